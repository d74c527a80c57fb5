"""Small helpers shared by the tests."""
import numpy as np


def ulp_distance(a, b) -> np.ndarray:
    """|a - b| in float32 units in the last place (sign-magnitude aware)."""
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def bits_equal(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def shrink(scene, width, height):
    """Same scene at another resolution (raydar_gb300.scene.resized)."""
    from raydar_gb300.scene import resized
    return resized(scene, width, height)
