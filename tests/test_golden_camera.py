"""Camera math (src/scene/camera.rs:210-231) against the matrices the
reference serialised into its own scene files: the only golden vectors the
reference holds for this path.  Both the library's rdc_camera_update_matrices
and the oracle's restatement must reproduce all four matrices of both scenes
bit for bit: view and projection from cgmath 0.18's look_at_lh / perspective,
the inverses from its float Matrix4::invert."""
import json

import numpy as np
import pytest

import oracle
from raydar_gb300.scene import Camera, Scene


def _cams(golden_dir):
    return json.loads((golden_dir / "reference_cameras.json").read_text())


def _bits(m):
    return np.ascontiguousarray(m, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_library_camera_matrices_match_reference_files(golden_dir, name):
    cam = Camera.from_json(_cams(golden_dir)[name])
    ref = [cam.view_matrix.copy(), cam.proj_matrix.copy(), cam.inverse_view_matrix.copy(),
           cam.inverse_proj_matrix.copy()]
    cam.update_matrices()
    mine = [cam.view_matrix, cam.proj_matrix, cam.inverse_view_matrix, cam.inverse_proj_matrix]
    for k, (a, b) in enumerate(zip(mine, ref)):
        assert np.array_equal(_bits(a), _bits(b)), (k, a, b)


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_oracle_camera_matrices_match_reference_files(golden_dir, name):
    cam = Camera.from_json(_cams(golden_dir)[name])
    mine = oracle.camera_matrices(cam.to_c())
    ref = [cam.view_matrix, cam.proj_matrix, cam.inverse_view_matrix, cam.inverse_proj_matrix]
    for k, (a, b) in enumerate(zip(mine, ref)):
        assert np.array_equal(_bits(a), _bits(b)), (k, a, b)


def test_library_and_oracle_cameras_agree_on_seeded_cameras():
    """Beyond the two stored cameras: random positions, targets, resolutions,
    fields of view and both projections give the same 64 floats from the
    library and the oracle, and a camera whose projection is singular by
    cgmath's test (|det| <= f32::EPSILON) is rejected by both."""
    rng = np.random.default_rng(2029)
    for k in range(300):
        pos = rng.uniform(-50, 50, 3).astype(np.float32)
        tgt = rng.uniform(-5, 5, 3).astype(np.float32)
        w, h = int(rng.integers(1, 4000)), int(rng.integers(1, 4000))
        proj = "Perspective" if k % 3 else "Orthographic"
        cam = Camera.new(pos, tgt, [0.0, 1.0, 0.0], w, h, float(np.float32(rng.uniform(0.001, 1.0))),
                         float(np.float32(rng.uniform(10.0, 5000.0))), projection=proj,
                         fov=float(np.float32(rng.uniform(10.0, 120.0))), size=float(np.float32(rng.uniform(0.5, 8.0))))
        lib = [cam.view_matrix, cam.proj_matrix, cam.inverse_view_matrix, cam.inverse_proj_matrix]
        orc = oracle.camera_matrices(cam.to_c())
        for a, b in zip(lib, orc):
            assert np.array_equal(_bits(a), _bits(b))
    # ortho with a huge size: det of the projection = 2/(2 s a) * 2/(2 s) * -2/(f - n), far below f32::EPSILON
    from raydar_gb300 import native
    big = Camera.new([0, 0, -5], [0, 0, 0], [0, 1, 0], 100, 100, 0.01, 1000.0, projection="Orthographic", size=1.0)
    big.size = 1e4
    with pytest.raises(native.RdcError):
        big.update_matrices()
    with pytest.raises(RuntimeError):
        oracle.camera_matrices(big.to_c())


def test_orthographic_projection_is_invertible_and_consistent():
    cam = Camera.new([1, 2, -5], [0, 0, 0], [0, 1, 0], 640, 360, 0.1, 100.0, projection="Orthographic",
                     size=3.0)
    v, p, iv, ip = oracle.camera_matrices(cam.to_c())
    assert np.array_equal(p, cam.proj_matrix)
    P = cam.proj_matrix.reshape(4, 4).T.astype(np.float64)
    IP = cam.inverse_proj_matrix.reshape(4, 4).T.astype(np.float64)
    assert np.allclose(P @ IP, np.eye(4), atol=1e-6)


def test_rscn_round_trip_preserves_every_float(golden_dir, tmp_path):
    for name in ("default", "benchmark"):
        scene = Scene.load(golden_dir / f"{name}.rscn")
        out = tmp_path / f"{name}.rscn"
        scene.save(out)
        again = Scene.load(out)
        assert json.dumps(again.to_json()) == json.dumps(scene.to_json())
        assert again.camera.resolution_x == scene.camera.resolution_x
        assert len(again.objects) == len(scene.objects)
        assert np.array_equal(again.camera.inverse_proj_matrix, scene.camera.inverse_proj_matrix)


def test_benchmark_scene_inventory(golden_dir):
    scene = Scene.load(golden_dir / "benchmark.rscn")
    kinds = [o.geometry for o in scene.objects]
    assert (scene.width, scene.height) == (3840, 2160)
    assert kinds.count("Sphere") == 70 and kinds.count("Cube") == 113
