"""Camera math (src/scene/camera.rs:210-231) against the matrices the
reference serialised into its own scene files: the only golden vectors the
reference holds for this path.  Both the library's rdc_camera_update_matrices
and the oracle's restatement are checked."""
import json

import numpy as np
import pytest

import oracle
from raydar_gb300.scene import Camera, Scene
from tests.helpers import ulp_distance

# view / projection are float formulas evaluated in the reference's order:
# bit-exact.  The inverses come from different (but exact-in-double)
# elimination, so they agree to rounding: 4 ulp, or 1e-6 absolute for the
# entries that are zero up to cancellation in the reference.
INV_ABS_TOL = 1e-6
INV_ULP_TOL = 4


def _cams(golden_dir):
    return json.loads((golden_dir / "reference_cameras.json").read_text())


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_library_camera_matrices_match_reference_files(golden_dir, name):
    cam = Camera.from_json(_cams(golden_dir)[name])
    ref = [cam.view_matrix.copy(), cam.proj_matrix.copy(), cam.inverse_view_matrix.copy(),
           cam.inverse_proj_matrix.copy()]
    cam.update_matrices()
    assert np.array_equal(cam.view_matrix.view(np.uint32), ref[0].view(np.uint32)) or \
        np.array_equal(cam.view_matrix, ref[0])
    assert np.array_equal(cam.proj_matrix, ref[1])
    for mine, r in ((cam.inverse_view_matrix, ref[2]), (cam.inverse_proj_matrix, ref[3])):
        ok = (np.abs(mine - r) <= INV_ABS_TOL) | (ulp_distance(mine, r) <= INV_ULP_TOL)
        assert ok.all(), (mine, r)


@pytest.mark.parametrize("name", ["default", "benchmark"])
def test_oracle_camera_matrices_match_reference_files(golden_dir, name):
    cam = Camera.from_json(_cams(golden_dir)[name])
    view, proj, iview, iproj = oracle.camera_matrices(cam.to_c())
    assert np.array_equal(view, cam.view_matrix)
    assert np.array_equal(proj, cam.proj_matrix)
    for mine, r in ((iview, cam.inverse_view_matrix), (iproj, cam.inverse_proj_matrix)):
        ok = (np.abs(mine - r) <= INV_ABS_TOL) | (ulp_distance(mine, r) <= INV_ULP_TOL)
        assert ok.all()


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
