"""The benchmark's reference arm times the CPU restatement of the reference
renderer; its process must not load the CUDA library at all.  It builds the
headline scene with the oracle's camera matrices, which must equal the
library's bit for bit, so both arms render the same scene."""
import json
import subprocess
import sys

import numpy as np

from tests.conftest import ROOT

PROBE = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
w = bench.reference_workload()
from raydar_gb300 import native
maps = open("/proc/self/maps").read()
cam = w.scene.camera
print(json.dumps({
    "lib_loaded": native._lib is not None or "libraydar_cuda" in maps,
    "oracle_loaded": "liboracle_raydar" in maps,
    "objects": len(w.scene.objects),
    "mats": [m.view(np.uint32).tolist() for m in (cam.view_matrix, cam.proj_matrix,
                                                 cam.inverse_view_matrix, cam.inverse_proj_matrix)],
}))
""".replace("import json, sys", "import json, sys\nimport numpy as np")


def test_reference_arm_never_loads_the_cuda_library():
    out = subprocess.run([sys.executable, "-c", PROBE, str(ROOT)], capture_output=True, text=True, check=True)
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert not d["lib_loaded"]
    assert d["oracle_loaded"]
    assert d["objects"] == 81

    import bench
    w = bench._workload()  # this process: the library's rdc_camera_update_matrices
    cam = w.scene.camera
    ours = [m.view(np.uint32).tolist() for m in (cam.view_matrix, cam.proj_matrix, cam.inverse_view_matrix,
                                                 cam.inverse_proj_matrix)]
    assert d["mats"] == ours
