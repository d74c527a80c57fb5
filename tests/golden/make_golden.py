"""Regenerate the golden fixtures from the reference checkout.

Reads the reference's two scene files (scenes/default.rscn and
scenes/benchmark.rscn) and writes, next to this script:
  reference_cameras.json   the camera block of each file: the inputs of
                           Camera::update_matrices (src/scene/camera.rs:210-231)
                           and the four matrices the reference computed and
                           serialised -- known-answer vectors for camera math
  default.rscn             scenes/default.rscn, re-serialised compactly
  benchmark.rscn           scenes/benchmark.rscn, re-serialised compactly (the
                           reference's own 3840x2160, 183-object benchmark scene)
Values are kept exactly as parsed (Python floats of the file's decimal text).

Usage: python tests/golden/make_golden.py REFERENCE_ROOT   (the root of a raydar checkout)
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    if not (ref / "scenes" / "default.rscn").exists():
        raise SystemExit(f"{ref}: not a raydar checkout (no scenes/default.rscn)")
    cams = {}
    for name in ("default", "benchmark"):
        data = json.loads((ref / "scenes" / f"{name}.rscn").read_text())
        cams[name] = data["camera"]
        (HERE / f"{name}.rscn").write_text(json.dumps(data, separators=(",", ":")))
    (HERE / "reference_cameras.json").write_text(json.dumps(cams, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
