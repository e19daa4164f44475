"""Regenerates tests/golden/ref_math.json from the reference's own math headers.

Runs only where a reference checkout exists (not on the GPU host): builds
oracle/_ref/ref_golden with oracle/build_ref.sh, runs it and freezes its JSON output.
The fixture then travels with the tests.

    AXIOM_REFERENCE=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent


def main() -> int:
    exe = subprocess.run([str(ROOT / "oracle" / "build_ref.sh")], check=True, capture_output=True,
                         text=True).stdout.strip().splitlines()[-1]
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    data = json.loads(out)
    data["_source"] = ("computed by include/axiom/math/{vec3,aabb,random}.hpp of "
                       "itsakeyfut/axiom-physics-engine via oracle/ref_golden.cpp")
    (HERE / "ref_math.json").write_text(json.dumps(data, separators=(",", ":")) + "\n")
    print(HERE / "ref_math.json")
    return 0


if __name__ == "__main__":
    sys.exit(main())
