"""Regenerate tests/golden/oracle_digests.json: SHA-256 digests of oracle
state after a few steps of each parity case, computed with the project libm
(identical on x86-64 and aarch64). They pin the oracle against silent changes;
the oracle itself is pinned by the published Cook-membrane results.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "mpm3d-f90_gb300")]

import numpy as np  # noqa: E402

import build  # noqa: E402
from gpu_cases import CASES  # noqa: E402

STEPS = 5
FIELDS = ("Mg", "PXg", "FXg", "Xp", "VXp", "SM", "SD", "VOL", "ie")


def main():
    build.build_oracle()
    import oracle

    out = {"note": "sha256 of little-endian float64 arrays after `steps` oracle steps (project libm)",
           "cases": {}}
    for name, (make, _) in sorted(CASES.items()):
        o = oracle.Oracle(deck_text=make(), libm="project")
        o.run(STEPS)
        out["cases"][name] = {"steps": STEPS, "digests": {
            f: hashlib.sha256(np.ascontiguousarray(o.download(f), dtype="<f8").tobytes()).hexdigest()
            for f in FIELDS}}
    with open(os.path.join(HERE, "oracle_digests.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
