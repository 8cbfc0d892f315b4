"""Make the particle-set fixture of the reference's soil-slope deck.

Data/Slopefail.mpm lists its 19640 particles point by point (a meshed
cross-section, not a generator rule), so tests/reference_decks.py cannot
write it from parameters. This script reads that list from the reference
tree and stores the values the reference reads (every real through GetReal,
FFI.f90:110-138, i.e. rounded to a 32-bit REAL) as
tests/golden/slopefail_points.npz: mass and x, y, z per particle, in order.

  python tests/golden/make_reference_fixtures.py [REFERENCE_TREE]

(default: $MPM3D_REFERENCE, else a 'reference' directory beside this
repository). The parser here is independent of the library's deck reader:
it splits the 'Particle point' body lines and rounds each number once from
its decimal text to float32 (numpy's correctly rounded conversion).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_point_list(path: str):
    rows, inside = [], False
    with open(path, errors="replace") as f:
        for line in f:
            t = line.replace(",", " ").replace("\t", " ").split("!")[0].split()
            if not t:
                continue
            if t[0].lower().startswith("part") and len(t) > 1 and t[1].lower().startswith("poin"):
                inside = True
                continue
            if inside:
                if t[0][0].isdigit() or t[0][0] == "-":
                    rows.append([np.float32(x.lower().replace("d", "e")) for x in t[2:6]])
                else:
                    inside = False
    a = np.array(rows, dtype=np.float32)
    return {"mass": a[:, 0], "x": a[:, 1], "y": a[:, 2], "z": a[:, 3]}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(
        "MPM3D_REFERENCE", os.path.join(os.path.dirname(os.path.dirname(HERE)), "..", "reference"))
    pts = read_point_list(os.path.join(ref, "Data", "Slopefail.mpm"))
    out = os.path.join(HERE, "slopefail_points.npz")
    np.savez_compressed(out, **pts)
    print(f"{out}: {pts['mass'].size} particles")


if __name__ == "__main__":
    main()
