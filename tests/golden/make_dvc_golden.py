"""Convert the reference's discrete-Voronoi-weights known answers into a small JSON fixture.

Reads PICellerator/Weights/tests/DVCWeightsSuite.c (the ten 3D and ten 2D point coordinates that
_DVCWeightsSuite_InitialiseParticleCoords / ...2D assign, on a 10 x 10 (x 10) grid over
[-1, 1]^dim) and the expected centroids and weights the suite compares against
(PICellerator/Weights/tests/expected/DVCWeightsSuite_testGetCentroids.txt, ...2D.txt, printed
with six decimals), from the read-only reference tree, and writes tests/golden/dvc_golden.json.
Run once in a checkout that has the reference tree; the fixture is committed.
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
SUITE = os.path.join(REF, "PICellerator/Weights/tests/DVCWeightsSuite.c")
EXPECTED = os.path.join(REF, "PICellerator/Weights/tests/expected")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dvc_golden.json")


def coords(src, func, name):
    body = src[src.index(func):]
    body = body[:body.index("\n}\n")]
    out = {}
    for axis in "xyz":
        vals = re.findall(r"data->%s\[i\]\.%s\s*=\s*([-+0-9.eE]+)\s*;" % (re.escape(name), axis), body)
        if vals:
            out[axis] = [float(v) for v in vals]
    return out


def expected(path, dim):
    txt = open(path).read()
    cen = re.findall(r"centroids: \((?:cx, cy, cz|cx, cy)\) = \(([^)]*)\)", txt)
    wts = re.findall(r"weight = ([-+0-9.eE]+)", txt)
    return [[float(v) for v in c.split(",")][:dim] for c in cen], [float(v) for v in wts]


def main():
    src = open(SUITE).read()
    c3 = coords(src, "void _DVCWeightsSuite_InitialiseParticleCoords(", "pList")
    c2 = coords(src, "void _DVCWeightsSuite_InitialiseParticleCoords2D(", "pList2D")
    cen3, w3 = expected(os.path.join(EXPECTED, "DVCWeightsSuite_testGetCentroids.txt"), 3)
    cen2, w2 = expected(os.path.join(EXPECTED, "DVCWeightsSuite_testGetCentroids2D.txt"), 2)
    out = {
        "source": "PICellerator/Weights/tests/DVCWeightsSuite.c, expected/DVCWeightsSuite_testGetCentroids{,2D}.txt",
        "tolerance_note": "expected values are printed with six decimals",
        "3d": {"res": [10, 10, 10], "xi": [list(p) for p in zip(c3["x"], c3["y"], c3["z"])],
               "centroids": cen3, "weights": w3},
        "2d": {"res": [10, 10], "xi": [list(p) for p in zip(c2["x"], c2["y"])], "centroids": cen2, "weights": w2},
    }
    assert len(out["3d"]["xi"]) == len(cen3) == len(w3) == 10
    assert len(out["2d"]["xi"]) == len(cen2) == len(w2) == 10
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
