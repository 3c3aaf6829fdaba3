"""Convert the reference's discrete-Voronoi-weights known answers into a small JSON fixture.

Reads PICellerator/Weights/tests/DVCWeightsSuite.c (the ten 3D and ten 2D point coordinates that
_DVCWeightsSuite_InitialiseParticleCoords / ...2D assign, on a 10 x 10 (x 10) grid over
[-1, 1]^dim), the expected centroids and weights the suite compares against
(PICellerator/Weights/tests/expected/DVCWeightsSuite_testGetCentroids.txt, ...2D.txt, printed
with six decimals) and the expected cell grids (links and centres,
DVCWeightsSuite_testConstructGrid.txt, ...2D.txt), and the PCDVC integration suite's setup and
expected error statistics (PICellerator/Utils/tests/input/testPCDVC.xml, testElementIntegral.xml,
expected/testPCDVC_{CircleInterface,PolynomialFunction,ExponentialInterface}.expected: a tolerance
and a value for the mean relative error, then for its standard deviation), and the same statistics
that PICellerator/Weights/tests/ConstantWeightsSuite.c states for ConstantWeights (its
WeightsSuite_TestElementIntegral calls, on input/testConstantWeights.xml), from the read-only
reference tree, and writes tests/golden/dvc_golden.json.
Run once with the reference tree's path as the only argument; the fixture is committed.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit(f"usage: python {os.path.basename(__file__)} <path of the Underworld 1.x source tree>")
REF = sys.argv[1]
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


def grid(path, dim):
    """cell links (N, S, E, W[, U, D]) and centres of _DVCWeights_ConstructGrid{,2D} as the suite's
    expected file prints them"""
    txt = open(path).read()
    keys = "NSEWUD"[:2 * dim]
    pat = r"Values: \(" + ", ".join(k + r": (-?\d+)" for k in keys) + r"\)"
    links = [[int(v) for v in m] for m in re.findall(pat, txt)]
    cen = [[float(v) for v in c.split(",")] for c in re.findall(r"Coords: \(([^)]*)\)", txt)]
    assert len(links) == len(cen)
    return links, cen


def _params(path):
    txt = re.sub(r"<!--.*?-->", "", open(path).read(), flags=re.S)
    return {k: v.strip() for k, v in re.findall(r'<param name="([^"]+)"[^>]*>([^<]*)</param>', txt)}


def pcdvc_suite():
    tests = os.path.join(REF, "PICellerator/Utils/tests")
    base = _params(os.path.join(tests, "input/testElementIntegral.xml"))
    pc = _params(os.path.join(tests, "input/testPCDVC.xml"))
    cases = {}
    for name in ("CircleInterface", "PolynomialFunction", "ExponentialInterface"):
        vals = [float(v) for v in open(os.path.join(tests, "expected", f"testPCDVC_{name}.expected")).read().split()[:4]]
        cases[name] = {"mean_tol": vals[0], "mean": vals[1], "sd_tol": vals[2], "sd": vals[3]}
    return {
        "source": "PICellerator/Utils/tests/PCDVCSuite.c with input/testPCDVC.xml",
        "elementRes": [int(base["elementResI"]), int(base["elementResJ"])],
        "min": [float(base["minX"]), float(base["minY"])],
        "max": [float(base["maxX"]), float(base["maxY"])],
        "particleCount": int(base["particleCount"]),
        "sampleSize": int(base["SampleSize"]),
        "res": [int(pc["resolutionX"]), int(pc["resolutionY"])],
        "maxDeletions": int(pc["maxDeletions"]), "maxSplits": int(pc["maxSplits"]),
        "cases": cases,
    }


def constant_weights_suite():
    tests = os.path.join(REF, "PICellerator/Weights/tests")
    base = _params(os.path.join(tests, "input/testElementIntegral.xml"))
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(tests, "ConstantWeightsSuite.c")).read(), flags=re.S)
    cases = {}
    for args in re.findall(r"WeightsSuite_TestElementIntegral\(\s*data->context,([^;]*)\);", src):
        a = [v.strip() for v in args.split(",")]
        name = a[0].strip('"')
        cases[name] = {"count": int(a[1]), "mean_tol": float(a[2]), "sd_tol": float(a[3]),
                       "mean": float(a[4]), "sd": float(a[5])}
    assert len(cases) == 6, cases
    return {
        "source": "PICellerator/Weights/tests/ConstantWeightsSuite.c with input/testConstantWeights.xml",
        "elementRes": [int(base["elementResI"]), int(base["elementResJ"])],
        "min": [float(base["minX"]), float(base["minY"])],
        "max": [float(base["maxX"]), float(base["maxY"])],
        "particleCount": int(base["particleCount"]),
        "cases": cases,
    }


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
    l3, g3 = grid(os.path.join(EXPECTED, "DVCWeightsSuite_testConstructGrid.txt"), 3)
    l2, g2 = grid(os.path.join(EXPECTED, "DVCWeightsSuite_testConstructGrid2D.txt"), 2)
    out["grid3d"] = {"res": [10, 10, 10], "links": l3, "centres": g3}
    out["grid2d"] = {"res": [10, 10], "links": l2, "centres": g2}
    assert len(l3) == 1000 and len(l2) == 100
    assert len(out["3d"]["xi"]) == len(cen3) == len(w3) == 10
    assert len(out["2d"]["xi"]) == len(cen2) == len(w2) == 10
    out["pcdvc_suite"] = pcdvc_suite()
    out["constant_weights_suite"] = constant_weights_suite()
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
