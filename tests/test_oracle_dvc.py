"""The oracle's discrete Voronoi cell weights (DVCWeights.c restated) against the reference's known
answers (PICellerator/Weights/tests/DVCWeightsSuite.c and its expected files, converted by
tests/golden/make_dvc_golden.py), the invariants of the construction, and the integration error
statistics of PICellerator/Utils/tests/PCDVCSuite.c and PICellerator/Weights/tests/
ConstantWeightsSuite.c."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "dvc_golden.json")


@pytest.mark.parametrize("key,dim", [("3d", 3), ("2d", 2)])
def test_dvc_matches_reference_known_answers(oracle, key, dim):
    g = json.load(open(GOLDEN))[key]
    cxi, w, passes = oracle.dvc_element(dim, g["res"], np.array(g["xi"]))
    # the expected files print six decimals
    assert np.abs(cxi - np.array(g["centroids"])).max() < 1e-6
    assert np.abs(w - np.array(g["weights"])).max() < 1e-6
    assert passes > 1


@pytest.mark.parametrize("key,dim", [("grid3d", 3), ("grid2d", 2)])
def test_dvc_grid_matches_reference_construction(oracle, key, dim):
    """Cell links and centres equal _DVCWeights_ConstructGrid{,2D}'s (the suite's expected grid
    files: links exactly, centres to their six printed decimals)."""
    g = json.load(open(GOLDEN))[key]
    centre, nbr = oracle.dvc_grid(dim, g["res"])
    assert np.array_equal(nbr, np.array(g["links"], dtype=np.int32))
    assert np.abs(centre - np.array(g["centres"])).max() < 1e-6


@pytest.mark.parametrize("dim,res", [(3, (10, 10, 10)), (2, (10, 10)), (3, (8, 6, 5)), (2, (32, 32))])
def test_dvc_partition_invariants(oracle, dim, res):
    """The regions tile the element: weights sum to 2^dim, every weight is a whole number of
    cells, and a region's centroid lies inside the element; duplicate points (a later point takes
    the shared cell) and points on the upper faces are handled."""
    rng = np.random.default_rng(4)
    h = 2.0 / np.array(res)
    da = np.prod(h)
    for n in (1, 2, 7, 27, 60):
        xi = rng.uniform(-1.0, 1.0, (n, dim))
        if n >= 7:
            xi[3] = xi[2]           # two points in one cell
            xi[4, 0] = 1.0          # on the upper x face
        cxi, w, _ = oracle.dvc_element(dim, res, xi)
        assert abs(w.sum() - 2.0 ** dim) < 1e-12
        cells = w / da
        assert np.allclose(cells, np.round(cells), atol=1e-9)
        held = w > 0
        assert np.all(np.abs(cxi[held]) <= 1.0)
        assert np.all(cxi[~held] == 0.0)


def _clustered_swarm(dim, nel, seed):
    """3..14 points per element, half of them crowded towards one corner; 20 % material 1."""
    rng = np.random.default_rng(seed)
    E = int(np.prod(nel))
    pts, mat = [], []
    for e in range(E):
        idx = [e % nel[0], (e // nel[0]) % nel[1]] + ([e // (nel[0] * nel[1])] if dim == 3 else [])
        for _ in range(int(rng.integers(3, 15))):
            loc = rng.uniform(0, 1, dim) ** 2.5 if rng.uniform() < 0.5 else rng.uniform(0, 1, dim)
            pts.append([(idx[d] + loc[d]) / nel[d] for d in range(dim)] + [0.0] * (3 - dim))
            mat.append(int(rng.uniform() < 0.2))
    order = rng.permutation(len(pts))
    return np.array(pts)[order], np.array(mat, np.int32)[order]


@pytest.mark.parametrize("dim,nel,res", [(2, (6, 5), (10, 10)), (3, (6, 5, 4), (10, 10, 10)),
                                         (3, (5, 4, 4), (8, 8, 8))])
def test_pcdvc_weights_follow_the_moved_points(oracle, dim, nel, res):
    """After a population-control pass the weight of every slot is the discrete Voronoi weight of
    its point within its element's final point set: a DVC pass over the final swarm (points mapped
    back to local coordinates) gives the same weights and centroids.  Deleting a point moves the
    swarm's last point into the hole; its weight moves with it (deleteIntParticleByIndexOnCPU,
    PICellerator/Utils/src/PCDVC.c:451-555)."""
    O = oracle
    pts, mat = _clustered_swarm(dim, nel, 1)
    m = O.make_mesh(dim, nel)
    _, off0, perm0, xi0, _ = O.map_points(m, pts)
    X, M, S, off2, perm2, xo, wo = O.pcdvc(m, res, pts, mat, off0, perm0, xi0, max_deletions=4, max_splits=5)
    assert len(X) != len(pts)
    _, off3, perm3, xi3, out = O.map_points(m, X)
    assert out == 0
    # the same points per element (the pass keeps its own order within an element)
    for e in range(int(np.prod(nel))):
        assert sorted(perm2[off2[e]:off2[e + 1]]) == sorted(perm3[off3[e]:off3[e + 1]])
    # local coordinates of the final swarm in the pass's slot order
    slot_of = np.empty(len(X), np.int64)
    slot_of[perm3] = np.arange(len(X))
    xi_final = xi3[slot_of[perm2]]
    cx, w = O.dvc_weights(m, res, off2, xi_final)
    assert np.allclose(w, wo, rtol=0, atol=1e-14)
    assert np.allclose(cx[:, :dim], xo[:, :dim], rtol=0, atol=1e-14)


# PICellerator/Utils/tests/PCDVCSuite.c: the integrands (functions of the local coordinates) and
# their exact integrals over the reference element [-1, 1]^2
PCDVC_CASES = {
    "CircleInterface": (lambda x, y: (x * x + y * y <= 1.0).astype(float), np.pi),
    "PolynomialFunction": (lambda x, y: 11 + 2 * x * x + 3 * x ** 3 * y + y + x ** 3 + 2 * y * y, 148.0 / 3.0),
    "ExponentialInterface": (lambda x, y: (y <= 0.1 * np.exp(2 * x)).astype(float),
                             0.05 * (np.exp(2.0) - np.exp(-2.0)) + 2.0),
}


def test_pcdvc_suite_integration_error_statistics(oracle):
    """PCDVCSuite.c: for seeds 0 .. SampleSize - 1, Swarm_Random_Seed(seed) and a RandomParticleLayout
    of 20 points per cell on a 2 x 2 mesh over [0, 4]^2; the integration points of element 0 get
    PCDVC weights (resolution 10, no splits or deletions, so the discrete Voronoi centroids and
    volumes); each integrand is integrated over the element at those points and weights.  The mean
    and the standard deviation of the relative error must lie within the suite's tolerances of its
    expected values (expected/testPCDVC_*.expected).  The oracle's layout restates the reference's
    Park-Miller stream, so the samples are the reference's own."""
    O = oracle
    g = json.load(open(GOLDEN))["pcdvc_suite"]
    assert g["maxDeletions"] == 0 and g["maxSplits"] == 0
    m = O.make_mesh(2, g["elementRes"] + [1], mn=g["min"] + [0.0], mx=g["max"] + [1.0])
    errs = {k: [] for k in PCDVC_CASES}
    for seed in range(g["sampleSize"]):
        xyz = O.random_layout(m, g["particleCount"], seed)
        _, off, perm, xi, outside = O.map_points(m, xyz)
        assert outside == 0 and off[1] - off[0] == g["particleCount"]
        cxi, w, _ = O.dvc_element(2, g["res"], xi[off[0]:off[1], :2])
        assert abs(w.sum() - 4.0) < 1e-12   # the element's local area; detJ = 1 for its 2 x 2 size
        for name, (f, exact) in PCDVC_CASES.items():
            errs[name].append(abs(np.sum(w * f(cxi[:, 0], cxi[:, 1])) - exact) / abs(exact))
    for name, c in g["cases"].items():
        e = np.array(errs[name])
        mean = e.mean()
        sd = np.sqrt((e * e).mean() - mean * mean)
        assert abs(c["mean"] - mean) < c["mean_tol"], (name, mean)
        assert abs(c["sd"] - sd) < c["sd_tol"], (name, sd)


# PICellerator/Weights/tests/ConstantWeightsSuite.c: integrands and exact integrals over [-1, 1]^2
CONSTANT_WEIGHTS_CASES = {
    "ConstantFunction": (lambda x, y: -3.0, -12.0),
    "LinearFunction": (lambda x, y: 2.0 + 2.2 * x - y, 8.0),
    "QuadraticFunction": (lambda x, y: 1 + x + x * x, 16.0 / 3.0),
    "PolynomialFunction": (lambda x, y: 11 + 2 * x * x + 3 * x * x * x * y + y + x * x * x + 2 * y * y, 148.0 / 3.0),
    "CircleInterface": (lambda x, y: float(x * x + y * y <= 1.0), np.pi),
    "ExponentialInterface": (lambda x, y: float(y <= 0.1 * np.exp(2 * x)), 0.05 * (np.exp(2.0) - np.exp(-2.0)) + 2.0),
}


def test_constant_weights_suite_integration_error_statistics(oracle):
    """ConstantWeightsSuite.c (WeightsSuite_TestElementIntegral): the same seeded layouts as the
    PCDVC suite, integrated over element 0 at the points' own local coordinates with the constant
    weights 4 / count (ConstantWeights.c:180-189); the reference states the mean and standard
    deviation of the relative error to six digits with a tolerance of 1e-6 (1e-10 for the constant
    integrand).  The oracle meets every one: its layout, element search, local coordinates and
    weights reproduce the reference's samples."""
    O = oracle
    g = json.load(open(GOLDEN))["constant_weights_suite"]
    m = O.make_mesh(2, g["elementRes"] + [1], mn=g["min"] + [0.0], mx=g["max"] + [1.0])
    count = {c["count"] for c in g["cases"].values()}
    assert len(count) == 1
    errs = {k: [] for k in CONSTANT_WEIGHTS_CASES}
    for seed in range(count.pop()):
        xyz = O.random_layout(m, g["particleCount"], seed)
        _, off, perm, xi, outside = O.map_points(m, xyz)
        assert outside == 0
        pts = xi[off[0]:off[1]]
        w = 4.0 / len(pts)
        for name, (f, exact) in CONSTANT_WEIGHTS_CASES.items():
            integral = 0.0
            for x, y in pts[:, :2]:          # in the swarm's order, as FeVariable_IntegrateElement sums
                integral += 1.0 * w * f(x, y)
            errs[name].append(abs(integral - exact) / abs(exact))
    for name, c in g["cases"].items():
        e = np.array(errs[name])
        mean = e.mean()
        sd = np.sqrt((e * e).mean() - mean * mean)
        assert abs(mean - c["mean"]) <= c["mean_tol"], (name, mean)
        assert abs(sd - c["sd"]) <= c["sd_tol"], (name, sd)
