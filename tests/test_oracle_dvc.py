"""The oracle's discrete Voronoi cell weights (DVCWeights.c restated) against the reference's known
answers (PICellerator/Weights/tests/DVCWeightsSuite.c and its expected files, converted by
tests/golden/make_dvc_golden.py), and the invariants of the construction."""
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
