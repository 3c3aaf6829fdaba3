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
