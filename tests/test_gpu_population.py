"""PCDVC population control (PICellerator/Utils/src/PCDVC.c:638-1060) on the GPU against the oracle's
sequential restatement: points with large Voronoi regions split at their region's centroid,
points with small regions deleted (the swarm's last point moving into the hole,
deleteIntParticleByIndexOnCPU :451-555), element after element.  The new point count, the cell
tables (bit-exact, in the reference's edited order), the coordinates, the integration points'
centroids and weights after the next assembly, and the element matrices assembled from them are
compared."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm((a - b).reshape(-1)) / max(np.linalg.norm(b.reshape(-1)), 1e-300)


def _clustered(dim, nel, seed):
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
    pts = np.array(pts)
    mat = np.array(mat, np.int32)
    order = rng.permutation(len(pts))   # swarm order not element ordered
    return pts[order], mat[order]


@pytest.mark.parametrize("dim,nel,res,kw", [(2, (6, 5), (10, 10), {}),
                                            (3, (6, 5, 4), (10, 10, 10), {}),
                                            (3, (5, 4, 4), (8, 8, 8), dict(max_deletions=4, max_splits=5,
                                                                             split_in_interface_cells=True,
                                                                             delete_in_interface_cells=True))])
def test_population_control_matches_oracle(oracle, uw, dim, nel, res, kw):
    O, U = oracle, uw
    pts, mat = _clustered(dim, nel, 1)
    mats = [U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0])], density=0.0),
            U.make_material([(U.LAW_MATERIAL_VISCOSITY, [10.0])], density=1.0)]
    with U.Context(0) as ctx:
        ctx.mesh_q1(dim, nel)
        ctx.bc_set(U.free_slip_mask(dim, nel))
        ctx.materials_set(mats)
        ctx.fields_set(None, 1.0, dim - 1)
        ctx.particles_upload(pts[:, 0], pts[:, 1], pts[:, 2] if dim == 3 else None, mat)
        perm0, off0, xi0 = ctx.bin_and_map()
        ctx.weights_set(U.WEIGHTS_DVC, res)
        n1 = ctx.population_control(**kw)
        perm1, off1 = ctx.cell_tables()
        x, y, z = ctx.particles()
        ctx.assemble()
        gxi, gw = ctx.integration_points()
        Ke, fe, Ge, Se = ctx.element_matrices()
    m = O.make_mesh(dim, nel)
    okw = {"max_deletions": kw.get("max_deletions", 2), "max_splits": kw.get("max_splits", 3),
           "split_in_interface": kw.get("split_in_interface_cells", False),
           "delete_in_interface": kw.get("delete_in_interface_cells", False)}
    X, M, S, off2, perm2, xo, wo = O.pcdvc(m, res, pts, mat, off0, perm0, xi0, **okw)
    print(f"{dim}D {nel}: {len(pts)} -> {n1} points (oracle {len(X)})")
    assert n1 == len(X) and n1 != len(pts)
    assert np.array_equal(off1, off2) and np.array_equal(perm1, perm2)
    got = np.stack([x, y] + ([z] if dim == 3 else []), axis=1)
    assert np.abs(got - X[:, :dim]).max() < 1e-15
    assert np.array_equal(gxi[:, :dim], xo[:, :dim]) and np.array_equal(gw, wo)
    # the assembly from the new points and weights against the oracle's
    f = O.make_fields(gravity=1.0, vert_axis=dim - 1)
    omats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [1.0])], density=0.0),
             O.make_material([(O.LAW_MATERIAL_VISCOSITY, [10.0])], density=1.0)]
    oK, ofe, oG, oS, _ = O.assemble(m, off2, perm2, xo, M, omats, f, weights=wo)
    assert _rel(Ke, oK) < 1e-12 and _rel(fe, ofe) < 1e-12 and _rel(Se, oS) < 1e-12
