"""Discrete Voronoi cell weights on the GPU (uwgpu_weights_set(UWGPU_WEIGHTS_DVC)) against the oracle's
restatement of PICellerator/Weights/src/DVCWeights.c and the reference's known answers, then the
assembly with those integration points and weights."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "dvc_golden.json")


def _rel(a, b):
    return np.linalg.norm((a - b).reshape(-1)) / max(np.linalg.norm(b.reshape(-1)), 1e-300)


@pytest.mark.parametrize("key,dim", [("3d", 3), ("2d", 2)])
def test_dvc_known_answers_through_the_abi(oracle, uw, key, dim):
    """The reference suite's ten points in one element of a 1 x 1 (x 1) mesh on the unit cube."""
    O, U = oracle, uw
    g = json.load(open(GOLDEN))[key]
    xi = np.array(g["xi"])
    x = (xi + 1.0) / 2.0
    nel = (1,) * dim
    ctx = U.Context(0)
    ctx.mesh_q1(dim, nel)
    ctx.bc_set(U.free_slip_mask(dim, nel))
    ctx.materials_set([U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0])], density=1.0)])
    ctx.fields_set(None, 1.0, dim - 1)
    ctx.particles_upload(x[:, 0], x[:, 1], x[:, 2] if dim == 3 else None, np.zeros(len(x), np.int32))
    perm, offsets, mxi = ctx.bin_and_map()
    ctx.weights_set(U.WEIGHTS_DVC, g["res"])
    ctx.assemble()
    gxi, gw = ctx.integration_points()
    ctx.close()
    order = np.argsort(perm)          # slot of each point
    assert np.abs(gxi[order, :dim] - np.array(g["centroids"])).max() < 1e-6
    assert np.abs(gw[order] - np.array(g["weights"])).max() < 1e-6
    # bit-exact against the oracle on the same local coordinates
    cxi, w, _ = O.dvc_element(dim, g["res"], mxi[:, :dim])
    assert np.array_equal(gxi[:, :dim], cxi) and np.array_equal(gw, w)


def _case(W, name):
    return {"spheres": lambda: W.spheres(nel=(8, 6, 10), nspheres=12, seed=4),
            "rt2d": lambda: W.rt2d(nel=(16, 12), ppc=20),
            "grf": lambda: W.grf(nel=(6, 6, 6), ppc=30, grid=32, corr=0.2)}[name]()


@pytest.mark.parametrize("name,res", [("spheres", (10, 10, 10)), ("rt2d", (10, 10)), ("grf", (8, 12, 10)),
                                      ("rt2d", (32, 32))])
def test_dvc_weights_bit_exact_and_assembly(oracle, uw, name, res):
    """Every element's centroids and weights equal the oracle's bit for bit; K_e, f_e assembled from
    them equal the oracle's assembly with the same points and weights."""
    from earthbyte_underworld_gb300 import workloads as W
    from test_gpu_parity import _mats_oracle
    O, U = oracle, uw
    w = _case(W, name)
    dim = w["dim"]
    ctx = U.Context(0)
    W.setup_context(ctx, w)
    perm, offsets, xi = ctx.bin_and_map()
    ctx.weights_set(U.WEIGHTS_DVC, res)
    ctx.assemble()
    gxi, gw = ctx.integration_points()
    Ke, fe, Ge, Se = ctx.element_matrices()
    ctx.close()
    m = O.make_mesh(dim, w["nel"])
    cxi, cw = O.dvc_weights(m, res, offsets, xi)
    assert np.array_equal(gxi, cxi)
    assert np.array_equal(gw, cw)
    # the weights tile every element
    esum = np.add.reduceat(cw, offsets[:-1].astype(np.int64))
    assert np.allclose(esum, 2.0 ** dim, rtol=0, atol=1e-12)
    f = O.make_fields(temperature=w.get("temperature"), gravity=w["gravity"], vert_axis=w["vert_axis"])
    oKe, ofe, oGe, oSe, _ = O.assemble(m, offsets, perm, cxi, w["material"], _mats_oracle(O, w["materials"]), f,
                                       point_eta=w.get("eta"), point_rho=w.get("rho"), weights=cw)
    assert _rel(Ke, oKe) < 1e-12 and _rel(fe, ofe) < 1e-12 and _rel(Se, oSe) < 1e-12


def test_dvc_ragged_element_and_solve(oracle, uw):
    """One element with 400 points beside elements with one or two: the growth and the centroid
    pass do not depend on the count; then a Stokes solve with the DVC weights converges."""
    O, U = oracle, uw
    nel = (3, 3, 3)
    rng = np.random.default_rng(5)
    pts = [[rng.uniform(0.0, 1 / 3), rng.uniform(0.0, 1 / 3), rng.uniform(0.0, 1 / 3)] for _ in range(400)]
    for e in range(27):
        i, j, k = e % 3, (e // 3) % 3, e // 9
        for _ in range(1 + e % 2):
            pts.append([(i + rng.uniform()) / 3, (j + rng.uniform()) / 3, (k + rng.uniform()) / 3])
    p = np.array(pts)[rng.permutation(len(pts))]
    mat = (p[:, 2] > 0.5).astype(np.int32)
    ctx = U.Context(0)
    ctx.mesh_q1(3, nel)
    ctx.bc_set(U.free_slip_mask(3, nel))
    ctx.materials_set([U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0 + 9.0 * k])], density=float(k))
                       for k in range(2)])
    ctx.fields_set(None, 1.0, 2)
    ctx.particles_upload(p[:, 0], p[:, 1], p[:, 2], mat)
    perm, offsets, xi = ctx.bin_and_map()
    ctx.weights_set(U.WEIGHTS_DVC, (10, 10, 10))
    ctx.assemble()
    gxi, gw = ctx.integration_points()
    cxi, cw = O.dvc_weights(O.make_mesh(3, nel), (10, 10, 10), offsets, xi)
    assert np.diff(offsets).max() >= 400
    assert np.array_equal(gxi, cxi) and np.array_equal(gw, cw)
    opts = U.default_opts(mg_levels=1, schur_type=1, schur_pc=0, scr_rtol=1e-8, a11_rtol=1e-10, back_rtol=1e-10,
                          max_outer=400, max_inner=2000)
    u, pr, rep = ctx.solve_bsscr(opts)
    ctx.close()
    assert rep.rel_residual < 1e-7
    # constant weights give a different operator: the switch reaches the assembly
    ctx2 = U.Context(0)
    ctx2.mesh_q1(3, nel)
    ctx2.bc_set(U.free_slip_mask(3, nel))
    ctx2.materials_set([U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0 + 9.0 * k])], density=float(k))
                        for k in range(2)])
    ctx2.fields_set(None, 1.0, 2)
    ctx2.particles_upload(p[:, 0], p[:, 1], p[:, 2], mat)
    ctx2.bin_and_map(want=False)
    ctx2.assemble()
    _, w0 = ctx2.integration_points()
    ctx2.close()
    assert not np.allclose(w0, gw)
    assert np.allclose(np.add.reduceat(w0, offsets[:-1].astype(np.int64)), 8.0)
