"""The inner operator of the scaled BFBt preconditioner, G^T W G with W = 1/rowmax(K)
(Solvers/KSPSolvers/src/BSSCR/pc_ScaledGtKG.c:735-760), in its three GPU forms through the C ABI
(uwgpu_bfbt_operator_apply): the FP64 element stencil, the FP32 matrix-free tiled apply of the
mixed form, and the FP32 stencil.  The reference product is formed here from the element G_e,
the oracle's assembled K (rows over free dofs, BCs removed) and its equation numbering."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _gtwg_reference(O, w, Ke, Ge):
    import scipy.sparse as sp
    dim, nel = w["dim"], w["nel"]
    m = O.make_mesh(dim, nel)
    rp, ci, v, eq, nf = O.global_csr(m, Ke, w["fixed"])
    rowmax = np.maximum.reduceat(v, rp[:-1])
    Wf = 1.0 / rowmax
    E = int(np.prod(nel))
    nnx, nny = nel[0] + 1, nel[1] + 1
    e = np.arange(E)
    ix, iy = e % nel[0], (e // nel[0]) % nel[1]
    iz = e // (nel[0] * nel[1]) if dim == 3 else np.zeros_like(e)
    rows, cols, vals = [], [], []
    for a in range(1 << dim):
        dx, dy, dz = a & 1, (a >> 1) & 1, (a >> 2) & 1
        node = (ix + dx) + nnx * ((iy + dy) + nny * (iz + dz)) if dim == 3 else (ix + dx) + nnx * (iy + dy)
        for d in range(dim):
            r = eq[node * dim + d]
            keep = r >= 0
            rows.append(r[keep])
            cols.append(e[keep])
            vals.append(Ge[keep, a * dim + d])
    G = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nf, E))
    return (G.T @ sp.diags(Wf) @ G).tocsr()


@pytest.mark.parametrize("case", ["rt2d", "rt2d_ragged", "spheres", "spheres_ragged"])
def test_bfbt_inner_operator_forms_match_reference(oracle, uw, case):
    """Every form against G^T W G assembled from the element matrices: FP64 to rounding, the FP32
    forms to FP32 rounding.  The ragged meshes leave partial tiles along every axis."""
    from earthbyte_underworld_gb300 import workloads as W
    O, U = oracle, uw
    w = {"rt2d": lambda: W.rt2d(nel=(32, 16), ppc=12),
         "rt2d_ragged": lambda: W.rt2d(nel=(37, 19), ppc=12),
         "spheres": lambda: W.spheres(nel=(16, 16, 16), nspheres=20, seed=5),
         "spheres_ragged": lambda: W.spheres(nel=(20, 10, 9), nspheres=12, seed=4)}[case]()
    ctx = U.Context(0)
    W.setup_context(ctx, w)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    Ke, fe, Ge, Se = ctx.element_matrices()
    ctx.operator_apply(np.zeros(ctx.nnodes * w["dim"]))   # builds the fine operator
    A = _gtwg_reference(O, w, Ke, Ge)
    rng = np.random.default_rng(7)
    x = rng.standard_normal(A.shape[0])
    yo = A @ x
    y0 = ctx.bfbt_operator_apply(x, form=0)
    y1 = ctx.bfbt_operator_apply(x, form=1)
    y2 = ctx.bfbt_operator_apply(x, form=2)
    ctx.close()
    assert _rel(y0, yo) < 1e-12
    assert _rel(y1, yo) < 1e-5
    assert _rel(y2, yo) < 1e-5


def test_bfbt_matrix_free_deep_tiles_match_stencil(uw):
    """A mesh large enough for the four-element-deep tiles (four tiles per SM), with a strongly
    varying W (GRF viscosity over six decades): the FP32 matrix-free apply against the FP64
    stencil."""
    from earthbyte_underworld_gb300 import workloads as W
    U = uw
    w = W.grf(nel=(96, 96, 112), ppc=4, grid=64, corr=0.1)
    ctx = U.Context(0)
    W.setup_context(ctx, w)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    ctx.operator_apply(np.zeros(ctx.nnodes * 3))
    rng = np.random.default_rng(1)
    x = rng.standard_normal(96 * 96 * 112)
    y0 = ctx.bfbt_operator_apply(x, form=0)
    y1 = ctx.bfbt_operator_apply(x, form=1)
    ctx.close()
    assert _rel(y1, y0) < 1e-5
