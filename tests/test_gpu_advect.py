"""Material-point advection (SwarmAdvector + TimeIntegrand) on the GPU against the oracle, with
the velocity of a real Stokes solve; then the ownership update (rebinning) of the moved points."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(U, W, case):
    w = W.rt2d(nel=(16, 16), ppc=12) if case == "rt2d" else W.spheres(nel=(8, 8, 8), nspheres=10, seed=9)
    ctx = U.Context(0)
    W.setup_context(ctx, w)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    opts = U.default_opts(mg_levels=3, schur_type=1, schur_pc=3, scr_rtol=1e-10, a11_rtol=1e-12, back_rtol=1e-12,
                          max_outer=400, bfbt_rtol=1e-6, bfbt_max_it=5000)
    u, p, rep = ctx.solve_bsscr(opts)
    assert rep.rel_residual < 1e-8
    return ctx, w, u


def _xyz(w):
    z = w["z"] if w["z"] is not None else np.zeros_like(w["x"])
    return np.stack([w["x"], w["y"], z], axis=1)


@pytest.mark.parametrize("case,order", [("rt2d", 2), ("spheres", 2), ("spheres", 1)])
def test_advection_matches_oracle_and_rebins(oracle, uw, case, order):
    from earthbyte_underworld_gb300 import workloads as W
    O, U = oracle, uw
    ctx, w, u = _setup(U, W, case)
    dim = w["dim"]
    h = 1.0 / max(w["nel"])
    dt = 0.4 * h / np.abs(u).max()          # up to 0.4 of an element per step
    m = O.make_mesh(dim, w["nel"])
    xyz = _xyz(w)
    for step in range(2):
        fb, left = ctx.advect(dt, order=order)
        ref, failed, ofb = O.advect(m, u.reshape(-1, dim), xyz, dt, order=order)
        assert failed == 0 and fb == ofb == 0
        x, y, z = ctx.particles()
        got = np.stack([x, y, z if dim == 3 else np.zeros_like(x)], axis=1)
        # closed-form local coordinates on the GPU, Newton in the oracle: rounding only
        assert np.max(np.abs(got - ref)) < 1e-13
        assert np.max(np.abs(got - xyz)) > 0.1 * h   # the points did move
        xyz = ref
        assert left == 0
        # ownership update: the moved points bin exactly as the oracle's moved points
        perm, offsets, xi = ctx.bin_and_map()
        _, ooff, operm, oxi, outside = O.map_points(m, ref)
        assert outside == 0
        assert np.array_equal(offsets, ooff) and np.array_equal(perm, operm)
    ctx.close()


def test_advection_fallback_and_refusal(oracle, uw):
    """A step long enough that predictors leave the mesh: without the first-order fallback the
    call is refused and no point moves; with it, the points whose predictor left use the
    first-order update, as the oracle does."""
    from earthbyte_underworld_gb300 import workloads as W
    O, U = oracle, uw
    ctx, w, u = _setup(U, W, "spheres")
    m = O.make_mesh(3, w["nel"])
    xyz = _xyz(w)
    dt = 6.0 / np.abs(u).max()                # several mesh widths per step
    with pytest.raises(U.UwgpuError) as err:
        ctx.advect(dt, order=2)
    assert err.value.code == U.ERR_DOMAIN
    x, y, z = ctx.particles()
    assert np.array_equal(np.stack([x, y, z], axis=1), xyz)
    ref, failed, ofb = O.advect(m, u.reshape(-1, 3), xyz, dt, order=2, allow_fallback=True)
    fb, left = ctx.advect(dt, order=2, allow_fallback=True)
    assert failed == 0 and fb == ofb and fb > 0
    x, y, z = ctx.particles()
    assert np.max(np.abs(np.stack([x, y, z], axis=1) - ref)) < 1e-12
    outside = np.sum(np.any((ref < 0.0) | (ref > 1.0), axis=1))
    assert left == outside
    ctx.close()
