"""Failure statuses of the solve, provoked on the host (no GPU fault involved).

- A NaN planted in a host input array before upload (a point density, or a point viscosity)
  reaches the Krylov residuals and the solve returns UWGPU_ERR_NAN: the reference declares
  KSP_DIVERGED_NAN when the residual norm is not a number
  (Solvers/KSPSolvers/src/BSSCR/bsscr-driver.c:528-531).
- A Schur iteration cap below what the tolerance needs, or a target residual the solve does not
  reach, returns UWGPU_ERR_NOT_CONVERGED with the report filled in.
- A Picard loop that does not meet its tolerance within max_iterations returns
  UWGPU_ERR_NOT_CONVERGED (SystemLinearEquations.c:908-914, "Failed to converge").
Every device loop is bounded by an iteration limit, so none of these can hang.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

UWGPU_ERR_NOT_CONVERGED = 6
UWGPU_ERR_NAN = 7


def _ctx(U, W, w):
    ctx = U.Context(0)
    W.setup_context(ctx, w)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    return ctx


def _opts(U, **kw):
    base = dict(mg_levels=3, schur_type=1, schur_pc=3, scr_rtol=1e-8, a11_rtol=1e-9, back_rtol=1e-9, max_outer=200,
                max_inner=500, bfbt_rtol=1e-4, bfbt_max_it=2000, smoother=1)
    base.update(kw)
    return U.default_opts(**base)


@pytest.mark.parametrize("field", ["rho", "eta"])
def test_nan_in_host_input_reports_nan(uw, field):
    from earthbyte_underworld_gb300 import workloads as W
    U = uw
    w = dict(W.grf(nel=(8, 8, 8), ppc=8, grid=32))
    arr = w[field].copy()
    arr[1234] = np.nan
    w[field] = arr
    ctx = _ctx(U, W, w)
    u, p, rep = ctx.solve_bsscr(_opts(U), check=False)
    assert rep.status == UWGPU_ERR_NAN, rep.status
    assert rep.converged == 0
    with pytest.raises(U.UwgpuError) as ei:
        ctx.solve_bsscr(_opts(U))
    assert ei.value.code == UWGPU_ERR_NAN
    ctx.close()


def test_iteration_cap_reports_not_converged(uw):
    from earthbyte_underworld_gb300 import workloads as W
    U = uw
    w = W.spheres(nel=(8, 8, 8), nspheres=10, seed=9)
    ctx = _ctx(U, W, w)
    # two Schur iterations cannot reach 1e-12
    u, p, rep = ctx.solve_bsscr(_opts(U, scr_rtol=1e-12, max_outer=2), check=False)
    assert rep.status == UWGPU_ERR_NOT_CONVERGED, rep.status
    assert rep.outer_its == 2 and rep.converged == 0
    assert np.isfinite(rep.rel_residual) and rep.rel_residual > 1e-12
    # a converged solve checked against a target residual it cannot meet
    u, p, rep = ctx.solve_bsscr(_opts(U, scr_rtol=1e-3, a11_rtol=1e-4, back_rtol=1e-4,
                                      target_rel_residual=1e-12), check=False)
    assert rep.status == UWGPU_ERR_NOT_CONVERGED, rep.status
    assert rep.rel_residual > 1e-12
    # the same solve with a target it meets
    u, p, rep = ctx.solve_bsscr(_opts(U, target_rel_residual=1e-5))
    assert rep.status == 0 and rep.rel_residual < 1e-5
    ctx.close()


def test_picard_not_converged(uw):
    from earthbyte_underworld_gb300 import workloads as W
    U = uw
    w = W.layers(nel=(6, 6, 8), ppc=20, cohesion_scale=1e-3)
    opts = _opts(U, mg_levels=2, scr_rtol=1e-10, a11_rtol=1e-12, back_rtol=1e-12)
    with U.Context(0) as ctx:
        W.setup_context(ctx, w)
        ctx.bin_and_map(want=False)
        u, p, rep, its, res = ctx.solve_picard(opts, tolerance=1e-14, max_iterations=2, check=False)
    assert rep.status == UWGPU_ERR_NOT_CONVERGED, rep.status
    assert its == 2 and res > 1e-14
