"""The GPU path on the reference's analytic-solution tests: solCx (viscosity jump 100 : 1 at
x = 0.5, Underworld/SysTest/PerformanceTests/testVelicSolCx.xml) and solKz (viscosity exp(2 y),
testVelicSolKz.xml), with 20 points per element on the Park-Miller layout, PCDVC population control
and DVC weights at resolution 10, binned, weighted, assembled and solved through the C ABI at 16^2,
32^2 and 64^2.  The L2 errors against the analytic solutions (the reference's own analytic plugins,
fixture tests/golden/velic_golden.npz) converge at the rates the reference's expected results state
(velocity 1.99 / 1.99 and 2.00 / 2.00, pressure 1.00, PerformanceTests/expected/
Underworld_Velic_sol{Cx,Kz}-analysis.cvg-convergence-rates.dat), in the FP64 and the mixed forms."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["cx", "kz"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_velic_convergence_rates_match_reference(uw, case, precision):
    from earthbyte_underworld_gb300 import workloads as W
    import velic_norms as VN
    U = uw
    g = VN.golden()
    ns = (16, 32, 64)
    prec = U.PREC_FP64 if precision == "fp64" else U.PREC_MIXED
    errs = []
    for n in ns:
        w = W.solcx(n) if case == "cx" else W.solkz(n)
        with U.Context(0) as ctx:
            W.setup_context(ctx, w)
            ctx.bin_and_map(want=False)
            ctx.weights_set(U.WEIGHTS_DVC, (10, 10))
            ctx.population_control(max_deletions=3, max_splits=3)
            ctx.assemble()
            u, p, rep = ctx.solve_bsscr(U.default_opts(mg_levels=3, schur_type=1, schur_pc=3, scr_rtol=1e-10,
                                                       a11_rtol=1e-11, back_rtol=1e-11, bfbt_rtol=1e-8,
                                                       bfbt_max_it=5000, max_outer=500, max_inner=4000,
                                                       precision=prec))
        assert rep.rel_residual < 1e-8
        errs.append(VN.errors(case, n, u.reshape(-1, 2), p, g))
    errs = np.array(errs)
    r = VN.rates(errs, ns)
    print(f"\nsol{case} {precision}: L2 errors {errs.tolist()}, rates {r.tolist()}")
    assert np.all(np.abs(r - g[f"{case}_expected_rates"]) < 0.1), r
