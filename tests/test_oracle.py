"""CPU checks of the oracle's restated rules (binning, layout stream, local coordinates, solve)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def test_park_miller_stream_matches_c(oracle):
    from earthbyte_underworld_gb300 import workloads as W
    O = oracle
    m = O.make_mesh(2, (4, 3, 1))
    xyz = O.random_layout(m, 5, 13)
    w = W.rt2d(nel=(4, 3), ppc=5, seed=13)
    assert np.array_equal(xyz[:, 0], w["x"]) and np.array_equal(xyz[:, 1], w["y"])


def test_search_element_tie_rules(oracle):
    """Mesh_RegularAlgorithms.c:194-226: a point on an interior face goes to the lower element
    (Num_Approx of the fractional part, eps 1e-12); a point at max goes to the last element."""
    O = oracle
    m = O.make_mesh(2, (4, 4, 1))
    pts = np.array([[0.25, 0.1, 0], [0.25 + 1e-13, 0.1, 0], [0.25 + 1e-9, 0.1, 0], [1.0, 1.0, 0],
                    [0.0, 0.0, 0], [1.0 + 5e-13, 0.5, 0], [1.0 + 1e-6, 0.5, 0], [-1e-9, 0.5, 0]])
    owning, offsets, perm, xi, outside = O.map_points(m, pts)
    assert owning[0] == 0                 # x on face 1 -> element 0
    assert owning[1] == 0                 # within eps of the face -> lower
    assert owning[2] == 1                 # beyond eps -> upper
    assert owning[3] == 15                # max corner -> last element
    assert owning[4] == 0
    assert owning[5] == 3 + 4 * 1         # x within eps of max -> last column; y on a face -> lower row
    assert owning[6] == 0xFFFFFFFF and owning[7] == 0xFFFFFFFF
    assert outside == 2


def test_map_is_stable_by_point_index(oracle):
    O = oracle
    m = O.make_mesh(3, (3, 2, 2))
    rng = np.random.default_rng(0)
    xyz = rng.uniform(0, 1, size=(500, 3))
    owning, offsets, perm, xi, outside = O.map_points(m, xyz)
    order = np.lexsort((np.arange(500), owning))
    assert np.array_equal(perm, order.astype(np.uint32))
    assert np.array_equal(np.diff(offsets.astype(np.int64)), np.bincount(owning, minlength=12))


def _drand48(n, seed=0):
    """POSIX srand48(seed) / drand48(): the 48-bit linear congruence X' = (0x5DEECE66D X + 0xB)
    mod 2^48 from X = (seed << 16) + 0x330E, returning X' / 2^48."""
    x = ((seed & 0xFFFFFFFF) << 16) | 0x330E
    out = []
    for _ in range(n):
        x = (0x5DEECE66D * x + 0xB) % (1 << 48)
        out.append(x / float(1 << 48))
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_element_type_suite_points_map_back(oracle, dim):
    """StgFEM/Discretisation/tests/ElementTypeSuite.c (TestLinear2D / TestLinear3D): 40 points
    drawn by srand48(0) / drand48() in a 6 x 6 (x 1) Q1 mesh over [0, 1.2]^dim are searched,
    converted to local coordinates and mapped back through the shape functions; the suite requires
    the round trip within 1e-8.  Here the oracle's element search and local coordinates (its
    Newton iteration and the closed form) must reproduce the points to that tolerance."""
    import ctypes
    try:
        libc = ctypes.CDLL("libc.so.6")
        libc.drand48.restype = ctypes.c_double
        libc.srand48(0)
        assert [libc.drand48() for _ in range(8)] == _drand48(8)   # the restated stream is libc's
    except OSError:
        pass
    O = oracle
    nel = (6, 6, 1)
    h = [1.2 / n for n in nel]
    m = O.make_mesh(dim, nel, mn=(0.0, 0.0, 0.0), mx=(1.2, 1.2, 1.2))
    r = _drand48(40 * dim)
    pts = np.zeros((40, 3))
    pts[:, :dim] = np.array(r).reshape(40, dim)
    for newton in (True, False):
        owning, offsets, perm, xi, outside = O.map_points(m, pts, use_newton=newton)
        assert outside == 0
        xi_pt = np.zeros_like(xi)
        xi_pt[perm] = xi                     # xi is in slot order
        e = owning.astype(np.int64)
        idx = [e % nel[0], (e // nel[0]) % nel[1], e // (nel[0] * nel[1])]
        back = np.zeros((40, dim))
        for d in range(dim):
            # Q1 shape functions on the rectangular element: sum_a N_a(xi) x_a
            lo = idx[d] * h[d]
            back[:, d] = lo * (1.0 - xi_pt[:, d]) / 2.0 + (lo + h[d]) * (1.0 + xi_pt[:, d]) / 2.0
        assert np.all(np.abs(xi_pt[:, :dim]) <= 1.0 + 1e-12)
        assert np.linalg.norm(back - pts[:, :dim], axis=1).max() < 1e-8


def test_newton_xi_equals_affine_closed_form(oracle):
    O = oracle
    m = O.make_mesh(3, (5, 3, 7))
    rng = np.random.default_rng(1)
    xyz = rng.uniform(0, 1, size=(2000, 3))
    _, off1, perm1, xi1, _ = O.map_points(m, xyz, use_newton=True)
    _, off2, perm2, xi2, _ = O.map_points(m, xyz, use_newton=False)
    assert np.array_equal(perm1, perm2)
    assert np.max(np.abs(xi1 - xi2)) < 1e-13
    assert np.all(np.abs(xi1) <= 1.0 + 1e-12)


def _small_problem(O, dim, nel, ppc=8, seed=0):
    m = O.make_mesh(dim, nel)
    rng = np.random.default_rng(seed)
    E = O.num_elements(m)
    xyz = O.random_layout(m, ppc, 17)
    mat = (xyz[:, 1] > 0.5).astype(np.int32)
    mats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [1.0])], density=0.0),
            O.make_material([(O.LAW_MATERIAL_VISCOSITY, [100.0])], density=1.0)]
    _, off, perm, xi, _ = O.map_points(m, xyz)
    f = O.make_fields(gravity=1.0, vert_axis=dim - 1)
    Ke, fe, Ge, Se, _ = O.assemble(m, off, perm, xi, mat, mats, f)
    return m, Ke, fe, Ge, Se


@pytest.mark.parametrize("dim,nel", [(2, (8, 8, 1)), (3, (4, 4, 4))])
def test_oracle_bsscr_matches_direct_solve(oracle, dim, nel):
    O = oracle
    m, Ke, fe, Ge, Se = _small_problem(O, dim, nel)
    fixed = O.free_slip_mask(m)
    u, p, rep = O.solve_bsscr(m, fixed, Ke, Ge, fe, Se, mg_levels=3 if dim == 2 else 2)
    # direct saddle-point solve with scipy
    rp, ci, v, eq, nf = O.global_csr(m, Ke, fixed)
    K = sp.csr_matrix((v, ci, rp), shape=(nf, nf))
    E = O.num_elements(m)
    nen = 1 << dim
    rows, cols, vals = [], [], []
    f = np.zeros(nf)
    for e in range(E):
        inc = np.zeros(8, np.int64)
        O.lib().uwr_element_nodes(__import__("ctypes").byref(m), e, inc.ctypes.data)
        for a in range(nen):
            for d in range(dim):
                q = eq[inc[a] * dim + d]
                if q >= 0:
                    rows.append(q); cols.append(e); vals.append(Ge[e, a * dim + d])
                    f[q] += fe[e, a * dim + d]
    G = sp.csr_matrix((vals, (rows, cols)), shape=(nf, E))
    A = sp.bmat([[K, G], [G.T, None]]).tocsc()
    # pin the constant pressure mode by adding a row/column (Lagrange multiplier)
    ones = sp.csr_matrix(np.concatenate([np.zeros(nf), np.ones(E)])[None, :])
    Aa = sp.bmat([[A, ones.T], [ones, None]]).tocsc()
    sol = spla.spsolve(Aa, np.concatenate([f, np.zeros(E), [0.0]]))
    ud, pd = sol[:nf], sol[nf:nf + E]
    uo = u.reshape(-1)[eq >= 0]
    assert rep.rel_residual < 1e-9
    assert np.linalg.norm(uo - ud) / np.linalg.norm(ud) < 1e-8
    assert np.linalg.norm(p - pd) / np.linalg.norm(pd) < 1e-8


def _full_saddle(O, m, Ke, Ge, fe):
    """K over every velocity dof, G (dofs x elements) and f assembled directly from the element
    matrices (independent of the oracle's own assembly and lift)."""
    import ctypes
    dim = m.dim
    nen = 1 << dim
    nd = nen * dim
    nn, E = O.num_nodes(m), O.num_elements(m)
    rows, cols, vals, grows, gcols, gvals = [], [], [], [], [], []
    f = np.zeros(nn * dim)
    for e in range(E):
        inc = np.zeros(8, np.int64)
        O.lib().uwr_element_nodes(ctypes.byref(m), e, inc.ctypes.data)
        dofs = (inc[:nen, None] * dim + np.arange(dim)[None, :]).reshape(-1)
        rows.append(np.repeat(dofs, nd)); cols.append(np.tile(dofs, nd)); vals.append(Ke[e].reshape(-1))
        grows.append(dofs); gcols.append(np.full(nd, e)); gvals.append(Ge[e])
        np.add.at(f, dofs, fe[e])
    K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nn * dim, nn * dim))
    G = sp.csr_matrix((np.concatenate(gvals), (np.concatenate(grows), np.concatenate(gcols))), shape=(nn * dim, E))
    return K, G, f


@pytest.mark.parametrize("dim,nel,kind", [(2, (8, 8, 1), "lid"), (2, (8, 6, 1), "extension"),
                                          (3, (4, 4, 4), "lid"), (3, (4, 6, 4), "extension")])
def test_oracle_bc_lift_matches_direct_solve(oracle, dim, nel, kind):
    """Non-zero Dirichlet values (StiffnessMatrix.c:900-925 lift): the oracle's BSSCR solution
    equals a direct solve of K_ff u_f + G_f p = f_f - K_fc u_c, G_f^T u_f = -G_c^T u_c, and its
    velocity carries the fixed values."""
    from earthbyte_underworld_gb300 import workloads as W
    O = oracle
    m, Ke, fe, Ge, Se = _small_problem(O, dim, nel)
    fixed, bcval = W.driven_walls(dim, nel[:dim], kind)
    u, p, rep = O.solve_bsscr(m, fixed, Ke, Ge, fe, Se, mg_levels=2, scr_rtol=1e-12, a11_rtol=1e-13,
                              back_rtol=1e-13, bcval=bcval)
    K, G, f = _full_saddle(O, m, Ke, Ge, fe)
    free = fixed == 0
    uc = np.where(free, 0.0, bcval)
    Kff = K[free][:, free]
    Gf = G[free]
    E = O.num_elements(m)
    rhs = np.concatenate([f[free] - K[free] @ uc, -(G.T @ uc)])
    A = sp.bmat([[Kff, Gf], [Gf.T, None]]).tocsc()
    closed = kind == "lid"
    if closed:   # constant pressure in the null space: pin its mean
        ones = sp.csr_matrix(np.concatenate([np.zeros(Kff.shape[0]), np.ones(E)])[None, :])
        A = sp.bmat([[A, ones.T], [ones, None]]).tocsc()
        rhs = np.concatenate([rhs, [0.0]])
    sol = spla.spsolve(A, rhs)
    ud = uc.copy()
    ud[free] = sol[:Kff.shape[0]]
    pd = sol[Kff.shape[0]:Kff.shape[0] + E]
    if closed:
        p = p - p.mean()
    assert rep.rel_residual < 1e-9
    assert np.array_equal(u.reshape(-1)[~free], bcval[~free])
    assert np.linalg.norm(u.reshape(-1) - ud) / np.linalg.norm(ud) < 1e-8
    assert np.linalg.norm(p - pd) / np.linalg.norm(pd) < 1e-8


def test_oracle_newton_form_without_yield_equals_picard(oracle):
    """With no yielding law the viscosity derivatives vanish and the 2D Newton element matrices
    (ConstitutiveMatrixCartesian.c:360-383) equal the Picard ones."""
    O = oracle
    m = O.make_mesh(2, (6, 5, 1))
    xyz = O.random_layout(m, 8, 5)
    _, off, perm, xi, _ = O.map_points(m, xyz)
    mats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [1.3])], density=1.0)]
    nn = O.num_nodes(m)
    u = np.random.default_rng(2).standard_normal((nn, 2))
    f0 = O.make_fields(velocity=u, previous_solution=True, gravity=1.0)
    f1 = O.make_fields(velocity=u, previous_solution=True, gravity=1.0, jacobian=True)
    K0, *_ = O.assemble(m, off, perm, xi, None, mats, f0)
    K1, *_ = O.assemble(m, off, perm, xi, None, mats, f1)
    assert np.abs(K1 - K0).max() < 1e-13 * np.abs(K0).max()


def test_oracle_refuses_meshes_that_do_not_coarsen(oracle):
    """The oracle's multigrid halves every axis per level: an odd element count on a level that
    is still coarsened is refused with an error instead of a broken hierarchy."""
    O = oracle
    m = O.make_mesh(2, (6, 5))
    nn, E = 7 * 6, 30
    fixed = np.zeros(nn * 2, np.uint8)
    Ke = np.tile(np.eye(8), (E, 1, 1))
    with pytest.raises(ValueError):
        O.solve_bsscr(m, fixed, Ke, np.zeros((E, 8)), np.zeros((E, 8)), np.ones(E), mg_levels=2)


@pytest.mark.parametrize("case", ["cx", "kz"])
def test_oracle_velic_convergence_rates_match_reference(oracle, case):
    """The oracle's particle-in-cell Stokes solve of the reference's analytic-solution tests
    (Underworld/SysTest/PerformanceTests/testVelicSolCx.xml: viscosity jump 100 : 1 at x = 0.5;
    testVelicSolKz.xml: viscosity exp(2 y)), with 20 points per element on the Park-Miller layout,
    PCDVC population control and DVC weights at resolution 10, at 16^2, 32^2, 64^2: the L2 errors
    against the analytic solutions (the reference's own analytic plugins, fixture
    tests/golden/velic_golden.npz) converge at the rates the reference's expected results state
    (PerformanceTests/expected/Underworld_Velic_sol{Cx,Kz}-analysis.cvg-convergence-rates.dat:
    velocity 1.99 / 1.99 and 2.00 / 2.00, pressure 1.00)."""
    from earthbyte_underworld_gb300 import workloads as W
    import velic_norms as VN
    O = oracle
    g = VN.golden()
    ns = (16, 32, 64)
    errs = []
    for n in ns:
        w = W.solcx(n) if case == "cx" else W.solkz(n)
        m = O.make_mesh(2, w["nel"])
        pts = np.stack([w["x"], w["y"], np.zeros_like(w["x"])], axis=1)
        _, off, perm, xi, _ = O.map_points(m, pts)
        X, M, S, off2, perm2, xo, wo = O.pcdvc(m, (10, 10), pts, w["material"], off, perm, xi, max_deletions=3,
                                             max_splits=3)
        mats = [O.make_material([(mm.laws[i].law, list(mm.laws[i].p)) for i in range(mm.n_laws)],
                                density=mm.density, alpha=mm.alpha, ref_temp=mm.ref_temp) for mm in w["materials"]]
        f = O.make_fields(temperature=w["temperature"], gravity=1.0, vert_axis=1)
        Ke, fe, Ge, Se, _ = O.assemble(m, off2, perm2, xo, M, mats, f, weights=wo)
        u, p, rep = O.solve_bsscr(m, w["fixed"], Ke, Ge, fe, Se, mg_levels=3, schur_type=1, schur_pc=3,
                                  scr_rtol=1e-10, a11_rtol=1e-12, back_rtol=1e-12, bfbt_rtol=1e-8, bfbt_max_it=5000)
        errs.append(VN.errors(case, n, u, p, g))
    errs = np.array(errs)
    r = VN.rates(errs, ns)
    print(f"\nsol{case}: L2 errors", errs.tolist(), "rates", r.tolist())
    assert np.all(np.abs(r - g[f"{case}_expected_rates"]) < 0.1), r


def _velic_fem_case(O, case, n):
    """solA / solB / solS of the reference's performance tests (testVelicSol{A,B,S}.xml): the FEM
    base application (ThermalConvectionBase.xml: 2 x 2 Gauss swarm, ThermalBuoyancyForceTerm with
    Ra = 1, StgFEM/Assembly/src/ThermalBuoyancyForceTerm.c:179-240, f_y = Ra T), isoviscous.
    The Gauss points are placed as points with constant weights (the same integral); the
    buoyancy Ra T is written as rho = -T (density 1e-12, expansivity 1e12 about T = 0)."""
    m = O.make_mesh(2, (n, n, 1))
    a = 1.0 / np.sqrt(3.0)
    e = np.arange(n * n)
    ex, ey = e % n, e // n
    pts = []
    for gy in (-a, a):
        for gx in (-a, a):
            pts.append(np.stack([(ex + 0.5 + 0.5 * gx) / n, (ey + 0.5 + 0.5 * gy) / n, np.zeros(n * n)], axis=1))
    pts = np.concatenate(pts)
    xn = O.node_coords(m)
    bc = None
    if case == "s":
        # velocityBC.topLidSinusoidal_NoSlipBottom.xml: top v_x = sin(pi x) (Velocity_SinusoidalLid,
        # StandardConditionFunctions.c:1076-1095), v_y = 0; bottom no-slip; sides v_x = 0
        mats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [1.0])], density=0.0)]
        T = None
        top, bot = np.isclose(xn[:, 1], 1.0), np.isclose(xn[:, 1], 0.0)
        side = np.isclose(xn[:, 0], 0.0) | np.isclose(xn[:, 0], 1.0)
        fixed = np.zeros((xn.shape[0], 2), np.uint8)
        fixed[top | bot, :] = 1
        fixed[side, 0] = 1
        bc = np.zeros((xn.shape[0], 2))
        bc[top, 0] = np.sin(np.pi * xn[top, 0])
        bc[side, 0] = 0.0
        fixed = fixed.reshape(-1)
    else:
        mats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [1.0])], density=1e-12, alpha=1e12, ref_temp=0.0)]
        if case == "a":   # VelicTemperatureIC (StandardConditionFunctions.c:1298-1338), wavenumberY 3.5
            T = np.sin(3.5 * np.pi * xn[:, 1]) * np.cos(np.pi * xn[:, 0])
        else:             # VelicTemperatureIC_SolB (StandardConditionFunctions.c:1341-1375), km = 2
            T = np.sinh(2.0 * xn[:, 1]) * np.cos(np.pi * xn[:, 0])
        fixed = O.free_slip_mask(m)
    _, off, perm, xi, outside = O.map_points(m, pts)
    assert outside == 0
    f = O.make_fields(temperature=T, gravity=1.0, vert_axis=1)
    Ke, fe, Ge, Se, _ = O.assemble(m, off, perm, xi, np.zeros(pts.shape[0], np.int32), mats, f)
    u, p, rep = O.solve_bsscr(m, fixed, Ke, Ge, fe, Se, mg_levels=3, schur_type=1, schur_pc=3, scr_rtol=1e-10,
                              a11_rtol=1e-12, back_rtol=1e-12, bfbt_rtol=1e-8, bfbt_max_it=5000, bcval=bc)
    return u, p


@pytest.mark.parametrize("case", ["a", "b", "s"])
def test_oracle_velic_fem_convergence_rates_match_reference(oracle, case):
    """solA (buoyancy from a non-integer vertical wavenumber), solB (a sinh temperature) and solS
    (a driven sinusoidal lid: non-zero Dirichlet values lifted into the right-hand side), on the
    reference's Gauss-swarm FEM setup at 16^2, 32^2, 64^2: the L2 errors against the reference's
    analytic plugins (Underworld/SysTest/AnalyticPlugins/Velic_sol{A,B,S}/sol{A,B,S}.c, fixture
    tests/golden/velic_golden.npz) converge at the rates the reference's expected results state
    (PerformanceTests/expected/Underworld_Velic_sol{A,B,S}-analysis.cvg-convergence-rates.dat)."""
    import velic_norms as VN
    O = oracle
    g = VN.golden()
    ns = (16, 32, 64)
    errs = np.array([VN.errors(case, n, *_velic_fem_case(O, case, n), g) for n in ns])
    r = VN.rates(errs, ns)
    print(f"\nsol{case}: L2 errors", errs.tolist(), "rates", r.tolist())
    assert np.all(np.abs(r - g[f"{case}_expected_rates"]) < 0.1), r


@pytest.mark.parametrize("order,radius_tol,theta_tol", [(1, 0.005, 1.0e-5), (2, 1.0e-7, 1.0e-5)])
def test_advection_suite_solid_body_rotation(oracle, order, radius_tol, theta_tol):
    """PICellerator/MaterialPoints/tests/AdvectionSuite.c (TestEuler / TestRK2 with
    input/testAdvection.xml, testEuler.xml, testRK2.xml): points inside the unit circle on a 20 x 20
    Q1 mesh over [-1.1, 1.1]^2, nodal velocity Velocity_SolidBodyRotation (StgFEM/plugins/
    StandardConditionFunctions/StandardConditionFunctions.c:665-693: (-y, x), omega 1), dt 0.01,
    ten steps; at every step the radius, the angle to the analytic rotation and the out-of-plane
    drift stay below the suite's tolerances (radius 0.005 / 1e-7, angle 1e-5, depth 1e-10)."""
    O = oracle
    m = O.make_mesh(2, (20, 20, 1), mn=(-1.1, -1.1, 0.0), mx=(1.1, 1.1, 0.0))
    xn = O.node_coords(m)
    u = np.stack([-xn[:, 1], xn[:, 0]], axis=1)
    rng = np.random.default_rng(0)
    r = np.sqrt(rng.random(4000))
    th = 2.0 * np.pi * rng.random(4000)
    x0 = np.stack([r * np.cos(th), r * np.sin(th), np.zeros_like(r)], axis=1)
    xyz = x0.copy()
    r0 = np.linalg.norm(x0[:, :2], axis=1)
    th0 = np.arctan2(x0[:, 1], x0[:, 0])
    dt, t = 0.01, 0.0
    for step in range(10):
        xyz, failed, _ = O.advect(m, u, xyz, dt, order=order)
        assert failed == 0
        t += dt
        ra = np.linalg.norm(xyz[:, :2], axis=1)
        ana = np.stack([r0 * np.cos(t + th0), r0 * np.sin(t + th0)], axis=1)
        cosang = np.sum(ana * xyz[:, :2], axis=1) / (np.linalg.norm(ana, axis=1) * ra)
        theta = np.arccos(np.clip(cosang, -1.0, 1.0))
        assert np.abs(ra - r0).max() < radius_tol
        assert theta.max() < theta_tol
        assert np.abs(xyz[:, 2] - x0[:, 2]).max() < 1e-10
