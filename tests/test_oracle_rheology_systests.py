"""The oracle's yield and power-law rheologies against the reference's rheology system tests.

Underworld/Rheology/tests/input/testYieldCriterion.xml compresses a 3 x 1 box of material points
(30 x 10 Q1 elements, a 2 x 2 Gauss layout of points per element, background MaterialViscosity
eta0 = 3.4) between side walls moving inward at 0.5, the top wall rising as
IncompressibleExtensionBC sets it (Underworld/plugins/IncompressibleExtensionBC/
IncompressibleExtensionBC.c:115-166: V_top = -(h (V_right - V_left)) / width with the reference
height at y = 0, V_bottom = 0), and a test codelet records every material point whose yield
indicator exceeds its criterion from the second non-linear iteration on, printing the time, the
step and the extent of those points (Underworld/Rheology/tests/VonMisesYieldingSuite.c).

- Byerlee (testByerleeYieldCriterion: cohesion 2, depthCoefficient 0.5333) yields at step 0 in
  the top half of the box.  Step 0 runs on the undeformed mesh, so the oracle reproduces it: the
  Picard loop of SystemLinearEquations.c:820-935 (tolerance 0.01 on the velocity change) on that
  mesh gives the same extent, printed the same way.
- VonMises (testVonMisesYieldCriterion: cohesion 3.0222222) first yields at step 12 of the
  deforming-mesh run; its input notes that the whole box yields at t = 0.75, where the box is
  2.25 wide.  The oracle does not deform meshes, so it is checked on that statement: nothing
  yields at step 0, every point yields in a box 2.2 wide (after t = 0.75), none in one 2.3 wide.

- NonNewtonian (testNonNewtonianShear.xml, run with stressExponent 3 and 4): simple shear of a
  unit box, 20 x 20 elements, eta0 = 100, the top wall moving at 0.5; the reference finds the
  velocity, strain rate, stress and viscosity within 1e-6, 1e-5, 1e-5 and 1e-4 of
  NonNewtonianShearSolution.c (v_x = y v / H, shear strain rate v / 2H, stress
  (eta0 v / H)^(1/n), viscosity eta0 (eta0 v / H)^(1/n - 1)) once the Picard loop has converged.
  The reference's side walls are periodic, which the oracle does not model; here they carry the
  same linear profile as Dirichlet values, which leaves the analytic solution unchanged, and the
  material points sit at the 2 x 2 Gauss points (exact for the linear field, as the reference's
  moment-balance weights are).

The fixture is tests/golden/rheology_systest_golden.json (made by
tests/golden/make_rheology_systest_golden.py).
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rheology_systest_golden.json")


@pytest.fixture(scope="module")
def golden():
    return json.load(open(GOLDEN))


def _gauss_points(nel, mn, mx):
    """GaussParticleLayout with two points per axis: the 2 x 2 Gauss points of every element."""
    g = np.array([-1.0, 1.0]) / np.sqrt(3.0)
    hx, hy = (mx[0] - mn[0]) / nel[0], (mx[1] - mn[1]) / nel[1]
    pts = []
    for j in range(nel[1]):
        for i in range(nel[0]):
            for b in g:
                for a in g:
                    pts.append((mn[0] + (i + 0.5 * (1 + a)) * hx, mn[1] + (j + 0.5 * (1 + b)) * hy, 0.0))
    return np.array(pts)


def _step0(O, model, law_id, cohesion, depth_coef, width=None):
    """One time step's Picard loop on the undeformed box (or on a box `width` wide with the same
    area): returns the coordinates of every point that yielded in an iteration after the first,
    and the final viscosities with the yielded mask of the last iteration."""
    nel = model["elementRes"]
    mn, mx = list(model["min"]), list(model["max"])
    if width is not None:
        area = (mx[0] - mn[0]) * (mx[1] - mn[1])
        mx = [mn[0] + width, mn[1] + area / width]
    m = O.make_mesh(2, nel, mn=(mn[0], mn[1], 0.0), mx=(mx[0], mx[1], 0.0))
    xyz = _gauss_points(nel, mn, mx)
    _, off, perm, xi, outside = O.map_points(m, xyz)
    assert outside == 0
    eta0 = model["eta0"]
    mats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [eta0]),
                             (law_id, [cohesion, depth_coef, 0.0, 0.0, 0.0, 0.0])])]
    material = np.zeros(xyz.shape[0], np.int32)
    # walls: vx on the sides, vy on top and bottom (IncompressibleExtensionBC, reference height 0)
    fixed = O.free_slip_mask(m)
    xn = O.node_coords(m)
    width_now, height = mx[0] - mn[0], mx[1] - mn[1]
    vl, vr = model["leftWallVelocity"], model["rightWallVelocity"]
    bc = np.zeros((xn.shape[0], 2))
    bc[np.isclose(xn[:, 0], mn[0]), 0] = vl
    bc[np.isclose(xn[:, 0], mx[0]), 0] = vr
    bc[np.isclose(xn[:, 1], mx[1]), 1] = -(mx[1] - 0.0) * (vr - vl) / width_now
    bc[np.isclose(xn[:, 1], mn[1]), 1] = (0.0 - mn[1]) * (vr - vl) / width_now
    free = fixed.reshape(-1) == 0
    u = p = None
    yielded_pts = np.zeros(xyz.shape[0], bool)
    last = None
    for it in range(50):
        f = O.make_fields(velocity=u, pressure=p, previous_solution=u is not None)
        Ke, fe, Ge, Se, eta = O.assemble(m, off, perm, xi, material, mats, f, want_eta=True)
        ys = eta < eta0 * (1.0 - 1e-12)          # slots whose viscosity the yield law corrected
        if it >= 1:                              # recorded from the second non-linear iteration
            yielded_pts[perm[ys]] = True
        last = (eta, ys)
        un, pn, rep = O.solve_bsscr(m, fixed, Ke, Ge, fe, Se, mg_levels=2, schur_type=1, schur_pc=0,
                                    scr_rtol=1e-10, a11_rtol=1e-12, back_rtol=1e-12, bcval=bc)
        un = un.reshape(-1)
        if u is not None:
            du = np.linalg.norm((un - u)[free]) / np.linalg.norm(un[free])
            u, p = un, pn
            if du < 0.01:
                break
        else:
            u, p = un, pn
    return xyz[yielded_pts], last, height, width_now


def _g(v):
    return "%12.4g" % v


def test_byerlee_yields_in_the_top_half_at_step_0(oracle, golden):
    law = golden["laws"]["Byerlee"]
    exp = law["expected"]
    assert exp["step"] == 0 and float(exp["time"]) == 0.0
    pts, (eta, ys), height, width = _step0(oracle, golden["model"], oracle.LAW_BYERLEE, law["cohesion"],
                                           law["depthCoefficient"])
    assert pts.shape[0] > 0
    got = {"x": [_g(pts[:, 0].min()).strip(), _g(pts[:, 0].max()).strip()],
           "y": [_g(pts[:, 1].min()).strip(), _g(pts[:, 1].max()).strip()]}
    assert got == {"x": exp["x"], "y": exp["y"]}, got
    # uniform pure shear: strain-rate invariant 1 / width, indicator 2 eta0 / width; the yielded
    # viscosity is the criterion over twice the strain-rate invariant
    m = golden["model"]
    ind = 2.0 * m["eta0"] / width
    assert abs(ind - 2.0 * 3.4 / 3.0) < 1e-12
    crit_top = law["cohesion"] + law["depthCoefficient"] * (height - 0.9789)
    assert crit_top < ind


def test_von_mises_yields_where_its_input_says(oracle, golden):
    law = golden["laws"]["VonMises"]
    m = golden["model"]
    assert law["expected"]["step"] > 0   # nothing printed at step 0
    pts, (eta, ys), _, _ = _step0(oracle, m, oracle.LAW_VON_MISES, law["cohesion"], 0.0)
    assert pts.shape[0] == 0 and not ys.any()
    # the box at t = 0.75 is 3 - 0.75 = 2.25 wide: 2 eta0 / 2.25 = cohesion
    assert abs(2.0 * m["eta0"] / 2.25 - law["cohesion"]) < 1e-6
    pts, (eta, ys), _, w = _step0(oracle, m, oracle.LAW_VON_MISES, law["cohesion"], 0.0, width=2.2)
    assert ys.all() and pts.shape[0] == ys.shape[0]
    # every point at the yielded viscosity cohesion / (2 / width)
    np.testing.assert_allclose(eta, law["cohesion"] * w / 2.0, rtol=1e-8)
    pts, (eta, ys), _, _ = _step0(oracle, m, oracle.LAW_VON_MISES, law["cohesion"], 0.0, width=2.3)
    assert pts.shape[0] == 0 and not ys.any()


@pytest.mark.parametrize("run", ["N3", "N4"])
def test_non_newtonian_shear_matches_the_analytic_solution(oracle, golden, run):
    O = oracle
    sh = golden["nonNewtonianShear"]
    n = sh["runs"][run]["stressExponent"]
    assert all(sh["runs"][run]["within"][f] for f in sh["tolerance"])   # the reference passed them
    nel, mn, mx = sh["elementRes"], sh["min"], sh["max"]
    H = mx[1] - mn[1]
    eta0 = sh["eta0"]
    m = O.make_mesh(2, nel, mn=(mn[0], mn[1], 0.0), mx=(mx[0], mx[1], 0.0))
    xyz = _gauss_points(nel, mn, mx)
    _, off, perm, xi, outside = O.map_points(m, xyz)
    assert outside == 0
    mats = [O.make_material([(O.LAW_MATERIAL_VISCOSITY, [eta0]), (9, [n, 0.0])])]   # 9: NonNewtonian
    material = np.zeros(xyz.shape[0], np.int32)
    xn = O.node_coords(m)
    on_wall = (np.isclose(xn[:, 0], mn[0]) | np.isclose(xn[:, 0], mx[0]) |
               np.isclose(xn[:, 1], mn[1]) | np.isclose(xn[:, 1], mx[1]))
    fixed = np.repeat(on_wall, 2).astype(np.uint8)
    for v in (sh["velocityTopOfBox"], 2.0 * sh["velocityTopOfBox"]):
        bc = np.zeros((xn.shape[0], 2))
        bc[:, 0] = (xn[:, 1] - mn[1]) / H * v
        u = p = None
        for it in range(50):
            f = O.make_fields(velocity=u, pressure=p, previous_solution=u is not None)
            Ke, fe, Ge, Se, eta = O.assemble(m, off, perm, xi, material, mats, f, want_eta=True)
            un, pn, rep = O.solve_bsscr(m, fixed, Ke, Ge, fe, Se, mg_levels=3, schur_type=1, schur_pc=0,
                                        scr_rtol=1e-12, a11_rtol=1e-13, back_rtol=1e-13, bcval=bc)
            un = un.reshape(-1)
            done = u is not None and np.linalg.norm(un - u) / np.linalg.norm(un) < sh["nonLinearTolerance"]
            u, p = un, pn
            if done:
                break
        # the first solve (eta0 everywhere) already gives the linear field, so the second repeats it
        assert done and it >= 1
        # the viscosity the last assembly evaluated, from the converged velocity
        f = O.make_fields(velocity=u, pressure=p, previous_solution=True)
        _, _, _, _, eta = O.assemble(m, off, perm, xi, material, mats, f, want_eta=True)
        eta_a = eta0 * (eta0 * v / H) ** (1.0 / n - 1.0)
        tau_a = (eta0 * v / H) ** (1.0 / n)
        ua = u.reshape(-1, 2)
        assert np.abs(ua[:, 0] - (xn[:, 1] - mn[1]) / H * v).max() < sh["tolerance"]["VelocityField"] * 1e-3
        assert np.abs(ua[:, 1]).max() < sh["tolerance"]["VelocityField"] * 1e-3
        assert np.abs(eta - eta_a).max() < sh["tolerance"]["ViscosityField"] * 1e-3 * eta_a
        # stress = 2 eta * shear strain rate, with the strain rate of the discrete solution
        assert abs(2.0 * eta.mean() * (v / (2.0 * H)) - tau_a) < sh["tolerance"]["StressField"] * 1e-3 * tau_a
