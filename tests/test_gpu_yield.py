"""Yield rheologies with a strain-weakening history (VonMises with cohesion softening and
strain-rate softening, Byerlee's depth-dependent yield stress, MohrCoulomb with friction and
cohesion softening on the principal stresses), through the GPU assembly against
the oracle: point viscosities, element matrices and the history's time derivative after a previous
solution, then one integration step of the history and a second assembly with the softened
cohesions (YieldRheology.c:198-243, VonMises.c:175-269, Byerlee.c:157-198,
MohrCoulomb.c:208-402, StrainWeakening.c:399-503).  The principal stresses follow the reference's
eigenvalue route (characteristic cubic, Jacobi rotations when an eigenvector formula fails), whose
branch decisions use absolute 1e-8 comparisons; both sides take the same branches here."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm((a - b).reshape(-1)) / max(np.linalg.norm(b.reshape(-1)), 1e-300)


LAWS = [
    [(1, [1.0]), (10, [0.5, 0.1, 1e-3, 0.5, 0.1, 0.0])],    # VonMises, cohesion softening and healing
    [(1, [2.0]), (11, [0.3, 1.0, 1e-3, 0.3, 0.0, 0.0])],    # Byerlee with a history
    [(1, [1.0]), (10, [0.4, 0.4, 1e-2, 0.0, 0.0, 1.0])],    # VonMises with strain-rate softening, no history
    [(1, [1.0]), (12, [0.05, 0.02, 0.6, 0.3, 0.0, 1e-3, 0.4, 0.05])],   # MohrCoulomb, friction and cohesion softening
]


@pytest.mark.parametrize("dim", [3, 2])
def test_yield_laws_with_strain_weakening(oracle, uw, dim):
    O, U = oracle, uw
    nel = (6, 5, 4)[:dim]
    rng = np.random.default_rng(12)
    E = int(np.prod(nel))
    n = E * 12
    e = np.repeat(np.arange(E), 12)
    idx = [e % nel[0], (e // nel[0]) % nel[1]] + ([e // (nel[0] * nel[1])] if dim == 3 else [])
    p = np.stack([(idx[d] + rng.uniform(size=n)) / nel[d] for d in range(dim)], axis=1)
    mat = rng.integers(0, len(LAWS), n).astype(np.int32)
    nodes = [v + 1 for v in nel]
    nn = int(np.prod(nodes))
    k = np.arange(nn)
    xn = (k % nodes[0]) / nel[0]
    yn = ((k // nodes[0]) % nodes[1]) / nel[1]
    comps = [0.2 * np.sin(np.pi * xn) * np.cos(np.pi * yn), -0.2 * np.cos(np.pi * xn) * np.sin(np.pi * yn)]
    if dim == 3:
        zn = (k // (nodes[0] * nodes[1])) / nel[2]
        comps.append(0.1 * np.sin(np.pi * zn) * xn)
    u = np.stack(comps, axis=1)
    pr = rng.uniform(-1.0, 1.0, E)
    pfw0 = rng.uniform(0.0, 0.4, n)
    dt = 0.05
    ctx = U.Context(0)
    ctx.mesh_q1(dim, nel)
    ctx.bc_set(U.free_slip_mask(dim, nel))
    ctx.materials_set([U.make_material(l, density=0.5) for l in LAWS])
    ctx.fields_set(None, 1.0, dim - 1)
    ctx.particles_upload(p[:, 0], p[:, 1], p[:, 2] if dim == 3 else None, mat)
    ctx.strain_weakening_set(pfw0)
    ctx.solution_set(u, pr)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    K1, _, _, _ = ctx.element_matrices()
    eta1 = ctx.point_viscosity()
    pfw_a, inc1 = ctx.strain_weakening()
    ctx.strain_weakening_advance(dt)
    ctx.assemble()
    K2, _, _, _ = ctx.element_matrices()
    eta2 = ctx.point_viscosity()
    pfw_b, inc2 = ctx.strain_weakening()
    ctx.close()

    m = O.make_mesh(dim, nel)
    pts = np.zeros((n, 3))
    pts[:, :dim] = p
    _, off, perm, xi, outside = O.map_points(m, pts)
    mats = [O.make_material(l, density=0.5) for l in LAWS]
    oinc1 = np.zeros(n)
    f = O.make_fields(gravity=1.0, vert_axis=dim - 1, velocity=u, pressure=pr, previous_solution=True, pfw=pfw0,
                      pfw_incr=oinc1)
    oK1, _, _, _, oeta1 = O.assemble(m, off, perm, xi, mat, mats, f, want_eta=True)
    opfw = O.strain_weakening_advance(pfw0, oinc1, dt)
    oinc2 = np.zeros(n)
    f = O.make_fields(gravity=1.0, vert_axis=dim - 1, velocity=u, pressure=pr, previous_solution=True, pfw=opfw,
                      pfw_incr=oinc2)
    oK2, _, _, _, oeta2 = O.assemble(m, off, perm, xi, mat, mats, f, want_eta=True)

    assert np.array_equal(pfw_a, pfw0)
    assert _rel(eta1, oeta1) < 1e-12 and _rel(K1, oK1) < 1e-12
    assert _rel(inc1, oinc1) < 1e-12
    assert _rel(pfw_b, opfw) < 1e-14
    assert _rel(eta2, oeta2) < 1e-12 and _rel(K2, oK2) < 1e-12
    assert _rel(inc2, oinc2) < 1e-12
    smat = mat[perm]
    base = np.array([1.0, 2.0, 1.0, 1.0])[smat]
    yielded = eta1 < base * (1 - 1e-12)
    # every law yields at some points and not at others; the history grows where points yield and
    # heals (VonMises, healing rate 0.1) where they do not
    for law in range(4):
        assert yielded[smat == law].any() and (~yielded[smat == law]).any(), law
    pmat = mat
    assert (inc1[pmat == 0] > 0).any() and (inc1[pmat == 0] < 0).any()
    assert np.all(inc1[pmat == 2] == 0.0)      # no history without a softening strain
    # the softened cohesion lowers the viscosity of yielding VonMises points in the second pass
    assert np.mean(eta2[smat == 0]) != np.mean(eta1[smat == 0])


def test_newton_jacobian_element_matrices_2d(oracle, uw):
    """The 2D Newton branch (ConstitutiveMatrixCartesian.c:360-383): with the Jacobian formed, the
    element matrices carry the yielding laws' viscosity derivatives and equal the oracle's entry by
    entry.  For these laws the derivative term is a
    rank-one update along the stress (VonMises.c:259-268 sets derivs[0,1,3,4] proportional to the
    stress components; Drucker-Prager adds only the pressure derivative derivs[8], which the
    velocity block does not read), so the Newton K_e stays symmetric."""
    O, U = oracle, uw
    laws = [[(1, [1.0]), (10, [0.2, 0.2, 1e-3, 0.0, 0.0, 0.0])],      # VonMises
            [(1, [2.0]), (5, [0.1, 0.6, 0.0, 1e-3])]]                  # Drucker-Prager
    nel = (8, 6)
    rng = np.random.default_rng(3)
    E = nel[0] * nel[1]
    e = np.repeat(np.arange(E), 10)
    p = np.stack([(e % nel[0] + rng.uniform(size=e.size)) / nel[0], (e // nel[0] + rng.uniform(size=e.size)) / nel[1]],
                 axis=1)
    mat = rng.integers(0, 2, e.size).astype(np.int32)
    nn = (nel[0] + 1) * (nel[1] + 1)
    k = np.arange(nn)
    xn, yn = (k % (nel[0] + 1)) / nel[0], (k // (nel[0] + 1)) / nel[1]
    u = np.stack([0.5 * np.sin(np.pi * xn) * np.cos(np.pi * yn), -0.5 * np.cos(np.pi * xn) * np.sin(np.pi * yn)], axis=1)
    pr = rng.uniform(-0.5, 0.5, E)
    out = {}
    for jac in (False, True):
        with U.Context(0) as ctx:
            ctx.mesh_q1(2, nel)
            ctx.bc_set(U.free_slip_mask(2, nel))
            ctx.materials_set([U.make_material(l, density=0.5) for l in laws])
            ctx.fields_set(None, 1.0, 1)
            ctx.particles_upload(p[:, 0], p[:, 1], None, mat)
            ctx.solution_set(u, pr)
            ctx.jacobian_set(jac)
            ctx.bin_and_map(want=False)
            ctx.assemble()
            out[jac] = ctx.element_matrices()
            if jac:
                with pytest.raises(U.UwgpuError):
                    ctx.solve_bsscr(U.default_opts(mg_levels=2))
    m = O.make_mesh(2, nel)
    pts = np.zeros((e.size, 3))
    pts[:, :2] = p
    _, off, perm, xi, _ = O.map_points(m, pts)
    mats = [O.make_material(l, density=0.5) for l in laws]
    f = O.make_fields(gravity=1.0, vert_axis=1, velocity=u, pressure=pr, previous_solution=True, jacobian=True)
    oK, _, _, oS, _ = O.assemble(m, off, perm, xi, mat, mats, f)
    K, _, _, S = out[True]
    assert _rel(K, oK) < 1e-12 and _rel(S, oS) < 1e-12
    asym = np.abs(K - K.transpose(0, 2, 1)).max() / np.abs(K).max()
    assert asym < 1e-12
    # elements with yielding points change by the (negative) derivative term
    Kp = out[False][0]
    dk = np.abs(K - Kp).max(axis=(1, 2)) / np.abs(Kp).max(axis=(1, 2))
    assert dk.max() > 1e-3
