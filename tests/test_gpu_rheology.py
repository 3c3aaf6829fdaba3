"""Point-wise rheologies beyond the benchmark's (LinearViscosity, DepthDependentViscosity,
NonNewtonian), alone and chained with the others, through the GPU assembly against the oracle:
before the first solve (NonNewtonian takes defaultStrainRateInvariant) and with a previous
velocity solution (the point's strain-rate invariant)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm((a - b).reshape(-1)) / max(np.linalg.norm(b.reshape(-1)), 1e-300)


LAWS = [
    [(7, [1.0, 0.5, -0.3, 0.2, 0.1, 0.05, -0.07, 0.3])],                 # LinearViscosity
    [(8, [2.0, 1.5, 0.3, 2.0])],                                          # DepthDependent along z
    [(1, [5.0]), (9, [3.0, 0.7])],                                        # MaterialViscosity + NonNewtonian
    [(8, [1.0, -2.0, 0.0, 0.0]), (9, [2.5, 0.0]), (4, [10.0, 0.1])],      # chained, limiter last
]


@pytest.mark.parametrize("previous", [False, True])
def test_new_rheologies_assembly_parity(oracle, uw, previous):
    O, U = oracle, uw
    nel = (6, 5, 4)
    rng = np.random.default_rng(8)
    E = int(np.prod(nel))
    pts = []
    for e in range(E):
        i, j, k = e % nel[0], (e // nel[0]) % nel[1], e // (nel[0] * nel[1])
        for _ in range(12):
            pts.append([(i + rng.uniform()) / nel[0], (j + rng.uniform()) / nel[1], (k + rng.uniform()) / nel[2]])
    p = np.array(pts)
    mat = rng.integers(0, len(LAWS), len(p)).astype(np.int32)
    nn = int(np.prod([n + 1 for n in nel]))
    # a smooth previous velocity and pressure
    idx = np.arange(nn)
    xn = (idx % 7) / 6.0
    yn = ((idx // 7) % 6) / 5.0
    zn = (idx // 42) / 4.0
    u = np.stack([np.sin(np.pi * xn) * np.cos(np.pi * yn), -np.cos(np.pi * xn) * np.sin(np.pi * yn),
                  0.3 * np.sin(np.pi * zn) * xn], axis=1)
    pr = rng.uniform(-1.0, 1.0, E)
    ctx = U.Context(0)
    ctx.mesh_q1(3, nel)
    ctx.bc_set(U.free_slip_mask(3, nel))
    ctx.materials_set([U.make_material(l, density=0.5) for l in LAWS])
    ctx.fields_set(None, 1.0, 2)
    ctx.particles_upload(p[:, 0], p[:, 1], p[:, 2], mat)
    if previous:
        ctx.solution_set(u, pr)
    ctx.bin_and_map(want=False)
    ctx.assemble()
    Ke, fe, Ge, Se = ctx.element_matrices()
    eta = ctx.point_viscosity()
    ctx.close()
    m = O.make_mesh(3, nel)
    _, off, perm, xi, outside = O.map_points(m, p)
    mats = [O.make_material(l, density=0.5) for l in LAWS]
    f = O.make_fields(gravity=1.0, vert_axis=2, velocity=u if previous else None, pressure=pr if previous else None,
                      previous_solution=previous)
    oKe, ofe, oGe, oSe, oeta = O.assemble(m, off, perm, xi, mat, mats, f, want_eta=True)
    assert _rel(eta, oeta) < 1e-12
    assert _rel(Ke, oKe) < 1e-12
    smat = mat[perm]                           # viscosities come in slot (element) order
    # every law moved the viscosity away from a constant
    assert np.std(eta[smat == 0]) > 0.01 and np.std(eta[smat == 1]) > 0.01
    if previous:
        assert np.std(eta[smat == 2]) > 0.01   # NonNewtonian with the point strain rates
    else:
        assert np.allclose(eta[smat == 2], (2 * 0.7) ** (1 / 3 - 1) * 5.0 ** (1 / 3))
