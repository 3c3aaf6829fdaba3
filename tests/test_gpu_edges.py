"""Edge cases of the mapper and the assembly through the C ABI, against the oracle: points on
element faces, edges, corners and the upper domain boundary (Num_Approx tie rules,
Mesh_RegularAlgorithms.c:194-226), ragged per-element counts (one element holding hundreds of
points next to elements holding one), and the inputs the library must refuse: points outside the
mesh, an element with no integration point, a material index out of range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm((a - b).reshape(-1)) / max(np.linalg.norm(b.reshape(-1)), 1e-300)


def _ctx(U, nel, x, y, z, mat, nmat=2):
    ctx = U.Context(0)
    ctx.mesh_q1(3, nel)
    ctx.bc_set(U.free_slip_mask(3, nel))
    mats = [U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0 + 9.0 * k])], density=float(k)) for k in range(nmat)]
    ctx.materials_set(mats)
    ctx.fields_set(None, 1.0, 2)
    ctx.particles_upload(x, y, z, mat)
    return ctx, mats


def _oracle_assemble(O, nel, x, y, z, mat, nmat=2):
    m = O.make_mesh(3, nel)
    _, off, perm, xi, outside = O.map_points(m, np.stack([x, y, z], axis=1))
    mats = [O.make_material([(1, [1.0 + 9.0 * k])], density=float(k)) for k in range(nmat)]
    f = O.make_fields(gravity=1.0, vert_axis=2)
    Ke, fe, Ge, Se, _ = O.assemble(m, off, perm, xi, mat, mats, f)
    return off, perm, xi, outside, Ke, fe, Ge, Se


def _face_points(nel, rng):
    """every element gets a few interior points; on top: points exactly on node coordinates,
    element faces and the upper boundary, and points within 1e-13 of a face (ties to the lower
    element by Num_Approx's 1e-12 relative epsilon)"""
    pts = []
    for e in range(int(np.prod(nel))):
        i, j, k = e % nel[0], (e // nel[0]) % nel[1], e // (nel[0] * nel[1])
        for _ in range(4):
            pts.append([(i + rng.uniform(0.05, 0.95)) / nel[0], (j + rng.uniform(0.05, 0.95)) / nel[1],
                        (k + rng.uniform(0.05, 0.95)) / nel[2]])
    for a in range(nel[0] + 1):
        for b in range(nel[1] + 1):
            pts.append([a / nel[0], b / nel[1], rng.integers(0, nel[2] + 1) / nel[2]])
    for t in range(60):
        base = [rng.integers(0, nel[d] + 1) / nel[d] for d in range(3)]
        d = t % 3
        base[d] = min(max(base[d] + rng.choice([-1e-13, 1e-13, 0.0]), 0.0), 1.0)
        pts.append(base)
    pts.append([1.0, 1.0, 1.0])
    pts.append([0.0, 0.0, 0.0])
    return np.array(pts)


def test_face_edge_corner_points_bin_bit_exactly(oracle, uw):
    O, U = oracle, uw
    nel = (4, 3, 5)
    rng = np.random.default_rng(21)
    p = _face_points(nel, rng)
    mat = rng.integers(0, 2, len(p)).astype(np.int32)
    ctx, _ = _ctx(U, nel, p[:, 0], p[:, 1], p[:, 2], mat)
    perm, offsets, xi = ctx.bin_and_map()
    ctx.assemble()
    Ke, fe, Ge, Se = ctx.element_matrices()
    ctx.close()
    ooff, operm, oxi, outside, oKe, ofe, oGe, oSe = _oracle_assemble(O, nel, p[:, 0], p[:, 1], p[:, 2], mat)
    assert outside == 0
    assert np.array_equal(offsets, ooff)
    assert np.array_equal(perm, operm)
    assert np.max(np.abs(xi - oxi)) < 1e-13
    assert _rel(Ke, oKe) < 1e-12 and _rel(fe, ofe) < 1e-12 and _rel(Se, oSe) < 1e-12


def test_ragged_cells_assembly_parity(oracle, uw):
    """one element with 400 points, most with one or two: the per-element loops and the
    warp-per-element ordering of the mapper must not depend on the count"""
    O, U = oracle, uw
    nel = (3, 3, 3)
    rng = np.random.default_rng(5)
    pts = [[rng.uniform(0.0, 1 / 3), rng.uniform(0.0, 1 / 3), rng.uniform(0.0, 1 / 3)] for _ in range(400)]
    for e in range(27):
        i, j, k = e % 3, (e // 3) % 3, e // 9
        for _ in range(1 + e % 2):
            pts.append([(i + rng.uniform()) / 3, (j + rng.uniform()) / 3, (k + rng.uniform()) / 3])
    p = np.array(pts)
    order = rng.permutation(len(p))
    p = p[order]
    mat = (p[:, 2] > 0.5).astype(np.int32)
    ctx, _ = _ctx(U, nel, p[:, 0], p[:, 1], p[:, 2], mat)
    perm, offsets, xi = ctx.bin_and_map()
    ctx.assemble()
    Ke, fe, Ge, Se = ctx.element_matrices()
    ctx.close()
    ooff, operm, oxi, outside, oKe, ofe, oGe, oSe = _oracle_assemble(O, nel, p[:, 0], p[:, 1], p[:, 2], mat)
    counts = np.diff(ooff)
    assert counts.max() >= 400 and counts.min() == 1
    assert np.array_equal(offsets, ooff) and np.array_equal(perm, operm)
    assert _rel(Ke, oKe) < 1e-12 and _rel(fe, ofe) < 1e-12


def test_points_outside_the_mesh_are_refused(oracle, uw):
    O, U = oracle, uw
    nel = (2, 2, 2)
    rng = np.random.default_rng(1)
    p = rng.uniform(0.0, 1.0, (200, 3))
    p[17] = [1.0 + 1e-9, 0.5, 0.5]
    p[99] = [0.5, -1e-9, 0.5]
    ctx, _ = _ctx(U, nel, p[:, 0], p[:, 1], p[:, 2], np.zeros(len(p), np.int32))
    with pytest.raises(U.UwgpuError) as err:
        ctx.bin_and_map()
    assert err.value.code == U.ERR_DOMAIN and "2 material points" in str(err.value)
    ctx.close()
    _, _, _, _, outside = O.map_points(O.make_mesh(3, nel), p)
    assert outside == 2


def test_empty_element_and_bad_material_are_refused(uw):
    U = uw
    nel = (2, 2, 2)
    rng = np.random.default_rng(2)
    p = rng.uniform(0.0, 0.49, (100, 3))   # only the first element is populated
    ctx, _ = _ctx(U, nel, p[:, 0], p[:, 1], p[:, 2], np.zeros(len(p), np.int32))
    ctx.bin_and_map(want=False)
    with pytest.raises(U.UwgpuError) as err:
        ctx.assemble()
    assert err.value.code == U.ERR_ARGUMENT and "no integration points" in str(err.value)
    ctx.close()
    p = rng.uniform(0.0, 1.0, (400, 3))
    mat = np.zeros(len(p), np.int32)
    mat[5] = 7
    ctx, _ = _ctx(U, nel, p[:, 0], p[:, 1], p[:, 2], mat)
    ctx.bin_and_map(want=False)
    with pytest.raises(U.UwgpuError) as err:
        ctx.assemble()
    assert err.value.code == U.ERR_ARGUMENT and "material index" in str(err.value)
    ctx.close()
