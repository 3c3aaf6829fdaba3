"""ctypes wrapper of the CPU oracle (``oracle/uwref.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The product library never
imports it.  Each wrapped routine restates the Underworld 1.x routine cited in ``uwref.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libuwref.so")
_lock = threading.Lock()
_lib = None

LAW_MATERIAL_VISCOSITY = 1
LAW_ARRHENIUS = 2
LAW_FRANK_KAMENETSKII = 3
LAW_VISCOSITY_LIMITER = 4
LAW_DRUCKER_PRAGER = 5
LAW_PARTICLE_VISCOSITY = 6
LAW_VON_MISES = 10
LAW_BYERLEE = 11
LAW_MOHR_COULOMB = 12


def strain_weakening_advance(pfw, incr, dt):
    """TimeIntegrand Euler step of postFailureWeakening with its stored time derivative, then
    _StrainWeakening_MakeValuesPositive (StrainWeakening.c:399-426; a higher-order integrator reads
    the same stored derivative at every stage, so the step is the same)."""
    out = pfw + dt * incr
    return np.where(out < 0.0, 0.0, out)


class Mesh(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nel", C.c_int32 * 3), ("min", C.c_double * 3), ("max", C.c_double * 3)]


class Law(C.Structure):
    _fields_ = [("law", C.c_int32), ("pad", C.c_int32), ("p", C.c_double * 8)]


class Material(C.Structure):
    _fields_ = [("n_laws", C.c_int32), ("pad", C.c_int32), ("laws", Law * 4),
                ("density", C.c_double), ("alpha", C.c_double), ("ref_temp", C.c_double)]


class Fields(C.Structure):
    _fields_ = [("temperature", C.c_void_p), ("velocity", C.c_void_p), ("pressure", C.c_void_p),
                ("previous_solution", C.c_int32), ("vert_axis", C.c_int32), ("gravity", C.c_double),
                ("pfw", C.c_void_p), ("pfw_incr", C.c_void_p), ("nl_form_jacobian", C.c_int32), ("pad", C.c_int32)]


class SolveOpts(C.Structure):
    _fields_ = [("mg_levels", C.c_int32), ("smooth_down", C.c_int32), ("smooth_up", C.c_int32),
                ("schur_type", C.c_int32), ("schur_pc", C.c_int32), ("restart", C.c_int32),
                ("max_outer", C.c_int32), ("max_inner", C.c_int32), ("scr_rtol", C.c_double),
                ("a11_rtol", C.c_double), ("back_rtol", C.c_double), ("remove_const_p", C.c_int32),
                ("nthreads", C.c_int32), ("bfbt_rtol", C.c_double), ("bfbt_max_it", C.c_int32), ("pad", C.c_int32)]


class PcdvcParams(C.Structure):
    _fields_ = [("upperT", C.c_double), ("lowerT", C.c_double), ("maxDeletions", C.c_int32), ("maxSplits", C.c_int32),
                ("splitInInterfaceCells", C.c_int32), ("deleteInInterfaceCells", C.c_int32)]


class Report(C.Structure):
    _fields_ = [("outer_its", C.c_int32), ("inner_its_total", C.c_int32), ("backsolve_its", C.c_int32),
                ("converged", C.c_int32), ("rel_residual", C.c_double), ("t_setup", C.c_double),
                ("t_solve", C.c_double)]


def build() -> str:
    """Compile the oracle with its Makefile (gcc, no GPU) and return the library path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                    os.path.join(_HERE, "uwref.c")):
                build()
            L = C.CDLL(_LIB_PATH)
            P = C.c_void_p
            L.uwr_num_nodes.restype = C.c_int64
            L.uwr_num_elements.restype = C.c_int64
            L.uwr_map.restype = C.c_int64
            L.uwr_map.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int32]
            L.uwr_random_layout.argtypes = [P, C.c_int32, C.c_uint32, P]
            L.uwr_assemble.argtypes = [P, C.c_int64, P, P, P, P, P, P, C.c_int32, P, P, P, P, P, P, P, P, C.c_int32]
            L.uwr_assemble_range.argtypes = [P, C.c_int64, C.c_int64, C.c_int64, P, P, P, P, P, P, C.c_int32, P, P,
                                             P, P, P, P, P, P, C.c_int32]
            L.uwr_dvc_element.argtypes = [C.c_int, P, C.c_int32, P, P, P]
            L.uwr_dvc_weights.argtypes = [P, P, P, P, P, P, C.c_int32]
            L.uwr_dvc_grid.argtypes = [C.c_int, P, P, P]
            L.uwr_pcdvc.restype = C.c_int64
            L.uwr_pcdvc.argtypes = [P, P, P, C.c_int64, C.c_int64, P, P, P, P, P, P, P, P, P, P]
            L.uwr_assemble_gauss.argtypes = [P, C.c_int32, P, P, P, P]
            L.uwr_eqnum.restype = C.c_int64
            L.uwr_eqnum.argtypes = [P, P, P]
            L.uwr_csr_nnz.restype = C.c_int64
            L.uwr_csr_nnz.argtypes = [P, P, C.c_int64, P]
            L.uwr_csr_fill.argtypes = [P, P, C.c_int64, P, P, P, P, C.c_int32]
            L.uwr_csr_spmv.argtypes = [C.c_int64, P, P, P, P, P, C.c_int32]
            L.uwr_solve_bsscr.argtypes = [P, P, P, P, P, P, P, P, P, P]
            L.uwr_solve_bsscr_bc.argtypes = [P, P, P, P, P, P, P, P, P, P, P]
            L.uwr_node_coords.argtypes = [P, P]
            L.uwr_global_to_local.argtypes = [P, C.c_int64, P, P]
            _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def make_mesh(dim, nel, mn=(0.0, 0.0, 0.0), mx=(1.0, 1.0, 1.0)) -> Mesh:
    m = Mesh()
    m.dim = dim
    for d in range(3):
        m.nel[d] = int(nel[d]) if d < len(nel) else 1
        m.min[d] = float(mn[d])
        m.max[d] = float(mx[d])
    return m


def make_material(laws, density=0.0, alpha=0.0, ref_temp=0.0) -> Material:
    """laws: list of (law_id, [params])."""
    mat = Material()
    mat.n_laws = len(laws)
    for i, (lid, params) in enumerate(laws):
        mat.laws[i].law = lid
        for j, v in enumerate(params):
            mat.laws[i].p[j] = float(v)
    mat.density = density
    mat.alpha = alpha
    mat.ref_temp = ref_temp
    return mat


def materials_array(mats):
    arr = (Material * len(mats))()
    for i, m in enumerate(mats):
        arr[i] = m
    return arr


def num_nodes(m):
    return lib().uwr_num_nodes(C.byref(m))


def num_elements(m):
    return lib().uwr_num_elements(C.byref(m))


def node_coords(m):
    xyz = np.zeros((num_nodes(m), 3))
    lib().uwr_node_coords(C.byref(m), _p(xyz))
    return xyz


def random_layout(m, ppc, seed):
    xyz = np.zeros((num_elements(m) * ppc, 3))
    lib().uwr_random_layout(C.byref(m), ppc, seed, _p(xyz))
    return xyz


def map_points(m, xyz, use_newton=True):
    """CoincidentMapper: returns (owning, offsets, perm, xi[perm order], n_outside)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = xyz.shape[0]
    E = num_elements(m)
    owning = np.zeros(n, np.uint32)
    offsets = np.zeros(E + 1, np.uint32)
    perm = np.zeros(n, np.uint32)
    xi = np.zeros((n, 3))
    outside = lib().uwr_map(C.byref(m), n, _p(xyz), _p(owning), _p(offsets), _p(perm), _p(xi),
                            1 if use_newton else 0)
    return owning, offsets, perm, xi, outside


def make_fields(temperature=None, velocity=None, pressure=None, previous_solution=False,
                vert_axis=1, gravity=0.0, pfw=None, pfw_incr=None, jacobian=False):
    """pfw: per-point postFailureWeakening (strain-weakening history); pfw_incr: a float64 array of
    the same length that the assembly fills with its time derivative."""
    f = Fields()
    keep = []
    if pfw_incr is not None:
        assert pfw_incr.dtype == np.float64 and pfw_incr.flags.c_contiguous
        f.pfw_incr = pfw_incr.ctypes.data
        keep.append(pfw_incr)
    for name, arr in (("temperature", temperature), ("velocity", velocity), ("pressure", pressure), ("pfw", pfw)):
        if arr is not None:
            arr = np.ascontiguousarray(arr, dtype=np.float64)
            keep.append(arr)
            setattr(f, name, arr.ctypes.data)
    f.previous_solution = 1 if previous_solution else 0
    f.nl_form_jacobian = 1 if jacobian else 0
    f.vert_axis = vert_axis
    f.gravity = gravity
    f._keep = keep
    return f


def assemble(m, offsets, perm, xi, material, mats, fields, point_eta=None, point_rho=None,
             nthreads=0, want_eta=False, weights=None):
    """Element matrices from the points in slot order (xi [slot][3]); weights: per-slot
    integration weights (e.g. dvc_weights), else the constant 2^dim / count."""
    dim = m.dim
    nen = 8 if dim == 3 else 4
    nd = nen * dim
    E = num_elements(m)
    n = perm.shape[0]
    Ke = np.zeros((E, nd, nd))
    fe = np.zeros((E, nd))
    Ge = np.zeros((E, nd))
    Se = np.zeros(E)
    eta = np.zeros(n) if want_eta else None
    material = None if material is None else np.ascontiguousarray(material, dtype=np.int32)
    point_eta = None if point_eta is None else np.ascontiguousarray(point_eta, dtype=np.float64)
    point_rho = None if point_rho is None else np.ascontiguousarray(point_rho, dtype=np.float64)
    weights = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    arr = materials_array(mats)
    rc = lib().uwr_assemble(C.byref(m), n, _p(offsets), _p(perm), _p(np.ascontiguousarray(xi)),
                            _p(material), _p(point_eta), _p(point_rho), len(mats), arr,
                            C.byref(fields), _p(Ke), _p(fe), _p(Ge), _p(Se), _p(eta), _p(weights), nthreads)
    if rc != 0:
        raise RuntimeError("oracle assembly failed (material index out of range)")
    return Ke, fe, Ge, Se, eta


def assemble_range(m, first, count, offsets, perm, xi, material, mats, fields, point_eta=None, point_rho=None,
                   nthreads=0):
    """Element matrices of elements [first, first + count) only (points in slot order, as in
    assemble): returns Ke (count, nd, nd), fe, Ge (count, nd), Se (count,)."""
    dim = m.dim
    nd = (8 if dim == 3 else 4) * dim
    Ke = np.zeros((count, nd, nd))
    fe = np.zeros((count, nd))
    Ge = np.zeros((count, nd))
    Se = np.zeros(count)
    material = None if material is None else np.ascontiguousarray(material, dtype=np.int32)
    point_eta = None if point_eta is None else np.ascontiguousarray(point_eta, dtype=np.float64)
    point_rho = None if point_rho is None else np.ascontiguousarray(point_rho, dtype=np.float64)
    arr = materials_array(mats)
    rc = lib().uwr_assemble_range(C.byref(m), int(first), int(count), perm.shape[0], _p(offsets), _p(perm),
                                  _p(np.ascontiguousarray(xi)), _p(material), _p(point_eta), _p(point_rho), len(mats),
                                  arr, C.byref(fields), _p(Ke), _p(fe), _p(Ge), _p(Se), None, None, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle assembly of a range failed ({rc})")
    return Ke, fe, Ge, Se


def dvc_element(dim, res, xi):
    """Discrete Voronoi weights of one element: xi (nump, dim) local coordinates -> (centroids
    (nump, dim), weights (nump,), growth passes)."""
    xi = np.ascontiguousarray(xi, dtype=np.float64).reshape(-1, dim)
    r = np.ascontiguousarray(list(res) + [1] * (3 - len(res)), dtype=np.int32)
    cxi = np.zeros_like(xi)
    w = np.zeros(xi.shape[0])
    passes = lib().uwr_dvc_element(dim, _p(r), xi.shape[0], _p(xi), _p(cxi), _p(w))
    if passes < 0:
        raise ValueError("DVC resolution out of range")
    return cxi, w, passes


def dvc_grid(dim, res):
    """(cell centres (nc, dim), face neighbours (nc, 2 dim): N, S, E, W[, U, D], -2 at the border)."""
    r = np.ascontiguousarray(list(res) + [1] * (3 - len(res)), dtype=np.int32)
    nc = int(np.prod(r[:dim]))
    centre = np.zeros((nc, dim))
    nbr = np.zeros((nc, 2 * dim), np.int32)
    lib().uwr_dvc_grid(dim, _p(r), _p(centre), _p(nbr))
    return centre, nbr


def dvc_weights(m, res, offsets, xi, nthreads=0):
    """Discrete Voronoi weights of every element, points in slot order: xi [slot][3] ->
    (centroids [slot][3], weights [slot])."""
    xi = np.ascontiguousarray(xi, dtype=np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(list(res) + [1] * (3 - len(res)), dtype=np.int32)
    cxi = np.zeros_like(xi)
    w = np.zeros(xi.shape[0])
    lib().uwr_dvc_weights(C.byref(m), _p(r), _p(np.ascontiguousarray(offsets, dtype=np.uint32)), _p(xi), _p(cxi),
                          _p(w), nthreads)
    return cxi, w


def pcdvc(m, res, xyz, material, offsets, perm, xi, upperT=25.0, lowerT=0.6, max_deletions=2, max_splits=3,
          split_in_interface=False, delete_in_interface=False):
    """One PCDVC population-control pass (non-inflow) over the cell tables of a CoincidentMapper pass
    (offsets, perm; xi [slot][3]).  Returns (xyz (n', 3), material, src (input point of every output
    point), offsets', perm', integration xi [slot][3], weights [slot])."""
    n = xyz.shape[0]
    E = num_elements(m)
    cap = n + max_splits * E
    X = np.zeros((cap, 3))
    X[:n] = xyz
    M = np.zeros(cap, np.int32)
    M[:n] = material
    S = np.zeros(cap, np.int64)
    off = np.zeros(E + 1, np.uint32)
    pr = np.zeros(cap, np.uint32)
    xo = np.zeros((cap, 3))
    wo = np.zeros(cap)
    pp = PcdvcParams(upperT, lowerT, max_deletions, max_splits, int(split_in_interface), int(delete_in_interface))
    r = np.ascontiguousarray(list(res) + [1] * (3 - len(res)), dtype=np.int32)
    cnt = lib().uwr_pcdvc(C.byref(m), _p(r), C.byref(pp), n, cap, _p(X), _p(M), _p(S),
                          _p(np.ascontiguousarray(offsets, dtype=np.uint32)), _p(np.ascontiguousarray(perm, dtype=np.uint32)),
                          _p(np.ascontiguousarray(xi, dtype=np.float64)), _p(off), _p(pr), _p(xo), _p(wo))
    if cnt < 0:
        raise RuntimeError(f"oracle PCDVC failed ({cnt})")
    return X[:cnt], M[:cnt], S[:cnt], off, pr[:cnt], xo[:cnt], wo[:cnt]


def assemble_gauss(m, mats, el_material, fields):
    dim = m.dim
    nd = (8 if dim == 3 else 4) * dim
    E = num_elements(m)
    Ke = np.zeros((E, nd, nd))
    elm = None if el_material is None else np.ascontiguousarray(el_material, dtype=np.int32)
    arr = materials_array(mats)
    rc = lib().uwr_assemble_gauss(C.byref(m), len(mats), arr, _p(elm), C.byref(fields), _p(Ke))
    if rc != 0:
        raise RuntimeError("oracle gauss assembly failed")
    return Ke


def eqnum(m, fixed=None):
    nn = num_nodes(m)
    eq = np.zeros(nn * m.dim, np.int64)
    fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
    nfree = lib().uwr_eqnum(C.byref(m), _p(fx), _p(eq))
    return eq, nfree


def global_csr(m, Ke, fixed=None, nthreads=0):
    """Assembled K over free dofs as (rowptr, cols, vals, eq, nfree)."""
    eq, nfree = eqnum(m, fixed)
    rowptr = np.zeros(nfree + 1, np.int64)
    nnz = lib().uwr_csr_nnz(C.byref(m), _p(eq), nfree, _p(rowptr))
    cols = np.zeros(nnz, np.int64)
    vals = np.zeros(nnz)
    lib().uwr_csr_fill(C.byref(m), _p(eq), nfree, _p(np.ascontiguousarray(Ke)), _p(rowptr), _p(cols),
                       _p(vals), nthreads)
    return rowptr, cols, vals, eq, nfree


def csr_spmv(rowptr, cols, vals, x, nthreads=0):
    y = np.zeros(rowptr.shape[0] - 1)
    lib().uwr_csr_spmv(rowptr.shape[0] - 1, _p(rowptr), _p(cols), _p(vals), _p(x), _p(y), nthreads)
    return y


def solve_bsscr(m, fixed, Ke, Ge, fe, Se, mg_levels=3, smooth=2, schur_type=1, schur_pc=0,
                scr_rtol=1e-10, a11_rtol=1e-12, back_rtol=1e-12, restart=30, max_outer=500,
                max_inner=2000, remove_const_p=True, nthreads=0, bfbt_rtol=1e-4, bfbt_max_it=500, bcval=None):
    """BSSCR solve; bcval (nn*dim, read where fixed) gives non-zero Dirichlet values, lifted into
    the right-hand sides as the reference's assembly does (None: homogeneous conditions)."""
    o = SolveOpts(mg_levels, smooth, smooth, schur_type, schur_pc, restart, max_outer, max_inner,
                  scr_rtol, a11_rtol, back_rtol, int(remove_const_p), nthreads, bfbt_rtol, bfbt_max_it, 0)
    nn = num_nodes(m)
    E = num_elements(m)
    u = np.zeros((nn, m.dim))
    p = np.zeros(E)
    rep = Report()
    fx = np.ascontiguousarray(fixed, dtype=np.uint8)
    bv = None if bcval is None else np.ascontiguousarray(bcval, dtype=np.float64).reshape(-1)
    rc = lib().uwr_solve_bsscr_bc(C.byref(m), _p(fx), _p(bv), _p(np.ascontiguousarray(Ke)),
                                  _p(np.ascontiguousarray(Ge)), _p(np.ascontiguousarray(fe)),
                                  _p(np.ascontiguousarray(Se)), C.byref(o), _p(u), _p(p), C.byref(rep))
    if rc == -3:
        raise ValueError(f"oracle BSSCR: {m.dim}D mesh {tuple(m.nel[:m.dim])} does not coarsen {mg_levels - 1} times")
    if rc != 0:
        raise RuntimeError("oracle BSSCR setup failed (coarse factorisation)")
    return u, p, rep


def advect(m, u_nodal, xyz, dt, order=2, allow_fallback=False):
    """SwarmAdvector step (first or second order) -> (new positions (n, 3), failed, fallbacks)"""
    out = np.ascontiguousarray(xyz, dtype=np.float64).copy()
    fb = C.c_int64()
    lib().uwr_advect.restype = C.c_int64
    failed = lib().uwr_advect(C.byref(m), _p(np.ascontiguousarray(u_nodal, dtype=np.float64)), out.shape[0], _p(out),
                              C.c_double(dt), order, 1 if allow_fallback else 0, C.byref(fb))
    return out, int(failed), fb.value


def free_slip_mask(m):
    """Free-slip walls: the normal velocity component is fixed on every wall."""
    nn = num_nodes(m)
    dim = m.dim
    nx, ny = m.nel[0] + 1, m.nel[1] + 1
    nz = m.nel[2] + 1 if dim == 3 else 1
    idx = np.arange(nn)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    fixed = np.zeros((nn, dim), np.uint8)
    fixed[(i == 0) | (i == nx - 1), 0] = 1
    fixed[(j == 0) | (j == ny - 1), 1] = 1
    if dim == 3:
        fixed[(k == 0) | (k == nz - 1), 2] = 1
    return fixed.reshape(-1)


def full_matrix_from_csr(rowptr, cols, vals, n):
    import scipy.sparse as sp
    return sp.csr_matrix((vals, cols, rowptr), shape=(n, n))
