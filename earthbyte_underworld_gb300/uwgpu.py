"""ctypes binding of libuwgpu (include/uwgpu.h) for Python callers, tests and the benchmark.

The library must be built (``earthbyte_underworld_gb300.build.build()``); loading fails loudly
when it is missing or when no CUDA device is present -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

_lock = threading.Lock()
_lib = None

OK = 0
ERR_ARGUMENT, ERR_CUDA, ERR_MEMORY, ERR_STATE, ERR_DOMAIN, ERR_NOT_CONVERGED, ERR_NAN, ERR_UNSUPPORTED, ERR_BREAKDOWN = range(1, 10)

LAW_MATERIAL_VISCOSITY = 1
LAW_ARRHENIUS = 2
LAW_FRANK_KAMENETSKII = 3
LAW_VISCOSITY_LIMITER = 4
LAW_DRUCKER_PRAGER = 5
LAW_PARTICLE_VISCOSITY = 6
LAW_LINEAR_VISCOSITY = 7
LAW_DEPTH_DEPENDENT = 8
LAW_NON_NEWTONIAN = 9
LAW_VON_MISES = 10
LAW_BYERLEE = 11
LAW_MOHR_COULOMB = 12

PREC_FP64 = 0
PREC_MIXED = 1
SCHUR_CG = 0
SCHUR_FGMRES = 1
SCHUR_PC_UW = 0
SCHUR_PC_GKGDIAG = 1
SCHUR_PC_NONE = 2
SCHUR_PC_SCALED_BFBT = 3
SMOOTHER_COLOUR_GS = 0
SMOOTHER_CHEBYSHEV = 1
ASSEMBLY_FP64 = 0
ASSEMBLY_TENSOR = 1

KERNEL_ASSEMBLY, KERNEL_APPLY, KERNEL_SMOOTH, KERNEL_BINNING, KERNEL_SCHUR_PC, KERNEL_VECTOR, KERNEL_TRANSFER, \
    KERNEL_LEARNED, KERNEL_SETUP = range(9)

WEIGHTS_CONSTANT = 0
WEIGHTS_DVC = 1


class UwgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"uwgpu error {code}: {msg}")
        self.code = code


class Law(C.Structure):
    _fields_ = [("law", C.c_int32), ("pad", C.c_int32), ("p", C.c_double * 8)]


class Material(C.Structure):
    _fields_ = [("n_laws", C.c_int32), ("pad", C.c_int32), ("laws", Law * 4),
                ("density", C.c_double), ("alpha", C.c_double), ("ref_temp", C.c_double)]


class SolveOpts(C.Structure):
    _fields_ = [("mg_levels", C.c_int32), ("smooth_down", C.c_int32), ("smooth_up", C.c_int32),
                ("schur_type", C.c_int32), ("schur_pc", C.c_int32), ("restart", C.c_int32),
                ("max_outer", C.c_int32), ("max_inner", C.c_int32), ("scr_rtol", C.c_double),
                ("a11_rtol", C.c_double), ("back_rtol", C.c_double), ("remove_const_p", C.c_int32),
                ("precision", C.c_int32), ("target_rel_residual", C.c_double), ("bfbt_rtol", C.c_double),
                ("bfbt_max_it", C.c_int32), ("smoother", C.c_int32), ("learned_pc", C.c_int32),
                ("learned_stagnation", C.c_int32), ("mg_cycle", C.c_int32), ("bfbt_inner_pc", C.c_int32)]


class PcdvcOpts(C.Structure):
    _fields_ = [("upper_t", C.c_double), ("lower_t", C.c_double), ("max_deletions", C.c_int32),
                ("max_splits", C.c_int32), ("split_in_interface_cells", C.c_int32),
                ("delete_in_interface_cells", C.c_int32)]


class Report(C.Structure):
    _fields_ = [("outer_its", C.c_int32), ("inner_its_total", C.c_int32), ("backsolve_its", C.c_int32),
                ("vcycles", C.c_int32), ("converged", C.c_int32), ("status", C.c_int32),
                ("rel_residual", C.c_double), ("t_setup_ms", C.c_double), ("t_solve_ms", C.c_double),
                ("pc_inner_its", C.c_int64), ("learned_applies", C.c_int32), ("learned_fallbacks", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libuwgpu.so; builds it first if it is absent (requires nvcc)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise UwgpuError(ERR_STATE, f"{path} is missing; build it with earthbyte_underworld_gb300.build")
            _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.uwgpu_abi_version.restype = C.c_int
        L.uwgpu_create.argtypes = [C.c_int32, C.POINTER(P)]
        L.uwgpu_destroy.argtypes = [P]
        L.uwgpu_destroy.restype = None
        L.uwgpu_last_error.argtypes = [P]
        L.uwgpu_last_error.restype = C.c_char_p
        L.uwgpu_synchronize.argtypes = [P]
        L.uwgpu_mesh_q1.argtypes = [P, C.c_int32, P, P, P]
        L.uwgpu_bc_set.argtypes = [P, P, P]
        L.uwgpu_materials_set.argtypes = [P, C.c_int32, P]
        L.uwgpu_fields_set.argtypes = [P, P, C.c_double, C.c_int32]
        L.uwgpu_solution_set.argtypes = [P, P, P]
        L.uwgpu_particles_upload.argtypes = [P, C.c_int64, P, P, P, P, P, P]
        L.uwgpu_bin_and_map.argtypes = [P, P, P, P]
        L.uwgpu_assemble.argtypes = [P]
        L.uwgpu_get_element_matrices.argtypes = [P, C.c_int64, C.c_int64, P, P, P, P]
        L.uwgpu_get_point_viscosity.argtypes = [P, P]
        L.uwgpu_operator_apply.argtypes = [P, C.c_int32, P, P]
        L.uwgpu_solve_bsscr.argtypes = [P, P, P, P, P]
        L.uwgpu_solve_picard.argtypes = [P, P, C.c_double, C.c_int32, C.c_int32, P, P, P, P, P]
        L.uwgpu_solve_opts_default.argtypes = [P]
        L.uwgpu_solve_opts_default.restype = None
        L.uwgpu_profile_enable.argtypes = [P, C.c_int32]
        L.uwgpu_profile_read.argtypes = [P, C.c_int32, P, P]
        L.uwgpu_profile_read_work.argtypes = [P, C.c_int32, P, P]
        L.uwgpu_get_stream.argtypes = [P, P]
        L.uwgpu_time_apply.argtypes = [P, C.c_int32, C.c_int32, P]
        L.uwgpu_time_smooth.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P]
        L.uwgpu_time_chebyshev.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, P]
        L.uwgpu_bfbt_operator_apply.argtypes = [P, C.c_int32, P, P]
        L.uwgpu_weights_set.argtypes = [P, C.c_int32, P]
        L.uwgpu_integration_points.argtypes = [P, P, P]
        L.uwgpu_time_bfbt_apply.argtypes = [P, C.c_int32, C.c_int32, P]
        L.uwgpu_launch_count.argtypes = [P]
        L.uwgpu_launch_count.restype = C.c_int64
        L.uwgpu_learned_create.argtypes = [P, C.c_int32, C.c_int32, C.c_uint64]
        L.uwgpu_learned_param_count.argtypes = [P, P]
        L.uwgpu_learned_get_params.argtypes = [P, P]
        L.uwgpu_learned_set_params.argtypes = [P, P]
        L.uwgpu_learned_forward.argtypes = [P, P, P]
        L.uwgpu_learned_backward.argtypes = [P, P, P, P]
        L.uwgpu_advect_particles.argtypes = [P, C.c_double, C.c_int32, C.c_int32, P, P]
        L.uwgpu_particles_download.argtypes = [P, P, P, P]
        L.uwgpu_learned_generate.argtypes = [P, P, C.c_int32, C.c_uint64]
        L.uwgpu_learned_train.argtypes = [P, C.c_int32, C.c_int32, C.c_float, C.c_uint64, P, P]
        L.uwgpu_tc_check.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P, P]
        L.uwgpu_assembly_set.argtypes = [P, C.c_int32]
        L.uwgpu_smoother_storage_set.argtypes = [P, C.c_int32]
        L.uwgpu_jacobian_set.argtypes = [P, C.c_int32]
        L.uwgpu_population_control.argtypes = [P, P, P]
        L.uwgpu_get_cell_tables.argtypes = [P, P, P]
        L.uwgpu_strain_weakening_set.argtypes = [P, P]
        L.uwgpu_strain_weakening_advance.argtypes = [P, C.c_double]
        L.uwgpu_strain_weakening_get.argtypes = [P, P, P]
        _lib = L
        return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def make_material(laws, density=0.0, alpha=0.0, ref_temp=0.0) -> Material:
    """laws: ordered list of (law_id, [params]) as in a RheologyMaterial's Rheology list."""
    if not 1 <= len(laws) <= 4:
        raise ValueError("a material takes 1..4 rheology laws")
    m = Material()
    m.n_laws = len(laws)
    for i, (lid, params) in enumerate(laws):
        m.laws[i].law = int(lid)
        for j, v in enumerate(params):
            m.laws[i].p[j] = float(v)
    m.density = float(density)
    m.alpha = float(alpha)
    m.ref_temp = float(ref_temp)
    return m


def default_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    load().uwgpu_solve_opts_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class Context:
    """One device context: mesh, material points, assembled system and solver state."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = C.c_void_p()
        rc = self._L.uwgpu_create(int(device), C.byref(h))
        if rc != OK:
            raise UwgpuError(rc, "uwgpu_create failed (no CUDA device?)")
        self._h = h
        self.dim = None
        self.nel = None

    def close(self):
        if getattr(self, "_h", None):
            self._L.uwgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != OK:
            msg = self._L.uwgpu_last_error(self._h)
            raise UwgpuError(rc, msg.decode() if msg else "")

    # ---- setup ----
    def mesh_q1(self, dim, nel, mn=(0.0, 0.0, 0.0), mx=(1.0, 1.0, 1.0)):
        n = (C.c_int32 * 3)(*(list(nel) + [1] * (3 - len(nel))))
        a = (C.c_double * 3)(*(list(mn) + [0.0] * (3 - len(mn))))
        b = (C.c_double * 3)(*(list(mx) + [1.0] * (3 - len(mx))))
        self._check(self._L.uwgpu_mesh_q1(self._h, dim, n, a, b))
        self.dim = dim
        self.nel = tuple(int(v) for v in list(nel)[:dim])
        self.nnodes = int(np.prod([v + 1 for v in self.nel]))
        self.nelements = int(np.prod(self.nel))

    def bc_set(self, fixed, values=None):
        fx = np.ascontiguousarray(fixed, dtype=np.uint8).reshape(-1)
        vals = None if values is None else np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        self._check(self._L.uwgpu_bc_set(self._h, _ptr(fx), _ptr(vals)))

    def materials_set(self, mats):
        arr = (Material * len(mats))(*mats)
        self._check(self._L.uwgpu_materials_set(self._h, len(mats), arr))

    def fields_set(self, temperature=None, gravity=0.0, vert_axis=1):
        t = None if temperature is None else np.ascontiguousarray(temperature, dtype=np.float64)
        self._check(self._L.uwgpu_fields_set(self._h, _ptr(t), float(gravity), int(vert_axis)))

    def solution_set(self, u, p):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1)
        self._check(self._L.uwgpu_solution_set(self._h, _ptr(u), _ptr(p)))

    def particles_upload(self, x, y, z=None, material=None, eta=None, rho=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        z = None if z is None else np.ascontiguousarray(z, dtype=np.float64)
        mat = None if material is None else np.ascontiguousarray(material, dtype=np.int32)
        eta = None if eta is None else np.ascontiguousarray(eta, dtype=np.float64)
        rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
        self._keep = (x, y, z, mat, eta, rho)
        self.npoints = x.shape[0]
        self._check(self._L.uwgpu_particles_upload(self._h, x.shape[0], _ptr(x), _ptr(y), _ptr(z), _ptr(mat),
                                                   _ptr(eta), _ptr(rho)))

    # ---- hot path ----
    def advect(self, dt, order=2, allow_fallback=False):
        """advect the material points with the current velocity -> (fallbacks, points that left the mesh)"""
        fb, lm = C.c_uint32(), C.c_uint32()
        self._check(self._L.uwgpu_advect_particles(self._h, dt, order, 1 if allow_fallback else 0, C.byref(fb),
                                                   C.byref(lm)))
        return fb.value, lm.value

    def particles(self):
        """current coordinates (x, y, z) of the material points"""
        n = self.npoints
        x, y, z = (np.zeros(n) for _ in range(3))
        self._check(self._L.uwgpu_particles_download(self._h, _ptr(x), _ptr(y), _ptr(z) if self.dim == 3 else None))
        return x, y, z

    def bin_and_map(self, want=True):
        if not want:
            self._check(self._L.uwgpu_bin_and_map(self._h, None, None, None))
            return None
        perm = np.zeros(self.npoints, np.uint32)
        offsets = np.zeros(self.nelements + 1, np.uint32)
        xi = np.zeros((self.npoints, 3))
        self._check(self._L.uwgpu_bin_and_map(self._h, _ptr(perm), _ptr(offsets), _ptr(xi)))
        return perm, offsets, xi

    def strain_weakening_set(self, pfw=None):
        """Upload the per-point strain-weakening history (None: zero) and enable it."""
        a = None if pfw is None else np.ascontiguousarray(pfw, dtype=np.float64)
        self._check(self._L.uwgpu_strain_weakening_set(self._h, _ptr(a)))

    def strain_weakening_advance(self, dt):
        self._check(self._L.uwgpu_strain_weakening_advance(self._h, float(dt)))

    def strain_weakening(self):
        """(history, time derivative from the last assembly), per point."""
        pfw = np.zeros(self.npoints)
        inc = np.zeros(self.npoints)
        self._check(self._L.uwgpu_strain_weakening_get(self._h, _ptr(pfw), _ptr(inc)))
        return pfw, inc

    def population_control(self, upper_t=25.0, lower_t=0.6, max_deletions=2, max_splits=3,
                           split_in_interface_cells=False, delete_in_interface_cells=False):
        """PCDVC split / delete pass (DVC weights must be selected); returns the new point count."""
        o = PcdvcOpts(upper_t, lower_t, max_deletions, max_splits, int(split_in_interface_cells),
                      int(delete_in_interface_cells))
        n = C.c_int64()
        self._check(self._L.uwgpu_population_control(self._h, C.byref(o), C.byref(n)))
        self.npoints = n.value
        return n.value

    def cell_tables(self):
        """(perm, offsets) of the current cell tables, without re-binning."""
        perm = np.zeros(self.npoints, np.uint32)
        offsets = np.zeros(self.nelements + 1, np.uint32)
        self._check(self._L.uwgpu_get_cell_tables(self._h, _ptr(perm), _ptr(offsets)))
        return perm, offsets

    def jacobian_set(self, on=True):
        """Newton (Jacobian) form of the 2D element matrices for the next assemblies."""
        self._check(self._L.uwgpu_jacobian_set(self._h, 1 if on else 0))

    def smoother_storage_set(self, bits):
        """16 (default): the mixed form smooths with FP16 row-scaled stencils; 32: FP32."""
        self._check(self._L.uwgpu_smoother_storage_set(self._h, int(bits)))

    def assembly_set(self, mode):
        """ASSEMBLY_FP64 (default) or ASSEMBLY_TENSOR (tensor-core contraction of the moments, 3D)."""
        self._check(self._L.uwgpu_assembly_set(self._h, int(mode)))

    def assemble(self):
        self._check(self._L.uwgpu_assemble(self._h))

    def element_matrices(self, first=0, count=None):
        if count is None:
            count = self.nelements - first
        nd = (1 << self.dim) * self.dim
        Ke = np.zeros((count, nd, nd))
        fe = np.zeros((count, nd))
        Ge = np.zeros((count, nd))
        Se = np.zeros(count)
        self._check(self._L.uwgpu_get_element_matrices(self._h, first, count, _ptr(Ke), _ptr(fe), _ptr(Ge), _ptr(Se)))
        return Ke, fe, Ge, Se

    def point_viscosity(self):
        eta = np.zeros(self.npoints)
        self._check(self._L.uwgpu_get_point_viscosity(self._h, _ptr(eta)))
        return eta

    def operator_apply(self, x, precision=PREC_FP64):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.zeros_like(x)
        self._check(self._L.uwgpu_operator_apply(self._h, precision, _ptr(x), _ptr(y)))
        return y

    def solve_bsscr(self, opts: SolveOpts | None = None, want=True, check=True):
        opts = opts or default_opts()
        rep = Report()
        u = np.zeros((self.nnodes, self.dim)) if want else None
        p = np.zeros(self.nelements) if want else None
        rc = self._L.uwgpu_solve_bsscr(self._h, C.byref(opts), _ptr(u), _ptr(p), C.byref(rep))
        if check:
            self._check(rc)
        return u, p, rep

    def solve_picard(self, opts: SolveOpts | None = None, tolerance=1e-4, max_iterations=20, min_iterations=1,
                     check=True):
        """Picard iteration (re-assemble with the current solution, re-solve) until the relative
        velocity change is below `tolerance` (tolerance <= 0: exactly max_iterations solves).
        Returns u, p, report, iterations, residual; with check=False a status other than OK is
        left in report.status instead of raised."""
        opts = opts or default_opts()
        rep = Report()
        u = np.zeros((self.nnodes, self.dim))
        p = np.zeros(self.nelements)
        its = C.c_int32()
        res = C.c_double()
        rc = self._L.uwgpu_solve_picard(self._h, C.byref(opts), float(tolerance), int(max_iterations),
                                        int(min_iterations), _ptr(u), _ptr(p), C.byref(rep), C.byref(its),
                                        C.byref(res))
        if check:
            self._check(rc)
        return u, p, rep, its.value, res.value

    def synchronize(self):
        self._check(self._L.uwgpu_synchronize(self._h))

    # ---- timing ----
    def profile_enable(self, on=True):
        self._check(self._L.uwgpu_profile_enable(self._h, 1 if on else 0))

    def profile_read(self, which):
        n = C.c_int64()
        ms = C.c_double()
        self._check(self._L.uwgpu_profile_read(self._h, which, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def profile_work(self, which):
        b = C.c_double()
        f = C.c_double()
        self._check(self._L.uwgpu_profile_read_work(self._h, which, C.byref(b), C.byref(f)))
        return b.value, f.value

    def time_apply(self, precision=PREC_FP64, iterations=20):
        ms = C.c_double()
        self._check(self._L.uwgpu_time_apply(self._h, precision, iterations, C.byref(ms)))
        return ms.value

    def time_smooth(self, precision=PREC_FP64, sweeps=2, iterations=10):
        ms = C.c_double()
        self._check(self._L.uwgpu_time_smooth(self._h, precision, sweeps, iterations, C.byref(ms)))
        return ms.value

    def weights_set(self, kind=0, res=(10, 10, 10)):
        """WEIGHTS_CONSTANT (2^dim / count) or WEIGHTS_DVC (discrete Voronoi cells, res per axis)."""
        r = np.ascontiguousarray(list(res) + [1] * (3 - len(res)), dtype=np.int32)
        self._check(self._L.uwgpu_weights_set(self._h, kind, _ptr(r)))

    def integration_points(self):
        """(local coordinates [slot][3], weights [slot]) the last assembly integrated with."""
        n = self.npoints
        xi = np.zeros((n, 3))
        w = np.zeros(n)
        self._check(self._L.uwgpu_integration_points(self._h, _ptr(xi), _ptr(w)))
        return xi, w

    def bfbt_operator_apply(self, x, form=0):
        """y = G^T W G x, the scaled BFBt inner operator of the current fine operator (form 0: FP64
        stencil, 1: FP32 matrix-free, 2: FP32 stencil)"""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self._check(self._L.uwgpu_bfbt_operator_apply(self._h, form, _ptr(x), _ptr(y)))
        return y

    def time_bfbt_apply(self, form=1, iterations=20):
        ms = C.c_double()
        self._check(self._L.uwgpu_time_bfbt_apply(self._h, form, iterations, C.byref(ms)))
        return ms.value

    def time_chebyshev(self, precision=PREC_FP64, degree=2, iterations=10):
        ms = C.c_double()
        self._check(self._L.uwgpu_time_chebyshev(self._h, precision, degree, iterations, C.byref(ms)))
        return ms.value

    def tc_check(self, a, b, layout=0, fmt=1):
        """Tensor-core self-check: a (128, k) and b (n, k) arrays of 16-bit patterns (uint16: bfloat16
        bits for fmt 1, half bits for fmt 0) -> a @ b.T (128, n) FP32 from one tcgen05 MMA sequence."""
        a = np.ascontiguousarray(a, dtype=np.uint16)
        b = np.ascontiguousarray(b, dtype=np.uint16)
        assert a.shape[0] == 128 and a.shape[1] == b.shape[1]
        d = np.zeros((128, b.shape[0]), np.float32)
        self._check(self._L.uwgpu_tc_check(self._h, int(layout), int(fmt), b.shape[0], a.shape[1], _ptr(a), _ptr(b),
                                           _ptr(d)))
        return d

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._L.uwgpu_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def launch_count(self):
        return int(self._L.uwgpu_launch_count(self._h))

    # ---- learned velocity preconditioner ----
    def learned_create(self, levels=3, base=8, seed=1):
        self._check(self._L.uwgpu_learned_create(self._h, levels, base, seed))

    def learned_param_count(self):
        n = C.c_int64()
        self._check(self._L.uwgpu_learned_param_count(self._h, C.byref(n)))
        return n.value

    def learned_params(self):
        p = np.zeros(self.learned_param_count(), np.float32)
        self._check(self._L.uwgpu_learned_get_params(self._h, _ptr(p)))
        return p

    def learned_set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == self.learned_param_count()
        self._check(self._L.uwgpu_learned_set_params(self._h, _ptr(p)))

    def learned_forward(self, inp):
        """inp: (7, nn) float32 (residual, V-cycle answer, log10 viscosity) -> (3, nn) float32"""
        x = np.ascontiguousarray(inp, dtype=np.float32).reshape(7, self.nnodes)
        out = np.zeros((3, self.nnodes), np.float32)
        self._check(self._L.uwgpu_learned_forward(self._h, _ptr(x), _ptr(out)))
        return out

    def learned_generate(self, opts, nsamples=64, seed=1):
        """training pairs (residual, error left by one V-cycle) from the assembled system"""
        self._check(self._L.uwgpu_learned_generate(self._h, C.byref(opts), nsamples, seed))

    def learned_train(self, epochs=10, batch=4, lr=1e-3, seed=1):
        """Adam on the generated pairs -> (last-epoch relative loss, held-out error ratio)"""
        tl, hr = C.c_double(), C.c_double()
        self._check(self._L.uwgpu_learned_train(self._h, epochs, batch, lr, seed, C.byref(tl), C.byref(hr)))
        return tl.value, hr.value

    def learned_backward(self, grad_out):
        """after learned_forward: gradient of the output (3, nn) -> (parameter gradient, input gradient (7, nn))"""
        g = np.ascontiguousarray(grad_out, dtype=np.float32).reshape(3, self.nnodes)
        gp = np.zeros(self.learned_param_count(), np.float32)
        gi = np.zeros((7, self.nnodes), np.float32)
        self._check(self._L.uwgpu_learned_backward(self._h, _ptr(g), _ptr(gp), _ptr(gi)))
        return gp, gi


def free_slip_mask(dim, nel):
    """Free-slip walls: the normal velocity component is fixed on each wall (node-major dofs)."""
    nx, ny = nel[0] + 1, nel[1] + 1
    nz = nel[2] + 1 if dim == 3 else 1
    idx = np.arange(nx * ny * nz)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    fixed = np.zeros((nx * ny * nz, dim), np.uint8)
    fixed[(i == 0) | (i == nx - 1), 0] = 1
    fixed[(j == 0) | (j == ny - 1), 1] = 1
    if dim == 3:
        fixed[(k == 0) | (k == nz - 1), 2] = 1
    return fixed.reshape(-1)
