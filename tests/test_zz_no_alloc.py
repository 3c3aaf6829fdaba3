"""The allocation-free binning entry point (uwgpu_bin_and_map_noalloc), through the C ABI.

Callers that cannot allocate device memory while running (a host framework owning every device
buffer through its own pool, or code where an allocation would synchronise the device) pass
their own device buffers; the entry point keeps its scratch in a fixed device array.  This test
hands it buffers allocated by the test itself, calls it twice in a row with different meshes
and point sets (so stale scratch from the first call would show up in the second), and checks
every output against the context-based uwgpu_bin_and_map.  Kept in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

UWGPU_OK = 0
UWGPU_ERR_TOO_LARGE = 10


def _lib():
    from earthbyte_underworld_gb300 import uwgpu as U
    L = U.load()
    P = C.c_void_p
    L.uwgpu_bin_and_map_noalloc.argtypes = [C.c_int32, P, P, P, C.c_int64, P, P, P, P, P, P, P, P]
    L.uwgpu_bin_and_map_noalloc.restype = C.c_int
    return L


def _reference(w):
    from earthbyte_underworld_gb300 import uwgpu as U
    with U.Context(0) as ctx:
        ctx.mesh_q1(w["dim"], w["nel"])
        ctx.particles_upload(w["x"], w["y"], w["z"])
        perm, offsets, xi = ctx.bin_and_map()
    return perm, offsets, xi


def _noalloc(L, w):
    torch = pytest.importorskip("torch")
    dim, nel = w["dim"], list(w["nel"]) + [1] * (3 - len(w["nel"]))
    n = w["x"].shape[0]
    ne = int(np.prod(w["nel"]))
    dev = torch.device("cuda", 0)
    x = torch.from_numpy(w["x"]).to(dev)
    y = torch.from_numpy(w["y"]).to(dev)
    z = torch.from_numpy(w["z"]).to(dev) if dim == 3 else None
    # outputs pre-filled with garbage so that unwritten entries would be caught
    perm = torch.full((n,), 0x7FFFFFFF, dtype=torch.int32, device=dev)
    offsets = torch.full((ne + 1,), -1, dtype=torch.int32, device=dev)
    xi = torch.full((dim * n,), float("nan"), dtype=torch.float64, device=dev)
    nel_a = (C.c_int32 * 3)(*nel)
    mn = (C.c_double * 3)(0.0, 0.0, 0.0)
    mx = (C.c_double * 3)(1.0, 1.0, 1.0)
    outside = C.c_uint32(123)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = L.uwgpu_bin_and_map_noalloc(dim, nel_a, mn, mx, n, x.data_ptr(), y.data_ptr(),
                                     z.data_ptr() if z is not None else None, perm.data_ptr(), offsets.data_ptr(),
                                     xi.data_ptr(), stream, C.byref(outside))
    assert rc == UWGPU_OK, rc
    assert outside.value == 0
    torch.cuda.synchronize()
    perm_h = perm.cpu().numpy().view(np.uint32)
    off_h = offsets.cpu().numpy().view(np.uint32)
    xi_h = xi.cpu().numpy().reshape(dim, n).T
    return perm_h, off_h, xi_h


def test_noalloc_matches_context_path_on_two_calls():
    from earthbyte_underworld_gb300 import workloads as W
    L = _lib()
    first = W.spheres(nel=(16, 12, 10), nspheres=8, seed=21)     # 3D, 51840 points
    second = W.rt2d(nel=(32, 24), ppc=20, seed=13)               # 2D, 15360 points
    for w in (first, second):
        perm, offsets, xi = _noalloc(L, w)
        rperm, roffsets, rxi = _reference(w)
        assert np.array_equal(offsets, roffsets)
        assert np.array_equal(perm, rperm)
        dim = w["dim"]
        # same closed form as the context path: agreement to rounding (tolerance of the
        # binning parity tests)
        assert np.max(np.abs(xi - rxi[:, :dim])) < 1e-13


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = _lib()
    nel = (C.c_int32 * 3)(8, 8, 8)
    mn = (C.c_double * 3)(0.0, 0.0, 0.0)
    mx = (C.c_double * 3)(1.0, 1.0, 1.0)
    rc = L.uwgpu_bin_and_map_noalloc(3, nel, mn, mx, (1 << 20) + 1, 8, 8, 8, 8, 8, 8, None, None)
    assert rc == UWGPU_ERR_TOO_LARGE
    big = (C.c_int32 * 3)(64, 64, 64)
    rc = L.uwgpu_bin_and_map_noalloc(3, big, mn, mx, 10, 8, 8, 8, 8, 8, 8, None, None)
    assert rc == UWGPU_ERR_TOO_LARGE
