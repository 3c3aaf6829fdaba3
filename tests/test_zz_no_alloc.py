"""The allocation-free binning entry point (uwgpu_bin_and_map_noalloc), through the C ABI.

Callers that cannot allocate device memory while running (a host framework owning every device
buffer through its own pool, or code where an allocation would synchronise the device) pass
their own device buffers; the entry point keeps its scratch in a fixed device array.  This test
hands it buffers allocated by the test itself, calls it twice in a row with different meshes
and point sets (so stale scratch from the first call would show up in the second), and checks
every output against the context-based uwgpu_bin_and_map.  It also covers a shifted and scaled
domain, points outside the mesh, an empty point set, sizes beyond the scratch (including element
counts whose product overflows 64 bits), and that a call takes no device memory.  Kept in its own
file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

UWGPU_OK = 0
UWGPU_ERR_DOMAIN = 5
UWGPU_ERR_TOO_LARGE = 10


def _lib():
    from earthbyte_underworld_gb300 import uwgpu as U
    L = U.load()
    P = C.c_void_p
    L.uwgpu_bin_and_map_noalloc.argtypes = [C.c_int32, P, P, P, C.c_int64, P, P, P, P, P, P, P, P]
    L.uwgpu_bin_and_map_noalloc.restype = C.c_int
    return L


def _reference(w, mn=(0.0, 0.0, 0.0), mx=(1.0, 1.0, 1.0)):
    from earthbyte_underworld_gb300 import uwgpu as U
    with U.Context(0) as ctx:
        ctx.mesh_q1(w["dim"], w["nel"], mn, mx)
        ctx.particles_upload(w["x"], w["y"], w["z"])
        perm, offsets, xi = ctx.bin_and_map()
    return perm, offsets, xi


def _noalloc(L, w, mn=(0.0, 0.0, 0.0), mx=(1.0, 1.0, 1.0), expect=UWGPU_OK):
    torch = pytest.importorskip("torch")
    dim, nel = w["dim"], list(w["nel"]) + [1] * (3 - len(w["nel"]))
    n = w["x"].shape[0]
    ne = int(np.prod(w["nel"]))
    dev = torch.device("cuda", 0)
    x = torch.from_numpy(w["x"]).to(dev)
    y = torch.from_numpy(w["y"]).to(dev)
    z = torch.from_numpy(w["z"]).to(dev) if dim == 3 else None
    # outputs pre-filled with garbage so that unwritten entries would be caught
    perm = torch.full((max(n, 1),), 0x7FFFFFFF, dtype=torch.int32, device=dev)
    offsets = torch.full((ne + 1,), -1, dtype=torch.int32, device=dev)
    xi = torch.full((max(dim * n, 1),), float("nan"), dtype=torch.float64, device=dev)
    nel_a = (C.c_int32 * 3)(*nel)
    mn_a = (C.c_double * 3)(*mn)
    mx_a = (C.c_double * 3)(*mx)
    outside = C.c_uint32(123)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    rc = L.uwgpu_bin_and_map_noalloc(dim, nel_a, mn_a, mx_a, n, x.data_ptr() if n else None,
                                     y.data_ptr() if n else None, z.data_ptr() if (z is not None and n) else None,
                                     perm.data_ptr(), offsets.data_ptr(), xi.data_ptr(), stream, C.byref(outside))
    free1 = torch.cuda.mem_get_info(dev)[0]
    assert rc == expect, rc
    torch.cuda.synchronize()
    perm_h = perm.cpu().numpy().view(np.uint32)[:n]
    off_h = offsets.cpu().numpy().view(np.uint32)
    xi_h = xi.cpu().numpy()[:dim * n].reshape(dim, n).T
    return perm_h, off_h, xi_h, outside.value, free0 - free1


def _check_equal(L, w, mn=(0.0, 0.0, 0.0), mx=(1.0, 1.0, 1.0)):
    perm, offsets, xi, outside, _ = _noalloc(L, w, mn, mx)
    assert outside == 0
    rperm, roffsets, rxi = _reference(w, mn, mx)
    assert np.array_equal(offsets, roffsets)
    assert np.array_equal(perm, rperm)
    # same closed form as the context path: agreement to rounding (tolerance of the binning
    # parity tests)
    dim = w["dim"]
    assert np.max(np.abs(xi - rxi[:, :dim])) < 1e-13


def test_noalloc_matches_context_path_on_two_calls():
    from earthbyte_underworld_gb300 import workloads as W
    L = _lib()
    first = W.spheres(nel=(16, 12, 10), nspheres=8, seed=21)     # 3D, 51840 points
    second = W.rt2d(nel=(32, 24), ppc=20, seed=13)               # 2D, 15360 points
    for w in (first, second):
        _check_equal(L, w)


def test_noalloc_shifted_scaled_domain():
    """A mesh over [-2, 1] x [0.5, 1.25] x [3, 7] with points mapped into it."""
    from earthbyte_underworld_gb300 import workloads as W
    L = _lib()
    w = W.spheres(nel=(12, 10, 14), nspheres=6, seed=7)
    mn, mx = (-2.0, 0.5, 3.0), (1.0, 1.25, 7.0)
    w = dict(w)
    w["x"] = mn[0] + (mx[0] - mn[0]) * w["x"]
    w["y"] = mn[1] + (mx[1] - mn[1]) * w["y"]
    w["z"] = mn[2] + (mx[2] - mn[2]) * w["z"]
    _check_equal(L, w, mn, mx)


def test_noalloc_outside_points_and_empty_set():
    from earthbyte_underworld_gb300 import workloads as W
    L = _lib()
    w = dict(W.spheres(nel=(8, 8, 8), nspheres=4, seed=3))
    x = w["x"].copy()
    x[[5, 77, 1000]] = [1.5, -0.25, 2.0]
    w["x"] = x
    _, _, _, outside, _ = _noalloc(L, w, expect=UWGPU_ERR_DOMAIN)
    assert outside == 3
    empty = {"dim": 3, "nel": (6, 5, 4), "x": np.zeros(0), "y": np.zeros(0), "z": np.zeros(0)}
    _, offsets, _, outside, _ = _noalloc(L, empty)
    assert outside == 0
    assert offsets.shape == (6 * 5 * 4 + 1,) and not offsets.any()


def test_noalloc_takes_no_device_memory():
    """After a first call on the device, further calls change the device's free memory by nothing."""
    from earthbyte_underworld_gb300 import workloads as W
    L = _lib()
    w = W.spheres(nel=(16, 16, 16), nspheres=8, seed=5)
    _noalloc(L, w)
    for _ in range(2):
        *_, taken = _noalloc(L, w)
        assert taken == 0


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
    # element counts whose 64-bit product wraps to 0 or to a negative number are refused before
    # anything is launched
    for dims in ((1 << 21, 1 << 21, 1 << 22), ((1 << 31) - 1, (1 << 31) - 1, 4), (1 << 17, 2, 1)):
        rc = L.uwgpu_bin_and_map_noalloc(3, (C.c_int32 * 3)(*dims), mn, mx, 10, 8, 8, 8, 8, 8, 8, None, None)
        assert rc == UWGPU_ERR_TOO_LARGE, dims
