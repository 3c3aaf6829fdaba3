"""The tcgen05 building blocks (csrc/tc.cuh) against a host product: D = A B^T from one tensor-core
MMA sequence, for the shared-memory operand layouts the library's tensor-core kernels use (both
operands K-major, both MN-major, A K-major with B MN-major), in BF16 and FP16 with FP32
accumulation.  The inputs are small integers times powers of two, so every product and sum is
exact in FP32 and the comparison is exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    return (np.asarray(x, np.float32).view(np.uint32) >> 16).astype(np.uint16)


def _f16_bits(x):
    return np.asarray(x, np.float16).view(np.uint16)


@pytest.mark.parametrize("layout", [0, 2, 4])
@pytest.mark.parametrize("fmt", [1, 0])
@pytest.mark.parametrize("n,k", [(64, 64), (16, 32), (128, 128), (256, 32)])
def test_tcgen05_product_exact(uw, layout, fmt, n, k):
    U = uw
    rng = np.random.default_rng(n * 1000 + k + layout)
    a = rng.integers(-8, 9, (128, k)).astype(np.float32) * 0.25
    b = rng.integers(-8, 9, (n, k)).astype(np.float32) * 0.5
    bits = _bf16_bits if fmt == 1 else _f16_bits
    with U.Context(0) as ctx:
        d = ctx.tc_check(bits(a), bits(b), layout=layout, fmt=fmt)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.array_equal(d.astype(np.float64), ref), np.abs(d - ref).max()
