"""Learned velocity preconditioner: the U-Net kernels against the CPU torch reference.

The reference (oracle/unet_ref.py) is the same network in torch with BF16 storage emulated, so
forward outputs and autograd gradients are compared with the GPU's own forward and backward
kernels through the C ABI (uwgpu_learned_forward / uwgpu_learned_backward)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def test_reference_conv_layout_matches_direct_sum():
    """The reference's tap layout equals the direct restatement of one layer."""
    from oracle import unet_ref as R
    rng = np.random.default_rng(0)
    cin, cout = 8, 16
    inp = rng.standard_normal((5, 6, 7, cin))
    w = rng.standard_normal((27, cin, cout))
    b = rng.standard_normal(cout)
    wt = torch.tensor(w).permute(2, 1, 0).reshape(cout, cin, 3, 3, 3)
    got = torch.nn.functional.conv3d(torch.tensor(inp).permute(3, 0, 1, 2)[None], wt, torch.tensor(b),
                                     padding=1)[0].permute(1, 2, 3, 0).numpy()
    assert np.abs(got - R.conv3_naive(inp, w, b)).max() < 1e-12
    assert R.param_count(4, 16) == 1462643   # the 4-level 16/32/64/128 network: ~1.5M parameters


def _quantized_params(R, levels, base, rng):
    """Small multiples of powers of two: BF16-exact weights, and FP32 sums that stay exact in
    any summation order, so the GPU and the reference must agree to rounding of the gradients."""
    ch, shapes = R.layer_shapes(levels, base)
    parts = []
    for cin, cout in shapes:
        parts.append(rng.integers(-2, 3, 27 * cin * cout) / 32.0)
        parts.append(rng.integers(-2, 3, cout) / 8.0)
    parts.append(rng.integers(-4, 5, ch[0] * 3) / 16.0)
    parts.append(rng.integers(-2, 3, 3) / 8.0)
    return np.concatenate(parts).astype(np.float32)


def _gpu_pass(U, nel, levels, base, params, inp, gout):
    with U.Context(0) as ctx:
        ctx.mesh_q1(3, nel)
        ctx.learned_create(levels=levels, base=base, seed=3)
        p0 = ctx.learned_params()
        ctx.learned_set_params(params)
        out = ctx.learned_forward(inp)
        gp, gi = ctx.learned_backward(gout)
        return p0, out, gp, gi


@pytest.mark.gpu
@pytest.mark.parametrize("nel,levels,base", [((7, 7, 7), 3, 8), ((8, 6, 9), 3, 8), ((5, 5, 5), 2, 16)])
def test_unet_forward_backward_match_reference(uw, nel, levels, base):
    """GPU forward and backward (parameter and input gradients) of <output, g> against torch
    autograd on the BF16-emulating reference, on meshes with and without padding of the node grid.
    (a) quantized weights and data: the FP32 sums are exact, so agreement is to ~1e-6 and every
    layer's block of the gradient is checked; (b) random FP32 data: BF16 roundings of activations
    may flip with the summation order, so the tolerance is looser, and the GPU must still sit
    much closer to the BF16-emulating reference than the plain FP32 network does."""
    from oracle import unet_ref as R
    U = uw
    nodes = tuple(n + 1 for n in nel)
    nn = int(np.prod(nodes))
    rng = np.random.default_rng(11)
    # (a) quantized
    params = _quantized_params(R, levels, base, rng)
    inp = (rng.integers(-3, 4, (4, nn)) / 2.0).astype(np.float32)
    gout = (rng.integers(-3, 4, (3, nn)) / 4.0).astype(np.float32)
    p0, out, gp, gi = _gpu_pass(U, nel, levels, base, params, inp, gout)
    assert p0.size == R.param_count(levels, base)
    assert np.all(p0[-3 * base - 3:] == 0.0)   # the head starts at zero: no correction
    rout, rgp, rgi = R.value_and_grads(params, inp, gout, nodes, levels, base, emulate_bf16=True)
    assert _rel(out, rout) < 1e-5
    assert _rel(gi, rgi) < 1e-4
    ch, shapes = R.layer_shapes(levels, base)
    off = 0
    for cin, cout in shapes:
        n = 27 * cin * cout + cout
        assert _rel(gp[off:off + n], rgp[off:off + n]) < 1e-4, (cin, cout)
        off += n
    assert _rel(gp[off:], rgp[off:]) < 1e-4   # head
    # (b) random FP32 data, He-scaled weights
    params = p0.copy()
    params[-3 * base - 3:] = rng.standard_normal(3 * base + 3).astype(np.float32) * 0.3
    inp = rng.standard_normal((4, nn)).astype(np.float32)
    gout = rng.standard_normal((3, nn)).astype(np.float32)
    _, out, gp, gi = _gpu_pass(U, nel, levels, base, params, inp, gout)
    rout, rgp, rgi = R.value_and_grads(params, inp, gout, nodes, levels, base, emulate_bf16=True)
    fout, fgp, _ = R.value_and_grads(params, inp, gout, nodes, levels, base, emulate_bf16=False)
    assert _rel(out, rout) < 1.5e-2 and _rel(gp, rgp) < 3e-2 and _rel(gi, rgi) < 3e-2
    assert _rel(out, rout) < 0.5 * _rel(fout, rout)
