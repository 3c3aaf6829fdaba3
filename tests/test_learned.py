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
    much closer to the BF16-emulating reference than the plain FP32 network does.  The convolutions
    run on the tensor core (tcgen05 implicit GEMM, BF16 operands, FP32 accumulation; FP32 gradients
    enter as hi + lo BF16 parts)."""
    from oracle import unet_ref as R
    U = uw
    nodes = tuple(n + 1 for n in nel)
    nn = int(np.prod(nodes))
    rng = np.random.default_rng(11)
    # (a) quantized
    params = _quantized_params(R, levels, base, rng)
    inp = (rng.integers(-3, 4, (7, nn)) / 2.0).astype(np.float32)
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
    inp = rng.standard_normal((7, nn)).astype(np.float32)
    gout = rng.standard_normal((3, nn)).astype(np.float32)
    _, out, gp, gi = _gpu_pass(U, nel, levels, base, params, inp, gout)
    rout, rgp, rgi = R.value_and_grads(params, inp, gout, nodes, levels, base, emulate_bf16=True)
    fout, fgp, _ = R.value_and_grads(params, inp, gout, nodes, levels, base, emulate_bf16=False)
    # BF16 roundings of activations flip with the tensor core's summation order; on these random
    # inputs the gradients then differ by a few percent from the emulating reference
    assert _rel(out, rout) < 1.5e-2 and _rel(gp, rgp) < 6e-2 and _rel(gi, rgi) < 6e-2
    assert _rel(out, rout) < 0.5 * _rel(fout, rout)


@pytest.mark.gpu
def test_learned_preconditioner_training_and_ablation(uw):
    """Train the U-Net on residual/error pairs of the multigrid solver (on the GPU, with its own
    kernels), then solve with and without it.  The gain on its task is asserted: on held-out pairs
    the network removes part of the error one V-cycle leaves (ratio < 1).  The solve with the
    learned correction reaches the same solution; the iteration counts of both are reported
    (flexible Krylov accepts any correction, and plain multigrid stays the fallback)."""
    from earthbyte_underworld_gb300 import workloads as W
    U = uw
    w = W.spheres(nel=(16, 16, 16), nspheres=20, seed=5)
    opts = U.default_opts(mg_levels=3, schur_type=1, schur_pc=3, scr_rtol=1e-6, a11_rtol=1e-6, back_rtol=1e-6,
                          max_outer=200, max_inner=2000, bfbt_rtol=1e-2, bfbt_max_it=2000, smoother=1,
                          smooth_down=2, smooth_up=2)
    with U.Context(0) as ctx:
        W.setup_context(ctx, w)
        ctx.bin_and_map(want=False)
        ctx.assemble()
        u0, p0, r0 = ctx.solve_bsscr(opts)
        ctx.learned_create(levels=3, base=8, seed=1)
        ctx.learned_generate(opts, nsamples=192, seed=5)
        loss, holdout = ctx.learned_train(epochs=60, batch=8, lr=1e-3, seed=2)
        opts.learned_pc = 1
        u1, p1, r1 = ctx.solve_bsscr(opts)
    print(f"\nU-Net: train loss {loss:.3f}, held-out error ratio {holdout:.3f}; "
          f"V-cycles plain {r0.vcycles}, learned {r1.vcycles} ({r1.learned_applies} corrections, "
          f"{r1.learned_fallbacks} fallbacks)")
    assert np.isfinite(loss) and holdout < 0.6   # deterministic training: 0.33 measured
    assert r1.rel_residual < 1e-5 and r1.learned_applies > 0
    assert _rel(u1, u0) < 1e-4 and _rel(p1, p0) < 1e-3


@pytest.mark.gpu
def test_learned_preconditioner_falls_back(uw):
    """A network that makes things worse (large random weights) must not break the solve: the
    stagnation test drops it and the plain V-cycle finishes the velocity solves."""
    from earthbyte_underworld_gb300 import workloads as W
    U = uw
    w = W.spheres(nel=(8, 8, 8), nspheres=8, seed=3)
    opts = U.default_opts(mg_levels=2, schur_type=1, schur_pc=0, scr_rtol=1e-6, a11_rtol=1e-7, back_rtol=1e-7,
                          max_outer=400, max_inner=2000)
    with U.Context(0) as ctx:
        W.setup_context(ctx, w)
        ctx.bin_and_map(want=False)
        ctx.assemble()
        u0, p0, r0 = ctx.solve_bsscr(opts)
        ctx.learned_create(levels=2, base=8, seed=4)
        rng = np.random.default_rng(0)
        ctx.learned_set_params(rng.standard_normal(ctx.learned_param_count()).astype(np.float32) * 3.0)
        opts.learned_pc = 1
        u1, p1, r1 = ctx.solve_bsscr(opts)
    assert r1.rel_residual < 1e-5
    assert _rel(u1, u0) < 1e-4
    assert r1.learned_applies > 0
