"""CPU reference of the learned velocity preconditioner's network (test infrastructure only).

The same U-Net as csrc/unet.cu, written with torch on the CPU so that autograd gives the
reference gradients: 3x3x3 convolutions with zero padding and ReLU (two per level), 2x2x2 average
pooling down, nearest upsampling + channel concatenation [up | skip] up, a 1x1x1 head to three
channels.  BF16 storage is emulated: weights of the 3x3x3 layers and every stored activation
(the input, each post-ReLU output, each pooled tensor) are rounded to bfloat16 (round to nearest
even) and back, the head weights stay FP32, and all arithmetic is FP32 (`emulate_bf16=False`
gives the plain FP32 network).  The rounding passes gradients through unchanged, which is what
the GPU backward does (it differentiates with the stored BF16 values).

Parameter layout (flat FP32 vector, as uwgpu_learned_get_params returns it): for every 3x3x3
layer W[27][cin][cout] then b[cout] -- encoder layers (level 0 first, two per level), then decoder
layers (level 0 first, two per level below the coarsest) -- then the head W[cin][3], b[3].
Tap t of W is the neighbour offset (t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) in (x, y, z).
"""
import numpy as np
import torch
import torch.nn.functional as F

IN_CHANNELS = 8


def layer_shapes(levels, base):
    ch = [base << l for l in range(levels)]
    cin = [IN_CHANNELS] + ch[:-1]
    shapes = []
    for l in range(levels):
        shapes.append((cin[l], ch[l]))
        shapes.append((ch[l], ch[l]))
    for l in range(levels - 1):
        shapes.append((ch[l + 1] + ch[l], ch[l]))
        shapes.append((ch[l], ch[l]))
    return ch, shapes


def param_count(levels, base):
    ch, shapes = layer_shapes(levels, base)
    return sum(27 * a * b + b for a, b in shapes) + ch[0] * 3 + 3


def padded(n, levels):
    m = 1 << (levels - 1)
    return (n + m - 1) // m * m


def _bf(x, on):
    """round the value to bfloat16; the gradient passes through in FP32 (a plain dtype cast would
    round the gradient to bfloat16 as well, which the GPU backward does not do)"""
    if not on:
        return x
    return x + (x.to(torch.bfloat16).to(torch.float32) - x).detach()


def forward_t(layers, hw, hb, inp, nodes, levels, emulate_bf16=True):
    """layers: [(conv3d weight [cout][cin][3][3][3], bias)], head (hw [cin][3], hb [3]);
    inp (7, nn) tensor (residual, V-cycle answer, log10 viscosity), node order x fastest;
    nodes = (nnx, nny, nnz) -> (3, nn)"""
    nnx, nny, nnz = nodes
    px, py, pz = (padded(n, levels) for n in nodes)
    bfon = emulate_bf16
    grid = inp.reshape(7, nnz, nny, nnx)
    x = torch.cat([F.pad(grid, (0, px - nnx, 0, py - nny, 0, pz - nnz)).unsqueeze(0),
                   torch.zeros(1, IN_CHANNELS - 7, pz, py, px)], dim=1)
    x = _bf(x, bfon)

    def conv(t, k):
        w, b = layers[k]
        return _bf(F.relu(F.conv3d(t, _bf(w, bfon), b, padding=1)), bfon)

    skips = []
    t = x
    for l in range(levels):
        t = conv(t, 2 * l)
        t = conv(t, 2 * l + 1)
        skips.append(t)
        if l + 1 < levels:
            t = _bf(F.avg_pool3d(t, 2), bfon)
    for l in range(levels - 2, -1, -1):
        up = F.interpolate(t, scale_factor=2, mode="nearest")
        t = torch.cat([up, skips[l]], dim=1)
        t = conv(t, 2 * levels + 2 * l)
        t = conv(t, 2 * levels + 2 * l + 1)
    out = torch.einsum("bczyx,cd->bdzyx", t, hw) + hb.reshape(1, 3, 1, 1, 1)
    return out[0, :, :nnz, :nny, :nnx].reshape(3, -1)


def value_and_grads(params, inp, grad_out, nodes, levels, base, emulate_bf16=True):
    """(output (3, nn), parameter gradient (flat), input gradient (7, nn)) of <output, grad_out>"""
    p = torch.tensor(np.asarray(params, dtype=np.float32), requires_grad=True)
    x = torch.tensor(np.asarray(inp, dtype=np.float32), requires_grad=True)
    ch, shapes = layer_shapes(levels, base)
    off = 0
    layers = []
    for cin, cout in shapes:
        w = p[off:off + 27 * cin * cout].reshape(27, cin, cout)
        off += 27 * cin * cout
        b = p[off:off + cout]
        off += cout
        # tap t -> (kz, ky, kx) = (t // 9, (t // 3) % 3, t % 3); conv3d is a correlation
        layers.append((w.permute(2, 1, 0).reshape(cout, cin, 3, 3, 3), b))
    hw = p[off:off + ch[0] * 3].reshape(ch[0], 3)
    off += ch[0] * 3
    hb = p[off:off + 3]
    out = forward_t(layers, hw, hb, x, nodes, levels, emulate_bf16)
    (out * torch.as_tensor(np.asarray(grad_out, dtype=np.float32))).sum().backward()
    return out.detach().numpy(), p.grad.numpy(), x.grad.numpy()


def conv3_naive(inp, w, b):
    """Direct restatement of one 3x3x3 layer on a channels-last grid: inp[z][y][x][ci],
    w[27][ci][co] -> out[z][y][x][co] = b[co] + sum_t sum_ci w[t][ci][co] inp[at offset t][ci]."""
    nz, ny, nx, cin = inp.shape
    out = np.tile(np.asarray(b, dtype=np.float64), (nz, ny, nx, 1))
    pad = np.zeros((nz + 2, ny + 2, nx + 2, cin))
    pad[1:-1, 1:-1, 1:-1] = inp
    for t in range(27):
        dx, dy, dz = t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1
        sl = pad[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
        out += sl @ w[t]
    return out
