// Learned velocity preconditioner: a 3D U-Net on the nodal grid (BF16 weights and activations,
// FP32 accumulation and gradients), with its own forward, backward and Adam kernels.
//
// Input channels per node: the three components of the residual r and of the multigrid
// V-cycle's answer V(r) (each scaled to unit RMS), and log10 of the node-averaged viscosity;
// output: the correction to add to V(r), in units of RMS(V(r)).  The node
// grid (nel+1 per axis) is zero-padded to a multiple of 2^(levels-1).  Level l has base * 2^l
// channels; each level is two 3x3x3 convolutions with ReLU, levels are joined by 2x2x2 average
// pooling on the way down and nearest upsampling + concatenation with the skip on the way up, and
// a 1x1x1 convolution maps the finest decoder output to the three velocity components.
//
// Layout: channels-last (voxel-major, channel fastest) so that one 16-byte load brings eight BF16
// channels of a voxel.  Weights of a 3x3x3 layer are W[tap][cin][cout]; the data-gradient pass
// runs the forward kernel on W'[tap][cout][cin] = W[26 - tap][cin][cout].
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "tc.cuh"
#include "unet.cuh"

namespace uwg {
namespace unet {

typedef __nv_bfloat16 bf16;

// ------------------------------------------------------------------------------------------
// Kernels
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void load8(const bf16* p, float v[8]) {
    uint4 raw = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&raw);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float2 f = __bfloat1622float2(h[k]);
        v[2 * k] = f.x;
        v[2 * k + 1] = f.y;
    }
}
__device__ __forceinline__ void load8(const float* p, float v[8]) {
    float4 a = *reinterpret_cast<const float4*>(p);
    float4 b = *reinterpret_cast<const float4*>(p + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void store8(bf16* p, const float v[8]) {
    uint4 raw;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&raw);
#pragma unroll
    for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
    *reinterpret_cast<uint4*>(p) = raw;
}
__device__ __forceinline__ void store8(float* p, const float v[8]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    *reinterpret_cast<float4*>(p + 4) = make_float4(v[4], v[5], v[6], v[7]);
}

// ---- tensor-core (tcgen05) forms of the 3x3x3 convolution --------------------------------------
// FP32 values enter a BF16 product as two parts, hi = bf16(x) and lo = bf16(x - hi), whose sum
// carries about 16 significant bits (the split of Henry, Tang and Heinecke, "Leveraging the
// bfloat16 artificial intelligence datatype for higher-precision computations", ARITH 2019);
// both parts are multiplied on the tensor core and accumulated in FP32.
__device__ __forceinline__ void split8(const float* p, uint4& hi, uint4& lo) {
    float v[8];
    load8(p, v);
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&hi);
    __nv_bfloat162* l = reinterpret_cast<__nv_bfloat162*>(&lo);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
        const float2 af = __bfloat1622float2(a);
        h[k] = a;
        l[k] = __floats2bfloat162_rn(v[2 * k] - af.x, v[2 * k + 1] - af.y);
    }
}

constexpr int kTcSmemBudget = 200 * 1024;   // dynamic shared memory a tensor-core conv kernel may use

// Shared-memory plan of k_conv3_tc: B (the weights) for all 27 taps when they fit, else two tap
// buffers; A double-buffered per tap, with a second (lo) part for FP32 inputs.
struct ConvTcPlan {
    int Kp, Np;
    int resident;
    size_t bytesB, bytesA, smem;
};
__host__ __device__ inline ConvTcPlan conv_tc_plan(int K, int N, bool split) {
    ConvTcPlan p;
    p.Kp = (K + 15) / 16 * 16;
    p.Np = (N + 15) / 16 * 16;
    p.bytesB = (size_t)p.Np * p.Kp * 2;
    p.bytesA = (size_t)128 * p.Kp * 2;
    const size_t a_total = 2 * (split ? 2 : 1) * p.bytesA;
    p.resident = 27 * p.bytesB + a_total <= (size_t)kTcSmemBudget ? 1 : 0;
    p.smem = (p.resident ? 27 : 2) * p.bytesB + a_total;
    return p;
}

// 3x3x3 convolution as an implicit GEMM on the tensor core: for a tile of 128 consecutive voxels
// (rows, M = 128) and all N output channels, D = sum over the 27 taps t of A_t B_t^T, with
// A_t[m][k] = in[v_m + off(t)][k] (zero outside the grid) and B_t[n][k] = W_t[k][n], read from the
// layer's other packing Wrev[26 - t][n][k] (for the forward pass the flipped transpose, for the
// data gradient the plain weights).  Operands are K-major in shared memory; the accumulator
// (128 x N FP32) lives in TMEM; one thread issues the MMAs of a tap while all threads stage the
// next tap into the other buffer.  The epilogue adds the bias, applies ReLU and stores BF16 (or
// FP32) rows.  CTAs are persistent over the voxel tiles.  FP32 inputs (gradients) enter as
// hi + lo BF16 parts (two MMAs per K step).
template <typename TI, typename TO>
__global__ void __launch_bounds__(128, 1) k_conv3_tc(Vol g, int K, int N, ConvTcPlan P, const TI* __restrict__ in,
                                                     const bf16* __restrict__ Wrev, const float* __restrict__ bias,
                                                     TO* __restrict__ out, int relu, uint32_t* __restrict__ err) {
    constexpr bool kSplit = sizeof(TI) == 4;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int Kp = P.Kp, Np = P.Np, kc8 = Kp / 8;
    unsigned char* sB = smem;
    unsigned char* sA = smem + (P.resident ? 27 : 2) * P.bytesB;   // [buf][part] of bytesA each
    const uint32_t ncols = tc::tmem_cols(Np);
    if (warp == 0) {
        tc::tmem_alloc(&tbase, ncols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    // B of tap t into `dst` (K-major, zero beyond N and K)
    auto stage_b = [&](int t, unsigned char* dst) {
        const bf16* src = Wrev + (size_t)(26 - t) * N * K;
        for (int idx = tid; idx < Np * kc8; idx += 128) {
            const int n = idx % Np, c8 = idx / Np;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (n < N && c8 * 8 < K) v = __ldg(reinterpret_cast<const uint4*>(src + (size_t)n * K + c8 * 8));
            *reinterpret_cast<uint4*>(dst + tc::k_major_offset(n, c8 * 8, Kp)) = v;
        }
    };
    if (P.resident)
        for (int t = 0; t < 27; ++t) stage_b(t, sB + (size_t)t * P.bytesB);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_f16(128, Np, tc::kFmtBF16, 0, 0);
    uint32_t phase[2] = {0u, 0u}, pend[2] = {0u, 0u};
    bool ok = true;
    auto wait_buf = [&](int b) {
        if (pend[b]) {
            ok = tc::mbar_wait(&bar[b], phase[b]) && ok;
            phase[b] ^= 1u;
            pend[b] = 0u;
        }
    };
    const int64_t ntiles = (g.nv + 127) / 128;
    const int64_t pxy = (int64_t)g.px * g.py;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t v = tile * 128 + tid;   // this thread's row
        const bool vin = v < g.nv;
        const int x = (int)(v % g.px), y = (int)((v / g.px) % g.py), z = (int)(v / pxy);
        for (int t = 0; t < 27; ++t) {
            const int b = t & 1;
            wait_buf(b);
            unsigned char* a0 = sA + (size_t)b * (kSplit ? 2 : 1) * P.bytesA;
            const int xx = x + t % 3 - 1, yy = y + (t / 3) % 3 - 1, zz = z + t / 9 - 1;
            const bool nb = vin && xx >= 0 && xx < g.px && yy >= 0 && yy < g.py && zz >= 0 && zz < g.pz;
            const TI* row = in + ((int64_t)xx + (int64_t)g.px * (yy + (int64_t)g.py * zz)) * K;
            for (int c8 = 0; c8 < kc8; ++c8) {
                const uint32_t off = tc::k_major_offset(tid, c8 * 8, Kp);
                const bool live = nb && c8 * 8 < K;
                if (kSplit) {
                    uint4 hi = make_uint4(0, 0, 0, 0), lo = make_uint4(0, 0, 0, 0);
                    if (live) split8(reinterpret_cast<const float*>(row) + c8 * 8, hi, lo);
                    *reinterpret_cast<uint4*>(a0 + off) = hi;
                    *reinterpret_cast<uint4*>(a0 + P.bytesA + off) = lo;
                } else {
                    uint4 val = make_uint4(0, 0, 0, 0);
                    if (live) val = __ldg(reinterpret_cast<const uint4*>(reinterpret_cast<const bf16*>(row) + c8 * 8));
                    *reinterpret_cast<uint4*>(a0 + off) = val;
                }
            }
            unsigned char* bt = P.resident ? sB + (size_t)t * P.bytesB : sB + (size_t)b * P.bytesB;
            if (!P.resident) stage_b(t, bt);
            tc::fence_proxy_async();
            tc::fence_before_sync();
            ok = __syncthreads_and(ok) != 0;
            if (!ok) break;
            tc::fence_after_sync();
            if (tid == 0) {
                const uint32_t sa = tc::smem_u32(a0), sb = tc::smem_u32(bt);
                for (int s = 0; s < Kp / 16; ++s) {
                    const uint64_t db = tc::k_major_desc(sb, s, Kp);
                    tc::mma_f16(taddr, tc::k_major_desc(sa, s, Kp), db, idesc, (t > 0 || s > 0) ? 1u : 0u);
                    if (kSplit) tc::mma_f16(taddr, tc::k_major_desc(sa + (uint32_t)P.bytesA, s, Kp), db, idesc, 1u);
                }
                tc::mma_commit(&bar[b]);
            }
            pend[b] = 1u;
        }
        wait_buf(0);
        wait_buf(1);
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        tc::fence_after_sync();
        // epilogue: this thread's row, 16 columns at a time
        for (int c = 0; c < Np; c += 16) {
            uint32_t r[16];
            tc::tmem_ld16(tc::tmem_addr(taddr, 32 * warp, c), r);
            tc::tmem_wait_ld();
            if (!vin) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c0 = c + 8 * h;
                if (c0 >= N) break;
                float o[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    float val = __uint_as_float(r[8 * h + j]) + (bias ? bias[c0 + j] : 0.0f);
                    o[j] = relu ? fmaxf(val, 0.0f) : val;
                }
                store8(out + v * N + c0, o);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    if (!ok) {
        if (tid == 0) atomicOr(err, 1u);
        // give MMAs still in flight a bounded time to finish before the TMEM is released
        for (int b = 0; b < 2; ++b)
            if (pend[b]) tc::mbar_wait(&bar[b], phase[b], 1u << 16);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, ncols);
    }
}

// Weight gradient on the tensor core: part[slice][t][ci][co] = sum over the slice's voxels v of
// in[v + off(t)][ci] g[v][co].  Rows M are the (tap, input channel) pairs, 128 per CTA (grid.x);
// N the output channels; K the voxels, 64 per stage, double-buffered.  Both operands are
// MN-major in shared memory: a 16-byte chunk holds 8 consecutive channels of one voxel, as the
// channels-last tensors store them.  The FP32 gradient enters as hi + lo BF16 parts.  Each CTA
// (grid.y) owns a fixed voxel slice, and the slices are summed in a fixed order afterwards, so the
// gradient is deterministic.
constexpr int kWgK = 64;   // voxels per stage
__host__ __device__ inline size_t wgrad_tc_smem(int Np) {
    return 2 * ((size_t)128 * kWgK * 2 + 2 * (size_t)Np * kWgK * 2);
}
__global__ void __launch_bounds__(128, 1) k_conv3_wgrad_tc(Vol g, int cin, int cout, int Np, int64_t vslice,
                                                           const bf16* __restrict__ in, const float* __restrict__ gout,
                                                           float* __restrict__ part, uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int rows = 27 * cin;
    const int r0 = blockIdx.x * 128;
    const size_t bytesA = (size_t)128 * kWgK * 2, bytesB = (size_t)Np * kWgK * 2;
    const size_t stage_bytes = bytesA + 2 * bytesB;
    const uint32_t ncols = tc::tmem_cols(Np);
    if (warp == 0) {
        tc::tmem_alloc(&tbase, ncols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_f16(128, Np, tc::kFmtBF16, 1, 1);
    const int64_t v0 = (int64_t)blockIdx.y * vslice;
    const int64_t v1 = v0 + vslice < g.nv ? v0 + vslice : g.nv;
    const int64_t pxy = (int64_t)g.px * g.py;
    uint32_t phase[2] = {0u, 0u}, pend[2] = {0u, 0u};
    bool ok = true;
    int step = 0;
    for (int64_t vb = v0; vb < v1; vb += kWgK, ++step) {
        const int b = step & 1;
        if (pend[b]) {
            ok = tc::mbar_wait(&bar[b], phase[b]) && ok;
            phase[b] ^= 1u;
            pend[b] = 0u;
        }
        unsigned char* sa = smem + (size_t)b * stage_bytes;
        unsigned char* sbh = sa + bytesA;
        unsigned char* sbl = sbh + bytesB;
        // A: 16 row groups (8 channels of one tap) x 64 voxels
        for (int idx = tid; idx < 16 * kWgK; idx += 128) {
            const int k = idx % kWgK, mg = idx / kWgK;   // consecutive threads: consecutive voxels
            const int r = r0 + mg * 8;
            const int64_t v = vb + k;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (r < rows && v < v1) {
                const int t = r / cin, ci = r % cin;
                const int x = (int)(v % g.px) + t % 3 - 1, y = (int)((v / g.px) % g.py) + (t / 3) % 3 - 1,
                          z = (int)(v / pxy) + t / 9 - 1;
                if (x >= 0 && x < g.px && y >= 0 && y < g.py && z >= 0 && z < g.pz)
                    val = __ldg(reinterpret_cast<const uint4*>(in + ((int64_t)x + (int64_t)g.px * (y + (int64_t)g.py * z)) * cin + ci));
            }
            *reinterpret_cast<uint4*>(sa + tc::mn_major_offset(mg * 8, k, 128)) = val;
        }
        // B: Np / 8 groups of output channels x 64 voxels, hi and lo parts
        for (int idx = tid; idx < (Np / 8) * kWgK; idx += 128) {
            const int k = idx % kWgK, ng = idx / kWgK;
            const int64_t v = vb + k;
            uint4 hi = make_uint4(0, 0, 0, 0), lo = make_uint4(0, 0, 0, 0);
            if (ng * 8 < cout && v < v1) split8(gout + v * cout + ng * 8, hi, lo);
            const uint32_t off = tc::mn_major_offset(ng * 8, k, Np);
            *reinterpret_cast<uint4*>(sbh + off) = hi;
            *reinterpret_cast<uint4*>(sbl + off) = lo;
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t a = tc::smem_u32(sa), bh = tc::smem_u32(sbh), bl = tc::smem_u32(sbl);
            for (int s = 0; s < kWgK / 16; ++s) {
                const uint64_t da = tc::mn_major_desc(a, s, 128);
                tc::mma_f16(taddr, da, tc::mn_major_desc(bh, s, Np), idesc, (step > 0 || s > 0) ? 1u : 0u);
                tc::mma_f16(taddr, da, tc::mn_major_desc(bl, s, Np), idesc, 1u);
            }
            tc::mma_commit(&bar[b]);
        }
        pend[b] = 1u;
    }
    for (int b = 0; b < 2; ++b)
        if (pend[b]) {
            ok = tc::mbar_wait(&bar[b], phase[b]) && ok;
            phase[b] ^= 1u;
            pend[b] = 0u;
        }
    ok = __syncthreads_and(ok) != 0;
    tc::fence_after_sync();
    const int r = r0 + tid;
    float* dst = part + ((int64_t)blockIdx.y * rows + r) * cout;
    for (int c = 0; c < Np && ok; c += 16) {
        uint32_t v[16];
        tc::tmem_ld16(tc::tmem_addr(taddr, 32 * warp, c), v);
        tc::tmem_wait_ld();
        if (r >= rows) continue;
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (c + j < cout) dst[c + j] = step > 0 ? __uint_as_float(v[j]) : 0.0f;
    }
    if (!ok && tid == 0) atomicOr(err, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, ncols);
    }
}

// dst[i] += sum_s part[s][i], s ascending
__global__ void k_sum_slices(int64_t n, int slices, const float* __restrict__ part, float* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a = 0.0f;
    for (int sl = 0; sl < slices; ++sl) a += part[(int64_t)sl * n + i];
    dst[i] += a;
}

// part[block][co] = sum over the block's voxels of g[v][co] (thread t covers channel t % cout of
// voxels t / cout + k * lanes); the lanes are combined in shared memory in a fixed order
__global__ void k_bias_grad(int64_t nv, int cout, const float* __restrict__ gout, float* __restrict__ part) {
    __shared__ float sp[256];
    const int lanes = blockDim.x / cout;
    const int co = threadIdx.x % cout, sub = threadIdx.x / cout;
    float a = 0.0f;
    for (int64_t v = (int64_t)blockIdx.x * lanes + sub; v < nv; v += (int64_t)gridDim.x * lanes) a += gout[v * cout + co];
    sp[threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.x < cout) {
        float b = 0.0f;
        for (int l = 0; l < lanes; ++l) b += sp[l * cout + threadIdx.x];
        part[(int64_t)blockIdx.x * cout + threadIdx.x] = b;
    }
}

// g = g * (y > 0): gradient through ReLU, y the stored BF16 output of the layer
__global__ void k_relu_bwd(int64_t n, const bf16* __restrict__ y, float* __restrict__ g) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !(__bfloat162float(y[i]) > 0.0f)) g[i] = 0.0f;
}

// 2x2x2 average pooling (fine -> coarse), BF16
__global__ void k_pool(Vol f, Vol c, int ch, const bf16* __restrict__ in, bf16* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nv * ch) return;
    const int64_t V = i / ch;
    const int cc = (int)(i % ch);
    const int X = (int)(V % c.px), Y = (int)((V / c.px) % c.py), Z = (int)(V / ((int64_t)c.px * c.py));
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int x = 2 * X + (k & 1), y = 2 * Y + ((k >> 1) & 1), z = 2 * Z + (k >> 2);
        s += __bfloat162float(in[((int64_t)x + (int64_t)f.px * (y + (int64_t)f.py * z)) * ch + cc]);
    }
    out[i] = __float2bfloat16_rn(0.125f * s);
}

// gradient of the pooling, added: gf[v][c] += gc[parent(v)][c] / 8
__global__ void k_pool_bwd_add(Vol f, Vol c, int ch, const float* __restrict__ gc, float* __restrict__ gf) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.nv * ch) return;
    const int64_t v = i / ch;
    const int cc = (int)(i % ch);
    const int x = (int)(v % f.px), y = (int)((v / f.px) % f.py), z = (int)(v / ((int64_t)f.px * f.py));
    const int64_t V = (x / 2) + (int64_t)c.px * ((y / 2) + (int64_t)c.py * (z / 2));
    gf[i] += 0.125f * gc[V * ch + cc];
}

// decoder input: out[v] = [ up(coarse)[v] (cu channels) | skip[v] (cs channels) ]
__global__ void k_up_concat(Vol f, Vol c, int cu, int cs, const bf16* __restrict__ coarse,
                            const bf16* __restrict__ skip, bf16* __restrict__ out) {
    const int ct = cu + cs;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.nv * ct) return;
    const int64_t v = i / ct;
    const int cc = (int)(i % ct);
    if (cc < cu) {
        const int x = (int)(v % f.px), y = (int)((v / f.px) % f.py), z = (int)(v / ((int64_t)f.px * f.py));
        const int64_t V = (x / 2) + (int64_t)c.px * ((y / 2) + (int64_t)c.py * (z / 2));
        out[i] = coarse[V * cu + cc];
    } else {
        out[i] = skip[v * cs + (cc - cu)];
    }
}

// gradient of k_up_concat: gc[V][c] = sum over the 8 children of g[v][c] (c < cu);
// gskip[v][c] += g[v][cu + c]
__global__ void k_up_concat_bwd_coarse(Vol f, Vol c, int cu, int cs, const float* __restrict__ g,
                                       float* __restrict__ gc) {
    const int ct = cu + cs;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nv * cu) return;
    const int64_t V = i / cu;
    const int cc = (int)(i % cu);
    const int X = (int)(V % c.px), Y = (int)((V / c.px) % c.py), Z = (int)(V / ((int64_t)c.px * c.py));
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int x = 2 * X + (k & 1), y = 2 * Y + ((k >> 1) & 1), z = 2 * Z + (k >> 2);
        s += g[((int64_t)x + (int64_t)f.px * (y + (int64_t)f.py * z)) * ct + cc];
    }
    gc[i] = s;
}
__global__ void k_up_concat_bwd_skip(Vol f, int cu, int cs, const float* __restrict__ g, float* __restrict__ gs) {
    const int ct = cu + cs;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.nv * cs) return;
    const int64_t v = i / cs;
    const int cc = (int)(i % cs);
    gs[i] += g[v * ct + cu + cc];
}

// head: out[d][v] = b[d] + sum_c W[c][d] x[v][c]   (d < 3, out SoA FP32)
__global__ void k_head(int64_t nv, int cin, const bf16* __restrict__ x, const float* __restrict__ W,
                       const float* __restrict__ b, float* __restrict__ out) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    float a0 = b[0], a1 = b[1], a2 = b[2];
    for (int c8 = 0; c8 < cin; c8 += 8) {
        float xv[8];
        load8(x + v * cin + c8, xv);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float* w = W + (c8 + c) * 3;
            a0 = fmaf(xv[c], w[0], a0);
            a1 = fmaf(xv[c], w[1], a1);
            a2 = fmaf(xv[c], w[2], a2);
        }
    }
    out[v] = a0;
    out[nv + v] = a1;
    out[2 * nv + v] = a2;
}

// head backward: gx[v][c] = sum_d W[c][d] g[d][v]; dW[c][d] += sum_v x[v][c] g[d][v]; db[d] += sum_v g[d][v]
// (warp sums first, then one shared-memory add per warp, then one global add per block)
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// part[block][0 .. 3 cin) = block sums of x[v][c] g[d][v], part[block][3 cin .. 3 cin + 3) = of g[d][v]
// (warp sums, then the warps in a fixed order); gx[v][c] = sum_d W[c][d] g[d][v]
__global__ void k_head_bwd(int64_t nv, int cin, const bf16* __restrict__ x, const float* __restrict__ W,
                           const float* __restrict__ g, float* __restrict__ gx, float* __restrict__ part) {
    extern __shared__ float swarp[];   // [warps][cin * 3 + 3]
    const int nq = cin * 3 + 3, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = v < nv;
    const float g0 = act ? g[v] : 0.0f, g1 = act ? g[nv + v] : 0.0f, g2 = act ? g[2 * nv + v] : 0.0f;
    const bool lead = (threadIdx.x & 31) == 0;
    for (int c = 0; c < cin; ++c) {
        const float* w = W + c * 3;
        const float xv = act ? __bfloat162float(x[v * cin + c]) : 0.0f;
        if (act) gx[v * cin + c] = w[0] * g0 + w[1] * g1 + w[2] * g2;
        const float s0 = warp_sum(xv * g0), s1 = warp_sum(xv * g1), s2 = warp_sum(xv * g2);
        if (lead) {
            swarp[warp * nq + c * 3 + 0] = s0;
            swarp[warp * nq + c * 3 + 1] = s1;
            swarp[warp * nq + c * 3 + 2] = s2;
        }
    }
    const float t0 = warp_sum(g0), t1 = warp_sum(g1), t2 = warp_sum(g2);
    if (lead) {
        swarp[warp * nq + cin * 3 + 0] = t0;
        swarp[warp * nq + cin * 3 + 1] = t1;
        swarp[warp * nq + cin * 3 + 2] = t2;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nq; k += blockDim.x) {
        float a = 0.0f;
        for (int w = 0; w < nw; ++w) a += swarp[w * nq + k];
        part[(int64_t)blockIdx.x * nq + k] = a;
    }
}

// FP32 master weights -> BF16 W[t][ci][co] and the flipped transpose W'[t][co][ci] = W[26-t][ci][co]
__global__ void k_pack(int taps, int cin, int cout, const float* __restrict__ w, bf16* __restrict__ w16,
                       bf16* __restrict__ wflip) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)taps * cin * cout;
    if (i >= n) return;
    const int t = (int)(i / ((int64_t)cin * cout));
    const int rem = (int)(i % ((int64_t)cin * cout));
    const int ci = rem / cout, co = rem % cout;
    const bf16 b = __float2bfloat16_rn(w[i]);
    w16[i] = b;
    if (wflip) wflip[((int64_t)(taps - 1 - t) * cout + co) * cin + ci] = b;
}

// Adam (Kingma & Ba 2015) with bias correction; bc1 = 1 - beta1^t, bc2 = 1 - beta2^t
__global__ void k_adam(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                       float gscale) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * gscale;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------
static unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

static int sm_count(Context& c) {
    int n = 0;
    UWG_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, c.device));
    return n > 0 ? n : 1;
}

void check_errors(Context& c, Net& n) {
    if (!n.tc_err.p) return;
    uint32_t e = 0;
    UWG_CUDA(cudaMemcpyAsync(&e, n.tc_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    if (e) {
        UWG_CUDA(cudaMemsetAsync(n.tc_err.p, 0, sizeof(uint32_t), c.stream));
        throw Error(UWGPU_ERR_CUDA, "U-Net tensor-core kernel: an MMA did not complete in time");
    }
}

// 3x3x3 convolution on the tensor core (k_conv3_tc).  W: the layer's weights as the convolution
// reads them ([27][K][N]); Wrev: the layer's other packing ([27][N][K] in reverse tap order).
template <typename TI, typename TO>
static void conv_launch_tc(Context& c, Net& n, const Vol& g, int K, int N, const TI* in, const bf16* Wrev,
                           const float* bias, TO* out, bool relu) {
    const ConvTcPlan P = conv_tc_plan(K, N, sizeof(TI) == 4);
    UWG_REQUIRE(P.Np <= 256, UWGPU_ERR_ARGUMENT, "U-Net layer too wide for the tensor-core convolution");
    int per_sm = 1;
    const size_t smem =
        tmem_safe_smem((const void*)k_conv3_tc<TI, TO>, c.device, P.smem, tc::tmem_cols(P.Np), &per_sm);
    const int64_t ntiles = (g.nv + 127) / 128;
    const int64_t cap = (int64_t)sm_count(c) * per_sm;
    const unsigned grid = (unsigned)(ntiles < cap ? ntiles : cap);
    LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
    k_conv3_tc<TI, TO><<<grid, 128, smem, c.stream>>>(g, K, N, P, in, Wrev, bias, out, relu ? 1 : 0, n.tc_err.p);
    note_work(c, UWGPU_KERNEL_LEARNED, (double)g.nv * (K * sizeof(TI) + N * sizeof(TO)),
              2.0 * 27.0 * K * N * (double)g.nv * (sizeof(TI) == 4 ? 2.0 : 1.0));
}

static void wgrad_launch_tc(Context& c, Net& n, const Vol& g, int cin, int cout, const bf16* in, const float* gout,
                            float* dW, DArray<float>& part) {
    const int Np = (cout + 15) / 16 * 16;
    UWG_REQUIRE(Np <= 256, UWGPU_ERR_ARGUMENT, "U-Net layer too wide for the tensor-core weight gradient");
    int per_sm = 1;
    const size_t smem =
        tmem_safe_smem((const void*)k_conv3_wgrad_tc, c.device, wgrad_tc_smem(Np), tc::tmem_cols(Np), &per_sm);
    const int rows = 27 * cin;
    const int mtiles = (rows + 127) / 128;
    int64_t slices = (2LL * sm_count(c) + mtiles - 1) / mtiles;
    const int64_t max_slices = (g.nv + 511) / 512;
    if (slices > max_slices) slices = max_slices;
    if (slices < 1) slices = 1;
    int64_t vslice = (g.nv + slices - 1) / slices;
    vslice = (vslice + kWgK - 1) / kWgK * kWgK;
    slices = (g.nv + vslice - 1) / vslice;
    const int64_t nw = (int64_t)rows * cout;
    part.ensure((size_t)slices * nw);
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_conv3_wgrad_tc<<<dim3(mtiles, (unsigned)slices), 128, smem, c.stream>>>(g, cin, cout, Np, vslice, in, gout,
                                                                                 part.p, n.tc_err.p);
    }
    LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
    k_sum_slices<<<nblk(nw, 256), 256, 0, c.stream>>>(nw, (int)slices, part.p, dW);
    note_work(c, UWGPU_KERNEL_LEARNED, (double)g.nv * 27.0 * (cin * 2 + cout * 4), 4.0 * 27.0 * cin * cout * (double)g.nv);
}

static void bias_grad_launch(Context& c, int64_t nv, int cout, const float* gout, float* db, DArray<float>& part) {
    const int blocks = 152;
    part.ensure((size_t)blocks * cout);
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_bias_grad<<<blocks, (256 / cout) * cout, 0, c.stream>>>(nv, cout, gout, part.p);
    }
    LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
    k_sum_slices<<<nblk(cout, 256), 256, 0, c.stream>>>(cout, blocks, part.p, db);
}

static void relu_bwd(Context& c, int64_t n, const bf16* y, float* g) {
    LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
    k_relu_bwd<<<nblk(n, 256), 256, 0, c.stream>>>(n, y, g);
}

// splitmix64 (Steele, Lea and Flood 2014) for reproducible initial weights
static uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void destroy(Net* n) { delete n; }

void create(Context& c, Net& n, int levels, int base, uint64_t seed) {
    const MeshDesc& m = c.mesh;
    UWG_REQUIRE(m.dim == 3, UWGPU_ERR_UNSUPPORTED, "the learned preconditioner is built for 3D meshes");
    UWG_REQUIRE(levels >= 1 && levels <= kMaxLevels, UWGPU_ERR_ARGUMENT, "U-Net levels must be 1..6");
    UWG_REQUIRE(base >= 8 && base % 8 == 0 && (base << (levels - 1)) <= 256, UWGPU_ERR_ARGUMENT,
                "U-Net base channels must be a multiple of 8, at most 256 at the coarsest level");
    n.levels = levels;
    n.base = base;
    n.nnx = m.nnx;
    n.nny = m.nny;
    n.nnz = m.nnz;
    n.nn = m.nn;
    const int64_t mult = (int64_t)1 << (levels - 1);
    Vol v0;
    v0.px = (int)((m.nnx + mult - 1) / mult * mult);
    v0.py = (int)((m.nny + mult - 1) / mult * mult);
    v0.pz = (int)((m.nnz + mult - 1) / mult * mult);
    for (int l = 0; l < levels; ++l) {
        Vol v;
        v.px = v0.px >> l;
        v.py = v0.py >> l;
        v.pz = v0.pz >> l;
        v.nv = (int64_t)v.px * v.py * v.pz;
        n.vol[l] = v;
        n.ch[l] = base << l;
    }
    // layers and parameter offsets
    {
        std::vector<Conv> fresh((size_t)(2 * levels + 2 * (levels - 1)));   // Conv owns device arrays: no copies
        n.convs.swap(fresh);
    }
    int64_t off = 0;
    auto add = [&](Conv& cv, int cin, int cout) {
        cv.cin = cin;
        cv.cout = cout;
        cv.w_off = off;
        off += (int64_t)27 * cin * cout;
        cv.b_off = off;
        off += cout;
    };
    for (int l = 0; l < levels; ++l) {
        add(n.convs[n.enc(l, 0)], n.cin_of_level(l), n.ch[l]);
        add(n.convs[n.enc(l, 1)], n.ch[l], n.ch[l]);
    }
    for (int l = 0; l + 1 < levels; ++l) {
        add(n.convs[n.dec(l, 0)], n.ch[l + 1] + n.ch[l], n.ch[l]);
        add(n.convs[n.dec(l, 1)], n.ch[l], n.ch[l]);
    }
    n.head_w = off;
    off += (int64_t)n.ch[0] * 3;
    n.head_b = off;
    off += 3;
    n.nparams = off;
    // He-uniform initial weights, zero biases, zero head (the untrained net adds nothing)
    std::vector<float> h((size_t)n.nparams, 0.0f);
    uint64_t s = seed;
    for (auto& cv : n.convs) {
        const float a = std::sqrt(6.0f / (27.0f * cv.cin));
        for (int64_t i = 0; i < (int64_t)27 * cv.cin * cv.cout; ++i) {
            const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
            h[(size_t)(cv.w_off + i)] = (float)((2.0 * u - 1.0) * a);
        }
    }
    for (auto* a : {&n.params, &n.grads, &n.adam_m, &n.adam_v}) a->ensure((size_t)n.nparams);
    UWG_CUDA(cudaMemcpy(n.params.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    UWG_CUDA(cudaMemset(n.grads.p, 0, h.size() * sizeof(float)));
    UWG_CUDA(cudaMemset(n.adam_m.p, 0, h.size() * sizeof(float)));
    UWG_CUDA(cudaMemset(n.adam_v.p, 0, h.size() * sizeof(float)));
    n.adam_t = 0;
    n.out_scale = 1.0f;
    // activations and gradients
    const Vol& f = n.vol[0];
    n.x0.ensure((size_t)f.nv * kInChannels);
    UWG_CUDA(cudaMemset(n.x0.p, 0, (size_t)f.nv * kInChannels * sizeof(bf16)));
    n.out.ensure((size_t)f.nv * 3);
    n.gout.ensure((size_t)f.nv * 3);
    for (int l = 0; l < levels; ++l) {
        const int64_t nv = n.vol[l].nv;
        const int C = n.ch[l];
        n.enc_a[l].ensure((size_t)nv * C);
        n.enc_b[l].ensure((size_t)nv * C);
        n.g_enc_a[l].ensure((size_t)nv * C);
        n.g_enc_b[l].ensure((size_t)nv * C);
        n.g_in[l].ensure((size_t)nv * n.cin_of_level(l));
        if (l + 1 < levels) {
            n.pool[l].ensure((size_t)n.vol[l + 1].nv * C);
            const int ct = n.ch[l + 1] + C;
            n.dec_cat[l].ensure((size_t)nv * ct);
            n.dec_a[l].ensure((size_t)nv * C);
            n.dec_b[l].ensure((size_t)nv * C);
            n.g_cat[l].ensure((size_t)nv * ct);
            n.g_dec_a[l].ensure((size_t)nv * C);
            n.g_dec_b[l].ensure((size_t)nv * C);
        }
    }
    for (auto& cv : n.convs) {
        cv.w16.ensure((size_t)27 * cv.cin * cv.cout);
        cv.wflip.ensure((size_t)27 * cv.cin * cv.cout);
    }
    n.tc_err.ensure(1);
    UWG_CUDA(cudaMemset(n.tc_err.p, 0, sizeof(uint32_t)));
    pack(c, n);
}

void pack(Context& c, Net& n) {
    for (auto& cv : n.convs) {
        const int64_t nw = (int64_t)27 * cv.cin * cv.cout;
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_pack<<<nblk(nw, 256), 256, 0, c.stream>>>(27, cv.cin, cv.cout, n.params.p + cv.w_off, cv.w16.p, cv.wflip.p);
    }
    check_launch("k_pack");
}

void forward(Context& c, Net& n) {
    const int L = n.levels;
    for (int l = 0; l < L; ++l) {
        const Vol& g = n.vol[l];
        const Conv& a = n.convs[n.enc(l, 0)];
        const Conv& b = n.convs[n.enc(l, 1)];
        const bf16* in = l == 0 ? n.x0.p : n.pool[l - 1].p;
        conv_launch_tc<bf16, bf16>(c, n, g, a.cin, a.cout, in, a.wflip.p, n.params.p + a.b_off, n.enc_a[l].p, true);
        conv_launch_tc<bf16, bf16>(c, n, g, b.cin, b.cout, n.enc_a[l].p, b.wflip.p, n.params.p + b.b_off, n.enc_b[l].p,
                                   true);
        if (l + 1 < L) {
            const int64_t cnt = n.vol[l + 1].nv * n.ch[l];
            LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
            k_pool<<<nblk(cnt, 256), 256, 0, c.stream>>>(g, n.vol[l + 1], n.ch[l], n.enc_b[l].p, n.pool[l].p);
        }
    }
    for (int l = L - 2; l >= 0; --l) {
        const Vol& g = n.vol[l];
        const int cu = n.ch[l + 1], cs = n.ch[l];
        const bf16* coarse = l == L - 2 ? n.enc_b[L - 1].p : n.dec_b[l + 1].p;
        {
            const int64_t cnt = g.nv * (cu + cs);
            LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
            k_up_concat<<<nblk(cnt, 256), 256, 0, c.stream>>>(g, n.vol[l + 1], cu, cs, coarse, n.enc_b[l].p,
                                                              n.dec_cat[l].p);
        }
        const Conv& a = n.convs[n.dec(l, 0)];
        const Conv& b = n.convs[n.dec(l, 1)];
        conv_launch_tc<bf16, bf16>(c, n, g, a.cin, a.cout, n.dec_cat[l].p, a.wflip.p, n.params.p + a.b_off, n.dec_a[l].p,
                                   true);
        conv_launch_tc<bf16, bf16>(c, n, g, b.cin, b.cout, n.dec_a[l].p, b.wflip.p, n.params.p + b.b_off, n.dec_b[l].p,
                                   true);
    }
    const bf16* fin = L == 1 ? n.enc_b[0].p : n.dec_b[0].p;
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_head<<<nblk(n.vol[0].nv, 256), 256, 0, c.stream>>>(n.vol[0].nv, n.ch[0], fin, n.params.p + n.head_w,
                                                              n.params.p + n.head_b, n.out.p);
    }
    check_launch("unet forward");
}

// gradient of one conv layer: g (pre-activation gradient, FP32, [nv][cout]) -> dW, db, and the
// gradient of its input (post-activation of the layer below) into gin
static void conv_backward(Context& c, Net& n, const Vol& g, const Conv& cv, const bf16* in, const float* gpre,
                          float* gin) {
    wgrad_launch_tc(c, n, g, cv.cin, cv.cout, in, gpre, n.grads.p + cv.w_off, n.part);
    bias_grad_launch(c, g.nv, cv.cout, gpre, n.grads.p + cv.b_off, n.part);
    // the data gradient is the convolution with W'[t][co][ci] = W[26 - t][ci][co]; its other
    // packing, read in reverse tap order, is the plain W
    conv_launch_tc<float, float>(c, n, g, cv.cout, cv.cin, gpre, cv.w16.p, nullptr, gin, false);
}

void backward(Context& c, Net& n) {
    const int L = n.levels;
    const Vol& f = n.vol[0];
    const bf16* fin = L == 1 ? n.enc_b[0].p : n.dec_b[0].p;
    float* gfin = L == 1 ? n.g_enc_b[0].p : n.g_dec_b[0].p;
    {
        const int nq = n.ch[0] * 3 + 3;
        const unsigned hb = nblk(f.nv, 256);
        n.part.ensure((size_t)hb * nq);
        {
            LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
            k_head_bwd<<<hb, 256, (size_t)8 * nq * sizeof(float), c.stream>>>(f.nv, n.ch[0], fin, n.params.p + n.head_w,
                                                                              n.gout.p, gfin, n.part.p);
        }
        // head_w and head_b are adjacent in the parameter vector: one ordered sum for both
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_sum_slices<<<nblk(nq, 256), 256, 0, c.stream>>>(nq, (int)hb, n.part.p, n.grads.p + n.head_w);
    }
    // skip gradients start at zero; the decoder adds into them
    for (int l = 0; l + 1 < L; ++l)
        UWG_CUDA(cudaMemsetAsync(n.g_enc_b[l].p, 0, (size_t)n.vol[l].nv * n.ch[l] * sizeof(float), c.stream));
    for (int l = 0; l + 1 < L; ++l) {
        const Vol& g = n.vol[l];
        const int cu = n.ch[l + 1], cs = n.ch[l];
        relu_bwd(c, g.nv * cs, n.dec_b[l].p, n.g_dec_b[l].p);
        conv_backward(c, n, g, n.convs[n.dec(l, 1)], n.dec_a[l].p, n.g_dec_b[l].p, n.g_dec_a[l].p);
        relu_bwd(c, g.nv * cs, n.dec_a[l].p, n.g_dec_a[l].p);
        conv_backward(c, n, g, n.convs[n.dec(l, 0)], n.dec_cat[l].p, n.g_dec_a[l].p, n.g_cat[l].p);
        float* gcoarse = l + 1 == L - 1 ? n.g_enc_b[L - 1].p : n.g_dec_b[l + 1].p;
        {
            LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
            k_up_concat_bwd_coarse<<<nblk(n.vol[l + 1].nv * cu, 256), 256, 0, c.stream>>>(g, n.vol[l + 1], cu, cs,
                                                                                           n.g_cat[l].p, gcoarse);
        }
        {
            LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
            k_up_concat_bwd_skip<<<nblk(g.nv * cs, 256), 256, 0, c.stream>>>(g, cu, cs, n.g_cat[l].p, n.g_enc_b[l].p);
        }
    }
    for (int l = L - 1; l >= 0; --l) {
        const Vol& g = n.vol[l];
        const int C = n.ch[l];
        if (l + 1 < L) {
            LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
            k_pool_bwd_add<<<nblk(g.nv * C, 256), 256, 0, c.stream>>>(g, n.vol[l + 1], C, n.g_in[l + 1].p,
                                                                      n.g_enc_b[l].p);
        }
        relu_bwd(c, g.nv * C, n.enc_b[l].p, n.g_enc_b[l].p);
        conv_backward(c, n, g, n.convs[n.enc(l, 1)], n.enc_a[l].p, n.g_enc_b[l].p, n.g_enc_a[l].p);
        relu_bwd(c, g.nv * C, n.enc_a[l].p, n.g_enc_a[l].p);
        const bf16* in = l == 0 ? n.x0.p : n.pool[l - 1].p;
        conv_backward(c, n, g, n.convs[n.enc(l, 0)], in, n.g_enc_a[l].p, n.g_in[l].p);
    }
    check_launch("unet backward");
}

// node (i, j, k) of the mesh sits at voxel (i, j, k) of the padded level-0 grid
__global__ void k_input_from_host_layout(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ in4,
                                         bf16* __restrict__ x0) {
    int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t i = node % nnx, j = (node / nnx) % nny, k = node / (nnx * nny);
    const int64_t v = i + (int64_t)g.px * (j + (int64_t)g.py * k);
#pragma unroll
    for (int ch = 0; ch < kUsedChannels; ++ch) x0[v * kInChannels + ch] = __float2bfloat16_rn(in4[(int64_t)ch * nn + node]);
}

__global__ void k_output_to_node_layout(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ out,
                                        float* __restrict__ o3) {
    int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t i = node % nnx, j = (node / nnx) % nny, k = node / (nnx * nny);
    const int64_t v = i + (int64_t)g.px * (j + (int64_t)g.py * k);
#pragma unroll
    for (int d = 0; d < 3; ++d) o3[(int64_t)d * nn + node] = out[(int64_t)d * g.nv + v];
}

void set_input_host(Context& c, Net& n, const float* input) {
    DArray<float> tmp;
    tmp.ensure((size_t)n.nn * kUsedChannels);
    UWG_CUDA(cudaMemcpyAsync(tmp.p, input, (size_t)n.nn * kUsedChannels * sizeof(float), cudaMemcpyHostToDevice,
                             c.stream));
    UWG_CUDA(cudaMemsetAsync(n.x0.p, 0, (size_t)n.vol[0].nv * kInChannels * sizeof(bf16), c.stream));
    LaunchScope ls(c, -1);
    k_input_from_host_layout<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], tmp.p, n.x0.p);
    UWG_CUDA(cudaStreamSynchronize(c.stream));
}

void get_output_host(Context& c, Net& n, float* output) {
    check_errors(c, n);
    DArray<float> tmp;
    tmp.ensure((size_t)n.nn * 3);
    {
        LaunchScope ls(c, -1);
        k_output_to_node_layout<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], n.out.p, tmp.p);
    }
    UWG_CUDA(cudaMemcpyAsync(output, tmp.p, (size_t)n.nn * 3 * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
}

__global__ void k_grad_from_node_layout(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ g3,
                                        float* __restrict__ gout) {
    int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t i = node % nnx, j = (node / nnx) % nny, k = node / (nnx * nny);
    const int64_t v = i + (int64_t)g.px * (j + (int64_t)g.py * k);
#pragma unroll
    for (int d = 0; d < 3; ++d) gout[(int64_t)d * g.nv + v] = g3[(int64_t)d * nn + node];
}

__global__ void k_input_grad_to_node_layout(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ gin,
                                            float* __restrict__ g4) {
    int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t i = node % nnx, j = (node / nnx) % nny, k = node / (nnx * nny);
    const int64_t v = i + (int64_t)g.px * (j + (int64_t)g.py * k);
#pragma unroll
    for (int ch = 0; ch < kUsedChannels; ++ch) g4[(int64_t)ch * nn + node] = gin[v * kInChannels + ch];
}

void set_grad_output_host(Context& c, Net& n, const float* grad) {
    DArray<float> tmp;
    tmp.ensure((size_t)n.nn * 3);
    UWG_CUDA(cudaMemcpyAsync(tmp.p, grad, (size_t)n.nn * 3 * sizeof(float), cudaMemcpyHostToDevice, c.stream));
    UWG_CUDA(cudaMemsetAsync(n.gout.p, 0, (size_t)n.vol[0].nv * 3 * sizeof(float), c.stream));
    LaunchScope ls(c, -1);
    k_grad_from_node_layout<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], tmp.p, n.gout.p);
    UWG_CUDA(cudaStreamSynchronize(c.stream));
}

void get_input_grad_host(Context& c, Net& n, float* grad_input) {
    check_errors(c, n);
    DArray<float> tmp;
    tmp.ensure((size_t)n.nn * kUsedChannels);
    {
        LaunchScope ls(c, -1);
        k_input_grad_to_node_layout<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], n.g_in[0].p,
                                                                            tmp.p);
    }
    UWG_CUDA(cudaMemcpyAsync(grad_input, tmp.p, (size_t)n.nn * kUsedChannels * sizeof(float), cudaMemcpyDeviceToHost,
                             c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
}

// ------------------------------------------------------------------------------------------
// The network as a preconditioner: residual -> input tensor, output -> velocity correction
// ------------------------------------------------------------------------------------------
// out[0] += sum x^2, in a fixed order: launched as one block of 1024 threads (deterministic)
template <typename T>
__global__ void __launch_bounds__(1024) k_sumsq(int64_t n, const T* __restrict__ x, double* __restrict__ out) {
    __shared__ double sw[32];
    float sf = 0.0f;   // each thread's strided partial in FP32 (fixed order), the tree in FP64
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float v = (float)x[i];
        sf = fmaf(v, v, sf);
    }
    double s = sf;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sw[w];
        out[0] += t;
    }
}

// node (i, j, k) of the mesh is voxel (i, j, k) of the padded level-0 grid
__device__ __forceinline__ int64_t node_voxel(int64_t node, int64_t nnx, int64_t nny, const Vol& g) {
    const int64_t i = node % nnx, j = (node / nnx) % nny, k = node / (nnx * nny);
    return i + (int64_t)g.px * (j + (int64_t)g.py * k);
}

// x0[v] = (r / rms(r), v / rms(v), log10 viscosity, 0) at node voxels; sumsq = (|r|^2, |v|^2)
template <typename T>
__global__ void k_make_input(int64_t nnx, int64_t nny, int64_t nn, Vol g, const T* __restrict__ r,
                             const T* __restrict__ vc, const double* __restrict__ sumsq,
                             const float* __restrict__ logeta, bf16* __restrict__ x0) {
    __shared__ float inv[2];
    if (threadIdx.x < 2)
        inv[threadIdx.x] = sumsq[threadIdx.x] > 0.0 ? (float)rsqrt(sumsq[threadIdx.x] / (double)(3 * nn)) : 0.0f;
    __syncthreads();
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t v = node_voxel(node, nnx, nny, g);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        x0[v * kInChannels + d] = __float2bfloat16_rn((float)r[(int64_t)d * nn + node] * inv[0]);
        x0[v * kInChannels + 3 + d] = __float2bfloat16_rn((float)vc[(int64_t)d * nn + node] * inv[1]);
    }
    x0[v * kInChannels + 6] = __float2bfloat16_rn(logeta[node]);
}

// z[d][node] += out_scale * rms(V(r)) * out[d][v] on free dofs (sumsq[1] = |V(r)|^2)
template <typename T>
__global__ void k_add_correction(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ out,
                                 const double* __restrict__ sumsq, float out_scale, const uint8_t* __restrict__ fixed,
                                 T* __restrict__ z) {
    __shared__ float s;
    if (threadIdx.x == 0) s = out_scale * (float)sqrt(sumsq[1] / (double)(3 * nn));
    __syncthreads();
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t v = node_voxel(node, nnx, nny, g);
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (!(fixed && fixed[node * 3 + d])) z[(int64_t)d * nn + node] += (T)(s * out[(int64_t)d * g.nv + v]);
}

// mean of log10(viscosity) over the material points of each element (0 for an empty element)
__global__ void k_elem_logeta(int64_t ne, const uint32_t* __restrict__ offsets, const double* __restrict__ eta,
                              float* __restrict__ elog) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const uint32_t a = offsets[e], b = offsets[e + 1];
    float s = 0.0f;
    for (uint32_t k = a; k < b; ++k) s += log10f(fmaxf((float)eta[k], 1e-30f));
    elog[e] = b > a ? s / (float)(b - a) : 0.0f;
}

// node value = mean over the (1..8) elements around the node
__global__ void k_node_logeta(int64_t nnx, int64_t nny, int64_t nn, int ex, int ey, int ez, const float* __restrict__ elog,
                              float* __restrict__ nlog) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t i = node % nnx, j = (node / nnx) % nny, k = node / (nnx * nny);
    float s = 0.0f;
    int cnt = 0;
    for (int o = 0; o < 8; ++o) {
        const int64_t a = i - (o & 1), b = j - ((o >> 1) & 1), cc = k - (o >> 2);
        if (a < 0 || a >= ex || b < 0 || b >= ey || cc < 0 || cc >= ez) continue;
        s += elog[a + (int64_t)ex * (b + (int64_t)ey * cc)];
        cnt++;
    }
    nlog[node] = cnt ? s / (float)cnt : 0.0f;
}

void prepare_viscosity(Context& c, Net& n) {
    UWG_REQUIRE(c.assembled && c.mapped, UWGPU_ERR_STATE, "learned preconditioner needs the assembled point viscosities");
    const MeshDesc& m = c.mesh;
    n.logeta.ensure((size_t)n.nn);
    DArray<float> elog;
    elog.ensure((size_t)m.ne);
    {
        LaunchScope ls(c, -1);
        k_elem_logeta<<<nblk(m.ne, 256), 256, 0, c.stream>>>(m.ne, c.offsets.p, c.seta_out.p, elog.p);
    }
    {
        LaunchScope ls(c, -1);
        k_node_logeta<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, m.nel[0], m.nel[1], m.nel[2], elog.p,
                                                             n.logeta.p);
    }
    UWG_CUDA(cudaStreamSynchronize(c.stream));   // elog is released on return
}

template <typename T>
void correct(Context& c, Net& n, const T* r, T* z) {
    n.sumsq.ensure(2);
    UWG_CUDA(cudaMemsetAsync(n.sumsq.p, 0, 2 * sizeof(double), c.stream));
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_sumsq<T><<<1, 1024, 0, c.stream>>>(3 * n.nn, r, n.sumsq.p);
    }
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_sumsq<T><<<1, 1024, 0, c.stream>>>(3 * n.nn, z, n.sumsq.p + 1);
    }
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_make_input<T><<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], r, z, n.sumsq.p,
                                                                n.logeta.p, n.x0.p);
    }
    forward(c, n);
    LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
    k_add_correction<T><<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], n.out.p, n.sumsq.p,
                                                                n.out_scale, c.levels[0].fixed.p, z);
}
template void correct<double>(Context&, Net&, const double*, double*);
template void correct<float>(Context&, Net&, const float*, float*);

// ------------------------------------------------------------------------------------------
// Training data: residual/error pairs of the multigrid solver (see solver.cu learned_generate)
// ------------------------------------------------------------------------------------------
struct Mode {
    float kx, ky, kz, phase, amp;
};

// e[d][node] = sum over the modes of component d of amp cos(2 pi k.x + phase), 0 on fixed dofs
__global__ void k_random_field(int64_t nnx, int64_t nny, int64_t nn, float hx, float hy, float hz,
                               const Mode* __restrict__ modes, int per_comp, const uint8_t* __restrict__ fixed,
                               double* __restrict__ e) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const float x = (float)(node % nnx) * hx, y = (float)((node / nnx) % nny) * hy, z = (float)(node / (nnx * nny)) * hz;
    for (int d = 0; d < 3; ++d) {
        float s = 0.0f;
        for (int m = 0; m < per_comp; ++m) {
            const Mode md = modes[d * per_comp + m];
            s += md.amp * cospif(2.0f * (md.kx * x + md.ky * y + md.kz * z) + md.phase);
        }
        e[(int64_t)d * nn + node] = (fixed && fixed[node * 3 + d]) ? 0.0 : (double)s;
    }
}

void random_field(Context& c, Net& n, uint64_t seed, double* e) {
    const MeshDesc& m = c.mesh;
    const int per = 16;
    uint64_t s = seed * 0x2545F4914F6CDD1Dull + 17;
    auto unif = [&]() { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); };
    // the largest wavenumber of this sample: from 1 (smooth) up to half the mesh resolution
    const int kcap = std::max(1, std::min(m.nel[0], std::min(m.nel[1], m.nel[2])) / 2);
    const double kmax = 1.0 + unif() * (kcap - 1);
    std::vector<Mode> h((size_t)3 * per);
    for (auto& md : h) {
        md.kx = (float)std::floor(unif() * (kmax + 1.0));
        md.ky = (float)std::floor(unif() * (kmax + 1.0));
        md.kz = (float)std::floor(unif() * (kmax + 1.0));
        const double kk = std::sqrt((double)md.kx * md.kx + (double)md.ky * md.ky + (double)md.kz * md.kz);
        md.phase = (float)(2.0 * unif());
        md.amp = (float)((2.0 * unif() - 1.0) / (1.0 + kk));
    }
    n.modes.ensure(h.size() * sizeof(Mode));
    UWG_CUDA(cudaMemcpyAsync(n.modes.p, h.data(), h.size() * sizeof(Mode), cudaMemcpyHostToDevice, c.stream));
    LaunchScope ls(c, -1);
    k_random_field<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, 1.0f / m.nel[0], 1.0f / m.nel[1],
                                                          1.0f / m.nel[2], reinterpret_cast<const Mode*>(n.modes.p), per,
                                                          c.levels[0].fixed.p, e);
    UWG_CUDA(cudaStreamSynchronize(c.stream));   // the host mode table is released on return
}

// sample k: xs = (r / rms(r), v / rms(v)) (FP32, [6][nn]), ys = (e - v) / rms(v) ([3][nn])
__global__ void k_store_sample(int64_t n3, const double* __restrict__ r, const double* __restrict__ e,
                               const double* __restrict__ v, const double* __restrict__ sumsq, int64_t nvec,
                               float* __restrict__ xs, float* __restrict__ ys) {
    __shared__ double inv[2];
    if (threadIdx.x < 2)
        inv[threadIdx.x] = sumsq[threadIdx.x] > 0.0 ? 1.0 / sqrt(sumsq[threadIdx.x] / (double)nvec) : 0.0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    xs[i] = (float)(r[i] * inv[0]);
    xs[n3 + i] = (float)(v[i] * inv[1]);
    ys[i] = (float)((e[i] - v[i]) * inv[1]);
}

void dataset_reserve(Context& c, Net& n, int nsamples) {
    n.data_x.ensure((size_t)nsamples * 6 * n.nn);
    n.data_y.ensure((size_t)nsamples * 3 * n.nn);
    n.ysq.assign((size_t)nsamples, 0.0);
    n.nsamples = 0;
    prepare_viscosity(c, n);
}

void dataset_add(Context& c, Net& n, const double* r, const double* e, const double* v) {
    const int k = n.nsamples;
    UWG_REQUIRE((size_t)k < n.ysq.size(), UWGPU_ERR_ARGUMENT, "training set is full");
    n.sumsq.ensure(2);
    UWG_CUDA(cudaMemsetAsync(n.sumsq.p, 0, 2 * sizeof(double), c.stream));
    const int64_t n3 = 3 * n.nn;
    {
        LaunchScope ls(c, -1);
        k_sumsq<double><<<1, 1024, 0, c.stream>>>(n3, r, n.sumsq.p);
        k_sumsq<double><<<1, 1024, 0, c.stream>>>(n3, v, n.sumsq.p + 1);
    }
    float* xs = n.data_x.p + (size_t)k * 2 * n3;
    float* ys = n.data_y.p + (size_t)k * n3;
    {
        LaunchScope ls(c, -1);
        k_store_sample<<<nblk(n3, 256), 256, 0, c.stream>>>(n3, r, e, v, n.sumsq.p, n3, xs, ys);
    }
    UWG_CUDA(cudaMemsetAsync(n.sumsq.p, 0, sizeof(double), c.stream));
    {
        LaunchScope ls(c, -1);
        k_sumsq<float><<<1, 1024, 0, c.stream>>>(n3, ys, n.sumsq.p);
    }
    double h = 0.0;
    UWG_CUDA(cudaMemcpyAsync(&h, n.sumsq.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    n.ysq[(size_t)k] = h;
    n.nsamples = k + 1;
}

__global__ void k_scale_f(int64_t n, float a, float* __restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= a;
}

// the network's targets are scaled to unit RMS; out_scale maps its output back
void dataset_finish(Context& c, Net& n) {
    UWG_REQUIRE(n.nsamples > 0, UWGPU_ERR_STATE, "empty training set");
    double tot = 0.0;
    for (int k = 0; k < n.nsamples; ++k) tot += n.ysq[(size_t)k];
    const double rms = std::sqrt(tot / ((double)n.nsamples * 3.0 * n.nn));
    UWG_REQUIRE(rms > 0.0 && std::isfinite(rms), UWGPU_ERR_NAN, "training targets are zero or not finite");
    n.out_scale = (float)rms;
    const int64_t tot_n = (int64_t)n.nsamples * 3 * n.nn;
    LaunchScope ls(c, -1);
    k_scale_f<<<nblk(tot_n, 256), 256, 0, c.stream>>>(tot_n, (float)(1.0 / rms), n.data_y.p);
    for (auto& v : n.ysq) v /= rms * rms;
    UWG_CUDA(cudaStreamSynchronize(c.stream));
}

// ------------------------------------------------------------------------------------------
// Training: relative squared error per sample, Adam
// ------------------------------------------------------------------------------------------
__global__ void k_sample_input(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ xs,
                               const float* __restrict__ logeta, bf16* __restrict__ x0) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nn) return;
    const int64_t v = node_voxel(node, nnx, nny, g);
#pragma unroll
    for (int d = 0; d < 6; ++d) x0[v * kInChannels + d] = __float2bfloat16_rn(xs[(int64_t)d * nn + node]);
    x0[v * kInChannels + 6] = __float2bfloat16_rn(logeta[node]);
}

// loss += |out - y|^2 / ysq over free dofs; gout = 2 (out - y) / ysq there (0 elsewhere)
__global__ void k_rel_mse(int64_t nnx, int64_t nny, int64_t nn, Vol g, const float* __restrict__ out,
                          const float* __restrict__ y, const uint8_t* __restrict__ fixed, float inv_ysq,
                          float* __restrict__ gout, double* __restrict__ loss) {
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (node < nn) {
        const int64_t v = node_voxel(node, nnx, nny, g);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float diff = out[(int64_t)d * g.nv + v] - y[(int64_t)d * nn + node];
            if (fixed && fixed[node * 3 + d]) diff = 0.0f;
            gout[(int64_t)d * g.nv + v] = 2.0f * diff * inv_ysq;
            l = fmaf(diff * diff, inv_ysq, l);
        }
    }
    l = warp_sum(l);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, (double)l);
}

// one sample: forward, loss and its gradient, backward (grads accumulate); returns the loss
static void sample_step(Context& c, Net& n, int k, bool train, double* dloss) {
    const int64_t n3 = 3 * n.nn;
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        k_sample_input<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], n.data_x.p + (size_t)k * 2 * n3,
                                                               n.logeta.p, n.x0.p);
    }
    forward(c, n);
    UWG_CUDA(cudaMemsetAsync(n.gout.p, 0, (size_t)n.vol[0].nv * 3 * sizeof(float), c.stream));
    {
        LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
        const double ysq = n.ysq[(size_t)k];
        k_rel_mse<<<nblk(n.nn, 256), 256, 0, c.stream>>>(n.nnx, n.nny, n.nn, n.vol[0], n.out.p, n.data_y.p + (size_t)k * n3,
                                                          c.levels[0].fixed.p, ysq > 0.0 ? (float)(1.0 / ysq) : 0.0f,
                                                          n.gout.p, dloss);
    }
    if (train) backward(c, n);
}

void train(Context& c, Net& n, int epochs, int batch, float lr, uint64_t seed, double* train_loss,
           double* holdout_ratio) {
    UWG_REQUIRE(n.nsamples >= 2, UWGPU_ERR_STATE, "training needs at least two samples (learned_generate)");
    UWG_REQUIRE(epochs >= 0 && batch >= 1, UWGPU_ERR_ARGUMENT, "bad epochs or batch");
    const int nhold = std::max(1, n.nsamples / 10);
    const int ntrain = n.nsamples - nhold;
    std::vector<int> order((size_t)ntrain);
    for (int k = 0; k < ntrain; ++k) order[(size_t)k] = k;
    uint64_t s = seed ^ 0xA0761D6478BD642Full;
    DArray<double> dl;
    dl.ensure(2);
    double last = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int k = ntrain - 1; k > 0; --k) std::swap(order[(size_t)k], order[(size_t)(splitmix(s) % (uint64_t)(k + 1))]);
        UWG_CUDA(cudaMemsetAsync(dl.p, 0, sizeof(double), c.stream));
        for (int b0 = 0; b0 < ntrain; b0 += batch) {
            const int nb = std::min(batch, ntrain - b0);
            UWG_CUDA(cudaMemsetAsync(n.grads.p, 0, (size_t)n.nparams * sizeof(float), c.stream));
            for (int q = 0; q < nb; ++q) sample_step(c, n, order[(size_t)(b0 + q)], true, dl.p);
            n.adam_t++;
            const float b1 = 0.9f, b2 = 0.999f;
            const float bc1 = 1.0f - std::pow(b1, (float)n.adam_t), bc2 = 1.0f - std::pow(b2, (float)n.adam_t);
            {
                LaunchScope ls(c, UWGPU_KERNEL_LEARNED);
                k_adam<<<nblk(n.nparams, 256), 256, 0, c.stream>>>(n.nparams, n.params.p, n.grads.p, n.adam_m.p,
                                                                   n.adam_v.p, lr, b1, b2, 1e-8f, bc1, bc2, 1.0f / nb);
            }
            pack(c, n);
        }
        UWG_CUDA(cudaMemcpyAsync(c.host_scalars, dl.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        last = c.host_scalars[0] / ntrain;
        if (!std::isfinite(last)) throw Error(UWGPU_ERR_NAN, "U-Net training diverged");
    }
    if (train_loss) *train_loss = last;
    // held-out samples: |y - N(x)|^2 / |y|^2 averaged (1 = no better than no correction)
    UWG_CUDA(cudaMemsetAsync(dl.p, 0, sizeof(double), c.stream));
    for (int k = ntrain; k < n.nsamples; ++k) sample_step(c, n, k, false, dl.p);
    UWG_CUDA(cudaMemcpyAsync(c.host_scalars, dl.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    if (holdout_ratio) *holdout_ratio = c.host_scalars[0] / nhold;
    check_errors(c, n);
}

}  // namespace unet
}  // namespace uwg
