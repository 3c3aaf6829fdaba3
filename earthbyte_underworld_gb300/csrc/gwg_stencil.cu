// Explicit element stencil of G^T W G and the Jacobi-preconditioned CG on it: the inner solves
// of the scaled BFBt Schur preconditioner (Solvers/KSPSolvers/src/BSSCR/pc_ScaledGtKG.c:242-310,
// the KSP on G^T W G built at pc_ScaledGtKG.c:735-760 with W = 1/rowmax(K)).
//
// G^T W G acts on P0 pressures (one unknown per element) and couples each element with the
// 3^dim elements that share a node with it.  Applying it matrix-free (G, scale by W, G^T) costs
// about 75 FP64 instructions per node and 50 per element, which on this part (FP64 at 1/58 of
// the FP32 rate) makes every CG iteration FP64-issue bound.  The stencil is built once per solve
// (A[q][e], entry-major, q = neighbour offset) and an iteration is then 27 FMAs per element
// with coalesced stencil reads; the 57 MB FP64 stencil of a 64^3 mesh can stay in L2.  In FP32
// the matrix-free chain is cheap, so the mixed form applies G^T W G matrix-free (k_cg_mf3_dir,
// k_cg_mf2_dir below) once its FP32 stencil would no longer fit in L2.
// Further down: the aggregation multigrid option for the inner solves, and the test and timing
// hooks on the inner operator.
//
// CG state lives in device memory and an iteration k is two kernels:
//   k_cg_update:   alpha = rz_k / pq_k; x += alpha p; r -= alpha q; z = Dinv r; rz_{k+1}, rr
//   k_cg_spmv_dir: beta = rz_{k+1} / rz_k; p = z + beta p; q = A z + beta q (= A p); pq_{k+1}
// (q = A p by linearity, so the direction update needs no neighbour of p and fuses into the spmv).
// The scalars are buffered so that no kernel clears a slot another block may still read:
//   scal[0..2] = rz (k mod 3)   scal[3..4] = pq (k mod 2)   scal[5..6] = rr (k mod 2)   scal[7] = r0.r0
// Twelve iterations (so both patterns repeat) are captured once as a CUDA graph and replayed; the
// host reads the residual norm after each replay.  The two kernels are launched with programmatic
// dependent launch (pdl_wait / pdl_trigger), so each one's blocks are resident when the previous
// one ends.
#include <algorithm>
#include <cmath>
#include <iterator>
#include <type_traits>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "internal.cuh"
#include "tc.cuh"

namespace uwg {

// fine-mesh element widths h[off[d] + i] (operator.cu), FP64 and FP32
const double* fine_widths(Context& c, int off[3]);
void bfbt_weights(Context& c, double* W);
void to_float(Context& c, const double* a, float* b, int64_t n);
void to_double(Context& c, const float* a, double* b, int64_t n);
void gwg_stencil_build(Context& c, const double* W, double* A, double* dinv);

namespace {

struct EGrid {
    int64_t ex, ey, ez, ne;
};

template <int DIM>
__host__ __device__ constexpr int stencil_points() { return DIM == 3 ? 27 : 9; }

// Block sum: products and the warp shuffle tree in the working precision T (FP64 work is 58x
// slower than FP32 on this part), the eight warp partials in FP64.
template <typename T>
__device__ __forceinline__ double block_sum(T v, double* sw) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sw[warp] = (double)v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sw[w];
    return t;  // valid in thread 0
}

// ratio of two device scalars, formed once per block (one FP64 division per block, not per thread)
template <typename T>
__device__ __forceinline__ T block_ratio(const double* num, const double* den, T* slot) {
    if (threadIdx.x == 0) *slot = (T)(*num / *den);
    __syncthreads();
    return *slot;
}

// Programmatic dependent launch between the CG kernels: a kernel waits for the grid before it
// (griddepcontrol.wait: that grid has completed and its writes are visible) before it reads
// anything, and lets the next grid start launching once all its own writes are issued, so the
// next kernel's blocks are resident when this one ends.  Without a programmatic predecessor the
// wait returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
void launch_pdl(void (*kern)(KArgs...), unsigned grid, unsigned block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    UWG_CUDA(cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
}

// A[q][e] = sum over the nodes n shared by e and f = e + off(q), and the free components d of n,
//           G_(n,d),e W_(n,d) G_(n,d),f   with  G_(n,d),e = -s prod_{k != d} h_k / 2^(dim-1),
// s = +1 when n is on the upper side of e along d (the P0 divergence term of the Q1 element,
// StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:160-250, integrated exactly); dinv = 1/A_ee.
template <int DIM>
__global__ void k_gwg_build(EGrid g, const double* __restrict__ h, int off1, int off2, int64_t nnx, int64_t nny,
                            int64_t nn, const double* __restrict__ W, const uint8_t* __restrict__ fixed,
                            double* __restrict__ A, double* __restrict__ dinv) {
    constexpr int NB = stencil_points<DIM>();
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.ne) return;
    const int64_t ei[3] = {e % g.ex, (e / g.ex) % g.ey, DIM == 3 ? e / (g.ex * g.ey) : 0};
    const int64_t ec[3] = {g.ex, g.ey, g.ez};
    const int offs[3] = {0, off1, off2};
    const double sc = DIM == 3 ? 0.25 : 0.5;
    double area_e[3];
    {
        double he[3] = {1.0, 1.0, 1.0};
#pragma unroll
        for (int d = 0; d < DIM; ++d) he[d] = h[offs[d] + ei[d]];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            area_e[d] = sc;
#pragma unroll
            for (int k = 0; k < DIM; ++k)
                if (k != d) area_e[d] *= he[k];
        }
    }
    for (int q = 0; q < NB; ++q) {
        const int o[3] = {q % 3 - 1, (q / 3) % 3 - 1, DIM == 3 ? q / 9 - 1 : 0};
        int64_t fi[3] = {0, 0, 0};
        bool valid = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            fi[d] = ei[d] + o[d];
            valid = valid && fi[d] >= 0 && fi[d] < ec[d];
        }
        double acc = 0.0;
        if (valid) {
            double hf[3] = {1.0, 1.0, 1.0}, area_f[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) hf[d] = h[offs[d] + fi[d]];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                area_f[d] = sc;
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                    if (k != d) area_f[d] *= hf[k];
            }
            // corners b of e whose node is also a corner (b - o) of f
            for (int b = 0; b < (1 << DIM); ++b) {
                int bb[3] = {b & 1, (b >> 1) & 1, (b >> 2) & 1};
                bool shared = true;
#pragma unroll
                for (int d = 0; d < DIM; ++d) shared = shared && (bb[d] - o[d] == 0 || bb[d] - o[d] == 1);
                if (!shared) continue;
                int64_t n = (ei[0] + bb[0]) + nnx * ((ei[1] + bb[1]) + nny * (DIM == 3 ? ei[2] + bb[2] : 0));
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    if (fixed && fixed[n * DIM + d]) continue;
                    double se = bb[d] ? -1.0 : 1.0;          // -s for corner b of e
                    double sf = (bb[d] - o[d]) ? -1.0 : 1.0;  // -s for corner b - o of f
                    acc += (se * area_e[d]) * W[(int64_t)d * nn + n] * (sf * area_f[d]);
                }
            }
        }
        A[(int64_t)q * g.ne + e] = acc;
        if (q == NB / 2) dinv[e] = 1.0 / acc;
    }
}

template <typename S, typename D>
__global__ void k_gwg_convert(int64_t n, const S* __restrict__ a, D* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (D)a[i];
}

// q = A p ; scal[0] += p.q ; clears the accumulators that the update kernel fills.
// Entries towards neighbours outside the mesh are stored as 0, so the neighbour index is clamped
// to the element itself and every load is unconditional (all 2 x 27 loads can be in flight).
// Index math is 32-bit (the host checks 27 ne < 2^31).
template <int DIM, typename T>
__global__ void __launch_bounds__(256) k_gwg_spmv(EGrid g, const T* __restrict__ A, const T* __restrict__ p,
                                                  T* __restrict__ q, double* __restrict__ scal, int parity) {
    constexpr int NB = stencil_points<DIM>();
    __shared__ double sw[32];
    const int ne = (int)g.ne, ex = (int)g.ex, ey = (int)g.ey, ez = (int)g.ez;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    T local = (T)0;
    if (e < ne) {
        const int exy = ex * ey;
        const int ix = e % ex, iy = (e / ex) % ey, iz = DIM == 3 ? e / exy : 0;
        const int dx[3] = {ix > 0 ? -1 : 0, 0, ix + 1 < ex ? 1 : 0};
        const int dy[3] = {iy > 0 ? -ex : 0, 0, iy + 1 < ey ? ex : 0};
        const int dz[3] = {DIM == 3 && iz > 0 ? -exy : 0, 0, DIM == 3 && iz + 1 < ez ? exy : 0};
        T a[NB], x[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k) a[k] = __ldg(A + (size_t)k * ne + e);
#pragma unroll
        for (int k = 0; k < NB; ++k) x[k] = __ldg(p + e + dx[k % 3] + dy[(k / 3) % 3] + dz[DIM == 3 ? k / 9 : 1]);
        T acc = (T)0;
#pragma unroll
        for (int k = 0; k < NB; ++k) acc = fma(a[k], x[k], acc);
        q[e] = acc;
        local = acc * x[NB / 2];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        scal[1 + (parity ^ 1)] = 0.0;
        scal[3] = 0.0;
    }
    double t = block_sum<T>(local, sw);
    if (threadIdx.x == 0) atomicAdd(&scal[0], t);
}

static double* rz_slot_host(double* scal, int k) { return scal + ((k % 3) + 3) % 3; }
__device__ __forceinline__ double* rz_slot(double* scal, int k) { return scal + ((k % 3) + 3) % 3; }
__device__ __forceinline__ double* pq_slot(double* scal, int k) { return scal + 3 + (((k % 2) + 2) % 2); }
__device__ __forceinline__ double* rr_slot(double* scal, int k) { return scal + 5 + (((k % 2) + 2) % 2); }

// iteration k, second kernel: p = z + beta p; q = A z + beta q; pq_{k+1} += p.q.  With first != 0
// (before iteration 0): p = z, q = A z, pq_0.  Clears rr_{k+1}'s slot.
template <int DIM, typename T>
__global__ void __launch_bounds__(256) k_cg_spmv_dir(EGrid g, const T* __restrict__ A, const T* __restrict__ z,
                                                     T* __restrict__ p, T* __restrict__ q, double* __restrict__ scal,
                                                     int k, int first) {
    constexpr int NB = stencil_points<DIM>();
    __shared__ double sw[32];
    __shared__ T s_beta;
    pdl_wait();
    const T beta = first ? (T)0 : block_ratio<T>(rz_slot(scal, k + 1), rz_slot(scal, k), &s_beta);
    const int ne = (int)g.ne, ex = (int)g.ex, ey = (int)g.ey, ez = (int)g.ez;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    T local = (T)0;
    if (e < ne) {
        const int exy = ex * ey;
        const int ix = e % ex, iy = (e / ex) % ey, iz = DIM == 3 ? e / exy : 0;
        const int dx[3] = {ix > 0 ? -1 : 0, 0, ix + 1 < ex ? 1 : 0};
        const int dy[3] = {iy > 0 ? -ex : 0, 0, iy + 1 < ey ? ex : 0};
        const int dz[3] = {DIM == 3 && iz > 0 ? -exy : 0, 0, DIM == 3 && iz + 1 < ez ? exy : 0};
        T a[NB], x[NB];
#pragma unroll
        for (int t = 0; t < NB; ++t) a[t] = __ldg(A + (size_t)t * ne + e);
#pragma unroll
        for (int t = 0; t < NB; ++t) x[t] = __ldg(z + e + dx[t % 3] + dy[(t / 3) % 3] + dz[DIM == 3 ? t / 9 : 1]);
        T az = (T)0;
#pragma unroll
        for (int t = 0; t < NB; ++t) az = fma(a[t], x[t], az);
        const T pe = first ? x[NB / 2] : fma(beta, p[e], x[NB / 2]);
        const T qe = first ? az : fma(beta, q[e], az);
        p[e] = pe;
        q[e] = qe;
        local = pe * qe;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *rr_slot(scal, k + 1) = 0.0;
    double t = block_sum<T>(local, sw);
    if (threadIdx.x == 0) atomicAdd(pq_slot(scal, k + 1), t);
    pdl_trigger();
}

// Elements per thread of the vector kernels: the block reduction (a shuffle tree, FP64 in the
// FP64 form) is paid once per kEpt elements.  Element k of a thread is base + k * blockDim.x,
// so every access stays coalesced.
constexpr int kEpt = 2;

// iteration k, first kernel: alpha = rz_k / pq_k; x += alpha p (unless with_x is 0: the direction
// kernel then updates x); r -= alpha q; z = dinv r; rz_{k+1} += r.z; and, when want_rr (the host's
// convergence check follows), rr_k += r.r.  Clears the slots of rz_{k+2} and pq_{k+1}.
// k_cg_update: 512 threads x 4 elements per block, so that few blocks (1,024 at 128^3) add their
// partial sums to the same two scalars (same-address atomics serialise in L2)
constexpr int kUpdThreads = 512, kUpdEpt = 4;

template <typename T>
__global__ void __launch_bounds__(kUpdThreads) k_cg_update(int64_t ne, const T* __restrict__ p, const T* __restrict__ q,
                            const T* __restrict__ dinv, T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                            double* __restrict__ scal, int k, int want_rr, int with_x) {
    __shared__ double sw[32];
    __shared__ T s_alpha;
    pdl_wait();
    // the vectors first: their loads are in flight while thread 0 fetches the scalars for alpha
    const int64_t base = (int64_t)blockIdx.x * blockDim.x * kUpdEpt + threadIdx.x;
    T pv[kUpdEpt], qv[kUpdEpt], xv[kUpdEpt], rv[kUpdEpt], dv[kUpdEpt];
#pragma unroll
    for (int m = 0; m < kUpdEpt; ++m) {
        const int64_t e = base + (int64_t)m * blockDim.x;
        const bool in = e < ne;
        pv[m] = in && with_x ? p[e] : (T)0;
        qv[m] = in ? q[e] : (T)0;
        xv[m] = in && with_x ? x[e] : (T)0;
        rv[m] = in ? r[e] : (T)0;
        dv[m] = in ? dinv[e] : (T)0;
    }
    const T alpha = block_ratio<T>(rz_slot(scal, k), pq_slot(scal, k), &s_alpha);
    T rz = (T)0, rr = (T)0;
#pragma unroll
    for (int m = 0; m < kUpdEpt; ++m) {
        const int64_t e = base + (int64_t)m * blockDim.x;
        if (e < ne) {
            if (with_x) x[e] = fma(alpha, pv[m], xv[m]);
            T re = fma(-alpha, qv[m], rv[m]);
            r[e] = re;
            T ze = re * dv[m];
            z[e] = ze;
            rz = fma(re, ze, rz);
            rr = fma(re, re, rr);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *rz_slot(scal, k + 2) = 0.0;
        *pq_slot(scal, k + 1) = 0.0;
    }
    double t1 = block_sum<T>(rz, sw);
    if (threadIdx.x == 0) atomicAdd(rz_slot(scal, k + 1), t1);
    if (want_rr) {
        __syncthreads();
        double t2 = block_sum<T>(rr, sw);
        if (threadIdx.x == 0) atomicAdd(rr_slot(scal, k), t2);
    }
    pdl_trigger();
}

// r = b, z = dinv r, x = 0 ; rz_0 (scal[0]) = r.z, scal[7] = r0.r0 (scal zeroed before; p and q
// are formed by the first k_cg_spmv_dir)
template <typename T>
__global__ void k_gwg_init(int64_t ne, const double* __restrict__ b, const T* __restrict__ dinv, T* __restrict__ x,
                           T* __restrict__ r, T* __restrict__ z, double* __restrict__ scal) {
    __shared__ double sw[32];
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T rz = (T)0, rr = (T)0;
    if (e < ne) {
        T re = (T)b[e];
        T ze = re * dinv[e];
        x[e] = (T)0;
        r[e] = re;
        z[e] = ze;
        rz = re * ze;
        rr = re * re;
    }
    double t1 = block_sum<T>(rz, sw);
    __syncthreads();
    double t2 = block_sum<T>(rr, sw);
    if (threadIdx.x == 0) {
        atomicAdd(&scal[0], t1);
        atomicAdd(&scal[7], t2);
    }
}

// ------------------------------------------------------------------------------------------
// Matrix-free FP32 apply (mixed form).  In FP32 the G, W, G^T chain is cheap arithmetic (FP32
// issues at 58x the FP64 rate), so the mixed form applies G^T W G without the stencil and streams
// z, p, q (read), p, q (written) and about one node's W per element instead of 27 stencil
// coefficients; on a 128^3 mesh every array an iteration touches fits in L2 together.
// The mesh is uniform, so G_(n,d),f = -s a_d with s = +1 when n is on the upper side of f along d
// and a_d = prod_{k != d} h_k / 2^(dim-1) (the convention of k_gwg_build).  With the folded
// weights Wc_(n,d) = a_d^2 W_(n,d) (zero on fixed components):
//   y_(n,d) = Wc_(n,d) D_d(n),  D_d(n) = sum over the 2^dim elements f around n of
//             (+1 if f is above n along d, else -1) z_f
//   (A z)_e = sum over the corners b of e and the components d of (-1 if b is the upper corner
//             along d, else +1) y_(n_b,d)
// ------------------------------------------------------------------------------------------
constexpr int kMfX = 32, kMfY = 8;

// 2D: one kMfX x kMfY tile of elements per block; z with its one-element halo and the tile's
// nodes staged in shared memory; fused with the direction update of k_cg_spmv_dir
__global__ void __launch_bounds__(kMfX * kMfY) k_cg_mf2_dir(int ex, int ey, int64_t nnx, int64_t nn,
                                                            const float* __restrict__ Wc, const float* __restrict__ z,
                                                            float* __restrict__ p, float* __restrict__ q,
                                                            double* __restrict__ scal, int k, int first) {
    constexpr int NT = kMfX * kMfY;
    constexpr int HX = kMfX + 2, HY = kMfY + 2, NX = kMfX + 1, NY = kMfY + 1, NN = NX * NY;
    __shared__ float zs[HY * HX];
    __shared__ float ys[2 * NN];
    __shared__ double sw[32];
    __shared__ float s_beta;
    const int ntx = (ex + kMfX - 1) / kMfX;
    const int x0 = (blockIdx.x % ntx) * kMfX, y0 = (blockIdx.x / ntx) * kMfY;
    const int tid = threadIdx.x, lx = tid % kMfX, ly = tid / kMfX;
    pdl_wait();
    for (int i = tid; i < HY * HX; i += NT) {
        const int gx = x0 - 1 + i % HX, gy = y0 - 1 + i / HX;
        zs[i] = (gx >= 0 && gx < ex && gy >= 0 && gy < ey) ? __ldg(z + gx + ex * gy) : 0.f;
    }
    const float beta = first ? 0.f : block_ratio<float>(rz_slot(scal, k + 1), rz_slot(scal, k), &s_beta);
    __syncthreads();
    for (int i = tid; i < NN; i += NT) {
        const int nx = i % NX, ny = i / NX, gx = x0 + nx, gy = y0 + ny;
        float y0v = 0.f, y1v = 0.f;
        if (gx <= ex && gy <= ey) {
            const int b = ny * HX + nx;
            const float z00 = zs[b], z10 = zs[b + 1], z01 = zs[b + HX], z11 = zs[b + HX + 1];
            const int64_t node = gx + nnx * gy;
            y0v = __ldg(Wc + node) * ((z10 - z00) + (z11 - z01));
            y1v = __ldg(Wc + nn + node) * ((z01 - z00) + (z11 - z10));
        }
        ys[i] = y0v;
        ys[NN + i] = y1v;
    }
    __syncthreads();
    float local = 0.f;
    const int gx = x0 + lx, gy = y0 + ly;
    if (gx < ex && gy < ey) {
        const int b = ly * NX + lx;
        const float out = (ys[b] - ys[b + 1] + ys[b + NX] - ys[b + NX + 1]) +
                          (ys[NN + b] + ys[NN + b + 1] - ys[NN + b + NX] - ys[NN + b + NX + 1]);
        const int e = gx + ex * gy;
        const float ze = zs[(ly + 1) * HX + lx + 1];
        const float pe = first ? ze : fmaf(beta, p[e], ze);
        const float qe = first ? out : fmaf(beta, q[e], out);
        p[e] = pe;
        q[e] = qe;
        local = pe * qe;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *rr_slot(scal, k + 1) = 0.0;
    double t = block_sum<float>(local, sw);
    if (threadIdx.x == 0) atomicAdd(pq_slot(scal, k + 1), t);
    pdl_trigger();
}

// 3D: a block owns a column of kMfX x kMfY elements over zc element planes and marches up z.  Step
// t stages element plane kk = zlo - 1 + t (with its one-element xy halo), forms node plane kk
// from element planes kk - 1 and kk, then element plane kk - 1 from node planes kk - 1 and kk.
// The next plane's z, W, p and q are loaded into registers while the current one is computed.
// Element planes rotate through three buffers and node planes through two, so that no thread
// overwrites a plane another thread may still read (two barriers per step).
struct Mf3 {
    int ex, ey, ez, zc;
    int64_t pitch, nny, nn;   // W layout [d][node plane][y][pitch]: row pitch, rows per plane, entries per d
};

__global__ void __launch_bounds__(kMfX * kMfY) k_cg_mf3_dir(Mf3 a, const float* __restrict__ Wc,
                                                            const float* __restrict__ z, float* __restrict__ p,
                                                            float* __restrict__ q, double* __restrict__ scal, int k,
                                                            int first) {
    constexpr int NT = kMfX * kMfY;
    constexpr int HX = kMfX + 2, HY = kMfY + 2, HP = HX * HY;   // element plane with halo
    constexpr int NX = kMfX + 1, NY = kMfY + 1, NP = NX * NY;   // node plane
    static_assert(HP <= 2 * NT && NP <= 2 * NT, "two slots per thread cover a plane");
    __shared__ float zb[3][HP];
    __shared__ float yb[2][3][NP];
    __shared__ double sw[32];
    __shared__ float s_beta, s_alpha;
    const int ex = a.ex, ey = a.ey, ez = a.ez;
    const int ntx = (ex + kMfX - 1) / kMfX, nty = (ey + kMfY - 1) / kMfY;
    int bi = blockIdx.x;
    const int x0 = (bi % ntx) * kMfX;
    bi /= ntx;
    const int y0 = (bi % nty) * kMfY;
    bi /= nty;
    const int zlo = bi * a.zc, zhi = min(zlo + a.zc, ez);
    const int tid = threadIdx.x, tx = tid % kMfX, ty = tid / kMfX;
    const int64_t exy = (int64_t)ex * ey, nxy = a.pitch * a.nny;
    // this thread's two element-halo slots and two node slots of a plane (offsets within a plane)
    int zo[2], nbase[2];
    bool zok[2], nok[2];
    int64_t no[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const int i = tid + s * NT;
        const int hx = i % HX, hy = i / HX, gx = x0 - 1 + hx, gy = y0 - 1 + hy;
        zok[s] = i < HP && gx >= 0 && gx < ex && gy >= 0 && gy < ey;
        zo[s] = zok[s] ? gx + ex * gy : 0;
        const int nx = i % NX, ny = i / NX;
        nok[s] = i < NP && x0 + nx <= ex && y0 + ny <= ey;
        no[s] = nok[s] ? (x0 + nx) + a.pitch * (y0 + ny) : 0;
        nbase[s] = ny * HX + nx;   // the node's lower-left element in the halo plane
    }
    const bool eok = x0 + tx < ex && y0 + ty < ey;
    const int eo = eok ? (x0 + tx) + ex * (y0 + ty) : 0;
    float zr[2], wr[2][3], pn = 0.f, qn = 0.f;
    auto load_z = [&](int plane) {
#pragma unroll
        for (int s = 0; s < 2; ++s)
            zr[s] = zok[s] && plane >= 0 && plane < ez ? __ldg(z + plane * exy + zo[s]) : 0.f;
    };
    auto load_w = [&](int plane) {
#pragma unroll
        for (int s = 0; s < 2; ++s)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                wr[s][d] = nok[s] && plane <= ez ? __ldg(Wc + d * a.nn + plane * nxy + no[s]) : 0.f;
    };
    auto load_pq = [&](int plane) {
        const bool ok = !first && eok && plane < zhi;
        pn = ok ? p[plane * exy + eo] : 0.f;
        qn = ok ? q[plane * exy + eo] : 0.f;
    };
    pdl_wait();
    const float beta = first ? 0.f : block_ratio<float>(rz_slot(scal, k + 1), rz_slot(scal, k), &s_beta);
    // prologue: element plane zlo - 1 into buffer 0; registers for plane zlo
    load_z(zlo - 1);
#pragma unroll
    for (int s = 0; s < 2; ++s)
        if (tid + s * NT < HP) zb[0][tid + s * NT] = zr[s];
    load_z(zlo);
    load_w(zlo);
    float lo[3][4], hi[3][4];
    float local = 0.f;
    const int ybase = ty * NX + tx;
    for (int t = 1; t <= zhi - zlo + 1; ++t) {
        const int kk = zlo - 1 + t;
        float* zc = zb[t % 3];
        const float* zp = zb[(t + 2) % 3];   // element plane kk - 1
#pragma unroll
        for (int s = 0; s < 2; ++s)
            if (tid + s * NT < HP) zc[tid + s * NT] = zr[s];
        float wc[2][3];
#pragma unroll
        for (int s = 0; s < 2; ++s)
#pragma unroll
            for (int d = 0; d < 3; ++d) wc[s][d] = wr[s][d];
        const float pc = pn, qc = qn;
        load_z(kk + 1);
        load_w(kk + 1);
        load_pq(kk);   // element plane kk, computed in the next step
        __syncthreads();
        float* yc = yb[t & 1][0];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int i = tid + s * NT;
            if (i < NP) {
                const int b = nbase[s];
                const float z000 = zp[b], z100 = zp[b + 1], z010 = zp[b + HX], z110 = zp[b + HX + 1];
                const float z001 = zc[b], z101 = zc[b + 1], z011 = zc[b + HX], z111 = zc[b + HX + 1];
                const float dx = (z100 - z000) + (z110 - z010) + (z101 - z001) + (z111 - z011);
                const float dy = (z010 - z000) + (z110 - z100) + (z011 - z001) + (z111 - z101);
                const float dz = (z001 - z000) + (z101 - z100) + (z011 - z010) + (z111 - z110);
                yc[i] = wc[s][0] * dx;
                yc[NP + i] = wc[s][1] * dy;
                yc[2 * NP + i] = wc[s][2] * dz;
            }
        }
        __syncthreads();
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4) {
            const int ni = ybase + (c4 >> 1) * NX + (c4 & 1);
#pragma unroll
            for (int d = 0; d < 3; ++d) hi[d][c4] = yc[d * NP + ni];
        }
        if (t >= 2 && eok) {
            // element plane kk - 1: corners (bx, by) on node planes kk - 1 (lo) and kk (hi)
            float out = 0.f;
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
                out += (c4 & 1) ? -(lo[0][c4] + hi[0][c4]) : (lo[0][c4] + hi[0][c4]);
                out += (c4 >> 1) ? -(lo[1][c4] + hi[1][c4]) : (lo[1][c4] + hi[1][c4]);
                out += lo[2][c4] - hi[2][c4];
            }
            const int64_t e = (int64_t)(kk - 1) * exy + eo;
            const float ze = zp[(ty + 1) * HX + tx + 1];
            const float pe = first ? ze : fmaf(beta, pc, ze);
            const float qe = first ? out : fmaf(beta, qc, out);
            p[e] = pe;
            q[e] = qe;
            local = fmaf(pe, qe, local);
        }
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
            for (int d = 0; d < 3; ++d) lo[d][c4] = hi[d][c4];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *rr_slot(scal, k + 1) = 0.0;
    double t = block_sum<float>(local, sw);
    if (threadIdx.x == 0) atomicAdd(pq_slot(scal, k + 1), t);
    pdl_trigger();
}

// The same direction update with every plane it reads staged by the tensor memory accelerator
// (cp.async.bulk.tensor), for element grids whose x extent is a multiple of 4 (so that every z row
// starts on 16 bytes).  Per z step one thread issues the copies of one stage into a ring of five:
// the element plane of z with its halo, as a 40 x 10 box from x0 - 4 (x aligned down to 16 bytes;
// coordinates outside the grid, the halo at the mesh boundary and the planes below and above the
// mesh, read as zero), the 36 x 9 x 3 box of the node plane's three weight components, and (after
// the first iteration) the tile's 32 x 8 plane of p and of q.  The copies complete on the stage's
// mbarrier.  Six warps: a thread forms two nodes of the 33 x 9 node plane (rows 2i and 2i + 1, one
// column; the element rows they share are summed once), then two elements of the 32 x 8 tile (rows
// 2j and 2j + 1; the node rows they share are combined once); one block barrier per step.  The
// arithmetic runs on FP32 pairs where the values come in twos (the two planes of a staged element
// row, the two columns of a node row, the two nodes or two elements of a thread): one packed add,
// multiply or fma (__fadd2_rn, __fmul2_rn, __ffma2_rn) does the work of two scalar ones.  A copy
// that has not arrived after a bounded wait makes the block report NaN in the iteration's p.q,
// which ends the inner solve with UWGPU_ERR_NAN.
constexpr int kTmThreads = 192;
constexpr int kTzX = kMfX + 8, kTzY = kMfY + 2;     // staged element plane: 40 x 10
constexpr int kTwX = kMfX + 4, kTwY = kMfY + 1;     // staged weight plane: 36 x 9, three components
constexpr int kTzBytes = kTzX * kTzY * 4, kTwBytes = 3 * kTwX * kTwY * 4, kTpBytes = kMfX * kMfY * 4;
constexpr int kTzSlot = (kTzBytes + 127) / 128 * 128, kTwSlot = (kTwBytes + 127) / 128 * 128;
constexpr int kTmStage = kTzSlot + kTwSlot + 2 * kTpBytes;   // z, W, p, q; every part 128-byte aligned
static_assert(kTpBytes % 128 == 0, "p and q slots stay 128-byte aligned");
// Ring of stages: step t reads stages t - 1 and t, so a slot is free again two steps after its
// stage was read; with kTmRing slots the copies run kTmRing - 2 stages ahead of the computation.
constexpr int kTmRing = 5;
constexpr int kTmNodes = (kMfX + 1) * (kMfY + 1);   // 297

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__global__ void __launch_bounds__(kTmThreads, 4) k_cg_mf3_dir_tma(Mf3 a, const __grid_constant__ CUtensorMap tz,
                                                                 const __grid_constant__ CUtensorMap tw,
                                                                 const __grid_constant__ CUtensorMap tp,
                                                                 const __grid_constant__ CUtensorMap tq,
                                                                 float* __restrict__ p, float* __restrict__ q,
                                                                 float* __restrict__ x, double* __restrict__ scal, int k,
                                                                 int first) {
    __shared__ __align__(128) unsigned char ring[kTmRing * kTmStage];
    __shared__ float yb[2][3][kTmNodes];
    __shared__ __align__(8) uint64_t bar[kTmRing];
    __shared__ double sw[32];
    __shared__ float s_beta, s_alpha;
    const int ex = a.ex, ey = a.ey, ez = a.ez;
    const int ntx = (ex + kMfX - 1) / kMfX, nty = (ey + kMfY - 1) / kMfY;
    int bi = blockIdx.x;
    const int x0 = (bi % ntx) * kMfX;
    bi /= ntx;
    const int y0 = (bi % nty) * kMfY;
    bi /= nty;
    const int zlo = bi * a.zc, zhi = min(zlo + a.zc, ez);
    const int nsteps = zhi - zlo + 2;   // stages: planes zlo - 1 .. zhi
    const int tid = threadIdx.x;
    const int64_t exy = (int64_t)ex * ey;
    if (tid == 0) {
        for (int i = 0; i < kTmRing; ++i) tc::mbar_init(&bar[i], 1);
    }
    // no thread may poll a barrier before it is initialised (the shared memory may still hold an
    // earlier block's state)
    __syncthreads();
    const uint32_t ring_s = tc::smem_u32(ring);
    // stage t = element plane zlo - 1 + t (z with halo; p and q of the tile when the plane is one of
    // the block's own and p, q are read), node plane zlo - 1 + t (W)
    auto issue = [&](int t) {
        const int slot = t % kTmRing, plane = zlo - 1 + t;
        const bool pq = !first && plane >= zlo && plane < zhi;
        const uint32_t b = tc::smem_u32(&bar[slot]), dst = ring_s + slot * kTmStage;
        mbar_expect_tx(b, (uint32_t)(kTzBytes + kTwBytes + (pq ? 2 * kTpBytes : 0)));
        tma_load_3d(dst, &tz, x0 - 4, y0 - 1, plane, b);
        tma_load_4d(dst + kTzSlot, &tw, x0, y0, plane, 0, b);
        if (pq) {
            tma_load_3d(dst + kTzSlot + kTwSlot, &tp, x0, y0, plane, b);
            tma_load_3d(dst + kTzSlot + kTwSlot + kTpBytes, &tq, x0, y0, plane, b);
        }
    };
    pdl_wait();
    // the first copies go out before the block waits for the scalars of beta
    int issued = 0;   // stages issued so far (thread 0)
    if (tid == 0)
        while (issued < nsteps && issued < kTmRing - 1) issue(issued++);
    // x += alpha_k p_k here when x is given (the update kernel then leaves x alone): p_k is the p
    // plane this kernel reads before it forms p_{k+1}
    const bool xupd = x != nullptr && !first;
    if (tid == 0) {
        s_beta = first ? 0.f : (float)(*rz_slot(scal, k + 1) / *rz_slot(scal, k));
        s_alpha = xupd ? (float)(*rz_slot(scal, k) / *pq_slot(scal, k)) : 0.f;
    }
    __syncthreads();
    const float beta = s_beta, alpha = s_alpha;
    // element role (threads 0..127): elements (tx, ty0) and (tx, ty0 + 1) of the 32 x 8 tile
    const bool elem = tid < kMfX * kMfY / 2;
    const int tx = tid % kMfX, ty0 = 2 * (tid / kMfX);
    const bool eok0 = elem && x0 + tx < ex && y0 + ty0 < ey;
    const bool eok1 = elem && x0 + tx < ex && y0 + ty0 + 1 < ey;
    const int eo = eok0 ? (x0 + tx) + ex * (y0 + ty0) : 0;   // element (tx, ty0); (tx, ty0 + 1) is ex further
    const int ybase = ty0 * (kMfX + 1) + tx;   // node (tx, ty0) in the node-plane buffers
    // node role (threads 0..164): nodes (nx, ny0) and (nx, ny0 + 1) of the 33 x 9 node block; warp
    // w < 5 takes columns 0..31 of row pair w, threads 160..164 column 32 of each pair; the last
    // pair (rows 8, 9) has only row 8
    const bool node = tid < 5 * kMfX + 5;
    const int nx = tid < 5 * kMfX ? tid % kMfX : kMfX;
    const int ny0 = 2 * (tid < 5 * kMfX ? tid / kMfX : tid - 5 * kMfX);
    const bool pair = ny0 + 1 <= kMfY;
    const int node_i = ny0 * (kMfX + 1) + nx;    // index of (nx, ny0) in the node-plane buffers
    const int zb_node = ny0 * kTzX + nx + 3;     // its lower-left element in the staged halo plane
    const int wb_node = ny0 * kTwX + nx;
    bool ok = true, bad = false;
    uint32_t phase_bits = 0;   // parity of the next wait, per slot
    auto wait_slot = [&](int slot) {
        ok = tc::mbar_wait(&bar[slot], (phase_bits >> slot) & 1u, 1u << 22) && ok;
        phase_bits ^= 1u << slot;
    };
    // node values of two node planes ([d][row 0..2] around the thread's elements, the two columns
    // as one pair), used in turn as lower and upper
    float2 la[3][3], lb[3][3];
    float2 local2 = make_float2(0.f, 0.f);
    float2 xn = make_float2(0.f, 0.f);   // x of the two elements of the plane computed in the next step
    const float2 beta2 = make_float2(beta, beta), alpha2 = make_float2(alpha, alpha);
    if (nsteps > 0) wait_slot(0);
    // element offsets fit 32 bits (mf_launch takes this kernel only below 2^32 elements)
    const uint32_t exy32 = (uint32_t)exy, emax = (uint32_t)(exy * ez), ex32 = (uint32_t)ex;
    uint32_t e_prev = (uint32_t)(zlo - 1) * exy32 + (uint32_t)eo;   // element (tx, ty0) in plane kk - 1
    int s_cur = 0, s_prev = 0;                        // ring slots of stages t and t - 1
    auto step = [&](int t, float2 (&lo)[3][3], float2 (&hi)[3][3]) -> bool {
        const int kk = zlo - 1 + t;
        s_prev = s_cur;
        s_cur = s_cur + 1 == kTmRing ? 0 : s_cur + 1;
        wait_slot(s_cur);
        const unsigned char* st_prev = ring + s_prev * kTmStage;
        const unsigned char* st_cur = ring + s_cur * kTmStage;
        const float* zp = reinterpret_cast<const float*>(st_prev);            // element plane kk - 1
        const float* zc = reinterpret_cast<const float*>(st_cur);             // element plane kk
        const float* wc = reinterpret_cast<const float*>(st_cur + kTzSlot);
        float* yc = yb[t & 1][0];
        if (node) {
            // per staged element row r around the nodes, with A = plane kk - 1, B = plane kk and
            // columns nx - 1 (0) and nx (1), the pairs (A0, B0) and (A1, B1) give
            // d = (A1 - A0, B1 - B0) and s = (A0 + A1, B0 + B1), and from them sx = dA + dB,
            // ss = sA + sB, sz = sB - sA.  A node between rows r and r + 1 has
            // D_x = sx(r) + sx(r+1), D_y = ss(r+1) - ss(r), D_z = sz(r) + sz(r+1).
            float sx[3], sz[3], ss[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                if (r < 2 || pair) {
                    const int b = zb_node + r * kTzX;
                    const float2 c0 = make_float2(zp[b], zc[b]), c1 = make_float2(zp[b + 1], zc[b + 1]);
                    const float2 d = __ffma2_rn(c0, make_float2(-1.f, -1.f), c1);
                    const float2 sm = __fadd2_rn(c0, c1);
                    sx[r] = d.x + d.y;
                    sz[r] = sm.y - sm.x;
                    ss[r] = sm.x + sm.y;
                } else {
                    sx[r] = sz[r] = ss[r] = 0.f;
                }
            }
            // the two nodes as one pair: (ny0, ny0 + 1)
            const int w1 = pair ? kTwX : 0;
            const float2 yx = __fmul2_rn(make_float2(wc[wb_node], wc[wb_node + w1]),
                                         make_float2(sx[0] + sx[1], sx[1] + sx[2]));
            const float2 yy = __fmul2_rn(make_float2(wc[kTwX * kTwY + wb_node], wc[kTwX * kTwY + wb_node + w1]),
                                         make_float2(ss[1] - ss[0], ss[2] - ss[1]));
            const float2 yz = __fmul2_rn(make_float2(wc[2 * kTwX * kTwY + wb_node], wc[2 * kTwX * kTwY + wb_node + w1]),
                                         make_float2(sz[0] + sz[1], sz[1] + sz[2]));
            yc[node_i] = yx.x;
            yc[kTmNodes + node_i] = yy.x;
            yc[2 * kTmNodes + node_i] = yz.x;
            if (pair) {
                yc[node_i + kMfX + 1] = yx.y;
                yc[kTmNodes + node_i + kMfX + 1] = yy.y;
                yc[2 * kTmNodes + node_i + kMfX + 1] = yz.y;
            }
        }
        const float2 xc = xn;
        if (xupd && eok0 && kk < zhi) {
            xn.x = x[e_prev + exy32];
            xn.y = eok1 ? x[e_prev + exy32 + ex32] : 0.f;
        }
        ok = __syncthreads_and(ok) != 0;
        if (!ok) return false;
        // the next stage, t + kTmRing - 2, goes to the slot of stage t - 2, which every thread
        // finished reading before this barrier
        if (tid == 0 && issued < nsteps) issue(issued++);
        if (elem) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float* yr = yc + d * kTmNodes + ybase + r * (kMfX + 1);
                    hi[d][r] = make_float2(yr[0], yr[1]);
                }
            if (t >= 2 && eok0) {
                // per node row r, over its two columns: u0 = lo0 + hi0, u1 = lo1 + hi1,
                // u2 = lo2 - hi2, X = u0(0) - u0(1), S1 = u1(0) + u1(1), S2 = u2(0) + u2(1); the
                // element between rows r and r + 1 gets X(r) + X(r+1) + S1(r) - S1(r+1) + S2(r) + S2(r+1)
                float X[3], S1[3], S2[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float2 u0 = __fadd2_rn(lo[0][r], hi[0][r]);
                    const float2 u1 = __fadd2_rn(lo[1][r], hi[1][r]);
                    const float2 u2 = __ffma2_rn(hi[2][r], make_float2(-1.f, -1.f), lo[2][r]);
                    X[r] = u0.x - u0.y;
                    S1[r] = u1.x + u1.y;
                    S2[r] = u2.x + u2.y;
                }
                const float2 out = make_float2((X[0] + X[1]) + (S1[0] - S1[1]) + (S2[0] + S2[1]),
                                               (X[1] + X[2]) + (S1[1] - S1[2]) + (S2[1] + S2[2]));
                const float* pq_prev = reinterpret_cast<const float*>(st_prev + kTzSlot + kTwSlot);
                const int lt = ty0 * kMfX + tx;   // element (tx, ty0) in the tile's p, q planes
                const int zi = (ty0 + 1) * kTzX + tx + 4;
                // the second element's row lies outside the mesh when !eok1: its staged z, p and q
                // read as zero there, so it adds nothing to p.q and is not stored
                const float2 ze = make_float2(zp[zi], zp[zi + kTzX]);
                // p and q of element plane kk - 1 arrived with stage t - 1 (the slot of zp)
                const float2 pv = make_float2(pq_prev[lt], pq_prev[lt + kMfX]);
                const float2 qv = make_float2(pq_prev[kMfX * kMfY + lt], pq_prev[kMfX * kMfY + lt + kMfX]);
                const float2 pe = first ? ze : __ffma2_rn(beta2, pv, ze);
                const float2 qe = first ? out : __ffma2_rn(beta2, qv, out);
                const float2 xv = __ffma2_rn(alpha2, pv, xc);
                const uint32_t e1 = e_prev + ex32;
                if (e_prev < emax && (!eok1 || e1 < emax)) {
                    p[e_prev] = pe.x;
                    q[e_prev] = qe.x;
                    if (xupd) x[e_prev] = xv.x;
                    if (eok1) {
                        p[e1] = pe.y;
                        q[e1] = qe.y;
                        if (xupd) x[e1] = xv.y;
                    }
                } else {
                    bad = true;
                }
                local2 = __ffma2_rn(pe, qe, local2);
            }
        }
        e_prev += exy32;
        return true;
    };
    for (int t = 1; t < nsteps; t += 2) {
        if (!step(t, la, lb)) break;
        if (t + 1 < nsteps && !step(t + 1, lb, la)) break;
    }
    float local = local2.x + local2.y;
    if (bad) local = __int_as_float(0x7fc00000);
    if (!ok) {
        // let copies still in flight land before the block's shared memory is released
        if (tid == 0)
            for (int t = 0; t < kTmRing; ++t) tc::mbar_wait(&bar[t], (phase_bits >> t) & 1u, 1u << 16);
        local = __int_as_float(0x7fc00000);   // NaN: the host ends the solve
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *rr_slot(scal, k + 1) = 0.0;
    double tsum = block_sum<float>(local, sw);
    if (threadIdx.x == 0) atomicAdd(pq_slot(scal, k + 1), tsum);
    pdl_trigger();
}

// Build-time check of k_cg_mf3_dir_tma's thread roles, restating the kernel's mapping: every
// index a thread forms into the staged z plane, the staged weight plane, the node-plane buffers
// and the tile's p and q planes lies inside that buffer, every node of the 33 x 9 block is formed
// by exactly one thread, and every element of the 32 x 8 tile by exactly one.
constexpr bool mf_tma_roles_ok() {
    int nodes[kTmNodes] = {};
    int elems[kMfX * kMfY] = {};
    for (int tid = 0; tid < kTmThreads; ++tid) {
        if (tid < 5 * kMfX + 5) {
            const int nx = tid < 5 * kMfX ? tid % kMfX : kMfX;
            const int ny0 = 2 * (tid < 5 * kMfX ? tid / kMfX : tid - 5 * kMfX);
            const bool pair = ny0 + 1 <= kMfY;
            const int node_i = ny0 * (kMfX + 1) + nx, zb = ny0 * kTzX + nx + 3, wb = ny0 * kTwX + nx;
            for (int r = 0; r < 3; ++r)
                if ((r < 2 || pair) && zb + r * kTzX + 1 >= kTzX * kTzY) return false;
            if (2 * kTwX * kTwY + wb + (pair ? kTwX : 0) >= 3 * kTwX * kTwY) return false;
            if (node_i + (pair ? kMfX + 1 : 0) >= kTmNodes) return false;
            ++nodes[node_i];
            if (pair) ++nodes[node_i + kMfX + 1];
        }
        if (tid < kMfX * kMfY / 2) {
            const int tx = tid % kMfX, ty0 = 2 * (tid / kMfX);
            if (ty0 * (kMfX + 1) + tx + 2 * (kMfX + 1) + 1 >= kTmNodes) return false;
            if ((ty0 + 1) * kTzX + tx + 4 + kTzX >= kTzX * kTzY) return false;
            if (ty0 * kMfX + tx + kMfX >= kMfX * kMfY) return false;
            ++elems[ty0 * kMfX + tx];
            ++elems[(ty0 + 1) * kMfX + tx];
        }
    }
    for (int i = 0; i < kTmNodes; ++i)
        if (nodes[i] != 1) return false;
    for (int i = 0; i < kMfX * kMfY; ++i)
        if (elems[i] != 1) return false;
    return true;
}
static_assert(mf_tma_roles_ok(), "k_cg_mf3_dir_tma: a thread role leaves its buffer or misses a node or element");

// Wc_(n,d) = a_d^2 W_(n,d) in FP32 (the weights of the matrix-free apply).  2D: [d][node].  3D:
// rows padded to `pitch` nodes (a multiple of 4, so that every row starts on 16 bytes as the
// tensor-memory-access copies need), [d][z][y][pitch], the padding zero.
__global__ void k_mf_weights(int64_t nn, int dim, int64_t nnx, int64_t nny, int64_t pitch, int64_t dstride, double a0,
                             double a1, double a2, const double* __restrict__ W, float* __restrict__ Wc) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    if (dim == 2) {
        Wc[n] = (float)(a0 * a0 * W[n]);
        Wc[nn + n] = (float)(a1 * a1 * W[nn + n]);
        return;
    }
    const int64_t x = n % nnx, y = (n / nnx) % nny, z = n / (nnx * nny);
    const int64_t o = x + pitch * (y + nny * z);
    Wc[o] = (float)(a0 * a0 * W[n]);
    Wc[dstride + o] = (float)(a1 * a1 * W[nn + n]);
    Wc[2 * dstride + o] = (float)(a2 * a2 * W[2 * nn + n]);
}



// the launch of the matrix-free direction kernel: in 3D the deepest column chunk (up to 16
// element planes) that still gives four blocks per SM, at least 2 planes
struct MfLaunch {
    int dim;
    int ex, ey;
    int64_t nnx, nn;
    Mf3 a3;
    const float* Wc;
    unsigned blocks;
    // tensor-memory-access form (3D, x extent a multiple of 4): maps of z, Wc, p and q
    bool tma;
    const float* tma_z;
    const float* tma_p;
    const float* tma_q;
    CUtensorMap tz;
    CUtensorMap tw;
    CUtensorMap tp;
    CUtensorMap tq;
};

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
        else
            (void)cudaGetLastError();
    }
    return fn;
}

// z, p, q: the vectors the direction kernel will read and update (the tensor maps are bound to them)
static MfLaunch mf_launch(const MeshDesc& m, EGrid g, const float* Wc, const float* z, const float* p, const float* q,
                          int sms) {
    MfLaunch L{};
    L.dim = m.dim;
    L.ex = (int)g.ex;
    L.ey = (int)g.ey;
    L.nnx = m.nnx;
    L.nn = m.nn;
    L.Wc = Wc;
    const int64_t txy = ((g.ex + kMfX - 1) / kMfX) * ((g.ey + kMfY - 1) / kMfY);
    if (m.dim == 2) {
        L.blocks = (unsigned)txy;
        return L;
    }
    int zc = 16;
    while (zc > 2 && txy * ((g.ez + zc - 1) / zc) < 4 * (int64_t)sms) zc /= 2;
    const int64_t pitch = (m.nnx + 3) / 4 * 4;
    L.a3 = Mf3{(int)g.ex, (int)g.ey, (int)g.ez, zc, pitch, m.nny, pitch * m.nny * m.nnz};
    L.blocks = (unsigned)(txy * ((g.ez + zc - 1) / zc));
    L.tma = false;
    auto enc = tensor_map_encoder();
    auto al16 = [](const void* v) { return v && (reinterpret_cast<uintptr_t>(v) & 15) == 0; };
    if (enc && g.ex % 4 == 0 && g.ne < ((int64_t)1 << 32) && al16(z) && al16(Wc) && al16(p) && al16(q)) {
        const cuuint64_t zdim[3] = {(cuuint64_t)g.ex, (cuuint64_t)g.ey, (cuuint64_t)g.ez};
        const cuuint64_t zstr[2] = {(cuuint64_t)g.ex * 4, (cuuint64_t)g.ex * g.ey * 4};
        const cuuint32_t zbox[3] = {(cuuint32_t)kTzX, (cuuint32_t)kTzY, 1};
        const cuuint64_t wdim[4] = {(cuuint64_t)pitch, (cuuint64_t)m.nny, (cuuint64_t)m.nnz, 3};
        const cuuint64_t wstr[3] = {(cuuint64_t)pitch * 4, (cuuint64_t)pitch * m.nny * 4,
                                    (cuuint64_t)pitch * m.nny * m.nnz * 4};
        const cuuint32_t wbox[4] = {(cuuint32_t)kTwX, (cuuint32_t)kTwY, 1, 3};
        const cuuint32_t one[4] = {1, 1, 1, 1};
        CUresult r1 = enc(&L.tz, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(z), zdim, zstr, zbox, one,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        CUresult r2 = enc(&L.tw, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(Wc), wdim, wstr, wbox, one,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        const cuuint32_t pbox[3] = {(cuuint32_t)kMfX, (cuuint32_t)kMfY, 1};
        CUresult r3 = enc(&L.tp, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(p), zdim, zstr, pbox, one,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        CUresult r4 = enc(&L.tq, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(q), zdim, zstr, pbox, one,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        L.tma = r1 == CUDA_SUCCESS && r2 == CUDA_SUCCESS && r3 == CUDA_SUCCESS && r4 == CUDA_SUCCESS;
        // four blocks of about 46 KB each per SM: ask for the largest shared-memory carveout
        if (L.tma && cudaFuncSetAttribute(k_cg_mf3_dir_tma, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            (void)cudaGetLastError();
        L.tma_z = z;
        L.tma_p = p;
        L.tma_q = q;
    }
    return L;
}

// whether mf_dir runs the TMA kernel for these vectors (it then also updates x when given one)
static bool mf_tma(const MfLaunch& L, const float* z, const float* p, const float* q) {
    return L.dim == 3 && L.tma && z == L.tma_z && p == L.tma_p && q == L.tma_q;
}

static void mf_dir(const MfLaunch& L, cudaStream_t st, const float* z, float* p, float* q, double* scal, int k,
                   int first, float* x = nullptr) {
    const unsigned nt = kMfX * kMfY;
    if (L.dim == 2) launch_pdl(k_cg_mf2_dir, L.blocks, nt, st, L.ex, L.ey, L.nnx, L.nn, L.Wc, z, p, q, scal, k, first);
    else if (mf_tma(L, z, p, q))
        launch_pdl(k_cg_mf3_dir_tma, L.blocks, (unsigned)kTmThreads, st, L.a3, L.tz, L.tw, L.tp, L.tq, p, q, x, scal, k,
                   first);
    else launch_pdl(k_cg_mf3_dir, L.blocks, nt, st, L.a3, L.Wc, z, p, q, scal, k, first);
}

// ------------------------------------------------------------------------------------------
// Multigrid preconditioner for the inner solves (option bfbt_inner_pc = 1): the element grid is
// coarsened 2:1 per axis by aggregation (a coarse element is the union of its 2^dim children;
// prolongation copies the parent's value, restriction sums the children), the coarse operator
// is the Galerkin product P^T A P (again a 3^dim element stencil), smoothing is Chebyshev on
// Dinv A (degree 2 before and after the coarse correction, the same polynomial, so the V-cycle
// is symmetric), and the coarsest level is a dense inverse (with the constant projector added
// when the operator has the constant null space).
// ------------------------------------------------------------------------------------------

// Ac[Q][E] = sum over the children e of E and their entries q whose neighbour's parent is at
// offset Q from E of Af[q][e]
template <int DIM>
__global__ void k_gmg_coarsen(EGrid f, EGrid c, const double* __restrict__ Af, double* __restrict__ Ac) {
    constexpr int NB = stencil_points<DIM>();
    const int64_t E = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (E >= c.ne) return;
    const int64_t Ei[3] = {E % c.ex, (E / c.ex) % c.ey, DIM == 3 ? E / (c.ex * c.ey) : 0};
    const int64_t fc[3] = {f.ex, f.ey, f.ez};
    double acc[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) acc[q] = 0.0;
    for (int ch = 0; ch < (1 << DIM); ++ch) {
        const int64_t fi[3] = {2 * Ei[0] + (ch & 1), 2 * Ei[1] + ((ch >> 1) & 1), DIM == 3 ? 2 * Ei[2] + ((ch >> 2) & 1) : 0};
        const int64_t e = fi[0] + f.ex * (fi[1] + f.ey * fi[2]);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int o[3] = {q % 3 - 1, (q / 3) % 3 - 1, DIM == 3 ? q / 9 - 1 : 0};
            int Q = 0, mul = 1;
            bool valid = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const int64_t nb = fi[d] + o[d];
                valid = valid && nb >= 0 && nb < fc[d];
                const int64_t P = nb >= 0 ? nb / 2 : -1;   // parent of the neighbour (floor)
                Q += (int)(P - Ei[d] + 1) * mul;
                mul *= 3;
            }
            if (valid) acc[Q] += Af[(int64_t)q * f.ne + e];
        }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) Ac[(int64_t)q * c.ne + E] = acc[q];
}

__global__ void k_gmg_dinv(int64_t ne, int center, const double* __restrict__ A, double* __restrict__ dinv) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < ne) dinv[e] = 1.0 / A[(int64_t)center * ne + e];
}

// (A x)_e with clamped neighbour indices (entries towards missing neighbours are 0)
template <int DIM, typename T>
__device__ __forceinline__ T gmg_row(const EGrid& g, int64_t e, const T* __restrict__ A, const T* __restrict__ x) {
    constexpr int NB = stencil_points<DIM>();
    const int64_t exy = g.ex * g.ey;
    const int64_t ix = e % g.ex, iy = (e / g.ex) % g.ey, iz = DIM == 3 ? e / exy : 0;
    const int64_t dx[3] = {ix > 0 ? -1 : 0, 0, ix + 1 < g.ex ? 1 : 0};
    const int64_t dy[3] = {iy > 0 ? -g.ex : 0, 0, iy + 1 < g.ey ? g.ex : 0};
    const int64_t dz[3] = {DIM == 3 && iz > 0 ? -exy : 0, 0, DIM == 3 && iz + 1 < g.ez ? exy : 0};
    T a[NB], xv[NB];
#pragma unroll
    for (int t = 0; t < NB; ++t) a[t] = __ldg(A + (size_t)t * g.ne + e);
#pragma unroll
    for (int t = 0; t < NB; ++t) xv[t] = x[e + dx[t % 3] + dy[(t / 3) % 3] + dz[DIM == 3 ? t / 9 : 1]];
    T acc = (T)0;
#pragma unroll
    for (int t = 0; t < NB; ++t) acc = fma(a[t], xv[t], acc);
    return acc;
}

// r = b - A x
template <int DIM, typename T>
__global__ void k_gmg_resid(EGrid g, const T* __restrict__ A, const T* __restrict__ x, const T* __restrict__ b,
                            T* __restrict__ r) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < g.ne) r[e] = b[e] - gmg_row<DIM, T>(g, e, A, x);
}

// Chebyshev step on Dinv A: z = dinv (b - A xin); d = c1 d + c2 z (c2 z first); xout = xin + d
// (xin == nullptr: zero guess)
template <int DIM, typename T>
__global__ void k_gmg_cheb(EGrid g, const T* __restrict__ A, const T* __restrict__ dinv, const T* __restrict__ b,
                           const T* __restrict__ xin, T* __restrict__ xout, T* __restrict__ d, T c1, T c2, int first) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.ne) return;
    T res = b[e];
    if (xin) res -= gmg_row<DIM, T>(g, e, A, xin);
    const T z = res * dinv[e];
    const T dn = first ? c2 * z : fma(c1, d[e], c2 * z);
    d[e] = dn;
    xout[e] = (xin ? xin[e] : (T)0) + dn;
}

// y = dinv (A x) (power iteration for the Chebyshev bounds)
template <int DIM>
__global__ void k_gmg_dax(EGrid g, const double* __restrict__ A, const double* __restrict__ dinv,
                          const double* __restrict__ x, double* __restrict__ y) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < g.ne) y[e] = dinv[e] * gmg_row<DIM, double>(g, e, A, x);
}

template <int DIM, typename T>
__global__ void k_gmg_restrict(EGrid f, EGrid c, const T* __restrict__ rf, T* __restrict__ bc) {
    const int64_t E = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (E >= c.ne) return;
    const int64_t Ei[3] = {E % c.ex, (E / c.ex) % c.ey, DIM == 3 ? E / (c.ex * c.ey) : 0};
    T acc = (T)0;
#pragma unroll
    for (int ch = 0; ch < (1 << DIM); ++ch) {
        const int64_t e = (2 * Ei[0] + (ch & 1)) +
                          f.ex * ((2 * Ei[1] + ((ch >> 1) & 1)) + f.ey * (DIM == 3 ? 2 * Ei[2] + ((ch >> 2) & 1) : 0));
        acc += rf[e];
    }
    bc[E] = acc;
}

template <int DIM, typename T>
__global__ void k_gmg_prolong_add(EGrid f, EGrid c, const T* __restrict__ xc, T* __restrict__ xf) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= f.ne) return;
    const int64_t ix = e % f.ex, iy = (e / f.ex) % f.ey, iz = DIM == 3 ? e / (f.ex * f.ey) : 0;
    xf[e] += xc[(ix / 2) + c.ex * ((iy / 2) + c.ey * (iz / 2))];
}

// dense coarsest matrix from the stencil, plus `shift` in every entry (the constant projector)
template <int DIM>
__global__ void k_gmg_dense(EGrid g, const double* __restrict__ A, double shift, double* __restrict__ M) {
    constexpr int NB = stencil_points<DIM>();
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.ne) return;
    for (int64_t j = 0; j < g.ne; ++j) M[e * g.ne + j] = shift;
    const int64_t ix = e % g.ex, iy = (e / g.ex) % g.ey, iz = DIM == 3 ? e / (g.ex * g.ey) : 0;
    for (int q = 0; q < NB; ++q) {
        const int ox = q % 3 - 1, oy = (q / 3) % 3 - 1, oz = DIM == 3 ? q / 9 - 1 : 0;
        if (ix + ox < 0 || ix + ox >= g.ex || iy + oy < 0 || iy + oy >= g.ey ||
            (DIM == 3 && (iz + oz < 0 || iz + oz >= g.ez)))
            continue;
        M[e * g.ne + e + ox + g.ex * (oy + g.ey * oz)] += A[(int64_t)q * g.ne + e];
    }
}

// CG kernels with the multigrid preconditioner: the update leaves z to the V-cycle; the dot
// kernel accumulates rz_{k+1} = r.z afterwards
template <typename T>
__global__ void k_cgm_update(int64_t ne, const T* __restrict__ p, const T* __restrict__ q, T* __restrict__ x,
                             T* __restrict__ r, double* __restrict__ scal, int k, int want_rr) {
    __shared__ double sw[32];
    __shared__ T s_alpha;
    const T alpha = block_ratio<T>(rz_slot(scal, k), pq_slot(scal, k), &s_alpha);
    const int64_t base = (int64_t)blockIdx.x * blockDim.x * kEpt + threadIdx.x;
    T rr = (T)0;
#pragma unroll
    for (int m = 0; m < kEpt; ++m) {
        const int64_t e = base + (int64_t)m * blockDim.x;
        if (e < ne) {
            x[e] = fma(alpha, p[e], x[e]);
            const T re = fma(-alpha, q[e], r[e]);
            r[e] = re;
            rr = fma(re, re, rr);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *rz_slot(scal, k + 2) = 0.0;
        *pq_slot(scal, k + 1) = 0.0;
    }
    if (want_rr) {
        double t = block_sum<T>(rr, sw);
        if (threadIdx.x == 0) atomicAdd(rr_slot(scal, k), t);
    }
}

template <typename T>
__global__ void k_cgm_dot(int64_t ne, const T* __restrict__ r, const T* __restrict__ z, double* __restrict__ out) {
    __shared__ double sw[32];
    const int64_t base = (int64_t)blockIdx.x * blockDim.x * kEpt + threadIdx.x;
    T rz = (T)0;
#pragma unroll
    for (int m = 0; m < kEpt; ++m) {
        const int64_t e = base + (int64_t)m * blockDim.x;
        if (e < ne) rz = fma(r[e], z[e], rz);
    }
    double t = block_sum<T>(rz, sw);
    if (threadIdx.x == 0) atomicAdd(out, t);
}

// r = b (copied, T), x = 0 ; scal[7] = r0.r0
template <typename T>
__global__ void k_cgm_init(int64_t ne, const double* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                           double* __restrict__ scal) {
    __shared__ double sw[32];
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T rr = (T)0;
    if (e < ne) {
        const T re = (T)b[e];
        x[e] = (T)0;
        r[e] = re;
        rr = re * re;
    }
    double t = block_sum<T>(rr, sw);
    if (threadIdx.x == 0) atomicAdd(&scal[7], t);
}

EGrid egrid_of(const MeshDesc& m) {
    EGrid g;
    g.ex = m.nel[0];
    g.ey = m.nel[1];
    g.ez = m.dim == 3 ? m.nel[2] : 1;
    g.ne = g.ex * g.ey * g.ez;
    return g;
}


// ------------------------------------------------------------------------------------------
// Coarse correction of the Jacobi inner solves on plane checkerboards (3D, option 4).
// Q1-P0's spurious pressure modes make G^T W G nearly singular on element checkerboards: the
// checkerboard (-1)^(i+j) of one z plane, multiplied by anything along z, is mapped to zero by G
// away from the walls, and likewise for the other two axis pairs.  Jacobi removes them slowly, and
// more slowly the finer the mesh.  The coarse space holds, per family F, one vector per plane:
//   xy: v_k0(e) = (-1)^(i+j) [k = k0]   xz: v_j0(e) = (-1)^(i+k) [j = j0]   yz: v_i0(e) = (-1)^(j+k) [i = i0]
// and the preconditioner is additive and block-diagonal over the families,
//   M^-1 r = D^-1 r + sum_F Z_F E_F^-1 Z_F^T r,   E_F = Z_F^T A Z_F (tridiagonal, A couples
// neighbouring planes only), still symmetric positive definite, so CG keeps its form.  Per
// iteration: Z^T r (k_cc_sums), y = E^-1 Z^T r and the extra r.z term s.y (k_cc_small), z += Z y
// (k_cc_zcorr).  Layout of s and y: the xy family (ez entries), then xz (ey), then yz (ex).
// ------------------------------------------------------------------------------------------
struct CcArgs {
    int ex, ey, ez;
    const double* einv;   // E_F^-1, row-major blocks ez^2 | ey^2 | ex^2
    double* s;            // [2][ez + ey + ex]
    double* y;            // [ez + ey + ex]
};
constexpr int kCcMaxX = 512;   // largest x extent (the column sums live in registers, 32 per lane)

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// s = Z^T r into buffer (k + 1) & 1: one warp per x row (j, k), lanes along x.  The row's
// alternating sum alt = sum_i (-1)^i r gives both of its plane sums ((-1)^j alt to xy bin k,
// (-1)^k alt to xz bin j); the yz bins (per i) are summed per lane over the warp's rows, then per
// block in shared memory.
template <typename T, int M>
__global__ void __launch_bounds__(256) k_cc_sums(CcArgs a, const T* __restrict__ r, int k) {
    __shared__ double col[kCcMaxX];
    pdl_wait();
    for (int i = threadIdx.x; i < a.ex; i += blockDim.x) col[i] = 0.0;
    __syncthreads();
    double* sb = a.s + (size_t)((k + 1) & 1) * (size_t)(a.ex + a.ey + a.ez);
    double* sxy = sb;
    double* sxz = sb + a.ez;
    double* syz = sb + a.ez + a.ey;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rows = a.ey * a.ez;
    double cacc[M];
#pragma unroll
    for (int m = 0; m < M; ++m) cacc[m] = 0.0;
    for (int row = blockIdx.x * 8 + warp; row < rows; row += gridDim.x * 8) {
        const int j = row % a.ey, kz = row / a.ey;
        const T* rr = r + (int64_t)row * a.ex;
        const bool neg = ((j + kz) & 1) != 0;
        double alt = 0.0;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const int i = lane + 32 * m;
            if (i < a.ex) {
                const double v = (double)rr[i];
                alt += (i & 1) ? -v : v;
                cacc[m] += neg ? -v : v;
            }
        }
        alt = warp_sum_d(alt);
        if (lane == 0) {
            atomicAdd(sxy + kz, (j & 1) ? -alt : alt);
            atomicAdd(sxz + j, (kz & 1) ? -alt : alt);
        }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const int i = lane + 32 * m;
        if (i < a.ex) atomicAdd(&col[i], cacc[m]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < a.ex; i += blockDim.x) atomicAdd(syz + i, col[i]);
    pdl_trigger();
}

// y = E^-1 s (one warp per coarse unknown), rz_{k+1} += s . y, and the other s buffer cleared for
// the next iteration
__global__ void __launch_bounds__(256) k_cc_small(CcArgs a, double* __restrict__ scal, int k) {
    __shared__ double sw[8];
    pdl_wait();
    const int n = a.ex + a.ey + a.ez;
    const double* sb = a.s + (size_t)((k + 1) & 1) * (size_t)n;
    double* so = a.s + (size_t)(k & 1) * (size_t)n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int b = blockIdx.x * 8 + warp;
    double part = 0.0;
    if (b < n) {
        int off, len;
        const double* E;
        if (b < a.ez) {
            off = 0;
            len = a.ez;
            E = a.einv + (size_t)b * a.ez;
        } else if (b < a.ez + a.ey) {
            off = a.ez;
            len = a.ey;
            E = a.einv + (size_t)a.ez * a.ez + (size_t)(b - off) * a.ey;
        } else {
            off = a.ez + a.ey;
            len = a.ex;
            E = a.einv + (size_t)a.ez * a.ez + (size_t)a.ey * a.ey + (size_t)(b - off) * a.ex;
        }
        double acc = 0.0;
        for (int cc = lane; cc < len; cc += 32) acc = fma(E[cc], sb[off + cc], acc);
        acc = warp_sum_d(acc);
        if (lane == 0) {
            a.y[b] = acc;
            part = acc * sb[b];
        }
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) so[t] = 0.0;
    if (lane == 0) sw[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += sw[w];
        if (t != 0.0) atomicAdd(rz_slot(scal, k + 1), t);
    }
    pdl_trigger();
}

// z += Z y: grid (x-y plane chunks, z planes)
template <typename T>
__global__ void __launch_bounds__(256) k_cc_zcorr(CcArgs a, T* __restrict__ z) {
    pdl_wait();
    const int pxy = blockIdx.x * blockDim.x + threadIdx.x, kz = blockIdx.y;
    if (pxy < a.ex * a.ey) {
        const int i = pxy % a.ex, j = pxy / a.ex;
        const double yxy = a.y[kz], yxz = a.y[a.ez + j], yyz = a.y[a.ez + a.ey + i];
        const double v = (((i + j) & 1) ? -yxy : yxy) + (((i + kz) & 1) ? -yxz : yxz) + (((j + kz) & 1) ? -yyz : yyz);
        const int64_t e = (int64_t)kz * a.ex * a.ey + pxy;
        z[e] = (T)((double)z[e] + v);
    }
    pdl_trigger();
}

// The three diagonals of every E_F from the element stencil A[q][e] (q = (dx+1) + 3 (dy+1) +
// 9 (dz+1), zero towards neighbours outside the mesh): E_xy[k][k+dz] = sum over the elements e of
// plane k and their neighbours f at dz of A_ef (-1)^(dx+dy) (the product of the two checkerboard
// signs), and the same for xz (offset dy, sign (-1)^(dx+dz)) and yz (offset dx, sign
// (-1)^(dy+dz)).  ed: [xy: ez][3] | [xz: ey][3] | [yz: ex][3].  One warp per x row.
template <int M>
__global__ void __launch_bounds__(256) k_cc_build(EGrid g, const double* __restrict__ A, double* __restrict__ ed) {
    __shared__ double col[kCcMaxX * 3];
    const int ex = (int)g.ex, ey = (int)g.ey, ez = (int)g.ez;
    for (int i = threadIdx.x; i < 3 * ex; i += blockDim.x) col[i] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rows = ey * ez;
    double cacc[M][3];
#pragma unroll
    for (int m = 0; m < M; ++m) cacc[m][0] = cacc[m][1] = cacc[m][2] = 0.0;
    for (int row = blockIdx.x * 8 + warp; row < rows; row += gridDim.x * 8) {
        const int j = row % ey, kz = row / ey;
        double vxy[3] = {0.0, 0.0, 0.0}, vxz[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const int i = lane + 32 * m;
            if (i < ex) {
                const int64_t e = (int64_t)row * ex + i;
                for (int q = 0; q < 27; ++q) {
                    const int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = q / 9 - 1;
                    const double v = A[(int64_t)q * g.ne + e];
                    vxy[dz + 1] += ((dx + dy) & 1) ? -v : v;
                    vxz[dy + 1] += ((dx + dz) & 1) ? -v : v;
                    cacc[m][dx + 1] += ((dy + dz) & 1) ? -v : v;
                }
            }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double sxy = warp_sum_d(vxy[d]), sxz = warp_sum_d(vxz[d]);
            if (lane == 0) {
                atomicAdd(ed + kz * 3 + d, sxy);
                atomicAdd(ed + 3 * ez + j * 3 + d, sxz);
            }
        }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const int i = lane + 32 * m;
        if (i < ex)
            for (int d = 0; d < 3; ++d) atomicAdd(&col[i * 3 + d], cacc[m][d]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * ex; t += blockDim.x) atomicAdd(ed + 3 * (ez + ey) + t, col[t]);
}

CcArgs cc_args(Context& c) {
    return CcArgs{c.cc.ex, c.cc.ey, c.cc.ez, c.cc.einv.p, c.cc.s.p, c.cc.y.p};
}

template <typename T>
void cc_sums_launch(Context& c, const T* r, int k) {
    const CcArgs a = cc_args(c);
    const unsigned blocks = (unsigned)std::min<int64_t>(((int64_t)a.ey * a.ez + 7) / 8, 256);
    if (a.ex <= 128) launch_pdl(k_cc_sums<T, 4>, blocks, 256u, c.stream, a, r, k);
    else if (a.ex <= 256) launch_pdl(k_cc_sums<T, 8>, blocks, 256u, c.stream, a, r, k);
    else launch_pdl(k_cc_sums<T, 16>, blocks, 256u, c.stream, a, r, k);
}

// the correction of iteration k: s = Z^T r, y = E^-1 s (and rz_{k+1} += s.y), z += Z y
template <typename T>
void cc_apply(Context& c, const T* r, T* z, double* scal, int k) {
    const CcArgs a = cc_args(c);
    cc_sums_launch<T>(c, r, k);
    launch_pdl(k_cc_small, (unsigned)((a.ex + a.ey + a.ez + 7) / 8), 256u, c.stream, a, scal, k);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((a.ex * a.ey + 255) / 256), (unsigned)a.ez);
    cfg.blockDim = dim3(256);
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    UWG_CUDA(cudaLaunchKernelEx(&cfg, k_cc_zcorr<T>, a, z));
}

}  // namespace

// Builds the FP64 stencil A (stencil_points * ne values, entry-major) and dinv = 1/diag for the
// velocity weights W (SoA [d][node]; fixed dofs excluded).
void gwg_stencil_build(Context& c, const double* W, double* A, double* dinv) {
    const Level& L = c.levels[0];
    const MeshDesc& m = L.mesh;
    EGrid g = egrid_of(m);
    UWG_REQUIRE(g.ne * (m.dim == 3 ? 27 : 9) < (int64_t)1 << 31, UWGPU_ERR_TOO_LARGE,
                "BFBt stencil: element count too large for 32-bit stencil indexing");
    int off[3];
    const double* h = fine_widths(c, off);
    {
        LaunchScope ls(c, -1);
        if (m.dim == 3)
            k_gwg_build<3><<<blocks_for(g.ne, 128), 128, 0, c.stream>>>(g, h, off[1], off[2], m.nnx, m.nny, m.nn, W,
                                                                        L.fixed.p, A, dinv);
        else
            k_gwg_build<2><<<blocks_for(g.ne, 128), 128, 0, c.stream>>>(g, h, off[1], off[2], m.nnx, m.nny, m.nn, W,
                                                                        L.fixed.p, A, dinv);
    }
    check_launch("k_gwg_build");
}

// FP32 copies of the stencil (skipped when A32 is null) and the inverse diagonal (mixed form)
void gwg_stencil_fp32(Context& c, const double* A, const double* dinv, float* A32, float* dinv32) {
    const MeshDesc& m = c.levels[0].mesh;
    int64_t ne = m.ne, na = ne * (m.dim == 3 ? 27 : 9);
    LaunchScope ls(c, -1);
    if (A32) k_gwg_convert<double, float><<<blocks_for(na, 256), 256, 0, c.stream>>>(na, A, A32);
    k_gwg_convert<double, float><<<blocks_for(ne, 256), 256, 0, c.stream>>>(ne, dinv, dinv32);
    c.launches++;
    check_launch("k_gwg_convert");
}

// y = A x (FP64); scal receives the unused p.q accumulators (8 doubles)
void gwg_stencil_apply(Context& c, const double* A, const double* x, double* y, double* scal) {
    const MeshDesc& m = c.levels[0].mesh;
    EGrid g = egrid_of(m);
    UWG_CUDA(cudaMemsetAsync(scal, 0, 8 * sizeof(double), c.stream));
    LaunchScope ls(c, -1);
    if (m.dim == 3) k_gwg_spmv<3, double><<<blocks_for(g.ne, 256), 256, 0, c.stream>>>(g, A, x, y, scal, 0);
    else k_gwg_spmv<2, double><<<blocks_for(g.ne, 256), 256, 0, c.stream>>>(g, A, x, y, scal, 0);
    check_launch("k_gwg_spmv");
}

// Builds the plane-checkerboard coarse correction for the FP64 element stencil A of G^T W G (3D):
// the tridiagonal E_F from the stencil on the device, their inverses on the host (column by column
// with the tridiagonal LDL^T factors; n^2 per family), and the device buffers.  Returns false (the
// inner solves keep plain Jacobi) in 2D, on meshes wider than 512 elements along x, or when an
// E_F is not positive definite.
bool gwg_cc_build(Context& c, const double* A) {
    const MeshDesc& m = c.levels[0].mesh;
    c.cc.on = false;
    if (m.dim != 3) return false;
    const EGrid g = egrid_of(m);
    if (g.ex > kCcMaxX || g.ey > 4096 || g.ez > 4096) return false;
    const int ex = (int)g.ex, ey = (int)g.ey, ez = (int)g.ez, n = ex + ey + ez;
    c.cc.ed.ensure((size_t)3 * n);
    UWG_CUDA(cudaMemsetAsync(c.cc.ed.p, 0, sizeof(double) * 3 * n, c.stream));
    {
        LaunchScope ls(c, -1);
        const unsigned blocks = (unsigned)std::min<int64_t>(((int64_t)ey * ez + 7) / 8, 1024);
        if (ex <= 128) k_cc_build<4><<<blocks, 256, 0, c.stream>>>(g, A, c.cc.ed.p);
        else if (ex <= 256) k_cc_build<8><<<blocks, 256, 0, c.stream>>>(g, A, c.cc.ed.p);
        else k_cc_build<16><<<blocks, 256, 0, c.stream>>>(g, A, c.cc.ed.p);
    }
    check_launch("k_cc_build");
    std::vector<double> ed((size_t)3 * n);
    UWG_CUDA(cudaMemcpyAsync(ed.data(), c.cc.ed.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> einv((size_t)ez * ez + (size_t)ey * ey + (size_t)ex * ex);
    const int lens[3] = {ez, ey, ex};
    size_t eoff = 0;
    int doff = 0;
    for (int f = 0; f < 3; ++f) {
        const int len = lens[f];
        const double* d3 = ed.data() + 3 * doff;
        // symmetric tridiagonal: diagonal d3[b][1], off-diagonal between b and b + 1 the mean of
        // d3[b][2] and d3[b + 1][0] (equal up to rounding, A being symmetric)
        std::vector<double> dg(len), od(len > 1 ? len - 1 : 1, 0.0);
        for (int b = 0; b < len; ++b) dg[b] = d3[3 * b + 1];
        for (int b = 0; b + 1 < len; ++b) od[b] = 0.5 * (d3[3 * b + 2] + d3[3 * (b + 1)]);
        // LDL^T: l[b] below the diagonal, D[b]
        std::vector<double> D(len), l(len, 0.0);
        double dmax = 0.0;
        for (int b = 0; b < len; ++b) dmax = std::max(dmax, std::fabs(dg[b]));
        for (int b = 0; b < len; ++b) {
            D[b] = dg[b] - (b > 0 ? l[b - 1] * od[b - 1] : 0.0);
            if (!(D[b] > 1e-12 * dmax)) return false;
            if (b + 1 < len) l[b] = od[b] / D[b];
        }
        // columns of the inverse: L D L^T x = e_col
        double* Ei = einv.data() + eoff;
        std::vector<double> x(len);
        for (int col = 0; col < len; ++col) {
            for (int b = 0; b < len; ++b) x[b] = b == col ? 1.0 : 0.0;
            for (int b = 1; b < len; ++b) x[b] -= l[b - 1] * x[b - 1];
            for (int b = 0; b < len; ++b) x[b] /= D[b];
            for (int b = len - 2; b >= 0; --b) x[b] -= l[b] * x[b + 1];
            for (int b = 0; b < len; ++b) Ei[(size_t)b * len + col] = x[b];
        }
        eoff += (size_t)len * len;
        doff += len;
    }
    c.cc.einv.ensure(einv.size());
    c.cc.s.ensure((size_t)2 * n);
    c.cc.y.ensure((size_t)n);
    UWG_CUDA(cudaMemcpyAsync(c.cc.einv.p, einv.data(), sizeof(double) * einv.size(), cudaMemcpyHostToDevice, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));   // the host copy is released on return
    c.cc.ex = ex;
    c.cc.ey = ey;
    c.cc.ez = ez;
    c.cc.on = true;
    return true;
}

// Solves A x = b (b projected off the constant by the caller when A has it) to
// ||r|| <= rtol ||b|| by Jacobi-preconditioned CG.  work holds 4*ne values of T, scal 8 doubles.
// With Wmf (FP32 only) A is applied matrix-free from the nodal weights instead of the stencil.
// Returns the iterations taken.
template <typename T>
static int gwg_cg_T(Context& c, const T* A, const float* Wmf, const T* dinv, const double* b, T* x, double rtol,
                    int maxit, T* work, double* scal) {
    const MeshDesc& m = c.levels[0].mesh;
    EGrid g = egrid_of(m);
    const int64_t ne = g.ne;
    const int nb = m.dim == 3 ? 27 : 9;
    MfLaunch mf{};
    if (Wmf) {
        int sms = 0;
        UWG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
        const float* w32 = reinterpret_cast<const float*>(work);
        mf = mf_launch(m, g, Wmf, w32 + ne, w32 + 2 * ne, w32 + 3 * ne, sms);
    }
    T* r = work;
    T* z = work + ne;
    T* p = work + 2 * ne;
    T* q = work + 3 * ne;
    const unsigned eb = blocks_for(ne, 256), ebv = blocks_for(ne, 256 * kEpt);
    // direction kernel of iteration k: p = z + beta p, q = A z + beta q, pq_{k+1}
    // the TMA direction kernel also updates x (x += alpha p with the p it reads), so the update
    // kernel then leaves x and p alone
    bool fused_x = false;
    if constexpr (std::is_same<T, float>::value) fused_x = Wmf && mf_tma(mf, z, p, q);
    auto dir = [&](int k, int first) {
        if constexpr (std::is_same<T, float>::value) {
            if (Wmf) {
                mf_dir(mf, c.stream, z, p, q, scal, k, first, fused_x ? x : nullptr);
                return;
            }
        }
        if (m.dim == 3) launch_pdl(k_cg_spmv_dir<3, T>, eb, 256, c.stream, g, A, z, p, q, scal, k, first);
        else launch_pdl(k_cg_spmv_dir<2, T>, eb, 256, c.stream, g, A, z, p, q, scal, k, first);
    };
    // the plane-checkerboard coarse correction, when the solver built it for this operator
    const bool cc = c.cc.on && m.dim == 3 && c.cc.ex == g.ex && c.cc.ey == g.ey && c.cc.ez == g.ez;
    UWG_CUDA(cudaMemsetAsync(scal, 0, 8 * sizeof(double), c.stream));
    if (cc) UWG_CUDA(cudaMemsetAsync(c.cc.s.p, 0, c.cc.s.n * sizeof(double), c.stream));
    {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_gwg_init<T><<<eb, 256, 0, c.stream>>>(ne, b, dinv, x, r, z, scal);
        if (cc) cc_apply<T>(c, r, z, scal, -1);
    }
    {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        dir(-1, 1);
    }
    double* hs = c.host_scalars;
    UWG_CUDA(cudaMemcpyAsync(hs, scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    const double r0 = std::sqrt(hs[7]);
    if (!(r0 > 0.0)) return 0;
    // Twelve iterations (the rz slots cycle with period 3, pq and rr with period 2) form one CUDA
    // graph per buffer set, replayed until converged; the host checks the residual once per replay.
    const int block = 12;
    auto issue = [&](int k) {
        launch_pdl(k_cg_update<T>, blocks_for(ne, kUpdThreads * kUpdEpt), (unsigned)kUpdThreads, c.stream, ne, p, q, dinv,
                   x, r, z, scal, k, (int)(k == block - 1), (int)!fused_x);
        if (cc) cc_apply<T>(c, r, z, scal, k);
        dir(k, 0);
    };
    const void* key[9] = {Wmf ? (const void*)Wmf : (const void*)A, dinv, x, work, scal, (const void*)(intptr_t)ne,
                          (const void*)(intptr_t)sizeof(T), (const void*)(intptr_t)(m.dim + (Wmf ? 48 : 16)),
                          cc ? (const void*)c.cc.einv.p : nullptr};
    Context::PcgGraph* pg = nullptr;
    for (auto& cand : c.pcg_graphs)
        if (std::equal(std::begin(key), std::end(key), std::begin(cand.key))) pg = &cand;
    if (!pg) {
        c.pcg_graphs.emplace_back();
        pg = &c.pcg_graphs.back();
        std::copy(std::begin(key), std::end(key), std::begin(pg->key));
        cudaGraph_t graph;
        UWG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < block; ++k) issue(k);
        UWG_CUDA(cudaStreamEndCapture(c.stream, &graph));
        UWG_CUDA(cudaGraphInstantiate(&pg->exec, graph, 0));
        UWG_CUDA(cudaGraphDestroy(graph));
    }
    // algorithmic traffic of one iteration: update (p, q, dinv, x, r read; x, r, z written) and
    // spmv+direction (the stencil, z, p, q read; p, q written; matrix-free: the dim nodal
    // weights of about one node per element in place of the stencil)
    const double it_bytes = (double)ne * sizeof(T) * (8 + (Wmf ? m.dim : nb) + 5 + (cc ? 3 : 0));
    const double it_flops = Wmf ? (double)ne * (m.dim == 3 ? 110.0 : 46.0) : (double)ne * (2.0 * nb + 14.0);
    int it = 0;
    while (it < maxit) {
        {
            LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
            UWG_CUDA(cudaGraphLaunch(pg->exec, c.stream));
        }
        note_work(c, UWGPU_KERNEL_SCHUR_PC, block * it_bytes, block * it_flops);
        c.launches += (cc ? 5 : 2) * block - 1;
        it += block;
        UWG_CUDA(cudaMemcpyAsync(hs, scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        const double rn = std::sqrt(hs[6]);   // rr of the block's last iteration (k = 11: slot 5 + 1)
        if (!std::isfinite(rn)) throw Error(UWGPU_ERR_NAN, "NaN in the BFBt inner solve");
        if (rn <= rtol * r0) break;
    }
    check_launch("gwg_cg");
    return it;
}

int gwg_cg(Context& c, const double* A, const double* dinv, const double* b, double* x, double rtol, int maxit,
           double* work, double* scal) {
    return gwg_cg_T<double>(c, A, nullptr, dinv, b, x, rtol, maxit, work, scal);
}

int gwg_cg32(Context& c, const float* A, const float* dinv, const double* b, float* x, double rtol, int maxit,
             float* work, double* scal) {
    return gwg_cg_T<float>(c, A, nullptr, dinv, b, x, rtol, maxit, work, scal);
}

// the mixed form's inner solve: G^T W G applied matrix-free from the folded weights Wc
// (gwg_mf_weights)
int gwg_cg32_mf(Context& c, const float* Wc, const float* dinv, const double* b, float* x, double rtol, int maxit,
                float* work, double* scal) {
    return gwg_cg_T<float>(c, nullptr, Wc, dinv, b, x, rtol, maxit, work, scal);
}

// Entries of the folded-weight array of the matrix-free apply (3D rows padded, see k_mf_weights).
int64_t mf_weights_size(const MeshDesc& m) {
    if (m.dim == 2) return m.nn * 2;
    const int64_t pitch = (m.nnx + 3) / 4 * 4;
    return 3 * pitch * m.nny * m.nnz;
}

// the folded weights of the matrix-free apply, Wc_(n,d) = a_d^2 W_(n,d) (FP32), for the uniform
// mesh's a_d = prod_{k != d} h_k / 2^(dim-1)
void gwg_mf_weights(Context& c, const double* W, float* Wc) {
    const MeshDesc& m = c.levels[0].mesh;
    double h[3] = {1.0, 1.0, 1.0};
    for (int d = 0; d < m.dim; ++d) h[d] = (m.max[d] - m.min[d]) / m.nel[d];
    const double sc = m.dim == 3 ? 0.25 : 0.5;
    double a[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < m.dim; ++d) {
        a[d] = sc;
        for (int k = 0; k < m.dim; ++k)
            if (k != d) a[d] *= h[k];
    }
    const int64_t pitch = (m.nnx + 3) / 4 * 4, dstride = pitch * m.nny * m.nnz;
    if (m.dim == 3) UWG_CUDA(cudaMemsetAsync(Wc, 0, (size_t)mf_weights_size(m) * sizeof(float), c.stream));
    LaunchScope ls(c, -1);
    k_mf_weights<<<blocks_for(m.nn, 256), 256, 0, c.stream>>>(m.nn, m.dim, m.nnx, m.nny, pitch, dstride, a[0], a[1],
                                                              a[2], W, Wc);
    check_launch("k_mf_weights");
}

// Test and timing hook on the inner operator of the current fine velocity operator: W, the FP64
// stencil and (form 2) its FP32 copy are built here, then the direction kernel of the inner CG
// runs with p = z, q = A z in the given form (0: FP64 stencil, 1: FP32 matrix-free, 2: FP32
// stencil).  With xh, y = A x is returned in yh; with iterations > 0 the kernel is launched that
// many times back to back and the elapsed device time is returned in ms.
void bfbt_operator_hook(Context& c, int form, const double* xh, double* yh, int iterations, double* ms) {
    UWG_REQUIRE(c.operator_built, UWGPU_ERR_STATE, "the fine velocity operator is not built (solve first)");
    UWG_REQUIRE(form >= 0 && form <= 2, UWGPU_ERR_ARGUMENT, "form must be 0, 1 or 2");
    const MeshDesc& m = c.levels[0].mesh;
    const EGrid g = egrid_of(m);
    const int nb = m.dim == 3 ? 27 : 9;
    const int64_t ne = g.ne, nv = m.nn * m.dim;
    UWG_REQUIRE(ne * nb < (int64_t)1 << 31, UWGPU_ERR_TOO_LARGE, "BFBt stencil: element count too large");
    DArray<double> W, A, dinv, x, pq, scal;
    DArray<float> W32, A32, x32, pq32;
    W.ensure((size_t)nv);
    A.ensure((size_t)nb * ne);
    dinv.ensure((size_t)ne);
    x.ensure((size_t)ne);
    pq.ensure((size_t)2 * ne);
    scal.ensure(8);
    bfbt_weights(c, W.p);
    gwg_stencil_build(c, W.p, A.p, dinv.p);
    if (xh) UWG_CUDA(cudaMemcpyAsync(x.p, xh, (size_t)ne * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    else UWG_CUDA(cudaMemsetAsync(x.p, 0, (size_t)ne * sizeof(double), c.stream));
    MfLaunch mf{};
    if (form != 0) {
        x32.ensure((size_t)ne);
        pq32.ensure((size_t)2 * ne);
        to_float(c, x.p, x32.p, ne);
        if (form == 1) {
            W32.ensure((size_t)mf_weights_size(m));
            gwg_mf_weights(c, W.p, W32.p);
            int sms = 0;
            UWG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
            mf = mf_launch(m, g, W32.p, x32.p, pq32.p, pq32.p + ne, sms);
        } else {
            A32.ensure((size_t)nb * ne);
            to_float(c, A.p, A32.p, (int64_t)nb * ne);
        }
    }
    auto launch = [&]() {
        const unsigned eb = blocks_for(ne, 256);
        if (form == 1) mf_dir(mf, c.stream, x32.p, pq32.p, pq32.p + ne, scal.p, -1, 1);
        else if (form == 2 && m.dim == 3) k_cg_spmv_dir<3, float><<<eb, 256, 0, c.stream>>>(g, A32.p, x32.p, pq32.p, pq32.p + ne, scal.p, -1, 1);
        else if (form == 2) k_cg_spmv_dir<2, float><<<eb, 256, 0, c.stream>>>(g, A32.p, x32.p, pq32.p, pq32.p + ne, scal.p, -1, 1);
        else if (m.dim == 3) k_cg_spmv_dir<3, double><<<eb, 256, 0, c.stream>>>(g, A.p, x.p, pq.p, pq.p + ne, scal.p, -1, 1);
        else k_cg_spmv_dir<2, double><<<eb, 256, 0, c.stream>>>(g, A.p, x.p, pq.p, pq.p + ne, scal.p, -1, 1);
    };
    UWG_CUDA(cudaMemsetAsync(scal.p, 0, 8 * sizeof(double), c.stream));
    launch();
    check_launch("bfbt operator hook");
    if (yh) {
        if (form != 0) to_double(c, pq32.p + ne, pq.p + ne, ne);
        UWG_CUDA(cudaMemcpyAsync(yh, pq.p + ne, (size_t)ne * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    }
    if (iterations > 0 && ms) {
        cudaEvent_t e0, e1;
        UWG_CUDA(cudaEventCreate(&e0));
        UWG_CUDA(cudaEventCreate(&e1));
        UWG_CUDA(cudaEventRecord(e0, c.stream));
        for (int i = 0; i < iterations; ++i) launch();
        UWG_CUDA(cudaEventRecord(e1, c.stream));
        UWG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        UWG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check_launch("bfbt operator hook timing");
        *ms = t;
        c.launches += iterations;
    }
    UWG_CUDA(cudaStreamSynchronize(c.stream));
}

// ---- multigrid hierarchy for G^T W G ----------------------------------------------------
void dense_inverse(Context& c, double* M, int64_t n);                      // operator.cu
template <typename T> void dense_apply(Context& c, const double* M, int64_t n, const T* b, T* x);

static EGrid egrid_level(const Context::GwgLevel& L) {
    EGrid g;
    g.ex = L.ex;
    g.ey = L.ey;
    g.ez = L.ez;
    g.ne = L.ne;
    return g;
}

// Builds the coarse levels, Chebyshev bounds and the coarsest inverse for the fine stencil A0
// (its inverse diagonal dinv0).  Returns false when the mesh does not coarsen to a dense size
// that fits (the caller keeps the Jacobi preconditioner then).
bool gwg_mg_build(Context& c, const double* A0, const double* dinv0, bool need32, bool const_null) {
    const MeshDesc& m = c.levels[0].mesh;
    // captured V-cycles carry this hierarchy's Chebyshev coefficients: drop them
    for (auto it = c.pcg_graphs.begin(); it != c.pcg_graphs.end();) {
        if ((intptr_t)it->key[7] >= 32 && (intptr_t)it->key[7] < 48) {
            if (it->exec) cudaGraphExecDestroy(it->exec);
            it = c.pcg_graphs.erase(it);
        } else {
            ++it;
        }
    }
    const int dim = m.dim, nb = dim == 3 ? 27 : 9;
    EGrid g = egrid_of(m);
    int nlev = 1;
    {
        auto& L0 = c.gwg[0];
        L0.ex = g.ex;
        L0.ey = g.ey;
        L0.ez = g.ez;
        L0.ne = g.ne;
    }
    while (nlev < kMaxLevels) {
        const auto& F = c.gwg[nlev - 1];
        const bool even = F.ex % 2 == 0 && F.ey % 2 == 0 && (dim == 2 || F.ez % 2 == 0);
        if (!even || F.ne <= 512) break;
        auto& C = c.gwg[nlev];
        C.ex = F.ex / 2;
        C.ey = F.ey / 2;
        C.ez = dim == 3 ? F.ez / 2 : 1;
        C.ne = C.ex * C.ey * C.ez;
        nlev++;
    }
    const auto& Lc = c.gwg[nlev - 1];
    if (Lc.ne > 4096) return false;
    c.gwg_nlev = nlev;
    // coarse stencils (FP64)
    for (int l = 1; l < nlev; ++l) {
        auto& C = c.gwg[l];
        C.A64.ensure((size_t)nb * C.ne);
        C.dinv64.ensure((size_t)C.ne);
        const double* Af = l == 1 ? A0 : c.gwg[l - 1].A64.p;
        LaunchScope ls(c, -1);
        if (dim == 3) k_gmg_coarsen<3><<<blocks_for(C.ne, 128), 128, 0, c.stream>>>(egrid_level(c.gwg[l - 1]), egrid_level(C), Af, C.A64.p);
        else k_gmg_coarsen<2><<<blocks_for(C.ne, 128), 128, 0, c.stream>>>(egrid_level(c.gwg[l - 1]), egrid_level(C), Af, C.A64.p);
        k_gmg_dinv<<<blocks_for(C.ne, 256), 256, 0, c.stream>>>(C.ne, nb / 2, C.A64.p, C.dinv64.p);
        c.launches++;
    }
    check_launch("k_gmg_coarsen");
    // work vectors
    for (int l = 0; l < nlev; ++l) {
        auto& L = c.gwg[l];
        for (auto* a : {&L.b64, &L.x64, &L.r64, &L.t64, &L.d64}) a->ensure((size_t)L.ne);
        if (need32)
            for (auto* a : {&L.b32, &L.x32, &L.r32, &L.t32, &L.d32}) a->ensure((size_t)L.ne);
    }
    // Chebyshev bounds: largest eigenvalue of Dinv A per smoothed level (power iteration)
    for (int l = 0; l + 1 < nlev; ++l) {
        auto& L = c.gwg[l];
        const double* A = l == 0 ? A0 : L.A64.p;
        const double* dinv = l == 0 ? dinv0 : L.dinv64.p;
        const EGrid gl = egrid_level(L);
        std::vector<double> h((size_t)L.ne);
        for (int64_t e = 0; e < L.ne; ++e) h[(size_t)e] = (double)((e * 2654435761ull >> 7) & 1023ull) / 1023.0 - 0.5;
        UWG_CUDA(cudaMemcpyAsync(L.x64.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        double lam = 1.0;
        for (int it = 0; it < 12; ++it) {
            {
                LaunchScope ls(c, -1);
                if (dim == 3) k_gmg_dax<3><<<blocks_for(L.ne, 256), 256, 0, c.stream>>>(gl, A, dinv, L.x64.p, L.t64.p);
                else k_gmg_dax<2><<<blocks_for(L.ne, 256), 256, 0, c.stream>>>(gl, A, dinv, L.x64.p, L.t64.p);
            }
            UWG_CUDA(cudaMemcpyAsync(h.data(), L.t64.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            UWG_CUDA(cudaStreamSynchronize(c.stream));
            double nrm = 0.0;
            for (double v : h) nrm += v * v;
            nrm = std::sqrt(nrm);
            if (!(nrm > 0.0) || !std::isfinite(nrm)) break;
            lam = nrm;
            for (double& v : h) v /= nrm;
            UWG_CUDA(cudaMemcpyAsync(L.x64.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        }
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        L.lmax = lam;
    }
    // coarsest: dense inverse of A (+ mean diagonal / n in every entry for the constant mode)
    {
        const auto& C = c.gwg[nlev - 1];
        const double* Ac = nlev == 1 ? A0 : C.A64.p;
        const int64_t n = C.ne;
        double shift = 0.0;
        if (const_null) {
            std::vector<double> dg((size_t)n);
            UWG_CUDA(cudaMemcpy(dg.data(), Ac + (size_t)(nb / 2) * n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
            double sdg = 0.0;
            for (double v : dg) sdg += v;
            shift = sdg / n / n;
        }
        c.gwg_Cinv.ensure((size_t)(n * n));
        c.gwg_ncoarse = n;
        {
            LaunchScope ls(c, -1);
            if (dim == 3) k_gmg_dense<3><<<blocks_for(n, 128), 128, 0, c.stream>>>(egrid_level(C), Ac, shift, c.gwg_Cinv.p);
            else k_gmg_dense<2><<<blocks_for(n, 128), 128, 0, c.stream>>>(egrid_level(C), Ac, shift, c.gwg_Cinv.p);
        }
        check_launch("k_gmg_dense");
        dense_inverse(c, c.gwg_Cinv.p, n);
    }
    // FP32 copies of the coarse levels (level 0's FP32 stencil belongs to the solve)
    if (need32)
        for (int l = 1; l < nlev; ++l) {
            auto& L = c.gwg[l];
            L.A32.ensure((size_t)nb * L.ne);
            L.dinv32.ensure((size_t)L.ne);
            LaunchScope ls(c, -1);
            k_gwg_convert<double, float><<<blocks_for((int64_t)nb * L.ne, 256), 256, 0, c.stream>>>((int64_t)nb * L.ne, L.A64.p, L.A32.p);
            k_gwg_convert<double, float><<<blocks_for(L.ne, 256), 256, 0, c.stream>>>(L.ne, L.dinv64.p, L.dinv32.p);
            c.launches++;
        }
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    return true;
}

// the level array of precision T
template <typename T> static T* lv(DArray<double>& a64, DArray<float>& a32);
template <> double* lv<double>(DArray<double>& a64, DArray<float>&) { return a64.p; }
template <> float* lv<float>(DArray<double>&, DArray<float>& a32) { return a32.p; }

// degree-2 Chebyshev smoothing on level l (xin == nullptr: zero guess); result in x (x may be xin)
template <typename T>
static void gmg_smooth(Context& c, int l, const T* A, const T* dinv, const T* b, const T* xin, T* x) {
    auto& L = c.gwg[l];
    const EGrid g = egrid_level(L);
    const double lmax = 1.1 * L.lmax, lmin = 0.1 * L.lmax;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    const double rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0);
    const double c2a = 1.0 / theta, c1b = rho1 * rho0, c2b = 2.0 * rho1 / delta;
    T* t = lv<T>(L.t64, L.t32);
    T* d = lv<T>(L.d64, L.d32);
    const unsigned nbk = blocks_for(L.ne, 256);
    if (c.mesh.dim == 3) {
        k_gmg_cheb<3, T><<<nbk, 256, 0, c.stream>>>(g, A, dinv, b, xin, t, d, (T)0, (T)c2a, 1);
        k_gmg_cheb<3, T><<<nbk, 256, 0, c.stream>>>(g, A, dinv, b, t, x, d, (T)c1b, (T)c2b, 0);
    } else {
        k_gmg_cheb<2, T><<<nbk, 256, 0, c.stream>>>(g, A, dinv, b, xin, t, d, (T)0, (T)c2a, 1);
        k_gmg_cheb<2, T><<<nbk, 256, 0, c.stream>>>(g, A, dinv, b, t, x, d, (T)c1b, (T)c2b, 0);
    }
}

// V-cycle x = M b on level l (zero initial guess); level 0 uses the solve's stencil A0 / dinv0
template <typename T>
static void gmg_vcycle(Context& c, int l, const T* A0, const T* dinv0, const T* b, T* x) {
    auto& L = c.gwg[l];
    if (l == c.gwg_nlev - 1) {
        dense_apply<T>(c, c.gwg_Cinv.p, c.gwg_ncoarse, b, x);
        return;
    }
    const T* A = l == 0 ? A0 : lv<T>(L.A64, L.A32);
    const T* dinv = l == 0 ? dinv0 : lv<T>(L.dinv64, L.dinv32);
    const EGrid g = egrid_level(L);
    auto& C = c.gwg[l + 1];
    const EGrid gc = egrid_level(C);
    T* r = lv<T>(L.r64, L.r32);
    T* bc = lv<T>(C.b64, C.b32);
    T* xc = lv<T>(C.x64, C.x32);
    gmg_smooth<T>(c, l, A, dinv, b, nullptr, x);
    const unsigned nbk = blocks_for(L.ne, 256), nbc = blocks_for(C.ne, 256);
    if (c.mesh.dim == 3) {
        k_gmg_resid<3, T><<<nbk, 256, 0, c.stream>>>(g, A, x, b, r);
        k_gmg_restrict<3, T><<<nbc, 256, 0, c.stream>>>(g, gc, r, bc);
    } else {
        k_gmg_resid<2, T><<<nbk, 256, 0, c.stream>>>(g, A, x, b, r);
        k_gmg_restrict<2, T><<<nbc, 256, 0, c.stream>>>(g, gc, r, bc);
    }
    gmg_vcycle<T>(c, l + 1, A0, dinv0, bc, xc);
    if (c.mesh.dim == 3) k_gmg_prolong_add<3, T><<<nbk, 256, 0, c.stream>>>(g, gc, xc, x);
    else k_gmg_prolong_add<2, T><<<nbk, 256, 0, c.stream>>>(g, gc, xc, x);
    // post-smoothing from x with the same polynomial; in place is safe: the first step reads x and
    // writes t, the second reads t and writes x
    gmg_smooth<T>(c, l, A, dinv, b, x, x);
}

// CG on A x = b preconditioned by the V-cycle; work holds 4*ne values of T, scal 8 doubles
template <typename T>
static int gwg_cg_mg_T(Context& c, const T* A, const T* dinv, const double* b, T* x, double rtol, int maxit,
                       T* work, double* scal) {
    const MeshDesc& m = c.levels[0].mesh;
    EGrid g = egrid_of(m);
    const int64_t ne = g.ne;
    const int nb = m.dim == 3 ? 27 : 9;
    T* r = work;
    T* z = work + ne;
    T* p = work + 2 * ne;
    T* q = work + 3 * ne;
    UWG_CUDA(cudaMemsetAsync(scal, 0, 8 * sizeof(double), c.stream));
    const unsigned eb = blocks_for(ne, 256), ebv = blocks_for(ne, 256 * kEpt);
    {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_cgm_init<T><<<eb, 256, 0, c.stream>>>(ne, b, x, r, scal);
    }
    gmg_vcycle<T>(c, 0, A, dinv, r, z);
    k_cgm_dot<T><<<ebv, 256, 0, c.stream>>>(ne, r, z, scal);   // rz_0 -> scal[0]
    if (m.dim == 3) k_cg_spmv_dir<3, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, -1, 1);
    else k_cg_spmv_dir<2, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, -1, 1);
    check_launch("gwg_cg_mg init");
    double* hs = c.host_scalars;
    UWG_CUDA(cudaMemcpyAsync(hs, scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    const double r0 = std::sqrt(hs[7]);
    if (!(r0 > 0.0)) return 0;
    // six iterations per graph: the rz slots cycle with period 3 and the pq / rr slots with 2, so
    // every launch of the graph finds its slots where the previous one left them
    const int block = 6;
    auto issue = [&](int k) {
        k_cgm_update<T><<<ebv, 256, 0, c.stream>>>(ne, p, q, x, r, scal, k, k == block - 1);
        gmg_vcycle<T>(c, 0, A, dinv, r, z);
        k_cgm_dot<T><<<ebv, 256, 0, c.stream>>>(ne, r, z, rz_slot_host(scal, k + 1));
        if (m.dim == 3) k_cg_spmv_dir<3, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, k, 0);
        else k_cg_spmv_dir<2, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, k, 0);
    };
    const void* key[9] = {A, dinv, x, work, scal, (const void*)(intptr_t)ne, (const void*)(intptr_t)sizeof(T),
                          (const void*)(intptr_t)(m.dim + 32), nullptr};
    Context::PcgGraph* pg = nullptr;
    for (auto& cand : c.pcg_graphs)
        if (std::equal(std::begin(key), std::end(key), std::begin(cand.key))) pg = &cand;
    if (!pg) {
        c.pcg_graphs.emplace_back();
        pg = &c.pcg_graphs.back();
        std::copy(std::begin(key), std::end(key), std::begin(pg->key));
        cudaGraph_t graph;
        UWG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < block; ++k) issue(k);
        UWG_CUDA(cudaStreamEndCapture(c.stream, &graph));
        UWG_CUDA(cudaGraphInstantiate(&pg->exec, graph, 0));
        UWG_CUDA(cudaGraphDestroy(graph));
    }
    // algorithmic traffic of one iteration: the two CG kernels, two smoothing steps before and two
    // after the coarse correction and the residual on every level (stencil + vectors)
    double lev_bytes = 0.0;
    for (int l = 0; l + 1 < c.gwg_nlev; ++l) lev_bytes += (double)c.gwg[l].ne * sizeof(T) * 5.0 * (nb + 4);
    const double it_bytes = (double)ne * sizeof(T) * (8 + nb + 5 + 2) + lev_bytes;
    const double it_flops = (double)ne * (2.0 * nb + 16.0) * 6.0;
    int it = 0;
    while (it < maxit) {
        {
            LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
            UWG_CUDA(cudaGraphLaunch(pg->exec, c.stream));
        }
        note_work(c, UWGPU_KERNEL_SCHUR_PC, block * it_bytes, block * it_flops);
        it += block;
        UWG_CUDA(cudaMemcpyAsync(hs, scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        const double rn = std::sqrt(hs[6]);   // rr of the block's last iteration (k = 5: slot 5 + 1)
        if (!std::isfinite(rn)) throw Error(UWGPU_ERR_NAN, "NaN in the BFBt inner solve");
        if (rn <= rtol * r0) break;
    }
    check_launch("gwg_cg_mg");
    return it;
}

int gwg_cg_mg(Context& c, const double* A, const double* dinv, const double* b, double* x, double rtol, int maxit,
              double* work, double* scal) {
    return gwg_cg_mg_T<double>(c, A, dinv, b, x, rtol, maxit, work, scal);
}

int gwg_cg_mg32(Context& c, const float* A, const float* dinv, const double* b, float* x, double rtol, int maxit,
                float* work, double* scal) {
    return gwg_cg_mg_T<float>(c, A, dinv, b, x, rtol, maxit, work, scal);
}

}  // namespace uwg
