// Explicit element stencil of G^T W G and the Jacobi-preconditioned CG on it: the inner solves
// of the scaled BFBt Schur preconditioner (Solvers/KSPSolvers/src/BSSCR/pc_ScaledGtKG.c:242-310,
// the KSP on G^T W G built at pc_ScaledGtKG.c:735-760 with W = 1/rowmax(K)).
//
// G^T W G acts on P0 pressures (one unknown per element) and couples each element with the
// 3^dim elements that share a node with it.  Applying it matrix-free (G, scale by W, G^T) costs
// about 75 FP64 instructions per node and 50 per element, which on this part (FP64 at 1/58 of
// the FP32 rate) makes every CG iteration FP64-issue bound.  The stencil is built once per solve
// (A[q][e], entry-major, q = neighbour offset) and an iteration is then 27 FMAs per element
// with coalesced stencil reads; the 57 MB FP64 stencil of a 64^3 mesh can stay in L2.
//
// CG state lives in device memory and an iteration k is two kernels:
//   k_cg_update:   alpha = rz_k / pq_k; x += alpha p; r -= alpha q; z = Dinv r; rz_{k+1}, rr
//   k_cg_spmv_dir: beta = rz_{k+1} / rz_k; p = z + beta p; q = A z + beta q (= A p); pq_{k+1}
// (q = A p by linearity, so the direction update needs no neighbour of p and fuses into the spmv).
// The scalars are buffered so that no kernel clears a slot another block may still read:
//   scal[0..2] = rz (k mod 3)   scal[3..4] = pq (k mod 2)   scal[5..6] = rr (k mod 2)   scal[7] = r0.r0
// Twelve iterations (so both patterns repeat) are captured once as a CUDA graph and replayed; the
// host reads the residual norm after each replay.
#include <algorithm>
#include <cmath>
#include <iterator>

#include "internal.cuh"

namespace uwg {

// fine-mesh element widths h[off[d] + i] (operator.cu)
const double* fine_widths(Context& c, int off[3]);

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
}

// Elements per thread of the vector kernels: the block reduction (a shuffle tree, FP64 in the
// FP64 form) is paid once per kEpt elements.  Element k of a thread is base + k * blockDim.x,
// so every access stays coalesced.
constexpr int kEpt = 2;

// iteration k, first kernel: alpha = rz_k / pq_k; x += alpha p; r -= alpha q; z = dinv r;
// rz_{k+1} += r.z; and, when want_rr (the host's convergence check follows), rr_k += r.r.
// Clears the slots of rz_{k+2} and pq_{k+1}.
template <typename T>
__global__ void k_cg_update(int64_t ne, const T* __restrict__ p, const T* __restrict__ q,
                            const T* __restrict__ dinv, T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                            double* __restrict__ scal, int k, int want_rr) {
    __shared__ double sw[32];
    __shared__ T s_alpha;
    const T alpha = block_ratio<T>(rz_slot(scal, k), pq_slot(scal, k), &s_alpha);
    const int64_t base = (int64_t)blockIdx.x * blockDim.x * kEpt + threadIdx.x;
    T rz = (T)0, rr = (T)0;
#pragma unroll
    for (int m = 0; m < kEpt; ++m) {
        const int64_t e = base + (int64_t)m * blockDim.x;
        if (e < ne) {
            x[e] = fma(alpha, p[e], x[e]);
            T re = fma(-alpha, q[e], r[e]);
            r[e] = re;
            T ze = re * dinv[e];
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

EGrid egrid_of(const MeshDesc& m) {
    EGrid g;
    g.ex = m.nel[0];
    g.ey = m.nel[1];
    g.ez = m.dim == 3 ? m.nel[2] : 1;
    g.ne = g.ex * g.ey * g.ez;
    return g;
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

// FP32 copies of the stencil and the inverse diagonal (mixed form)
void gwg_stencil_fp32(Context& c, const double* A, const double* dinv, float* A32, float* dinv32) {
    const MeshDesc& m = c.levels[0].mesh;
    int64_t ne = m.ne, na = ne * (m.dim == 3 ? 27 : 9);
    LaunchScope ls(c, -1);
    k_gwg_convert<double, float><<<blocks_for(na, 256), 256, 0, c.stream>>>(na, A, A32);
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

// Solves A x = b (b projected off the constant by the caller when A has it) to
// ||r|| <= rtol ||b|| by Jacobi-preconditioned CG.  work holds 4*ne values of T, scal 8 doubles.
// Returns the iterations taken.
template <typename T>
static int gwg_cg_T(Context& c, const T* A, const T* dinv, const double* b, T* x, double rtol, int maxit, T* work,
                    double* scal) {
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
        k_gwg_init<T><<<eb, 256, 0, c.stream>>>(ne, b, dinv, x, r, z, scal);
    }
    {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        if (m.dim == 3) k_cg_spmv_dir<3, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, -1, 1);
        else k_cg_spmv_dir<2, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, -1, 1);
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
        k_cg_update<T><<<ebv, 256, 0, c.stream>>>(ne, p, q, dinv, x, r, z, scal, k, k == block - 1);
        if (m.dim == 3) k_cg_spmv_dir<3, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, k, 0);
        else k_cg_spmv_dir<2, T><<<eb, 256, 0, c.stream>>>(g, A, z, p, q, scal, k, 0);
    };
    const void* key[8] = {A, dinv, x, work, scal, (const void*)(intptr_t)ne, (const void*)(intptr_t)sizeof(T),
                          (const void*)(intptr_t)(m.dim + 16)};
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
    // spmv+direction (the stencil, z, p, q read; p, q written)
    const double it_bytes = (double)ne * sizeof(T) * (8 + nb + 5);
    const double it_flops = (double)ne * (2.0 * nb + 14.0);
    int it = 0;
    while (it < maxit) {
        {
            LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
            UWG_CUDA(cudaGraphLaunch(pg->exec, c.stream));
        }
        note_work(c, UWGPU_KERNEL_SCHUR_PC, block * it_bytes, block * it_flops);
        c.launches += 2 * block - 1;
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
    return gwg_cg_T<double>(c, A, dinv, b, x, rtol, maxit, work, scal);
}

int gwg_cg32(Context& c, const float* A, const float* dinv, const double* b, float* x, double rtol, int maxit,
             float* work, double* scal) {
    return gwg_cg_T<float>(c, A, dinv, b, x, rtol, maxit, work, scal);
}

}  // namespace uwg
