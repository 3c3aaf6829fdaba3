// Velocity-block operator and geometric multigrid hierarchy.
//
// Reference behaviour (paths relative to the Underworld 1.x tree):
//   global K      StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:867-1017 (element scatter-add with
//                 the location matrix; BC dofs removed, FeEquationNumber.c:700-760)
//   transfers     StgFEM/SLE/SystemSetup/src/SROpGenerator.c:765-1060 (2:1 regular interpolation,
//                 weight 1/nPoints over 2^(#odd indices) coarse nodes; restriction = P^T)
//   coarse ops    StgFEM/SLE/SystemSetup/src/PETScMGSolver.c:493-549 (Galerkin P^T K P)
//   smoother      PETScMGSolver.c:641-716 (Richardson + SOR, multiplicative V-cycle)
//   coarse solve  PCMG's redundant direct solve on the coarsest level
//   G, G^T        GradientStiffnessMatrixTerm (P0 pressure, one dof per element)
//
// GPU design.  The assembled operator is kept as a node-block stencil: for every node the 3^dim
// neighbour blocks (dim x dim) are stored entry-major [q][r][c][node], so the apply is a pure
// gather (one thread per node, no atomics) and each load instruction of a warp is coalesced.
// Dirichlet dofs are identity rows/columns, so every vector keeps the full nodal length.
// The Gauss-Seidel smoother is colour-scheduled: the 2^dim parity colours of the nodes have no
// stencil coupling inside a colour, so a colour is relaxed in parallel without atomics.
// Coarse element matrices are formed element by element (P_c^T K_c P_c over the 2^dim children),
// which equals the Galerkin product for this interpolation.
#include <cooperative_groups.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>
#include <iterator>
#include <type_traits>

#include "internal.cuh"

namespace cg = cooperative_groups;

namespace uwg {

struct Grid {
    int dim;
    int64_t nx, ny, nz;  // nodes per axis
    int64_t nn;
    int ex, ey, ez;      // elements per axis
};

static Grid grid_of(const MeshDesc& m) {
    Grid g;
    g.dim = m.dim;
    g.nx = m.nnx;
    g.ny = m.nny;
    g.nz = m.nnz;
    g.nn = m.nn;
    g.ex = m.nel[0];
    g.ey = m.nel[1];
    g.ez = m.dim == 3 ? m.nel[2] : 1;
    return g;
}

template <int DIM>
__host__ __device__ constexpr int nblocks() { return DIM == 3 ? 27 : 9; }

// ------------------------------------------------------------------------------------------
// Stencil build from packed element matrices (gather per node, 9 accumulators per block).
// ------------------------------------------------------------------------------------------
template <int DIM>
__global__ void k_build_stencil(Grid g, int64_t ne, const double* __restrict__ Ke, const uint8_t* __restrict__ fixed,
                                double* __restrict__ A, double* __restrict__ Dinv) {
    constexpr int NEN = 1 << DIM, ND = NEN * DIM, NB = nblocks<DIM>();
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
    int64_t i = n % g.nx, j = (n / g.nx) % g.ny, k = DIM == 3 ? n / (g.nx * g.ny) : 0;
    int64_t nidx[3] = {i, j, k};
    int64_t ecount[3] = {g.ex, g.ey, g.ez};
    int64_t ncount[3] = {g.nx, g.ny, g.nz};
    bool rowfix[DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r) rowfix[r] = fixed ? fixed[n * DIM + r] != 0 : false;
    double diag[DIM][DIM];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        int off[3] = {q % 3 - 1, (q / 3) % 3 - 1, DIM == 3 ? q / 9 - 1 : 0};
        double acc[DIM][DIM];
#pragma unroll
        for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int cc = 0; cc < DIM; ++cc) acc[r][cc] = 0.0;
        bool valid = true;
        int64_t m[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            m[d] = nidx[d] + off[d];
            if (m[d] < 0 || m[d] >= ncount[d]) valid = false;
        }
        int64_t mnode = 0;
        bool colfix[DIM];
#pragma unroll
        for (int cc = 0; cc < DIM; ++cc) colfix[cc] = false;
        if (valid) {
            mnode = m[0] + g.nx * (m[1] + g.ny * (DIM == 3 ? m[2] : 0));
#pragma unroll
            for (int cc = 0; cc < DIM; ++cc) colfix[cc] = fixed ? fixed[mnode * DIM + cc] != 0 : false;
            // elements containing both nodes: per axis origin range
            int64_t lo[3], hi[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d >= DIM) { lo[d] = 0; hi[d] = 0; continue; }
                int64_t a = nidx[d] < m[d] ? nidx[d] : m[d];
                int64_t b = nidx[d] > m[d] ? nidx[d] : m[d];
                lo[d] = b - 1 < 0 ? 0 : b - 1;
                hi[d] = a > ecount[d] - 1 ? ecount[d] - 1 : a;
            }
            for (int64_t ez = lo[2]; ez <= hi[2]; ++ez)
                for (int64_t ey = lo[1]; ey <= hi[1]; ++ey)
                    for (int64_t ex = lo[0]; ex <= hi[0]; ++ex) {
                        int64_t e = ex + (int64_t)g.ex * (ey + (int64_t)g.ey * ez);
                        int la = (int)(i - ex) + 2 * (int)(j - ey) + (DIM == 3 ? 4 * (int)(k - ez) : 0);
                        int lb = (int)(m[0] - ex) + 2 * (int)(m[1] - ey) + (DIM == 3 ? 4 * (int)(m[2] - ez) : 0);
#pragma unroll
                        for (int r = 0; r < DIM; ++r)
#pragma unroll
                            for (int cc = 0; cc < DIM; ++cc) {
                                int R = la * DIM + r, C = lb * DIM + cc;
                                int pi = R <= C ? packed_index(ND, R, C) : packed_index(ND, C, R);
                                acc[r][cc] += Ke[(int64_t)pi * ne + e];
                            }
                    }
        }
#pragma unroll
        for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int cc = 0; cc < DIM; ++cc) {
                double v = acc[r][cc];
                if (rowfix[r] || colfix[cc]) v = 0.0;
                if (q == NB / 2 && r == cc && rowfix[r]) v = 1.0;
                A[((int64_t)(q * DIM + r) * DIM + cc) * g.nn + n] = v;
                if (q == NB / 2) diag[r][cc] = v;
            }
    }
    // inverse of the diagonal block
    double inv[DIM][DIM];
    if (DIM == 3) {
        double a = diag[0][0], b = diag[0][1], c = diag[0][2], d = diag[1][0], e = diag[1][1], f = diag[1][2],
               gg = diag[2][0], h = diag[2][1], ii = diag[2][2];
        double A0 = e * ii - f * h, B0 = -(d * ii - f * gg), C0 = d * h - e * gg;
        double det = a * A0 + b * B0 + c * C0;
        double id = 1.0 / det;
        inv[0][0] = A0 * id;
        inv[1][0] = B0 * id;
        inv[2][0] = C0 * id;
        inv[0][1] = -(b * ii - c * h) * id;
        inv[1][1] = (a * ii - c * gg) * id;
        inv[2][1] = -(a * h - b * gg) * id;
        inv[0][2] = (b * f - c * e) * id;
        inv[1][2] = -(a * f - c * d) * id;
        inv[2][2] = (a * e - b * d) * id;
    } else {
        double det = diag[0][0] * diag[1][1] - diag[0][1] * diag[1][0];
        double id = 1.0 / det;
        inv[0][0] = diag[1][1] * id;
        inv[0][1] = -diag[0][1] * id;
        inv[1][0] = -diag[1][0] * id;
        inv[1][1] = diag[0][0] * id;
    }
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int cc = 0; cc < DIM; ++cc) Dinv[(int64_t)(r * DIM + cc) * g.nn + n] = inv[r][cc];
}

template <typename S, typename D>
__global__ void k_convert(int64_t n, const S* __restrict__ a, D* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (D)a[i];
}

// ------------------------------------------------------------------------------------------
// Apply and smoothing.
// ------------------------------------------------------------------------------------------
// Neighbour offsets of node (i, j, k) per axis, 0 towards a missing neighbour.  Every stencil block
// towards a neighbour outside the mesh is stored as zero, so a row reads the node itself there
// and all loads of a row are unconditional (they can all be in flight at once).
struct NbrOffsets {
    int64_t dx[3], dy[3], dz[3];
};

template <int DIM>
__device__ __forceinline__ NbrOffsets nbr_offsets(const Grid& g, int64_t i, int64_t j, int64_t k) {
    NbrOffsets o;
    o.dx[0] = i > 0 ? -1 : 0;
    o.dx[1] = 0;
    o.dx[2] = i + 1 < g.nx ? 1 : 0;
    o.dy[0] = j > 0 ? -g.nx : 0;
    o.dy[1] = 0;
    o.dy[2] = j + 1 < g.ny ? g.nx : 0;
    o.dz[0] = DIM == 3 && k > 0 ? -g.nx * g.ny : 0;
    o.dz[1] = 0;
    o.dz[2] = DIM == 3 && k + 1 < g.nz ? g.nx * g.ny : 0;
    return o;
}

// (i, j, k) of node n with 32-bit division (node counts stay below 2^32, checked on the host)
template <int DIM>
__device__ __forceinline__ void node_ijk(const Grid& g, int64_t n, int64_t& i, int64_t& j, int64_t& k) {
    const unsigned un = (unsigned)n, nx = (unsigned)g.nx, ny = (unsigned)g.ny;
    const unsigned q = un / nx;
    i = un - q * nx;
    j = DIM == 3 ? q % ny : q;
    k = DIM == 3 ? q / ny : 0;
}

// Row-split layout: a block of kRowThreads threads covers kRowThreads/DIM nodes; warp w works on
// row w % DIM of 32 consecutive nodes (lanes), so every stencil load of a warp is coalesced and a
// node's DIM rows run on DIM threads (three times the parallelism of one thread per node).
constexpr int kRowThreads = 192;

// sum_q sum_c A[q][r][c][n] x[c][m(q)] for one row r of node n
template <int DIM, typename T>
__device__ __forceinline__ T stencil_row_r(const Grid& g, int64_t n, int64_t i, int64_t j, int64_t k, int r,
                                           const T* __restrict__ A, const T* __restrict__ x) {
    constexpr int NB = nblocks<DIM>();
    // Loads are issued in batches of QB neighbours (all stencil and x values of the batch before
    // its FMAs), so that enough bytes are in flight per thread to cover the memory latency:
    // 9 neighbours in FP32, 3 in FP64 (which is limited by the FP64 pipe, not by latency).
    constexpr int QB = sizeof(T) == 4 ? 9 : 3;
    const NbrOffsets o = nbr_offsets<DIM>(g, i, j, k);
    T out = (T)0;
#pragma unroll
    for (int q0 = 0; q0 < NB; q0 += QB) {
        T a[QB * DIM], xv[QB * DIM];
#pragma unroll
        for (int qq = 0; qq < QB; ++qq) {
            const int q = q0 + qq;
            const int64_t m = n + o.dx[q % 3] + o.dy[(q / 3) % 3] + o.dz[DIM == 3 ? q / 9 : 1];
#pragma unroll
            for (int cc = 0; cc < DIM; ++cc) {
                a[qq * DIM + cc] = __ldg(A + ((int64_t)(q * DIM + r) * DIM + cc) * g.nn + n);
                xv[qq * DIM + cc] = x[(int64_t)cc * g.nn + m];
            }
        }
#pragma unroll
        for (int t = 0; t < QB * DIM; ++t) out = fma(a[t], xv[t], out);
    }
    return out;
}

// The same row product from the FP16 row-scaled stencil (A / S16 per row), unscaled: the caller
// multiplies by S16[r][n].  The FP16 entries of neighbours q = 2p and 2p + 1 share one 32-bit word,
// [p][r][c][node], so a load brings two entries and one conversion widens both.  Loads go out in
// batches of five pairs.
template <int DIM>
__device__ __forceinline__ float stencil_row_h(const Grid& g, int64_t n, int64_t i, int64_t j, int64_t k, int r,
                                               const uint32_t* __restrict__ A, const float* __restrict__ x) {
    constexpr int NB = nblocks<DIM>(), NP = (NB + 1) / 2, PB = 5;
    const NbrOffsets o = nbr_offsets<DIM>(g, i, j, k);
    float out = 0.f;
#pragma unroll
    for (int p0 = 0; p0 < NP; p0 += PB) {
        uint32_t w[PB * DIM];
        float xv[2 * PB * DIM];
#pragma unroll
        for (int pp = 0; pp < PB; ++pp) {
            const int pr = p0 + pp;
            if (pr < NP) {
                const int q0 = 2 * pr, q1 = 2 * pr + 1;
                const int64_t m0 = n + o.dx[q0 % 3] + o.dy[(q0 / 3) % 3] + o.dz[DIM == 3 ? q0 / 9 : 1];
                const int64_t m1 = q1 < NB ? n + o.dx[q1 % 3] + o.dy[(q1 / 3) % 3] + o.dz[DIM == 3 ? q1 / 9 : 1] : n;
#pragma unroll
                for (int cc = 0; cc < DIM; ++cc) {
                    w[pp * DIM + cc] = __ldg(A + ((int64_t)(pr * DIM + r) * DIM + cc) * g.nn + n);
                    xv[(2 * pp) * DIM + cc] = x[(int64_t)cc * g.nn + m0];
                    xv[(2 * pp + 1) * DIM + cc] = q1 < NB ? x[(int64_t)cc * g.nn + m1] : 0.f;
                }
            }
        }
#pragma unroll
        for (int pp = 0; pp < PB; ++pp) {
            if (p0 + pp < NP) {
#pragma unroll
                for (int cc = 0; cc < DIM; ++cc) {
                    const uint32_t wv = w[pp * DIM + cc];
                    const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&wv));
                    out = fmaf(f.x, xv[(2 * pp) * DIM + cc], out);
                    out = fmaf(f.y, xv[(2 * pp + 1) * DIM + cc], out);
                }
            }
        }
    }
    return out;
}

// r = b - A x with the FP16 stencil (V-cycle residuals of the mixed form)
template <int DIM>
__global__ void __launch_bounds__(kRowThreads) k_residual_h(Grid g, const uint32_t* __restrict__ A,
                                                            const float* __restrict__ S, const float* __restrict__ x,
                                                            const float* __restrict__ b, float* __restrict__ y) {
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = warp % DIM, grp = warp / DIM;
    int64_t n = (int64_t)blockIdx.x * (kRowThreads / DIM) + grp * 32 + lane;
    if (n >= g.nn) return;
    int64_t i, j, k;
    node_ijk<DIM>(g, n, i, j, k);
    const int64_t idx = (int64_t)r * g.nn + n;
    y[idx] = b[idx] - S[idx] * stencil_row_h<DIM>(g, n, i, j, k, r, A, x);
}

// FP32 -> FP16 row-scaled stencil: S16[r][n] = max over the row's entries of |A|; the entries of
// A / S16 in FP16, neighbours 2p and 2p + 1 packed in word [p][r][c][n] (the last pair's upper half
// zero when the neighbour count is odd)
template <int DIM>
__global__ void k_to_fp16_rows(Grid g, const float* __restrict__ A, uint32_t* __restrict__ A16,
                               float* __restrict__ S16) {
    constexpr int NB = nblocks<DIM>(), NP = (NB + 1) / 2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)DIM * g.nn) return;
    const int r = (int)(t / g.nn);
    const int64_t n = t % g.nn;
    float mx = 0.f;
    for (int q = 0; q < NB; ++q)
        for (int cc = 0; cc < DIM; ++cc) mx = fmaxf(mx, fabsf(A[((int64_t)(q * DIM + r) * DIM + cc) * g.nn + n]));
    const float sc = mx > 0.f ? mx : 1.f, inv = 1.f / sc;
    S16[t] = sc;
    for (int pr = 0; pr < NP; ++pr)
        for (int cc = 0; cc < DIM; ++cc) {
            const int q0 = 2 * pr, q1 = 2 * pr + 1;
            const float a0 = A[((int64_t)(q0 * DIM + r) * DIM + cc) * g.nn + n] * inv;
            const float a1 = q1 < NB ? A[((int64_t)(q1 * DIM + r) * DIM + cc) * g.nn + n] * inv : 0.f;
            const uint32_t lo = __half_as_ushort(__float2half_rn(a0)), hi = __half_as_ushort(__float2half_rn(a1));
            A16[((int64_t)(pr * DIM + r) * DIM + cc) * g.nn + n] = lo | (hi << 16);
        }
}

// y = A x (or r = b - A x when b is given), row-split
template <int DIM, typename T>
__global__ void __launch_bounds__(kRowThreads) k_apply(Grid g, const T* __restrict__ A, const T* __restrict__ x,
                                                       const T* __restrict__ b, T* __restrict__ y) {
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = warp % DIM, grp = warp / DIM;
    int64_t n = (int64_t)blockIdx.x * (kRowThreads / DIM) + grp * 32 + lane;
    if (n >= g.nn) return;
    int64_t i, j, k;
    node_ijk<DIM>(g, n, i, j, k);
    T v = stencil_row_r<DIM, T>(g, n, i, j, k, r, A, x);
    y[(int64_t)r * g.nn + n] = b ? b[(int64_t)r * g.nn + n] - v : v;
}

// `sweeps` symmetric multicolour block Gauss-Seidel sweeps (colours ascending, then
// descending) in one cooperative launch: x_n += Dinv_n (b_n - (A x)_n).  Nodes of one parity
// colour are never stencil neighbours, so a colour is relaxed in parallel; the DIM row
// residuals of a node meet in shared memory before its update, and a grid-wide barrier
// separates colours.
template <int DIM, typename T>
__global__ void __launch_bounds__(kRowThreads) k_gs_sweeps(Grid g, const T* __restrict__ A, const T* __restrict__ Dinv,
                                                           const T* __restrict__ b, T* __restrict__ x, int sweeps,
                                                           int zero_init) {
    __shared__ T sres[kRowThreads];
    cg::grid_group grid = cg::this_grid();
    constexpr int NPB = kRowThreads / DIM;
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = warp % DIM, grp = warp / DIM;
    if (zero_init) {
        const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (int64_t t = tid; t < g.nn * DIM; t += stride) x[t] = (T)0;
        grid.sync();
    }
    constexpr int NCOL = 1 << DIM;
    for (int s = 0; s < sweeps; ++s) {
        for (int step = 0; step < 2 * NCOL; ++step) {
            int col = step < NCOL ? step : 2 * NCOL - 1 - step;
            int px = col & 1, py = (col >> 1) & 1, pz = (col >> 2) & 1;
            int64_t cx = (g.nx - px + 1) / 2, cy = (g.ny - py + 1) / 2;
            int64_t cz = DIM == 3 ? (g.nz - pz + 1) / 2 : 1;
            int64_t cnt = cx * cy * cz;
            for (int64_t base = (int64_t)blockIdx.x * NPB; base < cnt; base += (int64_t)gridDim.x * NPB) {
                int64_t t = base + grp * 32 + lane;
                bool act = t < cnt;
                int64_t n = 0;
                T res = (T)0;
                if (act) {
                    int64_t i = 2 * (t % cx) + px, j = 2 * ((t / cx) % cy) + py;
                    int64_t k = DIM == 3 ? 2 * (t / (cx * cy)) + pz : 0;
                    n = i + g.nx * (j + g.ny * k);
                    res = b[(int64_t)r * g.nn + n] - stencil_row_r<DIM, T>(g, n, i, j, k, r, A, x);
                }
                sres[threadIdx.x] = res;
                __syncthreads();
                if (act) {
                    T v = x[(int64_t)r * g.nn + n];
#pragma unroll
                    for (int cc = 0; cc < DIM; ++cc)
                        v = fma(Dinv[(int64_t)(r * DIM + cc) * g.nn + n], sres[(grp * DIM + cc) * 32 + lane], v);
                    x[(int64_t)r * g.nn + n] = v;
                }
                __syncthreads();
            }
            grid.sync();
        }
    }
}

// One Chebyshev step of the block-Jacobi preconditioned operator D^-1 A (row-split):
//   z = Dinv (b - A xin);  d = c1 d + c2 z (d = c2 z on the first step);  xout = xin + d.
// xin == nullptr stands for a zero initial guess.  Every node is relaxed from the old iterate, so
// no colouring and no grid barrier are needed.
template <int DIM, typename T>
__global__ void __launch_bounds__(kRowThreads) k_cheb_step(Grid g, const T* __restrict__ A, const T* __restrict__ Dinv,
                                                           const T* __restrict__ b, const T* __restrict__ xin,
                                                           T* __restrict__ xout, T* __restrict__ d, T c1, T c2,
                                                           int first) {
    __shared__ T sres[kRowThreads];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = warp % DIM, grp = warp / DIM;
    int64_t n = (int64_t)blockIdx.x * (kRowThreads / DIM) + grp * 32 + lane;
    bool act = n < g.nn;
    T res = (T)0;
    if (act) {
        int64_t i, j, k;
        node_ijk<DIM>(g, n, i, j, k);
        res = b[(int64_t)r * g.nn + n];
        if (xin) res -= stencil_row_r<DIM, T>(g, n, i, j, k, r, A, xin);
    }
    sres[threadIdx.x] = res;
    __syncthreads();
    if (!act) return;
    T z = (T)0;
#pragma unroll
    for (int cc = 0; cc < DIM; ++cc) z = fma(Dinv[(int64_t)(r * DIM + cc) * g.nn + n], sres[(grp * DIM + cc) * 32 + lane], z);
    int64_t idx = (int64_t)r * g.nn + n;
    T dn = first ? c2 * z : fma(c1, d[idx], c2 * z);
    d[idx] = dn;
    xout[idx] = (xin ? xin[idx] : (T)0) + dn;
}

// The Chebyshev step with the FP16 row-scaled stencil (mixed form)
template <int DIM>
__global__ void __launch_bounds__(kRowThreads) k_cheb_step_h(Grid g, const uint32_t* __restrict__ A,
                                                             const float* __restrict__ S, const float* __restrict__ Dinv,
                                                             const float* __restrict__ b, const float* __restrict__ xin,
                                                             float* __restrict__ xout, float* __restrict__ d, float c1,
                                                             float c2, int first) {
    __shared__ float sres[kRowThreads];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = warp % DIM, grp = warp / DIM;
    int64_t n = (int64_t)blockIdx.x * (kRowThreads / DIM) + grp * 32 + lane;
    bool act = n < g.nn;
    float res = 0.f;
    if (act) {
        int64_t i, j, k;
        node_ijk<DIM>(g, n, i, j, k);
        const int64_t idx = (int64_t)r * g.nn + n;
        res = b[idx];
        if (xin) res -= S[idx] * stencil_row_h<DIM>(g, n, i, j, k, r, A, xin);
    }
    sres[threadIdx.x] = res;
    __syncthreads();
    if (!act) return;
    float z = 0.f;
#pragma unroll
    for (int cc = 0; cc < DIM; ++cc) z = fmaf(Dinv[(int64_t)(r * DIM + cc) * g.nn + n], sres[(grp * DIM + cc) * 32 + lane], z);
    int64_t idx = (int64_t)r * g.nn + n;
    float dn = first ? c2 * z : fmaf(c1, d[idx], c2 * z);
    d[idx] = dn;
    xout[idx] = (xin ? xin[idx] : 0.f) + dn;
}

// z = Dinv y (block diagonal)
template <int DIM, typename T>
__global__ void k_dinv(Grid g, const T* __restrict__ Dinv, const T* __restrict__ y, T* __restrict__ z) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
    T yn[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) yn[c] = y[(int64_t)c * g.nn + n];
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
        T v = (T)0;
#pragma unroll
        for (int c = 0; c < DIM; ++c) v = fma(Dinv[(int64_t)(r * DIM + c) * g.nn + n], yn[c], v);
        z[(int64_t)r * g.nn + n] = v;
    }
}

// ------------------------------------------------------------------------------------------
// Transfers (trilinear 2:1, SROpGenerator weights), Dirichlet dofs masked.
// ------------------------------------------------------------------------------------------
template <int DIM, typename T>
__global__ void k_restrict(Grid gf, Grid gc, const T* __restrict__ rf, T* __restrict__ rc,
                           const uint8_t* __restrict__ fixf, const uint8_t* __restrict__ fixc) {
    int64_t N = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (N >= gc.nn) return;
    int64_t I = N % gc.nx, J = (N / gc.nx) % gc.ny, K = DIM == 3 ? N / (gc.nx * gc.ny) : 0;
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = (T)0;
#pragma unroll
    for (int dz = (DIM == 3 ? -1 : 0); dz <= (DIM == 3 ? 1 : 0); ++dz)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                int64_t i = 2 * I + dx, j = 2 * J + dy, k = 2 * K + dz;
                if (i < 0 || i >= gf.nx || j < 0 || j >= gf.ny || (DIM == 3 && (k < 0 || k >= gf.nz))) continue;
                T w = (T)((dx ? 0.5 : 1.0) * (dy ? 0.5 : 1.0) * (dz ? 0.5 : 1.0));
                int64_t n = i + gf.nx * (j + gf.ny * k);
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    if (!fixf || !fixf[n * DIM + d]) acc[d] = fma(w, rf[(int64_t)d * gf.nn + n], acc[d]);
            }
#pragma unroll
    for (int d = 0; d < DIM; ++d) rc[(int64_t)d * gc.nn + N] = (fixc && fixc[N * DIM + d]) ? (T)0 : acc[d];
}

template <int DIM, typename T>
__global__ void k_prolong_add(Grid gf, Grid gc, const T* __restrict__ xc, T* __restrict__ xf,
                              const uint8_t* __restrict__ fixf, const uint8_t* __restrict__ fixc) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= gf.nn) return;
    int64_t idx[3] = {n % gf.nx, (n / gf.nx) % gf.ny, DIM == 3 ? n / (gf.nx * gf.ny) : 0};
    int64_t c0[3], c1[3];
    int cnt[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= DIM) { c0[d] = c1[d] = 0; cnt[d] = 1; continue; }
        c0[d] = idx[d] >> 1;
        c1[d] = c0[d] + 1;
        cnt[d] = (idx[d] & 1) ? 2 : 1;
    }
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = (T)0;
    T w = (T)(1.0 / (double)(cnt[0] * cnt[1] * cnt[2]));
    for (int oz = 0; oz < cnt[2]; ++oz)
        for (int oy = 0; oy < cnt[1]; ++oy)
            for (int ox = 0; ox < cnt[0]; ++ox) {
                int64_t I = ox ? c1[0] : c0[0], J = oy ? c1[1] : c0[1], K = oz ? c1[2] : c0[2];
                int64_t N = I + gc.nx * (J + gc.ny * K);
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    if (!fixc || !fixc[N * DIM + d]) acc[d] = fma(w, xc[(int64_t)d * gc.nn + N], acc[d]);
            }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        if (!fixf || !fixf[n * DIM + d]) xf[(int64_t)d * gf.nn + n] += acc[d];
}

// ------------------------------------------------------------------------------------------
// Galerkin coarse element matrices: K_E = sum_children P_c^T K~_c P_c, where K~_c has the
// rows/columns of fixed fine dofs removed.
// ------------------------------------------------------------------------------------------
__host__ __device__ inline double interp_weight(int child_bit, int fine_bit, int coarse_bit) {
    int f = child_bit + fine_bit;   // fine position in half units: 0, 1, 2
    int cpos = 2 * coarse_bit;
    if (f == cpos) return 1.0;
    if (f == 1) return 0.5;
    return 0.0;
}

template <int DIM>
__global__ void k_galerkin(Grid gf, Grid gc, int64_t nef, int64_t nec, const double* __restrict__ Kf,
                           const uint8_t* __restrict__ fixf, double* __restrict__ Kc) {
    constexpr int NEN = 1 << DIM, ND = NEN * DIM, NP = ND * (ND + 1) / 2, NCH = 1 << DIM;
    extern __shared__ double sK[];  // NCH * ND * ND
    int64_t E = blockIdx.x;
    if (E >= nec) return;
    int64_t EI = E % gc.ex, EJ = (E / gc.ex) % gc.ey, EK = DIM == 3 ? E / ((int64_t)gc.ex * gc.ey) : 0;
    // load the children's full element matrices, fixed fine dofs zeroed
    for (int t = threadIdx.x; t < NCH * ND * ND; t += blockDim.x) {
        int ch = t / (ND * ND), rc = t % (ND * ND), R = rc / ND, C = rc % ND;
        int cx = ch & 1, cy = (ch >> 1) & 1, cz = (ch >> 2) & 1;
        int64_t fe = (2 * EI + cx) + (int64_t)gf.ex * ((2 * EJ + cy) + (int64_t)gf.ey * (DIM == 3 ? 2 * EK + cz : 0));
        int la = R / DIM, lb = C / DIM;
        int64_t fo = (2 * EI + cx) + gf.nx * ((2 * EJ + cy) + gf.ny * (DIM == 3 ? 2 * EK + cz : 0));
        int64_t na = fo + (la & 1) + ((la >> 1) & 1) * gf.nx + (DIM == 3 ? ((la >> 2) & 1) * gf.nx * gf.ny : 0);
        int64_t nb = fo + (lb & 1) + ((lb >> 1) & 1) * gf.nx + (DIM == 3 ? ((lb >> 2) & 1) * gf.nx * gf.ny : 0);
        bool fx = fixf && (fixf[na * DIM + R % DIM] || fixf[nb * DIM + C % DIM]);
        int pi = R <= C ? packed_index(ND, R, C) : packed_index(ND, C, R);
        sK[t] = fx ? 0.0 : Kf[(int64_t)pi * nef + fe];
    }
    __syncthreads();
    for (int o = threadIdx.x; o < NP; o += blockDim.x) {
        // decode packed (R, C), R <= C
        int R = 0, rem = o;
        while (rem >= ND - R) { rem -= ND - R; R++; }
        int C = R + rem;
        int I = R / DIM, a = R % DIM, J = C / DIM, b = C % DIM;
        double acc = 0.0;
        for (int ch = 0; ch < NCH; ++ch) {
            int cb[3] = {ch & 1, (ch >> 1) & 1, (ch >> 2) & 1};
            const double* K = sK + ch * ND * ND;
            for (int i = 0; i < NEN; ++i) {
                double wi = 1.0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) wi *= interp_weight(cb[d], (i >> d) & 1, (I >> d) & 1);
                if (wi == 0.0) continue;
                for (int j = 0; j < NEN; ++j) {
                    double wj = 1.0;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) wj *= interp_weight(cb[d], (j >> d) & 1, (J >> d) & 1);
                    if (wj == 0.0) continue;
                    acc += wi * wj * K[(i * DIM + a) * ND + j * DIM + b];
                }
            }
        }
        Kc[(int64_t)o * nec + E] = acc;
    }
}

// 3D form of the same product through the 27-node patch of the eight children: the patch matrix
// A (81 x 81), the children's element matrices added into it child after child (the 576 entries
// of one child land on distinct patch entries, so no two threads add to the same place), then
// B = A P and K_E = P^T B with the trilinear prolongation P (81 x 24), whose weights are products
// of 1 (fine node on the coarse node), 1/2 (fine node halfway) and 0 per axis.
__device__ __forceinline__ double half_weight(int fine_pos, int coarse_bit) {
    const int d = fine_pos - 2 * coarse_bit;
    return d == 0 ? 1.0 : (d == 1 || d == -1) ? 0.5 : 0.0;
}

__global__ void __launch_bounds__(256) k_galerkin3(Grid gf, Grid gc, int64_t nef, int64_t nec,
                                                  const double* __restrict__ Kf, const uint8_t* __restrict__ fixf,
                                                  double* __restrict__ Kc) {
    constexpr int ND = 24, NP = ND * (ND + 1) / 2, PN = 81;
    extern __shared__ double sm3[];
    double* sA = sm3;             // 81 x 81
    double* sB = sm3 + PN * PN;   // 81 x 24
    const int64_t E = blockIdx.x;
    if (E >= nec) return;
    const int64_t EI = E % gc.ex, EJ = (E / gc.ex) % gc.ey, EK = E / ((int64_t)gc.ex * gc.ey);
    for (int t = threadIdx.x; t < PN * PN; t += blockDim.x) sA[t] = 0.0;
    // every entry this thread adds, of all eight children, loaded first (the loads of one block
    // are then in flight together), then added child after child
    constexpr int KT = (ND * ND + 255) / 256;   // entries per thread and child (256 threads)
    double kv[8][KT];
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
        const int cx = ch & 1, cy = (ch >> 1) & 1, cz = (ch >> 2) & 1;
        const int64_t fe = (2 * EI + cx) + (int64_t)gf.ex * ((2 * EJ + cy) + (int64_t)gf.ey * (2 * EK + cz));
        const int64_t fo = (2 * EI + cx) + gf.nx * ((2 * EJ + cy) + gf.ny * (2 * EK + cz));
#pragma unroll
        for (int u = 0; u < KT; ++u) {
            const int t = threadIdx.x + u * 256;
            kv[ch][u] = 0.0;
            if (t < ND * ND) {
                const int R = t / ND, C = t % ND, la = R / 3, lb = C / 3;
                const int64_t na = fo + (la & 1) + ((la >> 1) & 1) * gf.nx + ((la >> 2) & 1) * gf.nx * gf.ny;
                const int64_t nb = fo + (lb & 1) + ((lb >> 1) & 1) * gf.nx + ((lb >> 2) & 1) * gf.nx * gf.ny;
                const bool fx = fixf && (fixf[na * 3 + R % 3] || fixf[nb * 3 + C % 3]);
                const int pi = R <= C ? packed_index(ND, R, C) : packed_index(ND, C, R);
                if (!fx) kv[ch][u] = Kf[(int64_t)pi * nef + fe];
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
        const int cx = ch & 1, cy = (ch >> 1) & 1, cz = (ch >> 2) & 1;
#pragma unroll
        for (int u = 0; u < KT; ++u) {
            const int t = threadIdx.x + u * 256;
            if (t < ND * ND) {
                const int R = t / ND, C = t % ND, la = R / 3, lb = C / 3;
                // patch nodes of the child's local nodes la, lb
                const int pa = (cx + (la & 1)) + 3 * (cy + ((la >> 1) & 1)) + 9 * (cz + ((la >> 2) & 1));
                const int pb = (cx + (lb & 1)) + 3 * (cy + ((lb >> 1) & 1)) + 9 * (cz + ((lb >> 2) & 1));
                sA[(pa * 3 + R % 3) * PN + pb * 3 + C % 3] += kv[ch][u];
            }
        }
        __syncthreads();
    }
    // B = A P (81 x 24)
    for (int t = threadIdx.x; t < PN * ND; t += blockDim.x) {
        const int P = t / ND, c = t % ND, C = c / 3, d = c % 3;
        const int X = C & 1, Y = (C >> 1) & 1, Z = (C >> 2) & 1;
        double acc = 0.0;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int x = X + (m & 1), y = Y + ((m >> 1) & 1), z = Z + ((m >> 2) & 1);   // the 8 fine nodes near C
            const double wgt = half_weight(x, X) * half_weight(y, Y) * half_weight(z, Z);
            acc = fma(wgt, sA[P * PN + (x + 3 * y + 9 * z) * 3 + d], acc);
        }
        sB[t] = acc;
    }
    __syncthreads();
    // K_E = P^T B, upper triangle in packed order
    for (int o = threadIdx.x; o < NP; o += blockDim.x) {
        int R = 0, rem = o;
        while (rem >= ND - R) {
            rem -= ND - R;
            R++;
        }
        const int C = R + rem;
        const int C1 = R / 3, d1 = R % 3;
        const int X = C1 & 1, Y = (C1 >> 1) & 1, Z = (C1 >> 2) & 1;
        double acc = 0.0;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int x = X + (m & 1), y = Y + ((m >> 1) & 1), z = Z + ((m >> 2) & 1);
            const double wgt = half_weight(x, X) * half_weight(y, Y) * half_weight(z, Z);
            acc = fma(wgt, sB[((x + 3 * y + 9 * z) * 3 + d1) * ND + C], acc);
        }
        Kc[(int64_t)o * nec + E] = acc;
    }
}

// coarse fixed mask by injection from the finer level
template <int DIM>
__global__ void k_inject_mask(Grid gf, Grid gc, const uint8_t* __restrict__ fixf, uint8_t* __restrict__ fixc) {
    int64_t N = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (N >= gc.nn) return;
    int64_t I = N % gc.nx, J = (N / gc.nx) % gc.ny, K = DIM == 3 ? N / (gc.nx * gc.ny) : 0;
    int64_t n = 2 * I + gf.nx * (2 * J + gf.ny * 2 * K);
#pragma unroll
    for (int d = 0; d < DIM; ++d) fixc[N * DIM + d] = fixf ? fixf[n * DIM + d] : 0;
}

// ------------------------------------------------------------------------------------------
// Coarsest level: dense operator (SoA dof order d*nn + node) and Gauss-Jordan inverse.
// ------------------------------------------------------------------------------------------
template <int DIM>
__global__ void k_dense_from_stencil(Grid g, const double* __restrict__ A, double* __restrict__ M) {
    constexpr int NB = nblocks<DIM>();
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
    int64_t N = g.nn * DIM;
    int64_t i = n % g.nx, j = (n / g.nx) % g.ny, k = DIM == 3 ? n / (g.nx * g.ny) : 0;
    for (int q = 0; q < NB; ++q) {
        int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = DIM == 3 ? q / 9 - 1 : 0;
        int64_t ii = i + dx, jj = j + dy, kk = k + dz;
        if (ii < 0 || ii >= g.nx || jj < 0 || jj >= g.ny || (DIM == 3 && (kk < 0 || kk >= g.nz))) continue;
        int64_t m = n + dx + g.nx * (dy + g.ny * dz);
        for (int r = 0; r < DIM; ++r)
            for (int cc = 0; cc < DIM; ++cc)
                M[((int64_t)r * g.nn + n) * N + (int64_t)cc * g.nn + m] = A[((int64_t)(q * DIM + r) * DIM + cc) * g.nn + n];
    }
}

// Gauss-Jordan inverse, one launch per pivot k.  rr / cc hold the pivot row and column of step k
// as they are before the step (unscaled); the step writes the row and column of pivot k + 1, as
// they are after it, into the other pair of buffers.  A block covers a tile of kGjRows rows x 256
// columns: each thread owns one column of the tile and walks its rows (independent loads, coalesced
// across the block), the tile's pivot-column entries and the reciprocal of the pivot sit in shared
// memory, and no thread divides an index.  In place, no pivoting: the coarse operator is SPD.
constexpr int kGjRows = 32;

__global__ void k_gj_first(int64_t n, const double* __restrict__ M, double* __restrict__ rr, double* __restrict__ cc) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        rr[t] = M[t];
        cc[t] = M[t * n];
    }
}

__global__ void __launch_bounds__(256) k_gj_step(int64_t n, int64_t k, double* __restrict__ M,
                                                 const double* __restrict__ rr, const double* __restrict__ cc,
                                                 double* __restrict__ rr_next, double* __restrict__ cc_next) {
    __shared__ double s_ip;
    __shared__ double s_c[kGjRows];
    const int64_t i0 = (int64_t)blockIdx.y * kGjRows;
    if (threadIdx.x == 0) s_ip = 1.0 / rr[k];
    if (threadIdx.x < kGjRows) s_c[threadIdx.x] = i0 + threadIdx.x < n ? cc[i0 + threadIdx.x] : 0.0;
    __syncthreads();
    const double ip = s_ip;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double rj = j == k ? 1.0 : rr[j] * ip;   // the scaled pivot row (its pivot entry unused below)
    const int rows = (int)(n - i0 < kGjRows ? n - i0 : kGjRows);
#pragma unroll 8
    for (int ri = 0; ri < rows; ++ri) {
        const int64_t i = i0 + ri;
        double* mij = M + i * n + j;
        double v;
        if (i == k) v = j == k ? ip : rj;
        else if (j == k) v = -s_c[ri] * ip;
        else v = fma(-s_c[ri], rj, *mij);
        *mij = v;
        if (i == k + 1) rr_next[j] = v;
        if (j == k + 1) cc_next[i] = v;
    }
}

// x = M b (one warp per row)
template <typename T>
__global__ void k_gemv(int64_t n, const double* __restrict__ M, const T* __restrict__ b, T* __restrict__ x) {
    int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0.0;
    for (int64_t j = lane; j < n; j += 32) s += M[row * n + j] * (double)b[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = (T)s;
}

// ------------------------------------------------------------------------------------------
// Host-side hierarchy construction.
// ------------------------------------------------------------------------------------------
static void build_stencil_level(Context& c, Level& L, const uint8_t* fixed) {
    Grid g = grid_of(L.mesh);
    int dim = L.mesh.dim;
    int nb = dim == 3 ? 27 : 9;
    L.A64.ensure((size_t)nb * dim * dim * g.nn);
    L.Dinv64.ensure((size_t)dim * dim * g.nn);
    {
        LaunchScope ls(c, -1);
        if (dim == 3)
            k_build_stencil<3><<<blocks_for(g.nn, 128), 128, 0, c.stream>>>(g, L.mesh.ne, L.Ke.p, fixed, L.A64.p, L.Dinv64.p);
        else
            k_build_stencil<2><<<blocks_for(g.nn, 128), 128, 0, c.stream>>>(g, L.mesh.ne, L.Ke.p, fixed, L.A64.p, L.Dinv64.p);
    }
    check_launch("k_build_stencil");
}

static void to_fp32(Context& c, const DArray<double>& a, DArray<float>& b) {
    b.ensure(a.n);
    LaunchScope ls(c, -1);
    k_convert<double, float><<<blocks_for((int64_t)a.n, 256), 256, 0, c.stream>>>((int64_t)a.n, a.p, b.p);
    check_launch("k_convert");
}

// In-place Gauss-Jordan inverse of an SPD dense n x n matrix (no pivoting), on the stream.
void dense_inverse(Context& c, double* M, int64_t n) {
    DArray<double> buf;
    buf.ensure((size_t)(4 * n));
    double* rr[2] = {buf.p, buf.p + n};
    double* cc[2] = {buf.p + 2 * n, buf.p + 3 * n};
    {
        LaunchScope ls(c, -1);
        k_gj_first<<<blocks_for(n, 256), 256, 0, c.stream>>>(n, M, rr[0], cc[0]);
    }
    const dim3 grid((unsigned)((n + 255) / 256), (unsigned)((n + kGjRows - 1) / kGjRows));
    for (int64_t k = 0; k < n; ++k) {
        LaunchScope ls(c, -1);
        k_gj_step<<<grid, 256, 0, c.stream>>>(n, k, M, rr[k & 1], cc[k & 1], rr[(k + 1) & 1], cc[(k + 1) & 1]);
    }
    check_launch("k_gj_step");
    UWG_CUDA(cudaStreamSynchronize(c.stream));   // the row and column buffers are released on return
}

// x = M b with a dense FP64 n x n matrix (one warp per row), vectors of type T
template <typename T>
void dense_apply(Context& c, const double* M, int64_t n, const T* b, T* x) {
    k_gemv<T><<<blocks_for(n * 32, 256), 256, 0, c.stream>>>(n, M, b, x);
}
template void dense_apply<double>(Context&, const double*, int64_t, const double*, double*);
template void dense_apply<float>(Context&, const double*, int64_t, const float*, float*);

static void coarse_inverse(Context& c, Level& L) {
    Grid g = grid_of(L.mesh);
    int dim = L.mesh.dim;
    int64_t n = g.nn * dim;
    UWG_REQUIRE(n <= 20000, UWGPU_ERR_ARGUMENT,
                "coarsest multigrid level too large for the dense solve; use more levels");
    L.ncoarse = n;
    L.Cinv.ensure((size_t)(n * n));
    UWG_CUDA(cudaMemsetAsync(L.Cinv.p, 0, (size_t)(n * n) * sizeof(double), c.stream));
    {
        LaunchScope ls(c, -1);
        if (dim == 3)
            k_dense_from_stencil<3><<<blocks_for(g.nn, 128), 128, 0, c.stream>>>(g, L.A64.p, L.Cinv.p);
        else
            k_dense_from_stencil<2><<<blocks_for(g.nn, 128), 128, 0, c.stream>>>(g, L.A64.p, L.Cinv.p);
    }
    check_launch("k_dense_from_stencil");
    dense_inverse(c, L.Cinv.p, n);
}

void build_operator(Context& c, int levels, bool need32) {
    UWG_REQUIRE(c.assembled, UWGPU_ERR_STATE, "operator requested before assembly");
    const MeshDesc& m = c.mesh;
    int dim = m.dim;
    UWG_REQUIRE(m.nn < ((int64_t)1 << 32), UWGPU_ERR_TOO_LARGE, "node count beyond 32-bit node indexing");
    // the number of levels the mesh admits (each coarsening halves every axis)
    int maxlev = 1;
    {
        int nel[3] = {m.nel[0], m.nel[1], dim == 3 ? m.nel[2] : 2};
        while (maxlev < kMaxLevels) {
            bool ok = true;
            for (int d = 0; d < dim; ++d) ok = ok && (nel[d] % 2 == 0) && nel[d] >= 2;
            if (!ok) break;
            for (int d = 0; d < dim; ++d) nel[d] /= 2;
            maxlev++;
        }
    }
    if (levels < 1) levels = 1;
    if (levels > maxlev) levels = maxlev;
    c.nlevels = levels;
    // captured inner-CG graphs bake in buffer addresses and mesh sizes: drop them on rebuild
    for (auto& pg : c.pcg_graphs)
        if (pg.exec) cudaGraphExecDestroy(pg.exec);
    c.pcg_graphs.clear();
    Level& L0 = c.levels[0];
    L0.mesh = m;
    L0.fixed.ensure((size_t)m.nn * dim);
    if (c.has_bc)
        UWG_CUDA(cudaMemcpyAsync(L0.fixed.p, c.fixed.p, (size_t)m.nn * dim, cudaMemcpyDeviceToDevice, c.stream));
    else
        UWG_CUDA(cudaMemsetAsync(L0.fixed.p, 0, (size_t)m.nn * dim, c.stream));
    build_stencil_level(c, L0, L0.fixed.p);
    for (int l = 1; l < levels; ++l) {
        Level& F = c.levels[l - 1];
        Level& C = c.levels[l];
        C.mesh = F.mesh;
        for (int d = 0; d < dim; ++d) C.mesh.nel[d] = F.mesh.nel[d] / 2;
        C.mesh.nnx = C.mesh.nel[0] + 1;
        C.mesh.nny = C.mesh.nel[1] + 1;
        C.mesh.nnz = dim == 3 ? C.mesh.nel[2] + 1 : 1;
        C.mesh.nn = C.mesh.nnx * C.mesh.nny * C.mesh.nnz;
        C.mesh.ne = (int64_t)C.mesh.nel[0] * C.mesh.nel[1] * (dim == 3 ? C.mesh.nel[2] : 1);
        Grid gf = grid_of(F.mesh), gc = grid_of(C.mesh);
        int nd = (1 << dim) * dim;
        C.Ke.ensure((size_t)packed_size(nd) * C.mesh.ne);
        C.fixed.ensure((size_t)C.mesh.nn * dim);
        {
            LaunchScope ls(c, -1);
            size_t smem = (size_t)(1 << dim) * nd * nd * sizeof(double);
            if (dim == 3) {
                const size_t smem3 = (size_t)(81 * 81 + 81 * 24) * sizeof(double);
                UWG_CUDA(cudaFuncSetAttribute(k_galerkin3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3));
                k_galerkin3<<<(unsigned)C.mesh.ne, 256, smem3, c.stream>>>(gf, gc, F.mesh.ne, C.mesh.ne, F.Ke.p, F.fixed.p,
                                                                          C.Ke.p);
            } else {
                k_galerkin<2><<<(unsigned)C.mesh.ne, 64, smem, c.stream>>>(gf, gc, F.mesh.ne, C.mesh.ne, F.Ke.p, F.fixed.p, C.Ke.p);
            }
        }
        check_launch("k_galerkin");
        {
            LaunchScope ls(c, -1);
            if (dim == 3)
                k_inject_mask<3><<<blocks_for(gc.nn, 256), 256, 0, c.stream>>>(gf, gc, F.fixed.p, C.fixed.p);
            else
                k_inject_mask<2><<<blocks_for(gc.nn, 256), 256, 0, c.stream>>>(gf, gc, F.fixed.p, C.fixed.p);
        }
        check_launch("k_inject_mask");
        build_stencil_level(c, C, C.fixed.p);
    }
    for (int l = 0; l < levels; ++l) {
        Level& L = c.levels[l];
        L.lmax = 0.0;
        size_t nv = (size_t)L.mesh.nn * dim;
        L.r64.ensure(nv);
        L.x64.ensure(nv);
        L.b64.ensure(nv);
        L.t64.ensure(nv);
        L.has32 = false;
        L.has16 = false;
        if (need32) {
            to_fp32(c, L.A64, L.A32);
            to_fp32(c, L.Dinv64, L.Dinv32);
            {
                const Grid g = grid_of(L.mesh);
                const int np = dim == 3 ? 14 : 5;   // neighbour pairs
                L.A16.ensure((size_t)np * dim * dim * g.nn);
                L.S16.ensure((size_t)dim * g.nn);
                LaunchScope ls(c, -1);
                if (dim == 3)
                    k_to_fp16_rows<3><<<blocks_for(3 * g.nn, 256), 256, 0, c.stream>>>(g, L.A32.p, L.A16.p, L.S16.p);
                else
                    k_to_fp16_rows<2><<<blocks_for(2 * g.nn, 256), 256, 0, c.stream>>>(g, L.A32.p, L.A16.p, L.S16.p);
                check_launch("k_to_fp16_rows");
                L.has16 = true;
            }
            L.r32.ensure(nv);
            L.x32.ensure(nv);
            L.b32.ensure(nv);
            L.t32.ensure(nv);
            L.has32 = true;
        }
    }
    if (levels > 1) coarse_inverse(c, c.levels[levels - 1]);
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    c.operator_built = true;
    c.operator_levels = levels;
    c.operator_has32 = need32;
}

// ------------------------------------------------------------------------------------------
// Level operations used by the solver.
// ------------------------------------------------------------------------------------------
template <typename T>
static const T* stencil_of(const Level& L);
template <>
const double* stencil_of<double>(const Level& L) { return L.A64.p; }
template <>
const float* stencil_of<float>(const Level& L) { return L.A32.p; }
template <typename T>
static const T* dinv_of(const Level& L);
template <>
const double* dinv_of<double>(const Level& L) { return L.Dinv64.p; }
template <>
const float* dinv_of<float>(const Level& L) { return L.Dinv32.p; }

template <typename T>
void level_apply(Context& c, const Level& L, const T* x, T* y) {
    Grid g = grid_of(L.mesh);
    int D = g.dim, NB = D == 3 ? 27 : 9;
    note_work(c, UWGPU_KERNEL_APPLY, (double)g.nn * (NB * D * D + 2 * D) * sizeof(T), 2.0 * g.nn * NB * D * D);
    LaunchScope ls(c, UWGPU_KERNEL_APPLY);
    if (g.dim == 3)
        k_apply<3, T><<<blocks_for(g.nn, kRowThreads / 3), kRowThreads, 0, c.stream>>>(g, stencil_of<T>(L), x, nullptr, y);
    else
        k_apply<2, T><<<blocks_for(g.nn, kRowThreads / 2), kRowThreads, 0, c.stream>>>(g, stencil_of<T>(L), x, nullptr, y);
}

template <typename T>
void level_residual(Context& c, const Level& L, const T* x, const T* b, T* r) {
    Grid g = grid_of(L.mesh);
    int D = g.dim, NB = D == 3 ? 27 : 9;
    if constexpr (std::is_same<T, float>::value) {
        if (L.has16 && c.smooth16) {
            note_work(c, UWGPU_KERNEL_APPLY, (double)g.nn * ((NB + 1) / 2 * D * D * 4 + 4 * D * 4), 2.0 * g.nn * NB * D * D);
            LaunchScope ls(c, UWGPU_KERNEL_APPLY);
            if (g.dim == 3)
                k_residual_h<3><<<blocks_for(g.nn, kRowThreads / 3), kRowThreads, 0, c.stream>>>(g, L.A16.p, L.S16.p, x, b, r);
            else
                k_residual_h<2><<<blocks_for(g.nn, kRowThreads / 2), kRowThreads, 0, c.stream>>>(g, L.A16.p, L.S16.p, x, b, r);
            return;
        }
    }
    note_work(c, UWGPU_KERNEL_APPLY, (double)g.nn * (NB * D * D + 3 * D) * sizeof(T), 2.0 * g.nn * NB * D * D);
    LaunchScope ls(c, UWGPU_KERNEL_APPLY);
    if (g.dim == 3)
        k_apply<3, T><<<blocks_for(g.nn, kRowThreads / 3), kRowThreads, 0, c.stream>>>(g, stencil_of<T>(L), x, b, r);
    else
        k_apply<2, T><<<blocks_for(g.nn, kRowThreads / 2), kRowThreads, 0, c.stream>>>(g, stencil_of<T>(L), x, b, r);
}

// symmetric sweep: colours ascending then descending
template <typename T>
void level_smooth(Context& c, const Level& L, const T* b, T* x, int sweeps, bool zero_init) {
    Grid g = grid_of(L.mesh);
    int D = g.dim, NB = D == 3 ? 27 : 9;
    note_work(c, UWGPU_KERNEL_SMOOTH, (double)sweeps * 2.0 * g.nn * (NB * D * D + D * D + 3 * D) * sizeof(T),
              (double)sweeps * 2.0 * 2.0 * g.nn * (NB * D * D + D * D));
    // one cooperative launch runs every colour of every sweep with grid-wide barriers between
    // colours; the grid is sized so that all of its blocks are resident (a requirement of the
    // cooperative launch), and each thread strides over the nodes of the current colour.
    static int max_blocks[2][2] = {{0, 0}, {0, 0}};
    int di = D == 3 ? 1 : 0, ti = sizeof(T) == 8 ? 1 : 0;
    void* fn = D == 3 ? (void*)k_gs_sweeps<3, T> : (void*)k_gs_sweeps<2, T>;
    if (max_blocks[di][ti] == 0) {
        int per_sm = 0, sms = 0, dev = 0;
        UWG_CUDA(cudaGetDevice(&dev));
        UWG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        UWG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kRowThreads, 0));
        UWG_REQUIRE(per_sm > 0, UWGPU_ERR_CUDA, "smoother kernel cannot be made resident");
        max_blocks[di][ti] = per_sm * sms;
    }
    int64_t per_colour = (g.nn + (1 << D) - 1) >> D;
    int64_t npb = kRowThreads / D;
    int64_t want = (per_colour + npb - 1) / npb;
    int blocks = (int)(want < max_blocks[di][ti] ? want : max_blocks[di][ti]);
    if (blocks < 1) blocks = 1;
    const T* A = stencil_of<T>(L);
    const T* Di = dinv_of<T>(L);
    int zi = zero_init ? 1 : 0;
    void* args[] = {(void*)&g, (void*)&A, (void*)&Di, (void*)&b, (void*)&x, (void*)&sweeps, (void*)&zi};
    LaunchScope ls(c, UWGPU_KERNEL_SMOOTH);
    UWG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kRowThreads), args, 0, c.stream));
}

template <typename T>
void level_restrict(Context& c, const Level& F, const Level& C, const T* rf, T* rc) {
    Grid gf = grid_of(F.mesh), gc = grid_of(C.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_TRANSFER);
    if (gf.dim == 3)
        k_restrict<3, T><<<blocks_for(gc.nn, 256), 256, 0, c.stream>>>(gf, gc, rf, rc, F.fixed.p, C.fixed.p);
    else
        k_restrict<2, T><<<blocks_for(gc.nn, 256), 256, 0, c.stream>>>(gf, gc, rf, rc, F.fixed.p, C.fixed.p);
}

template <typename T>
void level_prolong_add(Context& c, const Level& F, const Level& C, const T* xc, T* xf) {
    Grid gf = grid_of(F.mesh), gc = grid_of(C.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_TRANSFER);
    if (gf.dim == 3)
        k_prolong_add<3, T><<<blocks_for(gf.nn, 256), 256, 0, c.stream>>>(gf, gc, xc, xf, F.fixed.p, C.fixed.p);
    else
        k_prolong_add<2, T><<<blocks_for(gf.nn, 256), 256, 0, c.stream>>>(gf, gc, xc, xf, F.fixed.p, C.fixed.p);
}

template <typename T>
void level_coarse_solve(Context& c, const Level& L, const T* b, T* x) {
    LaunchScope ls(c, UWGPU_KERNEL_TRANSFER);
    k_gemv<T><<<blocks_for(L.ncoarse * 32, 256), 256, 0, c.stream>>>(L.ncoarse, L.Cinv.p, b, x);
}

template void level_apply<double>(Context&, const Level&, const double*, double*);
template void level_apply<float>(Context&, const Level&, const float*, float*);
template void level_residual<double>(Context&, const Level&, const double*, const double*, double*);
template void level_residual<float>(Context&, const Level&, const float*, const float*, float*);
template void level_smooth<double>(Context&, const Level&, const double*, double*, int, bool);
template void level_smooth<float>(Context&, const Level&, const float*, float*, int, bool);

template <typename T>
static T* tmp_of(Level& L);
template <>
double* tmp_of<double>(Level& L) { return L.t64.p; }
template <>
float* tmp_of<float>(Level& L) { return L.t32.p; }
template <typename T>
static T* dvec_of(Level& L);
template <>
double* dvec_of<double>(Level& L) { return L.r64.p; }
template <>
float* dvec_of<float>(Level& L) { return L.r32.p; }

// Chebyshev smoothing of `degree` steps on [lmax/10, 1.1 lmax] of D^-1 A (the eigenvalue
// bounds PETSc's Chebyshev smoother uses by default).  Uses the level's t and r vectors as the
// alternate iterate and the direction.
template <typename T>
void level_cheb(Context& c, Level& L, const T* b, T* x, int degree, bool zero_init) {
    Grid g = grid_of(L.mesh);
    int D = g.dim, NB = D == 3 ? 27 : 9;
    double lmax = 1.1 * L.lmax, lmin = 0.1 * L.lmax;
    double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    double sigma = theta / delta, rho = 1.0 / sigma;
    T* alt = tmp_of<T>(L);
    T* d = dvec_of<T>(L);
    bool half = false;
    if constexpr (std::is_same<T, float>::value) half = L.has16 && c.smooth16;
    if (half)
        note_work(c, UWGPU_KERNEL_SMOOTH, (double)degree * g.nn * ((NB + 1) / 2 * D * D * 4 + (D * D + 6 * D) * 4),
                  (double)degree * 2.0 * g.nn * (NB * D * D + D * D));
    else
        note_work(c, UWGPU_KERNEL_SMOOTH, (double)degree * g.nn * (NB * D * D + D * D + 5 * D) * sizeof(T),
                  (double)degree * 2.0 * g.nn * (NB * D * D + D * D));
    const T* cur = zero_init ? nullptr : x;
    for (int k = 0; k < degree; ++k) {
        T* dst = (k % 2 == 0) ? alt : x;
        double c1 = 0.0, c2;
        if (k == 0) {
            c2 = 1.0 / theta;
        } else {
            double rho_new = 1.0 / (2.0 * sigma - rho);
            c1 = rho_new * rho;
            c2 = 2.0 * rho_new / delta;
            rho = rho_new;
        }
        LaunchScope ls(c, UWGPU_KERNEL_SMOOTH);
        if constexpr (std::is_same<T, float>::value) {
            if (half) {
                if (D == 3)
                    k_cheb_step_h<3><<<blocks_for(g.nn, kRowThreads / 3), kRowThreads, 0, c.stream>>>(
                        g, L.A16.p, L.S16.p, L.Dinv32.p, b, cur, dst, d, (float)c1, (float)c2, k == 0);
                else
                    k_cheb_step_h<2><<<blocks_for(g.nn, kRowThreads / 2), kRowThreads, 0, c.stream>>>(
                        g, L.A16.p, L.S16.p, L.Dinv32.p, b, cur, dst, d, (float)c1, (float)c2, k == 0);
                cur = dst;
                continue;
            }
        }
        if (D == 3)
            k_cheb_step<3, T><<<blocks_for(g.nn, kRowThreads / 3), kRowThreads, 0, c.stream>>>(
                g, stencil_of<T>(L), dinv_of<T>(L), b, cur, dst, d, (T)c1, (T)c2, k == 0);
        else
            k_cheb_step<2, T><<<blocks_for(g.nn, kRowThreads / 2), kRowThreads, 0, c.stream>>>(
                g, stencil_of<T>(L), dinv_of<T>(L), b, cur, dst, d, (T)c1, (T)c2, k == 0);
        cur = dst;
    }
    if (degree % 2 == 1) UWG_CUDA(cudaMemcpyAsync(x, alt, (size_t)g.nn * D * sizeof(T), cudaMemcpyDeviceToDevice, c.stream));
    if (degree == 0 && zero_init) UWG_CUDA(cudaMemsetAsync(x, 0, (size_t)g.nn * D * sizeof(T), c.stream));
}

template <typename T>
void level_dinv(Context& c, const Level& L, const T* y, T* z) {
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, -1);
    if (g.dim == 3) k_dinv<3, T><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, dinv_of<T>(L), y, z);
    else k_dinv<2, T><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, dinv_of<T>(L), y, z);
}

template void level_cheb<double>(Context&, Level&, const double*, double*, int, bool);
template void level_cheb<float>(Context&, Level&, const float*, float*, int, bool);
template void level_dinv<double>(Context&, const Level&, const double*, double*);
template void level_restrict<double>(Context&, const Level&, const Level&, const double*, double*);
template void level_restrict<float>(Context&, const Level&, const Level&, const float*, float*);
template void level_prolong_add<double>(Context&, const Level&, const Level&, const double*, double*);
template void level_prolong_add<float>(Context&, const Level&, const Level&, const float*, float*);
template void level_coarse_solve<double>(Context&, const Level&, const double*, double*);
template void level_coarse_solve<float>(Context&, const Level&, const float*, float*);

void apply_fine(Context& c, bool fp32, const double* x, double* y) {
    Level& L = c.levels[0];
    if (!fp32) {
        level_apply<double>(c, L, x, y);
    } else {
        size_t nv = (size_t)L.mesh.nn * L.mesh.dim;
        {
            LaunchScope ls(c, -1);
            k_convert<double, float><<<blocks_for((int64_t)nv, 256), 256, 0, c.stream>>>((int64_t)nv, x, L.x32.p);
        }
        level_apply<float>(c, L, L.x32.p, L.r32.p);
        {
            LaunchScope ls(c, -1);
            k_convert<float, double><<<blocks_for((int64_t)nv, 256), 256, 0, c.stream>>>((int64_t)nv, L.r32.p, y);
        }
    }
    check_launch("apply_fine");
}

// ------------------------------------------------------------------------------------------
// Gradient operators on the fine level (P0 pressure).
// G_e[a][d] = -s_{d,a} * prod_{q != d} h_q / 2^(dim-1): the 2^dim-point Gauss integral of
// -dN_a/dx_d over the affine element.
// ------------------------------------------------------------------------------------------
// Element widths per axis, precomputed once per mesh (h[off[d] + i] = x_{i+1} - x_i along d), so
// the kernels do no FP64 division to recover the geometry.
struct GeoArgs {
    const double* h;
    int off[3];
};

template <int DIM>
__device__ __forceinline__ void element_h(const GeoArgs& a, int64_t ie, int64_t je, int64_t ke, double h[3]) {
    int64_t idx[3] = {ie, je, ke};
#pragma unroll
    for (int d = 0; d < DIM; ++d) h[d] = __ldg(a.h + a.off[d] + idx[d]);
}

template <int DIM>
__device__ __forceinline__ double gval(const double h[3], int a, int d) {
    double area = 1.0;
#pragma unroll
    for (int q = 0; q < DIM; ++q)
        if (q != d) area *= h[q];
    double s = ((a >> d) & 1) ? 1.0 : -1.0;
    return -s * area * (DIM == 3 ? 0.25 : 0.5);
}

// u = G p   (velocity SoA, fixed dofs zero)
template <int DIM>
__global__ void k_G(Grid g, GeoArgs geo, const double* __restrict__ p, const uint8_t* __restrict__ fixed,
                    double* __restrict__ u) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
    int64_t idx[3] = {n % g.nx, (n / g.nx) % g.ny, DIM == 3 ? n / (g.nx * g.ny) : 0};
    int64_t ecount[3] = {g.ex, g.ey, g.ez};
    double acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = 0.0;
#pragma unroll
    for (int o = 0; o < (1 << DIM); ++o) {
        int64_t e3[3];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d >= DIM) { e3[d] = 0; continue; }
            e3[d] = idx[d] - ((o >> d) & 1);
            if (e3[d] < 0 || e3[d] >= ecount[d]) ok = false;
        }
        if (!ok) continue;
        int a = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) a |= ((o >> d) & 1) << d;
        int64_t e = e3[0] + (int64_t)g.ex * (e3[1] + (int64_t)g.ey * e3[2]);
        double h[3];
        element_h<DIM>(geo, e3[0], e3[1], e3[2], h);
        double pe = p[e];
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += gval<DIM>(h, a, d) * pe;
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) u[(int64_t)d * g.nn + n] = (fixed && fixed[n * DIM + d]) ? 0.0 : acc[d];
}

// p = G^T u
template <int DIM>
__global__ void k_GT(Grid g, GeoArgs geo, const double* __restrict__ u, const uint8_t* __restrict__ fixed,
                     double* __restrict__ p) {
    int64_t ne = (int64_t)g.ex * g.ey * g.ez;
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int64_t ie = e % g.ex, je = (e / g.ex) % g.ey, ke = DIM == 3 ? e / ((int64_t)g.ex * g.ey) : 0;
    double h[3];
    element_h<DIM>(geo, ie, je, ke, h);
    int64_t base = ie + g.nx * (je + g.ny * ke);
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < (1 << DIM); ++a) {
        int64_t n = base + (a & 1) + ((a >> 1) & 1) * g.nx + (DIM == 3 ? ((a >> 2) & 1) * g.nx * g.ny : 0);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            if (!fixed || !fixed[n * DIM + d]) acc += gval<DIM>(h, a, d) * u[(int64_t)d * g.nn + n];
    }
    p[e] = acc;
}

// f (nodal SoA) = sum of element force vectors, fixed dofs zero
template <int DIM>
__global__ void k_gather_force(Grid g, const double* __restrict__ fe, int64_t ne, const uint8_t* __restrict__ fixed,
                               double* __restrict__ f) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
    int64_t idx[3] = {n % g.nx, (n / g.nx) % g.ny, DIM == 3 ? n / (g.nx * g.ny) : 0};
    int64_t ecount[3] = {g.ex, g.ey, g.ez};
    double acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = 0.0;
#pragma unroll
    for (int o = 0; o < (1 << DIM); ++o) {
        int64_t e3[3];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d >= DIM) { e3[d] = 0; continue; }
            e3[d] = idx[d] - ((o >> d) & 1);
            if (e3[d] < 0 || e3[d] >= ecount[d]) ok = false;
        }
        if (!ok) continue;
        int64_t e = e3[0] + (int64_t)g.ex * (e3[1] + (int64_t)g.ey * e3[2]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += fe[(int64_t)(o * DIM + d) * ne + e];
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) f[(int64_t)d * g.nn + n] = (fixed && fixed[n * DIM + d]) ? 0.0 : acc[d];
}

// gkgdiag: diag(G^T diag(K)^{-1} G) per element, using the assembled diagonal
template <int DIM>
__global__ void k_gkgdiag(Grid g, GeoArgs geo, const double* __restrict__ A, const uint8_t* __restrict__ fixed,
                          double* __restrict__ S) {
    int64_t ne = (int64_t)g.ex * g.ey * g.ez;
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    constexpr int NB = nblocks<DIM>();
    int64_t ie = e % g.ex, je = (e / g.ex) % g.ey, ke = DIM == 3 ? e / ((int64_t)g.ex * g.ey) : 0;
    double h[3];
    element_h<DIM>(geo, ie, je, ke, h);
    int64_t base = ie + g.nx * (je + g.ny * ke);
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < (1 << DIM); ++a) {
        int64_t n = base + (a & 1) + ((a >> 1) & 1) * g.nx + (DIM == 3 ? ((a >> 2) & 1) * g.nx * g.ny : 0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            if (fixed && fixed[n * DIM + d]) continue;
            double kd = A[((int64_t)((NB / 2) * DIM + d) * DIM + d) * g.nn + n];
            double gv = gval<DIM>(h, a, d);
            acc += gv * gv / kd;
        }
    }
    S[e] = acc;
}

static GeoArgs geo_of(Context& c, const MeshDesc& m) {
    // widths of the fine mesh, built on first use after the mesh was set
    if (c.elem_h_for != m.nel[0] + 4096LL * (m.nel[1] + 4096LL * m.nel[2]) || !c.elem_h.p) {
        std::vector<double> h;
        for (int d = 0; d < m.dim; ++d)
            for (int i = 0; i < m.nel[d]; ++i)
                h.push_back(node_coord_1d(i + 1, m.nel[d], m.min[d], m.max[d]) - node_coord_1d(i, m.nel[d], m.min[d], m.max[d]));
        c.elem_h.ensure(h.size());
        UWG_CUDA(cudaMemcpy(c.elem_h.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        c.elem_h_for = m.nel[0] + 4096LL * (m.nel[1] + 4096LL * m.nel[2]);
    }
    GeoArgs a;
    a.h = c.elem_h.p;
    a.off[0] = 0;
    a.off[1] = m.nel[0];
    a.off[2] = m.nel[0] + m.nel[1];
    return a;
}

const double* fine_widths(Context& c, int off[3]) {
    GeoArgs a = geo_of(c, c.levels[0].mesh);
    for (int d = 0; d < 3; ++d) off[d] = a.off[d];
    return a.h;
}

// ||G||_inf over the free velocity rows: max over free dofs (n, d) of sum_e |G_(n,d),e|
template <int DIM>
__global__ void k_g_rowsum_max(Grid g, GeoArgs geo, const uint8_t* __restrict__ fixed,
                               unsigned long long* __restrict__ out) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double best = 0.0;
    if (n < g.nn) {
        int64_t idx[3] = {n % g.nx, (n / g.nx) % g.ny, DIM == 3 ? n / (g.nx * g.ny) : 0};
        int64_t ecount[3] = {g.ex, g.ey, g.ez};
        double acc[3] = {0.0, 0.0, 0.0};
        for (int o = 0; o < (1 << DIM); ++o) {
            int64_t e3[3] = {0, 0, 0};
            bool ok = true;
            for (int d = 0; d < DIM; ++d) {
                e3[d] = idx[d] - ((o >> d) & 1);
                if (e3[d] < 0 || e3[d] >= ecount[d]) ok = false;
            }
            if (!ok) continue;
            double h[3];
            element_h<DIM>(geo, e3[0], e3[1], e3[2], h);
            for (int d = 0; d < DIM; ++d) acc[d] += fabs(gval<DIM>(h, o, d));
        }
        for (int d = 0; d < DIM; ++d)
            if (!(fixed && fixed[n * DIM + d])) best = fmax(best, acc[d]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
    // non-negative doubles order like their bit patterns
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

double g_inf_norm(Context& c) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    c.scratch.ensure(8);
    auto* out = reinterpret_cast<unsigned long long*>(c.scratch.p);
    UWG_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long), c.stream));
    {
        LaunchScope ls(c, -1);
        if (g.dim == 3)
            k_g_rowsum_max<3><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), L.fixed.p, out);
        else
            k_g_rowsum_max<2><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), L.fixed.p, out);
    }
    check_launch("k_g_rowsum_max");
    unsigned long long bits = 0;
    UWG_CUDA(cudaMemcpyAsync(c.host_scalars, out, sizeof(bits), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    std::memcpy(&bits, c.host_scalars, sizeof(bits));
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    return v;
}

void op_G(Context& c, const double* p, double* u) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    if (g.dim == 3)
        k_G<3><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), p, L.fixed.p, u);
    else
        k_G<2><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), p, L.fixed.p, u);
}

void op_GT(Context& c, const double* u, double* p) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    if (g.dim == 3)
        k_GT<3><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), u, L.fixed.p, p);
    else
        k_GT<2><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), u, L.fixed.p, p);
}

void op_GT_unmasked(Context& c, const double* u, double* p) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    if (g.dim == 3)
        k_GT<3><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), u, nullptr, p);
    else
        k_GT<2><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), u, nullptr, p);
}

void gather_force(Context& c, double* f) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    if (g.dim == 3)
        k_gather_force<3><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, c.fe.p, L.mesh.ne, L.fixed.p, f);
    else
        k_gather_force<2><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, c.fe.p, L.mesh.ne, L.fixed.p, f);
}

// Scaled BFBt weights W = 1/rowmax(K) per velocity dof (fixed dofs 0), pc_ScaledGtKG.c:735-760
template <int DIM>
__global__ void k_rowmax_weights(Grid g, const double* __restrict__ A, const uint8_t* __restrict__ fixed,
                                 double* __restrict__ W) {
    constexpr int NB = nblocks<DIM>();
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
        double mx = -1e300;
        for (int q = 0; q < NB; ++q)
#pragma unroll
            for (int cc = 0; cc < DIM; ++cc) {
                double v = A[((int64_t)(q * DIM + r) * DIM + cc) * g.nn + n];
                mx = v > mx ? v : mx;
            }
        W[(int64_t)r * g.nn + n] = (fixed && fixed[n * DIM + r]) ? 0.0 : 1.0 / mx;
    }
}

void bfbt_weights(Context& c, double* W) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, -1);
    if (g.dim == 3)
        k_rowmax_weights<3><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, L.A64.p, L.fixed.p, W);
    else
        k_rowmax_weights<2><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, L.A64.p, L.fixed.p, W);
}

// ------------------------------------------------------------------------------------------
// FP32 forms of G and G^T for the middle of the scaled BFBt apply in the mixed form
// (s = W G p, then G^T s); the inner G^T W G solves use its explicit stencil (gwg_stencil.cu).
// ------------------------------------------------------------------------------------------
template <typename T>
struct GeoT {
    const T* h;     // element widths per axis
    int off[3];
};

template <int DIM, typename T>
__device__ __forceinline__ T gvalT(const T h[3], int a, int d) {
    T area = (T)1;
#pragma unroll
    for (int q = 0; q < DIM; ++q)
        if (q != d) area *= h[q];
    T s = ((a >> d) & 1) ? (T)1 : (T)-1;
    return -s * area * (T)(DIM == 3 ? 0.25 : 0.5);
}

// s = W (G p)
template <int DIM, typename T>
__global__ void k_wgp(Grid g, GeoT<T> geo, const T* __restrict__ p, const T* __restrict__ W,
                         const uint8_t* __restrict__ fixed, T* __restrict__ s) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nn) return;
    int64_t idx[3] = {n % g.nx, (n / g.nx) % g.ny, DIM == 3 ? n / (g.nx * g.ny) : 0};
    int64_t ecount[3] = {g.ex, g.ey, g.ez};
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = (T)0;
#pragma unroll
    for (int o = 0; o < (1 << DIM); ++o) {
        int64_t e3[3] = {0, 0, 0};
        bool ok = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            e3[d] = idx[d] - ((o >> d) & 1);
            if (e3[d] < 0 || e3[d] >= ecount[d]) ok = false;
        }
        if (!ok) continue;
        int64_t e = e3[0] + (int64_t)g.ex * (e3[1] + (int64_t)g.ey * e3[2]);
        T h[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) h[d] = __ldg(geo.h + geo.off[d] + e3[d]);
        T pe = p[e];
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = fma(gvalT<DIM, T>(h, o, d), pe, acc[d]);
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        s[(int64_t)d * g.nn + n] = (fixed && fixed[n * DIM + d]) ? (T)0 : acc[d] * W[(int64_t)d * g.nn + n];
}

// q = G^T s
template <int DIM, typename T>
__global__ void k_gts(Grid g, GeoT<T> geo, const T* __restrict__ s, T* __restrict__ q) {
    int64_t ne = (int64_t)g.ex * g.ey * g.ez;
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int64_t i3[3] = {e % g.ex, (e / g.ex) % g.ey, DIM == 3 ? e / ((int64_t)g.ex * g.ey) : 0};
    T h[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) h[d] = __ldg(geo.h + geo.off[d] + i3[d]);
    int64_t base = i3[0] + g.nx * (i3[1] + g.ny * i3[2]);
    T acc = (T)0;
#pragma unroll
    for (int a = 0; a < (1 << DIM); ++a) {
        int64_t n = base + (a & 1) + ((a >> 1) & 1) * g.nx + (DIM == 3 ? ((a >> 2) & 1) * g.nx * g.ny : 0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc = fma(gvalT<DIM, T>(h, a, d), s[(int64_t)d * g.nn + n], acc);
    }
    q[e] = acc;
}

static GeoT<float> geo_f32(Context& c, const MeshDesc& m) {
    GeoArgs a = geo_of(c, m);
    size_t n = (size_t)m.nel[0] + m.nel[1] + (m.dim == 3 ? m.nel[2] : 0);
    if (c.elem_h32_for != c.elem_h_for) {
        c.elem_h32.ensure(n);
        LaunchScope ls(c, -1);
        k_convert<double, float><<<blocks_for((int64_t)n, 256), 256, 0, c.stream>>>((int64_t)n, a.h, c.elem_h32.p);
        c.elem_h32_for = c.elem_h_for;
    }
    GeoT<float> g;
    g.h = c.elem_h32.p;
    for (int d = 0; d < 3; ++d) g.off[d] = a.off[d];
    return g;
}

// FP32 pieces of the scaled BFBt apply: s = W (G p) and q = G^T s
void op_wg32(Context& c, const float* p, const float* W, float* s) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    GeoT<float> geo = geo_f32(c, L.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
    if (g.dim == 3) k_wgp<3, float><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, geo, p, W, L.fixed.p, s);
    else k_wgp<2, float><<<blocks_for(g.nn, 256), 256, 0, c.stream>>>(g, geo, p, W, L.fixed.p, s);
}

void op_gt32(Context& c, const float* s, float* q) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    GeoT<float> geo = geo_f32(c, L.mesh);
    LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
    if (g.dim == 3) k_gts<3, float><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo, s, q);
    else k_gts<2, float><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo, s, q);
}

void to_float(Context& c, const double* a, float* b, int64_t n) {
    LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
    k_convert<double, float><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, a, b);
}

void to_double(Context& c, const float* a, double* b, int64_t n) {
    LaunchScope ls(c, UWGPU_KERNEL_SCHUR_PC);
    k_convert<float, double><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, a, b);
}

void gkgdiag(Context& c, double* S) {
    const Level& L = c.levels[0];
    Grid g = grid_of(L.mesh);
    LaunchScope ls(c, -1);
    if (g.dim == 3)
        k_gkgdiag<3><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), L.A64.p, L.fixed.p, S);
    else
        k_gkgdiag<2><<<blocks_for(L.mesh.ne, 256), 256, 0, c.stream>>>(g, geo_of(c, L.mesh), L.A64.p, L.fixed.p, S);
}

}  // namespace uwg
