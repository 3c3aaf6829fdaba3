// BSSCR Schur-complement Stokes solve on the device.
//
// Reference behaviour (paths relative to the Underworld 1.x tree):
//   driver     Solvers/KSPSolvers/src/BSSCR/auglag-driver-DGTGD.c:53-441 (penalty 0):
//              h_hat = h - G^T K^{-1} f; Schur solve S p = h_hat with S = G^T K^{-1} G;
//              null-space removal (ksp_pressure_nullspace.c:82-176); back-solve u = K^{-1}(f - G p)
//   Schur PC   preconditioner.c:130-215 ("uw": approxS from UzawaPreconditionerTerm; "gkgdiag")
//   A11 solve  FGMRES preconditioned by a multiplicative V-cycle (mg.c:42-132, PETScMGSolver.c)
//
// Precision forms.  FP64: every vector, operator and smoother in FP64.  Mixed: each velocity
// (A11) solve is FP64 iterative refinement around an FP32 FGMRES whose V-cycle (stencils,
// smoothers, transfers) runs in FP32, with FP64 kept for the refinement residuals, the pressure
// Schur-complement iteration and the coarsest-level solve.
#include <chrono>
#include <cmath>
#include <cstring>

#include "internal.cuh"
#include "unet.cuh"

namespace uwg {

template <typename T> void level_apply(Context&, const Level&, const T*, T*);
template <typename T> void level_residual(Context&, const Level&, const T*, const T*, T*);
template <typename T> void level_smooth(Context&, const Level&, const T*, T*, int, bool);
template <typename T> void level_restrict(Context&, const Level&, const Level&, const T*, T*);
template <typename T> void level_prolong_add(Context&, const Level&, const Level&, const T*, T*);
template <typename T> void level_coarse_solve(Context&, const Level&, const T*, T*);
template <typename T> void level_cheb(Context&, Level&, const T*, T*, int, bool);
template <typename T> void level_dinv(Context&, const Level&, const T*, T*);
void op_G(Context& c, const double* p, double* u);
void op_GT(Context& c, const double* u, double* p);
void op_GT_unmasked(Context& c, const double* u, double* p);
void gather_force(Context& c, double* f);
void gkgdiag(Context& c, double* S);
void bfbt_weights(Context& c, double* W);
void gwg_stencil_build(Context& c, const double* W, double* A, double* dinv);
void gwg_stencil_fp32(Context& c, const double* A, const double* dinv, float* A32, float* dinv32);
void gwg_stencil_apply(Context& c, const double* A, const double* x, double* y, double* scal);
int gwg_cg(Context& c, const double* A, const double* dinv, const double* b, double* x, double rtol, int maxit,
           double* work, double* scal);
int gwg_cg32(Context& c, const float* A, const float* dinv, const double* b, float* x, double rtol, int maxit,
             float* work, double* scal);
double g_inf_norm(Context& c);
bool gwg_mg_build(Context& c, const double* A0, const double* dinv0, bool need32, bool const_null);
bool gwg_cc_build(Context& c, const double* A);
int gwg_cg_mg(Context& c, const double* A, const double* dinv, const double* b, double* x, double rtol, int maxit,
              double* work, double* scal);
int gwg_cg_mg32(Context& c, const float* A, const float* dinv, const double* b, float* x, double rtol, int maxit,
                float* work, double* scal);
int gwg_cg32_mf(Context& c, const float* Wc, const float* dinv, const double* b, float* x, double rtol, int maxit,
                float* work, double* scal);
void gwg_mf_weights(Context& c, const double* W, float* Wc);
int64_t mf_weights_size(const MeshDesc& m);
void op_wg32(Context& c, const float* p, const float* W, float* s);
void op_gt32(Context& c, const float* s, float* q);
void to_float(Context& c, const double* a, float* b, int64_t n);
void to_double(Context& c, const float* a, double* b, int64_t n);

// ------------------------------------------------------------------------------------------
// Vector kernels
// ------------------------------------------------------------------------------------------
constexpr int kRedBlocks = 608;   // 4 x 152 SMs
constexpr int kRedThreads = 256;

template <typename T>
__global__ void k_set(int64_t n, T v, T* __restrict__ x) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}

template <typename T>
__global__ void k_axpy(int64_t n, T a, const T* __restrict__ x, T* __restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = fma(a, x[i], y[i]);
}

template <typename T>
__global__ void k_scale(int64_t n, T a, const T* __restrict__ x, T* __restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i];
}

// y = x - y (used for r = b - Ax with Ax in y)
template <typename T>
__global__ void k_sub_from(int64_t n, const T* __restrict__ x, T* __restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] - y[i];
}

__global__ void k_pointwise_mul(int64_t n, const double* __restrict__ x, const double* __restrict__ d, double* __restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] * d[i];
}

__global__ void k_pointwise_mul32(int64_t n, const float* __restrict__ x, const float* __restrict__ d, float* __restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] * d[i];
}

__global__ void k_pointwise_div(int64_t n, const double* __restrict__ x, const double* __restrict__ d, double* __restrict__ y) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] / d[i];
}

template <typename S, typename D>
__global__ void k_cast(int64_t n, const S* __restrict__ a, D* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (D)a[i];
}

// y += (D) x
template <typename S, typename D>
__global__ void k_cast_add(int64_t n, const S* __restrict__ a, D* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] += (D)a[i];
}

// partial[j*G + block] = sum_i V[j*ldv + i] * w[i] for j < m.  Each thread's few products and
// the warp tree are in the vectors' precision T (FP64 arithmetic is 58x slower than FP32 on this
// part, so FP32 Krylov vectors are not widened element by element); warp partials onward in FP64.
template <typename T, int CH>
__global__ void __launch_bounds__(kRedThreads) k_multidot(int64_t n, const T* __restrict__ V, int64_t ldv, int m,
                                                          const T* __restrict__ w, double* __restrict__ partial) {
    __shared__ double sred[kRedThreads / 32][CH];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j0 = 0; j0 < m; j0 += CH) {
        T acc[CH];
#pragma unroll
        for (int q = 0; q < CH; ++q) acc[q] = (T)0;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            T wi = w[i];
#pragma unroll
            for (int q = 0; q < CH; ++q)
                if (j0 + q < m) acc[q] = fma(V[(int64_t)(j0 + q) * ldv + i], wi, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < CH; ++q) {
            T v = acc[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) sred[warp][q] = (double)v;
        }
        __syncthreads();
        if (threadIdx.x < CH && j0 + (int)threadIdx.x < m) {
            double s = 0.0;
            for (int wv = 0; wv < kRedThreads / 32; ++wv) s += sred[wv][threadIdx.x];
            partial[(int64_t)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
        }
        __syncthreads();
    }
}

__global__ void k_reduce_partials(int m, int nb, const double* __restrict__ partial, double* __restrict__ out) {
    int j = blockIdx.x;
    if (j >= m) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[(int64_t)j * nb + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double sw[32];
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sw[k];
        out[j] = t;
    }
}

// w += sign * sum_j h[j] V_j  (h on the device).  The coefficients are converted to T once per
// block in shared memory; the per-element arithmetic is in T.  (Block size >= 64.)
template <typename T>
__global__ void k_multi_axpy(int64_t n, const T* __restrict__ V, int64_t ldv, int m, const double* __restrict__ h,
                             T* __restrict__ w, double sign) {
    __shared__ T sh[64];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T acc = i < n ? w[i] : (T)0;
    for (int j0 = 0; j0 < m; j0 += 64) {
        __syncthreads();
        if (threadIdx.x < 64 && j0 + (int)threadIdx.x < m) sh[threadIdx.x] = (T)(sign * h[j0 + threadIdx.x]);
        __syncthreads();
        int jn = m - j0 < 64 ? m - j0 : 64;
        if (i < n)
            for (int j = 0; j < jn; ++j) acc = fma(sh[j], V[(int64_t)(j0 + j) * ldv + i], acc);
    }
    if (i < n) w[i] = acc;
}

// x += sum_j y[j] Z_j  (y on the device), coefficients staged as in k_multi_axpy
template <typename T>
__global__ void k_combine(int64_t n, const T* __restrict__ Z, int64_t ldz, int m, const double* __restrict__ y,
                          T* __restrict__ x) {
    __shared__ T sy[64];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T acc = i < n ? x[i] : (T)0;
    for (int j0 = 0; j0 < m; j0 += 64) {
        __syncthreads();
        if (threadIdx.x < 64 && j0 + (int)threadIdx.x < m) sy[threadIdx.x] = (T)y[j0 + threadIdx.x];
        __syncthreads();
        int jn = m - j0 < 64 ? m - j0 : 64;
        if (i < n)
            for (int j = 0; j < jn; ++j) acc = fma(sy[j], Z[(int64_t)(j0 + j) * ldz + i], acc);
    }
    if (i < n) x[i] = acc;
}

// deterministic oscillatory start vector for the power iteration (hash of the index)
__global__ void k_pattern(int64_t n, double* __restrict__ x) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = (double)(((uint64_t)i * 2654435761ull >> 7) & 1023ull) / 1023.0 - 0.5;
}

// element-parity indicators of the P0 pressure grid: t = 1 where i+j+k is even, v = 1 where odd
// (KSPBuildPressure_CB_Nullspace_BSSCR, ksp_pressure_nullspace.c:23-75)
__global__ void k_parity_fill(int64_t ex, int64_t ey, int64_t ne, double* __restrict__ t, double* __restrict__ v) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int64_t par = (e % ex + (e / ex) % ey + e / (ex * ey)) & 1;
    t[e] = par ? 0.0 : 1.0;
    v[e] = par ? 1.0 : 0.0;
}

__global__ void k_remove_mean(int64_t n, const double* __restrict__ sum, double* __restrict__ x) {
    __shared__ double mean;
    if (threadIdx.x == 0) mean = sum[0] / (double)n;   // one division per block
    __syncthreads();
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] -= mean;
}

// ------------------------------------------------------------------------------------------
// Solver state
// ------------------------------------------------------------------------------------------
struct Reducer {
    Context& c;
    DArray<double> partial, out;
    explicit Reducer(Context& ctx) : c(ctx) {
        partial.ensure((size_t)kRedBlocks * 64);
        out.ensure(64);
    }
    // out[0..m) = V_j . w on the device; optionally copied to host
    template <typename T>
    void multidot(int64_t n, const T* V, int64_t ldv, int m, const T* w, double* host) {
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            if (m <= 1)
                k_multidot<T, 1><<<kRedBlocks, kRedThreads, 0, c.stream>>>(n, V, ldv, m, w, partial.p);
            else
                k_multidot<T, 8><<<kRedBlocks, kRedThreads, 0, c.stream>>>(n, V, ldv, m, w, partial.p);
        }
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_reduce_partials<<<m, 256, 0, c.stream>>>(m, kRedBlocks, partial.p, out.p);
        }
        if (host) {
            UWG_CUDA(cudaMemcpyAsync(c.host_scalars, out.p, m * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            UWG_CUDA(cudaStreamSynchronize(c.stream));
            std::memcpy(host, c.host_scalars, m * sizeof(double));
        }
    }
    template <typename T>
    double dot(int64_t n, const T* a, const T* b) {
        double r;
        multidot<T>(n, a, 0, 1, b, &r);
        return r;
    }
    template <typename T>
    double norm(int64_t n, const T* a) {
        double d = dot<T>(n, a, a);
        return std::sqrt(d > 0 ? d : 0.0);
    }
};

template <typename T>
static void axpy(Context& c, int64_t n, double a, const T* x, T* y) {
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    k_axpy<T><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, (T)a, x, y);
}
template <typename T>
static void scale(Context& c, int64_t n, double a, const T* x, T* y) {
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    k_scale<T><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, (T)a, x, y);
}
template <typename T>
static void zero(Context& c, int64_t n, T* x) {
    UWG_CUDA(cudaMemsetAsync(x, 0, (size_t)n * sizeof(T), c.stream));
}
template <typename T>
static void copy(Context& c, int64_t n, const T* x, T* y) {
    UWG_CUDA(cudaMemcpyAsync(y, x, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, c.stream));
}
template <typename S, typename D>
static void cast(Context& c, int64_t n, const S* a, D* b) {
    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
    k_cast<S, D><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, a, b);
}

// Flexible GMRES(m), right preconditioning, zero initial guess; stops when ||r|| <= rtol ||b||
// or the iteration budget is spent.  Orthogonalisation: classical Gram-Schmidt with one
// re-orthogonalisation pass (batched dot products, one launch per pass).
template <typename T>
struct Fgmres {
    Context& c;
    Reducer& red;
    int64_t n = 0;
    int m = 30;
    DArray<T> V, Z, w;
    DArray<double> dvec;
    std::vector<double> H, cs, sn, g, y, hcol;
    Fgmres(Context& ctx, Reducer& r) : c(ctx), red(r) {}
    void setup(int64_t nn, int restart) {
        n = nn;
        m = restart < 1 ? 1 : (restart > 60 ? 60 : restart);
        V.ensure((size_t)(m + 1) * n);
        Z.ensure((size_t)m * n);
        w.ensure((size_t)n);
        dvec.ensure(64);
        H.assign((size_t)(m + 1) * m, 0.0);
        cs.assign(m, 0.0);
        sn.assign(m, 0.0);
        g.assign(m + 1, 0.0);
        y.assign(m, 0.0);
        hcol.assign(m + 1, 0.0);
    }
    // residual estimate after each iteration of the current solve, and the position of the
    // current iteration in its restart cycle (read by adaptive preconditioners)
    std::vector<double> hist;
    int cycle_k = 0;

    // A(x, y): y = A x ; M(v, z): z = M^{-1} v.  Returns iterations; *res = final ||r||.
    template <typename Aop, typename Mop>
    int solve(Aop&& A, Mop&& M, const T* b, T* x, double rtol, int maxit, double* res_out, double* bnorm_out,
              bool* nan_out) {
        hist.clear();
        zero<T>(c, n, x);
        double bnorm = red.norm<T>(n, b);
        if (bnorm_out) *bnorm_out = bnorm;
        if (nan_out) *nan_out = !std::isfinite(bnorm);
        if (!(bnorm > 0.0) || !std::isfinite(bnorm)) {
            if (res_out) *res_out = 0.0;
            return 0;
        }
        int its = 0;
        double beta = bnorm;
        // first cycle starts from x = 0, r = b
        copy<T>(c, n, b, V.p);
        bool first = true;
        while (true) {
            if (!first) {
                A(x, w.p);
                {
                    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
                    k_sub_from<T><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, b, w.p);
                }
                copy<T>(c, n, w.p, V.p);
                beta = red.norm<T>(n, V.p);
            }
            first = false;
            if (!std::isfinite(beta)) {
                if (nan_out) *nan_out = true;
                break;
            }
            if (beta <= rtol * bnorm || its >= maxit) break;
            scale<T>(c, n, 1.0 / beta, V.p, V.p);
            std::fill(g.begin(), g.end(), 0.0);
            g[0] = beta;
            int k = 0;
            bool done = false;
            for (; k < m && its < maxit; ++k) {
                T* vk = V.p + (int64_t)k * n;
                T* zk = Z.p + (int64_t)k * n;
                cycle_k = k;
                M(vk, zk);
                A(zk, w.p);
                // CGS2
                for (int pass = 0; pass < 2; ++pass) {
                    red.multidot<T>(n, V.p, n, k + 1, w.p, hcol.data() + 0);
                    UWG_CUDA(cudaMemcpyAsync(dvec.p, hcol.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, c.stream));
                    {
                        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
                        k_multi_axpy<T><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, V.p, n, k + 1, dvec.p, w.p, -1.0);
                    }
                    for (int j = 0; j <= k; ++j) {
                        if (pass == 0) H[(size_t)j * m + k] = hcol[j];
                        else H[(size_t)j * m + k] += hcol[j];
                    }
                }
                double hn = red.norm<T>(n, w.p);
                H[(size_t)(k + 1) * m + k] = hn;
                if (hn > 0.0) scale<T>(c, n, 1.0 / hn, w.p, V.p + (int64_t)(k + 1) * n);
                for (int j = 0; j < k; ++j) {
                    double t = cs[j] * H[(size_t)j * m + k] + sn[j] * H[(size_t)(j + 1) * m + k];
                    H[(size_t)(j + 1) * m + k] = -sn[j] * H[(size_t)j * m + k] + cs[j] * H[(size_t)(j + 1) * m + k];
                    H[(size_t)j * m + k] = t;
                }
                double a = H[(size_t)k * m + k], bb = H[(size_t)(k + 1) * m + k];
                double rr = std::sqrt(a * a + bb * bb);
                if (!(rr > 0.0)) {
                    done = true;
                    k++;
                    its++;
                    break;
                }
                cs[k] = a / rr;
                sn[k] = bb / rr;
                H[(size_t)k * m + k] = rr;
                H[(size_t)(k + 1) * m + k] = 0.0;
                g[k + 1] = -sn[k] * g[k];
                g[k] = cs[k] * g[k];
                its++;
                hist.push_back(std::fabs(g[k + 1]));
                if (!std::isfinite(g[k + 1])) {
                    if (nan_out) *nan_out = true;
                    done = true;
                    k++;
                    break;
                }
                if (std::fabs(g[k + 1]) <= rtol * bnorm || hn == 0.0) {
                    done = true;
                    k++;
                    break;
                }
            }
            // y = H^{-1} g, x += Z y
            for (int i = k - 1; i >= 0; --i) {
                double s = g[i];
                for (int j = i + 1; j < k; ++j) s -= H[(size_t)i * m + j] * y[j];
                y[i] = s / H[(size_t)i * m + i];
            }
            UWG_CUDA(cudaMemcpyAsync(dvec.p, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, c.stream));
            {
                LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
                k_combine<T><<<blocks_for(n, 256), 256, 0, c.stream>>>(n, Z.p, n, k, dvec.p, x);
            }
            beta = std::fabs(g[k]);
            if (done || its >= maxit) break;
        }
        if (res_out) *res_out = beta;
        return its;
    }
};

struct Bsscr {
    Context& c;
    const uwgpu_solve_opts& o;
    uwgpu_report& rep;
    Reducer red;
    Fgmres<double> gm64;
    Fgmres<float> gm32;
    Fgmres<double> gms;   // Schur (pressure)
    int dim = 0, nlev = 0;
    int64_t nv = 0, npres = 0;
    bool mixed = false;
    DArray<double> f, h, hhat, tu, tu2, t2, Sd, rhs_p, ref_r, ref_d;
    // scaled BFBt state: weights, G^T W G stencil and inverse diagonal, work vectors
    DArray<double> bw, bA, bd, bt, bt2, bs, bX, pr, pz, pp, pq, ptmp;
    // FP32 copies for the mixed form (the preconditioner runs in FP32 inside the FP64 Schur FGMRES)
    DArray<float> bw32, bA32, bd32, bt32, bt2_32, bs32, bX32, pz32, bwc32;
    DArray<double> scal32;
    int64_t bfbt_its = 0;
    // pressure null-space vectors (constant, or the two element-parity indicators), each used
    // only when G maps it to (nearly) zero; and whether G^T W G has the constant null space
    DArray<double> ns_t, ns_v;
    bool ns_use_t = false, ns_use_v = false;
    bool bbt_const = false;
    bool bfbt_mg = false;      // the inner solves use the multigrid preconditioner
    bool stencil32 = false;    // the mixed form's Jacobi inner solves read the FP32 stencil
    DArray<float> r32, d32;
    bool nan = false;
    bool inner_fail = false;

    Bsscr(Context& ctx, const uwgpu_solve_opts& opts, uwgpu_report& r)
        : c(ctx), o(opts), rep(r), red(ctx), gm64(ctx, red), gm32(ctx, red), gms(ctx, red) {}
    ~Bsscr() { c.cc.on = false; }   // the coarse correction belongs to this solve's operator

    // velocity hierarchy: operator, levels, Chebyshev bounds
    void setup_velocity() {
        dim = c.mesh.dim;
        int levels = o.mg_levels < 1 ? 1 : o.mg_levels;
        mixed = o.precision == UWGPU_PREC_MIXED;
        if (!c.operator_built || c.operator_levels != levels || (mixed && !c.operator_has32))
            build_operator(c, levels, mixed);
        nlev = c.nlevels;
        nv = c.mesh.nn * dim;
        if (o.smoother == UWGPU_SMOOTHER_CHEBYSHEV) estimate_lmax();
    }

    // ---- learned correction of the V-cycle (unet.cu): M(r) = S(V(r) + N(r, V(r))) ----
    // The network is trained on residuals of the multigrid iteration, so it is applied where
    // FGMRES hands the preconditioner a true (scaled) residual: the first iteration of each
    // restart cycle; the other Krylov directions get the plain V-cycle.  It stays active while
    // the velocity FGMRES makes progress; after `learned_stagnation` consecutive iterations that
    // reduce the residual estimate by less than 5%, the rest of that velocity solve uses the
    // plain V-cycle (the multigrid fallback).
    bool learned = false;      // requested and a network exists
    bool learned_on = false;   // within the current velocity solve
    template <typename T>
    void learned_check(const std::vector<double>& hist) {
        if (!learned_on) return;
        const int need = o.learned_stagnation > 0 ? o.learned_stagnation : 2;
        if ((int)hist.size() < need + 1) return;
        for (int q = 0; q < need; ++q) {
            const size_t i = hist.size() - 1 - q;
            if (!(hist[i] > 0.95 * hist[i - 1])) return;
        }
        learned_on = false;
        rep.learned_fallbacks++;
    }
    template <typename T>
    void precondition(const T* in, T* out, const std::vector<double>& hist, int cycle_k) {
        vcycle<T>(0, in, out);
        rep.vcycles++;
        learned_check<T>(hist);
        if (learned_on && cycle_k == 0) {
            unet::correct<T>(c, *c.net, in, out);
            // post-smoothing on the new residual, as after a coarse-grid correction: the rough
            // part of the network's error (its BF16 activations included) would otherwise be
            // amplified by K; the fine level's b and x buffers are free once the V-cycle is done
            Level& L0 = c.levels[0];
            level_residual<T>(c, L0, out, in, lvl_b<T>(L0));
            smooth<T>(L0, lvl_b<T>(L0), lvl_x<T>(L0), o.smooth_up > 0 ? o.smooth_up : 1, true);
            axpy<T>(c, nv, 1.0, lvl_x<T>(L0), out);
            rep.learned_applies++;
        }
    }

    // ---- multigrid V-cycle (zero initial guess), precision T ----
    template <typename T>
    T* lvl_x(Level& L);
    template <typename T>
    T* lvl_b(Level& L);
    template <typename T>
    T* lvl_r(Level& L);

    template <typename T>
    void smooth(Level& L, const T* b, T* x, int sweeps, bool zero_init) {
        if (o.smoother == UWGPU_SMOOTHER_CHEBYSHEV)
            level_cheb<T>(c, L, b, x, sweeps, zero_init);
        else
            level_smooth<T>(c, L, b, x, sweeps, zero_init);
    }

    // largest eigenvalue of Dinv A per smoothed level by power iteration (Chebyshev bounds)
    void estimate_lmax() {
        for (int l = 0; l < (nlev > 1 ? nlev - 1 : 1); ++l) {
            Level& L = c.levels[l];
            if (L.lmax > 0.0) continue;
            int64_t n = L.mesh.nn * dim;
            {
                LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
                k_pattern<<<blocks_for(n, 256), 256, 0, c.stream>>>(n, L.x64.p);
            }
            double nx = red.norm<double>(n, L.x64.p), lam = 1.0;
            scale<double>(c, n, 1.0 / nx, L.x64.p, L.x64.p);
            for (int it = 0; it < 15; ++it) {
                level_apply<double>(c, L, L.x64.p, L.t64.p);
                level_dinv<double>(c, L, L.t64.p, L.b64.p);
                lam = red.norm<double>(n, L.b64.p);
                if (!(lam > 0.0) || !std::isfinite(lam)) { lam = 1.0; break; }
                scale<double>(c, n, 1.0 / lam, L.b64.p, L.x64.p);
            }
            L.lmax = lam;
        }
    }

    template <typename T>
    void vcycle(int l, const T* b, T* x) {
        Level& L = c.levels[l];
        if (l == nlev - 1) {
            if (nlev > 1)
                level_coarse_solve<T>(c, L, b, x);
            else
                smooth<T>(L, b, x, o.smooth_down + o.smooth_up, true);
            return;
        }
        smooth<T>(L, b, x, o.smooth_down, true);
        T* r = lvl_r<T>(L);
        level_residual<T>(c, L, x, b, r);
        Level& C = c.levels[l + 1];
        T* bc = lvl_b<T>(C);
        T* xc = lvl_x<T>(C);
        level_restrict<T>(c, L, C, r, bc);
        vcycle<T>(l + 1, bc, xc);
        level_prolong_add<T>(c, L, C, xc, x);
        // W-cycle: a second coarse correction on the residual left by the first
        // (PCMG's -pc_mg_cycle_type w); the coarsest solve is exact, so it is not repeated there
        if (o.mg_cycle == 2 && l + 1 < nlev - 1) {
            level_residual<T>(c, L, x, b, r);
            level_restrict<T>(c, L, C, r, bc);
            vcycle<T>(l + 1, bc, xc);
            level_prolong_add<T>(c, L, C, xc, x);
        }
        smooth<T>(L, b, x, o.smooth_up, false);
    }

    // ---- velocity (A11) solve: x = K^{-1} b to relative tolerance rtol ----
    int a11(const double* b, double* x, double rtol) {
        int its = 0;
        Level& L0 = c.levels[0];
        int maxit = o.max_inner > 0 ? o.max_inner : 500;
        if (!mixed) {
            double res = 0.0, bn = 0.0;
            bool nn = false;
            learned_on = learned;
            its = gm64.solve([&](const double* in, double* out) { level_apply<double>(c, L0, in, out); },
                             [&](const double* in, double* out) { precondition<double>(in, out, gm64.hist, gm64.cycle_k); },
                             b, x, rtol, maxit, &res, &bn, &nn);
            if (nn) nan = true;
            if (!(res <= rtol * bn * 1.0000001) && bn > 0) inner_fail = true;
        } else {
            // FP64 iterative refinement around an FP32 FGMRES + FP32 V-cycle
            zero<double>(c, nv, x);
            double bn = red.norm<double>(nv, b);
            if (!(bn > 0.0)) return 0;
            if (!std::isfinite(bn)) { nan = true; return 0; }
            copy<double>(c, nv, b, ref_r.p);
            double rn = bn;
            int guard = 0;
            learned_on = learned;
            while (rn > rtol * bn && its < maxit && guard < 50) {
                guard++;
                cast<double, float>(c, nv, ref_r.p, r32.p);
                double res = 0.0, b32n = 0.0;
                bool nn = false;
                double inner_rtol = std::max(rtol * bn / rn, 1e-4);
                int k = gm32.solve([&](const float* in, float* out) { level_apply<float>(c, L0, in, out); },
                                   [&](const float* in, float* out) { precondition<float>(in, out, gm32.hist, gm32.cycle_k); },
                                   r32.p, d32.p, std::min(inner_rtol, 0.5), maxit - its, &res, &b32n, &nn);
                its += k;
                if (nn) { nan = true; break; }
                {
                    LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
                    k_cast_add<float, double><<<blocks_for(nv, 256), 256, 0, c.stream>>>(nv, d32.p, x);
                }
                level_residual<double>(c, L0, x, b, ref_r.p);
                rn = red.norm<double>(nv, ref_r.p);
                if (!std::isfinite(rn)) { nan = true; break; }
                if (k == 0) break;
            }
            if (rn > rtol * bn * 1.0000001) inner_fail = true;
        }
        rep.inner_its_total += its;
        return its;
    }

    // S v = G^T K^{-1} G v  (the positive form of PETSc's MatSchurComplement)
    void schur_apply(const double* v, double* y) {
        op_G(c, v, tu.p);
        a11(tu.p, tu2.p, o.a11_rtol);
        op_GT(c, tu2.p, y);
    }

    void pmul(int64_t n, const double* a, const double* b, double* y) {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_pointwise_mul<<<blocks_for(n, 256), 256, 0, c.stream>>>(n, a, b, y);
    }

    // Jacobi-preconditioned CG on G^T W G (the inner KSP of the scaled BFBt preconditioner), with
    // the right-hand side projected off the constant null space when G^T W G has it
    // (pc_ScaledGtKG.c:266-268, 829-831)
    void gwg_solve(const double* b, double* x) {
        int maxit = o.bfbt_max_it > 0 ? o.bfbt_max_it : 500;
        double rtol = o.bfbt_rtol > 0 ? o.bfbt_rtol : 1e-4;
        copy<double>(c, npres, b, pr.p);
        if (bbt_const) remove_constant_dev(pr.p);
        bfbt_its += bfbt_mg ? gwg_cg_mg(c, bA.p, bd.p, pr.p, x, rtol, maxit, pz.p, pz.p + 4 * npres)
                            : gwg_cg(c, bA.p, bd.p, pr.p, x, rtol, maxit, pz.p, pz.p + 4 * npres);
    }

    // FP32 inner solve of G^T W G into bt32: multigrid-preconditioned on the FP32 stencil, or
    // Jacobi on the FP32 stencil or with the matrix-free apply
    int inner32(const double* b) {
        int maxit = o.bfbt_max_it > 0 ? o.bfbt_max_it : 500;
        double rtol = o.bfbt_rtol > 0 ? o.bfbt_rtol : 1e-4;
        if (bfbt_mg) return gwg_cg_mg32(c, bA32.p, bd32.p, b, bt32.p, rtol, maxit, pz32.p, scal32.p);
        if (stencil32) return gwg_cg32(c, bA32.p, bd32.p, b, bt32.p, rtol, maxit, pz32.p, scal32.p);
        return gwg_cg32_mf(c, bwc32.p, bd32.p, b, bt32.p, rtol, maxit, pz32.p, scal32.p);
    }

    // the same preconditioner with FP32 operators, inner solves and vectors (mixed form)
    void bfbt_apply32(const double* x, double* y) {
        copy<double>(c, npres, x, pr.p);
        if (bbt_const) remove_constant_dev(pr.p);
        bfbt_its += inner32(pr.p);
        op_wg32(c, bt32.p, bw32.p, bs32.p);
        level_apply<float>(c, c.levels[0], bs32.p, bX32.p);
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_pointwise_mul32<<<blocks_for(nv, 256), 256, 0, c.stream>>>(nv, bX32.p, bw32.p, bX32.p);
        }
        op_gt32(c, bX32.p, bt2_32.p);
        to_double(c, bt2_32.p, pr.p, npres);
        if (bbt_const) remove_constant_dev(pr.p);
        bfbt_its += inner32(pr.p);
        to_double(c, bt32.p, y, npres);
    }

    // pc_ScaledGtKG.c:242-310: y = (G^T W G)^-1 G^T W K W G (G^T W G)^-1 x
    void bfbt_apply(const double* x, double* y) {
        if (mixed) {
            bfbt_apply32(x, y);
            return;
        }
        gwg_solve(x, bt.p);
        op_G(c, bt.p, bs.p);
        pmul(nv, bs.p, bw.p, bs.p);
        level_apply<double>(c, c.levels[0], bs.p, bX.p);
        pmul(nv, bX.p, bw.p, bX.p);
        op_GT(c, bX.p, bt2.p);
        gwg_solve(bt2.p, y);
    }

    void remove_constant_dev(double* x);
    void setup_nullspace();
    void project_nullspace(double* x);

    void schur_pc(const double* v, double* z) {
        if (o.schur_pc == UWGPU_SCHUR_PC_NONE) {
            copy<double>(c, npres, v, z);
        } else if (o.schur_pc == UWGPU_SCHUR_PC_SCALED_BFBT) {
            bfbt_apply(v, z);
        } else {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_pointwise_div<<<blocks_for(npres, 256), 256, 0, c.stream>>>(npres, v, Sd.p, z);
        }
    }

    // preconditioned CG on the Schur system (KSPCG), unpreconditioned residual test
    int schur_cg(const double* b, double* x, double rtol, int maxit) {
        DArray<double> r, z, p, q;
        r.ensure(npres);
        z.ensure(npres);
        p.ensure(npres);
        q.ensure(npres);
        zero<double>(c, npres, x);
        copy<double>(c, npres, b, r.p);
        double r0 = red.norm<double>(npres, r.p);
        if (!(r0 > 0)) return 0;
        schur_pc(r.p, z.p);
        double rz = red.dot<double>(npres, r.p, z.p);
        copy<double>(c, npres, z.p, p.p);
        int it = 0;
        double rn = r0;
        while (it < maxit && rn > rtol * r0) {
            schur_apply(p.p, q.p);
            double pq = red.dot<double>(npres, p.p, q.p);
            double alpha = rz / pq;
            axpy<double>(c, npres, alpha, p.p, x);
            axpy<double>(c, npres, -alpha, q.p, r.p);
            schur_pc(r.p, z.p);
            double rz2 = red.dot<double>(npres, r.p, z.p);
            double beta = rz2 / rz;
            rz = rz2;
            {
                // p = z + beta p
                scale<double>(c, npres, beta, p.p, p.p);
                axpy<double>(c, npres, 1.0, z.p, p.p);
            }
            rn = red.norm<double>(npres, r.p);
            it++;
            if (!std::isfinite(rn)) { nan = true; break; }
        }
        return it;
    }

    double full_residual(const double* u, const double* p) {
        // ||[f - K u - G p; h - G^T u]|| / ||[f; h]||
        Level& L0 = c.levels[0];
        level_apply<double>(c, L0, u, t2.p);
        op_G(c, p, tu.p);
        axpy<double>(c, nv, 1.0, tu.p, t2.p);
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_sub_from<double><<<blocks_for(nv, 256), 256, 0, c.stream>>>(nv, f.p, t2.p);
        }
        op_GT(c, u, rhs_p.p);
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_sub_from<double><<<blocks_for(npres, 256), 256, 0, c.stream>>>(npres, h.p, rhs_p.p);
        }
        double r2 = red.dot<double>(nv, t2.p, t2.p) + red.dot<double>(npres, rhs_p.p, rhs_p.p);
        double b2 = red.dot<double>(nv, f.p, f.p) + red.dot<double>(npres, h.p, h.p);
        return std::sqrt(r2 / (b2 > 0 ? b2 : 1.0));
    }

    void run();
};

template <>
double* Bsscr::lvl_x<double>(Level& L) { return L.x64.p; }
template <>
float* Bsscr::lvl_x<float>(Level& L) { return L.x32.p; }
template <>
double* Bsscr::lvl_b<double>(Level& L) { return L.b64.p; }
template <>
float* Bsscr::lvl_b<float>(Level& L) { return L.b32.p; }
template <>
double* Bsscr::lvl_r<double>(Level& L) { return L.r64.p; }
template <>
float* Bsscr::lvl_r<float>(Level& L) { return L.r32.p; }

__global__ void k_sum_partial(int64_t n, const double* __restrict__ x, double* __restrict__ out) {
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) s += x[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

static void remove_constant(Context& c, int64_t n, double* x, DArray<double>& tmp) {
    tmp.ensure(1);
    UWG_CUDA(cudaMemsetAsync(tmp.p, 0, sizeof(double), c.stream));
    {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_sum_partial<<<kRedBlocks, kRedThreads, 0, c.stream>>>(n, x, tmp.p);
    }
    {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_remove_mean<<<blocks_for(n, 256), 256, 0, c.stream>>>(n, tmp.p, x);
    }
}

// BC lift for non-zero Dirichlet values: f_free -= K_(free,fixed) u_b, h -= G^T u_b.
template <int DIM>
__global__ void k_bc_lift(int64_t nnx, int64_t nny, int64_t nnz, int64_t nn, int ex, int ey, int ez, int64_t ne,
                          const double* __restrict__ Ke, const uint8_t* __restrict__ fixed,
                          const double* __restrict__ val, double* __restrict__ f) {
    constexpr int NEN = 1 << DIM, ND = NEN * DIM;
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    int64_t idx[3] = {n % nnx, (n / nnx) % nny, DIM == 3 ? n / (nnx * nny) : 0};
    int64_t ecount[3] = {ex, ey, ez};
    double acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = 0.0;
    for (int o = 0; o < NEN; ++o) {
        int64_t e3[3] = {0, 0, 0};
        bool ok = true;
        for (int d = 0; d < DIM; ++d) {
            e3[d] = idx[d] - ((o >> d) & 1);
            if (e3[d] < 0 || e3[d] >= ecount[d]) ok = false;
        }
        if (!ok) continue;
        int64_t e = e3[0] + (int64_t)ex * (e3[1] + (int64_t)ey * e3[2]);
        int la = o;
        int64_t base = e3[0] + nnx * (e3[1] + nny * e3[2]);
        for (int b = 0; b < NEN; ++b) {
            int64_t m = base + (b & 1) + ((b >> 1) & 1) * nnx + (DIM == 3 ? ((b >> 2) & 1) * nnx * nny : 0);
            for (int cc = 0; cc < DIM; ++cc) {
                if (!fixed[m * DIM + cc]) continue;
                double v = val[m * DIM + cc];
                if (v == 0.0) continue;
                for (int r = 0; r < DIM; ++r) {
                    int R = la * DIM + r, C = b * DIM + cc;
                    int pi = R <= C ? packed_index(ND, R, C) : packed_index(ND, C, R);
                    acc[r] -= Ke[(int64_t)pi * ne + e] * v;
                }
            }
        }
    }
    for (int d = 0; d < DIM; ++d)
        if (!fixed[n * DIM + d]) f[(int64_t)d * nn + n] += acc[d];
}

// node-major BC values -> SoA vector with only the fixed comps set
template <int DIM>
__global__ void k_bc_vector(int64_t nn, const uint8_t* __restrict__ fixed, const double* __restrict__ val,
                            double* __restrict__ u) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    for (int d = 0; d < DIM; ++d) u[(int64_t)d * nn + n] = fixed[n * DIM + d] ? val[n * DIM + d] : 0.0;
}

void Bsscr::remove_constant_dev(double* x) { remove_constant(c, npres, x, ptmp); }

// KSPBuildPressure_Const_Nullspace_BSSCR / _CB_Nullspace_BSSCR (ksp_pressure_nullspace.c:23-115):
// remove_const_p = 1 builds the constant vector, 2 the even and odd element-parity indicators.
// KSPRemovePressureNullspace_BSSCR (ksp_pressure_nullspace.c:121-176) projects a vector w out
// only when ||G w|| / ||w|| < nstol ||G||_inf, nstol = 1e-7 (BSSCR.c:391).
void Bsscr::setup_nullspace() {
    int mode = o.remove_const_p;
    ns_use_t = ns_use_v = false;
    if (mode != 1 && mode != 2) return;
    const MeshDesc& m = c.mesh;
    ns_t.ensure(npres);
    if (mode == 1) {
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_set<double><<<blocks_for(npres, 256), 256, 0, c.stream>>>(npres, 1.0, ns_t.p);
    } else {
        ns_v.ensure(npres);
        LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
        k_parity_fill<<<blocks_for(npres, 256), 256, 0, c.stream>>>(m.nel[0], m.nel[1], npres, ns_t.p, ns_v.p);
    }
    const double ginf = g_inf_norm(c);
    auto in_nullspace = [&](const double* w) {
        op_G(c, w, tu.p);
        double gn = red.norm<double>(nv, tu.p), wn = red.norm<double>(npres, w);
        return wn > 0.0 && gn / wn < 1e-7 * ginf;
    };
    ns_use_t = in_nullspace(ns_t.p);
    if (mode == 2) ns_use_v = in_nullspace(ns_v.p);
}

void Bsscr::project_nullspace(double* x) {
    for (int k = 0; k < 2; ++k) {
        bool use = k == 0 ? ns_use_t : ns_use_v;
        const double* w = k == 0 ? ns_t.p : ns_v.p;
        if (!use) continue;
        double a1 = red.dot<double>(npres, w, x), a2 = red.dot<double>(npres, w, w);
        axpy<double>(c, npres, -a1 / a2, w, x);
    }
}

void Bsscr::run() {
    auto t0 = std::chrono::steady_clock::now();
    FamilyOverride setup_family(c, UWGPU_KERNEL_SETUP);
    setup_velocity();
    if (o.learned_pc) {
        UWG_REQUIRE(c.net != nullptr, UWGPU_ERR_STATE, "learned_pc requested but no network (uwgpu_learned_create)");
        UWG_REQUIRE(c.net->nn == c.mesh.nn, UWGPU_ERR_STATE, "the network was built for another mesh");
        unet::prepare_viscosity(c, *c.net);
        learned = true;
    }
    npres = c.mesh.ne;
    int restart = o.restart > 0 ? o.restart : 30;
    gm64.setup(nv, restart);
    if (mixed) gm32.setup(nv, restart);
    gms.setup(npres, restart);
    f.ensure(nv);
    h.ensure(npres);
    hhat.ensure(npres);
    tu.ensure(nv);
    tu2.ensure(nv);
    t2.ensure(nv);
    Sd.ensure(npres);
    rhs_p.ensure(npres);
    ref_r.ensure(nv);
    ref_d.ensure(nv);
    if (mixed) {
        r32.ensure(nv);
        d32.ensure(nv);
    }
    c.u_sol.ensure(nv);
    c.p_sol.ensure(npres);
    // right-hand sides
    gather_force(c, f.p);
    zero<double>(c, npres, h.p);
    DArray<double> ub;
    if (c.has_bc && c.bc_nonzero) {
        // BC lift (StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:900-925): f -= K_(free,fixed) u_b,
        // and for the transposed gradient block h -= G^T u_b
        const MeshDesc& m = c.mesh;
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            if (dim == 3)
                k_bc_lift<3><<<blocks_for(m.nn, 128), 128, 0, c.stream>>>(m.nnx, m.nny, m.nnz, m.nn, m.nel[0], m.nel[1],
                                                                          m.nel[2], m.ne, c.levels[0].Ke.p, c.fixed.p,
                                                                          c.bcval.p, f.p);
            else
                k_bc_lift<2><<<blocks_for(m.nn, 128), 128, 0, c.stream>>>(m.nnx, m.nny, m.nnz, m.nn, m.nel[0], m.nel[1], 1,
                                                                          m.ne, c.levels[0].Ke.p, c.fixed.p, c.bcval.p, f.p);
        }
        check_launch("k_bc_lift");
        ub.ensure(nv);
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            if (dim == 3)
                k_bc_vector<3><<<blocks_for(m.nn, 256), 256, 0, c.stream>>>(m.nn, c.fixed.p, c.bcval.p, ub.p);
            else
                k_bc_vector<2><<<blocks_for(m.nn, 256), 256, 0, c.stream>>>(m.nn, c.fixed.p, c.bcval.p, ub.p);
        }
        op_GT_unmasked(c, ub.p, h.p);
        scale<double>(c, npres, -1.0, h.p, h.p);
    }
    // Schur preconditioner
    if (o.schur_pc == UWGPU_SCHUR_PC_UW) copy<double>(c, npres, c.Se.p, Sd.p);
    else if (o.schur_pc == UWGPU_SCHUR_PC_GKGDIAG) gkgdiag(c, Sd.p);
    else if (o.schur_pc == UWGPU_SCHUR_PC_SCALED_BFBT) {
        for (auto* v : {&bw, &bs, &bX}) v->ensure(nv);
        for (auto* v : {&bd, &bt, &bt2, &pr}) v->ensure(npres);
        pz.ensure(4 * npres + 8);
        bfbt_weights(c, bw.p);
        bA.ensure((size_t)(dim == 3 ? 27 : 9) * npres);
        gwg_stencil_build(c, bw.p, bA.p, bd.p);
        // BSSCR_MatContainsConstNullSpace (Stokes_Nullspace.c:15-46) on G^T W G:
        // ||A (1/N)||_2 < 1e-7 attaches the constant null space to the inner solves
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_set<double><<<blocks_for(npres, 256), 256, 0, c.stream>>>(npres, 1.0 / (double)npres, bt.p);
        }
        gwg_stencil_apply(c, bA.p, bt.p, bt2.p, pz.p + 4 * npres);
        bbt_const = red.norm<double>(npres, bt2.p) < 1e-7;
        if (mixed) {
            for (auto* v : {&bw32, &bs32, &bX32}) v->ensure(nv);
            for (auto* v : {&bd32, &bt32, &bt2_32}) v->ensure(npres);
            pz32.ensure(4 * npres);
            scal32.ensure(8);
            to_float(c, bw.p, bw32.p, nv);
            bwc32.ensure((size_t)mf_weights_size(c.mesh));
            gwg_mf_weights(c, bw.p, bwc32.p);   // the matrix-free inner operator's folded weights
            // Jacobi inner solves: the FP32 stencil while it and the CG vectors take at most half
            // of L2 (streamed from L2 it is the faster form), else the matrix-free apply, which
            // moves about a fifth of the bytes; bfbt_inner_pc 2 / 3 force one form.  The
            // multigrid levels start from the FP32 stencil.
            int l2 = 0;
            UWG_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c.device));
            const double st_bytes = (double)npres * 4.0 * ((dim == 3 ? 27 : 9) + 6);
            stencil32 = o.bfbt_inner_pc == 2 ||
                        ((o.bfbt_inner_pc == 0 || o.bfbt_inner_pc == 4) && st_bytes <= 0.5 * l2);
            const bool want_stencil32 = stencil32 || o.bfbt_inner_pc == 1;
            if (want_stencil32) bA32.ensure((size_t)(dim == 3 ? 27 : 9) * npres);
            gwg_stencil_fp32(c, bA.p, bd.p, want_stencil32 ? bA32.p : nullptr, bd32.p);
        }
        if (o.bfbt_inner_pc == 1) bfbt_mg = gwg_mg_build(c, bA.p, bd.p, mixed, bbt_const);
        // option 4: Jacobi plus the plane-checkerboard coarse correction (3D; plain Jacobi in 2D)
        c.cc.on = false;
        if (o.bfbt_inner_pc == 4) gwg_cc_build(c, bA.p);
    }
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    auto t1 = std::chrono::steady_clock::now();
    rep.t_setup_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    c.family_override = setup_family.saved;

    // h_hat = h - G^T K^{-1} f
    a11(f.p, tu2.p, o.a11_rtol);
    op_GT(c, tu2.p, hhat.p);
    scale<double>(c, npres, -1.0, hhat.p, hhat.p);
    axpy<double>(c, npres, 1.0, h.p, hhat.p);
    // solve (G^T K^{-1} G) p = -h_hat
    scale<double>(c, npres, -1.0, hhat.p, rhs_p.p);
    setup_nullspace();
    project_nullspace(rhs_p.p);
    int maxo = o.max_outer > 0 ? o.max_outer : 500;
    int outer = 0;
    bool outer_fail = false;
    if (o.schur_type == UWGPU_SCHUR_CG) {
        outer = schur_cg(rhs_p.p, c.p_sol.p, o.scr_rtol, maxo);
    } else {
        double res = 0, bn = 0;
        bool nn = false;
        outer = gms.solve([&](const double* in, double* out) { schur_apply(in, out); },
                          [&](const double* in, double* out) { schur_pc(in, out); }, rhs_p.p, c.p_sol.p, o.scr_rtol,
                          maxo, &res, &bn, &nn);
        if (nn) nan = true;
        if (bn > 0 && res > o.scr_rtol * bn * 1.0000001) outer_fail = true;
    }
    project_nullspace(c.p_sol.p);
    // back-solve u = K^{-1} (f - G p)
    op_G(c, c.p_sol.p, t2.p);
    scale<double>(c, nv, -1.0, t2.p, t2.p);
    axpy<double>(c, nv, 1.0, f.p, t2.p);
    int before = rep.inner_its_total;
    a11(t2.p, c.u_sol.p, o.back_rtol);
    rep.backsolve_its = rep.inner_its_total - before;
    rep.outer_its = outer;
    rep.pc_inner_its = bfbt_its;
    // the residual of the lifted system, on the free dofs (before the fixed values are added)
    rep.rel_residual = full_residual(c.u_sol.p, c.p_sol.p);
    if (c.has_bc && c.bc_nonzero) axpy<double>(c, nv, 1.0, ub.p, c.u_sol.p);
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    if (learned) unet::check_errors(c, *c.net);
    auto t2c = std::chrono::steady_clock::now();
    rep.t_solve_ms = std::chrono::duration<double, std::milli>(t2c - t1).count();
    c.has_solution = true;
    if (nan || !std::isfinite(rep.rel_residual)) rep.status = UWGPU_ERR_NAN;
    else if (outer_fail) rep.status = UWGPU_ERR_NOT_CONVERGED;
    else rep.status = UWGPU_OK;
    if (o.target_rel_residual > 0 && rep.rel_residual > o.target_rel_residual && rep.status == UWGPU_OK)
        rep.status = UWGPU_ERR_NOT_CONVERGED;
    rep.converged = rep.status == UWGPU_OK && !inner_fail ? 1 : 0;
}

void solve_bsscr(Context& c, const uwgpu_solve_opts& o, uwgpu_report& rep) {
    UWG_REQUIRE(c.assembled, UWGPU_ERR_STATE, "solve requested before assembly");
    UWG_REQUIRE(!c.assembled_jacobian, UWGPU_ERR_UNSUPPORTED,
                "the Newton form's element matrices are not symmetric; the solver here takes the Picard form "
                "(uwgpu_jacobian_set(ctx, 0) and assemble again)");
    UWG_REQUIRE(o.precision == UWGPU_PREC_FP64 || o.precision == UWGPU_PREC_MIXED, UWGPU_ERR_ARGUMENT, "bad precision");
    UWG_REQUIRE(o.schur_type == UWGPU_SCHUR_CG || o.schur_type == UWGPU_SCHUR_FGMRES, UWGPU_ERR_ARGUMENT, "bad Schur type");
    UWG_REQUIRE(o.schur_pc >= 0 && o.schur_pc <= 3, UWGPU_ERR_ARGUMENT, "bad Schur preconditioner");
    UWG_REQUIRE(o.smoother == UWGPU_SMOOTHER_COLOUR_GS || o.smoother == UWGPU_SMOOTHER_CHEBYSHEV, UWGPU_ERR_ARGUMENT, "bad smoother");
    UWG_REQUIRE(o.remove_const_p >= 0 && o.remove_const_p <= 2, UWGPU_ERR_ARGUMENT, "bad pressure null-space mode");
    UWG_REQUIRE(o.learned_pc == 0 || o.learned_pc == 1, UWGPU_ERR_ARGUMENT, "bad learned_pc");
    UWG_REQUIRE(o.mg_cycle == 1 || o.mg_cycle == 2, UWGPU_ERR_ARGUMENT, "mg_cycle must be 1 (V) or 2 (W)");
    UWG_REQUIRE(o.bfbt_inner_pc >= 0 && o.bfbt_inner_pc <= 4, UWGPU_ERR_ARGUMENT, "bfbt_inner_pc must be 0..4");
    Bsscr s(c, o, rep);
    s.run();
}

// Largest eigenvalue of Dinv A on the fine level for the Chebyshev smoother (timing hooks).
void estimate_fine_lmax(Context& c, const uwgpu_solve_opts& o) {
    uwgpu_report rep;
    std::memset(&rep, 0, sizeof(rep));
    uwgpu_solve_opts oc = o;
    oc.smoother = UWGPU_SMOOTHER_CHEBYSHEV;
    Bsscr s(c, oc, rep);
    s.setup_velocity();
}

// Training pairs for the learned correction, produced by the multigrid solver of the assembled
// system.  For each right-hand side b (the assembled buoyancy force first, then random
// multi-scale fields, zero on Dirichlet dofs) the exact solution u* is computed by a tight
// FGMRES solve, and the plain multigrid iteration u <- u + V(b - K u) is run from u = 0.  Every
// iterate gives one pair: inputs the residual r = b - K u and the V-cycle's answer V(r), target
// the error left after that cycle, u* - u - V(r).  Late iterates carry the slowly converging
// modes that a velocity solve spends its iterations on.  Returns the number of pairs.
int learned_generate(Context& c, const uwgpu_solve_opts& o, int nsamples, uint64_t seed) {
    UWG_REQUIRE(c.assembled, UWGPU_ERR_STATE, "training data requested before assembly");
    UWG_REQUIRE(c.net != nullptr, UWGPU_ERR_STATE, "no network (uwgpu_learned_create)");
    UWG_REQUIRE(c.net->nn == c.mesh.nn, UWGPU_ERR_STATE, "the network was built for another mesh");
    UWG_REQUIRE(nsamples > 0, UWGPU_ERR_ARGUMENT, "nsamples must be positive");
    uwgpu_report rep;
    std::memset(&rep, 0, sizeof(rep));
    uwgpu_solve_opts o64 = o;
    o64.precision = UWGPU_PREC_FP64;
    o64.learned_pc = 0;
    Bsscr s(c, o64, rep);
    s.setup_velocity();
    s.gm64.setup(s.nv, o64.restart > 0 ? o64.restart : 30);
    unet::Net& n = *c.net;
    const int64_t nv = s.nv;
    const int per_rhs = 12;   // multigrid iterates per right-hand side
    DArray<double> b, us, u, r, v, e;
    for (auto* a : {&b, &us, &u, &r, &v, &e}) a->ensure(nv);
    unet::dataset_reserve(c, n, nsamples);
    const Level& L0 = c.levels[0];
    for (int src = 0; n.nsamples < nsamples; ++src) {
        if (src == 0) gather_force(c, b.p);
        else unet::random_field(c, n, seed + (uint64_t)src, b.p);
        double res = 0.0, bn = 0.0;
        bool nanflag = false;
        s.gm64.solve([&](const double* in, double* out) { level_apply<double>(c, L0, in, out); },
                     [&](const double* in, double* out) { s.vcycle<double>(0, in, out); }, b.p, us.p, 1e-11,
                     o64.max_inner > 0 ? o64.max_inner : 500, &res, &bn, &nanflag);
        UWG_REQUIRE(!nanflag, UWGPU_ERR_NAN, "NaN while generating training pairs");
        if (!(bn > 0.0)) continue;
        zero<double>(c, nv, u.p);
        const double un = s.red.norm<double>(nv, us.p);
        for (int k = 0; k < per_rhs && n.nsamples < nsamples; ++k) {
            level_residual<double>(c, L0, u.p, b.p, r.p);
            s.vcycle<double>(0, r.p, v.p);
            // e = u* - u (error before the cycle); the stored target is e - V(r)
            copy<double>(c, nv, us.p, e.p);
            axpy<double>(c, nv, -1.0, u.p, e.p);
            unet::dataset_add(c, n, r.p, e.p, v.p);
            axpy<double>(c, nv, 1.0, v.p, u.p);
            if (s.red.norm<double>(nv, e.p) <= 1e-8 * un) break;
        }
    }
    unet::dataset_finish(c, n);
    return n.nsamples;
}

}  // namespace uwg

namespace uwg {

// SystemLinearEquations_NonLinearExecute (SystemLinearEquations.c:750-935): the residual is the
// relative change of the velocity solution vector between successive solves.  With tol > 0, a
// loop that ends at max_iterations without reaching it reports UWGPU_ERR_NOT_CONVERGED (the
// reference's "Failed to converge" branch, SystemLinearEquations.c:908-914); tol <= 0 runs
// exactly max_iterations solves.
void solve_picard(Context& c, const uwgpu_solve_opts& o, double tol, int maxit, int minit, uwgpu_report& rep,
                  int& iterations, double& residual) {
    UWG_REQUIRE(c.mapped, UWGPU_ERR_STATE, "Picard iteration requested before bin_and_map");
    UWG_REQUIRE(maxit >= 1, UWGPU_ERR_ARGUMENT, "max_iterations must be positive");
    Reducer red(c);
    int64_t nv = c.mesh.nn * c.mesh.dim;
    DArray<double> prev;
    prev.ensure((size_t)nv);
    residual = 0.0;
    iterations = 0;
    bool converged = false;
    uwgpu_report r;
    for (int it = 0; it < maxit; ++it) {
        bool have_prev = c.has_solution;
        if (have_prev) UWG_CUDA(cudaMemcpyAsync(prev.p, c.u_sol.p, nv * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        assemble(c);
        std::memset(&r, 0, sizeof(r));
        solve_bsscr(c, o, r);
        iterations = it + 1;
        rep.outer_its += r.outer_its;
        rep.inner_its_total += r.inner_its_total;
        rep.backsolve_its += r.backsolve_its;
        rep.vcycles += r.vcycles;
        rep.pc_inner_its += r.pc_inner_its;
        rep.t_setup_ms += r.t_setup_ms;
        rep.t_solve_ms += r.t_solve_ms;
        rep.rel_residual = r.rel_residual;
        rep.status = r.status;
        rep.converged = r.converged;
        if (r.status != UWGPU_OK) return;
        if (!have_prev) continue;
        {
            LaunchScope ls(c, UWGPU_KERNEL_VECTOR);
            k_axpy<double><<<blocks_for(nv, 256), 256, 0, c.stream>>>(nv, -1.0, c.u_sol.p, prev.p);
        }
        double dn = red.norm<double>(nv, prev.p), un = red.norm<double>(nv, c.u_sol.p);
        residual = un > 0.0 ? dn / un : 0.0;
        if (!std::isfinite(residual)) {
            rep.status = UWGPU_ERR_NAN;
            return;
        }
        if (residual < tol && iterations >= minit) {
            converged = true;
            break;
        }
    }
    if (tol > 0.0 && !converged) {
        rep.status = UWGPU_ERR_NOT_CONVERGED;
        rep.converged = 0;
    }
}

}  // namespace uwg
