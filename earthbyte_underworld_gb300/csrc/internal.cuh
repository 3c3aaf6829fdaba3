// Internal declarations of libuwgpu: device context, buffers, launch accounting.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/uwgpu.h"

namespace uwg {

namespace unet {
struct Net;
void destroy(Net* n);
}

// Error carried from the internals to the C entry points, which turn it into a status code.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A failed runtime call also leaves its error as the thread's last error; it is cleared here so
// that a later launch check does not report it again.
#define UWG_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            (void)cudaGetLastError();                                                      \
            throw ::uwg::Error(e_ == cudaErrorMemoryAllocation ? UWGPU_ERR_MEMORY          \
                                                               : UWGPU_ERR_CUDA,           \
                               std::string(#call) + ": " + cudaGetErrorString(e_));        \
        }                                                                                  \
    } while (0)

#define UWG_REQUIRE(cond, code, msg)                                                       \
    do {                                                                                   \
        if (!(cond)) throw ::uwg::Error((code), (msg));                                    \
    } while (0)

// Owning device array (cudaMalloc / cudaFree), grown on demand, never shrunk.
// The stream of the API call in progress on this thread (the C entry points set it): device arrays
// are taken from and returned to the device's stream-ordered memory pool on it, whose release
// threshold keeps freed memory in the pool, so the work buffers of a solve cost no cudaMalloc or
// cudaFree after the first solve.  Outside an API call arrays use plain cudaMalloc.
inline cudaStream_t& alloc_stream() {
    static thread_local cudaStream_t s = nullptr;
    return s;
}

template <typename T>
struct DArray {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;   // stream it was allocated on (pooled arrays)
    bool pooled = false;
    DArray() = default;
    DArray(const DArray&) = delete;
    DArray& operator=(const DArray&) = delete;
    ~DArray() { release(); }
    void release() {
        if (p) {
            // a pooled array goes back to the pool in stream order; if its stream is gone the
            // synchronous free is the fallback
            if (!pooled || cudaFreeAsync(p, s) != cudaSuccess) {
                (void)cudaGetLastError();
                cudaFree(p);
            }
        }
        p = nullptr;
        n = 0;
        pooled = false;
    }
    void ensure(size_t count) {
        if (count <= n && p) return;
        release();
        if (count == 0) count = 1;
        cudaStream_t st = alloc_stream();
        if (st) {
            UWG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), st));
            // the allocation completes before any stream (and synchronous copies) may use it
            UWG_CUDA(cudaStreamSynchronize(st));
            s = st;
            pooled = true;
        } else {
            UWG_CUDA(cudaMalloc(&p, count * sizeof(T)));
        }
        n = count;
    }
    // exchanges the storage of two arrays (every field)
    void swap(DArray& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
        std::swap(s, o.s);
        std::swap(pooled, o.pooled);
    }
    T* get() const { return p; }
};

// Regular Cartesian Q1 mesh description (node index = i + nx*(j + ny*k), x fastest).
struct MeshDesc {
    int dim = 0;
    int nel[3] = {1, 1, 1};
    double min[3] = {0, 0, 0};
    double max[3] = {1, 1, 1};
    int64_t nnx = 1, nny = 1, nnz = 1;  // node counts per axis
    int64_t nn = 0, ne = 0;
};

// Node coordinate along axis d of node index i: CartesianGenerator_CalcGeom without contact
// depth (StgDomain/Mesh/src/CartesianGenerator.c:2275-2310).
__host__ __device__ inline double node_coord_1d(int64_t i, int nel, double mn, double mx) {
    if (i <= 0) return mn;
    if (i >= nel) return mx;
    return mn + ((double)i / (double)nel) * (mx - mn);
}

constexpr int kMaxLevels = 10;

// One level of the geometric hierarchy (level 0 = fine, as the solver sees it).
struct Level {
    MeshDesc mesh;
    DArray<double> Ke;       // packed upper-triangular element matrices, entry-major [k][e]
    DArray<double> A64;      // node-block stencil, entry-major [q][r][c][node]
    DArray<float> A32;
    DArray<double> Dinv64;   // inverse of the node's diagonal block [r][c][node]
    DArray<float> Dinv32;
    // FP16 copy of the stencil for the mixed form's smoothing and V-cycle residuals: each row
    // (r, node) divided by its largest magnitude S16[r][node]; IEEE half bits, the entries of
    // neighbours 2p and 2p + 1 in one word [p][r][c][node]
    DArray<uint32_t> A16;
    DArray<float> S16;
    bool has16 = false;
    DArray<uint8_t> fixed;   // per dof (node*dim+d), Dirichlet mask
    // work vectors (SoA by component: [d][node])
    DArray<double> r64, x64, b64, t64;
    DArray<float> r32, x32, b32, t32;
    // coarsest level: dense inverse of the full-dof operator
    DArray<double> Cinv;
    double lmax = 0.0;       // largest eigenvalue estimate of Dinv A (Chebyshev smoother)
    int64_t ncoarse = 0;
    bool has32 = false;
};

struct ProfileFamily {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
    size_t used = 0;
    int64_t launches = 0;
    double ms = 0.0;
    double bytes = 0.0;   // algorithmic bytes of the profiled launches
    double flops = 0.0;
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int64_t launches = 0;

    MeshDesc mesh;
    bool has_mesh = false;

    // boundary conditions (fine level)
    DArray<uint8_t> fixed;
    DArray<double> bcval;
    bool has_bc = false;
    bool bc_nonzero = false;

    // materials and fields
    DArray<uwgpu_material> mats;
    int nmat = 0;
    DArray<double> temperature;
    bool has_temperature = false;
    double gravity = 0.0;
    int vert_axis = 1;
    DArray<double> u_sol;     // nodal velocity, SoA [d][node]
    DArray<double> p_sol;     // element pressure
    bool has_solution = false;

    // material points
    int64_t np = 0;
    DArray<double> px, py, pz;
    DArray<double> qx, qy, qz;    // second coordinate set for advection (swapped in on success)
    DArray<int32_t> pmat;
    DArray<double> peta, prho;
    bool has_peta = false, has_prho = false;
    // strain-weakening history (postFailureWeakening) per point and its time derivative from the
    // last assembly (StrainWeakening.c), when set
    DArray<double> pfw, pfw_incr;
    bool has_pfw = false;
    bool has_points = false;

    // binning / mapping
    DArray<uint32_t> cell, counts, offsets, cursor, perm, tmp_perm, block_sums;
    DArray<uint32_t> err_count;
    DArray<double> sxi;       // [d][slot]
    // integration weights: constant 2^dim / count, or discrete Voronoi cells of dvc_res cells
    // per axis (centroids dvc_xi [d][slot], volumes dvc_w [slot], boundary sets dvc_bnd)
    int weights_kind = 0;
    int dvc_res[3] = {10, 10, 10};
    DArray<double> dvc_xi, dvc_w;
    DArray<uint32_t> dvc_bnd;
    DArray<int32_t> smat;
    DArray<double> seta_in, srho_in, seta_out;
    bool mapped = false;

    // assembly (fine level)
    DArray<double> fe;        // entry-major [k][e]
    DArray<double> Se;
    DArray<double> Ge;        // entry-major [k][e]
    bool assembled = false;
    int assembly_mode = UWGPU_ASSEMBLY_FP64;
    // Newton form of the 2D element matrices (SystemLinearEquations nlFormJacobian): full
    // non-symmetric K_e [64][e] of the last assembly
    bool jacobian = false;
    bool assembled_jacobian = false;
    DArray<double> Kjac;
    DArray<double> mom;       // 3D moments [27][e] of the tensor-core contraction

    // per-axis element widths of the fine mesh (device), and the mesh they belong to
    DArray<double> elem_h;
    int64_t elem_h_for = -1;
    DArray<float> elem_h32;
    int64_t elem_h32_for = -2;

    // solver state
    Level levels[kMaxLevels];
    int nlevels = 0;
    bool operator_built = false;
    int operator_levels = 0;
    bool operator_has32 = false;
    DArray<double> scratch;   // reductions
    double* host_scalars = nullptr;   // pinned

    bool profiling = false;
    ProfileFamily prof[UWGPU_KERNEL_COUNT];
    // while >= 0, every launch is counted in this family (the solver's setup phase)
    int family_override = -1;
    // the mixed form smooths (and forms V-cycle residuals) with the FP16 row-scaled stencils
    bool smooth16 = true;

    // multigrid hierarchy of the BFBt operator G^T W G (gwg_stencil.cu): element grids coarsened
    // 2:1 by aggregation; level 0's stencil belongs to the solve, the others live here, as do the
    // work vectors of every level (stable addresses for the captured CG graphs)
    struct GwgLevel {
        int64_t ex = 0, ey = 0, ez = 0, ne = 0;
        DArray<double> A64, dinv64, b64, x64, r64, t64, d64;
        DArray<float> A32, dinv32, b32, x32, r32, t32, d32;
        double lmax = 0.0;
    };
    GwgLevel gwg[kMaxLevels];
    int gwg_nlev = 0;
    DArray<double> gwg_Cinv;     // dense inverse on the coarsest level
    int64_t gwg_ncoarse = 0;

    // CUDA graphs of the BFBt inner-CG iteration block, one per buffer set
    struct PcgGraph {
        const void* key[9];
        cudaGraphExec_t exec = nullptr;
    };
    // Coarse correction of the BFBt inner solves on the element checkerboards of single planes
    // (gwg_stencil.cu), built per solve when requested: E_F^-1 per family (row-major blocks of
    // ez^2, ey^2, ex^2), the coarse residuals s (two buffers of ez + ey + ex) and the coarse
    // solution y
    struct CoarseCheckerboards {
        bool on = false;
        int ex = 0, ey = 0, ez = 0;
        DArray<double> einv, s, y, ed;
    } cc;
    std::vector<PcgGraph> pcg_graphs;

    // learned velocity preconditioner (csrc/unet.cu), created on request
    unet::Net* net = nullptr;

    ~Context() {
        unet::destroy(net);
        for (auto& g : pcg_graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
    }
};

// Launch bookkeeping: counts every launch, and brackets the launch with events when the
// family is being profiled.
struct LaunchScope {
    Context& c;
    int family;
    cudaEvent_t e1 = nullptr;
    LaunchScope(Context& ctx, int fam) : c(ctx), family(ctx.family_override >= 0 ? ctx.family_override : fam) {
        c.launches++;
        if (c.profiling && family >= 0) {
            ProfileFamily& f = c.prof[family];
            if (f.used == f.events.size()) {
                cudaEvent_t a, b;
                UWG_CUDA(cudaEventCreate(&a));
                UWG_CUDA(cudaEventCreate(&b));
                f.events.emplace_back(a, b);
            }
            auto& pr = f.events[f.used++];
            UWG_CUDA(cudaEventRecord(pr.first, c.stream));
            e1 = pr.second;
            f.launches++;
        }
    }
    ~LaunchScope() {
        if (e1) cudaEventRecord(e1, c.stream);
    }
};

// Counts every launch of its lifetime in one family (the solver's setup phase).
struct FamilyOverride {
    Context& c;
    int saved;
    FamilyOverride(Context& ctx, int fam) : c(ctx), saved(ctx.family_override) { c.family_override = fam; }
    ~FamilyOverride() { c.family_override = saved; }
};

// Records the algorithmic work of one launch of `family` while profiling.
inline void note_work(Context& c, int family, double bytes, double flops) {
    if (c.family_override >= 0) family = c.family_override;
    if (c.profiling && family >= 0) {
        c.prof[family].bytes += bytes;
        c.prof[family].flops += flops;
    }
}

inline void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(UWGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Dynamic shared memory for a tensor-core kernel that holds `ncols` TMEM columns per CTA: at
// least `need` bytes, and enough that at most 512 / ncols CTAs of it fit on an SM, so the SM's 512
// TMEM columns cover every resident CTA and no CTA waits for another one's columns.  Sets the
// kernel's dynamic shared-memory limit; *per_sm receives the CTAs per SM the request allows.
inline size_t tmem_safe_smem(const void* fn, int device, size_t need, uint32_t ncols, int* per_sm) {
    int optin = 0, sm_cap = 0;
    UWG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    UWG_CUDA(cudaDeviceGetAttribute(&sm_cap, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device));
    cudaFuncAttributes fa;
    UWG_CUDA(cudaFuncGetAttributes(&fa, fn));
    const size_t stat = fa.sharedSizeBytes, reserve = 1024;
    const size_t max_dyn = (size_t)optin - stat;
    UWG_REQUIRE(need <= max_dyn, UWGPU_ERR_ARGUMENT, "tensor-core kernel: shared memory plan too large");
    int max_cta = (int)(512 / ncols);
    if (max_cta > 16) max_cta = 16;
    size_t req = need;
    const size_t floor_total = (size_t)sm_cap / (size_t)(max_cta + 1) + 1;   // per-CTA footprint above which max_cta + 1 do not fit
    if (req + stat + reserve < floor_total) req = floor_total - stat - reserve;
    if (req > max_dyn) req = max_dyn;
    int fit = (int)((size_t)sm_cap / (req + stat + reserve));
    *per_sm = fit < 1 ? 1 : (fit < max_cta ? fit : max_cta);
    UWG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)req));
    return req;
}

inline unsigned blocks_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : b);
}

// ---- functions shared between translation units ----
void bin_and_map(Context& c);
void assemble(Context& c);
void strain_weakening_advance(Context& c, double dt);
int64_t population_control(Context& c, const uwgpu_pcdvc_opts& o);
void build_operator(Context& c, int levels, bool need32);
void apply_fine(Context& c, bool fp32, const double* x, double* y);  // device SoA vectors
void solve_bsscr(Context& c, const uwgpu_solve_opts& o, uwgpu_report& rep);
void estimate_fine_lmax(Context& c, const uwgpu_solve_opts& o);
void weights_set(Context& c, int kind, const int32_t res[3]);
void integration_points(Context& c, const double** xi, const double** w);
void integration_points_download(Context& c, double* xi, double* w);
void bfbt_operator_hook(Context& c, int form, const double* xh, double* yh, int iterations, double* ms);
int tc_check(int layout, int fmt, int N, int K, const uint16_t* A, const uint16_t* B, float* D);
void advect_particles(Context& c, double dt, int order, bool fallback, uint32_t& fell_back, uint32_t& left_mesh);
template <typename T> void level_cheb(Context&, Level&, const T*, T*, int, bool);
int learned_generate(Context& c, const uwgpu_solve_opts& o, int nsamples, uint64_t seed);
void solve_picard(Context& c, const uwgpu_solve_opts& o, double tol, int maxit, int minit, uwgpu_report& rep,
                  int& iterations, double& residual);
template <typename T> void level_apply(Context&, const Level&, const T*, T*);
template <typename T> void level_smooth(Context&, const Level&, const T*, T*, int, bool);

// Number of packed entries of a symmetric nd x nd element matrix.
__host__ __device__ constexpr int packed_size(int nd) { return nd * (nd + 1) / 2; }
// Packed index of (r, c) with r <= c, row-major upper triangle.
__host__ __device__ inline int packed_index(int nd, int r, int c) {
    return r * nd - (r * (r - 1)) / 2 + (c - r);
}

}  // namespace uwg
