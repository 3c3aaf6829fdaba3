// Allocation-free variant of the binning + integration-point mapping pass.
//
// Some callers cannot allocate device memory once they are running: a solver embedded in a
// host framework that owns every device buffer through its own pool, code running inside a
// region where allocation is forbidden (an allocation would synchronise the device or break the
// caller's memory budget), or a plugin that is handed pre-sized buffers.  For them this entry
// point needs no context and allocates nothing: the caller passes device-accessible inputs and
// outputs, and the scratch the pass needs (element of each point, per-element counts and
// cursors, the unordered permutation, a flag word) lives in one file-scope __device__ array of
// fixed size.  Sizes beyond that array are rejected with UWGPU_ERR_TOO_LARGE.
//
// The array exists once per device that loads the library and stays until the process exits.
// Every call shares it, so calls whose GPU work overlaps (for example on two streams) race;
// callers must order them.  The array keeps the previous call's contents: the counters and the
// flag are cleared at the start of every call.
//
// Host code cannot use the array's name as a device address (on the host it names a stand-in
// object); its device address is looked up once per device with cudaGetSymbolAddress, on the
// first call made while that device is current.
//
// Every call ends by copying the outside-point count to the host and synchronising its stream,
// so no call can be made while that stream is being captured into a CUDA graph.
#include <mutex>

#include "internal.cuh"

namespace uwg_noalloc {

constexpr int64_t kMaxPoints = UWGPU_NOALLOC_MAX_POINTS;
constexpr int64_t kMaxElements = UWGPU_NOALLOC_MAX_ELEMENTS;
// layout of the scratch words
constexpr int64_t kOffCell = 0;
constexpr int64_t kOffTmp = kOffCell + kMaxPoints;
constexpr int64_t kOffCount = kOffTmp + kMaxPoints;
constexpr int64_t kOffCursor = kOffCount + kMaxElements;
constexpr int64_t kOffFlag = kOffCursor + kMaxElements;
constexpr int64_t kWords = kOffFlag + 64;

static __device__ __align__(256) uint32_t g_scratch[kWords];

constexpr int kMaxDevices = 64;
static uint32_t* g_addr[kMaxDevices];
static std::mutex g_lock;

struct MeshP {
    int nel[3];
    double min[3], max[3];
};

__device__ __forceinline__ bool approx0(double v) { return v >= -1e-12 && v <= 1e-12; }

// Element of each point (Mesh_RegularAlgorithms_SearchElements rule) and per-element counts.
template <int DIM>
__global__ void k_na_locate(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ z, MeshP mp, uint32_t* __restrict__ s) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double pt[3] = {x[p], y[p], DIM == 3 ? z[p] : 0.0};
    unsigned ind[3] = {0u, 0u, 0u};
    bool ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double sep = (mp.max[d] - mp.min[d]) / mp.nel[d];
        if (!isfinite(pt[d])) {
            ok = false;
        } else if (approx0(pt[d] - mp.max[d])) {
            ind[d] = (unsigned)(mp.nel[d] - 1);
        } else if (pt[d] < mp.min[d] || pt[d] > mp.max[d]) {
            ok = false;
        } else {
            double out = (pt[d] - mp.min[d]) / sep;
            double whole = trunc(out);
            unsigned i = (unsigned)whole;
            if (i > 0 && approx0(out - whole)) i--;
            if (i >= (unsigned)mp.nel[d]) i = (unsigned)mp.nel[d] - 1;
            ind[d] = i;
        }
    }
    if (!ok) {
        s[kOffCell + p] = 0xffffffffu;
        atomicAdd(&s[kOffFlag], 1u);
        return;
    }
    unsigned e = ind[0] + (unsigned)mp.nel[0] * (ind[1] + (unsigned)mp.nel[1] * ind[2]);
    s[kOffCell + p] = e;
    atomicAdd(&s[kOffCount + e], 1u);
}

// Exclusive scan of the counts into offsets[0..ne] by one block (ne <= kMaxElements): the counts
// are read in tiles of blockDim.x consecutive words (one per thread, coalesced), each tile is
// scanned in the block and carried into the next.
__global__ void k_na_scan(int64_t ne, const uint32_t* __restrict__ s, uint32_t* __restrict__ offsets) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (int64_t t = 0; t < ne; t += blockDim.x) {
        const int64_t i = t + threadIdx.x;
        const uint32_t v = i < ne ? s[kOffCount + i] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < nwarps ? warp_tot[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += u;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        const uint32_t base = carry;
        const uint32_t excl = base + (warp ? warp_tot[warp - 1] : 0u) + incl - v;
        if (i < ne) offsets[i] = excl;
        __syncthreads();   // every thread has read carry and warp_tot
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[ne] = carry;
}

__global__ void k_na_scatter(int64_t n, const uint32_t* __restrict__ offsets, uint32_t* __restrict__ s) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t e = s[kOffCell + p];
    if (e == 0xffffffffu) return;
    uint32_t slot = offsets[e] + atomicAdd(&s[kOffCursor + e], 1u);
    s[kOffTmp + slot] = (uint32_t)p;
}

// Local coordinate of point v in element e along every axis, written to slot `slot` (SoA [d][slot]).
template <int DIM>
__device__ __forceinline__ void na_map_point(const int64_t idx[3], const MeshP& mp, uint32_t v, uint32_t slot, int64_t n,
                                             const double* __restrict__ x, const double* __restrict__ y,
                                             const double* __restrict__ z, double* __restrict__ xi) {
    double pt[3] = {x[v], y[v], DIM == 3 ? z[v] : 0.0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double x0 = uwg::node_coord_1d(idx[d], mp.nel[d], mp.min[d], mp.max[d]);
        double h = uwg::node_coord_1d(idx[d] + 1, mp.nel[d], mp.min[d], mp.max[d]) - x0;
        xi[(int64_t)d * n + slot] = (2.0 * (pt[d] - x0) - h) / h;
    }
}

// One warp per element: rank the element's points by index (the reference's append order),
// write the permutation and the local coordinates.  Elements with at most 32 points rank in
// registers (one point per lane, exchanged by shuffles); fuller elements re-read their run.
template <int DIM>
__global__ void k_na_sort_map(int64_t ne, int64_t n, MeshP mp, const uint32_t* __restrict__ offsets,
                              const uint32_t* __restrict__ s, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z,
                              uint32_t* __restrict__ perm, double* __restrict__ xi) {
    int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (e >= ne) return;
    uint32_t beg = offsets[e], cnt = offsets[e + 1] - beg;
    int64_t idx[3] = {e % mp.nel[0], (e / mp.nel[0]) % mp.nel[1], DIM == 3 ? e / ((int64_t)mp.nel[0] * mp.nel[1]) : 0};
    if (cnt <= 32u) {
        uint32_t v = lane < (int)cnt ? s[kOffTmp + beg + lane] : 0xffffffffu;
        uint32_t rank = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) rank += (__shfl_sync(0xffffffffu, v, j) < v) ? 1u : 0u;
        if (lane < (int)cnt) {
            perm[beg + rank] = v;
            na_map_point<DIM>(idx, mp, v, beg + rank, n, x, y, z, xi);
        }
        return;
    }
    for (uint32_t i = lane; i < cnt; i += 32) {
        uint32_t v = s[kOffTmp + beg + i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < cnt; ++j) rank += (s[kOffTmp + beg + j] < v) ? 1u : 0u;
        perm[beg + rank] = v;
        na_map_point<DIM>(idx, mp, v, beg + rank, n, x, y, z, xi);
    }
}

static uint32_t* scratch_address(int dev) {
    std::lock_guard<std::mutex> g(g_lock);
    if (!g_addr[dev]) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess) return nullptr;
        g_addr[dev] = (uint32_t*)ptr;
    }
    return g_addr[dev];
}

// Launches `fn` and returns the launch's own status (cudaLaunchKernel reports a bad
// configuration of this launch rather than an error left pending by earlier, unrelated work).
static cudaError_t launch(const void* fn, unsigned blocks, unsigned threads, cudaStream_t st, void** args) {
    return cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, 0, st);
}

}  // namespace uwg_noalloc

extern "C" int uwgpu_bin_and_map_noalloc(int32_t dim, const int32_t nel[3], const double min[3], const double max[3],
                                         int64_t n, const double* x, const double* y, const double* z,
                                         uint32_t* perm, uint32_t* offsets, double* xi, void* stream,
                                         uint32_t* outside) {
    using namespace uwg_noalloc;
    if ((dim != 2 && dim != 3) || !nel || !min || !max || n < 0 || !offsets) return UWGPU_ERR_ARGUMENT;
    if (n > 0 && (!x || !y || (dim == 3 && !z) || !perm || !xi)) return UWGPU_ERR_ARGUMENT;
    int64_t ne = 1;
    MeshP mp;
    for (int d = 0; d < 3; ++d) {
        mp.nel[d] = d < dim ? nel[d] : 1;
        mp.min[d] = min[d];
        mp.max[d] = max[d];
        if (d < dim && (nel[d] < 1 || !(max[d] > min[d]))) return UWGPU_ERR_ARGUMENT;
        // checked one factor at a time, so that the product cannot overflow
        if (mp.nel[d] > kMaxElements / ne) return UWGPU_ERR_TOO_LARGE;
        ne *= mp.nel[d];
    }
    if (n > kMaxPoints || ne > kMaxElements) return UWGPU_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return UWGPU_ERR_CUDA;
    uint32_t* s = scratch_address(dev);
    if (!s) return UWGPU_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // clear the counters, cursors and the flag left by the previous call
    if (cudaMemsetAsync(s + kOffCount, 0, (size_t)(kOffFlag + 1 - kOffCount) * sizeof(uint32_t), st) != cudaSuccess)
        return UWGPU_ERR_CUDA;
    if (n > 0) {
        void* args[] = {&n, (void*)&x, (void*)&y, (void*)&z, &mp, &s};
        const void* fn = dim == 3 ? (const void*)k_na_locate<3> : (const void*)k_na_locate<2>;
        if (launch(fn, (unsigned)((n + 255) / 256), 256, st, args) != cudaSuccess) return UWGPU_ERR_CUDA;
    }
    {
        void* args[] = {&ne, &s, &offsets};
        if (launch((const void*)k_na_scan, 1, 1024, st, args) != cudaSuccess) return UWGPU_ERR_CUDA;
    }
    if (n > 0) {
        void* sargs[] = {&n, &offsets, &s};
        if (launch((const void*)k_na_scatter, (unsigned)((n + 255) / 256), 256, st, sargs) != cudaSuccess)
            return UWGPU_ERR_CUDA;
        void* margs[] = {&ne, &n, &mp, &offsets, &s, (void*)&x, (void*)&y, (void*)&z, &perm, &xi};
        const void* fn = dim == 3 ? (const void*)k_na_sort_map<3> : (const void*)k_na_sort_map<2>;
        if (launch(fn, (unsigned)((ne * 32 + 255) / 256), 256, st, margs) != cudaSuccess) return UWGPU_ERR_CUDA;
    }
    uint32_t out = 0;
    if (cudaMemcpyAsync(&out, s + kOffFlag, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return UWGPU_ERR_CUDA;
    if (outside) *outside = out;
    return out ? UWGPU_ERR_DOMAIN : UWGPU_OK;
}
