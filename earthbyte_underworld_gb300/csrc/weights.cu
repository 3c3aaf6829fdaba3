// Discrete Voronoi cell weights of the integration points (PICellerator/Weights/src/DVCWeights.c),
// one warp per element.
//
// The element's local square / cube [-1, 1]^dim carries a fixed grid of res[0] x res[1] (x res[2])
// cells, x fastest, at most 1024 cells: cell c is bit (c & 31) of word (c >> 5), and lane l of
// the warp holds word l of every cell set.  Every point first claims the cell that holds it (a
// later point in the same cell takes it over).  Then the points grow their regions in passes, in
// point order, as the reference does (_DVCWeights_CreateVoronoi, DVCWeights.c:668-714):
//   claim   (_DVCWeights_ClaimCells, :261-317): every cell of the point's boundary set is taken
//           when free, or when held by another point that is farther from the cell's centre
//           (_DVCWeights_DistanceTest, :604-609, evaluated in the same operation order with
//           round-to-nearest intrinsics, so the contest is decided exactly as in FP64 C);
//   update  (_DVCWeights_UpdateBchain, :395-446): the new boundary set is the face neighbours of
//           the cells just taken that the point does not hold (bit shifts of the 1024-bit set
//           across the lanes, with row and plane masks so that no shift wraps around the grid).
// The cells a point tries in one claim are distinct and each decision reads only that cell's
// owner, so processing a boundary set in parallel gives the reference's sequential result.
// Passes end when one takes no cell (each cell changes owner only to a strictly nearer point, so
// the count of passes is bounded; a cap of cells x points + 2 passes flags an error).  Weight =
// cells held x cell volume; new local coordinate = mean of the held cells' centres, summed in
// cell order (_DVCWeights_GetCentroids, :203-231), lane j accumulating point j.
// Owners live in shared memory (4 KB per warp, transposed so that lane l's 32 cells are
// conflict-free); boundary sets live in a per-slot scratch array (32 words per point).
#include <algorithm>
#include <cstring>

#include "internal.cuh"

namespace uwg {

namespace {

constexpr int kDvcWarps = 4;

struct DvcArgs {
    int dim, nx, ny, nz, nc;
    double cen[3][32];   // cell centres per axis (accumulated as in _DVCWeights_ConstructGrid)
    double h[3];         // cell widths 2 / res
    double da;           // cell volume
    int64_t ne, nslots;
    const uint32_t* offsets;
    const double* sxi;   // [d][slot]
    double* oxi;         // [d][slot]
    double* ow;          // [slot]
    uint32_t* bnd;       // [slot][32]
    uint32_t* err;       // [0] elements whose passes hit the cap
};

__device__ __forceinline__ uint32_t shl_set(uint32_t w, int s, int lane) {
    // bit c of the result = bit c - s of the set
    const int q = s >> 5, r = s & 31;
    uint32_t a = __shfl_up_sync(0xffffffffu, w, q);
    uint32_t b = __shfl_up_sync(0xffffffffu, w, q + 1);
    a = lane >= q ? a : 0u;
    b = lane >= q + 1 ? b : 0u;
    return r ? (a << r) | (b >> (32 - r)) : a;
}

__device__ __forceinline__ uint32_t shr_set(uint32_t w, int s, int lane) {
    // bit c of the result = bit c + s of the set
    const int q = s >> 5, r = s & 31;
    uint32_t a = __shfl_down_sync(0xffffffffu, w, q);
    uint32_t b = __shfl_down_sync(0xffffffffu, w, q + 1);
    a = lane + q < 32 ? a : 0u;
    b = lane + q + 1 < 32 ? b : 0u;
    return r ? (a >> r) | (b << (32 - r)) : a;
}

// (x1 + x2 - x0 - x0)(x1 - x2) + (y1 + y2 - y0 - y0)(y1 - y2) [+ z term], left to right
__device__ __forceinline__ double dvc_contest(int dim, const double c0[3], const double p1[3], const double p2[3]) {
    double t = 0.0;
    for (int d = 0; d < dim; ++d) {
        const double a = __dsub_rn(__dsub_rn(__dadd_rn(p1[d], p2[d]), c0[d]), c0[d]);
        const double v = __dmul_rn(a, __dsub_rn(p1[d], p2[d]));
        t = d == 0 ? v : __dadd_rn(t, v);
    }
    return t;
}

__global__ void __launch_bounds__(32 * kDvcWarps) k_dvc(DvcArgs a) {
    __shared__ int owner_s[kDvcWarps][1024];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    int* own = owner_s[wl];
    const int64_t warps = (int64_t)gridDim.x * kDvcWarps;
    // this lane's word of the grid masks
    uint32_t valid = 0, xlo = 0, xhi = 0, ylo = 0, yhi = 0;
    for (int k = 0; k < 32; ++k) {
        const int c = 32 * lane + k;
        if (c >= a.nc) continue;
        const int x = c % a.nx, y = (c / a.nx) % a.ny;
        valid |= 1u << k;
        if (x == 0) xlo |= 1u << k;
        if (x == a.nx - 1) xhi |= 1u << k;
        if (y == 0) ylo |= 1u << k;
        if (y == a.ny - 1) yhi |= 1u << k;
    }
    const int sy = a.nx, sz = a.nx * a.ny;
    auto dilate = [&](uint32_t s) {
        uint32_t r = (shl_set(s, 1, lane) & ~xlo) | (shr_set(s, 1, lane) & ~xhi);
        r |= (shl_set(s, sy, lane) & ~ylo) | (shr_set(s, sy, lane) & ~yhi);
        if (a.dim == 3) r |= shl_set(s, sz, lane) | shr_set(s, sz, lane);
        return r & valid;
    };
    for (int64_t e = (int64_t)blockIdx.x * kDvcWarps + wl; e < a.ne; e += warps) {
        const uint32_t beg = a.offsets[e];
        const int np = (int)(a.offsets[e + 1] - beg);
        for (int k = 0; k < 32; ++k) own[k * 32 + lane] = -1;
        __syncwarp();
        // placement, in point order; the boundary of a point is the face neighbours of its cell
        for (int p = 0; p < np; ++p) {
            int idx[3] = {0, 0, 0};
            const int n3[3] = {a.nx, a.ny, a.nz};
            for (int d = 0; d < a.dim; ++d) {
                const double x = a.sxi[(int64_t)d * a.nslots + beg + p];
                idx[d] = (int)__ddiv_rn(__dadd_rn(x, 1.0), a.h[d]);
                if (idx[d] == n3[d]) idx[d]--;
                // mapped points lie in [-1, 1], where this changes nothing; it keeps any other
                // value inside the grid
                idx[d] = min(max(idx[d], 0), n3[d] - 1);
            }
            const int c = idx[0] + a.nx * (idx[1] + a.ny * idx[2]);
            if (lane == (c >> 5)) own[(c & 31) * 32 + lane] = p;
            const uint32_t one = lane == (c >> 5) ? 1u << (c & 31) : 0u;
            a.bnd[(int64_t)(beg + p) * 32 + lane] = dilate(one);
            __syncwarp();
        }
        // growth passes
        const int64_t cap = (int64_t)a.nc * np + 2;
        int64_t pass = 0;
        bool taken = np > 0;
        while (taken) {
            if (++pass > cap) {
                if (lane == 0) atomicAdd(&a.err[0], 1u);
                break;
            }
            int total = 0;
            for (int p = 0; p < np; ++p) {
                uint32_t* bw = a.bnd + (int64_t)(beg + p) * 32;
                uint32_t b = bw[lane];
                double xp[3] = {0.0, 0.0, 0.0};
                for (int d = 0; d < a.dim; ++d) xp[d] = a.sxi[(int64_t)d * a.nslots + beg + p];
                uint32_t got = 0;
                while (b) {
                    const int k = __ffs(b) - 1;
                    b &= b - 1;
                    const int c = 32 * lane + k;
                    const int o = own[k * 32 + lane];
                    bool take = o == -1;
                    if (!take && o != p) {
                        const double c0[3] = {a.cen[0][c % a.nx], a.cen[1][(c / a.nx) % a.ny],
                                              a.dim == 3 ? a.cen[2][c / (a.nx * a.ny)] : 0.0};
                        double xo[3] = {0.0, 0.0, 0.0};
                        for (int d = 0; d < a.dim; ++d) xo[d] = a.sxi[(int64_t)d * a.nslots + beg + o];
                        take = dvc_contest(a.dim, c0, xo, xp) > 0.0;
                    }
                    if (take) {
                        own[k * 32 + lane] = p;
                        got |= 1u << k;
                    }
                }
                __syncwarp();
                total += __popc(got);
                uint32_t mine = 0;
                for (int k = 0; k < 32; ++k) mine |= (own[k * 32 + lane] == p ? 1u : 0u) << k;
                bw[lane] = dilate(got) & ~mine;
                __syncwarp();
            }
            taken = __any_sync(0xffffffffu, total != 0);
        }
        // centroids and weights: lane j accumulates point j over the cells in index order
        for (int p0 = 0; p0 < np; p0 += 32) {
            const int p = p0 + lane;
            double s[3] = {0.0, 0.0, 0.0};
            int cnt = 0;
            int x = 0, y = 0, z = 0;
            for (int c = 0; c < a.nc; ++c) {
                if (own[(c & 31) * 32 + (c >> 5)] == p) {
                    s[0] = __dadd_rn(s[0], a.cen[0][x]);
                    s[1] = __dadd_rn(s[1], a.cen[1][y]);
                    if (a.dim == 3) s[2] = __dadd_rn(s[2], a.cen[2][z]);
                    ++cnt;
                }
                if (++x == a.nx) {
                    x = 0;
                    if (++y == a.ny) {
                        y = 0;
                        ++z;
                    }
                }
            }
            if (p < np) {
                a.ow[beg + p] = __dmul_rn((double)cnt, a.da);
                for (int d = 0; d < a.dim; ++d)
                    a.oxi[(int64_t)d * a.nslots + beg + p] = cnt != 0 ? __ddiv_rn(s[d], (double)cnt) : 0.0;
            }
        }
        __syncwarp();
    }
}

// the constant weights 2^dim / count of the element (ConstantWeights.c:180-189)
__global__ void k_const_weights(int64_t ne, int dim, const uint32_t* __restrict__ offsets, double* __restrict__ w) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const uint32_t beg = offsets[e], end = offsets[e + 1];
    const double v = (dim == 3 ? 8.0 : 4.0) / (double)(end - beg);
    for (uint32_t s = beg; s < end; ++s) w[s] = v;
}

}  // namespace

void weights_set(Context& c, int kind, const int32_t res[3]) {
    UWG_REQUIRE(kind == UWGPU_WEIGHTS_CONSTANT || kind == UWGPU_WEIGHTS_DVC, UWGPU_ERR_ARGUMENT,
                "weights kind must be UWGPU_WEIGHTS_CONSTANT or UWGPU_WEIGHTS_DVC");
    if (kind == UWGPU_WEIGHTS_DVC) {
        UWG_REQUIRE(res != nullptr, UWGPU_ERR_ARGUMENT, "DVC weights need a resolution");
        const int dim = c.has_mesh ? c.mesh.dim : 3;
        int64_t nc = 1;
        for (int d = 0; d < dim; ++d) {
            UWG_REQUIRE(res[d] >= 1 && res[d] <= 32, UWGPU_ERR_ARGUMENT, "DVC resolution must be 1..32 per axis");
            nc *= res[d];
        }
        UWG_REQUIRE(nc <= 1024, UWGPU_ERR_ARGUMENT, "DVC grid limited to 1024 cells per element");
        for (int d = 0; d < 3; ++d) c.dvc_res[d] = d < dim ? res[d] : 1;
    }
    c.weights_kind = kind;
    c.assembled = false;
    c.operator_built = false;
}

// The integration points of the next assembly: with DVC weights, the Voronoi centroids and
// volumes of the mapped points (c.dvc_xi, c.dvc_w); returns the local coordinates to assemble
// from and the per-slot weights (null: constant weights).
void integration_points(Context& c, const double** xi, const double** w) {
    const MeshDesc& m = c.mesh;
    if (c.weights_kind != UWGPU_WEIGHTS_DVC) {
        *xi = c.sxi.p;
        *w = nullptr;
        return;
    }
    const int dim = m.dim;
    int64_t nc = 1;
    for (int d = 0; d < dim; ++d) nc *= c.dvc_res[d];
    UWG_REQUIRE(nc <= 1024, UWGPU_ERR_ARGUMENT, "DVC grid limited to 1024 cells per element");
    const size_t ns = (size_t)(c.np > 0 ? c.np : 1);
    c.dvc_xi.ensure((size_t)dim * ns);
    c.dvc_w.ensure(ns);
    c.dvc_bnd.ensure(32 * ns);
    c.err_count.ensure(1);
    UWG_CUDA(cudaMemsetAsync(c.err_count.p, 0, sizeof(uint32_t), c.stream));
    DvcArgs a;
    std::memset(&a, 0, sizeof(a));
    a.dim = dim;
    a.nx = c.dvc_res[0];
    a.ny = c.dvc_res[1];
    a.nz = dim == 3 ? c.dvc_res[2] : 1;
    a.nc = (int)nc;
    const int n3[3] = {a.nx, a.ny, a.nz};
    for (int d = 0; d < 3; ++d) {
        // _DVCWeights_ConstructGrid: h = (1 - (-1)) / res, centre = -1 - h/2, then + h per cell
        const double h = 2.0 / n3[d];
        a.h[d] = h;
        double x = -1.0 - h / 2.0;
        for (int i = 0; i < n3[d] && i < 32; ++i) {
            x = x + h;
            a.cen[d][i] = x;
        }
    }
    a.da = dim == 3 ? a.h[0] * a.h[1] * a.h[2] : a.h[0] * a.h[1];
    a.ne = m.ne;
    a.nslots = c.np;
    a.offsets = c.offsets.p;
    a.sxi = c.sxi.p;
    a.oxi = c.dvc_xi.p;
    a.ow = c.dvc_w.p;
    a.bnd = c.dvc_bnd.p;
    a.err = c.err_count.p;
    if (m.ne > 0 && c.np > 0) {
        LaunchScope ls(c, UWGPU_KERNEL_ASSEMBLY);
        int sms = 0;
        UWG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
        const int64_t want = (m.ne + kDvcWarps - 1) / kDvcWarps;
        const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 16));
        k_dvc<<<blocks, 32 * kDvcWarps, 0, c.stream>>>(a);
        note_work(c, UWGPU_KERNEL_ASSEMBLY, (double)c.np * (dim * 16.0 + 8.0 + 256.0), (double)c.np * nc * 4.0);
    }
    check_launch("k_dvc");
    uint32_t err = 0;
    UWG_CUDA(cudaMemcpyAsync(&err, c.err_count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    if (err) throw Error(UWGPU_ERR_NOT_CONVERGED, "DVC weights: region growth did not settle");
    *xi = c.dvc_xi.p;
    *w = c.dvc_w.p;
}

// the local coordinates ([slot][3] on the host) and weights the last assembly integrated with
void integration_points_download(Context& c, double* xi, double* w) {
    UWG_REQUIRE(c.assembled, UWGPU_ERR_STATE, "nothing assembled");
    const int dim = c.mesh.dim;
    const size_t N = (size_t)c.np;
    if (N == 0) return;
    const double* src = c.weights_kind == UWGPU_WEIGHTS_DVC ? c.dvc_xi.p : c.sxi.p;
    if (xi) {
        std::vector<double> tmp((size_t)dim * N);
        UWG_CUDA(cudaMemcpyAsync(tmp.data(), src, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        for (size_t s = 0; s < N; ++s)
            for (int d = 0; d < 3; ++d) xi[3 * s + d] = d < dim ? tmp[(size_t)d * N + s] : 0.0;
    }
    if (w) {
        if (c.weights_kind == UWGPU_WEIGHTS_DVC) {
            UWG_CUDA(cudaMemcpyAsync(w, c.dvc_w.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        } else {
            DArray<double> tw;
            tw.ensure(N);
            {
                LaunchScope ls(c, -1);
                k_const_weights<<<blocks_for(c.mesh.ne, 256), 256, 0, c.stream>>>(c.mesh.ne, dim, c.offsets.p, tw.p);
            }
            check_launch("k_const_weights");
            UWG_CUDA(cudaMemcpyAsync(w, tw.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            UWG_CUDA(cudaStreamSynchronize(c.stream));
        }
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    }
}

}  // namespace uwg
