// Material point -> element binning and the integration-point mapper.
//
// Reference behaviour (paths relative to the Underworld 1.x tree):
//   element search   StgDomain/Mesh/src/Mesh_RegularAlgorithms.c:194-226 (sep from :154-175,
//                    Num_Approx epsilon 1e-12 from StGermain/Base/Foundation/src/Numerics.c:37-41)
//   cell tables      PICellerator/MaterialPoints/src/CoincidentMapper.c:176-242 appends points in
//                    ascending index order (StgDomain/Swarm/src/SwarmClass.c:1155-1184)
//   local coords     StgFEM/Discretisation/src/ElementType.c:227-350 (Newton; on the affine
//                    elements of a regular mesh it reproduces the closed form used here)
//
// GPU design: counting sort with integer atomics on HBM-resident counts, an exclusive scan,
// an unordered scatter, then one warp per element ranks its points by index so the final
// permutation equals the reference's append order exactly.  The same warp computes xi and
// gathers the per-point inputs into slot order (SoA), so assembly reads them coalesced.
#include "internal.cuh"

namespace uwg {

struct MeshParams {
    int dim;
    int nel[3];
    double min[3];
    double max[3];
};

static MeshParams params_of(const MeshDesc& m) {
    MeshParams p;
    p.dim = m.dim;
    for (int d = 0; d < 3; ++d) {
        p.nel[d] = m.nel[d];
        p.min[d] = m.min[d];
        p.max[d] = m.max[d];
    }
    return p;
}

__device__ __forceinline__ bool num_approx(double var, double val) {
    const double eps = 1e-12;
    return var >= val - eps && var <= val + eps;
}

template <int DIM>
__global__ void k_locate(int64_t np, const double* __restrict__ px, const double* __restrict__ py,
                         const double* __restrict__ pz, MeshParams mp, uint32_t* __restrict__ cell,
                         uint32_t* __restrict__ counts, uint32_t* __restrict__ err) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double pt[3];
    pt[0] = px[p];
    pt[1] = py[p];
    pt[2] = DIM == 3 ? pz[p] : 0.0;
    unsigned inds[3] = {0u, 0u, 0u};
    bool ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double sep = (mp.max[d] - mp.min[d]) / mp.nel[d];
        if (!isfinite(pt[d])) {
            ok = false;
        } else if (num_approx(pt[d] - mp.max[d], 0.0)) {
            inds[d] = (unsigned)(mp.nel[d] - 1);
        } else if (pt[d] < mp.min[d] || pt[d] > mp.max[d]) {
            ok = false;
        } else {
            double out = __ddiv_rn(pt[d] - mp.min[d], sep);
            double integer = trunc(out);
            double frac = out - integer;  // exact: modf of a non-negative value
            unsigned i = (unsigned)integer;
            if (i > 0 && num_approx(frac, 0.0)) i--;
            // a value that rounds onto the upper face is still inside the last element
            if (i >= (unsigned)mp.nel[d]) i = (unsigned)mp.nel[d] - 1;
            inds[d] = i;
        }
    }
    if (!ok) {
        cell[p] = 0xffffffffu;
        atomicAdd(err, 1u);
        return;
    }
    unsigned e = inds[0] + (unsigned)mp.nel[0] * (inds[1] + (unsigned)mp.nel[1] * inds[2]);
    cell[p] = e;
    atomicAdd(&counts[e], 1u);
}

// ---- exclusive scan of u32 counts: out[0..n] with out[n] = total ----
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem_warp, uint32_t& total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? smem_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) smem_warp[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = warp ? smem_warp[warp - 1] : 0u;
    total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void k_scan_tiles(int64_t n, const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                             uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t sw[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? in[base + i] : 0u;
        s += v[i];
    }
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, sw, total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = pre;
        pre += v[i];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Single block: exclusive scan of the tile sums in chunks, carrying the running total.
__global__ void k_scan_tile_sums(int64_t ntiles, uint32_t* __restrict__ tile_sums, uint32_t* __restrict__ grand) {
    __shared__ uint32_t sw[32];
    uint32_t carry = 0;
    for (int64_t base = 0; base < ntiles; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        uint32_t v = i < ntiles ? tile_sums[i] : 0u;
        uint32_t total;
        uint32_t pre = block_exclusive_scan(v, sw, total);
        if (i < ntiles) tile_sums[i] = carry + pre;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void k_scan_add(int64_t n, uint32_t* __restrict__ out, const uint32_t* __restrict__ tile_sums) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_sums[i / kScanTile];
}

static void exclusive_scan(Context& c, const uint32_t* in, uint32_t* out, int64_t n) {
    int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles < 1) ntiles = 1;
    c.block_sums.ensure((size_t)ntiles);
    {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, c.stream>>>(n, in, out, c.block_sums.p);
    }
    check_launch("k_scan_tiles");
    {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        k_scan_tile_sums<<<1, 1024, 0, c.stream>>>(ntiles, c.block_sums.p, out + n);
    }
    check_launch("k_scan_tile_sums");
    {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        k_scan_add<<<blocks_for(n, 256), 256, 0, c.stream>>>(n, out, c.block_sums.p);
    }
    check_launch("k_scan_add");
}

__global__ void k_scatter(int64_t np, const uint32_t* __restrict__ cell, const uint32_t* __restrict__ offsets,
                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ tmp_perm) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    uint32_t e = cell[p];
    if (e == 0xffffffffu) return;
    uint32_t slot = offsets[e] + atomicAdd(&cursor[e], 1u);
    tmp_perm[slot] = (uint32_t)p;
}

template <int DIM>
__device__ __forceinline__ void map_point(int64_t e, uint32_t p, uint32_t slot, int64_t nslots, const MeshParams& mp,
                                          const double* __restrict__ px, const double* __restrict__ py,
                                          const double* __restrict__ pz, const int32_t* __restrict__ pmat,
                                          const double* __restrict__ peta, const double* __restrict__ prho,
                                          double* __restrict__ sxi, int32_t* __restrict__ smat,
                                          double* __restrict__ seta, double* __restrict__ srho) {
    int64_t ie = e % mp.nel[0];
    int64_t je = (e / mp.nel[0]) % mp.nel[1];
    int64_t ke = DIM == 3 ? e / ((int64_t)mp.nel[0] * mp.nel[1]) : 0;
    int64_t idx[3] = {ie, je, ke};
    double x[3] = {px[p], py[p], DIM == 3 ? pz[p] : 0.0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double x0 = node_coord_1d(idx[d], mp.nel[d], mp.min[d], mp.max[d]);
        double x1 = node_coord_1d(idx[d] + 1, mp.nel[d], mp.min[d], mp.max[d]);
        double h = x1 - x0;
        sxi[(int64_t)d * nslots + slot] = (2.0 * (x[d] - x0) - h) / h;
    }
    smat[slot] = pmat[p];
    if (seta) seta[slot] = peta[p];
    if (srho) srho[slot] = prho[p];
}

// One warp per element: rank the element's points by point index (the append order of the
// reference cell table), write the permutation, then map every point of the element.
template <int DIM>
__global__ void k_sort_map(int64_t ne, int64_t nslots, MeshParams mp, const uint32_t* __restrict__ offsets,
                           const uint32_t* __restrict__ tmp_perm, uint32_t* __restrict__ perm,
                           const double* __restrict__ px, const double* __restrict__ py,
                           const double* __restrict__ pz, const int32_t* __restrict__ pmat,
                           const double* __restrict__ peta, const double* __restrict__ prho,
                           double* __restrict__ sxi, int32_t* __restrict__ smat, double* __restrict__ seta,
                           double* __restrict__ srho) {
    int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (e >= ne) return;
    uint32_t beg = offsets[e], end = offsets[e + 1];
    uint32_t n = end - beg;
    if (n <= 32) {
        uint32_t v = lane < (int)n ? tmp_perm[beg + lane] : 0xffffffffu;
        int rank = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            uint32_t o = __shfl_sync(0xffffffffu, v, j);
            rank += (o < v) ? 1 : 0;
        }
        if (lane < (int)n) {
            perm[beg + rank] = v;
            map_point<DIM>(e, v, beg + rank, nslots, mp, px, py, pz, pmat, peta, prho, sxi, smat, seta, srho);
        }
    } else {
        for (uint32_t i = lane; i < n; i += 32) {
            uint32_t v = tmp_perm[beg + i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < n; ++j) rank += (tmp_perm[beg + j] < v) ? 1u : 0u;
            perm[beg + rank] = v;
            map_point<DIM>(e, v, beg + rank, nslots, mp, px, py, pz, pmat, peta, prho, sxi, smat, seta, srho);
        }
    }
}

void bin_and_map(Context& c) {
    UWG_REQUIRE(c.has_mesh, UWGPU_ERR_STATE, "mesh not set");
    UWG_REQUIRE(c.has_points, UWGPU_ERR_STATE, "material points not uploaded");
    const int64_t np = c.np, ne = c.mesh.ne;
    MeshParams mp = params_of(c.mesh);
    c.cell.ensure((size_t)np);
    c.counts.ensure((size_t)ne);
    c.cursor.ensure((size_t)ne);
    c.offsets.ensure((size_t)ne + 1);
    c.perm.ensure((size_t)np);
    c.tmp_perm.ensure((size_t)np);
    c.err_count.ensure(1);
    c.sxi.ensure((size_t)np * c.mesh.dim);
    c.smat.ensure((size_t)np);
    c.seta_out.ensure((size_t)np);
    if (c.has_peta) c.seta_in.ensure((size_t)np);
    if (c.has_prho) c.srho_in.ensure((size_t)np);
    UWG_CUDA(cudaMemsetAsync(c.counts.p, 0, ne * sizeof(uint32_t), c.stream));
    UWG_CUDA(cudaMemsetAsync(c.cursor.p, 0, ne * sizeof(uint32_t), c.stream));
    UWG_CUDA(cudaMemsetAsync(c.err_count.p, 0, sizeof(uint32_t), c.stream));
    {
        // algorithmic bytes of the whole binning pass: per point coordinates read twice (locate,
        // map), cell id written/read, count/cursor atomics, unordered and final permutation,
        // material in, xi and material out (+ optional per-point inputs); per element counts,
        // cursor and offsets
        int dim = c.mesh.dim;
        double extra = (c.has_peta ? 16.0 : 0.0) + (c.has_prho ? 16.0 : 0.0);
        double per_point = 2 * dim * 8.0 + 8.0 + 16.0 + 12.0 + 8.0 + dim * 8.0 + extra;
        note_work(c, UWGPU_KERNEL_BINNING, per_point * np + 20.0 * ne, 0.0);
    }
    if (np > 0) {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        if (c.mesh.dim == 3)
            k_locate<3><<<blocks_for(np, 256), 256, 0, c.stream>>>(np, c.px.p, c.py.p, c.pz.p, mp, c.cell.p, c.counts.p, c.err_count.p);
        else
            k_locate<2><<<blocks_for(np, 256), 256, 0, c.stream>>>(np, c.px.p, c.py.p, nullptr, mp, c.cell.p, c.counts.p, c.err_count.p);
    }
    check_launch("k_locate");
    exclusive_scan(c, c.counts.p, c.offsets.p, ne);
    if (np > 0) {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        k_scatter<<<blocks_for(np, 256), 256, 0, c.stream>>>(np, c.cell.p, c.offsets.p, c.cursor.p, c.tmp_perm.p);
    }
    check_launch("k_scatter");
    {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        unsigned blocks = blocks_for(ne * 32, 256);
        double* seta = c.has_peta ? c.seta_in.p : nullptr;
        double* srho = c.has_prho ? c.srho_in.p : nullptr;
        if (c.mesh.dim == 3)
            k_sort_map<3><<<blocks, 256, 0, c.stream>>>(ne, np, mp, c.offsets.p, c.tmp_perm.p, c.perm.p, c.px.p, c.py.p,
                                                       c.pz.p, c.pmat.p, c.peta.p, c.prho.p, c.sxi.p, c.smat.p, seta, srho);
        else
            k_sort_map<2><<<blocks, 256, 0, c.stream>>>(ne, np, mp, c.offsets.p, c.tmp_perm.p, c.perm.p, c.px.p, c.py.p,
                                                       nullptr, c.pmat.p, c.peta.p, c.prho.p, c.sxi.p, c.smat.p, seta, srho);
    }
    check_launch("k_sort_map");
    uint32_t outside = 0;
    UWG_CUDA(cudaMemcpyAsync(&outside, c.err_count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    c.mapped = true;
    c.assembled = false;
    if (outside)
        throw Error(UWGPU_ERR_DOMAIN, std::to_string(outside) + " material points lie outside the mesh");
}

}  // namespace uwg
