// PCDVC population control of the material points (PICellerator/Utils/src/PCDVC.c): points whose
// discrete Voronoi region is large are split, points whose region is small are deleted, element
// by element, then the element's Voronoi weights are recomputed.
//
// Reference behaviour (non-inflow branch of _PCDVC_Calculate3D, :638-1060, and _PCDVC_Calculate2D):
//   for each element in index order, with its points in cell-table order:
//   - DVC weights and centroids of the points;
//   - interface cell: its points' materials differ; boundary cell: it touches the mesh boundary;
//   - split candidates: w > upperT % of the element's local volume, in cell order; delete
//     candidates: w < lowerT %, sorted by swarm index, largest first (compare_indexOnCPU, :621);
//     interface cells delete nothing unless deleteInInterfaceCells, and split nothing unless
//     splitInInterfaceCells or a boundary cell; maxDeletions > count - 4 becomes count / 2;
//   - a split appends a copy of the point to the swarm and the cell, at the centroid of the
//     point's region (splitIntParticleByIndexWithinCell, :556-619);
//   - a deletion takes the point out of its cell by moving the cell's last entry into its place
//     (Swarm_RemoveParticleFromCell, StgDomain/Swarm/src/SwarmClass.c:1055-1071) and fills its
//     swarm slot with the swarm's last point, whose cell entry is renumbered
//     (deleteIntParticleByIndexOnCPU, :451-555);
//   - after any change the element's DVC runs again in the new cell order.
// So the swarm order after the pass is a sequential function of every earlier element's edits.
//
// GPU design.  The Voronoi regions of all elements (k_dvc, weights.cu) and the per-element
// decisions' inputs (flags, candidate lists with their centroids) are computed in parallel on the
// device; only the candidates travel to the host, where the swarm edits are replayed in element
// order on an identity map of the points (point identities, their current swarm index, the cell
// tables of the elements that change).  The result (the swarm order as identities, the changed
// elements' cell tables, the new points' sources and centroids) returns to the device, where one
// gather rebuilds the point arrays and one pass the integration slots (perm, offsets, local
// coordinates, material, optional per-point inputs).  The next DVC evaluation (the assembly's)
// then runs in the new cell order, as the reference's second DVC pass does.
#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "internal.cuh"

namespace uwg {

namespace {

struct PcMesh {
    int dim;
    int nel[3];
    double min[3], max[3];
};

// per element: bit0 interface cell, bit1 boundary cell; split and delete candidate counts
__global__ void k_pc_flags(int64_t ne, PcMesh mp, const uint32_t* __restrict__ offsets, const int32_t* __restrict__ smat,
                           const double* __restrict__ w, double maxW, double minW, uint32_t* __restrict__ flags,
                           uint32_t* __restrict__ nsplit, uint32_t* __restrict__ ndel) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const uint32_t beg = offsets[e], end = offsets[e + 1];
    uint32_t f = 0, ns = 0, nd = 0;
    for (uint32_t s = beg; s < end; ++s) {
        if (smat[s] != smat[beg]) f |= 1u;
        if (w[s] > maxW) ++ns;
        if (w[s] < minW) ++nd;
    }
    const int64_t ei[3] = {e % mp.nel[0], (e / mp.nel[0]) % mp.nel[1],
                           mp.dim == 3 ? e / ((int64_t)mp.nel[0] * mp.nel[1]) : 0};
    for (int d = 0; d < mp.dim; ++d)
        if (ei[d] == 0 || ei[d] == mp.nel[d] - 1) f |= 2u;
    flags[e] = f;
    nsplit[e] = ns;
    ndel[e] = nd;
}

// candidate records of element e at its offsets: split (cell position, centroid), delete (cell
// position, point index)
__global__ void k_pc_collect(int64_t ne, int dim, int64_t nslots, const uint32_t* __restrict__ offsets,
                             const uint32_t* __restrict__ perm, const double* __restrict__ w,
                             const double* __restrict__ cxi, double maxW, double minW,
                             const uint32_t* __restrict__ soff, const uint32_t* __restrict__ doff,
                             uint32_t* __restrict__ spos, double* __restrict__ sxi3, uint32_t* __restrict__ dpos,
                             uint32_t* __restrict__ dpoint) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const uint32_t beg = offsets[e], end = offsets[e + 1];
    uint32_t so = soff[e], dof = doff[e];
    for (uint32_t s = beg; s < end; ++s) {
        if (w[s] > maxW) {
            spos[so] = s - beg;
            for (int d = 0; d < 3; ++d) sxi3[3 * (int64_t)so + d] = d < dim ? cxi[(int64_t)d * nslots + s] : 0.0;
            ++so;
        }
        if (w[s] < minW) {
            dpos[dof] = s - beg;
            dpoint[dof] = perm[s];
            ++dof;
        }
    }
}

// new point k: identity who[k]; identities below n0 are old points, the others new points with
// source point src_of_new[id - n0] at the global position xyz_new[id - n0]
__global__ void k_pc_gather(int64_t n, int64_t n0, const uint32_t* __restrict__ who, const uint32_t* __restrict__ new_src,
                            const double* __restrict__ new_xyz, const double* __restrict__ ox,
                            const double* __restrict__ oy, const double* __restrict__ oz, const int32_t* __restrict__ om,
                            const double* __restrict__ oeta, const double* __restrict__ orho,
                            const double* __restrict__ opfw, double* __restrict__ x, double* __restrict__ y,
                            double* __restrict__ z, int32_t* __restrict__ mat, double* __restrict__ eta,
                            double* __restrict__ rho, double* __restrict__ pfw) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t id = who[k];
    uint32_t srcp;
    if (id < n0) {
        srcp = id;
        x[k] = ox[id];
        y[k] = oy[id];
        if (z) z[k] = oz[id];
    } else {
        const int64_t j = id - n0;
        srcp = new_src[j];
        x[k] = new_xyz[3 * j];
        y[k] = new_xyz[3 * j + 1];
        if (z) z[k] = new_xyz[3 * j + 2];
    }
    mat[k] = om[srcp];
    if (eta) eta[k] = oeta[srcp];
    if (rho) rho[k] = orho[srcp];
    if (pfw) pfw[k] = opfw[srcp];
}

// the slots of the new cell tables: perm, owning element per point, local coordinates (closed
// form on the affine element; a split point keeps the centroid it was placed at), material and
// the optional per-point inputs
template <int DIM>
__global__ void k_pc_slots(int64_t ne, int64_t nslots, PcMesh mp, const uint32_t* __restrict__ offsets,
                           const uint32_t* __restrict__ perm, const uint32_t* __restrict__ who, int64_t n0,
                           const double* __restrict__ new_xi, const double* __restrict__ px,
                           const double* __restrict__ py, const double* __restrict__ pz,
                           const int32_t* __restrict__ pmat, const double* __restrict__ peta,
                           const double* __restrict__ prho, double* __restrict__ sxi, int32_t* __restrict__ smat,
                           double* __restrict__ seta, double* __restrict__ srho, uint32_t* __restrict__ cell) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int64_t idx[3] = {e % mp.nel[0], (e / mp.nel[0]) % mp.nel[1], DIM == 3 ? e / ((int64_t)mp.nel[0] * mp.nel[1]) : 0};
    for (uint32_t s = offsets[e]; s < offsets[e + 1]; ++s) {
        const uint32_t p = perm[s];
        cell[p] = (uint32_t)e;
        const uint32_t id = who[p];
        const double x[3] = {px[p], py[p], DIM == 3 ? pz[p] : 0.0};
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            double v;
            if (id >= n0) {
                v = new_xi[3 * (int64_t)(id - n0) + d];
            } else {
                const double x0 = node_coord_1d(idx[d], mp.nel[d], mp.min[d], mp.max[d]);
                const double h = node_coord_1d(idx[d] + 1, mp.nel[d], mp.min[d], mp.max[d]) - x0;
                v = (2.0 * (x[d] - x0) - h) / h;
            }
            sxi[(int64_t)d * nslots + s] = v;
        }
        smat[s] = pmat[p];
        if (seta) seta[s] = peta[p];
        if (srho) srho[s] = prho[p];
    }
}

}  // namespace

// FeMesh_CoordLocalToGlobal of local coordinate xi in element e: sum over the nodes of N_a x_a
static void local_to_global(const MeshDesc& m, int64_t e, const double* xi, double* xg) {
    const int dim = m.dim, nen = dim == 3 ? 8 : 4;
    const int64_t ei[3] = {e % m.nel[0], (e / m.nel[0]) % m.nel[1], dim == 3 ? e / ((int64_t)m.nel[0] * m.nel[1]) : 0};
    for (int d = 0; d < 3; ++d) xg[d] = 0.0;
    for (int a = 0; a < nen; ++a) {
        double N = dim == 3 ? 0.125 : 0.25;
        for (int d = 0; d < dim; ++d) N *= ((a >> d) & 1) ? (1.0 + xi[d]) : (1.0 - xi[d]);
        for (int d = 0; d < dim; ++d) {
            const int64_t i = ei[d] + ((a >> d) & 1);
            xg[d] += N * node_coord_1d(i, m.nel[d], m.min[d], m.max[d]);
        }
    }
}

int64_t population_control(Context& c, const uwgpu_pcdvc_opts& o) {
    UWG_REQUIRE(c.mapped, UWGPU_ERR_STATE, "population control requested before bin_and_map");
    UWG_REQUIRE(c.weights_kind == UWGPU_WEIGHTS_DVC, UWGPU_ERR_STATE,
                "population control needs DVC weights (uwgpu_weights_set with UWGPU_WEIGHTS_DVC)");
    UWG_REQUIRE(o.max_deletions >= 0 && o.max_splits >= 0 && o.upper_t >= 0.0 && o.lower_t >= 0.0, UWGPU_ERR_ARGUMENT,
                "bad population-control options");
    const MeshDesc& m = c.mesh;
    const int dim = m.dim;
    const int64_t ne = m.ne, n0 = c.np;
    const double vol = dim == 3 ? 8.0 : 4.0;
    const double maxW = o.upper_t * vol / 100.0, minW = o.lower_t * vol / 100.0;
    PcMesh mp;
    mp.dim = dim;
    for (int d = 0; d < 3; ++d) {
        mp.nel[d] = m.nel[d];
        mp.min[d] = m.min[d];
        mp.max[d] = m.max[d];
    }
    // 1. Voronoi regions of the current cell tables
    const double *cxi = nullptr, *w = nullptr;
    integration_points(c, &cxi, &w);
    // 2. flags and candidate counts per element, then the candidates themselves
    DArray<uint32_t> flags, nsp, ndl, soff, doff;
    for (auto* a : {&flags, &nsp, &ndl, &soff, &doff}) a->ensure((size_t)ne);
    {
        LaunchScope ls(c, -1);
        k_pc_flags<<<blocks_for(ne, 256), 256, 0, c.stream>>>(ne, mp, c.offsets.p, c.smat.p, w, maxW, minW, flags.p, nsp.p,
                                                             ndl.p);
    }
    check_launch("k_pc_flags");
    std::vector<uint32_t> hflags((size_t)ne), hns((size_t)ne), hnd((size_t)ne), hoff((size_t)ne + 1);
    UWG_CUDA(cudaMemcpyAsync(hflags.data(), flags.p, ne * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaMemcpyAsync(hns.data(), nsp.p, ne * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaMemcpyAsync(hnd.data(), ndl.p, ne * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaMemcpyAsync(hoff.data(), c.offsets.p, (ne + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<uint32_t> hso((size_t)ne), hdo((size_t)ne);
    uint64_t ts = 0, td = 0;
    for (int64_t e = 0; e < ne; ++e) {
        hso[e] = (uint32_t)ts;
        hdo[e] = (uint32_t)td;
        ts += hns[e];
        td += hnd[e];
        UWG_REQUIRE(hoff[e + 1] > hoff[e], UWGPU_ERR_ARGUMENT, "population control: an element holds no points");
    }
    DArray<uint32_t> spos, dpos, dpoint;
    DArray<double> sxi3;
    spos.ensure(ts ? ts : 1);
    sxi3.ensure(3 * (ts ? ts : 1));
    dpos.ensure(td ? td : 1);
    dpoint.ensure(td ? td : 1);
    UWG_CUDA(cudaMemcpyAsync(soff.p, hso.data(), ne * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
    UWG_CUDA(cudaMemcpyAsync(doff.p, hdo.data(), ne * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
    {
        LaunchScope ls(c, -1);
        k_pc_collect<<<blocks_for(ne, 256), 256, 0, c.stream>>>(ne, dim, c.np, c.offsets.p, c.perm.p, w, cxi, maxW, minW,
                                                               soff.p, doff.p, spos.p, sxi3.p, dpos.p, dpoint.p);
    }
    check_launch("k_pc_collect");
    std::vector<uint32_t> hspos(ts), hdpos(td), hdpoint(td);
    std::vector<double> hsxi(3 * ts);
    if (ts) {
        UWG_CUDA(cudaMemcpyAsync(hspos.data(), spos.p, ts * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaMemcpyAsync(hsxi.data(), sxi3.p, 3 * ts * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    }
    if (td) {
        UWG_CUDA(cudaMemcpyAsync(hdpos.data(), dpos.p, td * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaMemcpyAsync(hdpoint.data(), dpoint.p, td * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    }
    UWG_CUDA(cudaStreamSynchronize(c.stream));

    // 3. the swarm edits, replayed in element order.  Identities: old points keep their index as
    // identity, new points get n0, n0 + 1, ...  who / where map swarm index <-> identity for the
    // entries that changed; tables hold identities, in cell order, for the elements that change.
    std::unordered_map<uint32_t, uint32_t> who, where;   // absent: identity == index
    auto who_of = [&](uint32_t k) { auto it = who.find(k); return it == who.end() ? k : it->second; };
    auto where_of = [&](uint32_t id) { auto it = where.find(id); return it == where.end() ? id : it->second; };
    auto set_who = [&](uint32_t k, uint32_t id) {
        if (k == id) who.erase(k);
        else who[k] = id;
    };
    auto set_where = [&](uint32_t id, uint32_t k) {
        if (k == id) where.erase(id);
        else where[id] = k;
    };
    std::unordered_map<int64_t, std::vector<uint32_t>> tables;   // element -> identities in cell order
    auto table_of = [&](int64_t e) -> std::vector<uint32_t>& {
        auto it = tables.find(e);
        if (it != tables.end()) return it->second;
        std::vector<uint32_t>& t = tables[e];
        const uint32_t b = hoff[e], n = hoff[e + 1] - b;
        t.resize(n);
        UWG_CUDA(cudaMemcpy(t.data(), c.perm.p + b, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        return t;   // identities = the indices before the pass
    };
    std::vector<uint32_t> new_src;    // per new identity: the old point it copies
    std::vector<double> new_xi, new_xyz;
    int64_t count = n0;
    uint32_t next_id = (uint32_t)n0;
    for (int64_t e = 0; e < ne; ++e) {
        if (hns[e] == 0 && hnd[e] == 0) continue;
        const int64_t nump = hoff[e + 1] - hoff[e];
        const bool interface = hflags[e] & 1u, boundary = hflags[e] & 2u;
        int maxDel = o.max_deletions, maxSpl = o.max_splits;
        if (interface) {
            if (!o.delete_in_interface_cells) maxDel = 0;
            if (!o.split_in_interface_cells && !boundary) maxSpl = 0;
        }
        if (maxDel > nump - 4) maxDel = (int)(nump / 2);
        const int64_t nsplit = std::min<int64_t>(maxSpl, hns[e]);
        const int64_t ndel = std::min<int64_t>(maxDel, hnd[e]);
        if (nsplit == 0 && ndel == 0) continue;
        std::vector<uint32_t>& t = table_of(e);
        // delete list: the candidates' current swarm indices, largest first
        std::vector<uint32_t> dels;
        for (uint32_t k = 0; k < hnd[e]; ++k) dels.push_back(where_of(hdpoint[hdo[e] + k]));
        std::sort(dels.begin(), dels.end(), [](uint32_t a, uint32_t b) { return a > b; });
        for (int64_t k = 0; k < nsplit; ++k) {
            const uint32_t at = hspos[hso[e] + k];
            const uint32_t from = t[at];
            const uint32_t id = next_id++;
            const uint32_t idx = (uint32_t)count++;
            set_who(idx, id);
            set_where(id, idx);
            // an old point's source is itself; a new point copies its source's source
            new_src.push_back(from < n0 ? from : new_src[from - n0]);
            const double* xi3 = &hsxi[3 * (size_t)(hso[e] + k)];
            double xg[3];
            local_to_global(m, e, xi3, xg);
            for (int d = 0; d < 3; ++d) {
                new_xi.push_back(xi3[d]);
                new_xyz.push_back(xg[d]);
            }
            t.push_back(id);
        }
        for (int64_t k = 0; k < ndel; ++k) {
            const uint32_t P = dels[k];
            const uint32_t pid = who_of(P);
            // out of its cell: the cell's last entry takes its place
            auto pos = std::find(t.begin(), t.end(), pid);
            UWG_REQUIRE(pos != t.end(), UWGPU_ERR_STATE, "population control: delete candidate not in its cell");
            *pos = t.back();
            t.pop_back();
            // the swarm's last point fills the slot; its cell entry follows it (tables hold
            // identities, so only the index maps change)
            const uint32_t L = (uint32_t)(count - 1);
            if (P != L) {
                const uint32_t lid = who_of(L);
                set_who(P, lid);
                set_where(lid, P);
            }
            who.erase(L);
            where.erase(pid);
            count--;
        }
    }
    UWG_REQUIRE(count < (int64_t)0xffffffffLL, UWGPU_ERR_TOO_LARGE, "population control: too many points");
    const int64_t nnew = (int64_t)new_src.size();

    // 4. rebuild on the device: the swarm order (identity of every index), the points, the slots
    std::vector<uint32_t> hwho((size_t)count);
    for (int64_t k = 0; k < count; ++k) hwho[k] = who_of((uint32_t)k);
    std::vector<uint32_t> hcnt((size_t)ne);
    for (int64_t e = 0; e < ne; ++e) hcnt[e] = hoff[e + 1] - hoff[e];
    for (auto& kv : tables) hcnt[kv.first] = (uint32_t)kv.second.size();
    std::vector<uint32_t> noff((size_t)ne + 1);
    noff[0] = 0;
    for (int64_t e = 0; e < ne; ++e) noff[e + 1] = noff[e] + hcnt[e];
    UWG_REQUIRE((int64_t)noff[ne] == count, UWGPU_ERR_STATE, "population control: cell tables and swarm disagree");
    // new perm: unchanged elements keep their cell order (indices renumbered through where);
    // changed elements take their replayed tables
    std::vector<uint32_t> oldperm((size_t)n0);
    UWG_CUDA(cudaMemcpy(oldperm.data(), c.perm.p, n0 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> hperm((size_t)count);
    for (int64_t e = 0; e < ne; ++e) {
        auto it = tables.find(e);
        uint32_t s = noff[e];
        if (it == tables.end()) {
            for (uint32_t q = hoff[e]; q < hoff[e + 1]; ++q) hperm[s++] = where_of(oldperm[q]);
        } else {
            for (uint32_t id : it->second) hperm[s++] = where_of(id);
        }
    }
    const size_t N = (size_t)count;
    DArray<uint32_t> dwho, dsrc;
    DArray<double> dxyz, dxi;
    dwho.ensure(N);
    dsrc.ensure(nnew ? nnew : 1);
    dxyz.ensure(3 * (nnew ? nnew : 1));
    dxi.ensure(3 * (nnew ? nnew : 1));
    UWG_CUDA(cudaMemcpyAsync(dwho.p, hwho.data(), N * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
    if (nnew) {
        UWG_CUDA(cudaMemcpyAsync(dsrc.p, new_src.data(), nnew * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
        UWG_CUDA(cudaMemcpyAsync(dxyz.p, new_xyz.data(), 3 * nnew * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        UWG_CUDA(cudaMemcpyAsync(dxi.p, new_xi.data(), 3 * nnew * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    }
    DArray<double> nx, ny, nz, neta, nrho, npfw;
    DArray<int32_t> nmat;
    nx.ensure(N);
    ny.ensure(N);
    if (dim == 3) nz.ensure(N);
    nmat.ensure(N);
    if (c.has_peta) neta.ensure(N);
    if (c.has_prho) nrho.ensure(N);
    if (c.has_pfw) npfw.ensure(N);
    {
        LaunchScope ls(c, -1);
        k_pc_gather<<<blocks_for(count, 256), 256, 0, c.stream>>>(
            count, n0, dwho.p, dsrc.p, dxyz.p, c.px.p, c.py.p, dim == 3 ? c.pz.p : nullptr, c.pmat.p,
            c.has_peta ? c.peta.p : nullptr, c.has_prho ? c.prho.p : nullptr, c.has_pfw ? c.pfw.p : nullptr, nx.p, ny.p,
            dim == 3 ? nz.p : nullptr, nmat.p, c.has_peta ? neta.p : nullptr, c.has_prho ? nrho.p : nullptr,
            c.has_pfw ? npfw.p : nullptr);
    }
    check_launch("k_pc_gather");
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    c.px.swap(nx);
    c.py.swap(ny);
    if (dim == 3) {
        c.pz.swap(nz);
    }
    c.pmat.swap(nmat);
    if (c.has_peta) {
        c.peta.swap(neta);
    }
    if (c.has_prho) {
        c.prho.swap(nrho);
    }
    if (c.has_pfw) {
        c.pfw.swap(npfw);
        c.pfw_incr.ensure(N);
        UWG_CUDA(cudaMemsetAsync(c.pfw_incr.p, 0, N * sizeof(double), c.stream));
    }
    c.np = count;
    c.offsets.ensure((size_t)ne + 1);
    c.perm.ensure(N);
    c.cell.ensure(N);
    c.sxi.ensure((size_t)dim * N);
    c.smat.ensure(N);
    c.seta_out.ensure(N);
    if (c.has_peta) c.seta_in.ensure(N);
    if (c.has_prho) c.srho_in.ensure(N);
    c.tmp_perm.ensure(N);
    UWG_CUDA(cudaMemcpyAsync(c.offsets.p, noff.data(), (ne + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
    UWG_CUDA(cudaMemcpyAsync(c.perm.p, hperm.data(), N * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
    {
        LaunchScope ls(c, -1);
        if (dim == 3)
            k_pc_slots<3><<<blocks_for(ne, 128), 128, 0, c.stream>>>(
                ne, count, mp, c.offsets.p, c.perm.p, dwho.p, n0, dxi.p, c.px.p, c.py.p, c.pz.p, c.pmat.p,
                c.has_peta ? c.peta.p : nullptr, c.has_prho ? c.prho.p : nullptr, c.sxi.p, c.smat.p,
                c.has_peta ? c.seta_in.p : nullptr, c.has_prho ? c.srho_in.p : nullptr, c.cell.p);
        else
            k_pc_slots<2><<<blocks_for(ne, 128), 128, 0, c.stream>>>(
                ne, count, mp, c.offsets.p, c.perm.p, dwho.p, n0, dxi.p, c.px.p, c.py.p, nullptr, c.pmat.p,
                c.has_peta ? c.peta.p : nullptr, c.has_prho ? c.prho.p : nullptr, c.sxi.p, c.smat.p,
                c.has_peta ? c.seta_in.p : nullptr, c.has_prho ? c.srho_in.p : nullptr, c.cell.p);
    }
    check_launch("k_pc_slots");
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    c.mapped = true;
    c.assembled = false;
    c.operator_built = false;
    return count;
}

}  // namespace uwg
