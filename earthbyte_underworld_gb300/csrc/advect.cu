// Material-point advection on the device: the SwarmAdvector time integration of the particle
// coordinates with the current velocity solution.
//
// Reference (paths relative to the Underworld 1.x tree):
//   time derivative   PICellerator/MaterialPoints/src/SwarmAdvector.c:288-314: the velocity
//                     interpolated at the point (FieldVariable_InterpolateValueAt ->
//                     StgFEM/Discretisation/src/FeVariable.c:773-800); a point outside the mesh
//                     has no velocity
//   first order       StgDomain/Utils/src/TimeIntegrand.c:221-265: x = x0 + dt v(x0)
//   second order      TimeIntegrand.c:267-337: predictor x0 + dt/2 v(x0), corrector
//                     x0 + dt v(predictor); a predictor outside the mesh falls back to the
//                     first-order update when allowFallbackToFirstOrder is set, else stops
//   ownership         SwarmAdvector_AdvectionFinish -> Swarm_UpdateAllParticleOwners
//                     (SwarmAdvector.c:375-382): here the next uwgpu_bin_and_map
//
// Points are independent (the reference keeps each point's start value before its predictor),
// so the update is one thread per point: element search with the mapper's tie rules, the closed
// form local coordinate of the affine element, Q1 shape functions on the SoA nodal velocity.
// All points are written to a second coordinate set, which replaces the first only when every
// point succeeded, so a failed step leaves the swarm as it was.
#include <cmath>
#include <string>
#include <utility>

#include "internal.cuh"

namespace uwg {

namespace {

struct AdvMesh {
    int nel[3];
    double min[3], max[3];
    int64_t nnx, nny, nn;
};

__device__ __forceinline__ bool num_approx_adv(double var, double val) {
    const double eps = 1e-12;   // Num_Approx, StGermain/Base/Foundation/src/Numerics.c:37-41
    return var >= val - eps && var <= val + eps;
}

// element index along one axis (Mesh_RegularAlgorithms.c:194-226 rules); false when outside
__device__ __forceinline__ bool axis_element(double x, int nel, double mn, double mx, int64_t& idx) {
    if (!isfinite(x)) return false;
    if (num_approx_adv(x - mx, 0.0)) {
        idx = nel - 1;
        return true;
    }
    if (x < mn || x > mx) return false;
    const double out = __ddiv_rn(x - mn, (mx - mn) / nel);
    const double integer = trunc(out);
    int64_t i = (int64_t)integer;
    if (i > 0 && num_approx_adv(out - integer, 0.0)) i--;
    if (i >= nel) i = nel - 1;
    idx = i;
    return true;
}

// velocity at point x: Q1 interpolation of the SoA nodal velocity u[d][node]
template <int DIM>
__device__ __forceinline__ bool velocity_at(const AdvMesh& m, const double* __restrict__ u, const double x[3],
                                            double v[3]) {
    int64_t ie[3] = {0, 0, 0};
    double xi[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        if (!axis_element(x[d], m.nel[d], m.min[d], m.max[d], ie[d])) return false;
        const double x0 = node_coord_1d(ie[d], m.nel[d], m.min[d], m.max[d]);
        const double x1 = node_coord_1d(ie[d] + 1, m.nel[d], m.min[d], m.max[d]);
        const double h = x1 - x0;
        xi[d] = (2.0 * (x[d] - x0) - h) / h;
    }
    const int64_t base = ie[0] + m.nnx * (ie[1] + m.nny * ie[2]);
#pragma unroll
    for (int d = 0; d < DIM; ++d) v[d] = 0.0;
#pragma unroll
    for (int a = 0; a < (1 << DIM); ++a) {
        double N = 1.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) N *= 0.5 * (1.0 + (((a >> d) & 1) ? xi[d] : -xi[d]));
        const int64_t node = base + (a & 1) + ((a >> 1) & 1) * m.nnx + (DIM == 3 ? ((a >> 2) & 1) * m.nnx * m.nny : 0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) v[d] = fma(N, u[(int64_t)d * m.nn + node], v[d]);
    }
    return true;
}

// counters: [0] points without a velocity (start or, without fallback, predictor outside the
// mesh), [1] first-order fallbacks, [2] points that end outside the mesh
template <int DIM>
__global__ void k_advect(int64_t np, AdvMesh m, const double* __restrict__ u, double dt, int order, int fallback,
                         const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz,
                         double* __restrict__ qx, double* __restrict__ qy, double* __restrict__ qz,
                         uint32_t* __restrict__ counters) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const double x0[3] = {px[p], py[p], DIM == 3 ? pz[p] : 0.0};
    double v0[3] = {0, 0, 0}, v1[3] = {0, 0, 0}, x1[3] = {x0[0], x0[1], x0[2]};
    bool ok = velocity_at<DIM>(m, u, x0, v0);
    if (ok) {
        if (order == 1) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) x1[d] = x0[d] + dt * v0[d];
        } else {
            double xm[3] = {x0[0], x0[1], x0[2]};
#pragma unroll
            for (int d = 0; d < DIM; ++d) xm[d] = x0[d] + 0.5 * dt * v0[d];
            if (velocity_at<DIM>(m, u, xm, v1)) {
#pragma unroll
                for (int d = 0; d < DIM; ++d) x1[d] = x0[d] + dt * v1[d];
            } else if (fallback) {
#pragma unroll
                for (int d = 0; d < DIM; ++d) x1[d] = x0[d] + dt * v0[d];
                atomicAdd(&counters[1], 1u);
            } else {
                ok = false;
            }
        }
    }
    if (!ok) {
        atomicAdd(&counters[0], 1u);
    } else {
        int64_t dummy;
        bool inside = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) inside = inside && axis_element(x1[d], m.nel[d], m.min[d], m.max[d], dummy);
        if (!inside) atomicAdd(&counters[2], 1u);
    }
    qx[p] = x1[0];
    qy[p] = x1[1];
    if (DIM == 3) qz[p] = x1[2];
}

}  // namespace

void advect_particles(Context& c, double dt, int order, bool fallback, uint32_t& fell_back, uint32_t& left_mesh) {
    UWG_REQUIRE(c.has_points, UWGPU_ERR_STATE, "advection requested before particles_upload");
    UWG_REQUIRE(c.has_solution, UWGPU_ERR_STATE, "advection requested before a velocity solution");
    UWG_REQUIRE(order == 1 || order == 2, UWGPU_ERR_ARGUMENT, "advection order must be 1 or 2");
    UWG_REQUIRE(std::isfinite(dt), UWGPU_ERR_ARGUMENT, "dt must be finite");
    const MeshDesc& md = c.mesh;
    AdvMesh m;
    for (int d = 0; d < 3; ++d) {
        m.nel[d] = md.nel[d];
        m.min[d] = md.min[d];
        m.max[d] = md.max[d];
    }
    m.nnx = md.nnx;
    m.nny = md.nny;
    m.nn = md.nn;
    const int64_t np = c.np;
    c.qx.ensure((size_t)(np > 0 ? np : 1));
    c.qy.ensure((size_t)(np > 0 ? np : 1));
    if (md.dim == 3) c.qz.ensure((size_t)(np > 0 ? np : 1));
    c.err_count.ensure(4);
    UWG_CUDA(cudaMemsetAsync(c.err_count.p, 0, 4 * sizeof(uint32_t), c.stream));
    if (np > 0) {
        LaunchScope ls(c, UWGPU_KERNEL_BINNING);
        if (md.dim == 3)
            k_advect<3><<<blocks_for(np, 256), 256, 0, c.stream>>>(np, m, c.u_sol.p, dt, order, fallback ? 1 : 0, c.px.p,
                                                                   c.py.p, c.pz.p, c.qx.p, c.qy.p, c.qz.p, c.err_count.p);
        else
            k_advect<2><<<blocks_for(np, 256), 256, 0, c.stream>>>(np, m, c.u_sol.p, dt, order, fallback ? 1 : 0, c.px.p,
                                                                   c.py.p, nullptr, c.qx.p, c.qy.p, nullptr, c.err_count.p);
        note_work(c, UWGPU_KERNEL_BINNING, (double)np * md.dim * 16.0, (double)np * 80.0);
    }
    check_launch("k_advect");
    uint32_t counters[4] = {0, 0, 0, 0};
    UWG_CUDA(cudaMemcpyAsync(counters, c.err_count.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    if (counters[0] > 0)
        throw Error(UWGPU_ERR_DOMAIN, std::to_string(counters[0]) +
                                          " material points have no velocity (outside the mesh); the swarm is unchanged");
    c.px.swap(c.qx);
    c.py.swap(c.qy);
    if (md.dim == 3) {
        c.pz.swap(c.qz);
    }
    c.mapped = false;   // ownership changes: the next bin_and_map rebuilds the cell tables
    fell_back = counters[1];
    left_mesh = counters[2];
}

}  // namespace uwg
