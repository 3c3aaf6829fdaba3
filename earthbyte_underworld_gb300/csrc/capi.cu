// extern "C" entry points of libuwgpu (declared in include/uwgpu.h).  Each converts the
// internal uwg::Error exceptions into a status code plus a message.
#include <cmath>
#include <cstring>

#include "internal.cuh"
#include "unet.cuh"

using uwg::Context;
using uwg::Error;

struct uwgpu_ctx {
    Context c;
};

namespace {

template <typename F>
int guarded(uwgpu_ctx* ctx, F&& fn) {
    if (!ctx) return UWGPU_ERR_ARGUMENT;
    // device arrays of this call come from the pool on the context's stream
    struct AllocStream {
        cudaStream_t saved;
        explicit AllocStream(cudaStream_t s) : saved(uwg::alloc_stream()) { uwg::alloc_stream() = s; }
        ~AllocStream() { uwg::alloc_stream() = saved; }
    } as(ctx->c.stream);
    try {
        cudaSetDevice(ctx->c.device);
        fn(ctx->c);
        ctx->c.last_error.clear();
        return UWGPU_OK;
    } catch (const Error& e) {
        ctx->c.last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        ctx->c.last_error = e.what();
        return UWGPU_ERR_CUDA;
    }
}

template <typename T>
void upload(uwg::DArray<T>& dst, const T* src, size_t n, cudaStream_t s) {
    dst.ensure(n);
    UWG_CUDA(cudaMemcpyAsync(dst.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
}

}  // namespace

extern "C" {

int uwgpu_abi_version(void) { return UWGPU_ABI_VERSION; }

int uwgpu_create(int32_t device, uwgpu_ctx** out) {
    if (!out) return UWGPU_ERR_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return UWGPU_ERR_CUDA;
    if (device < 0 || device >= ndev) return UWGPU_ERR_ARGUMENT;
    uwgpu_ctx* ctx = new uwgpu_ctx();
    ctx->c.device = device;
    // freed device arrays stay in this process's pool of the device (reused by the next solve)
    {
        cudaMemPool_t pool;
        if (cudaSetDevice(device) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess)
                (void)cudaGetLastError();
        } else {
            (void)cudaGetLastError();
        }
    }
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&ctx->c.host_scalars, 1024 * sizeof(double)) != cudaSuccess) {
        delete ctx;
        return UWGPU_ERR_CUDA;
    }
    *out = ctx;
    return UWGPU_OK;
}

void uwgpu_destroy(uwgpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->c.device);
    cudaStreamSynchronize(ctx->c.stream);
    for (auto& f : ctx->c.prof)
        for (auto& pr : f.events) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    if (ctx->c.host_scalars) cudaFreeHost(ctx->c.host_scalars);
    cudaStream_t s = ctx->c.stream;
    delete ctx;  // frees device arrays
    if (s) cudaStreamDestroy(s);
}

const char* uwgpu_last_error(const uwgpu_ctx* ctx) {
    if (!ctx) return "null context";
    return ctx->c.last_error.c_str();
}

int uwgpu_synchronize(uwgpu_ctx* ctx) {
    return guarded(ctx, [&](Context& c) { UWG_CUDA(cudaStreamSynchronize(c.stream)); });
}

int uwgpu_mesh_q1(uwgpu_ctx* ctx, int32_t dim, const int32_t nel[3], const double mn[3],
                  const double mx[3]) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(dim == 2 || dim == 3, UWGPU_ERR_ARGUMENT, "dim must be 2 or 3");
        UWG_REQUIRE(nel && mn && mx, UWGPU_ERR_ARGUMENT, "null mesh argument");
        uwg::MeshDesc m;
        m.dim = dim;
        for (int d = 0; d < 3; ++d) {
            m.nel[d] = d < dim ? nel[d] : 1;
            m.min[d] = mn[d];
            m.max[d] = mx[d];
            if (d < dim) {
                UWG_REQUIRE(nel[d] >= 1, UWGPU_ERR_ARGUMENT, "element count must be positive");
                UWG_REQUIRE(mx[d] > mn[d], UWGPU_ERR_ARGUMENT, "max must exceed min");
            }
        }
        m.nnx = m.nel[0] + 1;
        m.nny = m.nel[1] + 1;
        m.nnz = dim == 3 ? m.nel[2] + 1 : 1;
        m.nn = m.nnx * m.nny * m.nnz;
        m.ne = (int64_t)m.nel[0] * m.nel[1] * (dim == 3 ? m.nel[2] : 1);
        UWG_REQUIRE(m.ne < (int64_t)0x7fffffff, UWGPU_ERR_ARGUMENT, "too many elements");
        c.mesh = m;
        c.has_mesh = true;
        c.elem_h_for = -1;
        c.has_bc = false;
        c.mapped = false;
        c.assembled = false;
        c.operator_built = false;
        c.has_solution = false;
        c.has_temperature = false;
    });
}

int uwgpu_bc_set(uwgpu_ctx* ctx, const uint8_t* fixed, const double* values) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_mesh, UWGPU_ERR_STATE, "mesh not set");
        UWG_REQUIRE(fixed, UWGPU_ERR_ARGUMENT, "fixed mask is null");
        size_t n = (size_t)c.mesh.nn * c.mesh.dim;
        // the device keeps the mask per dof, node-major like the host array
        upload(c.fixed, fixed, n, c.stream);
        c.bcval.ensure(n);
        c.bc_nonzero = false;
        if (values) {
            for (size_t i = 0; i < n; ++i)
                if (fixed[i] && values[i] != 0.0) { c.bc_nonzero = true; break; }
            UWG_CUDA(cudaMemcpyAsync(c.bcval.p, values, n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        } else {
            UWG_CUDA(cudaMemsetAsync(c.bcval.p, 0, n * sizeof(double), c.stream));
        }
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        c.has_bc = true;
        c.operator_built = false;
    });
}

int uwgpu_materials_set(uwgpu_ctx* ctx, int32_t n, const uwgpu_material* mats) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(n >= 1 && mats, UWGPU_ERR_ARGUMENT, "need at least one material");
        for (int i = 0; i < n; ++i) {
            UWG_REQUIRE(mats[i].n_laws >= 1 && mats[i].n_laws <= 4, UWGPU_ERR_ARGUMENT,
                        "material needs 1..4 rheology laws");
            for (int l = 0; l < mats[i].n_laws; ++l) {
                int law = mats[i].laws[l].law;
                UWG_REQUIRE(law >= UWGPU_LAW_MATERIAL_VISCOSITY && law <= UWGPU_LAW_MOHR_COULOMB,
                            UWGPU_ERR_UNSUPPORTED,
                            "rheology law " + std::to_string(law) + " is not provided by this library");
                if (law == UWGPU_LAW_DEPTH_DEPENDENT) {
                    const double axis = mats[i].laws[l].p[3];
                    UWG_REQUIRE(axis == 0.0 || axis == 1.0 || axis == 2.0, UWGPU_ERR_ARGUMENT,
                                "DepthDependentViscosity variationAxis must be 0, 1 or 2");
                }
            }
        }
        upload(c.mats, mats, (size_t)n, c.stream);
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        c.nmat = n;
    });
}

int uwgpu_fields_set(uwgpu_ctx* ctx, const double* nodal_temperature, double gravity, int32_t vert_axis) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_mesh, UWGPU_ERR_STATE, "mesh not set");
        UWG_REQUIRE(vert_axis >= 0 && vert_axis < c.mesh.dim, UWGPU_ERR_ARGUMENT, "bad vertical axis");
        if (nodal_temperature) {
            upload(c.temperature, nodal_temperature, (size_t)c.mesh.nn, c.stream);
            c.has_temperature = true;
        } else {
            c.has_temperature = false;
        }
        c.gravity = gravity;
        c.vert_axis = vert_axis;
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_solution_set(uwgpu_ctx* ctx, const double* u_nodal, const double* p) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_mesh, UWGPU_ERR_STATE, "mesh not set");
        UWG_REQUIRE(u_nodal && p, UWGPU_ERR_ARGUMENT, "null solution");
        int dim = c.mesh.dim;
        int64_t nn = c.mesh.nn;
        std::vector<double> soa((size_t)nn * dim);
        for (int64_t n = 0; n < nn; ++n)
            for (int d = 0; d < dim; ++d) soa[(size_t)d * nn + n] = u_nodal[n * dim + d];
        upload(c.u_sol, soa.data(), soa.size(), c.stream);
        upload(c.p_sol, p, (size_t)c.mesh.ne, c.stream);
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        c.has_solution = true;
    });
}

int uwgpu_particles_upload(uwgpu_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                           const int32_t* material, const double* eta, const double* rho) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_mesh, UWGPU_ERR_STATE, "mesh not set");
        UWG_REQUIRE(n >= 0 && n < (int64_t)0xffffffffLL, UWGPU_ERR_ARGUMENT, "bad point count");
        UWG_REQUIRE(n == 0 || (x && y && (c.mesh.dim == 2 || z)), UWGPU_ERR_ARGUMENT, "null coordinates");
        size_t N = (size_t)n;
        c.np = n;
        if (n > 0) {
            upload(c.px, x, N, c.stream);
            upload(c.py, y, N, c.stream);
            if (c.mesh.dim == 3) upload(c.pz, z, N, c.stream);
            if (material) {
                upload(c.pmat, material, N, c.stream);
            } else {
                c.pmat.ensure(N);
                UWG_CUDA(cudaMemsetAsync(c.pmat.p, 0, N * sizeof(int32_t), c.stream));
            }
            c.has_peta = eta != nullptr;
            c.has_prho = rho != nullptr;
            if (eta) upload(c.peta, eta, N, c.stream);
            if (rho) upload(c.prho, rho, N, c.stream);
        }
        c.has_points = true;
        c.has_pfw = false;   // a new point set: its strain-weakening history is set again if needed
        c.mapped = false;
        c.assembled = false;
    });
}

int uwgpu_get_cell_tables(uwgpu_ctx* ctx, uint32_t* perm, uint32_t* offsets) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.mapped, UWGPU_ERR_STATE, "points not mapped");
        if (perm && c.np > 0)
            UWG_CUDA(cudaMemcpyAsync(perm, c.perm.p, (size_t)c.np * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
        if (offsets)
            UWG_CUDA(cudaMemcpyAsync(offsets, c.offsets.p, (size_t)(c.mesh.ne + 1) * sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_population_control(uwgpu_ctx* ctx, const uwgpu_pcdvc_opts* opts, int64_t* count) {
    return guarded(ctx, [&](Context& c) {
        uwgpu_pcdvc_opts o;
        if (opts) o = *opts;
        else o = uwgpu_pcdvc_opts{25.0, 0.6, 2, 3, 0, 0};
        const int64_t n = uwg::population_control(c, o);
        if (count) *count = n;
    });
}

int uwgpu_strain_weakening_set(uwgpu_ctx* ctx, const double* pfw) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_points && c.np > 0, UWGPU_ERR_STATE, "material points not uploaded");
        const size_t N = (size_t)c.np;
        if (pfw) upload(c.pfw, pfw, N, c.stream);
        else {
            c.pfw.ensure(N);
            UWG_CUDA(cudaMemsetAsync(c.pfw.p, 0, N * sizeof(double), c.stream));
        }
        c.pfw_incr.ensure(N);
        UWG_CUDA(cudaMemsetAsync(c.pfw_incr.p, 0, N * sizeof(double), c.stream));
        c.has_pfw = true;
        c.assembled = false;
    });
}

int uwgpu_strain_weakening_advance(uwgpu_ctx* ctx, double dt) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_pfw, UWGPU_ERR_STATE, "strain-weakening history not set");
        UWG_REQUIRE(std::isfinite(dt), UWGPU_ERR_ARGUMENT, "dt must be finite");
        uwg::strain_weakening_advance(c, dt);
    });
}

int uwgpu_strain_weakening_get(uwgpu_ctx* ctx, double* pfw, double* increment) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_pfw, UWGPU_ERR_STATE, "strain-weakening history not set");
        const size_t N = (size_t)c.np;
        if (pfw) UWG_CUDA(cudaMemcpyAsync(pfw, c.pfw.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if (increment)
            UWG_CUDA(cudaMemcpyAsync(increment, c.pfw_incr.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_advect_particles(uwgpu_ctx* ctx, double dt, int32_t order, int32_t allow_first_order_fallback,
                           uint32_t* fell_back, uint32_t* left_mesh) {
    return guarded(ctx, [&](Context& c) {
        uint32_t fb = 0, lm = 0;
        uwg::advect_particles(c, dt, order, allow_first_order_fallback != 0, fb, lm);
        if (fell_back) *fell_back = fb;
        if (left_mesh) *left_mesh = lm;
    });
}

int uwgpu_particles_download(uwgpu_ctx* ctx, double* x, double* y, double* z) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_points, UWGPU_ERR_STATE, "no particles");
        const size_t n = (size_t)c.np;
        if (x && n) UWG_CUDA(cudaMemcpyAsync(x, c.px.p, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if (y && n) UWG_CUDA(cudaMemcpyAsync(y, c.py.p, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if (z && n && c.mesh.dim == 3)
            UWG_CUDA(cudaMemcpyAsync(z, c.pz.p, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_bin_and_map(uwgpu_ctx* ctx, uint32_t* perm, uint32_t* offsets, double* xi) {
    return guarded(ctx, [&](Context& c) {
        uwg::bin_and_map(c);
        size_t N = (size_t)c.np, E = (size_t)c.mesh.ne;
        if (perm && N) UWG_CUDA(cudaMemcpyAsync(perm, c.perm.p, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
        if (offsets) UWG_CUDA(cudaMemcpyAsync(offsets, c.offsets.p, (E + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
        if (xi && N) {
            std::vector<double> tmp(3 * N);
            int dim = c.mesh.dim;
            UWG_CUDA(cudaMemcpyAsync(tmp.data(), c.sxi.p, (size_t)dim * N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            UWG_CUDA(cudaStreamSynchronize(c.stream));
            for (size_t s = 0; s < N; ++s)
                for (int d = 0; d < 3; ++d) xi[3 * s + d] = d < dim ? tmp[(size_t)d * N + s] : 0.0;
        }
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_weights_set(uwgpu_ctx* ctx, int32_t kind, const int32_t res[3]) {
    return guarded(ctx, [&](Context& c) { uwg::weights_set(c, kind, res); });
}

int uwgpu_integration_points(uwgpu_ctx* ctx, double* xi, double* w) {
    return guarded(ctx, [&](Context& c) { uwg::integration_points_download(c, xi, w); });
}

int uwgpu_assemble(uwgpu_ctx* ctx) {
    return guarded(ctx, [&](Context& c) { uwg::assemble(c); });
}

int uwgpu_get_element_matrices(uwgpu_ctx* ctx, int64_t first, int64_t count, double* Ke, double* fe,
                               double* Ge, double* Se) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.assembled, UWGPU_ERR_STATE, "nothing assembled");
        int64_t E = c.mesh.ne;
        UWG_REQUIRE(first >= 0 && count >= 0 && first + count <= E, UWGPU_ERR_ARGUMENT, "element range");
        int dim = c.mesh.dim, nen = dim == 3 ? 8 : 4, nd = nen * dim, np = uwg::packed_size(nd);
        if (count == 0) return;
        auto fetch = [&](const double* base, int entries, std::vector<double>& out) {
            out.resize((size_t)entries * count);
            // entry-major [k][e]: one strided copy
            UWG_CUDA(cudaMemcpy2DAsync(out.data(), count * sizeof(double), base + first, E * sizeof(double),
                                       count * sizeof(double), entries, cudaMemcpyDeviceToHost, c.stream));
        };
        std::vector<double> hk, hf, hg;
        const bool full = c.assembled_jacobian;   // the Newton form's non-symmetric K_e, all entries
        if (Ke) fetch(full ? c.Kjac.p : c.levels[0].Ke.p, full ? nd * nd : np, hk);
        if (fe) fetch(c.fe.p, nd, hf);
        if (Ge) fetch(c.Ge.p, nd, hg);
        if (Se) UWG_CUDA(cudaMemcpyAsync(Se, c.Se.p + first, count * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        for (int64_t e = 0; e < count; ++e) {
            if (Ke && full) {
                for (int k = 0; k < nd * nd; ++k) Ke[e * nd * nd + k] = hk[(size_t)k * count + e];
            } else if (Ke) {
                double* K = Ke + e * nd * nd;
                for (int r = 0; r < nd; ++r)
                    for (int q = r; q < nd; ++q) {
                        double v = hk[(size_t)uwg::packed_index(nd, r, q) * count + e];
                        K[r * nd + q] = v;
                        K[q * nd + r] = v;
                    }
            }
            for (int k = 0; k < nd; ++k) {
                if (fe) fe[e * nd + k] = hf[(size_t)k * count + e];
                if (Ge) Ge[e * nd + k] = hg[(size_t)k * count + e];
            }
        }
    });
}

int uwgpu_get_point_viscosity(uwgpu_ctx* ctx, double* eta) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.assembled, UWGPU_ERR_STATE, "nothing assembled");
        UWG_REQUIRE(eta || c.np == 0, UWGPU_ERR_ARGUMENT, "null output");
        if (c.np) UWG_CUDA(cudaMemcpyAsync(eta, c.seta_out.p, c.np * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_operator_apply(uwgpu_ctx* ctx, int32_t precision, const double* x, double* y) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(x && y, UWGPU_ERR_ARGUMENT, "null vector");
        UWG_REQUIRE(precision == UWGPU_PREC_FP64 || precision == UWGPU_PREC_MIXED, UWGPU_ERR_ARGUMENT,
                    "bad precision");
        int dim = c.mesh.dim;
        int64_t nn = c.mesh.nn;
        if (!c.operator_built || (precision == UWGPU_PREC_MIXED && !c.operator_has32))
            uwg::build_operator(c, c.operator_built ? c.operator_levels : 1, precision == UWGPU_PREC_MIXED);
        std::vector<double> soa((size_t)nn * dim);
        for (int64_t n = 0; n < nn; ++n)
            for (int d = 0; d < dim; ++d) soa[(size_t)d * nn + n] = x[n * dim + d];
        uwg::DArray<double> dx, dy;
        dx.ensure(soa.size());
        dy.ensure(soa.size());
        UWG_CUDA(cudaMemcpyAsync(dx.p, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        uwg::apply_fine(c, precision == UWGPU_PREC_MIXED, dx.p, dy.p);
        UWG_CUDA(cudaMemcpyAsync(soa.data(), dy.p, soa.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        for (int64_t n = 0; n < nn; ++n)
            for (int d = 0; d < dim; ++d) y[n * dim + d] = soa[(size_t)d * nn + n];
    });
}

void uwgpu_solve_opts_default(uwgpu_solve_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->mg_levels = 4;
    o->smooth_down = 2;
    o->smooth_up = 2;
    o->schur_type = UWGPU_SCHUR_CG;
    o->schur_pc = UWGPU_SCHUR_PC_UW;
    o->restart = 30;
    o->max_outer = 500;
    o->max_inner = 500;
    o->scr_rtol = 1e-6;
    o->a11_rtol = 1e-8;
    o->back_rtol = 1e-8;
    o->remove_const_p = 1;
    o->precision = UWGPU_PREC_FP64;
    o->target_rel_residual = 0.0;
    o->bfbt_rtol = 1e-2;
    o->bfbt_max_it = 500;
    o->smoother = UWGPU_SMOOTHER_COLOUR_GS;
    o->learned_pc = 0;
    o->learned_stagnation = 2;
    o->mg_cycle = 1;
    o->bfbt_inner_pc = 0;
}

int uwgpu_solve_bsscr(uwgpu_ctx* ctx, const uwgpu_solve_opts* opts, double* u, double* p, uwgpu_report* report) {
    return guarded(ctx, [&](Context& c) {
        uwgpu_solve_opts o;
        if (opts) o = *opts; else uwgpu_solve_opts_default(&o);
        uwgpu_report rep;
        std::memset(&rep, 0, sizeof(rep));
        uwg::solve_bsscr(c, o, rep);
        int dim = c.mesh.dim;
        int64_t nn = c.mesh.nn;
        if (u) {
            std::vector<double> soa((size_t)nn * dim);
            UWG_CUDA(cudaMemcpyAsync(soa.data(), c.u_sol.p, soa.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            UWG_CUDA(cudaStreamSynchronize(c.stream));
            for (int64_t n = 0; n < nn; ++n)
                for (int d = 0; d < dim; ++d) u[n * dim + d] = soa[(size_t)d * nn + n];
        }
        if (p) UWG_CUDA(cudaMemcpyAsync(p, c.p_sol.p, c.mesh.ne * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        if (report) *report = rep;
        if (rep.status != UWGPU_OK) throw Error(rep.status, "BSSCR solve did not converge");
    });
}

int uwgpu_solve_picard(uwgpu_ctx* ctx, const uwgpu_solve_opts* opts, double tolerance, int32_t max_iterations,
                       int32_t min_iterations, double* u, double* p, uwgpu_report* report, int32_t* iterations,
                       double* residual) {
    return guarded(ctx, [&](Context& c) {
        uwgpu_solve_opts o;
        if (opts) o = *opts; else uwgpu_solve_opts_default(&o);
        uwgpu_report rep;
        std::memset(&rep, 0, sizeof(rep));
        int its = 0;
        double res = 0.0;
        uwg::solve_picard(c, o, tolerance, max_iterations, min_iterations, rep, its, res);
        int dim = c.mesh.dim;
        int64_t nn = c.mesh.nn;
        if (u) {
            std::vector<double> soa((size_t)nn * dim);
            UWG_CUDA(cudaMemcpyAsync(soa.data(), c.u_sol.p, soa.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            UWG_CUDA(cudaStreamSynchronize(c.stream));
            for (int64_t n = 0; n < nn; ++n)
                for (int d = 0; d < dim; ++d) u[n * dim + d] = soa[(size_t)d * nn + n];
        }
        if (p) UWG_CUDA(cudaMemcpyAsync(p, c.p_sol.p, c.mesh.ne * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        if (report) *report = rep;
        if (iterations) *iterations = its;
        if (residual) *residual = res;
        if (rep.status != UWGPU_OK) throw Error(rep.status, "Picard iteration: a Stokes solve did not converge");
    });
}

int uwgpu_profile_enable(uwgpu_ctx* ctx, int32_t on) {
    return guarded(ctx, [&](Context& c) {
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        for (auto& f : c.prof) {
            f.used = 0;
            f.launches = 0;
            f.ms = 0.0;
            f.bytes = 0.0;
            f.flops = 0.0;
        }
        c.profiling = on != 0;
    });
}

int uwgpu_profile_read(uwgpu_ctx* ctx, int32_t which, int64_t* launches, double* ms) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(which >= 0 && which < UWGPU_KERNEL_COUNT, UWGPU_ERR_ARGUMENT, "bad kernel family");
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        uwg::ProfileFamily& f = c.prof[which];
        double total = f.ms;
        for (size_t i = 0; i < f.used; ++i) {
            float t = 0.f;
            UWG_CUDA(cudaEventElapsedTime(&t, f.events[i].first, f.events[i].second));
            total += t;
        }
        f.ms = total;
        f.used = 0;
        if (launches) *launches = f.launches;
        if (ms) *ms = total;
    });
}

int uwgpu_profile_read_work(uwgpu_ctx* ctx, int32_t which, double* bytes, double* flops) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(which >= 0 && which < UWGPU_KERNEL_COUNT, UWGPU_ERR_ARGUMENT, "bad kernel family");
        if (bytes) *bytes = c.prof[which].bytes;
        if (flops) *flops = c.prof[which].flops;
    });
}

int64_t uwgpu_launch_count(const uwgpu_ctx* ctx) { return ctx ? ctx->c.launches : 0; }

int uwgpu_bfbt_operator_apply(uwgpu_ctx* ctx, int32_t form, const double* x, double* y) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(x && y, UWGPU_ERR_ARGUMENT, "x and y are required");
        uwg::bfbt_operator_hook(c, form, x, y, 0, nullptr);
    });
}

int uwgpu_jacobian_set(uwgpu_ctx* ctx, int32_t on) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(!on || (c.has_mesh && c.mesh.dim == 2), UWGPU_ERR_UNSUPPORTED,
                    "the Newton form of the element matrices is the reference's 2D branch");
        c.jacobian = on != 0;
        c.assembled = false;
    });
}

int uwgpu_assembly_set(uwgpu_ctx* ctx, int32_t mode) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(mode == UWGPU_ASSEMBLY_FP64 || mode == UWGPU_ASSEMBLY_TENSOR, UWGPU_ERR_ARGUMENT, "bad assembly mode");
        c.assembly_mode = mode;
    });
}

int uwgpu_smoother_storage_set(uwgpu_ctx* ctx, int32_t bits) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(bits == 16 || bits == 32, UWGPU_ERR_ARGUMENT, "smoother stencil storage must be 16 or 32 bits");
        c.smooth16 = bits == 16;
    });
}

int uwgpu_tc_check(uwgpu_ctx* ctx, int32_t layout, int32_t format, int32_t n, int32_t k, const uint16_t* a,
                   const uint16_t* b, float* d) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(a && b && d, UWGPU_ERR_ARGUMENT, "a, b and d are required");
        uwg::tc_check(layout, format, n, k, a, b, d);
    });
}

int uwgpu_time_bfbt_apply(uwgpu_ctx* ctx, int32_t form, int32_t iterations, double* ms) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(ms && iterations > 0, UWGPU_ERR_ARGUMENT, "bad arguments");
        uwg::bfbt_operator_hook(c, form, nullptr, nullptr, iterations, ms);
    });
}

int uwgpu_time_apply(uwgpu_ctx* ctx, int32_t precision, int32_t iterations, double* ms) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(ms && iterations > 0, UWGPU_ERR_ARGUMENT, "bad arguments");
        bool f32 = precision == UWGPU_PREC_MIXED;
        if (!c.operator_built || (f32 && !c.operator_has32))
            uwg::build_operator(c, c.operator_built ? c.operator_levels : 1, f32);
        uwg::Level& L = c.levels[0];
        size_t nv = (size_t)L.mesh.nn * L.mesh.dim;
        cudaEvent_t e0, e1;
        UWG_CUDA(cudaEventCreate(&e0));
        UWG_CUDA(cudaEventCreate(&e1));
        if (f32) {
            UWG_CUDA(cudaMemsetAsync(L.x32.p, 0, nv * sizeof(float), c.stream));
            UWG_CUDA(cudaEventRecord(e0, c.stream));
            for (int i = 0; i < iterations; ++i) uwg::level_apply<float>(c, L, L.x32.p, L.t32.p);
        } else {
            UWG_CUDA(cudaMemsetAsync(L.x64.p, 0, nv * sizeof(double), c.stream));
            UWG_CUDA(cudaEventRecord(e0, c.stream));
            for (int i = 0; i < iterations; ++i) uwg::level_apply<double>(c, L, L.x64.p, L.t64.p);
        }
        UWG_CUDA(cudaEventRecord(e1, c.stream));
        UWG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        UWG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *ms = t;
    });
}

int uwgpu_time_chebyshev(uwgpu_ctx* ctx, int32_t precision, int32_t degree, int32_t iterations, double* ms) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(ms && iterations > 0 && degree > 0, UWGPU_ERR_ARGUMENT, "bad arguments");
        const bool f32 = precision == UWGPU_PREC_MIXED;
        uwgpu_solve_opts o;
        uwgpu_solve_opts_default(&o);
        o.mg_levels = c.operator_built ? c.operator_levels : 1;
        o.precision = f32 ? UWGPU_PREC_MIXED : UWGPU_PREC_FP64;
        uwg::estimate_fine_lmax(c, o);
        uwg::Level& L = c.levels[0];
        const size_t nv = (size_t)L.mesh.nn * L.mesh.dim;
        cudaEvent_t e0, e1;
        UWG_CUDA(cudaEventCreate(&e0));
        UWG_CUDA(cudaEventCreate(&e1));
        // from the current iterate (not a zero guess), so every step applies the stencil
        if (f32) {
            UWG_CUDA(cudaMemsetAsync(L.b32.p, 0, nv * sizeof(float), c.stream));
            UWG_CUDA(cudaMemsetAsync(L.x32.p, 0, nv * sizeof(float), c.stream));
            UWG_CUDA(cudaEventRecord(e0, c.stream));
            for (int i = 0; i < iterations; ++i) uwg::level_cheb<float>(c, L, L.b32.p, L.x32.p, degree, false);
        } else {
            UWG_CUDA(cudaMemsetAsync(L.b64.p, 0, nv * sizeof(double), c.stream));
            UWG_CUDA(cudaMemsetAsync(L.x64.p, 0, nv * sizeof(double), c.stream));
            UWG_CUDA(cudaEventRecord(e0, c.stream));
            for (int i = 0; i < iterations; ++i) uwg::level_cheb<double>(c, L, L.b64.p, L.x64.p, degree, false);
        }
        UWG_CUDA(cudaEventRecord(e1, c.stream));
        UWG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        UWG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *ms = t;
    });
}

int uwgpu_time_smooth(uwgpu_ctx* ctx, int32_t precision, int32_t sweeps, int32_t iterations, double* ms) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(ms && iterations > 0 && sweeps > 0, UWGPU_ERR_ARGUMENT, "bad arguments");
        bool f32 = precision == UWGPU_PREC_MIXED;
        if (!c.operator_built || (f32 && !c.operator_has32))
            uwg::build_operator(c, c.operator_built ? c.operator_levels : 1, f32);
        uwg::Level& L = c.levels[0];
        size_t nv = (size_t)L.mesh.nn * L.mesh.dim;
        cudaEvent_t e0, e1;
        UWG_CUDA(cudaEventCreate(&e0));
        UWG_CUDA(cudaEventCreate(&e1));
        if (f32) {
            UWG_CUDA(cudaMemsetAsync(L.b32.p, 0, nv * sizeof(float), c.stream));
            UWG_CUDA(cudaEventRecord(e0, c.stream));
            for (int i = 0; i < iterations; ++i) uwg::level_smooth<float>(c, L, L.b32.p, L.x32.p, sweeps, true);
        } else {
            UWG_CUDA(cudaMemsetAsync(L.b64.p, 0, nv * sizeof(double), c.stream));
            UWG_CUDA(cudaEventRecord(e0, c.stream));
            for (int i = 0; i < iterations; ++i) uwg::level_smooth<double>(c, L, L.b64.p, L.x64.p, sweeps, true);
        }
        UWG_CUDA(cudaEventRecord(e1, c.stream));
        UWG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        UWG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *ms = t;
    });
}

int uwgpu_get_stream(uwgpu_ctx* ctx, void** stream) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(stream, UWGPU_ERR_ARGUMENT, "null output");
        *stream = (void*)c.stream;
    });
}

// ---- learned velocity preconditioner ----
static uwg::unet::Net& net_of(Context& c) {
    UWG_REQUIRE(c.net != nullptr, UWGPU_ERR_STATE, "no learned preconditioner: call uwgpu_learned_create");
    return *c.net;
}

int uwgpu_learned_create(uwgpu_ctx* ctx, int32_t levels, int32_t base_channels, uint64_t seed) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(c.has_mesh, UWGPU_ERR_STATE, "learned preconditioner requested before the mesh");
        auto* n = new uwg::unet::Net();
        try {
            uwg::unet::create(c, *n, levels, base_channels, seed);
        } catch (...) {
            delete n;
            throw;
        }
        uwg::unet::destroy(c.net);
        c.net = n;
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_learned_param_count(uwgpu_ctx* ctx, int64_t* count) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(count, UWGPU_ERR_ARGUMENT, "null count");
        *count = net_of(c).nparams;
    });
}

int uwgpu_learned_get_params(uwgpu_ctx* ctx, float* params) {
    return guarded(ctx, [&](Context& c) {
        auto& n = net_of(c);
        UWG_REQUIRE(params, UWGPU_ERR_ARGUMENT, "null params");
        UWG_CUDA(cudaMemcpyAsync(params, n.params.p, (size_t)n.nparams * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_learned_set_params(uwgpu_ctx* ctx, const float* params) {
    return guarded(ctx, [&](Context& c) {
        auto& n = net_of(c);
        UWG_REQUIRE(params, UWGPU_ERR_ARGUMENT, "null params");
        UWG_CUDA(cudaMemcpyAsync(n.params.p, params, (size_t)n.nparams * sizeof(float), cudaMemcpyHostToDevice, c.stream));
        uwg::unet::pack(c, n);
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_learned_forward(uwgpu_ctx* ctx, const float* input, float* output) {
    return guarded(ctx, [&](Context& c) {
        auto& n = net_of(c);
        UWG_REQUIRE(input && output, UWGPU_ERR_ARGUMENT, "null input or output");
        uwg::unet::set_input_host(c, n, input);
        uwg::unet::forward(c, n);
        uwg::unet::get_output_host(c, n, output);
    });
}

int uwgpu_learned_backward(uwgpu_ctx* ctx, const float* grad_output, float* grad_params, float* grad_input) {
    return guarded(ctx, [&](Context& c) {
        auto& n = net_of(c);
        UWG_REQUIRE(grad_output, UWGPU_ERR_ARGUMENT, "null grad_output");
        uwg::unet::set_grad_output_host(c, n, grad_output);
        UWG_CUDA(cudaMemsetAsync(n.grads.p, 0, (size_t)n.nparams * sizeof(float), c.stream));
        uwg::unet::backward(c, n);
        if (grad_params)
            UWG_CUDA(cudaMemcpyAsync(grad_params, n.grads.p, (size_t)n.nparams * sizeof(float), cudaMemcpyDeviceToHost,
                                     c.stream));
        if (grad_input) uwg::unet::get_input_grad_host(c, n, grad_input);
        UWG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int uwgpu_learned_generate(uwgpu_ctx* ctx, const uwgpu_solve_opts* opts, int32_t nsamples, uint64_t seed) {
    return guarded(ctx, [&](Context& c) {
        UWG_REQUIRE(opts, UWGPU_ERR_ARGUMENT, "null options");
        uwg::learned_generate(c, *opts, nsamples, seed);
    });
}

int uwgpu_learned_train(uwgpu_ctx* ctx, int32_t epochs, int32_t batch, float learning_rate, uint64_t seed,
                        double* train_loss, double* holdout_ratio) {
    return guarded(ctx, [&](Context& c) {
        uwg::unet::train(c, net_of(c), epochs, batch, learning_rate, seed, train_loss, holdout_ratio);
    });
}

}  // extern "C"
