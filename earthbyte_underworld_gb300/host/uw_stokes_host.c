/*
 * uw_stokes_host.c -- C host side of the GB300 Stokes path.
 *
 * Mirrors, in plain C against include/uwgpu.h, the calls an Underworld 1.x SLE execute makes on
 * this path (StgFEM/SLE/SystemSetup/src/SystemLinearEquations.c:87-98 hooks):
 *   IntegrationSetup -> _CoincidentMapper_Map          -> uwgpu_bin_and_map
 *   MatrixSetup / VectorSetup -> StiffnessMatrix and   -> uwgpu_assemble
 *       ForceVector assemble entry points
 *   ExecuteSolver -> StokesBlockKSPInterface / BSSCR   -> uwgpu_solve_bsscr
 * and reads its parameters the way Underworld's main reads command-line overrides
 * (`--key=value`, Underworld/src/main.c:77-79).  The three gpu_* functions below are what a
 * StGermain component shim (the GPU mapper, assembly hook and SLE solver) calls; main() runs them on a generated
 * Rayleigh-Taylor style layout so that the binding can be exercised without StGermain.
 *
 * Build: earthbyte_underworld_gb300/build.py (gcc -O2 ... -luwgpu -lm, rpath next to libuwgpu.so)
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "uwgpu.h"

typedef struct {
    int dim;
    int nel[3];
    int ppc;
    int levels;
    double eta_top, eta_bottom, rho_top, rho_bottom;
    double scr_rtol;
    int precision;
} host_params;

static void params_default(host_params* p) {
    p->dim = 2;
    p->nel[0] = 32;
    p->nel[1] = 32;
    p->nel[2] = 1;
    p->ppc = 20;
    p->levels = 3;
    p->eta_top = 1.0;
    p->eta_bottom = 0.01;
    p->rho_top = 1.0;
    p->rho_bottom = 0.0;
    p->scr_rtol = 1e-8;
    p->precision = UWGPU_PREC_FP64;
}

/* --key=value overrides */
static void params_parse(host_params* p, int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if (strncmp(a, "--", 2) != 0 || !strchr(a, '=')) continue;
        const char* v = strchr(a, '=') + 1;
        if (!strncmp(a, "--dim=", 6)) p->dim = atoi(v);
        else if (!strncmp(a, "--elementResI=", 14)) p->nel[0] = atoi(v);
        else if (!strncmp(a, "--elementResJ=", 14)) p->nel[1] = atoi(v);
        else if (!strncmp(a, "--elementResK=", 14)) p->nel[2] = atoi(v);
        else if (!strncmp(a, "--particlesPerCell=", 19)) p->ppc = atoi(v);
        else if (!strncmp(a, "--mgLevels=", 11)) p->levels = atoi(v);
        else if (!strncmp(a, "--scrRtol=", 10)) p->scr_rtol = atof(v);
        else if (!strncmp(a, "--mixed=", 8)) p->precision = atoi(v) ? UWGPU_PREC_MIXED : UWGPU_PREC_FP64;
    }
}

#define CHECK(call)                                                                   \
    do {                                                                              \
        int rc_ = (call);                                                             \
        if (rc_ != UWGPU_OK) {                                                        \
            fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, uwgpu_last_error(ctx)); \
            return rc_;                                                               \
        }                                                                             \
    } while (0)

/* IntegrationSetup: material points -> cell tables + local coordinates. */
int gpu_map_points(uwgpu_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                   const int32_t* material, uint32_t* cell_perm, uint32_t* cell_offsets) {
    CHECK(uwgpu_particles_upload(ctx, n, x, y, z, material, NULL, NULL));
    CHECK(uwgpu_bin_and_map(ctx, cell_perm, cell_offsets, NULL));
    return UWGPU_OK;
}

/* MatrixSetup + VectorSetup: K, G, f and the Schur preconditioner, on the device. */
int gpu_assemble(uwgpu_ctx* ctx) {
    CHECK(uwgpu_assemble(ctx));
    return UWGPU_OK;
}

/* ExecuteSolver: BSSCR with the options the PETSc options database would carry. */
int gpu_solve(uwgpu_ctx* ctx, const host_params* p, double* u, double* pr, uwgpu_report* rep) {
    uwgpu_solve_opts o;
    uwgpu_solve_opts_default(&o);
    o.mg_levels = p->levels;
    o.schur_type = UWGPU_SCHUR_FGMRES;
    o.schur_pc = UWGPU_SCHUR_PC_SCALED_BFBT;
    o.scr_rtol = p->scr_rtol;
    o.a11_rtol = p->scr_rtol * 1e-2;
    o.back_rtol = p->scr_rtol * 1e-2;
    o.bfbt_rtol = 1e-6;
    o.precision = p->precision;
    CHECK(uwgpu_solve_bsscr(ctx, &o, u, pr, rep));
    return UWGPU_OK;
}

/* Park-Miller stream of StgDomain/Swarm/src/Random.c (Schrage's method). */
static long pm_state;
static double pm_next(void) {
    long tmp = pm_state / 127773L;
    pm_state = 16807L * (pm_state - tmp * 127773L) - 2836L * tmp;
    if (pm_state < 0) pm_state += 2147483647L;
    return (double)pm_state / 2147483647.0;
}

int main(int argc, char** argv) {
    host_params p;
    params_default(&p);
    params_parse(&p, argc, argv);
    int dim = p.dim;
    int64_t E = (int64_t)p.nel[0] * p.nel[1] * (dim == 3 ? p.nel[2] : 1);
    int64_t nn = (int64_t)(p.nel[0] + 1) * (p.nel[1] + 1) * (dim == 3 ? p.nel[2] + 1 : 1);
    int64_t n = E * p.ppc;
    double* x = malloc(sizeof(double) * n);
    double* y = malloc(sizeof(double) * n);
    double* z = malloc(sizeof(double) * n);
    int32_t* mat = malloc(sizeof(int32_t) * n);
    uint8_t* fixed = calloc((size_t)(nn * dim), 1);
    double* u = malloc(sizeof(double) * nn * dim);
    double* pr = malloc(sizeof(double) * E);
    uint32_t* perm = malloc(sizeof(uint32_t) * n);
    uint32_t* offs = malloc(sizeof(uint32_t) * (E + 1));
    /* random layout, cell by cell, interface y = 0.2 + 0.02 cos(pi x) (BelowCosinePlane) */
    pm_state = 13L ^ 123459876L;
    for (int64_t e = 0; e < E; ++e) {
        int64_t ex = e % p.nel[0], ey = (e / p.nel[0]) % p.nel[1], ez = dim == 3 ? e / ((int64_t)p.nel[0] * p.nel[1]) : 0;
        for (int c = 0; c < p.ppc; ++c) {
            int64_t q = e * p.ppc + c;
            x[q] = (ex + pm_next()) / p.nel[0];
            y[q] = (ey + pm_next()) / p.nel[1];
            z[q] = dim == 3 ? (ez + pm_next()) / p.nel[2] : (pm_next(), 0.0);
            mat[q] = y[q] < 0.2 + 0.02 * cos(3.141592653589793 * x[q]) ? 1 : 0;
        }
    }
    /* free-slip walls: normal component fixed */
    int64_t nx = p.nel[0] + 1, ny = p.nel[1] + 1;
    for (int64_t k = 0; k < nn; ++k) {
        int64_t i = k % nx, j = (k / nx) % ny, l = k / (nx * ny);
        if (i == 0 || i == nx - 1) fixed[k * dim + 0] = 1;
        if (j == 0 || j == ny - 1) fixed[k * dim + 1] = 1;
        if (dim == 3 && (l == 0 || l == p.nel[2])) fixed[k * dim + 2] = 1;
    }
    uwgpu_material mats[2];
    memset(mats, 0, sizeof(mats));
    mats[0].n_laws = 1;
    mats[0].laws[0].law = UWGPU_LAW_MATERIAL_VISCOSITY;
    mats[0].laws[0].p[0] = p.eta_top;
    mats[0].density = p.rho_top;
    mats[1] = mats[0];
    mats[1].laws[0].p[0] = p.eta_bottom;
    mats[1].density = p.rho_bottom;

    uwgpu_ctx* ctx = NULL;
    if (uwgpu_create(0, &ctx) != UWGPU_OK) {
        fprintf(stderr, "uwgpu_create failed: no usable GPU\n");
        return 1;
    }
    double mn[3] = {0, 0, 0}, mx[3] = {1, 1, 1};
    int rc = 0;
    uwgpu_report rep;
    memset(&rep, 0, sizeof(rep));
    if ((rc = uwgpu_mesh_q1(ctx, dim, p.nel, mn, mx)) != UWGPU_OK ||
        (rc = uwgpu_bc_set(ctx, fixed, NULL)) != UWGPU_OK ||
        (rc = uwgpu_materials_set(ctx, 2, mats)) != UWGPU_OK ||
        (rc = uwgpu_fields_set(ctx, NULL, 1.0, dim - 1)) != UWGPU_OK ||
        (rc = gpu_map_points(ctx, n, x, y, z, mat, perm, offs)) != UWGPU_OK ||
        (rc = gpu_assemble(ctx)) != UWGPU_OK || (rc = gpu_solve(ctx, &p, u, pr, &rep)) != UWGPU_OK) {
        fprintf(stderr, "failed: %d %s\n", rc, uwgpu_last_error(ctx));
    } else {
        double vmax = 0.0;
        for (int64_t k = 0; k < nn * dim; ++k) vmax = u[k] > vmax ? u[k] : (-u[k] > vmax ? -u[k] : vmax);
        printf("{\"points\": %lld, \"elements\": %lld, \"outer_its\": %d, \"inner_its\": %d, "
               "\"rel_residual\": %.3e, \"vmax\": %.9e, \"solve_ms\": %.3f}\n",
               (long long)n, (long long)E, rep.outer_its, rep.inner_its_total, rep.rel_residual, vmax,
               rep.t_solve_ms);
    }
    uwgpu_destroy(ctx);
    free(x); free(y); free(z); free(mat); free(fixed); free(u); free(pr); free(perm); free(offs);
    return rc;
}
