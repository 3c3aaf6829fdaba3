/*
 * uwref.c -- CPU restatement of the Underworld 1.x particle-in-cell Stokes hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the parity tests, the smoke check and the CPU
 * baseline of bench.py run.  The GPU library never links or calls this file.
 *
 * Each function names the reference routine it restates (paths relative to the
 * Underworld 1.x tree).  Loop orders and floating-point expressions follow those routines
 * so that results agree to rounding; where a PETSc routine is used by the reference
 * (SOR, FGMRES, CG, MatPtAP, LU) the published algorithm is restated.
 */
#define _POSIX_C_SOURCE 200809L
#include "uwref.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* StGermain/Base/Foundation/src/Numerics.c:37-41 */
static const double kNumEpsilon = 1e-12;
static int num_approx(double var, double val) {
    return var >= val - kNumEpsilon && var <= val + kNumEpsilon;
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------------------ */
/* Mesh                                                                                 */
/* ------------------------------------------------------------------------------------ */

int64_t uwr_num_nodes(const uwr_mesh* m) {
    int64_t n = 1;
    for (int d = 0; d < m->dim; ++d) n *= (m->nel[d] + 1);
    return n;
}

int64_t uwr_num_elements(const uwr_mesh* m) {
    int64_t n = 1;
    for (int d = 0; d < m->dim; ++d) n *= m->nel[d];
    return n;
}

/* StgDomain/Mesh/src/CartesianGenerator.c:2275-2310 (CartesianGenerator_CalcGeom, no contact
 * depth): first node at crdMin, last at crdMax, interior min + (i/(n-1))*(max-min). */
static double node_coord_1d(const uwr_mesh* m, int d, int64_t i) {
    int64_t sizes = m->nel[d] + 1;
    if (i <= 0) return m->min[d];
    if (i >= sizes - 1) return m->max[d];
    return m->min[d] + ((double)i / (double)(sizes - 1)) * (m->max[d] - m->min[d]);
}

void uwr_node_coords(const uwr_mesh* m, double* xyz) {
    int64_t nx = m->nel[0] + 1, ny = m->nel[1] + 1, nz = (m->dim == 3) ? m->nel[2] + 1 : 1;
    for (int64_t k = 0; k < nz; ++k)
        for (int64_t j = 0; j < ny; ++j)
            for (int64_t i = 0; i < nx; ++i) {
                int64_t n = i + nx * (j + ny * k);
                xyz[3 * n + 0] = node_coord_1d(m, 0, i);
                xyz[3 * n + 1] = node_coord_1d(m, 1, j);
                xyz[3 * n + 2] = (m->dim == 3) ? node_coord_1d(m, 2, k) : 0.0;
            }
}

/* StgDomain/Mesh/src/CartesianGenerator.c:976-1035 (element-vertex incidence) with
 * Grid_Project (StgDomain/Mesh/src/Grid.c:257-275, basis = x fastest). */
void uwr_element_nodes(const uwr_mesh* m, int64_t e, int64_t* inc) {
    int64_t ex = m->nel[0], ey = m->nel[1];
    int64_t i = e % ex, j = (e / ex) % ey, k = (m->dim == 3) ? e / (ex * ey) : 0;
    int64_t nx = ex + 1, ny = ey + 1;
    int64_t base = i + nx * (j + ny * k);
    inc[0] = base;
    inc[1] = base + 1;
    inc[2] = base + nx;
    inc[3] = base + nx + 1;
    if (m->dim == 3) {
        int64_t s = nx * ny;
        inc[4] = base + s;
        inc[5] = base + s + 1;
        inc[6] = base + s + nx;
        inc[7] = base + s + nx + 1;
    }
}

static void element_node_xyz(const uwr_mesh* m, int64_t e, double xyz[8][3]) {
    int64_t inc[8];
    int64_t nx = m->nel[0] + 1, ny = m->nel[1] + 1;
    int nen = (m->dim == 3) ? 8 : 4;
    uwr_element_nodes(m, e, inc);
    for (int a = 0; a < nen; ++a) {
        int64_t n = inc[a];
        int64_t i = n % nx, j = (n / nx) % ny, k = n / (nx * ny);
        xyz[a][0] = node_coord_1d(m, 0, i);
        xyz[a][1] = node_coord_1d(m, 1, j);
        xyz[a][2] = (m->dim == 3) ? node_coord_1d(m, 2, k) : 0.0;
    }
}

/* ------------------------------------------------------------------------------------ */
/* Inputs                                                                               */
/* ------------------------------------------------------------------------------------ */

/* StgDomain/Swarm/src/Random.c:43-73 (Park-Miller minimal standard, Schrage's method). */
typedef struct { long state; } pm_rng;
static void pm_seed(pm_rng* r, long seed) { r->state = seed ^ 123459876L; }
static double pm_random(pm_rng* r) {
    const long q = 127773, rr = 2836, a = 16807, mx = 2147483647L;
    long tmp = r->state / q;
    r->state = a * (r->state - tmp * q) - rr * tmp;
    if (r->state < 0) r->state += mx;
    return (double)r->state;
}
static double pm_random_minmax(pm_rng* r, double mn, double mx) {
    return (mx - mn) * pm_random(r) / (double)2147483647L + mn;
}

/* StgDomain/Swarm/src/RandomParticleLayout.c:194-213: per cell, per point, three draws
 * (x, y, z) in the cell's bounding box. */
void uwr_random_layout(const uwr_mesh* m, int32_t ppc, uint32_t seed, double* xyz) {
    pm_rng r;
    pm_seed(&r, (long)seed);
    int64_t E = uwr_num_elements(m);
    for (int64_t e = 0; e < E; ++e) {
        double nodes[8][3];
        element_node_xyz(m, e, nodes);
        int nen = (m->dim == 3) ? 8 : 4;
        double mn[3] = {nodes[0][0], nodes[0][1], nodes[0][2]};
        double mx[3] = {nodes[nen - 1][0], nodes[nen - 1][1], nodes[nen - 1][2]};
        if (m->dim == 2) { mn[2] = 0.0; mx[2] = 0.0; }
        for (int32_t c = 0; c < ppc; ++c) {
            double* x = xyz + 3 * (e * ppc + c);
            for (int d = 0; d < 3; ++d) x[d] = pm_random_minmax(&r, mn[d], mx[d]);
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* Binning                                                                              */
/* ------------------------------------------------------------------------------------ */

/* StgDomain/Mesh/src/Mesh_RegularAlgorithms.c:154-175 (sep) and :194-226 (search). */
int uwr_search_element(const uwr_mesh* m, const double* pt, uint32_t* el) {
    unsigned inds[3] = {0, 0, 0};
    for (int d = 0; d < m->dim; ++d) {
        double sep = (m->max[d] - m->min[d]) / m->nel[d];
        if (num_approx(pt[d] - m->max[d], 0.0)) {
            inds[d] = (unsigned)(m->nel[d] - 1);
        } else if (pt[d] < m->min[d] || pt[d] > m->max[d]) {
            return 0;
        } else {
            double integer;
            double out = (pt[d] - m->min[d]) / sep;
            double frac = modf(out, &integer);
            inds[d] = (unsigned)integer;
            if (inds[d] > 0 && num_approx(frac, 0.0)) inds[d]--;
        }
    }
    *el = inds[0] + (unsigned)m->nel[0] * (inds[1] + (unsigned)m->nel[1] * inds[2]);
    return 1;
}

/* Velocity at a point: FieldVariable_InterpolateValueAt -> _FeVariable_InterpolateValueAt
 * (StgFEM/Discretisation/src/FeVariable.c:773-800): element search, global->local (Newton), Q1
 * shape functions on the element's nodal values.  u_nodal is node-major (node * dim + d). */
static int velocity_at(const uwr_mesh* m, const double* u_nodal, const double* pt, double* v) {
    uint32_t e;
    if (!uwr_search_element(m, pt, &e)) return 0;
    double xi[3] = {0, 0, 0}, N[8];
    int64_t inc[8];
    uwr_global_to_local(m, e, pt, xi);
    uwr_shape(m->dim, xi, N);
    uwr_element_nodes(m, e, inc);
    int nen = m->dim == 3 ? 8 : 4;
    for (int d = 0; d < m->dim; ++d) {
        v[d] = 0.0;
        for (int a = 0; a < nen; ++a) v[d] += N[a] * u_nodal[inc[a] * m->dim + d];
    }
    return 1;
}

/* Particle advection: _SwarmAdvector_TimeDeriv (PICellerator/MaterialPoints/src/SwarmAdvector.c:
 * 288-314) in TimeIntegrand_FirstOrder (StgDomain/Utils/src/TimeIntegrand.c:221-265,
 * x = x0 + dt v(x0)) or TimeIntegrand_SecondOrder (:267-337: predictor x0 + dt/2 v(x0), then
 * x0 + dt v(predictor); a predictor outside the mesh falls back to the first-order update when
 * allowed).  Points are independent.  Returns the number of points whose velocity could not be
 * found (the reference stops there); such points are left unmoved. */
int64_t uwr_advect(const uwr_mesh* m, const double* u_nodal, int64_t n, double* xyz, double dt, int32_t order,
                   int32_t allow_fallback, int64_t* fallbacks) {
    int64_t failed = 0, fb = 0;
    for (int64_t p = 0; p < n; ++p) {
        double x0[3] = {xyz[p * 3], xyz[p * 3 + 1], xyz[p * 3 + 2]}, v0[3] = {0, 0, 0}, v1[3] = {0, 0, 0};
        if (!velocity_at(m, u_nodal, x0, v0)) {
            failed++;
            continue;
        }
        double x1[3] = {x0[0], x0[1], x0[2]};
        if (order == 1) {
            for (int d = 0; d < m->dim; ++d) x1[d] = x0[d] + dt * v0[d];
        } else {
            double xm[3] = {x0[0], x0[1], x0[2]};
            for (int d = 0; d < m->dim; ++d) xm[d] = x0[d] + 0.5 * dt * v0[d];
            if (velocity_at(m, u_nodal, xm, v1)) {
                for (int d = 0; d < m->dim; ++d) x1[d] = x0[d] + dt * v1[d];
            } else if (allow_fallback) {
                for (int d = 0; d < m->dim; ++d) x1[d] = x0[d] + dt * v0[d];
                fb++;
            } else {
                failed++;
                continue;
            }
        }
        for (int d = 0; d < m->dim; ++d) xyz[p * 3 + d] = x1[d];
    }
    if (fallbacks) *fallbacks = fb;
    return failed;
}

/* PICellerator/MaterialPoints/src/CoincidentMapper.c:176-242 with
 * StgDomain/Swarm/src/SwarmClass.c:1155-1184 (append => ascending point order per cell),
 * StgFEM/Discretisation/src/ElementType.c:227-350 for xi. */
int64_t uwr_map(const uwr_mesh* m, int64_t n, const double* xyz, uint32_t* owning,
                uint32_t* offsets, uint32_t* perm, double* xi, int32_t use_newton) {
    int64_t E = uwr_num_elements(m);
    int64_t outside = 0;
    uint32_t* count = (uint32_t*)calloc((size_t)E, sizeof(uint32_t));
    for (int64_t p = 0; p < n; ++p) {
        uint32_t el;
        if (uwr_search_element(m, xyz + 3 * p, &el)) {
            owning[p] = el;
            count[el]++;
        } else {
            owning[p] = 0xffffffffu;
            outside++;
        }
    }
    offsets[0] = 0;
    for (int64_t e = 0; e < E; ++e) offsets[e + 1] = offsets[e] + count[e];
    memset(count, 0, (size_t)E * sizeof(uint32_t));
    for (int64_t p = 0; p < n; ++p) {
        uint32_t el = owning[p];
        if (el == 0xffffffffu) continue;
        perm[offsets[el] + count[el]++] = (uint32_t)p;
    }
    free(count);
    if (xi) {
        int64_t total = offsets[E];
#pragma omp parallel for schedule(static)
        for (int64_t s = 0; s < total; ++s) {
            /* element of slot s: binary search in offsets */
            int64_t lo = 0, hi = E;
            while (hi - lo > 1) {
                int64_t mid = (lo + hi) / 2;
                if (offsets[mid] <= (uint32_t)s) lo = mid; else hi = mid;
            }
            const double* x = xyz + 3 * (int64_t)perm[s];
            if (use_newton) {
                uwr_global_to_local(m, lo, x, xi + 3 * s);
            } else {
                double nodes[8][3];
                element_node_xyz(m, lo, nodes);
                int nen = (m->dim == 3) ? 8 : 4;
                for (int d = 0; d < 3; ++d) {
                    if (d < m->dim) {
                        double h = nodes[nen - 1][d] - nodes[0][d];
                        xi[3 * s + d] = (2.0 * (x[d] - nodes[0][d]) - h) / h;
                    } else {
                        xi[3 * s + d] = 0.0;
                    }
                }
            }
        }
    }
    return outside;
}

/* ------------------------------------------------------------------------------------ */
/* Shape functions                                                                      */
/* ------------------------------------------------------------------------------------ */

/* StgFEM/Discretisation/src/BilinearElementType.c:212-244 and TrilinearElementType.c:249-306 */
void uwr_shape(int dim, const double* xi, double* N) {
    if (dim == 2) {
        double x = xi[0], y = xi[1];
        N[0] = 0.25 * (1.0 - x) * (1.0 - y);
        N[1] = 0.25 * (1.0 + x) * (1.0 - y);
        N[2] = 0.25 * (1.0 - x) * (1.0 + y);
        N[3] = 0.25 * (1.0 + x) * (1.0 + y);
    } else {
        double x = xi[0], y = xi[1], z = xi[2];
        N[0] = 0.125 * (1.0 - x) * (1.0 - y) * (1.0 - z);
        N[2] = 0.125 * (1.0 - x) * (1.0 + y) * (1.0 - z);
        N[3] = 0.125 * (1.0 + x) * (1.0 + y) * (1.0 - z);
        N[1] = 0.125 * (1.0 + x) * (1.0 - y) * (1.0 - z);
        N[4] = 0.125 * (1.0 - x) * (1.0 - y) * (1.0 + z);
        N[6] = 0.125 * (1.0 - x) * (1.0 + y) * (1.0 + z);
        N[7] = 0.125 * (1.0 + x) * (1.0 + y) * (1.0 + z);
        N[5] = 0.125 * (1.0 + x) * (1.0 - y) * (1.0 + z);
    }
}

void uwr_shape_local_derivs(int dim, const double* xi, double* G) {
    if (dim == 2) {
        double x = xi[0], y = xi[1];
        double* g0 = G;
        double* g1 = G + 4;
        g0[0] = -0.25 * (1.0 - y);
        g0[1] = 0.25 * (1.0 - y);
        g0[3] = 0.25 * (1.0 + y);
        g0[2] = -0.25 * (1.0 + y);
        g1[0] = -0.25 * (1.0 - x);
        g1[1] = -0.25 * (1.0 + x);
        g1[3] = 0.25 * (1.0 + x);
        g1[2] = 0.25 * (1.0 - x);
    } else {
        double x = xi[0], y = xi[1], z = xi[2];
        double* g0 = G;
        double* g1 = G + 8;
        double* g2 = G + 16;
        g0[0] = -0.125 * (1.0 - y) * (1.0 - z);
        g0[2] = -0.125 * (1.0 + y) * (1.0 - z);
        g0[3] = 0.125 * (1.0 + y) * (1.0 - z);
        g0[1] = 0.125 * (1.0 - y) * (1.0 - z);
        g0[4] = -0.125 * (1.0 - y) * (1.0 + z);
        g0[6] = -0.125 * (1.0 + y) * (1.0 + z);
        g0[7] = 0.125 * (1.0 + y) * (1.0 + z);
        g0[5] = 0.125 * (1.0 - y) * (1.0 + z);
        g1[0] = -0.125 * (1.0 - x) * (1.0 - z);
        g1[2] = 0.125 * (1.0 - x) * (1.0 - z);
        g1[3] = 0.125 * (1.0 + x) * (1.0 - z);
        g1[1] = -0.125 * (1.0 + x) * (1.0 - z);
        g1[4] = -0.125 * (1.0 - x) * (1.0 + z);
        g1[6] = 0.125 * (1.0 - x) * (1.0 + z);
        g1[7] = 0.125 * (1.0 + x) * (1.0 + z);
        g1[5] = -0.125 * (1.0 + x) * (1.0 + z);
        g2[0] = -0.125 * (1.0 - x) * (1.0 - y);
        g2[2] = -0.125 * (1.0 - x) * (1.0 + y);
        g2[3] = -0.125 * (1.0 + x) * (1.0 + y);
        g2[1] = -0.125 * (1.0 + x) * (1.0 - y);
        g2[4] = 0.125 * (1.0 - x) * (1.0 - y);
        g2[6] = 0.125 * (1.0 - x) * (1.0 + y);
        g2[7] = 0.125 * (1.0 + x) * (1.0 + y);
        g2[5] = 0.125 * (1.0 + x) * (1.0 - y);
    }
}

/* StgDomain/Geometry/src/TensorMath.c:980-1043 (Cramer's rule; FT3D_ij = row-major). */
static void tensor_solve(const double* A, double* s, const double* b, int dim) {
    if (dim == 3) {
        double det = +A[0] * (A[4] * A[8] - A[7] * A[5])
                     - A[1] * (A[3] * A[8] - A[5] * A[6])
                     + A[2] * (A[3] * A[7] - A[4] * A[6]);
        s[0] = (b[0] * (A[4] * A[8] - A[7] * A[5])
                - A[1] * (b[1] * A[8] - A[5] * b[2])
                + A[2] * (b[1] * A[7] - A[4] * b[2])) / det;
        s[1] = (A[0] * (b[1] * A[8] - b[2] * A[5])
                - b[0] * (A[3] * A[8] - A[5] * A[6])
                + A[2] * (A[3] * b[2] - b[1] * A[6])) / det;
        s[2] = (A[0] * (A[4] * b[2] - A[7] * b[1])
                - A[1] * (A[3] * b[2] - b[1] * A[6])
                + b[0] * (A[3] * A[7] - A[4] * A[6])) / det;
    } else {
        double det = A[0] * A[3] - A[2] * A[1];
        s[0] = (b[0] * A[3] - A[1] * b[1]) / det;
        s[1] = (b[1] * A[0] - A[2] * b[0]) / det;
    }
}

/* StgFEM/Discretisation/src/ElementType.c:227-350 (Newton-Raphson global -> local). */
void uwr_global_to_local(const uwr_mesh* m, int64_t e, const double* x, double* xi) {
    int dim = m->dim, nen = (dim == 3) ? 8 : 4;
    double nodes[8][3], N[8], G[24];
    element_node_xyz(m, e, nodes);
    memset(xi, 0, sizeof(double) * dim);
    for (int it = 0; it < 100; ++it) {
        double J[9] = {0}, rhs[3] = {0}, inc[3] = {0};
        uwr_shape(dim, xi, N);
        uwr_shape_local_derivs(dim, xi, G);
        for (int a = 0; a < nen; ++a) {
            double sf = N[a];
            const double* c = nodes[a];
            J[0 * dim + 0] += G[0 * nen + a] * c[0];
            J[0 * dim + 1] += G[1 * nen + a] * c[0];
            J[1 * dim + 0] += G[0 * nen + a] * c[1];
            J[1 * dim + 1] += G[1 * nen + a] * c[1];
            rhs[0] -= sf * c[0];
            rhs[1] -= sf * c[1];
            if (dim == 3) {
                J[0 * 3 + 2] += G[2 * nen + a] * c[0];
                J[1 * 3 + 2] += G[2 * nen + a] * c[1];
                J[2 * 3 + 0] += G[0 * nen + a] * c[2];
                J[2 * 3 + 1] += G[1 * nen + a] * c[2];
                J[2 * 3 + 2] += G[2 * nen + a] * c[2];
                rhs[2] -= sf * c[2];
            }
        }
        rhs[0] += x[0];
        rhs[1] += x[1];
        if (dim == 3) rhs[2] += x[2];
        tensor_solve(J, inc, rhs, dim);
        xi[0] += inc[0];
        xi[1] += inc[1];
        if (dim == 3) xi[2] += inc[2];
        double mr = fabs(inc[0]);
        if (mr < fabs(inc[1])) mr = fabs(inc[1]);
        if (dim == 3 && mr < fabs(inc[2])) mr = fabs(inc[2]);
        if (mr < 0.0001) return;
    }
    xi[0] = 1.1;
}

/* StgFEM/Discretisation/src/ElementType.c:354-495 (ElementType_ShapeFunctionsGlobalDerivs). */
static void global_derivs_nodes(int dim, double nodes[8][3], const double* xi, double* detJ, double* GNx) {
    int nen = (dim == 3) ? 8 : 4;
    double G[24], jac[3][3], cof[3][3], D = 0.0;
    uwr_shape_local_derivs(dim, xi, G);
    if (dim == 2) {
        jac[0][0] = jac[0][1] = jac[1][0] = jac[1][1] = 0.0;
        for (int n = 0; n < nen; ++n) {
            jac[0][0] = jac[0][0] + G[0 * nen + n] * nodes[n][0];
            jac[0][1] = jac[0][1] + G[0 * nen + n] * nodes[n][1];
            jac[1][0] = jac[1][0] + G[1 * nen + n] * nodes[n][0];
            jac[1][1] = jac[1][1] + G[1 * nen + n] * nodes[n][1];
        }
        D = jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0];
        double tmp = jac[0][0];
        jac[0][0] = jac[1][1] / D;
        jac[1][1] = tmp / D;
        jac[0][1] = -jac[0][1] / D;
        jac[1][0] = -jac[1][0] / D;
    } else {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) jac[i][j] = 0.0;
        for (int n = 0; n < nen; ++n)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) jac[i][j] = jac[i][j] + G[i * nen + n] * nodes[n][j];
        D = jac[0][0] * (jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1])
            - jac[0][1] * (jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0])
            + jac[0][2] * (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]);
        cof[0][0] = jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1];
        cof[1][0] = -(jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0]);
        cof[2][0] = jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0];
        cof[0][1] = -(jac[0][1] * jac[2][2] - jac[0][2] * jac[2][1]);
        cof[1][1] = jac[0][0] * jac[2][2] - jac[0][2] * jac[2][0];
        cof[2][1] = -(jac[0][0] * jac[2][1] - jac[0][1] * jac[2][0]);
        cof[0][2] = jac[0][1] * jac[1][2] - jac[0][2] * jac[1][1];
        cof[1][2] = -(jac[0][0] * jac[1][2] - jac[0][2] * jac[1][0]);
        cof[2][2] = jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) jac[i][j] = cof[i][j] / D;
    }
    *detJ = D;
    for (int dx = 0; dx < dim; ++dx)
        for (int n = 0; n < nen; ++n) {
            double v = 0.0;
            for (int dxi = 0; dxi < dim; ++dxi) v = v + G[dxi * nen + n] * jac[dx][dxi];
            GNx[dx * nen + n] = v;
        }
}

void uwr_global_derivs(const uwr_mesh* m, int64_t e, const double* xi, double* detJ, double* GNx) {
    double nodes[8][3];
    element_node_xyz(m, e, nodes);
    global_derivs_nodes(m->dim, nodes, xi, detJ, GNx);
}

/* ------------------------------------------------------------------------------------ */
/* Rheology                                                                             */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    const uwr_mesh* m;
    const uwr_fields* f;
    int64_t e;
    const int64_t* inc;
    const double* xi;
    const double* N;        /* shape functions at xi */
    const double* GNx;      /* global derivatives at xi */
    double nodes[8][3];
    double point_eta;
    int64_t p;              /* material point index (strain-weakening history) */
} rheo_point;

static double interp_temperature(const rheo_point* rp) {
    int nen = (rp->m->dim == 3) ? 8 : 4;
    double T = 0.0;
    for (int a = 0; a < nen; ++a) T += rp->N[a] * rp->f->temperature[rp->inc[a]];
    return T;
}

/* Underworld/Rheology/src/ConstitutiveMatrixCartesian.c:669-699 (isDiagonal stress) and
 * StgDomain/Geometry/src/TensorMath.c:430-458 (second invariant). */
static double stress_invariant(const rheo_point* rp, double eta) {
    int dim = rp->m->dim, nen = (dim == 3) ? 8 : 4;
    double L[3][3] = {{0}};
    if (rp->f->velocity) {
        for (int a = 0; a < nen; ++a)
            for (int i = 0; i < dim; ++i)
                for (int j = 0; j < dim; ++j)
                    L[i][j] += rp->GNx[j * nen + a] * rp->f->velocity[rp->inc[a] * dim + i];
    }
    if (dim == 3) {
        double sr[6] = {L[0][0], L[1][1], L[2][2], 0.5 * (L[0][1] + L[1][0]),
                        0.5 * (L[0][2] + L[2][0]), 0.5 * (L[1][2] + L[2][1])};
        double st[6] = {2.0 * eta * sr[0], 2.0 * eta * sr[1], 2.0 * eta * sr[2],
                        eta * 2.0 * sr[3], eta * 2.0 * sr[4], eta * 2.0 * sr[5]};
        double inv = 0.5 * (st[0] * st[0] + st[1] * st[1] + st[2] * st[2])
                     + st[3] * st[3] + st[4] * st[4] + st[5] * st[5];
        return sqrt(inv);
    } else {
        double sr[3] = {L[0][0], L[1][1], 0.5 * (L[0][1] + L[1][0])};
        double st[3] = {2.0 * eta * sr[0], 2.0 * eta * sr[1], eta * 2.0 * sr[2]};
        double inv = 0.5 * (st[0] * st[0] + st[1] * st[1]) + st[2] * st[2];
        return sqrt(inv);
    }
}

/* velocity gradient L[i][j] = du_i/dx_j at the point (FeVariable_InterpolateDerivatives_WithGNx) */
static void velocity_gradient(const rheo_point* rp, double L[3][3]) {
    int dim = rp->m->dim, nen = (dim == 3) ? 8 : 4;
    memset(L, 0, 9 * sizeof(double));
    if (!rp->f->velocity) return;
    for (int a = 0; a < nen; ++a)
        for (int i = 0; i < dim; ++i)
            for (int j = 0; j < dim; ++j) L[i][j] += rp->GNx[j * nen + a] * rp->f->velocity[rp->inc[a] * dim + i];
}

/* the Newton terms of _VonMises_HasYielded (VonMises.c:259-268), with the viscosity before the
 * correction, the stored criterion and the stress (2D [xx, yy, xy], 3D [xx, yy, zz, ...]) of the
 * yield indicator */
static void yield_derivs(const rheo_point* rp, double visc0, double crit, double ind, double* derivs) {
    if (!derivs || !rp->f->nl_form_jacobian) return;
    double L[3][3];
    velocity_gradient(rp, L);
    double st[3];
    st[0] = 2.0 * visc0 * L[0][0];
    st[1] = 2.0 * visc0 * L[1][1];
    st[2] = rp->m->dim == 3 ? 2.0 * visc0 * L[2][2] : visc0 * 2.0 * (0.5 * (L[0][1] + L[1][0]));
    double coef = -visc0 * crit / (2.0 * ind * ind * ind);
    derivs[0] += coef * 2.0 * visc0 * st[0];
    derivs[4] += coef * 2.0 * visc0 * st[1];
    derivs[1] += coef * 2.0 * visc0 * st[2];
    derivs[3] += coef * 2.0 * visc0 * st[2];
}

/* ---- eigenvalues of a symmetric stress tensor (StgDomain/Geometry/src/TensorMath.c) ---------
 * Storage: 2D [xx, yy, xy], 3D [xx, yy, zz, xy, xz, yz].  EQL is the reference's absolute
 * comparison |a - b| < 1e-8 (TensorMath.c:760). */
#define UWR_EQL(A, B) (fabs((A) - (B)) < 1.0e-8)
#define UWR_PI 3.14159265358979323846   /* M_PI of math.h */

/* CubicSolver_OnlyRealRoots (TensorMath.c:941-975) */
static void cubic_real_roots(double a2, double a1, double a0, double* root) {
    double Q = (3.0 * a1 - a2 * a2) / 9.0;
    double R = (9.0 * a2 * a1 - 27.0 * a0 - 2.0 * a2 * a2 * a2) / 54.0;
    double D = Q * Q * Q + R * R;
    if (UWR_EQL(D, 0.0)) {
        double halfB = R < 0.0 ? -pow(-R, 1.0 / 3.0) : pow(R, 1.0 / 3.0);
        root[0] = -a2 / 3.0 + 2.0 * halfB;
        root[1] = root[2] = -a2 / 3.0 - halfB;
        return;
    }
    double theta = acos(R / sqrt(-Q * Q * Q)) / 3.0;
    double factor = 2.0 * sqrt(-Q);
    root[0] = factor * cos(theta) - a2 / 3.0;
    root[1] = factor * cos(theta + 2.0 * UWR_PI / 3.0) - a2 / 3.0;
    root[2] = factor * cos(theta + 4.0 * UWR_PI / 3.0) - a2 / 3.0;
}

/* SymmetricTensor_CalcEigenvector3D's test (TensorMath.c:726-758): false when no eigenvector
 * formula applies for this eigenvalue */
static int eigvec3_ok(const double* t, double lam) {
    double A = t[0] - lam, B = t[1] - lam, d = t[3], e = t[4], f = t[5];
    if (!UWR_EQL(B * e, f * d) && !UWR_EQL(e, 0.0)) return 1;
    if (!UWR_EQL(f * A, d * e) && !UWR_EQL(e, 0.0)) return 1;
    if (!UWR_EQL(d * d, B * A) && !UWR_EQL(d, 0.0)) return 1;
    return 0;
}

/* Matrix_CalcAllEigenvectorsJacobi (TensorMath.c:820-909): cyclic Jacobi rotations with the
 * threshold sweeps of Numerical Recipes in C (2nd ed., section 11.1); eigenvalues only */
static void jacobi_eigenvalues3(const double* t, double* ev) {
    double a[3][3] = {{t[0], t[3], t[4]}, {t[3], t[1], t[5]}, {t[4], t[5], t[2]}};
    double b[3], z[3];
    for (int ip = 0; ip < 3; ++ip) {
        b[ip] = ev[ip] = a[ip][ip];
        z[ip] = 0.0;
    }
    for (int sweep = 1; sweep <= 50; ++sweep) {
        double sum = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        if (sum == 0.0) break;
        double tresh = sweep < 4 ? 0.2 * sum / 9.0 : 0.0;
        for (int ip = 0; ip < 2; ++ip)
            for (int iq = ip + 1; iq < 3; ++iq) {
                double g = 100.0 * fabs(a[ip][iq]);
                if (sweep > 4 && (fabs(ev[ip]) + g) == fabs(ev[ip]) && (fabs(ev[iq]) + g) == fabs(ev[iq])) {
                    a[ip][iq] = 0.0;
                } else if (fabs(a[ip][iq]) > tresh) {
                    double h = ev[iq] - ev[ip], tt;
                    if ((double)(fabs(h) + g) == (double)fabs(h)) {
                        tt = a[ip][iq] / h;
                    } else {
                        double theta = 0.5 * h / a[ip][iq];
                        tt = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
                        if (theta < 0.0) tt = -tt;
                    }
                    double c = 1.0 / sqrt(1 + tt * tt), sn = tt * c, tau = sn / (1.0 + c);
                    h = tt * a[ip][iq];
                    z[ip] -= h;
                    z[iq] += h;
                    ev[ip] -= h;
                    ev[iq] += h;
                    a[ip][iq] = 0.0;
                    for (int j = 0; j <= ip - 1; ++j) {
                        double g1 = a[j][ip], h1 = a[j][iq];
                        a[j][ip] = g1 - sn * (h1 + g1 * tau);
                        a[j][iq] = h1 + sn * (g1 - h1 * tau);
                    }
                    for (int j = ip + 1; j <= iq - 1; ++j) {
                        double g1 = a[ip][j], h1 = a[j][iq];
                        a[ip][j] = g1 - sn * (h1 + g1 * tau);
                        a[j][iq] = h1 + sn * (g1 - h1 * tau);
                    }
                    for (int j = iq + 1; j < 3; ++j) {
                        double g1 = a[ip][j], h1 = a[iq][j];
                        a[ip][j] = g1 - sn * (h1 + g1 * tau);
                        a[iq][j] = h1 + sn * (g1 - h1 * tau);
                    }
                }
            }
        for (int ip = 0; ip < 3; ++ip) {
            b[ip] += z[ip];
            ev[ip] = b[ip];
            z[ip] = 0.0;
        }
    }
}

static void sort3(double* v) {
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2 - i; ++j)
            if (v[j] > v[j + 1]) { double t = v[j]; v[j] = v[j + 1]; v[j + 1] = t; }
}

/* SymmetricTensor_CalcAllEigenvectors (TensorMath.c:619-776): ascending eigenvalues */
static void sym_eigenvalues(const double* t, int dim, double* ev) {
    if (dim == 2) {   /* SymmetricTensor_CalcAllEigenvalues2D */
        double r = sqrt(0.25 * (t[0] - t[1]) * (t[0] - t[1]) + t[2] * t[2]);
        double avg = 0.5 * (t[0] + t[1]);
        ev[0] = avg - r;
        ev[1] = avg + r;
        return;
    }
    double a2 = -t[0] - t[1] - t[2];
    double a1 = (t[0] * t[1]) + (t[0] * t[2]) + (t[1] * t[2]) - (t[3] * t[3]) - (t[4] * t[4]) - (t[5] * t[5]);
    double a0 = -(t[0] * t[1] * t[2]) - 2.0 * (t[3] * t[4] * t[5]) + (t[0] * t[5] * t[5]) + (t[1] * t[4] * t[4]) +
                (t[2] * t[3] * t[3]);
    cubic_real_roots(a2, a1, a0, ev);
    for (int i = 0; i < 3; ++i)
        if (!eigvec3_ok(t, ev[i])) {
            jacobi_eigenvalues3(t, ev);
            break;
        }
    sort3(ev);
}

/* deviatoric strain rate at the point (MohrCoulomb.c:355-402: the strain rate with its trace
 * divided among the diagonal removed), symmetric storage */
static void deviatoric_strain_rate(const rheo_point* rp, double* sr) {
    int dim = rp->m->dim, nen = (dim == 3) ? 8 : 4;
    double L[3][3] = {{0}};
    if (rp->f->velocity) {
        for (int a = 0; a < nen; ++a)
            for (int i = 0; i < dim; ++i)
                for (int j = 0; j < dim; ++j)
                    L[i][j] += rp->GNx[j * nen + a] * rp->f->velocity[rp->inc[a] * dim + i];
    }
    if (dim == 3) {
        sr[0] = L[0][0]; sr[1] = L[1][1]; sr[2] = L[2][2];
        sr[3] = 0.5 * (L[0][1] + L[1][0]); sr[4] = 0.5 * (L[0][2] + L[2][0]); sr[5] = 0.5 * (L[1][2] + L[2][1]);
        double tr = sr[0] + sr[1] + sr[2];
        for (int i = 0; i < 3; ++i) sr[i] -= tr / 3.0;
    } else {
        sr[0] = L[0][0]; sr[1] = L[1][1]; sr[2] = 0.5 * (L[0][1] + L[1][0]);
        double tr = sr[0] + sr[1];
        for (int i = 0; i < 2; ++i) sr[i] -= tr / 2.0;
    }
}

/* global coordinate of the point: FeMesh_CoordLocalToGlobal = sum_a N_a(xi) x_a */
static void point_coord(const rheo_point* rp, double* x) {
    int nen = (rp->m->dim == 3) ? 8 : 4;
    for (int d = 0; d < 3; ++d) {
        x[d] = 0.0;
        for (int a = 0; a < nen; ++a) x[d] += rp->N[a] * rp->nodes[a][d];
    }
}

/* second invariant of the strain rate at the point (StrainRateInvariantField:
 * TensorMath.c:430-458 on the symmetric velocity gradient) */
static double strain_rate_invariant(const rheo_point* rp) {
    int dim = rp->m->dim, nen = (dim == 3) ? 8 : 4;
    double L[3][3] = {{0}};
    if (rp->f->velocity) {
        for (int a = 0; a < nen; ++a)
            for (int i = 0; i < dim; ++i)
                for (int j = 0; j < dim; ++j)
                    L[i][j] += rp->GNx[j * nen + a] * rp->f->velocity[rp->inc[a] * dim + i];
    }
    if (dim == 3) {
        double e0 = L[0][0], e1 = L[1][1], e2 = L[2][2], e3 = 0.5 * (L[0][1] + L[1][0]), e4 = 0.5 * (L[0][2] + L[2][0]),
               e5 = 0.5 * (L[1][2] + L[2][1]);
        return sqrt(0.5 * (e0 * e0 + e1 * e1 + e2 * e2) + e3 * e3 + e4 * e4 + e5 * e5);
    }
    double e0 = L[0][0], e1 = L[1][1], e2 = 0.5 * (L[0][1] + L[1][0]);
    return sqrt(0.5 * (e0 * e0 + e1 * e1) + e2 * e2);
}

/* The rheology list of a RheologyMaterial (Underworld/Rheology/src/Rheology_Register.c:61-77).
 * Every law in scope keeps D isotropic, so the constitutive matrix is tracked by eta:
 * SetIsotropicViscosity (ConstitutiveMatrix.c:362-367) sets it, IsotropicCorrection adds to it. */
/* derivs (9, may be NULL): the constitutive matrix's viscosity derivatives of the Newton form
 * (ConstitutiveMatrix.c:362-367 zeroes them with every SetIsotropicViscosity; the VonMises-family
 * _HasYielded adds its terms when the SLE forms the Jacobian, VonMises.c:259-268). */
#define UWR_SET_VISC(v)                                             \
    do {                                                            \
        eta = (v);                                                  \
        if (derivs) memset(derivs, 0, 9 * sizeof(double));          \
    } while (0)
static double run_rheologies(const uwr_material* mat, const rheo_point* rp, double* derivs) {
    double eta = 0.0;
    int dim = rp->m->dim;
    if (derivs) memset(derivs, 0, 9 * sizeof(double));
    for (int l = 0; l < mat->n_laws; ++l) {
        const uwr_law* law = &mat->laws[l];
        switch (law->law) {
        case UWR_LAW_MATERIAL_VISCOSITY: /* MaterialViscosity.c:119-139 */
            UWR_SET_VISC(law->p[0]);
            break;
        case UWR_LAW_ARRHENIUS: { /* Arrhenius.c:156-200 */
            double T = rp->f->temperature ? interp_temperature(rp) : 0.0;
            if (law->p[2] > (0.0 + 1e-12)) {
                int nen = (dim == 3) ? 8 : 4;
                double y = 0.0;
                for (int a = 0; a < nen; ++a) y += rp->N[a] * rp->nodes[a][1];
                double depth = rp->m->max[1] - y;
                UWR_SET_VISC(law->p[0] * exp((law->p[1] + law->p[2] * depth) / (T + law->p[3])));
            } else {
                UWR_SET_VISC(law->p[0] * exp((law->p[1]) / (T + law->p[3])));
            }
            break;
        }
        case UWR_LAW_FRANK_KAMENETSKII: { /* FrankKamenetskii.c:134-152 */
            double T = rp->f->temperature ? interp_temperature(rp) : 0.0;
            UWR_SET_VISC(law->p[0] * exp(-law->p[1] * T));
            break;
        }
        case UWR_LAW_VISCOSITY_LIMITER: { /* ViscosityLimiter.c:106-126 */
            double v = eta;
            if (v > law->p[0]) v = law->p[0];
            if (v < law->p[1]) v = law->p[1];
            UWR_SET_VISC(v);
            break;
        }
        case UWR_LAW_DRUCKER_PRAGER: { /* YieldRheology.c:198-243, VonMises.c:206-269, DruckerPrager.c:236-345 */
            double minVisc = law->p[3];
            if (!rp->f->previous_solution) break;
            double ind = stress_invariant(rp, eta);
            double pressure = rp->f->pressure ? rp->f->pressure[rp->e] : 0.0;
            double phi = atan(law->p[1]);
            double dpFric, dpCoh;
            if (dim == 3) {
                double sinphi = sin(phi);
                double ood = 1.0 / (sqrt(3.0) * (3.0 - sinphi));
                dpFric = 6.0 * sinphi * ood;
                dpCoh = 6.0 * law->p[0] * cos(phi) * ood;
            } else {
                dpCoh = law->p[0] * cos(phi);
                dpFric = sin(phi);
            }
            double crit = dpFric * pressure + dpCoh;
            if (crit < law->p[2]) crit = law->p[2];
            if (crit < ind) {
                double visc0 = eta;
                double beta = 1.0 - crit / ind;
                double corr = -eta * beta;
                if ((eta + corr) < minVisc) corr = minVisc - eta;
                eta += corr;
                yield_derivs(rp, visc0, crit, ind, derivs);
            }
            if (eta < minVisc) UWR_SET_VISC(minVisc);
            break;
        }
        case UWR_LAW_PARTICLE_VISCOSITY:
            UWR_SET_VISC(rp->point_eta);
            break;
        case UWR_LAW_LINEAR_VISCOSITY: { /* LinearViscosity.c:154-190, coordinate by FeMesh_CoordLocalToGlobal */
            double x[3];
            point_coord(rp, x);
            double v = law->p[1] * x[0] + law->p[2] * x[1] + law->p[4] * x[0] * x[1] + law->p[0];
            if (dim == 3)
                v += law->p[3] * x[2] + law->p[5] * x[0] * x[2] + law->p[6] * x[1] * x[2] + law->p[7] * x[0] * x[1] * x[2];
            UWR_SET_VISC(v);
            break;
        }
        case UWR_LAW_DEPTH_DEPENDENT: { /* DepthDependentViscosity.c:165-188 */
            double x[3];
            point_coord(rp, x);
            int axis = (int)law->p[3];
            UWR_SET_VISC(law->p[0] * exp(law->p[1] * (x[axis] - law->p[2])));
            break;
        }
        case UWR_LAW_VON_MISES:     /* YieldRheology.c:198-243 with VonMises.c:175-269 */
        case UWR_LAW_BYERLEE: {     /* Byerlee.c:157-198: criterion cohesion + depthCoefficient (max_y - y) */
            if (!rp->f->previous_solution) break;
            const double minVisc = law->p[2], soft = law->p[3], healing = law->p[4];
            double ind = stress_invariant(rp, eta);                 /* _VonMises_GetYieldIndicator */
            /* StrainWeakening_CalcRatio (StrainWeakening.c:484-503) */
            double pfw = (rp->f->pfw && rp->p >= 0) ? rp->f->pfw[rp->p] : 0.0;
            if (pfw < 0.0) pfw = 0.0;
            double ratio = 0.0;
            if (soft > 0.0) {
                ratio = pfw / soft;
                if (ratio > 1.0) ratio = 1.0;
            }
            double crit;
            if (law->law == UWR_LAW_VON_MISES) {
                crit = law->p[0] * (1.0 - ratio) + law->p[1] * ratio;  /* _VonMises_GetYieldCriterion */
            } else {
                double x[3];
                point_coord(rp, x);
                crit = law->p[0] + law->p[1] * (rp->m->max[1] - x[1]);
            }
            /* StrainWeakening_AssignIncrement -> _StrainWeakening_CalcIncrementIsotropic (:428-481),
             * with the viscosity before the yield correction */
            if (soft > 0.0 && rp->f->pfw_incr && rp->p >= 0) {
                double beta = (crit == 0.0 || ind == 0.0) ? 0.0 : 1.0 - crit / ind;
                rp->f->pfw_incr[rp->p] = beta <= 0.0 ? -healing * pfw
                                                     : (crit / eta) * (beta / (1.0 - beta) - healing * pfw);
            }
            if (crit < ind) {   /* _VonMises_HasYielded */
                double visc0 = eta;
                if (law->p[5] != 0.0) {
                    UWR_SET_VISC(2.0 * crit * crit * eta / (crit * crit + ind * ind));
                } else {
                    double beta = 1.0 - crit / ind;
                    double corr = -eta * beta;
                    if ((eta + corr) < minVisc) corr = minVisc - eta;
                    eta += corr;
                }
                /* the Newton terms use the criterion the law stored; Byerlee's criterion
                 * (Byerlee.c:157-198) stores none, taken as 0 here (no terms) */
                yield_derivs(rp, visc0, law->law == UWR_LAW_VON_MISES ? crit : 0.0, ind, derivs);
            }
            if (eta < minVisc) UWR_SET_VISC(minVisc);
            break;
        }
        case UWR_LAW_MOHR_COULOMB: { /* MohrCoulomb.c:208-402 via YieldRheology.c:198-243 */
            if (!rp->f->previous_solution) break;
            const double minVisc = law->p[5], soft = law->p[6], healing = law->p[7];
            double sr[6], st[6], ev[3];
            deviatoric_strain_rate(rp, sr);
            int ns = dim == 3 ? 6 : 3;
            for (int i = 0; i < ns; ++i) st[i] = 2.0 * eta * sr[i];   /* isotropic D, isDiagonal */
            sym_eigenvalues(st, dim, ev);
            double pfw = (rp->f->pfw && rp->p >= 0) ? rp->f->pfw[rp->p] : 0.0;
            if (pfw < 0.0) pfw = 0.0;
            double ratio = 0.0;
            if (soft > 0.0) {
                ratio = pfw / soft;
                if (ratio > 1.0) ratio = 1.0;
            }
            const double alpha = law->p[2] * (1.0 - ratio) + law->p[3] * ratio;   /* effective friction */
            const double coh = law->p[0] * (1.0 - ratio) + law->p[1] * ratio;     /* effective cohesion */
            /* _MohrCoulomb_GetYieldIndicator */
            double smin = ev[0], smax = dim == 2 ? ev[1] : ev[2];
            double sigma_ns = 0.5 * (smax - smin);
            if (dim == 3) {
                double theta = 0.5 * atan(1.0 / alpha);
                double factor = 1 / (sin(2 * theta) - alpha * cos(2 * theta));
                sigma_ns -= (smax + smin) * 0.5 * alpha * factor;
            }
            double ind = fabs(sigma_ns);
            /* _MohrCoulomb_GetYieldCriterion */
            double pressure = rp->f->pressure ? rp->f->pressure[rp->e] : 0.0;
            double theta = 0.5 * atan(1.0 / alpha);
            double factor = sin(2 * theta);
            double crit = alpha * pressure * factor + coh * factor;
            double minYS = law->p[4] == 0.0 ? coh : law->p[4];
            if (crit < minYS * factor) crit = minYS * factor;
            if (soft > 0.0 && rp->f->pfw_incr && rp->p >= 0) {
                double beta = (crit == 0.0 || ind == 0.0) ? 0.0 : 1.0 - crit / ind;
                rp->f->pfw_incr[rp->p] = beta <= 0.0 ? -healing * pfw
                                                     : (crit / eta) * (beta / (1.0 - beta) - healing * pfw);
            }
            if (crit < ind) {   /* _MohrCoulomb_HasYielded */
                double beta = 1.0 - crit / ind;
                double corr = -eta * beta;
                if ((eta + corr) < minVisc) corr = minVisc - eta;
                eta += corr;
            }
            if (eta < minVisc) UWR_SET_VISC(minVisc);
            break;
        }
        case UWR_LAW_NON_NEWTONIAN: { /* NonNewtonian.c:139-171 */
            double sri = rp->f->previous_solution ? strain_rate_invariant(rp) : law->p[1];
            if (sri == 0) break;
            double n = law->p[0];
            if (fabs(n - 1.0) < 1.0e-10) break;
            UWR_SET_VISC(pow(2.0 * sri, 1.0 / n - 1.0) * pow(eta, 1.0 / n));
            break;
        }
        default:
            break;
        }
    }
    return eta;
}

/* ------------------------------------------------------------------------------------ */
/* Element assembly                                                                     */
/* ------------------------------------------------------------------------------------ */

/* Underworld/Rheology/src/ConstitutiveMatrixCartesian.c:202-412 with the isDiagonal D_B of
 * :556-649.  Accumulates elStiffMat[colDof][rowDof] exactly as the reference loop does. */
static void accumulate_Ke(int dim, int nen, double eta, double factor, const double* GNx, double* Ke) {
    int nd = nen * dim;
    if (dim == 2) {
        double D00 = 2.0 * eta * factor, D11 = 2.0 * eta * factor, D22 = eta * factor;
        for (int r = 0; r < nen; ++r) {
            double dx = GNx[0 * nen + r], dy = GNx[1 * nen + r];
            double DB[3][2] = {{D00 * dx, 0.0}, {0.0, D11 * dy}, {D22 * dy, D22 * dx}};
            for (int c = 0; c < nen; ++c) {
                double bx = GNx[0 * nen + c], by = GNx[1 * nen + c];
                double* K0 = Ke + (c * 2 + 0) * nd + r * 2;
                double* K1 = Ke + (c * 2 + 1) * nd + r * 2;
                K0[0] += bx * DB[0][0] + by * DB[2][0];
                K0[1] += bx * DB[0][1] + by * DB[2][1];
                K1[0] += by * DB[1][0] + bx * DB[2][0];
                K1[1] += by * DB[1][1] + bx * DB[2][1];
            }
        }
    } else {
        double Dn = 2.0 * eta * factor, Ds = eta * factor;
        for (int r = 0; r < nen; ++r) {
            double dx = GNx[0 * nen + r], dy = GNx[1 * nen + r], dz = GNx[2 * nen + r];
            double DB[6][3] = {{Dn * dx, 0.0, 0.0}, {0.0, Dn * dy, 0.0}, {0.0, 0.0, Dn * dz},
                               {Ds * dy, Ds * dx, 0.0}, {Ds * dz, 0.0, Ds * dx}, {0.0, Ds * dz, Ds * dy}};
            for (int c = 0; c < nen; ++c) {
                double bx = GNx[0 * nen + c], by = GNx[1 * nen + c], bz = GNx[2 * nen + c];
                double* K0 = Ke + (c * 3 + 0) * nd + r * 3;
                double* K1 = Ke + (c * 3 + 1) * nd + r * 3;
                double* K2 = Ke + (c * 3 + 2) * nd + r * 3;
                for (int j = 0; j < 3; ++j) {
                    K0[j] += bx * DB[0][j] + by * DB[3][j] + bz * DB[4][j];
                    K1[j] += by * DB[1][j] + bx * DB[3][j] + bz * DB[5][j];
                    K2[j] += bz * DB[2][j] + bx * DB[4][j] + by * DB[5][j];
                }
            }
        }
    }
}

/* The Newton (Jacobian) branch of the 2D element loop, ConstitutiveMatrixCartesian.c:360-383:
 * elStiffMat[col][row] with the viscosity derivatives of the point.  (The reference's Ni term is
 * multiplied by derivs[2] and derivs[5], which no law sets: it is left out.) */
static void accumulate_Ke_jacobian2d(double eta, const double* derivs, double L[3][3], double intFac,
                                     const double* GNx, double* Ke) {
    const int nen = 4, nd = 8;
    double DuDx = L[0][0], DuDy = L[0][1], DvDx = L[1][0], DvDy = L[1][1];
    for (int r = 0; r < nen; ++r) {
        double Bj_x = GNx[0 * nen + r], Bj_y = GNx[1 * nen + r];
        double DetaDu = derivs[0] * Bj_x + derivs[1] * Bj_y;
        double DetaDv = derivs[3] * Bj_x + derivs[4] * Bj_y;
        for (int c = 0; c < nen; ++c) {
            double Bi_x = GNx[0 * nen + c], Bi_y = GNx[1 * nen + c];
            double fac = eta * Bj_y + DuDy * DetaDu + DvDx * DetaDu;
            Ke[(c * 2) * nd + r * 2] += intFac * (2.0 * Bi_x * (eta * Bj_x + DuDx * DetaDu) + Bi_y * fac);
            Ke[(c * 2 + 1) * nd + r * 2] += intFac * (2.0 * Bi_y * DvDy * DetaDu + Bi_x * fac);
            fac = eta * Bj_x + DvDx * DetaDv + DuDy * DetaDv;
            Ke[(c * 2) * nd + r * 2 + 1] += intFac * (2.0 * Bi_x * DuDx * DetaDv + Bi_y * fac);
            Ke[(c * 2 + 1) * nd + r * 2 + 1] += intFac * (2.0 * Bi_y * (eta * Bj_y + DvDy * DetaDv) + Bi_x * fac);
        }
    }
}

/* StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:160-250 on the Gauss swarm
 * (2^dim points at +-1/sqrt(3), unit weights: GaussParticleLayout.c:218-336). */
void uwr_gauss_G(const uwr_mesh* m, int64_t e, double* Ge) {
    int dim = m->dim, nen = (dim == 3) ? 8 : 4, nd = nen * dim;
    double nodes[8][3];
    element_node_xyz(m, e, nodes);
    memset(Ge, 0, sizeof(double) * nd);
    double a = -1.0 / sqrt(3.0);
    double ab[2] = {a, -a};
    int ng = 1 << dim;
    for (int g = 0; g < ng; ++g) {
        double xi[3] = {ab[g & 1], ab[(g >> 1) & 1], ab[(g >> 2) & 1]};
        double detJ, GNx[24];
        global_derivs_nodes(dim, nodes, xi, &detJ, GNx);
        double weight = 1.0;
        for (int r = 0; r < nen; ++r)
            for (int d = 0; d < dim; ++d) Ge[r * dim + d] += +weight * (-detJ) * (GNx[d * nen + r] * 1.0);
    }
}

int uwr_assemble(const uwr_mesh* m, int64_t n, const uint32_t* offsets, const uint32_t* perm,
                 const double* xi, const int32_t* material, const double* point_eta,
                 const double* point_rho, int32_t nmat, const uwr_material* mats,
                 const uwr_fields* f, double* Ke, double* fe, double* Ge, double* Se,
                 double* eta_out, const double* slot_weight, int32_t nthreads) {
    return uwr_assemble_range(m, 0, uwr_num_elements(m), n, offsets, perm, xi, material, point_eta, point_rho,
                              nmat, mats, f, Ke, fe, Ge, Se, eta_out, slot_weight, nthreads);
}

/* uwr_assemble restricted to elements [first, first + count): outputs Ke, fe, Ge, Se are indexed
 * from `first` (element first + i at position i); eta_out stays indexed by slot.  Lets a caller
 * check a large mesh chunk by chunk with bounded memory. */
int uwr_assemble_range(const uwr_mesh* m, int64_t first, int64_t count, int64_t n, const uint32_t* offsets,
                       const uint32_t* perm, const double* xi, const int32_t* material, const double* point_eta,
                       const double* point_rho, int32_t nmat, const uwr_material* mats,
                       const uwr_fields* f, double* Ke, double* fe, double* Ge, double* Se,
                       double* eta_out, const double* slot_weight, int32_t nthreads) {
    (void)n;
    set_threads(nthreads);
    int dim = m->dim, nen = (dim == 3) ? 8 : 4, nd = nen * dim;
    int64_t E = uwr_num_elements(m);
    if (first < 0 || count < 0 || first + count > E) return -2;
    /* WeightsCalculator.c:83 cellLocalVolume = 2^dim; ConstantWeights.c:180-189 */
    const double cellVolume = pow(2.0, (double)dim);
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
    for (int64_t e = first; e < first + count; ++e) {
        const int64_t eo = e - first;   /* output position */
        int64_t inc[8];
        uwr_element_nodes(m, e, inc);
        rheo_point rp;
        rp.m = m;
        rp.f = f;
        rp.e = e;
        rp.inc = inc;
        element_node_xyz(m, e, rp.nodes);
        double* K = Ke ? Ke + eo * nd * nd : NULL;
        double Kloc[576];
        if (!K) K = Kloc;
        memset(K, 0, sizeof(double) * nd * nd);
        double floc[24] = {0};
        uint32_t beg = offsets[e], end = offsets[e + 1];
        uint32_t cnt = end - beg;
        double weight = cellVolume / (double)cnt;
        for (uint32_t s = beg; s < end; ++s) {
            uint32_t p = perm[s];
            const double* x = xi + 3 * (int64_t)s;
            if (slot_weight) weight = slot_weight[s];
            double detJ, GNx[24], N[8];
            global_derivs_nodes(dim, rp.nodes, x, &detJ, GNx);
            uwr_shape(dim, x, N);
            rp.xi = x;
            rp.N = N;
            rp.GNx = GNx;
            rp.point_eta = point_eta ? point_eta[p] : 0.0;
            rp.p = p;
            int32_t mi = material ? material[p] : 0;
            if (mi < 0 || mi >= nmat) { bad |= 1; continue; }
            const uwr_material* mat = &mats[mi];
            double derivs[9];
            double eta = run_rheologies(mat, &rp, derivs);
            if (eta_out) eta_out[s] = eta;
            if (f->nl_form_jacobian && dim == 2) {
                double L[3][3];
                velocity_gradient(&rp, L);
                accumulate_Ke_jacobian2d(eta, derivs, L, detJ * weight, GNx, K);
            } else {
                accumulate_Ke(dim, nen, eta, detJ * weight, GNx, K);
            }
            /* PICellerator/Utils/src/BuoyancyForceTerm.c:374-450 */
            double T = f->temperature ? interp_temperature(&rp) : 0.0;
            double rho0 = point_rho ? point_rho[p] : mat->density;
            double density = rho0 * (1.0 - mat->alpha * (T - mat->ref_temp));
            double force = density * f->gravity;
            double factor = detJ * weight * 1.0 * force;
            for (int a = 0; a < nen; ++a) floc[a * dim + f->vert_axis] += -1.0 * factor * N[a];
        }
        double G[24];
        uwr_gauss_G(m, e, G);
        if (fe) memcpy(fe + eo * nd, floc, sizeof(double) * nd);
        if (Ge) memcpy(Ge + eo * nd, G, sizeof(double) * nd);
        if (Se) {
            /* StgFEM/SLE/ProvidedSystems/StokesFlow/src/UzawaPreconditionerTerm.c:194-214 */
            double s = 0.0;
            for (int v = 0; v < nd; ++v) s += G[v] * (G[v] / K[v * nd + v]);
            Se[eo] = s;
        }
    }
    return bad ? -1 : 0;
}

/* ---- discrete Voronoi cell weights (PICellerator/Weights/src/DVCWeights.c) --------------------
 * An element's local square / cube [-1, 1]^dim carries a fixed grid of res[0] x res[1] (x res[2])
 * cells, x fastest (_DVCWeights_ConstructGrid, :500-594: the cell centres are accumulated from
 * -1 - h/2 by repeated additions of h = 2 / res, as below).  Every point first claims the cell
 * that holds it (cell index = (int)((xi + 1) / h), the upper face folded into the last cell; a
 * later point in the same cell takes it over).  Then the points grow their regions in passes
 * (_DVCWeights_CreateVoronoi, :668-714): in point order, each point tries the cells of its
 * boundary (_DVCWeights_ClaimCells, :261-317).  It takes a free cell, and a cell held by another
 * point when it is strictly nearer to the cell's centre by _DVCWeights_DistanceTest (:604-609,
 * evaluated in the same order: (x1 + x2 - x0 - x0)(x1 - x2) + ... > 0, owner 1, challenger 2,
 * centre 0).  Its boundary becomes the face neighbours of the cells it has just taken that it
 * does not hold (_DVCWeights_UpdateBchain, :395-446).  The passes end when one takes no cell.
 * Weight = cells held x cell volume; the new local coordinate is the mean of the held cells'
 * centres, summed in cell order (_DVCWeights_GetCentroids, :203-231); a point that holds no
 * cell keeps weight 0 and coordinate 0. */
static void dvc_centres(int n, double* c) {
    const double h = 2.0 / n;
    double x = -1.0 - h / 2.0;
    for (int i = 0; i < n; ++i) {
        x = x + h;
        c[i] = x;
    }
}

/* face neighbours of cell c in the order N (y + 1), S (y - 1), E (x + 1), W (x - 1), U (z + 1),
 * D (z - 1); -2 where the grid ends (_DVCWeights_ConstructGrid's links, :510-580) */
static void dvc_neighbours(int c, int nx, int ny, int nz, int q[6]) {
    const int x = c % nx, y = (c / nx) % ny, z = c / (nx * ny);
    q[0] = y < ny - 1 ? c + nx : -2;
    q[1] = y > 0 ? c - nx : -2;
    q[2] = x < nx - 1 ? c + 1 : -2;
    q[3] = x > 0 ? c - 1 : -2;
    q[4] = z < nz - 1 ? c + nx * ny : -2;
    q[5] = z > 0 ? c - nx * ny : -2;
}

void uwr_dvc_grid(int dim, const int32_t res[3], double* centre /* nc*dim */, int32_t* nbr /* nc*2dim */) {
    const int nx = res[0], ny = res[1], nz = dim == 3 ? res[2] : 1;
    double cen[3][64];
    dvc_centres(nx, cen[0]);
    dvc_centres(ny, cen[1]);
    if (dim == 3) dvc_centres(nz, cen[2]);
    for (int c = 0; c < nx * ny * nz; ++c) {
        int q[6];
        dvc_neighbours(c, nx, ny, nz, q);
        for (int k = 0; k < 2 * dim; ++k) nbr[c * 2 * dim + k] = q[k];
        centre[c * dim + 0] = cen[0][c % nx];
        centre[c * dim + 1] = cen[1][(c / nx) % ny];
        if (dim == 3) centre[c * dim + 2] = cen[2][c / (nx * ny)];
    }
}

static double dvc_contest(int dim, const double* c0, const double* p1, const double* p2) {
    double t = (p1[0] + p2[0] - c0[0] - c0[0]) * (p1[0] - p2[0]) + (p1[1] + p2[1] - c0[1] - c0[1]) * (p1[1] - p2[1]);
    if (dim == 3) t = t + (p1[2] + p2[2] - c0[2] - c0[2]) * (p1[2] - p2[2]);
    return t;
}

int uwr_dvc_element(int dim, const int32_t res[3], int32_t nump, const double* xi, double* cxi, double* w) {
    const int nx = res[0], ny = res[1], nz = dim == 3 ? res[2] : 1;
    const int nc = nx * ny * nz;
    if (nx < 1 || ny < 1 || nz < 1 || nx > 64 || ny > 64 || nz > 64 || nc > 4096) return -1;
    double cen[3][64];
    dvc_centres(nx, cen[0]);
    dvc_centres(ny, cen[1]);
    if (dim == 3) dvc_centres(nz, cen[2]);
    const double h[3] = {2.0 / nx, 2.0 / ny, dim == 3 ? 2.0 / nz : 1.0};
    int* owner = (int*)malloc(sizeof(int) * (size_t)nc);
    unsigned char* mark = (unsigned char*)calloc((size_t)nc, 1);
    int* bnd = (int*)malloc(sizeof(int) * (size_t)nc * (size_t)(nump > 0 ? nump : 1));
    int* nbnd = (int*)calloc((size_t)(nump > 0 ? nump : 1), sizeof(int));
    int* took = (int*)malloc(sizeof(int) * (size_t)nc);
    for (int c = 0; c < nc; ++c) owner[c] = -1;
    /* the boundary of p after it took the cells took[0..ntook) */
#define DVC_BOUNDARY(p, ntook)                                                                       \
    do {                                                                                             \
        int* B = bnd + (size_t)(p) * nc;                                                             \
        int nb = 0;                                                                                  \
        for (int t_ = 0; t_ < (ntook); ++t_) {                                                       \
            int q[6];                                                                                \
            dvc_neighbours(took[t_], nx, ny, nz, q);                                                 \
            for (int k_ = 0; k_ < 6; ++k_)                                                           \
                if (q[k_] >= 0 && owner[q[k_]] != (p) && !mark[q[k_]]) {                             \
                    mark[q[k_]] = 1;                                                                 \
                    B[nb++] = q[k_];                                                                 \
                }                                                                                    \
        }                                                                                            \
        for (int k_ = 0; k_ < nb; ++k_) mark[B[k_]] = 0;                                             \
        nbnd[p] = nb;                                                                                \
    } while (0)
    for (int p = 0; p < nump; ++p) {
        int idx[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) {
            const int n = d == 0 ? nx : (d == 1 ? ny : nz);
            idx[d] = (int)((xi[p * dim + d] - -1.0) / h[d]);
            if (idx[d] == n) idx[d]--;
        }
        const int c = idx[0] + nx * (idx[1] + ny * idx[2]);
        owner[c] = p;
        took[0] = c;
        DVC_BOUNDARY(p, 1);
    }
    int passes = 0, taken = nump > 0;
    while (taken) {
        taken = 0;
        ++passes;
        for (int p = 0; p < nump; ++p) {
            const int* B = bnd + (size_t)p * nc;
            int ntook = 0;
            for (int k = 0; k < nbnd[p]; ++k) {
                const int c = B[k];
                int take = 0;
                if (owner[c] == -1) {
                    take = 1;
                } else if (owner[c] != p) {
                    const double c0[3] = {cen[0][c % nx], cen[1][(c / nx) % ny], dim == 3 ? cen[2][c / (nx * ny)] : 0.0};
                    take = dvc_contest(dim, c0, xi + (size_t)owner[c] * dim, xi + (size_t)p * dim) > 0.0;
                }
                if (take) {
                    owner[c] = p;
                    took[ntook++] = c;
                }
            }
            taken += ntook;
            DVC_BOUNDARY(p, ntook);
        }
    }
#undef DVC_BOUNDARY
    const double da = dim == 3 ? h[0] * h[1] * h[2] : h[0] * h[1];
    int* count = (int*)calloc((size_t)(nump > 0 ? nump : 1), sizeof(int));
    for (int p = 0; p < nump * dim; ++p) cxi[p] = 0.0;
    for (int c = 0; c < nc; ++c) {
        const int p = owner[c];
        if (p < 0) continue;
        cxi[p * dim + 0] += cen[0][c % nx];
        cxi[p * dim + 1] += cen[1][(c / nx) % ny];
        if (dim == 3) cxi[p * dim + 2] += cen[2][c / (nx * ny)];
        count[p]++;
    }
    for (int p = 0; p < nump; ++p) {
        w[p] = count[p] * da;
        if (count[p] != 0)
            for (int d = 0; d < dim; ++d) cxi[p * dim + d] /= count[p];
    }
    free(count);
    free(took);
    free(nbnd);
    free(bnd);
    free(mark);
    free(owner);
    return passes;
}

void uwr_dvc_weights(const uwr_mesh* m, const int32_t res[3], const uint32_t* offsets, const double* xi,
                     double* cxi, double* w, int32_t nthreads) {
    set_threads(nthreads);
    const int dim = m->dim;
    const int64_t E = uwr_num_elements(m);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t e = 0; e < E; ++e) {
        const uint32_t beg = offsets[e], n = offsets[e + 1] - beg;
        double pin[3 * 512], pout[3 * 512];
        double* a = n <= 512 ? pin : (double*)malloc(sizeof(double) * 3 * n);
        double* b = n <= 512 ? pout : (double*)malloc(sizeof(double) * 3 * n);
        for (uint32_t i = 0; i < n; ++i)
            for (int d = 0; d < dim; ++d) a[i * dim + d] = xi[3 * (int64_t)(beg + i) + d];
        uwr_dvc_element(dim, res, (int32_t)n, a, b, w + beg);
        for (uint32_t i = 0; i < n; ++i) {
            for (int d = 0; d < dim; ++d) cxi[3 * (int64_t)(beg + i) + d] = b[i * dim + d];
            if (dim == 2) cxi[3 * (int64_t)(beg + i) + 2] = 0.0;
        }
        if (a != pin) free(a);
        if (b != pout) free(b);
    }
}

/* ---- PCDVC population control (PICellerator/Utils/src/PCDVC.c) ----------------------------
 * The non-inflow branch of _PCDVC_Calculate3D (:638-1060) and _PCDVC_Calculate2D (:1063-...),
 * element after element in index order, on the swarm as the cell tables leave it after a
 * CoincidentMapper pass (slot order = cell-table order):
 *   DVC weights of the element's points in cell order; interface cell = its points' materials
 *   differ; boundary cell = the element touches the mesh boundary; maxW / minW = upperT / lowerT
 *   percent of the element's local volume 2^dim; splits: points with w > maxW in cell order,
 *   deletions: points with w < minW sorted by swarm index, largest first (compare_indexOnCPU :621);
 *   interface cells delete nothing unless deleteInInterfaceCells and split nothing unless
 *   splitInInterfaceCells or a boundary cell; maxDeletions > count - 4 becomes count / 2.
 *   A split appends a copy of the point to the swarm and to the cell, at the centroid of the
 *   point's Voronoi region (splitIntParticleByIndexWithinCell :556-619).  A deletion removes the
 *   point from its cell by moving the cell's last entry into its place (Swarm_RemoveParticleFromCell,
 *   StgDomain/Swarm/src/SwarmClass.c:1055-1071) and fills its swarm slot with the swarm's last point,
 *   whose own cell entry is renumbered (deleteIntParticleByIndexOnCPU :451-555).  After any change
 *   the element's DVC is recomputed in its new cell order.  Every integration point ends at the
 *   centroid of its region with the region's volume as weight (:1040-1048).
 * The inflow branch (libc rand()) is not restated.
 * Arrays of capacity `cap` points; returns the new point count, or -1 (cap too small / an empty
 * element), -2 (DVC resolution out of range). */
typedef struct {
    uint32_t* v;
    int64_t n, cap;
} u32vec;
static void u32vec_push(u32vec* a, uint32_t x) {
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 8;
        a->v = (uint32_t*)realloc(a->v, sizeof(uint32_t) * (size_t)a->cap);
    }
    a->v[a->n++] = x;
}
static int64_t u32vec_find(const u32vec* a, uint32_t x) {
    for (int64_t i = 0; i < a->n; ++i)
        if (a->v[i] == x) return i;
    return -1;
}
typedef struct {
    int64_t pos;
    uint32_t index;
} pc_del;
static int pc_del_cmp(const void* A, const void* B) {   /* descending swarm index */
    const pc_del* a = (const pc_del*)A;
    const pc_del* b = (const pc_del*)B;
    return a->index < b->index ? 1 : (a->index > b->index ? -1 : 0);
}

int64_t uwr_pcdvc(const uwr_mesh* m, const int32_t res[3], const uwr_pcdvc_params* pp, int64_t n, int64_t cap,
                  double* xyz, int32_t* material, int64_t* src, const uint32_t* offsets, const uint32_t* perm,
                  const double* xi_slot, uint32_t* offsets_out, uint32_t* perm_out, double* xi_out, double* w_out) {
    const int dim = m->dim;
    const int64_t E = uwr_num_elements(m);
    const double vol = dim == 3 ? 8.0 : 4.0;
    const double maxW = pp->upperT * vol / 100.0, minW = pp->lowerT * vol / 100.0;
    if (cap < n) return -1;
    /* per swarm index: integration xi, owning cell */
    double* pxi = (double*)malloc(sizeof(double) * 3 * (size_t)cap);
    int64_t* cell = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
    u32vec* tab = (u32vec*)calloc((size_t)E, sizeof(u32vec));
    for (int64_t e = 0; e < E; ++e)
        for (uint32_t s = offsets[e]; s < offsets[e + 1]; ++s) {
            uint32_t p = perm[s];
            u32vec_push(&tab[e], p);
            cell[p] = e;
            for (int d = 0; d < 3; ++d) pxi[3 * (int64_t)p + d] = xi_slot[3 * (int64_t)s + d];
        }
    for (int64_t p = 0; p < n; ++p) src[p] = p;
    int64_t count = n;
    int rc = 0;
    double* a = NULL;
    double* cx = NULL;
    double* w = NULL;
    int64_t abuf = 0;
    for (int64_t e = 0; e < E && rc == 0; ++e) {
        int64_t nump = tab[e].n;
        if (nump == 0) { rc = -1; break; }
        if (nump + pp->maxSplits > abuf) {
            abuf = 2 * (nump + pp->maxSplits);
            a = (double*)realloc(a, sizeof(double) * 3 * (size_t)abuf);
            cx = (double*)realloc(cx, sizeof(double) * 3 * (size_t)abuf);
            w = (double*)realloc(w, sizeof(double) * (size_t)abuf);
        }
        for (int64_t i = 0; i < nump; ++i)
            for (int d = 0; d < dim; ++d) a[i * dim + d] = pxi[3 * (int64_t)tab[e].v[i] + d];
        if (uwr_dvc_element(dim, res, (int32_t)nump, a, cx, w) < 0) { rc = -2; break; }
        /* interface and boundary cells */
        int interface = 0;
        for (int64_t i = 1; i < nump; ++i)
            if (material[tab[e].v[i]] != material[tab[e].v[0]]) { interface = 1; break; }
        int64_t ei[3] = {e % m->nel[0], (e / m->nel[0]) % m->nel[1], dim == 3 ? e / ((int64_t)m->nel[0] * m->nel[1]) : 0};
        int boundary = 0;
        for (int d = 0; d < dim; ++d)
            if (ei[d] == 0 || ei[d] == m->nel[d] - 1) boundary = 1;
        int maxDel = pp->maxDeletions, maxSpl = pp->maxSplits;
        if (interface) {
            if (!pp->deleteInInterfaceCells) maxDel = 0;
            if (!pp->splitInInterfaceCells && !boundary) maxSpl = 0;
        }
        int64_t* splits = (int64_t*)malloc(sizeof(int64_t) * (size_t)nump);
        pc_del* dels = (pc_del*)malloc(sizeof(pc_del) * (size_t)nump);
        int64_t ns = 0, nd = 0;
        for (int64_t i = 0; i < nump; ++i) {
            if (w[i] > maxW) splits[ns++] = i;
            if (w[i] < minW) { dels[nd].pos = i; dels[nd].index = tab[e].v[i]; nd++; }
        }
        qsort(dels, (size_t)nd, sizeof(pc_del), pc_del_cmp);
        if (maxDel > nump - 4) maxDel = (int)(nump / 2);
        int changed = 0;
        int64_t cnt = maxSpl > ns ? ns : maxSpl;
        for (int64_t i = 0; i < cnt; ++i) {
            if (count >= cap) { rc = -1; break; }
            int64_t at = splits[i];
            uint32_t from = tab[e].v[at];
            int64_t k = count++;
            for (int d = 0; d < 3; ++d) xyz[3 * k + d] = xyz[3 * (int64_t)from + d];
            material[k] = material[from];
            src[k] = src[from];
            double cxi[3] = {cx[at * dim + 0], cx[at * dim + 1], dim == 3 ? cx[at * dim + 2] : 0.0};
            for (int d = 0; d < 3; ++d) pxi[3 * k + d] = cxi[d];
            /* FeMesh_CoordLocalToGlobal of the centroid */
            double nodes[8][3], N[8];
            element_node_xyz(m, e, nodes);
            uwr_shape(dim, cxi, N);
            for (int d = 0; d < 3; ++d) {
                double v = 0.0;
                for (int q = 0; q < (dim == 3 ? 8 : 4); ++q) v += N[q] * nodes[q][d];
                xyz[3 * k + d] = v;
            }
            cell[k] = e;
            u32vec_push(&tab[e], (uint32_t)k);
            changed = 1;
        }
        int64_t cntd = maxDel > nd ? nd : maxDel;
        for (int64_t i = 0; i < cntd && rc == 0; ++i) {
            uint32_t P = dels[i].index;
            u32vec* t = &tab[cell[P]];
            int64_t pos = u32vec_find(t, P);
            t->v[pos] = t->v[t->n - 1];
            t->n--;
            int64_t L = count - 1;
            if ((int64_t)P != L) {
                for (int d = 0; d < 3; ++d) {
                    xyz[3 * (int64_t)P + d] = xyz[3 * L + d];
                    pxi[3 * (int64_t)P + d] = pxi[3 * L + d];
                }
                /* the moved point keeps the weight its element gave it (when that element was
                   already processed; otherwise the element writes it later under index P) */
                w_out[P] = w_out[L];
                material[P] = material[L];
                src[P] = src[L];
                int64_t f = cell[L];
                cell[P] = f;
                u32vec* tf = &tab[f];
                tf->v[u32vec_find(tf, (uint32_t)L)] = P;
            }
            count--;
            changed = 1;
        }
        free(splits);
        free(dels);
        if (rc) break;
        nump = tab[e].n;
        if (changed) {
            if (nump > abuf) {
                abuf = 2 * nump;
                a = (double*)realloc(a, sizeof(double) * 3 * (size_t)abuf);
                cx = (double*)realloc(cx, sizeof(double) * 3 * (size_t)abuf);
                w = (double*)realloc(w, sizeof(double) * (size_t)abuf);
            }
            for (int64_t i = 0; i < nump; ++i)
                for (int d = 0; d < dim; ++d) a[i * dim + d] = pxi[3 * (int64_t)tab[e].v[i] + d];
            if (uwr_dvc_element(dim, res, (int32_t)nump, a, cx, w) < 0) { rc = -2; break; }
        }
        /* the element's integration points move to their centroids */
        for (int64_t i = 0; i < nump; ++i) {
            int64_t p = tab[e].v[i];
            for (int d = 0; d < dim; ++d) pxi[3 * p + d] = cx[i * dim + d];
        }
        /* weights per point, reordered by slot when the tables are written out */
        for (int64_t i = 0; i < nump; ++i) w_out[tab[e].v[i]] = w[i];
    }
    if (rc == 0) {
        int64_t sidx = 0;
        for (int64_t e = 0; e < E; ++e) {
            offsets_out[e] = (uint32_t)sidx;
            for (int64_t i = 0; i < tab[e].n; ++i, ++sidx) perm_out[sidx] = tab[e].v[i];
        }
        offsets_out[E] = (uint32_t)sidx;
        /* per slot: integration xi and weight (w_out was filled per point index; reorder) */
        double* wtmp = (double*)malloc(sizeof(double) * (size_t)(count > 0 ? count : 1));
        memcpy(wtmp, w_out, sizeof(double) * (size_t)count);
        for (int64_t s = 0; s < sidx; ++s) {
            int64_t p = perm_out[s];
            for (int d = 0; d < 3; ++d) xi_out[3 * s + d] = d < dim ? pxi[3 * p + d] : 0.0;
            w_out[s] = wtmp[p];
        }
        free(wtmp);
    }
    for (int64_t e = 0; e < E; ++e) free(tab[e].v);
    free(tab);
    free(pxi);
    free(cell);
    free(a);
    free(cx);
    free(w);
    return rc ? rc : count;
}

int uwr_assemble_gauss(const uwr_mesh* m, int32_t nmat, const uwr_material* mats,
                       const int32_t* el_material, const uwr_fields* f, double* Ke) {
    int dim = m->dim, nen = (dim == 3) ? 8 : 4, nd = nen * dim;
    int64_t E = uwr_num_elements(m);
    double a = -1.0 / sqrt(3.0);
    double ab[2] = {a, -a};
    int ng = 1 << dim;
    for (int64_t e = 0; e < E; ++e) {
        int64_t inc[8];
        uwr_element_nodes(m, e, inc);
        rheo_point rp;
        rp.m = m;
        rp.f = f;
        rp.e = e;
        rp.inc = inc;
        element_node_xyz(m, e, rp.nodes);
        double* K = Ke + e * nd * nd;
        memset(K, 0, sizeof(double) * nd * nd);
        int32_t mi = el_material ? el_material[e] : 0;
        if (mi < 0 || mi >= nmat) return -1;
        for (int g = 0; g < ng; ++g) {
            double xi[3] = {ab[g & 1], ab[(g >> 1) & 1], ab[(g >> 2) & 1]};
            double detJ, GNx[24], N[8];
            global_derivs_nodes(dim, rp.nodes, xi, &detJ, GNx);
            uwr_shape(dim, xi, N);
            rp.xi = xi;
            rp.N = N;
            rp.GNx = GNx;
            rp.point_eta = 0.0;
            rp.p = -1;
            double eta = run_rheologies(&mats[mi], &rp, NULL);
            accumulate_Ke(dim, nen, eta, detJ * 1.0, GNx, K);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Global system                                                                        */
/* ------------------------------------------------------------------------------------ */

/* StgFEM/Discretisation/src/FeEquationNumber.c:700-760: node order, dof order; BC -> -1. */
int64_t uwr_eqnum(const uwr_mesh* m, const uint8_t* fixed, int64_t* eq) {
    int64_t nn = uwr_num_nodes(m), cur = 0;
    for (int64_t n = 0; n < nn; ++n)
        for (int d = 0; d < m->dim; ++d) {
            int64_t k = n * m->dim + d;
            eq[k] = (fixed && fixed[k]) ? -1 : cur++;
        }
    return cur;
}

typedef struct { int64_t nx, ny, nz; } grid3;
static grid3 node_grid(const uwr_mesh* m) {
    grid3 g = {m->nel[0] + 1, m->nel[1] + 1, (m->dim == 3) ? m->nel[2] + 1 : 1};
    return g;
}

/* Neighbours (incl. self) of node n in ascending index order. */
static int node_neighbours(const uwr_mesh* m, int64_t n, int64_t* nb) {
    grid3 g = node_grid(m);
    int64_t i = n % g.nx, j = (n / g.nx) % g.ny, k = n / (g.nx * g.ny);
    int cnt = 0;
    int kz0 = (m->dim == 3) ? -1 : 0, kz1 = (m->dim == 3) ? 1 : 0;
    for (int dk = kz0; dk <= kz1; ++dk)
        for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
                int64_t ii = i + di, jj = j + dj, kk = k + dk;
                if (ii < 0 || jj < 0 || kk < 0 || ii >= g.nx || jj >= g.ny || kk >= g.nz) continue;
                nb[cnt++] = ii + g.nx * (jj + g.ny * kk);
            }
    return cnt;
}

/* Elements containing node n and the node's local index in each. */
static int node_elements(const uwr_mesh* m, int64_t n, int64_t* els, int* loc) {
    grid3 g = node_grid(m);
    int64_t i = n % g.nx, j = (n / g.nx) % g.ny, k = n / (g.nx * g.ny);
    int cnt = 0;
    int kz0 = (m->dim == 3) ? -1 : 0;
    for (int dk = kz0; dk <= 0; ++dk)
        for (int dj = -1; dj <= 0; ++dj)
            for (int di = -1; di <= 0; ++di) {
                int64_t ei = i + di, ej = j + dj, ek = k + dk;
                if (ei < 0 || ej < 0 || ek < 0 || ei >= m->nel[0] || ej >= m->nel[1]) continue;
                if (m->dim == 3 && ek >= m->nel[2]) continue;
                els[cnt] = ei + m->nel[0] * (ej + m->nel[1] * ek);
                loc[cnt] = (int)((-di) + 2 * (-dj) + ((m->dim == 3) ? 4 * (-dk) : 0));
                cnt++;
            }
    return cnt;
}

int64_t uwr_csr_nnz(const uwr_mesh* m, const int64_t* eq, int64_t nfree, int64_t* rowptr) {
    int64_t nn = uwr_num_nodes(m);
    int dim = m->dim;
    rowptr[0] = 0;
    int64_t r = 0;
    for (int64_t n = 0; n < nn; ++n) {
        int64_t nb[27];
        int nnb = node_neighbours(m, n, nb);
        int cols = 0;
        for (int b = 0; b < nnb; ++b)
            for (int d = 0; d < dim; ++d) cols += eq[nb[b] * dim + d] >= 0;
        for (int d = 0; d < dim; ++d) {
            if (eq[n * dim + d] < 0) continue;
            rowptr[r + 1] = rowptr[r] + cols;
            r++;
        }
    }
    (void)nfree;
    return rowptr[r];
}

/* StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:867-1017: element loop with MatSetValues
 * ADD_VALUES through the location matrix (negative equation numbers dropped).  Restated
 * as a row gather so that rows are built independently. */
void uwr_csr_fill(const uwr_mesh* m, const int64_t* eq, int64_t nfree, const double* Ke,
                  const int64_t* rowptr, int64_t* cols, double* vals, int32_t nthreads) {
    set_threads(nthreads);
    int64_t nn = uwr_num_nodes(m);
    int dim = m->dim, nen = (dim == 3) ? 8 : 4, nd = nen * dim;
    /* first free row of every node */
    int64_t* rowOf = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nn + 1));
    int64_t r = 0;
    for (int64_t n = 0; n < nn; ++n) {
        rowOf[n] = r;
        for (int d = 0; d < dim; ++d) r += eq[n * dim + d] >= 0;
    }
    rowOf[nn] = r;
    (void)nfree;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t n = 0; n < nn; ++n) {
        int64_t nb[27];
        int nnb = node_neighbours(m, n, nb);
        int64_t els[8];
        int loc[8];
        int ne = node_elements(m, n, els, loc);
        int64_t rr = rowOf[n];
        for (int d = 0; d < dim; ++d) {
            if (eq[n * dim + d] < 0) continue;
            int64_t base = rowptr[rr];
            int c = 0;
            for (int b = 0; b < nnb; ++b)
                for (int db = 0; db < dim; ++db) {
                    int64_t q = eq[nb[b] * dim + db];
                    if (q < 0) continue;
                    double v = 0.0;
                    for (int ie = 0; ie < ne; ++ie) {
                        int64_t inc[8];
                        uwr_element_nodes(m, els[ie], inc);
                        for (int a = 0; a < nen; ++a)
                            if (inc[a] == nb[b]) {
                                const double* K = Ke + els[ie] * nd * nd;
                                v += K[(loc[ie] * dim + d) * nd + a * dim + db];
                            }
                    }
                    cols[base + c] = q;
                    vals[base + c] = v;
                    c++;
                }
            rr++;
        }
    }
    free(rowOf);
}

void uwr_csr_spmv(int64_t nrows, const int64_t* rowptr, const int64_t* cols, const double* vals,
                  const double* x, double* y, int32_t nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < nrows; ++r) {
        double s = 0.0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += vals[k] * x[cols[k]];
        y[r] = s;
    }
}

/* ------------------------------------------------------------------------------------ */
/* Sparse matrices for the multigrid restatement                                        */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    int64_t nr, nc;
    int64_t* rp;
    int64_t* ci;
    double* v;
} csr;

static void csr_free(csr* a) {
    free(a->rp);
    free(a->ci);
    free(a->v);
    a->rp = NULL;
    a->ci = NULL;
    a->v = NULL;
}

static void csr_mv(const csr* a, const double* x, double* y) {
#pragma omp parallel for schedule(static) if (a->nr > 20000)
    for (int64_t r = 0; r < a->nr; ++r) {
        double s = 0.0;
        for (int64_t k = a->rp[r]; k < a->rp[r + 1]; ++k) s += a->v[k] * x[a->ci[k]];
        y[r] = s;
    }
}

static csr csr_transpose(const csr* a) {
    csr t;
    t.nr = a->nc;
    t.nc = a->nr;
    t.rp = (int64_t*)calloc((size_t)(t.nr + 1), sizeof(int64_t));
    int64_t nnz = a->rp[a->nr];
    t.ci = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
    t.v = (double*)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    for (int64_t k = 0; k < nnz; ++k) t.rp[a->ci[k] + 1]++;
    for (int64_t r = 0; r < t.nr; ++r) t.rp[r + 1] += t.rp[r];
    int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (size_t)(t.nr + 1));
    memcpy(pos, t.rp, sizeof(int64_t) * (size_t)(t.nr + 1));
    for (int64_t r = 0; r < a->nr; ++r)
        for (int64_t k = a->rp[r]; k < a->rp[r + 1]; ++k) {
            int64_t c = a->ci[k];
            t.ci[pos[c]] = r;
            t.v[pos[c]] = a->v[k];
            pos[c]++;
        }
    free(pos);
    return t;
}

/* Gustavson sparse product C = A B (columns sorted). */
static csr csr_matmul(const csr* A, const csr* B) {
    csr C;
    C.nr = A->nr;
    C.nc = B->nc;
    C.rp = (int64_t*)calloc((size_t)(C.nr + 1), sizeof(int64_t));
    int64_t* mark = (int64_t*)malloc(sizeof(int64_t) * (size_t)B->nc);
    for (int64_t c = 0; c < B->nc; ++c) mark[c] = -1;
    for (int64_t r = 0; r < A->nr; ++r) {
        int64_t cnt = 0;
        for (int64_t k = A->rp[r]; k < A->rp[r + 1]; ++k) {
            int64_t a = A->ci[k];
            for (int64_t q = B->rp[a]; q < B->rp[a + 1]; ++q)
                if (mark[B->ci[q]] != r) { mark[B->ci[q]] = r; cnt++; }
        }
        C.rp[r + 1] = C.rp[r] + cnt;
    }
    int64_t nnz = C.rp[C.nr];
    C.ci = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
    C.v = (double*)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    double* acc = (double*)calloc((size_t)B->nc, sizeof(double));
    for (int64_t c = 0; c < B->nc; ++c) mark[c] = -1;
    for (int64_t r = 0; r < A->nr; ++r) {
        int64_t cnt = 0, base = C.rp[r];
        for (int64_t k = A->rp[r]; k < A->rp[r + 1]; ++k) {
            int64_t a = A->ci[k];
            double av = A->v[k];
            for (int64_t q = B->rp[a]; q < B->rp[a + 1]; ++q) {
                int64_t c = B->ci[q];
                if (mark[c] != r) { mark[c] = r; C.ci[base + cnt++] = c; acc[c] = 0.0; }
                acc[c] += av * B->v[q];
            }
        }
        /* sort columns (insertion sort; rows are short) */
        for (int64_t i = 1; i < cnt; ++i) {
            int64_t key = C.ci[base + i], j = i - 1;
            while (j >= 0 && C.ci[base + j] > key) { C.ci[base + j + 1] = C.ci[base + j]; j--; }
            C.ci[base + j + 1] = key;
        }
        for (int64_t i = 0; i < cnt; ++i) C.v[base + i] = acc[C.ci[base + i]];
    }
    free(mark);
    free(acc);
    return C;
}

/* StgFEM/SLE/SystemSetup/src/SROpGenerator.c:765-1060 (finest level: rows = fine free dofs,
 * columns = every coarse dof node*nDofs+k, weight 1/nPoints over the 2^(#odd indices)
 * coarse nodes) and :1086- (coarser levels: every dof). */
static csr sr_prolongation(const uwr_mesh* fine, const int64_t* fine_eq, int64_t nfine_rows) {
    int dim = fine->dim;
    grid3 gf = node_grid(fine);
    int64_t cnx = fine->nel[0] / 2 + 1, cny = fine->nel[1] / 2 + 1;
    int64_t cnz = (dim == 3) ? fine->nel[2] / 2 + 1 : 1;
    int64_t nfn = gf.nx * gf.ny * gf.nz;
    csr P;
    P.nr = nfine_rows;
    P.nc = cnx * cny * cnz * dim;
    P.rp = (int64_t*)calloc((size_t)(P.nr + 1), sizeof(int64_t));
    P.ci = (int64_t*)malloc(sizeof(int64_t) * (size_t)(P.nr * 8 + 1));
    P.v = (double*)malloc(sizeof(double) * (size_t)(P.nr * 8 + 1));
    int64_t nnz = 0;
    for (int64_t n = 0; n < nfn; ++n) {
        int64_t ind[3] = {n % gf.nx, (n / gf.nx) % gf.ny, n / (gf.nx * gf.ny)};
        int noff[3] = {1, 1, 1};
        for (int d = 0; d < dim; ++d) noff[d] = (ind[d] & 1) ? 2 : 1;
        int npts = noff[0] * noff[1] * noff[2];
        int64_t nodes[8];
        int c = 0;
        for (int oz = 0; oz < noff[2]; ++oz)
            for (int oy = 0; oy < noff[1]; ++oy)
                for (int ox = 0; ox < noff[0]; ++ox) {
                    int64_t ci = (ind[0] >> 1) + ox, cj = (ind[1] >> 1) + oy;
                    int64_t ck = (dim == 3) ? (ind[2] >> 1) + oz : 0;
                    nodes[c++] = ci + cnx * (cj + cny * ck);
                }
        double frac = 1.0 / (double)npts;
        for (int k = 0; k < dim; ++k) {
            int64_t row = fine_eq ? fine_eq[n * dim + k] : n * dim + k;
            if (row < 0) continue;
            P.rp[row + 1] = npts;
            for (int j = 0; j < npts; ++j) {
                P.ci[row * 8 + j] = nodes[j] * dim + k;
                P.v[row * 8 + j] = frac;
            }
        }
    }
    /* compact (rows were laid out with stride 8) */
    for (int64_t r = 0; r < P.nr; ++r) {
        int64_t len = P.rp[r + 1];
        for (int64_t j = 0; j < len; ++j) {
            P.ci[nnz + j] = P.ci[r * 8 + j];
            P.v[nnz + j] = P.v[r * 8 + j];
        }
        /* sort the row */
        for (int64_t i = 1; i < len; ++i) {
            int64_t key = P.ci[nnz + i];
            double kv = P.v[nnz + i];
            int64_t j = i - 1;
            while (j >= 0 && P.ci[nnz + j] > key) { P.ci[nnz + j + 1] = P.ci[nnz + j]; P.v[nnz + j + 1] = P.v[nnz + j]; j--; }
            P.ci[nnz + j + 1] = key;
            P.v[nnz + j + 1] = kv;
        }
        P.rp[r + 1] = nnz + len;
        nnz += len;
    }
    P.rp[0] = 0;
    return P;
}

/* Dense Cholesky of the coarsest operator (PETSc's redundant LU on one rank). */
typedef struct { int64_t n; double* L; } chol;
static int chol_factor(const csr* A, chol* c) {
    int64_t n = A->nr;
    c->n = n;
    c->L = (double*)calloc((size_t)(n * n), sizeof(double));
    for (int64_t r = 0; r < n; ++r)
        for (int64_t k = A->rp[r]; k < A->rp[r + 1]; ++k) c->L[r * n + A->ci[k]] = A->v[k];
    for (int64_t j = 0; j < n; ++j) {
        double d = c->L[j * n + j];
        for (int64_t k = 0; k < j; ++k) d -= c->L[j * n + k] * c->L[j * n + k];
        if (!(d > 0.0)) return -1;
        d = sqrt(d);
        c->L[j * n + j] = d;
#pragma omp parallel for schedule(static)
        for (int64_t i = j + 1; i < n; ++i) {
            double s = c->L[i * n + j];
            for (int64_t k = 0; k < j; ++k) s -= c->L[i * n + k] * c->L[j * n + k];
            c->L[i * n + j] = s / d;
        }
    }
    return 0;
}
static void chol_solve(const chol* c, const double* b, double* x) {
    int64_t n = c->n;
    for (int64_t i = 0; i < n; ++i) {
        double s = b[i];
        for (int64_t k = 0; k < i; ++k) s -= c->L[i * n + k] * x[k];
        x[i] = s / c->L[i * n + i];
    }
    for (int64_t i = n - 1; i >= 0; --i) {
        double s = x[i];
        for (int64_t k = i + 1; k < n; ++k) s -= c->L[k * n + i] * x[k];
        x[i] = s / c->L[i * n + i];
    }
}

/* PCSOR default (SOR_LOCAL_SYMMETRIC_SWEEP, omega = 1): forward then backward Gauss-Seidel. */
static void sor_symmetric(const csr* A, const double* b, double* x, int its) {
    for (int it = 0; it < its; ++it) {
        for (int64_t r = 0; r < A->nr; ++r) {
            double s = b[r], d = 1.0;
            for (int64_t k = A->rp[r]; k < A->rp[r + 1]; ++k) {
                if (A->ci[k] == r) d = A->v[k]; else s -= A->v[k] * x[A->ci[k]];
            }
            x[r] = s / d;
        }
        for (int64_t r = A->nr - 1; r >= 0; --r) {
            double s = b[r], d = 1.0;
            for (int64_t k = A->rp[r]; k < A->rp[r + 1]; ++k) {
                if (A->ci[k] == r) d = A->v[k]; else s -= A->v[k] * x[A->ci[k]];
            }
            x[r] = s / d;
        }
    }
}

typedef struct {
    int nlev;           /* level 0 = coarsest */
    csr A[12];
    csr P[12];          /* P[l]: level l-1 -> level l */
    csr PT[12];
    chol coarse;
    int down, up;
    double* work[12][3];
} mg_t;

/* PETScMGSolver.c:459-549 (Galerkin MatPtAP hierarchy) + PCMG multiplicative V-cycle with
 * Richardson/SOR smoothers (PETScMGSolver.c:641-716). */
static int mg_setup(mg_t* mg, const uwr_mesh* m, const int64_t* eq, const csr* K, int levels, int down, int up) {
    memset(mg, 0, sizeof(*mg));
    /* every coarsening halves each axis: the element counts must stay even down to level 1 */
    {
        uwr_mesh t = *m;
        for (int l = levels - 1; l >= 1; --l)
            for (int d = 0; d < t.dim; ++d) {
                if (t.nel[d] < 2 || (t.nel[d] & 1)) return -3;
                t.nel[d] /= 2;
            }
    }
    mg->nlev = levels;
    mg->down = down;
    mg->up = up;
    int L = levels - 1;
    mg->A[L] = *K;
    uwr_mesh cur = *m;
    for (int l = L; l >= 1; --l) {
        mg->P[l] = sr_prolongation(&cur, (l == L) ? eq : NULL, mg->A[l].nr);
        mg->PT[l] = csr_transpose(&mg->P[l]);
        csr AP = csr_matmul(&mg->A[l], &mg->P[l]);
        mg->A[l - 1] = csr_matmul(&mg->PT[l], &AP);
        csr_free(&AP);
        for (int d = 0; d < cur.dim; ++d) cur.nel[d] /= 2;
    }
    for (int l = 0; l < levels; ++l)
        for (int w = 0; w < 3; ++w) mg->work[l][w] = (double*)calloc((size_t)mg->A[l].nr, sizeof(double));
    return chol_factor(&mg->A[0], &mg->coarse);
}

static void mg_free(mg_t* mg) {
    for (int l = 0; l < mg->nlev; ++l) {
        if (l < mg->nlev - 1) csr_free(&mg->A[l]);
        if (l > 0) { csr_free(&mg->P[l]); csr_free(&mg->PT[l]); }
        for (int w = 0; w < 3; ++w) free(mg->work[l][w]);
    }
    free(mg->coarse.L);
}

static void vcycle(mg_t* mg, int l, const double* b, double* x) {
    if (l == 0) {
        chol_solve(&mg->coarse, b, x);
        return;
    }
    const csr* A = &mg->A[l];
    double* r = mg->work[l][0];
    memset(x, 0, sizeof(double) * (size_t)A->nr);
    sor_symmetric(A, b, x, mg->down);
    csr_mv(A, x, r);
    for (int64_t i = 0; i < A->nr; ++i) r[i] = b[i] - r[i];
    double* bc = mg->work[l - 1][1];
    double* xc = mg->work[l - 1][2];
    csr_mv(&mg->PT[l], r, bc);
    vcycle(mg, l - 1, bc, xc);
    double* t = mg->work[l][1];
    csr_mv(&mg->P[l], xc, t);
    for (int64_t i = 0; i < A->nr; ++i) x[i] += t[i];
    sor_symmetric(A, b, x, mg->up);
}

static double dot(int64_t n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 50000)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* Right-preconditioned FGMRES(restart) (the PETSc KSPFGMRES algorithm, zero initial guess,
 * stop when ||r|| <= rtol*||b||). Returns iterations. */
typedef void (*op_fn)(void* ctx, const double* x, double* y);
static int fgmres(int64_t n, op_fn A, void* actx, op_fn M, void* mctx, const double* b,
                  double* x, double rtol, int restart, int maxit) {
    double** V = (double**)malloc(sizeof(double*) * (size_t)(restart + 1));
    double** Z = (double**)malloc(sizeof(double*) * (size_t)restart);
    for (int i = 0; i <= restart; ++i) V[i] = (double*)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < restart; ++i) Z[i] = (double*)malloc(sizeof(double) * (size_t)n);
    double* H = (double*)calloc((size_t)((restart + 1) * restart), sizeof(double));
    double* cs = (double*)malloc(sizeof(double) * (size_t)restart);
    double* sn = (double*)malloc(sizeof(double) * (size_t)restart);
    double* g = (double*)malloc(sizeof(double) * (size_t)(restart + 1));
    double* w = (double*)malloc(sizeof(double) * (size_t)n);
    memset(x, 0, sizeof(double) * (size_t)n);
    double bnorm = sqrt(dot(n, b, b));
    int its = 0;
    if (bnorm == 0.0) goto done;
    for (;;) {
        A(actx, x, w);
        for (int64_t i = 0; i < n; ++i) V[0][i] = b[i] - w[i];
        double beta = sqrt(dot(n, V[0], V[0]));
        if (beta <= rtol * bnorm || its >= maxit) break;
        for (int64_t i = 0; i < n; ++i) V[0][i] /= beta;
        memset(g, 0, sizeof(double) * (size_t)(restart + 1));
        g[0] = beta;
        int k = 0;
        for (; k < restart && its < maxit; ++k) {
            M(mctx, V[k], Z[k]);
            A(actx, Z[k], w);
            for (int j = 0; j <= k; ++j) {
                double h = dot(n, w, V[j]);
                H[j * restart + k] = h;
                for (int64_t i = 0; i < n; ++i) w[i] -= h * V[j][i];
            }
            double hn = sqrt(dot(n, w, w));
            H[(k + 1) * restart + k] = hn;
            for (int64_t i = 0; i < n; ++i) V[k + 1][i] = w[i] / (hn > 0 ? hn : 1.0);
            for (int j = 0; j < k; ++j) {
                double t = cs[j] * H[j * restart + k] + sn[j] * H[(j + 1) * restart + k];
                H[(j + 1) * restart + k] = -sn[j] * H[j * restart + k] + cs[j] * H[(j + 1) * restart + k];
                H[j * restart + k] = t;
            }
            double a = H[k * restart + k], bb = H[(k + 1) * restart + k];
            double rr = sqrt(a * a + bb * bb);
            cs[k] = a / rr;
            sn[k] = bb / rr;
            H[k * restart + k] = rr;
            H[(k + 1) * restart + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            its++;
            if (fabs(g[k + 1]) <= rtol * bnorm) { k++; break; }
        }
        /* back substitution */
        double y[256];
        for (int i = k - 1; i >= 0; --i) {
            double s = g[i];
            for (int j = i + 1; j < k; ++j) s -= H[i * restart + j] * y[j];
            y[i] = s / H[i * restart + i];
        }
        for (int j = 0; j < k; ++j)
            for (int64_t i = 0; i < n; ++i) x[i] += y[j] * Z[j][i];
        if (fabs(g[k]) <= rtol * bnorm || its >= maxit) break;
    }
done:
    for (int i = 0; i <= restart; ++i) free(V[i]);
    for (int i = 0; i < restart; ++i) free(Z[i]);
    free(V);
    free(Z);
    free(H);
    free(cs);
    free(sn);
    free(g);
    free(w);
    return its;
}

typedef struct {
    csr K, G, GT;
    mg_t mg;
    double a11_rtol;
    int restart, max_inner;
    int64_t inner_its;
    double* Sdiag;
    double* tu;
    double* tu2;
    /* scaled BFBt (Solvers/KSPSolvers/src/BSSCR/pc_ScaledGtKG.c:242-310) */
    int bfbt;
    double bfbt_rtol;
    int bfbt_max_it;
    double* W;      /* 1/rowmax(K), pc_ScaledGtKG.c:735-760 */
    double* gwgd;   /* diag(G^T W G) */
    double *pr, *pz, *pp, *pq, *pt, *pt2, *vs, *vX;
    int64_t bfbt_its;
    int bbt_const;  /* G^T W G has the constant null space (Stokes_Nullspace.c:15-46) */
} bsscr_t;

static void op_K(void* c, const double* x, double* y) { csr_mv(&((bsscr_t*)c)->K, x, y); }
static void op_mg(void* c, const double* x, double* y) {
    bsscr_t* s = (bsscr_t*)c;
    vcycle(&s->mg, s->mg.nlev - 1, x, y);
}
static int a11_solve(bsscr_t* s, const double* b, double* x, double rtol) {
    int its = fgmres(s->K.nr, op_K, s, op_mg, s, b, x, rtol, s->restart, s->max_inner);
    s->inner_its += its;
    return its;
}
/* S v = G^T K^{-1} G v (the positive form; PETSc's MatSchurComplement is its negative). */
static void op_S(void* c, const double* v, double* y) {
    bsscr_t* s = (bsscr_t*)c;
    csr_mv(&s->G, v, s->tu);
    a11_solve(s, s->tu, s->tu2, s->a11_rtol);
    csr_mv(&s->GT, s->tu2, y);
}
static void gwg_apply(bsscr_t* s, const double* x, double* y) {
    csr_mv(&s->G, x, s->vs);
    for (int64_t i = 0; i < s->G.nr; ++i) s->vs[i] *= s->W[i];
    csr_mv(&s->GT, s->vs, y);
}

/* inner KSP of the scaled BFBt preconditioner: Jacobi-preconditioned CG on G^T W G, the
 * right-hand side projected off the constant null space when G^T W G has it
 * (pc_ScaledGtKG.c:266-268, 829-831) */
static void gwg_solve(bsscr_t* s, const double* b, double* x) {
    int64_t n = s->G.nc;
    double mean = 0.0;
    if (s->bbt_const) {
        for (int64_t i = 0; i < n; ++i) mean += b[i];
        mean /= (double)n;
    }
    for (int64_t i = 0; i < n; ++i) { x[i] = 0.0; s->pr[i] = b[i] - mean; }
    double r0 = sqrt(dot(n, s->pr, s->pr));
    if (!(r0 > 0.0)) return;
    for (int64_t i = 0; i < n; ++i) { s->pz[i] = s->pr[i] / s->gwgd[i]; s->pp[i] = s->pz[i]; }
    double rz = dot(n, s->pr, s->pz), rn = r0;
    int it = 0;
    while (it < s->bfbt_max_it && rn > s->bfbt_rtol * r0) {
        gwg_apply(s, s->pp, s->pq);
        double pq = dot(n, s->pp, s->pq);
        if (!(pq > 0.0)) break;
        double alpha = rz / pq;
        for (int64_t i = 0; i < n; ++i) { x[i] += alpha * s->pp[i]; s->pr[i] -= alpha * s->pq[i]; s->pz[i] = s->pr[i] / s->gwgd[i]; }
        double rz2 = dot(n, s->pr, s->pz);
        double beta = rz2 / rz;
        rz = rz2;
        for (int64_t i = 0; i < n; ++i) s->pp[i] = s->pz[i] + beta * s->pp[i];
        rn = sqrt(dot(n, s->pr, s->pr));
        it++;
    }
    s->bfbt_its += it;
}

static void op_Spc(void* c, const double* v, double* y) {
    bsscr_t* s = (bsscr_t*)c;
    if (s->bfbt) {
        /* y = (G^T W G)^-1 G^T W K W G (G^T W G)^-1 v */
        gwg_solve(s, v, s->pt);
        csr_mv(&s->G, s->pt, s->vs);
        for (int64_t i = 0; i < s->G.nr; ++i) s->vs[i] *= s->W[i];
        csr_mv(&s->K, s->vs, s->vX);
        for (int64_t i = 0; i < s->G.nr; ++i) s->vX[i] *= s->W[i];
        csr_mv(&s->GT, s->vX, s->pt2);
        gwg_solve(s, s->pt2, y);
        return;
    }
    for (int64_t i = 0; i < s->G.nc; ++i) y[i] = s->Sdiag ? v[i] / s->Sdiag[i] : v[i];
}

/* Preconditioned CG (PETSc KSPCG), zero initial guess, stopped on the unpreconditioned
 * residual ||r|| <= rtol ||b|| so that every solver here uses the same test. */
static int pcg(int64_t n, op_fn A, void* actx, op_fn M, void* mctx, const double* b, double* x,
               double rtol, int maxit) {
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    double* z = (double*)malloc(sizeof(double) * (size_t)n);
    double* p = (double*)malloc(sizeof(double) * (size_t)n);
    double* q = (double*)malloc(sizeof(double) * (size_t)n);
    memset(x, 0, sizeof(double) * (size_t)n);
    memcpy(r, b, sizeof(double) * (size_t)n);
    M(mctx, r, z);
    double rz = dot(n, r, z), r0 = sqrt(dot(n, r, r));
    memcpy(p, z, sizeof(double) * (size_t)n);
    int it = 0;
    while (it < maxit && sqrt(dot(n, r, r)) > rtol * r0) {
        A(actx, p, q);
        double alpha = rz / dot(n, p, q);
        for (int64_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
        M(mctx, r, z);
        double rz2 = dot(n, r, z);
        double beta = rz2 / rz;
        rz = rz2;
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        it++;
    }
    free(r);
    free(z);
    free(p);
    free(q);
    return it;
}

/* Pressure null-space vectors (ksp_pressure_nullspace.c:23-115): mode 1 the constant, mode 2 the
 * even and odd element-parity indicators (i+j+k even / odd).  A vector is used only when
 * ||G w|| / ||w|| < nstol ||G||_inf with nstol = 1e-7 (BSSCR.c:391, ksp_pressure_nullspace.c:140-170). */
typedef struct {
    int use[2];
    double* w[2];
} nullspace_t;

static void nullspace_setup(nullspace_t* ns, const uwr_mesh* m, const csr* G, int mode) {
    int64_t E = G->nc;
    memset(ns, 0, sizeof(*ns));
    if (mode != 1 && mode != 2) return;
    double ginf = 0.0;
    for (int64_t r = 0; r < G->nr; ++r) {
        double a = 0.0;
        for (int64_t k = G->rp[r]; k < G->rp[r + 1]; ++k) a += fabs(G->v[k]);
        ginf = a > ginf ? a : ginf;
    }
    int nvec = mode == 1 ? 1 : 2;
    double* gw = (double*)malloc(sizeof(double) * (size_t)(G->nr > 0 ? G->nr : 1));
    for (int k = 0; k < nvec; ++k) {
        ns->w[k] = (double*)malloc(sizeof(double) * (size_t)E);
        for (int64_t e = 0; e < E; ++e) {
            if (mode == 1) {
                ns->w[k][e] = 1.0;
            } else {
                int64_t i = e % m->nel[0], j = (e / m->nel[0]) % m->nel[1];
                int64_t l = m->dim == 3 ? e / ((int64_t)m->nel[0] * m->nel[1]) : 0;
                ns->w[k][e] = ((i + j + l) % 2 == k) ? 1.0 : 0.0;
            }
        }
        csr_mv(G, ns->w[k], gw);
        double gn = sqrt(dot(G->nr, gw, gw)), wn = sqrt(dot(E, ns->w[k], ns->w[k]));
        ns->use[k] = wn > 0.0 && gn / wn < 1e-7 * ginf;
    }
    free(gw);
}

static void nullspace_project(const nullspace_t* ns, int64_t n, double* x) {
    for (int k = 0; k < 2; ++k) {
        if (!ns->use[k]) continue;
        double a1 = dot(n, ns->w[k], x), a2 = dot(n, ns->w[k], ns->w[k]);
        for (int64_t i = 0; i < n; ++i) x[i] -= a1 / a2 * ns->w[k][i];
    }
}

static void nullspace_free(nullspace_t* ns) {
    free(ns->w[0]);
    free(ns->w[1]);
}

/* Solvers/KSPSolvers/src/BSSCR/auglag-driver-DGTGD.c:53-441 with penalty 0:
 * h_hat = h - G^T K^{-1} f; Schur solve with the approxS (uw) or gkgdiag preconditioner;
 * constant null-space removal (ksp_pressure_nullspace.c:82-176); back-solve u = K^{-1}(f - G p). */
int uwr_solve_bsscr(const uwr_mesh* m, const uint8_t* fixed, const double* Ke, const double* Ge,
                    const double* fe, const double* Se, const uwr_solve_opts* o,
                    double* u_nodal, double* p, uwr_report* rep) {
    return uwr_solve_bsscr_bc(m, fixed, NULL, Ke, Ge, fe, Se, o, u_nodal, p, rep);
}

/* BSSCR solve with Dirichlet values bcval (nn*dim, read where fixed; NULL: homogeneous).  The
 * element loop lifts the fixed values into both right-hand sides the way __StiffnessMatrix_NewAssemble
 * does (StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:900-925): for the velocity block
 * f_row -= K_e[row][col] bc_col over free rows and fixed columns; for the gradient block, whose
 * transposed right-hand side is the continuity equation's h, h_e -= G_e[row] bc_row over fixed
 * rows.  The Schur right-hand side is then G^T K^-1 f - h, the residual includes h - G^T u, and
 * the returned nodal velocity carries the fixed values. */
int uwr_solve_bsscr_bc(const uwr_mesh* m, const uint8_t* fixed, const double* bcval, const double* Ke,
                       const double* Ge, const double* fe, const double* Se, const uwr_solve_opts* o,
                       double* u_nodal, double* p, uwr_report* rep) {
    set_threads(o->nthreads);
    double t0 = now_s();
    int dim = m->dim, nen = (dim == 3) ? 8 : 4, nd = nen * dim;
    int64_t nn = uwr_num_nodes(m), E = uwr_num_elements(m);
    int64_t* eq = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nn * dim));
    int64_t nfree = uwr_eqnum(m, fixed, eq);
    bsscr_t s;
    memset(&s, 0, sizeof(s));
    s.K.nr = s.K.nc = nfree;
    s.K.rp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nfree + 1));
    int64_t nnz = uwr_csr_nnz(m, eq, nfree, s.K.rp);
    s.K.ci = (int64_t*)malloc(sizeof(int64_t) * (size_t)nnz);
    s.K.v = (double*)malloc(sizeof(double) * (size_t)nnz);
    uwr_csr_fill(m, eq, nfree, Ke, s.K.rp, s.K.ci, s.K.v, o->nthreads);
    /* G: free velocity dofs x elements (P0) */
    s.G.nr = nfree;
    s.G.nc = E;
    s.G.rp = (int64_t*)calloc((size_t)(nfree + 1), sizeof(int64_t));
    {
        int64_t* cnt = s.G.rp;
        for (int64_t e = 0; e < E; ++e) {
            int64_t inc[8];
            uwr_element_nodes(m, e, inc);
            for (int a = 0; a < nen; ++a)
                for (int d = 0; d < dim; ++d) {
                    int64_t q = eq[inc[a] * dim + d];
                    if (q >= 0) cnt[q + 1]++;
                }
        }
        for (int64_t r = 0; r < nfree; ++r) s.G.rp[r + 1] += s.G.rp[r];
        int64_t gn = s.G.rp[nfree];
        s.G.ci = (int64_t*)malloc(sizeof(int64_t) * (size_t)gn);
        s.G.v = (double*)malloc(sizeof(double) * (size_t)gn);
        int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nfree + 1));
        memcpy(pos, s.G.rp, sizeof(int64_t) * (size_t)(nfree + 1));
        for (int64_t e = 0; e < E; ++e) {
            int64_t inc[8];
            uwr_element_nodes(m, e, inc);
            for (int a = 0; a < nen; ++a)
                for (int d = 0; d < dim; ++d) {
                    int64_t q = eq[inc[a] * dim + d];
                    if (q < 0) continue;
                    s.G.ci[pos[q]] = e;
                    s.G.v[pos[q]] = Ge[e * nd + a * dim + d];
                    pos[q]++;
                }
        }
        free(pos);
    }
    s.GT = csr_transpose(&s.G);
    double* f = (double*)calloc((size_t)nfree, sizeof(double));
    for (int64_t e = 0; e < E; ++e) {
        int64_t inc[8];
        uwr_element_nodes(m, e, inc);
        for (int a = 0; a < nen; ++a)
            for (int d = 0; d < dim; ++d) {
                int64_t q = eq[inc[a] * dim + d];
                if (q >= 0) f[q] += fe[e * nd + a * dim + d];
            }
    }
    double* h = (double*)calloc((size_t)(E > 0 ? E : 1), sizeof(double));
    if (bcval) {
        for (int64_t e = 0; e < E; ++e) {
            int64_t inc[8];
            uwr_element_nodes(m, e, inc);
            const double* K = Ke + (size_t)e * nd * nd;
            for (int b = 0; b < nen; ++b)
                for (int d2 = 0; d2 < dim; ++d2) {
                    int64_t gc = inc[b] * dim + d2;
                    if (eq[gc] >= 0) continue;
                    double bc = bcval[gc];
                    int col = b * dim + d2;
                    for (int a = 0; a < nen; ++a)
                        for (int d = 0; d < dim; ++d) {
                            int64_t q = eq[inc[a] * dim + d];
                            if (q >= 0) f[q] -= bc * K[(a * dim + d) * nd + col];
                        }
                    h[e] -= bc * Ge[e * nd + col];
                }
        }
    }
    /* Schur preconditioner diagonal */
    double* Sd = (double*)malloc(sizeof(double) * (size_t)E);
    if (o->schur_pc == 0) {
        memcpy(Sd, Se, sizeof(double) * (size_t)E);
        s.Sdiag = Sd;
    } else if (o->schur_pc == 1) {
        /* BSSCR_FormSchurApproximationDiag: diag(G^T diag(K)^{-1} G) */
        double* kd = (double*)malloc(sizeof(double) * (size_t)nfree);
        for (int64_t r = 0; r < nfree; ++r)
            for (int64_t k = s.K.rp[r]; k < s.K.rp[r + 1]; ++k)
                if (s.K.ci[k] == r) kd[r] = s.K.v[k];
        for (int64_t e = 0; e < E; ++e) {
            double acc = 0.0;
            for (int64_t k = s.GT.rp[e]; k < s.GT.rp[e + 1]; ++k) acc += s.GT.v[k] * s.GT.v[k] / kd[s.GT.ci[k]];
            Sd[e] = acc;
        }
        free(kd);
        s.Sdiag = Sd;
    } else {
        s.Sdiag = NULL;
        if (o->schur_pc == 3) {
            s.bfbt = 1;
            s.bfbt_rtol = o->bfbt_rtol > 0 ? o->bfbt_rtol : 1e-4;
            s.bfbt_max_it = o->bfbt_max_it > 0 ? o->bfbt_max_it : 500;
            s.W = (double*)malloc(sizeof(double) * (size_t)nfree);
            for (int64_t r = 0; r < nfree; ++r) {
                double mx = -1e300;
                for (int64_t k = s.K.rp[r]; k < s.K.rp[r + 1]; ++k) mx = s.K.v[k] > mx ? s.K.v[k] : mx;
                s.W[r] = 1.0 / mx;
            }
            s.gwgd = (double*)calloc((size_t)E, sizeof(double));
            for (int64_t e = 0; e < E; ++e)
                for (int64_t k = s.GT.rp[e]; k < s.GT.rp[e + 1]; ++k) s.gwgd[e] += s.GT.v[k] * s.GT.v[k] * s.W[s.GT.ci[k]];
            double** bufs[] = {&s.pr, &s.pz, &s.pp, &s.pq, &s.pt, &s.pt2};
            for (int b = 0; b < 6; ++b) *bufs[b] = (double*)malloc(sizeof(double) * (size_t)E);
            s.vs = (double*)malloc(sizeof(double) * (size_t)nfree);
            s.vX = (double*)malloc(sizeof(double) * (size_t)nfree);
            /* BSSCR_MatContainsConstNullSpace (Stokes_Nullspace.c:15-46): ||A (1/N)||_2 < 1e-7 */
            for (int64_t e = 0; e < E; ++e) s.pt[e] = 1.0 / (double)E;
            gwg_apply(&s, s.pt, s.pt2);
            s.bbt_const = sqrt(dot(E, s.pt2, s.pt2)) < 1e-7;
        }
    }
    s.a11_rtol = o->a11_rtol;
    s.restart = o->restart > 0 ? o->restart : 30;
    s.max_inner = o->max_inner > 0 ? o->max_inner : 1000;
    s.tu = (double*)malloc(sizeof(double) * (size_t)nfree);
    s.tu2 = (double*)malloc(sizeof(double) * (size_t)nfree);
    int rc = mg_setup(&s.mg, m, eq, &s.K, o->mg_levels, o->smooth_down, o->smooth_up);
    double t1 = now_s();
    if (rc != 0) goto cleanup;

    {
        double* utmp = (double*)malloc(sizeof(double) * (size_t)nfree);
        double* hhat = (double*)malloc(sizeof(double) * (size_t)E);
        a11_solve(&s, f, utmp, o->a11_rtol);
        csr_mv(&s.GT, utmp, hhat);   /* h_hat = h - G^T K^{-1} f */
        for (int64_t e = 0; e < E; ++e) hhat[e] = h[e] - hhat[e];
        /* solve (G^T K^{-1} G) p = -h_hat */
        double* rhs = (double*)malloc(sizeof(double) * (size_t)E);
        for (int64_t e = 0; e < E; ++e) rhs[e] = -hhat[e];
        nullspace_t ns;
        nullspace_setup(&ns, m, &s.G, o->remove_const_p);
        nullspace_project(&ns, E, rhs);
        int outer;
        if (o->schur_type == 0)
            outer = pcg(E, op_S, &s, op_Spc, &s, rhs, p, o->scr_rtol, o->max_outer > 0 ? o->max_outer : 1000);
        else
            outer = fgmres(E, op_S, &s, op_Spc, &s, rhs, p, o->scr_rtol, s.restart, o->max_outer > 0 ? o->max_outer : 1000);
        nullspace_project(&ns, E, p);
        nullspace_free(&ns);
        /* back-solve */
        double* t = (double*)malloc(sizeof(double) * (size_t)nfree);
        csr_mv(&s.G, p, t);
        for (int64_t r = 0; r < nfree; ++r) t[r] = f[r] - t[r];
        int64_t before = s.inner_its;
        a11_solve(&s, t, utmp, o->back_rtol);
        /* true residual */
        double* ku = (double*)malloc(sizeof(double) * (size_t)nfree);
        double* gtu = (double*)malloc(sizeof(double) * (size_t)E);
        csr_mv(&s.K, utmp, ku);
        csr_mv(&s.G, p, t);
        double r2 = 0.0, b2 = dot(nfree, f, f) + dot(E, h, h);
        for (int64_t r = 0; r < nfree; ++r) { double d = f[r] - ku[r] - t[r]; r2 += d * d; }
        csr_mv(&s.GT, utmp, gtu);
        for (int64_t e = 0; e < E; ++e) { double d = h[e] - gtu[e]; r2 += d * d; }
        memset(u_nodal, 0, sizeof(double) * (size_t)(nn * dim));
        for (int64_t k = 0; k < nn * dim; ++k)
            if (eq[k] >= 0) u_nodal[k] = utmp[eq[k]];
            else if (bcval) u_nodal[k] = bcval[k];
        if (rep) {
            rep->outer_its = outer;
            rep->backsolve_its = (int32_t)(s.inner_its - before);
            rep->inner_its_total = (int32_t)s.inner_its;
            rep->rel_residual = sqrt(r2 / (b2 > 0 ? b2 : 1.0));
            rep->converged = 1;
        }
        free(utmp);
        free(hhat);
        free(rhs);
        free(t);
        free(ku);
        free(gtu);
    }
cleanup:
    if (rep) {
        rep->t_setup = t1 - t0;
        rep->t_solve = now_s() - t1;
    }
    mg_free(&s.mg);
    csr_free(&s.K);
    csr_free(&s.G);
    csr_free(&s.GT);
    free(f);
    free(h);
    free(Sd);
    free(s.tu);
    free(s.tu2);
    if (s.bfbt) {
        free(s.W); free(s.gwgd); free(s.pr); free(s.pz); free(s.pp); free(s.pq); free(s.pt); free(s.pt2);
        free(s.vs); free(s.vX);
    }
    free(eq);
    return rc;
}
