/*
 * uwref.h -- CPU restatement of the Underworld 1.x particle-in-cell Stokes hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: the parity tests, the smoke check
 * and the CPU-baseline leg of bench.py call it to check and to time the GPU library.  The
 * product (libuwgpu) never links, loads or calls it.
 *
 * Every routine follows a cited reference routine (paths relative to the Underworld tree).
 * The reference itself cannot be built here (it needs MPI, PETSc 3.5.4, libxml2 and HDF5),
 * so the parity anchor for element assembly is the reference's own golden matrices
 * (Underworld/Rheology/tests/expected/test*.matrix), which this restatement reproduces.
 */
#ifndef UWREF_H
#define UWREF_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Regular Cartesian Q1 mesh (CartesianGenerator without contact depth). */
typedef struct {
    int32_t dim;
    int32_t nel[3];
    double min[3];
    double max[3];
} uwr_mesh;

/* Rheology laws: one entry of a RheologyMaterial's rheology list. */
enum {
    UWR_LAW_NONE = 0,
    UWR_LAW_MATERIAL_VISCOSITY = 1,   /* p[0]=eta0                                         */
    UWR_LAW_ARRHENIUS = 2,            /* p[0]=eta0 p[1]=activationEnergy p[2]=activationVolume p[3]=referenceTemperature */
    UWR_LAW_FRANK_KAMENETSKII = 3,    /* p[0]=eta0 p[1]=theta                              */
    UWR_LAW_VISCOSITY_LIMITER = 4,    /* p[0]=maxViscosity p[1]=minViscosity               */
    UWR_LAW_DRUCKER_PRAGER = 5,       /* p[0]=cohesion p[1]=frictionCoefficient p[2]=minimumYieldStress p[3]=minimumViscosity */
    UWR_LAW_PARTICLE_VISCOSITY = 6,   /* eta = per-point viscosity input                   */
    UWR_LAW_LINEAR_VISCOSITY = 7,     /* p0..p7 = C X Y Z XY XZ YZ XYZ                      */
    UWR_LAW_DEPTH_DEPENDENT = 8,      /* p0=eta0 p1=gamma p2=referencePoint p3=axis         */
    UWR_LAW_NON_NEWTONIAN = 9,        /* p0=stressExponent p1=defaultStrainRateInvariant    */
    UWR_LAW_VON_MISES = 10,           /* p0=cohesion p1=cohesionAfterSoftening p2=minimumViscosity
                                         p3=softeningStrain (<= 0: no strain weakening) p4=healingRate
                                         p5=strainRateSoftening (0/1)                        */
    UWR_LAW_BYERLEE = 11,             /* p0=cohesion p1=depthCoefficient p2=minimumViscosity
                                         p3=softeningStrain p4=healingRate p5=strainRateSoftening */
    UWR_LAW_MOHR_COULOMB = 12         /* p0=cohesion p1=cohesionAfterSoftening p2=frictionCoefficient
                                         p3=frictionCoefficientAfterSoftening p4=minimumYieldStress
                                         p5=minimumViscosity p6=softeningStrain p7=healingRate   */
};

typedef struct {
    int32_t law;
    int32_t pad;
    double p[8];
} uwr_law;

typedef struct {
    int32_t n_laws;
    int32_t pad;
    uwr_law laws[4];
    double density;     /* BuoyancyForceTerm material density                        */
    double alpha;       /* thermal expansivity                                       */
    double ref_temp;    /* BuoyancyForceTerm referenceTemperature                    */
} uwr_material;

/* Fields the rheology chain and the force term may read. */
typedef struct {
    const double* temperature;   /* nodal, nnode (NULL: none)                        */
    const double* velocity;      /* nodal, nnode*dim (NULL: zero)                    */
    const double* pressure;      /* per element, P0 (NULL: zero)                     */
    int32_t previous_solution;   /* YieldRheology yields only if a solve happened    */
    int32_t vert_axis;           /* BuoyancyForceTerm VerticalAxis                   */
    double gravity;              /* BuoyancyForceTerm gravity                        */
    const double* pfw;           /* StrainWeakening postFailureWeakening per point (NULL: 0) */
    double* pfw_incr;            /* out: its time derivative per point (NULL: not written)  */
    int32_t nl_form_jacobian;    /* SystemLinearEquations nlFormJacobian: 2D Newton element matrices */
    int32_t pad;
} uwr_fields;

/* Mesh geometry -------------------------------------------------------------------------- */
int64_t uwr_num_nodes(const uwr_mesh* m);
int64_t uwr_num_elements(const uwr_mesh* m);
void uwr_node_coords(const uwr_mesh* m, double* xyz /* nnode*3 */);
void uwr_element_nodes(const uwr_mesh* m, int64_t e, int64_t* inc /* 2^dim */);

/* Input layouts ------------------------------------------------------------------------ */
/* Park-Miller stream of StgDomain/Swarm/src/Random.c, three draws per point as in
 * RandomParticleLayout; writes points cell by cell (cell order = element order). */
void uwr_random_layout(const uwr_mesh* m, int32_t ppc, uint32_t seed, double* xyz /* E*ppc*3 */);

/* Binning + integration-point mapping --------------------------------------------------- */
int uwr_search_element(const uwr_mesh* m, const double* pt, uint32_t* el);
/* Returns number of points outside the domain (those get owning = 0xffffffff and are skipped). */
int64_t uwr_map(const uwr_mesh* m, int64_t n, const double* xyz /* n*3 */,
                uint32_t* owning /* n */, uint32_t* offsets /* E+1 */, uint32_t* perm /* n */,
                double* xi /* n*3, in perm order */, int32_t use_newton);

/* Shape functions ---------------------------------------------------------------------- */
int64_t uwr_advect(const uwr_mesh* m, const double* u_nodal /* nnode*dim */, int64_t n, double* xyz /* n*3, in/out */,
                   double dt, int32_t order, int32_t allow_fallback, int64_t* fallbacks);
void uwr_shape(int dim, const double* xi, double* N);
void uwr_shape_local_derivs(int dim, const double* xi, double* GNi /* dim*nen */);
void uwr_global_to_local(const uwr_mesh* m, int64_t e, const double* x, double* xi);
void uwr_global_derivs(const uwr_mesh* m, int64_t e, const double* xi, double* detJ, double* GNx /* dim*nen */);

/* Assembly ----------------------------------------------------------------------------- */
/* Per element: Ke (nd*nd, row-major, dof = node*dim+comp), fe (nd), Ge (nd, Gauss swarm),
 * Se (UzawaPreconditionerTerm approxS), eta_out (per point, perm order, may be NULL). */
int uwr_assemble(const uwr_mesh* m, int64_t n, const uint32_t* offsets, const uint32_t* perm,
                 const double* xi, const int32_t* material, const double* point_eta,
                 const double* point_rho, int32_t nmat, const uwr_material* mats,
                 const uwr_fields* f, double* Ke, double* fe, double* Ge, double* Se,
                 double* eta_out, const double* slot_weight /* NULL: constant weights */,
                 int32_t nthreads);
/* uwr_assemble over elements [first, first + count) only; Ke, fe, Ge, Se indexed from first. */
int uwr_assemble_range(const uwr_mesh* m, int64_t first, int64_t count, int64_t n, const uint32_t* offsets,
                       const uint32_t* perm, const double* xi, const int32_t* material, const double* point_eta,
                       const double* point_rho, int32_t nmat, const uwr_material* mats,
                       const uwr_fields* f, double* Ke, double* fe, double* Ge, double* Se,
                       double* eta_out, const double* slot_weight, int32_t nthreads);

/* Discrete Voronoi cell weights (PICellerator/Weights/src/DVCWeights.c) --------------------- */
/* One element: nump points at local coordinates xi[p*dim + d]; res[d] cells per axis
 * (res[0]*res[1](*res[2]) <= 4096).  Out: the new local coordinates (the centroids of the
 * points' discrete Voronoi regions) cxi[p*dim + d] and the weights w[p] (region volume in local
 * coordinates).  Returns the number of growth passes. */
int uwr_dvc_element(int dim, const int32_t res[3], int32_t nump, const double* xi, double* cxi, double* w);
/* The cell grid: centres (nc*dim, accumulated as the reference does) and face neighbours
 * (nc*2*dim: N, S, E, W[, U, D], -2 where the grid ends). */
void uwr_dvc_grid(int dim, const int32_t res[3], double* centre, int32_t* nbr);
/* Every element of the mesh, points in slot order: xi and cxi are [slot][3] (z unused in 2D). */
void uwr_dvc_weights(const uwr_mesh* m, const int32_t res[3], const uint32_t* offsets, const double* xi,
                     double* cxi, double* w, int32_t nthreads);

/* Gauss-swarm element matrices (2^dim Gauss points, unit weights). */
void uwr_gauss_G(const uwr_mesh* m, int64_t e, double* Ge /* nd */);
/* Gauss-swarm isoviscous-like assembly with the given rheology: used by the golden tests. */
int uwr_assemble_gauss(const uwr_mesh* m, int32_t nmat, const uwr_material* mats,
                       const int32_t* el_material, const uwr_fields* f, double* Ke);

/* Global system ------------------------------------------------------------------------ */
/* FeEquationNumber: free dofs numbered in node order; fixed -> -1. Returns #free. */
int64_t uwr_eqnum(const uwr_mesh* m, const uint8_t* fixed /* nnode*dim */, int64_t* eq);
/* CSR of K over free dofs (columns sorted).  Two passes: rowptr/nnz, then cols/vals. */
int64_t uwr_csr_nnz(const uwr_mesh* m, const int64_t* eq, int64_t nfree, int64_t* rowptr);
void uwr_csr_fill(const uwr_mesh* m, const int64_t* eq, int64_t nfree, const double* Ke,
                  const int64_t* rowptr, int64_t* cols, double* vals, int32_t nthreads);

/* BSSCR solve -------------------------------------------------------------------------- */
typedef struct {
    int32_t mg_levels;        /* total levels incl. fine                          */
    int32_t smooth_down, smooth_up;
    int32_t schur_type;       /* 0 = CG, 1 = FGMRES                               */
    int32_t schur_pc;         /* 0 = uw (approxS), 1 = gkgdiag, 2 = none, 3 = scaled BFBt */
    int32_t restart;          /* FGMRES restart                                   */
    int32_t max_outer, max_inner;
    double scr_rtol;          /* -scr_ksp_rtol                                    */
    double a11_rtol;          /* -A11_ksp_rtol                                    */
    double back_rtol;         /* -backsolveA11_ksp_rtol                           */
    int32_t remove_const_p;   /* 1 constant, 2 checkerboard pressure null space     */
    int32_t nthreads;
    double bfbt_rtol;         /* inner G^T W G tolerance of the scaled BFBt PC      */
    int32_t bfbt_max_it;
    int32_t pad;
} uwr_solve_opts;

typedef struct {
    int32_t outer_its, inner_its_total, backsolve_its, converged;
    double rel_residual;      /* ||[f-Ku-Gp; h-G^T u]|| / ||[f;h]||                */
    double t_setup, t_solve;
} uwr_report;

/* PCDVC population control parameters (PICellerator/Utils/src/PCDVC.c:247-284 defaults:
 * upperT 25, lowerT 0.6, maxDeletions 2, maxSplits 3, interface switches False). */
typedef struct {
    double upperT, lowerT;   /* percent of the element's local volume */
    int32_t maxDeletions, maxSplits;
    int32_t splitInInterfaceCells, deleteInInterfaceCells;
} uwr_pcdvc_params;
/* One PCDVC pass (non-inflow branch) over every element; see uwref.c.  xyz (cap*3), material (cap),
 * src (cap: the input point each output point copies) are updated in place; offsets_out (E+1),
 * perm_out, xi_out (3 per slot), w_out (per slot; cap entries of scratch) receive the new cell
 * tables and integration points.  Returns the new point count or a negative error. */
int64_t uwr_pcdvc(const uwr_mesh* m, const int32_t res[3], const uwr_pcdvc_params* pp, int64_t n, int64_t cap,
                  double* xyz, int32_t* material, int64_t* src, const uint32_t* offsets, const uint32_t* perm,
                  const double* xi_slot, uint32_t* offsets_out, uint32_t* perm_out, double* xi_out, double* w_out);

int uwr_solve_bsscr(const uwr_mesh* m, const uint8_t* fixed, const double* Ke, const double* Ge,
                    const double* fe, const double* Se, const uwr_solve_opts* o,
                    double* u_nodal /* nnode*dim */, double* p /* E */, uwr_report* rep);
/* The same with non-zero Dirichlet values (bcval: nn*dim, read where fixed), lifted into f and h as
 * StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:900-925 does. */
int uwr_solve_bsscr_bc(const uwr_mesh* m, const uint8_t* fixed, const double* bcval, const double* Ke,
                       const double* Ge, const double* fe, const double* Se, const uwr_solve_opts* o,
                       double* u_nodal, double* p, uwr_report* rep);

/* Sparse kernels used by the CPU baseline timing. */
void uwr_csr_spmv(int64_t nrows, const int64_t* rowptr, const int64_t* cols, const double* vals,
                  const double* x, double* y, int32_t nthreads);

#ifdef __cplusplus
}
#endif
#endif
