/*
 * uwgpu.h -- C ABI of the GB300 particle-in-cell Stokes library (libuwgpu.so).
 *
 * The library replaces the hot path of an Underworld 1.x Stokes solve:
 *   material point -> element binning and the integration-point mapper,
 *   per-point rheology and Q1 element assembly (K_e, f_e, G_e, approxS_e),
 *   the velocity-block operator and the geometric multigrid inside the BSSCR
 *   Schur-complement solver.
 * Host code (a StGermain component, or any C/C++/Python caller) owns its data in host
 * memory and passes plain pointers; the library copies what it needs into device memory it
 * owns.  Every entry point returns an int status (UWGPU_OK on success) and records a message
 * readable with uwgpu_last_error().  A context is bound to one device and one CUDA stream;
 * calls on one context must not be made from several threads at once.
 *
 * Each declaration names the reference interface it stands in for (paths are relative to
 * the Underworld 1.x source tree).
 */
#ifndef UWGPU_H
#define UWGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UWGPU_ABI_VERSION 2

/* Status codes. */
enum {
    UWGPU_OK = 0,
    UWGPU_ERR_ARGUMENT = 1,      /* bad argument (NULL pointer, size, index)                 */
    UWGPU_ERR_CUDA = 2,          /* a CUDA runtime call failed                               */
    UWGPU_ERR_MEMORY = 3,        /* device allocation failed                                 */
    UWGPU_ERR_STATE = 4,         /* call out of order (e.g. assemble before binning)         */
    UWGPU_ERR_DOMAIN = 5,        /* material points outside the mesh                         */
    UWGPU_ERR_NOT_CONVERGED = 6, /* a Krylov solve hit its iteration limit                   */
    UWGPU_ERR_NAN = 7,           /* NaN/Inf detected in a residual                           */
    UWGPU_ERR_UNSUPPORTED = 8,   /* rheology law or option not provided by this library      */
    UWGPU_ERR_BREAKDOWN = 9,     /* Krylov breakdown (zero pivot / non-SPD coarse operator)  */
    UWGPU_ERR_TOO_LARGE = 10     /* input larger than the fixed scratch of uwgpu_bin_and_map_noalloc */
};

/* Rheology laws (one entry of a RheologyMaterial's rheology list, applied in order). */
enum {
    UWGPU_LAW_MATERIAL_VISCOSITY = 1, /* Underworld/Rheology/src/MaterialViscosity.c:119   p0=eta0 */
    UWGPU_LAW_ARRHENIUS = 2,          /* Underworld/Rheology/src/Arrhenius.c:156          p0=eta0 p1=activationEnergy p2=activationVolume p3=referenceTemperature */
    UWGPU_LAW_FRANK_KAMENETSKII = 3,  /* Underworld/Rheology/src/FrankKamenetskii.c:134   p0=eta0 p1=theta */
    UWGPU_LAW_VISCOSITY_LIMITER = 4,  /* Underworld/Rheology/src/ViscosityLimiter.c:106   p0=maxViscosity p1=minViscosity */
    UWGPU_LAW_DRUCKER_PRAGER = 5,     /* Underworld/Rheology/src/DruckerPrager.c:236 via YieldRheology.c:198, VonMises.c:232
                                         p0=cohesion p1=frictionCoefficient p2=minimumYieldStress p3=minimumViscosity */
    UWGPU_LAW_PARTICLE_VISCOSITY = 6, /* eta taken from the per-point viscosity array passed to uwgpu_particles_upload */
    UWGPU_LAW_LINEAR_VISCOSITY = 7,   /* Underworld/Rheology/src/LinearViscosity.c:154-190  eta = C + X x + Y y + XY x y
                                         (+ Z z + XZ x z + YZ y z + XYZ x y z in 3D); p0..p7 = C X Y Z XY XZ YZ XYZ */
    UWGPU_LAW_DEPTH_DEPENDENT = 8,    /* Underworld/Rheology/src/DepthDependentViscosity.c:165-188  eta = eta0 exp(gamma (x_axis - referencePoint));
                                         p0=eta0 p1=gamma p2=referencePoint p3=variationAxis (0, 1, 2) */
    UWGPU_LAW_NON_NEWTONIAN = 9,      /* Underworld/Rheology/src/NonNewtonian.c:139-171  eta = (2 e_II)^(1/n - 1) eta^(1/n), e_II the point's
                                         strain-rate invariant (defaultStrainRateInvariant before the first solve);
                                         p0=stressExponent p1=defaultStrainRateInvariant */
    UWGPU_LAW_VON_MISES = 10,         /* Underworld/Rheology/src/VonMises.c:175-269 via YieldRheology.c:198-243, with the
                                         StrainWeakening of its cohesion (StrainWeakening.c:428-503); p0=cohesion
                                         p1=cohesionAfterSoftening p2=minimumViscosity p3=softeningStrain (<= 0: no weakening)
                                         p4=healingRate p5=strainRateSoftening (0/1) */
    UWGPU_LAW_BYERLEE = 11,           /* Underworld/Rheology/src/Byerlee.c:157-198: the VonMises law with the yield stress
                                         cohesion + depthCoefficient (max_y - y); p0=cohesion p1=depthCoefficient, p2..p5 as
                                         for VON_MISES (p3, p4: the strain-weakening history it updates) */
    UWGPU_LAW_MOHR_COULOMB = 12       /* Underworld/Rheology/src/MohrCoulomb.c:208-402: indicator from the principal stresses
                                         of the deviatoric strain rate's stress, criterion (C + mu p) sin 2 theta; p0=cohesion
                                         p1=cohesionAfterSoftening p2=frictionCoefficient p3=frictionCoefficientAfterSoftening
                                         p4=minimumYieldStress (0: the effective cohesion) p5=minimumViscosity
                                         p6=softeningStrain (<= 0: no weakening) p7=healingRate */
};

typedef struct {
    int32_t law;
    int32_t pad;
    double p[8];
} uwgpu_law;

/* One RheologyMaterial (Underworld/Rheology/src/RheologyMaterial.c:240-270) plus the
 * BuoyancyForceTerm material extension (PICellerator/Utils/src/BuoyancyForceTerm.c:217-221). */
typedef struct {
    int32_t n_laws;     /* 1..4 */
    int32_t pad;
    uwgpu_law laws[4];
    double density;
    double alpha;
    double ref_temp;
} uwgpu_material;

/* Solver options: the PETSc options the BSSCR driver reads
 * (Solvers/KSPSolvers/src/BSSCR/auglag-driver-DGTGD.c, mg.c; StgFEM PETScMGSolver.c). */
enum { UWGPU_PREC_FP64 = 0, UWGPU_PREC_MIXED = 1 };
enum { UWGPU_SCHUR_CG = 0, UWGPU_SCHUR_FGMRES = 1 };
/* Schur preconditioners (-Q22_pc_type): uw = approxS of UzawaPreconditionerTerm; gkgdiag =
 * diag(G^T diag(K)^-1 G); scaled BFBt = the "gtkg" preconditioner of
 * Solvers/KSPSolvers/src/BSSCR/pc_ScaledGtKG.c:242-310, (G^T W G)^-1 (G^T W K W G) (G^T W G)^-1 with
 * W = 1/rowmax(K), whose inner G^T W G solves are Jacobi-preconditioned CG. */
enum { UWGPU_SCHUR_PC_UW = 0, UWGPU_SCHUR_PC_GKGDIAG = 1, UWGPU_SCHUR_PC_NONE = 2, UWGPU_SCHUR_PC_SCALED_BFBT = 3 };

/* Multigrid smoothers: symmetric multicolour block Gauss-Seidel (the colour-scheduled form of
 * the reference's Richardson/SOR level smoother, PETScMGSolver.c:674-709), or Chebyshev
 * iteration on the block-Jacobi preconditioned operator (PETSc KSPCHEBYSHEV, eigenvalue bounds
 * [0.1, 1.1] x the power-iteration estimate). */
enum { UWGPU_SMOOTHER_COLOUR_GS = 0, UWGPU_SMOOTHER_CHEBYSHEV = 1 };

typedef struct {
    int32_t mg_levels;        /* mgLevels: levels including the fine one (>= 2)          */
    int32_t smooth_down;      /* downIterations: symmetric colour sweeps before restrict  */
    int32_t smooth_up;        /* upIterations                                            */
    int32_t schur_type;       /* -scr_ksp_type: UWGPU_SCHUR_CG or UWGPU_SCHUR_FGMRES      */
    int32_t schur_pc;         /* -Q22_pc_type: uw (approxS), gkgdiag, none               */
    int32_t restart;          /* FGMRES restart length (PETSc default 30)                */
    int32_t max_outer;        /* -scr_ksp_max_it                                         */
    int32_t max_inner;        /* -A11_ksp_max_it (per velocity solve)                    */
    double scr_rtol;          /* -scr_ksp_rtol                                           */
    double a11_rtol;          /* -A11_ksp_rtol                                           */
    double back_rtol;         /* -backsolveA11_ksp_rtol                                  */
    int32_t remove_const_p;   /* pressure null space projected out of the Schur rhs and p:
                                 0 none, 1 constant (-remove_constant_pressure_null_space),
                                 2 even/odd element parity (-remove_checkerboard_pressure_null_space);
                                 a vector is used only when ||G w||/||w|| < 1e-7 ||G||_inf
                                 (ksp_pressure_nullspace.c:23-176, BSSCR.c:330-347)            */
    int32_t precision;        /* UWGPU_PREC_FP64 or UWGPU_PREC_MIXED                     */
    double target_rel_residual; /* > 0: the report's status is UWGPU_ERR_NOT_CONVERGED when the
                                   full Stokes residual ||[f-Ku-Gp; h-G^T u]|| / ||[f;h]|| after
                                   the solve is above this value (a check, not a stopping rule) */
    double bfbt_rtol;         /* inner G^T W G solve tolerance of the scaled BFBt preconditioner */
    int32_t bfbt_max_it;      /* inner iteration limit of those solves                   */
    int32_t smoother;         /* UWGPU_SMOOTHER_COLOUR_GS (default) or UWGPU_SMOOTHER_CHEBYSHEV:
                                 smooth_down/up are then polynomial degrees              */
    int32_t learned_pc;       /* 1: velocity preconditioner V-cycle + trained U-Net correction
                                 (uwgpu_learned_*), 0: V-cycle only (default)                */
    int32_t learned_stagnation; /* consecutive velocity iterations with < 5% residual reduction
                                 after which a velocity solve drops the U-Net (default 2)    */
    int32_t mg_cycle;         /* coarse corrections per level visit: 1 V-cycle (default), 2 W-cycle
                                 (-pc_mg_cycle_type v|w of the velocity PCMG)                */
    int32_t bfbt_inner_pc;    /* preconditioner of the scaled BFBt inner G^T W G solves: 0 Jacobi (default,
                                 as the reference's KSP; the mixed form reads the FP32 stencil
                                 while it fits in half of L2, else applies G^T W G matrix-free),
                                 1 aggregation multigrid V-cycle, 2 Jacobi on the FP32 stencil,
                                 3 Jacobi with the matrix-free FP32 apply (2, 3: mixed form),
                                 4 Jacobi plus an additive coarse correction on the element
                                 checkerboards of single planes, Q1-P0's near-null pressure
                                 modes (3D; the operator form chosen as for 0; 2D: as 0).  No
                                 reference counterpart: the reference's inner KSP is Jacobi. */
} uwgpu_solve_opts;

typedef struct {
    int32_t outer_its;        /* Schur (pressure) iterations                             */
    int32_t inner_its_total;  /* velocity (A11) Krylov iterations, all solves            */
    int32_t backsolve_its;    /* iterations of the final velocity back-solve             */
    int32_t vcycles;          /* multigrid V-cycles applied                              */
    int32_t converged;
    int32_t status;
    double rel_residual;      /* ||[f-Ku-Gp; h-G^T u]|| / ||[f;h]|| of the returned u, p  */
    double t_setup_ms;        /* stencil build + multigrid hierarchy                     */
    double t_solve_ms;
    int64_t pc_inner_its;     /* inner iterations of the Schur preconditioner (scaled BFBt) */
    int32_t learned_applies;  /* U-Net corrections applied                                  */
    int32_t learned_fallbacks; /* velocity solves that fell back to the plain V-cycle       */
} uwgpu_report;

typedef struct uwgpu_ctx uwgpu_ctx;

/* Lifetime ------------------------------------------------------------------------------ */
/* The GPU components create their context in their Build phase and free it in their Destroy
 * phase (Stg_Component_Build / Stg_Component_Destroy, StGermain/Base/Automation/src/
 * Stg_Component.c:228,339); the last error message is what they pass to Journal_Firewall
 * (StGermain/Base/IO/src/Journal.c:519).  uwgpu_abi_version and uwgpu_synchronize have no
 * reference counterpart. */
int uwgpu_abi_version(void);
/* Creates a context on `device` with its own stream. */
int uwgpu_create(int32_t device, uwgpu_ctx** out);
void uwgpu_destroy(uwgpu_ctx* ctx);
const char* uwgpu_last_error(const uwgpu_ctx* ctx);
int uwgpu_synchronize(uwgpu_ctx* ctx);

/* Mesh: regular Cartesian Q1 mesh of CartesianGenerator (StgDomain/Mesh/src/CartesianGenerator.c
 * :976-1035 incidence, :2275-2310 coordinates) with a P0 pressure mesh. */
int uwgpu_mesh_q1(uwgpu_ctx* ctx, int32_t dim, const int32_t nel[3], const double min[3],
                  const double max[3]);

/* Velocity boundary conditions: fixed[n*dim+d] != 0 fixes dof d of node n to values[n*dim+d]
 * (values may be NULL for homogeneous conditions).  Replaces the WallVC/CompositeVC lookup
 * the equation numbering uses (StgFEM/Discretisation/src/FeEquationNumber.c:700-760). */
int uwgpu_bc_set(uwgpu_ctx* ctx, const uint8_t* fixed, const double* values);

/* Materials: device-side descriptors of the Materials_Register walk the constitutive matrix
 * does at build time (Underworld/Rheology/src/ConstitutiveMatrix.c:214-243). */
int uwgpu_materials_set(uwgpu_ctx* ctx, int32_t n, const uwgpu_material* mats);

/* Fields the rheology and force terms read (Ppc lookups, PICellerator/Common/src/PpcManager.c:503):
 * nodal temperature (may be NULL), gravity magnitude, vertical axis (BuoyancyForceTerm
 * VerticalAxis).  Velocity and pressure for strain-rate and pressure dependent laws are the
 * context's last solution (see uwgpu_solution_set). */
int uwgpu_fields_set(uwgpu_ctx* ctx, const double* nodal_temperature, double gravity,
                     int32_t vert_axis);
/* Sets the current solution (nodal velocity nnode*dim, element pressure) used by
 * strain-rate / pressure dependent rheologies; marks a previous solution as present
 * (ConstitutiveMatrix previousSolutionExists, Underworld/Rheology/src/YieldRheology.c:210). */
int uwgpu_solution_set(uwgpu_ctx* ctx, const double* u_nodal, const double* p);

/* Material points: coordinates as three arrays (x, y, z; z ignored in 2D), material index per
 * point, optional per-point viscosity and density (NULL if unused).  Copied to the device.
 * Stands in for the MaterialPointsSwarm particle array (PICellerator/MaterialPoints). */
int uwgpu_particles_upload(uwgpu_ctx* ctx, int64_t n, const double* x, const double* y,
                           const double* z, const int32_t* material, const double* eta,
                           const double* rho);

/* Strain-weakening history of the material points (the postFailureWeakening particle variable of
 * a StrainWeakening component, StgDomain TimeIntegrand; Underworld/Rheology/src/StrainWeakening.c).
 * _set uploads it (n values in point order; NULL: all zero) and enables the history: the next
 * assemblies give every point of a VON_MISES / BYERLEE law with softeningStrain > 0 a softened
 * cohesion and store the history's time derivative (_StrainWeakening_CalcIncrementIsotropic).
 * _advance integrates one step of length dt with that derivative and clamps the history at zero
 * (_StrainWeakening_TimeDerivative, _StrainWeakening_MakeValuesPositive, :399-426).  _get copies the
 * history and the last derivative to the host (either may be NULL).  The initial random damage of
 * _StrainWeakening_Initialise (libc rand()) stays on the host. */
int uwgpu_strain_weakening_set(uwgpu_ctx* ctx, const double* pfw);
int uwgpu_strain_weakening_advance(uwgpu_ctx* ctx, double dt);
int uwgpu_strain_weakening_get(uwgpu_ctx* ctx, double* pfw, double* increment);

/* Binning + integration-point mapping: _CoincidentMapper_Map
 * (PICellerator/MaterialPoints/src/CoincidentMapper.c:150-253) with the regular-mesh element
 * search (StgDomain/Mesh/src/Mesh_RegularAlgorithms.c:194-226), the cell-table append order of
 * Swarm_AddParticleToCell (StgDomain/Swarm/src/SwarmClass.c:1155-1184) and ConstantWeights
 * (PICellerator/Weights/src/ConstantWeights.c:180-189).  Optional host outputs: perm (n: point
 * index of each integration slot, element by element, ascending within an element), offsets
 * (nel+1) and xi (3 per slot).  Returns UWGPU_ERR_DOMAIN if points lie outside the mesh. */
int uwgpu_bin_and_map(uwgpu_ctx* ctx, uint32_t* perm, uint32_t* offsets, double* xi);

/* Material-point advection with the current velocity solution: _SwarmAdvector_TimeDeriv
 * (PICellerator/MaterialPoints/src/SwarmAdvector.c:288-314) integrated by TimeIntegrand_FirstOrder
 * (order 1) or TimeIntegrand_SecondOrder (order 2, StgDomain/Utils/src/TimeIntegrand.c:221-337).
 * A point with no velocity (outside the mesh; with order 2 also a predictor outside the mesh
 * unless allow_first_order_fallback) makes the call return UWGPU_ERR_DOMAIN and leaves every
 * point where it was.  fell_back: points updated to first order; left_mesh: points now outside
 * the mesh (the next uwgpu_bin_and_map refuses them).  The positions change on the device: the
 * next uwgpu_bin_and_map redoes the ownership (SwarmAdvector_AdvectionFinish,
 * SwarmAdvector.c:375-382). */
int uwgpu_advect_particles(uwgpu_ctx* ctx, double dt, int32_t order, int32_t allow_first_order_fallback,
                           uint32_t* fell_back, uint32_t* left_mesh);
/* Current particle coordinates to host arrays (n each; z ignored in 2D): the host copy of
 * GlobalParticle.coord (StgDomain/Swarm/src/StandardParticle.h:77) for output and analysis. */
int uwgpu_particles_download(uwgpu_ctx* ctx, double* x, double* y, double* z);

/* Integration weights of the next assemblies (the WeightsCalculator of the integration swarm).
 * UWGPU_WEIGHTS_CONSTANT (default): ConstantWeights, 2^dim / points in the element
 * (PICellerator/Weights/src/ConstantWeights.c:180-189).  UWGPU_WEIGHTS_DVC: DVCWeights
 * (PICellerator/Weights/src/DVCWeights.c:763-942) on res[0] x res[1] (x res[2]) cells over the
 * element's local coordinates (the component's resolutionX/Y/Z, default 10 each; at most 32 per
 * axis and 1024 cells per element): every integration point moves to the centroid of its
 * discrete Voronoi region and weighs that region's volume.  res is ignored for CONSTANT. */
enum { UWGPU_WEIGHTS_CONSTANT = 0, UWGPU_WEIGHTS_DVC = 1 };
int uwgpu_weights_set(uwgpu_ctx* ctx, int32_t kind, const int32_t res[3]);
/* PCDVC population control (PICellerator/Utils/src/PCDVC.c:638-1060, non-inflow branch; defaults of
 * PCDVC.c:260-268 in brackets): with DVC weights selected and the points mapped, every element in
 * index order splits its points whose Voronoi region exceeds upper_t percent of the element's local
 * volume [25] (at most max_splits [3], at the region's centroid) and deletes those below lower_t
 * percent [0.6] (at most max_deletions [2], largest swarm index first, the swarm's last point moving
 * into the hole), with no deletions in interface cells (mixed materials) unless
 * delete_in_interface_cells [0] and no splits there unless split_in_interface_cells [0] or the
 * element touches the mesh boundary.  The points (coordinates, material, per-point viscosity,
 * density and strain-weakening history) and the cell tables are replaced on the device in the
 * reference's order; *count (optional) receives the new number of points.  The next assembly's
 * DVC weights follow the new cell order (the reference's second DVC pass). */
typedef struct {
    double upper_t, lower_t;
    int32_t max_deletions, max_splits;
    int32_t split_in_interface_cells, delete_in_interface_cells;
} uwgpu_pcdvc_opts;
int uwgpu_population_control(uwgpu_ctx* ctx, const uwgpu_pcdvc_opts* opts, int64_t* count);

/* The current cell tables (the integration swarm's cellParticleTbl, in slot order): perm (point
 * of every slot) and offsets (nel + 1), without re-binning (after uwgpu_population_control they
 * hold the reference's edited order).  Either may be NULL. */
int uwgpu_get_cell_tables(uwgpu_ctx* ctx, uint32_t* perm, uint32_t* offsets);

/* Local coordinates ([slot][3], z = 0 in 2D) and weights (slot order) of the integration points
 * the last assembly used: IntegrationPoint.xi and .weight (StgDomain/Swarm/src/
 * IntegrationPoint.h:47, StandardParticle.h:70) for CPU readers of the integration swarm.
 * Either output may be NULL. */
int uwgpu_integration_points(uwgpu_ctx* ctx, double* xi, double* w);

/* Element assembly of every element: replaces the StiffnessMatrix assemble entry point
 * (StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:799-1017) for the terms
 * ConstitutiveMatrixCartesian (Underworld/Rheology/src/ConstitutiveMatrixCartesian.c:202-412),
 * BuoyancyForceTerm (PICellerator/Utils/src/BuoyancyForceTerm.c:310-452),
 * GradientStiffnessMatrixTerm (StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:160-250) and
 * UzawaPreconditionerTerm (StgFEM/SLE/ProvidedSystems/StokesFlow/src/UzawaPreconditionerTerm.c:155-238).
 * Results stay on the device. */
int uwgpu_assemble(uwgpu_ctx* ctx);

/* How the next assemblies contract the per-element moments into K_e (3D; 2D always uses FP64):
 * UWGPU_ASSEMBLY_FP64 (default): FP64 arithmetic on the CUDA cores, the drop-in form.
 * UWGPU_ASSEMBLY_TENSOR: the 63 pair tables of every element are one batched product of the
 * moments with a small integer matrix, run on the tcgen05 tensor core in FP16 with FP64 accuracy
 * (each moment cut into five 11-bit slices, every slice product exact in the FP32 accumulator;
 * Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 59, 2012); relative error of K_e about 2^-53.
 * Replaces the B^T D B accumulation of ConstitutiveMatrixCartesian.c:388-407 in the same way. */
enum { UWGPU_ASSEMBLY_FP64 = 0, UWGPU_ASSEMBLY_TENSOR = 1 };
int uwgpu_assembly_set(uwgpu_ctx* ctx, int32_t mode);

/* Storage of the stencils the mixed form's V-cycle smooths with (no reference counterpart: the
 * reference's PCMG smooths in FP64): 16 (default) keeps an FP16 copy of every level's stencil with
 * each row divided by its largest magnitude (relative error 2^-11 of the row's largest entry),
 * read by the Chebyshev smoother and the V-cycle residuals, which halves their stencil bytes; the
 * Krylov products and the FP64 refinement residuals keep the FP32 / FP64 stencils, so the
 * converged answer is unchanged.  32: the FP32 stencil everywhere. */
int uwgpu_smoother_storage_set(uwgpu_ctx* ctx, int32_t bits);

/* Newton form of the element matrices (the SLE's nlFormJacobian, 2D): with on != 0 the next
 * assemblies add the viscosity's derivatives with respect to the velocity gradient that yielding
 * laws (VON_MISES, DRUCKER_PRAGER) provide to the viscous term, as the 2D branch of
 * ConstitutiveMatrixCartesian.c:360-383 does, around the context's current solution.  The
 * general form is not symmetric (for these two laws the added term is a symmetric rank-one update
 * along the stress, which can make K_e indefinite): uwgpu_get_element_matrices returns all
 * nd x nd entries (row = test function dof), and uwgpu_solve_bsscr refuses it with
 * UWGPU_ERR_UNSUPPORTED (the solver here takes the Picard form).  3D: UWGPU_ERR_UNSUPPORTED (the
 * reference has no 3D branch). */
int uwgpu_jacobian_set(uwgpu_ctx* ctx, int32_t on);

/* Per-element results of the last assembly, copied to the host: the per-element callback
 * StiffnessMatrixTerm_AssembleElementFunction (StgFEM/SLE/SystemSetup/src/StiffnessMatrixTerm.c
 * :247-266) reads element e from here.  Ke: count*(nd*nd) row-major, dof = node*dim + comp;
 * fe, Ge: count*nd; Se: count.  Any output may be NULL. */
int uwgpu_get_element_matrices(uwgpu_ctx* ctx, int64_t first, int64_t count, double* Ke,
                               double* fe, double* Ge, double* Se);
/* Viscosity evaluated at every integration slot by the last assembly (n, slot order): the
 * isotropic viscosity the constitutive matrix holds per point (ConstitutiveMatrixCartesian.c:332,
 * matrixData[2][2] in 2D) for output and tests. */
int uwgpu_get_point_viscosity(uwgpu_ctx* ctx, double* eta);

/* Velocity-block operator y = K x on nodal vectors (nnode*dim, fixed dofs act as identity):
 * the MatMult of the assembled K the BSSCR solver applies (PETSc MatMult on the k_matrix).
 * precision: UWGPU_PREC_FP64 or UWGPU_PREC_MIXED (FP32 operator).  Builds the operator if
 * needed. */
int uwgpu_operator_apply(uwgpu_ctx* ctx, int32_t precision, const double* x, double* y);

/* Stokes solve by Schur-complement reduction: KSPSolve_BSSCR
 * (Solvers/KSPSolvers/src/BSSCR/BSSCR.c:151-229, auglag-driver-DGTGD.c:53-441) invoked through
 * the SLE_Solver interface (StgFEM/SLE/SystemSetup/src/SLE_Solver.c:226-257,
 * Solvers/KSPSolvers/src/StokesBlockKSPInterface.c:211-328).  u (nnode*dim) and p (nel) are
 * host outputs (either may be NULL to leave the result on the device). */
int uwgpu_solve_bsscr(uwgpu_ctx* ctx, const uwgpu_solve_opts* opts, double* u, double* p,
                      uwgpu_report* report);

/* Picard iteration of a nonlinear Stokes system: SystemLinearEquations_NonLinearExecute
 * (StgFEM/SLE/SystemSetup/src/SystemLinearEquations.c:750-935).  Each iteration re-runs the
 * rheology and assembly with the current velocity and pressure (strain-rate and pressure
 * dependent laws; yielding starts after the first solve, YieldRheology.c:210-212) and solves again,
 * until ||u_k - u_(k-1)|| / ||u_k|| < tolerance (after at least min_iterations) or max_iterations
 * solves.  Requires uwgpu_bin_and_map first.  *iterations and *residual (optional) report the
 * solves done and the last relative change; u, p as in uwgpu_solve_bsscr.  With tolerance > 0,
 * reaching max_iterations without meeting it returns UWGPU_ERR_NOT_CONVERGED (the reference's
 * "Failed to converge", SystemLinearEquations.c:908-914); tolerance <= 0 runs exactly
 * max_iterations solves. */
int uwgpu_solve_picard(uwgpu_ctx* ctx, const uwgpu_solve_opts* opts, double tolerance, int32_t max_iterations,
                       int32_t min_iterations, double* u, double* p, uwgpu_report* report, int32_t* iterations,
                       double* residual);

/* Default options: the BSSCR driver's defaults (CG Schur iteration, KSPSetType "cg" in
 * auglag-driver-DGTGD.c:266, with the uw approxS preconditioner, preconditioner.c:137), 4 levels,
 * 2+2 smoothing sweeps. */
void uwgpu_solve_opts_default(uwgpu_solve_opts* opts);

/* Kernel timing: when enabled, launches of the kernel family `which` are bracketed by CUDA
 * events on the context stream and summed (count, milliseconds). */
enum { UWGPU_KERNEL_ASSEMBLY = 0, UWGPU_KERNEL_APPLY = 1, UWGPU_KERNEL_SMOOTH = 2,
       UWGPU_KERNEL_BINNING = 3, UWGPU_KERNEL_SCHUR_PC = 4 /* scaled-BFBt inner solves */,
       UWGPU_KERNEL_VECTOR = 5 /* Krylov vector work, reductions, G and G^T */,
       UWGPU_KERNEL_TRANSFER = 6 /* restriction, prolongation, coarsest solve */,
       UWGPU_KERNEL_LEARNED = 7 /* U-Net preconditioner: forward, backward, Adam */,
       UWGPU_KERNEL_SETUP = 8 /* solver setup: stencils, multigrid hierarchy, Chebyshev bounds, BFBt operator */,
       UWGPU_KERNEL_COUNT = 9 };
/* (Measurement hooks, no reference counterpart.) */
int uwgpu_profile_enable(uwgpu_ctx* ctx, int32_t on);
int uwgpu_profile_read(uwgpu_ctx* ctx, int32_t which, int64_t* launches, double* ms);
/* Algorithmic work of the profiled launches of family `which`: bytes the kernels must move
 * (each operand read or written once) and floating-point operations, summed on the host at
 * launch time while profiling is enabled. */
int uwgpu_profile_read_work(uwgpu_ctx* ctx, int32_t which, double* bytes, double* flops);
/* Number of library kernel launches issued since the context was created. */
int64_t uwgpu_launch_count(const uwgpu_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), so callers can order their own work and
 * record timing events on it. */
int uwgpu_get_stream(uwgpu_ctx* ctx, void** stream);

/* Timing hook (no reference counterpart): `iterations` Chebyshev smoothing calls of `degree`
 * steps on the fine level (k_cheb_step, each step a full stencil pass from the current iterate),
 * total ms by CUDA events. */
int uwgpu_time_chebyshev(uwgpu_ctx* ctx, int32_t precision, int32_t degree, int32_t iterations, double* ms);

/* Kernel timing hooks (no reference counterpart; used by the benchmark and the profiles).
 * Each runs `iterations` back-to-back launches on the fine level, on vectors resident in the
 * context, and returns the elapsed device time in milliseconds (CUDA events on the context
 * stream).  uwgpu_time_apply: the operator apply y = K x; uwgpu_time_smooth: one smoothing call
 * of `sweeps` symmetric colour Gauss-Seidel sweeps.  precision as in uwgpu_operator_apply. */
int uwgpu_time_apply(uwgpu_ctx* ctx, int32_t precision, int32_t iterations, double* ms);
int uwgpu_time_smooth(uwgpu_ctx* ctx, int32_t precision, int32_t sweeps, int32_t iterations, double* ms);

/* Test and timing hooks on the inner operator of the scaled BFBt preconditioner, G^T W G with
 * W = 1/rowmax(K) of the current fine velocity operator (pc_ScaledGtKG.c:735-760; built by a
 * previous solve, else UWGPU_ERR_STATE).  form 0: the FP64 element stencil; 1: the FP32
 * matrix-free apply of the mixed form; 2: the FP32 stencil.  uwgpu_bfbt_operator_apply: y = A x
 * (host arrays of one value per element).  uwgpu_time_bfbt_apply: `iterations` launches of the
 * inner CG's operator kernel in that form, elapsed device milliseconds in ms. */
int uwgpu_bfbt_operator_apply(uwgpu_ctx* ctx, int32_t form, const double* x, double* y);
int uwgpu_time_bfbt_apply(uwgpu_ctx* ctx, int32_t form, int32_t iterations, double* ms);

/* Tensor-core self-check (no reference counterpart): D = A B^T for A 128 x k and B n x k (row-major
 * 16-bit values: bfloat16 bits for format 1, IEEE half bits for format 0), D 128 x n FP32, computed
 * by one tcgen05 MMA sequence with the operands staged in shared memory in the layout `layout`
 * (0: both K-major, 2: both MN-major, 4: A K-major and B MN-major; odd values exchange the
 * descriptors' two stride fields, a diagnostic).  n and k: multiples of 16, 16..256. */
int uwgpu_tc_check(uwgpu_ctx* ctx, int32_t layout, int32_t format, int32_t n, int32_t k, const uint16_t* a,
                   const uint16_t* b, float* d);

/* Allocation-free binning + mapping.  This entry point has no counterpart in the reference; it
 * exists for callers that cannot allocate device memory while they run (a host framework that
 * owns every device buffer through its own pool, or code where an allocation would synchronise
 * the device).  It needs no context and calls no allocator: the caller passes device-accessible
 * inputs (x, y, z coordinates of n points) and outputs (perm: n, offsets: nel+1, xi: dim*n laid
 * out [d][slot]), and the pass's scratch lives in one fixed __device__ array of about 9 MB that
 * every device loading the library keeps until the process exits.  Limits: at most
 * UWGPU_NOALLOC_MAX_POINTS points and UWGPU_NOALLOC_MAX_ELEMENTS elements, else
 * UWGPU_ERR_TOO_LARGE.  Results equal uwgpu_bin_and_map's.  The first call on a device looks up
 * the array's device address.  Calls share the array: calls whose GPU work overlaps race, so
 * order them (e.g. one stream).  Runs on `stream` (NULL: the default stream) and synchronises it
 * to read the outside-point count, so it cannot be called while that stream is being captured;
 * *outside (optional, host) receives the number of points outside the mesh, reported as
 * UWGPU_ERR_DOMAIN. */
#define UWGPU_NOALLOC_MAX_POINTS (1 << 20)
#define UWGPU_NOALLOC_MAX_ELEMENTS (1 << 17)
int uwgpu_bin_and_map_noalloc(int32_t dim, const int32_t nel[3], const double min[3], const double max[3],
                              int64_t n, const double* x, const double* y, const double* z, uint32_t* perm,
                              uint32_t* offsets, double* xi, void* stream, uint32_t* outside);

/* ---- Learned velocity preconditioner ------------------------------------------------------
 * A 3D U-Net (BF16 weights and activations, FP32 accumulation) that maps the velocity residual,
 * the multigrid V-cycle's answer to it and log10 viscosity on the node grid to a correction of
 * that answer.  It has no counterpart in the
 * reference: it augments the multigrid preconditioner of the velocity solve (BSSCR/mg.c:42-132,
 * PCMG) inside the flexible Krylov iteration, with plain multigrid as its fallback.  3D only. */

/* Builds the network for the context's mesh: `levels` resolution levels (1..6), `base_channels`
 * channels at the finest level (multiple of 8), doubling per level; weights from `seed`. */
int uwgpu_learned_create(uwgpu_ctx* ctx, int32_t levels, int32_t base_channels, uint64_t seed);
int uwgpu_learned_param_count(uwgpu_ctx* ctx, int64_t* count);
/* Parameters (FP32 master copy, layout: per 3x3x3 layer W[27][cin][cout] then bias[cout], encoder
 * layers by level, then decoder layers by level, then the 1x1x1 head W[cin][3], bias[3]). */
int uwgpu_learned_get_params(uwgpu_ctx* ctx, float* params);
int uwgpu_learned_set_params(uwgpu_ctx* ctx, const float* params);
/* Test hooks: one forward pass on host input[7][nn] (channels: three residual components, three
 * components of the V-cycle's answer, log10 viscosity; node order of the mesh) -> output[3][nn];
 * then the backward pass of grad_output[3][nn] -> grad_params[param_count] (overwritten) and
 * grad_input[7][nn]. */
int uwgpu_learned_forward(uwgpu_ctx* ctx, const float* input, float* output);
int uwgpu_learned_backward(uwgpu_ctx* ctx, const float* grad_output, float* grad_params, float* grad_input);

/* Training set from the assembled system: `nsamples` residual/error pairs of the multigrid
 * solver (random velocity fields e, r = K e, inputs r and V(r), target e - V(r) for one V-cycle V
 * of the hierarchy `opts` describes); replaces any previous set. */
int uwgpu_learned_generate(uwgpu_ctx* ctx, const uwgpu_solve_opts* opts, int32_t nsamples, uint64_t seed);
/* Adam on the relative squared error of the correction; the last 10% of the samples are held
 * out.  train_loss: mean relative error of the last epoch; holdout_ratio: |target - N|^2/|target|^2
 * on the held-out pairs (below 1: the network reduces the error the V-cycle leaves). */
int uwgpu_learned_train(uwgpu_ctx* ctx, int32_t epochs, int32_t batch, float learning_rate, uint64_t seed,
                        double* train_loss, double* holdout_ratio);

#ifdef __cplusplus
}
#endif
#endif /* UWGPU_H */
