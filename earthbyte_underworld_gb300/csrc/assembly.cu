// Element assembly on the integration points of every element.
//
// Reference behaviour (paths relative to the Underworld 1.x tree):
//   K_e  Underworld/Rheology/src/ConstitutiveMatrixCartesian.c:202-412: sum over the cell's
//        points of B^T (detJ w D) B with the isotropic D of ConstitutiveMatrix_SetIsotropicViscosity
//        (ConstitutiveMatrix.c:362-374, ConstitutiveMatrixCartesian.c:470-481)
//   eta  the RheologyMaterial law list (Rheology_Register.c:61-77): MaterialViscosity.c:119-139,
//        Arrhenius.c:156-200, FrankKamenetskii.c:134-152, ViscosityLimiter.c:106-126,
//        YieldRheology.c:198-243 + VonMises.c:206-269 + DruckerPrager.c:236-345
//   w    ConstantWeights.c:180-189 (cellLocalVolume 2^dim / count, WeightsCalculator.c:83), or
//        the discrete Voronoi weights and centroids of weights.cu (DVCWeights.c)
//   f_e  PICellerator/Utils/src/BuoyancyForceTerm.c:310-452
//   G_e  StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:160-250 on the 2^dim Gauss swarm
//   S_e  StgFEM/SLE/ProvidedSystems/StokesFlow/src/UzawaPreconditionerTerm.c:155-238
//
// GPU design.  On the affine elements of a regular mesh every product of shape-function
// derivatives is a polynomial of degree <= 2 per axis in the local coordinates, so
//   K_e = sum over 3^dim moments mu_abc = sum_p w eta_p xi^a eta^b zeta^c of fixed matrices.
// One thread owns one element: it streams the element's points (slot order, SoA) once,
// evaluates the rheology, accumulates the 27 (3D) / 9 (2D) moments in FP64 registers, then
// contracts them axis by axis into the 300 (3D) / 36 (2D) distinct entries of K_e.  This
// needs ~50 FP64 operations per point instead of the ~1000 of the per-point B^T D B loop,
// which matters on a part whose FP64 rate is 1/58 of its FP32 rate.  K_e, f_e, G_e are
// written entry-major ([entry][element]) so a warp's stores coalesce.
#include <cuda_fp16.h>

#include "internal.cuh"
#include "tc.cuh"

namespace uwg {

struct AssemblyArgs {
    int dim;
    int nel[3];
    double min[3], max[3];
    int64_t ne, nslots;
    const uint32_t* offsets;
    const double* sxi;       // [d][slot]
    const double* sw;        // per-slot weights, or null: 2^dim / count
    const int32_t* smat;
    const double* seta_in;   // optional
    const double* srho_in;   // optional
    const uwgpu_material* mats;
    int nmat;
    const double* temperature;  // nodal or null
    const double* u;            // nodal SoA [d][node] or null
    const double* p;            // per element or null
    int previous_solution;
    int vert_axis;
    double gravity;
    int64_t nnx, nny, nn;
    double* Ke;    // packed, entry-major
    double* fe;    // entry-major
    double* Ge;    // entry-major
    double* Se;
    double* eta_out;
    uint32_t* flags;  // bit0: empty element, bit1: bad material index
    double* mom;      // 3D, tensor-core contraction: moments out ([27][e]) instead of K_e and S_e
    const uint32_t* perm;   // point of each slot
    const double* pfw;      // strain-weakening history per point, or null
    double* pfw_incr;       // its time derivative per point (written by yielding laws), or null
};

// G_e entry of node a, component d on a 3D element of widths h: the integral of -dN_a/dx_d
// (exact for the 2x2x2 Gauss rule)
__host__ __device__ inline double ge_entry(const double h[3], int a, int d) {
    double area = 1.0;
    for (int q = 0; q < 3; ++q)
        if (q != d) area *= h[q];
    const double sa = ((a >> d) & 1) ? 1.0 : -1.0;
    return -sa * area * 0.25;
}

// ---- eigenvalues of a symmetric stress tensor, as the reference computes them
// (StgDomain/Geometry/src/TensorMath.c:619-975): the real roots of the characteristic cubic, or,
// when an eigenvector formula fails for one of them, cyclic Jacobi rotations (Numerical Recipes
// in C, 2nd ed., section 11.1); the same decisions, with the reference's absolute 1e-8
// comparisons, so that both sides take the same branch.  Storage: 2D [xx, yy, xy],
// 3D [xx, yy, zz, xy, xz, yz].  Ascending order.
__device__ __forceinline__ bool eql8(double a, double b) { return fabs(a - b) < 1.0e-8; }

__device__ inline void jacobi_eig3(const double* t, double* ev) {
    double a01 = t[3], a02 = t[4], a12 = t[5];
    double b[3] = {t[0], t[1], t[2]}, z[3] = {0.0, 0.0, 0.0};
    ev[0] = t[0];
    ev[1] = t[1];
    ev[2] = t[2];
    for (int sweep = 1; sweep <= 50; ++sweep) {
        const double sum = fabs(a01) + fabs(a02) + fabs(a12);
        if (sum == 0.0) break;
        const double tresh = sweep < 4 ? 0.2 * sum / 9.0 : 0.0;
        for (int pr = 0; pr < 3; ++pr) {
            const int ip = pr < 2 ? 0 : 1, iq = pr == 0 ? 1 : 2;   // (0,1), (0,2), (1,2)
            double& apq = pr == 0 ? a01 : (pr == 1 ? a02 : a12);
            const double g = 100.0 * fabs(apq);
            if (sweep > 4 && (fabs(ev[ip]) + g) == fabs(ev[ip]) && (fabs(ev[iq]) + g) == fabs(ev[iq])) {
                apq = 0.0;
            } else if (fabs(apq) > tresh) {
                double h = ev[iq] - ev[ip], tt;
                if ((double)(fabs(h) + g) == (double)fabs(h)) {
                    tt = apq / h;
                } else {
                    const double theta = 0.5 * h / apq;
                    tt = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
                    if (theta < 0.0) tt = -tt;
                }
                const double c = 1.0 / sqrt(1 + tt * tt), sn = tt * c, tau = sn / (1.0 + c);
                h = tt * apq;
                z[ip] -= h;
                z[iq] += h;
                ev[ip] -= h;
                ev[iq] += h;
                apq = 0.0;
                // the rotation of the remaining off-diagonal entry (the third index r)
                if (pr == 0) {          // (0,1): r = 2 -> a02 (row ip), a12 (row iq)
                    const double g1 = a02, h1 = a12;
                    a02 = g1 - sn * (h1 + g1 * tau);
                    a12 = h1 + sn * (g1 - h1 * tau);
                } else if (pr == 1) {   // (0,2): r = 1 lies between ip and iq -> a01 (row ip), a12 (column iq)
                    const double g1 = a01, h1 = a12;
                    a01 = g1 - sn * (h1 + g1 * tau);
                    a12 = h1 + sn * (g1 - h1 * tau);
                } else {                // (1,2): r = 0 below ip -> a01, a02
                    const double g1 = a01, h1 = a02;
                    a01 = g1 - sn * (h1 + g1 * tau);
                    a02 = h1 + sn * (g1 - h1 * tau);
                }
            }
        }
        for (int i = 0; i < 3; ++i) {
            b[i] += z[i];
            ev[i] = b[i];
            z[i] = 0.0;
        }
    }
}

__device__ inline void sym_eigenvalues(const double* t, int dim, double* ev) {
    if (dim == 2) {
        const double r = sqrt(0.25 * (t[0] - t[1]) * (t[0] - t[1]) + t[2] * t[2]);
        const double avg = 0.5 * (t[0] + t[1]);
        ev[0] = avg - r;
        ev[1] = avg + r;
        return;
    }
    const double a2 = -t[0] - t[1] - t[2];
    const double a1 = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(t[0], t[1]), __dmul_rn(t[0], t[2])),
                                                          __dmul_rn(t[1], t[2])),
                                                -__dmul_rn(t[3], t[3])),
                                      -__dmul_rn(t[4], t[4])),
                            -__dmul_rn(t[5], t[5]));
    const double a0 = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(-__dmul_rn(__dmul_rn(t[0], t[1]), t[2]),
                                                          -__dmul_rn(2.0, __dmul_rn(__dmul_rn(t[3], t[4]), t[5]))),
                                                __dmul_rn(__dmul_rn(t[0], t[5]), t[5])),
                                      __dmul_rn(__dmul_rn(t[1], t[4]), t[4])),
                            __dmul_rn(__dmul_rn(t[2], t[3]), t[3]));
    // the real roots of l^3 + a2 l^2 + a1 l + a0 (Cardano, trigonometric form)
    const double Q = __ddiv_rn(__dsub_rn(__dmul_rn(3.0, a1), __dmul_rn(a2, a2)), 9.0);
    const double R = __ddiv_rn(__dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(9.0, a2), a1), __dmul_rn(27.0, a0)),
                                         __dmul_rn(__dmul_rn(__dmul_rn(2.0, a2), a2), a2)),
                               54.0);
    const double D = __dadd_rn(__dmul_rn(__dmul_rn(Q, Q), Q), __dmul_rn(R, R));
    if (eql8(D, 0.0)) {
        const double halfB = R < 0.0 ? -pow(-R, 1.0 / 3.0) : pow(R, 1.0 / 3.0);
        ev[0] = -a2 / 3.0 + 2.0 * halfB;
        ev[1] = ev[2] = -a2 / 3.0 - halfB;
    } else {
        const double theta = acos(R / sqrt(-__dmul_rn(__dmul_rn(Q, Q), Q))) / 3.0;
        const double factor = 2.0 * sqrt(-Q);
        const double pi = 3.14159265358979323846;
        ev[0] = factor * cos(theta) - a2 / 3.0;
        ev[1] = factor * cos(theta + 2.0 * pi / 3.0) - a2 / 3.0;
        ev[2] = factor * cos(theta + 4.0 * pi / 3.0) - a2 / 3.0;
    }
    // an eigenvector formula must apply to every root (TensorMath.c:726-758), else Jacobi
    bool ok = true;
    for (int i = 0; i < 3; ++i) {
        const double A = t[0] - ev[i], B = t[1] - ev[i], d = t[3], e = t[4], f = t[5];
        const bool good = (!eql8(B * e, f * d) && !eql8(e, 0.0)) || (!eql8(f * A, d * e) && !eql8(e, 0.0)) ||
                          (!eql8(d * d, B * A) && !eql8(d, 0.0));
        ok = ok && good;
    }
    if (!ok) jacobi_eig3(t, ev);
    // ascending
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2 - i; ++j)
            if (ev[j] > ev[j + 1]) {
                const double tmp = ev[j];
                ev[j] = ev[j + 1];
                ev[j + 1] = tmp;
            }
}

// Per-point rheology chain.  Every law in scope keeps D isotropic, so the constitutive matrix
// is carried as its viscosity (D[3][3] in 3D, D[2][2] in 2D).
template <int DIM>
__device__ __forceinline__ double run_rheology(const uwgpu_material& m, const double* N, const double* Tn,
                                               bool hasT, const double* xg, double ymax, double point_eta,
                                               const double (*L)[3], double pressure, int prev, double pfw,
                                               double* pfw_incr, double* derivs = nullptr, bool jacobian = false) {
    const double yglobal = xg[1];
    double eta = 0.0;
    // derivs: the viscosity derivatives of the Newton form (9 entries; zeroed with every
    // SetIsotropicViscosity, ConstitutiveMatrix.c:362-367; VonMises-family yielding adds its terms
    // when the Jacobian is formed, VonMises.c:259-268)
    if (derivs)
        for (int k = 0; k < 9; ++k) derivs[k] = 0.0;
    auto set_visc = [&](double v) {
        eta = v;
        if (derivs)
            for (int k = 0; k < 9; ++k) derivs[k] = 0.0;
    };
    auto yield_derivs = [&](double visc0, double crit, double ind) {
        if (!derivs || !jacobian) return;
        const double st0 = 2.0 * visc0 * L[0][0], st1 = 2.0 * visc0 * L[1][1];
        const double st2 = DIM == 3 ? 2.0 * visc0 * L[2][2] : visc0 * 2.0 * (0.5 * (L[0][1] + L[1][0]));
        const double coef = -visc0 * crit / (2.0 * ind * ind * ind);
        derivs[0] += coef * 2.0 * visc0 * st0;
        derivs[4] += coef * 2.0 * visc0 * st1;
        derivs[1] += coef * 2.0 * visc0 * st2;
        derivs[3] += coef * 2.0 * visc0 * st2;
    };
    for (int l = 0; l < m.n_laws; ++l) {
        const uwgpu_law& law = m.laws[l];
        switch (law.law) {
        case UWGPU_LAW_MATERIAL_VISCOSITY:
            set_visc(law.p[0]);
            break;
        case UWGPU_LAW_ARRHENIUS: {
            double T = 0.0;
            if (hasT) {
#pragma unroll
                for (int a = 0; a < (1 << DIM); ++a) T += N[a] * Tn[a];
            }
            if (law.p[2] > (0.0 + 1e-12)) {
                double depth = ymax - yglobal;
                set_visc(law.p[0] * exp((law.p[1] + law.p[2] * depth) / (T + law.p[3])));
            } else {
                set_visc(law.p[0] * exp((law.p[1]) / (T + law.p[3])));
            }
            break;
        }
        case UWGPU_LAW_FRANK_KAMENETSKII: {
            double T = 0.0;
            if (hasT) {
#pragma unroll
                for (int a = 0; a < (1 << DIM); ++a) T += N[a] * Tn[a];
            }
            set_visc(law.p[0] * exp(-law.p[1] * T));
            break;
        }
        case UWGPU_LAW_VISCOSITY_LIMITER: {
            double v = eta;
            if (v > law.p[0]) v = law.p[0];
            if (v < law.p[1]) v = law.p[1];
            set_visc(v);
            break;
        }
        case UWGPU_LAW_DRUCKER_PRAGER: {
            double minVisc = law.p[3];
            if (!prev) break;
            // yield indicator: second invariant of the stress D . strain-rate
            double inv;
            if (DIM == 3) {
                double s0 = 2.0 * eta * L[0][0], s1 = 2.0 * eta * L[1][1], s2 = 2.0 * eta * L[2][2];
                double s3 = eta * 2.0 * (0.5 * (L[0][1] + L[1][0]));
                double s4 = eta * 2.0 * (0.5 * (L[0][2] + L[2][0]));
                double s5 = eta * 2.0 * (0.5 * (L[1][2] + L[2][1]));
                inv = 0.5 * (s0 * s0 + s1 * s1 + s2 * s2) + s3 * s3 + s4 * s4 + s5 * s5;
            } else {
                double s0 = 2.0 * eta * L[0][0], s1 = 2.0 * eta * L[1][1];
                double s2 = eta * 2.0 * (0.5 * (L[0][1] + L[1][0]));
                inv = 0.5 * (s0 * s0 + s1 * s1) + s2 * s2;
            }
            double ind = sqrt(inv);
            double phi = atan(law.p[1]);
            double dpFric, dpCoh;
            if (DIM == 3) {
                double sinphi = sin(phi);
                double ood = 1.0 / (sqrt(3.0) * (3.0 - sinphi));
                dpFric = 6.0 * sinphi * ood;
                dpCoh = 6.0 * law.p[0] * cos(phi) * ood;
            } else {
                dpCoh = law.p[0] * cos(phi);
                dpFric = sin(phi);
            }
            double crit = dpFric * pressure + dpCoh;
            if (crit < law.p[2]) crit = law.p[2];
            if (crit < ind) {
                const double visc0 = eta;
                double beta = 1.0 - crit / ind;
                double corr = -eta * beta;
                if ((eta + corr) < minVisc) corr = minVisc - eta;
                eta += corr;
                yield_derivs(visc0, crit, ind);
            }
            if (eta < minVisc) set_visc(minVisc);
            break;
        }
        case UWGPU_LAW_VON_MISES:
        case UWGPU_LAW_BYERLEE: {
            // YieldRheology.c:198-243: indicator, criterion, strain-weakening increment (with the
            // viscosity before the correction), the yield correction, the minimum viscosity
            if (!prev) break;
            const double minVisc = law.p[2], soft = law.p[3], healing = law.p[4];
            double inv;
            if (DIM == 3) {
                double s0 = 2.0 * eta * L[0][0], s1 = 2.0 * eta * L[1][1], s2 = 2.0 * eta * L[2][2];
                double s3 = eta * 2.0 * (0.5 * (L[0][1] + L[1][0]));
                double s4 = eta * 2.0 * (0.5 * (L[0][2] + L[2][0]));
                double s5 = eta * 2.0 * (0.5 * (L[1][2] + L[2][1]));
                inv = 0.5 * (s0 * s0 + s1 * s1 + s2 * s2) + s3 * s3 + s4 * s4 + s5 * s5;
            } else {
                double s0 = 2.0 * eta * L[0][0], s1 = 2.0 * eta * L[1][1];
                double s2 = eta * 2.0 * (0.5 * (L[0][1] + L[1][0]));
                inv = 0.5 * (s0 * s0 + s1 * s1) + s2 * s2;
            }
            const double ind = sqrt(inv);
            // StrainWeakening_CalcRatio (StrainWeakening.c:484-503)
            const double w = pfw < 0.0 ? 0.0 : pfw;
            double ratio = 0.0;
            if (soft > 0.0) {
                ratio = w / soft;
                if (ratio > 1.0) ratio = 1.0;
            }
            // VonMises.c:175-198 (softened cohesion) or Byerlee.c:157-198 (cohesion + depth term,
            // depth below the mesh's largest y)
            const double crit = law.law == UWGPU_LAW_VON_MISES ? law.p[0] * (1.0 - ratio) + law.p[1] * ratio
                                                               : law.p[0] + law.p[1] * (ymax - yglobal);
            if (soft > 0.0 && pfw_incr) {   // _StrainWeakening_CalcIncrementIsotropic (:428-481)
                const double beta = (crit == 0.0 || ind == 0.0) ? 0.0 : 1.0 - crit / ind;
                *pfw_incr = beta <= 0.0 ? -healing * w : (crit / eta) * (beta / (1.0 - beta) - healing * w);
            }
            if (crit < ind) {   // _VonMises_HasYielded (VonMises.c:232-269)
                const double visc0 = eta;
                if (law.p[5] != 0.0) {
                    set_visc(2.0 * crit * crit * eta / (crit * crit + ind * ind));
                } else {
                    const double beta = 1.0 - crit / ind;
                    double corr = -eta * beta;
                    if ((eta + corr) < minVisc) corr = minVisc - eta;
                    eta += corr;
                }
                // Newton terms with the criterion the law stored (Byerlee.c stores none: no terms)
                yield_derivs(visc0, law.law == UWGPU_LAW_VON_MISES ? crit : 0.0, ind);
            }
            if (eta < minVisc) set_visc(minVisc);
            break;
        }
        case UWGPU_LAW_MOHR_COULOMB: {
            // MohrCoulomb.c:208-402 via YieldRheology.c:198-243: principal stresses of the stress
            // of the deviatoric strain rate, a friction-modified stress difference as indicator,
            // the pressure-dependent strength as criterion
            if (!prev) break;
            const double minVisc = law.p[5], soft = law.p[6], healing = law.p[7];
            double st[6], ev[3];
            if (DIM == 3) {
                const double tr = L[0][0] + L[1][1] + L[2][2];
                st[0] = 2.0 * eta * (L[0][0] - tr / 3.0);
                st[1] = 2.0 * eta * (L[1][1] - tr / 3.0);
                st[2] = 2.0 * eta * (L[2][2] - tr / 3.0);
                st[3] = 2.0 * eta * (0.5 * (L[0][1] + L[1][0]));
                st[4] = 2.0 * eta * (0.5 * (L[0][2] + L[2][0]));
                st[5] = 2.0 * eta * (0.5 * (L[1][2] + L[2][1]));
            } else {
                const double tr = L[0][0] + L[1][1];
                st[0] = 2.0 * eta * (L[0][0] - tr / 2.0);
                st[1] = 2.0 * eta * (L[1][1] - tr / 2.0);
                st[2] = 2.0 * eta * (0.5 * (L[0][1] + L[1][0]));
            }
            sym_eigenvalues(st, DIM, ev);
            const double w = pfw < 0.0 ? 0.0 : pfw;
            double ratio = 0.0;
            if (soft > 0.0) {
                ratio = w / soft;
                if (ratio > 1.0) ratio = 1.0;
            }
            const double alpha = law.p[2] * (1.0 - ratio) + law.p[3] * ratio;
            const double coh = law.p[0] * (1.0 - ratio) + law.p[1] * ratio;
            const double smin = ev[0], smax = DIM == 2 ? ev[1] : ev[2];
            double sigma_ns = 0.5 * (smax - smin);
            if (DIM == 3) {
                const double th = 0.5 * atan(1.0 / alpha);
                const double fac = 1 / (sin(2 * th) - alpha * cos(2 * th));
                sigma_ns -= (smax + smin) * 0.5 * alpha * fac;
            }
            const double ind = fabs(sigma_ns);
            const double th = 0.5 * atan(1.0 / alpha);
            const double fac = sin(2 * th);
            double crit = alpha * pressure * fac + coh * fac;
            const double minYS = law.p[4] == 0.0 ? coh : law.p[4];
            if (crit < minYS * fac) crit = minYS * fac;
            if (soft > 0.0 && pfw_incr) {
                const double beta = (crit == 0.0 || ind == 0.0) ? 0.0 : 1.0 - crit / ind;
                *pfw_incr = beta <= 0.0 ? -healing * w : (crit / eta) * (beta / (1.0 - beta) - healing * w);
            }
            if (crit < ind) {
                const double beta = 1.0 - crit / ind;
                double corr = -eta * beta;
                if ((eta + corr) < minVisc) corr = minVisc - eta;
                eta += corr;
            }
            if (eta < minVisc) set_visc(minVisc);
            break;
        }
        case UWGPU_LAW_PARTICLE_VISCOSITY:
            set_visc(point_eta);
            break;
        case UWGPU_LAW_LINEAR_VISCOSITY:
        {
            double v = law.p[1] * xg[0] + law.p[2] * xg[1] + law.p[4] * xg[0] * xg[1] + law.p[0];
            if (DIM == 3)
                v += law.p[3] * xg[2] + law.p[5] * xg[0] * xg[2] + law.p[6] * xg[1] * xg[2] +
                     law.p[7] * xg[0] * xg[1] * xg[2];
            set_visc(v);
            break;
        }
        case UWGPU_LAW_DEPTH_DEPENDENT: {
            const int axis = (int)law.p[3];
            set_visc(law.p[0] * exp(law.p[1] * (xg[axis < 0 ? 0 : (axis > 2 ? 2 : axis)] - law.p[2])));
            break;
        }
        case UWGPU_LAW_NON_NEWTONIAN: {
            // strain-rate invariant of the previous solution at the point (TensorMath.c:430-458)
            double sri = law.p[1];
            if (prev) {
                if (DIM == 3) {
                    double e3 = 0.5 * (L[0][1] + L[1][0]), e4 = 0.5 * (L[0][2] + L[2][0]), e5 = 0.5 * (L[1][2] + L[2][1]);
                    sri = sqrt(0.5 * (L[0][0] * L[0][0] + L[1][1] * L[1][1] + L[2][2] * L[2][2]) + e3 * e3 + e4 * e4 +
                               e5 * e5);
                } else {
                    double e2 = 0.5 * (L[0][1] + L[1][0]);
                    sri = sqrt(0.5 * (L[0][0] * L[0][0] + L[1][1] * L[1][1]) + e2 * e2);
                }
            }
            const double n = law.p[0];
            if (sri == 0.0 || fabs(n - 1.0) < 1.0e-10) break;
            set_visc(pow(2.0 * sri, 1.0 / n - 1.0) * pow(eta, 1.0 / n));
            break;
        }
        default:
            break;
        }
    }
    return eta;
}

// Coefficients of (1 + s_i x)(1 + s_j x) in the monomials 1, x, x^2, by pair type:
// type 0: s_i = s_j = +1, type 1: s_i = s_j = -1, type 2: s_i != s_j.
__device__ __constant__ double kQ[3][3] = {{1.0, 2.0, 1.0}, {1.0, -2.0, 1.0}, {1.0, 0.0, -1.0}};
// Coefficients of (1 + s x) in 1, x by type: 0: s = +1, 1: s = -1.
__device__ __constant__ double kL[2][2] = {{1.0, 1.0}, {1.0, -1.0}};

__device__ __forceinline__ int qtype(int si, int sj) { return si == sj ? (si > 0 ? 0 : 1) : 2; }
__device__ __forceinline__ int ltype(int s) { return s > 0 ? 0 : 1; }

// The 63 pair tables of a 3D element: same-axis tables Dkk[t1][t2] (the node-pair types of the two
// other axes) and mixed-axis tables Mkl[t_k][t_l][t_other], each an integer combination of the 27
// moments mu[a][b][c] (a, b, c: powers of xi, eta, zeta).
struct Tables3 {
    double Dxx[3][3], Dyy[3][3], Dzz[3][3];
    double Mxy[2][2][3], Mxz[2][2][3], Myz[2][2][3];
};

// Coefficient of moment m = 9a + 3b + c in table q (the ordering of Tables3 flattened:
// Dxx, Dyy, Dzz as [t1][t2], then Mxy, Mxz, Myz as [ta][tb][to]); the same combinations
// tables_from_moments forms.  Values are 0, +-1, +-2, +-4.
__host__ __device__ inline int table_coefficient(int q, int m) {
    const int Q[3][3] = {{1, 2, 1}, {1, -2, 1}, {1, 0, -1}};
    const int L[2][2] = {{1, 1}, {1, -1}};
    const int a = m / 9, b = (m / 3) % 3, c = m % 3;
    if (q < 27) {
        const int axis = q / 9, t1 = (q % 9) / 3, t2 = q % 3;
        // the axis of the table carries power 0; (u, v) the powers of the two other axes in order
        int zero, u, v;
        if (axis == 0) { zero = a; u = b; v = c; }
        else if (axis == 1) { zero = b; u = a; v = c; }
        else { zero = c; u = a; v = b; }
        return zero == 0 ? Q[t1][u] * Q[t2][v] : 0;
    }
    if (q >= 63) return 0;
    const int r = q - 27, pair = r / 12, ta = (r % 12) / 6, tb = (r % 6) / 3, to = r % 3;
    int u, v, o;   // powers of the pair's first axis, second axis, and the other axis
    if (pair == 0) { u = a; v = b; o = c; }        // xy
    else if (pair == 1) { u = a; v = c; o = b; }   // xz
    else { u = b; v = c; o = a; }                  // yz
    if (u > 1 || v > 1) return 0;
    return L[ta][u] * L[tb][v] * Q[to][o];
}

__device__ __forceinline__ void tables_from_moments(const double* mu, Tables3& T) {
#pragma unroll
    for (int t1 = 0; t1 < 3; ++t1)
#pragma unroll
        for (int t2 = 0; t2 < 3; ++t2) {
            double sx = 0.0, sy = 0.0, sz = 0.0;
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int v = 0; v < 3; ++v) {
                    double q = kQ[t1][u] * kQ[t2][v];
                    sx += q * mu[0 * 9 + u * 3 + v];   // axes y (u), z (v)
                    sy += q * mu[u * 9 + 0 * 3 + v];   // axes x (u), z (v)
                    sz += q * mu[u * 9 + v * 3 + 0];   // axes x (u), y (v)
                }
            T.Dxx[t1][t2] = sx;
            T.Dyy[t1][t2] = sy;
            T.Dzz[t1][t2] = sz;
        }
#pragma unroll
    for (int ta = 0; ta < 2; ++ta)
#pragma unroll
        for (int tb = 0; tb < 2; ++tb)
#pragma unroll
            for (int to = 0; to < 3; ++to) {
                double sxy = 0.0, sxz = 0.0, syz = 0.0;
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int v = 0; v < 2; ++v) {
                        double l2 = kL[ta][u] * kL[tb][v];
#pragma unroll
                        for (int o = 0; o < 3; ++o) {
                            double q = l2 * kQ[to][o];
                            sxy += q * mu[u * 9 + v * 3 + o];   // x^u y^v z^o
                            sxz += q * mu[u * 9 + o * 3 + v];   // x^u z^v y^o
                            syz += q * mu[o * 9 + u * 3 + v];   // y^u z^v x^o
                        }
                    }
                T.Mxy[ta][tb][to] = sxy;
                T.Mxz[ta][tb][to] = sxz;
                T.Myz[ta][tb][to] = syz;
            }
}

// Packed K_e (entry-major) of element e from its tables; diag receives the 24 diagonal entries.
__device__ __forceinline__ void ke_from_tables(const Tables3& T, double detJ, const double g[3], int64_t e, int64_t ne,
                                               double* __restrict__ Ke, double diag[24]) {
    constexpr int NEN = 8, ND = 24;
    const double inv64 = 1.0 / 64.0;
    // M_kl[i][j] for node pair (i, j)
    auto Mkl = [&](int k, int l, int i, int j) -> double {
        int si[3] = {((i & 1) << 1) - 1, (((i >> 1) & 1) << 1) - 1, (((i >> 2) & 1) << 1) - 1};
        int sj[3] = {((j & 1) << 1) - 1, (((j >> 1) & 1) << 1) - 1, (((j >> 2) & 1) << 1) - 1};
        double sc = detJ * g[k] * g[l] * inv64 * (double)(si[k] * sj[l]);
        if (k == l) {
            if (k == 0) return sc * T.Dxx[qtype(si[1], sj[1])][qtype(si[2], sj[2])];
            if (k == 1) return sc * T.Dyy[qtype(si[0], sj[0])][qtype(si[2], sj[2])];
            return sc * T.Dzz[qtype(si[0], sj[0])][qtype(si[1], sj[1])];
        }
        // k < l: derivative axis k on node i, l on node j
        if (k > l) {
            // M_kl[i][j] = M_lk[j][i]
            int t = k; k = l; l = t;
            int tmp[3] = {si[0], si[1], si[2]};
            for (int q = 0; q < 3; ++q) { si[q] = sj[q]; sj[q] = tmp[q]; }
        }
        if (k == 0 && l == 1) return sc * T.Mxy[ltype(sj[0])][ltype(si[1])][qtype(si[2], sj[2])];
        if (k == 0 && l == 2) return sc * T.Mxz[ltype(sj[0])][ltype(si[2])][qtype(si[1], sj[1])];
        return sc * T.Myz[ltype(sj[1])][ltype(si[2])][qtype(si[0], sj[0])];
    };
#pragma unroll
    for (int i = 0; i < NEN; ++i)
#pragma unroll
        for (int j = i; j < NEN; ++j) {
            double tr = Mkl(0, 0, i, j) + Mkl(1, 1, i, j) + Mkl(2, 2, i, j);
#pragma unroll
            for (int al = 0; al < 3; ++al)
#pragma unroll
                for (int be = 0; be < 3; ++be) {
                    int r = i * 3 + al, cix = j * 3 + be;
                    if (r > cix) continue;
                    // K[(i,al),(j,be)] = delta * tr + M_{be,al}[i][j]
                    double v = Mkl(be, al, i, j) + (al == be ? tr : 0.0);
                    Ke[(int64_t)packed_index(ND, r, cix) * ne + e] = v;
                    if (r == cix) diag[r] = v;
                }
        }
}

template <int DIM>
__global__ void __launch_bounds__(128) k_assemble(AssemblyArgs A) {
    constexpr int NEN = 1 << DIM;
    constexpr int ND = NEN * DIM;
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.ne) return;
    int64_t ie = e % A.nel[0];
    int64_t je = (e / A.nel[0]) % A.nel[1];
    int64_t ke = DIM == 3 ? e / ((int64_t)A.nel[0] * A.nel[1]) : 0;
    int64_t idx[3] = {ie, je, ke};
    double x0[3], h[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        x0[d] = node_coord_1d(idx[d], A.nel[d], A.min[d], A.max[d]);
        h[d] = node_coord_1d(idx[d] + 1, A.nel[d], A.min[d], A.max[d]) - x0[d];
    }
    // element nodes (CartesianGenerator incidence order, x fastest)
    int64_t base = ie + A.nnx * (je + A.nny * ke);
    int64_t inc[NEN];
#pragma unroll
    for (int a = 0; a < NEN; ++a)
        inc[a] = base + (a & 1) + ((a >> 1) & 1) * A.nnx + (DIM == 3 ? ((a >> 2) & 1) * A.nnx * A.nny : 0);
    double Tn[NEN];
    bool hasT = A.temperature != nullptr;
#pragma unroll
    for (int a = 0; a < NEN; ++a) Tn[a] = hasT ? A.temperature[inc[a]] : 0.0;
    bool needL = A.u != nullptr && A.previous_solution;
    double un[DIM][NEN];
    if (needL) {
#pragma unroll
        for (int d = 0; d < DIM; ++d)
#pragma unroll
            for (int a = 0; a < NEN; ++a) un[d][a] = A.u[(int64_t)d * A.nn + inc[a]];
    }
    double pressure = A.p ? A.p[e] : 0.0;

    uint32_t beg = A.offsets[e], end = A.offsets[e + 1];
    uint32_t cnt = end - beg;
    if (cnt == 0) atomicOr(A.flags, 1u);
    const double cellVolume = DIM == 3 ? 8.0 : 4.0;
    double w = cellVolume / (double)cnt;

    constexpr int NM = DIM == 3 ? 27 : 9;
    constexpr int NF = NEN;
    double mu[NM];
    double phi[NF];
#pragma unroll
    for (int i = 0; i < NM; ++i) mu[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NF; ++i) phi[i] = 0.0;

    for (uint32_t s = beg; s < end; ++s) {
        double xi[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xi[d] = A.sxi[(int64_t)d * A.nslots + s];
        if (DIM == 2) xi[2] = 0.0;
        int mi = A.smat[s];
        if (mi < 0 || mi >= A.nmat) {
            atomicOr(A.flags, 2u);
            mi = 0;
        }
        const uwgpu_material& m = A.mats[mi];
        // shape functions at xi (TrilinearElementType.c:249-263 / BilinearElementType.c:212-220)
        double N[NEN];
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            double v = DIM == 3 ? 0.125 : 0.25;
#pragma unroll
            for (int d = 0; d < DIM; ++d) v *= ((a >> d) & 1) ? (1.0 + xi[d]) : (1.0 - xi[d]);
            N[a] = v;
        }
        double L[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (needL) {
            // velocity gradient L[i][j] = du_i/dx_j from the global derivatives at xi
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                double gx[3];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    double v = (2.0 / h[d]) * (DIM == 3 ? 0.125 : 0.25) * (((a >> d) & 1) ? 1.0 : -1.0);
#pragma unroll
                    for (int q = 0; q < DIM; ++q)
                        if (q != d) v *= ((a >> q) & 1) ? (1.0 + xi[q]) : (1.0 - xi[q]);
                    gx[d] = v;
                }
#pragma unroll
                for (int i = 0; i < DIM; ++i)
#pragma unroll
                    for (int j = 0; j < DIM; ++j) L[i][j] += gx[j] * un[i][a];
            }
        }
        // global coordinate of the point (FeMesh_CoordLocalToGlobal on the affine element)
        double xg[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < DIM; ++d) xg[d] = x0[d] + 0.5 * h[d] * (xi[d] + 1.0);
        double peta = A.seta_in ? A.seta_in[s] : 0.0;
        const uint32_t pidx = A.perm[s];
        double eta = run_rheology<DIM>(m, N, Tn, hasT, xg, A.max[1], peta, L, pressure, A.previous_solution,
                                       A.pfw ? A.pfw[pidx] : 0.0, A.pfw_incr ? A.pfw_incr + pidx : nullptr);
        if (A.eta_out) A.eta_out[s] = eta;
        double rho0 = A.srho_in ? A.srho_in[s] : m.density;
        double T = 0.0;
        if (hasT && m.alpha != 0.0) {
#pragma unroll
            for (int a = 0; a < NEN; ++a) T += N[a] * Tn[a];
        }
        double rho = rho0 * (1.0 - m.alpha * (T - m.ref_temp));

        const double ws = A.sw ? A.sw[s] : w;
        double c = ws * eta;
        double r = ws * rho;
        if (DIM == 3) {
            double x1 = xi[0], y1 = xi[1], z1 = xi[2];
            double x2 = x1 * x1;
            double cz0 = c, cz1 = c * z1, cz2 = cz1 * z1;
            double cyz[3][3];
            cyz[0][0] = cz0;
            cyz[0][1] = cz1;
            cyz[0][2] = cz2;
            cyz[1][0] = cz0 * y1;
            cyz[1][1] = cz1 * y1;
            cyz[1][2] = cz2 * y1;
            cyz[2][0] = cyz[1][0] * y1;
            cyz[2][1] = cyz[1][1] * y1;
            cyz[2][2] = cyz[1][2] * y1;
#pragma unroll
            for (int b = 0; b < 3; ++b)
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) {
                    double v = cyz[b][cc];
                    mu[0 * 9 + b * 3 + cc] += v;
                    mu[1 * 9 + b * 3 + cc] = fma(x1, v, mu[1 * 9 + b * 3 + cc]);
                    mu[2 * 9 + b * 3 + cc] = fma(x2, v, mu[2 * 9 + b * 3 + cc]);
                }
            double rz = r * z1, ry = r * y1, ryz = ry * z1;
            phi[0] += r;
            phi[1] = fma(x1, r, phi[1]);
            phi[2] += ry;
            phi[3] = fma(x1, ry, phi[3]);
            phi[4] += rz;
            phi[5] = fma(x1, rz, phi[5]);
            phi[6] += ryz;
            phi[7] = fma(x1, ryz, phi[7]);
        } else {
            double x1 = xi[0], y1 = xi[1];
            double x2 = x1 * x1;
            double cy0 = c, cy1 = c * y1, cy2 = cy1 * y1;
            double cy[3] = {cy0, cy1, cy2};
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                mu[0 * 3 + b] += cy[b];
                mu[1 * 3 + b] = fma(x1, cy[b], mu[1 * 3 + b]);
                mu[2 * 3 + b] = fma(x2, cy[b], mu[2 * 3 + b]);
            }
            double ry = r * y1;
            phi[0] += r;
            phi[1] = fma(x1, r, phi[1]);
            phi[2] += ry;
            phi[3] = fma(x1, ry, phi[3]);
        }
    }

    // ---- contraction of the moments into K_e ----
    // detJ of the affine element and derivative scales (ElementType.c:354-495 reduces to these)
    double detJ = DIM == 3 ? (0.5 * h[0]) * (0.5 * h[1]) * (0.5 * h[2]) : (0.5 * h[0]) * (0.5 * h[1]);
    double g[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) g[d] = 2.0 / h[d];
    const double inv64 = DIM == 3 ? 1.0 / 64.0 : 1.0 / 16.0;

    if (DIM == 3) {
        const int64_t ne = A.ne;
        double diag[ND];
        if (A.mom) {
            // moments out; K_e and S_e come from the tensor-core contraction (k_contract_tc)
#pragma unroll
            for (int m = 0; m < NM; ++m) A.mom[(int64_t)m * ne + e] = mu[m];
        } else {
            Tables3 T;
            tables_from_moments(mu, T);
            ke_from_tables(T, detJ, g, e, ne, A.Ke, diag);
        }
        // G_e: integral of -dN_a/dx_d over the element (exact for the 2x2x2 Gauss rule)
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double G = ge_entry(h, a, d);
                A.Ge[(int64_t)(a * 3 + d) * ne + e] = G;
                if (!A.mom) s += G * (G / diag[a * 3 + d]);
            }
        if (!A.mom) A.Se[e] = s;
        // f_e: -g detJ sum_p w rho N_a on the vertical component
        double fs = -A.gravity * detJ * 0.125;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            double sx = (a & 1) ? 1.0 : -1.0, sy = ((a >> 1) & 1) ? 1.0 : -1.0, sz = ((a >> 2) & 1) ? 1.0 : -1.0;
            double v = phi[0] + sx * phi[1] + sy * phi[2] + sx * sy * phi[3] + sz * phi[4] + sx * sz * phi[5] +
                       sy * sz * phi[6] + sx * sy * sz * phi[7];
#pragma unroll
            for (int d = 0; d < 3; ++d) A.fe[(int64_t)(a * 3 + d) * ne + e] = (d == A.vert_axis) ? fs * v : 0.0;
        }
    } else {
        double Dxx[3], Dyy[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            double sx = 0.0, sy = 0.0;
#pragma unroll
            for (int u = 0; u < 3; ++u) {
                sx += kQ[t][u] * mu[0 * 3 + u];
                sy += kQ[t][u] * mu[u * 3 + 0];
            }
            Dxx[t] = sx;
            Dyy[t] = sy;
        }
        double Mxy[2][2];
#pragma unroll
        for (int ta = 0; ta < 2; ++ta)
#pragma unroll
            for (int tb = 0; tb < 2; ++tb) {
                double v = 0.0;
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int q = 0; q < 2; ++q) v += kL[ta][u] * kL[tb][q] * mu[u * 3 + q];
                Mxy[ta][tb] = v;
            }
        auto Mkl = [&](int k, int l, int i, int j) -> double {
            int si[2] = {((i & 1) << 1) - 1, (((i >> 1) & 1) << 1) - 1};
            int sj[2] = {((j & 1) << 1) - 1, (((j >> 1) & 1) << 1) - 1};
            double sc = detJ * g[k] * g[l] * inv64 * (double)(si[k] * sj[l]);
            if (k == l) {
                if (k == 0) return sc * Dxx[qtype(si[1], sj[1])];
                return sc * Dyy[qtype(si[0], sj[0])];
            }
            if (k > l) {
                for (int q = 0; q < 2; ++q) { int t = si[q]; si[q] = sj[q]; sj[q] = t; }
            }
            return sc * Mxy[ltype(sj[0])][ltype(si[1])];
        };
        const int64_t ne = A.ne;
        double diag[ND];
#pragma unroll
        for (int i = 0; i < NEN; ++i)
#pragma unroll
            for (int j = i; j < NEN; ++j) {
                double tr = Mkl(0, 0, i, j) + Mkl(1, 1, i, j);
#pragma unroll
                for (int al = 0; al < 2; ++al)
#pragma unroll
                    for (int be = 0; be < 2; ++be) {
                        int r = i * 2 + al, cix = j * 2 + be;
                        if (r > cix) continue;
                        double v = Mkl(be, al, i, j) + (al == be ? tr : 0.0);
                        A.Ke[(int64_t)packed_index(ND, r, cix) * ne + e] = v;
                        if (r == cix) diag[r] = v;
                    }
            }
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                double sa = ((a >> d) & 1) ? 1.0 : -1.0;
                double G = -sa * h[1 - d] * 0.5;
                A.Ge[(int64_t)(a * 2 + d) * ne + e] = G;
                s += G * (G / diag[a * 2 + d]);
            }
        A.Se[e] = s;
        double fs = -A.gravity * detJ * 0.25;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            double sx = (a & 1) ? 1.0 : -1.0, sy = ((a >> 1) & 1) ? 1.0 : -1.0;
            double v = phi[0] + sx * phi[1] + sy * phi[2] + sx * sy * phi[3];
#pragma unroll
            for (int d = 0; d < 2; ++d) A.fe[(int64_t)(a * 2 + d) * ne + e] = (d == A.vert_axis) ? fs * v : 0.0;
        }
    }
}

// ---- the Newton (Jacobian) form of the 2D element matrices ---------------------------------
// ConstitutiveMatrixCartesian.c:360-383: with the SLE's nlFormJacobian the 2D loop adds, per point,
// the viscosity's derivatives with respect to the velocity gradient (set by yielding laws) to the
// viscous term, so K_e is no longer symmetric and the moment form does not apply: each point is
// accumulated directly into the 64 entries, element-major per entry ([i][j][e], i the matrix row
// (test function), j the column).  S_e is formed from this K_e's diagonal.  (The reference's
// Ni term multiplies derivs[2] and derivs[5], which no law sets; it is left out.)
__global__ void __launch_bounds__(128) k_assemble_jacobian2d(AssemblyArgs A, double* __restrict__ Kj) {
    constexpr int NEN = 4, ND = 8;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.ne) return;
    const int64_t ie = e % A.nel[0], je = e / A.nel[0];
    const int64_t idx[2] = {ie, je};
    double x0[3] = {0.0, 0.0, 0.0}, h[2];
    for (int d = 0; d < 2; ++d) {
        x0[d] = node_coord_1d(idx[d], A.nel[d], A.min[d], A.max[d]);
        h[d] = node_coord_1d(idx[d] + 1, A.nel[d], A.min[d], A.max[d]) - x0[d];
    }
    const int64_t base = ie + A.nnx * je;
    int64_t inc[NEN];
    for (int a = 0; a < NEN; ++a) inc[a] = base + (a & 1) + ((a >> 1) & 1) * A.nnx;
    double Tn[NEN];
    const bool hasT = A.temperature != nullptr;
    for (int a = 0; a < NEN; ++a) Tn[a] = hasT ? A.temperature[inc[a]] : 0.0;
    double un[2][NEN];
    for (int d = 0; d < 2; ++d)
        for (int a = 0; a < NEN; ++a) un[d][a] = A.u ? A.u[(int64_t)d * A.nn + inc[a]] : 0.0;
    const double pressure = A.p ? A.p[e] : 0.0;
    const uint32_t beg = A.offsets[e], end = A.offsets[e + 1];
    const uint32_t cnt = end - beg;
    const double w = 4.0 / (double)(cnt ? cnt : 1);
    const double detJ = (0.5 * h[0]) * (0.5 * h[1]);
    double K[ND * ND];
#pragma unroll
    for (int k = 0; k < ND * ND; ++k) K[k] = 0.0;
    for (uint32_t s = beg; s < end; ++s) {
        double xi[3] = {A.sxi[s], A.sxi[A.nslots + s], 0.0};
        int mi = A.smat[s];
        if (mi < 0 || mi >= A.nmat) mi = 0;
        const uwgpu_material& m = A.mats[mi];
        double N[NEN], G[2][NEN];
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            const double sx = (a & 1) ? 1.0 : -1.0, sy = ((a >> 1) & 1) ? 1.0 : -1.0;
            N[a] = 0.25 * (1.0 + sx * xi[0]) * (1.0 + sy * xi[1]);
            G[0][a] = (2.0 / h[0]) * 0.25 * sx * (1.0 + sy * xi[1]);
            G[1][a] = (2.0 / h[1]) * 0.25 * sy * (1.0 + sx * xi[0]);
        }
        double L[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) L[i][j] += G[j][a] * un[i][a];
        double xg[3] = {x0[0] + 0.5 * h[0] * (xi[0] + 1.0), x0[1] + 0.5 * h[1] * (xi[1] + 1.0), 0.0};
        const double peta = A.seta_in ? A.seta_in[s] : 0.0;
        const uint32_t pidx = A.perm[s];
        double derivs[9];
        const double eta = run_rheology<2>(m, N, Tn, hasT, xg, A.max[1], peta, L, pressure, A.previous_solution,
                                           A.pfw ? A.pfw[pidx] : 0.0, nullptr, derivs, true);
        const double intFac = (A.sw ? A.sw[s] : w) * detJ;
        const double DuDx = L[0][0], DuDy = L[0][1], DvDx = L[1][0], DvDy = L[1][1];
#pragma unroll
        for (int r = 0; r < NEN; ++r) {
            const double Bj_x = G[0][r], Bj_y = G[1][r];
            const double DetaDu = derivs[0] * Bj_x + derivs[1] * Bj_y;
            const double DetaDv = derivs[3] * Bj_x + derivs[4] * Bj_y;
#pragma unroll
            for (int c = 0; c < NEN; ++c) {
                const double Bi_x = G[0][c], Bi_y = G[1][c];
                double fac = eta * Bj_y + DuDy * DetaDu + DvDx * DetaDu;
                K[(c * 2) * ND + r * 2] += intFac * (2.0 * Bi_x * (eta * Bj_x + DuDx * DetaDu) + Bi_y * fac);
                K[(c * 2 + 1) * ND + r * 2] += intFac * (2.0 * Bi_y * DvDy * DetaDu + Bi_x * fac);
                fac = eta * Bj_x + DvDx * DetaDv + DuDy * DetaDv;
                K[(c * 2) * ND + r * 2 + 1] += intFac * (2.0 * Bi_x * DuDx * DetaDv + Bi_y * fac);
                K[(c * 2 + 1) * ND + r * 2 + 1] += intFac * (2.0 * Bi_y * (eta * Bj_y + DvDy * DetaDv) + Bi_x * fac);
            }
        }
    }
    const int64_t ne = A.ne;
#pragma unroll
    for (int k = 0; k < ND * ND; ++k) Kj[(int64_t)k * ne + e] = K[k];
    double sacc = 0.0;
#pragma unroll
    for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            const double sa = ((a >> d) & 1) ? 1.0 : -1.0;
            const double Gv = -sa * h[1 - d] * 0.5;
            sacc += Gv * (Gv / K[(a * 2 + d) * ND + a * 2 + d]);
        }
    A.Se[e] = sacc;
}

// ---- tensor-core contraction of the 3D moments into K_e -------------------------------------
// The 63 pair tables are integer combinations of the 27 moments (table_coefficient), so for a
// tile of 128 elements they form one product Tab = Mom C^T with C (63 x 27) of small integers.
// It runs on the tensor core in FP16 with FP64 accuracy by the error-free splitting of Ozaki,
// Ogita, Oishi and Rump ("Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms 59, 2012): each
// element's moments are scaled by a power of two s_e >= max |mu| and cut into five slices of 11
// bits, mu = s_e sum_j a_j 2^(-11 (j+1)) with integers |a_j| < 2^11 (exact in FP16).  A slice
// times C is an integer below 27 * 2^11 * 4 < 2^24, exact in the FP32 accumulator, so the only
// error is the truncation after 55 bits (relative 2^-55 of the element's largest moment) and the
// FP64 sum of the five slice products.  The epilogue forms K_e and S_e from the tables in FP64
// (ke_from_tables, as the FP64 path does).
constexpr int kSlices = 5;
constexpr int kTabN = 64;   // 63 tables + a zero row
constexpr int kMomK = 32;   // 27 moments + zero columns

struct ContractArgs {
    int nel[3];
    double min[3], max[3];
    int64_t ne;
    const double* mom;   // [27][e]
    double* Ke;          // packed, entry-major
    double* Se;
    uint32_t* err;
};

__global__ void __launch_bounds__(128, 1) k_contract_tc(ContractArgs A) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    unsigned char* sB = smem;                                   // 64 x 32 FP16, K-major
    unsigned char* sA = smem + kTabN * kMomK * 2;               // kSlices x (128 x 32 FP16)
    const uint32_t bytesA = 128 * kMomK * 2;
    constexpr uint32_t kCols = 512;                             // 5 x 64 accumulator columns
    if (warp == 0) {
        tc::tmem_alloc(&tbase, kCols);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&bar, 1);
    for (int idx = tid; idx < kTabN * kMomK; idx += 128) {
        const int q = idx / kMomK, m = idx % kMomK;
        const float v = m < 27 ? (float)table_coefficient(q, m) : 0.0f;
        *reinterpret_cast<__half*>(sB + tc::k_major_offset(q, m, kMomK)) = __float2half_rn(v);
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_f16(128, kTabN, tc::kFmtF16, 0, 0);
    const int64_t ne = A.ne;
    const int64_t ntiles = (ne + 127) / 128;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e = tile * 128 + tid;
        const bool live = e < ne;
        // this element's moments, scaled by 2^-ex so that |t| < 1, cut into five 11-bit slices
        double t[27];
        double mx = 0.0;
#pragma unroll
        for (int m = 0; m < 27; ++m) {
            t[m] = live ? A.mom[(int64_t)m * ne + e] : 0.0;
            mx = fmax(mx, fabs(t[m]));
        }
        int ex = 0;
        frexp(mx, &ex);   // mx < 2^ex
#pragma unroll
        for (int m = 0; m < 27; ++m) t[m] = ldexp(t[m], -ex);
#pragma unroll
        for (int j = 0; j < kSlices; ++j) {
#pragma unroll
            for (int c8 = 0; c8 < kMomK / 8; ++c8) {
                uint4 chunk;
                __half* hv = reinterpret_cast<__half*>(&chunk);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int m = c8 * 8 + i;
                    float a = 0.0f;
                    if (m < 27) {
                        const double u = t[m] * 2048.0;
                        const double w = trunc(u);
                        t[m] = u - w;
                        a = (float)w;
                    }
                    hv[i] = __float2half_rn(a);
                }
                *reinterpret_cast<uint4*>(sA + j * bytesA + tc::k_major_offset(tid, c8 * 8, kMomK)) = chunk;
            }
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t b = tc::smem_u32(sB), a0 = tc::smem_u32(sA);
#pragma unroll
            for (int j = 0; j < kSlices; ++j)
#pragma unroll
                for (int s = 0; s < kMomK / 16; ++s)
                    tc::mma_f16(taddr + (uint32_t)(j * kTabN), tc::k_major_desc(a0 + j * bytesA, s, kMomK),
                                tc::k_major_desc(b, s, kMomK), idesc, s > 0 ? 1u : 0u);
            tc::mma_commit(&bar);
        }
        ok = tc::mbar_wait(&bar, phase) && ok;
        phase ^= 1u;
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        tc::fence_after_sync();
        // tables = 2^ex sum_j D_j 2^(-11 (j+1)), each D_j an exact integer in FP32
        double T[kTabN];
#pragma unroll
        for (int q = 0; q < kTabN; ++q) T[q] = 0.0;
#pragma unroll
        for (int j = 0; j < kSlices; ++j) {
            const double sc = ldexp(1.0, ex - 11 * (j + 1));
#pragma unroll
            for (int c = 0; c < kTabN; c += 16) {
                uint32_t r[16];
                tc::tmem_ld16(tc::tmem_addr(taddr, 32 * warp, j * kTabN + c), r);
                tc::tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) T[c + i] = fma((double)__uint_as_float(r[i]), sc, T[c + i]);
            }
        }
        tc::fence_before_sync();
        if (live) {
            Tables3 tb;
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                tb.Dxx[i / 3][i % 3] = T[i];
                tb.Dyy[i / 3][i % 3] = T[9 + i];
                tb.Dzz[i / 3][i % 3] = T[18 + i];
            }
#pragma unroll
            for (int i = 0; i < 12; ++i) {
                tb.Mxy[i / 6][(i / 3) % 2][i % 3] = T[27 + i];
                tb.Mxz[i / 6][(i / 3) % 2][i % 3] = T[39 + i];
                tb.Myz[i / 6][(i / 3) % 2][i % 3] = T[51 + i];
            }
            const int64_t ie = e % A.nel[0], je = (e / A.nel[0]) % A.nel[1], ke = e / ((int64_t)A.nel[0] * A.nel[1]);
            const int64_t idx[3] = {ie, je, ke};
            double h[3], g[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double x0 = node_coord_1d(idx[d], A.nel[d], A.min[d], A.max[d]);
                h[d] = node_coord_1d(idx[d] + 1, A.nel[d], A.min[d], A.max[d]) - x0;
                g[d] = 2.0 / h[d];
            }
            const double detJ = (0.5 * h[0]) * (0.5 * h[1]) * (0.5 * h[2]);
            double diag[24];
            ke_from_tables(tb, detJ, g, e, ne, A.Ke, diag);
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const double G = ge_entry(h, a, d);
                    s += G * (G / diag[a * 3 + d]);
                }
            A.Se[e] = s;
        }
    }
    if (!ok && tid == 0) atomicOr(A.err, 4u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, kCols);
    }
}

// One TimeIntegrand Euler step of the strain-weakening history with the derivative the last
// assembly stored, then the clamp at zero (StrainWeakening.c:399-426).
__global__ void k_pfw_advance(int64_t n, double dt, const double* __restrict__ incr, double* __restrict__ pfw) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = pfw[i] + dt * incr[i];
    pfw[i] = v < 0.0 ? 0.0 : v;
}

void strain_weakening_advance(Context& c, double dt) {
    {
        LaunchScope ls(c, UWGPU_KERNEL_ASSEMBLY);
        k_pfw_advance<<<blocks_for(c.np, 256), 256, 0, c.stream>>>(c.np, dt, c.pfw_incr.p, c.pfw.p);
    }
    check_launch("k_pfw_advance");
    c.assembled = false;
}

void assemble(Context& c) {
    UWG_REQUIRE(c.mapped, UWGPU_ERR_STATE, "assemble called before bin_and_map");
    UWG_REQUIRE(c.nmat > 0, UWGPU_ERR_STATE, "materials not set");
    const MeshDesc& m = c.mesh;
    int dim = m.dim, nen = 1 << dim, nd = nen * dim;
    int64_t ne = m.ne;
    Level& L0 = c.levels[0];
    L0.mesh = m;
    L0.Ke.ensure((size_t)packed_size(nd) * ne);
    c.fe.ensure((size_t)nd * ne);
    c.Ge.ensure((size_t)nd * ne);
    c.Se.ensure((size_t)ne);
    c.seta_out.ensure((size_t)(c.np > 0 ? c.np : 1));
    c.err_count.ensure(1);
    UWG_CUDA(cudaMemsetAsync(c.err_count.p, 0, sizeof(uint32_t), c.stream));

    AssemblyArgs A;
    A.dim = dim;
    for (int d = 0; d < 3; ++d) {
        A.nel[d] = m.nel[d];
        A.min[d] = m.min[d];
        A.max[d] = m.max[d];
    }
    A.ne = ne;
    A.nslots = c.np;
    A.offsets = c.offsets.p;
    integration_points(c, &A.sxi, &A.sw);
    A.smat = c.smat.p;
    A.seta_in = c.has_peta ? c.seta_in.p : nullptr;
    A.srho_in = c.has_prho ? c.srho_in.p : nullptr;
    A.mats = c.mats.p;
    A.nmat = c.nmat;
    A.temperature = c.has_temperature ? c.temperature.p : nullptr;
    A.u = c.has_solution ? c.u_sol.p : nullptr;
    A.p = c.has_solution ? c.p_sol.p : nullptr;
    A.previous_solution = c.has_solution ? 1 : 0;
    A.vert_axis = c.vert_axis;
    A.gravity = c.gravity;
    A.nnx = m.nnx;
    A.nny = m.nny;
    A.nn = m.nn;
    A.Ke = L0.Ke.p;
    A.fe = c.fe.p;
    A.Ge = c.Ge.p;
    A.Se = c.Se.p;
    A.eta_out = c.seta_out.p;
    A.flags = c.err_count.p;
    A.perm = c.perm.p;
    A.pfw = c.has_pfw ? c.pfw.p : nullptr;
    A.pfw_incr = c.has_pfw ? c.pfw_incr.p : nullptr;
    const bool tcpath = dim == 3 && c.assembly_mode == UWGPU_ASSEMBLY_TENSOR;
    A.mom = nullptr;
    if (tcpath) {
        c.mom.ensure((size_t)27 * ne);
        A.mom = c.mom.p;
    }
    {
        // algorithmic bytes: per point xi + material (+ optional inputs) read, viscosity written;
        // per element offsets read, packed K_e, f_e, G_e, S_e written
        double per_point = dim * 8.0 + 4.0 + 8.0 + (c.has_peta ? 8.0 : 0.0) + (c.has_prho ? 8.0 : 0.0) +
                           (A.sw ? 8.0 : 0.0);
        // (the tensor-core form writes the 27 moments instead of K_e and S_e, and its contraction
        // kernel reads them back: 2 x 216 B more per element)
        double per_el = 4.0 + packed_size(nd) * 8.0 + 2.0 * nd * 8.0 + 8.0 + (tcpath ? 2.0 * 27 * 8.0 : 0.0);
        double flops_point = dim == 3 ? 120.0 : 50.0, flops_el = dim == 3 ? 3600.0 : 300.0;
        note_work(c, UWGPU_KERNEL_ASSEMBLY, per_point * c.np + per_el * ne, flops_point * c.np + flops_el * ne);
        LaunchScope ls(c, UWGPU_KERNEL_ASSEMBLY);
        if (dim == 3)
            k_assemble<3><<<blocks_for(ne, 128), 128, 0, c.stream>>>(A);
        else
            k_assemble<2><<<blocks_for(ne, 128), 128, 0, c.stream>>>(A);
    }
    check_launch("k_assemble");
    if (tcpath) {
        ContractArgs C;
        for (int d = 0; d < 3; ++d) {
            C.nel[d] = m.nel[d];
            C.min[d] = m.min[d];
            C.max[d] = m.max[d];
        }
        C.ne = ne;
        C.mom = c.mom.p;
        C.Ke = L0.Ke.p;
        C.Se = c.Se.p;
        C.err = c.err_count.p;
        // 512 TMEM columns per CTA: the shared-memory request keeps one CTA per SM
        int per_sm = 1;
        const size_t smem = tmem_safe_smem((const void*)k_contract_tc, c.device,
                                           (size_t)kTabN * kMomK * 2 + (size_t)kSlices * 128 * kMomK * 2, 512, &per_sm);
        int nsm = 1;
        UWG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
        const int64_t ntiles = (ne + 127) / 128;
        LaunchScope ls(c, UWGPU_KERNEL_ASSEMBLY);
        k_contract_tc<<<(unsigned)(ntiles < nsm ? ntiles : nsm), 128, smem, c.stream>>>(C);
    }
    check_launch("k_contract_tc");
    uint32_t flags = 0;
    UWG_CUDA(cudaMemcpyAsync(&flags, c.err_count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    UWG_CUDA(cudaStreamSynchronize(c.stream));
    c.assembled = true;
    c.operator_built = false;
    if (flags & 4u) throw Error(UWGPU_ERR_CUDA, "tensor-core contraction: an MMA did not complete in time");
    c.assembled_jacobian = false;
    if (c.jacobian && dim == 2 && !(flags & 3u)) {
        c.Kjac.ensure((size_t)64 * ne);
        {
            LaunchScope ls(c, UWGPU_KERNEL_ASSEMBLY);
            k_assemble_jacobian2d<<<blocks_for(ne, 128), 128, 0, c.stream>>>(A, c.Kjac.p);
        }
        check_launch("k_assemble_jacobian2d");
        UWG_CUDA(cudaStreamSynchronize(c.stream));
        c.assembled_jacobian = true;
    }
    if (flags & 2u) throw Error(UWGPU_ERR_ARGUMENT, "material index out of range");
    if (flags & 1u)
        throw Error(UWGPU_ERR_ARGUMENT,
                    "an element holds no integration points (zero element contribution is not allowed)");
}

}  // namespace uwg
