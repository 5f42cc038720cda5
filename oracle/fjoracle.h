/*
 * fjoracle.h -- CPU oracle for the fJmodels density / moment hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference algorithm (lposti/fJmodels) used as the checker for the CUDA
 * path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  It is never linked into the product library.
 *
 * Pinning: the restatement is checked against fixtures produced by the
 * reference's own, unmodified C++ sources compiled against a GSL stand-in
 * (oracle/ref_build, tests/golden).  The GSL algorithms themselves (Brent,
 * QAGS/QAGIU, the orbit integrator) are restated from their published
 * descriptions; parity at that boundary is unpinned.
 *
 * All arrays are row-major: a [nr][npoly] table element (n, l) is t[n*npoly+l].
 */
#ifndef FJORACLE_H
#define FJORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* DF variants */
#define ORC_DF_DPL 0      /* double power law + k*tanh(chi*Jphi/J0) rotation (DF.cpp:65-76,108-123) */
#define ORC_DF_QUASIISO 1 /* quasi-isothermal DF, the reference's live branch (DF.cpp:94-106)      */

typedef struct orc_model {
    int nr, npoly, ngauss, ngrid;
    const double *ar;              /* [nr] radial grid                         */
    const double *phil, *Pr, *Pr2; /* [nr*npoly] potential multipoles          */
    const double *Egrid, *Dgrid;   /* [ngrid] focal-distance table (Dgrid=D^2) */
    int df_kind;
    double alpha, beta, J0, mass;
    double dphi_h, dz_h, dphi_g, dz_g, chi, k;
    int nq;                        /* velocity rule, same on the three axes */
    const double *xq, *wq;
    int jquad;                     /* 0: QAGS (GSL wrapper semantics); n>0: n-point Gauss-Legendre */
} orc_model;

typedef struct orc_stats {
    long long nodes, bound, phi_evals, grad_evals, brent_iters, quad_evals, failures;
} orc_stats;

/* ---- numerics ---- */
void orc_gauleg(double x1, double x2, int n, double *x, double *w);
int orc_brent_wrapped(double (*f)(double, void *), void *p, double lo, double hi, double *root);
int orc_qags(double (*f)(double, void *), void *p, double a, double b, double epsabs,
             double epsrel, int limit, double *result, double *abserr);
int orc_qagiu(double (*f)(double, void *), void *p, double a, double epsabs, double epsrel,
              int limit, double *result, double *abserr);

/* ---- potential (Potential.cpp, UtilsLeg.h) ---- */
void orc_evenlegend(int npoly, double c, double *pol);
double orc_phi(const orc_model *m, double R, double z);
double orc_dR(const orc_model *m, double R, double z);
double orc_dz(const orc_model *m, double R, double z);
void orc_getfreqs(const orc_model *m, double R, double *kappa, double *nu, double *Omega);
void orc_log_grid(double rmin, double rmax, int n, double *ar);

/* ---- actions (uvOrb.cpp) ---- */
double orc_deltafn(const orc_model *m, double E);
/* returns 1 if bound; Jr/Jz are 1e31 for an unbound orbit */
int orc_actions(const orc_model *m, double Delta, double R, double z, double Phi, double pR,
                double vphi, double pz, double *Jr, double *Jz, orc_stats *st);

/* ---- DF, moments (DF.cpp, Integ.cpp, potLeg.cpp) ---- */
double orc_df(const orc_model *m, double R, double z, double Phi, const double *V, orc_stats *st);
double orc_rhofDF(const orc_model *m, double R, double z, double *mom6, orc_stats *st);
/* grid of moments (rho, vrot, sigR, sigp, sigz, sigRz) on [nr][ngauss] points;
   points with index in [p0, p1) only (p = n*ngauss+g); nthreads OpenMP threads */
void orc_moment_grid(const orc_model *m, int p0, int p1, double *grids6, int nthreads, orc_stats *st);
/* rho[0][0] extrapolation (potLeg.cpp:68) + 6-field projection (UtilsLeg.h:200-253) */
void orc_project6(int nr, int ngauss, int npoly, const double *ar, double *grids6, double *coef6);
/* Poisson solve (Potential.cpp:110-200): rhl -> phil, Pr, Pr2 */
void orc_compute_phil(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                      double *Pr, double *Pr2);
/* the same solve with the radial integrals taken without adaptive
   quadrature (Gauss-Legendre per grid interval, running sums) */
void orc_compute_phil_cumulative(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                                 double *Pr, double *Pr2);
/* guess density multipoles (Potential.cpp:63-80): kind 0 Hernquist, 1 Isochrone, 2 NFW */
void orc_guess_rhl(int nr, int ngauss, int npoly, const double *ar, int kind, double mass,
                   double r0, double q, double *rhl);
/* tensor virial (Stats.cpp:12-41): out = {KRR, Kzz, WRR, Wzz, pot, mass_pr, mass_sum} */
void orc_vir2(const orc_model *m, const double *coef6, double *out7);
/* max |dphil|/|phil_0| (UtilsLeg.h:266-278 distance only) */
double orc_merge_distance(int nr, int npoly, const double *phil_new, const double *phil_old);
/* focal-distance table (tabulate.cpp:13-38 + Delta.cpp) */
int orc_tabulate_delta(const orc_model *m, double *Egrid, double *Dgrid);

/* ---- projected density, line profile, velocity distributions (Integ.cpp:32-43,63-135,168-220) ---- */
#define ORC_LOS_SIGMA 0  /* SigmaDF(R, z) from the density multipoles rhl      */
#define ORC_LOS_LINE 1   /* line_profile(R, z, vx): v = vx in units of Ve      */
#define ORC_LOS_PVPHI 2  /* P_vp(R, z, vphi)                                   */
#define ORC_LOS_PVZ 3    /* P_vz(R, z, vz)                                     */
#define ORC_LOS_PVR 4    /* P_vr(R, z, vR)                                     */
/* the 22-point tanh-sinh table on [0,1] of include/GaussPts.h (xpt01/xw01) */
void orc_tanh_sinh01(double *x, double *w);
/* one value; the model's rule (xq, wq) is the [-1,1] rule (xpt11/xw11), x01/w01 the
   [0,1] rule (22 points), rhl [nr*npoly] the density multipoles for SigmaDF */
double orc_los(const orc_model *m, const double *rhl, int kind, double R, double z, double v,
               const double *x01, const double *w01, orc_stats *st);

#ifdef __cplusplus
}
#endif
#endif
