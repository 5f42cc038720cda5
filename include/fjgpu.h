/*
 * fjgpu.h -- C ABI of the GB300 (sm_103a) implementation of the fJmodels
 * density / moment evaluation path.
 *
 * Conventions
 *   - Every table is contiguous row-major: a [nr][npoly] multipole table
 *     stores coefficient l=2*np at radius ar[n] in t[n*npoly+np]; a
 *     [nr][ngauss] meridional grid stores point (ar[n], cos theta_g) in
 *     g[n*ngauss+g].  The reference keeps the same matrices as row-pointer
 *     double** (include/Utils.h:71-75); a row-pointer matrix is adapted by
 *     copying its rows into (or out of) one contiguous buffer.
 *   - "device" pointers are CUDA global-memory pointers on the context's
 *     device; "host" pointers are ordinary memory.  Every call is ordered on
 *     the context's stream and returns after its work is queued unless the
 *     comment says it synchronises.
 *   - Return value: FJ_OK (0) or an FJ_ERR_* code; the reference's exit(n)
 *     paths become error codes (fj_last_error gives the text).  Per-node
 *     numerical failures (a capped bracket, Brent or QAGS limit) never abort:
 *     a capped bracket or root makes the node's DF contribute 0, as the
 *     reference's NaN guard does (df/DF.cpp:105); a full QAGS list keeps the
 *     integral's estimate so far; the counts are reported in fj_moment_stats.
 *   - One context per host thread; calls on one context are not re-entrant.
 */
#ifndef FJGPU_H
#define FJGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FJ_OK 0
#define FJ_ERR_ARG 1
#define FJ_ERR_CUDA 2
#define FJ_ERR_NOMEM 3
#define FJ_ERR_IO 4
#define FJ_ERR_NODEVICE 5

/* distribution function variants */
#define FJ_DF_DPL 0      /* double power law + k*tanh(chi*Jphi/J0) (df/DF.cpp:65-76,108-123) */
#define FJ_DF_QUASIISO 1 /* quasi-isothermal, the reference binary's live branch (df/DF.cpp:94-106) */

/* arithmetic of the phase-space kernel */
#define FJ_PREC_FP64 0  /* plain form: everything in FP64 */
#define FJ_PREC_MIXED 1 /* FP32 turning points, momentum quadrature and DF; FP64 node setup,
                           turning points at the u/v limits and accumulation (DPL DF, QAGS only) */

/* momentum integrals of the actions: 0 = adaptive QAGS as the reference
   (include/Utils.h:173-185); n > 0 = fixed n-point Gauss-Legendre */
#define FJ_JQUAD_QAGS 0

/* guess densities (pot/models.cpp:40-56), and the density of the external
   halo (rhoNFWext, pot/models.cpp:61-65: GM / (m/a (a + m)) / 4 pi, the
   reference's a = 25, GM = 0.01 passed as r0 and mass) */
#define FJ_GUESS_HERNQUIST 0
#define FJ_GUESS_ISOCHRONE 1
#define FJ_GUESS_NFW 2
#define FJ_GUESS_NFWEXT 3

typedef struct fj_ctx fj_ctx;

/* Multipole potential on a radial grid: the reference's global ar/phil/Pr/Pr2
   (include/Grid.h:19-22).  Requires 11 <= nr and 1 <= npoly <= 24. */
typedef struct fj_potential {
    int nr, npoly;
    const double *ar;   /* [nr]        */
    const double *phil; /* [nr*npoly]  */
    const double *Pr;   /* [nr*npoly]  dPhi_l/dr   */
    const double *Pr2;  /* [nr*npoly]  d2Phi_l/dr2 */
} fj_potential;

/* Focal-distance table of delta/tabulate.cpp (Egrid, Dgrid = Delta^2). */
typedef struct fj_delta_table {
    int ngrid;
    const double *Egrid, *Dgrid;
} fj_delta_table;

/* DF parameters of one component (df/DF.cpp:18-63, pot/models.cpp:13). */
typedef struct fj_df_params {
    int kind;                         /* FJ_DF_DPL or FJ_DF_QUASIISO */
    double alpha, beta;               /* slopes A, B */
    double J0, mass;                  /* J0 = sqrt(mass*r0) */
    double dphi_h, dz_h, dphi_g, dz_g;
    double chi, k;                    /* rotation: f*(1 + k*tanh(chi*Jphi/J0)) when chi > 0 */
} fj_df_params;

/* Velocity quadrature (the same nq-point rule on [-1,1] for vR, vphi, vz;
   include/GaussPts.h:79-88 is the reference's live rule), host arrays. */
typedef struct fj_quad_rule {
    int nq;            /* <= 64 */
    const double *xq;  /* [nq] host */
    const double *wq;  /* [nq] host */
    int jquad;         /* FJ_JQUAD_QAGS or Gauss-Legendre order (<= 64) */
    int precision;     /* FJ_PREC_FP64 or FJ_PREC_MIXED */
} fj_quad_rule;

typedef struct fj_moment_stats {
    long long nodes;     /* phase-space evaluations (grid points x nq^3) */
    long long bound;     /* nodes with H < 0 */
    long long failures;  /* nodes whose action solve hit a cap (after any FP64 re-solve) */
    double kernel_ms;    /* device time of the phase-space kernel (CUDA events) */
    long long escalated; /* FJ_PREC_MIXED: nodes whose turning points were solved in FP64 */
    /* failures by kind (a node can count in more than one): a momentum
       integral's QAGS list full (its estimate so far is kept, as QUADPACK
       returns it), a bracket walk or Brent at its step cap (the DF counts 0) */
    long long fail_quad, fail_bracket, fail_root;
    long long resolved64; /* FJ_PREC_MIXED: nodes whose FP32 solve hit a cap and were
                             solved again by the plain FP64 solve */
} fj_moment_stats;

/* ---------------------------------------------------------------- context */
const char *fj_version(void);
int fj_ctx_create(int device, fj_ctx **out);
int fj_ctx_destroy(fj_ctx *ctx);
/* Order subsequent work on the given cudaStream_t (passed as void*, used as
   is: NULL is the legacy default stream).  A new context works on its own
   stream, which is a blocking stream and so also orders after work on the
   legacy default stream. */
int fj_ctx_set_stream(fj_ctx *ctx, void *stream);
/* The context's own stream (to go back to it with fj_ctx_set_stream). */
void *fj_ctx_own_stream(fj_ctx *ctx);
int fj_ctx_synchronize(fj_ctx *ctx);
const char *fj_last_error(fj_ctx *ctx);

/* ----------------------------------------------------- hot path (device) */

/* Integ density/moment integrals over the meridional grid.
   Backs rhofDF(R,z,p,&vrot,&sigR,&sigp,&sigz,&sigRz) (include/Integ.h:19,
   integ/Integ.cpp:150-163) as called by computeRhl's grid loop
   (pot/potLeg.cpp:54-58).  The grid points are (ar[n]*sqrt(1-c_g^2), ar[n]*c_g)
   with c_g the ngauss Gauss-Legendre nodes on (0,1) (potLeg.cpp:43-47).
   grids6: device [6][nr*ngauss] = rho, vrot, sigR, sigp, sigz, sigRz. */
int fj_moments(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta,
               const fj_df_params *df, const fj_quad_rule *rule, int ngauss, double *grids6,
               fj_moment_stats *stats);

/* Same, for an explicit list of npts meridional points Rz (device [npts][2]);
   out6 device [6][npts].  The one-point form backs the 8-argument rhofDF. */
int fj_moments_points(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta,
                      const fj_df_params *df, const fj_quad_rule *rule, const double *Rz, int npts,
                      double *out6, fj_moment_stats *stats);

/* Projected density, line-of-sight velocity profile and velocity
   distributions: SigmaDF, line_profile, P_vp, P_vz, P_vr (integ/Integ.cpp:
   168-220 with SigmaInteg :32-43, lineProfile :63-92, Pvphi/Pvz/Pvr
   :97-135), n values of one kind at device Rzv [n][3] = (R, z, v):
     FJ_LOS_SIGMA  v unused: 2 x the line-of-sight integral of the density
                   from R to ar[nr-1] at height z, from the multipoles rhl;
     FJ_LOS_LINE   v = vx in units of the escape speed: the [-1,1]^3 rule over
                   (vy, x, vz), divided by SigmaDF (so rhl is needed too);
     FJ_LOS_PVPHI, FJ_LOS_PVZ, FJ_LOS_PVR  v = the fixed velocity component.
   The [-1,1] axes take `rule` (host arrays; precision FJ_PREC_FP64; jquad as
   for the moments), the [0,1] axes the reference's 22-point tanh-sinh table
   (fj_tanh_sinh01).  rhl device [nr*npoly] (may be NULL for PVPHI, PVZ,
   PVR); out device [n].  Plain FP64; a value's nodes in blocks of 1024, summed in a fixed order. */
#define FJ_LOS_SIGMA 0
#define FJ_LOS_LINE 1
#define FJ_LOS_PVPHI 2
#define FJ_LOS_PVZ 3
#define FJ_LOS_PVR 4
int fj_los(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
           const fj_quad_rule *rule, const double *rhl, int kind, const double *Rzv, int n, double *out,
           fj_moment_stats *stats);
/* The 22-point tanh-sinh table on [0,1] of include/GaussPts.h:91-134
   (xpt01/xw01), regenerated from its formula; host x[22], w[22]. */
int fj_tanh_sinh01(double *x, double *w);

/* Many models' phase-space integrals in one launch (no reference counterpart:
   the reference builds one model per process).  Item m is one model's
   computeRhl grid (pot/potLeg.cpp:35-70): its own device potential, Delta
   table, DF and polar node count, output grids6 device [6][nr*ngauss]; all
   items share the velocity rule (and form).  Blocks are assigned to models
   by a prefix table; the results are those of fj_moments per item. */
typedef struct fj_batch_item {
    fj_potential pot;
    fj_delta_table delta;
    fj_df_params df;
    int ngauss;
    double *grids6;
} fj_batch_item;
int fj_moments_batch(fj_ctx *ctx, int n, const fj_batch_item *items, const fj_quad_rule *rule,
                     fj_moment_stats *stats);

/* BF16 GEMM on the tensor cores (tcgen05, FP32 accumulation in tensor
   memory), the building block of the action surrogate; no reference
   counterpart.  C[M][N] = A[M][K] B[N][K]^T with A, B device BF16 (K
   contiguous, lda/ldb multiples of 8, 16-byte aligned), C device FP32 (row
   stride ldc), N and K multiples of 16; ksplit > 1 splits K across CTAs and
   accumulates with atomics.  Synchronises the stream.  FJ_ERR_CUDA if a
   tensor-core wait timed out. */
int fj_tc_gemm(int M, int N, int K, const void *A, int lda, const void *B, int ldb, float *C, int ldc, int ksplit,
               void *stream);

/* The action surrogate (no reference counterpart): an MLP 16 -> 128 x 4
   (GELU) -> 16 mapping normalised phase-space features (13 used, zero padded)
   to log h and log g of the double-power-law DF (outputs 0 and 1), trained and evaluated with the
   tensor-core GEMMs: BF16 weights and activations, FP32 accumulation and
   master weights, Adam.  batch = samples per training step (a multiple of
   128); work runs on the context's stream.  X device f32 [n][16], T device
   f32 [n][2] targets, Y device f32 [n][16] outputs.  fj_surrogate_params
   copies the parameters out (host_out) and/or in (host_in), laid out per
   layer as W [rows][cols] then b [rows]; fj_surrogate_gradients gives the
   mean-squared-error gradient of one batch (the first `batch` rows). */
/* Mixed form: also write (Jr, Jz) of every bound velocity node of the grid
   (device f32 [npts][nq^3][2], point-major as the grid; unbound nodes are
   left NaN) on subsequent fj_moments / fj_moments_points / fj_compute_new_phi
   calls of this context; NULL turns it off.  Feeds fj_surrogate_fit. */
int fj_set_action_output(fj_ctx *ctx, float *jout);

typedef struct fj_surrogate fj_surrogate;
int fj_surrogate_create(fj_ctx *ctx, int batch, unsigned long long seed, fj_surrogate **out);
int fj_surrogate_destroy(fj_surrogate *s);
long long fj_surrogate_nparam(const fj_surrogate *s);
int fj_surrogate_params(fj_surrogate *s, double *host_out, const double *host_in);
int fj_surrogate_gradients(fj_surrogate *s, const float *X, const float *T, double *grad_out, double *loss);
int fj_surrogate_train(fj_surrogate *s, const float *X, const float *T, long long n, int epochs, float lr,
                       double *final_loss);
int fj_surrogate_predict(fj_surrogate *s, const float *X, long long n, float *Y);
/* Fit to the exact actions J of a grid iteration (from fj_set_action_output,
   in potential pot): `samples` rows drawn with `seed` among bound nodes,
   features built on the device, targets log h and log g of the DF df,
   `epochs` of Adam at lr.  rho (device [nr*ngauss], the same iteration's
   densities; may be NULL) weights each row by 0.2 + nq^3 x the node's share
   of its point's density, so the fit concentrates where the density is. */
int fj_surrogate_fit(fj_surrogate *s, const fj_potential *pot, const fj_df_params *df, int ngauss,
                     const fj_quad_rule *rule, const float *J, const double *rho, long long samples,
                     unsigned long long seed, int epochs, float lr, double *loss);
/* computeRhl with the surrogate's actions: the features of every bound
   velocity node of the grid, the MLP on the tensor cores, the double-power-law
   DF and the moment sums into grids6 device [6][nr*ngauss]; ms = device time.
   fused = 1: one kernel per grid point (weights resident in shared memory,
   accumulators in tensor memory, nothing but the sums leaves the chip);
   fused = 0: features, GEMMs and sums as separate passes through memory. */
int fj_surrogate_moments(fj_surrogate *s, const fj_potential *pot, const fj_df_params *df, const fj_quad_rule *rule,
                         int ngauss, double *grids6, double *ms, int fused);

/* Configuration of the mixed-precision phase-space kernel (no reference
   counterpart: the reference has one CPU loop).  variant 0..7: 0..3 give
   each thread a fixed share of a block's velocity nodes, 4..7 let a thread
   take the next untaken node when it finishes one (the time per node varies
   by two orders of magnitude); within each, the register budget of the build
   (launch bounds of 3, 4, 6, 8 resident blocks per SM),
   nodes_per_block = velocity nodes of one point per block (128..8192).
   fj_autotune_mixed times every variant x {1024, 2048, 4096} with
   fj_moments_points on the given device sample points (out6 device
   [6][npts] scratch), keeps the fastest in the context and returns its
   kernel time (all_ms, if not NULL: host [8][3] times of every variant x
   {1024, 2048, 4096}); results are the same in every configuration up to
   the summation order of the per-thread sums (the two forms give the same
   bits at the same nodes_per_block). */
int fj_set_mixed_config(fj_ctx *ctx, int variant, int nodes_per_block);
int fj_get_mixed_config(fj_ctx *ctx, int *variant, int *nodes_per_block);
int fj_autotune_mixed(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
                      const fj_quad_rule *rule, const double *Rz, int npts, double *out6, double *best_ms,
                      double *all_ms);

/* rho[0][0] extrapolation (pot/potLeg.cpp:68) and the 6-field Legendre
   projection get_Ylm (include/UtilsLeg.h:200-253).  grids6 device
   [6][nr*ngauss] (read only), coef6 device [6][nr*npoly] = rhl, vrotl, sigRl,
   sigpl, sigzl, sigRzl. */
int fj_legendre_project(fj_ctx *ctx, int nr, int ngauss, int npoly, const double *ar,
                        const double *grids6, double *coef6);

/* Poisson solve Potential::computePhil (pot/Potential.cpp:110-200):
   QAGS / QAGIU radial integrals with the reference's tolerances and retry
   rule, then phil, Pr, Pr2.  All device [nr*npoly]. */
int fj_poisson(fj_ctx *ctx, int nr, int npoly, const double *ar, const double *rhl,
               double *phil, double *Pr, double *Pr2);

/* Poisson solve that allocates nothing and needs no context.  It has no
   counterpart in the reference: it is fj_poisson for callers that hold no
   fj_ctx or cannot allocate device memory on their call path (an
   application whose device memory belongs to its own pool allocator, a
   latency-bound loop).  The quadrature workspace lives in the kernel's
   shared memory.  Inputs and outputs are device pointers on the current
   device, work is queued on `stream` (a cudaStream_t; NULL = legacy default
   stream); calls on different streams are independent.  Any nr >= 2 and
   1 <= npoly <= 24 is accepted.  The kernel's per-thread stack must fit the
   device's current stack limit (CUDA's default 1024 bytes does): otherwise
   the call returns FJ_ERR_NOMEM without launching, since the launch would
   make the driver enlarge the local-memory reservation. */
int fj_poisson_noalloc(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                       double *Pr, double *Pr2, void *stream);
/* The per-thread stack (bytes) fj_poisson_noalloc's kernel needs, and the
   current device's per-thread stack limit (cudaLimitStackSize); either
   pointer may be NULL.  No counterpart in the reference. */
int fj_poisson_noalloc_stack(size_t *need, size_t *limit);

/* How fj_poisson (and every call that solves the Poisson equation on the
   context: fj_compute_new_phi, the model loops) takes the radial integrals:
     FJ_POISSON_QAGS        the reference's adaptive QAGS / QAGIU with its
                            tolerances and retry rule (the default; parity);
     FJ_POISSON_CUMULATIVE  the same integrands (the linear interpolation of
                            the density multipoles, the r^-4 tail beyond the
                            grid) integrated exactly, interval by interval,
                            as prefix sums in a fixed order (nr <= 4096).
   The adaptive form's answer moves by up to ~1e-3 of the potential when a
   small change of the density flips one of its subdivision decisions; the
   cumulative form is a smooth function of the density, so a self-consistent
   loop can converge below that level.  No counterpart in the reference. */
#define FJ_POISSON_QAGS 0
#define FJ_POISSON_CUMULATIVE 1
int fj_set_poisson(fj_ctx *ctx, int mode);
int fj_get_poisson(fj_ctx *ctx, int *mode);

/* updatePhil (pot/potLeg.cpp:21-29): out = a + b element-wise on the three
   tables (device [nr*npoly] each). */
int fj_sum_potentials(fj_ctx *ctx, int n, const double *phil_a, const double *Pr_a,
                      const double *Pr2_a, const double *phil_b, const double *Pr_b,
                      const double *Pr2_b, double *phil, double *Pr, double *Pr2);

/* computeNewPhi (pot/potLeg.cpp:76-82): moments, projection and Poisson in
   one stream-ordered call.  grids6, coef6 and the three output tables are
   device buffers; the output tables may not alias pot's tables. */
int fj_compute_new_phi(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta,
                       const fj_df_params *df, const fj_quad_rule *rule, int ngauss,
                       double *grids6, double *coef6, double *phil_out, double *Pr_out,
                       double *Pr2_out, fj_moment_stats *stats);

/* Staeckel-fudge actions: uvOrb(Delta, Lz, Phi, x, p, pot).Ju()/.Jv()
   (include/uvOrb.h:15,23-24; uvOrb/uvOrb.cpp:15-262) for n phase points
   pts device [n][5] = (R, z, vR, vphi, vz), with Delta = Deltafn(H)
   (delta/tabulate.cpp:40-44) as df() does.  out device [n][2] = (Jr, Jz);
   (-1,-1) marks H >= 0, 1e31 an unbound orbit.  jquad: FJ_JQUAD_QAGS or GL order. */
int fj_actions(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta,
               const double *pts, size_t n, int jquad, double *out);

/* Potential::operator(), dR, dz (pot/Potential.cpp:206-276) at n points
   Rz device [n][2]; out device [n][3] = (Phi, dPhi/dR, dPhi/dz). */
int fj_potential_eval(fj_ctx *ctx, const fj_potential *pot, const double *Rz, size_t n, double *out);

/* Tensor virial sums vir2 (libs/Stats.cpp:12-41).  coef6 device (as from
   fj_legendre_project).  out7 HOST = KRR, Kzz, WRR, Wzz, PE, mass from Pr at
   the last radius, mass from the density sum.  Synchronises. */
int fj_vir2(fj_ctx *ctx, const fj_potential *pot, int ngauss, const double *coef6, double *out7);

/* FMA throughput of the current device in TFLOP/s (fp32 = 0: FP64, 1: FP32),
   from a kernel of independent FMA chains; the roofline denominator of the
   phase-space kernel.  No counterpart in the reference (a measurement aid). */
int fj_measure_fma_peak(int fp32, double *tflops);

/* ------------------------------------------- host-side setup (run once) */

/* Logarithmic radial grid (include/Utils.h:76-81 with an explicit rmin). */
int fj_log_grid(double rmin, double rmax, int n, double *ar);
/* Gauss-Legendre nodes/weights on [x1,x2] (include/UtilsLeg.h:18-39). */
int fj_gauleg(double x1, double x2, int n, double *x, double *w);
/* Guess-density multipoles computeGuessRhl (pot/Potential.cpp:63-80), host arrays. */
int fj_guess_rhl(int nr, int ngauss, int npoly, const double *ar, int kind, double mass,
                 double r0, double q, double *rhl);
/* Focal-distance table tabulateDelta (delta/tabulate.cpp:13-38, delta/Delta.cpp),
   evaluated on the host from HOST potential tables.  Egrid/Dgrid host [ngrid]. */
int fj_tabulate_delta(const fj_potential *pot_host, int ngrid, double *Egrid, double *Dgrid);
/* The same tables of n models on the GPU, one thread per (model, energy)
   running the host's code (no reference counterpart: the reference tabulates
   one model).  pots host [n] of DEVICE potential tables (nr >= 11); Egrid,
   Dgrid device [n][ngrid]; status host [n] (may be NULL): FJ_OK, or
   FJ_ERR_ARG where a bracket or root search hit its cap (the host call's
   return value).  The energies agree with the host's to rounding; the focal
   distances are another draw of the same fit (the fit is not continuous in
   the rounding of the device's transcendental functions: entries move by
   ~10-20 %, the densities they give by a few per cent). */
int fj_tabulate_delta_batch(fj_ctx *ctx, int n, const fj_potential *pots, int ngrid, double *Egrid, double *Dgrid,
                            int *status);

/* Coefficient file writer _writeOut (io/writeOut.cpp:74-138): byte-identical
   output for identical arrays.  mats9 host [9][nr*npoly] in the file order
   rhl, vrotl, sigRl, sigpl, sigzl, sigRzl, phil, Pr, Pr2. */
int fj_write_out(const char *path, int nr, int npoly, int ngauss, const double *hdr10,
                 const double *ar, const double *mats9);
/* The same file with `digits` significant digits per value (0 = the
   reference's default stream precision, i.e. fj_write_out; 17 = every double
   read back exactly, for a full-precision restart). */
int fj_write_out_digits(const char *path, int nr, int npoly, int ngauss, const double *hdr10,
                        const double *ar, const double *mats9, int digits);
/* Reader of that file format (no reference counterpart: the reference writes
   its models but never reads them back).  Call with ar = mats9 = NULL to get
   nr, npoly, ngauss and hdr10[0..8] (dphi_h dz_h dphi_g dz_g chi mass r0 A B);
   then with host ar [nr] and mats9 [9][nr*npoly] for the arrays.  FJ_ERR_IO
   if the file cannot be opened, FJ_ERR_ARG if it is not in the format. */
int fj_read_out(const char *path, int *nr, int *npoly, int *ngauss, double *hdr10, double *ar,
                double *mats9);

/* ------------------------------------------- whole model (host buffers) */

/* One component of a self-consistent run (fJmodels.cpp:86-144 oneComp). */
typedef struct fj_model_config {
    int nr, ngauss, npoly, ngrid;
    double rmin, rmax;
    int guess;                   /* FJ_GUESS_* */
    double mass, r0, q;
    fj_df_params df;
    fj_quad_rule rule;           /* host arrays */
    int itermax;                 /* iterations */
    double tol;                  /* stop when max|dphil/phil_0| < tol (UtilsLeg.h:266-278); <= 0: run itermax */
    const double *Egrid_in;      /* optional host focal-distance table [ngrid] to use instead of */
    const double *Dgrid_in;      /* tabulating it from the guess potential; NULL: tabulate       */
    /* second component (fJmodels.cpp:38-84); ncomp 0 or 1 = one component */
    int ncomp;
    int guess2;                  /* FJ_GUESS_* of component 2 */
    double mass2, r0_2, q2;
    fj_df_params df2;
    int twocomp_order;           /* FJ_TWOCOMP_* */
    /* restart from written tables (fj_read_out; fj_run_model only): optional
       host arrays, NULL = start from the guess density's potential */
    const double *ar_in;         /* radial grid [nr] instead of the log grid of (rmin, rmax) */
    const double *phil_in;       /* total potential tables [nr*npoly] to iterate from; */
    const double *Pr_in;         /* the focal-distance table is tabulated from them unless */
    const double *Pr2_in;        /* Egrid_in/Dgrid_in are given                           */
    /* focal-distance table (no reference counterpart: the reference tabulates
       once, on the host, from the guess potential) */
    int delta_gpu;               /* 1: tabulate on the GPU (fj_tabulate_delta_batch) */
    int delta_every;             /* k > 0: re-tabulate from the new potential after every k-th
                                    iteration (fj_run_model_batch: 0 or 1, with delta_gpu) */
    /* a fixed external potential added to the model's own (the reference's
       commented-out external mode, fJmodels.cpp:120-125, 134: updatePhil after
       the guess and after every iteration); host [nr*npoly] tables, NULL = none.
       A restart's tables are taken as the total.  fj_run_model only. */
    const double *ext_phil, *ext_Pr, *ext_Pr2;
    /* Anderson mixing of the iteration (no reference counterpart: the reference
       iterates the plain map, fJmodels.cpp:131-143): 0 = the plain iteration;
       m in [1, FJ_ANDERSON_MAX_DEPTH] = each next input potential mixed from
       the last m + 1 outputs (fj_anderson_step).  With tol > 0 the loop ends
       with a plain step: a change below tol after a mixed step is confirmed by
       one plain step from that output, whose change must be below tol too.
       fj_run_model only. */
    int accel;
    double accel_beta;           /* the mixing factor of fj_anderson_reset, (0, 4]; 0 = 1 */
} fj_model_config;

/* Two-component iteration order.  SUMMED: both components' moments in the
   current total potential, one Poisson solve of the summed density
   multipoles.  REFERENCE: the reference's order (fJmodels.cpp:66-80 with
   Potential.cpp:182-188): component 1 in the total potential, whose own new
   potential then replaces the total, component 2 in that, total = sum of the
   two components' potentials (updatePhil, potLeg.cpp:21-29). */
#define FJ_TWOCOMP_SUMMED 0
#define FJ_TWOCOMP_REFERENCE 1

typedef struct fj_model_result {
    /* host arrays the caller allocated: ar [nr], coef6 [6][nr*npoly],
       phil/Pr/Pr2 [nr*npoly], Egrid/Dgrid [ngrid], grids6 [6][nr*ngauss] (may be NULL) */
    double *ar, *coef6, *phil, *Pr, *Pr2, *Egrid, *Dgrid, *grids6;
    double vir7[7];              /* vir2 sums after the last iteration */
    int iterations;
    double last_change;          /* max|dphil/phil_0| of the last iteration */
    long long bound, failures;
    double wall_ms, kernel_ms;
    double setup_ms;             /* wall time before the first iteration (grid, guess, Poisson, Delta table) */
    double *coef6_2;             /* two components: component 2's coefficients [6][nr*npoly] (may be NULL);
                                    coef6, vir7 and grids6 are component 1's */
    double vir7_2[7];            /* two components: vir2 sums of component 2 in the total potential */
} fj_model_result;

int fj_run_model(fj_ctx *ctx, const fj_model_config *cfg, fj_model_result *res);

/* Anderson mixing of the self-consistent iteration x <- G(x) over the
   potential tables (no reference counterpart).  The context keeps the history
   of one iteration: fj_anderson_reset starts it with depth m (0 = plain steps)
   and mixing factor beta in (0, 4].
   fj_anderson_step takes the device tables x (the input of the last
   computeNewPhi, [3][nr*npoly]: phil, Pr, Pr2) and g (its output), sets
   *change (may be NULL) to the plain step's change max|g_phil - x_phil| /
   |g_phil(r, 0)| (fj_run_model's stopping test) and overwrites x with the next
   input: with gbar = g - sum_j gamma_j (g_{j+1} - g_j) over the last m + 1
   outputs and xbar the same combination of the inputs, gamma the
   least-squares fit of the residual by the residual differences (the
   residual weighted as the stopping test), x = xbar + beta (gbar - xbar)
   (beta = 1: x = gbar).  The history restarts when the change grew by more
   than a factor 2 (that step then has no history: x + beta (g - x)).  Host
   work and two small copies on the context's stream; synchronous. */
#define FJ_ANDERSON_MAX_DEPTH 8
int fj_anderson_reset(fj_ctx *ctx, int depth, double beta);
int fj_anderson_step(fj_ctx *ctx, int nr, int npoly, double *x, const double *g, double *change);

/* The same mixing without a context, on host tables (a loop that keeps the
   potential on the host, as the reference's does): fj_anderson_create(m,
   beta, &a) holds one iteration's history; fj_anderson_host_step(a, nr,
   npoly, x, g, &change) as fj_anderson_step with host x and g.  No device
   work; FJ_ERR_ARG for bad arguments. */
typedef struct fj_anderson fj_anderson;
int fj_anderson_create(int depth, double beta, fj_anderson **out);
int fj_anderson_destroy(fj_anderson *a);
int fj_anderson_host_step(fj_anderson *a, int nr, int npoly, double *x, const double *g, double *change);

/* n models iterated together (no reference counterpart): one- and
   two-component models (the latter in the summed order, FJ_TWOCOMP_SUMMED:
   both components' grids in the one launch), per iteration one
   fj_moments_batch launch over every model's grid, then each
   model's projection and Poisson solve; with use_graph the iteration is
   captured once as a CUDA graph after running eagerly and replayed.  All
   models share cfgs[0].rule; each runs max(itermax) iterations or until every
   model's tol is met.  res[m] as fj_run_model, except wall_ms, setup_ms,
   kernel_ms (eager iterations only), bound and failures, which are totals of
   the batch. */
int fj_run_model_batch(fj_ctx *ctx, int n, const fj_model_config *cfgs, fj_model_result *res, int use_graph);

/* Surrogate-accelerated self-consistent loop (no reference counterpart).
   Iterations [0, exact_first) and the last exact_last run the mixed-precision
   phase-space kernel and fit the surrogate to that iteration's exact actions
   (samples rows, seeded; epochs_first Adam epochs on the first fit, epochs
   later); the iterations between use the surrogate's actions, except at grid
   points with r < r_exact, which keep the exact kernel, and with an audit:
   every audit_stride-th grid point is also computed exactly and, if the
   largest relative density difference there exceeds audit_tol, the iteration
   is redone exactly (a fallback).  cfg as fj_run_model (mixed rule,
   double-power-law DF, one component). */
typedef struct fj_surrogate_schedule {
    int exact_first, exact_last;
    long long samples;
    int epochs_first, epochs;
    float lr;
    unsigned long long seed;
    double r_exact;
    int audit_stride;
    double audit_tol;
} fj_surrogate_schedule;

typedef struct fj_surrogate_report {
    int surrogate_iterations, fallback_iterations, fits;
    double last_audit_err, max_audit_err, last_fit_loss;
    double surrogate_ms, exact_ms, fit_ms;  /* wall time in each kind of step */
} fj_surrogate_report;

int fj_run_model_surrogate(fj_ctx *ctx, const fj_model_config *cfg, const fj_surrogate_schedule *sch,
                           fj_surrogate *sg, fj_model_result *res, fj_surrogate_report *rep);


#ifdef __cplusplus
}
#endif
#endif
