// fj_device.cuh -- device (and host) math of the fJmodels phase-space path:
// multipole potential and gradient, Brent roots, QUADPACK QAGS, the Staeckel
// fudge and the distribution function.
//
// Written for one thread per (meridional point, velocity node).  Everything
// a thread needs lives in registers; the only indexed per-thread storage is
// the QAGS interval list, which the compiler keeps in local memory and only
// touches when an integral is subdivided.
//
// Arithmetic follows the reference's expression order where that is free,
// so FP64 results agree with the reference to rounding level.  Deliberate
// differences (all rounding-level): Phi and its gradient at one point share
// one interpolation; cos(acos(c)) is replaced by c; pow(x, 2k+1) by repeated
// products; Phi(pi/2) of the v-equation is evaluated once per orbit.
#pragma once

#include <cfloat>
#include <cmath>

#include "fj_kronrod.h"

#if defined(__CUDACC__)
#define FJ_HD __host__ __device__ __forceinline__
#define FJ_HDNI static __host__ __device__ __noinline__
#define FJ_UNROLL _Pragma("unroll")
#else
#define FJ_HD inline
#define FJ_HDNI static inline
#define FJ_UNROLL
#endif

namespace fj {

// literals of include/Utils.h:56-60
constexpr double kPI = 3.141592653589793;
constexpr double kPIH = 1.570796326794897;
constexpr double kTPI = 6.283185307179586;
constexpr double kFPI = 12.56637061435917;
constexpr double kTINY = 1e-12;

constexpr int kMaxPoly = 24;      // largest supported npoly (l_max = 46)
constexpr int kLoopCap = 4096;    // cap on every bracketing loop (unbounded in the reference)
constexpr int kRootMaxIt = 200;   // cap on Brent iterations
constexpr int kQagsCap = 128;     // interval capacity of the per-thread QAGS list

// status bits of one phase-space evaluation
constexpr unsigned kFailBracket = 1u;  // a bracketing loop hit kLoopCap
constexpr unsigned kFailRoot = 2u;     // Brent hit kRootMaxIt
constexpr unsigned kFailQuad = 4u;     // QAGS interval list full (estimate kept)

FJ_HD double dmax(double a, double b) { return a > b ? a : b; }  // MAX of include/Utils.h:47-48

// ----------------------------------------------------------------------------
// multipole potential: tables of include/Grid.h:19-22
// ----------------------------------------------------------------------------
struct PotView {
    int nr, npoly;
    const double *ar, *phil, *Pr, *Pr2;
};

// bracketing search with the semantics of topbottom (include/Utils.h:103-119)
FJ_HD int topbottom(const double *xm, int n, double x, int &bot, int &top)
{
    int t = n - 1, b = 0;
    if ((xm[t] - x) * (x - xm[b]) < 0.) {
        if (fabs(xm[t] - x) < 1e-5 * fabs(x - xm[b])) { top = t; bot = t - 1; return 1; }
        if (fabs(x - xm[b]) < 1e-5 * fabs(x - xm[t])) { top = b + 1; bot = b; return 1; }
        return 0;
    }
    while (t - b > 1) {
        int m = (t + b) / 2;
        if ((xm[t] - x) * (x - xm[m]) >= 0) b = m; else t = m;
    }
    top = t; bot = b;
    return 1;
}

// interpolation weights of intpo2 (include/UtilsLeg.h:96-158) at one radius
struct Interp {
    int bot, top, thr;
    bool ext, quad;
    double f1, f2, f3, x;  // x = ar[nr-1]/r beyond the grid
};

FJ_HD void interp_setup(const PotView &P, double r, Interp &I)
{
    const double *ar = P.ar;
    const int nr = P.nr;
    // every field is set on both branches: the callers' ternaries read both
    I.bot = I.top = I.thr = 0;
    I.f1 = I.f2 = I.f3 = 0.0;
    I.x = 0.0;
    if (r >= ar[nr - 1]) { I.ext = true; I.quad = false; I.x = ar[nr - 1] / r; return; }
    I.ext = false;
    int top = 0, bot = 0;
    topbottom(ar, nr, r, bot, top);
    const double db = r - ar[bot];
    I.f1 = db / (ar[top] - ar[bot]);
    I.bot = bot; I.top = top;
    I.quad = top < 10;
    if (I.quad) {
        const int thr = (I.f1 < 0.5 && bot > 0) ? bot - 1 : top + 1;
        const double dt = r - ar[top];
        I.f2 = dt * db / ((ar[thr] - ar[top]) * (ar[thr] - ar[bot]));
        I.f3 = (ar[thr] - ar[bot]) / (ar[top] - ar[bot]);
        I.thr = thr;
    } else {
        I.thr = top; I.f2 = 0; I.f3 = 0;
    }
}

FJ_HD double interp_in(const Interp &I, const double *T, int npoly, int k)
{
    const double vt = T[I.top * npoly + k], vb = T[I.bot * npoly + k];
    double v = I.f1 * vt + (1 - I.f1) * vb;
    if (I.quad) {
        const double vh = T[I.thr * npoly + k];
        v += I.f2 * (vh - vb - I.f3 * (vt - vb));
    }
    return v;
}

// next even Legendre polynomial P_{2np} from P_{2np-4}, P_{2np-2} (UtilsLeg.h:68-79), np >= 2
FJ_HD double evenleg_next(int np, double c2, double pm2, double pm1)
{
    const int l = 2 * (np - 1), l2 = 2 * l;
    double p = -pm2 * l * (l - 1) / (double)((l2 + 1) * (l2 - 1)) +
               pm1 * (c2 - (l2 * l + l2 - 1) / (double)((l2 - 1) * (l2 + 3)));
    p *= (l2 + 1) * (l2 + 3) / (double)((l + 1) * (l + 2));
    return p;
}

// Phi(R,z): Potential::operator() (pot/Potential.cpp:206-219)
FJ_HDNI double pot_phi(const PotView &P, double R, double z)
{
    const double r = sqrt(R * R + z * z);
    const double c = z / r;
    Interp I;
    interp_setup(P, (r >= P.ar[P.nr - 1]) ? r : dmax(r, P.ar[0]), I);
    const int np_ = P.npoly;
    const double *T = P.phil;
    const double x2 = I.ext ? I.x * I.x : 0.0;
    double xp = I.x;
    double phi = I.ext ? T[(P.nr - 1) * np_] * xp : interp_in(I, T, np_, 0);
    if (np_ < 2) return phi;
    const double c2 = c * c;
    double pm2 = 1.0, pm1 = 1.5 * c2 - .5;
    xp *= x2;
    phi += (I.ext ? T[(P.nr - 1) * np_ + 1] * xp : interp_in(I, T, np_, 1)) * pm1;
    for (int k = 2; k < np_; k++) {
        const double pk = evenleg_next(k, c2, pm2, pm1);
        xp *= x2;
        phi += (I.ext ? T[(P.nr - 1) * np_ + k] * xp : interp_in(I, T, np_, k)) * pk;
        pm2 = pm1; pm1 = pk;
    }
    return phi;
}

// Phi, dPhi/dR, dPhi/dz at one point: operator(), dR, dz of pot/Potential.cpp:206-276
// sharing one bracket search.  dtheta uses the full Legendre recurrence
// (dlegend, UtilsLeg.h:43-57), dr the even one, as the reference does.
FJ_HDNI void pot_grad(const PotView &P, double R, double z, double &phi, double &dR, double &dz)
{
    const double *ar = P.ar;
    const int np_ = P.npoly, nr = P.nr;
    const double r0 = sqrt(R * R + z * z);
    const double cphi = z / r0;
    double r = r0;
    if (r < ar[0]) r = ar[0];
    const double s = R / r;
    double c = z / r;
    if (c == 1) c -= 1e-8;
    Interp I;
    interp_setup(P, r, I);
    const double x2 = I.ext ? I.x * I.x : 0.0;
    double xp = I.x;
    const double cp2 = cphi * cphi, cc2 = c * c;
    // even polys at cphi (potential) and at c (radial derivative)
    double ep2 = 1, ep1 = 0, ec2 = 1, ec1 = 0;
    // full recurrence at c: Pl_m1 = P_{n-1}, Pl = P_n
    double Pl_m1 = 0, Pl = 1;
    int nfull = 0;
    double gphi = 0, gdr = 0, gdth = 0;
    for (int k = 0; k < np_; k++) {
        double ph, dph;
        if (I.ext) {
            const double t = P.phil[(nr - 1) * np_ + k];
            ph = t * xp;
            dph = -(2 * k + 1) * t * xp / r;
            xp *= x2;
        } else {
            ph = interp_in(I, P.phil, np_, k);
            dph = interp_in(I, P.Pr, np_, k);
        }
        double pe_phi, pe_c;
        if (k == 0) { pe_phi = 1; pe_c = 1; }
        else if (k == 1) { pe_phi = 1.5 * cp2 - .5; pe_c = 1.5 * cc2 - .5; ep1 = pe_phi; ec1 = pe_c; }
        else {
            pe_phi = evenleg_next(k, cp2, ep2, ep1); ep2 = ep1; ep1 = pe_phi;
            pe_c = evenleg_next(k, cc2, ec2, ec1); ec2 = ec1; ec1 = pe_c;
        }
        // advance the full recurrence to n = 2k
        double dleg = 0;
        if (k > 0) {
            const int n = 2 * k;
            while (nfull < n) {
                const int i = nfull + 1;
                double Pn;
                if (i == 1) Pn = c;
                else Pn = ((2 * i - 1) * c * Pl - (i - 1) * Pl_m1) / (double)i;
                Pl_m1 = Pl; Pl = Pn; nfull = i;
            }
            dleg = (n * Pl_m1 - n * c * Pl) / (1 - c * c);
        }
        if (k == 0) gphi = ph; else gphi += ph * pe_phi;
        gdr += dph * pe_c;
        gdth += ph * dleg;
    }
    gdth *= -sqrt(1 - c * c);
    phi = gphi;
    dR = gdth * (c / r) + gdr * s;
    dz = gdth * (-s / r) + gdr * c;
}

// Potential::dr with its second derivative (pot/Potential.cpp:224-234); r not clamped
FJ_HD double pot_dr2(const PotView &P, double r, double c, double &d2)
{
    const int np_ = P.npoly, nr = P.nr;
    Interp I;
    interp_setup(P, r, I);
    const double x2 = I.ext ? I.x * I.x : 0.0, cc2 = c * c;
    double xp = I.x, ec2 = 1, ec1 = 0, g1 = 0, g2 = 0;
    for (int k = 0; k < np_; k++) {
        double dph, d2ph;
        if (I.ext) {
            const double t = P.phil[(nr - 1) * np_ + k];
            dph = -(2 * k + 1) * t * xp / r;
            d2ph = (2 * k + 2) * (2 * k + 1) * t * xp / r / r;
            xp *= x2;
        } else {
            dph = interp_in(I, P.Pr, np_, k);
            d2ph = interp_in(I, P.Pr2, np_, k);
        }
        double pe;
        if (k == 0) pe = 1;
        else if (k == 1) { pe = 1.5 * cc2 - .5; ec1 = pe; }
        else { pe = evenleg_next(k, cc2, ec2, ec1); ec2 = ec1; ec1 = pe; }
        g1 += dph * pe;
        g2 += d2ph * pe;
    }
    d2 = g2;
    return g1;
}

// sum_k Phi_k(r) * dP_{2k}/dc and * d2P_{2k}/dc2 (dtheta / d2theta pieces, Potential.cpp:235-255)
FJ_HD void pot_theta_sums(const PotView &P, double r, double c, double &s1, double &s2)
{
    const int np_ = P.npoly, nr = P.nr;
    Interp I;
    interp_setup(P, (r >= P.ar[nr - 1]) ? r : dmax(r, P.ar[0]), I);
    const double x2 = I.ext ? I.x * I.x : 0.0;
    double xp = I.x, Pl_m1 = 0, Pl = 1;
    int nfull = 0;
    s1 = 0; s2 = 0;
    for (int k = 0; k < np_; k++) {
        double ph;
        if (I.ext) { ph = P.phil[(nr - 1) * np_ + k] * xp; xp *= x2; }
        else ph = interp_in(I, P.phil, np_, k);
        double d1 = 0, dd2 = 0;
        const int n = 2 * k;
        if (k > 0) {
            while (nfull < n) {
                const int i = nfull + 1;
                const double Pn = (i == 1) ? c : ((2 * i - 1) * c * Pl - (i - 1) * Pl_m1) / (double)i;
                Pl_m1 = Pl; Pl = Pn; nfull = i;
            }
            d1 = (n * Pl_m1 - n * c * Pl) / (1 - c * c);
        }
        dd2 = (2 * c * d1 - n * (n + 1) * Pl) / (1. - c * c);
        s1 += ph * d1;
        s2 += ph * dd2;
    }
}

// epicycle frequencies getfreqs (pot/Potential.cpp:281-296)
FJ_HDNI void pot_freqs(const PotView &P, double R, double &kappa, double &nu, double &Omega)
{
    const double cth = 6.123233995736766e-17;  // cos(asin(1)) in double
    double d2, phi, dRv, dzv;
    pot_dr2(P, R, cth, d2);
    const double d2R = d2;
    const double g1 = pot_dr2(P, R, cth, d2);
    double s1, s2;
    pot_theta_sums(P, R, 0.0, s1, s2);
    const double dth = s1 * -sqrt(1 - 0.0 * 0.0);
    double d2th = s2 * (1 - 0.0 * 0.0);
    d2th += ((dth * 0.0) / sqrt(1 - 0.0 * 0.0));
    const double d2z = (1. / R) * g1 + (1. / (R * R)) * d2th;
    pot_grad(P, R, 0, phi, dRv, dzv);
    kappa = sqrt(d2R + 3 / R * dRv);
    nu = sqrt(d2z);
    Omega = sqrt(dRv / R);
}

// ----------------------------------------------------------------------------
// Brent root with the stopping rule of wrp_GSLroots (include/Utils.h:134-167)
// ----------------------------------------------------------------------------
FJ_HD bool same_sign(double x, double y) { return (x < 0 && y < 0) || (x > 0 && y > 0); }

template <class F>
FJ_HDNI unsigned brent_root(F &f, double lo, double hi, double &root)
{
    const double flo = f(lo);
    if (fabs(flo) < 5e-4) { root = lo; return 0; }
    const double fhi = f(hi);
    if (fabs(fhi) < 5e-4) { root = hi; return 0; }
    double a = lo, fa = flo, b = hi, fb = fhi, c = hi, fc = fhi, d = hi - lo, e = hi - lo;
    double xr = 0.5 * (lo + hi), xlo = lo, xhi = hi;
    for (int it = 0; it < kRootMaxIt; it++) {
        bool secant = false;
        if (same_sign(fb, fc)) { secant = true; c = a; fc = fa; d = b - a; e = b - a; }
        if (fabs(fc) < fabs(fb)) { secant = true; a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
        const double tol = 0.5 * DBL_EPSILON * fabs(b);
        const double m = 0.5 * (c - b);
        if (fb == 0) { xr = b; xlo = b; xhi = b; }
        else if (fabs(m) <= tol) { xr = b; xlo = b < c ? b : c; xhi = b < c ? c : b; }
        else {
            if (fabs(e) < tol || fabs(fa) <= fabs(fb)) { d = m; e = m; }
            else {
                const double sr = fb / fa;
                double pn, q;
                if (secant) { pn = 2 * m * sr; q = 1 - sr; }
                else {
                    q = fa / fc;
                    const double r = fb / fc;
                    pn = sr * (2 * m * q * (q - r) - (b - a) * (r - 1));
                    q = (q - 1) * (r - 1) * (sr - 1);
                }
                if (pn > 0) q = -q; else pn = -pn;
                const double lim1 = 3 * m * q - fabs(tol * q), lim2 = fabs(e * q);
                if (2 * pn < (lim1 < lim2 ? lim1 : lim2)) { e = d; d = pn / q; }
                else { d = m; e = m; }
            }
            a = b; fa = fb;
            if (fabs(d) > tol) b += d; else b += (m > 0 ? +tol : -tol);
            fb = f(b);
            xr = b;
            const double cc = same_sign(fb, fc) ? a : c;
            xlo = b < cc ? b : cc;
            xhi = b < cc ? cc : b;
        }
        const double alo = fabs(xlo), ahi = fabs(xhi);
        const double mn = ((xlo > 0 && xhi > 0) || (xlo < 0 && xhi < 0)) ? (alo < ahi ? alo : ahi) : 0.0;
        if (fabs(xhi - xlo) < 1e-8 + 1e-6 * mn && !(xhi - xlo > 1e-8)) { root = xr; return 0; }
    }
    root = xr;
    return kFailRoot;
}

// ----------------------------------------------------------------------------
// QUADPACK QAGS (Piessens et al. 1983: DQAGSE, DQK21/DQK15, DQPSRT, DQELG;
// the epsilon table's result count advances only on completed updates, as in
// GSL).  The interval list holds kQagsCap entries; a full list stops the
// refinement, keeps the current estimate and sets kFailQuad.
// ----------------------------------------------------------------------------
FJ_HD double rescale_err(double err, double resabs, double resasc)
{
    err = fabs(err);
    if (resasc != 0 && err != 0) {
        const double scale = pow(200 * err / resasc, 1.5);
        err = scale < 1 ? resasc * scale : resasc;
    }
    if (resabs > DBL_MIN / (50 * DBL_EPSILON)) {
        const double min_err = 50 * DBL_EPSILON * resabs;
        if (min_err > err) err = min_err;
    }
    return err;
}

// Gauss-Kronrod panels (DQK21, DQK15) as abscissas and sums, so that one
// lane or a whole warp can evaluate a panel's function values: the e-th
// abscissa (e < 2 nk - 1) in the evaluation order of the QUADPACK routine --
// the centre, then -/+ the Gauss-point offsets xgk[1], xgk[3], .., then -/+
// xgk[0], xgk[2], .. -- and the sums over the values in that order.
template <int RULE>
struct GKRule {
    static constexpr int nk = RULE == 21 ? 11 : 8;  // Kronrod abscissas in [0, 1]
    static constexpr int npts = 2 * nk - 1;         // function values per panel
    static constexpr int n1 = (nk - 1) / 2;         // Gauss-point pairs
};

FJ_HD double dmul_rn(double x, double y)
{
#ifdef __CUDA_ARCH__
    return __dmul_rn(x, y);
#else
    return x * y;
#endif
}
FJ_HD double dadd_rn(double x, double y)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(x, y);
#else
    return x + y;
#endif
}

template <int RULE>
FJ_HD void gk_tables(const double *&xgk, const double *&wgk, const double *&wg)
{
#ifdef __CUDA_ARCH__
    xgk = RULE == 21 ? fj_xgk21_d : fj_xgk15_d;
    wgk = RULE == 21 ? fj_wgk21_d : fj_wgk15_d;
    wg = RULE == 21 ? fj_wg10_d : fj_wg7_d;
#else
    xgk = RULE == 21 ? fj_xgk21 : fj_xgk15;
    wgk = RULE == 21 ? fj_wgk21 : fj_wgk15;
    wg = RULE == 21 ? fj_wg10 : fj_wg7;
#endif
}

template <int RULE>
FJ_HD double gk_abscissa(double a, double b, int e)
{
    using G = GKRule<RULE>;
    const double *xgk, *wgk, *wg;
    gk_tables<RULE>(xgk, wgk, wg);
    const double center = dmul_rn(0.5, dadd_rn(a, b)), half = dmul_rn(0.5, dadd_rn(b, -a));
    if (e == 0) return center;
    const int jj = e <= 2 * G::n1 ? 2 * ((e - 1) >> 1) + 1 : 2 * ((e - 1 - 2 * G::n1) >> 1);
    const double x = dmul_rn(half, xgk[jj]);
    return ((e - 1) & 1) ? dadd_rn(center, x) : dadd_rn(center, -x);
}

template <int RULE>
FJ_HD void gk_sum(double a, double b, const double *v, double &res, double &abserr, double &resabs, double &resasc)
{
    using G = GKRule<RULE>;
    constexpr int nk = G::nk, n1 = G::n1;
    const double *xgk, *wgk, *wg;
    gk_tables<RULE>(xgk, wgk, wg);
    const double half = dmul_rn(0.5, dadd_rn(b, -a)), ahalf = fabs(half);
    const double fc = v[0];
    double rg = 0, rk = fc * wgk[nk - 1], ra = fabs(rk);
    if (nk % 2 == 0) rg = fc * wg[nk / 2 - 1];
FJ_UNROLL
    for (int j = 0; j < n1; j++) {
        const int jj = 2 * j + 1;
        const double f1 = v[1 + 2 * j], f2 = v[2 + 2 * j];
        rg += wg[j] * (f1 + f2);
        rk += wgk[jj] * (f1 + f2);
        ra += wgk[jj] * (fabs(f1) + fabs(f2));
    }
FJ_UNROLL
    for (int j = 0; j < nk / 2; j++) {
        const int jj = 2 * j;
        const double f1 = v[1 + 2 * n1 + 2 * j], f2 = v[2 + 2 * n1 + 2 * j];
        rk += wgk[jj] * (f1 + f2);
        ra += wgk[jj] * (fabs(f1) + fabs(f2));
    }
    const double mean = 0.5 * rk;
    double rasc = wgk[nk - 1] * fabs(fc - mean);
FJ_UNROLL
    for (int jj = 0; jj < nk - 1; jj++) {
        const int em = (jj & 1) ? jj : 1 + 2 * n1 + jj;
        rasc += wgk[jj] * (fabs(v[em] - mean) + fabs(v[em + 1] - mean));
    }
    const double err = (rk - rg) * half;
    rk *= half; ra *= ahalf; rasc *= ahalf;
    res = rk; resabs = ra; resasc = rasc;
    abserr = rescale_err(err, ra, rasc);
}

template <int RULE, class F>
FJ_HD void gk_panel(F &f, double a, double b, double &res, double &abserr, double &resabs, double &resasc)
{
    double v[GKRule<RULE>::npts];
FJ_UNROLL
    for (int e = 0; e < GKRule<RULE>::npts; e++) v[e] = f(gk_abscissa<RULE>(a, b, e));
    gk_sum<RULE>(a, b, v, res, abserr, resabs, resasc);
}

// Wynn epsilon step (DQELG); tab[0..n-1] with room for n+2
FJ_HD void qelg(double *tab, int &n_io, double *res3, int &nres, double &result, double &abserr)
{
    const int n = n_io - 1;
    const double current = tab[n];
    result = current;
    abserr = DBL_MAX;
    if (n < 2) return;
    tab[n + 2] = tab[n];
    tab[n] = DBL_MAX;
    const int newelm = n / 2;
    int n_final = n;
    for (int i = 0; i < newelm; i++) {
        double res = tab[n - 2 * i + 2];
        const double e0 = tab[n - 2 * i - 2], e1 = tab[n - 2 * i - 1], e2 = res;
        const double e1abs = fabs(e1);
        const double delta2 = e2 - e1, err2 = fabs(delta2);
        const double tol2 = (fabs(e2) > e1abs ? fabs(e2) : e1abs) * DBL_EPSILON;
        const double delta3 = e1 - e0, err3 = fabs(delta3);
        const double tol3 = (e1abs > fabs(e0) ? e1abs : fabs(e0)) * DBL_EPSILON;
        if (err2 <= tol2 && err3 <= tol3) {
            const double rel = 5 * DBL_EPSILON * fabs(res);
            result = res;
            abserr = (err2 + err3) > rel ? (err2 + err3) : rel;
            return;
        }
        const double e3 = tab[n - 2 * i];
        tab[n - 2 * i] = e1;
        const double delta1 = e1 - e3, err1 = fabs(delta1);
        const double tol1 = (e1abs > fabs(e3) ? e1abs : fabs(e3)) * DBL_EPSILON;
        if (err1 <= tol1 || err2 <= tol2 || err3 <= tol3) { n_final = 2 * i; break; }
        const double ss = (1 / delta1 + 1 / delta2) - 1 / delta3;
        if (fabs(ss * e1) <= 0.0001) { n_final = 2 * i; break; }
        res = e1 + 1 / ss;
        tab[n - 2 * i] = res;
        const double error = err2 + fabs(res - e2) + err3;
        if (error <= abserr) { abserr = error; result = res; }
    }
    if (n_final == 49) n_final = 48;
    if (n % 2 == 1) { for (int i = 0; i <= newelm; i++) tab[1 + 2 * i] = tab[2 * i + 3]; }
    else { for (int i = 0; i <= newelm; i++) tab[2 * i] = tab[2 * i + 2]; }
    if (n != n_final) for (int i = 0; i <= n_final; i++) tab[i] = tab[n - n_final + i];
    n_io = n_final + 1;
    if (nres < 3) { res3[nres] = result; abserr = DBL_MAX; }
    else {
        abserr = fabs(result - res3[2]) + fabs(result - res3[1]) + fabs(result - res3[0]);
        res3[0] = res3[1]; res3[1] = res3[2]; res3[2] = result;
    }
    nres += 1;
    const double rel = 5 * DBL_EPSILON * fabs(result);
    if (rel > abserr) abserr = rel;
}

// Interval list of one QAGS call: per-thread local arrays in the phase-space
// kernel, a slice of context scratch in the Poisson kernel.
struct QagsWs {
    double *alist, *blist, *rlist, *elist;
    int *iord;
    int cap;
};

// QAGS on [a,b].  limit is the reference's nominal limit (it only enters the
// ordering rule of DQPSRT); ws.cap is the storage actually available.
// Returns the QUADPACK error class (0 = success); fail gets kFailQuad on overflow.
// The first panel's early exits: returns the QUADPACK error class of a
// finished call (result and abserr set), or -1 when the bisection goes on.
FJ_HD int qags_head(double res0, double err0, double resabs0, double resasc0, double epsabs, double epsrel, int limit,
                    double &result, double &abserr)
{
    const double tol = epsabs > epsrel * fabs(res0) ? epsabs : epsrel * fabs(res0);
    if (err0 <= 100 * DBL_EPSILON * resabs0 && err0 > tol) { result = res0; abserr = err0; return 2; }
    if ((err0 <= tol && err0 != resasc0) || err0 == 0.0) { result = res0; abserr = err0; return 0; }
    if (limit == 1) { result = res0; abserr = err0; return 1; }
    return -1;
}

// The rest of QAGS after a first panel (res0, err0, resabs0) that did not
// finish it: Pn::two evaluates the two half-interval panels of each bisection
// (LanePanels64: one thread; the Poisson kernel's warp form: one warp).
template <int RULE, class Pn>
FJ_HDNI int qags_rest(Pn &pn, double a, double b, double res0, double err0, double resabs0, double epsabs,
                      double epsrel, int limit, double &result, double &abserr, unsigned &fail, const QagsWs &ws)
{
    const int CAP = ws.cap;
    double *alist = ws.alist, *blist = ws.blist, *rlist = ws.rlist, *elist = ws.elist;
    int *iord = ws.iord;
    double rlist2[52], res3la[3];
    int nres = 0, numrl2 = 1;
    alist[0] = a; blist[0] = b; rlist[0] = res0; elist[0] = err0; iord[0] = 0;
    rlist2[0] = res0;
    double area = res0, errsum = err0, errmax = err0;
    int maxerr = 0, nrmax = 0, last = 1, ier = 0;
    double res_ext = res0, err_ext = DBL_MAX, correc = 0, ertest = 0, erlarg = 0, small = 0;
    int ktmin = 0, ierro = 0;
    bool extrap = false, noext = false, done_sum = false;
    int iroff1 = 0, iroff2 = 0, iroff3 = 0;
    const int ksgn = fabs(res0) >= (1 - 50 * DBL_EPSILON) * resabs0 ? 1 : -1;

    for (last = 1; last < limit; last++) {
        if (last >= CAP) { fail |= kFailQuad; last = CAP - 1; done_sum = true; break; }
        const double a1 = alist[maxerr], b1 = 0.5 * (alist[maxerr] + blist[maxerr]);
        const double a2 = b1, b2 = blist[maxerr];
        const double erlast = errmax;
        double area1, error1, ra1, rasc1, area2, error2, ra2, rasc2;
        pn.two(a1, b1, a2, b2, area1, error1, ra1, rasc1, area2, error2, ra2, rasc2);
        const double area12 = area1 + area2, erro12 = error1 + error2;
        errsum = errsum + erro12 - errmax;
        area = area + area12 - rlist[maxerr];
        if (!(rasc1 == error1 || rasc2 == error2)) {
            if (fabs(rlist[maxerr] - area12) <= 1e-5 * fabs(area12) && erro12 >= 0.99 * errmax) {
                if (extrap) iroff2++; else iroff1++;
            }
            if (last > 9 && erro12 > errmax) iroff3++;
        }
        rlist[maxerr] = area1;
        rlist[last] = area2;
        const double errbnd = epsabs > epsrel * fabs(area) ? epsabs : epsrel * fabs(area);
        if (iroff1 + iroff2 >= 10 || iroff3 >= 20) ier = 2;
        if (iroff2 >= 5) ierro = 3;
        if (last == limit - 1) ier = 1;
        const double mx = fabs(a1) > fabs(b2) ? fabs(a1) : fabs(b2);
        if (mx <= (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN)) ier = 4;
        if (!(error2 > error1)) {
            alist[last] = a2; blist[maxerr] = b1; blist[last] = b2;
            elist[maxerr] = error1; elist[last] = error2;
        } else {
            alist[maxerr] = a2; alist[last] = a1; blist[last] = b1;
            rlist[maxerr] = area2; rlist[last] = area1;
            elist[maxerr] = error2; elist[last] = error1;
        }
        {   // DQPSRT with 1-based positions
            const int L = last + 1;
            if (L <= 2) { iord[0] = 0; iord[1] = 1; }
            else {
                const double em = elist[maxerr];
                int nr1 = nrmax + 1;
                if (nr1 != 1) {
                    const int ido = nr1 - 1;
                    for (int i = 1; i <= ido; i++) {
                        const int isucc = iord[nr1 - 2];
                        if (em <= elist[isucc]) break;
                        iord[nr1 - 1] = isucc;
                        nr1--;
                    }
                }
                int jupbn = L;
                if (L > limit / 2 + 2) jupbn = limit + 3 - L;
                const double errmin = elist[L - 1];
                const int jbnd = jupbn - 1, ibeg = nr1 + 1;
                int i = ibeg;
                bool found = false;
                if (ibeg <= jbnd) {
                    for (i = ibeg; i <= jbnd; i++) {
                        const int isucc = iord[i - 1];
                        if (em >= elist[isucc]) { found = true; break; }
                        iord[i - 2] = isucc;
                    }
                }
                if (!found) { iord[jbnd - 1] = maxerr; iord[jupbn - 1] = L - 1; }
                else {
                    iord[i - 2] = maxerr;
                    int k = jbnd;
                    bool ins = false;
                    for (int j = i; j <= jbnd; j++) {
                        const int isucc = iord[k - 1];
                        if (errmin < elist[isucc]) { iord[k] = L - 1; ins = true; break; }
                        iord[k] = isucc;
                        k--;
                    }
                    if (!ins) iord[i - 1] = L - 1;
                }
                nrmax = nr1 - 1;
            }
            maxerr = iord[nrmax];
            errmax = elist[maxerr];
        }
        if (errsum <= errbnd) { done_sum = true; break; }
        if (ier) break;
        if (last == 1) {
            small = fabs(b - a) * 0.375;
            erlarg = errsum;
            ertest = errbnd;
            rlist2[1] = area; numrl2 = 2;
            continue;
        }
        if (noext) continue;
        erlarg -= erlast;
        if (fabs(b1 - a1) > small) erlarg += erro12;
        if (!extrap) {
            if (fabs(blist[maxerr] - alist[maxerr]) > small) continue;
            extrap = true;
            nrmax = 1;
        }
        bool do_ext = true;
        if (!(ierro == 3 || erlarg <= ertest)) {
            int jupbnd = last + 1;
            if (last + 1 > 2 + limit / 2) jupbnd = limit + 3 - (last + 1);
            for (int k = nrmax + 1; k <= jupbnd; k++) {
                maxerr = iord[nrmax];
                errmax = elist[maxerr];
                if (fabs(blist[maxerr] - alist[maxerr]) > small) { do_ext = false; break; }
                nrmax++;
            }
        }
        if (!do_ext) continue;
        rlist2[numrl2] = area; numrl2++;
        double reseps, abseps;
        qelg(rlist2, numrl2, res3la, nres, reseps, abseps);
        ktmin++;
        if (ktmin > 5 && err_ext < 1e-3 * errsum) ier = 5;
        if (abseps < err_ext) {
            ktmin = 0;
            err_ext = abseps;
            res_ext = reseps;
            correc = erlarg;
            ertest = epsabs > epsrel * fabs(reseps) ? epsabs : epsrel * fabs(reseps);
            if (err_ext <= ertest) break;
        }
        if (numrl2 == 1) noext = true;
        if (ier == 5) break;
        maxerr = iord[0];
        errmax = elist[maxerr];
        nrmax = 0;
        extrap = false;
        small *= 0.5;
        erlarg = errsum;
    }
    bool take_sum = done_sum;
    if (!done_sum) {
        result = res_ext;
        abserr = err_ext;
        if (err_ext == DBL_MAX) take_sum = true;
        else {
            bool skip_div = false;
            if (ier + ierro != 0) {
                if (ierro == 3) err_ext += correc;
                if (ier == 0) ier = 3;
                if (res_ext != 0.0 && area != 0.0) {
                    if (err_ext / fabs(res_ext) > errsum / fabs(area)) take_sum = true;
                } else if (err_ext > errsum) take_sum = true;
                else if (area == 0.0) skip_div = true;
                abserr = err_ext;
            }
            if (!take_sum && !skip_div) {
                const double mxa = fabs(res_ext) > fabs(area) ? fabs(res_ext) : fabs(area);
                if (!(ksgn == -1 && mxa <= resabs0 * 0.01)) {
                    const double ratio = res_ext / area;
                    if (ratio < 0.01 || ratio > 100.0 || errsum > fabs(area)) ier = 6;
                }
            }
        }
    }
    if (take_sum) {
        double s = 0;
        for (int k = 0; k <= last; k++) s += rlist[k];
        result = s;
        abserr = errsum;
    }
    if (ier > 2) ier--;
    return ier;
}

template <int RULE, class F>
struct LanePanels64 {
    F &f;
    FJ_HD void two(double a1, double b1, double a2, double b2, double &r1, double &e1, double &ra1, double &rc1,
                   double &r2, double &e2, double &ra2, double &rc2)
    {
        gk_panel<RULE>(f, a1, b1, r1, e1, ra1, rc1);
        gk_panel<RULE>(f, a2, b2, r2, e2, ra2, rc2);
    }
};

template <int RULE, class F>
FJ_HDNI int qags(F &f, double a, double b, double epsabs, double epsrel, int limit, double &result,
               double &abserr, unsigned &fail, const QagsWs &ws)
{
    double res0, err0, resabs0, resasc0;
    gk_panel<RULE>(f, a, b, res0, err0, resabs0, resasc0);
    const int h = qags_head(res0, err0, resabs0, resasc0, epsabs, epsrel, limit, result, abserr);
    if (h >= 0) return h;
    LanePanels64<RULE, F> pn{f};
    return qags_rest<RULE>(pn, a, b, res0, err0, resabs0, epsabs, epsrel, limit, result, abserr, fail, ws);
}

// ----------------------------------------------------------------------------
// Staeckel fudge (uvOrb/uvOrb.cpp, uvOrb/Uvpt.cpp) in FP64
// ----------------------------------------------------------------------------
struct Fudge {
    PotView P;
    double Delta, E, Er, Iv, Lzsq;
    double u, v, shu2, sv, cv, sv2;
    double sinv, cosv;     // sin(v), cos(v) as pt(Delta,u,v) recomputes them
    double sinhu, coshu;   // sinh(u), cosh(u) of the point
    double sh1sq, ch1sq, Phiu1, PhivPIH;
    double uinner, uouter, umid, vturn, ubar, Deltau;
    unsigned fail;

    FJ_HD double Phiu(double shu, double chu) const { return pot_phi(P, Delta * shu * sinv, Delta * chu * cosv); }
    FJ_HD double dU(double u_) const
    {
        const double shu = sinh(u_);
        return (shu * shu + sv2) * Phiu(shu, cosh(u_)) - (sh1sq + sv2) * Phiu1;
    }
    FJ_HD double Phiv(double sn, double cs) const { return pot_phi(P, Delta * sinhu * sn, Delta * coshu * cs); }
    FJ_HD double vturnfn(double v_) const
    {
        double sn, cs;
        sincos(v_, &sn, &cs);
        const double s2 = sn * sn;
        const double dV = (1 + shu2) * PhivPIH - (shu2 + s2) * Phiv(sn, cs);
        return E * s2 + Iv + dV - .5 * Lzsq / (Delta * Delta * s2);
    }
    FJ_HD double uturnfn(double u_) const
    {
        const double shu = sinh(u_), chu = cosh(u_), s2 = shu * shu;
        const double dUv = (s2 + sv2) * Phiu(shu, chu) - (sh1sq + sv2) * Phiu1;
        return E * (s2 - sh1sq) + Er * ch1sq - dUv - .5 * Lzsq / (Delta * Delta) * (1 / s2 - 1 / sh1sq);
    }
    FJ_HD double duturnfn(double u_) const
    {
        const double shu = sinh(u_), chu = cosh(u_), s2 = shu * shu;
        double phi0, f0, f1;
        pot_grad(P, Delta * shu * sinv, Delta * chu * cosv, phi0, f0, f1);
        const double dPhidu = Delta * (f0 * chu * sv + f1 * shu * cv);
        return 2 * (E - phi0) * shu * chu - (s2 + sv2) * dPhidu + Lzsq * chu / (Delta * Delta * s2 * shu);
    }
};

struct UturnF { const Fudge *o; FJ_HD double operator()(double x) const { return o->uturnfn(x); } };
struct DuturnF { const Fudge *o; FJ_HD double operator()(double x) const { return o->duturnfn(x); } };
struct VturnF { const Fudge *o; FJ_HD double operator()(double x) const { return o->vturnfn(x); } };
struct JuIntF {
    const Fudge *o;
    FJ_HD double operator()(double psi) const
    {
        double sn, cs;
        sincos(psi, &sn, &cs);
        return sqrt(dmax(0., o->uturnfn(o->ubar - o->Deltau * cs))) * sn;
    }
};
struct JvIntF {
    const Fudge *o;
    FJ_HD double operator()(double psi) const
    {
        double sn, cs;
        sincos(psi, &sn, &cs);
        return sqrt(dmax(0., o->vturnfn(kPIH - (kPIH - o->vturn) * cs))) * sn;
    }
};

// uvOrb::Getu0 (uvOrb.cpp:109-129)
FJ_HDNI void getu0(Fudge &o, double utry)
{
    DuturnF f{&o};
    double ui = utry, uo = utry, dut = f(utry);
    int it = 0;
    if (dut > 0) {
        while (dut > 0) {
            ui = utry; utry *= 1.2; dut = f(utry);
            if (++it > kLoopCap) { o.fail |= kFailBracket; break; }
        }
        uo = utry;
    } else {
        while (dut < 0) {
            uo = utry; utry *= .8; dut = f(utry);
            if (++it > kLoopCap) { o.fail |= kFailBracket; break; }
        }
        ui = utry;
    }
    o.fail |= brent_root(f, ui, uo, o.umid);
}

// uvOrb::GetTurnu (uvOrb.cpp:131-201)
FJ_HDNI void get_turn_u(Fudge &o, double utry)
{
    UturnF U{&o};
    DuturnF D{&o};
    double u1 = utry, u2 = utry;
    double ut = U(utry), dut = D(utry), eps = .1;
    int it = 0;
    bool capped = false;
#define FJ_CAP()                                                        \
    if (++it > kLoopCap) { capped = true; break; }
    if (ut < 0) {
        if (dut > 0) {
            o.uinner = utry;
            while (!capped) {
                while (ut < 0 && dut > 0) {
                    o.uinner = utry; utry *= (1 + eps);
                    ut = U(utry); dut = D(utry);
                    FJ_CAP();
                }
                if (capped) break;
                if (ut >= 0) { u1 = utry; break; }
                utry /= (1 + eps); eps *= .2;
                if (eps < kTINY) { o.uinner = o.uouter = utry; return; }
                utry *= (1 + eps);
                ut = U(utry); dut = D(utry);
                FJ_CAP();
            }
            while (!capped && ut > 0) { u2 = utry; utry *= 1.1; ut = U(utry); FJ_CAP(); }
            o.uouter = utry;
        } else {
            while (!capped) {
                while (ut < 0 && dut < 0) {
                    o.uouter = utry; utry /= (1 + eps);
                    ut = U(utry); dut = D(utry);
                    FJ_CAP();
                }
                if (capped) break;
                if (ut >= 0) { u2 = utry; break; }
                utry *= (1 + eps); eps *= .2;
                if (eps < kTINY) { o.uinner = o.uouter = utry; return; }
                utry /= (1 + eps);
                ut = U(utry); dut = D(utry);
                FJ_CAP();
            }
            while (!capped && ut > 0) { u1 = utry; utry *= .9; ut = U(utry); FJ_CAP(); }
            o.uinner = utry;
        }
    } else {
        const double fu1 = ut;
        while (ut > 0) { u2 = utry; utry *= 1.1; ut = U(utry); FJ_CAP(); }
        o.uouter = utry;
        ut = fu1;
        while (!capped && ut > 0) { u1 = utry; utry *= .9; ut = U(utry); FJ_CAP(); }
        o.uinner = utry;
    }
#undef FJ_CAP
    if (capped) { o.fail |= kFailBracket; o.uinner = o.uouter = utry; return; }
    o.fail |= brent_root(U, o.uinner, u1, o.uinner);
    o.fail |= brent_root(U, u2, o.uouter, o.uouter);
}

// uvOrb::GetTurnv (uvOrb.cpp:203-224)
FJ_HDNI double get_turn_v(Fudge &o, double vtry)
{
    VturnF V{&o};
    double vtop = vtry, vbot = vtry;
    int it = 0;
    if (V(vtry) < 0) {
        while (V(vbot) < 0) {
            vbot = .5 * (kPIH + vbot);
            if (kPIH - vbot < kTINY) return kPIH;
            if (++it > kLoopCap) { o.fail |= kFailBracket; return kPIH; }
        }
    } else {
        while (V(vtop) > 0) {
            vtop *= .5;
            if (vtop < kTINY) return 0;
            if (++it > kLoopCap) { o.fail |= kFailBracket; return 0; }
        }
    }
    double r;
    if (!(vbot < vtop)) o.fail |= brent_root(V, vtop, vbot, r);
    else o.fail |= brent_root(V, vbot, vtop, r);
    return r;
}

// Momentum-integral rule: QAGS as wrp_GSLinteg (include/Utils.h:173-185) or fixed GL.
struct GLRule {
    int n;              // 0 = QAGS
    const double *x01;  // nodes on (0,1)
    const double *w01;  // weights on (0,1)
};

template <class F>
FJ_HDNI double mom_integral(F &f, double b, const GLRule &gl, unsigned &fail)
{
    if (gl.n <= 0) {
        double al[kQagsCap], bl[kQagsCap], rl[kQagsCap], el[kQagsCap];
        int io[kQagsCap];
        const QagsWs ws{al, bl, rl, el, io, kQagsCap};
        double r, e;
        qags<21>(f, 0.0, b, 1e-5, 1e-3, 1000, r, e, fail, ws);
        return r;
    }
    double s = 0;
    for (int i = 0; i < gl.n; i++) s += (b * gl.w01[i]) * f(b * gl.x01[i]);
    return s;
}

// The momentum integrals of one thread: QAGS or fixed Gauss-Legendre (mom_integral)
struct SerialMomInt {
    const GLRule *gl;
    template <class F>
    FJ_HD double operator()(F &f, double b, unsigned &fail) const { return mom_integral(f, b, *gl, fail); }
};

// Actions of one phase-space point: uvOrb ctor (uvOrb.cpp:15-36), Ju, Jv, the
// momentum integrals by mi(integrand, upper limit, fail).
// Returns false for an unbound orbit (Jr = Jz = 1e31).
template <class MI>
FJ_HDNI bool fudge_actions_with(const PotView &P, double Delta, double R, double z, double Phi, double pR,
                                double vphi, double pz, const MI &mi, double &Jr, double &Jz, unsigned &fail)
{
    Fudge o;
    o.P = P;
    o.fail = 0;
    o.Delta = Delta;
    const double Lz = R * vphi;
    o.Lzsq = Lz * Lz;
    // pt(Delta, x, p): Uvpt.cpp:11-24
    const double Delta2 = Delta * Delta, R2 = R * R, z2 = z * z, r2 = R2 + z2;
    const double dmr = Delta2 - r2, dpr = Delta2 + r2;
    const double shu2 = .5 * (r2 - Delta2 + sqrt(dmr * dmr + 4 * Delta2 * R2)) / Delta2;
    const double shu = sqrt(shu2);
    o.u = asinh(shu);
    const double chu = sqrt(1 + shu2);
    const double cv2 = .5 * (r2 + Delta2 - sqrt(dpr * dpr - 4 * Delta2 * z2)) / Delta2;
    const double cv = z < 0 ? -sqrt(cv2) : sqrt(cv2);
    o.v = acos(cv);
    o.sv = sin(o.v);
    o.sv2 = 1 - cv2;
    o.shu2 = shu2;
    o.cv = cv;
    const double p2 = pR * pR + pz * pz;
    const double pu = Delta * (pR * chu * o.sv + pz * shu * cv);
    const double pv = Delta * (pR * shu * cv - pz * chu * o.sv);
    o.E = .5 * p2 + .5 * o.Lzsq / (R * R) + Phi;
    if (o.E >= 0 || isnan(o.E)) { Jr = Jz = 1e31; return false; }
    sincos(o.v, &o.sinv, &o.cosv);
    o.sinhu = sinh(o.u);
    o.coshu = cosh(o.u);
    const double us = 58;
    {
        const double s = sinh(us), c = cosh(us);
        o.sh1sq = s * s; o.ch1sq = c * c;
    }
    getu0(o, us);
    {
        const double s = sinh(o.umid), c = cosh(o.umid);
        o.sh1sq = s * s; o.ch1sq = c * c;
        o.Phiu1 = o.Phiu(s, c);
    }
    o.PhivPIH = o.Phiv(sin(kPIH), cos(kPIH));
    o.Er = -o.E * (shu2 - o.sh1sq) / o.ch1sq + .5 * (pu * pu) / (Delta2 * o.ch1sq) +
           .5 * o.Lzsq / (Delta2 * o.ch1sq) * (1 / shu2 - 1 / o.sh1sq) + o.dU(o.u) / o.ch1sq;
    {
        double sn, cs;
        sincos(o.v, &sn, &cs);
        const double dVv = (1 + o.shu2) * o.PhivPIH - (o.shu2 + sn * sn) * o.Phiv(sn, cs);
        o.Iv = .5 * (pv * pv) / Delta2 - o.E * o.sv2 + .5 * o.Lzsq / (Delta2 * o.sv2) - dVv;
    }
    const double rtwo = sqrt(2.0);
    // Ju (uvOrb.cpp:226-239)
    get_turn_u(o, 1);
    if (fabs(o.uouter - o.uinner) < kTINY) Jr = 0;
    else {
        o.ubar = .5 * (o.uinner + o.uouter);
        o.Deltau = .5 * (o.uouter - o.uinner);
        JuIntF fju{&o};
        Jr = rtwo * Delta * o.Deltau * mi(fju, kPI, o.fail) / kPI;
    }
    // Jv (uvOrb.cpp:247-257)
    o.vturn = get_turn_v(o, .5 * kPIH);
    if (fabs(o.vturn - kPIH) < kTINY) Jz = 0;
    else {
        JvIntF fjv{&o};
        Jz = 2 * rtwo * Delta * (kPIH - o.vturn) * mi(fjv, kPIH, o.fail) / kPI;
    }
    fail |= o.fail;
    return true;
}

FJ_HDNI bool fudge_actions(const PotView &P, double Delta, double R, double z, double Phi, double pR,
                         double vphi, double pz, const GLRule &gl, double &Jr, double &Jz, unsigned &fail)
{
    return fudge_actions_with(P, Delta, R, z, Phi, pR, vphi, pz, SerialMomInt{&gl}, Jr, Jz, fail);
}

// ----------------------------------------------------------------------------
// focal distance and DF
// ----------------------------------------------------------------------------
// Deltafn (delta/tabulate.cpp:40-44) with linterp (Utils.h:122-128)
FJ_HD double deltafn(const double *Eg, const double *Dg, int n, double E)
{
    if (E < Eg[0]) return sqrt(dmax(.000001, Dg[0]));
    if (E < Eg[n - 1]) {
        double y;
        if (E <= Eg[0]) y = Dg[0];
        else {
            int top = 0, bot = 0;
            topbottom(Eg, n, E, bot, top);
            y = Dg[bot] + (E - Eg[bot]) / (Eg[top] - Eg[bot]) * (Dg[top] - Dg[bot]);
        }
        return sqrt(dmax(.000001, y));
    }
    return sqrt(dmax(.000001, Dg[n - 1]));
}

struct DFDev {
    int kind;
    double alpha, beta, J0, norm, tpi3, dphi_h, dz_h, dphi_g, dz_g, chi, k;
};

// GetRc (include/Utils.h:195-214): circular radius for Lz^2
FJ_HDNI double get_rc(const PotView &P, double Lzsq, double R, unsigned &fail)
{
    struct RcF {
        const PotView *P; double Lzsq;
        FJ_HD double operator()(double x) const
        {
            double phi, dR, dz;
            pot_grad(*P, x, 0, phi, dR, dz);
            return Lzsq / (x * x * x) - dR;
        }
    } f{&P, Lzsq};
    double Ri = R, Ro = R, dfRt = f(R);
    int it = 0;
    if (dfRt > 0) {
        while (dfRt > 0) { Ri = R; R *= 1.2; dfRt = f(R); if (++it > kLoopCap) { fail |= kFailBracket; break; } }
        Ro = R;
    } else {
        while (dfRt < 0) { Ro = R; R *= .8; dfRt = f(R); if (++it > kLoopCap) { fail |= kFailBracket; break; } }
        Ri = R;
    }
    double r;
    fail |= brent_root(f, Ri, Ro, r);
    return r;
}

// df() (df/DF.cpp:78-124) from the actions; NaN -> 0 as DF.cpp:105
FJ_HD double df_value(const DFDev &d, const PotView &P, double R, double Jr, double Jz, double Jphi,
                      unsigned &fail)
{
    double DF;
    if (d.kind == 1) {
        const double rc = get_rc(P, Jphi * Jphi, R, fail);
        double kappa, nu, Omega;
        pot_freqs(P, rc, kappa, nu, Omega);
        const double sigmar = exp(-rc / 2.) * 5.;
        const double sigmaz = exp(-rc / 4.) * .316;
        const double fr = Omega * 1e-1 * exp(-rc / 1.) / (kPI * sigmar * sigmar * kappa) * (1. + tanh(Jphi / .1)) *
                          exp(-kappa * Jr / (sigmar * sigmar));
        const double fz = nu / (2 * kPI * sigmaz * sigmaz) * exp(-2 * Jz / (sigmaz * sigmaz));
        DF = dmax(0., fr * fz);
    } else {
        const double h = Jr + d.dphi_h * fabs(Jphi) + d.dz_h * Jz;
        const double g = Jr + d.dphi_g * fabs(Jphi) + d.dz_g * Jz;
        const double DFeven = d.norm * dmax(0., pow(1. + d.J0 / h, d.alpha) / (pow(1. + g / d.J0, d.beta))) / d.tpi3;
        DF = d.chi == 0. ? DFeven : DFeven + d.k * tanh(d.chi * Jphi / d.J0) * DFeven;
    }
    if (isnan(DF)) return 0.;
    return DF;
}

}  // namespace fj
