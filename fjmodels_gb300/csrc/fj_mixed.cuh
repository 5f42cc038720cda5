// fj_mixed.cuh -- mixed-precision phase-space evaluation.
//
// The same algorithm as the plain form (fj_device.cuh: the reference's
// bracketing, Brent roots, QAGS momentum integrals with its tolerances, the
// double-power-law DF) with the bulk arithmetic in FP32:
//   FP64  per-point setup (Phi, escape speed), the node's velocity, energy
//         and focal distance, the prolate-spheroidal transform, the moment
//         accumulation, and the turning-point search whenever it reaches the
//         u/v limits (the bracket refinement below FP32 resolution, v within
//         1e-6 of the equatorial or polar limit), which reruns in FP64;
//   FP32  potential and gradient evaluations from FP32 copies of the tables,
//         the u/v turning-point functions, the bracket search and Brent
//         iterations away from the limits, QAGS (GK21) and the DF.
// The reference point u0 of the u-equation is the orbit's own u instead of
// the root of d/du (uvOrb.cpp:109-129): the u-equation does not depend on u0
// (it cancels exactly), and u0 = 58 overflows FP32 (sinh(58)^2 > FLT_MAX).
// With u0 = u, Er*cosh^2(u0) reduces to pu^2/(2 Delta^2) exactly.
#pragma once

#include "fj_device.cuh"

namespace fj {

constexpr float kPIHf = 1.570796326794897f;
constexpr float kPIf = 3.141592653589793f;

// FP32 view of the multipole potential.  The monopole column of phil holds
// Phi_0(r) - shift (shift = the potential at the phase point of the block):
// the u and v equations only involve E - Phi, and near the point the
// shifted values are small, so their FP32 rounding is relative to the local
// potential differences rather than to |Phi|.  out0 = the unshifted outer
// monopole phil[nr-1][0] for the r >= ar[nr-1] extrapolation.
// The interpolation of pot/Potential.cpp:206-276 (linear, plus the quadratic
// correction in the ten innermost intervals) uses per-interval constants:
// ih[n] = 1/(ar[n+1]-ar[n]) and, for n < kQuadIntervals, qc[4n..4n+3] =
// {q, f3} with the third point below (n-1) and above (n+2), where
// q = 1/((ar[thr]-ar[n+1])(ar[thr]-ar[n])), f3 = (ar[thr]-ar[n])/(ar[n+1]-ar[n]).
// The interval of r is found from the logarithmic spacing of the grid
// (lr0 = log ar[0], idl = (nr-1)/log(ar[nr-1]/ar[0])) and corrected by
// neighbour tests, so any increasing grid gives the bracketing interval.
constexpr int kQuadIntervals = 9;  // intervals whose top node is below 10
struct PotViewF {
    int nr, npoly;
    const float *ar, *phil, *Pr, *ih, *qc;
    float out0, shift, lr0, idl;
    float c2pt;         // cos^2 of the polar angle of the grid point
    const float *pyl;   // P_2k(c2pt), k < npoly
};

// even-Legendre recurrence P_2k from P_2k-2, P_2k-4 (include/UtilsLeg.h:43-50)
// as P_2k = (P_2k-2 (c^2 - B_k) - A_k P_2k-4) C_k, constants per k
struct LegCoefF { float A[kMaxPoly], B[kMaxPoly], C[kMaxPoly], inv[2 * kMaxPoly + 1]; };
constexpr LegCoefF make_leg_f()
{
    LegCoefF o{};
    for (int k = 0; k < kMaxPoly; k++) {
        const double l = 2.0 * (k - 1), l2 = 2 * l;
        o.A[k] = k >= 2 ? (float)(l * (l - 1) / ((l2 + 1) * (l2 - 1))) : 0.f;
        o.B[k] = k >= 2 ? (float)((l2 * l + l2 - 1) / ((l2 - 1) * (l2 + 3))) : 0.f;
        o.C[k] = k >= 2 ? (float)((l2 + 1) * (l2 + 3) / ((l + 1) * (l + 2))) : 0.f;
    }
    for (int i = 0; i <= 2 * kMaxPoly; i++) o.inv[i] = i ? (float)(1.0 / i) : 0.f;
    return o;
}
static __constant__ LegCoefF kLegF_d = make_leg_f();
static constexpr LegCoefF kLegF_h = make_leg_f();
FJ_HD const LegCoefF &leg_f()
{
#ifdef __CUDA_ARCH__
    return kLegF_d;
#else
    return kLegF_h;
#endif
}

// log for the interval guess only (corrected by neighbour tests)
FJ_HD float fast_logf(float x)
{
#ifdef __CUDA_ARCH__
    return __logf(x);
#else
    return logf(x);
#endif
}

// sin and cos of a quadrature angle psi in [0, pi]: absolute error 4e-7 of the
// hardware approximation is below the QAGS tolerances
FJ_HD void sincos_psi(float x, float *s, float *c)
{
#ifdef __CUDA_ARCH__
    __sincosf(x, s, c);
#else
    sincosf(x, s, c);
#endif
}

// sinh x and cosh x - 1 from one expm1 (relative precision for small |x|)
FJ_HD void sinh_coshm1(float x, float &sh, float &chm1)
{
    const float em = expm1f(x), h = em / (2.f * (em + 1.f));  // (e^x - 1) / (2 e^x)
    sh = h * (em + 2.f);
    chm1 = h * em;
}

struct InterpF {
    int bot, thr;
    bool ext, quad;
    float f1, f2, f3, q, x;
};

FJ_HD void interp_setup_f(const PotViewF &P, float r, InterpF &I)
{
    const float *ar = P.ar;
    const int nr = P.nr;
    I.bot = I.thr = 0;
    I.f1 = I.f2 = I.f3 = I.q = 0.f;
    I.quad = false;
    I.x = 0.f;
    if (r >= ar[nr - 1]) { I.ext = true; I.x = ar[nr - 1] / r; return; }
    I.ext = false;
    int b = (int)((fast_logf(r) - P.lr0) * P.idl);
    b = b < 0 ? 0 : (b > nr - 2 ? nr - 2 : b);
    while (b > 0 && r < ar[b]) --b;
    while (b < nr - 2 && r > ar[b + 1]) ++b;
    I.bot = b;
    I.f1 = (r - ar[b]) * P.ih[b];
    I.quad = b < kQuadIntervals;
    if (I.quad) {
        const bool lo = I.f1 < 0.5f && b > 0;
        I.thr = lo ? b - 1 : b + 2;
        const float *q = P.qc + 4 * b + (lo ? 0 : 2);
        I.q = q[0];
        I.f2 = (r - ar[b + 1]) * (r - ar[b]) * q[0];
        I.f3 = q[1];
    }
}

FJ_HD float interp_in_f(const InterpF &I, const float *T, int npoly, int k)
{
    const float vb = T[I.bot * npoly + k], d = T[(I.bot + 1) * npoly + k] - vb;
    float v = vb + I.f1 * d;
    if (I.quad) v += I.f2 * (T[I.thr * npoly + k] - vb - I.f3 * d);
    return v;
}

FJ_HDNI float pot_phi_f(const PotViewF &P, float R, float z)
{
    const float r = sqrtf(R * R + z * z);
    const float c = z / r;
    InterpF I;
    interp_setup_f(P, (r >= P.ar[P.nr - 1]) ? r : fmaxf(r, P.ar[0]), I);
    const int np_ = P.npoly;
    const float *T = P.phil;
    const LegCoefF &L = leg_f();
    const float x2 = I.x * I.x;
    float xp = I.x;
    float phi = I.ext ? P.out0 * xp - P.shift : interp_in_f(I, T, np_, 0);
    if (np_ < 2) return phi;
    const float c2 = c * c;
    float pm2 = 1.f, pm1 = 1.5f * c2 - .5f;
    xp *= x2;
    phi += (I.ext ? T[(P.nr - 1) * np_ + 1] * xp : interp_in_f(I, T, np_, 1)) * pm1;
    for (int k = 2; k < np_; k++) {
        const float pk = (pm1 * (c2 - L.B[k]) - L.A[k] * pm2) * L.C[k];
        xp *= x2;
        phi += (I.ext ? T[(P.nr - 1) * np_ + k] * xp : interp_in_f(I, T, np_, k)) * pk;
        pm2 = pm1; pm1 = pk;
    }
    return phi;
}

// Phi, dPhi/dR, dPhi/dz (pot/Potential.cpp:206-276) in FP32
FJ_HDNI void pot_grad_f(const PotViewF &P, float R, float z, float &phi, float &dR, float &dz)
{
    const float *ar = P.ar;
    const int np_ = P.npoly, nr = P.nr;
    const LegCoefF &L = leg_f();
    const float r0 = sqrtf(R * R + z * z);
    const float cphi = z / r0;
    float r = r0 < ar[0] ? ar[0] : r0;
    const float s = R / r;
    float c = z / r;
    if (c >= 1.f) c = 1.f - 1e-7f;
    InterpF I;
    interp_setup_f(P, r, I);
    const float x2 = I.x * I.x;
    float xp = I.x;
    const float cp2 = cphi * cphi, cc2 = c * c, i1mc2 = 1.f / (1.f - cc2);
    float ep2 = 1, ep1 = 0, ec2 = 1, ec1 = 0, Pl_m1 = 0, Pl = 1;
    int nfull = 0;
    float gphi = 0, gdr = 0, gdth = 0;
    for (int k = 0; k < np_; k++) {
        float ph, dph;
        if (I.ext) {
            const float t = k == 0 ? P.out0 : P.phil[(nr - 1) * np_ + k];
            ph = k == 0 ? t * xp - P.shift : t * xp;
            dph = -(float)(2 * k + 1) * t * xp / r;
            xp *= x2;
        } else {
            ph = interp_in_f(I, P.phil, np_, k);
            dph = interp_in_f(I, P.Pr, np_, k);
        }
        float pe_phi, pe_c;
        if (k == 0) { pe_phi = 1; pe_c = 1; }
        else if (k == 1) { pe_phi = 1.5f * cp2 - .5f; pe_c = 1.5f * cc2 - .5f; ep1 = pe_phi; ec1 = pe_c; }
        else {
            pe_phi = (ep1 * (cp2 - L.B[k]) - L.A[k] * ep2) * L.C[k]; ep2 = ep1; ep1 = pe_phi;
            pe_c = (ec1 * (cc2 - L.B[k]) - L.A[k] * ec2) * L.C[k]; ec2 = ec1; ec1 = pe_c;
        }
        float dleg = 0;
        if (k > 0) {
            const int n = 2 * k;
            while (nfull < n) {
                const int i = nfull + 1;
                const float Pn = (i == 1) ? c : ((float)(2 * i - 1) * c * Pl - (float)(i - 1) * Pl_m1) * L.inv[i];
                Pl_m1 = Pl; Pl = Pn; nfull = i;
            }
            dleg = (float)n * (Pl_m1 - c * Pl) * i1mc2;
        }
        if (k == 0) gphi = ph; else gphi += ph * pe_phi;
        gdr += dph * pe_c;
        gdth += ph * dleg;
    }
    gdth *= -sqrtf(1.f - c * c);
    phi = gphi;
    dR = gdth * (c / r) + gdr * s;
    dz = gdth * (-s / r) + gdr * c;
}

// Phi(R, z) - Phi(point) for a position on a coordinate line through the
// phase point, with the differences of the geometry given exactly:
// dr2 = r^2 - rpt^2 and dc2 = c^2 - c2pt (c = z/r).  When r and the point share
// an interpolation interval (the point may sit on its end node) the
// difference is formed inside the interpolation formula and by the difference
// recurrence of the even Legendre polynomials,
//   d_k = C_k ((x - B_k) d_k-1 + (x - y) P_k-1(y) - A_k d_k-2),  x = c^2, y = c2pt,
// so it keeps its relative precision however close the position is to the
// point; otherwise it is the direct interpolation (or the r >= ar[nr-1]
// extrapolation) minus Phipt, the FP32 potential at the point.  All three
// run in the same loop over the multipoles, each l's term being
//   vb a_l + (vt - vb) b_l + (v_thr - vb - f3 (vt - vb)) g_l
// with per-position coefficients selected without branches, so the lanes of
// a warp do not split between them.  P_k(y) is the point's table P.pyl.
struct DState {
    int mode;  // 0: difference, 1: direct, 2: extrapolated
    int b, thr;
    bool quad;
    float f1, f2, f3, f1p, f2p, df1, df2, x, dc2, xe2, xp1, sum0, phipt;
};

FJ_HD void dphi_setup(const PotViewF &P, float R, float z, float rpt, float dr2, float dc2, float Phipt, DState &s)
{
    const float r = sqrtf(R * R + z * z);
    const float *ar = P.ar;
    const int nr = P.nr;
    const float a0 = ar[0], rmax = ar[nr - 1];
    s.b = nr - 2; s.thr = 0; s.quad = false;
    s.f1 = s.f2 = s.f3 = s.f1p = s.f2p = s.df1 = s.df2 = 0.f;
    s.xe2 = 1.f; s.xp1 = 1.f; s.sum0 = 0.f;
    s.phipt = Phipt; s.dc2 = dc2;
    if (r >= rmax) {  // phi_l = phil[nr-1][l] (rmax/r)^(2l+1); the monopole from the unshifted table value
        s.mode = 2;
        const float xe = rmax / r;
        s.xe2 = xe * xe;
        s.xp1 = xe * s.xe2;
        s.sum0 = P.out0 * xe - P.shift;
    } else {
        const float re = fmaxf(r, a0), rpe = fmaxf(rpt, a0);
        InterpF I;
        interp_setup_f(P, re, I);
        s.b = I.bot; s.thr = I.thr; s.quad = I.quad; s.f1 = I.f1; s.f2 = I.f2; s.f3 = I.f3;
        const float ab = ar[s.b], at = ar[s.b + 1];
        s.mode = 1;
        if (rpt < rmax && rpe >= ab && rpe <= at) {
            const float fp = (rpe - ab) * P.ih[s.b];
            const int thr_p = (fp < 0.5f && s.b > 0) ? s.b - 1 : s.b + 2;
            if (!s.quad || thr_p == s.thr || rpe == ab || rpe == at) {
                s.mode = 0;
                s.f1p = fp;
                s.f2p = s.quad ? (rpe - at) * (rpe - ab) * I.q : 0.f;
                const float dr = (r >= a0 && rpt >= a0) ? dr2 / (r + rpt) : re - rpe;
                s.df1 = dr * P.ih[s.b];
                s.df2 = s.quad ? I.q * dr * (re + rpe - ab - at) : 0.f;
            }
        }
    }
    s.x = s.mode == 0 ? P.c2pt + dc2 : (z * z) / (r * r);
}

// the term of multipole k: px = P_k(x), dk = P_k(x) - P_k(y), xp the
// extrapolation factor (1 in the other modes)
FJ_HD void dphi_acc(const PotViewF &P, const DState &s, float &sum, int k, float px, float dk, float xp)
{
    const int np_ = P.npoly;
    const float *T = P.phil;
    const float vb = T[s.b * np_ + k], d = T[(s.b + 1) * np_ + k] - vb;
    const float e = s.quad ? T[s.thr * np_ + k] - vb - s.f3 * d : 0.f;
    const float t = xp * px;
    const bool m0 = s.mode == 0, m1 = s.mode == 1;
    const float ca = m0 ? dk : t;
    const float cb = m0 ? s.df1 * px + s.f1p * dk : (m1 ? s.f1 * px : t);
    const float cg = m0 ? s.df2 * px + s.f2p * dk : s.f2 * px;
    sum += vb * ca + d * cb + e * cg;
}

FJ_HD float dphi_end(const DState &s, float sum) { return s.mode == 0 ? sum : sum - s.phipt; }

// one multipole chain: Legendre recurrences of x and of the difference
struct DChain {
    float px1, px2, d1, d2, xp, sum;
    FJ_HD void begin(const PotViewF &P, const DState &s)
    {
        sum = s.sum0;
        dphi_acc(P, s, sum, 0, 1.f, 0.f, s.mode == 2 ? 0.f : 1.f);  // the extrapolated monopole is in sum0
        px2 = 1.f; d2 = 0.f;
        if (P.npoly > 1) {
            px1 = 1.5f * s.x - .5f;
            d1 = 1.5f * s.dc2;
            dphi_acc(P, s, sum, 1, px1, d1, s.xp1);
        }
        xp = s.xp1 * s.xe2;
    }
    FJ_HD void step(const PotViewF &P, const LegCoefF &L, const DState &s, int k)
    {
        const float px = ((s.x - L.B[k]) * px1 - L.A[k] * px2) * L.C[k];
        const float dk = ((s.x - L.B[k]) * d1 + s.dc2 * P.pyl[k - 1] - L.A[k] * d2) * L.C[k];
        dphi_acc(P, s, sum, k, px, dk, xp);
        xp *= s.xe2;
        px2 = px1; px1 = px; d2 = d1; d1 = dk;
    }
};

FJ_HD float pot_dphi_f(const PotViewF &P, float R, float z, float rpt, float dr2, float dc2, float Phipt)
{
    DState s;
    dphi_setup(P, R, z, rpt, dr2, dc2, Phipt, s);
    DChain c;
    c.begin(P, s);
    const LegCoefF &L = leg_f();
    for (int k = 2; k < P.npoly; k++) c.step(P, L, s, k);
    return dphi_end(s, c.sum);
}

// Brent root (wrp_GSLroots rule, include/Utils.h:134-167) in FP32; the
// absolute bracket tolerance is raised to the FP32 resolution of the root.
template <class F>
FJ_HDNI unsigned brent_root_f(F &f, float lo, float hi, float &root)
{
    const float flo = f(lo);
    if (fabsf(flo) < 5e-4f) { root = lo; return 0; }
    const float fhi = f(hi);
    if (fabsf(fhi) < 5e-4f) { root = hi; return 0; }
    float a = lo, fa = flo, b = hi, fb = fhi, c = hi, fc = fhi, d = hi - lo, e = hi - lo;
    float xr = 0.5f * (lo + hi), xlo = lo, xhi = hi;
    for (int it = 0; it < kRootMaxIt; it++) {
        bool secant = false;
        if ((fb < 0 && fc < 0) || (fb > 0 && fc > 0)) { secant = true; c = a; fc = fa; d = b - a; e = b - a; }
        if (fabsf(fc) < fabsf(fb)) { secant = true; a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
        const float tol = 0.5f * FLT_EPSILON * fabsf(b);
        const float m = 0.5f * (c - b);
        if (fb == 0) { xr = b; xlo = b; xhi = b; }
        else if (fabsf(m) <= tol) { xr = b; xlo = fminf(b, c); xhi = fmaxf(b, c); }
        else {
            if (fabsf(e) < tol || fabsf(fa) <= fabsf(fb)) { d = m; e = m; }
            else {
                const float sr = fb / fa;
                float pn, q;
                if (secant) { pn = 2 * m * sr; q = 1 - sr; }
                else {
                    q = fa / fc;
                    const float r = fb / fc;
                    pn = sr * (2 * m * q * (q - r) - (b - a) * (r - 1));
                    q = (q - 1) * (r - 1) * (sr - 1);
                }
                if (pn > 0) q = -q; else pn = -pn;
                if (2 * pn < fminf(3 * m * q - fabsf(tol * q), fabsf(e * q))) { e = d; d = pn / q; }
                else { d = m; e = m; }
            }
            a = b; fa = fb;
            if (fabsf(d) > tol) b += d; else b += (m > 0 ? +tol : -tol);
            fb = f(b);
            xr = b;
            const float cc = ((fb < 0 && fc < 0) || (fb > 0 && fc > 0)) ? a : c;
            xlo = fminf(b, cc);
            xhi = fmaxf(b, cc);
        }
        const float alo = fabsf(xlo), ahi = fabsf(xhi);
        const float mn = ((xlo > 0 && xhi > 0) || (xlo < 0 && xhi < 0)) ? fminf(alo, ahi) : 0.f;
        const float abstol = fmaxf(1e-8f, 4.f * FLT_EPSILON * fmaxf(alo, ahi));
        if (fabsf(xhi - xlo) < abstol + 1e-6f * mn && !(xhi - xlo > abstol)) { root = xr; return 0; }
    }
    root = xr;
    return kFailRoot;
}

// ---------------------------------------------------------------- QAGS, FP32
FJ_HD float rescale_err_f(float err, float resabs, float resasc)
{
    err = fabsf(err);
    if (resasc != 0 && err != 0) {
        const float scale = powf(200 * err / resasc, 1.5f);
        err = scale < 1 ? resasc * scale : resasc;
    }
    if (resabs > FLT_MIN / (50 * FLT_EPSILON)) {
        const float min_err = 50 * FLT_EPSILON * resabs;
        if (min_err > err) err = min_err;
    }
    return err;
}

struct GK21f { float xgk[11], wgk[11], wg[5]; };

// FP32 products and sums that are never contracted into an FMA: the panel
// abscissas have the same bits wherever the code is compiled (device, host)
FJ_HD float mul_rn(float x, float y)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(x, y);
#else
    return x * y;
#endif
}
FJ_HD float add_rn(float x, float y)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(x, y);
#else
    return x + y;
#endif
}

// The e-th (0..20) abscissa of the 21-point Gauss-Kronrod panel on [a, b], in
// the evaluation order of gk21_f: the centre, then -/+ the Gauss-point
// offsets xgk[1], xgk[3], .., xgk[9], then -/+ xgk[0], xgk[2], .., xgk[8]
FJ_HD float gk21_abscissa(const GK21f &K, float a, float b, int e)
{
    const float center = mul_rn(0.5f, add_rn(a, b)), half = mul_rn(0.5f, add_rn(b, -a));
    if (e == 0) return center;
    const int jj = e <= 10 ? 2 * ((e - 1) >> 1) + 1 : 2 * ((e - 11) >> 1);
    const float x = mul_rn(half, K.xgk[jj]);
    return ((e - 1) & 1) ? add_rn(center, x) : add_rn(center, -x);
}

// The panel's sums (QUADPACK DQK21) over the 21 values v[e] in that order
FJ_HD void gk21_sum(const GK21f &K, float a, float b, const float *v, float &res, float &abserr, float &resabs,
                    float &resasc)
{
    const float half = mul_rn(0.5f, add_rn(b, -a)), ahalf = fabsf(half);
    const float fc = v[0];
    float rg = 0, rk = fc * K.wgk[10], ra = fabsf(rk);
    FJ_UNROLL
    for (int j = 0; j < 5; j++) {
        const int jj = 2 * j + 1;
        const float f1 = v[1 + 2 * j], f2 = v[2 + 2 * j];
        rg += K.wg[j] * (f1 + f2);
        rk += K.wgk[jj] * (f1 + f2);
        ra += K.wgk[jj] * (fabsf(f1) + fabsf(f2));
    }
    FJ_UNROLL
    for (int j = 0; j < 5; j++) {
        const int jj = 2 * j;
        const float f1 = v[11 + 2 * j], f2 = v[12 + 2 * j];
        rk += K.wgk[jj] * (f1 + f2);
        ra += K.wgk[jj] * (fabsf(f1) + fabsf(f2));
    }
    const float mean = 0.5f * rk;
    float rasc = K.wgk[10] * fabsf(fc - mean);
    FJ_UNROLL
    for (int jj = 0; jj < 10; jj++) {
        const float f1 = (jj & 1) ? v[jj] : v[11 + jj], f2 = (jj & 1) ? v[jj + 1] : v[12 + jj];
        rasc += K.wgk[jj] * (fabsf(f1 - mean) + fabsf(f2 - mean));
    }
    const float err = (rk - rg) * half;
    rk *= half; ra *= ahalf; rasc *= ahalf;
    res = rk; resabs = ra; resasc = rasc;
    abserr = rescale_err_f(err, ra, rasc);
}

template <class F>
FJ_HDNI void gk21_f(F &f, const GK21f &K, float a, float b, float &res, float &abserr, float &resabs, float &resasc)
{
    float v[21];
    FJ_UNROLL
    for (int e = 0; e < 21; e++) v[e] = f(gk21_abscissa(K, a, b, e));
    gk21_sum(K, a, b, v, res, abserr, resabs, resasc);
}

FJ_HD void qelg_f(float *tab, int &n_io, float *res3, int &nres, float &result, float &abserr)
{
    const int n = n_io - 1;
    const float current = tab[n];
    result = current;
    abserr = FLT_MAX;
    if (n < 2) return;
    tab[n + 2] = tab[n];
    tab[n] = FLT_MAX;
    const int newelm = n / 2;
    int n_final = n;
    for (int i = 0; i < newelm; i++) {
        float res = tab[n - 2 * i + 2];
        const float e0 = tab[n - 2 * i - 2], e1 = tab[n - 2 * i - 1], e2 = res;
        const float e1abs = fabsf(e1);
        const float delta2 = e2 - e1, err2 = fabsf(delta2);
        const float tol2 = fmaxf(fabsf(e2), e1abs) * FLT_EPSILON;
        const float delta3 = e1 - e0, err3 = fabsf(delta3);
        const float tol3 = fmaxf(e1abs, fabsf(e0)) * FLT_EPSILON;
        if (err2 <= tol2 && err3 <= tol3) {
            result = res;
            abserr = fmaxf(err2 + err3, 5 * FLT_EPSILON * fabsf(res));
            return;
        }
        const float e3 = tab[n - 2 * i];
        tab[n - 2 * i] = e1;
        const float delta1 = e1 - e3, err1 = fabsf(delta1);
        const float tol1 = fmaxf(e1abs, fabsf(e3)) * FLT_EPSILON;
        if (err1 <= tol1 || err2 <= tol2 || err3 <= tol3) { n_final = 2 * i; break; }
        const float ss = (1 / delta1 + 1 / delta2) - 1 / delta3;
        if (fabsf(ss * e1) <= 0.0001f) { n_final = 2 * i; break; }
        res = e1 + 1 / ss;
        tab[n - 2 * i] = res;
        const float error = err2 + fabsf(res - e2) + err3;
        if (error <= abserr) { abserr = error; result = res; }
    }
    if (n_final == 49) n_final = 48;
    if (n % 2 == 1) { for (int i = 0; i <= newelm; i++) tab[1 + 2 * i] = tab[2 * i + 3]; }
    else { for (int i = 0; i <= newelm; i++) tab[2 * i] = tab[2 * i + 2]; }
    if (n != n_final) for (int i = 0; i <= n_final; i++) tab[i] = tab[n - n_final + i];
    n_io = n_final + 1;
    if (nres < 3) { res3[nres] = result; abserr = FLT_MAX; }
    else {
        abserr = fabsf(result - res3[2]) + fabsf(result - res3[1]) + fabsf(result - res3[0]);
        res3[0] = res3[1]; res3[1] = res3[2]; res3[2] = result;
    }
    nres += 1;
    abserr = fmaxf(abserr, 5 * FLT_EPSILON * fabsf(result));
}

#ifndef FJ_MIXED_QAGS_CAP
#define FJ_MIXED_QAGS_CAP 64
#endif
constexpr int kQagsCapF = FJ_MIXED_QAGS_CAP;  // intervals of the FP32 QAGS list (a full list: the node is re-solved in FP64)
static_assert(kQagsCapF <= 256, "qags_f keeps interval indices as bytes");

// QAGS (DQAGSE) in FP32 on [a,b] with the reference's tolerances; interval
// list of kQagsCapF entries on the thread's stack.
template <class F>
FJ_HDNI float qags_f(F &f, const GK21f &K, float a, float b, float epsabs, float epsrel, unsigned &fail)
{
    const int limit = 1000;
    float res0, err0, resabs0, resasc0;
    gk21_f(f, K, a, b, res0, err0, resabs0, resasc0);
    const float tol = fmaxf(epsabs, epsrel * fabsf(res0));
    if (err0 <= 100 * FLT_EPSILON * resabs0 && err0 > tol) return res0;
    if ((err0 <= tol && err0 != resasc0) || err0 == 0.0f) return res0;

    float alist[kQagsCapF], blist[kQagsCapF], rlist[kQagsCapF], elist[kQagsCapF];
    unsigned char iord[kQagsCapF];  // interval indices < kQagsCapF
    float rlist2[52], res3la[3];
    int nres = 0, numrl2 = 1;
    alist[0] = a; blist[0] = b; rlist[0] = res0; elist[0] = err0; iord[0] = 0;
    rlist2[0] = res0;
    float area = res0, errsum = err0, errmax = err0;
    int maxerr = 0, nrmax = 0, last = 1, ier = 0;
    float res_ext = res0, err_ext = FLT_MAX, correc = 0, ertest = 0, erlarg = 0, small = 0;
    int ktmin = 0, ierro = 0, iroff1 = 0, iroff2 = 0, iroff3 = 0;
    bool extrap = false, noext = false, done_sum = false;
    const int ksgn = fabsf(res0) >= (1 - 50 * FLT_EPSILON) * resabs0 ? 1 : -1;
    for (last = 1; last < limit; last++) {
        if (last >= kQagsCapF) { fail |= kFailQuad; last = kQagsCapF - 1; done_sum = true; break; }
        const float a1 = alist[maxerr], b1 = 0.5f * (alist[maxerr] + blist[maxerr]);
        const float a2 = b1, b2 = blist[maxerr];
        const float erlast = errmax;
        float area1, error1, ra1, rasc1, area2, error2, ra2, rasc2;
        gk21_f(f, K, a1, b1, area1, error1, ra1, rasc1);
        gk21_f(f, K, a2, b2, area2, error2, ra2, rasc2);
        const float area12 = area1 + area2, erro12 = error1 + error2;
        errsum = errsum + erro12 - errmax;
        area = area + area12 - rlist[maxerr];
        if (!(rasc1 == error1 || rasc2 == error2)) {
            if (fabsf(rlist[maxerr] - area12) <= 1e-5f * fabsf(area12) && erro12 >= 0.99f * errmax) {
                if (extrap) iroff2++; else iroff1++;
            }
            if (last > 9 && erro12 > errmax) iroff3++;
        }
        rlist[maxerr] = area1;
        rlist[last] = area2;
        const float errbnd = fmaxf(epsabs, epsrel * fabsf(area));
        if (iroff1 + iroff2 >= 10 || iroff3 >= 20) ier = 2;
        if (iroff2 >= 5) ierro = 3;
        if (fmaxf(fabsf(a1), fabsf(b2)) <= (1 + 100 * FLT_EPSILON) * (fabsf(a2) + 1000 * FLT_MIN)) ier = 4;
        if (!(error2 > error1)) {
            alist[last] = a2; blist[maxerr] = b1; blist[last] = b2;
            elist[maxerr] = error1; elist[last] = error2;
        } else {
            alist[maxerr] = a2; alist[last] = a1; blist[last] = b1;
            rlist[maxerr] = area2; rlist[last] = area1;
            elist[maxerr] = error2; elist[last] = error1;
        }
        {   // DQPSRT
            const int L = last + 1;
            if (L <= 2) { iord[0] = 0; iord[1] = 1; }
            else {
                const float em = elist[maxerr];
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
                const int jupbn = L, jbnd = jupbn - 1, ibeg = nr1 + 1;
                const float errmin = elist[L - 1];
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
            small = fabsf(b - a) * 0.375f;
            erlarg = errsum;
            ertest = errbnd;
            rlist2[1] = area; numrl2 = 2;
            continue;
        }
        if (noext) continue;
        erlarg -= erlast;
        if (fabsf(b1 - a1) > small) erlarg += erro12;
        if (!extrap) {
            if (fabsf(blist[maxerr] - alist[maxerr]) > small) continue;
            extrap = true;
            nrmax = 1;
        }
        bool do_ext = true;
        if (!(ierro == 3 || erlarg <= ertest)) {
            for (int k = nrmax + 1; k <= last + 1; k++) {
                maxerr = iord[nrmax];
                errmax = elist[maxerr];
                if (fabsf(blist[maxerr] - alist[maxerr]) > small) { do_ext = false; break; }
                nrmax++;
            }
        }
        if (!do_ext) continue;
        rlist2[numrl2] = area; numrl2++;
        float reseps, abseps;
        qelg_f(rlist2, numrl2, res3la, nres, reseps, abseps);
        ktmin++;
        if (ktmin > 5 && err_ext < 1e-3f * errsum) ier = 5;
        if (abseps < err_ext) {
            ktmin = 0;
            err_ext = abseps;
            res_ext = reseps;
            correc = erlarg;
            ertest = fmaxf(epsabs, epsrel * fabsf(reseps));
            if (err_ext <= ertest) break;
        }
        if (numrl2 == 1) noext = true;
        if (ier == 5) break;
        maxerr = iord[0];
        errmax = elist[maxerr];
        nrmax = 0;
        extrap = false;
        small *= 0.5f;
        erlarg = errsum;
    }
    bool take_sum = done_sum;
    float result = res_ext;
    if (!done_sum) {
        if (err_ext == FLT_MAX) take_sum = true;
        else if (ier + ierro != 0) {
            if (ierro == 3) err_ext += correc;
            if (res_ext != 0.0f && area != 0.0f) {
                if (err_ext / fabsf(res_ext) > errsum / fabsf(area)) take_sum = true;
            } else if (err_ext > errsum) take_sum = true;
        }
    }
    if (take_sum) {
        float s = 0;
        for (int k = 0; k <= last; k++) s += rlist[k];
        result = s;
    }
    (void)ksgn;
    return result;
}

// ----------------------------------------------------------- fudge, FP32
// The u and v equations of uvOrb.cpp:38-52 written about the phase point
// itself, in offsets that keep their relative precision when the orbit's
// excursion is small (a near-circular orbit, a thin disc orbit):
//   u = u_pt + t:  U(t) = Ds K + EC + Lt Ds / (s^2 sh^2) - (s^2 + sv^2) dPhi,
//                  s = sinh(u), sh = sinh(u_pt), Ds = s^2 - sh^2 formed for
//                  |t| < 1/2 from sinh(t) and cosh(t) - 1 (one expm1); for
//                  |t| >= 1/2, Ds K + EC = s^2 K + C0 with C0 = EC - sh^2 K
//                  formed in FP64 (far from the focus sh^2 K and EC are ~(r/Delta)^2
//                  times larger than U);
//   v = pi/2 - w:  V(w) = Dv (K + Lt / (sv^2 cos^2 w)) + pv^2/(2 Delta^2) - (sh^2 + cos^2 w) dPhi,
//                  Dv = cos^2 v_pt - sin^2 w = (|cos v_pt| - sin w)(|cos v_pt| + sin w);
// Lt = Lz^2/(2 Delta^2), EC = pu^2/(2 Delta^2), K = E - Phi_pt the kinetic
// energy of the node, dPhi = Phi - Phi_pt from pot_dphi_f (on these lines
// r^2 - r_pt^2 = Delta^2 Ds and -Delta^2 Dv).  Both follow from the reference's equations with the
// reference point u0 = u_pt (the u-equation does not depend on u0; it cancels
// exactly) and the Phi(pi/2) terms of Iv and dV cancelled.  The v-equation
// near the pole (v -> 0) keeps v itself as the variable, with
// Dv = sin^2 v - sin^2 v_pt formed as (sin v - sin v_pt)(sin v + sin v_pt).
struct FudgeF {
    PotViewF P;
    float Delta, D2, K, EC, C0, Lt, shu2, sv2, swp, svp, sinv, cosv, sinhu, coshu, pvterm;
    float rpt, Phipt;  // the point: radius and FP32 potential
    double u_pt;
    float tb, Dt;  // Ju: centre and half-width of [t_in, t_out]
    float wt;      // Jv: turning point in w
};

// What fudge_eval evaluates at x: the u-equation U(t), the v-equation V(w) or
// V(v), and the momentum integrands of Ju (uvOrb.cpp:226-239, u = ubar -
// Deltau cos psi) and Jv (uvOrb.cpp:247-257, v = pi/2 - (pi/2 - vturn) cos psi).
enum : int { kEvU = 0, kEvVw = 1, kEvVv = 2, kEvJu = 3, kEvJv = 4 };

// geometry of a position on the coordinate line, and U or V = A + Bc dPhi
struct FGeo {
    float R, z, dr2, dc2, A, Bc, fac;
};

FJ_HD void fudge_geom(const FudgeF &o, int mode, float x, FGeo &G)
{
    float fac = 1.f;
    int m = mode;
    if (mode >= kEvJu) {
        float sn, cs;
        sincos_psi(x, &sn, &cs);
        fac = sn;
        if (mode == kEvJu) { x = o.tb - o.Dt * cs; m = kEvU; }
        else {
            const float w = o.wt * cs;
            if (w <= .5f * kPIHf) { x = w; m = kEvVw; }
            else { x = kPIHf - w; m = kEvVv; }
        }
    }
    G.fac = fac;
    if (m == kEvU) {
        float s, c, Ds, KE;
        if (fabsf(x) < .5f) {  // offsets: no cancellation for |t| < 1/2
            float st, cm1;
            sinh_coshm1(x, st, cm1);
            const float ds = o.sinhu * cm1 + o.coshu * st;  // sinh(u_pt + t) - sinh(u_pt)
            s = o.sinhu + ds;
            c = o.coshu + o.coshu * cm1 + o.sinhu * st;
            Ds = ds * (s + o.sinhu);
            KE = Ds * o.K + o.EC;
        } else {  // far from the point the direct form has no cancellation
            float cm1;
            sinh_coshm1((float)o.u_pt + x, s, cm1);
            c = 1.f + cm1;
            Ds = s * s - o.shu2;
            KE = s * s * o.K + o.C0;
        }
        const float s2 = s * s, cv2 = o.swp * o.swp;
        G.R = o.Delta * s * o.sinv;
        G.z = o.Delta * c * o.cosv;
        G.dr2 = o.D2 * Ds;
        G.dc2 = -cv2 * o.sv2 * Ds / ((s2 + cv2) * (o.shu2 + cv2));
        G.A = KE + (o.Lt > 0.f ? o.Lt * Ds / (s2 * o.shu2) : 0.f);
        G.Bc = -(s2 + o.sv2);
    } else {
        float sn, cs, Dv;
        sincosf(x, &sn, &cs);
        if (m == kEvVw) {  // x = w: sin v = cos w, cos v = sin w
            Dv = (o.swp - sn) * (o.swp + sn);  // cos^2 v_pt - sin^2 w
            const float t_ = sn; sn = cs; cs = t_;
        } else {
            Dv = (sn - o.svp) * (sn + o.svp);  // sin^2 v - sin^2 v_pt
        }
        const float s2 = sn * sn;
        G.R = o.Delta * o.sinhu * sn;
        G.z = o.Delta * o.coshu * cs;
        G.dr2 = -o.D2 * Dv;
        G.dc2 = -(1.f + o.shu2) * o.shu2 * Dv / ((o.shu2 + cs * cs) * (o.shu2 + o.swp * o.swp));
        G.A = Dv * (o.K + (o.Lt > 0.f ? o.Lt / (o.sv2 * s2) : 0.f)) + o.pvterm;
        G.Bc = -(o.shu2 + s2);
    }
}

FJ_HD float fudge_finish(int mode, const FGeo &G, float dphi)
{
    const float val = G.A + G.Bc * dphi;
    return mode >= kEvJu ? sqrtf(fmaxf(0.f, val)) * G.fac : val;
}

// The one evaluator of every FP32 turning-point search and momentum
// integral: the position on the coordinate line and the exact geometry
// differences, a single pot_dphi_f, then U or V as A + B dPhi.  Kept out of
// line, so Brent, the bracket walks and QAGS each exist once in the binary
// and the divergent warps' working set fits the instruction cache.
FJ_HDNI float fudge_eval(const FudgeF &o, int mode, float x)
{
    FGeo G;
    fudge_geom(o, mode, x, G);
    return fudge_finish(mode, G, pot_dphi_f(o.P, G.R, G.z, o.rpt, G.dr2, G.dc2, o.Phipt));
}

// dU/du for the bracket's slope tests (uvOrb.cpp:54-61); E - Phi = K - (Phi - Phi_pt)
FJ_HDNI float fudge_du(const FudgeF &o, float u)
{
    float shu, chm1;
    sinh_coshm1(u, shu, chm1);
    const float chu = 1.f + chm1, s2 = shu * shu;
    const float sv = sqrtf(o.sv2), cv = o.cosv < 0.f ? -o.swp : o.swp;
    float phi0, f0, f1;
    pot_grad_f(o.P, o.Delta * shu * o.sinv, o.Delta * chu * o.cosv, phi0, f0, f1);
    const float dPhidu = o.Delta * (f0 * chu * sv + f1 * shu * cv);
    return 2.f * (o.K - (phi0 - o.Phipt)) * shu * chu - (s2 + o.sv2) * dPhidu + 2.f * o.Lt * chu / (s2 * shu);
}

// fudge_eval as a functor of x for Brent and QAGS (one type, one instance each)
struct FudgeFn {
    const FudgeF *o;
    int mode;
    FJ_HD float operator()(float x) const { return fudge_eval(*o, mode, x); }
};

// uvOrb::GetTurnu (uvOrb.cpp:131-201): the bracket walk in FP64 positions
// (cheap scalar steps, the same step sequence as the reference down to its
// 1e-12 refinement limit, where Jr = 0), the u-equation in FP32, Brent in
// t = u - u_pt.  Returns false when the u-equation leaves the FP32 range
// (sinh(u)^2 overflows beyond u ~ 44) or at the step cap; the caller then
// redoes the u solve in FP64.
FJ_HDNI bool get_turn_u_f(FudgeF &o, double utry, float &tin, float &tout, unsigned &fail)
{
    const FudgeFn U{&o, kEvU};
    const double u0 = o.u_pt;
    double u1 = utry, u2 = utry, uin = utry, uout = utry, eps = .1;
    float ut = U((float)(utry - u0)), dut = fudge_du(o, (float)utry);
    int it = 0;
#define FJ_STEP_U(x) { ut = U((float)((x) - u0)); if (++it > kLoopCap || !isfinite(ut)) return false; }
#define FJ_STEP_UD(x) { ut = U((float)((x) - u0)); dut = fudge_du(o, (float)(x)); \
                        if (++it > kLoopCap || !isfinite(ut)) return false; }
    if (!isfinite(ut)) return false;
    if (ut < 0) {
        if (dut > 0) {
            uin = utry;
            for (;;) {
                while (ut < 0 && dut > 0) { uin = utry; utry *= (1 + eps); FJ_STEP_UD(utry); }
                if (ut >= 0) { u1 = utry; break; }
                utry /= (1 + eps); eps *= .2;
                if (eps < kTINY) { tin = tout = (float)(utry - u0); return true; }
                utry *= (1 + eps);
                FJ_STEP_UD(utry);
            }
            while (ut > 0) { u2 = utry; utry *= 1.1; FJ_STEP_U(utry); }
            uout = utry;
        } else {
            for (;;) {
                while (ut < 0 && dut < 0) { uout = utry; utry /= (1 + eps); FJ_STEP_UD(utry); }
                if (ut >= 0) { u2 = utry; break; }
                utry *= (1 + eps); eps *= .2;
                if (eps < kTINY) { tin = tout = (float)(utry - u0); return true; }
                utry /= (1 + eps);
                FJ_STEP_UD(utry);
            }
            while (ut > 0) { u1 = utry; utry *= .9; FJ_STEP_U(utry); }
            uin = utry;
        }
    } else {
        const float fu1 = ut;
        while (ut > 0) { u2 = utry; utry *= 1.1; FJ_STEP_U(utry); }
        uout = utry;
        ut = fu1;
        while (ut > 0) { u1 = utry; utry *= .9; FJ_STEP_U(utry); }
        uin = utry;
    }
#undef FJ_STEP_U
#undef FJ_STEP_UD
    fail |= brent_root_f(U, (float)(uin - u0), (float)(u1 - u0), tin);
    fail |= brent_root_f(U, (float)(u2 - u0), (float)(uout - u0), tout);
    return true;
}

// uvOrb::GetTurnv (uvOrb.cpp:203-224) with the turning point returned as
// w = pi/2 - v.  Towards the equator the walk halves w, towards the pole it
// halves v (both exact in FP32), down to the reference's 1e-12 limits.
// Returns false at the step cap (the caller redoes the v solve in FP64).
FJ_HDNI bool get_turn_v_f(FudgeF &o, float &wturn, unsigned &fail)
{
    const float q = .5f * kPIHf;  // vtry = pi/4
    int it = 0;
    if (fudge_eval(o, kEvVw, q) < 0) {
        const FudgeFn V{&o, kEvVw};
        float wbot = q;
        while (V(wbot) < 0) {
            wbot *= .5f;
            if (wbot < 1e-12f) { wturn = 0.f; return true; }
            if (++it > kLoopCap) return false;
        }
        fail |= brent_root_f(V, q, wbot, wturn);
    } else {
        const FudgeFn V{&o, kEvVv};
        float vtop = q;
        while (V(vtop) > 0) {
            vtop *= .5f;
            if (vtop < 1e-12f) { wturn = kPIHf; return true; }
            if (++it > kLoopCap) return false;
        }
        float vt;
        fail |= brent_root_f(V, vtop, q, vt);
        wturn = kPIHf - vt;
    }
    return true;
}

// FP64 fudge state with the reference point u0 at the orbit's own u
// (the u-equation does not depend on u0), for turning points at the limits.
FJ_HDNI void fudge64_at_point(Fudge &o, const PotView &P, double Delta, double Lzsq, double E, double u, double v,
                              double shu2, double sv, double cv, double sv2, double pu, double pv)
{
    o.P = P; o.fail = 0; o.Delta = Delta; o.Lzsq = Lzsq; o.E = E;
    o.u = u; o.v = v; o.shu2 = shu2; o.sv = sv; o.cv = cv; o.sv2 = sv2;
    sincos(v, &o.sinv, &o.cosv);
    o.sinhu = sinh(u);
    o.coshu = cosh(u);
    o.sh1sq = o.sinhu * o.sinhu;
    o.ch1sq = o.coshu * o.coshu;
    o.umid = u;
    o.Phiu1 = o.Phiu(o.sinhu, o.coshu);
    o.PhivPIH = o.Phiv(sin(kPIH), cos(kPIH));
    const double D2 = Delta * Delta;
    o.Er = .5 * (pu * pu) / (D2 * o.ch1sq);
    double sn, cs;
    sincos(v, &sn, &cs);
    const double dVv = (1 + shu2) * o.PhivPIH - (shu2 + sn * sn) * o.Phiv(sn, cs);
    o.Iv = .5 * (pv * pv) / D2 - E * sv2 + .5 * Lzsq / (D2 * sv2) - dVv;
}

// FP32 tables of PotViewF for the phase point whose potential is Phi_h;
// entries i0, i0 + stride, ... (a block's threads share the work).  ih has
// nr-1 entries, qc 4*kQuadIntervals.
// cos^2 of the polar angle of the grid point (R, z) and the even Legendre
// polynomials there, P_2k(c2) for k < npoly, by the recurrence of leg_f
FJ_HD float point_c2_f(double R, double z)
{
    const double r2 = R * R + z * z;
    return r2 > 0 ? (float)(z * z / r2) : 1.f;
}

FJ_HD void point_legendre_f(float y, int npoly, float *pyl)
{
    const LegCoefF &L = leg_f();
    float p1 = 1.f, p2 = 1.f;
    for (int k = 0; k < npoly; k++) {
        const float pk = k == 0 ? 1.f : (k == 1 ? 1.5f * y - .5f : ((y - L.B[k]) * p1 - L.A[k] * p2) * L.C[k]);
        pyl[k] = pk;
        p2 = p1; p1 = pk;
    }
}

// FP32 tables of one grid point (R, z): radii, potential multipoles shifted by
// Phi_h, interval reciprocals, quadratic-correction constants and P_2k(c2pt);
// threads i0, i0 + stride, ... share the work
FJ_HD void mixed_tables_f(int nr, int npoly, const double *ar, const double *phil, const double *Pr, double Phi_h,
                          double R, double z, float *far, float *fphil, float *fPr, float *ih, float *qc, float *pyl,
                          int i0, int stride)
{
    for (int i = i0; i < nr; i += stride) far[i] = (float)ar[i];
    for (int i = i0; i < nr - 1; i += stride) ih[i] = (float)(1.0 / (ar[i + 1] - ar[i]));
    for (int i = i0; i < 4 * kQuadIntervals; i += stride) {
        const int n = i / 4, j = i % 4, thr = j < 2 ? n - 1 : n + 2;
        double v = 0;
        if (thr >= 0 && thr < nr && n + 1 < nr)
            v = j % 2 == 0 ? 1.0 / ((ar[thr] - ar[n + 1]) * (ar[thr] - ar[n])) : (ar[thr] - ar[n]) / (ar[n + 1] - ar[n]);
        qc[i] = (float)v;
    }
    for (int i = i0; i < nr * npoly; i += stride) {
        fphil[i] = (float)(i % npoly == 0 ? phil[i] - Phi_h : phil[i]);
        fPr[i] = (float)Pr[i];
    }
    if (i0 == 0) point_legendre_f(point_c2_f(R, z), npoly, pyl);
}

// PotViewF over tables built by mixed_tables_f
FJ_HD PotViewF mixed_view_f(int nr, int npoly, const double *ar, const double *phil, double Phi_h, double R, double z,
                            const float *far, const float *fphil, const float *fPr, const float *ih, const float *qc,
                            const float *pyl)
{
    PotViewF v;
    v.nr = nr; v.npoly = npoly; v.ar = far; v.phil = fphil; v.Pr = fPr; v.ih = ih; v.qc = qc;
    v.out0 = (float)phil[(nr - 1) * npoly];
    v.shift = (float)Phi_h;
    v.lr0 = (float)log(ar[0]);
    v.idl = (float)((nr - 1) / log(ar[nr - 1] / ar[0]));
    v.c2pt = point_c2_f(R, z);
    v.pyl = pyl;
    return v;
}

// One velocity node of the mixed form: the prolate-spheroidal transform of
// the phase point (Uvpt.cpp:11-24) in FP64, Ju and Jv (uvOrb.cpp:226-257)
// with FP32 turning points and QAGS, FP64 turning points at the limits, and
// the double-power-law DF (DF.cpp:65-76,108-119) in FP32.  PF is shifted by
// PF.shift = Phi_h (mixed_tables_f); the node's energy enters shifted too.
// Returns the DF (NaN -> 0 as DF.cpp:105); fail gets the kFail* bits,
// esc = 1 when the FP64 turning-point path ran; J (optional) the actions.
FJ_HDNI double mixed_node_df(const PotView &P, const PotViewF &PF, const GK21f &K, const DFDev &d, double Delta,
                             double R, double z, double Phi_h, double V0, double V1, double V2, unsigned &fail,
                             unsigned &esc, double *J = nullptr)
{
    const double Lz = R * V1, Lzsq = Lz * Lz;
    const double D2 = Delta * Delta, R2 = R * R, z2 = z * z, r2 = R2 + z2;
    const double dmr = D2 - r2, dpr = D2 + r2;
    const double shu2 = .5 * (r2 - D2 + sqrt(dmr * dmr + 4 * D2 * R2)) / D2;
    const double shu = sqrt(shu2), chu = sqrt(1 + shu2);
    const double u = asinh(shu);
    const double cv2 = .5 * (r2 + D2 - sqrt(dpr * dpr - 4 * D2 * z2)) / D2;
    const double cv = z < 0 ? -sqrt(cv2) : sqrt(cv2);
    const double v = acos(cv), sv = sin(v), sv2 = 1 - cv2;
    const double pu = Delta * (V0 * chu * sv + V2 * shu * cv);
    const double pv = Delta * (V0 * shu * cv - V2 * chu * sv);
    const double E = .5 * (V0 * V0 + V2 * V2) + .5 * Lzsq / R2 + Phi_h;
    double Jr = 1e31, Jz = 1e31;
    if (!(E >= 0 || isnan(E))) {
        FudgeF o;
        o.P = PF;
        o.Delta = (float)Delta;
        o.D2 = (float)D2;
        o.K = (float)(.5 * (V0 * V0 + V2 * V2) + .5 * Lzsq / R2);
        o.EC = (float)(.5 * (pu * pu) / D2);
        o.C0 = (float)(.5 * (pu * pu) / D2 - shu2 * (.5 * (V0 * V0 + V2 * V2) + .5 * Lzsq / R2));
        o.Lt = (float)(.5 * Lzsq / D2);
        o.shu2 = (float)shu2;
        o.sv2 = (float)sv2;
        o.swp = (float)fabs(cv);
        o.svp = (float)sqrt(sv2);
        double sn, cs;
        sincos(v, &sn, &cs);
        o.sinv = (float)sn; o.cosv = (float)cs;
        o.sinhu = (float)shu; o.coshu = (float)chu;
        o.pvterm = (float)(.5 * (pv * pv) / D2);
        o.u_pt = u;
        o.rpt = (float)(Delta * sqrt(shu2 + cv2));
        o.Phipt = pot_phi_f(PF, o.Delta * o.sinhu * o.sinv, o.Delta * o.coshu * o.cosv);
        Fudge o64;
        bool have64 = false;
        const float rtwo = 1.41421356237309505f;
        float tin, tout;
        if (!get_turn_u_f(o, 1.0, tin, tout, fail)) {  // u limit: FP64 (uvOrb.cpp:131-201)
            fudge64_at_point(o64, P, Delta, Lzsq, E, u, v, shu2, sv, cv, sv2, pu, pv);
            have64 = true;
            get_turn_u(o64, 1);
            fail |= o64.fail;
            tin = (float)(o64.uinner - u); tout = (float)(o64.uouter - u);
            esc = 1u;
        }
        if (fabsf(tout - tin) < 1e-12f) Jr = 0;
        else {
            o.tb = .5f * (tin + tout);
            o.Dt = .5f * (tout - tin);
            const FudgeFn fju{&o, kEvJu};
            Jr = (double)(rtwo * o.Delta * o.Dt * qags_f(fju, K, 0.f, kPIf, 1e-5f, 1e-3f, fail) / kPIf);
        }
        float wt;
        if (!get_turn_v_f(o, wt, fail)) {  // v at the pole: FP64 (uvOrb.cpp:203-224)
            if (!have64) fudge64_at_point(o64, P, Delta, Lzsq, E, u, v, shu2, sv, cv, sv2, pu, pv);
            const double v64 = get_turn_v(o64, .5 * kPIH);
            fail |= o64.fail;
            wt = (float)(kPIH - v64);
            esc = 1u;
        }
        if (wt < 1e-12f) Jz = 0;
        else {
            o.wt = wt;
            const FudgeFn fjv{&o, kEvJv};
            Jz = (double)(2.f * rtwo * o.Delta * wt * qags_f(fjv, K, 0.f, kPIHf, 1e-5f, 1e-3f, fail) / kPIf);
        }
    }
    if (J) { J[0] = Jr; J[1] = Jz; }
    const float Jphi = (float)Lz, jr = (float)Jr, jz = (float)Jz, J0 = (float)d.J0;
    const float h = jr + (float)d.dphi_h * fabsf(Jphi) + (float)d.dz_h * jz;
    const float g = jr + (float)d.dphi_g * fabsf(Jphi) + (float)d.dz_g * jz;
    const float ev = (float)d.norm * fmaxf(0.f, powf(1.f + J0 / h, (float)d.alpha) / powf(1.f + g / J0, (float)d.beta)) /
                     (float)d.tpi3;
    float f = d.chi == 0. ? ev : ev + (float)d.k * tanhf((float)d.chi * Jphi / J0) * ev;
    if (isnan(f)) f = 0.f;
    return (double)f;
}

}  // namespace fj
