/*
 * orc_numerics.c -- oracle numerics: Gauss-Legendre nodes, Brent root
 * bracketing wrapper, QUADPACK QAGS / QAGIU, and the adaptive orbit
 * integrator used by the focal-distance tabulation.
 *
 * TEST INFRASTRUCTURE ONLY (see fjoracle.h).
 *
 * The reference delegates these to GSL (not vendored, version unpinned:
 * configure.ac:108-124 only probes for libgsl; .travis.yml installs the
 * distribution's GSL 1.x).  They are restated here from the published
 * algorithms:
 *   - Brent, "Algorithms for Minimization without Derivatives" (1973), ch. 4,
 *     in the one-step-per-call form of GSL's documented root-solver interface;
 *   - Piessens, de Doncker-Kapenga, Ueberhuber, Kahaner, "QUADPACK" (1983):
 *     DQAGSE with DQK21, DQPSRT and DQELG; QAGIU as DQAGSE applied to
 *     f(a+(1-t)/t)/t^2 on (0,1] with the 15-point Kronrod rule;
 *   - the Runge-Kutta 8(7) pair of Prince & Dormand (1981), RK8(7)13M (the
 *     stepper the reference names, gsl_odeiv2_step_rk8pd), with the y-error
 *     step-size controller described in the GSL manual (odeiv2).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fjoracle.h"
#include "orc_internal.h"
#include "orc_kronrod.h"
#include "orc_rk8pd.h"

/* Gauss-Legendre nodes on [x1,x2] (UtilsLeg.h:18-39, NGAUSS replaced by n). */
void orc_gauleg(double x1, double x2, int n, double *x, double *w)
{
    const double eps = 3.0e-11;
    int m = (n + 1) / 2;
    double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1), pp = 0.0, z1;
    for (int i = 0; i < m; i++) {
        double z = cos(3.141592654 * (i + 0.75) / (n + 0.5));
        do {
            double p1 = 1, p2 = 0, p3;
            for (int j = 0; j < n; j++) {
                p3 = p2;
                p2 = p1;
                p1 = ((2 * (j + 1) - 1) * z * p2 - j * p3) / (double)(j + 1);
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            z1 = z;
            z = z1 - p1 / pp;
        } while (fabs(z - z1) > eps);
        x[i] = xm - xl * z;
        x[n - i - 1] = xm + xl * z;
        w[i] = 2 * xl / ((1 - z * z) * pp * pp);
        w[n - i - 1] = w[i];
    }
}

/* ------------------------------------------------------------------------
 * Brent root finding with the reference wrapper's stopping rule
 * (include/Utils.h:134-167): return an end point whose |f| < 5e-4; otherwise
 * iterate Brent steps until the bracket passes the interval test
 * |hi-lo| < 1e-8 + 1e-6*min(|lo|,|hi|) (0 if the bracket holds 0) AND
 * hi-lo <= 1e-8.  Returns 0 on success, 1 if the iteration cap was hit.
 * ---------------------------------------------------------------------- */
#define ROOT_EPSABS 1e-8
#define ROOT_EPSREL 1e-6
#define ROOT_MAXIT 2000

static int same_sign(double x, double y) { return (x < 0 && y < 0) || (x > 0 && y > 0); }

_Thread_local long long orc_brent_iterations = 0;

void orc_brent_init(orc_brent *s, double (*f)(double, void *), void *p, double lo, double hi,
                    double flo, double fhi)
{
    s->f = f; s->p = p;
    s->a = lo; s->fa = flo; s->b = hi; s->fb = fhi; s->c = hi; s->fc = fhi;
    s->d = hi - lo; s->e = hi - lo;
    s->root = 0.5 * (lo + hi); s->lo = lo; s->hi = hi;
}

/* One step of Brent's method (zeroin): inverse quadratic / secant step
   when it is safe, bisection otherwise.  Reports the current best root and
   the bracket [min(b,c), max(b,c)]. */
void orc_brent_step(orc_brent *s)
{
    double a = s->a, b = s->b, c = s->c, fa = s->fa, fb = s->fb, fc = s->fc, d = s->d, e = s->e;
    orc_brent_iterations++;
    int secant = 0;
    if (same_sign(fb, fc)) { secant = 1; c = a; fc = fa; d = b - a; e = b - a; }
    if (fabs(fc) < fabs(fb)) { secant = 1; a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
    double tol = 0.5 * DBL_EPSILON * fabs(b);
    double m = 0.5 * (c - b);
    if (fb == 0) { s->root = b; s->lo = b; s->hi = b; return; }
    if (fabs(m) <= tol) { s->root = b; s->lo = b < c ? b : c; s->hi = b < c ? c : b; return; }
    if (fabs(e) < tol || fabs(fa) <= fabs(fb)) { d = m; e = m; }
    else {
        double sr = fb / fa, pn, q, r;
        if (secant) { pn = 2 * m * sr; q = 1 - sr; }
        else {
            q = fa / fc; r = fb / fc;
            pn = sr * (2 * m * q * (q - r) - (b - a) * (r - 1));
            q = (q - 1) * (r - 1) * (sr - 1);
        }
        if (pn > 0) q = -q; else pn = -pn;
        double lim1 = 3 * m * q - fabs(tol * q), lim2 = fabs(e * q);
        if (2 * pn < (lim1 < lim2 ? lim1 : lim2)) { e = d; d = pn / q; }
        else { d = m; e = m; }
    }
    a = b; fa = fb;
    if (fabs(d) > tol) b += d; else b += (m > 0 ? +tol : -tol);
    fb = s->f(b, s->p);
    s->a = a; s->b = b; s->c = c; s->fa = fa; s->fb = fb; s->fc = fc; s->d = d; s->e = e;
    s->root = b;
    double cc = same_sign(fb, fc) ? a : c;
    s->lo = b < cc ? b : cc;
    s->hi = b < cc ? cc : b;
}

/* GSL's documented interval test: |hi-lo| < epsabs + epsrel*min(|lo|,|hi|),
   with min replaced by 0 when the interval contains the origin. */
int orc_root_test_interval(double lo, double hi, double epsabs, double epsrel)
{
    double alo = fabs(lo), ahi = fabs(hi);
    double mn = ((lo > 0 && hi > 0) || (lo < 0 && hi < 0)) ? (alo < ahi ? alo : ahi) : 0.0;
    return fabs(hi - lo) < epsabs + epsrel * mn;
}

int orc_brent_wrapped(double (*f)(double, void *), void *p, double lo, double hi, double *root)
{
    double flo = f(lo, p);
    if (fabs(flo) < 5e-4) { *root = lo; return 0; }
    double fhi = f(hi, p);
    if (fabs(fhi) < 5e-4) { *root = hi; return 0; }
    orc_brent s;
    orc_brent_init(&s, f, p, lo, hi, flo, fhi);
    for (int it = 0; it < ROOT_MAXIT; it++) {
        orc_brent_step(&s);
        if (orc_root_test_interval(s.lo, s.hi, ROOT_EPSABS, ROOT_EPSREL) && !(s.hi - s.lo > ROOT_EPSABS)) {
            *root = s.root;
            return 0;
        }
    }
    *root = s.root;
    return 1;
}

/* ------------------------------------------------------------------------
 * QUADPACK
 * ---------------------------------------------------------------------- */
typedef double (*orc_fn)(double, void *);

static double rescale_err(double err, double resabs, double resasc)
{
    err = fabs(err);
    if (resasc != 0 && err != 0) {
        double scale = pow(200 * err / resasc, 1.5);
        err = scale < 1 ? resasc * scale : resasc;
    }
    if (resabs > DBL_MIN / (50 * DBL_EPSILON)) {
        double min_err = 50 * DBL_EPSILON * resabs;
        if (min_err > err) err = min_err;
    }
    return err;
}

/* One Gauss-Kronrod panel.  nk = number of non-negative Kronrod nodes
   (11 for 21 points, 8 for 15 points); xgk descending with 0 last. */
static void gk_panel(orc_fn f, void *p, double a, double b, int nk, const double *xgk,
                     const double *wgk, const double *wg, double *res, double *abserr,
                     double *resabs, double *resasc)
{
    double fv1[11], fv2[11];
    double center = 0.5 * (a + b), half = 0.5 * (b - a), ahalf = fabs(half);
    double fc = f(center, p);
    double rg = 0, rk = fc * wgk[nk - 1], ra = fabs(rk);
    if (nk % 2 == 0) rg = fc * wg[nk / 2 - 1];
    for (int j = 0; j < (nk - 1) / 2; j++) {
        int jj = 2 * j + 1;
        double x = half * xgk[jj];
        double f1 = f(center - x, p), f2 = f(center + x, p);
        fv1[jj] = f1; fv2[jj] = f2;
        rg += wg[j] * (f1 + f2);
        rk += wgk[jj] * (f1 + f2);
        ra += wgk[jj] * (fabs(f1) + fabs(f2));
    }
    for (int j = 0; j < nk / 2; j++) {
        int jj = 2 * j;
        double x = half * xgk[jj];
        double f1 = f(center - x, p), f2 = f(center + x, p);
        fv1[jj] = f1; fv2[jj] = f2;
        rk += wgk[jj] * (f1 + f2);
        ra += wgk[jj] * (fabs(f1) + fabs(f2));
    }
    double mean = 0.5 * rk;
    double rasc = wgk[nk - 1] * fabs(fc - mean);
    for (int j = 0; j < nk - 1; j++) rasc += wgk[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
    double err = (rk - rg) * half;
    rk *= half; ra *= ahalf; rasc *= ahalf;
    *res = rk; *resabs = ra; *resasc = rasc;
    *abserr = rescale_err(err, ra, rasc);
}

typedef struct { orc_fn f; void *p; double a; } infmap;
static double inf_transform(double t, void *vp)
{
    infmap *m = (infmap *)vp;
    double x = m->a + (1 - t) / t;
    double y = m->f(x, m->p);
    return (y / t) / t;
}

/* Wynn epsilon extrapolation (DQELG).  tab holds n entries (n>=1, room for
   n+2); res3 and *nres keep the last three results.  As in the GSL variant,
   *nres only advances when the table is actually processed. */
static void qelg(double *tab, int *n_io, double *res3, int *nres, double *result, double *abserr)
{
    int n = *n_io - 1; /* index of newest entry */
    double current = tab[n];
    *result = current;
    *abserr = DBL_MAX;
    if (n < 2) {
        double rel = 5 * DBL_EPSILON * fabs(current);
        *abserr = DBL_MAX > rel ? DBL_MAX : rel;
        return;
    }
    tab[n + 2] = tab[n];
    tab[n] = DBL_MAX;
    int newelm = n / 2, n_orig = n, n_final = n;
    for (int i = 0; i < newelm; i++) {
        double res = tab[n - 2 * i + 2];
        double e0 = tab[n - 2 * i - 2], e1 = tab[n - 2 * i - 1], e2 = res;
        double e1abs = fabs(e1);
        double delta2 = e2 - e1, err2 = fabs(delta2);
        double tol2 = (fabs(e2) > e1abs ? fabs(e2) : e1abs) * DBL_EPSILON;
        double delta3 = e1 - e0, err3 = fabs(delta3);
        double tol3 = (e1abs > fabs(e0) ? e1abs : fabs(e0)) * DBL_EPSILON;
        if (err2 <= tol2 && err3 <= tol3) {
            double rel = 5 * DBL_EPSILON * fabs(res);
            *result = res;
            *abserr = (err2 + err3) > rel ? (err2 + err3) : rel;
            return;
        }
        double e3 = tab[n - 2 * i];
        tab[n - 2 * i] = e1;
        double delta1 = e1 - e3, err1 = fabs(delta1);
        double tol1 = (e1abs > fabs(e3) ? e1abs : fabs(e3)) * DBL_EPSILON;
        if (err1 <= tol1 || err2 <= tol2 || err3 <= tol3) { n_final = 2 * i; break; }
        double ss = (1 / delta1 + 1 / delta2) - 1 / delta3;
        if (fabs(ss * e1) <= 0.0001) { n_final = 2 * i; break; }
        res = e1 + 1 / ss;
        tab[n - 2 * i] = res;
        double error = err2 + fabs(res - e2) + err3;
        if (error <= *abserr) { *abserr = error; *result = res; }
    }
    if (n_final == 49) n_final = 2 * (49 / 2);
    if (n_orig % 2 == 1) { for (int i = 0; i <= newelm; i++) tab[1 + 2 * i] = tab[2 * i + 3]; }
    else { for (int i = 0; i <= newelm; i++) tab[2 * i] = tab[2 * i + 2]; }
    if (n_orig != n_final) for (int i = 0; i <= n_final; i++) tab[i] = tab[n_orig - n_final + i];
    *n_io = n_final + 1;
    if (*nres < 3) { res3[*nres] = *result; *abserr = DBL_MAX; }
    else {
        *abserr = fabs(*result - res3[2]) + fabs(*result - res3[1]) + fabs(*result - res3[0]);
        res3[0] = res3[1]; res3[1] = res3[2]; res3[2] = *result;
    }
    *nres += 1;
    double rel = 5 * DBL_EPSILON * fabs(*result);
    if (rel > *abserr) *abserr = rel;
}

/* Adaptive bisection with extrapolation (DQAGSE).  rule 21 or 15.
   Returns 0 on success, a positive QUADPACK error class otherwise. */
_Thread_local int orc_qags_hist[8];
static int qags_core(orc_fn f, void *p, double a, double b, double epsabs, double epsrel, int limit,
                     int rule, double *result, double *abserr)
{
    const double *xgk = rule == 21 ? orc_xgk21 : orc_xgk15;
    const double *wgk = rule == 21 ? orc_wgk21 : orc_wgk15;
    const double *wg = rule == 21 ? orc_wg10 : orc_wg7;
    int nk = rule == 21 ? 11 : 8;

    double *alist = malloc(sizeof(double) * 4 * (size_t)limit);
    double *blist = alist + limit, *rlist = blist + limit, *elist = rlist + limit;
    int *iord = malloc(sizeof(int) * (size_t)limit);
    double rlist2[52], res3la[3];
    int nres = 0, numrl2;

    double res0, err0, resabs0, resasc0;
    gk_panel(f, p, a, b, nk, xgk, wgk, wg, &res0, &err0, &resabs0, &resasc0);
    alist[0] = a; blist[0] = b; rlist[0] = res0; elist[0] = err0; iord[0] = 0;
    double tol = epsabs > epsrel * fabs(res0) ? epsabs : epsrel * fabs(res0);
    int ier = 0;
    if (err0 <= 100 * DBL_EPSILON * resabs0 && err0 > tol) ier = 2;
    else if ((err0 <= tol && err0 != resasc0) || err0 == 0.0) { orc_qags_hist[0]++; *result = res0; *abserr = err0; free(alist); free(iord); return 0; }
    else if (limit == 1) ier = 1;
    if (ier) { *result = res0; *abserr = err0; free(alist); free(iord); return ier; }

    rlist2[0] = res0; numrl2 = 1;
    double area = res0, errsum = err0, errmax = err0;
    int maxerr = 0, nrmax = 0, last = 1;
    double res_ext = res0, err_ext = DBL_MAX, correc = 0, ertest = 0, erlarg = 0, small = 0;
    int ktmin = 0, extrap = 0, noext = 0, iroff1 = 0, iroff2 = 0, iroff3 = 0, ierro = 0;
    int ksgn = fabs(res0) >= (1 - 50 * DBL_EPSILON) * resabs0 ? 1 : -1;
    int done_sum = 0; /* 1: take the plain sum of panels */

    for (last = 1; last < limit; last++) {
        double a1 = alist[maxerr], b1 = 0.5 * (alist[maxerr] + blist[maxerr]);
        double a2 = b1, b2 = blist[maxerr];
        double erlast = errmax;
        double area1, error1, ra1, rasc1, area2, error2, ra2, rasc2;
        gk_panel(f, p, a1, b1, nk, xgk, wgk, wg, &area1, &error1, &ra1, &rasc1);
        gk_panel(f, p, a2, b2, nk, xgk, wgk, wg, &area2, &error2, &ra2, &rasc2);
        double area12 = area1 + area2, erro12 = error1 + error2;
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
        double errbnd = epsabs > epsrel * fabs(area) ? epsabs : epsrel * fabs(area);
        if (iroff1 + iroff2 >= 10 || iroff3 >= 20) ier = 2;
        if (iroff2 >= 5) ierro = 3;
        if (last == limit - 1) ier = 1;
        double mx = fabs(a1) > fabs(b2) ? fabs(a1) : fabs(b2);
        if (mx <= (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN)) ier = 4;
        if (!(error2 > error1)) {
            alist[last] = a2; blist[maxerr] = b1; blist[last] = b2;
            elist[maxerr] = error1; elist[last] = error2;
        } else {
            alist[maxerr] = a2; alist[last] = a1; blist[last] = b1;
            rlist[maxerr] = area2; rlist[last] = area1;
            elist[maxerr] = error2; elist[last] = error1;
        }
        /* DQPSRT: keep iord descending in error; pick the nrmax-th */
        {
            /* positions and "last" are 1-based here, as in the published
               routine; array subscripts convert with -1 */
            int L = last + 1;
            if (L <= 2) { iord[0] = 0; iord[1] = 1; }
            else {
                double em = elist[maxerr];
                int nr1 = nrmax + 1;
                if (nr1 != 1) {
                    int ido = nr1 - 1;
                    for (int i = 1; i <= ido; i++) {
                        int isucc = iord[nr1 - 2];
                        if (em <= elist[isucc]) break;
                        iord[nr1 - 1] = isucc;
                        nr1--;
                    }
                }
                int jupbn = L;
                if (L > limit / 2 + 2) jupbn = limit + 3 - L;
                double errmin = elist[L - 1];
                int jbnd = jupbn - 1, ibeg = nr1 + 1, i = ibeg, found = 0;
                if (ibeg <= jbnd) {
                    for (i = ibeg; i <= jbnd; i++) {
                        int isucc = iord[i - 1];
                        if (em >= elist[isucc]) { found = 1; break; }
                        iord[i - 2] = isucc;
                    }
                }
                if (!found) { iord[jbnd - 1] = maxerr; iord[jupbn - 1] = L - 1; }
                else {
                    iord[i - 2] = maxerr;
                    int k = jbnd, ins = 0;
                    for (int j = i; j <= jbnd; j++) {
                        int isucc = iord[k - 1];
                        if (errmin < elist[isucc]) { iord[k] = L - 1; ins = 1; break; }
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
        if (errsum <= errbnd) { done_sum = 1; break; }
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
            extrap = 1;
            nrmax = 1;
        }
        int do_ext = 1;
        if (!(ierro == 3 || erlarg <= ertest)) {
            int id = nrmax + 1, jupbnd = last + 1, found_large = 0;
            if (last + 1 > 2 + limit / 2) jupbnd = limit + 3 - (last + 1);
            for (int k = id; k <= jupbnd; k++) {
                maxerr = iord[nrmax];
                errmax = elist[maxerr];
                if (fabs(blist[maxerr] - alist[maxerr]) > small) { found_large = 1; break; }
                nrmax++;
            }
            if (found_large) do_ext = 0;
        }
        if (!do_ext) continue;
        rlist2[numrl2] = area; numrl2++;
        double reseps, abseps;
        qelg(rlist2, &numrl2, res3la, &nres, &reseps, &abseps);
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
        if (numrl2 == 1) noext = 1;
        if (ier == 5) break;
        maxerr = iord[0];
        errmax = elist[maxerr];
        nrmax = 0;
        extrap = 0;
        small *= 0.5;
        erlarg = errsum;
    }

    int take_sum = done_sum;
    if (!done_sum) {
        *result = res_ext;
        *abserr = err_ext;
        if (err_ext == DBL_MAX) take_sum = 1;
        else {
            int skip_div = 0;
            if (ier + ierro != 0) {
                if (ierro == 3) err_ext += correc;
                if (ier == 0) ier = 3;
                if (res_ext != 0.0 && area != 0.0) {
                    if (err_ext / fabs(res_ext) > errsum / fabs(area)) take_sum = 1;
                } else if (err_ext > errsum) take_sum = 1;
                else if (area == 0.0) skip_div = 1;
                *abserr = err_ext;
            }
            if (!take_sum && !skip_div) {
                double mxa = fabs(res_ext) > fabs(area) ? fabs(res_ext) : fabs(area);
                if (!(ksgn == -1 && mxa <= resabs0 * 0.01)) {
                    double ratio = res_ext / area;
                    if (ratio < 0.01 || ratio > 100.0 || errsum > fabs(area)) ier = 6;
                }
            }
        }
    }
    if (take_sum) {
        double s = 0;
        for (int k = 0; k <= last && k < limit; k++) s += rlist[k];
        *result = s;
        *abserr = errsum;
    }
    {
        int L = last + 1, b = L <= 1 ? 0 : L <= 4 ? 1 : L <= 8 ? 2 : L <= 16 ? 3 : L <= 32 ? 4 : L <= 64 ? 5 : L <= 128 ? 6 : 7;
        orc_qags_hist[b]++;
    }
    if (ier > 2) ier--;
    free(alist);
    free(iord);
    return ier;
}

int orc_qags(orc_fn f, void *p, double a, double b, double epsabs, double epsrel, int limit,
             double *result, double *abserr)
{
    return qags_core(f, p, a, b, epsabs, epsrel, limit, 21, result, abserr);
}

void orc_qags_histogram(int *out8)
{
    for (int i = 0; i < 8; i++) out8[i] = orc_qags_hist[i];
}

int orc_qagiu(orc_fn f, void *p, double a, double epsabs, double epsrel, int limit,
              double *result, double *abserr)
{
    infmap m = {f, p, a};
    return qags_core(inf_transform, &m, 0.0, 1.0, epsabs, epsrel, limit, 15, result, abserr);
}

/* ------------------------------------------------------------------------
 * Orbit integrator for the focal-distance tabulation (delta/Delta.cpp:53-90).
 * One step is the 13-stage RK8(7) pair of Prince & Dormand (orc_rk8pd.h,
 * generated from the published tableau by rk8pd_tableau.py, which checks its
 * order conditions): y1 from the 8th-order weights, the error estimate from
 * the difference of the 8th- and 7th-order weights.  The controller follows
 * the GSL manual's standard y-error control with the method's order 8.
 * ---------------------------------------------------------------------- */
static void rk8pd_step(orc_rhs rhs, void *p, double t, double h, const double *y0, double *y1, double *yerr)
{
    double k[RK8PD_STAGES][4], ys[4];
    for (int st = 0; st < RK8PD_STAGES; st++) {
        for (int i = 0; i < 4; i++) {
            double acc = 0;
            for (int j = 0; j < st; j++) acc += rk8pd_a[st][j] * k[j][i];
            ys[i] = y0[i] + h * acc;
        }
        rhs(t + rk8pd_c[st] * h, ys, k[st], p);
    }
    for (int i = 0; i < 4; i++) {
        double s8 = 0, se = 0;
        for (int st = 0; st < RK8PD_STAGES; st++) {
            s8 += rk8pd_b8[st] * k[st][i];
            se += (rk8pd_b8[st] - rk8pd_b7[st]) * k[st][i];
        }
        y1[i] = y0[i] + h * s8;
        yerr[i] = h * se;
    }
}

int orc_evolve_apply(orc_rhs rhs, void *p, double *t, double t1, double *h, double *y,
                     double epsabs, double epsrel)
{
    const double S = 0.9, ord = 8.0;
    double dt = t1 - *t, h0 = *h;
    int final = 0;
    if (h0 > dt) { h0 = dt; final = 1; }
    double y1[4], yerr[4];
    for (int tries = 0; tries < 200; tries++) {
        rk8pd_step(rhs, p, *t, h0, y, y1, yerr);
        double rmax = 0;
        for (int i = 0; i < 4; i++) {
            double D0 = epsrel * fabs(y1[i]) + epsabs;
            double r = fabs(yerr[i]) / fabs(D0);
            if (r > rmax) rmax = r;
        }
        if (rmax > 1.1 && h0 > 0) {
            double r = S / pow(rmax, 1.0 / ord);
            if (r < 0.2) r = 0.2;
            h0 *= r;
            final = 0;
            continue;
        }
        *t = final ? t1 : *t + h0;
        for (int i = 0; i < 4; i++) y[i] = y1[i];
        if (rmax < 0.5) {
            double r = S / pow(rmax, 1.0 / (ord + 1.0));
            if (r > 5.0) r = 5.0;
            if (r < 1.0) r = 1.0;
            *h = r * h0;
        } else *h = h0;
        return 0;
    }
    return 1;
}
