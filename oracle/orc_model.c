/*
 * orc_model.c -- oracle restatement of the fJmodels hot path: multipole
 * potential and its derivatives, prolate-spheroidal coordinates, Staeckel
 * fudge actions, the DF, the 3-D velocity quadrature, the Legendre
 * projection, the Poisson solve, the tensor-virial sums and the focal
 * distance table.
 *
 * TEST INFRASTRUCTURE ONLY (see fjoracle.h).  Each function names the
 * reference file:line it restates.  Unbounded loops of the reference are
 * capped here; hitting a cap counts a failure instead of hanging.
 */
#include <float.h>
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fjoracle.h"
#include "orc_internal.h"

/* reference literals (include/Utils.h:56-60) */
#define PI 3.141592653589793
#define PIH 1.570796326794897
#define TPI 6.283185307179586
#define FPI 12.56637061435917
#define TINY 1e-12
#define LOOP_CAP 100000
#define MAXP 64 /* max npoly in the oracle */

#define MAX(A, B) ((A) > (B) ? (A) : (B))

/* ---------------- grids and interpolation (include/Utils.h) ---------------- */

/* Utils.h:103-119 */
static int topbottom(const double *xm, int n, double x, int *botx, int *topx)
{
    int m, top = n - 1, bot = 0;
    if ((xm[top] - x) * (x - xm[bot]) < 0.) {
        if (fabs(xm[top] - x) < 1e-5 * fabs(x - xm[bot])) { *topx = top; *botx = top - 1; return 1; }
        else if (fabs(x - xm[bot]) < 1e-5 * fabs(x - xm[top])) { *topx = bot + 1; *botx = bot; return 1; }
        else return 0;
    }
    while (top - bot > 1) {
        m = (top + bot) / 2;
        if ((xm[top] - x) * (x - xm[m]) >= 0) bot = m; else top = m;
    }
    *topx = top; *botx = bot;
    return 1;
}

/* Utils.h:122-128 */
static double linterp(const double *xm, const double *ym, int np, double x)
{
    int top = 0, bot = 0;
    if (x <= xm[0]) return ym[0];
    if (x >= xm[np - 1]) return ym[np - 1];
    topbottom(xm, np, x, &bot, &top);
    return ym[bot] + (x - xm[bot]) / (xm[top] - xm[bot]) * (ym[top] - ym[bot]);
}

/* Utils.h:76-81 / 91-97 with an explicit (rmin, rmax) pair */
void orc_log_grid(double rmin, double rmax, int n, double *ar)
{
    for (int i = 0; i < n; i++)
        ar[i] = pow(10., log10(rmin) + (log10(rmax) - log10(rmin)) * i / (n - 1));
}

/* ---------------- Legendre polynomials (include/UtilsLeg.h) ---------------- */

/* UtilsLeg.h:43-50 */
static void legend(double *allpol, double c, int npoly)
{
    npoly++;
    allpol[0] = 1;
    if (npoly < 2) return;
    allpol[1] = c;
    for (int i = 2; i < npoly; i++)
        allpol[i] = ((2 * i - 1) * c * allpol[i - 1] - (i - 1) * allpol[i - 2]) / (double)i;
}

/* UtilsLeg.h:51-57 */
static double dlegend(double c, int n)
{
    if (n == 0) return 0;
    double allpol[2 * MAXP + 2];
    legend(allpol, c, n);
    return (n * allpol[n - 1] - n * c * allpol[n]) / (1 - c * c);
}

/* UtilsLeg.h:58-63 */
static double d2legend(double c, int n)
{
    double allpol[2 * MAXP + 2];
    legend(allpol, c, n);
    return (2 * c * dlegend(c, n) - n * (n + 1) * allpol[n]) / (1. - c * c);
}

/* UtilsLeg.h:68-79: P_0, P_2, ..., P_{2(npoly-1)} */
void orc_evenlegend(int npoly, double c, double *pol)
{
    double c2 = c * c;
    pol[0] = 1;
    if (npoly < 2) return;
    pol[1] = 1.5 * c2 - .5;
    for (int np = 2; np < npoly; np++) {
        int l = 2 * (np - 1), l2 = 2 * l;
        pol[np] = -pol[np - 2] * l * (l - 1) / (double)((l2 + 1) * (l2 - 1)) +
                  pol[np - 1] * (c2 - (l2 * l + l2 - 1) / (double)((l2 - 1) * (l2 + 3)));
        pol[np] *= (l2 + 1) * (l2 + 3) / (double)((l + 1) * (l + 2));
    }
}

/* ---------------- potential (UtilsLeg.h:96-158, Potential.cpp:206-296) ---------------- */

#define TAB(t, n, k) ((t)[(n) * m->npoly + (k)])

/* UtilsLeg.h:96-124 */
static void intpo2_phi(const orc_model *m, double r, double *phip)
{
    int nr = m->nr, npoly = m->npoly;
    const double *ar = m->ar;
    if (r >= ar[nr - 1]) {
        for (int k = 0; k < npoly; k++) phip[k] = TAB(m->phil, nr - 1, k) * pow(ar[nr - 1] / r, 2 * k + 1);
    } else {
        int top = 0, bot = 0;
        r = MAX(r, ar[0]);
        topbottom(ar, nr, r, &bot, &top);
        double db = r - ar[bot], f1 = db / (ar[top] - ar[bot]);
        for (int k = 0; k < npoly; k++) phip[k] = f1 * TAB(m->phil, top, k) + (1 - f1) * TAB(m->phil, bot, k);
        if (top < 10) {
            int thr;
            if (f1 < 0.5 && bot > 0) thr = bot - 1; else thr = top + 1;
            double dt = r - ar[top];
            double f2 = dt * db / ((ar[thr] - ar[top]) * (ar[thr] - ar[bot])),
                   f3 = (ar[thr] - ar[bot]) / (ar[top] - ar[bot]);
            for (int k = 0; k < npoly; k++)
                phip[k] += f2 * (TAB(m->phil, thr, k) - TAB(m->phil, bot, k) -
                                 f3 * (TAB(m->phil, top, k) - TAB(m->phil, bot, k)));
        }
    }
}

/* UtilsLeg.h:127-158 */
static void intpo2_all(const orc_model *m, double r, double *phip, double *dphip, double *d2phip)
{
    int nr = m->nr, npoly = m->npoly;
    const double *ar = m->ar;
    if (r >= ar[nr - 1]) {
        for (int k = 0; k < npoly; k++) {
            phip[k] = TAB(m->phil, nr - 1, k) * pow(ar[nr - 1] / r, 2 * k + 1);
            dphip[k] = -(2 * k + 1) * TAB(m->phil, nr - 1, k) * pow(ar[nr - 1] / r, 2 * k + 1) / r;
            d2phip[k] = (2 * k + 2) * (2 * k + 1) * TAB(m->phil, nr - 1, k) * pow(ar[nr - 1] / r, 2 * k + 1) / r / r;
        }
    } else {
        int top = 0, bot = 0;
        topbottom(ar, nr, r, &bot, &top);
        double db = r - ar[bot], f1 = db / (ar[top] - ar[bot]);
        for (int k = 0; k < npoly; k++) {
            phip[k] = f1 * TAB(m->phil, top, k) + (1 - f1) * TAB(m->phil, bot, k);
            dphip[k] = f1 * TAB(m->Pr, top, k) + (1 - f1) * TAB(m->Pr, bot, k);
            d2phip[k] = f1 * TAB(m->Pr2, top, k) + (1 - f1) * TAB(m->Pr2, bot, k);
        }
        if (top < 10) {
            int thr;
            if (f1 < 0.5 && bot > 0) thr = bot - 1; else thr = top + 1;
            double dt = r - ar[top];
            double f2 = dt * db / ((ar[thr] - ar[top]) * (ar[thr] - ar[bot])),
                   f3 = (ar[thr] - ar[bot]) / (ar[top] - ar[bot]);
            for (int k = 0; k < npoly; k++) {
                phip[k] += f2 * (TAB(m->phil, thr, k) - TAB(m->phil, bot, k) - f3 * (TAB(m->phil, top, k) - TAB(m->phil, bot, k)));
                dphip[k] += f2 * (TAB(m->Pr, thr, k) - TAB(m->Pr, bot, k) - f3 * (TAB(m->Pr, top, k) - TAB(m->Pr, bot, k)));
                d2phip[k] += f2 * (TAB(m->Pr2, thr, k) - TAB(m->Pr2, bot, k) - f3 * (TAB(m->Pr2, top, k) - TAB(m->Pr2, bot, k)));
            }
        }
    }
}

/* Potential.cpp:206-219 */
double orc_phi(const orc_model *m, double R, double z)
{
    double pol[MAXP], phip[MAXP];
    double c = z / sqrt(R * R + z * z), r = sqrt(R * R + z * z);
    intpo2_phi(m, r, phip);
    orc_evenlegend(m->npoly, c, pol);
    double phi = phip[0];
    for (int np = 1; np < m->npoly; np++) phi += phip[np] * pol[np];
    return phi;
}

/* Potential.cpp:224-234 */
static double pot_dr(const orc_model *m, double r, double theta, double *d2)
{
    double pol[MAXP], phip[MAXP], dphip[MAXP], d2phip[MAXP], g1 = 0, g2 = 0;
    orc_evenlegend(m->npoly, cos(theta), pol);
    intpo2_all(m, r, phip, dphip, d2phip);
    for (int np = 0; np < m->npoly; np++) { g1 += dphip[np] * pol[np]; g2 += d2phip[np] * pol[np]; }
    *d2 = g2;
    return g1;
}

/* Potential.cpp:235-244 */
static double pot_dtheta(const orc_model *m, double r, double c)
{
    double d = 0, dpol[MAXP], phinterp[MAXP];
    intpo2_phi(m, r, phinterp);
    for (int k = 0; k < m->npoly; k++) dpol[k] = dlegend(c, 2 * k);
    for (int j = 0; j < m->npoly; j++) d += phinterp[j] * dpol[j];
    d *= -sqrt(1 - c * c);
    return d;
}

/* Potential.cpp:245-255 */
static double pot_d2theta(const orc_model *m, double r, double c)
{
    double d = 0, d2pol[MAXP], phinterp[MAXP];
    intpo2_phi(m, r, phinterp);
    for (int k = 0; k < m->npoly; k++) d2pol[k] = d2legend(c, 2 * k);
    for (int j = 0; j < m->npoly; j++) d += phinterp[j] * d2pol[j];
    d *= (1 - c * c);
    d += ((pot_dtheta(m, r, c) * c) / sqrt(1 - c * c));
    return d;
}

/* Potential.cpp:261-268 */
double orc_dR(const orc_model *m, double R, double z)
{
    double r = sqrt(z * z + R * R);
    if (r < m->ar[0]) r = m->ar[0];
    double s = R / r, c = z / r;
    if (c == 1) c -= 1e-8;
    double theta = acos(c), d2;
    return pot_dtheta(m, r, c) * (c / r) + pot_dr(m, r, theta, &d2) * s;
}

/* Potential.cpp:269-276 */
double orc_dz(const orc_model *m, double R, double z)
{
    double r = sqrt(z * z + R * R);
    if (r < m->ar[0]) r = m->ar[0];
    double s = R / r, c = z / r;
    if (c == 1) c -= 1e-8;
    double theta = acos(c), d2;
    return pot_dtheta(m, r, c) * (-s / r) + pot_dr(m, r, theta, &d2) * c;
}

/* Potential.cpp:281-296 */
void orc_getfreqs(const orc_model *m, double R, double *kappa, double *nu, double *Omega)
{
    double theta = asin(1), d2;
    pot_dr(m, R, theta, &d2);
    double d2R = d2;
    double d2z = (1. / R) * pot_dr(m, R, theta, &d2) + (1. / (R * R)) * pot_d2theta(m, R, 0);
    *kappa = sqrt(d2R + 3 / R * orc_dR(m, R, 0));
    *nu = sqrt(d2z);
    *Omega = sqrt(orc_dR(m, R, 0) / R);
}

/* ---------------- prolate spheroidal coordinates (uvOrb/Uvpt.cpp) ---------------- */

typedef struct { double Delta2, u, v, shu2, sv, cv, sv2, p2, pu, pv; } orc_pt;

/* Uvpt.cpp:11-24 */
static void pt_from_Rz(double Delta, double R, double z, double pR, double pz, orc_pt *X)
{
    double Delta2 = Delta * Delta, R2 = R * R, z2 = z * z, r2 = R2 + z2;
    X->Delta2 = Delta2;
    double shu2 = .5 * (r2 - Delta2 + sqrt(pow(Delta2 - r2, 2) + 4 * Delta2 * R2)) / Delta2;
    double shu = sqrt(shu2);
    X->u = asinh(shu);
    double chu = sqrt(1 + shu2);
    double cv2 = .5 * (r2 + Delta2 - sqrt(pow(Delta2 + r2, 2) - 4 * Delta2 * z2)) / Delta2;
    double cv = z < 0 ? -sqrt(cv2) : sqrt(cv2);
    X->v = acos(cv);
    X->sv = sin(X->v);
    X->sv2 = 1 - cv2;
    X->shu2 = shu2;
    X->cv = cv;
    X->p2 = pR * pR + pz * pz;
    X->pu = Delta * (pR * chu * X->sv + pz * shu * cv);
    X->pv = Delta * (pR * shu * cv - pz * chu * X->sv);
}

/* ---------------- Staeckel fudge (uvOrb/uvOrb.cpp) ---------------- */

typedef struct {
    const orc_model *m;
    orc_stats *st;
    double Delta, u, v, E, Er, Iv, Lzsq;
    double shu2, sh1sq, ch1sq, Phiu1, sv, cv, sv2;
    double uinner, uouter, umid, vturn, ubar, Deltau;
    int fail;
} orc_uv;

static double uv_phi(orc_uv *o, double R, double z)
{
    if (o->st) o->st->phi_evals++;
    return orc_phi(o->m, R, z);
}

/* uvOrb.cpp:57-60: pt(Delta,u,v) then Phi(R,z) (Uvpt.cpp:25-35) */
static double Phiu(orc_uv *o, double u)
{
    return uv_phi(o, o->Delta * sinh(u) * sin(o->v), o->Delta * cosh(u) * cos(o->v));
}
/* uvOrb.cpp:42-45 */
static double Phiv(orc_uv *o, double v)
{
    return uv_phi(o, o->Delta * sinh(o->u) * sin(v), o->Delta * cosh(o->u) * cos(v));
}
/* uvOrb.cpp:61-63 */
static double dU(orc_uv *o, double u) { return (pow(sinh(u), 2) + o->sv2) * Phiu(o, u) - (o->sh1sq + o->sv2) * o->Phiu1; }
/* uvOrb.cpp:46-48 */
static double dV(orc_uv *o, double v) { return (1 + o->shu2) * Phiv(o, PIH) - (o->shu2 + pow(sin(v), 2)) * Phiv(o, v); }
/* uvOrb.cpp:49-52 */
static double vturnfn(double v, void *p)
{
    orc_uv *o = (orc_uv *)p;
    double sv2 = pow(sin(v), 2);
    return o->E * sv2 + o->Iv + dV(o, v) - .5 * o->Lzsq / (o->Delta * o->Delta * sv2);
}
/* uvOrb.cpp:53-56 */
static double Jvint(double psi, void *p)
{
    orc_uv *o = (orc_uv *)p;
    double v = PIH - (PIH - o->vturn) * cos(psi);
    if (o->st) o->st->quad_evals++;
    return sqrt(MAX(0., vturnfn(v, p))) * sin(psi);
}
/* uvOrb.cpp:64-69 */
static double dPhiu(orc_uv *o, double u, double *f)
{
    double R = o->Delta * sinh(u) * sin(o->v), z = o->Delta * cosh(u) * cos(o->v);
    if (o->st) o->st->grad_evals++;
    f[0] = orc_dR(o->m, R, z);
    f[1] = orc_dz(o->m, R, z);
    return uv_phi(o, R, z);
}
/* uvOrb.cpp:70-73 */
static double uturnfn(double u, void *p)
{
    orc_uv *o = (orc_uv *)p;
    double shu2 = pow(sinh(u), 2);
    return o->E * (shu2 - o->sh1sq) + o->Er * o->ch1sq - dU(o, u) -
           .5 * o->Lzsq / (o->Delta * o->Delta) * (1 / shu2 - 1 / o->sh1sq);
}
/* uvOrb.cpp:74-79 */
static double duturnfn(double u, void *p)
{
    orc_uv *o = (orc_uv *)p;
    double shu = sinh(u), chu = cosh(u), shu2 = shu * shu, f[2];
    double Phi0 = dPhiu(o, u, f);
    double dPhidu = o->Delta * (f[0] * chu * o->sv + f[1] * shu * o->cv);
    return 2 * (o->E - Phi0) * shu * chu - (shu2 + o->sv2) * dPhidu +
           o->Lzsq * chu / (o->Delta * o->Delta * shu2 * shu);
}
/* uvOrb.cpp:80-83 */
static double Juint(double psi, void *p)
{
    orc_uv *o = (orc_uv *)p;
    double u = o->ubar - o->Deltau * cos(psi);
    if (o->st) o->st->quad_evals++;
    return sqrt(MAX(0., uturnfn(u, p))) * sin(psi);
}

static double roots(orc_uv *o, double (*f)(double, void *), double lo, double hi)
{
    double r;
    long long before = orc_brent_iterations;
    if (orc_brent_wrapped(f, o, lo, hi, &r)) o->fail = 1;
    if (o->st) o->st->brent_iters += orc_brent_iterations - before;
    return r;
}

/* uvOrb.cpp:109-129 */
static void Getu0(orc_uv *o, double utry)
{
    double ui = utry, uo = utry, dut = duturnfn(utry, o);
    int it = 0;
    if (dut > 0) {
        while (dut > 0) {
            ui = utry; utry *= 1.2; dut = duturnfn(utry, o);
            if (++it > LOOP_CAP) { o->fail = 1; break; }
        }
        uo = utry;
    } else {
        while (dut < 0) {
            uo = utry; utry *= .8; dut = duturnfn(utry, o);
            if (++it > LOOP_CAP) { o->fail = 1; break; }
        }
        ui = utry;
    }
    o->umid = roots(o, duturnfn, ui, uo);
}

/* uvOrb.cpp:131-201 */
static void GetTurnu(orc_uv *o, double utry)
{
    double u1 = utry, u2 = utry;
    double ut = uturnfn(utry, o), dut = duturnfn(utry, o), eps = .1;
    int it = 0;
#define CAP() do { if (++it > LOOP_CAP) { o->fail = 1; o->uinner = o->uouter = utry; return; } } while (0)
    if (ut < 0) {
        if (dut > 0) { /* inside peri */
            o->uinner = utry;
            while (1) {
                while (ut < 0 && dut > 0) {
                    o->uinner = utry; utry *= (1 + eps);
                    ut = uturnfn(utry, o); dut = duturnfn(utry, o);
                    CAP();
                }
                if (ut >= 0) { u1 = utry; break; }
                else {
                    utry /= (1 + eps); eps *= .2;
                    if (eps < TINY) { o->uinner = o->uouter = utry; return; }
                    utry *= (1 + eps);
                    ut = uturnfn(utry, o); dut = duturnfn(utry, o);
                    CAP();
                }
            }
            while (ut > 0) { u2 = utry; utry *= 1.1; ut = uturnfn(utry, o); CAP(); }
            o->uouter = utry;
        } else { /* outside apo */
            while (1) {
                while (ut < 0 && dut < 0) {
                    o->uouter = utry; utry /= (1 + eps);
                    ut = uturnfn(utry, o); dut = duturnfn(utry, o);
                    CAP();
                }
                if (ut >= 0) { u2 = utry; break; }
                else {
                    utry *= (1 + eps); eps *= .2;
                    if (eps < TINY) { o->uinner = o->uouter = utry; return; }
                    utry /= (1 + eps);
                    ut = uturnfn(utry, o); dut = duturnfn(utry, o);
                    CAP();
                }
            }
            while (ut > 0) { u1 = utry; utry *= .9; ut = uturnfn(utry, o); CAP(); }
            o->uinner = utry;
        }
    } else { /* allowed region; the inward sweep starts from the outer point, as in the reference */
        double fu1 = ut;
        while (ut > 0) { u2 = utry; utry *= 1.1; ut = uturnfn(utry, o); CAP(); }
        o->uouter = utry;
        ut = fu1;
        while (ut > 0) { u1 = utry; utry *= .9; ut = uturnfn(utry, o); CAP(); }
        o->uinner = utry;
    }
#undef CAP
    o->uinner = roots(o, uturnfn, o->uinner, u1);
    o->uouter = roots(o, uturnfn, u2, o->uouter);
}

/* uvOrb.cpp:203-224 */
static double GetTurnv(orc_uv *o, double vtry)
{
    double vtop = vtry, vbot = vtry;
    int it = 0;
    if (vturnfn(vtry, o) < 0) {
        while (vturnfn(vbot, o) < 0) {
            vbot = .5 * (PIH + vbot);
            if (PIH - vbot < TINY) return PIH;
            if (++it > LOOP_CAP) { o->fail = 1; return PIH; }
        }
    } else {
        while (vturnfn(vtop, o) > 0) {
            vtop *= .5;
            if (vtop < TINY) return 0;
            if (++it > LOOP_CAP) { o->fail = 1; return 0; }
        }
    }
    if (!(vbot < vtop)) return roots(o, vturnfn, vtop, vbot);
    else return roots(o, vturnfn, vbot, vtop);
}

static double mom_integral(orc_uv *o, double (*f)(double, void *), double b)
{
    const orc_model *m = o->m;
    if (m->jquad <= 0) {
        double r, e;
        orc_qags(f, o, 0, b, 1e-5, 1e-3, 1000, &r, &e); /* Utils.h:173-185 */
        return r;
    }
    double x[256], w[256], s = 0;
    int n = m->jquad > 256 ? 256 : m->jquad;
    orc_gauleg(0, b, n, x, w);
    for (int i = 0; i < n; i++) s += w[i] * f(x[i], o);
    return s;
}

/* uvOrb.cpp:15-36 (bound branch) then Ju (226-245) and Jv (247-262) */
int orc_actions(const orc_model *m, double Delta, double R, double z, double Phi, double pR,
                double vphi, double pz, double *Jr, double *Jz, orc_stats *st)
{
    orc_uv o;
    memset(&o, 0, sizeof o);
    o.m = m; o.st = st; o.Delta = Delta;
    double Lz = R * vphi;
    o.Lzsq = Lz * Lz;
    orc_pt X;
    pt_from_Rz(Delta, R, z, pR, pz, &X);
    o.u = X.u; o.v = X.v; o.shu2 = X.shu2; o.sv = X.sv; o.cv = X.cv; o.sv2 = X.sv2;
    o.E = .5 * X.p2 + .5 * o.Lzsq / pow(R, 2) + Phi;
    if (o.E >= 0 || isnan(o.E)) { *Jr = *Jz = 1e31; return 0; }
    /* the pre-Getu0 evaluation of Iu/Er at u=58 is overwritten before use */
    const double us = 58;
    o.sh1sq = pow(sinh(us), 2); o.ch1sq = pow(cosh(us), 2);
    Getu0(&o, us);
    o.sh1sq = pow(sinh(o.umid), 2); o.ch1sq = pow(cosh(o.umid), 2);
    o.Phiu1 = Phiu(&o, o.umid);
    o.Er = -o.E * (X.shu2 - o.sh1sq) / o.ch1sq + .5 * pow(X.pu, 2) / (X.Delta2 * o.ch1sq) +
           .5 * o.Lzsq / (X.Delta2 * o.ch1sq) * (1 / X.shu2 - 1 / o.sh1sq) + dU(&o, X.u) / o.ch1sq;
    o.Iv = .5 * pow(X.pv, 2) / X.Delta2 - o.E * X.sv2 + .5 * o.Lzsq / (X.Delta2 * X.sv2) - dV(&o, X.v);
    const double rtwo = sqrt(2);
    /* Ju: uvOrb.cpp:226-239 */
    GetTurnu(&o, 1);
    if (fabs(o.uouter - o.uinner) < TINY) *Jr = 0;
    else {
        o.ubar = .5 * (o.uinner + o.uouter);
        o.Deltau = .5 * (o.uouter - o.uinner);
        *Jr = rtwo * Delta * o.Deltau * mom_integral(&o, Juint, PI) / PI;
    }
    /* Jv: uvOrb.cpp:247-257 */
    o.vturn = GetTurnv(&o, .5 * PIH);
    if (fabs(o.vturn - PIH) < TINY) *Jz = 0;
    else *Jz = 2 * rtwo * Delta * (PIH - o.vturn) * mom_integral(&o, Jvint, PIH) / PI;
    if (o.fail && st) st->failures++;
    return 1;
}

/* ---------------- focal distance lookup (delta/tabulate.cpp:40-44) ---------------- */
double orc_deltafn(const orc_model *m, double E)
{
    int n = m->ngrid;
    if (E < m->Egrid[0]) return sqrt(MAX(.000001, m->Dgrid[0]));
    else if (E < m->Egrid[n - 1]) return sqrt(MAX(.000001, linterp(m->Egrid, m->Dgrid, n, E)));
    else return sqrt(MAX(.000001, m->Dgrid[n - 1]));
}

/* ---------------- circular radius (include/Utils.h:190-214) ---------------- */
typedef struct { const orc_model *m; double E, Lzsq; int fail; } orc_pelz;

static double Rcfn(double R, void *p)
{
    orc_pelz *q = (orc_pelz *)p;
    return q->Lzsq / pow(R, 3) - orc_dR(q->m, R, 0);
}

static double GetRc(const orc_model *m, double Lzsq, double R, int *fail)
{
    orc_pelz par = {m, 0., Lzsq, 0};
    double Ri = R, Ro = R, dfRt = Rcfn(R, &par);
    int it = 0;
    if (dfRt > 0) {
        while (dfRt > 0) { Ri = R; R *= 1.2; dfRt = Rcfn(R, &par); if (++it > LOOP_CAP) { *fail = 1; break; } }
        Ro = R;
    } else {
        while (dfRt < 0) { Ro = R; R *= .8; dfRt = Rcfn(R, &par); if (++it > LOOP_CAP) { *fail = 1; break; } }
        Ri = R;
    }
    double r;
    if (orc_brent_wrapped(Rcfn, &par, Ri, Ro, &r)) *fail = 1;
    return r;
}

/* ---------------- DF (df/DF.cpp:65-124) ---------------- */
double orc_df(const orc_model *m, double R, double z, double Phi, const double *V, orc_stats *st)
{
    double Lz = R * V[1];
    double H = .5 * (pow(V[0], 2) + pow(V[1], 2) + pow(V[2], 2)) + Phi;
    if (H >= 0) return 0.;
    if (st) st->bound++;
    double Jr, Jz, Jphi = Lz;
    orc_actions(m, orc_deltafn(m, H), R, z, Phi, V[0], V[1], V[2], &Jr, &Jz, st);
    double DF;
    if (m->df_kind == ORC_DF_QUASIISO) {
        int fail = 0;
        double rc = GetRc(m, Jphi * Jphi, R, &fail), Omega, kappa, nu;
        orc_getfreqs(m, rc, &kappa, &nu, &Omega);
        double sigmar = exp(-rc / 2.) * 5.;
        double sigmaz = exp(-rc / 4.) * .316;
        double fr = Omega * 1e-1 * exp(-rc / 1.) / (PI * sigmar * sigmar * kappa) * (1. + tanh(Jphi / .1)) *
                    exp(-kappa * Jr / (sigmar * sigmar));
        double fz = nu / (2 * PI * sigmaz * sigmaz) * exp(-2 * Jz / (sigmaz * sigmaz));
        DF = MAX(0., fr * fz);
        if (fail && st) st->failures++;
    } else {
        double h = Jr + m->dphi_h * fabs(Jphi) + m->dz_h * Jz;
        double g = Jr + m->dphi_g * fabs(Jphi) + m->dz_g * Jz;
        double DFeven = m->mass / pow(m->J0, 3) *
                        MAX(0., pow(1. + m->J0 / h, m->alpha) / (pow(1. + g / m->J0, m->beta))) / (pow(TPI, 3.));
        if (m->chi == 0.) DF = DFeven;
        else DF = DFeven + m->k * tanh(m->chi * Jphi / m->J0) * DFeven;
    }
    if (isnan(DF)) return 0.; /* DF.cpp:105 guard, applied to both variants */
    return DF;
}

/* ---------------- moments (integ/Integ.cpp:46-62,150-163; GaussQuad.cpp:160-180) ---------------- */
double orc_rhofDF(const orc_model *m, double R, double z, double *mom6, orc_stats *st)
{
    double Phi_h = orc_phi(m, R, z);
    double rmax = m->ar[m->nr - 1];
    double Ve = sqrt(-2 * (Phi_h - orc_phi(m, 10 * rmax, 10 * rmax)));
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < m->nq; i++)
        for (int j = 0; j < m->nq; j++)
            for (int k = 0; k < m->nq; k++) {
                double V[3] = {1e-6 + Ve * m->xq[i], 1e-6 + Ve * m->xq[j], 1e-6 + Ve * m->xq[k]};
                double jacob = Ve * Ve * Ve;
                if (st) st->nodes++;
                double DF = orc_df(m, R, z, Phi_h, V, st);
                double r[6] = {jacob * DF, jacob * DF * V[1], jacob * DF * V[0] * V[0],
                               jacob * DF * V[1] * V[1], jacob * DF * V[2] * V[2], jacob * DF * V[0] * V[2]};
                double w = m->wq[i] * m->wq[j] * m->wq[k];
                for (int q = 0; q < 6; q++) s[q] += w * r[q];
            }
    mom6[0] = s[0];
    mom6[1] = s[1] / s[0];
    mom6[2] = sqrt(s[2] / s[0]);
    mom6[3] = sqrt(s[3] / s[0]);
    mom6[4] = sqrt(s[4] / s[0]);
    mom6[5] = sqrt(fabs(s[5]) / s[0]);
    return s[0];
}

/* potLeg.cpp:35-58 grid loop; grids6 is [6][nr*ngauss] */
void orc_moment_grid(const orc_model *m, int p0, int p1, double *grids6, int nthreads, orc_stats *st)
{
    int ng = m->ngauss, npts = m->nr * ng;
    double *ci = malloc(sizeof(double) * ng), *wi = malloc(sizeof(double) * ng);
    orc_gauleg(0, 1, ng, ci, wi);
    orc_stats tot;
    memset(&tot, 0, sizeof tot);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int p = p0; p < p1; p++) {
        int n = p / ng, g = p % ng;
        double si = sqrt(1 - ci[g] * ci[g]);
        orc_stats loc;
        memset(&loc, 0, sizeof loc);
        double mom[6];
        orc_rhofDF(m, m->ar[n] * si, m->ar[n] * ci[g], mom, &loc);
        for (int q = 0; q < 6; q++) grids6[q * npts + p] = mom[q];
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            tot.nodes += loc.nodes; tot.bound += loc.bound; tot.phi_evals += loc.phi_evals;
            tot.grad_evals += loc.grad_evals; tot.brent_iters += loc.brent_iters;
            tot.quad_evals += loc.quad_evals; tot.failures += loc.failures;
        }
    }
    (void)nthreads;
    if (st) {
        st->nodes += tot.nodes; st->bound += tot.bound; st->phi_evals += tot.phi_evals;
        st->grad_evals += tot.grad_evals; st->brent_iters += tot.brent_iters;
        st->quad_evals += tot.quad_evals; st->failures += tot.failures;
    }
    free(ci);
    free(wi);
}

/* potLeg.cpp:68 then UtilsLeg.h:200-253.  grids6 [6][nr*ngauss] (rho row 0
   is modified in place as the reference does), coef6 [6][nr*npoly]. */
void orc_project6(int nr, int ngauss, int npoly, const double *ar, double *grids6, double *coef6)
{
    int npts = nr * ngauss, ncoef = nr * npoly;
    double *rho = grids6;
    /* potLeg.cpp:68 */
    rho[0 * ngauss + 0] = (rho[2 * ngauss + 0] - rho[1 * ngauss + 0]) / (ar[2] - ar[1]) * (ar[0] - ar[1]) + rho[1 * ngauss + 0];
    double *ci = malloc(sizeof(double) * ngauss), *wi = malloc(sizeof(double) * ngauss);
    double *poly = malloc(sizeof(double) * npoly * ngauss), pol[MAXP];
    orc_gauleg(0, 1, ngauss, ci, wi);
    for (int g = 0; g < ngauss; g++) {
        orc_evenlegend(npoly, ci[g], pol);
        for (int np = 0; np < npoly; np++) poly[np * ngauss + g] = 2 * pol[np] * wi[g];
    }
    for (int j = 1; j < ngauss; j++) rho[j] = rho[0];
    for (int q = 0; q < 6; q++) {
        const double *Q = grids6 + q * npts;
        double *Ql = coef6 + q * ncoef;
        for (int n = 0; n < nr; n++)
            for (int np = 0; np < npoly; np++) {
                double s = 0;
                for (int g = 0; g < ngauss; g++) s += poly[np * ngauss + g] * Q[n * ngauss + g];
                Ql[n * npoly + np] = s;
            }
        Ql[0] = 2 * Q[0];
        for (int np = 1; np < npoly; np++) Ql[np] = 0;
    }
    free(ci); free(wi); free(poly);
}

/* ---------------- Poisson (pot/Potential.cpp:82-200) ---------------- */
typedef struct { int l, nr; const double *ar, *rhl_h; } orc_ipar;

static double I_internal(double x, void *p)
{
    orc_ipar *q = (orc_ipar *)p;
    return pow(x, q->l + 2) * linterp(q->ar, q->rhl_h, q->nr, x);
}
static double I_external(double x, void *p)
{
    orc_ipar *q = (orc_ipar *)p;
    double rhol;
    if (x > q->ar[q->nr - 1]) rhol = MAX(0., q->rhl_h[q->nr - 1] * pow(q->ar[q->nr - 1] / x, 4));
    else rhol = linterp(q->ar, q->rhl_h, q->nr, x);
    return rhol / pow(x, q->l - 1);
}

void orc_compute_phil(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                      double *Pr, double *Pr2)
{
    double *rhl_h = malloc(sizeof(double) * nr);
    for (int np = 0; np < npoly; np++) {
        int l = 2 * np;
        double G = 1;
        for (int i = 0; i < nr; i++) rhl_h[i] = rhl[i * npoly + np];
        for (int n = 0; n < nr; n++) {
            orc_ipar par = {l, nr, ar, rhl_h};
            double Iint, Iext, err;
            orc_qags(I_internal, &par, 0., ar[n], 1e-4, 1e-3, 1000, &Iint, &err);
            double epsabs = 1e-4, epsrel = 1e-3;
            int status = 1, tries = 0;
            while (status != 0 && tries < 60) {
                status = orc_qagiu(I_external, &par, ar[n], epsabs, epsrel, 1000, &Iext, &err);
                epsabs *= 2; epsrel *= 2; tries++;
            }
            phil[n * npoly + np] = -TPI * G * (Iint / pow(ar[n], l + 1) + Iext * pow(ar[n], l));
            Pr[n * npoly + np] = -TPI * G * (-(l + 1) * Iint / pow(ar[n], l + 2) + l * Iext * pow(ar[n], l - 1));
            Pr2[n * npoly + np] = -TPI * G * ((l + 2) * (l + 1) * Iint / pow(ar[n], l + 3) +
                                              (l - 1) * l * Iext * pow(ar[n], l - 2) - (2 * l + 1) * rhl[n * npoly + np]);
        }
    }
    free(rhl_h);
}

/* The same integrands as computeInts (pot/Potential.cpp:82-155: x^(l+2)
   linterp(rho_l) inside, linterp(rho_l) / x^(l-1) outside with the
   max(0, rho_N (R/x)^4) tail) integrated without adaptivity: each grid
   interval by a 24-point Gauss-Legendre rule (exact for the polynomial
   integrands inside; to rounding for the negative powers outside, whose
   intervals span a small ratio of radii), [0, ar[0]] the same way with
   rho = rhl[0] (linterp's clamp), the tail in closed form; running sums
   from the centre (internal) and from the tail (external). */
/* Gauss-Legendre nodes and weights on (0,1) to full double precision (Newton
   on the Legendre recurrence until the step stops shrinking; the reference's
   gauleg stops at 3e-11 with pi = 3.141592654, too coarse for this check) */
static void gauleg_full(int n, double *x, double *w)
{
    for (int i = 0; i < (n + 1) / 2; i++) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0, dz = 1;
        for (int it = 0; it < 100; it++) {
            double p1 = 1, p2 = 0;
            for (int j = 0; j < n; j++) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2 * j + 1) * z * p2 - j * p3) / (j + 1);
            }
            pp = n * (z * p1 - p2) / (z * z - 1);
            const double step = p1 / pp;
            z -= step;
            if (fabs(step) >= fabs(dz) && fabs(step) < 1e-14) break;
            dz = step;
        }
        x[i] = 0.5 * (1 - z);
        x[n - 1 - i] = 0.5 * (1 + z);
        w[i] = w[n - 1 - i] = 1 / ((1 - z * z) * pp * pp);
    }
}

void orc_compute_phil_cumulative(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                                 double *Pr, double *Pr2)
{
    enum { NGL = 24 };
    double xg[NGL], wg[NGL];
    gauleg_full(NGL, xg, wg);
    double *Iint = malloc(sizeof(double) * nr), *Iext = malloc(sizeof(double) * nr);
    for (int np = 0; np < npoly; np++) {
        const int l = 2 * np;
        double acc = 0;
        for (int k = 0; k < NGL; k++) {
            const double x = ar[0] * xg[k];
            acc += ar[0] * wg[k] * pow(x, l + 2) * rhl[np];
        }
        Iint[0] = acc;
        for (int n = 1; n < nr; n++) {
            const double a = ar[n - 1], b = ar[n], ya = rhl[(n - 1) * npoly + np], yb = rhl[n * npoly + np];
            double seg = 0;
            for (int k = 0; k < NGL; k++) {
                const double x = a + (b - a) * xg[k];
                seg += (b - a) * wg[k] * pow(x, l + 2) * (ya + (x - a) / (b - a) * (yb - ya));
            }
            acc += seg;
            Iint[n] = acc;
        }
        const double R = ar[nr - 1], yN = rhl[(nr - 1) * npoly + np];
        acc = MAX(0., yN) * pow(R, 2 - l) / (l + 2);
        Iext[nr - 1] = acc;
        for (int n = nr - 2; n >= 0; n--) {
            const double a = ar[n], b = ar[n + 1], ya = rhl[n * npoly + np], yb = rhl[(n + 1) * npoly + np];
            double seg = 0;
            for (int k = 0; k < NGL; k++) {
                const double x = a + (b - a) * xg[k];
                seg += (b - a) * wg[k] * (ya + (x - a) / (b - a) * (yb - ya)) / pow(x, l - 1);
            }
            acc += seg;
            Iext[n] = acc;
        }
        for (int n = 0; n < nr; n++) {
            const double r = ar[n], G = 1;
            phil[n * npoly + np] = -TPI * G * (Iint[n] / pow(r, l + 1) + Iext[n] * pow(r, l));
            Pr[n * npoly + np] = -TPI * G * (-(l + 1) * Iint[n] / pow(r, l + 2) + l * Iext[n] * pow(r, l - 1));
            Pr2[n * npoly + np] = -TPI * G * ((l + 2) * (l + 1) * Iint[n] / pow(r, l + 3) +
                                              (l - 1) * l * Iext[n] * pow(r, l - 2) - (2 * l + 1) * rhl[n * npoly + np]);
        }
    }
    free(Iint);
    free(Iext);
}

/* ---------------- guess densities (pot/models.cpp:40-56; Potential.cpp:63-80) ---------------- */
static double guess_rho(int kind, double mass, double r0, double q, double R, double z)
{
    double q2 = q * q, m = sqrt(R * R + z * z / q2);
    if (kind == 1) {
        double a = sqrt(r0 * r0 + m * m);
        return mass / FPI / (q * pow((a + r0) * a, 2) * a) * r0 * (r0 + 2 * a);
    }
    if (kind == 2) return mass / (m / r0 * pow(r0 + m, 2)) / FPI;
    return mass / (m / r0 * pow(r0 + m, 3)) / TPI;
}

void orc_guess_rhl(int nr, int ngauss, int npoly, const double *ar, int kind, double mass,
                   double r0, double q, double *rhl)
{
    double *ci = malloc(sizeof(double) * ngauss), *wi = malloc(sizeof(double) * ngauss), pol[MAXP];
    orc_gauleg(0, 1, ngauss, ci, wi);
    for (int n = 0; n < nr; n++)
        for (int np = 0; np < npoly; np++) rhl[n * npoly + np] = 0.;
    for (int n = 0; n < nr; n++)
        for (int np = 0; np < npoly; np++)
            for (int g = 0; g < ngauss; g++) {
                double si = sqrt(1 - ci[g] * ci[g]);
                orc_evenlegend(npoly, ci[g], pol);
                rhl[n * npoly + np] += 2 * pol[np] * wi[g] * guess_rho(kind, mass, r0, q, ar[n] * si, ar[n] * ci[g]);
            }
    double si0 = sqrt(1 - ci[0] * ci[0]);
    rhl[0] = 2 * guess_rho(kind, mass, r0, q, ar[0] * si0, ar[0] * ci[0]);
    free(ci); free(wi);
}

/* ---------------- tensor virial (libs/Stats.cpp:12-41; UtilsLeg.h:285-354) ---------------- */
void orc_vir2(const orc_model *m, const double *coef6, double *out7)
{
    int nr = m->nr, npoly = m->npoly, ng = m->ngauss, nc = nr * npoly;
    const double *ar = m->ar, *rhl = coef6, *vrotl = coef6 + nc, *sigRl = coef6 + 2 * nc,
                 *sigpl = coef6 + 3 * nc, *sigzl = coef6 + 4 * nc;
    double *ci = malloc(sizeof(double) * ng), *wi = malloc(sizeof(double) * ng);
    orc_gauleg(0, 1, ng, ci, wi);
    double pot = 0, KRR = 0, Kzz = 0, WRR = 0, Wzz = 0, pol[MAXP];
    for (int i = 1; i < nr; i++) {
        double r = .5 * (ar[i - 1] + ar[i]), dr = ar[i] - ar[i - 1];
        for (int j = 0; j < ng; j++) {
            double sij = sqrt(1 - ci[j] * ci[j]);
            double z = r * ci[j], R = r * sij;
            /* ev_dens, 5-field (UtilsLeg.h:337-354) with the float weight of int_dens (:312) */
            double c = z / sqrt(R * R + z * z), rr = sqrt(R * R + z * z);
            double densp[MAXP], Vrotp[MAXP], sigup[MAXP], sigpp[MAXP], sigvp[MAXP];
            densp[0] = Vrotp[0] = sigup[0] = sigpp[0] = sigvp[0] = 0; /* npoly >= 1 overwrites */
            orc_evenlegend(npoly, c, pol);
            if (rr > ar[nr - 1]) {
                for (int k = 0; k < npoly; k++) densp[k] = Vrotp[k] = sigup[k] = sigpp[k] = sigvp[k] = 0;
            } else {
                int top = 0, bot = 0;
                topbottom(ar, nr, rr, &bot, &top);
                float f = (float)((rr - ar[bot]) / (ar[top] - ar[bot]));
                float omf = 1 - f;
                for (int k = 0; k < npoly; k++) {
                    densp[k] = f * rhl[top * npoly + k] + omf * rhl[bot * npoly + k];
                    sigup[k] = f * sigRl[top * npoly + k] + omf * sigRl[bot * npoly + k];
                    sigpp[k] = f * sigpl[top * npoly + k] + omf * sigpl[bot * npoly + k];
                    sigvp[k] = f * sigzl[top * npoly + k] + omf * sigzl[bot * npoly + k];
                    Vrotp[k] = f * vrotl[top * npoly + k] + omf * vrotl[bot * npoly + k];
                }
            }
            double dens = .5 * densp[0], Sigu = .5 * sigup[0], Sigp = .5 * sigpp[0], Sigv = .5 * sigvp[0];
            for (int np = 1; np < npoly; np++) {
                double fac = .5 * (4 * np + 1);
                dens += fac * densp[np] * pol[np];
                Sigu += fac * sigup[np] * pol[np];
                Sigp += fac * sigpp[np] * pol[np];
                Sigv += fac * sigvp[np] * pol[np];
            }
            pot += .5 * wi[j] * dens * orc_phi(m, R, z) * r * r * dr;
            KRR += .5 * wi[j] * dens * (pow(r * Sigu, 2) + pow(r * Sigp, 2)) * dr;
            Kzz += .5 * wi[j] * dens * pow(r * Sigv, 2) * dr;
            WRR -= wi[j] * dens * R * orc_dR(m, R, z) * r * r * dr;
            Wzz -= wi[j] * dens * z * orc_dz(m, R, z) * r * r * dr;
        }
    }
    KRR *= 4 * PI; Kzz *= 4 * PI; WRR *= 4 * PI; Wzz *= 4 * PI; pot *= 4 * PI;
    /* mass check (Stats.cpp:35-37): ev_dens(ar[i],0), 1-field with a double weight */
    double sum = 0.;
    for (int i = 0; i < nr; i++) {
        orc_evenlegend(npoly, 0.0, pol);
        int top = 0, bot = 0;
        topbottom(ar, nr, ar[i], &bot, &top);
        double f = (ar[i] - ar[bot]) / (ar[top] - ar[bot]);
        double dens = .5 * (f * rhl[top * npoly] + (1 - f) * rhl[bot * npoly]);
        for (int np = 1; np < npoly; np++)
            dens += .5 * (4 * np + 1) * (f * rhl[top * npoly + np] + (1 - f) * rhl[bot * npoly + np]) * pol[np];
        sum += 2 * TPI * ar[i] * ar[i] * dens;
    }
    out7[0] = KRR; out7[1] = Kzz; out7[2] = WRR; out7[3] = Wzz; out7[4] = pot;
    out7[5] = pow(ar[nr - 1], 2) * m->Pr[(nr - 1) * npoly + 0];
    out7[6] = sum;
    free(ci); free(wi);
}

/* UtilsLeg.h:266-278 (distance part only) */
double orc_merge_distance(int nr, int npoly, const double *phil_new, const double *phil_old)
{
    double maxd = 0;
    for (int i = 0; i < nr; i++)
        for (int j = 0; j < npoly; j++) {
            double d = fabs((phil_new[i * npoly + j] - phil_old[i * npoly + j]) / phil_new[i * npoly]);
            if (d > maxd) maxd = d;
        }
    return maxd;
}

/* ---------------- focal-distance tabulation (delta/tabulate.cpp:13-38, delta/Delta.cpp) ---------------- */
#define ORB_SIZE 200

typedef struct {
    const orc_model *m;
    double E, Lz, Rc, R0;
    double D2, sqDR, v0, cv, sv, Ri, zi;
    double R[ORB_SIZE], z[ORB_SIZE];
    int N, fail;
} orc_delta;

static void eqs_motion(double t, const double *y, double *f, void *p)
{
    orc_delta *d = (orc_delta *)p;
    (void)t;
    f[0] = y[2];
    f[1] = y[3];
    f[2] = -orc_dR(d->m, y[0], y[1]) + pow(d->Lz, 2.0) / pow(y[0], 3.0);
    f[3] = -orc_dz(d->m, y[0], y[1]);
}

static double vsq(orc_delta *d, double x) { return 2 * (d->E - (orc_phi(d->m, x, 0.) + .5 * pow(d->Lz / x, 2))); }

/* Delta.cpp:53-90; cond 0: z>=0, 1: pz>=0 */
static int evolve_orbit(orc_delta *d, double x0, int cond)
{
    double steph = 2e-3, y[4], t = 0;
    y[0] = x0; y[1] = 0.; y[2] = 0.; y[3] = sqrt(vsq(d, x0));
    int i = 0;
    d->R[0] = y[0]; d->z[0] = y[1];
    double t1 = 5 * x0 / sqrt(vsq(d, x0));
    while (i < ORB_SIZE - 1 && (cond == 0 ? y[1] >= 0. : y[3] >= 0.)) {
        if (orc_evolve_apply(eqs_motion, d, &t, t1, &steph, y, 1e-10, 1e-9)) d->fail = 1;
        i++;
        d->R[i] = y[0]; d->z[i] = y[1];
    }
    return i;
}

/* Delta.cpp:93-104 */
static double getDR(double x0, void *p)
{
    orc_delta *d = (orc_delta *)p;
    int N = evolve_orbit(d, x0, 0);
    double *R = d->R, *z = d->z;
    if (fabs(z[N - 1] - z[N]) > 0 && fabs(R[N - 1] - R[N]) != 0)
        return x0 - (R[N] - z[N] * (R[N - 1] - R[N]) / (z[N - 1] - z[N]));
    return x0 - R[N];
}

static double dPhiEff(orc_delta *d, double x) { return orc_dR(d->m, x, 0) - pow(d->Lz, 2) / pow(x, 3); }

/* Delta.cpp:116-124 */
static double ensureVsq(orc_delta *d, double x0)
{
    int count = 0;
    while (vsq(d, x0) < 0) {
        if (dPhiEff(d, x0) < 0) x0 *= 1.1; else x0 *= .9;
        if (++count > 50) { d->fail = 1; break; }
    }
    return x0;
}

/* Delta.cpp:129-164 */
static double getJr0(orc_delta *d)
{
    double x0 = d->Rc, x1, dx0, dx1, A = .8;
    int k = 0;
    x0 = ensureVsq(d, x0); dx0 = getDR(x0, d);
    x1 = ensureVsq(d, x0 / A); dx1 = getDR(x1, d);
    while (dx0 * dx1 > 0) {
        if (fabs(dx1) < fabs(dx0)) { x0 = x1; dx0 = dx1; }
        else A = pow(A, -0.9);
        x1 = ensureVsq(d, x0 * A); dx1 = getDR(x1, d);
        k++;
        if (k == 21) {
            if (fabs(dx0) < 1.e-7) return -x0;
            return -1; /* the reference reports "problem in get_closed()" and goes on with -1 */
        }
    }
    double lo = x0 < x1 ? x0 : x1, hi = x0 < x1 ? x1 : x0, r;
    if (orc_brent_wrapped(getDR, d, lo, hi, &r)) d->fail = 1;
    return r;
}

/* Delta.cpp:170-172 */
static double ds2dv(double v, void *p)
{
    orc_delta *d = (orc_delta *)p;
    return 2 * (d->zi * d->sqDR * sin(v) - cos(v) * (d->Ri * d->R0 + d->D2 * sin(v)));
}

/* Delta.cpp:189-208 */
static void getv(orc_delta *d)
{
    double lo = 0, hi = PIH;
    if (fabs(ds2dv(lo, d)) < 1e-8) d->v0 = lo;
    else if (fabs(ds2dv(hi, d)) < 1e-8) d->v0 = hi;
    else if (orc_brent_wrapped(ds2dv, d, lo, hi, &d->v0)) d->fail = 1;
    d->sv = sin(d->v0); d->cv = cos(d->v0);
}

/* Delta.cpp:210-234 */
static double ds2dD2TOT(double D2h, void *p)
{
    orc_delta *d = (orc_delta *)p;
    d->D2 = D2h; d->sqDR = sqrt(d->D2 + d->R0 * d->R0);
    double sum = 0.;
    for (int i = 0; i < d->N; i++) {
        d->Ri = d->R[i]; d->zi = d->z[i];
        getv(d);
        double sv = d->sv, cv = d->cv, zi = d->zi, sqDR = d->sqDR;
        double dvdD2 = .5 * sv * (zi / sqDR - 2 * cv) / (cv * zi * sqDR + sv * d->Ri * d->R0 - d->D2 * (cv * cv - sv * sv));
        sum += (cv - zi / sqDR) * cv + ds2dv(d->v0, d) * dvdD2;
    }
    return sum;
}

static double RcEfn(double R, void *p)
{
    orc_pelz *q = (orc_pelz *)p;
    return .5 * R * orc_dR(q->m, R, 0) + orc_phi(q->m, R, 0) - q->E;
}

/* Utils.h:220-236 */
static double RcE(const orc_model *m, double E, double Rc, int *fail)
{
    orc_pelz par = {m, E, 0., 0};
    double R0 = .8 * Rc, f0 = RcEfn(R0, &par);
    int it = 0;
    while (f0 > 0) { R0 *= .8; f0 = RcEfn(R0, &par); if (++it > LOOP_CAP) { *fail = 1; break; } }
    double R1 = 1.2 * Rc, f1 = RcEfn(R1, &par);
    it = 0;
    while (f1 < 0) { R1 *= 1.2; f1 = RcEfn(R1, &par); if (++it > LOOP_CAP) { *fail = 1; break; } }
    double r;
    if (orc_brent_wrapped(RcEfn, &par, R0, R1, &r)) *fail = 1;
    return r;
}

/* Delta.cpp:248-294 (returns D^2) */
static double getBestDelta(orc_delta *d)
{
    d->R0 = getJr0(d);
    d->N = evolve_orbit(d, d->R0, 1);
    double lo = -0.001, hi = 5, D2out = 0;
    double Dmin = ds2dD2TOT(lo, d), Dmax = ds2dD2TOT(hi, d);
    int it = 0;
    while (Dmin * Dmax > 0 && fabs(Dmax) > 1e-4 && fabs(Dmin) > 1e-4) {
        if (Dmax < 0) { hi *= 5; Dmax = ds2dD2TOT(hi, d); }
        else { lo -= .1; Dmin = ds2dD2TOT(lo, d); }
        if (++it > 1000000) { d->fail = 1; break; }
    }
    if (fabs(ds2dD2TOT(lo, d)) < 1e-8) D2out = lo;
    else if (fabs(ds2dD2TOT(hi, d)) < 1e-8) D2out = hi;
    else if (orc_brent_wrapped(ds2dD2TOT, d, lo, hi, &D2out)) d->fail = 1;
    return D2out;
}

int orc_tabulate_delta(const orc_model *m, double *Egrid, double *Dgrid)
{
    int nr = m->nr, fail = 0;
    const double *ar = m->ar;
    double Rmax = ar[nr - 1];
    double Lzmax = Rmax * 0.98 * sqrt(-2 * orc_phi(m, Rmax, 0)), Rmin = 1e-3 * Rmax;
    double Lzmin = Rmin * sqrt(Rmin * orc_dR(m, Rmin, 0)), R = .01 * Rmax;
    /* only entries 0 and 1 of the reference's per-radius loop feed the table */
    double Lz1 = 0, Rg1 = 0, Ec1 = 0, Vmax1 = 0;
    for (int i = 0; i < 2; i++) {
        double Lzi = Lzmin + i * (Lzmax - Lzmin) / (double)(nr - 1);
        double Lzsq = pow(Lzi, 2);
        R = GetRc(m, Lzsq, R, &fail);
        double vc2 = R * orc_dR(m, R, 0);
        double Ec = .5 * vc2 + orc_phi(m, R, 0);
        Lz1 = Lzi; Rg1 = R; Ec1 = Ec; Vmax1 = .98 * sqrt(-2 * Ec);
    }
    orc_delta *d = malloc(sizeof(orc_delta));
    for (int nE = 0; nE < m->ngrid; nE++) {
        Egrid[nE] = Ec1 + .5 * pow(Vmax1 * (nE + 1) / (double)m->ngrid, 2);
        memset(d, 0, sizeof *d);
        d->m = m; d->E = Egrid[nE]; d->Lz = .25 * Lz1;
        d->Rc = RcE(m, d->E, Rg1, &fail);
        Dgrid[nE] = getBestDelta(d);
        if (d->fail) fail = 1;
    }
    free(d);
    return fail;
}

/* ---------------- projected density, line profile, velocity distributions ---------------- */
/* The 22-point tanh-sinh rule on [0,1] tabulated in include/GaussPts.h:91-134 (xpt01/xw01):
   x_k = (1 + tanh(pi/2 sinh(k h)))/2, w_k = h pi/4 cosh(k h) / cosh^2(pi/2 sinh(k h)),
   h = 2/11, k = -11..10, each printed to 12 significant digits. */
void orc_tanh_sinh01(double *x, double *w)
{
    const double h = 2. / 11.;
    for (int i = 0; i < 22; i++) {
        const double t = (i - 11) * h, u = PI / 2 * sinh(t);
        char buf[32];
        snprintf(buf, sizeof buf, "%.12g", .5 * (1 + tanh(u)));
        x[i] = strtod(buf, NULL);
        snprintf(buf, sizeof buf, "%.12g", h * PI / 4 * cosh(t) / pow(cosh(u), 2));
        w[i] = strtod(buf, NULL);
    }
}

/* ev_dens, 1-field (include/UtilsLeg.h:285-298, 323-334): density from the multipoles rhl */
static double ev_dens1(const orc_model *m, const double *rhl, double R, double z)
{
    const int nr = m->nr, np = m->npoly;
    double pol[64], densp[64] = {0};
    const double c = z / sqrt(R * R + z * z), r = sqrt(R * R + z * z);
    orc_evenlegend(np, c, pol);
    if (r > m->ar[nr - 1]) {
        for (int i = 0; i < np; i++) densp[i] = 0;
    } else {
        int top, bot;
        topbottom(m->ar, nr, r, &bot, &top);
        const double f = (r - m->ar[bot]) / (m->ar[top] - m->ar[bot]);
        for (int i = 0; i < np; i++) densp[i] = f * rhl[top * np + i] + (1 - f) * rhl[bot * np + i];
    }
    double dens = .5 * densp[0];
    for (int l = 1; l < np; l++) dens += .5 * (4 * l + 1) * densp[l] * pol[l];
    return dens;
}

/* SigmaDF (Integ.cpp:168-172) with SigmaInteg (:32-43) on the [0,1] rule */
static double sigma_df(const orc_model *m, const double *rhl, double R, double z, const double *x01,
                       const double *w01)
{
    const double rmax = m->ar[m->nr - 1], jac = rmax - R;
    double s = 0;
    for (int i = 0; i < 22; i++) s += w01[i] * (jac * ev_dens1(m, rhl, R + x01[i] * jac, z));
    return 2 * s;
}

double orc_los(const orc_model *m, const double *rhl, int kind, double R, double z, double v,
               const double *x01, const double *w01, orc_stats *st)
{
    if (kind == ORC_LOS_SIGMA) return sigma_df(m, rhl, R, z, x01, w01);
    const double rmax = m->ar[m->nr - 1];
    const double Phi = orc_phi(m, R, z), Ve = sqrt(-2 * (Phi - orc_phi(m, 10 * rmax, 10 * rmax)));
    const int nq = m->nq;
    const double *x11 = m->xq, *w11 = m->wq;
    double sum = 0;
    if (kind == ORC_LOS_LINE) {  /* Int3D_111111 of lineProfile (Integ.cpp:63-92, 177-186) */
        for (int i = 0; i < nq; i++)
            for (int j = 0; j < nq; j++)
                for (int k = 0; k < nq; k++) {
                    const double vy = x11[i], x = x11[j], vz = x11[k];
                    const double Rp = sqrt(pow(R, 2) + pow(x * rmax, 2)), y = R;
                    const double vabs = sqrt(v * v + vy * vy);
                    const double alpha = acos(v / vabs), theta = atan2(y, x);
                    const double vr = vabs * cos(alpha + theta), vphi = vabs * sin(alpha + theta);
                    const double V[3] = {1e-6 + Ve * vr, 1e-6 + Ve * vphi, 1e-6 + Ve * vz};
                    const double jacob = Ve * Ve * (fabs(x) * pow(rmax, 2)) / Rp;
                    sum += w11[i] * w11[j] * w11[k] * (jacob * orc_df(m, R, z, Phi, V, st));
                }
        return sum / sigma_df(m, rhl, R, z, x01, w01);
    }
    if (kind == ORC_LOS_PVPHI) {  /* Int2D_0101 of Pvphi (Integ.cpp:97-109, 191-198) */
        for (int i = 0; i < 22; i++)
            for (int j = 0; j < 22; j++) {
                const double V[3] = {1e-6 + Ve * x01[i], v, 1e-6 + Ve * x01[j]};
                sum += w01[i] * w01[j] * (Ve * Ve * orc_df(m, R, z, Phi, V, st));
            }
        return sum;
    }
    /* Int2D_0111 of Pvz / Pvr (Integ.cpp:110-135, 202-220) */
    for (int i = 0; i < 22; i++)
        for (int j = 0; j < nq; j++) {
            double V[3];
            if (kind == ORC_LOS_PVZ) { V[0] = 1e-6 + Ve * x01[i]; V[1] = 1e-6 + Ve * x11[j]; V[2] = v; }
            else { V[0] = v; V[1] = 1e-6 + Ve * x11[j]; V[2] = 1e-6 + Ve * x01[i]; }
            sum += w01[i] * w11[j] * (Ve * Ve * orc_df(m, R, z, Phi, V, st));
        }
    return sum;
}
