// fj_delta.cuh -- the focal-distance table: tabulateDelta (delta/tabulate.cpp:
// 13-38) and the Delta class (delta/Delta.cpp), as host and device code.
// Orbits use the reference's stepper, the Runge-Kutta 8(7) pair of Prince &
// Dormand (gsl_odeiv2_step_rk8pd, Delta.cpp:59-60; fj_rk8pd.h), under the
// y-error step control of its integrator setup (abs 1e-10, rel 1e-9,
// Delta.cpp:59-69).  One energy of the table is independent of the
// others (delta_energy): the host loops over them, the batched kernel gives
// each (model, energy) pair a thread.
#pragma once
#include "fj_device.cuh"
#include "fj_rk8pd.h"

namespace fj {

constexpr int kOrbSize = 200;

struct DeltaFit {
    PotView P;
    double E, Lz, Lz2, Rc, R0, D2, sqDR, v0, cv, sv, Ri, zi;  // Lz2 = pow(Lz, 2.0), once per fit
    double R[kOrbSize], z[kOrbSize];
    int N;
    bool bad;
};

FJ_HD void orbit_rhs(const DeltaFit &d, const double *y, double *f)
{
    double phi, dR, dz;
    pot_grad(d.P, y[0], y[1], phi, dR, dz);
    f[0] = y[2];
    f[1] = y[3];
    f[2] = -dR + d.Lz2 / pow(y[0], 3.0);  // Delta.cpp's pow(Lz, 2.0), taken once per fit
    f[3] = -dz;
}

FJ_HD const RK8PDTab &rk8pd_tab()
{
#ifdef __CUDA_ARCH__
    return kRK8PD_d;
#else
    return kRK8PD_h;
#endif
}

// One RK8(7) step: y1 from the 8th-order weights, yerr = h sum (b8 - b7) k
FJ_HDNI void rk8pd_step(const DeltaFit &d, double h, const double *y0, double *y1, double *yerr)
{
    const RK8PDTab &T = rk8pd_tab();
    double k[13][4], ys[4];
    for (int st = 0; st < 13; st++) {
        for (int i = 0; i < 4; i++) {
            double acc = 0;
            for (int j = 0; j < st; j++) acc += T.a[st][j] * k[j][i];
            ys[i] = y0[i] + h * acc;
        }
        orbit_rhs(d, ys, k[st]);
    }
    for (int i = 0; i < 4; i++) {
        double s8 = 0, se = 0;
        for (int st = 0; st < 13; st++) {
            s8 += T.b8[st] * k[st][i];
            se += (T.b8[st] - T.b7[st]) * k[st][i];
        }
        y1[i] = y0[i] + h * s8;
        yerr[i] = h * se;
    }
}

FJ_HDNI bool evolve_step(const DeltaFit &d, double &t, double t1, double &h, double *y)
{
    const double S = 0.9, ord = 8.0, epsabs = 1e-10, epsrel = 1e-9;
    double h0 = h;
    bool final = false;
    if (h0 > t1 - t) { h0 = t1 - t; final = true; }
    double y1[4], yerr[4];
    for (int tries = 0; tries < 200; tries++) {
        rk8pd_step(d, h0, y, y1, yerr);
        double rmax = 0;
        for (int i = 0; i < 4; i++) {
            const double D0 = epsrel * fabs(y1[i]) + epsabs;
            const double r = fabs(yerr[i]) / fabs(D0);
            if (r > rmax) rmax = r;
        }
        if (rmax > 1.1 && h0 > 0) {
            double r = S / pow(rmax, 1.0 / ord);
            if (r < 0.2) r = 0.2;
            h0 *= r;
            final = false;
            continue;
        }
        t = final ? t1 : t + h0;
        for (int i = 0; i < 4; i++) y[i] = y1[i];
        if (rmax < 0.5) {
            double r = S / pow(rmax, 1.0 / (ord + 1.0));
            if (r > 5.0) r = 5.0;
            if (r < 1.0) r = 1.0;
            h = r * h0;
        } else h = h0;
        return true;
    }
    return false;
}

FJ_HD double vsq(const DeltaFit &d, double x) { return 2 * (d.E - (pot_phi(d.P, x, 0.) + .5 * pow(d.Lz / x, 2))); }

FJ_HDNI int evolve_orbit(DeltaFit &d, double x0, int cond)
{
    double steph = 2e-3, y[4] = {x0, 0., 0., sqrt(vsq(d, x0))}, t = 0;
    int i = 0;
    d.R[0] = y[0];
    d.z[0] = y[1];
    const double t1 = 5 * x0 / sqrt(vsq(d, x0));
    while (i < kOrbSize - 1 && (cond == 0 ? y[1] >= 0. : y[3] >= 0.)) {
        if (!evolve_step(d, t, t1, steph, y)) d.bad = true;
        i++;
        d.R[i] = y[0];
        d.z[i] = y[1];
    }
    return i;
}

struct GetDRF {
    DeltaFit *d;
    __host__ __device__ double operator()(double x0) const
    {
        const int N = evolve_orbit(*d, x0, 0);
        const double *R = d->R, *z = d->z;
        if (fabs(z[N - 1] - z[N]) > 0 && fabs(R[N - 1] - R[N]) != 0)
            return x0 - (R[N] - z[N] * (R[N - 1] - R[N]) / (z[N - 1] - z[N]));
        return x0 - R[N];
    }
};

FJ_HD double dphi_eff(const DeltaFit &d, double x)
{
    double phi, dR, dz;
    pot_grad(d.P, x, 0, phi, dR, dz);
    return dR - pow(d.Lz, 2) / pow(x, 3);
}

FJ_HDNI double ensure_vsq(DeltaFit &d, double x0)
{
    int count = 0;
    while (vsq(d, x0) < 0) {
        if (dphi_eff(d, x0) < 0) x0 *= 1.1; else x0 *= .9;
        if (++count > 50) { d.bad = true; break; }
    }
    return x0;
}

FJ_HDNI double get_jr0(DeltaFit &d)
{
    GetDRF f{&d};
    double x0 = d.Rc, x1, dx0, dx1, A = .8;
    int k = 0;
    x0 = ensure_vsq(d, x0); dx0 = f(x0);
    x1 = ensure_vsq(d, x0 / A); dx1 = f(x1);
    while (dx0 * dx1 > 0) {
        if (fabs(dx1) < fabs(dx0)) { x0 = x1; dx0 = dx1; }
        else A = pow(A, -0.9);
        x1 = ensure_vsq(d, x0 * A); dx1 = f(x1);
        if (++k == 21) {
            if (fabs(dx0) < 1.e-7) return -x0;
            return -1;  // Delta.cpp:145-151 goes on with -1
        }
    }
    double r;
    if (brent_root(f, x0 < x1 ? x0 : x1, x0 < x1 ? x1 : x0, r)) d.bad = true;
    return r;
}

struct Ds2dvF {
    DeltaFit *d;
    __host__ __device__ double operator()(double v) const { return 2 * (d->zi * d->sqDR * sin(v) - cos(v) * (d->Ri * d->R0 + d->D2 * sin(v))); }
};

struct Ds2dD2F {
    DeltaFit *d;
    __host__ __device__ double operator()(double D2h) const
    {
        d->D2 = D2h;
        d->sqDR = sqrt(d->D2 + d->R0 * d->R0);
        Ds2dvF g{d};
        double sum = 0.;
        for (int i = 0; i < d->N; i++) {
            d->Ri = d->R[i];
            d->zi = d->z[i];
            const double lo = 0, hi = kPIH;
            if (fabs(g(lo)) < 1e-8) d->v0 = lo;
            else if (fabs(g(hi)) < 1e-8) d->v0 = hi;
            else if (brent_root(g, lo, hi, d->v0)) d->bad = true;
            d->sv = sin(d->v0);
            d->cv = cos(d->v0);
            const double sv = d->sv, cv = d->cv, zi = d->zi, sq = d->sqDR;
            const double dvdD2 = .5 * sv * (zi / sq - 2 * cv) / (cv * zi * sq + sv * d->Ri * d->R0 - d->D2 * (cv * cv - sv * sv));
            sum += (cv - zi / sq) * cv + g(d->v0) * dvdD2;
        }
        return sum;
    }
};

FJ_HD double get_rc_flag(const PotView &P, double Lzsq, double R, bool &bad)
{
    unsigned f = 0;
    const double r = get_rc(P, Lzsq, R, f);
    if (f) bad = true;
    return r;
}

struct RcEF {
    PotView P; double E;
    __host__ __device__ double operator()(double R) const
    {
        double phi, dR, dz;
        pot_grad(P, R, 0, phi, dR, dz);
        return .5 * R * dR + pot_phi(P, R, 0) - E;
    }
};


// The model's constants of the table (tabulate.cpp:13-38): only entries 0 and
// 1 of the reference's per-radius loop feed it -- the circular orbit of the
// second angular momentum sets the lowest energy and the speed scale.
struct DeltaBase {
    double Lz1, Rg1, Ec1, Vmax1;
    bool bad;
};

FJ_HDNI DeltaBase delta_base(const PotView &P)
{
    DeltaBase b{0, 0, 0, 0, false};
    const double *ar = P.ar;
    const int nr = P.nr;
    const double Rmax = ar[nr - 1];
    double phi, dRv, dzv;
    const double Lzmax = Rmax * 0.98 * sqrt(-2 * pot_phi(P, Rmax, 0)), Rmin = 1e-3 * Rmax;
    pot_grad(P, Rmin, 0, phi, dRv, dzv);
    const double Lzmin = Rmin * sqrt(Rmin * dRv);
    double R = .01 * Rmax;
    for (int i = 0; i < 2; i++) {
        const double Lzi = Lzmin + i * (Lzmax - Lzmin) / (double)(nr - 1);
        R = get_rc_flag(P, pow(Lzi, 2), R, b.bad);
        pot_grad(P, R, 0, phi, dRv, dzv);
        const double vc2 = R * dRv;
        const double Ec = .5 * vc2 + pot_phi(P, R, 0);
        b.Lz1 = Lzi; b.Rg1 = R; b.Ec1 = Ec; b.Vmax1 = .98 * sqrt(-2 * Ec);
    }
    return b;
}

// Entry nE of the table: its energy E and the squared focal distance of the
// best-fitting prolate coordinates of an orbit of that energy (getBestDelta,
// Delta.cpp:248-294).  d is scratch (an orbit of kOrbSize points); bad is set
// when a bracket or root search hit its cap.  The bracket of the focal
// distance widens by 0.1 per step on the negative side, as in the reference;
// some tables need thousands of steps (D^2 near -545 in an NFW table), each a
// root search per orbit point, so the cap is the caller's: the reference's
// 10^6 on the host, kDeltaWalkCapDevice on the GPU.
constexpr int kDeltaWalkCapHost = 1000000;
constexpr int kDeltaWalkCapDevice = 20000;

FJ_HDNI double delta_energy(const PotView &P, const DeltaBase &b, int nE, int ngrid, double &E, DeltaFit &d, bool &bad,
                            int walk_cap)
{
    E = b.Ec1 + .5 * pow(b.Vmax1 * (nE + 1) / (double)ngrid, 2);
    d = DeltaFit{};
    d.P = P;
    d.E = E;
    d.Lz = .25 * b.Lz1;
    d.Lz2 = pow(d.Lz, 2.0);
    // RcE (include/Utils.h:220-236)
    RcEF fe{P, d.E};
    double R0 = .8 * b.Rg1, f0 = fe(R0);
    for (int it = 0; f0 > 0 && it < kLoopCap; it++) { R0 *= .8; f0 = fe(R0); }
    double R1 = 1.2 * b.Rg1, f1 = fe(R1);
    for (int it = 0; f1 < 0 && it < kLoopCap; it++) { R1 *= 1.2; f1 = fe(R1); }
    if (brent_root(fe, R0, R1, d.Rc)) bad = true;
    d.R0 = get_jr0(d);
    d.N = evolve_orbit(d, d.R0, 1);
    Ds2dD2F g{&d};
    double lo = -0.001, hi = 5, D2out = 0;
    double Dmin = g(lo), Dmax = g(hi);
    for (int it = 0; Dmin * Dmax > 0 && fabs(Dmax) > 1e-4 && fabs(Dmin) > 1e-4; it++) {
        if (Dmax < 0) { hi *= 5; Dmax = g(hi); } else { lo -= .1; Dmin = g(lo); }
        if (it > walk_cap) { bad = true; break; }
    }
    if (fabs(g(lo)) < 1e-8) D2out = lo;
    else if (fabs(g(hi)) < 1e-8) D2out = hi;
    else if (brent_root(g, lo, hi, D2out)) bad = true;
    if (d.bad) bad = true;
    return D2out;
}

}  // namespace fj
