// fj_mixed_wave.cuh -- the mixed-precision node solve as a resumable state
// machine ("wavefront" form).
//
// mixed_node_df (fj_mixed.cuh) runs one node's solve as nested loops: the u
// bracket walk, two Brent roots, QAGS for Ju, the v walk, Brent, QAGS for Jv.
// In a warp each lane is somewhere else in that nest, so the lanes that need
// a potential difference reach fudge_eval from different call sites and the
// warp issues the evaluation once per distinct site.  Here the same steps are
// restated as a state machine that consumes one function value and returns
// the next (mode, x) it needs; the kernel loop then evaluates every lane's
// request at one call site each step, and only the bookkeeping between
// evaluations diverges.  The arithmetic and its order are those of
// mixed_node_df: a lane produces the same values bit for bit.
#pragma once

#include "fj_mixed.cuh"

namespace fj {

// Brent root of the wrapper's rule (brent_root_f) one function value at a time.
struct BrentSM {
    float lo, hi, flo;
    float a, fa, b, fb, c, fc, d, e, xr, xlo, xhi;
    int it, stage;  // 0: wants f(lo), 1: wants f(hi), 2: wants f(b)
    FJ_HD float start(float lo_, float hi_)
    {
        lo = lo_; hi = hi_; stage = 0; it = 0;
        return lo;
    }
    // Feeds f at the requested point.  Returns true with the root in xr, or
    // false with the next point in x.
    FJ_HD bool feed(float f, float &x, unsigned &fail)
    {
        if (stage == 0) {
            if (fabsf(f) < 5e-4f) { xr = lo; return true; }
            flo = f; stage = 1; x = hi;
            return false;
        }
        if (stage == 1) {
            if (fabsf(f) < 5e-4f) { xr = hi; return true; }
            a = lo; fa = flo; b = hi; fb = f; c = hi; fc = f; d = hi - lo; e = hi - lo;
            xr = 0.5f * (lo + hi); xlo = lo; xhi = hi;
            stage = 2;
            it = 0;
            return iterate(x, fail);
        }
        // the value at the b of iteration `it`: finish that iteration
        fb = f;
        xr = b;
        const float cc = ((fb < 0 && fc < 0) || (fb > 0 && fc > 0)) ? a : c;
        xlo = fminf(b, cc);
        xhi = fmaxf(b, cc);
        if (converged()) return true;
        if (++it >= kRootMaxIt) { fail |= kFailRoot; return true; }
        return iterate(x, fail);
    }
    FJ_HD bool converged() const
    {
        const float alo = fabsf(xlo), ahi = fabsf(xhi);
        const float mn = ((xlo > 0 && xhi > 0) || (xlo < 0 && xhi < 0)) ? fminf(alo, ahi) : 0.f;
        const float abstol = fmaxf(1e-8f, 4.f * FLT_EPSILON * fmaxf(alo, ahi));
        return fabsf(xhi - xlo) < abstol + 1e-6f * mn && !(xhi - xlo > abstol);
    }
    // Runs iterations `it`, it+1, ... until one needs a function value (false,
    // x = that point) or the search ends (true).
    FJ_HD bool iterate(float &x, unsigned &fail)
    {
        for (;;) {
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
                x = b;
                return false;
            }
            if (converged()) return true;
            if (++it >= kRootMaxIt) { fail |= kFailRoot; return true; }
        }
    }
};

// QAGS (qags_f) one function value at a time: Gauss-Kronrod panels are filled
// node by node in gk21_f's order, the DQAGSE bookkeeping runs between panels.
struct QagsSM {
    float A, Bnd, epsabs, epsrel;
    // panel being filled
    float pa, pb, center, half, fc, rg, rk, ra, fv1[11], fv2[11];
    int j, stage;  // stage 0: first panel, 1: left half, 2: right half
    // DQAGSE state
    float alist[kQagsCapF], blist[kQagsCapF], rlist[kQagsCapF], elist[kQagsCapF];
    int iord[kQagsCapF];
    float rlist2[52], res3la[3];
    int nres, numrl2, maxerr, nrmax, last, ier, ktmin, ierro, iroff1, iroff2, iroff3;
    float area, errsum, errmax, res_ext, err_ext, correc, ertest, erlarg, small;
    float a1, b1, a2, b2, erlast, area1, error1, rasc1;
    bool extrap, noext;
    float result;

    // node n of the panel in gk21_f's order: 0 = centre, then the Gauss nodes
    // (jj = 1, 3, .., 9) and the Kronrod nodes (jj = 0, 2, .., 8), each pair
    // centre - x, centre + x
    FJ_HD float node_x(const GK21f &K, int n) const
    {
        if (n == 0) return center;
        const int k = (n - 1) >> 1, jj = k < 5 ? 2 * k + 1 : 2 * (k - 5);
        const float x = half * K.xgk[jj];
        return (n & 1) ? center - x : center + x;
    }
    FJ_HD float begin_panel(const GK21f &K, float a_, float b_)
    {
        pa = a_; pb = b_;
        center = 0.5f * (a_ + b_);
        half = 0.5f * (b_ - a_);
        j = 0;
        return node_x(K, 0);
    }
    // accumulates one panel value; true when the panel is complete
    FJ_HD bool panel_feed(const GK21f &K, float f)
    {
        if (j == 0) {
            fc = f; rg = 0; rk = f * K.wgk[10]; ra = fabsf(rk);
        } else {
            const int k = (j - 1) >> 1, jj = k < 5 ? 2 * k + 1 : 2 * (k - 5);
            if (j & 1) fv1[jj] = f;
            else {
                fv2[jj] = f;
                const float f1 = fv1[jj], f2 = f;
                if (k < 5) rg += K.wg[k] * (f1 + f2);
                rk += K.wgk[jj] * (f1 + f2);
                ra += K.wgk[jj] * (fabsf(f1) + fabsf(f2));
            }
        }
        return ++j == 21;
    }
    FJ_HD void panel_result(const GK21f &K, float &res, float &abserr, float &resabs, float &resasc) const
    {
        const float mean = 0.5f * rk;
        float rasc = K.wgk[10] * fabsf(fc - mean);
        for (int q = 0; q < 10; q++) rasc += K.wgk[q] * (fabsf(fv1[q] - mean) + fabsf(fv2[q] - mean));
        const float ahalf = fabsf(half);
        const float err = (rk - rg) * half;
        res = rk * half;
        resabs = ra * ahalf;
        resasc = rasc * ahalf;
        abserr = rescale_err_f(err, resabs, resasc);
    }

    FJ_HD float start(const GK21f &K, float a_, float b_, float epsabs_, float epsrel_)
    {
        A = a_; Bnd = b_; epsabs = epsabs_; epsrel = epsrel_;
        stage = 0;
        return begin_panel(K, a_, b_);
    }
    // Feeds the value at the requested point; true with the integral in
    // result, or false with the next point in x.
    FJ_HD bool feed(const GK21f &K, float f, float &x, unsigned &fail)
    {
        if (!panel_feed(K, f)) { x = node_x(K, j); return false; }
        float res, err, resabs, resasc;
        panel_result(K, res, err, resabs, resasc);
        if (stage == 0) {
            const float tol = fmaxf(epsabs, epsrel * fabsf(res));
            if (err <= 100 * FLT_EPSILON * resabs && err > tol) { result = res; return true; }
            if ((err <= tol && err != resasc) || err == 0.0f) { result = res; return true; }
            nres = 0; numrl2 = 1;
            alist[0] = A; blist[0] = Bnd; rlist[0] = res; elist[0] = err; iord[0] = 0;
            rlist2[0] = res;
            area = res; errsum = err; errmax = err;
            maxerr = 0; nrmax = 0; ier = 0;
            res_ext = res; err_ext = FLT_MAX; correc = 0; ertest = 0; erlarg = 0; small = 0;
            ktmin = 0; ierro = 0; iroff1 = 0; iroff2 = 0; iroff3 = 0;
            extrap = false; noext = false;
            last = 1;
            return next_bisection(K, x, fail);
        }
        if (stage == 1) {
            area1 = res; error1 = err; rasc1 = resasc;
            (void)resabs;
            stage = 2;
            x = begin_panel(K, a2, b2);
            return false;
        }
        // stage 2: the right half is complete, the DQAGSE step of qags_f
        const float area2 = res, error2 = err, rasc2 = resasc;
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
                    for (int jq = i; jq <= jbnd; jq++) {
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
        if (errsum <= errbnd) return finish(true);
        if (ier) return finish(false);
        if (last == 1) {
            small = fabsf(Bnd - A) * 0.375f;
            erlarg = errsum;
            ertest = errbnd;
            rlist2[1] = area; numrl2 = 2;
            last++;
            return next_bisection(K, x, fail);
        }
        if (noext) { last++; return next_bisection(K, x, fail); }
        erlarg -= erlast;
        if (fabsf(b1 - a1) > small) erlarg += erro12;
        if (!extrap) {
            if (fabsf(blist[maxerr] - alist[maxerr]) > small) { last++; return next_bisection(K, x, fail); }
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
        if (!do_ext) { last++; return next_bisection(K, x, fail); }
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
            if (err_ext <= ertest) return finish(false);
        }
        if (numrl2 == 1) noext = true;
        if (ier == 5) return finish(false);
        maxerr = iord[0];
        errmax = elist[maxerr];
        nrmax = 0;
        extrap = false;
        small *= 0.5f;
        erlarg = errsum;
        last++;
        return next_bisection(K, x, fail);
    }
    // top of qags_f's bisection loop for the current `last`
    FJ_HD bool next_bisection(const GK21f &K, float &x, unsigned &fail)
    {
        static_assert(kQagsCapF < 1000, "the interval cap ends the bisection before DQAGSE's limit");
        if (last >= kQagsCapF) { fail |= kFailQuad; last = kQagsCapF - 1; return finish(true); }
        a1 = alist[maxerr]; b1 = 0.5f * (alist[maxerr] + blist[maxerr]);
        a2 = b1; b2 = blist[maxerr];
        erlast = errmax;
        stage = 1;
        x = begin_panel(K, a1, b1);
        return false;
    }
    // the end of qags_f: the extrapolated result or the sum of the panels
    FJ_HD bool finish(bool done_sum)
    {
        bool take_sum = done_sum;
        result = res_ext;
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
        return true;
    }
};

// One node of the mixed form (mixed_node_df) as a state machine.
struct MixedLane {
    enum : int { kIdle = 0, kWalkU, kBrentUin, kBrentUout, kQagsU, kWalkVeq, kWalkVpole, kBrentVeq, kBrentVpole,
                 kQagsV, kDone };
    FudgeF o;
    double Lz, Delta, E, u, v, shu2, sv, cv, sv2, pu, pv;  // FP64 node state (fallback, DF)
    double utry, u1, u2, uin, uout, eps;                  // u walk (FP64 positions)
    float ut, dut, fu1, wbot, vtop, tin, tout, wt;
    double Jr, Jz;
    unsigned fail, esc;
    int phase, wstage, it;
    bool have64;
    int mode;     // request: fudge_eval(o, mode, x)
    float x;
    bool want_du; // and fudge_du(o, xdu) alongside
    float xdu;
    BrentSM br;
    QagsSM qs;

    // Node setup (mixed_node_df up to the u walk's first request); returns
    // false when the node is unbound (E >= 0: Jr = Jz = 1e31, no request).
    FJ_HD bool begin(const PotViewF &PF, double Delta_, double R, double z, double Phi_h, double V0, double V1,
                     double V2)
    {
        Delta = Delta_;
        Lz = R * V1;
        const double Lzsq = Lz * Lz;
        const double D2 = Delta * Delta, R2 = R * R, z2 = z * z, r2 = R2 + z2;
        const double dmr = D2 - r2, dpr = D2 + r2;
        shu2 = .5 * (r2 - D2 + sqrt(dmr * dmr + 4 * D2 * R2)) / D2;
        const double shu = sqrt(shu2), chu = sqrt(1 + shu2);
        u = asinh(shu);
        const double cv2 = .5 * (r2 + D2 - sqrt(dpr * dpr - 4 * D2 * z2)) / D2;
        cv = z < 0 ? -sqrt(cv2) : sqrt(cv2);
        v = acos(cv);
        sv = sin(v);
        sv2 = 1 - cv2;
        pu = Delta * (V0 * chu * sv + V2 * shu * cv);
        pv = Delta * (V0 * shu * cv - V2 * chu * sv);
        E = .5 * (V0 * V0 + V2 * V2) + .5 * Lzsq / R2 + Phi_h;
        fail = 0; esc = 0; have64 = false;
        Jr = 1e31; Jz = 1e31;
        if (E >= 0 || isnan(E)) { phase = kDone; return false; }
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
        o.c2pt = (float)((1 + shu2) * cv2 / (shu2 + cv2));
        o.Phipt = pot_phi_f(PF, o.Delta * o.sinhu * o.sinv, o.Delta * o.coshu * o.cosv);
        // get_turn_u_f: ut = U(utry), dut = dU(utry) at utry = 1
        utry = 1.0; u1 = u2 = uin = uout = utry; eps = .1; it = 0;
        phase = kWalkU; wstage = 0;
        request_u(utry, true);
        return true;
    }
    FJ_HD void request_u(double at, bool du)
    {
        mode = kEvU; x = (float)(at - o.u_pt); want_du = du; xdu = (float)at;
    }

    // FP64 solves for the turning points at the limits (the same calls as mixed_node_df)
    FJ_HD void fallback_u(const PotView &P)
    {
        Fudge o64;
        fudge64_at_point(o64, P, Delta, Lz * Lz, E, u, v, shu2, sv, cv, sv2, pu, pv);
        have64 = true;
        get_turn_u(o64, 1);
        fail |= o64.fail;
        tin = (float)(o64.uinner - u); tout = (float)(o64.uouter - u);
        esc = 1u;
    }
    FJ_HD void fallback_v(const PotView &P)
    {
        Fudge o64;
        fudge64_at_point(o64, P, Delta, Lz * Lz, E, u, v, shu2, sv, cv, sv2, pu, pv);
        const double v64 = get_turn_v(o64, .5 * kPIH);
        fail |= o64.fail;
        wt = (float)(kPIH - v64);
        esc = 1u;
    }

    // u walk (get_turn_u_f) after a value: true when it ended (tin, tout set
    // or the FP64 fallback ran), false with a new request.
    FJ_HD bool walk_u(const PotView &P, float val, float dval)
    {
        ut = val;
        if (want_du) dut = dval;
        if (wstage == 0) {  // the first value, at utry = 1
            if (!isfinite(ut)) { fallback_u(P); return true; }
            if (ut < 0) {
                if (dut > 0) { uin = utry; wstage = 1; }
                else wstage = 3;
            } else { fu1 = ut; wstage = 5; }
        } else {
            if (++it > kLoopCap || !isfinite(ut)) { fallback_u(P); return true; }
        }
        for (;;) {
            switch (wstage) {
            case 1:  // while (ut < 0 && dut > 0) walk out; then refine eps
                if (ut < 0 && dut > 0) { uin = utry; utry *= (1 + eps); request_u(utry, true); return false; }
                if (ut >= 0) { u1 = utry; wstage = 2; continue; }
                utry /= (1 + eps); eps *= .2;
                if (eps < kTINY) { tin = tout = (float)(utry - o.u_pt); return true; }
                utry *= (1 + eps);
                request_u(utry, true);
                return false;
            case 2:  // while (ut > 0) { u2 = utry; utry *= 1.1 }
                if (ut > 0) { u2 = utry; utry *= 1.1; request_u(utry, false); return false; }
                uout = utry;
                return start_brent_u();
            case 3:  // while (ut < 0 && dut < 0) walk in; then refine eps
                if (ut < 0 && dut < 0) { uout = utry; utry /= (1 + eps); request_u(utry, true); return false; }
                if (ut >= 0) { u2 = utry; wstage = 4; continue; }
                utry *= (1 + eps); eps *= .2;
                if (eps < kTINY) { tin = tout = (float)(utry - o.u_pt); return true; }
                utry /= (1 + eps);
                request_u(utry, true);
                return false;
            case 4:  // while (ut > 0) { u1 = utry; utry *= .9 }
                if (ut > 0) { u1 = utry; utry *= .9; request_u(utry, false); return false; }
                uin = utry;
                return start_brent_u();
            case 5:  // ut >= 0 at the start: outward
                if (ut > 0) { u2 = utry; utry *= 1.1; request_u(utry, false); return false; }
                uout = utry;
                ut = fu1;
                wstage = 6;
                continue;
            default:  // 6: inward from the outer position
                if (ut > 0) { u1 = utry; utry *= .9; request_u(utry, false); return false; }
                uin = utry;
                return start_brent_u();
            }
        }
    }
    FJ_HD bool start_brent_u()
    {
        phase = kBrentUin;
        mode = kEvU; want_du = false;
        x = br.start((float)(uin - o.u_pt), (float)(u1 - o.u_pt));
        return false;
    }

    FJ_HD void start_v()
    {
        phase = kWalkVeq; wstage = 0; it = 0;
        mode = kEvVw; x = .5f * kPIHf; want_du = false;
    }

    // Feeds the requested value(s).  Returns true when the node's actions are
    // complete (Jr, Jz).
    FJ_HD bool feed(const PotView &P, const GK21f &K, float val, float dval)
    {
        const float rtwo = 1.41421356237309505f;
        for (;;) {
            switch (phase) {
            case kWalkU: {
                bool ended = walk_u(P, val, dval);
                if (!ended) return false;
                if (phase == kBrentUin) return false;  // a Brent request is pending
                // the walk ended without Brent (Jr = 0 limit or the FP64 fallback)
                phase = kQagsU;
                if (fabsf(tout - tin) < 1e-12f) { Jr = 0; start_v(); return false; }
                o.tb = .5f * (tin + tout); o.Dt = .5f * (tout - tin);
                mode = kEvJu; want_du = false;
                x = qs.start(K, 0.f, kPIf, 1e-5f, 1e-3f);
                return false;
            }
            case kBrentUin:
                if (!br.feed(val, x, fail)) return false;
                tin = br.xr;
                phase = kBrentUout;
                x = br.start((float)(u2 - o.u_pt), (float)(uout - o.u_pt));
                return false;
            case kBrentUout:
                if (!br.feed(val, x, fail)) return false;
                tout = br.xr;
                if (fabsf(tout - tin) < 1e-12f) { Jr = 0; start_v(); return false; }
                o.tb = .5f * (tin + tout); o.Dt = .5f * (tout - tin);
                phase = kQagsU;
                mode = kEvJu;
                x = qs.start(K, 0.f, kPIf, 1e-5f, 1e-3f);
                return false;
            case kQagsU:
                if (!qs.feed(K, val, x, fail)) return false;
                Jr = (double)(rtwo * o.Delta * o.Dt * qs.result / kPIf);
                start_v();
                return false;
            case kWalkVeq:
                if (wstage == 0) {  // V(pi/4) in the w form decides the side
                    if (val < 0) { wbot = .5f * kPIHf; wstage = 1; continue; }
                    phase = kWalkVpole; vtop = .5f * kPIHf; it = 0;
                    mode = kEvVv; x = vtop;
                    return false;
                }
                // wstage 1: val = V(wbot) (the first is the value at pi/4 again)
                if (val < 0) {
                    wbot *= .5f;
                    if (wbot < 1e-12f) { wt = 0.f; return start_qags_v(K); }
                    if (++it > kLoopCap) { fallback_v(P); return start_qags_v(K); }
                    x = wbot;
                    return false;
                }
                phase = kBrentVeq;
                x = br.start(.5f * kPIHf, wbot);
                return false;
            case kWalkVpole:
                if (val > 0) {
                    vtop *= .5f;
                    if (vtop < 1e-12f) { wt = kPIHf; return start_qags_v(K); }
                    if (++it > kLoopCap) { fallback_v(P); return start_qags_v(K); }
                    x = vtop;
                    return false;
                }
                phase = kBrentVpole;
                x = br.start(vtop, .5f * kPIHf);
                return false;
            case kBrentVeq:
                if (!br.feed(val, x, fail)) return false;
                wt = br.xr;
                return start_qags_v(K);
            case kBrentVpole:
                if (!br.feed(val, x, fail)) return false;
                wt = kPIHf - br.xr;
                return start_qags_v(K);
            case kQagsV:
                if (!qs.feed(K, val, x, fail)) return false;
                Jz = (double)(2.f * rtwo * o.Delta * o.wt * qs.result / kPIf);
                phase = kDone;
                return true;
            default:
                return true;
            }
        }
    }
    FJ_HD bool start_qags_v(const GK21f &K)
    {
        if (wt < 1e-12f) { Jz = 0; phase = kDone; return true; }
        o.wt = wt;
        phase = kQagsV;
        mode = kEvJv; want_du = false;
        x = qs.start(K, 0.f, kPIHf, 1e-5f, 1e-3f);
        return false;
    }

    // the double-power-law DF of mixed_node_df from the actions
    FJ_HD double df(const DFDev &d) const
    {
        const float Jphi = (float)Lz, jr = (float)Jr, jz = (float)Jz, J0 = (float)d.J0;
        const float h = jr + (float)d.dphi_h * fabsf(Jphi) + (float)d.dz_h * jz;
        const float g = jr + (float)d.dphi_g * fabsf(Jphi) + (float)d.dz_g * jz;
        const float ev = (float)d.norm *
                         fmaxf(0.f, powf(1.f + J0 / h, (float)d.alpha) / powf(1.f + g / J0, (float)d.beta)) /
                         (float)d.tpi3;
        float f = d.chi == 0. ? ev : ev + (float)d.k * tanhf((float)d.chi * Jphi / J0) * ev;
        if (isnan(f)) f = 0.f;
        return (double)f;
    }
};

}  // namespace fj
