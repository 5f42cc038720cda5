// fj_qags_warp.cuh -- QUADPACK QAGS (DQAGSE) run by a whole warp.
//
// The function values of each Gauss-Kronrod panel (21 or 15 points, twice that
// per bisection) are spread over the 32 lanes and exchanged through shared
// memory; every lane forms the panel sums from them in the same order, and the
// adaptive bookkeeping (qags_rest of fj_device.cuh) runs uniformly on every
// lane over an interval list in the warp's shared memory (identical values,
// identical writes).  The result is that of one thread running the same QAGS:
// the same function values enter the same sums in the same order.  Every lane
// of the warp must call it with the same arguments.
#pragma once

#include "fj_device.cuh"

namespace fj {

template <int RULE, class F>
struct WarpPanels64 {
    F &f;
    double *buf;
    int lane;
    __device__ void one(double a, double b, double &r, double &e, double &ra, double &rc)
    {
        constexpr int n = GKRule<RULE>::npts;
        for (int i = lane; i < n; i += 32) buf[i] = f(gk_abscissa<RULE>(a, b, i));
        __syncwarp();
        gk_sum<RULE>(a, b, buf, r, e, ra, rc);
        __syncwarp();
    }
    __device__ void two(double a1, double b1, double a2, double b2, double &r1, double &e1, double &ra1,
                        double &rc1, double &r2, double &e2, double &ra2, double &rc2)
    {
        constexpr int n = GKRule<RULE>::npts;
        for (int i = lane; i < 2 * n; i += 32) {
            const bool second = i >= n;
            buf[i] = f(gk_abscissa<RULE>(second ? a2 : a1, second ? b2 : b1, second ? i - n : i));
        }
        __syncwarp();
        gk_sum<RULE>(a1, b1, buf, r1, e1, ra1, rc1);
        gk_sum<RULE>(a2, b2, buf + n, r2, e2, ra2, rc2);
        __syncwarp();
    }
};

template <int RULE, class F>
__device__ int qags_warp(F &f, double a, double b, double epsabs, double epsrel, int limit, double &result,
                         double &abserr, unsigned &fail, const QagsWs &ws, double *buf, int lane)
{
    WarpPanels64<RULE, F> pn{f, buf, lane};
    double res0, err0, resabs0, resasc0;
    pn.one(a, b, res0, err0, resabs0, resasc0);
    const int h = qags_head(res0, err0, resabs0, resasc0, epsabs, epsrel, limit, result, abserr);
    if (h >= 0) return h;
    return qags_rest<RULE>(pn, a, b, res0, err0, resabs0, epsabs, epsrel, limit, result, abserr, fail, ws);
}


// workspace of one warp: an interval list of `cap` entries and the panel values
struct WarpQagsWs {
    double *list;  // [4 * cap]
    int *iord;     // [cap]
    double *buf;   // [42]
    int cap;
    __device__ QagsWs ws() const { return QagsWs{list, list + cap, list + 2 * cap, list + 3 * cap, iord, cap}; }
};

}  // namespace fj
