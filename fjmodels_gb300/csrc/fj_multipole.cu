// fj_multipole.cu -- the multipole side of one iteration: Legendre
// projection of the moment grids, the radial Poisson integrals, the sum of
// component potentials and the tensor-virial sums.  All FP64; each is small
// next to the phase-space kernel.
#include "fj_internal.h"
#include "fj_qags_warp.cuh"

namespace fj {

// get_Ylm, 6 fields (include/UtilsLeg.h:200-253), with computeRhl's rho[0][0]
// extrapolation (pot/potLeg.cpp:68).  One thread per output coefficient.
__global__ void k_project(int nr, int ngauss, int npoly, const double *ar, const double *poly,
                          const double *grids6, double *coef6)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncoef = nr * npoly, npts = nr * ngauss;
    if (t >= 6 * ncoef) return;
    const int q = t / ncoef, n = (t % ncoef) / npoly, l = t % npoly;
    const double *Q = grids6 + (size_t)q * npts;
    double v;
    if (n == 0) {
        if (l != 0) v = 0;
        else if (q == 0)
            v = 2 * ((Q[2 * ngauss] - Q[ngauss]) / (ar[2] - ar[1]) * (ar[0] - ar[1]) + Q[ngauss]);
        else v = 2 * Q[0];
    } else {
        double s = 0;
        for (int g = 0; g < ngauss; g++) s += poly[l * ngauss + g] * Q[n * ngauss + g];
        v = s;
    }
    coef6[t] = v;
}

cudaError_t launch_project(int nr, int ngauss, int npoly, const double *ar, const double *poly,
                           const double *grids6, double *coef6, cudaStream_t s)
{
    const int n = 6 * nr * npoly;
    k_project<<<(n + 127) / 128, 128, 0, s>>>(nr, ngauss, npoly, ar, poly, grids6, coef6);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ Poisson
// linear interpolation of one multipole column (include/Utils.h:122-128)
__device__ __forceinline__ double linterp_col(const double *ar, const double *rhl, int npoly, int l, int nr, double x)
{
    if (x <= ar[0]) return rhl[l];
    if (x >= ar[nr - 1]) return rhl[(nr - 1) * npoly + l];
    int top = 0, bot = 0;
    topbottom(ar, nr, x, bot, top);
    const double yb = rhl[bot * npoly + l], yt = rhl[top * npoly + l];
    return yb + (x - ar[bot]) / (ar[top] - ar[bot]) * (yt - yb);
}

struct IInternal {  // I_internal (pot/Potential.cpp:83-89); multipole column col, degree l = 2*col
    const double *ar, *rhl; int npoly, col, l, nr;
    __device__ double operator()(double x) const { return pow(x, l + 2) * linterp_col(ar, rhl, npoly, col, nr, x); }
};
struct IExternalT {  // I_external (pot/Potential.cpp:90-101) on x = a + (1-t)/t, divided by t^2
    const double *ar, *rhl; int npoly, col, l, nr; double a;
    __device__ double operator()(double t) const
    {
        const double x = a + (1 - t) / t;
        double rhol;
        if (x > ar[nr - 1]) rhol = dmax(0., rhl[(nr - 1) * npoly + col] * pow(ar[nr - 1] / x, 4));
        else rhol = linterp_col(ar, rhl, npoly, col, nr, x);
        const double y = rhol / pow(x, l - 1);
        return (y / t) / t;
    }
};

// One warp per (n, l) pair.  The QAGS calls of a pair run on all 32 lanes
// at once: the function values of each Gauss-Kronrod panel (21 or 15, 42 or
// 30 per bisection) are spread over the lanes and exchanged through shared
// memory, every lane forms the panel sums from them in the same order, and
// the adaptive bookkeeping runs uniformly on every lane over an interval
// list in the warp's shared memory (identical values, identical writes).
// The results are those of one thread running the same QAGS: the same
// function values enter the same sums in the same order.  With one thread
// per pair the 2 nr npoly integrals (560 on 80 x 7) sat on a few SMs, each
// thread evaluating its thousands of integrand values one after another.
constexpr int kPoissonWarps = 4;

// computeInts + computePhil (pot/Potential.cpp:110-200)
__global__ void __launch_bounds__(32 * kPoissonWarps) k_poisson(int nr, int npoly, const double *ar,
                                                                 const double *rhl, double *phil, double *Pr,
                                                                 double *Pr2, unsigned long long *counters)
{
    __shared__ double s_list[kPoissonWarps][4 * kPoissonCap];
    __shared__ int s_iord[kPoissonWarps][kPoissonCap];
    __shared__ double s_vals[kPoissonWarps][42];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kPoissonWarps + warp;
    const int nt = nr * npoly;
    if (t >= nt) return;  // the whole warp
    const int n = t / npoly, np = t % npoly, l = 2 * np;
    double *dws = s_list[warp];
    const QagsWs W{dws, dws + kPoissonCap, dws + 2 * kPoissonCap, dws + 3 * kPoissonCap, s_iord[warp], kPoissonCap};
    unsigned fail = 0;
    double Iint, Iext, err;
    IInternal fi{ar, rhl, npoly, np, l, nr};
    qags_warp<21>(fi, 0., ar[n], 1e-4, 1e-3, 1000, Iint, err, fail, W, s_vals[warp], lane);
    IExternalT fe{ar, rhl, npoly, np, l, nr, ar[n]};
    double epsabs = 1e-4, epsrel = 1e-3;
    int status = 1, tries = 0;
    while (status != 0 && tries < 60) {
        status = qags_warp<15>(fe, 0.0, 1.0, epsabs, epsrel, 1000, Iext, err, fail, W, s_vals[warp], lane);
        epsabs *= 2; epsrel *= 2; tries++;
    }
    if (lane != 0) return;
    if (fail && counters) atomicAdd(&counters[kCntPoisson], 1ull);
    const double r = ar[n];
    const double G = 1;
    phil[t] = -kTPI * G * (Iint / pow(r, l + 1) + Iext * pow(r, l));
    Pr[t] = -kTPI * G * (-(l + 1) * Iint / pow(r, l + 2) + l * Iext * pow(r, l - 1));
    Pr2[t] = -kTPI * G * ((l + 2) * (l + 1) * Iint / pow(r, l + 3) + (l - 1) * l * Iext * pow(r, l - 2) -
                          (2 * l + 1) * rhl[t]);
}

cudaError_t launch_poisson(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                           double *Pr, double *Pr2, unsigned long long *counters, cudaStream_t s)
{
    const int nt = nr * npoly;
    k_poisson<<<(nt + kPoissonWarps - 1) / kPoissonWarps, 32 * kPoissonWarps, 0, s>>>(nr, npoly, ar, rhl, phil, Pr,
                                                                                      Pr2, counters);
    return cudaGetLastError();
}

// ------------------------------------------- exact cumulative Poisson solve
// The integrals of computeInts (pot/Potential.cpp:82-155) taken exactly: the
// integrands are x^(l+2) rho_l(x) and rho_l(x) x^(1-l) with rho_l the linear
// interpolation of the density multipoles (linterp, include/Utils.h:122-128:
// constant below ar[0]) and rho_l(x) = max(0, rho_l[nr-1] (ar[nr-1]/x)^4)
// beyond the grid (Potential.cpp:90-99), so each grid interval contributes a
// closed form and the integrals are prefix sums over the intervals, added in
// a fixed order.  No adaptive decisions: the potential is a smooth function of
// the density, where the reference's QAGS (epsabs 1e-4, epsrel 1e-3) moves it
// by up to ~1e-3 when a small change of the density flips a subdivision.
// One block per multipole l, a thread per interval, then one thread per radius.

// int_a^b x^m (c0 + c1 x) dx
__device__ __forceinline__ double seg_power_integral(double a, double b, int m, double c0, double c1)
{
    const double t0 = m == -1 ? log(b / a) : (pow(b, m + 1) - pow(a, m + 1)) / (m + 1);
    const double t1 = m == -2 ? log(b / a) : (pow(b, m + 2) - pow(a, m + 2)) / (m + 2);
    return c0 * t0 + c1 * t1;
}

__global__ void k_poisson_cumulative(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                                     double *Pr, double *Pr2)
{
    extern __shared__ double sh[];
    double *s_in = sh, *s_ex = sh + nr;  // interval i = [ar[i], ar[i+1]] (s_in[nr-1]: [0, ar[0]]; s_ex[nr-1]: tail)
    const int np = blockIdx.x, l = 2 * np;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        if (i < nr - 1) {
            const double a = ar[i], b = ar[i + 1], ya = rhl[i * npoly + np], yb = rhl[(i + 1) * npoly + np];
            const double s = (yb - ya) / (b - a), c0 = ya - s * a;
            s_in[i] = seg_power_integral(a, b, l + 2, c0, s);
            s_ex[i] = seg_power_integral(a, b, 1 - l, c0, s);
        } else {
            const double a0 = ar[0], R = ar[nr - 1], yN = rhl[(nr - 1) * npoly + np];
            s_in[i] = rhl[np] * pow(a0, l + 3) / (l + 3);
            s_ex[i] = (yN > 0 ? yN : 0.) * pow(R, 2 - l) / (l + 2);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // prefix sums in place: s_in[n] = I_int(ar[n]), s_ex[n] = I_ext(ar[n])
        double acc = s_in[nr - 1], seg = s_in[0];
        s_in[0] = acc;
        for (int n = 1; n < nr; n++) {
            acc += seg;
            seg = s_in[n];
            s_in[n] = acc;
        }
        acc = s_ex[nr - 1];
        for (int n = nr - 1; n >= 0; n--) {
            const double cur = n < nr - 1 ? s_ex[n] : 0.;
            if (n < nr - 1) acc += cur;
            s_ex[n] = acc;
        }
    }
    __syncthreads();
    for (int n = threadIdx.x; n < nr; n += blockDim.x) {  // computePhil (Potential.cpp:163-200)
        const double r = ar[n], Ii = s_in[n], Ie = s_ex[n], G = 1;
        const int t = n * npoly + np;
        phil[t] = -kTPI * G * (Ii / pow(r, l + 1) + Ie * pow(r, l));
        Pr[t] = -kTPI * G * (-(l + 1) * Ii / pow(r, l + 2) + l * Ie * pow(r, l - 1));
        Pr2[t] = -kTPI * G * ((l + 2) * (l + 1) * Ii / pow(r, l + 3) + (l - 1) * l * Ie * pow(r, l - 2) -
                              (2 * l + 1) * rhl[t]);
    }
}

cudaError_t launch_poisson_cumulative(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                                      double *Pr, double *Pr2, cudaStream_t s)
{
    if (nr < 2 || nr > kPoissonCumulativeMaxNr) return cudaErrorInvalidValue;
    k_poisson_cumulative<<<npoly, 128, 2 * nr * sizeof(double), s>>>(nr, npoly, ar, rhl, phil, Pr, Pr2);
    return cudaGetLastError();
}

// ------------------------------------------------------------ updatePhil
__global__ void k_sum3(int n, const double *a0, const double *a1, const double *a2, const double *b0,
                       const double *b1, const double *b2, double *o0, double *o1, double *o2)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    o0[t] = a0[t] + b0[t];
    o1[t] = a1[t] + b1[t];
    o2[t] = a2[t] + b2[t];
}

cudaError_t launch_sum3(int n, const double *a0, const double *a1, const double *a2, const double *b0,
                        const double *b1, const double *b2, double *o0, double *o1, double *o2, cudaStream_t s)
{
    k_sum3<<<(n + 255) / 256, 256, 0, s>>>(n, a0, a1, a2, b0, b1, b2, o0, o1, o2);
    return cudaGetLastError();
}

__global__ void k_add(int n, const double *a, const double *b, double *o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) o[i] = a[i] + b[i];
}

cudaError_t launch_add(int n, const double *a, const double *b, double *o, cudaStream_t s)
{
    k_add<<<(n + 255) / 256, 256, 0, s>>>(n, a, b, o);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ vir2
constexpr int kVirBlock = 256;

// vir2 (libs/Stats.cpp:12-41) with the 5-field ev_dens / int_dens of
// include/UtilsLeg.h:300-354, whose interpolation weight is a float (:312).
__global__ void __launch_bounds__(kVirBlock) k_vir2(PotView P, int ngauss, const double *ci, const double *wi,
                                                   const double *coef6, double *out7)
{
    const int nr = P.nr, npoly = P.npoly, nc = nr * npoly;
    const double *ar = P.ar, *rhl = coef6, *sigRl = coef6 + 2 * nc, *sigpl = coef6 + 3 * nc, *sigzl = coef6 + 4 * nc;
    double acc[5] = {0, 0, 0, 0, 0};  // pot, KRR, Kzz, WRR, Wzz
    const int ncell = (nr - 1) * ngauss;
    for (int cell = threadIdx.x; cell < ncell; cell += kVirBlock) {
        const int i = 1 + cell / ngauss, j = cell % ngauss;
        const double r = .5 * (ar[i - 1] + ar[i]), dr = ar[i] - ar[i - 1];
        const double sij = sqrt(1 - ci[j] * ci[j]);
        const double z = r * ci[j], R = r * sij;
        const double rr = sqrt(R * R + z * z), c = z / rr;
        double dens = 0, Su = 0, Sp = 0, Sv = 0;
        if (!(rr > ar[nr - 1])) {
            int top = 0, bot = 0;
            topbottom(ar, nr, rr, bot, top);
            const float f = (float)((rr - ar[bot]) / (ar[top] - ar[bot]));
            const float omf = 1 - f;
            const double c2 = c * c;
            double pm2 = 1, pm1 = 0;
            for (int np = 0; np < npoly; np++) {
                const double dp = f * rhl[top * npoly + np] + omf * rhl[bot * npoly + np];
                const double up = f * sigRl[top * npoly + np] + omf * sigRl[bot * npoly + np];
                const double pp = f * sigpl[top * npoly + np] + omf * sigpl[bot * npoly + np];
                const double vp = f * sigzl[top * npoly + np] + omf * sigzl[bot * npoly + np];
                if (np == 0) { dens = .5 * dp; Su = .5 * up; Sp = .5 * pp; Sv = .5 * vp; continue; }
                double pol;
                if (np == 1) { pol = 1.5 * c2 - .5; pm1 = pol; }
                else { pol = evenleg_next(np, c2, pm2, pm1); pm2 = pm1; pm1 = pol; }
                const double fac = .5 * (4 * np + 1);
                dens += fac * dp * pol;
                Su += fac * up * pol;
                Sp += fac * pp * pol;
                Sv += fac * vp * pol;
            }
        }
        double phi, dR, dz;
        pot_grad(P, R, z, phi, dR, dz);
        acc[0] += .5 * wi[j] * dens * phi * r * r * dr;
        acc[1] += .5 * wi[j] * dens * ((r * Su) * (r * Su) + (r * Sp) * (r * Sp)) * dr;
        acc[2] += .5 * wi[j] * dens * ((r * Sv) * (r * Sv)) * dr;
        acc[3] -= wi[j] * dens * R * dR * r * r * dr;
        acc[4] -= wi[j] * dens * z * dz * r * r * dr;
    }
    __shared__ double red[kVirBlock / 32][5];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        double v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[5] = {0, 0, 0, 0, 0};
        for (int w = 0; w < kVirBlock / 32; w++)
            for (int q = 0; q < 5; q++) s[q] += red[w][q];
        const double fpi = 4 * kPI;
        out7[0] = s[1] * fpi;  // KRR
        out7[1] = s[2] * fpi;  // Kzz
        out7[2] = s[3] * fpi;  // WRR
        out7[3] = s[4] * fpi;  // Wzz
        out7[4] = s[0] * fpi;  // PE
        out7[5] = ar[nr - 1] * ar[nr - 1] * P.Pr[(nr - 1) * npoly];
        // mass check (Stats.cpp:35-37)
        double sum = 0.;
        for (int i = 0; i < nr; i++) {
            int top = 0, bot = 0;
            topbottom(ar, nr, ar[i], bot, top);
            const double f = (ar[i] - ar[bot]) / (ar[top] - ar[bot]);
            double dens = .5 * (f * rhl[top * npoly] + (1 - f) * rhl[bot * npoly]);
            double pm2 = 1, pm1 = 0;
            for (int np = 1; np < npoly; np++) {
                double pol;
                if (np == 1) { pol = -.5; pm1 = pol; }
                else { pol = evenleg_next(np, 0.0, pm2, pm1); pm2 = pm1; pm1 = pol; }
                dens += .5 * (4 * np + 1) * (f * rhl[top * npoly + np] + (1 - f) * rhl[bot * npoly + np]) * pol;
            }
            sum += 2 * kTPI * ar[i] * ar[i] * dens;
        }
        out7[6] = sum;
    }
}

cudaError_t launch_vir2(PotView P, int ngauss, const double *ci, const double *wi, const double *coef6,
                        double *out7, cudaStream_t s)
{
    k_vir2<<<1, kVirBlock, 0, s>>>(P, ngauss, ci, wi, coef6, out7);
    return cudaGetLastError();
}

size_t poisson_local_bytes()
{
    cudaFuncAttributes at;
    return cudaFuncGetAttributes(&at, k_poisson) == cudaSuccess ? at.localSizeBytes : 0;
}

size_t multipole_local_bytes()
{
    size_t m = 0;
    cudaFuncAttributes at;
    if (cudaFuncGetAttributes(&at, k_poisson) == cudaSuccess && at.localSizeBytes > m) m = at.localSizeBytes;
    if (cudaFuncGetAttributes(&at, k_vir2) == cudaSuccess && at.localSizeBytes > m) m = at.localSizeBytes;
    return m;
}

}  // namespace fj
