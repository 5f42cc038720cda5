// Host build of the mixed-precision node solve (fjmodels_gb300/csrc/fj_mixed.cuh,
// the same host/device source the GPU kernel compiles): the moments of given
// meridional points, per point as the kernel's block does it (potential and
// escape speed in FP64, the FP32 tables shifted by the point's potential, every
// bound velocity node through mixed_node_df, the moments summed in FP64) and
// normalised as k_moments_finalize (integ/Integ.cpp:160-162).  Test
// infrastructure for tests/test_mixed_host.py: it takes its inputs as one binary
// file and prints the moments.  The GPU's FP64 re-solve of capped nodes is not
// mirrored: capped nodes are counted and printed.
//
//   host_mixed <input.bin>
//   input: int32 nr, npoly, ngrid, nq, npts; float64 ar[nr], phil, Pr, Pr2 [nr*npoly],
//          Egrid, Dgrid [ngrid], xq, wq [nq], Rz [npts][2],
//          df: kind, alpha, beta, J0, mass, dphi_h, dz_h, dphi_g, dz_g, chi, k
//   output: per point one line of the six moments (rho, vrot, sigR, sigphi, sigz, sigRz),
//           then "capped <n>"
#define __constant__
#include <cmath>
using std::isfinite;
using std::isnan;
#include <cstdio>
#include <cstring>
#include <vector>

#include "fj_mixed.cuh"

using namespace fj;

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[5];
    if (fread(hdr, sizeof(int), 5, f) != 5) return 2;
    const int nr = hdr[0], npoly = hdr[1], ngrid = hdr[2], nq = hdr[3], npts = hdr[4];
    auto rd = [&](size_t n) {
        std::vector<double> v(n);
        if (fread(v.data(), sizeof(double), n, f) != n) v.clear();
        return v;
    };
    const auto ar = rd(nr), phil = rd((size_t)nr * npoly), Pr = rd((size_t)nr * npoly), Pr2 = rd((size_t)nr * npoly);
    const auto Eg = rd(ngrid), Dg = rd(ngrid), xq = rd(nq), wq = rd(nq), Rz = rd(2 * (size_t)npts), dfv = rd(11);
    fclose(f);
    if (dfv.size() != 11 || npoly > kMaxPoly) return 2;
    DFDev d;
    memset(&d, 0, sizeof d);  // as df_dev (fj_api.cu)
    d.kind = (int)dfv[0];
    d.alpha = dfv[1]; d.beta = dfv[2]; d.J0 = dfv[3];
    d.norm = dfv[4] / pow(dfv[3], 3);
    d.tpi3 = pow(kTPI, 3.);
    d.dphi_h = dfv[5]; d.dz_h = dfv[6]; d.dphi_g = dfv[7]; d.dz_g = dfv[8]; d.chi = dfv[9]; d.k = dfv[10];
    GK21f K;
    for (int i = 0; i < 11; i++) {
        K.xgk[i] = (float)fj_xgk21[i];
        K.wgk[i] = (float)fj_wgk21[i];
        if (i < 5) K.wg[i] = (float)fj_wg10[i];
    }
    const PotView P{nr, npoly, ar.data(), phil.data(), Pr.data(), Pr2.data()};
    std::vector<float> far(nr), fphil((size_t)nr * npoly), fPr((size_t)nr * npoly), ih(nr), qc(4 * kQuadIntervals),
        pyl(npoly);
    long capped = 0;
    for (int p = 0; p < npts; p++) {
        const double R = Rz[2 * p], z = Rz[2 * p + 1];
        const double rmax = ar[nr - 1];
        const double Phi_h = pot_phi(P, R, z);
        const double Ve = sqrt(-2 * (Phi_h - pot_phi(P, 10 * rmax, 10 * rmax)));
        mixed_tables_f(nr, npoly, ar.data(), phil.data(), Pr.data(), Phi_h, R, z, far.data(), fphil.data(), fPr.data(),
                       ih.data(), qc.data(), pyl.data(), 0, 1);
        const PotViewF PF = mixed_view_f(nr, npoly, ar.data(), phil.data(), Phi_h, R, z, far.data(), fphil.data(),
                                         fPr.data(), ih.data(), qc.data(), pyl.data());
        const double jacob = Ve * Ve * Ve;
        double m[6] = {0, 0, 0, 0, 0, 0};
        for (int i = 0; i < nq; i++)
            for (int j = 0; j < nq; j++)
                for (int k = 0; k < nq; k++) {
                    const double V0 = 1e-6 + Ve * xq[i], V1 = 1e-6 + Ve * xq[j], V2 = 1e-6 + Ve * xq[k];
                    const double H = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h;
                    if (!(H < 0)) continue;
                    unsigned fail = 0, esc = 0;
                    const double Delta = deltafn(Eg.data(), Dg.data(), ngrid, H);
                    double DF = mixed_node_df(P, PF, K, d, Delta, R, z, Phi_h, V0, V1, V2, fail, esc);
                    if (fail) capped++;
                    if (fail & (kFailBracket | kFailRoot)) DF = 0;
                    const double jd = (wq[i] * wq[j] * wq[k]) * (jacob * DF);
                    m[0] += jd;
                    m[1] += jd * V1;
                    m[2] += jd * V0 * V0;
                    m[3] += jd * V1 * V1;
                    m[4] += jd * V2 * V2;
                    m[5] += jd * V0 * V2;
                }
        printf("%.17g %.17g %.17g %.17g %.17g %.17g\n", m[0], m[1] / m[0], sqrt(m[2] / m[0]), sqrt(m[3] / m[0]),
               sqrt(m[4] / m[0]), sqrt(fabs(m[5]) / m[0]));
    }
    printf("capped %ld\n", capped);
    return 0;
}
