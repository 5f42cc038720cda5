// fj_delta.cu -- the focal-distance tables of many models at once: one thread
// per (model, energy) runs delta_energy (fj_delta.cuh), the same code as the
// host's fj_tabulate_delta.  The energies' searches take very different paths
// and lengths (most of a fit is the search for its Jr = 0 orbit: repeated
// adaptive orbit integrations), and the launch lasts as long as its slowest
// fits, so every fit starts at once and the fits are spread evenly over the
// SMs: small blocks of kDeltaThreads.  256 models x 30 energies on the GB300:
// 10.7 s with 8 threads per block, 11.0 s with 16, 11.8 s with 32 or 64, and
// 22.3 s with one thread per block (the SMs' 32-block limit made two waves).
// A warp per fit, its lanes sharing the sums over the orbit points of the
// focal-distance walk, was not faster: those sums are a small part of a fit.
// Built without FMA contraction, like the host code.
//
// The fit of the focal distance to an orbit is not a continuous function of
// rounding: a change of one unit in the last place of the orbit equations
// moves some entries of the table by tens of per cent (the host code itself,
// with pow(y, 3) written as y*y*y, does the same).  The device's libm rounds
// differently from the host's, so the GPU table is another table of the same
// algorithm, not the host's bits; the energies agree to rounding.
#include "fj_internal.h"
#include "fj_delta.cuh"

namespace fj {

namespace {

constexpr int kDeltaThreads = 8;  // fits per block

__global__ void __launch_bounds__(kDeltaThreads) k_tabulate_delta(const PotView *pots, double *const *Eg,
                                                               double *const *Dg, int n, int ngrid, int *bad)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * ngrid) return;
    const int m = t / ngrid, nE = t % ngrid;
    const PotView P = pots[m];
    const DeltaBase base = delta_base(P);
    bool b = base.bad;
    DeltaFit d;
    double E;
    const double D2 = delta_energy(P, base, nE, ngrid, E, d, b, kDeltaWalkCapDevice);
    Eg[m][nE] = E;
    Dg[m][nE] = D2;
    if (b) atomicOr(&bad[m], 1);
}

}  // namespace

cudaError_t launch_tabulate_delta(const PotView *pots, double *const *Eg, double *const *Dg, int n, int ngrid,
                                  int *bad, cudaStream_t s)
{
    const int nt = n * ngrid;
    k_tabulate_delta<<<(nt + kDeltaThreads - 1) / kDeltaThreads, kDeltaThreads, 0, s>>>(pots, Eg, Dg, n, ngrid, bad);
    return cudaGetLastError();
}

size_t delta_local_bytes()
{
    cudaFuncAttributes at;
    return cudaFuncGetAttributes(&at, k_tabulate_delta) == cudaSuccess ? at.localSizeBytes : 0;
}

}  // namespace fj
