// fj_delta.cu -- the focal-distance tables of many models at once: one thread
// per (model, energy) runs delta_energy (fj_delta.cuh), the same code as the
// host's fj_tabulate_delta.  Each thread integrates its orbits alone (FP64,
// serial Bulirsch-Stoer steps), so the kernel is latency-bound and pays off
// with many models (or a table per iteration), not for one.  Built without
// FMA contraction, like the host restatement it shares its arithmetic with.
#include "fj_internal.h"
#include "fj_delta.cuh"

namespace fj {

namespace {

constexpr int kDeltaBlock = 32;

__global__ void __launch_bounds__(kDeltaBlock) k_tabulate_delta(const PotView *pots, double *const *Eg,
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
    k_tabulate_delta<<<(nt + kDeltaBlock - 1) / kDeltaBlock, kDeltaBlock, 0, s>>>(pots, Eg, Dg, n, ngrid, bad);
    return cudaGetLastError();
}

size_t delta_local_bytes()
{
    cudaFuncAttributes at;
    return cudaFuncGetAttributes(&at, k_tabulate_delta) == cudaSuccess ? at.localSizeBytes : 0;
}

}  // namespace fj
