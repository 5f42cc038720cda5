// fj_noalloc.cu -- a Poisson solve that allocates no memory.
//
// Some callers cannot call cudaMalloc on their call path: an application
// whose device memory is entirely reserved by its own pool allocator (where a
// driver allocation fails or stalls), or a latency-bound loop that must not
// pay for an allocation.  fj_poisson needs scratch for the adaptive
// quadrature's interval lists and gets it from a context; this variant uses a
// file-scope device array instead, so the caller passes only its inputs,
// outputs and a stream.
//
// The array is part of the library's device image: every GPU that loads the
// library holds it (9 MiB) until the process exits.  All calls share it, so
// calls whose work overlaps on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.  The kernel
// writes every workspace entry before reading it, so nothing has to be
// cleared between calls.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fjgpu.h"
#include "fj_internal.h"

namespace {

constexpr int kMaxIntegrals = FJ_POISSON_NOALLOC_MAX_COEFS;  // nr * npoly
constexpr size_t kScratchBytes = (size_t)kMaxIntegrals * fj::kPoissonCap * (4 * sizeof(double) + sizeof(int));

static __device__ __align__(256) unsigned char g_poisson_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void *g_scratch_addr[kMaxDevices];  // device address of the array, per device, filled on first use
std::mutex g_mu;

}  // namespace

extern "C" int fj_poisson_noalloc(int nr, int npoly, const double *ar, const double *rhl, double *phil, double *Pr,
                                  double *Pr2, void *stream)
{
    if (nr < 2 || npoly < 1 || npoly > fj::kMaxPoly || !ar || !rhl || !phil || !Pr || !Pr2) return FJ_ERR_ARG;
    if ((long long)nr * npoly > kMaxIntegrals) return FJ_ERR_ARG;  // beyond the static workspace
    static_assert(kScratchBytes >= (size_t)kMaxIntegrals * fj::kPoissonCap * (4 * sizeof(double) + sizeof(int)),
                  "workspace layout of the Poisson kernel");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FJ_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return FJ_ERR_ARG;
    void *ws = nullptr;
    {
        // first call on this device: look up the array's device address with the device current
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_poisson_scratch) != cudaSuccess || !p) return FJ_ERR_CUDA;
            g_scratch_addr[dev] = p;
        }
        ws = g_scratch_addr[dev];
    }
    const cudaError_t e =
        fj::launch_poisson(nr, npoly, ar, rhl, phil, Pr, Pr2, ws, nullptr, (cudaStream_t)stream);
    return e == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}
