// fj_noalloc.cu -- the Poisson solve without a context.
//
// For callers that hold no fj_ctx or cannot allocate device memory on their
// call path (an application whose device memory is entirely reserved by its
// own pool allocator, or a latency-bound loop that must not pay for an
// allocation).  The Poisson kernel keeps its quadrature workspace in shared
// memory, so this entry point needs nothing but its inputs, outputs and a
// stream, and calls on different streams are independent.
//
// The one device memory a launch can still claim is per-thread local memory:
// a kernel whose stack is larger than the device's current stack limit makes
// the CUDA driver enlarge the context's local-memory reservation at launch.
// The call therefore compares the kernel's stack with the current limit and
// refuses (FJ_ERR_NOMEM) instead of launching when the limit is too small.
// CUDA's default limit (1024 bytes per thread) covers the kernel.
#include <cuda_runtime.h>

#include "../../include/fjgpu.h"
#include "fj_internal.h"

extern "C" int fj_poisson_noalloc_stack(size_t *need, size_t *limit)
{
    if (!need && !limit) return FJ_ERR_ARG;
    if (need) *need = fj::poisson_local_bytes();
    if (limit && cudaDeviceGetLimit(limit, cudaLimitStackSize) != cudaSuccess) return FJ_ERR_CUDA;
    return FJ_OK;
}

extern "C" int fj_poisson_noalloc(int nr, int npoly, const double *ar, const double *rhl, double *phil, double *Pr,
                                  double *Pr2, void *stream)
{
    if (nr < 2 || npoly < 1 || npoly > fj::kMaxPoly || !ar || !rhl || !phil || !Pr || !Pr2) return FJ_ERR_ARG;
    size_t need = 0, limit = 0;
    if (fj_poisson_noalloc_stack(&need, &limit) != FJ_OK) return FJ_ERR_CUDA;
    if (need > limit) return FJ_ERR_NOMEM;
    const cudaError_t e = fj::launch_poisson(nr, npoly, ar, rhl, phil, Pr, Pr2, nullptr, (cudaStream_t)stream);
    return e == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}
