// fj_noalloc.cu -- the Poisson solve without a context.
//
// For callers that hold no fj_ctx or cannot allocate device memory on their
// call path (an application whose device memory is entirely reserved by its
// own pool allocator, or a latency-bound loop that must not pay for an
// allocation).  The Poisson kernel keeps its quadrature workspace in shared
// memory, so this entry point needs nothing but its inputs, outputs and a
// stream, and calls on different streams are independent.
#include <cuda_runtime.h>

#include "../../include/fjgpu.h"
#include "fj_internal.h"

extern "C" int fj_poisson_noalloc(int nr, int npoly, const double *ar, const double *rhl, double *phil, double *Pr,
                                  double *Pr2, void *stream)
{
    if (nr < 2 || npoly < 1 || npoly > fj::kMaxPoly || !ar || !rhl || !phil || !Pr || !Pr2) return FJ_ERR_ARG;
    const cudaError_t e = fj::launch_poisson(nr, npoly, ar, rhl, phil, Pr, Pr2, nullptr, (cudaStream_t)stream);
    return e == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}
