// fj_peak.cu -- FMA-throughput micro-benchmark: the FP64 / FP32 peaks the
// phase-space kernels' rooflines are quoted against (a copy-bandwidth or BF16
// GEMM measurement says nothing about these pipes).
#include <cuda_runtime.h>

#include "../../include/fjgpu.h"

namespace {

template <class T>
__global__ void k_fma_chain(T *out, int iters, T a, T b)
{
    // 8 independent dependency chains per thread keep the pipe busy
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-1.2345) out[blockIdx.x] = s;  // keeps the chains live
}

template <class T>
double run(int iters)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    if (cudaMalloc(&out, blocks * sizeof(T)) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_chain<T><<<blocks, threads>>>(out, iters / 8, (T)0.999999, (T)1e-7);  // warm-up
    cudaEventRecord(e0);
    k_fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    return ms > 0 ? flops / (ms * 1e-3) / 1e12 : -1;
}

}  // namespace

extern "C" int fj_measure_fma_peak(int fp32, double *tflops)
{
    if (!tflops) return FJ_ERR_ARG;
    *tflops = fp32 ? run<float>(1 << 16) : run<double>(1 << 12);
    return *tflops > 0 ? FJ_OK : FJ_ERR_CUDA;
}
