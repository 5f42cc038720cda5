// fj_mlp.cu -- tensor-core (tcgen05) GEMM and the action surrogate built on it.
#include <cuda_bf16.h>

#include <cstdint>

#include "../../include/fjgpu.h"
#include "fj_internal.h"
#include "fj_tc.cuh"

namespace fj {

using tc::Epilogue;

constexpr int kPadSmem = 23 * 1024;

// C tile (blockIdx.x: rows of 128, blockIdx.y: columns of 128, blockIdx.z:
// K split of kslice columns of K) of A[M][K] * B[N][K]^T.  M any, N and K
// multiples of 16, lda/ldb multiples of 8 elements, A and B 16-byte aligned.
__global__ void __launch_bounds__(tc::kThreads) k_gemm_tc(const __nv_bfloat16 *__restrict__ A, int lda,
                                                          const __nv_bfloat16 *__restrict__ B, int ldb, int M, int N,
                                                          int K, int kslice, Epilogue ep)
{
    __shared__ __align__(1024) unsigned char sA[tc::kTileM * tc::kSliceK * 2];
    __shared__ __align__(1024) unsigned char sB[tc::kTileN * tc::kSliceK * 2];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * tc::kTileM, n0 = blockIdx.y * tc::kTileN;
    const int bn = min(tc::kTileN, N - n0);  // a multiple of 16
    const int k_begin = blockIdx.z * kslice, k_end = min(K, k_begin + kslice);
    const uint32_t bar_a = tc::smem_addr(&bar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc::smem_addr(&tmem_slot)),
                     "r"(tc::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar_a), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(tc::kTileM, bn);
    const uint32_t sA_a = tc::smem_addr(sA), sB_a = tc::smem_addr(sB);

    uint32_t phase = 0;
    bool first = true;
    for (int kc = k_begin; kc < k_end; kc += tc::kSliceK) {
        // stage A[m0.., kc..kc+63] and B[n0.., kc..]: one 16-byte core-matrix row per piece
        for (int p = tid; p < tc::kTileM * 8; p += tc::kThreads) {
            const int r = p >> 3, q = p & 7, k = kc + q * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (m0 + r < M && k < k_end) v = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * lda + k);
            *reinterpret_cast<uint4 *>(sA + (q >> 1) * 4096 + (r >> 3) * 256 + (q & 1) * 128 + (r & 7) * 16) = v;
        }
        for (int p = tid; p < bn * 8; p += tc::kThreads) {
            const int r = p >> 3, q = p & 7, k = kc + q * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (k < k_end) v = *reinterpret_cast<const uint4 *>(B + (size_t)(n0 + r) * ldb + k);
            *reinterpret_cast<uint4 *>(sB + (q >> 1) * (bn * 32) + (r >> 3) * 256 + (q & 1) * 128 + (r & 7) * 16) = v;
        }
        // generic-proxy stores -> visible to the tensor core's (async proxy) reads
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int ks = 0; ks < 4 && kc + ks * 16 < k_end; ks++) {
                const uint64_t ad = tc::smem_desc(sA_a + ks * 4096, 128, 256);
                const uint64_t bd = tc::smem_desc(sB_a + ks * (bn * 32), 128, 256);
                const uint32_t acc = first ? 0u : 1u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
                first = false;
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_a)
                         : "memory");
        }
        // every thread waits for the slice's MMAs before the buffers are refilled
        if (!tc::mbar_wait(bar_a, phase)) abort_flag = 1;
        phase ^= 1u;
        __syncthreads();
        if (abort_flag) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (!abort_flag && k_end > k_begin) {
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < bn; c0 += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int col = n0 + c0 + j;
                    float v = __uint_as_float(r[j]);
                    const size_t o = (size_t)row * ep.ldo + col;
                    switch (ep.mode) {
                    case tc::kEpiStoreF32: ep.outf[o] = v + (ep.bias ? ep.bias[col] : 0.f); break;
                    case tc::kEpiAtomicF32: atomicAdd(ep.outf + o, v); break;
                    case tc::kEpiBiasGelu: {
                        const float z = v + (ep.bias ? ep.bias[col] : 0.f);
                        if (ep.zout) ep.zout[o] = z;
                        ep.outb[o] = __float2bfloat16_rn(tc::gelu(z));
                        break;
                    }
                    case tc::kEpiGeluGrad: ep.outb[o] = __float2bfloat16_rn(v * tc::gelu_grad(ep.zin[o])); break;
                    default: ep.outb[o] = __float2bfloat16_rn(v + (ep.bias ? ep.bias[col] : 0.f)); break;
                    }
                }
            }
        }
    }
    if (abort_flag && tid == 0 && ep.err) atomicExch(ep.err, 1);
    if (abort_flag) tc::mbar_wait(bar_a, phase ^ 1u);  // let an outstanding commit land before freeing TMEM
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kTmemCols)
                     : "memory");
}

cudaError_t launch_gemm_tc(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                           int ksplit, const Epilogue &ep, cudaStream_t s)
{
    if (M < 1 || N < 16 || N % 16 || K < 16 || K % 16 || lda % 8 || ldb % 8 || ksplit < 1) return cudaErrorInvalidValue;
    if (((uintptr_t)A | (uintptr_t)B) & 15) return cudaErrorInvalidValue;
    int kslice = (K + ksplit - 1) / ksplit;
    kslice = (kslice + tc::kSliceK - 1) / tc::kSliceK * tc::kSliceK;
    const dim3 grid((M + tc::kTileM - 1) / tc::kTileM, (N + tc::kTileN - 1) / tc::kTileN, (K + kslice - 1) / kslice);
    // 23 KB of unused dynamic shared memory hold residency at 4 CTAs per SM,
    // whose 4 x 128 TMEM columns are exactly the SM's 512: no CTA waits in alloc
    k_gemm_tc<<<grid, tc::kThreads, kPadSmem, s>>>(A, lda, B, ldb, M, N, K, kslice, ep);
    return cudaGetLastError();
}

}  // namespace fj

extern "C" int fj_tc_gemm(int M, int N, int K, const void *A, int lda, const void *B, int ldb, float *C, int ldc,
                          int ksplit, void *stream)
{
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return FJ_ERR_NOMEM;
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(err, 0, sizeof(int), s);
    fj::tc::Epilogue ep{ksplit > 1 ? fj::tc::kEpiAtomicF32 : fj::tc::kEpiStoreF32, nullptr, C, nullptr, nullptr, nullptr,
                        ldc, err};
    if (ksplit > 1) cudaMemsetAsync(C, 0, (size_t)(M - 1) * ldc * sizeof(float) + N * sizeof(float), s);
    cudaError_t e = fj::launch_gemm_tc((const __nv_bfloat16 *)A, lda, (const __nv_bfloat16 *)B, ldb, M, N, K, ksplit,
                                       ep, s);
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(err);
    if (e != cudaSuccess) return e == cudaErrorInvalidValue ? FJ_ERR_ARG : FJ_ERR_CUDA;
    return h ? FJ_ERR_CUDA : FJ_OK;
}
