// fj_tc.cuh -- BF16 GEMM on the 5th-generation tensor cores (tcgen05).
//
// C[M][N] (+epilogue) = A[M][K] * B[N][K]^T, A and B BF16 with K contiguous
// (K-major), FP32 accumulation in tensor memory.  One CTA of 128 threads owns
// a 128 x BN tile of C (BN <= 128, a multiple of 16): its warp 0 allocates
// 128 TMEM columns, all threads stage 128 x 64 slices of A and BN x 64 of B in
// shared memory in the canonical no-swizzle K-major layout, one thread issues
// four tcgen05.mma (K = 16 each) per slice and commits them to an mbarrier,
// and after the last slice every warp reads its 32 TMEM lanes (rows) with
// tcgen05.ld for the epilogue.  Waits on the mbarrier are bounded in time;
// a CTA that gives up sets the error flag, drains, frees its TMEM and returns.
//
// Shared-memory operand layout (per 16-wide K step): core matrices of 8 rows
// x 16 bytes, 128 contiguous bytes each; the two core matrices of a row group
// that cover K = 0..7 and 8..15 are adjacent (leading-dimension byte offset
// 128), row groups are 256 bytes apart (stride-dimension byte offset 256).
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace fj {
namespace tc {

constexpr int kThreads = 128;
constexpr int kTileM = 128;
constexpr int kTileN = 128;
constexpr int kSliceK = 64;
constexpr int kTmemCols = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

enum : int {
    kEpiStoreF32 = 0,    // outf = acc (+ bias)
    kEpiAtomicF32 = 1,   // outf += acc (split K)
    kEpiBiasGelu = 2,    // z = acc + bias -> zout (f32), outb = gelu(z) (bf16)
    kEpiGeluGrad = 3,    // outb = acc * gelu'(zin) (bf16)
    kEpiStoreBF16 = 4,   // outb = acc (+ bias) (bf16)
};

struct Epilogue {
    int mode;
    const float *bias;    // [N] or null
    float *outf;          // f32 output, row stride ldo
    __nv_bfloat16 *outb;  // bf16 output, row stride ldo
    float *zout;          // kEpiBiasGelu: pre-activations, row stride ldo
    const float *zin;     // kEpiGeluGrad: pre-activations, row stride ldo
    int ldo;
    int *err;             // set to 1 when a wait gave up
};

// tanh-form GELU and its derivative
__device__ __forceinline__ float gelu(float z)
{
    const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
    return 0.5f * z * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float z)
{
    const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
    const float t = tanhf(u);
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * 0.7978845608028654f * (1.f + 3.f * 0.044715f * z * z);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading/stride byte offsets
// (bits 0-13, 16-29, 32-45, each >> 4), descriptor version 1 (bits 46-47),
// base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 (bits 17-22), M >> 4 (bits 24-28)
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bounded wait for the completion of mbarrier phase `parity`
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const unsigned long long t0 = global_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

}  // namespace tc
}  // namespace fj
