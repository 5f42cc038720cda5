// fj_mlp.cu -- tensor-core (tcgen05) GEMM and the action surrogate built on it.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

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
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kPadSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
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

// ======================================================================
// The action surrogate: an MLP 16 -> 128 -> 128 -> 128 -> 128 -> 16 (GELU),
// inputs padded from 13 features, outputs 0 and 1 used (log Jr, log Jz),
// trained with Adam on mean-squared error.  Master weights FP32, BF16 copies
// (and their transposes, for the backward data products) feed the GEMMs.
// ======================================================================
namespace fj {
namespace {

constexpr int kIn = 16, kHid = 128, kOut = 16, kLayers = 5, kUsedOut = 2;

__global__ void k_to_bf16(int n, const float *x, __nv_bfloat16 *y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// y[c][r] = x[r][c] (bf16, r < R, c < C), 32 x 32 tiles through shared memory
__global__ void k_transpose_bf16(int R, int C, const __nv_bfloat16 *x, int ldx, __nv_bfloat16 *y, int ldy)
{
    __shared__ __nv_bfloat16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < R && c < C) t[i][threadIdx.x] = x[(size_t)r * ldx + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < R && c < C) y[(size_t)c * ldy + r] = t[threadIdx.x][i];
    }
}

// f32 -> transposed bf16 copy of a weight matrix W[rows][cols] -> WT[cols][rows]
__global__ void k_weight_t(int rows, int cols, const float *w, __nv_bfloat16 *wt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int r = i / cols, c = i % cols;
    wt[(size_t)c * rows + r] = __float2bfloat16_rn(w[i]);
}

// dY = 2 w (Y - T) / (B * kUsedOut) on the used outputs (bf16, zero elsewhere),
// w = per-row weight (1 if wt is null); loss = the weighted mean of squares
__global__ void k_mse_grad(int B, const float *y, const float *t, const float *wt, __nv_bfloat16 *dy, float *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < B * kOut) {
        const int b = i / kOut, o = i % kOut;
        float g = 0.f;
        if (o < kUsedOut) {
            const float w = wt ? wt[b] : 1.f;
            const float d = y[i] - t[b * kUsedOut + o];
            g = 2.f * w * d / (float)(B * kUsedOut);
            l = w * d * d;
        }
        dy[i] = __float2bfloat16_rn(g);
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l / (float)(B * kUsedOut));
}

// column sums of a [B][N] bf16 matrix into g[N] (f32, accumulated)
__global__ void k_colsum(int B, int N, const __nv_bfloat16 *x, float *g)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float s = 0.f;
    for (int b = blockIdx.y; b < B; b += gridDim.y) s += __bfloat162float(x[(size_t)b * N + c]);
    atomicAdd(g + c, s);
}

// Adam (Kingma & Ba 2015) on n parameters; bias-corrected step size alpha_t
__global__ void k_adam(int n, float *w, const float *g, float *m, float *v, float alpha_t, float b1, float b2,
                       float eps, const unsigned char *mask)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (mask && !mask[i])) return;
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    w[i] -= alpha_t * m[i] / (sqrtf(v[i]) + eps);
}

}  // namespace
}  // namespace fj

struct fj_surrogate {
    fj_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    int batch = 0;  // samples per training step
    int rows[5], cols[5];
    size_t woff[5], boff[5], nparam = 0;
    // parameters (f32 masters), gradients, Adam moments, masks of trainable entries
    float *P = nullptr, *G = nullptr, *Mom = nullptr, *Var = nullptr;
    unsigned char *mask = nullptr;
    __nv_bfloat16 *Wb = nullptr, *WbT = nullptr;  // bf16 weights and transposes, at woff
    // activations of one batch
    __nv_bfloat16 *X = nullptr, *XT = nullptr, *H = nullptr, *HT = nullptr, *dZ = nullptr, *dZT = nullptr;
    float *Z = nullptr, *Y = nullptr, *loss = nullptr;
    int *err = nullptr;
    __nv_bfloat16 *Xi = nullptr, *Hi = nullptr;  // inference workspace
    float *Xf = nullptr, *Yf = nullptr;           // f32 features / outputs of one inference pass
    float *fitX = nullptr, *fitT = nullptr, *fitW = nullptr;  // training rows (fj_surrogate_fit), fit_cap rows
    long long *fitIdx = nullptr;
    long long fit_cap = 0;
    double *partial = nullptr;                    // surrogate moment sums [npts][6]
    long long partial_cap = 0;
    double *points = nullptr;                     // per grid point: Phi, Ve
    long long points_cap = 0;
    long long step = 0;
    std::vector<void *> owned;
};

namespace {

using fj::tc::Epilogue;

constexpr int kInferRows = 1 << 20;  // rows per inference pass (2 x 256 MB of activations)

int sg_alloc(fj_surrogate *s, void **p, size_t bytes)
{
    if (cudaMalloc(p, bytes) != cudaSuccess) return FJ_ERR_NOMEM;
    s->owned.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes, s->stream) == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}

#define SG_CUDA(call)                                   \
    do {                                                \
        if ((call) != cudaSuccess) return FJ_ERR_CUDA;  \
    } while (0)

// bf16 copies of the weights and of their transposes
int sg_refresh(fj_surrogate *s)
{
    for (int l = 0; l < fj::kLayers; l++) {
        const int n = s->rows[l] * s->cols[l];
        fj::k_to_bf16<<<(n + 255) / 256, 256, 0, s->stream>>>(n, s->P + s->woff[l], s->Wb + s->woff[l]);
        fj::k_weight_t<<<(n + 255) / 256, 256, 0, s->stream>>>(s->rows[l], s->cols[l], s->P + s->woff[l],
                                                               s->WbT + s->woff[l]);
    }
    return cudaGetLastError() == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}

int sg_gemm(fj_surrogate *s, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
            int ksplit, Epilogue ep)
{
    ep.err = s->err;
    return fj::launch_gemm_tc(A, lda, B, ldb, M, N, K, ksplit, ep, s->stream) == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}

int sg_transpose(fj_surrogate *s, int R, int C, const __nv_bfloat16 *x, __nv_bfloat16 *y)
{
    const dim3 grid((C + 31) / 32, (R + 31) / 32);
    fj::k_transpose_bf16<<<grid, dim3(32, 8), 0, s->stream>>>(R, C, x, C, y, R);
    return cudaGetLastError() == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}

// forward pass of n rows of X (bf16 [n][16]) through the layers; keep
// (training, n = batch): pre-activations to Z[l] and activations to H[l];
// else the hidden layers ping-pong between the two halves of Hbuf, each of
// hcap rows.  Output f32 [n][16] in out.
int sg_forward(fj_surrogate *s, const __nv_bfloat16 *X, int n, float *out, bool keep, __nv_bfloat16 *Hbuf,
               size_t hcap)
{
    const size_t hb = hcap * fj::kHid;
    const __nv_bfloat16 *in = X;
    int inw = fj::kIn, rc;
    for (int l = 0; l < 4; l++) {
        __nv_bfloat16 *h = Hbuf + (keep ? l : (l & 1)) * hb;
        Epilogue ep{fj::tc::kEpiBiasGelu, s->P + s->boff[l], nullptr, h, keep ? s->Z + l * hb : nullptr, nullptr,
                    fj::kHid, nullptr};
        if ((rc = sg_gemm(s, in, inw, s->Wb + s->woff[l], s->cols[l], n, fj::kHid, inw, 1, ep))) return rc;
        in = h;
        inw = fj::kHid;
    }
    Epilogue ep{fj::tc::kEpiStoreF32, s->P + s->boff[4], out, nullptr, nullptr, nullptr, fj::kOut, nullptr};
    return sg_gemm(s, in, fj::kHid, s->Wb + s->woff[4], fj::kHid, n, fj::kOut, fj::kHid, 1, ep);
}

// gradients of the mean-squared error of one training batch (after sg_forward
// with keep) into G; T f32 [batch][2]
int sg_backward(fj_surrogate *s, const float *T, const float *Wt)
{
    const int B = s->batch, ks = (B + 4095) / 4096;
    const size_t hb = (size_t)B * fj::kHid;
    int rc;
    SG_CUDA(cudaMemsetAsync(s->G, 0, s->nparam * sizeof(float), s->stream));
    __nv_bfloat16 *dY = s->dZ + hb;  // [B][16], after the two dZ buffers' first
    fj::k_mse_grad<<<(B * fj::kOut + 255) / 256, 256, 0, s->stream>>>(B, s->Y, T, Wt, dY, s->loss);
    // output layer: gW4 = dY^T H3, gb4 = colsum(dY), dZ3 = (dY W4) * gelu'(Z3)
    if ((rc = sg_transpose(s, B, fj::kOut, dY, s->dZT))) return rc;
    if ((rc = sg_transpose(s, B, fj::kHid, s->H + 3 * hb, s->HT))) return rc;
    Epilogue gw{fj::tc::kEpiAtomicF32, nullptr, s->G + s->woff[4], nullptr, nullptr, nullptr, fj::kHid, nullptr};
    if ((rc = sg_gemm(s, s->dZT, B, s->HT, B, fj::kOut, fj::kHid, B, ks, gw))) return rc;
    fj::k_colsum<<<dim3(1, 64), fj::kOut, 0, s->stream>>>(B, fj::kOut, dY, s->G + s->boff[4]);
    __nv_bfloat16 *dz = s->dZ, *dz2 = s->dZ + (size_t)2 * hb;
    Epilogue gg{fj::tc::kEpiGeluGrad, nullptr, nullptr, dz, nullptr, s->Z + 3 * hb, fj::kHid, nullptr};
    if ((rc = sg_gemm(s, dY, fj::kOut, s->WbT + s->woff[4], fj::kOut, B, fj::kHid, fj::kOut, 1, gg))) return rc;
    for (int l = 3; l >= 0; l--) {
        // gW_l = dZ_l^T H_{l-1} (X for l = 0), gb_l = colsum(dZ_l)
        const __nv_bfloat16 *prev = l > 0 ? s->H + (size_t)(l - 1) * hb : s->X;
        const int pw = l > 0 ? fj::kHid : fj::kIn;
        if ((rc = sg_transpose(s, B, fj::kHid, dz, s->dZT))) return rc;
        if ((rc = sg_transpose(s, B, pw, prev, s->HT))) return rc;
        Epilogue g2{fj::tc::kEpiAtomicF32, nullptr, s->G + s->woff[l], nullptr, nullptr, nullptr, pw, nullptr};
        if ((rc = sg_gemm(s, s->dZT, B, s->HT, B, fj::kHid, pw, B, ks, g2))) return rc;
        fj::k_colsum<<<dim3(1, 64), fj::kHid, 0, s->stream>>>(B, fj::kHid, dz, s->G + s->boff[l]);
        if (l == 0) break;
        // dZ_{l-1} = (dZ_l W_l) * gelu'(Z_{l-1})
        Epilogue g3{fj::tc::kEpiGeluGrad, nullptr, nullptr, dz2, nullptr, s->Z + (size_t)(l - 1) * hb, fj::kHid,
                    nullptr};
        if ((rc = sg_gemm(s, dz, fj::kHid, s->WbT + s->woff[l], fj::kHid, B, fj::kHid, fj::kHid, 1, g3))) return rc;
        std::swap(dz, dz2);
    }
    return cudaGetLastError() == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}

// the inference workspace: kInferRows rows per pass (bf16 inputs, two hidden
// buffers, f32 features and outputs), allocated on first use
fj::DFDev sg_df(const fj_df_params *df)
{
    fj::DFDev d;
    d.kind = df->kind; d.alpha = df->alpha; d.beta = df->beta; d.J0 = df->J0;
    d.norm = df->mass / pow(df->J0, 3); d.tpi3 = pow(2 * fj::kPI, 3.);
    d.dphi_h = df->dphi_h; d.dz_h = df->dz_h; d.dphi_g = df->dphi_g; d.dz_g = df->dz_g; d.chi = df->chi; d.k = df->k;
    return d;
}

int sg_infer_buffers(fj_surrogate *s)
{
    if (s->Xi && s->Hi && s->Xf && s->Yf) return FJ_OK;
    int rc;
    void *q;
    if ((rc = sg_alloc(s, &q, (size_t)kInferRows * fj::kIn * sizeof(__nv_bfloat16)))) return rc;
    s->Xi = (__nv_bfloat16 *)q;
    if ((rc = sg_alloc(s, &q, (size_t)2 * kInferRows * fj::kHid * sizeof(__nv_bfloat16)))) return rc;
    s->Hi = (__nv_bfloat16 *)q;
    if ((rc = sg_alloc(s, &q, (size_t)kInferRows * fj::kIn * sizeof(float)))) return rc;
    s->Xf = (float *)q;
    if ((rc = sg_alloc(s, &q, (size_t)kInferRows * fj::kOut * sizeof(float)))) return rc;
    s->Yf = (float *)q;
    return FJ_OK;
}

int sg_check_err(fj_surrogate *s)
{
    int h = 0;
    SG_CUDA(cudaMemcpyAsync(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    SG_CUDA(cudaStreamSynchronize(s->stream));
    return h ? FJ_ERR_CUDA : FJ_OK;
}

// one training step on rows [r0, r0 + batch) of X f32 [n][16], T f32 [n][2]
int sg_step(fj_surrogate *s, const float *X, const float *T, const float *Wt, float lr)
{
    const int B = s->batch;
    fj::k_to_bf16<<<(B * fj::kIn + 255) / 256, 256, 0, s->stream>>>(B * fj::kIn, X, s->X);
    int rc;
    if ((rc = sg_forward(s, s->X, B, s->Y, true, s->H, B))) return rc;
    if ((rc = sg_backward(s, T, Wt))) return rc;
    s->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float alpha = lr * sqrtf(1.f - powf(b2, (float)s->step)) / (1.f - powf(b1, (float)s->step));
    fj::k_adam<<<(unsigned)((s->nparam + 255) / 256), 256, 0, s->stream>>>((int)s->nparam, s->P, s->G, s->Mom, s->Var,
                                                                           alpha, b1, b2, 1e-8f, s->mask);
    return sg_refresh(s);
}

}  // namespace

extern "C" {

int fj_surrogate_create(fj_ctx *ctx, int batch, unsigned long long seed, fj_surrogate **out)
{
    if (!out || batch < 128 || batch % 128) return FJ_ERR_ARG;
    fj_surrogate *s = new fj_surrogate;
    s->ctx = ctx;
    s->stream = ctx ? fj::context_stream(ctx) : nullptr;
    s->batch = batch;
    const int rows[5] = {fj::kHid, fj::kHid, fj::kHid, fj::kHid, fj::kOut};
    const int cols[5] = {fj::kIn, fj::kHid, fj::kHid, fj::kHid, fj::kHid};
    size_t o = 0;
    for (int l = 0; l < fj::kLayers; l++) {
        s->rows[l] = rows[l]; s->cols[l] = cols[l];
        s->woff[l] = o; o += (size_t)rows[l] * cols[l];
        s->boff[l] = o; o += rows[l];
    }
    s->nparam = o;
    // seeded initialisation: uniform(-a, a), a = sqrt(6 / (fan_in + fan_out)); zero biases; the
    // output rows beyond the two used outputs are zero and frozen
    std::vector<float> p(o, 0.f);
    std::vector<unsigned char> mask(o, 1);
    unsigned long long z = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto uni = [&]() {  // splitmix64
        z += 0x9E3779B97F4A7C15ull;
        unsigned long long x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < fj::kLayers; l++) {
        const double a = sqrt(6.0 / (rows[l] + cols[l]));
        for (int r = 0; r < rows[l]; r++)
            for (int c = 0; c < cols[l]; c++) p[s->woff[l] + (size_t)r * cols[l] + c] = (float)(a * (2 * uni() - 1));
        if (l == fj::kLayers - 1)
            for (int r = fj::kUsedOut; r < rows[l]; r++) {
                for (int c = 0; c < cols[l]; c++) {
                    p[s->woff[l] + (size_t)r * cols[l] + c] = 0.f;
                    mask[s->woff[l] + (size_t)r * cols[l] + c] = 0;
                }
                mask[s->boff[l] + r] = 0;
            }
    }
    const size_t hb = (size_t)batch * fj::kHid;
    int rc = FJ_OK;
    void *q;
    auto A = [&](void **dst, size_t bytes) { if (!rc) rc = sg_alloc(s, dst, bytes); };
    A(&q, o * sizeof(float)); s->P = (float *)q;
    A(&q, o * sizeof(float)); s->G = (float *)q;
    A(&q, o * sizeof(float)); s->Mom = (float *)q;
    A(&q, o * sizeof(float)); s->Var = (float *)q;
    A(&q, o); s->mask = (unsigned char *)q;
    A(&q, o * sizeof(__nv_bfloat16)); s->Wb = (__nv_bfloat16 *)q;
    A(&q, o * sizeof(__nv_bfloat16)); s->WbT = (__nv_bfloat16 *)q;
    A(&q, (size_t)batch * fj::kIn * sizeof(__nv_bfloat16)); s->X = (__nv_bfloat16 *)q;
    A(&q, 4 * hb * sizeof(__nv_bfloat16)); s->H = (__nv_bfloat16 *)q;
    A(&q, hb * sizeof(__nv_bfloat16)); s->HT = (__nv_bfloat16 *)q;
    A(&q, 4 * hb * sizeof(float)); s->Z = (float *)q;
    A(&q, (3 * hb) * sizeof(__nv_bfloat16)); s->dZ = (__nv_bfloat16 *)q;
    A(&q, hb * sizeof(__nv_bfloat16)); s->dZT = (__nv_bfloat16 *)q;
    A(&q, (size_t)batch * fj::kOut * sizeof(float)); s->Y = (float *)q;
    A(&q, sizeof(float)); s->loss = (float *)q;
    A(&q, sizeof(int)); s->err = (int *)q;
    if (!rc && cudaMemcpyAsync(s->P, p.data(), o * sizeof(float), cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        rc = FJ_ERR_CUDA;
    if (!rc && cudaMemcpyAsync(s->mask, mask.data(), o, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        rc = FJ_ERR_CUDA;
    if (!rc) rc = sg_refresh(s);
    if (!rc && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = FJ_ERR_CUDA;
    if (rc) { fj_surrogate_destroy(s); return rc; }
    *out = s;
    return FJ_OK;
}

int fj_surrogate_destroy(fj_surrogate *s)
{
    if (!s) return FJ_ERR_ARG;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void *p : s->owned) cudaFree(p);
    delete s;
    return FJ_OK;
}

int fj_surrogate_params(fj_surrogate *s, double *host_out, const double *host_in)
{
    if (!s) return FJ_ERR_ARG;
    std::vector<float> p(s->nparam);
    if (host_in) {
        for (size_t i = 0; i < s->nparam; i++) p[i] = (float)host_in[i];
        SG_CUDA(cudaMemcpyAsync(s->P, p.data(), s->nparam * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        int rc = sg_refresh(s);
        if (rc) return rc;
    }
    if (host_out) {
        SG_CUDA(cudaMemcpyAsync(p.data(), s->P, s->nparam * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        SG_CUDA(cudaStreamSynchronize(s->stream));
        for (size_t i = 0; i < s->nparam; i++) host_out[i] = p[i];
    }
    SG_CUDA(cudaStreamSynchronize(s->stream));
    return FJ_OK;
}

long long fj_surrogate_nparam(const fj_surrogate *s) { return s ? (long long)s->nparam : -1; }

int fj_surrogate_gradients(fj_surrogate *s, const float *X, const float *T, double *grad_out, double *loss)
{
    if (!s || !X || !T || !grad_out) return FJ_ERR_ARG;
    const int B = s->batch;
    SG_CUDA(cudaMemsetAsync(s->loss, 0, sizeof(float), s->stream));
    fj::k_to_bf16<<<(B * fj::kIn + 255) / 256, 256, 0, s->stream>>>(B * fj::kIn, X, s->X);
    int rc;
    if ((rc = sg_forward(s, s->X, B, s->Y, true, s->H, B))) return rc;
    if ((rc = sg_backward(s, T, nullptr))) return rc;
    if ((rc = sg_check_err(s))) return rc;
    std::vector<float> g(s->nparam);
    float l = 0;
    SG_CUDA(cudaMemcpyAsync(g.data(), s->G, s->nparam * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    SG_CUDA(cudaMemcpyAsync(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    SG_CUDA(cudaStreamSynchronize(s->stream));
    for (size_t i = 0; i < s->nparam; i++) grad_out[i] = g[i];
    if (loss) *loss = l;
    return FJ_OK;
}

static int sg_train(fj_surrogate *s, const float *X, const float *T, const float *Wt, long long n, int epochs,
                    float lr, double *final_loss);

int fj_surrogate_train(fj_surrogate *s, const float *X, const float *T, long long n, int epochs, float lr,
                       double *final_loss)
{
    return sg_train(s, X, T, nullptr, n, epochs, lr, final_loss);
}

}  // extern "C"

static int sg_train(fj_surrogate *s, const float *X, const float *T, const float *Wt, long long n, int epochs,
                    float lr, double *final_loss)
{
    if (!s || !X || !T || n < s->batch || epochs < 1 || !(lr > 0)) return FJ_ERR_ARG;
    const long long steps = n / s->batch;
    int rc;
    for (int e = 0; e < epochs; e++)
        for (long long k = 0; k < steps; k++) {
            if (e == epochs - 1 && k == steps - 1) SG_CUDA(cudaMemsetAsync(s->loss, 0, sizeof(float), s->stream));
            if ((rc = sg_step(s, X + (size_t)k * s->batch * fj::kIn, T + (size_t)k * s->batch * fj::kUsedOut,
                              Wt ? Wt + (size_t)k * s->batch : nullptr, lr)))
                return rc;
        }
    if ((rc = sg_check_err(s))) return rc;
    if (final_loss) {
        float l = 0;
        SG_CUDA(cudaMemcpyAsync(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        SG_CUDA(cudaStreamSynchronize(s->stream));
        *final_loss = l;
    }
    return FJ_OK;
}

extern "C" {

int fj_surrogate_predict(fj_surrogate *s, const float *X, long long n, float *Y)
{
    if (!s || !X || !Y || n < 1) return FJ_ERR_ARG;
    int rc;
    if ((rc = sg_infer_buffers(s))) return rc;
    for (long long r0 = 0; r0 < n; r0 += kInferRows) {
        const int m = (int)std::min<long long>(kInferRows, n - r0);
        fj::k_to_bf16<<<(m * fj::kIn + 255) / 256, 256, 0, s->stream>>>(m * fj::kIn, X + (size_t)r0 * fj::kIn, s->Xi);
        if ((rc = sg_forward(s, s->Xi, m, Y + (size_t)r0 * fj::kOut, false, s->Hi, kInferRows))) return rc;
    }
    return sg_check_err(s);
}

}  // extern "C"

// ======================================================================
// Surrogate features, targets and the surrogate moment sums.
//
// Features of node (i, j, k) of grid point p = (ar[n], cos theta_g) (table
// values at the grid radius, nothing interpolated):
//   0: (log r - mu) / sigma over the grid's log-radius range,   1: cos theta,
//   2, 3, 4: vR / Ve, vz / Ve, vphi / Ve (the node's rule coordinates),
//   5: Phi_0(r) / Phi_0(ar[0]),   6..12: Phi_l(r) / |Phi_0(r)|, l = 1..7,
//   13: log(H / Phi(point)) / 5 (-> -inf as the orbit becomes unbound),
//   14, 15: 0.
// Outputs: log h and log g of the double-power-law DF (DF.cpp:65-76),
// h = Jr + dphi_h |Jphi| + dz_h Jz and g likewise: the DF needs nothing else
// (Jphi = R vphi is exact), and their logs are smooth with no cancellation.
// Regressing log J of each action is dominated by the circular (Jr = 0) and
// near-unbound tails; recovering Jr + Jz from a predicted total action loses
// the near-circular in-plane orbits, where the DF peaks.
// ======================================================================
namespace fj {

struct SgGrid {
    PotView P;
    const double *ci;  // polar nodes
    int ngauss, nq;
    const double *xq;
    double lmu, lsig;     // log-radius normalisation
    const double *point;  // [npts][2]: Phi at the point, escape speed Ve
};

__global__ void k_sg_points(SgGrid g, int npts, double *point)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int n = p / g.ngauss, gg = p % g.ngauss;
    const double c = g.ci[gg], si = sqrt(1 - c * c);
    const double Phi_h = pot_phi(g.P, g.P.ar[n] * si, g.P.ar[n] * c);
    const double rmax = g.P.ar[g.P.nr - 1];
    point[2 * p] = Phi_h;
    point[2 * p + 1] = sqrt(-2 * (Phi_h - pot_phi(g.P, 10 * rmax, 10 * rmax)));
}

__device__ __forceinline__ void sg_velocity(const SgGrid &g, int p, int node, double &V0, double &V1, double &V2,
                                            double &H, double &R)
{
    const int nq = g.nq;
    const double Phi_h = g.point[2 * p], Ve = g.point[2 * p + 1];
    V0 = 1e-6 + Ve * g.xq[node / (nq * nq)];
    V1 = 1e-6 + Ve * g.xq[(node / nq) % nq];
    V2 = 1e-6 + Ve * g.xq[node % nq];
    H = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h;
    const double c = g.ci[p % g.ngauss];
    R = g.P.ar[p / g.ngauss] * sqrt(1 - c * c);
}

// features of nodes idx[0..m) (idx = p * nq^3 + node; NULL: rows 0..m-1 are nodes
// first .. first+m-1), X f32 [m][16]
__global__ void k_sg_features(SgGrid g, const long long *idx, long long first, long long m, float *X)
{
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= m) return;
    const long long id = idx ? idx[s] : first + s;
    const int nq = g.nq, nq3 = nq * nq * nq;
    const int p = (int)(id / nq3), node = (int)(id % nq3);
    const int n = p / g.ngauss, gg = p % g.ngauss, np_ = g.P.npoly;
    float *x = X + s * 16;
    x[0] = (float)((log(g.P.ar[n]) - g.lmu) / g.lsig);
    x[1] = (float)g.ci[gg];
    x[2] = (float)g.xq[node / (nq * nq)];
    x[3] = (float)g.xq[node % nq];
    x[4] = (float)g.xq[(node / nq) % nq];
    const double p0 = g.P.phil[n * np_];
    x[5] = (float)(p0 / g.P.phil[0]);
    for (int l = 1; l < 8; l++) x[5 + l] = l < np_ ? (float)(g.P.phil[n * np_ + l] / fabs(p0)) : 0.f;
    double V0, V1, V2, H, R;
    sg_velocity(g, p, node, V0, V1, V2, H, R);
    x[13] = (float)(log(fmax(H / g.point[2 * p], 1e-12)) / 5);
    x[14] = x[15] = 0.f;
}

// training rows from exact actions J [npts * nq^3][2] (unbound or E >= 0: NaN or
// 1e31): sample s takes node hash(seed, s) (the next valid one after it, within 64)
__global__ void k_sg_sample(SgGrid g, DFDev df, const float *J, const double *rho, const double *wq, long long total,
                            unsigned long long seed, long long ns, long long *idx, float *T, float *Wt)
{
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= ns) return;
    unsigned long long hs = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(s + 1);
    hs = (hs ^ (hs >> 30)) * 0xBF58476D1CE4E5B9ull;
    hs = (hs ^ (hs >> 27)) * 0x94D049BB133111EBull;
    hs ^= hs >> 31;
    long long id = (long long)(hs % (unsigned long long)total);
    bool ok = false;
    for (int t = 0; t < 64 && !ok; t++) {
        const long long q = (id + t) % total;
        const float jr = J[2 * q], jz = J[2 * q + 1];
        if (jr >= 0.f && jz >= 0.f && jr < 1e30f && jz < 1e30f) { id = q; ok = true; }
    }
    idx[s] = id;
    const int nq3 = g.nq * g.nq * g.nq, p = (int)(id / nq3), node = (int)(id % nq3);
    double V0, V1, V2, H, R;
    sg_velocity(g, p, node, V0, V1, V2, H, R);
    const double jr = ok ? J[2 * id] : 0., jz = ok ? J[2 * id + 1] : 0., jp = fabs(R * V1);
    const double h = jr + df.dphi_h * jp + df.dz_h * jz, gg = jr + df.dphi_g * jp + df.dz_g * jz;
    T[2 * s] = (float)log(h + 1e-12);
    T[2 * s + 1] = (float)log(gg + 1e-12);
    // weight: a floor plus the node's share of its point's density (x nq^3)
    float w = ok ? 1.f : 0.f;
    if (ok && rho && rho[p] > 0) {
        const double Jphi = R * V1, Ve = g.point[2 * p + 1];
        double f = df.norm * fmax(0., pow(1. + df.J0 / h, df.alpha) / pow(1. + gg / df.J0, df.beta)) / df.tpi3;
        if (df.chi != 0.) f += df.k * tanh(df.chi * Jphi / df.J0) * f;
        const int nq = g.nq;
        const double share = wq[node / (nq * nq)] * wq[(node / nq) % nq] * wq[node % nq] * Ve * Ve * Ve * f / rho[p];
        w = (float)fmin(100., 0.2 + (double)nq3 * share);
    }
    Wt[s] = w;
}

// moment sums of grid point p0 + blockIdx.x from the surrogate outputs Y (rows from
// node `first` of the grid, [.][16])
__global__ void __launch_bounds__(128) k_sg_moments(SgGrid g, const double *wq, DFDev df, const float *Y,
                                                    long long first, int p0, double *partial)
{
    __shared__ double s_red[6 * 4];
    const int p = p0 + blockIdx.x, nq = g.nq, nq3 = nq * nq * nq;
    const double Ve = g.point[2 * p + 1], jacob = Ve * Ve * Ve;
    double m[6] = {0, 0, 0, 0, 0, 0};
    for (int node = threadIdx.x; node < nq3; node += blockDim.x) {
        double V0, V1, V2, H, R;
        sg_velocity(g, p, node, V0, V1, V2, H, R);
        if (!(H < 0)) continue;
        const float *y = Y + ((long long)p * nq3 + node - first) * 16;
        const float Jphi = (float)(R * V1), J0 = (float)df.J0;
        const float h = expf(y[0]), gg = expf(y[1]);
        const float ev = (float)df.norm *
                         fmaxf(0.f, powf(1.f + J0 / h, (float)df.alpha) / powf(1.f + gg / J0, (float)df.beta)) /
                         (float)df.tpi3;
        float f = df.chi == 0. ? ev : ev + (float)df.k * tanhf((float)df.chi * Jphi / J0) * ev;
        if (isnan(f)) f = 0.f;
        const int i = node / (nq * nq), j = (node / nq) % nq, k = node % nq;
        const double jd = (wq[i] * wq[j] * wq[k]) * (jacob * (double)f);
        m[0] += jd;
        m[1] += jd * V1;
        m[2] += jd * V0 * V0;
        m[3] += jd * V1 * V1;
        m[4] += jd * V2 * V2;
        m[5] += jd * V0 * V2;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = 0; q < 6; q++) {
        double v = m[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) s_red[warp * 6 + q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w = 0; w < 4; w++) s += s_red[w * 6 + threadIdx.x];
        partial[(size_t)p * 6 + threadIdx.x] = s;
    }
}

}  // namespace fj

// ======================================================================
// Fused surrogate moments: features, the MLP on the tensor cores and the DF
// moment sums of one grid point's bound nodes in one kernel.  One CTA per
// (grid point, node range); two groups of four warps each own a 128-node
// tile in flight (own activation buffer, 128 TMEM columns, mbarrier) and
// share the five layers' BF16 weights, resident in shared memory in the
// canonical K-major layout.  Per tile: each thread writes its node's 16
// features into the operand buffer; one thread issues the layer's
// tcgen05.mma chain; after the commit the group reads the accumulators back
// (tcgen05.ld), applies bias and GELU and writes the BF16 activations into
// the same buffer as the next layer's operand; the output layer's log h and
// log g go straight into the DF and the FP64 moment sums.
// ======================================================================
namespace fj {

struct SgWeights {
    const __nv_bfloat16 *W[5];  // [rows][cols] row-major
    const float *b[5];
};

constexpr int kFusedThreads = 256;     // two groups of 128
constexpr int kFusedMaxNodes = 12288;  // node range of one CTA (bound-node list in shared memory)

// canonical no-swizzle K-major offset (bytes) of element (row, k) of a [rows][K]
// bf16 operand: K steps of 16 are rows*32 bytes apart
__device__ __forceinline__ uint32_t kmaj_off(int row, int k, int rows)
{
    return (uint32_t)((k >> 4) * rows * 32 + (row >> 3) * 256 + ((k >> 3) & 1) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared memory: W0 4 KB | W1..W3 96 KB | W4 4 KB | biases 2112 B | 2 x act 32 KB | list | misc
constexpr int kSmW0 = 0, kSmW1 = 4096, kSmW4 = kSmW1 + 3 * 32768, kSmBias = kSmW4 + 4096;
constexpr int kSmAct = kSmBias + 4 * 128 * 4 + 16 * 4 + 192;  // 1024-aligned below
constexpr int kSmActAligned = (kSmAct + 1023) / 1024 * 1024;
constexpr int kSmList = kSmActAligned + 2 * 32768;
constexpr size_t fused_smem_bytes() { return (size_t)kSmList + kFusedMaxNodes * 2 + 256; }

__global__ void __launch_bounds__(kFusedThreads, 1) k_sg_fused(SgGrid g, SgWeights wts, const double *wq, DFDev df,
                                                               int blocks_per_point, double *partial, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) unsigned long long bars[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_wc[8];
    __shared__ double s_red[8 * 6];
    unsigned short *s_list = (unsigned short *)(sm + kSmList);
    float *s_bias = (float *)(sm + kSmBias);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, grp = tid >> 7, gt = tid & 127;
    const int B = blocks_per_point, p = blockIdx.x / B, chunk = blockIdx.x % B;
    const int nq = g.nq, nq3 = nq * nq * nq;
    const int n0 = (int)((long long)chunk * nq3 / B), n1 = (int)((long long)(chunk + 1) * nq3 / B);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc::smem_addr(&tmem_slot)),
                     "r"(256)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < 2) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc::smem_addr(&bars[tid])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // weights -> canonical layout (16-byte pieces), biases
    {
        const int rows[5] = {128, 128, 128, 128, 16}, cols[5] = {16, 128, 128, 128, 128};
        const int base[5] = {kSmW0, kSmW1, kSmW1 + 32768, kSmW1 + 65536, kSmW4};
        for (int l = 0; l < 5; l++) {
            const int pieces = rows[l] * cols[l] / 8;
            for (int q = tid; q < pieces; q += kFusedThreads) {
                const int r = q / (cols[l] / 8), k = (q % (cols[l] / 8)) * 8;
                *reinterpret_cast<uint4 *>(sm + base[l] + kmaj_off(r, k, rows[l])) =
                    *reinterpret_cast<const uint4 *>(wts.W[l] + (size_t)r * cols[l] + k);
            }
        }
        for (int q = tid; q < 4 * 128 + 16; q += kFusedThreads) s_bias[q] = wts.b[q >> 7 < 4 ? q >> 7 : 4][q < 512 ? q & 127 : q - 512];
    }
    // bound nodes of [n0, n1) in node order
    const double Phi_h = g.point[2 * p], Ve = g.point[2 * p + 1];
    int nbound = 0;
    for (int base = n0; base < n1; base += kFusedThreads) {
        const int node = base + tid;
        bool b = false;
        if (node < n1) {
            double V0, V1, V2, H, R;
            sg_velocity(g, p, node, V0, V1, V2, H, R);
            b = H < 0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, b);
        if (lane == 0) s_wc[warp] = __popc(bal);
        __syncthreads();
        int off = nbound, tot = 0;
        for (int w = 0; w < 8; w++) {
            if (w < warp) off += s_wc[w];
            tot += s_wc[w];
        }
        if (b) s_list[off + __popc(bal & ((1u << lane) - 1u))] = (unsigned short)(node - n0);
        __syncthreads();
        nbound += tot;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot + (uint32_t)(grp * 128);
    const uint32_t bar = tc::smem_addr(&bars[grp]);
    unsigned char *act = sm + kSmActAligned + grp * 32768;
    const uint32_t act_a = tc::smem_addr(act), w_a = tc::smem_addr(sm);
    const int n = p / g.ngauss, np_ = g.P.npoly;
    const double c = g.ci[p % g.ngauss], R = g.P.ar[n] * sqrt(1 - c * c), jacob = Ve * Ve * Ve;
    // per-point features
    float fx[14];
    fx[0] = (float)((log(g.P.ar[n]) - g.lmu) / g.lsig);
    fx[1] = (float)c;
    const double p0v = g.P.phil[n * np_];
    fx[5] = (float)(p0v / g.P.phil[0]);
    for (int l = 1; l < 8; l++) fx[5 + l] = l < np_ ? (float)(g.P.phil[n * np_ + l] / fabs(p0v)) : 0.f;
    double m[6] = {0, 0, 0, 0, 0, 0};
    uint32_t phase = 0;
    const float J0 = (float)df.J0;
    auto group_sync = [&]() { asm volatile("bar.sync %0, 128;" ::"r"(1 + grp) : "memory"); };
    // true in every thread of the group when v is true in any of them (also a group barrier)
    auto group_any = [&](bool v) {
        uint32_t r;
        asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, 128, p;\n"
                     " selp.u32 %0, 1, 0, q;\n}\n"
                     : "=r"(r)
                     : "r"((uint32_t)v), "r"(1 + grp)
                     : "memory");
        return r != 0;
    };
    // one layer's MMAs; false (in the whole group) if the completion wait gave up
    auto mma_chain = [&](int k_steps, uint32_t b_base, int n_cols) {
        if (gt == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t idesc = tc::idesc_bf16(128, n_cols);
            for (int ks = 0; ks < k_steps; ks++) {
                const uint64_t ad = tc::smem_desc(act_a + ks * 4096, 128, 256);
                const uint64_t bd = tc::smem_desc(w_a + b_base + ks * (n_cols * 32), 128, 256);
                const uint32_t acc = ks ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                         : "memory");
        }
        const bool ok = tc::mbar_wait(bar, phase);
        phase ^= 1u;
        const bool bad = group_any(!ok);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        return !bad;
    };
    const int ntiles = (nbound + 127) / 128;
    bool aborted = false;
    for (int t = grp; t < ntiles && !aborted; t += 2) {
        const int q = t * 128 + gt;
        const bool valid = q < nbound;
        const int node = valid ? n0 + s_list[q] : n0;
        double V0, V1, V2, H, Rr;
        sg_velocity(g, p, node, V0, V1, V2, H, Rr);
        // features of this thread's node, row gt of the K = 16 operand
        {
            float x[16];
            for (int i = 0; i < 14; i++) x[i] = fx[i];
            x[2] = (float)g.xq[node / (nq * nq)];
            x[3] = (float)g.xq[node % nq];
            x[4] = (float)g.xq[(node / nq) % nq];
            x[13] = valid ? (float)(log(fmax(H / Phi_h, 1e-12)) / 5) : 0.f;
            x[14] = x[15] = 0.f;
            for (int h8 = 0; h8 < 2; h8++) {
                __align__(16) __nv_bfloat16 v[8];
                for (int e = 0; e < 8; e++) v[e] = __float2bfloat16_rn(x[h8 * 8 + e]);
                *reinterpret_cast<uint4 *>(act + kmaj_off(gt, h8 * 8, 128)) = *reinterpret_cast<const uint4 *>(v);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        group_sync();
        // hidden layers: acc -> bias + GELU -> bf16 operand of the next layer
        for (int l = 0; l < 4 && !aborted; l++) {
            if (!mma_chain(l == 0 ? 1 : 8, l == 0 ? kSmW0 : kSmW1 + (l - 1) * 32768, 128)) { aborted = true; break; }
            for (int c0 = 0; c0 < 128; c0 += 16) {
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                __align__(16) __nv_bfloat16 v[16];
                for (int e = 0; e < 16; e++) v[e] = __float2bfloat16_rn(tc::gelu(__uint_as_float(r[e]) + s_bias[l * 128 + c0 + e]));
                *reinterpret_cast<uint4 *>(act + kmaj_off(gt, c0, 128)) = *reinterpret_cast<const uint4 *>(v);
                *reinterpret_cast<uint4 *>(act + kmaj_off(gt, c0 + 8, 128)) = *reinterpret_cast<const uint4 *>(v + 8);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            group_sync();
        }
        if (aborted) break;
        // output layer (N = 16): columns 0, 1 = log h, log g
        if (!mma_chain(8, kSmW4, 16)) { aborted = true; break; }
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(tmem + ((uint32_t)((warp & 3) * 32) << 16)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        group_sync();  // the operand buffer and TMEM are free for the group's next tile
        if (valid) {
            const float h = expf(__uint_as_float(r[0]) + s_bias[512]), gg = expf(__uint_as_float(r[1]) + s_bias[513]);
            const float Jphi = (float)(R * V1);
            const float ev = (float)df.norm *
                             fmaxf(0.f, powf(1.f + J0 / h, (float)df.alpha) / powf(1.f + gg / J0, (float)df.beta)) /
                             (float)df.tpi3;
            float f = df.chi == 0. ? ev : ev + (float)df.k * tanhf((float)df.chi * Jphi / J0) * ev;
            if (isnan(f)) f = 0.f;
            const int i = node / (nq * nq), j = (node / nq) % nq, k = node % nq;
            const double jd = (wq[i] * wq[j] * wq[k]) * (jacob * (double)f);
            m[0] += jd;
            m[1] += jd * V1;
            m[2] += jd * V0 * V0;
            m[3] += jd * V1 * V1;
            m[4] += jd * V2 * V2;
            m[5] += jd * V0 * V2;
        }
    }
    for (int qq = 0; qq < 6; qq++) {
        double v = m[qq];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) s_red[warp * 6 + qq] = v;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid < 6) {
        double sacc = 0;
        for (int w = 0; w < 8; w++) sacc += s_red[w * 6 + tid];
        partial[((size_t)p * B + chunk) * 6 + tid] = sacc;
    }
    if (aborted) {  // let the group's outstanding commit land before TMEM is freed
        tc::mbar_wait(bar, phase ^ 1u);
        if (gt == 0 && err) atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_slot), "r"(256) : "memory");
}

}  // namespace fj

namespace {

int sg_grid(fj_surrogate *s, const fj_potential *pot, int ngauss, const fj_quad_rule *rule, fj::SgGrid &g)
{
    if (!s->ctx || !pot || !rule || ngauss < 1 || pot->nr < 2 || pot->npoly < 1) return FJ_ERR_ARG;
    const double *ci, *xq, *wq;
    int rc = fj::context_grid_inputs(s->ctx, ngauss, rule, &ci, &xq, &wq);
    if (rc) return rc;
    std::vector<double> ar2(2);
    SG_CUDA(cudaMemcpyAsync(ar2.data(), pot->ar, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    SG_CUDA(cudaMemcpyAsync(ar2.data() + 1, pot->ar + pot->nr - 1, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    SG_CUDA(cudaStreamSynchronize(s->stream));
    g.P = fj::PotView{pot->nr, pot->npoly, pot->ar, pot->phil, pot->Pr, pot->Pr2};
    g.ci = ci; g.ngauss = ngauss; g.nq = rule->nq; g.xq = xq;
    g.lmu = .5 * (log(ar2[0]) + log(ar2[1]));
    g.lsig = .5 * (log(ar2[1]) - log(ar2[0]));
    const int npts = pot->nr * ngauss;
    if (npts > s->points_cap) {
        void *q;
        int rc2 = sg_alloc(s, &q, (size_t)npts * 2 * sizeof(double));
        if (rc2) return rc2;
        s->points = (double *)q;
        s->points_cap = npts;
    }
    g.point = s->points;
    fj::k_sg_points<<<(npts + 127) / 128, 128, 0, s->stream>>>(g, npts, s->points);
    return cudaGetLastError() == cudaSuccess ? FJ_OK : FJ_ERR_CUDA;
}


}  // namespace

extern "C" {

int fj_surrogate_fit(fj_surrogate *s, const fj_potential *pot, const fj_df_params *df, int ngauss,
                     const fj_quad_rule *rule, const float *J, const double *rho, long long nsamples,
                     unsigned long long seed, int epochs, float lr, double *loss)
{
    if (!s || !J || !df || nsamples < s->batch || epochs < 1) return FJ_ERR_ARG;
    fj::SgGrid g;
    int rc = sg_grid(s, pot, ngauss, rule, g);
    if (rc) return rc;
    const long long ns = nsamples / s->batch * s->batch;
    if (ns > s->fit_cap) {
        void *q;
        if ((rc = sg_alloc(s, &q, (size_t)ns * fj::kIn * sizeof(float)))) return rc;
        s->fitX = (float *)q;
        if ((rc = sg_alloc(s, &q, (size_t)ns * fj::kUsedOut * sizeof(float)))) return rc;
        s->fitT = (float *)q;
        if ((rc = sg_alloc(s, &q, (size_t)ns * sizeof(long long)))) return rc;
        s->fitIdx = (long long *)q;
        if ((rc = sg_alloc(s, &q, (size_t)ns * sizeof(float)))) return rc;
        s->fitW = (float *)q;
        s->fit_cap = ns;
    }
    const long long total = (long long)pot->nr * ngauss * rule->nq * rule->nq * rule->nq;
    const double *ci, *xq, *wq;
    if ((rc = fj::context_grid_inputs(s->ctx, ngauss, rule, &ci, &xq, &wq))) return rc;
    fj::k_sg_sample<<<(unsigned)((ns + 255) / 256), 256, 0, s->stream>>>(g, sg_df(df), J, rho, wq, total, seed, ns,
                                                                         s->fitIdx, s->fitT, s->fitW);
    fj::k_sg_features<<<(unsigned)((ns + 255) / 256), 256, 0, s->stream>>>(g, s->fitIdx, 0, ns, s->fitX);
    return sg_train(s, s->fitX, s->fitT, s->fitW, ns, epochs, lr, loss);
}

int fj_surrogate_moments(fj_surrogate *s, const fj_potential *pot, const fj_df_params *df, const fj_quad_rule *rule,
                         int ngauss, double *grids6, double *ms, int fused)
{
    if (!s || !df || !grids6 || df->kind != FJ_DF_DPL) return FJ_ERR_ARG;
    fj::SgGrid g;
    int rc = sg_grid(s, pot, ngauss, rule, g);
    if (rc) return rc;
    const double *ci, *xq, *wq;
    if ((rc = fj::context_grid_inputs(s->ctx, ngauss, rule, &ci, &xq, &wq))) return rc;
    const int npts = pot->nr * ngauss, nq3 = rule->nq * rule->nq * rule->nq;
    const int B = fused ? (nq3 + fj::kFusedMaxNodes - 1) / fj::kFusedMaxNodes : 1;
    if ((long long)npts * B > s->partial_cap) {
        void *q;
        if ((rc = sg_alloc(s, &q, (size_t)npts * B * 6 * sizeof(double)))) return rc;
        s->partial = (double *)q;
        s->partial_cap = (long long)npts * B;
    }
    const fj::DFDev dd = sg_df(df);
    if (fused) {  // features, MLP and moment sums in one kernel
        static bool attr = false;
        const size_t smem = fj::fused_smem_bytes();
        if (!attr) {
            if (cudaFuncSetAttribute(fj::k_sg_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
                return FJ_ERR_CUDA;
            attr = true;
        }
        fj::SgWeights w;
        for (int l = 0; l < fj::kLayers; l++) { w.W[l] = s->Wb + s->woff[l]; w.b[l] = s->P + s->boff[l]; }
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s->stream);
        fj::k_sg_fused<<<npts * B, fj::kFusedThreads, smem, s->stream>>>(g, w, wq, dd, B, s->partial, s->err);
        cudaEventRecord(e1, s->stream);
        if (cudaGetLastError() != cudaSuccess) return FJ_ERR_CUDA;
        fj::MomentArgs a{};
        a.partial = s->partial; a.npts = npts; a.blocks_per_point = B; a.out6 = grids6;
        if (fj::launch_moments_finalize(a, s->stream) != cudaSuccess) return FJ_ERR_CUDA;
        if ((rc = sg_check_err(s))) return rc;
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (ms) *ms = t;
        return FJ_OK;
    }
    if ((rc = sg_infer_buffers(s))) return rc;
    if (nq3 > kInferRows) return FJ_ERR_ARG;
    const int per = kInferRows / nq3;  // whole grid points per inference pass
    const fj::DFDev &d = dd;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s->stream);
    for (int p0 = 0; p0 < npts; p0 += per) {
        const int np = std::min(per, npts - p0);
        const long long first = (long long)p0 * nq3, m = (long long)np * nq3;
        fj::k_sg_features<<<(unsigned)((m + 255) / 256), 256, 0, s->stream>>>(g, nullptr, first, m, s->Xf);
        fj::k_to_bf16<<<(unsigned)((m * fj::kIn + 255) / 256), 256, 0, s->stream>>>((int)(m * fj::kIn), s->Xf, s->Xi);
        if ((rc = sg_forward(s, s->Xi, (int)m, s->Yf, false, s->Hi, kInferRows))) return rc;
        fj::k_sg_moments<<<np, 128, 0, s->stream>>>(g, wq, d, s->Yf, first, p0, s->partial);
    }
    cudaEventRecord(e1, s->stream);
    fj::MomentArgs a{};
    a.partial = s->partial; a.npts = npts; a.blocks_per_point = 1; a.out6 = grids6;
    if (fj::launch_moments_finalize(a, s->stream) != cudaSuccess) return FJ_ERR_CUDA;
    if ((rc = sg_check_err(s))) return rc;
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t;
    return FJ_OK;
}

}  // extern "C"


