// fj_internal.h -- launch interface between the C-ABI layer and the kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "fj_device.cuh"

struct fj_ctx;
struct fj_quad_rule;

namespace fj {

struct DeferWork;  // scratch of the mixed form's FP64 pass (below)
constexpr int kMomentBlock = 128;  // threads per block of the phase-space kernel
// Device counters of one call (fj_moment_stats): nodes with H < 0, nodes whose
// action solve still hit a cap (any kind), Poisson integrals that hit theirs,
// nodes whose turning points ran in FP64 (mixed form), the final failures by
// kind (a node can count in several), and mixed-form nodes re-solved by the
// plain FP64 solve because their FP32 solve hit a cap.
enum : int {
    kCntBound = 0, kCntFailed = 1, kCntPoisson = 2, kCntEscalated = 3,
    kCntFailQuad = 4, kCntFailBracket = 5, kCntFailRoot = 6, kCntResolved64 = 7, kNumCounters = 8
};
constexpr int kPlainChunk = 1024;  // velocity nodes of one point per block (FP64 form)
// per-thread stack the kernels need: the QAGS interval list (kQagsCap entries
// of four doubles and an int), the epsilon table and the call frames
constexpr size_t kStackBytes = 8192;
static_assert(kQagsCap * (4 * sizeof(double) + sizeof(int)) + 52 * sizeof(double) + 1024 < kStackBytes,
              "stack floor below the QAGS workspace");

// Arguments of the phase-space (moment) kernel.  All pointers are device memory.
struct MomentArgs {
    PotView P;
    const double *Eg, *Dg;
    int ngrid;
    const double *xq, *wq;   // velocity rule [nq]
    int nq;
    GLRule gl;               // momentum-integral rule (n = 0: QAGS)
    DFDev df;
    const double *ci;        // grid mode: ngauss polar GL nodes on (0,1); else NULL
    int ngauss;
    const double *Rz;        // point mode: [npts][2]; else NULL
    int npts;
    int blocks_per_point;
    int mixed_chunk;         // mixed form: nodes per block (<= kMixedMaxNodes)
    float *jout;             // mixed form, optional: (Jr, Jz) of every bound node [npts][nq^3][2]
    double *partial;         // [npts][blocks_per_point][6]
    unsigned *defer;         // mixed form: [npts * blocks_per_point][mixed_chunk / 32] bitmaps of the nodes
                             // left to the FP64 pass
    int *defer_count;        // mixed form: [npts * blocks_per_point] how many nodes each block left
    unsigned long long *counters;  // [kNumCounters], the slots below
    double *out6;            // [6][npts]
};

// Projected density, line profiles and velocity distributions (fj_los.cu):
// n values at Rzv [n][3] (R, z, v) of one kind (FJ_LOS_*), on m's potential,
// focal-distance table, [-1,1] rule and DF, with the 22-point [0,1] table
constexpr int kLos01 = 22;
struct LosArgs {
    MomentArgs m;
    const double *rhl;  // [nr*npoly] density multipoles (SigmaDF)
    int kind;
    const double *Rzv;
    int n;
    double *out;        // [n]
    double x01[kLos01], w01[kLos01];
    int blocks_per_item;  // blocks sharing one value's nodes (kLosChunk nodes each)
    double *partial;      // [n][blocks_per_item] block sums, added in order by k_los_finalize
};
constexpr int kLosChunk = 1024;  // nodes of one value per block
cudaError_t launch_los(const LosArgs &a, cudaStream_t s);
int los_blocks_per_item(int kind, int nq);
size_t los_local_bytes();

// Focal-distance tables of n models (fj_delta.cu): one thread per (model,
// energy); pots, Eg, Dg device arrays [n] (tables [ngrid] each), bad device [n]
// (set to 1 where a bracket or root search hit its cap)
cudaError_t launch_tabulate_delta(const PotView *pots, double *const *Eg, double *const *Dg, int n, int ngrid,
                                  int *bad, cudaStream_t s);
size_t delta_local_bytes();

// Several models' phase-space launches in one grid: model m owns blocks
// [block_start[m], block_start[m+1]) and grid points [point_start[m],
// point_start[m+1]) of the batched finalize.  All pointers are device memory;
// n = 0: a single launch described by the kernel's MomentArgs parameter.
struct MomentBatch {
    const MomentArgs *args;
    const int *block_start, *point_start;
    int n;
};

// per-node status tallies of one thread: nodes with any cap, and by kind
struct FailTally {
    unsigned any = 0, quad = 0, bracket = 0, root = 0;
    __device__ __forceinline__ void add(unsigned fail)
    {
        any += fail ? 1u : 0u;
        quad += (fail & kFailQuad) ? 1u : 0u;
        bracket += (fail & kFailBracket) ? 1u : 0u;
        root += (fail & kFailRoot) ? 1u : 0u;
    }
};

// adds a warp's values of v to *ctr (one atomic per warp, none for a zero sum);
// every lane of the warp must call it
__device__ __forceinline__ void warp_count(unsigned long long *ctr, unsigned v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(ctr, (unsigned long long)v);
}

__device__ __forceinline__ void warp_count_fails(unsigned long long *counters, const FailTally &t)
{
    warp_count(&counters[kCntFailed], t.any);
    warp_count(&counters[kCntFailQuad], t.quad);
    warp_count(&counters[kCntFailBracket], t.bracket);
    warp_count(&counters[kCntFailRoot], t.root);
}

// the model of block (or point) `i` of a batch: largest m with start[m] <= i
__device__ __forceinline__ int batch_model(const int *start, int n, int i)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

size_t moment_smem_bytes(const MomentArgs &a);
cudaError_t launch_moments(const MomentArgs &a, cudaStream_t s);
// batched forms: grid = total blocks, smem = the largest model's
// work queue of the persistent mixed kernel: item i is block order[i] (order
// NULL: block i) of the launch's layout; cost[b] receives block b's cycles
struct ItemQueue {
    unsigned *next;    // device counter, zeroed by the launch
    const int *order;  // [total] or NULL
    float *cost;       // [total] or NULL
    int total;
};
cudaError_t launch_moments_batch(const MomentArgs &a0, const MomentBatch &b, int nblocks, size_t smem, bool mixed,
                                 int variant, const DeferWork &dw, const ItemQueue &q, cudaStream_t s);
cudaError_t launch_moments_finalize_batch(const MomentBatch &b, int npoints, cudaStream_t s);
// dst6[q][idx[t]] = src6[q][t] (moments of n points into a grid of npts)
cudaError_t launch_scatter6(int n, const int *idx, const double *src6, int npts, double *dst6, cudaStream_t s);
// the per-point sums of the block partials (shared by both forms)
cudaError_t launch_moments_finalize(const MomentArgs &a, cudaStream_t s);
// mixed-precision form (FJ_PREC_MIXED, double-power-law DF, QAGS momentum
// integrals); counters[3] gets the nodes whose turning points ran in FP64
constexpr int kMixedBlock = 128;     // threads per block of the mixed kernel
// A mixed-form node whose FP32 solve hits a cap is not re-solved in the block
// (one FP64 solve would hold its warp and block for as long as hundreds of FP32
// ones): its block marks it in a bitmap of its node range, leaves it out of its
// sums and records how many it left.  The FP64 pass (launch_deferred) then lists
// every launch's left nodes compactly, block by block in node order (an
// exclusive scan of the counts gives each block its offset), solves them all in
// parallel, one thread per node, and adds each block's nodes to its partial
// sums in list order: the same sums whatever order the threads ran in.
struct DeferWork {
    int *count;      // [nblocks] the blocks' counts (the launch's defer_count arrays, in block order)
    int *offset;     // [nblocks] exclusive prefix of the blocks' counts
    int *chunk_sum;  // [nblocks / kScanChunk + 2] scan carries; [nchunks] = the launch's total
    int *node;       // [cap] listed nodes (index within the point's nq^3 rule)
    int *block;      // [cap] global block index of each listed node
    double *mom;     // [cap][6] moment contributions of the listed nodes
    int cap;         // list capacity; nodes beyond it are solved by their block's adding thread
};
constexpr int kScanChunk = 1024;  // blocks per chunk of the count scan
constexpr int kMixedMaxNodes = 8192; // largest node range of one block (shared-memory list)
FJ_HD int defer_words(int chunk) { return (chunk + 31) / 32; }  // bitmap words of one block
constexpr int kMixedVariants = 8;    // builds of the mixed kernel (2 forms x 4 register budgets)
size_t moment_mixed_smem_bytes(const MomentArgs &a);
int mixed_blocks_per_point(long long nq3, int chunk);
cudaError_t launch_moments_mixed(const MomentArgs &a, int variant, const DeferWork &dw, const ItemQueue &q,
                                 cudaStream_t s);

cudaError_t launch_actions(PotView P, const double *Eg, const double *Dg, int ngrid, GLRule gl,
                           const double *pts, size_t n, double *out, cudaStream_t s);
cudaError_t launch_potential_eval(PotView P, const double *Rz, size_t n, double *out, cudaStream_t s);

// projection: poly [npoly][ngauss] = 2 P_2l(c_g) w_g
cudaError_t launch_project(int nr, int ngauss, int npoly, const double *ar, const double *poly,
                           const double *grids6, double *coef6, cudaStream_t s);
// Poisson: one warp per (n, l), QAGS interval lists of kPoissonCap entries in
// shared memory (no device workspace)
constexpr int kPoissonCap = 256;
cudaError_t launch_poisson(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                           double *Pr, double *Pr2, unsigned long long *counters, cudaStream_t s);
// Poisson with the radial integrals taken exactly over the linear interpolation
// of the density multipoles (prefix sums, no adaptive quadrature): one block per l
constexpr int kPoissonCumulativeMaxNr = 4096;
cudaError_t launch_poisson_cumulative(int nr, int npoly, const double *ar, const double *rhl, double *phil,
                                      double *Pr, double *Pr2, cudaStream_t s);
cudaError_t launch_sum3(int n, const double *a0, const double *a1, const double *a2, const double *b0,
                        const double *b1, const double *b2, double *o0, double *o1, double *o2, cudaStream_t s);
// o = a + b elementwise (summed component densities)
cudaError_t launch_add(int n, const double *a, const double *b, double *o, cudaStream_t s);
// vir2: ci, wi = ngauss polar nodes/weights on (0,1); out7 device
cudaError_t launch_vir2(PotView P, int ngauss, const double *ci, const double *wi, const double *coef6,
                        double *out7, cudaStream_t s);

// the stream a context orders its work on; the device copies of a grid's polar
// nodes and of a velocity rule
cudaStream_t context_stream(::fj_ctx *ctx);
int context_grid_inputs(::fj_ctx *ctx, int ngauss, const struct ::fj_quad_rule *rule, const double **ci,
                        const double **xq, const double **wq);
// BF16 tensor-core GEMM (fj_mlp.cu): C = A B^T with a fused epilogue
namespace tc { struct Epilogue; }
cudaError_t launch_gemm_tc(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                           int ksplit, const tc::Epilogue &ep, cudaStream_t s);

// largest per-thread local memory (stack) any kernel of the library needs
size_t moments_local_bytes();
size_t moments_mixed_local_bytes();
size_t multipole_local_bytes();
size_t poisson_local_bytes();  // per-thread local memory (stack) of the Poisson kernel

}  // namespace fj
