// fj_moments_mixed.cu -- the mixed-precision phase-space kernel (FJ_PREC_MIXED).
//
// Same decomposition as k_moments (one thread per node, fixed-order block
// partials); the per-node arithmetic follows fj_mixed.cuh: FP64 for the
// node's velocity, energy, focal distance and prolate-spheroidal transform,
// FP32 for the turning-point searches, the QAGS momentum integrals and the
// DF, FP64 again for turning points at the u/v limits and for the moments.
// Built with FMA contraction (the plain form is the rounding-faithful one).
#include <cstdint>

#include "fj_internal.h"
#include "fj_mixed.cuh"
#include "fj_order.cuh"
#include "fj_qags_warp.cuh"

namespace fj {

// Work layout: a block takes one contiguous range of at most a.mixed_chunk
// nodes of one point (mixed_blocks_per_point blocks per point), compacts the
// bound ones (H < 0; about 40% of the cube) into a shared-memory list in node
// order, and its threads take the list round-robin.  So no lane idles on an
// unbound node, each thread's nodes are summed in a fixed order, and the
// per-block sums are added in a fixed order by k_moments_finalize.
// The kernel is built in two forms and each in four register budgets (launch
// bounds of 3, 4, 6 and 8 resident blocks per SM: 168, 128, 80 and 64
// registers): kMixedVariants builds.
//  - static: thread t takes list entries t, t + 128, .. and sums its nodes'
//    moments as it goes;
//  - dynamic: a lane that finishes a node takes the next untaken entry
//    (shared counter), stores the node's DF in a shared array, and after
//    the list the threads sum the moments of entries t, t + 128, .. from it.
//    The time per node varies by two orders of magnitude (QAGS takes 1 to
//    ~60 panels per integral), so with static shares the block waits for its
//    unluckiest thread; the dynamic form keeps all lanes busy to the end.
//    Its sums are those of the static form term by term, so both give the
//    same bits.
// Which one, and the chunk size, is a per-context setting (fj_autotune_mixed).
// Shared memory holds only what the node solves read: the FP32 tables, the
// radii, the focal-distance table, the velocity rule and the node list.  The
// FP64 potential tables are read from global memory (the point setup, the
// FP32 table build and the rare FP64 turning-point path): kept out of shared
// memory they leave L1 to the threads' local memory (QAGS lists, call
// frames), which took the 80x40 launch from ~347 to ~311 ms.
int mixed_blocks_per_point(long long nq3, int chunk) { return (int)((nq3 + chunk - 1) / chunk); }

// capacity of a block's node list: the next power of two >= the node range (the sort pads to it)
__host__ __device__ static int mixed_list_cap(int chunk)
{
    int c = 1;
    while (c < chunk) c <<= 1;
    return c;
}

size_t moment_mixed_smem_bytes(const MomentArgs &a)
{
    const size_t nt = (size_t)a.P.nr * a.P.npoly;
    return (a.P.nr + 2 * a.ngrid + 2 * a.nq + 6 * (kMixedBlock / 32) + 4) * sizeof(double) +
           (2 * a.P.nr + 2 * nt + 4 * kQuadIntervals + a.P.npoly) * sizeof(float) + sizeof(GK21f) + 16 +
           (kMixedBlock / 32) * sizeof(int) + (size_t)mixed_list_cap(a.mixed_chunk) * sizeof(unsigned short) + 16 +
           (size_t)mixed_list_cap(a.mixed_chunk) * sizeof(float) + sizeof(int);
}


// One work item: the node range `bid` (global over the launch's models) of
// one grid point, as described at the top of the file.
template <bool DYN>
__device__ __forceinline__ void mixed_item(const MomentArgs &a0, const MomentBatch &batch, int bid, double *sm,
                                           unsigned *s_bits, int &s_nleft)
{
    MomentArgs a = a0;
    for (int i = threadIdx.x; i < kMixedMaxNodes / 32; i += blockDim.x) s_bits[i] = 0u;
    if (threadIdx.x == 0) s_nleft = 0;
    __syncthreads();
    if (batch.n > 0) {
        const int m = batch_model(batch.block_start, batch.n, bid);
        a = batch.args[m];
        bid -= batch.block_start[m];
    }
    const int nr = a.P.nr, npoly = a.P.npoly, nt = nr * npoly;
    double *s_ar = sm;
    double *s_Eg = s_ar + nr, *s_Dg = s_Eg + a.ngrid, *s_xq = s_Dg + a.ngrid, *s_wq = s_xq + a.nq;
    double *s_red = s_wq + a.nq, *s_pt = s_red + 6 * (kMixedBlock / 32);
    float *f_ar = (float *)(s_pt + 4), *f_phil = f_ar + nr, *f_Pr = f_phil + nt, *f_ih = f_Pr + nt;
    float *f_qc = f_ih + nr, *f_pyl = f_qc + 4 * kQuadIntervals;
    GK21f *sK = (GK21f *)(((uintptr_t)(f_pyl + npoly) + 15) & ~(uintptr_t)15);
    int *s_wc = (int *)(sK + 1);
    unsigned short *s_list = (unsigned short *)(s_wc + kMixedBlock / 32);
    const int cap = mixed_list_cap(a.mixed_chunk);
    float *s_df = (float *)(((uintptr_t)(s_list + cap) + 15) & ~(uintptr_t)15);
    int *s_next = (int *)(s_df + cap);
    for (int i = threadIdx.x; i < nr; i += blockDim.x) s_ar[i] = a.P.ar[i];
    for (int i = threadIdx.x; i < a.ngrid; i += blockDim.x) { s_Eg[i] = a.Eg[i]; s_Dg[i] = a.Dg[i]; }
    for (int i = threadIdx.x; i < a.nq; i += blockDim.x) { s_xq[i] = a.xq[i]; s_wq[i] = a.wq[i]; }
    if (threadIdx.x < 11) {
        sK->xgk[threadIdx.x] = (float)fj_xgk21_d[threadIdx.x];
        sK->wgk[threadIdx.x] = (float)fj_wgk21_d[threadIdx.x];
        if (threadIdx.x < 5) sK->wg[threadIdx.x] = (float)fj_wg10_d[threadIdx.x];
    }
    const PotView P{nr, npoly, s_ar, a.P.phil, a.P.Pr, a.P.Pr2};
    const int B = a.blocks_per_point;
    const int p = bid / B, chunk = bid % B;
    __syncthreads();
    if (threadIdx.x == 0) {  // per-point FP64 setup, shared by the block (integ/Integ.cpp:46-62,150-151)
        double R, z;
        if (a.Rz) { R = a.Rz[2 * p]; z = a.Rz[2 * p + 1]; }
        else {
            const int n = p / a.ngauss, g = p % a.ngauss;
            const double c = a.ci[g], si = sqrt(1 - c * c);
            R = s_ar[n] * si; z = s_ar[n] * c;
        }
        const double rmax = s_ar[nr - 1];
        const double Phi_h = pot_phi(P, R, z);
        s_pt[0] = R; s_pt[1] = z; s_pt[2] = Phi_h;
        s_pt[3] = sqrt(-2 * (Phi_h - pot_phi(P, 10 * rmax, 10 * rmax)));
    }
    __syncthreads();
    const double R = s_pt[0], z = s_pt[1], Phi_h = s_pt[2], Ve = s_pt[3];
    mixed_tables_f(nr, npoly, s_ar, a.P.phil, a.P.Pr, Phi_h, R, z, f_ar, f_phil, f_Pr, f_ih, f_qc, f_pyl, threadIdx.x,
                   blockDim.x);
    const int nq = a.nq, nq2 = nq * nq;
    const long long nq3 = (long long)nq2 * nq;
    const int n0 = (int)(chunk * nq3 / B), n1 = (int)((chunk + 1) * nq3 / B);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    // bound nodes of [n0, n1) in node order
    int nbound = 0;
    for (int base = n0; base < n1; base += kMixedBlock) {
        const int node = base + threadIdx.x;
        bool b = false;
        if (node < n1) {
            const double V0 = 1e-6 + Ve * s_xq[node / nq2], V1 = 1e-6 + Ve * s_xq[(node / nq) % nq],
                         V2 = 1e-6 + Ve * s_xq[node % nq];
            b = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h < 0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, b);
        if (lane == 0) s_wc[warp] = __popc(bal);
        __syncthreads();
        int off = nbound, tot = 0;
        for (int w = 0; w < kMixedBlock / 32; w++) {
            if (w < warp) off += s_wc[w];
            tot += s_wc[w];
        }
        if (b) s_list[off + __popc(bal & ((1u << lane) - 1u))] = (unsigned short)(node - n0);
        __syncthreads();
        nbound += tot;
    }
    for (int q = threadIdx.x; q < nbound; q += kMixedBlock) {  // cost keys, in s_df until the solves
        const int node = n0 + s_list[q];
        s_df[q] = node_cost_key((float)s_xq[node / nq2], (float)s_xq[(node / nq) % nq], (float)s_xq[node % nq]);
    }
    sort_list(s_list, s_df, nbound);
    const PotViewF PF = mixed_view_f(nr, npoly, s_ar, a.P.phil, Phi_h, R, z, f_ar, f_phil, f_Pr, f_ih, f_qc, f_pyl);
    const double jacob = Ve * Ve * Ve;

    double m[6] = {0, 0, 0, 0, 0, 0};
    unsigned esc = 0;
    FailTally tally;
    // one node's solve; returns the DF that enters the moments.  A node whose
    // FP32 solve hits a cap (a full QAGS list, a bracket walk or Brent at its
    // step limit) is marked in the block's bitmap and counts 0 here: k_moments_deferred
    // solves it again with the plain form's FP64 solve (QAGS lists of kQagsCap
    // intervals) and adds it to this block's sums.  Only what that solve still
    // caps is a failure, with the plain form's policy (a capped bracket or root:
    // DF 0; a full QAGS list: the estimate so far, as QUADPACK returns it).
    auto solve = [&](int q) {
        const int node = n0 + s_list[q];
        const int i = node / nq2, j = (node / nq) % nq, k = node % nq;
        const double V0 = 1e-6 + Ve * s_xq[i], V1 = 1e-6 + Ve * s_xq[j], V2 = 1e-6 + Ve * s_xq[k];
        const double H = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h;
        unsigned fail = 0, e = 0;
        const double Delta = deltafn(s_Eg, s_Dg, a.ngrid, H);
        double J[2];
        double f = mixed_node_df(P, PF, *sK, a.df, Delta, R, z, Phi_h, V0, V1, V2, fail, e, J);
        esc += e;
        if (fail && a.defer) {
            atomicOr(&s_bits[(node - n0) >> 5], 1u << ((node - n0) & 31));
            atomicAdd(&s_nleft, 1);
            return 0.;
        }
        if (a.jout) {
            float *jo = a.jout + ((size_t)p * nq3 + node) * 2;
            jo[0] = (float)J[0];
            jo[1] = (float)J[1];
        }
        tally.add(fail);
        return (fail & (kFailBracket | kFailRoot)) ? 0. : f;
    };
    auto accumulate = [&](int q, double DF) {
        const int node = n0 + s_list[q];
        const int i = node / nq2, j = (node / nq) % nq, k = node % nq;
        const double V0 = 1e-6 + Ve * s_xq[i], V1 = 1e-6 + Ve * s_xq[j], V2 = 1e-6 + Ve * s_xq[k];
        const double jd = (s_wq[i] * s_wq[j] * s_wq[k]) * (jacob * DF);
        m[0] += jd;
        m[1] += jd * V1;
        m[2] += jd * V0 * V0;
        m[3] += jd * V1 * V1;
        m[4] += jd * V2 * V2;
        m[5] += jd * V0 * V2;
    };
    if (DYN) {
        if (threadIdx.x == 0) *s_next = kMixedBlock;
        __syncthreads();
        for (int q = threadIdx.x; q < nbound;) {
            s_df[q] = (float)solve(q);  // the DF is an FP32 value
            q = atomicAdd(s_next, 1);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < nbound; q += kMixedBlock) accumulate(q, (double)s_df[q]);
    } else {
        for (int q = threadIdx.x; q < nbound; q += kMixedBlock) accumulate(q, solve(q));
    }
#pragma unroll
    for (int q = 0; q < 6; q++) {
        double v = m[q];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) s_red[warp * 6 + q] = v;
    }
    warp_count_fails(a.counters, tally);
    warp_count(&a.counters[kCntEscalated], esc);
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w = 0; w < kMixedBlock / 32; w++) s += s_red[w * 6 + threadIdx.x];
        a.partial[((size_t)p * B + chunk) * 6 + threadIdx.x] = s;
    }
    if (a.defer) {  // the block's bitmap of deferred nodes and their number
        const int nw = defer_words(a.mixed_chunk);
        for (int i = threadIdx.x; i < nw; i += blockDim.x) a.defer[((size_t)p * B + chunk) * nw + i] = s_bits[i];
        if (threadIdx.x == 0) a.defer_count[(size_t)p * B + chunk] = s_nleft;
    }
    if (threadIdx.x == 0 && nbound) atomicAdd(&a.counters[kCntBound], (unsigned long long)nbound);
}

// The persistent kernel: a grid of at most as many blocks as fit on the GPU at
// once takes work items from the queue (an atomic counter) until none is
// left, in the queue's order (most expensive first, from the previous launch's
// measured cycles, when the context has them), and records each item's cycles.
// Blocks free up as their items finish and take the next one, so the uneven
// cost of the root finding and quadrature is balanced across the GPU.
template <int MINB, bool DYN>
__global__ void __launch_bounds__(kMixedBlock, MINB) k_moments_mixed(MomentArgs a0, MomentBatch batch, ItemQueue q)
{
    extern __shared__ double sm[];
    __shared__ unsigned s_bits[kMixedMaxNodes / 32];  // nodes left to the FP64 pass
    __shared__ int s_nleft, s_item;
    for (;;) {
        __syncthreads();  // every thread is done with the previous item's shared data
        if (threadIdx.x == 0) s_item = (int)atomicAdd(q.next, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= q.total) return;
        const int bid = q.order ? q.order[it] : it;
        const long long t0 = clock64();
        mixed_item<DYN>(a0, batch, bid, sm, s_bits, s_nleft);
        if (q.cost && threadIdx.x == 0) q.cost[bid] = (float)(clock64() - t0);
    }
}

// ------------------------------------------------------ the FP64 pass
// Over the nodes the mixed kernel left (launch_deferred): a scan of the
// blocks' counts, the compact list, one thread per listed node, one thread per
// block adding its nodes in list order.

// the arguments and the model-local index of global block g of a launch
__device__ __forceinline__ const MomentArgs &block_args(const MomentArgs &a0, const MomentBatch &b, int g, int &bid)
{
    bid = g;
    if (b.n == 0) return a0;
    const int m = batch_model(b.block_start, b.n, g);
    bid -= b.block_start[m];
    return b.args[m];
}

// the block's point, its potential and escape speed (as the mixed kernel's setup)
__device__ void defer_point(const MomentArgs &a, int bid, double &R, double &z, double &Phi_h, double &Ve)
{
    const int nr = a.P.nr, p = bid / a.blocks_per_point;
    if (a.Rz) { R = a.Rz[2 * p]; z = a.Rz[2 * p + 1]; }
    else {
        const int n = p / a.ngauss, gg = p % a.ngauss;
        const double c = a.ci[gg], si = sqrt(1 - c * c);
        R = a.P.ar[n] * si; z = a.P.ar[n] * c;
    }
    const PotView P{nr, a.P.npoly, a.P.ar, a.P.phil, a.P.Pr, a.P.Pr2};
    const double rmax = a.P.ar[nr - 1];
    Phi_h = pot_phi(P, R, z);
    Ve = sqrt(-2 * (Phi_h - pot_phi(P, 10 * rmax, 10 * rmax)));
}

// The momentum integrals of a warp: QAGS with the panels spread over the lanes
struct WarpMomInt {
    WarpQagsWs w;
    int lane;
    template <class F>
    FJ_HD double operator()(F &f, double b, unsigned &fail) const
    {
#ifdef __CUDA_ARCH__
        double r, e;
        qags_warp<21>(f, 0.0, b, 1e-5, 1e-3, 1000, r, e, fail, w.ws(), w.buf, lane);
        return r;
#else
        (void)f; (void)b; (void)fail;
        return 0.;
#endif
    }
};

// one left node with the plain form's FP64 solve (the actions with QAGS lists
// of kQagsCap intervals, df_value) by a whole warp (every lane calls it with the
// same node; the turning points run on every lane, the momentum integrals
// spread their panels over the lanes): its six moment contributions
__device__ void defer_solve(const MomentArgs &a, int bid, int node, double *c6, FailTally &tally,
                            const WarpQagsWs &w, int lane)
{
    double R, z, Phi_h, Ve;
    defer_point(a, bid, R, z, Phi_h, Ve);
    const PotView P{a.P.nr, a.P.npoly, a.P.ar, a.P.phil, a.P.Pr, a.P.Pr2};
    const int nq = a.nq, nq2 = nq * nq;
    const int i = node / nq2, j = (node / nq) % nq, l = node % nq;
    const double V0 = 1e-6 + Ve * a.xq[i], V1 = 1e-6 + Ve * a.xq[j], V2 = 1e-6 + Ve * a.xq[l];
    const double H = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h;
    unsigned fail = 0;
    double Jr, Jz;
    fudge_actions_with(P, deltafn(a.Eg, a.Dg, a.ngrid, H), R, z, Phi_h, V0, V1, V2, WarpMomInt{w, lane}, Jr, Jz,
                       fail);
    double DF = df_value(a.df, P, R, Jr, Jz, R * V1, fail);
    if (fail & (kFailBracket | kFailRoot)) DF = 0.;
    if (lane == 0) {
        tally.add(fail);
        if (a.jout) {
            float *jo = a.jout + ((size_t)(bid / a.blocks_per_point) * nq2 * nq + node) * 2;
            jo[0] = (float)Jr;
            jo[1] = (float)Jz;
        }
    }
    const double jd = (a.wq[i] * a.wq[j] * a.wq[l]) * (Ve * Ve * Ve * DF);
    c6[0] = jd; c6[1] = jd * V1; c6[2] = jd * V0 * V0;
    c6[3] = jd * V1 * V1; c6[4] = jd * V2 * V2; c6[5] = jd * V0 * V2;
}

__device__ void add_tally(unsigned long long *counters, const FailTally &t, unsigned solved)
{
    if (solved) atomicAdd(&counters[kCntResolved64], (unsigned long long)solved);
    if (!t.any) return;
    atomicAdd(&counters[kCntFailed], (unsigned long long)t.any);
    if (t.quad) atomicAdd(&counters[kCntFailQuad], (unsigned long long)t.quad);
    if (t.bracket) atomicAdd(&counters[kCntFailBracket], (unsigned long long)t.bracket);
    if (t.root) atomicAdd(&counters[kCntFailRoot], (unsigned long long)t.root);
}

// exclusive scan of the counts: per chunk of kScanChunk blocks, then the chunk
// carries (one CTA; chunk_sum[nchunks] = the total), then the carries added
__device__ __forceinline__ int block_exclusive_scan(int v, int *s_warp, int &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nwarp ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nwarp) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[nwarp - 1];
    const int res = x - v + (warp ? s_warp[warp - 1] : 0);
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanChunk) k_defer_scan_chunks(DeferWork dw, int nblocks)
{
    __shared__ int s_warp[32];
    const int i = blockIdx.x * kScanChunk + threadIdx.x;
    int total;
    const int ex = block_exclusive_scan(i < nblocks ? dw.count[i] : 0, s_warp, total);
    if (i < nblocks) dw.offset[i] = ex;
    if (threadIdx.x == 0) dw.chunk_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanChunk) k_defer_scan_carries(DeferWork dw, int nchunks)
{
    __shared__ int s_warp[32];
    int carry = 0;
    for (int base = 0; base < nchunks; base += kScanChunk) {
        const int i = base + threadIdx.x;
        const int v = i < nchunks ? dw.chunk_sum[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, s_warp, total);
        if (i < nchunks) dw.chunk_sum[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) dw.chunk_sum[nchunks] = carry;
}

// adds the carries and lists each block's left nodes in node order (a warp per block)
constexpr int kListWarps = 4;
__global__ void __launch_bounds__(32 * kListWarps) k_defer_list(MomentArgs a0, MomentBatch batch, DeferWork dw,
                                                                 int nblocks)
{
    const int lane = threadIdx.x & 31;
    const int g = blockIdx.x * kListWarps + (threadIdx.x >> 5);
    if (g >= nblocks) return;  // the whole warp
    const int off = dw.offset[g] + dw.chunk_sum[g / kScanChunk];
    __syncwarp();
    if (lane == 0) dw.offset[g] = off;
    const int cnt = dw.count[g];
    if (cnt == 0) return;
    int bid;
    const MomentArgs &a = block_args(a0, batch, g, bid);
    const int nw = defer_words(a.mixed_chunk), B = a.blocks_per_point, chunk = bid % B;
    const long long nq3 = (long long)a.nq * a.nq * a.nq;
    const int n0 = (int)(chunk * nq3 / B);
    const unsigned *bits = a.defer + (size_t)bid * nw;
    int rank = 0;
    for (int w = 0; w < nw && rank < cnt; w++) {
        const unsigned word = bits[w];  // the same word on every lane
        if ((word >> lane) & 1u) {
            const int e = off + rank + __popc(word & ((1u << lane) - 1u));
            if (e < dw.cap) { dw.node[e] = n0 + w * 32 + lane; dw.block[e] = g; }
        }
        rank += __popc(word);
    }
}

// one warp per listed node (grid-stride over the launch's total)
constexpr int kSolveWarps = 4;
__global__ void __launch_bounds__(32 * kSolveWarps) k_defer_solve(MomentArgs a0, MomentBatch batch, DeferWork dw,
                                                                   int nchunks)
{
    __shared__ double s_list[kSolveWarps][4 * kQagsCap];
    __shared__ int s_iord[kSolveWarps][kQagsCap];
    __shared__ double s_buf[kSolveWarps][42];
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const WarpQagsWs w{s_list[wq], s_iord[wq], s_buf[wq], kQagsCap};
    const int total = min(dw.chunk_sum[nchunks], dw.cap);
    FailTally tally;
    unsigned solved = 0;
    unsigned long long *counters = a0.counters;
    for (int e = blockIdx.x * kSolveWarps + wq; e < total; e += gridDim.x * kSolveWarps) {
        int bid;
        const MomentArgs &a = block_args(a0, batch, dw.block[e], bid);
        counters = a.counters;
        double c6[6];
        defer_solve(a, bid, dw.node[e], c6, tally, w, lane);
        if (lane == 0) {
            for (int q = 0; q < 6; q++) dw.mom[(size_t)e * 6 + q] = c6[q];
            solved++;
        }
    }
    if (lane == 0) add_tally(counters, tally, solved);
}

// one warp per block: its listed nodes added in list order by lane 0 (nodes
// beyond the list's capacity solved here by the warp, in node order)
constexpr int kAddWarps = 4;
__global__ void __launch_bounds__(32 * kAddWarps) k_defer_add(MomentArgs a0, MomentBatch batch, DeferWork dw,
                                                               int nblocks)
{
    __shared__ double s_list[kAddWarps][4 * kQagsCap];
    __shared__ int s_iord[kAddWarps][kQagsCap];
    __shared__ double s_buf[kAddWarps][42];
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const int g = blockIdx.x * kAddWarps + wq;
    if (g >= nblocks) return;  // the whole warp
    const int cnt = dw.count[g];
    if (cnt == 0) return;
    int bid;
    const MomentArgs &a = block_args(a0, batch, g, bid);
    const int off = dw.offset[g];
    const WarpQagsWs w{s_list[wq], s_iord[wq], s_buf[wq], kQagsCap};
    double msum[6] = {0, 0, 0, 0, 0, 0};
    FailTally tally;
    unsigned solved = 0;
    for (int k = 0; k < cnt; k++) {
        const int e = off + k;
        if (e < dw.cap) {
            for (int q = 0; q < 6; q++) msum[q] += dw.mom[(size_t)e * 6 + q];
            continue;
        }
        // past the list: the block's k-th left node, from its bitmap
        const int nw = defer_words(a.mixed_chunk), B = a.blocks_per_point;
        const long long nq3 = (long long)a.nq * a.nq * a.nq;
        const int n0 = (int)((bid % B) * nq3 / B);
        const unsigned *bits = a.defer + (size_t)bid * nw;
        int r = k, wd = 0;
        while (r >= __popc(bits[wd])) r -= __popc(bits[wd++]);
        unsigned word = bits[wd];
        for (int t = 0; t < r; t++) word &= word - 1;
        double c6[6];
        defer_solve(a, bid, n0 + wd * 32 + (__ffs((int)word) - 1), c6, tally, w, lane);
        solved++;
        for (int q = 0; q < 6; q++) msum[q] += c6[q];
    }
    if (lane == 0) {
        double *pt = a.partial + (size_t)bid * 6;
        for (int q = 0; q < 6; q++) pt[q] += msum[q];
        add_tally(a.counters, tally, solved);
    }
}

static cudaError_t launch_deferred(const MomentArgs &a, const MomentBatch &b, long long nblocks, const DeferWork &dw,
                                   cudaStream_t s)
{
    if (!dw.count) return cudaSuccess;
    const int nb = (int)nblocks, nchunks = (nb + kScanChunk - 1) / kScanChunk;
    k_defer_scan_chunks<<<nchunks, kScanChunk, 0, s>>>(dw, nb);
    k_defer_scan_carries<<<1, kScanChunk, 0, s>>>(dw, nchunks);
    k_defer_list<<<(nb + kListWarps - 1) / kListWarps, 32 * kListWarps, 0, s>>>(a, b, dw, nb);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    k_defer_solve<<<4 * (nsm > 0 ? nsm : 1), 32 * kSolveWarps, 0, s>>>(a, b, dw, nchunks);
    k_defer_add<<<(nb + kAddWarps - 1) / kAddWarps, 32 * kAddWarps, 0, s>>>(a, b, dw, nb);
    return cudaGetLastError();
}

namespace {
template <int MINB, bool DYN>
cudaError_t launch_variant(const MomentArgs &a, const MomentBatch &b, const ItemQueue &q, size_t smem, cudaStream_t s)
{
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_moments_mixed<MINB, DYN>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int dev = 0, nsm = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_moments_mixed<MINB, DYN>, kMixedBlock, smem);
    if (e != cudaSuccess) return e;
    const long long resident = (long long)(per_sm > 0 ? per_sm : 1) * (nsm > 0 ? nsm : 1);
    const long long grid = q.total < resident ? q.total : resident;
    if ((e = cudaMemsetAsync(q.next, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
    k_moments_mixed<MINB, DYN><<<(unsigned)grid, kMixedBlock, smem, s>>>(a, b, q);
    return cudaGetLastError();
}

cudaError_t launch_mixed_any(const MomentArgs &a, const MomentBatch &b, const ItemQueue &q, size_t smem, int variant,
                             cudaStream_t s)
{
    switch (variant) {
    case 0: return launch_variant<3, false>(a, b, q, smem, s);
    case 1: return launch_variant<4, false>(a, b, q, smem, s);
    case 2: return launch_variant<6, false>(a, b, q, smem, s);
    case 3: return launch_variant<8, false>(a, b, q, smem, s);
    case 4: return launch_variant<3, true>(a, b, q, smem, s);
    case 5: return launch_variant<4, true>(a, b, q, smem, s);
    case 6: return launch_variant<6, true>(a, b, q, smem, s);
    case 7: return launch_variant<8, true>(a, b, q, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int MINB, bool DYN>
size_t local_bytes()
{
    cudaFuncAttributes at;
    return cudaFuncGetAttributes(&at, k_moments_mixed<MINB, DYN>) == cudaSuccess ? at.localSizeBytes : 0;
}
}  // namespace

cudaError_t launch_moments_mixed(const MomentArgs &a, int variant, const DeferWork &dw, const ItemQueue &q,
                                 cudaStream_t s)
{
    if (a.mixed_chunk < kMixedBlock || a.mixed_chunk > kMixedMaxNodes) return cudaErrorInvalidValue;
    const size_t smem = moment_mixed_smem_bytes(a);
    const MomentBatch none{nullptr, nullptr, nullptr, 0};
    const long long nblocks = (long long)a.npts * a.blocks_per_point;
    if (q.total != nblocks) return cudaErrorInvalidValue;
    cudaError_t e = launch_mixed_any(a, none, q, smem, variant, s);
    if (e == cudaSuccess) e = launch_deferred(a, none, nblocks, dw, s);
    if (e != cudaSuccess) return e;
    return launch_moments_finalize(a, s);
}

cudaError_t launch_moments_plain_batch(const MomentArgs &a0, const MomentBatch &b, int nblocks, size_t smem,
                                      cudaStream_t s);

cudaError_t launch_moments_batch(const MomentArgs &a0, const MomentBatch &b, int nblocks, size_t smem, bool mixed,
                                 int variant, const DeferWork &dw, const ItemQueue &q, cudaStream_t s)
{
    if (!mixed) return launch_moments_plain_batch(a0, b, nblocks, smem, s);
    if (q.total != nblocks) return cudaErrorInvalidValue;
    const cudaError_t e = launch_mixed_any(a0, b, q, smem, variant, s);
    return e == cudaSuccess ? launch_deferred(a0, b, nblocks, dw, s) : e;
}

size_t moments_mixed_local_bytes()
{
    const size_t v[kMixedVariants] = {local_bytes<3, false>(), local_bytes<4, false>(), local_bytes<6, false>(),
                                      local_bytes<8, false>(), local_bytes<3, true>(), local_bytes<4, true>(),
                                      local_bytes<6, true>(), local_bytes<8, true>()};
    size_t m = 0;
    for (size_t x : v) m = x > m ? x : m;
    cudaFuncAttributes at;
    for (const void *k : {(const void *)k_defer_solve, (const void *)k_defer_add})
        if (cudaFuncGetAttributes(&at, k) == cudaSuccess && at.localSizeBytes > m) m = at.localSizeBytes;
    return m;
}

}  // namespace fj
