// fj_api.cu -- the C ABI of include/fjgpu.h: context, cached rule tables,
// launches of the hot path, and the host-side setup the reference also runs
// once on the host (grid, guess density, focal-distance table, coefficient
// file writer) plus the one-component self-consistent loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fjgpu.h"
#include "fj_internal.h"
#include "fj_delta.cuh"

// the host-only functors below instantiate the __host__ __device__ Brent template on the host only
#pragma nv_diag_suppress 20011, 20014

using namespace fj;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// The history of one Anderson-mixed iteration (fj_anderson_step, fj_anderson_host_step)
struct fj_anderson {
    int depth = 0;
    double beta = 1;                               // mixing factor (1: the next input is the mixed output)
    double last = -1;                              // the previous step's change
    std::vector<std::vector<double>> f, g, x;      // weighted phil residuals [nt], outputs, inputs [3 nt]
};

struct fj_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own = nullptr;
    std::string err;
    DevBuf partial, counters, rule, misc, defer;
    std::map<int, DevBuf> gauss_nodes;                 // ngauss -> [2][ngauss] (ci, wi)
    std::map<std::pair<int, int>, DevBuf> poly;        // (ngauss, npoly) -> [npoly][ngauss]
    std::map<int, DevBuf> gl_rules;                    // jquad -> [2][n]
    std::vector<double> rule_host;                     // last uploaded velocity rule
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int mixed_variant = 0, mixed_chunk = kMixedMaxNodes;  // mixed kernel configuration (fj_autotune_mixed)
    int poisson = FJ_POISSON_QAGS;                     // radial integrals of fj_poisson (fj_set_poisson)
    float *jout = nullptr;                             // mixed form: actions of every bound node (fj_set_action_output)
    DevBuf batch;                                      // batched launch: MomentArgs[n] | block_start | point_start
    std::vector<char> batch_host;                      // what `batch` holds (re-uploaded only when it changes)
    DevBuf delta_ws;                                   // GPU focal-distance tables: views | Eg ptrs | Dg ptrs | flags
    DevBuf queue;                                      // mixed kernel's work queue: counter | order | costs
    int q_total = 0;                                   // items of the launch whose costs the queue holds
    bool q_costs = false, q_order = false;             // costs recorded / order taken from them
    int q_launches = 0;                                // launches since the order was last taken
    fj_anderson anderson;                              // the mixing history of fj_anderson_step
};

namespace fj {
cudaStream_t context_stream(fj_ctx *ctx) { return ctx->stream; }
}  // namespace fj

namespace {

int fail(fj_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_fail(fj_ctx *c, cudaError_t e, const char *what)
{
    return fail(c, FJ_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define FJ_CUDA(call)                                      \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

int ensure(fj_ctx *ctx, DevBuf &b, size_t bytes)
{
    if (b.bytes >= bytes) return FJ_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) return fail(ctx, FJ_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b.bytes = bytes;
    return FJ_OK;
}

// Scratch of the mixed form's FP64 pass over capped nodes for a launch of
// nblocks blocks (nw bitmap words each) and `nodes` phase-space nodes, in one
// buffer: bitmaps | counts | offsets | scan carries | list (nodes, blocks,
// moments).  The list holds 1/256 of the nodes (at least 64 Ki, at most 4 Mi
// entries); a launch that leaves more is still exact (the extra nodes are
// solved by their block's adding thread), only slower.
int defer_setup(fj_ctx *ctx, long long nblocks, int nw, long long nodes, DeferWork &dw, unsigned *&bitmaps)
{
    const long long nchunks = (nblocks + kScanChunk - 1) / kScanChunk;
    long long cap = nodes / 256;
    cap = cap < 65536 ? 65536 : (cap > (4ll << 20) ? (4ll << 20) : cap);
    const size_t ints = (size_t)nblocks * nw + 2 * (size_t)nblocks + nchunks + 2 + 2 * (size_t)cap;
    const size_t off_mom = (ints * sizeof(int) + 15) / 16 * 16;
    int rc = ensure(ctx, ctx->defer, off_mom + (size_t)cap * 6 * sizeof(double));
    if (rc) return rc;
    int *base = (int *)ctx->defer.p;
    bitmaps = (unsigned *)base;
    dw.count = base + (size_t)nblocks * nw;
    dw.offset = dw.count + nblocks;
    dw.chunk_sum = dw.offset + nblocks;
    dw.node = dw.chunk_sum + nchunks + 2;
    dw.block = dw.node + cap;
    dw.mom = (double *)((char *)ctx->defer.p + off_mom);
    dw.cap = (int)cap;
    return FJ_OK;
}

// The persistent mixed kernel's work queue for a launch of `total` items.  The
// kernel records every item's cycles; the next launch of the same size (outside
// a graph capture) takes the items most expensive first, the order refreshed
// from the latest costs every kReorderEvery launches.  A captured launch keeps
// the order in place at capture (refresh_queue_order takes one before).
constexpr int kReorderEvery = 4;

int refresh_queue_order(fj_ctx *ctx)
{
    if (!ctx->q_costs || ctx->q_total < 1) return FJ_OK;
    const int n = ctx->q_total;
    int *order = (int *)((char *)ctx->queue.p + 16);
    float *cost = (float *)(order + n);
    std::vector<float> c(n);
    FJ_CUDA(cudaMemcpyAsync(c.data(), cost, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return c[x] > c[y]; });
    FJ_CUDA(cudaMemcpyAsync(order, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->q_order = true;
    ctx->q_launches = 0;
    return FJ_OK;
}

int queue_setup(fj_ctx *ctx, long long total, ItemQueue &q)
{
    if (total < 1 || total > 0x7fffffffLL) return fail(ctx, FJ_ERR_ARG, "moments: too many work items");
    const int n = (int)total;
    if (n != ctx->q_total) {
        int rc = ensure(ctx, ctx->queue, 16 + (size_t)n * (sizeof(int) + sizeof(float)));
        if (rc) return rc;
        ctx->q_total = n;
        ctx->q_costs = ctx->q_order = false;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FJ_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone && ctx->q_costs && (!ctx->q_order || ctx->q_launches >= kReorderEvery)) {
        int rc = refresh_queue_order(ctx);
        if (rc) return rc;
    }
    int *order = (int *)((char *)ctx->queue.p + 16);
    q.next = (unsigned *)ctx->queue.p;
    q.order = ctx->q_order ? order : nullptr;
    q.cost = (float *)(order + n);
    q.total = n;
    ctx->q_costs = true;  // this launch records them
    ctx->q_launches++;
    return FJ_OK;
}

// Gauss-Legendre on [x1,x2] with the iteration of include/UtilsLeg.h:18-39
void gauleg_host(double x1, double x2, int n, double *x, double *w)
{
    const double eps = 3.0e-11;
    const int m = (n + 1) / 2;
    const double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
    double pp = 0, z1;
    for (int i = 0; i < m; i++) {
        double z = cos(3.141592654 * (i + 0.75) / (n + 0.5));
        do {
            double p1 = 1, p2 = 0, p3;
            for (int j = 0; j < n; j++) {
                p3 = p2;
                p2 = p1;
                p1 = ((2 * (j + 1) - 1) * z * p2 - j * p3) / (double)(j + 1);
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            z1 = z;
            z = z1 - p1 / pp;
        } while (fabs(z - z1) > eps);
        x[i] = xm - xl * z;
        x[n - i - 1] = xm + xl * z;
        w[i] = 2 * xl / ((1 - z * z) * pp * pp);
        w[n - i - 1] = w[i];
    }
}

void evenlegend_host(int npoly, double c, double *pol)
{
    const double c2 = c * c;
    pol[0] = 1;
    if (npoly < 2) return;
    pol[1] = 1.5 * c2 - .5;
    for (int np = 2; np < npoly; np++) pol[np] = evenleg_next(np, c2, pol[np - 2], pol[np - 1]);
}

int gauss_nodes(fj_ctx *ctx, int ngauss, const double **dptr)
{
    auto it = ctx->gauss_nodes.find(ngauss);
    if (it == ctx->gauss_nodes.end()) {
        std::vector<double> h(2 * ngauss);
        gauleg_host(0, 1, ngauss, h.data(), h.data() + ngauss);
        DevBuf b;
        int rc = ensure(ctx, b, h.size() * sizeof(double));
        if (rc) return rc;
        FJ_CUDA(cudaMemcpy(b.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        it = ctx->gauss_nodes.emplace(ngauss, b).first;
    }
    *dptr = (const double *)it->second.p;
    return FJ_OK;
}

int poly_table(fj_ctx *ctx, int ngauss, int npoly, const double **dptr)
{
    auto key = std::make_pair(ngauss, npoly);
    auto it = ctx->poly.find(key);
    if (it == ctx->poly.end()) {
        std::vector<double> ci(ngauss), wi(ngauss), pol(npoly), h((size_t)npoly * ngauss);
        gauleg_host(0, 1, ngauss, ci.data(), wi.data());
        for (int g = 0; g < ngauss; g++) {
            evenlegend_host(npoly, ci[g], pol.data());
            for (int np = 0; np < npoly; np++) h[(size_t)np * ngauss + g] = 2 * pol[np] * wi[g];
        }
        DevBuf b;
        int rc = ensure(ctx, b, h.size() * sizeof(double));
        if (rc) return rc;
        FJ_CUDA(cudaMemcpy(b.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        it = ctx->poly.emplace(key, b).first;
    }
    *dptr = (const double *)it->second.p;
    return FJ_OK;
}

int gl_rule(fj_ctx *ctx, int n, GLRule *out)
{
    memset(out, 0, sizeof *out);
    if (n <= 0) return FJ_OK;
    auto it = ctx->gl_rules.find(n);
    if (it == ctx->gl_rules.end()) {
        std::vector<double> h(2 * n);
        gauleg_host(0, 1, n, h.data(), h.data() + n);
        DevBuf b;
        int rc = ensure(ctx, b, h.size() * sizeof(double));
        if (rc) return rc;
        FJ_CUDA(cudaMemcpy(b.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        it = ctx->gl_rules.emplace(n, b).first;
    }
    const double *p = (const double *)it->second.p;
    out->n = n;
    out->x01 = p;
    out->w01 = p + n;
    return FJ_OK;
}

int upload_rule(fj_ctx *ctx, const fj_quad_rule *r, const double **xq, const double **wq)
{
    std::vector<double> h(r->xq, r->xq + r->nq);
    h.insert(h.end(), r->wq, r->wq + r->nq);
    if (h != ctx->rule_host) {
        int rc = ensure(ctx, ctx->rule, h.size() * sizeof(double));
        if (rc) return rc;
        FJ_CUDA(cudaMemcpyAsync(ctx->rule.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        FJ_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->rule_host = h;
    }
    *xq = (const double *)ctx->rule.p;
    *wq = *xq + r->nq;
    return FJ_OK;
}

// Descriptors reach the device as bytes and fj_moments_batch compares them
// with the last upload (a graph capture must not upload): padding is zeroed.
DFDev df_dev(const fj_df_params *d)
{
    DFDev o;
    memset(&o, 0, sizeof o);
    o.kind = d->kind;
    o.alpha = d->alpha; o.beta = d->beta; o.J0 = d->J0;
    o.norm = d->mass / pow(d->J0, 3);
    o.tpi3 = pow(kTPI, 3.);
    o.dphi_h = d->dphi_h; o.dz_h = d->dz_h; o.dphi_g = d->dphi_g; o.dz_g = d->dz_g;
    o.chi = d->chi; o.k = d->k;
    return o;
}

int check_pot(fj_ctx *ctx, const fj_potential *p)
{
    if (!p || p->nr < 11 || p->npoly < 1 || p->npoly > kMaxPoly || !p->ar || !p->phil || !p->Pr || !p->Pr2)
        return fail(ctx, FJ_ERR_ARG, "potential: need 11 <= nr, 1 <= npoly <= 24 and all tables");
    return FJ_OK;
}

PotView view(const fj_potential *p) { return PotView{p->nr, p->npoly, p->ar, p->phil, p->Pr, p->Pr2}; }

// Validates one phase-space call and fills its launch arguments (without the
// scratch pointers).  mixed = the rule asks for the mixed-precision form.
int build_args(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
               const fj_quad_rule *rule, int ngauss, const double *Rz, int npts, double *out6, MomentArgs &a,
               bool &mixed)
{
    memset(&a, 0, sizeof a);  // padding too (the batch descriptors are compared as bytes)
    int rc = check_pot(ctx, pot);
    if (rc) return rc;
    if (!delta || delta->ngrid < 2 || !delta->Egrid || !delta->Dgrid) return fail(ctx, FJ_ERR_ARG, "delta table");
    if (!df || !rule || rule->nq < 1 || rule->nq > 64 || rule->jquad < 0 || rule->jquad > 64 || !out6 || npts < 1)
        return fail(ctx, FJ_ERR_ARG, "moments: bad rule, df or sizes");
    if (rule->precision != FJ_PREC_FP64 && rule->precision != FJ_PREC_MIXED)
        return fail(ctx, FJ_ERR_ARG, "moments: unknown precision mode");
    mixed = rule->precision == FJ_PREC_MIXED;
    if (mixed && (df->kind != FJ_DF_DPL || rule->jquad != FJ_JQUAD_QAGS))
        return fail(ctx, FJ_ERR_ARG, "moments: the mixed form takes the double-power-law DF and QAGS momentum integrals");
    a.P = view(pot);
    a.Eg = delta->Egrid; a.Dg = delta->Dgrid; a.ngrid = delta->ngrid;
    if ((rc = upload_rule(ctx, rule, &a.xq, &a.wq))) return rc;
    a.nq = rule->nq;
    if ((rc = gl_rule(ctx, rule->jquad, &a.gl))) return rc;
    a.df = df_dev(df);
    a.ci = nullptr; a.ngauss = ngauss; a.Rz = Rz; a.npts = npts;
    if (!Rz) {
        const double *gn;
        if ((rc = gauss_nodes(ctx, ngauss, &gn))) return rc;
        a.ci = gn;
    }
    const long long nq3 = (long long)rule->nq * rule->nq * rule->nq;
    a.mixed_chunk = ctx->mixed_chunk;
    a.blocks_per_point =
        mixed ? mixed_blocks_per_point(nq3, a.mixed_chunk) : (int)((nq3 + kPlainChunk - 1) / kPlainChunk);
    a.out6 = out6;
    a.jout = nullptr;
    return FJ_OK;
}

int read_stats(fj_ctx *ctx, long long nodes, fj_moment_stats *stats)
{
    unsigned long long h[kNumCounters];
    FJ_CUDA(cudaMemcpyAsync(h, ctx->counters.p, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats->nodes = nodes;
    stats->bound = (long long)h[kCntBound];
    stats->failures = (long long)h[kCntFailed];
    stats->kernel_ms = ms;
    stats->escalated = (long long)h[kCntEscalated];
    stats->fail_quad = (long long)h[kCntFailQuad];
    stats->fail_bracket = (long long)h[kCntFailBracket];
    stats->fail_root = (long long)h[kCntFailRoot];
    stats->resolved64 = (long long)h[kCntResolved64];
    return FJ_OK;
}

int run_moments(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
                const fj_quad_rule *rule, int ngauss, const double *Rz, int npts, double *out6,
                fj_moment_stats *stats)
{
    MomentArgs a;
    bool mixed = false;
    int rc = build_args(ctx, pot, delta, df, rule, ngauss, Rz, npts, out6, a, mixed);
    if (rc) return rc;
    if ((rc = ensure(ctx, ctx->partial, (size_t)npts * a.blocks_per_point * 6 * sizeof(double)))) return rc;
    const long long nq3 = (long long)rule->nq * rule->nq * rule->nq;
    DeferWork dw{};
    if (mixed) {
        const long long nb = (long long)npts * a.blocks_per_point;
        if ((rc = defer_setup(ctx, nb, defer_words(a.mixed_chunk), (long long)npts * nq3, dw, a.defer))) return rc;
        a.defer_count = dw.count;
    }
    if ((rc = ensure(ctx, ctx->counters, kNumCounters * sizeof(unsigned long long)))) return rc;
    a.partial = (double *)ctx->partial.p;
    a.counters = (unsigned long long *)ctx->counters.p;
    if (mixed && ctx->jout) {  // unbound nodes keep the all-ones (NaN) pattern
        a.jout = ctx->jout;
        FJ_CUDA(cudaMemsetAsync(a.jout, 0xFF, (size_t)npts * nq3 * 2 * sizeof(float), ctx->stream));
    }
    FJ_CUDA(cudaMemsetAsync(a.counters, 0, kNumCounters * sizeof(unsigned long long), ctx->stream));
    FJ_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    ItemQueue q{};
    if (mixed && (rc = queue_setup(ctx, (long long)npts * a.blocks_per_point, q))) return rc;
    FJ_CUDA(mixed ? launch_moments_mixed(a, ctx->mixed_variant, dw, q, ctx->stream) : launch_moments(a, ctx->stream));
    FJ_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    return stats ? read_stats(ctx, nq3 * npts, stats) : FJ_OK;
}

}  // namespace

namespace fj {
int context_grid_inputs(fj_ctx *ctx, int ngauss, const fj_quad_rule *rule, const double **ci, const double **xq,
                        const double **wq)
{
    int rc = gauss_nodes(ctx, ngauss, ci);
    if (rc) return rc;
    return upload_rule(ctx, rule, xq, wq);
}
}  // namespace fj

// =================================================================== ABI
extern "C" {

int fj_set_action_output(fj_ctx *ctx, float *jout)
{
    if (!ctx) return FJ_ERR_ARG;
    ctx->jout = jout;
    return FJ_OK;
}


const char *fj_version(void) { return "fjmodels-gb300 0.1 (sm_103a)"; }

int fj_ctx_create(int device, fj_ctx **out)
{
    if (!out) return FJ_ERR_ARG;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) return FJ_ERR_NODEVICE;
    fj_ctx *c = new fj_ctx;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->own, cudaStreamDefault) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        delete c;
        return FJ_ERR_CUDA;
    }
    c->stream = c->own;
    // The phase-space kernels keep the QAGS interval list on the per-thread
    // call stack (about 5.5 KB, ptxas "cumulative stack size"); the function
    // attributes do not report call-stack frames, so the floor is explicit.
    size_t need = moments_local_bytes();
    for (size_t n2 : {multipole_local_bytes(), moments_mixed_local_bytes(), delta_local_bytes(), los_local_bytes()})
        if (n2 > need) need = n2;
    need = (need + 1024 + 1023) / 1024 * 1024;
    if (need < kStackBytes) need = kStackBytes;
    size_t cur = 0;
    if (cudaDeviceGetLimit(&cur, cudaLimitStackSize) != cudaSuccess ||
        (cur < need && cudaDeviceSetLimit(cudaLimitStackSize, need) != cudaSuccess)) {
        cudaEventDestroy(c->ev0);
        cudaEventDestroy(c->ev1);
        cudaStreamDestroy(c->own);
        delete c;
        return FJ_ERR_CUDA;
    }
    *out = c;
    return FJ_OK;
}

int fj_ctx_destroy(fj_ctx *ctx)
{
    if (!ctx) return FJ_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (DevBuf *b : {&ctx->partial, &ctx->counters, &ctx->rule, &ctx->misc, &ctx->defer, &ctx->queue})
        if (b->p) cudaFree(b->p);
    for (auto &kv : ctx->gauss_nodes) cudaFree(kv.second.p);
    for (auto &kv : ctx->poly) cudaFree(kv.second.p);
    for (auto &kv : ctx->gl_rules) cudaFree(kv.second.p);
    cudaEventDestroy(ctx->ev0);
    cudaEventDestroy(ctx->ev1);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
    return FJ_OK;
}

int fj_ctx_set_stream(fj_ctx *ctx, void *stream)
{
    if (!ctx) return FJ_ERR_ARG;
    ctx->stream = (cudaStream_t)stream;
    return FJ_OK;
}

void *fj_ctx_own_stream(fj_ctx *ctx) { return ctx ? (void *)ctx->own : nullptr; }

int fj_ctx_synchronize(fj_ctx *ctx)
{
    if (!ctx) return FJ_ERR_ARG;
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    return FJ_OK;
}

const char *fj_last_error(fj_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int fj_moments(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
               const fj_quad_rule *rule, int ngauss, double *grids6, fj_moment_stats *stats)
{
    if (!ctx || !pot || ngauss < 1) return fail(ctx, FJ_ERR_ARG, "moments: bad arguments");
    return run_moments(ctx, pot, delta, df, rule, ngauss, nullptr, pot->nr * ngauss, grids6, stats);
}

int fj_moments_points(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
                      const fj_quad_rule *rule, const double *Rz, int npts, double *out6, fj_moment_stats *stats)
{
    if (!ctx || !Rz) return fail(ctx, FJ_ERR_ARG, "moments_points: bad arguments");
    return run_moments(ctx, pot, delta, df, rule, 0, Rz, npts, out6, stats);
}

int fj_moments_batch(fj_ctx *ctx, int n, const fj_batch_item *items, const fj_quad_rule *rule,
                     fj_moment_stats *stats)
{
    if (!ctx || n < 1 || !items || !rule) return fail(ctx, FJ_ERR_ARG, "moments_batch: bad arguments");
    std::vector<MomentArgs> args(n);
    std::vector<int> bs(n + 1, 0), ps(n + 1, 0);
    size_t smem = 0, partial = 0, defer_words_total = 0;
    bool mixed = false;
    long long nodes = 0;
    const long long nq3 = (long long)rule->nq * rule->nq * rule->nq;
    for (int m = 0; m < n; m++) {
        const fj_batch_item &it = items[m];
        if (it.ngauss < 1) return fail(ctx, FJ_ERR_ARG, "moments_batch: ngauss");
        const int npts = it.pot.nr * it.ngauss;
        bool mx = false;
        int rc = build_args(ctx, &it.pot, &it.delta, &it.df, rule, it.ngauss, nullptr, npts, it.grids6, args[m], mx);
        if (rc) return rc;
        mixed = mx;
        const long long nb = (long long)npts * args[m].blocks_per_point;
        if (bs[m] + nb > 0x7fffffffLL) return fail(ctx, FJ_ERR_ARG, "moments_batch: too many blocks");
        bs[m + 1] = bs[m] + (int)nb;
        ps[m + 1] = ps[m] + npts;
        args[m].partial = reinterpret_cast<double *>(partial);  // offset, made a pointer below
        partial += (size_t)nb * 6;
        if (mixed) {  // offsets, made pointers below
            args[m].defer = reinterpret_cast<unsigned *>(defer_words_total);
            args[m].defer_count = reinterpret_cast<int *>((size_t)bs[m]);
            defer_words_total += (size_t)nb * defer_words(args[m].mixed_chunk);
        }
        const size_t sm = mixed ? moment_mixed_smem_bytes(args[m]) : moment_smem_bytes(args[m]);
        smem = sm > smem ? sm : smem;
        nodes += nq3 * npts;
    }
    int rc;
    if ((rc = ensure(ctx, ctx->partial, partial * sizeof(double)))) return rc;
    DeferWork dw{};
    unsigned *bitmaps = nullptr;
    if (mixed && (rc = defer_setup(ctx, bs[n], defer_words(ctx->mixed_chunk), nodes, dw, bitmaps))) return rc;
    if ((rc = ensure(ctx, ctx->counters, kNumCounters * sizeof(unsigned long long)))) return rc;
    for (int m = 0; m < n; m++) {
        args[m].partial = (double *)ctx->partial.p + reinterpret_cast<size_t>(args[m].partial);
        if (mixed) {
            args[m].defer = bitmaps + reinterpret_cast<size_t>(args[m].defer);
            args[m].defer_count = dw.count + reinterpret_cast<size_t>(args[m].defer_count);
        }
        args[m].counters = (unsigned long long *)ctx->counters.p;
    }
    // descriptor block: MomentArgs[n] | block_start[n+1] | point_start[n+1]
    const size_t bytes = n * sizeof(MomentArgs) + 2 * (n + 1) * sizeof(int);
    std::vector<char> host(bytes);
    memcpy(host.data(), args.data(), n * sizeof(MomentArgs));
    memcpy(host.data() + n * sizeof(MomentArgs), bs.data(), (n + 1) * sizeof(int));
    memcpy(host.data() + n * sizeof(MomentArgs) + (n + 1) * sizeof(int), ps.data(), (n + 1) * sizeof(int));
    if (ctx->batch_host != host) {  // unchanged descriptors are not re-sent (graph capture repeats the call)
        if ((rc = ensure(ctx, ctx->batch, bytes))) return rc;
        FJ_CUDA(cudaMemcpyAsync(ctx->batch.p, host.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
        FJ_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->batch_host.swap(host);
    }
    const char *db = (const char *)ctx->batch.p;
    const MomentBatch b{(const MomentArgs *)db, (const int *)(db + n * sizeof(MomentArgs)),
                        (const int *)(db + n * sizeof(MomentArgs) + (n + 1) * sizeof(int)), n};
    FJ_CUDA(cudaMemsetAsync(ctx->counters.p, 0, kNumCounters * sizeof(unsigned long long), ctx->stream));
    FJ_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    ItemQueue q{};
    if (mixed && (rc = queue_setup(ctx, bs[n], q))) return rc;
    FJ_CUDA(launch_moments_batch(args[0], b, bs[n], smem, mixed, ctx->mixed_variant, dw, q, ctx->stream));
    FJ_CUDA(launch_moments_finalize_batch(b, ps[n], ctx->stream));
    FJ_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    return stats ? read_stats(ctx, nodes, stats) : FJ_OK;
}

int fj_set_mixed_config(fj_ctx *ctx, int variant, int nodes_per_block)
{
    if (!ctx || variant < 0 || variant >= kMixedVariants || nodes_per_block < kMixedBlock ||
        nodes_per_block > kMixedMaxNodes)
        return fail(ctx, FJ_ERR_ARG, "set_mixed_config: variant or nodes per block out of range");
    ctx->mixed_variant = variant;
    ctx->mixed_chunk = nodes_per_block;
    return FJ_OK;
}

int fj_get_mixed_config(fj_ctx *ctx, int *variant, int *nodes_per_block)
{
    if (!ctx || !variant || !nodes_per_block) return FJ_ERR_ARG;
    *variant = ctx->mixed_variant;
    *nodes_per_block = ctx->mixed_chunk;
    return FJ_OK;
}

int fj_autotune_mixed(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
                      const fj_quad_rule *rule, const double *Rz, int npts, double *out6, double *best_ms,
                      double *all_ms)
{
    if (!ctx || !rule || rule->precision != FJ_PREC_MIXED || !Rz || npts < 1 || !out6)
        return fail(ctx, FJ_ERR_ARG, "autotune_mixed: needs a mixed-precision rule and sample points");
    static const int chunks[] = {1024, 2048, 4096};
    const int v0 = ctx->mixed_variant, c0 = ctx->mixed_chunk;
    int bv = v0, bc = c0;
    double best = -1;
    for (int v = 0; v < kMixedVariants; v++)
        for (int ci = 0; ci < 3; ci++) {
            ctx->mixed_variant = v;
            ctx->mixed_chunk = chunks[ci];
            double ms = -1;
            for (int rep = 0; rep < 2; rep++) {  // the faster of two launches (the first may pay one-time costs)
                fj_moment_stats st;
                int rc = run_moments(ctx, pot, delta, df, rule, 0, Rz, npts, out6, &st);
                if (rc) { ctx->mixed_variant = v0; ctx->mixed_chunk = c0; return rc; }
                if (ms < 0 || st.kernel_ms < ms) ms = st.kernel_ms;
            }
            if (all_ms) all_ms[v * 3 + ci] = ms;
            if (best < 0 || ms < best) { best = ms; bv = v; bc = chunks[ci]; }
        }
    ctx->mixed_variant = bv;
    ctx->mixed_chunk = bc;
    if (best_ms) *best_ms = best;
    return FJ_OK;
}

int fj_legendre_project(fj_ctx *ctx, int nr, int ngauss, int npoly, const double *ar, const double *grids6,
                        double *coef6)
{
    if (!ctx || nr < 3 || ngauss < 1 || npoly < 1 || npoly > kMaxPoly || !ar || !grids6 || !coef6)
        return fail(ctx, FJ_ERR_ARG, "legendre_project: bad arguments");
    const double *poly;
    int rc = poly_table(ctx, ngauss, npoly, &poly);
    if (rc) return rc;
    FJ_CUDA(launch_project(nr, ngauss, npoly, ar, poly, grids6, coef6, ctx->stream));
    return FJ_OK;
}

int fj_poisson(fj_ctx *ctx, int nr, int npoly, const double *ar, const double *rhl, double *phil, double *Pr,
               double *Pr2)
{
    if (!ctx || nr < 2 || npoly < 1 || npoly > kMaxPoly || !ar || !rhl || !phil || !Pr || !Pr2)
        return fail(ctx, FJ_ERR_ARG, "poisson: bad arguments");
    if (ctx->poisson == FJ_POISSON_CUMULATIVE) {
        if (nr > kPoissonCumulativeMaxNr) return fail(ctx, FJ_ERR_ARG, "poisson: too many radii");
        FJ_CUDA(launch_poisson_cumulative(nr, npoly, ar, rhl, phil, Pr, Pr2, ctx->stream));
        return FJ_OK;
    }
    int rc = ensure(ctx, ctx->counters, kNumCounters * sizeof(unsigned long long));
    if (rc) return rc;
    FJ_CUDA(launch_poisson(nr, npoly, ar, rhl, phil, Pr, Pr2, (unsigned long long *)ctx->counters.p, ctx->stream));
    return FJ_OK;
}

int fj_set_poisson(fj_ctx *ctx, int mode)
{
    if (!ctx || (mode != FJ_POISSON_QAGS && mode != FJ_POISSON_CUMULATIVE))
        return fail(ctx, FJ_ERR_ARG, "set_poisson: unknown mode");
    ctx->poisson = mode;
    return FJ_OK;
}

int fj_get_poisson(fj_ctx *ctx, int *mode)
{
    if (!ctx || !mode) return FJ_ERR_ARG;
    *mode = ctx->poisson;
    return FJ_OK;
}

int fj_sum_potentials(fj_ctx *ctx, int n, const double *phil_a, const double *Pr_a, const double *Pr2_a,
                      const double *phil_b, const double *Pr_b, const double *Pr2_b, double *phil, double *Pr,
                      double *Pr2)
{
    if (!ctx || n < 1) return fail(ctx, FJ_ERR_ARG, "sum_potentials: bad arguments");
    FJ_CUDA(launch_sum3(n, phil_a, Pr_a, Pr2_a, phil_b, Pr_b, Pr2_b, phil, Pr, Pr2, ctx->stream));
    return FJ_OK;
}

int fj_compute_new_phi(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
                       const fj_quad_rule *rule, int ngauss, double *grids6, double *coef6, double *phil_out,
                       double *Pr_out, double *Pr2_out, fj_moment_stats *stats)
{
    int rc = fj_moments(ctx, pot, delta, df, rule, ngauss, grids6, stats);
    if (rc) return rc;
    if ((rc = fj_legendre_project(ctx, pot->nr, ngauss, pot->npoly, pot->ar, grids6, coef6))) return rc;
    return fj_poisson(ctx, pot->nr, pot->npoly, pot->ar, coef6, phil_out, Pr_out, Pr2_out);
}

int fj_actions(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const double *pts, size_t n,
               int jquad, double *out)
{
    if (!ctx) return FJ_ERR_ARG;
    int rc = check_pot(ctx, pot);
    if (rc) return rc;
    if (!delta || delta->ngrid < 2 || !pts || !out || jquad < 0 || jquad > 64)
        return fail(ctx, FJ_ERR_ARG, "actions: bad arguments");
    GLRule gl;
    if ((rc = gl_rule(ctx, jquad, &gl))) return rc;
    FJ_CUDA(launch_actions(view(pot), delta->Egrid, delta->Dgrid, delta->ngrid, gl, pts, n, out, ctx->stream));
    return FJ_OK;
}

int fj_potential_eval(fj_ctx *ctx, const fj_potential *pot, const double *Rz, size_t n, double *out)
{
    if (!ctx) return FJ_ERR_ARG;
    int rc = check_pot(ctx, pot);
    if (rc) return rc;
    if (!Rz || !out) return fail(ctx, FJ_ERR_ARG, "potential_eval: bad arguments");
    FJ_CUDA(launch_potential_eval(view(pot), Rz, n, out, ctx->stream));
    return FJ_OK;
}

int fj_vir2(fj_ctx *ctx, const fj_potential *pot, int ngauss, const double *coef6, double *out7)
{
    if (!ctx) return FJ_ERR_ARG;
    int rc = check_pot(ctx, pot);
    if (rc) return rc;
    if (ngauss < 1 || !coef6 || !out7) return fail(ctx, FJ_ERR_ARG, "vir2: bad arguments");
    const double *gn;
    if ((rc = gauss_nodes(ctx, ngauss, &gn))) return rc;
    if ((rc = ensure(ctx, ctx->misc, 8 * sizeof(double)))) return rc;
    FJ_CUDA(launch_vir2(view(pot), ngauss, gn, gn + ngauss, coef6, (double *)ctx->misc.p, ctx->stream));
    FJ_CUDA(cudaMemcpyAsync(out7, ctx->misc.p, 7 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    return FJ_OK;
}

// ------------------------------------------- line of sight, velocity PDFs
// the 22-point [0,1] tanh-sinh table of include/GaussPts.h:91-134:
// x_k = (1 + tanh(pi/2 sinh(k h)))/2, w_k = h pi/4 cosh(k h)/cosh^2(pi/2 sinh(k h)),
// h = 2/11, k = -11..10, each rounded to the table's 12 significant digits
int fj_tanh_sinh01(double *x, double *w)
{
    if (!x || !w) return FJ_ERR_ARG;
    const double h = 2. / 11.;
    for (int i = 0; i < kLos01; i++) {
        const double t = (i - 11) * h, u = kPI / 2 * sinh(t);
        char buf[40];
        snprintf(buf, sizeof buf, "%.12g", .5 * (1 + tanh(u)));
        x[i] = strtod(buf, nullptr);
        snprintf(buf, sizeof buf, "%.12g", h * kPI / 4 * cosh(t) / pow(cosh(u), 2));
        w[i] = strtod(buf, nullptr);
    }
    return FJ_OK;
}

int fj_los(fj_ctx *ctx, const fj_potential *pot, const fj_delta_table *delta, const fj_df_params *df,
           const fj_quad_rule *rule, const double *rhl, int kind, const double *Rzv, int n, double *out,
           fj_moment_stats *stats)
{
    if (!ctx) return FJ_ERR_ARG;
    if (kind < FJ_LOS_SIGMA || kind > FJ_LOS_PVR || !Rzv || n < 1 || !out)
        return fail(ctx, FJ_ERR_ARG, "los: bad kind, points or output");
    if ((kind == FJ_LOS_SIGMA || kind == FJ_LOS_LINE) && !rhl)
        return fail(ctx, FJ_ERR_ARG, "los: SigmaDF needs the density multipoles");
    if (!rule || rule->precision != FJ_PREC_FP64) return fail(ctx, FJ_ERR_ARG, "los: FP64 rule only");
    LosArgs a;
    bool mixed = false;
    int rc = build_args(ctx, pot, delta, df, rule, 0, Rzv, n, out, a.m, mixed);
    if (rc) return rc;
    if ((rc = ensure(ctx, ctx->counters, kNumCounters * sizeof(unsigned long long)))) return rc;
    a.m.counters = (unsigned long long *)ctx->counters.p;
    a.rhl = rhl; a.kind = kind; a.Rzv = Rzv; a.n = n; a.out = out;
    fj_tanh_sinh01(a.x01, a.w01);
    a.blocks_per_item = los_blocks_per_item(kind, rule->nq);
    if ((long long)n * a.blocks_per_item > 0x7fffffffLL) return fail(ctx, FJ_ERR_ARG, "los: too many values");
    if ((rc = ensure(ctx, ctx->partial, (size_t)n * a.blocks_per_item * sizeof(double)))) return rc;
    a.partial = (double *)ctx->partial.p;
    FJ_CUDA(cudaMemsetAsync(ctx->counters.p, 0, kNumCounters * sizeof(unsigned long long), ctx->stream));
    FJ_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    FJ_CUDA(launch_los(a, ctx->stream));
    FJ_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (stats) {
        const long long nq = rule->nq;
        const long long per = kind == FJ_LOS_LINE ? nq * nq * nq
                              : kind == FJ_LOS_PVPHI ? (long long)kLos01 * kLos01
                              : kind == FJ_LOS_SIGMA ? 0 : kLos01 * nq;
        return read_stats(ctx, per * n, stats);
    }
    return FJ_OK;
}

// ------------------------------------------------------------ host setup
int fj_log_grid(double rmin, double rmax, int n, double *ar)
{
    if (n < 2 || !(rmin > 0) || !(rmax > rmin) || !ar) return FJ_ERR_ARG;
    for (int i = 0; i < n; i++) ar[i] = pow(10., log10(rmin) + (log10(rmax) - log10(rmin)) * i / (n - 1));
    return FJ_OK;
}

int fj_gauleg(double x1, double x2, int n, double *x, double *w)
{
    if (n < 1 || !x || !w) return FJ_ERR_ARG;
    gauleg_host(x1, x2, n, x, w);
    return FJ_OK;
}

int fj_guess_rhl(int nr, int ngauss, int npoly, const double *ar, int kind, double mass, double r0, double q,
                 double *rhl)
{
    if (nr < 1 || ngauss < 1 || npoly < 1 || npoly > kMaxPoly || !ar || !rhl || kind < 0 || kind > 3)
        return FJ_ERR_ARG;
    const double q2 = q * q;
    auto rho = [&](double R, double z) {  // pot/models.cpp:40-56
        const double m = sqrt(R * R + z * z / q2);
        if (kind == FJ_GUESS_ISOCHRONE) {
            const double a = sqrt(r0 * r0 + m * m);
            return mass / kFPI / (q * pow((a + r0) * a, 2) * a) * r0 * (r0 + 2 * a);
        }
        if (kind == FJ_GUESS_NFW) return mass / (m / r0 * pow(r0 + m, 2)) / kFPI;
        if (kind == FJ_GUESS_NFWEXT) return mass / (m / r0 * pow(r0 + m, 1)) / kFPI;
        return mass / (m / r0 * pow(r0 + m, 3)) / kTPI;
    };
    std::vector<double> ci(ngauss), wi(ngauss), si(ngauss), pol(npoly);
    gauleg_host(0, 1, ngauss, ci.data(), wi.data());
    for (int g = 0; g < ngauss; g++) si[g] = sqrt(1 - ci[g] * ci[g]);
    std::vector<double> poly((size_t)npoly * ngauss);
    for (int g = 0; g < ngauss; g++) {
        evenlegend_host(npoly, ci[g], pol.data());
        for (int np = 0; np < npoly; np++) poly[(size_t)np * ngauss + g] = 2 * pol[np] * wi[g];
    }
    for (int n = 0; n < nr; n++)
        for (int np = 0; np < npoly; np++) {
            double s = 0.;
            for (int g = 0; g < ngauss; g++) s += poly[(size_t)np * ngauss + g] * rho(ar[n] * si[g], ar[n] * ci[g]);
            rhl[n * npoly + np] = s;
        }
    rhl[0] = 2 * rho(ar[0] * si[0], ar[0] * ci[0]);
    return FJ_OK;
}

}  // extern "C"

// --------------------------------------------------- focal-distance table
// tabulateDelta (delta/tabulate.cpp:13-38) on the host (fj_delta.cuh); the
// energies are independent, so host threads take them in turn (each entry is
// the same computation whichever thread runs it: the same bits as one thread).
// fj_tabulate_delta_batch runs the same code per (model, energy) on the GPU.
extern "C" int fj_tabulate_delta(const fj_potential *pot, int ngrid, double *Egrid, double *Dgrid)
{
    if (!pot || pot->nr < 11 || pot->npoly < 1 || pot->npoly > kMaxPoly || ngrid < 2 || !Egrid || !Dgrid)
        return FJ_ERR_ARG;
    const PotView P = view(pot);
    const DeltaBase base = delta_base(P);
    const int nthreads = (int)std::max(1u, std::min((unsigned)ngrid, std::thread::hardware_concurrency()));
    std::vector<DeltaFit> fits(nthreads);
    std::vector<char> bad(nthreads, base.bad ? 1 : 0);
    auto work = [&](int t) {
        bool b = false;
        for (int nE = t; nE < ngrid; nE += nthreads)
            Dgrid[nE] = delta_energy(P, base, nE, ngrid, Egrid[nE], fits[t], b, kDeltaWalkCapHost);
        if (b) bad[t] = 1;
    };
    // a share whose thread cannot be started runs on the calling thread (no
    // exception crosses the C ABI)
    std::vector<std::thread> pool;
    int started = 1;
    try {
        for (; started < nthreads; started++) pool.emplace_back(work, started);
    } catch (...) {
    }
    work(0);
    for (int t = started; t < nthreads; t++) work(t);
    for (auto &th : pool) th.join();
    for (char b : bad)
        if (b) return FJ_ERR_ARG;
    return FJ_OK;
}

// The focal-distance tables of n models on the GPU (fj_delta.cu): views of
// the models' device potentials and the device tables to fill, uploaded to
// the context; fixed addresses, so a launch can be captured in a graph.
namespace {
struct DeltaDev {
    const PotView *views;
    double *const *Eg;
    double *const *Dg;
    int *bad;
    int n;
};

int delta_prepare(fj_ctx *ctx, int n, const PotView *views, double *const *Eg, double *const *Dg, DeltaDev &dd)
{
    const size_t bytes = n * (sizeof(PotView) + 2 * sizeof(double *) + sizeof(int));
    int rc = ensure(ctx, ctx->delta_ws, bytes);
    if (rc) return rc;
    std::vector<char> h(bytes);
    char *p = h.data();
    memcpy(p, views, n * sizeof(PotView));
    memcpy(p + n * sizeof(PotView), Eg, n * sizeof(double *));
    memcpy(p + n * (sizeof(PotView) + sizeof(double *)), Dg, n * sizeof(double *));
    memset(p + n * (sizeof(PotView) + 2 * sizeof(double *)), 0, n * sizeof(int));
    char *d = (char *)ctx->delta_ws.p;
    FJ_CUDA(cudaMemcpyAsync(d, h.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));  // h is pageable and goes out of scope
    dd.views = (const PotView *)d;
    dd.Eg = (double *const *)(d + n * sizeof(PotView));
    dd.Dg = (double *const *)(d + n * (sizeof(PotView) + sizeof(double *)));
    dd.bad = (int *)(d + n * (sizeof(PotView) + 2 * sizeof(double *)));
    dd.n = n;
    return FJ_OK;
}

// n status flags back to the host: 0, or FJ_ERR_ARG where a search hit its cap
int delta_status(fj_ctx *ctx, const DeltaDev &dd, int *status)
{
    std::vector<int> h(dd.n);
    FJ_CUDA(cudaMemcpyAsync(h.data(), dd.bad, dd.n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    int any = 0;
    for (int m = 0; m < dd.n; m++) {
        if (status) status[m] = h[m] ? FJ_ERR_ARG : FJ_OK;
        any |= h[m];
    }
    return any;
}
}  // namespace

extern "C" int fj_tabulate_delta_batch(fj_ctx *ctx, int n, const fj_potential *pots, int ngrid, double *Egrid,
                                       double *Dgrid, int *status)
{
    if (!ctx) return FJ_ERR_ARG;
    if (n < 1 || !pots || ngrid < 2 || !Egrid || !Dgrid) return fail(ctx, FJ_ERR_ARG, "tabulate_delta_batch: arguments");
    std::vector<PotView> views(n);
    std::vector<double *> eg(n), dg(n);
    for (int m = 0; m < n; m++) {
        int rc = check_pot(ctx, &pots[m]);
        if (rc) return rc;
        if (pots[m].nr < 11) return fail(ctx, FJ_ERR_ARG, "tabulate_delta_batch: nr < 11");
        views[m] = view(&pots[m]);
        eg[m] = Egrid + (size_t)m * ngrid;
        dg[m] = Dgrid + (size_t)m * ngrid;
    }
    DeltaDev dd;
    int rc = delta_prepare(ctx, n, views.data(), eg.data(), dg.data(), dd);
    if (rc) return rc;
    FJ_CUDA(launch_tabulate_delta(dd.views, dd.Eg, dd.Dg, n, ngrid, dd.bad, ctx->stream));
    delta_status(ctx, dd, status);
    return FJ_OK;
}

// ------------------------------------------------------ coefficient file
extern "C" int fj_write_out(const char *path, int nr, int npoly, int ngauss, const double *hdr10, const double *ar,
                            const double *mats9)
{
    return fj_write_out_digits(path, nr, npoly, ngauss, hdr10, ar, mats9, 0);
}

extern "C" int fj_write_out_digits(const char *path, int nr, int npoly, int ngauss, const double *hdr10,
                                   const double *ar, const double *mats9, int digits)
{
    if (!path || nr < 1 || npoly < 1 || !hdr10 || !ar || !mats9 || digits < 0 || digits > 17) return FJ_ERR_ARG;
    std::ofstream outF(path, std::ios::out);
    if (!outF.is_open()) return FJ_ERR_IO;
    if (digits > 0) outF.precision(digits);
    // header (io/writeOut.cpp:81-85): sizes, h/g coefficients, chi mass r0, A B
    outF << nr << " " << npoly << " " << ngauss << std::endl;
    outF << hdr10[0] << " " << hdr10[1] << " " << hdr10[2] << " " << hdr10[3] << std::endl;
    outF << hdr10[4] << " " << hdr10[5] << " " << hdr10[6] << std::endl;
    outF << hdr10[7] << " " << hdr10[8] << std::endl;
    for (int i = 0; i < nr; i++) outF << ar[i] << std::endl;  // writeArr (:45-49)
    for (int m = 0; m < 9; m++)                                  // writeMat (:51-59)
        for (int i = 0; i < nr; i++) {
            for (int j = 0; j < npoly; j++) outF << mats9[(size_t)m * nr * npoly + (size_t)i * npoly + j] << " ";
            outF << std::endl;
        }
    outF.close();
    return outF.fail() ? FJ_ERR_IO : FJ_OK;
}

// The file of fj_write_out read back: header, ar, nine [nr][npoly] tables.
extern "C" int fj_read_out(const char *path, int *nr, int *npoly, int *ngauss, double *hdr10, double *ar,
                           double *mats9)
{
    if (!path || !nr || !npoly || !ngauss || !hdr10 || (!ar != !mats9)) return FJ_ERR_ARG;
    std::ifstream in(path);
    if (!in.is_open()) return FJ_ERR_IO;
    long long n = 0, np = 0, ng = 0;
    if (!(in >> n >> np >> ng) || n < 1 || np < 1 || ng < 0 || n > (1 << 20) || np > (1 << 10)) return FJ_ERR_ARG;
    for (int i = 0; i < 9; i++)
        if (!(in >> hdr10[i])) return FJ_ERR_ARG;
    hdr10[9] = 0;
    *nr = (int)n; *npoly = (int)np; *ngauss = (int)ng;
    if (!ar) return FJ_OK;
    for (long long i = 0; i < n; i++)
        if (!(in >> ar[i])) return FJ_ERR_ARG;
    for (long long i = 0; i < 9 * n * np; i++)
        if (!(in >> mats9[i])) return FJ_ERR_ARG;
    double extra;
    return (in >> extra) ? FJ_ERR_ARG : FJ_OK;  // nothing may follow the last table
}

// ------------------------------------------------------------ whole model
static bool anderson_args_ok(int depth, double beta)
{
    return depth >= 0 && depth <= FJ_ANDERSON_MAX_DEPTH && beta > 0 && beta <= 4;
}

extern "C" int fj_anderson_reset(fj_ctx *ctx, int depth, double beta)
{
    if (!ctx || !anderson_args_ok(depth, beta))
        return fail(ctx, FJ_ERR_ARG, "anderson_reset: depth in [0, FJ_ANDERSON_MAX_DEPTH] and beta in (0, 4]");
    ctx->anderson = fj_anderson{};
    ctx->anderson.depth = depth;
    ctx->anderson.beta = beta;
    return FJ_OK;
}

extern "C" int fj_anderson_create(int depth, double beta, fj_anderson **out)
{
    if (!out || !anderson_args_ok(depth, beta)) return FJ_ERR_ARG;
    *out = new (std::nothrow) fj_anderson;
    if (!*out) return FJ_ERR_NOMEM;
    (*out)->depth = depth;
    (*out)->beta = beta;
    return FJ_OK;
}

extern "C" int fj_anderson_destroy(fj_anderson *a)
{
    delete a;
    return FJ_OK;
}

// Least squares min |r - sum_j c_j A_j| over the columns A_j (modified Gram-Schmidt;
// a column whose remaining norm is below 1e-12 of its own is left out, c_j = 0).
static std::vector<double> lsq_columns(const std::vector<std::vector<double>> &A, const std::vector<double> &r)
{
    const int m = (int)A.size(), n = (int)r.size();
    std::vector<std::vector<double>> Q(A);
    std::vector<double> R((size_t)m * m, 0.0), c(m, 0.0);
    std::vector<bool> keep(m, true);
    for (int j = 0; j < m; j++) {
        double n0 = 0;
        for (int i = 0; i < n; i++) n0 += A[j][i] * A[j][i];
        for (int k = 0; k < j; k++) {
            if (!keep[k]) continue;
            double d = 0;
            for (int i = 0; i < n; i++) d += Q[k][i] * Q[j][i];
            R[k * m + j] = d;
            for (int i = 0; i < n; i++) Q[j][i] -= d * Q[k][i];
        }
        double nn = 0;
        for (int i = 0; i < n; i++) nn += Q[j][i] * Q[j][i];
        if (!(nn > 1e-24 * n0) || nn == 0) { keep[j] = false; continue; }
        nn = std::sqrt(nn);
        R[j * m + j] = nn;
        for (int i = 0; i < n; i++) Q[j][i] /= nn;
    }
    std::vector<double> qr(m, 0.0);
    for (int j = 0; j < m; j++)
        if (keep[j])
            for (int i = 0; i < n; i++) qr[j] += Q[j][i] * r[i];
    for (int j = m - 1; j >= 0; j--) {
        if (!keep[j]) continue;
        double v = qr[j];
        for (int k = j + 1; k < m; k++)
            if (keep[k]) v -= R[j * m + k] * c[k];
        c[j] = v / R[j * m + j];
    }
    return c;
}

// One mixing step on host tables: hx the last input, hg its output ([3][nr*npoly]
// each), xn the next input; *change (may be NULL) the plain step's change.
static void anderson_update(fj_anderson &H, int nr, int npoly, const std::vector<double> &hx,
                            const std::vector<double> &hg, std::vector<double> &xn, double *change)
{
    const int nt = nr * npoly, n = 3 * nt;
    // the residual as the stopping test weighs it: phil, per radius over |phil(r, 0)|
    std::vector<double> res(nt);
    double maxd = 0;
    for (int i = 0; i < nr; i++)
        for (int j = 0; j < npoly; j++) {
            res[i * npoly + j] = (hg[i * npoly + j] - hx[i * npoly + j]) / std::fabs(hg[i * npoly]);
            maxd = std::fmax(maxd, std::fabs(res[i * npoly + j]));
        }
    if (change) *change = maxd;
    if (H.last >= 0 && maxd > 2 * H.last) { H.f.clear(); H.g.clear(); H.x.clear(); }  // diverging: restart
    H.last = maxd;
    xn = hg;
    if (H.depth > 0) {
        const bool relax = H.beta != 1;
        H.f.push_back(res);
        H.g.push_back(hg);
        if (relax) H.x.push_back(hx);
        if ((int)H.f.size() > H.depth + 1) {
            H.f.erase(H.f.begin());
            H.g.erase(H.g.begin());
            if (relax) H.x.erase(H.x.begin());
        }
        const int m = (int)H.f.size() - 1;
        std::vector<double> xbar(hx);
        if (m > 0) {
            std::vector<std::vector<double>> dF(m, std::vector<double>(nt));
            for (int j = 0; j < m; j++)
                for (int i = 0; i < nt; i++) dF[j][i] = H.f[j + 1][i] - H.f[j][i];
            const std::vector<double> c = lsq_columns(dF, res);
            for (int j = 0; j < m; j++)
                for (int i = 0; i < n; i++) {
                    xn[i] -= c[j] * (H.g[j + 1][i] - H.g[j][i]);
                    if (relax) xbar[i] -= c[j] * (H.x[j + 1][i] - H.x[j][i]);
                }
        }
        // beta != 1: the mixed input plus beta times the mixed residual
        if (relax)
            for (int i = 0; i < n; i++) xn[i] = xbar[i] + H.beta * (xn[i] - xbar[i]);
    }
}

extern "C" int fj_anderson_step(fj_ctx *ctx, int nr, int npoly, double *x, const double *g, double *change)
{
    if (!ctx || nr < 1 || npoly < 1 || !x || !g) return fail(ctx, FJ_ERR_ARG, "anderson_step: bad arguments");
    const int n = 3 * nr * npoly;
    std::vector<double> hx(n), hg(n), xn;
    FJ_CUDA(cudaMemcpyAsync(hx.data(), x, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FJ_CUDA(cudaMemcpyAsync(hg.data(), g, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    anderson_update(ctx->anderson, nr, npoly, hx, hg, xn, change);
    FJ_CUDA(cudaMemcpyAsync(x, xn.data(), n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    FJ_CUDA(cudaStreamSynchronize(ctx->stream));
    return FJ_OK;
}

extern "C" int fj_anderson_host_step(fj_anderson *a, int nr, int npoly, double *x, const double *g, double *change)
{
    if (!a || nr < 1 || npoly < 1 || !x || !g) return FJ_ERR_ARG;
    const int n = 3 * nr * npoly;
    std::vector<double> hx(x, x + n), hg(g, g + n), xn;
    anderson_update(*a, nr, npoly, hx, hg, xn, change);
    std::copy(xn.begin(), xn.end(), x);
    return FJ_OK;
}

extern "C" int fj_run_model(fj_ctx *ctx, const fj_model_config *cfg, fj_model_result *res)
{
    if (!ctx || !cfg || !res || !res->ar || !res->coef6 || !res->phil || !res->Pr || !res->Pr2 || !res->Egrid ||
        !res->Dgrid)
        return fail(ctx, FJ_ERR_ARG, "run_model: missing result buffers");
    const int nr = cfg->nr, ng = cfg->ngauss, npl = cfg->npoly, ngrid = cfg->ngrid, nt = nr * npl;
    if (nr < 11 || ng < 1 || npl < 1 || npl > kMaxPoly || ngrid < 2 || cfg->itermax < 1)
        return fail(ctx, FJ_ERR_ARG, "run_model: bad sizes");
    if (cfg->ncomp < 0 || cfg->ncomp > 2 ||
        (cfg->ncomp == 2 && cfg->twocomp_order != FJ_TWOCOMP_SUMMED && cfg->twocomp_order != FJ_TWOCOMP_REFERENCE))
        return fail(ctx, FJ_ERR_ARG, "run_model: ncomp must be 1 or 2 with a known two-component order");
    const bool two = cfg->ncomp == 2;
    const bool ref_order = two && cfg->twocomp_order == FJ_TWOCOMP_REFERENCE;
    auto t0 = std::chrono::steady_clock::now();
    int rc = FJ_OK;
    if (cfg->delta_every < 0) return fail(ctx, FJ_ERR_ARG, "run_model: delta_every must be >= 0");
    if (cfg->accel < 0 || cfg->accel > FJ_ANDERSON_MAX_DEPTH)
        return fail(ctx, FJ_ERR_ARG, "run_model: accel must be in [0, FJ_ANDERSON_MAX_DEPTH]");
    const int accel = cfg->accel;
    if (!(cfg->accel_beta >= 0 && cfg->accel_beta <= 4))
        return fail(ctx, FJ_ERR_ARG, "run_model: accel_beta must be in [0, 4] (0: 1)");
    const double beta = cfg->accel_beta > 0 ? cfg->accel_beta : 1.0;
    if (accel && (rc = fj_anderson_reset(ctx, accel, beta))) return rc;
    const bool ext = cfg->ext_phil || cfg->ext_Pr || cfg->ext_Pr2;
    if (ext && !(cfg->ext_phil && cfg->ext_Pr && cfg->ext_Pr2))
        return fail(ctx, FJ_ERR_ARG, "run_model: an external potential needs ext_phil, ext_Pr and ext_Pr2");
    const bool resume = cfg->phil_in || cfg->Pr_in || cfg->Pr2_in;
    if (resume && !(cfg->phil_in && cfg->Pr_in && cfg->Pr2_in))
        return fail(ctx, FJ_ERR_ARG, "run_model: a restart needs phil_in, Pr_in and Pr2_in");
    if (cfg->ar_in) {
        for (int i = 0; i < nr; i++)
            if (!(cfg->ar_in[i] > 0) || (i && !(cfg->ar_in[i] > cfg->ar_in[i - 1])))
                return fail(ctx, FJ_ERR_ARG, "run_model: ar_in must be positive and increasing");
        memcpy(res->ar, cfg->ar_in, nr * sizeof(double));
    } else if ((rc = fj_log_grid(cfg->rmin, cfg->rmax, nr, res->ar))) return fail(ctx, rc, "run_model: grid");
    std::vector<double> rhl(2 * (size_t)nt);
    if (!resume) {
        if ((rc = fj_guess_rhl(nr, ng, npl, res->ar, cfg->guess, cfg->mass, cfg->r0, cfg->q, rhl.data())))
            return fail(ctx, rc, "run_model: guess");
        if (two &&
            (rc = fj_guess_rhl(nr, ng, npl, res->ar, cfg->guess2, cfg->mass2, cfg->r0_2, cfg->q2, rhl.data() + nt)))
            return fail(ctx, rc, "run_model: guess of component 2");
    }
    // device layout: ar | rhl (2) | pot A, B (total, 3 tables each) | pot C, D (components) | Eg | Dg |
    // grids6 (2) | coef6 (2) | external potential (3)
    const size_t nd =
        nr + 2 * (size_t)nt + 12 * (size_t)nt + 2 * ngrid + 12 * (size_t)nr * ng + 12 * (size_t)nt + 3 * (size_t)nt;
    double *dbuf = nullptr;
    FJ_CUDA(cudaMalloc(&dbuf, nd * sizeof(double)));
    struct Free { double *p; ~Free() { cudaFree(p); } } guard{dbuf};
    double *d_ar = dbuf, *d_rhl = d_ar + nr, *potA = d_rhl + 2 * nt, *potB = potA + 3 * nt, *potC = potB + 3 * nt,
           *potD = potC + 3 * nt, *d_Eg = potD + 3 * nt, *d_Dg = d_Eg + ngrid, *d_grids = d_Dg + ngrid,
           *d_grids2 = d_grids + 6 * (size_t)nr * ng, *d_coef = d_grids2 + 6 * (size_t)nr * ng,
           *d_coef2 = d_coef + 6 * (size_t)nt, *potE = d_coef2 + 6 * (size_t)nt;
    cudaStream_t s = ctx->stream;
    FJ_CUDA(cudaMemcpyAsync(d_ar, res->ar, nr * sizeof(double), cudaMemcpyHostToDevice, s));
    FJ_CUDA(cudaMemcpyAsync(d_rhl, rhl.data(), 2 * nt * sizeof(double), cudaMemcpyHostToDevice, s));
    if (ext) {
        FJ_CUDA(cudaMemcpyAsync(potE, cfg->ext_phil, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(potE + nt, cfg->ext_Pr, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(potE + 2 * nt, cfg->ext_Pr2, nt * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    // updatePhil with the external potential (potLeg.cpp:21-29): pot += ext, all three tables
    auto add_ext = [&](double *pot) { return launch_add(3 * nt, pot, potE, pot, s); };
    if (resume) {  // the written total potential (fJmodels.cpp:63 state at the restart iteration)
        FJ_CUDA(cudaMemcpyAsync(potA, cfg->phil_in, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(potA + nt, cfg->Pr_in, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(potA + 2 * nt, cfg->Pr2_in, nt * sizeof(double), cudaMemcpyHostToDevice, s));
    } else if (!two) {
        if ((rc = fj_poisson(ctx, nr, npl, d_ar, d_rhl, potA, potA + nt, potA + 2 * nt))) return rc;
    } else {  // each component's guess potential, total = their sum (fJmodels.cpp:49-59)
        if ((rc = fj_poisson(ctx, nr, npl, d_ar, d_rhl, potC, potC + nt, potC + 2 * nt))) return rc;
        if ((rc = fj_poisson(ctx, nr, npl, d_ar, d_rhl + nt, potD, potD + nt, potD + 2 * nt))) return rc;
        FJ_CUDA(launch_sum3(nt, potC, potC + nt, potC + 2 * nt, potD, potD + nt, potD + 2 * nt, potA, potA + nt,
                            potA + 2 * nt, s));
    }
    if (ext && !resume) FJ_CUDA(add_ext(potA));  // fJmodels.cpp:120-125
    // focal-distance table from the guess (or restart) potential (fJmodels.cpp:63, 127);
    // again from the new potential after every delta_every-th iteration if asked
    std::vector<double> hp(3 * nt);
    FJ_CUDA(cudaMemcpyAsync(hp.data(), potA, 3 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaStreamSynchronize(s));
    auto tabulate = [&](const double *dpot) -> int {  // dpot: device tables [3][nt]
        if (cfg->delta_gpu) {
            const fj_potential dp{nr, npl, d_ar, dpot, dpot + nt, dpot + 2 * nt};
            int r2 = fj_tabulate_delta_batch(ctx, 1, &dp, ngrid, d_Eg, d_Dg, nullptr);
            if (r2) return r2;
            FJ_CUDA(cudaMemcpyAsync(res->Egrid, d_Eg, ngrid * sizeof(double), cudaMemcpyDeviceToHost, s));
            FJ_CUDA(cudaMemcpyAsync(res->Dgrid, d_Dg, ngrid * sizeof(double), cudaMemcpyDeviceToHost, s));
            FJ_CUDA(cudaStreamSynchronize(s));
            return FJ_OK;
        }
        std::vector<double> tp(3 * nt);
        FJ_CUDA(cudaMemcpyAsync(tp.data(), dpot, 3 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaStreamSynchronize(s));
        const fj_potential hpot{nr, npl, res->ar, tp.data(), tp.data() + nt, tp.data() + 2 * nt};
        fj_tabulate_delta(&hpot, ngrid, res->Egrid, res->Dgrid);
        FJ_CUDA(cudaMemcpyAsync(d_Eg, res->Egrid, ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(d_Dg, res->Dgrid, ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaStreamSynchronize(s));
        return FJ_OK;
    };
    if (cfg->Egrid_in && cfg->Dgrid_in) {
        memcpy(res->Egrid, cfg->Egrid_in, ngrid * sizeof(double));
        memcpy(res->Dgrid, cfg->Dgrid_in, ngrid * sizeof(double));
        FJ_CUDA(cudaMemcpyAsync(d_Eg, res->Egrid, ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(d_Dg, res->Dgrid, ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
    } else if ((rc = tabulate(potA))) return rc;
    fj_delta_table dt{ngrid, d_Eg, d_Dg};
    double *cur = potA, *nxt = potB;
    std::vector<double> old(nt), neu(nt);
    memcpy(old.data(), hp.data(), nt * sizeof(double));
    res->bound = res->failures = 0;
    res->kernel_ms = 0;
    res->last_change = -1;
    FJ_CUDA(cudaStreamSynchronize(s));
    res->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    auto tally = [&](const fj_moment_stats &st) {
        res->bound += st.bound;
        res->failures += st.failures;
        res->kernel_ms += st.kernel_ms;
    };
    int k = 0;
    bool confirmed = false;
    for (k = 0; k < cfg->itermax; k++) {
        fj_moment_stats st;
        const fj_potential pot{nr, npl, d_ar, cur, cur + nt, cur + 2 * nt};
        if (!two) {
            if ((rc = fj_compute_new_phi(ctx, &pot, &dt, &cfg->df, &cfg->rule, ng, d_grids, d_coef, nxt, nxt + nt,
                                         nxt + 2 * nt, &st)))
                return rc;
            tally(st);
        } else if (!ref_order) {
            // both components in the current total potential, one solve of the summed density
            if ((rc = fj_moments(ctx, &pot, &dt, &cfg->df, &cfg->rule, ng, d_grids, &st))) return rc;
            tally(st);
            if ((rc = fj_legendre_project(ctx, nr, ng, npl, d_ar, d_grids, d_coef))) return rc;
            if ((rc = fj_moments(ctx, &pot, &dt, &cfg->df2, &cfg->rule, ng, d_grids2, &st))) return rc;
            tally(st);
            if ((rc = fj_legendre_project(ctx, nr, ng, npl, d_ar, d_grids2, d_coef2))) return rc;
            FJ_CUDA(launch_add(nt, d_coef, d_coef2, d_rhl, s));
            if ((rc = fj_poisson(ctx, nr, npl, d_ar, d_rhl, nxt, nxt + nt, nxt + 2 * nt))) return rc;
        } else {
            // component 1 in the total potential; its own new potential replaces the total
            // (Potential.cpp:182-188); component 2 in that; total = sum (updatePhil)
            if ((rc = fj_compute_new_phi(ctx, &pot, &dt, &cfg->df, &cfg->rule, ng, d_grids, d_coef, potC, potC + nt,
                                         potC + 2 * nt, &st)))
                return rc;
            tally(st);
            const fj_potential pot1{nr, npl, d_ar, potC, potC + nt, potC + 2 * nt};
            if ((rc = fj_compute_new_phi(ctx, &pot1, &dt, &cfg->df2, &cfg->rule, ng, d_grids2, d_coef2, potD, potD + nt,
                                         potD + 2 * nt, &st)))
                return rc;
            tally(st);
            FJ_CUDA(launch_sum3(nt, potC, potC + nt, potC + 2 * nt, potD, potD + nt, potD + 2 * nt, nxt, nxt + nt,
                                nxt + 2 * nt, s));
        }
        if (ext) FJ_CUDA(add_ext(nxt));  // fJmodels.cpp:134
        FJ_CUDA(cudaMemcpyAsync(neu.data(), nxt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaStreamSynchronize(s));
        double maxd = 0;
        for (int i = 0; i < nr; i++)
            for (int j = 0; j < npl; j++)
                maxd = fmax(maxd, fabs((neu[i * npl + j] - old[i * npl + j]) / neu[i * npl]));
        res->last_change = maxd;
        const bool below = cfg->tol > 0 && maxd < cfg->tol;
        if (!accel || below || k + 1 >= cfg->itermax) {  // a plain step: the next input is this output
            old.swap(neu);
            std::swap(cur, nxt);
            if (below && (!accel || confirmed)) { k++; break; }
            confirmed = below;  // mixed: a change below tol is confirmed by one plain step
        } else {                // mixed: the next input from the last outputs
            if ((rc = fj_anderson_step(ctx, nr, npl, cur, nxt, nullptr))) return rc;
            FJ_CUDA(cudaMemcpyAsync(old.data(), cur, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
            FJ_CUDA(cudaStreamSynchronize(s));
            confirmed = false;
        }
        if (cfg->delta_every > 0 && (k + 1) % cfg->delta_every == 0 && k + 1 < cfg->itermax) {
            if ((rc = tabulate(cur))) return rc;
            if (accel && (rc = fj_anderson_reset(ctx, accel, beta))) return rc;  // a new map: a new history
        }
    }
    res->iterations = k;
    const fj_potential pot{nr, npl, d_ar, cur, cur + nt, cur + 2 * nt};
    if ((rc = fj_vir2(ctx, &pot, ng, d_coef, res->vir7))) return rc;
    if (two && (rc = fj_vir2(ctx, &pot, ng, d_coef2, res->vir7_2))) return rc;
    FJ_CUDA(cudaMemcpyAsync(res->coef6, d_coef, 6 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (two && res->coef6_2)
        FJ_CUDA(cudaMemcpyAsync(res->coef6_2, d_coef2, 6 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaMemcpyAsync(res->phil, cur, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaMemcpyAsync(res->Pr, cur + nt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaMemcpyAsync(res->Pr2, cur + 2 * nt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (res->grids6)
        FJ_CUDA(cudaMemcpyAsync(res->grids6, d_grids, 6 * (size_t)nr * ng * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaStreamSynchronize(s));
    res->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return FJ_OK;
}

// ------------------------------------------------------------ many models
extern "C" int fj_run_model_batch(fj_ctx *ctx, int n, const fj_model_config *cfgs, fj_model_result *res,
                                  int use_graph)
{
    if (!ctx || n < 1 || !cfgs || !res) return fail(ctx, FJ_ERR_ARG, "run_model_batch: bad arguments");
    const fj_quad_rule &rule = cfgs[0].rule;
    int itermax = cfgs[0].itermax;
    for (int m = 0; m < n; m++) {
        const fj_model_config &c = cfgs[m];
        const fj_model_result &r = res[m];
        if (!r.ar || !r.coef6 || !r.phil || !r.Pr || !r.Pr2 || !r.Egrid || !r.Dgrid)
            return fail(ctx, FJ_ERR_ARG, "run_model_batch: missing result buffers");
        if (c.nr < 11 || c.ngauss < 1 || c.npoly < 1 || c.npoly > kMaxPoly || c.ngrid < 2 || c.itermax < 1 ||
            c.ncomp < 0 || c.ncomp > 2)
            return fail(ctx, FJ_ERR_ARG, "run_model_batch: bad sizes or component count");
        if (c.ncomp == 2 && c.twocomp_order != FJ_TWOCOMP_SUMMED)
            return fail(ctx, FJ_ERR_ARG, "run_model_batch: two components in the summed order (the reference's "
                                         "order is a fj_run_model option)");
        if (c.ar_in || c.phil_in || c.Pr_in || c.Pr2_in || c.ext_phil || c.ext_Pr || c.ext_Pr2 || c.accel)
            return fail(ctx, FJ_ERR_ARG, "run_model_batch: restart tables, external potentials and Anderson mixing "
                                         "are fj_run_model options");
        if (c.delta_every != cfgs[0].delta_every || c.delta_every < 0 || c.delta_every > 1 ||
            (c.delta_every && !c.delta_gpu))
            return fail(ctx, FJ_ERR_ARG, "run_model_batch: delta_every is 0 or 1 (with delta_gpu) for all models");
        if (c.rule.nq != rule.nq || c.rule.precision != rule.precision || c.rule.jquad != rule.jquad ||
            memcmp(c.rule.xq, rule.xq, rule.nq * sizeof(double)) || memcmp(c.rule.wq, rule.wq, rule.nq * sizeof(double)))
            return fail(ctx, FJ_ERR_ARG, "run_model_batch: all models must share one velocity rule");
        itermax = c.itermax > itermax ? c.itermax : itermax;
    }
    auto t0 = std::chrono::steady_clock::now();
    // per-model device block: ar | rhl | cur (3 tables) | nxt (3) | Eg | Dg | grids6 | coef6, and for a
    // second component (summed order, fj_run_model's FJ_TWOCOMP_SUMMED): | grids6 | coef6
    std::vector<size_t> off(n + 1, 0), nts(n);
    for (int m = 0; m < n; m++) {
        const fj_model_config &c = cfgs[m];
        const size_t nt = (size_t)c.nr * c.npoly, g6 = 6 * (size_t)c.nr * c.ngauss;
        nts[m] = nt;
        off[m + 1] = off[m] + c.nr + nt + 6 * nt + 2 * c.ngrid + g6 + 6 * nt + (c.ncomp == 2 ? g6 + 6 * nt : 0);
    }
    double *dbuf = nullptr, *hmono = nullptr;
    FJ_CUDA(cudaMalloc(&dbuf, off[n] * sizeof(double)));
    struct Free {
        double *p, *h;
        ~Free() { cudaFree(p); if (h) cudaFreeHost(h); }
    } guard{dbuf, nullptr};
    size_t ntsum = 0;
    for (int m = 0; m < n; m++) ntsum += nts[m];
    FJ_CUDA(cudaMallocHost(&hmono, ntsum * sizeof(double)));
    guard.h = hmono;
    struct Dev { double *ar, *rhl, *cur, *nxt, *Eg, *Dg, *grids, *coef, *mono, *grids2, *coef2; };
    std::vector<Dev> d(n);
    std::vector<int> gpu_delta;  // models whose focal-distance table is tabulated on the GPU
    cudaStream_t s = ctx->stream;
    int rc;
    size_t monooff = 0;
    for (int m = 0; m < n; m++) {
        const fj_model_config &c = cfgs[m];
        const size_t nt = nts[m];
        double *b = dbuf + off[m];
        const size_t g6 = 6 * (size_t)c.nr * c.ngauss;
        double *coef = b + c.nr + 7 * nt + 2 * c.ngrid + g6;
        d[m] = Dev{b, b + c.nr, b + c.nr + nt, b + c.nr + 4 * nt, b + c.nr + 7 * nt, b + c.nr + 7 * nt + c.ngrid,
                   b + c.nr + 7 * nt + 2 * c.ngrid, coef, hmono + monooff, nullptr, nullptr};
        if (c.ncomp == 2) { d[m].grids2 = coef + 6 * nt; d[m].coef2 = d[m].grids2 + g6; }
        monooff += nt;
        if ((rc = fj_log_grid(c.rmin, c.rmax, c.nr, res[m].ar))) return fail(ctx, rc, "run_model_batch: grid");
        std::vector<double> rhl(2 * nt);
        if ((rc = fj_guess_rhl(c.nr, c.ngauss, c.npoly, res[m].ar, c.guess, c.mass, c.r0, c.q, rhl.data())))
            return fail(ctx, rc, "run_model_batch: guess");
        if (c.ncomp == 2 &&
            (rc = fj_guess_rhl(c.nr, c.ngauss, c.npoly, res[m].ar, c.guess2, c.mass2, c.r0_2, c.q2, rhl.data() + nt)))
            return fail(ctx, rc, "run_model_batch: guess of component 2");
        FJ_CUDA(cudaMemcpyAsync(d[m].ar, res[m].ar, c.nr * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(d[m].rhl, rhl.data(), nt * sizeof(double), cudaMemcpyHostToDevice, s));
        if (c.ncomp == 2)  // component 2's guess multipoles in nxt for its Poisson solve (fJmodels.cpp:49-59)
            FJ_CUDA(cudaMemcpyAsync(d[m].nxt + 2 * nt, rhl.data() + nt, nt * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaStreamSynchronize(s));
        if ((rc = fj_poisson(ctx, c.nr, c.npoly, d[m].ar, d[m].rhl, d[m].cur, d[m].cur + nt, d[m].cur + 2 * nt)))
            return rc;
        if (c.ncomp == 2) {  // each component's guess potential, total = their sum
            double *pD = d[m].coef;  // scratch: 3 tables of component 2 (coef is written by the iterations)
            if ((rc = fj_poisson(ctx, c.nr, c.npoly, d[m].ar, d[m].nxt + 2 * nt, pD, pD + nt, pD + 2 * nt))) return rc;
            FJ_CUDA(launch_add(3 * (int)nt, d[m].cur, pD, d[m].cur, s));
        }
        std::vector<double> hp(3 * nt);
        FJ_CUDA(cudaMemcpyAsync(hp.data(), d[m].cur, 3 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaStreamSynchronize(s));
        memcpy(d[m].mono, hp.data(), nt * sizeof(double));
        fj_potential hpot{c.nr, c.npoly, res[m].ar, hp.data(), hp.data() + nt, hp.data() + 2 * nt};
        if (c.Egrid_in && c.Dgrid_in) {
            memcpy(res[m].Egrid, c.Egrid_in, c.ngrid * sizeof(double));
            memcpy(res[m].Dgrid, c.Dgrid_in, c.ngrid * sizeof(double));
        } else if (c.delta_gpu) {
            gpu_delta.push_back(m);  // all together on the GPU below
        } else fj_tabulate_delta(&hpot, c.ngrid, res[m].Egrid, res[m].Dgrid);
        if (!c.delta_gpu || (c.Egrid_in && c.Dgrid_in)) {
            FJ_CUDA(cudaMemcpyAsync(d[m].Eg, res[m].Egrid, c.ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
            FJ_CUDA(cudaMemcpyAsync(d[m].Dg, res[m].Dgrid, c.ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
        }
        res[m].bound = res[m].failures = 0;
        res[m].kernel_ms = 0;
        res[m].last_change = -1;
    }
    std::vector<fj_batch_item> items;  // one per component: both components of a model in its total potential
    for (int m = 0; m < n; m++) {
        const fj_model_config &c = cfgs[m];
        const size_t nt = nts[m];
        const fj_potential pot{c.nr, c.npoly, d[m].ar, d[m].cur, d[m].cur + nt, d[m].cur + 2 * nt};
        items.push_back(fj_batch_item{pot, fj_delta_table{c.ngrid, d[m].Eg, d[m].Dg}, c.df, c.ngauss, d[m].grids});
        if (c.ncomp == 2)
            items.push_back(fj_batch_item{pot, fj_delta_table{c.ngrid, d[m].Eg, d[m].Dg}, c.df2, c.ngauss, d[m].grids2});
    }
    // GPU focal-distance tables in one launch: the models that asked for them now,
    // and with delta_every = 1 every model again before each later iteration (from
    // cur, which the iteration refreshes in place, so the launch replays in a graph)
    const bool retab = cfgs[0].delta_every == 1;
    std::vector<int> tab_models = gpu_delta;
    if (retab) {
        tab_models.resize(n);
        for (int m = 0; m < n; m++) tab_models[m] = m;
    }
    DeltaDev dd{nullptr, nullptr, nullptr, nullptr, 0};
    const int ngrid0 = tab_models.empty() ? 0 : cfgs[tab_models[0]].ngrid;
    auto prepare = [&](const std::vector<int> &ms, DeltaDev &out) -> int {
        std::vector<PotView> views;
        std::vector<double *> eg, dg;
        for (int m : ms) {
            if (cfgs[m].ngrid != ngrid0)
                return fail(ctx, FJ_ERR_ARG, "run_model_batch: GPU focal-distance tables need one ngrid");
            const size_t nt = nts[m];
            views.push_back(PotView{cfgs[m].nr, cfgs[m].npoly, d[m].ar, d[m].cur, d[m].cur + nt, d[m].cur + 2 * nt});
            eg.push_back(d[m].Eg);
            dg.push_back(d[m].Dg);
        }
        return delta_prepare(ctx, (int)ms.size(), views.data(), eg.data(), dg.data(), out);
    };
    if (!gpu_delta.empty()) {  // first tables of the models that asked (the others have theirs)
        DeltaDev d0;
        if ((rc = prepare(gpu_delta, d0))) return rc;
        FJ_CUDA(launch_tabulate_delta(d0.views, d0.Eg, d0.Dg, d0.n, ngrid0, d0.bad, s));
    }
    if (retab && (rc = prepare(tab_models, dd))) return rc;  // stream-ordered after the launch above
    FJ_CUDA(cudaStreamSynchronize(s));
    const double setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    std::vector<double> old(ntsum);
    memcpy(old.data(), hmono, ntsum * sizeof(double));
    // one iteration of every model: batched phase-space launch, then each model's
    // projection and Poisson solve into nxt, nxt copied to cur (fixed addresses, so
    // the sequence can be replayed as a graph) and its multipoles to the host
    auto iteration = [&](fj_moment_stats *st, bool tab) -> int {
        if (tab) FJ_CUDA(launch_tabulate_delta(dd.views, dd.Eg, dd.Dg, dd.n, ngrid0, dd.bad, s));
        int r2 = fj_moments_batch(ctx, (int)items.size(), items.data(), &rule, st);
        if (r2) return r2;
        for (int m = 0; m < n; m++) {
            const fj_model_config &c = cfgs[m];
            const size_t nt = nts[m];
            if ((r2 = fj_legendre_project(ctx, c.nr, c.ngauss, c.npoly, d[m].ar, d[m].grids, d[m].coef))) return r2;
            const double *dens = d[m].coef;
            if (c.ncomp == 2) {  // one solve of the summed density multipoles
                if ((r2 = fj_legendre_project(ctx, c.nr, c.ngauss, c.npoly, d[m].ar, d[m].grids2, d[m].coef2)))
                    return r2;
                FJ_CUDA(launch_add((int)nt, d[m].coef, d[m].coef2, d[m].rhl, s));
                dens = d[m].rhl;
            }
            if ((r2 = fj_poisson(ctx, c.nr, c.npoly, d[m].ar, dens, d[m].nxt, d[m].nxt + nt, d[m].nxt + 2 * nt)))
                return r2;
            FJ_CUDA(cudaMemcpyAsync(d[m].cur, d[m].nxt, 3 * nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
            FJ_CUDA(cudaMemcpyAsync(d[m].mono, d[m].nxt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        return FJ_OK;
    };
    auto converged = [&](int k) {
        bool all = true;
        size_t o = 0;
        for (int m = 0; m < n; m++) {
            const fj_model_config &c = cfgs[m];
            double maxd = 0;
            for (int i = 0; i < c.nr; i++)
                for (int j = 0; j < c.npoly; j++)
                    maxd = fmax(maxd, fabs((hmono[o + i * c.npoly + j] - old[o + i * c.npoly + j]) /
                                           hmono[o + i * c.npoly]));
            res[m].last_change = maxd;
            res[m].iterations = k + 1;
            if (!(c.tol > 0 && maxd < c.tol)) all = false;
            o += nts[m];
        }
        memcpy(old.data(), hmono, ntsum * sizeof(double));
        return all;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    struct GraphFree {
        cudaGraph_t *g; cudaGraphExec_t *e;
        ~GraphFree() { if (*e) cudaGraphExecDestroy(*e); if (*g) cudaGraphDestroy(*g); }
    } gguard{&graph, &exec};
    double kernel_ms = 0;
    long long bound = 0, failures = 0;
    for (int k = 0; k < itermax; k++) {
        if (use_graph && exec) {
            FJ_CUDA(cudaGraphLaunch(exec, s));
            FJ_CUDA(cudaStreamSynchronize(s));
        } else {
            fj_moment_stats st;
            if ((rc = iteration(&st, retab && k > 0))) return rc;
            FJ_CUDA(cudaStreamSynchronize(s));
            kernel_ms += st.kernel_ms;
            bound += st.bound;
            failures += st.failures;
            if (use_graph && k + 1 < itermax) {  // capture the sequence once it has run eagerly
                // the captured launches take the items in the order of this iteration's costs
                if (cfgs[0].rule.precision == FJ_PREC_MIXED && (rc = refresh_queue_order(ctx))) return rc;
                FJ_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                rc = iteration(nullptr, retab);
                cudaGraph_t g = nullptr;
                const cudaError_t ce = cudaStreamEndCapture(s, &g);
                if (rc) { if (g) cudaGraphDestroy(g); return rc; }
                if (ce != cudaSuccess) return cuda_fail(ctx, ce, "run_model_batch: graph capture");
                graph = g;
                FJ_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            }
        }
        if (converged(k)) break;
    }
    for (int m = 0; m < n; m++) {
        const fj_model_config &c = cfgs[m];
        const size_t nt = nts[m];
        const fj_potential pot{c.nr, c.npoly, d[m].ar, d[m].cur, d[m].cur + nt, d[m].cur + 2 * nt};
        if ((rc = fj_vir2(ctx, &pot, c.ngauss, d[m].coef, res[m].vir7))) return rc;
        FJ_CUDA(cudaMemcpyAsync(res[m].coef6, d[m].coef, 6 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (c.ncomp == 2) {
            if ((rc = fj_vir2(ctx, &pot, c.ngauss, d[m].coef2, res[m].vir7_2))) return rc;
            if (res[m].coef6_2)
                FJ_CUDA(cudaMemcpyAsync(res[m].coef6_2, d[m].coef2, 6 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        FJ_CUDA(cudaMemcpyAsync(res[m].phil, d[m].cur, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaMemcpyAsync(res[m].Pr, d[m].cur + nt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaMemcpyAsync(res[m].Pr2, d[m].cur + 2 * nt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (res[m].grids6)
            FJ_CUDA(cudaMemcpyAsync(res[m].grids6, d[m].grids, 6 * (size_t)c.nr * c.ngauss * sizeof(double),
                                    cudaMemcpyDeviceToHost, s));
    }
    for (int m : tab_models) {  // the GPU tables of the last iteration
        FJ_CUDA(cudaMemcpyAsync(res[m].Egrid, d[m].Eg, cfgs[m].ngrid * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaMemcpyAsync(res[m].Dgrid, d[m].Dg, cfgs[m].ngrid * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    FJ_CUDA(cudaStreamSynchronize(s));
    const double wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (int m = 0; m < n; m++) {
        res[m].wall_ms = wall;
        res[m].setup_ms = setup_ms;
        res[m].kernel_ms = kernel_ms;
        res[m].bound = bound;
        res[m].failures = failures;
    }
    return FJ_OK;
}

// ------------------------------------------------------------ surrogate loop
extern "C" int fj_run_model_surrogate(fj_ctx *ctx, const fj_model_config *cfg, const fj_surrogate_schedule *sch,
                                      fj_surrogate *sg, fj_model_result *res, fj_surrogate_report *rep)
{
    if (!ctx || !cfg || !sch || !sg || !res || !res->ar || !res->coef6 || !res->phil || !res->Pr || !res->Pr2 ||
        !res->Egrid || !res->Dgrid)
        return fail(ctx, FJ_ERR_ARG, "run_model_surrogate: missing arguments");
    const int nr = cfg->nr, ng = cfg->ngauss, npl = cfg->npoly, ngrid = cfg->ngrid, nt = nr * npl;
    if (nr < 11 || ng < 1 || npl < 1 || npl > kMaxPoly || ngrid < 2 || cfg->itermax < 1 || cfg->ncomp > 1 ||
        cfg->rule.precision != FJ_PREC_MIXED || cfg->df.kind != FJ_DF_DPL || sch->exact_first < 1 ||
        sch->exact_last < 0 || sch->audit_stride < 1 || sch->samples < 1 || sch->epochs_first < 1 || sch->epochs < 1)
        return fail(ctx, FJ_ERR_ARG, "run_model_surrogate: needs one DPL component, the mixed rule and a valid schedule");
    if (cfg->ar_in || cfg->phil_in || cfg->Pr_in || cfg->Pr2_in || cfg->delta_gpu || cfg->delta_every ||
        cfg->ext_phil || cfg->ext_Pr || cfg->ext_Pr2 || cfg->accel)
        return fail(ctx, FJ_ERR_ARG, "run_model_surrogate: restart tables, GPU or repeated Delta tables and "
                                     "Anderson mixing are fj_run_model options");
    fj_surrogate_report rp{};
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto ms_since = [](std::chrono::steady_clock::time_point t) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
    };
    auto t0 = now();
    int rc;
    if ((rc = fj_log_grid(cfg->rmin, cfg->rmax, nr, res->ar))) return fail(ctx, rc, "run_model_surrogate: grid");
    std::vector<double> rhl(nt);
    if ((rc = fj_guess_rhl(nr, ng, npl, res->ar, cfg->guess, cfg->mass, cfg->r0, cfg->q, rhl.data())))
        return fail(ctx, rc, "run_model_surrogate: guess");
    const int npts = nr * ng;
    const long long nq3 = (long long)cfg->rule.nq * cfg->rule.nq * cfg->rule.nq;
    // exact points: r < r_exact, and the audit points (every audit_stride-th of the rest)
    std::vector<double> ci(ng), wi(ng);
    gauleg_host(0., 1., ng, ci.data(), wi.data());
    std::vector<int> ex_idx, audit;
    std::vector<double> ex_rz;
    for (int p = 0; p < npts; p++) {
        const int n = p / ng, g = p % ng;
        const bool inner = res->ar[n] < sch->r_exact, aud = !inner && p % sch->audit_stride == 0;
        if (!inner && !aud) continue;
        if (aud) audit.push_back((int)ex_idx.size());
        ex_idx.push_back(p);
        ex_rz.push_back(res->ar[n] * sqrt(1 - ci[g] * ci[g]));
        ex_rz.push_back(res->ar[n] * ci[g]);
    }
    const int ne = (int)ex_idx.size();
    // device: ar | rhl | pot A, B | Eg | Dg | grids6 | coef6 | exact Rz | exact out6 ; actions (floats) ; exact index
    const size_t nd = nr + nt + 6 * (size_t)nt + 2 * ngrid + 6 * (size_t)npts + 6 * (size_t)nt + 2 * (size_t)ne +
                      6 * (size_t)ne;
    double *dbuf = nullptr;
    float *jout = nullptr;
    int *d_idx = nullptr;
    FJ_CUDA(cudaMalloc(&dbuf, nd * sizeof(double)));
    struct Free {
        double *p; float *j; int *i;
        ~Free() { cudaFree(p); cudaFree(j); cudaFree(i); }
    } guard{dbuf, nullptr, nullptr};
    FJ_CUDA(cudaMalloc(&jout, (size_t)npts * nq3 * 2 * sizeof(float)));
    guard.j = jout;
    FJ_CUDA(cudaMalloc(&d_idx, (ne > 0 ? ne : 1) * sizeof(int)));
    guard.i = d_idx;
    double *d_ar = dbuf, *d_rhl = d_ar + nr, *potA = d_rhl + nt, *potB = potA + 3 * nt, *d_Eg = potB + 3 * nt,
           *d_Dg = d_Eg + ngrid, *d_grids = d_Dg + ngrid, *d_coef = d_grids + 6 * (size_t)npts,
           *d_exrz = d_coef + 6 * (size_t)nt, *d_ex6 = d_exrz + 2 * (size_t)ne;
    cudaStream_t s = ctx->stream;
    FJ_CUDA(cudaMemcpyAsync(d_ar, res->ar, nr * sizeof(double), cudaMemcpyHostToDevice, s));
    FJ_CUDA(cudaMemcpyAsync(d_rhl, rhl.data(), nt * sizeof(double), cudaMemcpyHostToDevice, s));
    if (ne) {
        FJ_CUDA(cudaMemcpyAsync(d_exrz, ex_rz.data(), 2 * ne * sizeof(double), cudaMemcpyHostToDevice, s));
        FJ_CUDA(cudaMemcpyAsync(d_idx, ex_idx.data(), ne * sizeof(int), cudaMemcpyHostToDevice, s));
    }
    if ((rc = fj_poisson(ctx, nr, npl, d_ar, d_rhl, potA, potA + nt, potA + 2 * nt))) return rc;
    std::vector<double> hp(3 * nt);
    FJ_CUDA(cudaMemcpyAsync(hp.data(), potA, 3 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaStreamSynchronize(s));
    fj_potential hpot{nr, npl, res->ar, hp.data(), hp.data() + nt, hp.data() + 2 * nt};
    if (cfg->Egrid_in && cfg->Dgrid_in) {
        memcpy(res->Egrid, cfg->Egrid_in, ngrid * sizeof(double));
        memcpy(res->Dgrid, cfg->Dgrid_in, ngrid * sizeof(double));
    } else fj_tabulate_delta(&hpot, ngrid, res->Egrid, res->Dgrid);
    FJ_CUDA(cudaMemcpyAsync(d_Eg, res->Egrid, ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
    FJ_CUDA(cudaMemcpyAsync(d_Dg, res->Dgrid, ngrid * sizeof(double), cudaMemcpyHostToDevice, s));
    const fj_delta_table dt{ngrid, d_Eg, d_Dg};
    double *cur = potA, *nxt = potB;
    std::vector<double> old(nt), neu(nt), ex6(6 * (size_t)ne), sg6(6 * (size_t)npts);
    memcpy(old.data(), hp.data(), nt * sizeof(double));
    res->bound = res->failures = 0;
    res->kernel_ms = 0;
    res->last_change = -1;
    FJ_CUDA(cudaStreamSynchronize(s));
    res->setup_ms = ms_since(t0);
    int k = 0;
    for (k = 0; k < cfg->itermax; k++) {
        const fj_potential pot{nr, npl, d_ar, cur, cur + nt, cur + 2 * nt};
        bool exact = k < sch->exact_first || k >= cfg->itermax - sch->exact_last;
        if (!exact) {
            auto ts = now();
            double sms = 0;
            if ((rc = fj_surrogate_moments(sg, &pot, &cfg->df, &cfg->rule, ng, d_grids, &sms, 1)))
                return fail(ctx, rc, "run_model_surrogate: surrogate moments");
            double err = 0;
            if (ne) {
                fj_moment_stats st;
                if ((rc = run_moments(ctx, &pot, &dt, &cfg->df, &cfg->rule, 0, d_exrz, ne, d_ex6, &st))) return rc;
                res->bound += st.bound;
                res->failures += st.failures;
                FJ_CUDA(cudaMemcpyAsync(ex6.data(), d_ex6, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
                FJ_CUDA(cudaMemcpyAsync(sg6.data(), d_grids, npts * sizeof(double), cudaMemcpyDeviceToHost, s));
                FJ_CUDA(cudaStreamSynchronize(s));
                for (int a : audit)
                    if (ex6[a] > 0) err = fmax(err, fabs(sg6[ex_idx[a]] - ex6[a]) / ex6[a]);
                FJ_CUDA(launch_scatter6(ne, d_idx, d_ex6, npts, d_grids, s));
            }
            rp.last_audit_err = err;
            rp.max_audit_err = fmax(rp.max_audit_err, err);
            if (err > sch->audit_tol) {
                exact = true;
                rp.fallback_iterations++;
            } else {
                if ((rc = fj_legendre_project(ctx, nr, ng, npl, d_ar, d_grids, d_coef))) return rc;
                if ((rc = fj_poisson(ctx, nr, npl, d_ar, d_coef, nxt, nxt + nt, nxt + 2 * nt))) return rc;
                rp.surrogate_iterations++;
            }
            FJ_CUDA(cudaStreamSynchronize(s));
            rp.surrogate_ms += ms_since(ts);
        }
        if (exact) {
            auto ts = now();
            // fit while a surrogate iteration is still ahead
            const bool fit = k + 1 < cfg->itermax - sch->exact_last;
            fj_set_action_output(ctx, fit ? jout : nullptr);
            fj_moment_stats st;
            rc = fj_compute_new_phi(ctx, &pot, &dt, &cfg->df, &cfg->rule, ng, d_grids, d_coef, nxt, nxt + nt,
                                    nxt + 2 * nt, &st);
            fj_set_action_output(ctx, nullptr);
            if (rc) return rc;
            res->bound += st.bound;
            res->failures += st.failures;
            res->kernel_ms += st.kernel_ms;
            FJ_CUDA(cudaStreamSynchronize(s));
            rp.exact_ms += ms_since(ts);
            if (fit) {
                auto tf = now();
                double loss = 0;
                if ((rc = fj_surrogate_fit(sg, &pot, &cfg->df, ng, &cfg->rule, jout, d_grids, sch->samples,
                                           sch->seed + (unsigned)k,
                                           rp.fits ? sch->epochs : sch->epochs_first, sch->lr, &loss)))
                    return fail(ctx, rc, "run_model_surrogate: fit");
                rp.fits++;
                rp.last_fit_loss = loss;
                rp.fit_ms += ms_since(tf);
            }
        }
        FJ_CUDA(cudaMemcpyAsync(neu.data(), nxt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
        FJ_CUDA(cudaStreamSynchronize(s));
        double maxd = 0;
        for (int i = 0; i < nr; i++)
            for (int j = 0; j < npl; j++)
                maxd = fmax(maxd, fabs((neu[i * npl + j] - old[i * npl + j]) / neu[i * npl]));
        res->last_change = maxd;
        old.swap(neu);
        std::swap(cur, nxt);
        if (cfg->tol > 0 && maxd < cfg->tol && k >= cfg->itermax - sch->exact_last) { k++; break; }
    }
    res->iterations = k;
    const fj_potential pot{nr, npl, d_ar, cur, cur + nt, cur + 2 * nt};
    if ((rc = fj_vir2(ctx, &pot, ng, d_coef, res->vir7))) return rc;
    FJ_CUDA(cudaMemcpyAsync(res->coef6, d_coef, 6 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaMemcpyAsync(res->phil, cur, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaMemcpyAsync(res->Pr, cur + nt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaMemcpyAsync(res->Pr2, cur + 2 * nt, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (res->grids6)
        FJ_CUDA(cudaMemcpyAsync(res->grids6, d_grids, 6 * (size_t)npts * sizeof(double), cudaMemcpyDeviceToHost, s));
    FJ_CUDA(cudaStreamSynchronize(s));
    res->wall_ms = ms_since(t0);
    if (rep) *rep = rp;
    return FJ_OK;
}

