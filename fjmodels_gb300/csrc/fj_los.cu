// fj_los.cu -- projected density, line-of-sight velocity profiles and
// velocity distributions of a model (integ/Integ.cpp:32-43, 63-135, 168-220):
// the phase-space kernel's node body (Staeckel-fudge actions + DF, plain FP64)
// under 3-D and 2-D tensor rules.
//
// A value's nodes are split into ranges of kLosChunk nodes, one block each
// (a line profile's 22^3 nodes: 11 blocks), so a few hundred values fill the
// GPU.  As in the phase-space kernels, a block compacts its bound nodes,
// orders them by the cost proxy of fj_order.cuh and hands them to threads as
// they free up, storing each node's DF; thread t then sums list entries t,
// t + kLosBlock, .. from the stored DFs, the block adds the thread sums in a
// fixed order and k_los_finalize adds the blocks' sums in order, so a value
// is the same run to run.
//   SIGMA  SigmaDF(R, z) = 2 sum_i w01_i (rmax - R) rho(R + x01_i (rmax - R), z),
//          rho from the density multipoles (ev_dens, UtilsLeg.h:285-298, 323-334)
//   LINE   line_profile(R, z, vx): [-1,1]^3 rule over (vy, x, vz), the DF at the
//          point's (R, z, Phi) with the velocity rotated by the line-of-sight
//          angle and the Jacobian Ve^2 |x| rmax^2 / R' (Integ.cpp:63-92), / SigmaDF
//   PVPHI  P_vp(R, z, vphi): [0,1]^2 over (vR, vz)                 (Integ.cpp:97-109)
//   PVZ    P_vz(R, z, vz):   [0,1] x [-1,1] over (vR, vphi)       (Integ.cpp:110-122)
//   PVR    P_vr(R, z, vR):   [0,1] x [-1,1] over (vz, vphi)       (Integ.cpp:123-135)
// Built without FMA contraction, like the phase-space kernel it shares its
// arithmetic with.
#include "../../include/fjgpu.h"
#include "fj_internal.h"
#include "fj_order.cuh"

namespace fj {

namespace {

constexpr int kLosBlock = 128;

__device__ __forceinline__ double los_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ev_dens, 1-field (include/UtilsLeg.h:285-298, 323-334)
__device__ double ev_dens1(const PotView &P, const double *rhl, double R, double z)
{
    const int nr = P.nr, np = P.npoly;
    double pol[kMaxPoly], densp[kMaxPoly];
    const double c = z / sqrt(R * R + z * z), r = sqrt(R * R + z * z);
    const double c2 = c * c;
    pol[0] = 1;
    if (np > 1) pol[1] = 1.5 * c2 - .5;
    for (int l = 2; l < np; l++) pol[l] = evenleg_next(l, c2, pol[l - 2], pol[l - 1]);
    if (r > P.ar[nr - 1]) {
        for (int i = 0; i < np; i++) densp[i] = 0;
    } else {
        int top = 0, bot = 0;
        topbottom(P.ar, nr, r, bot, top);
        const double f = (r - P.ar[bot]) / (P.ar[top] - P.ar[bot]);
        for (int i = 0; i < np; i++) densp[i] = f * rhl[top * np + i] + (1 - f) * rhl[bot * np + i];
    }
    double dens = .5 * densp[0];
    for (int l = 1; l < np; l++) dens += .5 * (4 * l + 1) * densp[l] * pol[l];
    return dens;
}

__device__ double sigma_df(const PotView &P, const double *rhl, const LosArgs &a, double R, double z)
{
    const double rmax = P.ar[P.nr - 1], jac = rmax - R;
    double s = 0;
    for (int i = 0; i < kLos01; i++) s += a.w01[i] * (jac * ev_dens1(P, rhl, R + a.x01[i] * jac, z));
    return 2 * s;
}

__global__ void __launch_bounds__(kLosBlock) k_los(LosArgs a)
{
    extern __shared__ double sm[];
    const MomentArgs &m = a.m;
    const int nr = m.P.nr, npoly = m.P.npoly, nt = nr * npoly;
    double *s_ar = sm, *s_phil = s_ar + nr, *s_Pr = s_phil + nt, *s_Pr2 = s_Pr + nt;
    double *s_Eg = s_Pr2 + nt, *s_Dg = s_Eg + m.ngrid, *s_xq = s_Dg + m.ngrid, *s_wq = s_xq + m.nq;
    double *s_glx = s_wq + m.nq, *s_glw = s_glx + m.gl.n, *s_rhl = s_glw + m.gl.n, *s_red = s_rhl + nt;
    double *s_df = s_red + kLosBlock / 32;                          // [kLosChunk] DF of the list entries
    float *s_key = (float *)(s_df + kLosChunk);                       // [kLosChunk] cost keys
    unsigned short *s_list = (unsigned short *)(s_key + kLosChunk);   // [kLosChunk] bound nodes
    int *s_wc = (int *)(s_list + kLosChunk), *s_next = s_wc + kLosBlock / 32;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) s_ar[i] = m.P.ar[i];
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        s_phil[i] = m.P.phil[i]; s_Pr[i] = m.P.Pr[i]; s_Pr2[i] = m.P.Pr2[i];
        s_rhl[i] = a.rhl ? a.rhl[i] : 0.;
    }
    for (int i = threadIdx.x; i < m.ngrid; i += blockDim.x) { s_Eg[i] = m.Eg[i]; s_Dg[i] = m.Dg[i]; }
    for (int i = threadIdx.x; i < m.nq; i += blockDim.x) { s_xq[i] = m.xq[i]; s_wq[i] = m.wq[i]; }
    for (int i = threadIdx.x; i < m.gl.n; i += blockDim.x) { s_glx[i] = m.gl.x01[i]; s_glw[i] = m.gl.w01[i]; }
    __syncthreads();
    const PotView P{nr, npoly, s_ar, s_phil, s_Pr, s_Pr2};
    const GLRule gl{m.gl.n, s_glx, s_glw};
    const int B = a.blocks_per_item, item = blockIdx.x / B, chunk = blockIdx.x % B;
    const double R = a.Rzv[3 * item], z = a.Rzv[3 * item + 1], v = a.Rzv[3 * item + 2];
    if (a.kind == FJ_LOS_SIGMA) {
        if (threadIdx.x == 0) a.out[item] = sigma_df(P, s_rhl, a, R, z);
        return;
    }
    const double rmax = s_ar[nr - 1];
    const double Phi = pot_phi(P, R, z), Ve = sqrt(-2 * (Phi - pot_phi(P, 10 * rmax, 10 * rmax)));
    const int nq = m.nq;
    const int nnodes = a.kind == FJ_LOS_LINE ? nq * nq * nq : (a.kind == FJ_LOS_PVPHI ? kLos01 * kLos01 : kLos01 * nq);
    const int n0 = (int)((long long)chunk * nnodes / B), n1 = (int)((long long)(chunk + 1) * nnodes / B);
    // a node's velocity, weight and Jacobian
    auto node_vel = [&](int node, double *V, double &w, double &jacob) {
        if (a.kind == FJ_LOS_LINE) {  // lineProfile(vy, x, vz), Integ.cpp:63-92
            const int i = node / (nq * nq), j = (node / nq) % nq, k = node % nq;
            const double vy = s_xq[i], x = s_xq[j], vz = s_xq[k];
            const double Rp = sqrt(R * R + (x * rmax) * (x * rmax)), y = R;
            const double vabs = sqrt(v * v + vy * vy);
            const double alpha = acos(v / vabs), theta = atan2(y, x);
            const double vr = vabs * cos(alpha + theta), vphi = vabs * sin(alpha + theta);
            V[0] = 1e-6 + Ve * vr; V[1] = 1e-6 + Ve * vphi; V[2] = 1e-6 + Ve * vz;
            jacob = Ve * Ve * (fabs(x) * (rmax * rmax)) / Rp;
            w = s_wq[i] * s_wq[j] * s_wq[k];
        } else if (a.kind == FJ_LOS_PVPHI) {  // Pvphi(vr, vz), Integ.cpp:97-109
            const int i = node / kLos01, j = node % kLos01;
            V[0] = 1e-6 + Ve * a.x01[i]; V[1] = v; V[2] = 1e-6 + Ve * a.x01[j];
            jacob = Ve * Ve;
            w = a.w01[i] * a.w01[j];
        } else {  // Pvz(vr, vphi) / Pvr(vz, vphi), Integ.cpp:110-135
            const int i = node / nq, j = node % nq;
            if (a.kind == FJ_LOS_PVZ) { V[0] = 1e-6 + Ve * a.x01[i]; V[1] = 1e-6 + Ve * s_xq[j]; V[2] = v; }
            else { V[0] = v; V[1] = 1e-6 + Ve * s_xq[j]; V[2] = 1e-6 + Ve * a.x01[i]; }
            jacob = Ve * Ve;
            w = a.w01[i] * s_wq[j];
        }
    };
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // bound nodes of [n0, n1) in node order, then ordered by the cost proxy of
    // the phase-space kernels (most expensive first), taken as threads free up
    int nbound = 0;
    for (int base = n0; base < n1; base += kLosBlock) {
        const int node = base + threadIdx.x;
        bool b = false;
        if (node < n1) {
            double V[3], w, jacob;
            node_vel(node, V, w, jacob);
            b = .5 * (V[0] * V[0] + V[1] * V[1] + V[2] * V[2]) + Phi < 0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, b);
        if (lane == 0) s_wc[warp] = __popc(bal);
        __syncthreads();
        int off = nbound, tot = 0;
        for (int q = 0; q < kLosBlock / 32; q++) {
            if (q < warp) off += s_wc[q];
            tot += s_wc[q];
        }
        if (b) s_list[off + __popc(bal & ((1u << lane) - 1u))] = (unsigned short)(node - n0);
        __syncthreads();
        nbound += tot;
    }
    const double iVe = 1. / Ve;
    for (int q = threadIdx.x; q < nbound; q += kLosBlock) {
        double V[3], w, jacob;
        node_vel(n0 + s_list[q], V, w, jacob);
        s_key[q] = node_cost_key((float)(V[0] * iVe), (float)(V[1] * iVe), (float)(V[2] * iVe));
    }
    sort_list(s_list, s_key, nbound);
    if (threadIdx.x == 0) *s_next = kLosBlock;
    __syncthreads();
    unsigned failed = 0;
    for (int q = threadIdx.x; q < nbound;) {  // df(), DF.cpp:78-124
        double V[3], w, jacob;
        node_vel(n0 + s_list[q], V, w, jacob);
        const double H = .5 * (V[0] * V[0] + V[1] * V[1] + V[2] * V[2]) + Phi;
        unsigned fail = 0;
        double Jr, Jz;
        fudge_actions(P, deltafn(s_Eg, s_Dg, m.ngrid, H), R, z, Phi, V[0], V[1], V[2], gl, Jr, Jz, fail);
        double DF = df_value(m.df, P, R, Jr, Jz, R * V[1], fail);
        if (fail & (kFailBracket | kFailRoot)) DF = 0.;
        failed += fail ? 1u : 0u;
        s_df[q] = DF;
        q = atomicAdd(s_next, 1);
    }
    __syncthreads();
    double sum = 0;  // fixed order: thread t adds list entries t, t + kLosBlock, ..
    for (int q = threadIdx.x; q < nbound; q += kLosBlock) {
        double V[3], w, jacob;
        node_vel(n0 + s_list[q], V, w, jacob);
        sum += w * (jacob * s_df[q]);
    }
    const double ws = los_warp_sum(sum);
    unsigned nfw = failed;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nfw += __shfl_xor_sync(0xffffffffu, nfw, o);
    if (lane == 0) { s_red[warp] = ws; s_wc[warp] = (int)nfw; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        unsigned nf = 0;
        for (int q = 0; q < kLosBlock / 32; q++) { s += s_red[q]; nf += (unsigned)s_wc[q]; }
        a.partial[blockIdx.x] = s;
        if (a.m.counters) {
            if (nbound) atomicAdd(&a.m.counters[kCntBound], (unsigned long long)nbound);
            if (nf) atomicAdd(&a.m.counters[kCntFailed], (unsigned long long)nf);
        }
    }
}

// a value's block sums in order; a line profile is divided by SigmaDF at the
// point (Integ.cpp:92), from the tables in global memory
__global__ void k_los_finalize(LosArgs a)
{
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= a.n || a.kind == FJ_LOS_SIGMA) return;
    const int B = a.blocks_per_item;
    double s = 0;
    for (int c = 0; c < B; c++) s += a.partial[(size_t)item * B + c];
    if (a.kind == FJ_LOS_LINE) s /= sigma_df(a.m.P, a.rhl, a, a.Rzv[3 * item], a.Rzv[3 * item + 1]);
    a.out[item] = s;
}

}  // namespace

int los_blocks_per_item(int kind, int nq)
{
    const long long nnodes = kind == FJ_LOS_LINE ? (long long)nq * nq * nq
                             : kind == FJ_LOS_PVPHI ? (long long)kLos01 * kLos01 : (long long)kLos01 * nq;
    return kind == FJ_LOS_SIGMA ? 1 : (int)((nnodes + kLosChunk - 1) / kLosChunk);
}

size_t los_smem_bytes(const MomentArgs &m)
{
    const size_t nt = (size_t)m.P.nr * m.P.npoly;
    return (m.P.nr + 4 * nt + 2 * m.ngrid + 2 * m.nq + 2 * m.gl.n + kLosBlock / 32 + kLosChunk) * sizeof(double) +
           kLosChunk * (sizeof(float) + sizeof(unsigned short)) + (kLosBlock / 32 + 1) * sizeof(int);
}

size_t los_local_bytes()
{
    cudaFuncAttributes at;
    return cudaFuncGetAttributes(&at, k_los) == cudaSuccess ? at.localSizeBytes : 0;
}

cudaError_t launch_los(const LosArgs &a, cudaStream_t s)
{
    const size_t smem = los_smem_bytes(a.m);
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k_los, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_los<<<(unsigned)((long long)a.n * a.blocks_per_item), kLosBlock, smem, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || a.kind == FJ_LOS_SIGMA) return e;
    k_los_finalize<<<(a.n + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fj
