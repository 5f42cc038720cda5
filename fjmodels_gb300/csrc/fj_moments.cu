// fj_moments.cu -- the phase-space kernel: one thread per (meridional point,
// velocity node) evaluates the Staeckel-fudge actions and the DF and the
// block reduces the six velocity moments; plus the batched action and
// potential kernels.
//
// Work unit: node q = (i, j, k) of the nq^3 tensor rule (integ/GaussQuad.cpp:
// 160-180), velocity V = 1e-6 + Ve*(x_i, x_j, x_k) (integ/Integ.cpp:46-62).
// A block takes kPlainChunk consecutive nodes of one point, compacts the bound
// ones (H < 0) into a shared list, orders it by the cost proxy of fj_order.cuh
// and its threads take the entries as they free up; each node's DF goes to a
// shared array, and after the list thread t sums the moments of entries t,
// t + 128, .. in order.  The per-block sums go to a scratch array and a second
// kernel adds them in a fixed order, so results are deterministic run to run.
#include <cstdint>

#include "fj_internal.h"
#include "fj_order.cuh"

namespace fj {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

size_t moment_smem_bytes(const MomentArgs &a)
{
    const size_t nd = a.P.nr + 3 * (size_t)a.P.nr * a.P.npoly + 2 * a.ngrid + 2 * a.nq + 2 * a.gl.n;
    return nd * sizeof(double) + 6 * (kMomentBlock / 32) * sizeof(double) + 4 * sizeof(double) +
           kPlainChunk * (sizeof(double) + sizeof(float) + sizeof(unsigned short)) + (kMomentBlock / 32 + 1) * sizeof(int) +
           16;
}

__global__ void __launch_bounds__(kMomentBlock) k_moments(MomentArgs a0, MomentBatch batch)
{
    extern __shared__ double sm[];
    MomentArgs a = a0;
    int bid = blockIdx.x;
    if (batch.n > 0) {
        const int m = batch_model(batch.block_start, batch.n, bid);
        a = batch.args[m];
        bid -= batch.block_start[m];
    }
    const int nr = a.P.nr, npoly = a.P.npoly, nt = nr * npoly;
    double *s_ar = sm, *s_phil = s_ar + nr, *s_Pr = s_phil + nt, *s_Pr2 = s_Pr + nt;
    double *s_Eg = s_Pr2 + nt, *s_Dg = s_Eg + a.ngrid, *s_xq = s_Dg + a.ngrid, *s_wq = s_xq + a.nq;
    double *s_glx = s_wq + a.nq, *s_glw = s_glx + a.gl.n, *s_red = s_glw + a.gl.n;
    double *s_pt = s_red + 6 * (kMomentBlock / 32), *s_df = s_pt + 4;
    float *s_key = (float *)(s_df + kPlainChunk);
    unsigned short *s_list = (unsigned short *)(s_key + kPlainChunk);
    int *s_wc = (int *)(((uintptr_t)(s_list + kPlainChunk) + 15) & ~(uintptr_t)15), *s_next = s_wc + kMomentBlock / 32;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) s_ar[i] = a.P.ar[i];
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        s_phil[i] = a.P.phil[i]; s_Pr[i] = a.P.Pr[i]; s_Pr2[i] = a.P.Pr2[i];
    }
    for (int i = threadIdx.x; i < a.ngrid; i += blockDim.x) { s_Eg[i] = a.Eg[i]; s_Dg[i] = a.Dg[i]; }
    for (int i = threadIdx.x; i < a.nq; i += blockDim.x) { s_xq[i] = a.xq[i]; s_wq[i] = a.wq[i]; }
    for (int i = threadIdx.x; i < a.gl.n; i += blockDim.x) { s_glx[i] = a.gl.x01[i]; s_glw[i] = a.gl.w01[i]; }
    __syncthreads();

    const PotView P{nr, npoly, s_ar, s_phil, s_Pr, s_Pr2};
    const GLRule gl{a.gl.n, s_glx, s_glw};
    const int B = a.blocks_per_point;
    const int p = bid / B, chunk = bid % B;
    const int nq = a.nq, nq2 = nq * nq, nq3 = nq2 * nq;
    const int n0 = chunk * kPlainChunk, n1 = min(n0 + kPlainChunk, nq3);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {  // the point (integ/Integ.cpp:150-151)
        double R, z;
        if (a.Rz) { R = a.Rz[2 * p]; z = a.Rz[2 * p + 1]; }
        else {
            const int n = p / a.ngauss, g = p % a.ngauss;
            const double c = a.ci[g], si = sqrt(1 - c * c);
            R = s_ar[n] * si; z = s_ar[n] * c;
        }
        const double Phi_h = pot_phi(P, R, z), rmax = s_ar[nr - 1];
        s_pt[0] = R; s_pt[1] = z; s_pt[2] = Phi_h;
        s_pt[3] = sqrt(-2 * (Phi_h - pot_phi(P, 10 * rmax, 10 * rmax)));
        *s_next = kMomentBlock;
    }
    __syncthreads();
    const double R = s_pt[0], z = s_pt[1], Phi_h = s_pt[2], Ve = s_pt[3];
    auto velocity = [&](int node, double &V0, double &V1, double &V2) {
        V0 = 1e-6 + Ve * s_xq[node / nq2]; V1 = 1e-6 + Ve * s_xq[(node / nq) % nq]; V2 = 1e-6 + Ve * s_xq[node % nq];
    };
    // bound nodes of [n0, n1) in node order
    int nbound = 0;
    for (int base = n0; base < n1; base += kMomentBlock) {
        const int node = base + threadIdx.x;
        bool b = false;
        if (node < n1) {
            double V0, V1, V2;
            velocity(node, V0, V1, V2);
            b = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h < 0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, b);
        if (lane == 0) s_wc[warp] = __popc(bal);
        __syncthreads();
        int off = nbound, tot = 0;
        for (int w = 0; w < kMomentBlock / 32; w++) {
            if (w < warp) off += s_wc[w];
            tot += s_wc[w];
        }
        if (b) s_list[off + __popc(bal & ((1u << lane) - 1u))] = (unsigned short)(node - n0);
        __syncthreads();
        nbound += tot;
    }
    for (int q = threadIdx.x; q < nbound; q += kMomentBlock) {
        const int node = n0 + s_list[q];
        s_key[q] = node_cost_key((float)s_xq[node / nq2], (float)s_xq[(node / nq) % nq], (float)s_xq[node % nq]);
    }
    sort_list(s_list, s_key, nbound);
    // the solves, nodes taken as threads free up
    FailTally tally;
    for (int q = threadIdx.x; q < nbound;) {
        const int node = n0 + s_list[q];
        double V0, V1, V2;
        velocity(node, V0, V1, V2);
        const double H = .5 * (V0 * V0 + V1 * V1 + V2 * V2) + Phi_h;
        unsigned fail = 0;
        double Jr, Jz;
        fudge_actions(P, deltafn(s_Eg, s_Dg, a.ngrid, H), R, z, Phi_h, V0, V1, V2, gl, Jr, Jz, fail);
        double DF = df_value(a.df, P, R, Jr, Jz, R * V1, fail);
        if (fail & (kFailBracket | kFailRoot)) DF = 0.;
        tally.add(fail);
        s_df[q] = DF;
        q = atomicAdd(s_next, 1);
    }
    __syncthreads();
    double m[6] = {0, 0, 0, 0, 0, 0};
    const double jacob = Ve * Ve * Ve;
    for (int q = threadIdx.x; q < nbound; q += kMomentBlock) {
        const int node = n0 + s_list[q];
        double V0, V1, V2;
        velocity(node, V0, V1, V2);
        const double w = s_wq[node / nq2] * s_wq[(node / nq) % nq] * s_wq[node % nq];
        const double jd = jacob * s_df[q];
        m[0] += w * jd;
        m[1] += w * (jd * V1);
        m[2] += w * (jd * V0 * V0);
        m[3] += w * (jd * V1 * V1);
        m[4] += w * (jd * V2 * V2);
        m[5] += w * (jd * V0 * V2);
    }
    // block reduction in a fixed order
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const double v = warp_sum(m[q]);
        if (lane == 0) s_red[warp * 6 + q] = v;
    }
    warp_count_fails(a.counters, tally);
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w = 0; w < kMomentBlock / 32; w++) s += s_red[w * 6 + threadIdx.x];
        a.partial[((size_t)p * B + chunk) * 6 + threadIdx.x] = s;
    }
    if (threadIdx.x == 0 && nbound) atomicAdd(&a.counters[kCntBound], (unsigned long long)nbound);
}

// sums the per-block partials of each point and normalises as rhofDF does
// (integ/Integ.cpp:160-162)
__device__ __forceinline__ void finalize_point(const double *partial, int npts, int B, double *out6, int p)
{
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < B; c++)
#pragma unroll
        for (int q = 0; q < 6; q++) s[q] += partial[((size_t)p * B + c) * 6 + q];
    out6[0 * (size_t)npts + p] = s[0];
    out6[1 * (size_t)npts + p] = s[1] / s[0];
    out6[2 * (size_t)npts + p] = sqrt(s[2] / s[0]);
    out6[3 * (size_t)npts + p] = sqrt(s[3] / s[0]);
    out6[4 * (size_t)npts + p] = sqrt(s[4] / s[0]);
    out6[5 * (size_t)npts + p] = sqrt(fabs(s[5]) / s[0]);
}

__global__ void k_moments_finalize(const double *partial, int npts, int B, double *out6)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < npts) finalize_point(partial, npts, B, out6, p);
}

__global__ void k_moments_finalize_batch(MomentBatch batch, int npoints)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npoints) return;
    const int m = batch_model(batch.point_start, batch.n, t);
    const MomentArgs &a = batch.args[m];
    finalize_point(a.partial, a.npts, a.blocks_per_point, a.out6, t - batch.point_start[m]);
}

__global__ void k_scatter6(int n, const int *idx, const double *src6, int npts, double *dst6)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    for (int q = 0; q < 6; q++) dst6[(size_t)q * npts + idx[t]] = src6[(size_t)q * n + t];
}

cudaError_t launch_scatter6(int n, const int *idx, const double *src6, int npts, double *dst6, cudaStream_t s)
{
    k_scatter6<<<(n + 127) / 128, 128, 0, s>>>(n, idx, src6, npts, dst6);
    return cudaGetLastError();
}

cudaError_t launch_moments_finalize_batch(const MomentBatch &b, int npoints, cudaStream_t s)
{
    k_moments_finalize_batch<<<(npoints + 127) / 128, 128, 0, s>>>(b, npoints);
    return cudaGetLastError();
}

cudaError_t launch_moments(const MomentArgs &a, cudaStream_t s)
{
    const size_t smem = moment_smem_bytes(a);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_moments, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const long long nblocks = (long long)a.npts * a.blocks_per_point;
    k_moments<<<(unsigned)nblocks, kMomentBlock, smem, s>>>(a, MomentBatch{nullptr, nullptr, nullptr, 0});
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_moments_finalize(a, s);
}

cudaError_t launch_moments_plain_batch(const MomentArgs &a0, const MomentBatch &b, int nblocks, size_t smem,
                                      cudaStream_t s)
{
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_moments, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_moments<<<(unsigned)nblocks, kMomentBlock, smem, s>>>(a0, b);
    return cudaGetLastError();
}

cudaError_t launch_moments_finalize(const MomentArgs &a, cudaStream_t s)
{
    k_moments_finalize<<<(a.npts + 127) / 128, 128, 0, s>>>(a.partial, a.npts, a.blocks_per_point, a.out6);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- actions
__global__ void k_actions(PotView P, const double *Eg, const double *Dg, int ngrid, GLRule gl,
                          const double *pts, size_t n, double *out)
{
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double R = pts[5 * t], z = pts[5 * t + 1], vR = pts[5 * t + 2], vp = pts[5 * t + 3], vz = pts[5 * t + 4];
    const double Phi = pot_phi(P, R, z);
    const double H = .5 * (vR * vR + vp * vp + vz * vz) + Phi;
    if (H >= 0) { out[2 * t] = -1; out[2 * t + 1] = -1; return; }
    double Jr, Jz;
    unsigned fail = 0;
    fudge_actions(P, deltafn(Eg, Dg, ngrid, H), R, z, Phi, vR, vp, vz, gl, Jr, Jz, fail);
    out[2 * t] = Jr;
    out[2 * t + 1] = Jz;
}

cudaError_t launch_actions(PotView P, const double *Eg, const double *Dg, int ngrid, GLRule gl,
                           const double *pts, size_t n, double *out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_actions<<<(unsigned)((n + 63) / 64), 64, 0, s>>>(P, Eg, Dg, ngrid, gl, pts, n, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- potential
__global__ void k_potential_eval(PotView P, const double *Rz, size_t n, double *out)
{
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    double phi, dR, dz;
    pot_grad(P, Rz[2 * t], Rz[2 * t + 1], phi, dR, dz);
    out[3 * t] = phi;
    out[3 * t + 1] = dR;
    out[3 * t + 2] = dz;
}

cudaError_t launch_potential_eval(PotView P, const double *Rz, size_t n, double *out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_potential_eval<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P, Rz, n, out);
    return cudaGetLastError();
}

size_t moments_local_bytes()
{
    size_t m = 0;
    cudaFuncAttributes at;
    if (cudaFuncGetAttributes(&at, k_moments) == cudaSuccess && at.localSizeBytes > m) m = at.localSizeBytes;
    if (cudaFuncGetAttributes(&at, k_actions) == cudaSuccess && at.localSizeBytes > m) m = at.localSizeBytes;
    if (cudaFuncGetAttributes(&at, k_potential_eval) == cudaSuccess && at.localSizeBytes > m) m = at.localSizeBytes;
    return m;
}

}  // namespace fj
