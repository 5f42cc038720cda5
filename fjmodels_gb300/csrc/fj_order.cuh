// fj_order.cuh -- the order in which a block of the phase-space kernels
// works through its bound velocity nodes (both the FP64 and the mixed form).
#pragma once
#include <math.h>

namespace fj {

// The bound nodes of a block, ordered by a cost proxy before the solves.  The
// time of a node's solve follows its orbit: the energy sets how far the
// bracket walks go and how many interpolation kinks the momentum integrals
// cross (so how many QAGS panels they need), the angular momentum where the
// inner turning point lies.  Lanes that take neighbouring entries of a list
// sorted by x0^2 + x2^2 + 1.25 x1^2 (the node's velocity in units of the
// escape speed; x1 the azimuthal one) spend similar times in each phase of
// the solve, so a warp's lanes diverge less; the most expensive nodes come
// first, so the dynamic assignment ends on cheap ones.  On the 80x40 workload
// this takes the mixed kernel from 464 to ~310 ms (the weight 1.25 chosen
// among 0, 1, 1.25, 1.5, 2, 3 by timing; energy alone: 335 ms).
__device__ __forceinline__ float node_cost_key(float x0, float x1, float x2)
{
    return -(x0 * x0 + x2 * x2 + 1.25f * x1 * x1);
}

// Bitonic sort of list[0, n) by key, padded to the next power of two (the
// arrays hold that many entries); all threads of the block take part.
static __device__ void sort_list(unsigned short *list, float *key, int n)
{
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int q = n + threadIdx.x; q < n2; q += blockDim.x) { key[q] = INFINITY; list[q] = 0; }
    __syncthreads();
    for (int kb = 2; kb <= n2; kb <<= 1)
        for (int jb = kb >> 1; jb > 0; jb >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int ixj = i ^ jb;
                if (ixj > i) {
                    const bool up = (i & kb) == 0;
                    const float ki = key[i], kj = key[ixj];
                    if ((ki > kj) == up) {
                        key[i] = kj; key[ixj] = ki;
                        const unsigned short t = list[i]; list[i] = list[ixj]; list[ixj] = t;
                    }
                }
            }
            __syncthreads();
        }
}

}  // namespace fj
