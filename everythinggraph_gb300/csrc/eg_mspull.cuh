// Bottom-up (pull) level of the bit-sliced multi-source BFS: for every
// vertex v still unseen by some live source, next[v] = OR of the frontier
// words of its in-neighbours, restricted to those sources.  The scan of v's
// in-list stops as soon as every source still missing v has been found
// (the bottom-up early exit of bfs_simple.c:104-229's pull, one word per 64
// sources).
//
// A serial scan per vertex is fine for the common low-degree vertex but not
// for a hub whose sources stay unsatisfied (it would read its whole in-list,
// 10^5..10^6 entries, from one thread).  So the level runs in two parts:
//   k_msp_light  one thread per vertex scans at most EG_MSP_LIGHT in-entries;
//                a vertex still unsatisfied with entries left goes to the
//                heavy list, its partial word parked in next[v];
//   k_msp_heavy  one CTA per heavy vertex scans the rest 1024 entries per
//                step (4 per thread, coalesced), ORs the warps' words in
//                shared memory and stops once the need is met.
#pragma once
#include "eg_internal.cuh"

#define EG_MSP_LIGHT 32u

namespace {

__global__ void __launch_bounds__(256) k_msp_light(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                   uint32_t n, unsigned long long all,
                                                   const unsigned long long *__restrict__ seen,
                                                   const unsigned long long *__restrict__ front,
                                                   unsigned long long *__restrict__ next, uint32_t *__restrict__ heavy,
                                                   uint32_t *heavy_count, const int *gate = nullptr) {
    if (gate && !*gate) return;  // a device-driven loop chose push for this level
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    // uniform trip count per warp for the ballot
    for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < n; v0 += stride) {
        const uint32_t v = v0 + lane;
        bool hv = false;
        if (v < n) {
            const unsigned long long need = all & ~seen[v];
            unsigned long long acc = 0ull;
            if (need) {
                const uint32_t b = ptr[v], e = ptr[v + 1];
                const uint32_t lim = e - b > EG_MSP_LIGHT ? b + EG_MSP_LIGHT : e;
                for (uint32_t p = b; p < lim; p++) {
                    acc |= __ldg(front + col[p]);
                    if ((acc & need) == need) break;
                }
                hv = (acc & need) != need && lim < e;
            }
            next[v] = hv ? acc : (acc & need);
        }
        const uint32_t ball = __ballot_sync(EG_FULL_MASK, hv);
        if (ball) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(heavy_count, (uint32_t)__popc(ball));
            base = __shfl_sync(EG_FULL_MASK, base, 0);
            if (hv) heavy[base + __popc(ball & eg_lanemask_lt())] = v;
        }
    }
}

__global__ void __launch_bounds__(256) k_msp_heavy(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                   unsigned long long all, const unsigned long long *__restrict__ seen,
                                                   const unsigned long long *__restrict__ front,
                                                   unsigned long long *__restrict__ next,
                                                   const uint32_t *__restrict__ heavy, const uint32_t *heavy_count,
                                                   const int *gate = nullptr) {
    __shared__ unsigned long long s_acc;
    if (gate && !*gate) return;
    const uint32_t nh = *(volatile const uint32_t *)heavy_count;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t i = blockIdx.x; i < nh; i += gridDim.x) {
        const uint32_t v = heavy[i];
        const unsigned long long need = all & ~seen[v];
        if (threadIdx.x == 0) s_acc = next[v];  // the light scan's partial word
        __syncthreads();
        const uint32_t e = ptr[v + 1];
        for (uint32_t base = ptr[v] + EG_MSP_LIGHT; base < e; base += 1024u) {
            unsigned long long acc = 0ull;
#pragma unroll
            for (uint32_t k = 0; k < 4; k++) {
                const uint32_t p = base + k * 256u + threadIdx.x;
                if (p < e) acc |= __ldg(front + col[p]);
            }
            const uint32_t lo = __reduce_or_sync(EG_FULL_MASK, (uint32_t)acc);
            const uint32_t hi = __reduce_or_sync(EG_FULL_MASK, (uint32_t)(acc >> 32));
            if (lane == 0 && (lo | hi)) atomicOr(&s_acc, ((unsigned long long)hi << 32) | lo);
            __syncthreads();
            const bool stop = (s_acc & need) == need;
            __syncthreads();  // every thread has read s_acc before the next step adds to it
            if (stop) break;
        }
        if (threadIdx.x == 0) next[v] = s_acc & need;
        __syncthreads();  // s_acc is reset for the next vertex only after the write
    }
}

}  // namespace
