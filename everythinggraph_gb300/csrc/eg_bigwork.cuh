// Deferred high-degree frontier items (RMAT hubs with 10^3..10^6 edges),
// shared out over the whole grid in fixed-size chunks of edges.
//
// A push kernel appends the items whose vertex has more than its warp limit
// of edges to a side list.  k_big_offsets (one block) turns that list into an
// exclusive prefix of chunk counts, off[i] = sum over items before i of
// ceil(deg / chunk), with off[nbig] = the total; a consumer CTA takes chunk
// indices c = blockIdx.x, blockIdx.x + gridDim.x, ... and finds its item as
// the last i with off[i] <= c (binary search).  The cost of an item is then
// proportional to its degree, instead of one grid-wide latency chain per item.
//
// An item is vertex * per + word (per = 1 for one source, the number of
// 32-source words for the batched kernels).
//
// eg_warp_grab / eg_cta_grab hand out work units from a counter zeroed
// before the launch, so that a grid with more CTAs than fit on the SMs at
// once, or units of uneven cost, leave no tail of idle SMs.
#pragma once
#include "eg_internal.cuh"

namespace {

// Next unit for the calling warp (lane 0 takes it, every lane gets it).
__device__ __forceinline__ uint32_t eg_warp_grab(uint32_t *counter) {
    uint32_t c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(counter, 1u);
    return __shfl_sync(EG_FULL_MASK, c, 0);
}

// Next unit for the calling CTA (every thread calls it).
__device__ __forceinline__ uint32_t eg_cta_grab(uint32_t *counter) {
    __shared__ uint32_t s_unit;
    __syncthreads();  // every thread has read the previous unit
    if (threadIdx.x == 0) s_unit = atomicAdd(counter, 1u);
    __syncthreads();
    return s_unit;
}

__global__ void __launch_bounds__(1024) k_big_offsets(const uint32_t *__restrict__ items,
                                                      const uint32_t *__restrict__ count, uint32_t per,
                                                      const uint32_t *__restrict__ ptr, uint32_t chunk,
                                                      uint32_t *__restrict__ off) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_run;
    const uint32_t nb = *(volatile const uint32_t *)count;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_run = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nb; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        uint32_t c = 0;
        if (i < nb) {
            const uint32_t v = items[i] / per;
            c = (ptr[v + 1] - ptr[v] + chunk - 1) / chunk;
        }
        uint32_t x = c;  // inclusive warp scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(EG_FULL_MASK, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t t = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(EG_FULL_MASK, t, o);
                if (lane >= (uint32_t)o) t += y;
            }
            s_warp[lane] = t;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t run = s_run;
        const uint32_t before = (warp ? s_warp[warp - 1] : 0u) + x - c;
        if (i < nb) off[i] = run + before;
        __syncthreads();  // every thread has read s_run and s_warp
        if (threadIdx.x == 0) s_run = run + s_warp[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) off[nb] = s_run;
}

// The item holding chunk c: the last i in [0, nb) with off[i] <= c.
__device__ __forceinline__ uint32_t eg_big_item(const uint32_t *__restrict__ off, uint32_t nb, uint32_t c) {
    uint32_t lo = 0, hi = nb;  // off[lo] <= c < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= c) lo = mid;
        else hi = mid;
    }
    return lo;
}

}  // namespace
