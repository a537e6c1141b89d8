// Frontier building blocks shared by the single-source BFS and SSSP loops.
//
// eg_warp_lists  a warp walks the out-lists of its 32 lanes' vertices
//                together, 32 edges per step: an inclusive scan of the list
//                lengths gives each edge slot its owner lane by a 5-step
//                shuffle search, so every lane has an edge whatever the
//                degrees (one warp per vertex leaves most lanes idle on
//                low-degree frontiers).
// k_bm_queue     frontier bitmap -> vertex-id queue: a thread per bitmap
//                word, a block-wide exclusive scan of the words' popcounts
//                places the ids, one atomic per block reserves the space;
//                optionally clears the words it read.
#pragma once
#include "eg_internal.cuh"

namespace {

// Lane i holds vertex u, list start b and length d (d = 0: nothing).  For
// every edge slot f(valid, owner_lane, owner_vertex, edge_index) is called
// by all 32 lanes together (so f may use warp collectives); edge_index is
// meaningful only where valid.
template <class F>
__device__ __forceinline__ void eg_warp_lists(uint32_t u, uint32_t b, uint32_t d, F &&f) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t inc = d;  // inclusive scan of the lengths
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(EG_FULL_MASK, inc, o);
        if (lane >= o) inc += y;
    }
    const uint32_t total = __shfl_sync(EG_FULL_MASK, inc, 31);
    const uint32_t exc = inc - d;
    for (uint32_t p0 = 0; p0 < total; p0 += 32) {
        const uint32_t x = p0 + lane;
        uint32_t lo = 0;  // owner of slot x: the first lane whose inclusive sum exceeds x
#pragma unroll
        for (uint32_t step = 16; step > 0; step >>= 1) {
            const uint32_t probe = __shfl_sync(EG_FULL_MASK, inc, lo + step - 1);
            if (probe <= x) lo += step;
        }
        const uint32_t ob = __shfl_sync(EG_FULL_MASK, b, lo);
        const uint32_t oe = __shfl_sync(EG_FULL_MASK, exc, lo);
        const uint32_t ou = __shfl_sync(EG_FULL_MASK, u, lo);
        const bool valid = x < total;
        f(valid, lo, ou, valid ? ob + (x - oe) : 0u);
    }
}

__global__ void __launch_bounds__(256) k_bm_queue(uint32_t *__restrict__ bm, uint32_t n, uint32_t *queue,
                                                  uint32_t *qsize, int clear) {
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_base;
    const uint32_t nw = (n + 31) >> 5;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t w0 = blockIdx.x * blockDim.x; w0 < nw; w0 += gridDim.x * blockDim.x) {
        const uint32_t w = w0 + threadIdx.x;
        const uint32_t word = w < nw ? bm[w] : 0u;
        if (clear && word) bm[w] = 0u;
        const uint32_t c = __popc(word);
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(EG_FULL_MASK, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int i = 0; i < 8; i++) {
                const uint32_t v = s_warp[i];
                s_warp[i] = t;
                t += v;
            }
            s_base = t ? atomicAdd(qsize, t) : 0u;
        }
        __syncthreads();
        uint32_t pos = s_base + s_warp[warp] + x - c;
        uint32_t bits = word;
        while (bits) {
            const int bb = __ffs(bits) - 1;
            bits &= bits - 1;
            queue[pos++] = (w << 5) + (uint32_t)bb;
        }
        __syncthreads();
    }
}

}  // namespace
