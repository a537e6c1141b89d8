// Batched (vertex-major) SSSP relaxation of one frontier vertex's out-edges
// for one word of 32 sources: lane l owns source 32*j + l, whose distances
// sit in dist[v*K + s] (one 128-byte row segment per vertex and word).
//
// The warp walks the edges 32 at a time: lane k loads the k-th column and
// computes that edge's weight once (the weight rule is per edge, the same for
// every source), the values are broadcast by shuffles, and four edges are
// relaxed per step with their four distance rows loaded before any of their
// atomicMin updates, so four independent row loads are in flight instead of
// one dependent col -> dist -> atomic chain per edge.
//
// sink(v, ball) is called by lane 0 for every edge that lowered the distance
// of the sources in `ball`; it records v in the next frontier.
#pragma once
#include "eg_internal.cuh"

template <class Sink>
__device__ __forceinline__ void eg_mrelax_span(uint32_t u, uint32_t p0, uint32_t p1, const uint32_t *__restrict__ col,
                                               const eg_wrule &w, bool on, uint32_t du, uint32_t s, uint32_t K,
                                               uint32_t *dist, Sink &sink) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c0 = p0; c0 < p1; c0 += 32) {
        const uint32_t pl = c0 + lane;
        const uint32_t myv = pl < p1 ? __ldg(col + pl) : u;  // u: skipped like a self-loop
        const uint32_t myw = pl < p1 ? w.weight(u, myv) : 0u;
        const uint32_t cnt = p1 - c0 < 32 ? p1 - c0 : 32;
        for (uint32_t k = 0; k < cnt; k += 4) {
            uint32_t vv[4], nd[4], cur[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                vv[q] = __shfl_sync(EG_FULL_MASK, myv, (k + q) & 31);
                const uint32_t wt = __shfl_sync(EG_FULL_MASK, myw, (k + q) & 31);
                if (k + q >= cnt) vv[q] = u;
                nd[q] = w.add(du, wt);
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                cur[q] = (on && vv[q] != u) ? __ldcg(dist + (uint64_t)vv[q] * K + s) : 0u;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                bool improved = false;
                if (on && vv[q] != u && nd[q] < cur[q])  // self-loops skipped (sssp_pushpull.c:80)
                    improved = nd[q] < atomicMin(dist + (uint64_t)vv[q] * K + s, nd[q]);
                const uint32_t ball = __ballot_sync(EG_FULL_MASK, improved);
                if (ball && lane == 0) sink(vv[q], ball);
            }
        }
    }
}
