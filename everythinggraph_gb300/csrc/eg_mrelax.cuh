// Batched (vertex-major) SSSP relaxation of one frontier vertex's out-edges
// [p0, p1) for one word j of 32 sources: source s = 32*j + l has its
// distances in dist[v*K + s]; `a` holds the word's sources whose distance at
// u dropped last round, `du` is lane l's own distance at u (valid when bit l
// of `a` is set).  Two forms, picked per item by the number of active sources:
//
//  * row form (many active sources): lane l relaxes source 32*j + l.  The
//    warp walks the edges 32 at a time: lane k loads the k-th column and its
//    weight (`wts`: the rule's weights materialised in CSR order, the same
//    for every source), the values are broadcast by shuffles, and four edges
//    are relaxed per step with their four 128-byte distance rows loaded before
//    any of their atomicMin updates.
//  * edge form (few active sources): lane k relaxes edge k of the chunk, once
//    per active source (scattered 4-byte distance accesses), so a word with
//    2 active sources costs 2 warp steps per 32 edges instead of 32.
//
// An update counts as an improvement when nd is below the distance read just
// before it; the atomicMin's old value is not awaited.  When another
// relaxation of the same (vertex, source) got below nd in between, that one
// improved and marks the same frontier bit, so the next frontier is the same
// set as with the old value tested, and one memory round trip leaves each
// relaxation's critical path.
//
// The Sink records the next frontier:
//   row(v, ball)      lane 0: sources `ball` of word j improved at v
//   mark(v, bit)      one lane: source bit `bit` improved at v; returns true
//                     if v newly entered the next frontier queue bitmap
//   append(q, v)      whole warp: appends the lanes' newly queued vertices
//   any(bit)          lane 0: source bit `bit` improved somewhere this step
#pragma once
#include "eg_internal.cuh"

#ifndef EG_MRELAX_SPARSE
// at most this many active sources: edge form.  Directed RMAT-23, 256
// sources (u32 / fp32 weights): 0 (row form always) 325 / 635 ms, 1 296 / 590,
// 2 290 / 560, 3 291 / 568, 4 294 / 585, 8 339 / 725, 16 506 / 1055
#define EG_MRELAX_SPARSE 2
#endif
#define EG_MSSSP_MINB 8     // resident CTAs per SM asked of the compiler for the item kernels (32 registers)

template <class Sink>
__device__ __forceinline__ void eg_mrelax_rows(uint32_t u, uint32_t p0, uint32_t p1, const uint32_t *__restrict__ col,
                                               const uint32_t *__restrict__ wts, const eg_wrule &w, bool on,
                                               uint32_t du, uint32_t s, uint32_t K, uint32_t *dist, Sink &sink) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c0 = p0; c0 < p1; c0 += 32) {
        const uint32_t pl = c0 + lane;
        const uint32_t myv = pl < p1 ? __ldg(col + pl) : u;  // u: skipped like a self-loop
        const uint32_t myw = pl < p1 ? __ldg(wts + pl) : 0u;
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
                // self-loops skipped (sssp_pushpull.c:80); the atomic's old
                // value is not awaited (see the header)
                const bool improved = on && vv[q] != u && nd[q] < cur[q];
                if (improved) atomicMin(dist + (uint64_t)vv[q] * K + s, nd[q]);
                const uint32_t ball = __ballot_sync(EG_FULL_MASK, improved);
                if (ball && lane == 0) sink.row(vv[q], ball);
            }
        }
    }
}

template <class Sink>
__device__ __forceinline__ void eg_mrelax_edges(uint32_t u, uint32_t p0, uint32_t p1,
                                                const uint32_t *__restrict__ col, const uint32_t *__restrict__ wts,
                                                const eg_wrule &w, uint32_t a,
                                                uint32_t du, uint32_t j, uint32_t K, uint32_t *dist, Sink &sink) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c0 = p0; c0 < p1; c0 += 32) {
        const uint32_t pl = c0 + lane;
        const bool valid = pl < p1;
        const uint32_t v = valid ? __ldg(col + pl) : u;
        const uint32_t wt = valid ? __ldg(wts + pl) : 0u;
        for (uint32_t aa = a; aa; aa &= aa - 1) {
            const uint32_t sl = (uint32_t)__ffs(aa) - 1;
            const uint32_t s = 32 * j + sl;
            const uint32_t nd = w.add(__shfl_sync(EG_FULL_MASK, du, sl), wt);
            bool improved = false;
            if (v != u) {  // self-loops (and lanes past the end) skipped
                uint32_t *dp = dist + (uint64_t)v * K + s;
                if (nd < __ldcg(dp)) {
                    atomicMin(dp, nd);
                    improved = true;
                }
            }
            const bool q = improved && sink.mark(v, 1u << sl);
            if (__ballot_sync(EG_FULL_MASK, improved) && lane == 0) sink.any(1u << sl);
            sink.append(q, v);
        }
    }
}

template <class Sink>
__device__ __forceinline__ void eg_mrelax(uint32_t u, uint32_t p0, uint32_t p1, const uint32_t *__restrict__ col,
                                          const uint32_t *__restrict__ wts, const eg_wrule &w, uint32_t a, uint32_t du,
                                          uint32_t j, uint32_t K, uint32_t *dist, Sink &sink) {
    if (__popc(a) > EG_MRELAX_SPARSE) {
        const uint32_t lane = threadIdx.x & 31;
        eg_mrelax_rows(u, p0, p1, col, wts, w, (a >> lane) & 1u, du, 32 * j + lane, K, dist, sink);
    } else {
        eg_mrelax_edges(u, p0, p1, col, wts, w, a, du, j, K, dist, sink);
    }
}

// Frontier items it = qi * kw + j (qi: queue index, j: source word) taken 32
// per warp step: lane l loads item base + l's vertex, active word and list
// bounds (independent loads, so their latencies overlap), hubs with more than
// big_deg edges go to the big list for a grid-wide kernel, and the warp then
// relaxes the other items one after another with their metadata broadcast by
// shuffles; the next item's source distances are loaded before the current
// item is relaxed.  `scanned` (lane 0) counts (edge, source) relaxations.
template <class Sink>
__device__ __forceinline__ void eg_mrelax_items(uint64_t base, uint64_t items, const uint32_t *__restrict__ queue,
                                                uint32_t kw, const uint32_t *__restrict__ ptr,
                                                const uint32_t *__restrict__ col, const uint32_t *__restrict__ wts,
                                                const eg_wrule &w, uint32_t K, uint32_t *dist,
                                                const uint32_t *__restrict__ act, uint32_t big_deg, uint32_t *big,
                                                uint32_t *nbig, Sink &sink, unsigned long long &scanned) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t it = base + lane;
    const bool valid = it < items;
    const uint32_t ul = valid ? __ldg(queue + it / kw) : 0u;
    const uint32_t jl = (uint32_t)(it % kw);
    const uint32_t al = valid ? __ldg(act + (uint64_t)ul * kw + jl) : 0u;
    const uint32_t bl = al ? __ldg(ptr + ul) : 0u, el = al ? __ldg(ptr + ul + 1) : 0u;
    const bool isbig = al && el - bl > big_deg;
    const uint32_t bigball = __ballot_sync(EG_FULL_MASK, isbig);
    if (bigball) {
        uint32_t at = 0;
        if (lane == 0) at = atomicAdd(nbig, (uint32_t)__popc(bigball));
        at = __shfl_sync(EG_FULL_MASK, at, 0);
        if (isbig) big[at + __popc(bigball & eg_lanemask_lt())] = (uint32_t)((uint64_t)ul * kw + jl);
    }
    uint32_t work = __ballot_sync(EG_FULL_MASK, al && !isbig);
    if (!work) return;
    uint32_t k = (uint32_t)__ffs(work) - 1;
    uint32_t u = __shfl_sync(EG_FULL_MASK, ul, k), j = __shfl_sync(EG_FULL_MASK, jl, k);
    uint32_t a = __shfl_sync(EG_FULL_MASK, al, k);
    uint32_t du = ((a >> lane) & 1u) ? __ldcg(dist + (uint64_t)u * K + 32 * j + lane) : 0u;
    while (work) {
        k = (uint32_t)__ffs(work) - 1;
        work &= work - 1;
        const uint32_t b = __shfl_sync(EG_FULL_MASK, bl, k), e = __shfl_sync(EG_FULL_MASK, el, k);
        uint32_t u2 = 0, j2 = 0, a2 = 0, du2 = 0;
        if (work) {  // the next item's distances, loaded ahead
            const uint32_t k2 = (uint32_t)__ffs(work) - 1;
            u2 = __shfl_sync(EG_FULL_MASK, ul, k2);
            j2 = __shfl_sync(EG_FULL_MASK, jl, k2);
            a2 = __shfl_sync(EG_FULL_MASK, al, k2);
            du2 = ((a2 >> lane) & 1u) ? __ldcg(dist + (uint64_t)u2 * K + 32 * j2 + lane) : 0u;
        }
        if (lane == 0) scanned += (unsigned long long)(e - b) * (unsigned long long)__popc(a);
        sink.j = j;
        eg_mrelax(u, b, e, col, wts, w, a, du, j, K, dist, sink);
        u = u2;
        j = j2;
        a = a2;
        du = du2;
    }
}
