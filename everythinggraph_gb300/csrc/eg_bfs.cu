// Direction-optimising BFS with a bitmap frontier, and bit-sliced
// multi-source BFS.
//
// Replaces bfs_simple.c (bfs_push 121-134, bfs_pull 104-120, the switch rule
// 191-197) and bfsgrid_cilk.c (get_bfs 48-65, iterator 121-168).  The
// reference's frontier is a byte map plus id lists (random.c:74-77,
// buffer.c:62-297); here it is a bitmap in the style of Gemini's Bitmap
// (bitmap.h:16-50), written one 32-bit word per warp with __ballot_sync, plus
// a compacted id queue for push levels.
//
// Levels follow the reference: level[root] = 1, unreached = 0 (the value
// bfsgrid_cilk and the edge-centric bfs_simple write into dist[]).
#include <stdlib.h>
#include <string.h>

#include "eg_bigwork.cuh"
#include "eg_frontier.cuh"
#include "eg_internal.cuh"
#include "eg_mspull.cuh"

namespace {

struct BfsCounters {
    unsigned long long next_deg;  // sum of out-degrees of the new frontier
    uint32_t next_count;          // vertices in the new frontier
    uint32_t qsize;               // entries in the next queue
    uint32_t nbig;                // frontier vertices deferred to the cooperative kernel
    uint32_t qbuilt;              // ids written by k_bm_queue (the frontier count is known already)
};

// Frontier vertices with more out-edges than a threshold are expanded by the
// whole grid (k_*_push_big) instead of one warp: an RMAT hub has 10^5..10^6.
#define EG_BFS_WARP_EDGES 256u          // pushes with 32 lists per warp (8192 edges at most)
#define EG_BFS_SMALL_BIG 64u            // single-source levels with few frontier vertices
#define EG_BFS_CHUNK 4096u              // edges of a deferred hub per CTA work unit
#define EG_BFS_QUEUE_EDGES (1u << 18)   // push levels over more edges build no next queue
#define EG_NO_VERTEX 0xffffffffu

// Block-level reduction of per-thread counters: one atomic per block.
__device__ __forceinline__ void block_add_counters(BfsCounters *c, uint32_t cnt, unsigned long long deg) {
    __shared__ uint32_t s_cnt[32];
    __shared__ unsigned long long s_deg[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_down_sync(EG_FULL_MASK, cnt, o);
        deg += __shfl_down_sync(EG_FULL_MASK, deg, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_cnt[w] = cnt;
        s_deg[w] = deg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tc = 0;
        unsigned long long td = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            tc += s_cnt[i];
            td += s_deg[i];
        }
        if (tc) {
            atomicAdd(&c->next_count, tc);
            atomicAdd(&c->next_deg, td);
        }
    }
}

// noin (may be NULL): a bit per vertex without in-neighbours.  Such a vertex
// can only be the root, so it starts out visited: the pull levels then skip
// it, and skip whole words of them (on undirected RMAT about half the ids
// are isolated).  Its level and parent stay those of an unreached vertex.
__global__ void k_bfs_init(uint32_t n, int32_t *level, int32_t *parent, uint32_t *visited, uint32_t *cur_bm,
                           uint32_t nw, uint32_t root, uint32_t *queue, const uint32_t *deg, BfsCounters *cnt,
                           const uint32_t *__restrict__ noin) {
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        level[v] = v == root ? 1 : 0;
        if (parent) parent[v] = v == root ? (int32_t)root : -1;
    }
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += stride) {
        uint32_t bit = (root >> 5) == w ? 1u << (root & 31) : 0u;
        visited[w] = bit | (noin ? noin[w] : 0u);
        cur_bm[w] = bit;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        queue[0] = root;
        cnt->next_count = 1;
        cnt->qsize = 1;
        cnt->next_deg = deg[root];
    }
}

// Claims v for the next level if it is unvisited (atomicOr on its visited
// bit); returns true for the one thread that set the bit.
__device__ __forceinline__ bool bfs_claim(uint32_t v, uint32_t u, uint32_t *visited, uint32_t *next_bm, int32_t *level,
                                          int32_t *parent, int32_t next_level) {
    const uint32_t bit = 1u << (v & 31);
    if (__ldcg(visited + (v >> 5)) & bit) return false;
    const uint32_t old = atomicOr(visited + (v >> 5), bit);
    if (old & bit) return false;
    level[v] = next_level;
    if (parent) parent[v] = (int32_t)u;
    atomicOr(next_bm + (v >> 5), bit);
    return true;
}

// Appends the claimed vertices of a warp to the next queue (one atomic per
// warp) and counts them.  next_queue NULL: count only — the next frontier is
// the next_bm bitmap alone (a level with many claims would otherwise meet on
// the one queue counter).
__device__ __forceinline__ void warp_append(bool claimed, uint32_t v, uint32_t *next_queue, BfsCounters *cnt,
                                            const uint32_t *__restrict__ deg, uint32_t &my_cnt,
                                            unsigned long long &my_deg) {
    if (!next_queue) {
        if (claimed) {
            my_cnt++;
            my_deg += deg[v];
        }
        return;
    }
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t ball = __ballot_sync(EG_FULL_MASK, claimed);
    if (ball) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&cnt->qsize, __popc(ball));
        base = __shfl_sync(EG_FULL_MASK, base, 0);
        if (claimed) {
            next_queue[base + __popc(ball & eg_lanemask_lt())] = v;
            my_cnt++;
            my_deg += deg[v];
        }
    }
}

// Expands the out-lists of a warp's 32 lanes' vertices together
// (eg_warp_lists): claims the unvisited targets for the next level.
__device__ __forceinline__ void bfs_expand_warp(uint32_t u, uint32_t b, uint32_t d, const uint32_t *__restrict__ col,
                                                const uint32_t *__restrict__ deg, uint32_t *visited,
                                                uint32_t *next_bm, uint32_t *next_queue, int32_t *level,
                                                int32_t *parent, int32_t next_level, BfsCounters *cnt,
                                                uint32_t &my_cnt, unsigned long long &my_deg) {
    eg_warp_lists(u, b, d, [&](bool valid, uint32_t, uint32_t ou, uint32_t p) {
        bool claimed = false;
        uint32_t v = 0;
        if (valid) {
            v = col[p];
            claimed = bfs_claim(v, ou, visited, next_bm, level, parent, next_level);
        }
        warp_append(claimed, v, next_queue, cnt, deg, my_cnt, my_deg);
    });
}

// Top-down step: a warp takes 32 frontier vertices (one per lane) and
// expands them together (bfs_expand_warp).  Vertices with more than big_deg
// out-edges go to a side list that k_bfs_push_big expands with every thread
// of the grid.
__global__ void __launch_bounds__(256) k_bfs_push(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                  const uint32_t *__restrict__ deg, const uint32_t *__restrict__ queue,
                                                  uint32_t qlen, uint32_t *visited, uint32_t *next_bm,
                                                  uint32_t *next_queue, int32_t *level, int32_t *parent,
                                                  int32_t next_level, BfsCounters *cnt, uint32_t *big,
                                                  uint32_t big_deg) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t my_cnt = 0;
    unsigned long long my_deg = 0;
    // uniform trip count per warp (q0 is the same for all lanes)
    for (uint32_t q0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; q0 < qlen; q0 += warps * 32) {
        const uint32_t qi = q0 + lane;
        uint32_t u = 0, b = 0, d = 0;
        if (qi < qlen) {
            u = queue[qi];
            b = ptr[u];
            d = ptr[u + 1] - b;
            if (d > big_deg) {
                big[atomicAdd(&cnt->nbig, 1u)] = u;
                d = 0;
            }
        }
        bfs_expand_warp(u, b, d, col, deg, visited, next_bm, next_queue, level, parent, next_level, cnt, my_cnt,
                        my_deg);
    }
    block_add_counters(cnt, my_cnt, my_deg);
}

// Small push levels back to back in one CTA (1024 threads): the root's level
// and the tail levels after the pull levels have a few hundred to a few
// thousand frontier vertices, and as separate launches each paid ~25 us of
// launches and host round trip for a few us of work.  The frontier lives in
// shared memory (two queues of EG_SMALL_Q ids); a level runs here only while
// its frontier has at most EG_SMALL_Q vertices and out-edges (so the next
// frontier, at most one id per edge, always fits) and, in auto mode, the
// switch rule still asks for push.  Larger caps lose: one SM walking 4K-16K
// edges per level with dependent claims took longer than a full grid plus
// its launch overhead (RMAT-24: 1K 0.637 ms per BFS, 4K 0.650, 16K 0.728,
// none 0.651).  Block barriers only; the frontier is
// handed back through `queue` and the host loop continues from it.
#define EG_SMALL_Q 1024u
#define EG_FDEG_UNKNOWN (~0ull)
struct BfsSmallOut {
    uint32_t qlen;     // frontier size handed back
    uint32_t levels;   // levels run (0: the incoming frontier was not small)
    int32_t lvl;       // level number of the frontier handed back
    uint32_t pad;
    unsigned long long fdeg, reached, traversed;
    unsigned long long fdeg_in;  // out-degree sum of the incoming frontier
};

// fdeg = EG_FDEG_UNKNOWN: the kernel sums the incoming frontier's degrees
// itself (the root's level, launched right after k_bfs_init without a host
// round trip).  The level counters `cnt` are cleared for the next level.
__global__ void __launch_bounds__(1024) k_bfs_small(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                    const uint32_t *__restrict__ deg, uint32_t *visited,
                                                    int32_t *level, int32_t *parent, uint32_t *queue, uint32_t qlen,
                                                    unsigned long long fdeg, int32_t lvl, double threshold,
                                                    int auto_dir, BfsSmallOut *out, BfsCounters *cnt) {
    __shared__ uint32_t s_q[2 * EG_SMALL_Q];
    __shared__ uint32_t s_n;
    __shared__ unsigned long long s_deg;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const bool fits = qlen <= EG_SMALL_Q;
    if (fits)
        for (uint32_t i = threadIdx.x; i < qlen; i += blockDim.x) s_q[i] = queue[i];
    if (threadIdx.x == 0) {
        s_deg = 0;
        cnt->next_deg = 0;
        cnt->next_count = 0;
        cnt->qsize = 0;
        cnt->nbig = 0;
        cnt->qbuilt = 0;
    }
    __syncthreads();
    if (fits && fdeg == EG_FDEG_UNKNOWN) {
        unsigned long long my = 0;
        for (uint32_t i = threadIdx.x; i < qlen; i += blockDim.x) my += deg[s_q[i]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) my += __shfl_down_sync(EG_FULL_MASK, my, o);
        if (lane == 0 && my) atomicAdd(&s_deg, my);
        __syncthreads();
        fdeg = s_deg;
        __syncthreads();
    }
    const unsigned long long fdeg_in = fdeg;
    if (!fits || fdeg > EG_SMALL_Q || (auto_dir && (double)qlen + (double)fdeg > threshold)) {
        if (threadIdx.x == 0) {  // not a small level: nothing run
            out->qlen = qlen;
            out->levels = 0;
            out->lvl = lvl;
            out->fdeg = fdeg;
            out->reached = 0;
            out->traversed = 0;
            out->fdeg_in = fdeg_in;
        }
        return;
    }
    int c = 0;
    uint32_t levels = 0;
    unsigned long long reached = 0, traversed = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            s_n = 0;
            s_deg = 0;
        }
        __syncthreads();
        const uint32_t *cq = s_q + (c ? EG_SMALL_Q : 0u);
        uint32_t *nq = s_q + (c ? 0u : EG_SMALL_Q);
        const int32_t next_level = lvl + 1;
        unsigned long long my_deg = 0;
        for (uint32_t q0 = warp * 32; q0 < qlen; q0 += nwarps * 32) {  // uniform per warp
            const uint32_t qi = q0 + lane;
            uint32_t u = 0, b = 0, d = 0;
            if (qi < qlen) {
                u = cq[qi];
                b = ptr[u];
                d = ptr[u + 1] - b;
            }
            eg_warp_lists(u, b, d, [&](bool valid, uint32_t, uint32_t ou, uint32_t p) {
                bool claimed = false;
                uint32_t v = 0;
                if (valid) {
                    v = col[p];
                    const uint32_t bit = 1u << (v & 31);
                    if (!(__ldcg(visited + (v >> 5)) & bit) && !(atomicOr(visited + (v >> 5), bit) & bit)) {
                        claimed = true;
                        level[v] = next_level;
                        if (parent) parent[v] = (int32_t)ou;
                    }
                }
                const uint32_t ball = __ballot_sync(EG_FULL_MASK, claimed);
                if (ball) {
                    uint32_t base = 0;
                    if (lane == 0) base = atomicAdd(&s_n, (uint32_t)__popc(ball));
                    base = __shfl_sync(EG_FULL_MASK, base, 0);
                    if (claimed) {
                        nq[base + __popc(ball & eg_lanemask_lt())] = v;
                        my_deg += deg[v];
                    }
                }
            });
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) my_deg += __shfl_down_sync(EG_FULL_MASK, my_deg, o);
        if (lane == 0 && my_deg) atomicAdd(&s_deg, my_deg);
        __syncthreads();
        qlen = s_n;
        fdeg = s_deg;
        __syncthreads();  // every thread has read s_n and s_deg before the next level resets them
        levels++;
        lvl++;
        reached += qlen;
        traversed += fdeg;
        c ^= 1;
        if (qlen == 0 || qlen > EG_SMALL_Q || fdeg > EG_SMALL_Q ||
            (auto_dir && (double)qlen + (double)fdeg > threshold))
            break;
    }
    const uint32_t *cq = s_q + (c ? EG_SMALL_Q : 0u);
    for (uint32_t i = threadIdx.x; i < qlen; i += blockDim.x) queue[i] = cq[i];
    if (threadIdx.x == 0) {
        out->qlen = qlen;
        out->levels = levels;
        out->lvl = lvl;
        out->fdeg = fdeg;
        out->reached = reached;
        out->traversed = traversed;
        out->fdeg_in = fdeg_in;
    }
}

// Frontier queue -> bitmap (the bitmap zeroed before).
__global__ void k_queue_bm(const uint32_t *__restrict__ queue, uint32_t qlen, uint32_t *bm) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x) {
        const uint32_t v = queue[i];
        atomicOr(bm + (v >> 5), 1u << (v & 31));
    }
}

// Expands the deferred high-degree frontier vertices: their out-lists cut
// into chunks of `chunk` edges (as k_big_offsets counted them), one CTA per
// chunk.
__global__ void __launch_bounds__(256) k_bfs_push_big(const uint32_t *__restrict__ ptr,
                                                      const uint32_t *__restrict__ col,
                                                      const uint32_t *__restrict__ deg, const uint32_t *big,
                                                      const uint32_t *__restrict__ bigoff, uint32_t *visited,
                                                      uint32_t *next_bm, uint32_t *next_queue, int32_t *level,
                                                      int32_t *parent, int32_t next_level, BfsCounters *cnt,
                                                      uint32_t chunk) {
    const uint32_t nbig = *(volatile uint32_t *)&cnt->nbig;
    uint32_t my_cnt = 0;
    unsigned long long my_deg = 0;
    const uint32_t total = nbig ? bigoff[nbig] : 0u;
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t u = big[i];
        const uint32_t b = ptr[u] + (c - bigoff[i]) * chunk, e = min(ptr[u + 1], b + chunk);
        // warp-uniform trip count: each warp covers 32 consecutive entries
        for (uint32_t p0 = b + (threadIdx.x & ~31u); p0 < e; p0 += blockDim.x) {
            const uint32_t p = p0 + (threadIdx.x & 31);
            bool claimed = false;
            uint32_t v = 0;
            if (p < e) {
                v = col[p];
                claimed = bfs_claim(v, u, visited, next_bm, level, parent, next_level);
            }
            warp_append(claimed, v, next_queue, cnt, deg, my_cnt, my_deg);
        }
    }
    block_add_counters(cnt, my_cnt, my_deg);
}

// An unvisited vertex's bottom-up scan: first[] (one coalesced word per
// vertex) names the in-neighbour with the largest out-degree, most often in
// the frontier; the list is read, in order, only when that one is not.  The
// parent is that in-neighbour or the first one in list order in the frontier.
__device__ __forceinline__ bool pull_scan(uint32_t v, const uint32_t *__restrict__ ptr,
                                          const uint32_t *__restrict__ col, const uint32_t *__restrict__ first,
                                          const uint32_t *cur_bm, int32_t *level, int32_t *parent,
                                          int32_t next_level) {
    const uint32_t f0 = __ldg(first + v);
    if (f0 == EG_NO_VERTEX) return false;  // no in-neighbours
    // the frontier bitmap is not written during a pull level: read through L1,
    // which keeps the words of the hub ids
    uint32_t u = f0;
    bool hit = (__ldg(cur_bm + (u >> 5)) >> (u & 31)) & 1u;
    if (!hit) {
        // four entries per step, their loads all in flight before the tests
        // (a long list is a chain of dependent loads otherwise); the first
        // hit in list order is kept
        uint32_t p = ptr[v];
        const uint32_t e = ptr[v + 1];
        for (; p + 4 <= e; p += 4) {
            const uint32_t u0 = col[p], u1 = col[p + 1], u2 = col[p + 2], u3 = col[p + 3];
            const uint32_t w0 = __ldg(cur_bm + (u0 >> 5)), w1 = __ldg(cur_bm + (u1 >> 5));
            const uint32_t w2 = __ldg(cur_bm + (u2 >> 5)), w3 = __ldg(cur_bm + (u3 >> 5));
            const bool h0 = (w0 >> (u0 & 31)) & 1u, h1 = (w1 >> (u1 & 31)) & 1u;
            const bool h2 = (w2 >> (u2 & 31)) & 1u, h3 = (w3 >> (u3 & 31)) & 1u;
            if (h0 | h1 | h2 | h3) {
                u = h0 ? u0 : (h1 ? u1 : (h2 ? u2 : u3));
                hit = true;
                break;
            }
        }
        for (; !hit && p < e; p++) {
            u = col[p];
            hit = (__ldg(cur_bm + (u >> 5)) >> (u & 31)) & 1u;
        }
    }
    if (hit) {
        level[v] = next_level;
        if (parent) parent[v] = (int32_t)u;
    }
    return hit;
}

// first[v] = v's in-neighbour with the largest out-degree (the smallest id
// among equals), EG_NO_VERTEX when the in-list is empty: the in-neighbour
// most likely to be in a large frontier, checked before the list is read.
// One warp per vertex, 32 entries per step.
__global__ void k_first_in(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                           const uint32_t *__restrict__ deg, uint32_t n, uint32_t *__restrict__ first) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        const uint32_t b = ptr[v], e = ptr[v + 1];
        unsigned long long best = 0ull;  // (degree << 32) | ~id: the max is the largest degree, then the smallest id
        for (uint32_t p = b + lane; p < e; p += 32) {
            const uint32_t u = col[p];
            const unsigned long long key = ((unsigned long long)deg[u] << 32) | (uint32_t)~u;
            best = key > best ? key : best;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_down_sync(EG_FULL_MASK, best, o);
            best = y > best ? y : best;
        }
        if (lane == 0) first[v] = b < e ? ~(uint32_t)best : EG_NO_VERTEX;
    }
}

// bits[w]: bit l set when vertex 32w + l has no in-neighbours (ids past n: set)
__global__ void k_no_in_bits(const uint32_t *__restrict__ first, uint32_t n, uint32_t nw, uint32_t *bits) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;  // a multiple of 32: warps stay whole
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < (uint64_t)nw * 32; v += stride) {
        const bool none = v >= n || first[v] == EG_NO_VERTEX;
        const uint32_t b = __ballot_sync(EG_FULL_MASK, none);
        if ((threadIdx.x & 31) == 0) bits[v >> 5] = b;
    }
}

// Bottom-up step: one thread per vertex, warps over 32 consecutive vertices
// (one bitmap word).  An unvisited vertex scans its in-list and stops at the
// first neighbour in the frontier.  The new frontier word is the warp ballot.
__global__ void __launch_bounds__(256) k_bfs_pull(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                  const uint32_t *__restrict__ first,
                                                  const uint32_t *__restrict__ deg, uint32_t n,
                                                  const uint32_t *__restrict__ cur_bm, uint32_t *visited,
                                                  uint32_t *next_bm, int32_t *level, int32_t *parent,
                                                  int32_t next_level, BfsCounters *cnt) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (n + 31) >> 5;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t my_cnt = 0;
    unsigned long long my_deg = 0;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += warps) {
        const uint32_t vis = visited[w];
        if (vis == EG_FULL_MASK) {
            if (lane == 0) next_bm[w] = 0;
            continue;
        }
        const uint32_t v = (w << 5) + lane;
        bool found = false;
        if (v < n && !(vis & (1u << lane)))
            found = pull_scan(v, ptr, col, first, cur_bm, level, parent, next_level);
        const uint32_t ball = __ballot_sync(EG_FULL_MASK, found);
        if (lane == 0) {
            next_bm[w] = ball;
            if (ball) visited[w] = vis | ball;
        }
        if (found) {
            my_cnt++;
            my_deg += deg[v];
        }
    }
    block_add_counters(cnt, my_cnt, my_deg);
}

// ---------------------------------------------------------------- device-driven levels
// The level loop as a CUDA graph: a start kernel, then a while node whose
// body runs one level (prep, push, push_big, pull, end).  Every kernel reads
// the level's direction and buffer parity from BfsGState and returns at once
// when it is not this level's step; the end kernel folds the counters,
// picks the next direction with the reference's rule and clears the while
// condition when the frontier is empty.
struct BfsGState {
    uint32_t parity;      // frontier buffers in use: bm[parity], q[parity]
    uint32_t pull;        // this level runs bottom-up
    uint32_t need_queue;  // the frontier exists only as a bitmap
    uint32_t qlen;        // queue length when !need_queue
    uint32_t qfill;       // queue length built by the prep kernel
    uint32_t lvl;         // level of the current frontier (root = 1)
    uint32_t levels, pull_levels;
    uint32_t root, dirmode, n, err;
    unsigned long long fdeg, reached, traversed;
    double threshold;
};

__global__ void k_bfsg_start(BfsGState *st, const uint32_t *__restrict__ deg, int32_t *level, int32_t *parent,
                             uint32_t *visited, uint32_t *bm0, uint32_t nw, uint32_t *q0, BfsCounters *cnt,
                             const uint32_t *__restrict__ noin) {
    const uint32_t n = st->n, root = st->root;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        level[v] = v == root ? 1 : 0;
        if (parent) parent[v] = v == root ? (int32_t)root : -1;
    }
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += stride) {
        const uint32_t bit = (root >> 5) == w ? 1u << (root & 31) : 0u;
        visited[w] = bit | (noin ? noin[w] : 0u);  // as in k_bfs_init
        bm0[w] = bit;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q0[0] = root;
        const unsigned long long d = deg[root];
        st->parity = 0;
        st->need_queue = 0;
        st->qlen = 1;
        st->qfill = 0;
        st->lvl = 1;
        st->levels = 0;
        st->pull_levels = 0;
        st->err = 0;
        st->fdeg = d;
        st->reached = 1;
        st->traversed = d;
        st->pull = st->dirmode == EG_BFS_PULL_ONLY || (st->dirmode == EG_BFS_AUTO && 1.0 + (double)d > st->threshold);
        cnt->next_deg = 0;
        cnt->next_count = 0;
        cnt->qsize = 0;
        cnt->nbig = 0;
    }
}

// Push levels: clear the next bitmap; after a pull level, list the frontier
// (bitmap -> queue, one atomic per block).
__global__ void __launch_bounds__(256) k_bfsg_prep(BfsGState *st, uint32_t *bm0, uint32_t *bm1, uint32_t *q0,
                                                   uint32_t *q1, uint32_t nw) {
    if (st->pull) return;
    const uint32_t par = st->parity;
    uint32_t *cur = par ? bm1 : bm0, *nxt = par ? bm0 : bm1, *q = par ? q1 : q0;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) nxt[w] = 0;
    if (!st->need_queue) return;
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_base;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t w0 = blockIdx.x * blockDim.x; w0 < nw; w0 += gridDim.x * blockDim.x) {
        const uint32_t w = w0 + threadIdx.x;
        const uint32_t word = w < nw ? cur[w] : 0u;
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
            s_base = t ? atomicAdd(&st->qfill, t) : 0u;
        }
        __syncthreads();
        uint32_t pos = s_base + s_warp[warp] + x - c;
        uint32_t bits = word;
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            q[pos++] = (w << 5) + (uint32_t)b;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_bfsg_push(const BfsGState *st, const uint32_t *__restrict__ ptr,
                                                   const uint32_t *__restrict__ col, const uint32_t *__restrict__ deg,
                                                   uint32_t *q0, uint32_t *q1, uint32_t *bm0, uint32_t *bm1,
                                                   uint32_t *visited, int32_t *level, int32_t *parent,
                                                   BfsCounters *cnt, uint32_t *big) {
    if (st->pull) return;
    const uint32_t par = st->parity;
    const uint32_t qlen = st->need_queue ? st->qfill : st->qlen;
    const uint32_t *queue = par ? q1 : q0;
    uint32_t *next_queue = par ? q0 : q1, *next_bm = par ? bm0 : bm1;
    const int32_t next_level = (int32_t)st->lvl + 1;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t my_cnt = 0;
    unsigned long long my_deg = 0;
    for (uint32_t q0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; q0 < qlen; q0 += warps * 32) {
        const uint32_t qi = q0 + lane;
        uint32_t u = 0, b = 0, d = 0;
        if (qi < qlen) {
            u = queue[qi];
            b = ptr[u];
            d = ptr[u + 1] - b;
            if (d > EG_BFS_WARP_EDGES) {
                big[atomicAdd(&cnt->nbig, 1u)] = u;
                d = 0;
            }
        }
        bfs_expand_warp(u, b, d, col, deg, visited, next_bm, next_queue, level, parent, next_level, cnt, my_cnt,
                        my_deg);
    }
    block_add_counters(cnt, my_cnt, my_deg);
}

__global__ void __launch_bounds__(256) k_bfsg_push_big(const BfsGState *st, const uint32_t *__restrict__ ptr,
                                                       const uint32_t *__restrict__ col,
                                                       const uint32_t *__restrict__ deg, const uint32_t *big,
                                                       const uint32_t *__restrict__ bigoff, uint32_t *q0, uint32_t *q1,
                                                       uint32_t *bm0, uint32_t *bm1, uint32_t *visited, int32_t *level,
                                                       int32_t *parent, BfsCounters *cnt) {
    if (st->pull) return;
    const uint32_t nbig = *(volatile uint32_t *)&cnt->nbig;
    if (!nbig) return;
    const uint32_t par = st->parity;
    uint32_t *next_queue = par ? q0 : q1, *next_bm = par ? bm0 : bm1;
    const int32_t next_level = (int32_t)st->lvl + 1;
    uint32_t my_cnt = 0;
    unsigned long long my_deg = 0;
    const uint32_t total = bigoff[nbig];
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t u = big[i];
        const uint32_t b = ptr[u] + (c - bigoff[i]) * EG_BFS_CHUNK, e = min(ptr[u + 1], b + EG_BFS_CHUNK);
        for (uint32_t p0 = b + (threadIdx.x & ~31u); p0 < e; p0 += blockDim.x) {
            const uint32_t p = p0 + (threadIdx.x & 31);
            bool claimed = false;
            uint32_t v = 0;
            if (p < e) {
                v = col[p];
                claimed = bfs_claim(v, u, visited, next_bm, level, parent, next_level);
            }
            warp_append(claimed, v, next_queue, cnt, deg, my_cnt, my_deg);
        }
    }
    block_add_counters(cnt, my_cnt, my_deg);
}

__global__ void __launch_bounds__(256) k_bfsg_pull(const BfsGState *st, const uint32_t *__restrict__ ptr,
                                                   const uint32_t *__restrict__ col,
                                                   const uint32_t *__restrict__ first, const uint32_t *__restrict__ deg,
                                                   uint32_t *bm0, uint32_t *bm1, uint32_t *visited, int32_t *level,
                                                   int32_t *parent, BfsCounters *cnt) {
    if (!st->pull) return;
    const uint32_t n = st->n;
    const uint32_t par = st->parity;
    const uint32_t *cur_bm = par ? bm1 : bm0;
    uint32_t *next_bm = par ? bm0 : bm1;
    const int32_t next_level = (int32_t)st->lvl + 1;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (n + 31) >> 5;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t my_cnt = 0;
    unsigned long long my_deg = 0;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += warps) {
        const uint32_t vis = visited[w];
        if (vis == EG_FULL_MASK) {
            if (lane == 0) next_bm[w] = 0;
            continue;
        }
        const uint32_t v = (w << 5) + lane;
        bool found = false;
        if (v < n && !(vis & (1u << lane)))
            found = pull_scan(v, ptr, col, first, cur_bm, level, parent, next_level);
        const uint32_t ball = __ballot_sync(EG_FULL_MASK, found);
        if (lane == 0) {
            next_bm[w] = ball;
            if (ball) visited[w] = vis | ball;
        }
        if (found) {
            my_cnt++;
            my_deg += deg[v];
        }
    }
    block_add_counters(cnt, my_cnt, my_deg);
}

__global__ void k_bfsg_end(BfsGState *st, BfsCounters *cnt, cudaGraphConditionalHandle handle) {
    const uint32_t count = cnt->next_count;
    const unsigned long long fdeg = cnt->next_deg;
    st->levels += 1;
    if (st->pull) st->pull_levels += 1;
    st->reached += count;
    st->traversed += fdeg;
    if (count == 0 || st->lvl > st->n + 1) {
        if (count != 0) st->err = 1;
        cudaGraphSetConditional(handle, 0);
        return;
    }
    st->need_queue = st->pull ? 1u : 0u;  // a pull level leaves only a bitmap
    st->qlen = cnt->qsize;
    st->qfill = 0;
    st->parity ^= 1u;
    st->lvl += 1;
    st->fdeg = fdeg;
    st->pull = st->dirmode == EG_BFS_PULL_ONLY ||
               (st->dirmode == EG_BFS_AUTO && (double)count + (double)fdeg > st->threshold);
    cnt->next_count = 0;
    cnt->next_deg = 0;
    cnt->qsize = 0;
    cnt->nbig = 0;
}
}  // namespace

extern "C" void eg_bfs_opts_default(eg_bfs_opts *o) {
    if (!o) return;
    o->direction = EG_BFS_AUTO;
    o->switch_divisor = -1.0;
    o->device_parents = 0;
    o->host_loop = -1;
}

static uint32_t blocks_for(eg_ctx *ctx, uint64_t threads) {
    uint64_t b = (threads + 255) / 256;
    uint64_t cap = (uint64_t)ctx->sm_count * 8;
    if (b > cap) b = cap;
    return b ? (uint32_t)b : 1u;
}

// Captures the level loop of eg_bfs for the current buffers (see BfsGState).
static int bfs_graph_build(eg_graph *g, eg_bfs_graph &bg, const void *const key[8], BfsGState *st,
                           const uint32_t *deg, int32_t *level, int32_t *parent, uint32_t *visited, uint32_t *bm0,
                           uint32_t *bm1, uint32_t *q0, uint32_t *q1, uint32_t *big, uint32_t *bigoff,
                           BfsCounters *cnt, const eg_adj *in_adj) {
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n, nw = (n + 31) >> 5;
    if (bg.exec) cudaGraphExecDestroy(bg.exec);
    if (bg.graph) cudaGraphDestroy(bg.graph);
    bg.exec = nullptr;
    bg.graph = nullptr;
    cudaGraph_t graph = nullptr;
    EG_CUDA(cudaGraphCreate(&graph, 0));
    bg.graph = graph;
    const uint32_t blocks = (uint32_t)ctx->sm_count * 8;
    // start kernel
    EG_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_bfsg_start<<<blocks, 256, 0, ctx->stream>>>(st, deg, level, parent, visited, bm0, nw, q0, cnt,
                                                  in_adj ? bp<uint32_t>(g->first_in) + n : nullptr);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (ce != cudaSuccess) return eg_fail(EG_ECUDA, "BFS graph capture: %s", cudaGetErrorString(ce));
    cudaGraphNode_t start_node;
    size_t nnodes = 1;
    EG_CUDA(cudaGraphGetNodes(graph, &start_node, &nnodes));
    // while node
    cudaGraphConditionalHandle handle;
    EG_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    EG_CUDA(cudaGraphAddNode(&wnode, graph, &start_node, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    EG_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const uint32_t *iptr = in_adj ? bp<uint32_t>(in_adj->ptr) : nullptr;
    const uint32_t *icol = in_adj ? bp<uint32_t>(in_adj->col) : nullptr;
    k_bfsg_prep<<<blocks, 256, 0, ctx->stream>>>(st, bm0, bm1, q0, q1, nw);
    k_bfsg_push<<<blocks, 256, 0, ctx->stream>>>(st, bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), deg, q0, q1,
                                                bm0, bm1, visited, level, parent, cnt, big);
    k_big_offsets<<<1, 1024, 0, ctx->stream>>>(big, &cnt->nbig, 1u, bp<uint32_t>(g->csr.ptr), EG_BFS_CHUNK, bigoff);
    k_bfsg_push_big<<<blocks, 256, 0, ctx->stream>>>(st, bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), deg, big,
                                                    bigoff, q0, q1, bm0, bm1, visited, level, parent, cnt);
    if (iptr)
        k_bfsg_pull<<<blocks, 256, 0, ctx->stream>>>(st, iptr, icol, bp<uint32_t>(g->first_in), deg, bm0, bm1, visited,
                                                     level, parent, cnt);
    k_bfsg_end<<<1, 1, 0, ctx->stream>>>(st, cnt, handle);
    ce = cudaStreamEndCapture(ctx->stream, &body);
    if (ce != cudaSuccess) return eg_fail(EG_ECUDA, "BFS level capture: %s", cudaGetErrorString(ce));
    cudaGraphExec_t exec = nullptr;
    EG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    bg.exec = exec;
    for (int i = 0; i < 8; i++) bg.key[i] = key[i];
    return EG_OK;
}

static int bfs_check(eg_graph *g, const eg_bfs_opts *opts, eg_bfs_opts &o) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (!(g->built & EG_LAYOUT_CSR)) return eg_fail(EG_ENOTBUILT, "BFS needs the CSR");
    if (opts) o = *opts;
    else eg_bfs_opts_default(&o);
    if (o.direction < EG_BFS_AUTO || o.direction > EG_BFS_PULL_ONLY) return eg_fail(EG_EINVAL, "bad direction");
    return EG_OK;
}

// One BFS from `root` into the device arrays of output slot `slot` (g->level
// / g->parent, or g->level_s / g->parent_s), on the context stream.  When
// level_out / parent_out are given, the copies to them are queued before the
// final wait; returns once the traversal (and those copies) are done.
static int bfs_core(eg_graph *g, uint32_t root, const eg_bfs_opts &o, int slot, bool want_parent, int32_t *level_out,
                    int32_t *parent_out, eg_bfs_stats *stats) {
    if (root >= g->n) return eg_fail(EG_EINVAL, "root %u >= n %u", root, g->n);
    const bool undirected = (g->flags & EG_UNDIRECTED) != 0;
    // in-lists: the CSC when built (sorted by source id, so RMAT hubs come first
    // and bottom-up scans stop early); an undirected CSR is its own transpose
    eg_adj *in_adj = (g->built & EG_LAYOUT_CSC) ? &g->csc : (undirected ? &g->csr : nullptr);
    if (!in_adj && o.direction != EG_BFS_PUSH_ONLY)
        return eg_fail(EG_ENOTBUILT, "bottom-up BFS on a directed graph needs the CSC");
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    const uint32_t nw = (n + 31) >> 5;
    if (in_adj && g->first_in_src != in_adj->col.p) {  // once per graph and in-list array
        // first_in[0 .. n), then the bit per vertex without in-neighbours
        EG_TRY(eg_buf_ensure(ctx, g->first_in, ((uint64_t)n + nw) * 4));
        k_first_in<<<(uint32_t)ctx->sm_count * 8, 256, 0, ctx->stream>>>(
            bp<uint32_t>(in_adj->ptr), bp<uint32_t>(in_adj->col), bp<uint32_t>(g->out_deg), n, bp<uint32_t>(g->first_in));
        EG_LAUNCHED(ctx);
        k_no_in_bits<<<blocks_for(ctx, (uint64_t)nw * 32), 256, 0, ctx->stream>>>(bp<uint32_t>(g->first_in), n, nw,
                                                                                  bp<uint32_t>(g->first_in) + n);
        EG_LAUNCHED(ctx);
        g->first_in_src = in_adj->col.p;
    }
    eg_buf &lbuf = slot ? g->level_s[slot - 1] : g->level, &pbuf = slot ? g->parent_s[slot - 1] : g->parent;
    EG_TRY(eg_buf_ensure(ctx, lbuf, (uint64_t)n * 4));
    if (want_parent) EG_TRY(eg_buf_ensure(ctx, pbuf, (uint64_t)n * 4));
    // work: visited | bm0 | bm1 | queue0 | queue1 | big list | counters | graph state
    // (the counters are followed by a BfsSmallOut: 24 words leave room for both)
    const uint64_t off_bm0 = (uint64_t)nw, off_bm1 = 2ull * nw, off_q0 = 3ull * nw, off_q1 = off_q0 + n,
                   off_big = off_q1 + n, off_bigoff = off_big + n, off_cnt = (off_bigoff + n + 1 + 7) & ~7ull,
                   off_st = off_cnt + 24;
    static_assert(sizeof(BfsCounters) + sizeof(BfsSmallOut) <= 24 * 4, "counter area");
    EG_TRY(eg_buf_ensure(ctx, g->bfs_work, (off_st + 64) * 4));
    uint32_t *wk = bp<uint32_t>(g->bfs_work);
    uint32_t *visited = wk, *bm[2] = {wk + off_bm0, wk + off_bm1}, *q[2] = {wk + off_q0, wk + off_q1};
    uint32_t *big = wk + off_big, *bigoff = wk + off_bigoff;
    BfsCounters *cnt = reinterpret_cast<BfsCounters *>(wk + off_cnt);
    BfsGState *gst = reinterpret_cast<BfsGState *>(wk + off_st);
    int32_t *level = bp<int32_t>(lbuf);
    int32_t *parent = want_parent ? bp<int32_t>(pbuf) : nullptr;
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    const double divisor = o.switch_divisor < 0 ? g->bfs_divisor : o.switch_divisor;
    const double threshold = divisor > 0 ? (double)g->m / divisor : 0.0;

    const bool host_loop = o.host_loop < 0 ? g->bfs_host_loop != 0 : o.host_loop != 0;
    if (!host_loop) {
        eg_bfs_graph &bg = g->bfsg[slot * 2 + (want_parent ? 1 : 0)];
        const void *key[8] = {wk, level, parent, (const void *)((uintptr_t)deg ^ ((uintptr_t)g->first_in.p << 1)),
                              g->csr.col.p, in_adj ? in_adj->col.p : nullptr, g->csr.ptr.p,
                              (const void *)(uintptr_t)ctx->stream};
        bool fresh = bg.exec != nullptr;
        for (int i = 0; i < 8 && fresh; i++) fresh = bg.key[i] == key[i];
        if (!fresh)
            EG_TRY(bfs_graph_build(g, bg, key, gst, deg, level, parent, visited, bm[0], bm[1], q[0], q[1], big, bigoff,
                                   cnt, in_adj));
        BfsGState *h = (BfsGState *)ctx->h_pinned;
        memset(h, 0, sizeof(BfsGState));
        h->root = root;
        h->dirmode = (uint32_t)o.direction;
        h->n = n;
        h->threshold = threshold;
        EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
        EG_CUDA(cudaMemcpyAsync(gst, h, sizeof(BfsGState), cudaMemcpyHostToDevice, ctx->stream));
        EG_CUDA(cudaGraphLaunch(bg.exec, ctx->stream));
        ctx->launches += 1;
        EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
        if (level_out) EG_CUDA(cudaMemcpyAsync(level_out, level, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (parent_out)
            EG_CUDA(cudaMemcpyAsync(parent_out, parent, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        BfsGState *hs = h + 1;
        EG_TRY(eg_readback(ctx, hs, gst, sizeof(BfsGState), ctx->stream));
        EG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (hs->err) return eg_fail(EG_ETIMEOUT, "BFS did not terminate");
        if (stats) {
            stats->levels = (int)hs->levels;
            stats->reached = (uint32_t)hs->reached;
            stats->edges_traversed = hs->traversed;
            stats->pull_levels = (int)hs->pull_levels;
            EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
        }
        return EG_OK;
    }

    // host-driven level loop
    BfsCounters *h = (BfsCounters *)ctx->h_pinned;
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    k_bfs_init<<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(n, level, parent, visited, bm[0], nw, root, q[0], deg, cnt,
                                                            in_adj ? bp<uint32_t>(g->first_in) + n : nullptr);
    EG_LAUNCHED(ctx);
    uint32_t count = 1, qlen = 1;
    unsigned long long fdeg = 0;
    int cur = 0;
    bool have_queue = true;  // q[cur] lists the frontier
    int32_t lvl = 1;
    int pull_levels = 0;
    uint64_t reached = 1, traversed = 0;
    bool bm_valid = true;  // bm[cur] holds the frontier (not so after k_bfs_small)
    BfsSmallOut *hsm = reinterpret_cast<BfsSmallOut *>(h + 1);
    BfsSmallOut *dsm = reinterpret_cast<BfsSmallOut *>(cnt + 1);
    if (o.direction != EG_BFS_PULL_ONLY) {
        // the root's level goes straight to the small-level kernel, which
        // finds the root's degree itself (no round trip after k_bfs_init)
        k_bfs_small<<<1, 1024, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), deg, visited,
                                                 level, parent, q[0], 1u, EG_FDEG_UNKNOWN, 1, threshold,
                                                 o.direction == EG_BFS_AUTO ? 1 : 0, dsm, cnt);
        EG_LAUNCHED(ctx);
        EG_TRY(eg_readback_wait(ctx, hsm, dsm, sizeof(BfsSmallOut), ctx->stream));
        count = qlen = hsm->qlen;
        fdeg = hsm->fdeg;
        reached += hsm->reached;
        traversed = hsm->fdeg_in + hsm->traversed;
        lvl = hsm->lvl;
        bm_valid = hsm->levels == 0;  // else bm[0] still holds only the root
    } else {
        EG_TRY(eg_readback_wait(ctx, h, cnt, sizeof(BfsCounters), ctx->stream, true));  // and clears them
        fdeg = h->next_deg;
        traversed = fdeg;
    }
    while (count > 0) {
        bool pull;
        if (o.direction == EG_BFS_PUSH_ONLY) pull = false;
        else if (o.direction == EG_BFS_PULL_ONLY) pull = true;
        else pull = (double)count + (double)fdeg > threshold;
        if (!pull && have_queue && qlen <= EG_SMALL_Q && fdeg <= EG_SMALL_Q) {
            // small levels back to back in one CTA
            k_bfs_small<<<1, 1024, 0, ctx->stream>>>(
                bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), deg, visited, level, parent, q[cur], qlen, fdeg,
                lvl, threshold, o.direction == EG_BFS_AUTO ? 1 : 0, dsm, cnt);
            EG_LAUNCHED(ctx);
            EG_TRY(eg_readback_wait(ctx, hsm, dsm, sizeof(BfsSmallOut), ctx->stream));
            count = qlen = hsm->qlen;
            fdeg = hsm->fdeg;
            reached += hsm->reached;
            traversed += hsm->traversed;
            lvl = hsm->lvl;
            bm_valid = false;
            if (lvl > (int32_t)n + 1) return eg_fail(EG_ETIMEOUT, "BFS did not terminate");
            continue;  // the frontier in q[cur] left the small range, needs pull, or is empty
        }
        const int nxt = cur ^ 1;
        if (pull && !bm_valid) {  // the frontier is a queue only: set its bits
            EG_TRY(eg_zero(ctx, bm[cur], (uint64_t)nw * 4, ctx->stream));
            k_queue_bm<<<blocks_for(ctx, qlen), 256, 0, ctx->stream>>>(q[cur], qlen, bm[cur]);
            EG_LAUNCHED(ctx);
        }
        bm_valid = true;
        if (pull) {
            k_bfs_pull<<<blocks_for(ctx, (uint64_t)nw * 32), 256, 0, ctx->stream>>>(
                bp<uint32_t>(in_adj->ptr), bp<uint32_t>(in_adj->col), bp<uint32_t>(g->first_in), deg, n, bm[cur],
                visited, bm[nxt], level, parent, lvl + 1, cnt);
            EG_LAUNCHED(ctx);
            pull_levels++;
            have_queue = false;
        } else {
            if (!have_queue) {  // the queue from the bitmap; its length is the frontier count
                k_bm_queue<<<blocks_for(ctx, (uint64_t)nw * 32), 256, 0, ctx->stream>>>(bm[cur], n, q[cur],
                                                                                       &cnt->qbuilt, 0);
                EG_LAUNCHED(ctx);
                qlen = count;
            }
            EG_TRY(eg_zero(ctx, bm[nxt], (uint64_t)nw * 4, ctx->stream));
            // A frontier with fewer vertices than a full grid has warps (the
            // first levels: a root and its hubs' neighbours) would leave most
            // SMs idle behind the warps walking long lists: there every list
            // over EG_BFS_SMALL_BIG edges goes to the chunked kernel, with
            // chunks sized to spread the level's edges over the grid.
            const uint32_t grid_ctas = (uint32_t)ctx->sm_count * 8;
            // a level over many edges leaves the next frontier as a bitmap
            // only; a push level after it rebuilds the queue (k_bm_queue)
            const bool make_queue = fdeg <= EG_BFS_QUEUE_EDGES;
            uint32_t big_deg = EG_BFS_WARP_EDGES, chunk = EG_BFS_CHUNK;
            if ((uint64_t)qlen < (uint64_t)grid_ctas * 8) {
                big_deg = EG_BFS_SMALL_BIG;
                const uint64_t per = (fdeg / grid_ctas + 255) & ~255ull;
                chunk = (uint32_t)(per < 256 ? 256 : (per > EG_BFS_CHUNK ? EG_BFS_CHUNK : per));
            }
            k_bfs_push<<<blocks_for(ctx, qlen), 256, 0, ctx->stream>>>(
                bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), deg, q[cur], qlen, visited, bm[nxt],
                make_queue ? q[nxt] : nullptr, level, parent, lvl + 1, cnt, big, big_deg);
            EG_LAUNCHED(ctx);
            if (fdeg > big_deg) {  // a frontier vertex may exceed the threshold
                k_big_offsets<<<1, 1024, 0, ctx->stream>>>(big, &cnt->nbig, 1u, bp<uint32_t>(g->csr.ptr), chunk,
                                                           bigoff);
                EG_LAUNCHED(ctx);
                k_bfs_push_big<<<grid_ctas, 256, 0, ctx->stream>>>(
                    bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), deg, big, bigoff, visited, bm[nxt],
                    make_queue ? q[nxt] : nullptr, level, parent, lvl + 1, cnt, chunk);
                EG_LAUNCHED(ctx);
            }
            have_queue = make_queue;
        }
        EG_TRY(eg_readback_wait(ctx, h, cnt, sizeof(BfsCounters), ctx->stream, true));  // and clears them
        count = h->next_count;
        fdeg = h->next_deg;
        qlen = h->qsize;
        reached += count;
        traversed += fdeg;
        cur = nxt;
        lvl++;
        if (lvl > (int32_t)n + 1) return eg_fail(EG_ETIMEOUT, "BFS did not terminate");
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (level_out) EG_CUDA(cudaMemcpyAsync(level_out, level, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (parent_out) EG_CUDA(cudaMemcpyAsync(parent_out, parent, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->levels = lvl - 1;
        stats->reached = (uint32_t)reached;
        stats->edges_traversed = traversed;
        stats->pull_levels = pull_levels;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}

extern "C" int eg_bfs(eg_graph *g, uint32_t root, const eg_bfs_opts *opts, int32_t *level_out, int32_t *parent_out,
                      eg_bfs_stats *stats) {
    eg_bfs_opts o;
    EG_TRY(bfs_check(g, opts, o));
    EG_CUDA(cudaSetDevice(g->ctx->device));
    return bfs_core(g, root, o, 0, parent_out != nullptr || o.device_parents, level_out, parent_out, stats);
}

// BFS from each root in turn; root i's levels (and parents) go to
// level_out + i * n (parent_out + i * n).  Root i is traversed into output
// slot i % EG_OUT_SLOTS and copied out on the copy stream while the next
// roots are traversed into the other slots; a slot is rewritten only after
// its previous copy-out.
extern "C" int eg_bfs_batch(eg_graph *g, const uint32_t *roots, uint32_t k, const eg_bfs_opts *opts,
                            int32_t *level_out, int32_t *parent_out, eg_bfs_stats *stats) {
    eg_bfs_opts o;
    EG_TRY(bfs_check(g, opts, o));
    if (!roots && k) return eg_fail(EG_EINVAL, "NULL roots");
    for (uint32_t i = 0; i < k; i++)
        if (roots[i] >= g->n) return eg_fail(EG_EINVAL, "root %u >= n %u", roots[i], g->n);
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint64_t n = g->n;
    const bool want_parent = parent_out != nullptr || o.device_parents;
    int rc = EG_OK;
    for (uint32_t i = 0; i < k && rc == EG_OK; i++) {
        const int slot = (int)(i % EG_OUT_SLOTS);
        if (i >= EG_OUT_SLOTS) EG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_out[EG_OUT_SLOTS + slot], 0));
        rc = bfs_core(g, roots[i], o, slot, want_parent, nullptr, nullptr, stats ? stats + i : nullptr);
        if (rc != EG_OK) break;
        if (level_out || parent_out) {
            const int32_t *level = bp<int32_t>(slot ? g->level_s[slot - 1] : g->level);
            const int32_t *parent = want_parent ? bp<int32_t>(slot ? g->parent_s[slot - 1] : g->parent) : nullptr;
            EG_CUDA(cudaEventRecord(ctx->ev_out[slot], ctx->stream));
            EG_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_out[slot], 0));
            if (level_out)
                EG_CUDA(cudaMemcpyAsync(level_out + i * n, level, n * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
            if (parent_out)
                EG_CUDA(cudaMemcpyAsync(parent_out + i * n, parent, n * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
            EG_CUDA(cudaEventRecord(ctx->ev_out[EG_OUT_SLOTS + slot], ctx->copy_stream));
        }
    }
    const cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
    if (rc == EG_OK && e != cudaSuccess) return eg_fail(EG_ECUDA, "BFS batch copies: %s", cudaGetErrorString(e));
    return rc;
}

// ============================================================== multi-source
// Bit-sliced BFS: bit s of seen[v] / front[v] belongs to source s (k <= 64).
namespace {
struct MsCounters {
    unsigned long long deg;   // sum of out-degrees of vertices with a nonzero new word
    unsigned long long tdeg;  // sum over new (vertex, source) pairs of the vertex's out-degree
    unsigned long long disc;  // new (vertex, source) pairs
    uint32_t count;           // vertices with a nonzero new word
    uint32_t nbig;            // frontier vertices deferred to k_ms_push_big
};

__global__ void k_ms_init(uint32_t n, unsigned long long *seen, unsigned long long *front) {
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        seen[v] = 0ull;
        front[v] = 0ull;
    }
}

// Device state of the multi-source level loop (one CUDA graph, see
// msbfs_graph_build): the frontier's size and out-degree sum, the direction
// chosen for the level, and the totals for the stats.
struct MsGState {
    uint32_t count;  // vertices in the frontier
    int32_t lvl;     // level of the frontier (roots: 1)
    int pull;        // this level runs bottom-up
    int pull_levels;
    unsigned long long fdeg;       // out-degree sum of the frontier's vertices
    unsigned long long reached;    // (vertex, source) pairs reached
    unsigned long long traversed;  // sum over those pairs of the vertex's out-degree
    unsigned long long m;          // adjacency entries (switch rule)
    uint32_t n;
    uint32_t pad;
};

// Roots: seen/front bits, level 1, and the first frontier (distinct roots)
// with its statistics.  One block of 64 threads.
__global__ void k_ms_roots(const uint32_t *roots, int k, uint32_t n, unsigned long long *seen, unsigned long long *front,
                           int32_t *levels, const uint32_t *__restrict__ deg, uint32_t *queue, MsGState *st,
                           unsigned long long m) {
    __shared__ unsigned int s_count;
    __shared__ unsigned long long s_fdeg, s_rdeg;
    const int s = threadIdx.x;
    if (s == 0) {
        s_count = 0;
        s_fdeg = 0;
        s_rdeg = 0;
    }
    __syncthreads();
    if (s < k) {
        const uint32_t r = roots[s];
        atomicOr(seen + r, 1ull << s);
        const unsigned long long was = atomicOr(front + r, 1ull << s);
        if (levels) levels[(uint64_t)s * n + r] = 1;
        const unsigned long long d = deg[r];
        atomicAdd(&s_rdeg, d);
        if (!was) {  // the first source at this vertex lists it
            queue[atomicAdd(&s_count, 1u)] = r;
            atomicAdd(&s_fdeg, d);
        }
    }
    __syncthreads();
    if (s == 0) {
        st->count = s_count;
        st->lvl = 1;
        st->pull = 0;
        st->pull_levels = 0;
        st->fdeg = s_fdeg;
        st->reached = (unsigned long long)k;
        st->traversed = s_rdeg;
        st->m = m;
        st->n = n;
    }
}

// Level start: the reference's switch rule (bfs_simple.c:191-197) on the
// frontier's size and out-degrees, and cleared level counters.
__global__ void k_msg_prep(MsGState *st, MsCounters *cnt) {
    st->pull = (double)st->count + (double)st->fdeg > (double)st->m / 20.0;
    cnt->deg = 0;
    cnt->tdeg = 0;
    cnt->disc = 0;
    cnt->count = 0;
    cnt->nbig = 0;
}

// Pull: a vertex ORs the frontier words of its in-neighbours, stopping early
// once every source it still lacks has been found.
// Push: 32 vertices with a nonzero frontier word per warp (eg_warp_lists); lists with more
// than EG_BFS_WARP_EDGES out-edges go to a side list for k_ms_push_big.
__global__ void __launch_bounds__(256) k_ms_push(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                 const uint32_t *__restrict__ queue, const MsGState *st,
                                                 const unsigned long long *__restrict__ seen,
                                                 const unsigned long long *__restrict__ front,
                                                 unsigned long long *__restrict__ next, uint32_t *big,
                                                 MsCounters *cnt) {
    if (st->pull) return;
    const uint32_t qlen = st->count;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    // 32 frontier vertices per warp, their lists walked together (eg_warp_lists)
    for (uint32_t q0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; q0 < qlen; q0 += warps * 32) {
        const uint32_t qi = q0 + lane;
        uint32_t u = 0, b = 0, d = 0;
        unsigned long long f = 0ull;
        if (qi < qlen) {
            u = queue[qi];
            b = ptr[u];
            d = ptr[u + 1] - b;
            if (d > EG_BFS_WARP_EDGES) {
                big[atomicAdd(&cnt->nbig, 1u)] = u;
                d = 0;
            } else {
                f = front[u];
            }
        }
        eg_warp_lists(u, b, d, [&](bool valid, uint32_t lo, uint32_t, uint32_t p) {
            const unsigned long long of = __shfl_sync(EG_FULL_MASK, f, lo);
            if (valid) {
                const uint32_t v = col[p];
                const unsigned long long add = of & ~__ldcg(seen + v);
                if (add && (__ldcg(next + v) & add) != add) atomicOr(next + v, add);
            }
        });
    }
}

// The deferred high-degree frontier vertices: every thread of the grid
// strides over each one's out-list in turn.
__global__ void __launch_bounds__(256) k_ms_push_big(const uint32_t *__restrict__ ptr,
                                                     const uint32_t *__restrict__ col, const uint32_t *big,
                                                     const uint32_t *__restrict__ bigoff,
                                                     const unsigned long long *__restrict__ seen,
                                                     const unsigned long long *__restrict__ front,
                                                     unsigned long long *__restrict__ next, const MsCounters *cnt) {
    const uint32_t nbig = *(volatile const uint32_t *)&cnt->nbig;
    if (!nbig) return;
    const uint32_t total = bigoff[nbig];
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t u = big[i];
        const unsigned long long f = front[u];
        const uint32_t b = ptr[u] + (c - bigoff[i]) * EG_BFS_CHUNK, e = min(ptr[u + 1], b + EG_BFS_CHUNK);
        for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) {
            const uint32_t v = col[p];
            const unsigned long long add = f & ~__ldcg(seen + v);
            if (add && (__ldcg(next + v) & add) != add) atomicOr(next + v, add);
        }
    }
}

// Level end: the new frontier's counters into the loop state; the while node
// repeats the level body while the frontier is non-empty (and at most n + 1
// levels, a bound the loop can never need).
__global__ void k_msg_end(MsGState *st, const MsCounters *cnt, cudaGraphConditionalHandle handle) {
    st->count = cnt->count;
    st->fdeg = cnt->deg;
    st->reached += cnt->disc;
    st->traversed += cnt->tdeg;
    st->pull_levels += st->pull;
    st->lvl += 1;
    cudaGraphSetConditional(handle, (cnt->count > 0 && (uint32_t)st->lvl <= st->n + 1) ? 1u : 0u);
}

// Folds the new words into seen, records levels, makes them the frontier and
// lists the frontier vertices for a following push step.
__global__ void k_ms_fold(uint32_t n, int k, unsigned long long *seen, unsigned long long *front,
                          unsigned long long *next, int clear_next, int32_t *levels, const MsGState *st,
                          const uint32_t *__restrict__ deg, uint32_t *queue, MsCounters *cnt) {
    const int32_t lvl = st->lvl + 1;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt = eg_lanemask_lt();
    uint32_t stride = gridDim.x * blockDim.x;
    // uniform trip count per warp for the ballots
    for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < n; v0 += stride) {
        const uint32_t v = v0 + lane;
        unsigned long long x = 0ull;
        if (v < n) {
            x = next[v] & ~seen[v];
            if (clear_next) next[v] = 0ull;
            front[v] = x;
            if (x) {
                seen[v] |= x;
                if (levels) {
                    unsigned long long y = x;
                    while (y) {
                        int s = __ffsll((long long)y) - 1;
                        y &= y - 1;
                        levels[(uint64_t)s * n + v] = lvl;
                    }
                }
            }
        }
        const uint32_t ball = __ballot_sync(EG_FULL_MASK, x != 0ull);
        if (ball) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&cnt->count, __popc(ball));
            base = __shfl_sync(EG_FULL_MASK, base, 0);
            unsigned long long d = x ? (unsigned long long)deg[v] : 0ull;
            unsigned long long pc = (unsigned long long)__popcll((long long)x);
            unsigned long long td = d * pc;
            if (x) queue[base + __popc(ball & lt)] = v;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                d += __shfl_down_sync(EG_FULL_MASK, d, o);
                td += __shfl_down_sync(EG_FULL_MASK, td, o);
                pc += __shfl_down_sync(EG_FULL_MASK, pc, o);
            }
            if (lane == 0) {
                atomicAdd(&cnt->deg, d);
                atomicAdd(&cnt->tdeg, td);
                atomicAdd(&cnt->disc, pc);
            }
        }
    }
}
}  // namespace

// The level loop of eg_bfs_multi as one CUDA graph: a while node whose body
// is prep (direction), push (+ hubs in chunks) or the two-part pull, fold,
// and end (counters into the state, loop condition).  Valid while the
// buffers and k it was captured with (key) stay the same.
static int msbfs_graph_build(eg_graph *g, const void *const key[8], const eg_adj *in_adj, int k,
                             unsigned long long all, unsigned long long *seen, unsigned long long *front,
                             unsigned long long *next, uint32_t *queue, uint32_t *big, uint32_t *bigoff, int32_t *levels,
                             MsGState *st, MsCounters *cnt) {
    eg_ctx *ctx = g->ctx;
    eg_bfs_graph &bg = g->msg;
    const uint32_t n = g->n;
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    if (bg.exec) cudaGraphExecDestroy(bg.exec);
    if (bg.graph) cudaGraphDestroy(bg.graph);
    bg.exec = nullptr;
    bg.graph = nullptr;
    cudaGraph_t graph = nullptr;
    EG_CUDA(cudaGraphCreate(&graph, 0));
    bg.graph = graph;
    cudaGraphConditionalHandle handle;
    EG_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    EG_CUDA(cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const uint32_t blocks = (uint32_t)ctx->sm_count * 8;
    EG_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_msg_prep<<<1, 1, 0, ctx->stream>>>(st, cnt);
    k_ms_push<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), queue, st, seen,
                                               front, next, big, cnt);
    k_big_offsets<<<1, 1024, 0, ctx->stream>>>(big, &cnt->nbig, 1u, bp<uint32_t>(g->csr.ptr), EG_BFS_CHUNK, bigoff);
    k_ms_push_big<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), big, bigoff,
                                                   seen, front, next, cnt);
    // the heavy list reuses the push side list (idle in a pull level)
    k_msp_light<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(in_adj->ptr), bp<uint32_t>(in_adj->col), n, all, seen,
                                                 front, next, big, &cnt->nbig, &st->pull);
    k_msp_heavy<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(in_adj->ptr), bp<uint32_t>(in_adj->col), all, seen, front,
                                                 next, big, &cnt->nbig, &st->pull);
    k_ms_fold<<<blocks, 256, 0, ctx->stream>>>(n, k, seen, front, next, 1, levels, st, deg, queue, cnt);
    k_msg_end<<<1, 1, 0, ctx->stream>>>(st, cnt, handle);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &body);
    if (ce != cudaSuccess) return eg_fail(EG_ECUDA, "multi-source BFS capture: %s", cudaGetErrorString(ce));
    cudaGraphExec_t exec = nullptr;
    EG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    bg.exec = exec;
    for (int i = 0; i < 8; i++) bg.key[i] = key[i];
    return EG_OK;
}

extern "C" int eg_bfs_multi(eg_graph *g, const uint32_t *roots, int k, int32_t *levels_out, eg_bfs_stats *stats) {
    if (!g || !roots) return eg_fail(EG_EINVAL, "NULL argument");
    if (k < 1 || k > 64) return eg_fail(EG_EINVAL, "k=%d sources: bit-sliced BFS takes 1..64", k);
    if (!(g->built & EG_LAYOUT_CSR)) return eg_fail(EG_ENOTBUILT, "BFS needs the CSR");
    const bool undirected = (g->flags & EG_UNDIRECTED) != 0;
    // in-lists: the CSC when built (sorted by source id, so RMAT hubs come first
    // and bottom-up scans stop early); an undirected CSR is its own transpose
    eg_adj *in_adj = (g->built & EG_LAYOUT_CSC) ? &g->csc : (undirected ? &g->csr : nullptr);
    if (!in_adj) return eg_fail(EG_ENOTBUILT, "multi-source BFS on a directed graph needs the CSC");
    for (int s = 0; s < k; s++)
        if (roots[s] >= g->n) return eg_fail(EG_EINVAL, "root %u >= n", roots[s]);
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    // work: seen | front | next (u64 each) | queue (u32) | big list (u32) | roots | counters | state |
    //       big chunk offsets
    const uint64_t bytes = 3ull * n * 8 + 2ull * n * 4 + 64 * 4 + 64 + 64 + ((uint64_t)n + 1) * 4;
    EG_TRY(eg_buf_ensure(ctx, g->msbfs_work, bytes));
    unsigned long long *seen = bp<unsigned long long>(g->msbfs_work);
    unsigned long long *front = seen + n, *next = seen + 2ull * n;
    uint32_t *queue = reinterpret_cast<uint32_t *>(seen + 3ull * n);
    uint32_t *big = queue + n;
    uint32_t *d_roots = big + n;
    MsCounters *cnt = reinterpret_cast<MsCounters *>(d_roots + 64);
    MsGState *st = reinterpret_cast<MsGState *>(d_roots + 64 + 16);
    uint32_t *bigoff = d_roots + 64 + 32;
    int32_t *levels = nullptr;
    if (levels_out) {
        EG_TRY(eg_buf_ensure(ctx, g->level, (uint64_t)k * n * 4));
        levels = bp<int32_t>(g->level);
    }
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    const unsigned long long all = k == 64 ? ~0ull : ((1ull << k) - 1ull);
    const void *key[8] = {g->msbfs_work.p, levels, g->csr.col.p, in_adj->col.p, (const void *)(uintptr_t)k, g->csr.ptr.p,
                          in_adj->ptr.p, g->out_deg.p};
    bool same = g->msg.exec != nullptr;
    for (int i = 0; i < 8 && same; i++) same = g->msg.key[i] == key[i];
    if (!same)
        EG_TRY(msbfs_graph_build(g, key, in_adj, k, all, seen, front, next, queue, big, bigoff, levels, st, cnt));
    EG_CUDA(cudaMemcpyAsync(d_roots, roots, (uint64_t)k * 4, cudaMemcpyHostToDevice, ctx->stream));
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    if (levels) EG_CUDA(cudaMemsetAsync(levels, 0, (uint64_t)k * n * 4, ctx->stream));
    k_ms_init<<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(n, seen, front);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemsetAsync(next, 0, (uint64_t)n * 8, ctx->stream));
    k_ms_roots<<<1, 64, 0, ctx->stream>>>(d_roots, k, n, seen, front, levels, deg, queue, st, g->m);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaGraphLaunch(g->msg.exec, ctx->stream));
    ctx->launches++;
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    MsGState *h = (MsGState *)ctx->h_pinned;
    EG_CUDA(cudaMemcpyAsync(h, st, sizeof(MsGState), cudaMemcpyDeviceToHost, ctx->stream));
    if (levels_out) EG_CUDA(cudaMemcpyAsync(levels_out, levels, (uint64_t)k * n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if ((uint32_t)h->lvl > n + 1) return eg_fail(EG_ETIMEOUT, "multi-source BFS did not terminate");
    if (stats) {
        stats->levels = h->lvl - 1;
        stats->reached = (uint32_t)(h->reached > 0xffffffffull ? 0xffffffffull : h->reached);
        stats->edges_traversed = h->traversed;
        stats->pull_levels = h->pull_levels;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}

int eg_bfs_tune(eg_graph *g, float *ms_graph, float *ms_host, int *host_loop, double *divisor) {
    // per-root times vary several-fold (an early switch to pull costs a few
    // roots a lot), so the mean is taken over 48 sampled roots
    static const double kDiv[5] = {20.0, 40.0, 80.0, 160.0, 320.0};
    constexpr int R = 48;
    uint32_t roots[R];
    EG_TRY(eg_sample_roots(g, R, 12345, roots));
    float best[2] = {0.f, 0.f};
    double best_div[2] = {20.0, 20.0};
    for (int form = 0; form < 2; form++) {
        for (int d = 0; d < 5; d++) {
            eg_bfs_opts o;
            eg_bfs_opts_default(&o);
            o.host_loop = form;
            o.switch_divisor = kDiv[d];
            o.device_parents = 1;
            eg_bfs_stats st;
            EG_TRY(eg_bfs(g, roots[0], &o, nullptr, nullptr, &st));  // warm-up (graph capture, buffers)
            float t = 0.f;
            for (int r = 0; r < R; r++) {
                EG_TRY(eg_bfs(g, roots[r], &o, nullptr, nullptr, &st));
                t += st.ms / (float)R;
            }
            if (d == 0 || t < best[form]) {
                best[form] = t;
                best_div[form] = kDiv[d];
            }
        }
    }
    g->bfs_host_loop = best[1] < best[0] ? 1 : 0;
    g->bfs_divisor = best_div[g->bfs_host_loop];
    *ms_graph = best[0];
    *ms_host = best[1];
    *host_loop = g->bfs_host_loop;
    *divisor = g->bfs_divisor;
    return EG_OK;
}
