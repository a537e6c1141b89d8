// Single- and multi-source SSSP: frontier Bellman-Ford with atomicMin.
//
// Replaces sssp_pushpull.c: the push relax (sssp_algo, 39-56, which the
// reference runs with unit weights) and the weighted pull relax
// (sssp_algo_pull, 69-98) iterated to a fixed point (iterator, 127-190).  The
// fixed point is the exact shortest-path distance, which is what both this
// code and the reference's pull-only run (-a 1 -r) produce.  dist[root] = 0,
// unreached = UINT32_MAX-1 (sssp_pushpull.c:8).
//
// Weights are computed from the edge's endpoints, like the reference's
// CREATE_WEIGHT path (init_all.c:661-686): no weight array is stored or read.
#include <stdlib.h>
#include <string.h>

#include "eg_internal.cuh"
#include "eg_bigwork.cuh"
#include "eg_frontier.cuh"
#include "eg_mrelax.cuh"

namespace {

using WRule = eg_wrule;

struct SsspCounters {
    unsigned long long relax;  // entries scanned
    uint32_t qsize;
    uint32_t nbig;             // frontier vertices deferred to the grid-wide kernel
    unsigned long long reached;
    uint32_t grab, grab_big;   // work units handed out (batched kernels), zeroed per round
};

// Frontier vertices with more out-edges than this are relaxed by the whole
// grid instead of one warp (RMAT hubs have 10^5..10^6 out-edges).
#ifndef EG_SSSP_BIG_DEG
#define EG_SSSP_BIG_DEG 2048u
#endif

__global__ void k_sssp_init(uint32_t n, uint32_t *dist, uint32_t root, uint32_t *queue, SsspCounters *cnt,
                            uint32_t inf) {
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) dist[v] = v == root ? 0u : inf;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        queue[0] = root;
        cnt->qsize = 1;
        cnt->relax = 0;
    }
}

// A relaxation that lowers dist[v] marks v in the next frontier bitmap; the
// next queue is built from the bitmap afterwards (k_bm_queue), so no warp
// waits on a shared queue counter.  The atomicMin's old value is not
// awaited: when another relaxation got below nd first, that one marks v, so
// the frontier is the same set either way.
__device__ __forceinline__ void sssp_relax(uint32_t u, uint32_t du, uint32_t v, uint32_t wt, const WRule &w,
                                           uint32_t *dist, uint32_t *next_bm) {
    if (v == u) return;  // self-loops skipped (sssp_pushpull.c:80)
    const uint32_t nd = w.add(du, wt);
    if (nd >= __ldcg(dist + v)) return;
    atomicMin(dist + v, nd);
    atomicOr(next_bm + (v >> 5), 1u << (v & 31));
}

// Relaxes the deferred high-degree frontier vertices: chunks of
// EG_SSSP_CHUNK edges shared out over the grid (one CTA per chunk).
#define EG_SSSP_CHUNK 2048u
__global__ void __launch_bounds__(256) k_sssp_push_big(const uint32_t *__restrict__ ptr,
                                                       const uint32_t *__restrict__ col,
                                                       const uint32_t *__restrict__ wts, const uint32_t *big,
                                                       const uint32_t *__restrict__ bigoff, uint32_t *dist,
                                                       uint32_t *next_bm, WRule w, SsspCounters *cnt) {
    const uint32_t nbig = *(volatile uint32_t *)&cnt->nbig;
    if (!nbig) return;
    const uint32_t total = bigoff[nbig];
    unsigned long long scanned = 0;
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t u = big[i];
        const uint32_t du = __ldcg(dist + u);
        const uint32_t vb = ptr[u], ve = ptr[u + 1];
        const uint32_t b = vb + (c - bigoff[i]) * EG_SSSP_CHUNK;
        const uint32_t e = ve - b > EG_SSSP_CHUNK ? b + EG_SSSP_CHUNK : ve;
        if (threadIdx.x == 0) scanned += e - b;
        for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x)
            sssp_relax(u, du, __ldg(col + p), __ldg(wts + p), w, dist, next_bm);
    }
    if (scanned) atomicAdd(&cnt->relax, scanned);
}

// A warp takes 32 frontier vertices (one per lane) and relaxes their
// out-lists together (eg_warp_lists); lists over EG_SSSP_WARP_EDGES go to
// the side list for k_sssp_push_big.
#define EG_SSSP_WARP_EDGES 256u
__global__ void __launch_bounds__(256) k_sssp_push(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                   const uint32_t *__restrict__ wts,
                                                   const uint32_t *__restrict__ queue, uint32_t qlen, uint32_t *dist,
                                                   uint32_t *next_bm, WRule w, SsspCounters *cnt, uint32_t *big) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long scanned = 0;
    for (uint32_t q0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; q0 < qlen; q0 += warps * 32) {
        const uint32_t qi = q0 + lane;
        uint32_t u = 0, b = 0, d = 0, du = 0;
        if (qi < qlen) {
            u = queue[qi];
            b = ptr[u];
            d = ptr[u + 1] - b;
            if (d > EG_SSSP_WARP_EDGES) {
                big[atomicAdd(&cnt->nbig, 1u)] = u;
                d = 0;
            } else {
                du = __ldcg(dist + u);
                scanned += d;
            }
        }
        eg_warp_lists(u, b, d, [&](bool valid, uint32_t lo, uint32_t ou, uint32_t p) {
            const uint32_t odu = __shfl_sync(EG_FULL_MASK, du, lo);
            if (valid) sssp_relax(ou, odu, __ldg(col + p), __ldg(wts + p), w, dist, next_bm);
        });
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) scanned += __shfl_down_sync(EG_FULL_MASK, scanned, o);
    if (lane == 0 && scanned) atomicAdd(&cnt->relax, scanned);
}

__global__ void k_count_reached(const uint32_t *__restrict__ dist, uint64_t len, unsigned long long *out,
                                uint32_t inf) {
    unsigned long long c = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x)
        c += dist[i] != inf;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(EG_FULL_MASK, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void k_edge_weights(const uint32_t *__restrict__ rid, const uint32_t *__restrict__ col, uint32_t m,
                               WRule w, uint32_t *__restrict__ out) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x)
        out[p] = w.weight(__ldg(rid + p), __ldg(col + p));
}

uint32_t blocks_for(eg_ctx *ctx, uint64_t threads) {
    uint64_t b = (threads + 255) / 256;
    uint64_t cap = (uint64_t)ctx->sm_count * 8;
    if (b > cap) b = cap;
    return b ? (uint32_t)b : 1u;
}

int check_weights(const eg_weights *w) {
    if (!w) return EG_OK;
    if (w->rule != EG_W_REF && w->rule != EG_W_HASH && w->rule != EG_W_UNIT && w->rule != EG_W_HASH_F32)
        return eg_fail(EG_EINVAL, "unknown weight rule %d", w->rule);
    if (w->rule == EG_W_HASH && w->hi < w->lo) return eg_fail(EG_EINVAL, "weight range hi < lo");
    return EG_OK;
}

}  // namespace

int eg_fill_weights(eg_graph *g, const eg_wrule &w, uint32_t *out) {
    eg_ctx *ctx = g->ctx;
    const eg_adj &a = g->csr;
    if (g->m) {
        k_edge_weights<<<blocks_for(ctx, g->m), 256, 0, ctx->stream>>>(bp<uint32_t>(a.rid), bp<uint32_t>(a.col),
                                                                      (uint32_t)g->m, w, out);
        EG_LAUNCHED(ctx);
    }
    return EG_OK;
}

int eg_edge_weights(eg_graph *g, const eg_wrule &w, const uint32_t **out) {
    const uint64_t key[3] = {(uint64_t)w.rule, w.seed, ((uint64_t)w.lo << 32) ^ w.span};
    if (g->wts.p && !memcmp(key, g->wts_key, sizeof(key))) {
        *out = bp<uint32_t>(g->wts);
        return EG_OK;
    }
    EG_TRY(eg_buf_ensure(g->ctx, g->wts, g->m * 4 + 16));
    EG_TRY(eg_fill_weights(g, w, bp<uint32_t>(g->wts)));
    memcpy(g->wts_key, key, sizeof(key));
    *out = bp<uint32_t>(g->wts);
    return EG_OK;
}

extern "C" int eg_sssp(eg_graph *g, uint32_t root, const eg_weights *wrule_in, uint32_t *dist_out,
                       eg_sssp_stats *stats) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (root >= g->n) return eg_fail(EG_EINVAL, "root %u >= n %u", root, g->n);
    if (!(g->built & EG_LAYOUT_CSR)) return eg_fail(EG_ENOTBUILT, "SSSP needs the CSR");
    EG_TRY(check_weights(wrule_in));
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n, nw = (n + 31) >> 5;
    const WRule w = eg_make_wrule(wrule_in);
    const uint32_t *wts = nullptr;
    EG_TRY(eg_edge_weights(g, w, &wts));
    EG_TRY(eg_buf_ensure(ctx, g->dist, (uint64_t)n * 4));
    const uint64_t off_q0 = nw, off_q1 = off_q0 + n, off_big = off_q1 + n, off_bigoff = off_big + n,
                   off_cnt = (off_bigoff + n + 1 + 7) & ~7ull;
    EG_TRY(eg_buf_ensure(ctx, g->sssp_work, (off_cnt + 16) * 4));
    uint32_t *wk = bp<uint32_t>(g->sssp_work);
    uint32_t *bm = wk, *q[2] = {wk + off_q0, wk + off_q1}, *big = wk + off_big, *bigoff = wk + off_bigoff;
    SsspCounters *cnt = reinterpret_cast<SsspCounters *>(wk + off_cnt);
    SsspCounters *h = (SsspCounters *)ctx->h_pinned;
    uint32_t *dist = bp<uint32_t>(g->dist);
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    EG_CUDA(cudaMemsetAsync(bm, 0, (uint64_t)nw * 4, ctx->stream));
    k_sssp_init<<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(n, dist, root, q[0], cnt, w.inf());
    EG_LAUNCHED(ctx);
    uint32_t qlen = 1;
    int cur = 0, rounds = 0;
    unsigned long long relax = 0;
    while (qlen > 0) {
        const int nxt = cur ^ 1;
        EG_CUDA(cudaMemsetAsync(&cnt->qsize, 0, 8, ctx->stream));  // qsize and nbig
        k_sssp_push<<<blocks_for(ctx, qlen), 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col),
                                                                   wts, q[cur], qlen, dist, bm, w, cnt, big);
        EG_LAUNCHED(ctx);
        k_big_offsets<<<1, 1024, 0, ctx->stream>>>(big, &cnt->nbig, 1u, bp<uint32_t>(g->csr.ptr), EG_SSSP_CHUNK,
                                                   bigoff);
        EG_LAUNCHED(ctx);
        k_sssp_push_big<<<(uint32_t)ctx->sm_count * 8, 256, 0, ctx->stream>>>(
            bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), wts, big, bigoff, dist, bm, w, cnt);
        EG_LAUNCHED(ctx);
        // the marked vertices become the next queue; their bits are cleared
        k_bm_queue<<<blocks_for(ctx, (uint64_t)nw * 32), 256, 0, ctx->stream>>>(bm, n, q[nxt], &cnt->qsize, 1);
        EG_LAUNCHED(ctx);
        EG_TRY(eg_readback_wait(ctx, h, cnt, sizeof(SsspCounters), ctx->stream));
        qlen = h->qsize;
        relax = h->relax;
        cur = nxt;
        rounds++;
        if (rounds > (int)(4 * (uint64_t)n + 16)) return eg_fail(EG_ETIMEOUT, "SSSP did not converge");
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (dist_out) EG_CUDA(cudaMemcpyAsync(dist_out, dist, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    unsigned long long *dcount = &cnt->reached;
    if (stats) {
        EG_CUDA(cudaMemsetAsync(dcount, 0, 8, ctx->stream));
        k_count_reached<<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(dist, n, dcount, w.inf());
        EG_LAUNCHED(ctx);
        EG_CUDA(cudaMemcpyAsync(h, dcount, 8, cudaMemcpyDeviceToHost, ctx->stream));
    }
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->reached = (uint32_t) * (unsigned long long *)h;
        stats->rounds = rounds;
        stats->relaxations = relax;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}

// ============================================================== multi-source
// dist is vertex-major: dist[v*k + s].  The frontier is a bit per
// (vertex, source): act[v*KW + j] holds sources 32j..32j+31.  One warp takes
// one (frontier vertex, source word) and walks the vertex's out-list; its 32
// lanes relax 32 sources of the same edge (coalesced 128-byte rows).
namespace {
// Round-loop state of the batched SSSP graph: the current frontier's length,
// the rounds run, and an error flag when the round bound was hit.
struct MsState {
    uint32_t qlen;
    uint32_t rounds;
    uint32_t limit;
    uint32_t err;
};

// Round start: the counters the round's kernels accumulate into are cleared.
__global__ void k_msssp_prep(SsspCounters *cnt) {
    cnt->qsize = 0;
    cnt->nbig = 0;
    cnt->grab = 0;
    cnt->grab_big = 0;
}

// Round end: the next frontier becomes the current one; the while node runs
// the body (two rounds) again while a frontier is left and the bound allows.
__global__ void k_msssp_end(MsState *st, const SsspCounters *cnt, cudaGraphConditionalHandle handle, int last) {
    if (st->qlen) st->rounds += 1;
    st->qlen = cnt->qsize;
    if (st->qlen && st->rounds >= st->limit) {
        st->err = 1;
        st->qlen = 0;
    }
    if (last) cudaGraphSetConditional(handle, st->qlen ? 1u : 0u);
}

__global__ void k_msssp_init(uint32_t n, int k, uint32_t kw, uint32_t *dist, uint32_t *act0, uint32_t *act1,
                             uint32_t inf) {
    uint64_t total = (uint64_t)n * k;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
        dist[i] = inf;
    uint64_t tw = (uint64_t)n * kw;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < tw; i += (uint64_t)gridDim.x * blockDim.x) {
        act0[i] = 0;
        act1[i] = 0;
    }
}

__global__ void k_msssp_roots(const uint32_t *roots, int k, uint32_t kw, uint32_t *dist, uint32_t *act,
                              uint32_t *inq, uint32_t *queue, SsspCounters *cnt) {
    for (int s = threadIdx.x; s < k; s += blockDim.x) {
        uint32_t r = roots[s];
        dist[(uint64_t)r * k + s] = 0;
        atomicOr(act + (uint64_t)r * kw + (s >> 5), 1u << (s & 31));
        uint32_t bit = 1u << (r & 31);
        if (!(atomicOr(inq + (r >> 5), bit) & bit)) queue[atomicAdd(&cnt->qsize, 1u)] = r;
    }
}

// Records v in the next frontier for sources of word j (eg_mrelax's Sink).
struct MsSink {
    uint32_t j, kw;
    uint32_t *next_act, *next_inq, *next_queue;
    SsspCounters *cnt;
    __device__ __forceinline__ bool enqueue_bit(uint32_t v) {
        const uint32_t bit = 1u << (v & 31);
        return !(atomicOr(next_inq + (v >> 5), bit) & bit);
    }
    __device__ __forceinline__ void row(uint32_t v, uint32_t ball) {
        atomicOr(next_act + (uint64_t)v * kw + j, ball);
        if (enqueue_bit(v)) next_queue[atomicAdd(&cnt->qsize, 1u)] = v;
    }
    __device__ __forceinline__ bool mark(uint32_t v, uint32_t bit) {
        atomicOr(next_act + (uint64_t)v * kw + j, bit);
        return enqueue_bit(v);
    }
    __device__ __forceinline__ void append(bool q, uint32_t v) {
        const uint32_t ball = __ballot_sync(EG_FULL_MASK, q);
        if (!ball) return;
        uint32_t base = 0;
        if ((threadIdx.x & 31) == 0) base = atomicAdd(&cnt->qsize, (uint32_t)__popc(ball));
        base = __shfl_sync(EG_FULL_MASK, base, 0);
        if (q) next_queue[base + __popc(ball & eg_lanemask_lt())] = v;
    }
    __device__ __forceinline__ void any(uint32_t) {}
};

__global__ void __launch_bounds__(256, EG_MSSSP_MINB) k_msssp_push(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                    const uint32_t *__restrict__ wts, const uint32_t *__restrict__ queue,
                                                    const MsState *st, int k,
                                                    uint32_t kw, uint32_t *dist, const uint32_t *__restrict__ act,
                                                    uint32_t *next_act, uint32_t *next_inq, uint32_t *next_queue,
                                                    WRule w, SsspCounters *cnt, uint32_t *big) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long scanned = 0;
    const uint64_t items = (uint64_t)st->qlen * kw;
    MsSink sink{0, kw, next_act, next_inq, next_queue, cnt};
    for (;;) {  // 32 items per unit
        const uint64_t base = (uint64_t)eg_warp_grab(&cnt->grab) * 32;
        if (base >= items) break;
        eg_mrelax_items(base, items, queue, kw, ptr, col, wts, w, (uint32_t)k, dist, act, EG_SSSP_BIG_DEG, big,
                        &cnt->nbig, sink, scanned);
    }
    if (lane == 0 && scanned) atomicAdd(&cnt->relax, scanned);
}

// The deferred (high-degree vertex, source word) items: chunks of
// EG_MSSSP_CHUNK edges handed out to the CTAs, one warp per 32 edges of a
// chunk.
#define EG_MSSSP_CHUNK 256u  // one CTA work unit: its 8 warps take 32 edges each
__global__ void __launch_bounds__(256) k_msssp_push_big(const uint32_t *__restrict__ ptr,
                                                        const uint32_t *__restrict__ col,
                                                        const uint32_t *__restrict__ wts, int k, uint32_t kw,
                                                        uint32_t *dist, const uint32_t *__restrict__ act,
                                                        uint32_t *next_act, uint32_t *next_inq, uint32_t *next_queue,
                                                        WRule w, SsspCounters *cnt, const uint32_t *big,
                                                        const uint32_t *__restrict__ bigoff) {
    const uint32_t nbig = *(volatile uint32_t *)&cnt->nbig;
    if (!nbig) return;
    const uint32_t total = bigoff[nbig];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long scanned = 0;
    for (;;) {
        const uint32_t c = eg_cta_grab(&cnt->grab_big);
        if (c >= total) break;
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t item = big[i];
        const uint32_t u = item / kw, j = item % kw;
        const uint32_t a = act[(uint64_t)u * kw + j];
        const uint32_t s = j * 32 + lane;
        const bool on = (a >> lane) & 1u;
        const uint32_t du = on ? __ldcg(dist + (uint64_t)u * k + s) : 0u;
        const uint32_t vb = ptr[u], ve = ptr[u + 1];
        const uint32_t off = c - bigoff[i];
        if (off == 0 && threadIdx.x == 0) scanned += (ve - vb) * (unsigned long long)__popc(a);
        const uint32_t b = vb + off * EG_MSSSP_CHUNK + 32u * warp;
        if (b < ve) {
            MsSink sink{j, kw, next_act, next_inq, next_queue, cnt};
            eg_mrelax(u, b, ve - b > 32 ? b + 32 : ve, col, wts, w, a, du, j, (uint32_t)k, dist, sink);
        }
    }
    if (scanned) atomicAdd(&cnt->relax, scanned);
}

// Clears the frontier words and queued bits of the vertices in a queue.
__global__ void k_msssp_clear(const uint32_t *__restrict__ queue, const MsState *st, uint32_t kw, uint32_t *act,
                              uint32_t *inq) {
    const uint32_t qlen = st->qlen;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (uint64_t)qlen * kw;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = queue[i / kw];
        act[(uint64_t)v * kw + i % kw] = 0;
        if (i % kw == 0) atomicAnd(inq + (v >> 5), ~(1u << (v & 31)));
    }
}

__global__ void k_transpose_dist(const uint32_t *__restrict__ dvk, uint32_t n, int k, uint32_t *__restrict__ dkv) {
    __shared__ uint32_t t[32][33];
    uint32_t v0 = blockIdx.x * 32, s0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        uint32_t v = v0 + r, s = s0 + threadIdx.x;
        t[r][threadIdx.x] = (v < n && s < (uint32_t)k) ? dvk[(uint64_t)v * k + s] : 0u;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        uint32_t s = s0 + r, v = v0 + threadIdx.x;
        if (v < n && s < (uint32_t)k) dkv[(uint64_t)s * n + v] = t[threadIdx.x][r];
    }
}
}  // namespace

namespace {
// Loop state from the roots' queue: qlen = the roots' frontier, no rounds yet.
__global__ void k_msssp_state(MsState *st, const SsspCounters *cnt, uint32_t limit) {
    st->qlen = cnt->qsize;
    st->rounds = 0;
    st->limit = limit;
    st->err = 0;
}
}  // namespace

// The round loop of eg_sssp_multi as one CUDA graph: a while node whose body
// runs two rounds (frontier buffers 0 -> 1, then 1 -> 0), each round = clear
// the counters, relax the frontier's (vertex, source word) items, cut the
// hubs' deferred items into chunks and relax them, clear the old frontier,
// and move the next frontier's length into the state.  Every kernel takes
// its work from counters (fixed grids), so a round with an empty frontier
// does nothing.  Valid while the buffers, k and the weight array it was
// captured with (key) stay the same.
static int msssp_graph_build(eg_graph *g, const void *const key[8], const uint32_t *wts, int k, uint32_t kw, WRule w,
                             uint32_t *dist, uint32_t *const act[2], uint32_t *const inq[2], uint32_t *const q[2],
                             uint32_t *big, uint32_t *bigoff, MsState *st, SsspCounters *cnt) {
    eg_ctx *ctx = g->ctx;
    eg_bfs_graph &bg = g->ssg;
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
    const uint32_t *ptr = bp<uint32_t>(g->csr.ptr), *col = bp<uint32_t>(g->csr.col);
    EG_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    for (int cur = 0; cur < 2; cur++) {
        const int nxt = cur ^ 1;
        k_msssp_prep<<<1, 1, 0, ctx->stream>>>(cnt);
        k_msssp_push<<<blocks, 256, 0, ctx->stream>>>(ptr, col, wts, q[cur], st, k, kw, dist, act[cur], act[nxt],
                                                       inq[nxt], q[nxt], w, cnt, big);
        k_big_offsets<<<1, 1024, 0, ctx->stream>>>(big, &cnt->nbig, kw, ptr, EG_MSSSP_CHUNK, bigoff);
        k_msssp_push_big<<<blocks, 256, 0, ctx->stream>>>(ptr, col, wts, k, kw, dist, act[cur], act[nxt], inq[nxt],
                                                           q[nxt], w, cnt, big, bigoff);
        // the current frontier's words and bits are cleared for reuse as "next"
        k_msssp_clear<<<blocks, 256, 0, ctx->stream>>>(q[cur], st, kw, act[cur], inq[cur]);
        k_msssp_end<<<1, 1, 0, ctx->stream>>>(st, cnt, handle, cur);
    }
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &body);
    if (ce != cudaSuccess) return eg_fail(EG_ECUDA, "batched SSSP capture: %s", cudaGetErrorString(ce));
    cudaGraphExec_t exec = nullptr;
    EG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    bg.exec = exec;
    for (int i = 0; i < 8; i++) bg.key[i] = key[i];
    return EG_OK;
}

extern "C" int eg_sssp_multi(eg_graph *g, const uint32_t *roots, int k, const eg_weights *wrule_in,
                             uint32_t *dist_out, eg_sssp_stats *stats) {
    if (!g || !roots) return eg_fail(EG_EINVAL, "NULL argument");
    if (k < 1 || k > 1024) return eg_fail(EG_EINVAL, "k=%d: batched SSSP takes 1..1024 sources", k);
    if (!(g->built & EG_LAYOUT_CSR)) return eg_fail(EG_ENOTBUILT, "SSSP needs the CSR");
    EG_TRY(check_weights(wrule_in));
    for (int s = 0; s < k; s++)
        if (roots[s] >= g->n) return eg_fail(EG_EINVAL, "root %u >= n", roots[s]);
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n, nw = (n + 31) >> 5, kw = (uint32_t)((k + 31) / 32);
    const WRule w = eg_make_wrule(wrule_in);
    const uint32_t *wts = nullptr;
    EG_TRY(eg_edge_weights(g, w, &wts));
    // work: dist[n*k] | act0, act1 [n*kw] | inq0, inq1 [nw] | q0, q1 [n] | roots | counters
    if ((uint64_t)n * kw >= 0xffffffffull) return eg_fail(EG_EINVAL, "n * ceil(k/32) must be < 2^32");
    const uint64_t off_act0 = (uint64_t)n * k, off_act1 = off_act0 + (uint64_t)n * kw, off_inq0 = off_act1 + (uint64_t)n * kw,
                   off_inq1 = off_inq0 + nw, off_q0 = off_inq1 + nw, off_q1 = off_q0 + n, off_big = off_q1 + n,
                   off_bigoff = off_big + (uint64_t)n * kw, off_roots = off_bigoff + (uint64_t)n * kw + 1,
                   off_cnt = (off_roots + 1024 + 7) & ~7ull;
    EG_TRY(eg_buf_ensure(ctx, g->sssp_work, (off_cnt + 16) * 4));
    uint32_t *wk = bp<uint32_t>(g->sssp_work);
    uint32_t *dist = wk, *act[2] = {wk + off_act0, wk + off_act1}, *inq[2] = {wk + off_inq0, wk + off_inq1},
             *q[2] = {wk + off_q0, wk + off_q1}, *d_roots = wk + off_roots, *big = wk + off_big,
             *bigoff = wk + off_bigoff;
    SsspCounters *cnt = reinterpret_cast<SsspCounters *>(wk + off_cnt);
    MsState *st = reinterpret_cast<MsState *>(wk + off_cnt + 8);
    SsspCounters *h = (SsspCounters *)ctx->h_pinned;
    EG_CUDA(cudaMemcpyAsync(d_roots, roots, (uint64_t)k * 4, cudaMemcpyHostToDevice, ctx->stream));
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    k_msssp_init<<<blocks_for(ctx, (uint64_t)n * k), 256, 0, ctx->stream>>>(n, k, kw, dist, act[0], act[1], w.inf());
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemsetAsync(inq[0], 0, 2ull * nw * 4, ctx->stream));
    EG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(SsspCounters), ctx->stream));
    k_msssp_roots<<<1, 256, 0, ctx->stream>>>(d_roots, k, kw, dist, act[0], inq[0], q[0], cnt);
    EG_LAUNCHED(ctx);
    // the round loop: one CUDA graph launch (built once per graph, buffers,
    // k and weight array; a while node over a body of two rounds, so that
    // each half keeps its frontier buffers fixed)
    k_msssp_state<<<1, 1, 0, ctx->stream>>>(st, cnt, (uint32_t)(4 * (uint64_t)n + 16));
    EG_LAUNCHED(ctx);
    const void *key[8] = {wk, wts, g->csr.col.p, (const void *)(uintptr_t)k, (const void *)(uintptr_t)kw,
                          (const void *)(uintptr_t)w.rule, (const void *)(uintptr_t)n, nullptr};
    eg_bfs_graph &bg = g->ssg;
    bool same = bg.exec != nullptr;
    for (int i = 0; i < 8 && same; i++) same = bg.key[i] == key[i];
    if (!same) EG_TRY(msssp_graph_build(g, key, wts, k, kw, w, dist, act, inq, q, big, bigoff, st, cnt));
    EG_CUDA(cudaGraphLaunch(bg.exec, ctx->stream));
    ctx->launches += 1;
    EG_TRY(eg_readback(ctx, h + 1, st, sizeof(MsState), ctx->stream));
    EG_TRY(eg_readback(ctx, h, cnt, sizeof(SsspCounters), ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    const MsState *hst = reinterpret_cast<const MsState *>(h + 1);
    if (hst->err) return eg_fail(EG_ETIMEOUT, "batched SSSP did not converge");
    const int rounds = (int)hst->rounds;
    const unsigned long long relax = h->relax;
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (dist_out) {
        EG_TRY(eg_buf_ensure(ctx, g->dist, (uint64_t)n * k * 4));
        dim3 grid(eg_div_up(n, 32), eg_div_up((uint64_t)k, 32)), block(32, 8);
        k_transpose_dist<<<grid, block, 0, ctx->stream>>>(dist, n, k, bp<uint32_t>(g->dist));
        EG_LAUNCHED(ctx);
        EG_CUDA(cudaMemcpyAsync(dist_out, g->dist.p, (uint64_t)n * k * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        unsigned long long *dcount = &cnt->reached;
        EG_CUDA(cudaMemsetAsync(dcount, 0, 8, ctx->stream));
        k_count_reached<<<blocks_for(ctx, (uint64_t)n * k), 256, 0, ctx->stream>>>(dist, (uint64_t)n * k, dcount,
                                                                                   w.inf());
        EG_LAUNCHED(ctx);
        EG_CUDA(cudaMemcpyAsync(h, dcount, 8, cudaMemcpyDeviceToHost, ctx->stream));
        EG_CUDA(cudaStreamSynchronize(ctx->stream));
        unsigned long long rc = *(unsigned long long *)h;
        stats->reached = (uint32_t)(rc > 0xffffffffull ? 0xffffffffull : rc);
        stats->rounds = rounds;
        stats->relaxations = relax;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}
