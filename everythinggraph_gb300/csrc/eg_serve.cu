// Query server: continuous batching of BFS, SSSP and personalised-PageRank
// queries over one resident graph.
//
// No counterpart in the reference (it runs one algorithm per process).  Each
// query kind has an engine with a fixed number of slots whose state lives in
// HBM for the server's lifetime:
//   BFS   64 slots, bit-sliced: bit s of seen[v]/front[v] (u64) is slot s
//   SSSP  64 slots, dist[v][s] vertex-major, per-(vertex, slot) frontier bits
//   PPR   32 lanes, x[v][q] vertex-major (the eg_ppr_multi iteration)
// A scheduler tick admits queued queries into free slots (slot counts are
// capped by the HBM budget), advances every engine that has live slots by one
// step (one BFS level, one Bellman-Ford round, one PPR iteration) and retires
// the slots whose query finished.  A slot's arithmetic never reads another
// slot's values, so a query's result does not depend on what else is in the
// batch.  Each engine's step is the same code whatever the slot occupancy.
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <deque>
#include <vector>

#include "eg_bigwork.cuh"
#include "eg_mrelax.cuh"
#include "eg_mspull.cuh"
#include "eg_ppr.cuh"

#define SV_INF 0xfffffffeu
#define SV_BFS_SLOTS 64
#define SV_SSSP_SLOTS 64
#define SV_PPR_LANES 32
#define SV_BIG_DEG 2048u

namespace {

double now_s() {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

struct SvCounters {
    unsigned long long deg;         // out-degree sum of the new frontier
    unsigned long long newmask;     // BFS: slots that discovered vertices this level
    unsigned long long actmask[4];  // SSSP: slots still relaxing (bits of the next frontier)
    uint32_t count;                 // vertices in the new frontier
    uint32_t qsize;
    uint32_t nbig;
    uint32_t grab, grab_big;  // SSSP work units handed out this step
    uint32_t pad;
};

// ------------------------------------------------------------------ BFS engine
__global__ void k_sv_bfs_admit(const uint32_t *roots, const uint32_t *slots, int k, uint32_t n,
                               unsigned long long *seen, unsigned long long *front, int32_t *levels) {
    const int i = threadIdx.x;
    if (i < k) {
        const uint32_t r = roots[i], s = slots[i];
        atomicOr(seen + r, 1ull << s);
        atomicOr(front + r, 1ull << s);
        levels[(uint64_t)s * n + r] = 1;
    }
}

// pull: OR the frontier words of the in-neighbours (early exit when every
// missing slot is found)
__global__ void k_sv_front_queue(const unsigned long long *__restrict__ front, uint32_t n, uint32_t *queue,
                                 SvCounters *cnt) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < n; v0 += gridDim.x * blockDim.x) {
        const uint32_t v = v0 + lane;
        const bool on = v < n && front[v] != 0ull;
        const uint32_t ball = __ballot_sync(EG_FULL_MASK, on);
        if (ball) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&cnt->qsize, __popc(ball));
            base = __shfl_sync(EG_FULL_MASK, base, 0);
            if (on) queue[base + __popc(ball & eg_lanemask_lt())] = v;
        }
    }
}

__global__ void __launch_bounds__(256) k_sv_bfs_push(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                     const uint32_t *__restrict__ queue, const SvCounters *qc,
                                                     const unsigned long long *__restrict__ seen,
                                                     const unsigned long long *__restrict__ front,
                                                     unsigned long long *__restrict__ next, uint32_t *big,
                                                     SvCounters *cnt) {
    const uint32_t qlen = qc->qsize;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; qi < qlen; qi += warps) {
        const uint32_t u = queue[qi];
        const uint32_t b = ptr[u], e = ptr[u + 1];
        if (e - b > SV_BIG_DEG) {
            if (lane == 0) big[atomicAdd(&cnt->nbig, 1u)] = u;
            continue;
        }
        const unsigned long long f = front[u];
        for (uint32_t p = b + lane; p < e; p += 32) {
            const uint32_t v = col[p];
            const unsigned long long add = f & ~__ldcg(seen + v);
            if (add && (__ldcg(next + v) & add) != add) atomicOr(next + v, add);
        }
    }
}

#define SV_BFS_CHUNK 4096u  // edges of a deferred hub per CTA work unit
__global__ void __launch_bounds__(256) k_sv_bfs_push_big(const uint32_t *__restrict__ ptr,
                                                         const uint32_t *__restrict__ col, const uint32_t *big,
                                                         const uint32_t *__restrict__ bigoff,
                                                         const unsigned long long *__restrict__ seen,
                                                         const unsigned long long *__restrict__ front,
                                                         unsigned long long *__restrict__ next, const SvCounters *cnt) {
    const uint32_t nbig = *(volatile const uint32_t *)&cnt->nbig;
    if (!nbig) return;
    const uint32_t total = bigoff[nbig];
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t u = big[i];
        const unsigned long long f = front[u];
        const uint32_t b = ptr[u] + (c - bigoff[i]) * SV_BFS_CHUNK, e = min(ptr[u + 1], b + SV_BFS_CHUNK);
        for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) {
            const uint32_t v = col[p];
            const unsigned long long add = f & ~__ldcg(seen + v);
            if (add && (__ldcg(next + v) & add) != add) atomicOr(next + v, add);
        }
    }
}

// seen |= new, levels of the new bits = slot level + 1, front = new, next = 0
__global__ void k_sv_bfs_fold(uint32_t n, unsigned long long *seen, unsigned long long *front,
                              unsigned long long *next, int32_t *levels, const int32_t *__restrict__ slot_level,
                              const uint32_t *__restrict__ deg, SvCounters *cnt) {
    unsigned long long my_new = 0ull, my_deg = 0ull;
    uint32_t my_cnt = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const unsigned long long x = next[v] & ~seen[v];
        next[v] = 0ull;
        front[v] = x;
        if (x) {
            seen[v] |= x;
            my_new |= x;
            my_cnt++;
            my_deg += deg[v];
            unsigned long long y = x;
            while (y) {
                const int s = __ffsll((long long)y) - 1;
                y &= y - 1;
                levels[(uint64_t)s * n + v] = slot_level[s] + 1;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        my_new |= __shfl_down_sync(EG_FULL_MASK, my_new, o);
        my_deg += __shfl_down_sync(EG_FULL_MASK, my_deg, o);
        my_cnt += __shfl_down_sync(EG_FULL_MASK, my_cnt, o);
    }
    if ((threadIdx.x & 31) == 0 && my_cnt) {
        atomicOr(&cnt->newmask, my_new);
        atomicAdd(&cnt->deg, my_deg);
        atomicAdd(&cnt->count, my_cnt);
    }
}

// retiring slots: clear their bits everywhere
__global__ void k_sv_bfs_clear(uint32_t n, unsigned long long keep, unsigned long long *seen,
                               unsigned long long *front) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        seen[v] &= keep;
        front[v] &= keep;
    }
}

// reached count and deepest level of a slot's level row
__global__ void k_sv_level_summary(const int32_t *__restrict__ row, uint32_t n, unsigned long long *out) {
    unsigned long long c = 0, mx = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int32_t l = row[v];
        c += l > 0;
        mx = l > (int32_t)mx ? (unsigned long long)l : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_down_sync(EG_FULL_MASK, c, o);
        mx = max(mx, __shfl_down_sync(EG_FULL_MASK, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, c);
        atomicMax(out + 1, mx);
    }
}

// ------------------------------------------------------------------ SSSP engine
using SvW = eg_wrule;  // integer rules only (the server keeps u32 distances)

__global__ void k_sv_sssp_admit(const uint32_t *roots, const uint32_t *slots, int k, uint32_t *dist, uint32_t *act,
                                uint32_t *inq, uint32_t *queue, SvCounters *cnt) {
    const int i = threadIdx.x;
    if (i < k) {
        const uint32_t r = roots[i], s = slots[i];
        dist[(uint64_t)r * SV_SSSP_SLOTS + s] = 0;
        atomicOr(act + (uint64_t)r * 2 + (s >> 5), 1u << (s & 31));
        const uint32_t bit = 1u << (r & 31);
        if (!(atomicOr(inq + (r >> 5), bit) & bit)) queue[atomicAdd(&cnt->qsize, 1u)] = r;
    }
}

// Records v in the next frontier for slots of word j (eg_mrelax's Sink).
// The slots that improved anything collect in lane 0's registers (am) and
// reach cnt->actmask once per warp (flush), not once per improved edge.
struct SvSink {
    uint32_t j;
    uint32_t *next_act, *next_inq, *next_queue;
    SvCounters *cnt;
    uint32_t am[2];
    __device__ __forceinline__ bool enqueue_bit(uint32_t v) {
        const uint32_t bit = 1u << (v & 31);
        return !(atomicOr(next_inq + (v >> 5), bit) & bit);
    }
    __device__ __forceinline__ void row(uint32_t v, uint32_t ball) {
        atomicOr(next_act + (uint64_t)v * 2 + j, ball);
        am[j] |= ball;
        if (enqueue_bit(v)) next_queue[atomicAdd(&cnt->qsize, 1u)] = v;
    }
    __device__ __forceinline__ bool mark(uint32_t v, uint32_t bit) {
        atomicOr(next_act + (uint64_t)v * 2 + j, bit);
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
    __device__ __forceinline__ void any(uint32_t bit) { am[j] |= bit; }
    __device__ __forceinline__ void flush() {
        if ((threadIdx.x & 31) != 0) return;
        if (am[0]) atomicOr(&cnt->actmask[0], (unsigned long long)am[0]);
        if (am[1]) atomicOr(&cnt->actmask[1], (unsigned long long)am[1]);
    }
};

__global__ void __launch_bounds__(256, EG_MSSSP_MINB) k_sv_sssp_push(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                                      const uint32_t *__restrict__ wts, const uint32_t *__restrict__ queue, const SvCounters *qc,
                                                      uint32_t *dist, const uint32_t *__restrict__ act,
                                                      uint32_t *next_act, uint32_t *next_inq, uint32_t *next_queue,
                                                      SvW w, SvCounters *cnt, uint32_t *big) {
    const uint32_t qlen = qc->qsize;
    unsigned long long scanned = 0;
    SvSink sink{0, next_act, next_inq, next_queue, cnt, {0u, 0u}};
    for (;;) {  // 32 items per unit
        const uint64_t base = (uint64_t)eg_warp_grab(&cnt->grab) * 32;
        if (base >= 2ull * qlen) break;
        eg_mrelax_items(base, 2ull * qlen, queue, 2u, ptr, col, wts, w, SV_SSSP_SLOTS, dist, act, SV_BIG_DEG, big,
                        &cnt->nbig, sink, scanned);
    }
    sink.flush();
}

// Deferred (hub, word) items in chunks of SV_SSSP_CHUNK edges handed out to
// the CTAs, one warp per 32 edges of a chunk.
#define SV_SSSP_CHUNK 256u  // one CTA work unit: its 8 warps take 32 edges each
__global__ void __launch_bounds__(256) k_sv_sssp_push_big(const uint32_t *__restrict__ ptr,
                                                          const uint32_t *__restrict__ col,
                                                          const uint32_t *__restrict__ wts, uint32_t *dist,
                                                          const uint32_t *__restrict__ act, uint32_t *next_act,
                                                          uint32_t *next_inq, uint32_t *next_queue, SvW w,
                                                          SvCounters *cnt, const uint32_t *big,
                                                          const uint32_t *__restrict__ bigoff) {
    const uint32_t nbig = *(volatile uint32_t *)&cnt->nbig;
    if (!nbig) return;
    const uint32_t total = bigoff[nbig];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    SvSink sink{0, next_act, next_inq, next_queue, cnt, {0u, 0u}};
    for (;;) {
        const uint32_t c = eg_cta_grab(&cnt->grab_big);
        if (c >= total) break;
        const uint32_t i = eg_big_item(bigoff, nbig, c);
        const uint32_t u = big[i] >> 1, j = big[i] & 1;
        const uint32_t a = act[(uint64_t)u * 2 + j];
        const uint32_t s = j * 32 + lane;
        const bool on = (a >> lane) & 1u;
        const uint32_t du = on ? __ldcg(dist + (uint64_t)u * SV_SSSP_SLOTS + s) : 0u;
        const uint32_t ve = ptr[u + 1];
        const uint32_t b = ptr[u] + (c - bigoff[i]) * SV_SSSP_CHUNK + 32u * warp;
        if (b < ve) {
            sink.j = j;
            eg_mrelax(u, b, ve - b > 32 ? b + 32 : ve, col, wts, w, a, du, j, SV_SSSP_SLOTS, dist, sink);
        }
    }
    sink.flush();
}

__global__ void k_sv_sssp_clear_frontier(const uint32_t *__restrict__ queue, const SvCounters *qc, uint32_t *act,
                                         uint32_t *inq) {
    const uint32_t qlen = qc->qsize;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x) {
        const uint32_t v = queue[i];
        act[(uint64_t)v * 2] = 0;
        act[(uint64_t)v * 2 + 1] = 0;
        atomicAnd(inq + (v >> 5), ~(1u << (v & 31)));
    }
}

__global__ void k_sv_sssp_reset(uint32_t n, unsigned long long mask, uint32_t *dist) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        unsigned long long y = mask;
        while (y) {
            const int s = __ffsll((long long)y) - 1;
            y &= y - 1;
            dist[(uint64_t)v * SV_SSSP_SLOTS + s] = SV_INF;
        }
    }
}

// reached count and largest distance of every slot in `done`, two words per
// slot in out[]: a warp takes 32 vertices and walks the done slots, so slots
// that share a 32-byte sector of a vertex row reuse it from L1
__global__ void __launch_bounds__(256) k_sv_dist_summary(const uint32_t *__restrict__ dist, uint32_t n,
                                                         unsigned long long done, unsigned long long *out) {
    __shared__ unsigned long long s_c[SV_SSSP_SLOTS];
    __shared__ unsigned int s_m[SV_SSSP_SLOTS];
    for (uint32_t i = threadIdx.x; i < SV_SSSP_SLOTS; i += blockDim.x) {
        s_c[i] = 0;
        s_m[i] = 0;
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < n; v0 += gridDim.x * blockDim.x) {
        const uint32_t v = v0 + lane;
        for (unsigned long long y = done; y; y &= y - 1) {
            const int sl = __ffsll((long long)y) - 1;
            const uint32_t d = v < n ? dist[(uint64_t)v * SV_SSSP_SLOTS + sl] : SV_INF;
            const bool r = d != SV_INF;
            const uint32_t c = (uint32_t)__popc(__ballot_sync(EG_FULL_MASK, r));
            const uint32_t m = __reduce_max_sync(EG_FULL_MASK, r ? d : 0u);
            if (lane == 0 && c) {
                atomicAdd(&s_c[sl], (unsigned long long)c);
                atomicMax(&s_m[sl], m);
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < SV_SSSP_SLOTS; i += blockDim.x)
        if (((done >> i) & 1ull) && s_c[i]) {
            atomicAdd(out + 2 * i, s_c[i]);
            atomicMax(out + 2 * i + 1, (unsigned long long)s_m[i]);
        }
}

__global__ void k_sv_column(const uint32_t *__restrict__ m, uint32_t n, uint32_t width, uint32_t s, uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        out[v] = m[(uint64_t)v * width + s];
}

// ------------------------------------------------------------------ PPR engine
// Uses the batched PPR kernels (eg_ppr.cuh); lane q's seeds sit at
// seeds[8q .. 8q + nseeds).
__global__ void k_sv_ppr_column(const float *__restrict__ R, uint32_t n, uint32_t q, float *out, double *sum) {
    double s = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const float r = R[(uint64_t)v * EG_PPR_LANES + q];
        if (out) out[v] = r;
        s += (double)r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(EG_FULL_MASK, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

}  // namespace

// ------------------------------------------------------------------ server
struct Pending {
    uint64_t id;
    eg_query q;
};

struct eg_server {
    eg_graph *g;
    eg_serve_opts opts;
    uint64_t next_id = 1;
    std::deque<Pending> queue;
    std::vector<eg_query_result> done;
    std::vector<std::vector<uint32_t>> kept;  // per result (keep_results): full result as u32 words
    double t0;
    int bfs_cap, sssp_cap, ppr_cap;
    // BFS engine
    eg_buf bfs_buf;
    unsigned long long bfs_seen_mask = 0;  // slots in use
    int32_t bfs_level[SV_BFS_SLOTS];
    uint64_t bfs_id[SV_BFS_SLOTS];
    double bfs_admit[SV_BFS_SLOTS], bfs_arrival[SV_BFS_SLOTS];
    unsigned long long bfs_count = 0, bfs_fdeg = 0;
    // SSSP engine
    eg_buf sssp_buf;
    unsigned long long sssp_mask = 0;
    uint64_t sssp_id[SV_SSSP_SLOTS];
    double sssp_admit[SV_SSSP_SLOTS], sssp_arrival[SV_SSSP_SLOTS];
    int sssp_cur = 0;
    int sssp_rounds[SV_SSSP_SLOTS];
    // PPR engine
    eg_buf ppr_buf;
    uint32_t ppr_mask = 0;
    uint64_t ppr_id[SV_PPR_LANES];
    double ppr_admit[SV_PPR_LANES], ppr_arrival[SV_PPR_LANES];
    eg_buf wts_buf;                      // SSSP weights of the CSR entries (the server's own copy)
    const uint32_t *wts = nullptr;
    PprQ *hq = nullptr;                  // host mirror of the lanes' state (pinned, updated every iteration)
    uint32_t pseeds[SV_PPR_LANES * 8] = {};  // seeds of each lane (8 per lane)
    uint32_t pnseeds[SV_PPR_LANES] = {};
    eg_buf small;  // counters, admission lists, summaries (device)
    uint64_t ticks = 0;
    // engines run on their own streams; a step is in flight until its event completes
    cudaStream_t st[3] = {};
    cudaEvent_t ev_begin[3] = {}, ev_end[3] = {};
    bool inflight[3] = {false, false, false};
    int turn = 0;            // engine offered the GPU first at the next launch
    bool ppr_dirty = false;  // host lane table changed since its last upload
    unsigned long long step_mask[3] = {0, 0, 0};  // slots live in the step in flight
    unsigned char *hpin = nullptr;                // pinned host staging, a region per engine
    double eng_ms[3] = {0.0, 0.0, 0.0};
    uint64_t eng_steps[3] = {0, 0, 0};
    uint64_t admitted[3] = {0, 0, 0}, completed[3] = {0, 0, 0};
};

// Device small-buffer layout (bytes) and host staging layout (bytes).
enum : uint32_t {
    SM_BCNT = 0, SM_SCNT = 256, SM_SNEXT = 512, SM_BROOTS = 1024, SM_SROOTS = 1536, SM_BSLOTS = 2048,
    SM_SSLOTS = 2560, SM_BLEVEL = 3072, SM_PPRQ = 4096, SM_PSEEDS = 8192, SM_PSBEG = 9216, SM_PSEND = 9344,
    SM_SUM = 12544,  // 64 bytes per engine
    SM_RSUM = 16384,  // retire summaries: 16 bytes per slot, BFS then SSSP
    HP_BCNT = 0, HP_SCNT = 256, HP_PPRQ = 1024, HP_PSEEDS = 4096, HP_SUM = 8192,  // 64 per engine
    HP_BADM = 12288, HP_SADM = 13312, HP_BLEVEL = 14336, HP_RSUM = 16384, HP_BYTES = 20480
};

static uint32_t sv_blocks(eg_ctx *ctx, uint64_t threads) {
    uint64_t b = (threads + 255) / 256;
    const uint64_t cap = (uint64_t)ctx->sm_count * 8;
    return (uint32_t)(b > cap ? cap : (b ? b : 1));
}

extern "C" void eg_serve_opts_default(eg_serve_opts *o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->hbm_budget = 64ull << 30;
    o->max_bfs = SV_BFS_SLOTS;
    o->max_sssp = SV_SSSP_SLOTS;
    o->max_ppr = SV_PPR_LANES;
    o->weights.rule = EG_W_HASH;
    o->weights.seed = 6;
    o->weights.lo = 1;
    o->weights.hi = 255;
    o->ppr_damping = 0.85f;
    o->ppr_max_iters = 50;
    o->keep_results = 0;
    o->exclusive = 0;
    o->gang = 1;
}

// Device bytes per slot of each engine (the admission cost of one query).
static void sv_slot_bytes(uint32_t n, uint64_t *bfs, uint64_t *sssp, uint64_t *ppr) {
    *bfs = (uint64_t)n * 4;        // level row
    *sssp = (uint64_t)n * 4;       // dist column
    *ppr = (uint64_t)n * 4 * 3;    // R, X, Y columns
}

extern "C" int eg_serve_open(eg_graph *g, const eg_serve_opts *opts, eg_server **out) {
    if (!g || !out) return eg_fail(EG_EINVAL, "NULL argument");
    if (!(g->built & EG_LAYOUT_CSR) || !(g->built & EG_LAYOUT_CSC))
        return eg_fail(EG_ENOTBUILT, "the server needs the CSR and the CSC");
    eg_serve_opts o;
    if (opts) o = *opts;
    else eg_serve_opts_default(&o);
    if (o.weights.rule != EG_W_REF && o.weights.rule != EG_W_HASH && o.weights.rule != EG_W_UNIT)
        return eg_fail(EG_EINVAL, "the server takes integer weight rules (EG_W_REF, EG_W_HASH, EG_W_UNIT)");
    if (o.weights.rule == EG_W_HASH && o.weights.hi < o.weights.lo) return eg_fail(EG_EINVAL, "weight range hi < lo");
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    uint64_t sb, ss, sp;
    sv_slot_bytes(n, &sb, &ss, &sp);
    // shared per-engine state, then as many slots as the budget allows
    const uint64_t shared_bfs = (uint64_t)n * 8 * 3 + (uint64_t)n * 8 + ((uint64_t)n + 1) * 4;
    const uint64_t shared_sssp = (uint64_t)n * 8 * 2 + (uint64_t)n * 4 * 2 + (uint64_t)n * 4 * 4;
    const uint64_t shared_ppr = 0;
    const uint64_t base = shared_bfs + shared_sssp + shared_ppr;
    if (o.hbm_budget && o.hbm_budget < base + sb + ss + sp)
        return eg_fail(EG_ENOMEM, "HBM budget %llu below one slot of each engine (%llu)", (unsigned long long)o.hbm_budget,
                       (unsigned long long)(base + sb + ss + sp));
    const uint64_t avail = o.hbm_budget ? o.hbm_budget - base : ~0ull;
    // split the budget evenly in bytes between the three engines
    auto cap = [&](int want, int hard, uint64_t per) {
        int c = want < 1 ? 1 : (want > hard ? hard : want);
        uint64_t lim = avail / 3 / per;
        if ((uint64_t)c > lim) c = (int)(lim < 1 ? 1 : lim);
        return c;
    };
    eg_server *s = new eg_server();
    s->g = g;
    s->opts = o;
    s->bfs_cap = cap(o.max_bfs, SV_BFS_SLOTS, sb);
    s->sssp_cap = cap(o.max_sssp, SV_SSSP_SLOTS, ss);
    s->ppr_cap = cap(o.max_ppr, SV_PPR_LANES, sp);
    int rc = EG_OK;
    // BFS: seen | front | next (u64) | queue+big (u32 x 2n) | levels (64 rows) | big chunk offsets
    if (rc == EG_OK)
        rc = eg_buf_ensure(ctx, s->bfs_buf, (uint64_t)n * 8 * 3 + (uint64_t)n * 8 + (uint64_t)SV_BFS_SLOTS * n * 4 +
                                                ((uint64_t)n + 1) * 4);
    // SSSP: dist [n][64] | act x2 [n][2] | inq x2 | queue x2 | big | big chunk offsets
    if (rc == EG_OK)
        rc = eg_buf_ensure(ctx, s->sssp_buf, (uint64_t)n * 4 * SV_SSSP_SLOTS + (uint64_t)n * 8 * 2 + (uint64_t)((n + 31) / 32) * 4 * 2 +
                                                 (uint64_t)n * 4 * 4 + 4);
    // PPR: R, X, Y [n][32] | parts
    const uint64_t ptiles = g->m ? (g->m + EG_PPR_TILE - 1) / EG_PPR_TILE : 0;
    if (rc == EG_OK)
        rc = eg_buf_ensure(ctx, s->ppr_buf, (uint64_t)n * 4 * EG_PPR_LANES * 3 + ptiles * EG_PPR_LANES * 4 * 2 +
                                                 ((ptiles + 63) & ~63ull) * 4 + (uint64_t)ctx->sm_count * 4 * 32 * 16 + 256);
    if (rc == EG_OK) rc = eg_buf_ensure(ctx, s->small, 64 * 1024);
    if (rc == EG_OK) rc = eg_buf_ensure(ctx, s->wts_buf, g->m * 4 + 16);
    if (rc == EG_OK) rc = eg_fill_weights(g, eg_make_wrule(&o.weights), bp<uint32_t>(s->wts_buf));
    if (rc == EG_OK) s->wts = bp<uint32_t>(s->wts_buf);
    // stream priorities by step length: the blocks of a BFS level (~1 ms)
    // are scheduled ahead of those of a Bellman-Ford round or a PPR sweep
    // (~13 ms), so that the short queries do not queue behind long steps;
    // SSSP and PPR share the lower priority
    int lo_prio = 0, hi_prio = 0;
    if (rc == EG_OK && cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio) != cudaSuccess)
        rc = eg_fail(EG_ECUDA, "stream priority range");
    const int prio[3] = {hi_prio, lo_prio, lo_prio};  // BFS, SSSP, PPR
    for (int e = 0; e < 3 && rc == EG_OK; e++) {
        if (cudaStreamCreateWithPriority(&s->st[e], cudaStreamNonBlocking, prio[e]) != cudaSuccess ||
            cudaEventCreate(&s->ev_begin[e]) != cudaSuccess || cudaEventCreate(&s->ev_end[e]) != cudaSuccess)
            rc = eg_fail(EG_ECUDA, "server streams/events");
    }
    if (rc == EG_OK && cudaMallocHost(&s->hpin, HP_BYTES) != cudaSuccess) rc = eg_fail(EG_ECUDA, "server staging");
    if (rc == EG_OK) {
        s->hq = (PprQ *)(s->hpin + HP_PPRQ);
        memset(s->hpin, 0, HP_BYTES);
    }
    if (rc != EG_OK) {
        for (int e = 0; e < 3; e++) {
            if (s->st[e]) cudaStreamDestroy(s->st[e]);
            if (s->ev_begin[e]) cudaEventDestroy(s->ev_begin[e]);
            if (s->ev_end[e]) cudaEventDestroy(s->ev_end[e]);
        }
        if (s->hpin) cudaFreeHost(s->hpin);
        eg_buf_free(ctx, s->bfs_buf);
        eg_buf_free(ctx, s->sssp_buf);
        eg_buf_free(ctx, s->ppr_buf);
        eg_buf_free(ctx, s->small);
        eg_buf_free(ctx, s->wts_buf);
        delete s;
        return rc;
    }
    // initial state
    unsigned char *bb = bp<unsigned char>(s->bfs_buf);
    EG_CUDA(cudaMemsetAsync(bb, 0, (uint64_t)n * 8 * 3, ctx->stream));
    EG_CUDA(cudaMemsetAsync(bb + (uint64_t)n * 8 * 4, 0, (uint64_t)SV_BFS_SLOTS * n * 4, ctx->stream));
    unsigned char *sbuf = bp<unsigned char>(s->sssp_buf);
    EG_CUDA(cudaMemsetAsync(sbuf, 0xff, (uint64_t)n * 4 * SV_SSSP_SLOTS, ctx->stream));  // reset below to SV_INF
    k_sv_sssp_reset<<<sv_blocks(ctx, (uint64_t)n * SV_SSSP_SLOTS), 256, 0, ctx->stream>>>(n, ~0ull, (uint32_t *)sbuf);
    ctx->launches++;
    EG_CUDA(cudaMemsetAsync(sbuf + (uint64_t)n * 4 * SV_SSSP_SLOTS, 0,
                            (uint64_t)n * 8 * 2 + (uint64_t)((n + 31) / 32) * 4 * 2, ctx->stream));
    EG_CUDA(cudaMemsetAsync(s->small.p, 0, 64 * 1024, ctx->stream));
    EG_CUDA(cudaMemsetAsync(s->ppr_buf.p, 0, (uint64_t)n * 4 * EG_PPR_LANES * 2, ctx->stream));
    if (n >= 0x80000000u) return eg_fail(EG_EINVAL, "the server takes n < 2^31");
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    s->t0 = now_s();
    *out = s;
    return EG_OK;
}

extern "C" int eg_serve_close(eg_server *s) {
    if (!s) return EG_OK;
    eg_ctx *ctx = s->g->ctx;
    cudaStreamSynchronize(ctx->stream);
    for (int e = 0; e < 3; e++) {
        cudaStreamSynchronize(s->st[e]);
        cudaStreamDestroy(s->st[e]);
        cudaEventDestroy(s->ev_begin[e]);
        cudaEventDestroy(s->ev_end[e]);
    }
    cudaFreeHost(s->hpin);
    eg_buf_free(ctx, s->bfs_buf);
    eg_buf_free(ctx, s->sssp_buf);
    eg_buf_free(ctx, s->ppr_buf);
    eg_buf_free(ctx, s->small);
    eg_buf_free(ctx, s->wts_buf);
    delete s;
    return EG_OK;
}

extern "C" int eg_serve_submit(eg_server *s, const eg_query *q, uint64_t *id_out) {
    if (!s || !q) return eg_fail(EG_EINVAL, "NULL argument");
    const uint32_t n = s->g->n;
    if (q->kind == EG_Q_BFS || q->kind == EG_Q_SSSP) {
        if (q->source >= n) return eg_fail(EG_EINVAL, "source %u >= n", q->source);
    } else if (q->kind == EG_Q_PPR) {
        if (q->nseeds < 1 || q->nseeds > 8) return eg_fail(EG_EINVAL, "a PPR query has 1..8 seeds");
        for (uint32_t i = 0; i < q->nseeds; i++)
            if (q->seeds[i] >= n) return eg_fail(EG_EINVAL, "seed %u >= n", q->seeds[i]);
    } else {
        return eg_fail(EG_EINVAL, "unknown query kind %d", q->kind);
    }
    Pending p;
    p.id = s->next_id++;
    p.q = *q;
    if (p.q.arrival_s <= 0.0) p.q.arrival_s = now_s() - s->t0;
    s->queue.push_back(p);
    if (id_out) *id_out = p.id;
    return EG_OK;
}

static void sv_finish(eg_server *s, uint64_t id, int kind, double arrival, double admit, uint32_t reached,
                      uint32_t depth, int iters, double value) {
    eg_query_result r;
    memset(&r, 0, sizeof(r));
    r.id = id;
    r.kind = kind;
    r.arrival_s = arrival;
    r.admit_s = admit;
    r.done_s = now_s() - s->t0;
    r.reached = reached;
    r.depth = depth;
    r.iterations = iters;
    r.value = value;
    s->done.push_back(r);
    s->completed[kind - 1]++;
}

// ---------------------------------------------------------------- engines
// Each engine (BFS, SSSP, PPR) advances on its own stream: a step (one BFS
// level, one Bellman-Ford round, one PPR iteration over all live slots) is
// launched, its counters are copied to pinned host memory behind it, and an
// event marks its end.  eg_serve_step polls the events: an engine whose step
// finished has its finished slots retired and its free slots refilled from
// the queue, then its next step is launched.  Engines never wait for one
// another, so a slow Bellman-Ford round does not hold back BFS levels.
enum { E_BFS = 0, E_SSSP = 1, E_PPR = 2 };

static int sv_poll(eg_server *s, int e, bool *ready) {
    *ready = false;
    if (!s->inflight[e]) return EG_OK;
    const cudaError_t q = cudaEventQuery(s->ev_end[e]);
    if (q == cudaErrorNotReady) return EG_OK;
    if (q != cudaSuccess) return eg_fail(EG_ECUDA, "server engine %d: %s", e, cudaGetErrorString(q));
    float ms = 0.f;
    EG_CUDA(cudaEventElapsedTime(&ms, s->ev_begin[e], s->ev_end[e]));
    s->eng_ms[e] += ms;
    s->eng_steps[e]++;
    s->inflight[e] = false;
    *ready = true;
    return EG_OK;
}

// ---- BFS
static int sv_bfs_retire(eg_server *s, unsigned long long done) {
    eg_graph *g = s->g;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    cudaStream_t st = s->st[E_BFS];
    unsigned long long *seen = bp<unsigned long long>(s->bfs_buf);
    unsigned long long *front = seen + n;
    int32_t *levels = reinterpret_cast<int32_t *>(reinterpret_cast<uint32_t *>(seen + 3ull * n) + 2ull * n);
    unsigned long long *d_sum = (unsigned long long *)(bp<unsigned char>(s->small) + SM_RSUM);
    unsigned long long *hsum = (unsigned long long *)(s->hpin + HP_RSUM);
    std::vector<std::vector<uint32_t>> keep;
    EG_CUDA(cudaMemsetAsync(d_sum, 0, 16 * SV_BFS_SLOTS, st));
    for (int sl = 0; sl < SV_BFS_SLOTS; sl++) {
        if (!((done >> sl) & 1ull)) continue;
        int32_t *row = levels + (uint64_t)sl * n;
        k_sv_level_summary<<<sv_blocks(ctx, n), 256, 0, st>>>(row, n, d_sum + 2 * sl);
        EG_LAUNCHED(ctx);
        if (s->opts.keep_results) {
            keep.emplace_back(n);
            EG_CUDA(cudaMemcpyAsync(keep.back().data(), row, (uint64_t)n * 4, cudaMemcpyDeviceToHost, st));
        }
        EG_CUDA(cudaMemsetAsync(row, 0, (uint64_t)n * 4, st));
    }
    EG_CUDA(cudaMemcpyAsync(hsum, d_sum, 16 * SV_BFS_SLOTS, cudaMemcpyDeviceToHost, st));
    EG_CUDA(cudaStreamSynchronize(st));  // one wait for every retiring slot
    size_t k = 0;
    for (int sl = 0; sl < SV_BFS_SLOTS; sl++) {
        if (!((done >> sl) & 1ull)) continue;
        sv_finish(s, s->bfs_id[sl], EG_Q_BFS, s->bfs_arrival[sl], s->bfs_admit[sl], (uint32_t)hsum[2 * sl],
                  (uint32_t)hsum[2 * sl + 1], s->bfs_level[sl] - 1, 0.0);
        if (s->opts.keep_results) s->kept.push_back(std::move(keep[k++]));
    }
    k_sv_bfs_clear<<<sv_blocks(ctx, n), 256, 0, st>>>(n, ~done, seen, front);
    EG_LAUNCHED(ctx);
    s->bfs_seen_mask &= ~done;
    return EG_OK;
}

static int sv_bfs_advance(eg_server *s, bool *progress, bool launch, bool *launched) {
    bool ready;
    EG_TRY(sv_poll(s, E_BFS, &ready));
    if (ready) {
        const SvCounters *hc = (const SvCounters *)(s->hpin + HP_BCNT);
        const unsigned long long live = s->step_mask[E_BFS];
        s->bfs_count = hc->count;
        s->bfs_fdeg = hc->deg;
        for (int sl = 0; sl < SV_BFS_SLOTS; sl++)
            if ((live >> sl) & 1ull) s->bfs_level[sl] += 1;
        const unsigned long long done = live & ~hc->newmask;  // no discovery this level: finished
        if (done) EG_TRY(sv_bfs_retire(s, done));
        *progress = true;
    }
    if (!launch || s->inflight[E_BFS]) return EG_OK;
    eg_graph *g = s->g;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    cudaStream_t st = s->st[E_BFS];
    unsigned char *small = bp<unsigned char>(s->small);
    SvCounters *bcnt = (SvCounters *)(small + SM_BCNT);
    // admission: FIFO into free slots; with gangs, only while no BFS slot is
    // live, so that the sources of a word advance level by level together
    // (the push and pull steps of slots at different depths cost as much as
    // the deepest one: 5.1 ms per step mixed against ~1.6 ms in step)
    uint32_t *hroots = (uint32_t *)(s->hpin + HP_BADM), *hslots = hroots + 64;
    int nadm = 0;
    unsigned long long taken = 0;
    const double tnow = now_s() - s->t0;
    const bool closed = s->opts.gang && s->bfs_seen_mask != 0ull;
    for (auto it = s->queue.begin(); !closed && it != s->queue.end();) {
        if (it->q.kind != EG_Q_BFS) {
            ++it;
            continue;
        }
        int sl = 0;
        while (sl < s->bfs_cap && (((s->bfs_seen_mask | taken) >> sl) & 1ull)) sl++;
        if (sl >= s->bfs_cap) break;
        taken |= 1ull << sl;
        hroots[nadm] = it->q.source;
        hslots[nadm] = (uint32_t)sl;
        nadm++;
        s->bfs_id[sl] = it->id;
        s->bfs_arrival[sl] = it->q.arrival_s;
        s->bfs_admit[sl] = tnow;
        it = s->queue.erase(it);
    }
    unsigned long long *seen = bp<unsigned long long>(s->bfs_buf);
    unsigned long long *front = seen + n, *next = seen + 2ull * n;
    uint32_t *bq = reinterpret_cast<uint32_t *>(seen + 3ull * n), *bbig = bq + n;
    int32_t *levels = reinterpret_cast<int32_t *>(bbig + n);
    uint32_t *bbigoff = reinterpret_cast<uint32_t *>(levels + (uint64_t)SV_BFS_SLOTS * n);
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    if (nadm) {
        EG_CUDA(cudaMemcpyAsync(small + SM_BROOTS, hroots, (uint64_t)nadm * 4, cudaMemcpyHostToDevice, st));
        EG_CUDA(cudaMemcpyAsync(small + SM_BSLOTS, hslots, (uint64_t)nadm * 4, cudaMemcpyHostToDevice, st));
        k_sv_bfs_admit<<<1, 64, 0, st>>>((const uint32_t *)(small + SM_BROOTS), (const uint32_t *)(small + SM_BSLOTS), nadm,
                                         n, seen, front, levels);
        EG_LAUNCHED(ctx);
        for (int i = 0; i < nadm; i++) {
            s->bfs_seen_mask |= 1ull << hslots[i];
            s->bfs_level[hslots[i]] = 1;
            s->bfs_fdeg += 1;  // keeps the first step of new roots in push mode unless the frontier is large
        }
        s->admitted[E_BFS] += nadm;
        *progress = true;
    }
    const unsigned long long live = s->bfs_seen_mask;
    if (!live) return EG_OK;
    int32_t *hlev = (int32_t *)(s->hpin + HP_BLEVEL);
    memcpy(hlev, s->bfs_level, sizeof(s->bfs_level));
    EG_CUDA(cudaEventRecord(s->ev_begin[E_BFS], st));
    EG_CUDA(cudaMemcpyAsync(small + SM_BLEVEL, hlev, sizeof(s->bfs_level), cudaMemcpyHostToDevice, st));
    EG_CUDA(cudaMemsetAsync(bcnt, 0, sizeof(SvCounters), st));
    const bool pull = (double)s->bfs_count + (double)s->bfs_fdeg > (double)g->m / 20.0;
    if (pull) {
        k_msp_light<<<sv_blocks(ctx, n), 256, 0, st>>>(bp<uint32_t>(g->csc.ptr), bp<uint32_t>(g->csc.col), n, live, seen,
                                                       front, next, bbig, &bcnt->nbig);
        EG_LAUNCHED(ctx);
        k_msp_heavy<<<(uint32_t)ctx->sm_count * 8, 256, 0, st>>>(bp<uint32_t>(g->csc.ptr), bp<uint32_t>(g->csc.col), live,
                                                                 seen, front, next, bbig, &bcnt->nbig);
        EG_LAUNCHED(ctx);
    } else {
        k_sv_front_queue<<<sv_blocks(ctx, n), 256, 0, st>>>(front, n, bq, bcnt);
        EG_LAUNCHED(ctx);
        k_sv_bfs_push<<<(uint32_t)ctx->sm_count * 8, 256, 0, st>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), bq,
                                                                   bcnt, seen, front, next, bbig, bcnt);
        EG_LAUNCHED(ctx);
        k_big_offsets<<<1, 1024, 0, st>>>(bbig, &bcnt->nbig, 1u, bp<uint32_t>(g->csr.ptr), SV_BFS_CHUNK, bbigoff);
        EG_LAUNCHED(ctx);
        k_sv_bfs_push_big<<<(uint32_t)ctx->sm_count * 8, 256, 0, st>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col),
                                                                       bbig, bbigoff, seen, front, next, bcnt);
        EG_LAUNCHED(ctx);
    }
    EG_CUDA(cudaMemsetAsync(bcnt, 0, sizeof(SvCounters), st));
    k_sv_bfs_fold<<<sv_blocks(ctx, n), 256, 0, st>>>(n, seen, front, next, levels, (const int32_t *)(small + SM_BLEVEL),
                                                     deg, bcnt);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemcpyAsync(s->hpin + HP_BCNT, bcnt, sizeof(SvCounters), cudaMemcpyDeviceToHost, st));
    EG_CUDA(cudaEventRecord(s->ev_end[E_BFS], st));
    s->inflight[E_BFS] = true;
    *launched = true;
    s->step_mask[E_BFS] = live;
    *progress = true;
    return EG_OK;
}

// ---- SSSP
static int sv_sssp_retire(eg_server *s, unsigned long long done) {
    eg_graph *g = s->g;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    cudaStream_t st = s->st[E_SSSP];
    uint32_t *dist = bp<uint32_t>(s->sssp_buf);
    unsigned long long *d_sum = (unsigned long long *)(bp<unsigned char>(s->small) + SM_RSUM + 16 * SV_BFS_SLOTS);
    unsigned long long *hsum = (unsigned long long *)(s->hpin + HP_RSUM + 16 * SV_BFS_SLOTS);
    EG_CUDA(cudaMemsetAsync(d_sum, 0, 16 * SV_SSSP_SLOTS, st));
    k_sv_dist_summary<<<sv_blocks(ctx, n), 256, 0, st>>>(dist, n, done, d_sum);
    EG_LAUNCHED(ctx);
    std::vector<std::vector<uint32_t>> keep;
    if (s->opts.keep_results) {
        EG_TRY(eg_buf_ensure(ctx, g->spmv_y, (uint64_t)n * 8));
        uint32_t *col = bp<uint32_t>(g->spmv_y);
        for (int sl = 0; sl < SV_SSSP_SLOTS; sl++) {
            if (!((done >> sl) & 1ull)) continue;
            keep.emplace_back(n);
            k_sv_column<<<sv_blocks(ctx, n), 256, 0, st>>>(dist, n, SV_SSSP_SLOTS, (uint32_t)sl, col);
            EG_LAUNCHED(ctx);
            EG_CUDA(cudaMemcpyAsync(keep.back().data(), col, (uint64_t)n * 4, cudaMemcpyDeviceToHost, st));
            EG_CUDA(cudaStreamSynchronize(st));  // col is reused by the next slot
        }
    }
    EG_CUDA(cudaMemcpyAsync(hsum, d_sum, 16 * SV_SSSP_SLOTS, cudaMemcpyDeviceToHost, st));
    EG_CUDA(cudaStreamSynchronize(st));  // one wait for every retiring slot
    size_t k = 0;
    for (int sl = 0; sl < SV_SSSP_SLOTS; sl++) {
        if (!((done >> sl) & 1ull)) continue;
        sv_finish(s, s->sssp_id[sl], EG_Q_SSSP, s->sssp_arrival[sl], s->sssp_admit[sl], (uint32_t)hsum[2 * sl],
                  (uint32_t)hsum[2 * sl + 1], s->sssp_rounds[sl], 0.0);
        if (s->opts.keep_results) s->kept.push_back(std::move(keep[k++]));
    }
    k_sv_sssp_reset<<<sv_blocks(ctx, (uint64_t)n * SV_SSSP_SLOTS), 256, 0, st>>>(n, done, dist);
    EG_LAUNCHED(ctx);
    s->sssp_mask &= ~done;
    return EG_OK;
}

static int sv_sssp_advance(eg_server *s, bool *progress, bool launch, bool *launched) {
    bool ready;
    EG_TRY(sv_poll(s, E_SSSP, &ready));
    if (ready) {
        const SvCounters *hc = (const SvCounters *)(s->hpin + HP_SCNT);
        const unsigned long long live = s->step_mask[E_SSSP];
        const unsigned long long still = hc->actmask[0] | (hc->actmask[1] << 32);
        for (int sl = 0; sl < SV_SSSP_SLOTS; sl++)
            if ((live >> sl) & 1ull) s->sssp_rounds[sl] += 1;
        const unsigned long long done = live & ~still;
        if (done) EG_TRY(sv_sssp_retire(s, done));
        *progress = true;
    }
    if (!launch || s->inflight[E_SSSP]) return EG_OK;
    eg_graph *g = s->g;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n, nw = (n + 31) / 32;
    cudaStream_t st = s->st[E_SSSP];
    unsigned char *small = bp<unsigned char>(s->small);
    SvCounters *scur = (SvCounters *)(small + SM_SCNT), *snext = (SvCounters *)(small + SM_SNEXT);
    uint32_t *dist = bp<uint32_t>(s->sssp_buf);
    uint32_t *act0 = dist + (uint64_t)n * SV_SSSP_SLOTS, *act1 = act0 + 2ull * n;
    uint32_t *inq0 = act1 + 2ull * n, *inq1 = inq0 + nw;
    uint32_t *sq0 = inq1 + nw, *sq1 = sq0 + n, *sbig = sq1 + n, *sbigoff = sbig + n;
    uint32_t *act[2] = {act0, act1}, *inq[2] = {inq0, inq1}, *sq[2] = {sq0, sq1};
    uint32_t *hroots = (uint32_t *)(s->hpin + HP_SADM), *hslots = hroots + 64;
    int nadm = 0;
    unsigned long long taken = 0;
    const double tnow = now_s() - s->t0;
    // gang admission: a 32-source word with a live source takes no new one
    unsigned long long closed = s->sssp_mask;
    if (s->opts.gang)
        for (int j = 0; j < 2; j++)
            if ((s->sssp_mask >> (32 * j)) & 0xffffffffull) closed |= 0xffffffffull << (32 * j);
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        if (it->q.kind != EG_Q_SSSP) {
            ++it;
            continue;
        }
        int sl = 0;
        while (sl < s->sssp_cap && (((closed | taken) >> sl) & 1ull)) sl++;
        if (sl >= s->sssp_cap) break;
        taken |= 1ull << sl;
        hroots[nadm] = it->q.source;
        hslots[nadm] = (uint32_t)sl;
        nadm++;
        s->sssp_id[sl] = it->id;
        s->sssp_arrival[sl] = it->q.arrival_s;
        s->sssp_admit[sl] = tnow;
        s->sssp_rounds[sl] = 0;
        it = s->queue.erase(it);
    }
    const int c = s->sssp_cur, nx = c ^ 1;
    if (nadm) {
        EG_CUDA(cudaMemcpyAsync(small + SM_SROOTS, hroots, (uint64_t)nadm * 4, cudaMemcpyHostToDevice, st));
        EG_CUDA(cudaMemcpyAsync(small + SM_SSLOTS, hslots, (uint64_t)nadm * 4, cudaMemcpyHostToDevice, st));
        k_sv_sssp_admit<<<1, 64, 0, st>>>((const uint32_t *)(small + SM_SROOTS), (const uint32_t *)(small + SM_SSLOTS),
                                          nadm, dist, act[c], inq[c], sq[c], scur);
        EG_LAUNCHED(ctx);
        for (int i = 0; i < nadm; i++) s->sssp_mask |= 1ull << hslots[i];
        s->admitted[E_SSSP] += nadm;
        *progress = true;
    }
    if (!s->sssp_mask) return EG_OK;
    SvW w = eg_make_wrule(&s->opts.weights);
    const uint32_t *wts = s->wts;
    EG_CUDA(cudaEventRecord(s->ev_begin[E_SSSP], st));
    EG_CUDA(cudaMemsetAsync(snext, 0, sizeof(SvCounters), st));
    k_sv_sssp_push<<<(uint32_t)ctx->sm_count * 8, 256, 0, st>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), wts,
                                                                sq[c], scur, dist, act[c], act[nx], inq[nx], sq[nx], w,
                                                                snext, sbig);
    EG_LAUNCHED(ctx);
    k_big_offsets<<<1, 1024, 0, st>>>(sbig, &snext->nbig, 2u, bp<uint32_t>(g->csr.ptr), SV_SSSP_CHUNK, sbigoff);
    EG_LAUNCHED(ctx);
    k_sv_sssp_push_big<<<(uint32_t)ctx->sm_count * 8, 256, 0, st>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col),
                                                                    wts, dist, act[c], act[nx], inq[nx], sq[nx], w, snext,
                                                                    sbig, sbigoff);
    EG_LAUNCHED(ctx);
    k_sv_sssp_clear_frontier<<<sv_blocks(ctx, n), 256, 0, st>>>(sq[c], scur, act[c], inq[c]);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemcpyAsync(scur, snext, sizeof(SvCounters), cudaMemcpyDeviceToDevice, st));
    EG_CUDA(cudaMemcpyAsync(s->hpin + HP_SCNT, snext, sizeof(SvCounters), cudaMemcpyDeviceToHost, st));
    EG_CUDA(cudaEventRecord(s->ev_end[E_SSSP], st));
    s->sssp_cur = nx;
    s->inflight[E_SSSP] = true;
    *launched = true;
    s->step_mask[E_SSSP] = s->sssp_mask;
    *progress = true;
    return EG_OK;
}

// ---- PPR
static int sv_ppr_advance(eg_server *s, bool *progress, bool launch, bool *launched) {
    bool ready;
    EG_TRY(sv_poll(s, E_PPR, &ready));
    eg_graph *g = s->g;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    cudaStream_t st = s->st[E_PPR];
    unsigned char *small = bp<unsigned char>(s->small);
    PprQ *d_ppr = (PprQ *)(small + SM_PPRQ);
    uint32_t *d_pseeds = (uint32_t *)(small + SM_PSEEDS);
    uint32_t *d_sbeg = (uint32_t *)(small + SM_PSBEG), *d_send = (uint32_t *)(small + SM_PSEND);
    float *R = bp<float>(s->ppr_buf), *X = R + (uint64_t)n * EG_PPR_LANES, *Y = X + (uint64_t)n * EG_PPR_LANES;
    PprQ *hp = s->hq;
    if (ready) {
        uint32_t done = 0;
        for (int q = 0; q < EG_PPR_LANES; q++)
            if (((s->ppr_mask >> q) & 1u) && hp[q].active && hp[q].done) done |= 1u << q;
        double *dsum = (double *)(small + SM_RSUM + 16 * (SV_BFS_SLOTS + SV_SSSP_SLOTS));
        double *hsum = (double *)(s->hpin + HP_RSUM + 16 * (SV_BFS_SLOTS + SV_SSSP_SLOTS));
        std::vector<std::vector<uint32_t>> keep;
        if (done) EG_CUDA(cudaMemsetAsync(dsum, 0, 8 * EG_PPR_LANES, st));
        for (int q = 0; q < EG_PPR_LANES; q++) {
            if (!((done >> q) & 1u)) continue;
            float *col = nullptr;
            if (s->opts.keep_results) {
                EG_TRY(eg_buf_ensure(ctx, g->spmv_y, (uint64_t)n * 8));
                col = bp<float>(g->spmv_y);
                keep.emplace_back(n);
            }
            k_sv_ppr_column<<<sv_blocks(ctx, n), 256, 0, st>>>(R, n, (uint32_t)q, col, dsum + q);
            EG_LAUNCHED(ctx);
            if (col) {
                EG_CUDA(cudaMemcpyAsync(keep.back().data(), col, (uint64_t)n * 4, cudaMemcpyDeviceToHost, st));
                EG_CUDA(cudaStreamSynchronize(st));  // col is reused by the next lane
            }
        }
        if (done) {
            EG_CUDA(cudaMemcpyAsync(hsum, dsum, 8 * EG_PPR_LANES, cudaMemcpyDeviceToHost, st));
            EG_CUDA(cudaStreamSynchronize(st));  // one wait for every retiring lane
        }
        size_t kk = 0;
        for (int q = 0; q < EG_PPR_LANES; q++) {
            if (!((done >> q) & 1u)) continue;
            sv_finish(s, s->ppr_id[q], EG_Q_PPR, s->ppr_arrival[q], s->ppr_admit[q], 0u, 0u, hp[q].iters, hsum[q]);
            if (s->opts.keep_results) s->kept.push_back(std::move(keep[kk++]));
            hp[q].active = 0;
            hp[q].done = 0;
            s->pnseeds[q] = 0;
        }
        s->ppr_mask &= ~done;
        if (done) s->ppr_dirty = true;  // the lane table goes up with the next launch
        *progress = true;
    }
    if (!launch || s->inflight[E_PPR]) return EG_OK;
    uint32_t new_ppr = 0;
    const double tnow = now_s() - s->t0;
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        if (it->q.kind != EG_Q_PPR) {
            ++it;
            continue;
        }
        int sl = 0;
        while (sl < s->ppr_cap && (((s->ppr_mask | new_ppr) >> sl) & 1u)) sl++;
        if (sl >= s->ppr_cap) break;
        const eg_query &q = it->q;
        PprQ &p = hp[sl];
        memset(&p, 0, sizeof(p));
        p.tol = q.tol > 0 ? q.tol : 1e-6f;
        p.max_iters = s->opts.ppr_max_iters;
        p.active = 1;
        p.nseeds = (int)q.nseeds;
        for (uint32_t k = 0; k < q.nseeds; k++) s->pseeds[8 * sl + k] = q.seeds[k];
        s->pnseeds[sl] = q.nseeds;
        new_ppr |= 1u << sl;
        s->ppr_id[sl] = it->id;
        s->ppr_arrival[sl] = q.arrival_s;
        s->ppr_admit[sl] = tnow;
        it = s->queue.erase(it);
    }
    if (new_ppr || s->ppr_dirty) {
        s->ppr_dirty = false;
        uint32_t *hseeds = (uint32_t *)(s->hpin + HP_PSEEDS), *hbeg = hseeds + 256, *hend = hbeg + 32;
        for (int q = 0; q < EG_PPR_LANES; q++) {
            hbeg[q] = 8u * q;
            hend[q] = 8u * q + (hp[q].active ? s->pnseeds[q] : 0u);
            for (int k = 0; k < 8; k++) hseeds[8 * q + k] = s->pseeds[8 * q + k];
        }
        EG_CUDA(cudaMemcpyAsync(d_ppr, hp, sizeof(PprQ) * EG_PPR_LANES, cudaMemcpyHostToDevice, st));
        EG_CUDA(cudaMemcpyAsync(d_pseeds, hseeds, 256 * 4, cudaMemcpyHostToDevice, st));
        EG_CUDA(cudaMemcpyAsync(d_sbeg, hbeg, 32 * 4, cudaMemcpyHostToDevice, st));
        EG_CUDA(cudaMemcpyAsync(d_send, hend, 32 * 4, cudaMemcpyHostToDevice, st));
    }
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    if (new_ppr) {
        k_ppr_init<<<sv_blocks(ctx, (uint64_t)n * 32), 256, 0, st>>>(n, new_ppr, R, X);
        EG_LAUNCHED(ctx);
        k_ppr_init_seeds<<<1, 32, 0, st>>>(d_pseeds, d_sbeg, d_send, new_ppr, d_ppr, deg, R, X);
        EG_LAUNCHED(ctx);
        k_ppr_init_dangling<<<1, 32, 0, st>>>(d_pseeds, d_sbeg, d_send, new_ppr, deg, R, d_ppr);
        EG_LAUNCHED(ctx);
        s->ppr_mask |= new_ppr;
        s->admitted[E_PPR] += __builtin_popcount(new_ppr);
        *progress = true;
    }
    if (!s->ppr_mask) return EG_OK;
    const uint32_t pm = (uint32_t)g->m;
    const uint32_t ptiles = pm ? eg_div_up(pm, EG_PPR_TILE) : 0;
    float *phv = Y + (uint64_t)n * EG_PPR_LANES, *ptv = phv + (uint64_t)ptiles * EG_PPR_LANES;
    uint32_t *phr = reinterpret_cast<uint32_t *>(ptv + (uint64_t)ptiles * EG_PPR_LANES);
    double2 *ppart = reinterpret_cast<double2 *>(phr + ((ptiles + 63) & ~63u));
    const uint32_t fb = (uint32_t)ctx->sm_count * 4;
    const uint32_t rb = ptiles ? eg_div_up((uint64_t)ptiles * 32, 256) : 0;
    EG_CUDA(cudaEventRecord(s->ev_begin[E_PPR], st));
    if (rb) {
        k_ppr_rows<<<rb, 256, 0, st>>>(bp<uint32_t>(g->csc.rid), bp<uint32_t>(g->csc.col), pm, ptiles, X, Y, phv, ptv, phr);
        EG_LAUNCHED(ctx);
        k_ppr_fixup<<<rb, 256, 0, st>>>(bp<uint32_t>(g->csc.ptr), ptiles, phr, phv, ptv, Y);
        EG_LAUNCHED(ctx);
    }
    k_ppr_empty<<<(uint32_t)ctx->sm_count * 8, 256, 0, st>>>(bp<uint32_t>(g->csc.ptr), n, Y);
    EG_LAUNCHED(ctx);
    k_ppr_seeds<<<1, 32, 0, st>>>(d_pseeds, d_sbeg, d_send, 32, d_ppr, s->opts.ppr_damping, Y);
    EG_LAUNCHED(ctx);
    k_ppr_finish<<<fb, 256, 0, st>>>(Y, deg, n, s->opts.ppr_damping, d_ppr, R, X, ppart);
    EG_LAUNCHED(ctx);
    k_ppr_reduce<<<1, 32, 0, st>>>(ppart, fb, d_ppr, 1);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemcpyAsync(hp, d_ppr, sizeof(PprQ) * EG_PPR_LANES, cudaMemcpyDeviceToHost, st));
    EG_CUDA(cudaEventRecord(s->ev_end[E_PPR], st));
    s->inflight[E_PPR] = true;
    *launched = true;
    s->step_mask[E_PPR] = s->ppr_mask;
    *progress = true;
    return EG_OK;
}

// One scheduler pass: every engine whose step has finished is retired,
// refilled and relaunched.  When no engine was ready the call waits briefly
// (about a millisecond at most) so that a polling caller does not spin the host.
extern "C" int eg_serve_step(eg_server *s, int *active_out) {
    if (!s) return eg_fail(EG_EINVAL, "NULL server");
    EG_CUDA(cudaSetDevice(s->g->ctx->device));
    s->ticks++;
    bool progress = false;
    typedef int (*advance_fn)(eg_server *, bool *, bool, bool *);
    static const advance_fn adv[3] = {sv_bfs_advance, sv_sssp_advance, sv_ppr_advance};
    for (int spin = 0; spin < 20 && !progress; spin++) {
        bool launched = false;
        for (int e = 0; e < 3; e++) EG_TRY(adv[e](s, &progress, false, &launched));  // retire finished steps
        for (int t = 0; t < 3; t++) {  // refill and launch, engines taking turns first
            const int e = (s->turn + t) % 3;
            if (s->opts.exclusive && (s->inflight[E_BFS] || s->inflight[E_SSSP] || s->inflight[E_PPR])) break;
            launched = false;
            EG_TRY(adv[e](s, &progress, true, &launched));
            if (launched) s->turn = (e + 1) % 3;
        }
        if (!progress) {
            if (!s->inflight[E_BFS] && !s->inflight[E_SSSP] && !s->inflight[E_PPR]) break;  // idle
            struct timespec ts = {0, 1000};
            nanosleep(&ts, nullptr);
        }
    }
    if (active_out)
        *active_out = __builtin_popcountll(s->bfs_seen_mask) + __builtin_popcountll(s->sssp_mask) +
                      __builtin_popcount(s->ppr_mask) + (int)s->queue.size();
    return EG_OK;
}

extern "C" int eg_serve_stats(eg_server *s, eg_serve_stats_t *out) {
    if (!s || !out) return eg_fail(EG_EINVAL, "NULL argument");
    memset(out, 0, sizeof(*out));
    out->ticks = s->ticks;
    for (int e = 0; e < 3; e++) {
        out->engine_ms[e] = s->eng_ms[e];
        out->engine_steps[e] = s->eng_steps[e];
        out->admitted[e] = s->admitted[e];
        out->completed[e] = s->completed[e];
    }
    out->queued = s->queue.size();
    return EG_OK;
}

extern "C" int eg_serve_poll(eg_server *s, eg_query_result *out, int max, int *count) {
    if (!s || !count) return eg_fail(EG_EINVAL, "NULL argument");
    int c = (int)s->done.size();
    if (c > max) c = max;
    for (int i = 0; i < c; i++) out[i] = s->done[i];
    s->done.erase(s->done.begin(), s->done.begin() + c);
    *count = c;
    return EG_OK;
}

extern "C" int eg_serve_take_result(eg_server *s, uint32_t *out, uint32_t n) {
    if (!s || !out) return eg_fail(EG_EINVAL, "NULL argument");
    if (s->kept.empty()) return eg_fail(EG_EINVAL, "no kept result (keep_results off or none left)");
    if (n != s->g->n) return eg_fail(EG_EINVAL, "buffer holds %u, the graph has %u vertices", n, s->g->n);
    memcpy(out, s->kept.front().data(), (size_t)n * 4);
    s->kept.erase(s->kept.begin());
    return EG_OK;
}

extern "C" int eg_serve_info(eg_server *s, int *bfs_slots, int *sssp_slots, int *ppr_slots, double *clock_s) {
    if (!s) return eg_fail(EG_EINVAL, "NULL server");
    if (bfs_slots) *bfs_slots = s->bfs_cap;
    if (sssp_slots) *sssp_slots = s->sssp_cap;
    if (ppr_slots) *ppr_slots = s->ppr_cap;
    if (clock_s) *clock_s = now_s() - s->t0;
    return EG_OK;
}
