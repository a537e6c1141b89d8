// Internal declarations shared by the CUDA translation units of libeg_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "eg_gpu.h"

#define EG_FULL_MASK 0xffffffffu
#define EG_TROW_SPAN 512  // entries per row-of-entry sample (eg_graph::csc_p_trow)
#define EG_STARTS_PAD 8   // zero words after the row-start bits

// ---------------------------------------------------------------- errors
int eg_fail(int code, const char *fmt, ...);
void eg_clear_error();

#define EG_CUDA(call)                                                                               \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return eg_fail(EG_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
    } while (0)

#define EG_TRY(call)                 \
    do {                             \
        int rc_ = (call);            \
        if (rc_ != EG_OK) return rc_; \
    } while (0)

// Checks the last launch and counts it.
#define EG_LAUNCHED(ctx)                                                                           \
    do {                                                                                           \
        (ctx)->launches++;                                                                         \
        cudaError_t e_ = cudaGetLastError();                                                       \
        if (e_ != cudaSuccess)                                                                     \
            return eg_fail(EG_ECUDA, "%s:%d launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_)); \
    } while (0)

// ---------------------------------------------------------------- context
#define EG_KEV 8        // kernel launches timed individually per call
#define EG_OUT_SLOTS 4  // device output slots of eg_bfs_batch (copy-out pipeline depth)
#define EG_SB_MAX 64    // source blocks of the blocked CSC at most
struct eg_ctx {
    int device;
    int sm_count;
    cudaStream_t stream;
    uint64_t budget;
    uint64_t in_use;
    uint64_t launches;
    void *h_pinned;      // 1 MiB pinned staging for small readbacks
    void *h_pinned_dev;  // the same memory as the device addresses it
    cudaEvent_t ev0, ev1;
    cudaEvent_t evk[2 * EG_KEV];  // begin/end pairs around single kernel launches
    int live_graphs;              // eg_close refuses while graphs are alive
    cudaStream_t copy_stream;     // device-to-host copies overlapped with the next traversal
    cudaEvent_t ev_out[2 * EG_OUT_SLOTS];  // [slot]: outputs ready, [EG_OUT_SLOTS + slot]: copied out
    uint32_t rb_seq = 0;                   // eg_readback_wait: the last flag value asked for
};
// eg_readback_wait's flag word: the last 64 bytes of the pinned staging area
#define EG_RB_FLAG_OFF ((1u << 20) - 64u)

int eg_dmalloc(eg_ctx *ctx, void **p, uint64_t bytes);
void eg_dfree(eg_ctx *ctx, void *p, uint64_t bytes);

// A device buffer tracked against the context budget.
struct eg_buf {
    void *p = nullptr;
    uint64_t bytes = 0;
};
int eg_buf_ensure(eg_ctx *ctx, eg_buf &b, uint64_t bytes);  // grows (contents lost)
// Small device-to-host readback into ctx->h_pinned (host_dst lies in it) by a
// one-warp kernel on `st` instead of a copy engine, so that it does not queue
// behind large copies another stream has on the engine.  Valid on the host
// after `st` is synchronised.
// With `clear` the kernel also zeroes the device words after reading them.
int eg_readback(eg_ctx *ctx, void *host_dst, const void *dev_src, uint32_t bytes, cudaStream_t st,
                bool clear = false);
// The same, and returns once the words are on the host: the kernel raises a
// flag in pinned memory after them and the host polls it (no stream
// synchronisation per call).  The poll gives up after a second and falls back
// to synchronising `st`, which reports any device error.
int eg_readback_wait(eg_ctx *ctx, void *host_dst, const void *dev_src, uint32_t bytes, cudaStream_t st,
                     bool clear = false);
// Zeroes `bytes` (a multiple of 4, 4-byte aligned) of device memory with a
// kernel, for the same reason: a memset may be carried out by a copy engine.
int eg_zero(eg_ctx *ctx, void *dev, uint64_t bytes, cudaStream_t st);
void eg_buf_free(eg_ctx *ctx, eg_buf &b);
template <class T>
static inline T *bp(const eg_buf &b) {
    return (T *)b.p;
}

// ---------------------------------------------------------------- graph
struct eg_adj {
    eg_buf ptr;  // uint32[n+1]
    eg_buf col;  // uint32[m]
    eg_buf rid;  // uint32[m]: row of each entry (COO form), kept from the sort
};


// A BFS level loop captured as a CUDA graph with a device-side while node,
// valid while the buffers it was captured with (key) stay in place.
struct eg_bfs_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void *key[8] = {};
};

// A copy of an adjacency with its entries split by source block (for row
// sums over an x larger than L2): block b holds the len[b] entries with
// source in [b << shift, (b+1) << shift), in the adjacency's order, from
// entry start[b] (a multiple of 4: the row kernel reads 16-byte vectors from
// the block's base); ptr holds one row-pointer array of n + 1 per block;
// perm[i] is the adjacency entry placed at i (for values kept per entry).
struct eg_sblocks {
    uint32_t shift = 0, blocks = 0;
    eg_buf ptr, rid, col, perm, vals, yerr;
    uint64_t start[EG_SB_MAX] = {}, len[EG_SB_MAX] = {};
    int vals_kind = 0;
    uint64_t vals_seed = 0;
};

// PageRank's destination-partition layout of the relabelled CSC (eg_pcol.cu):
// the rows with entries are cut into partitions of 2^shift rows; inside a
// partition the entries are ordered by source (then row), so each source's
// entries into the partition form one run whose contribution is gathered
// once.  Partitions start at chunk boundaries (EG_PC_CHUNK entries); the
// entries past a partition's last (up to the next chunk) are padding that
// adds into row 2^shift, a slot outside the partition.
#define EG_PC_CHUNK 256
struct eg_pcols {
    uint32_t shift = 0;  // 0: not built
    uint32_t parts = 0, segs = 0;
    uint64_t chunks = 0, runs = 0;
    eg_buf dst;     // uint16[chunks * EG_PC_CHUNK]: the entry's row within its partition
    eg_buf ridx;    // uint8[chunks * EG_PC_CHUNK]: each entry's run within its chunk, transposed like dst
    eg_buf crun;    // uint32[chunks]: run of each chunk's first entry
    eg_buf rsrc;    // uint32[runs]: source of each run
    eg_buf seg;     // uint4[segs] (first chunk, end chunk, partition, segments of that partition), longest first
    eg_buf acc;     // uint64[rows with entries]: sums of the partitions split over several segments
    eg_buf ticket;  // uint32[parts + 2]: segments finished per partition; [parts]: the next segment to take; [parts + 1]: CTAs done
};

struct eg_graph {
    eg_ctx *ctx;
    uint32_t n;
    uint64_t m_in;  // input edges
    uint64_t m;     // adjacency entries
    unsigned flags;
    unsigned built;
    float build_ms;
    eg_buf pairs;  // uint32[2*m_in]
    eg_adj csr, csc;
    eg_buf out_deg, in_deg;  // uint32[n]
    // PageRank's copy of the CSC with vertices relabelled by descending
    // out-degree (hot sources contiguous), the vertices without in-edges
    // last: perm[old] = new, deg_p[new]; rows [csc_p_rows, n) have no entries
    eg_adj csc_p;
    eg_buf perm, deg_p;
    bool relabeled = false;
    uint32_t csc_p_rows = 0;
    // csc_p's rows as row-start bits (1 per entry, EG_STARTS_PAD zero words
    // after them) and the row of every EG_TROW_SPAN-th entry: the row kernel's
    // compact form of the row-id stream (valid because rows 0 .. csc_p_rows-1
    // all have entries)
    eg_buf csc_p_starts, csc_p_trow;
    // edge array (load modes 7, 8, 9): sources and destinations of every
    // adjacency entry in the order edge_order (EG_EDGES_*), and the
    // edge-centric BFS's bitmaps and counters
    eg_buf esrc, edst, edge_work;
    int edge_order = -1;
    // grid
    uint32_t grid_p;
    eg_buf cell_ptr, gsrc, gdst;
    // grid SpMV/PageRank: cell visiting order, work-unit offsets, edge values,
    // accumulators (eg_grid.cu)
    eg_buf grid_order, grid_units, grid_off, grid_vals, grid_acc;
    uint32_t grid_order_p = 0, grid_block = 0;
    int grid_vals_kind = 0;
    uint64_t grid_vals_seed = 0;
    // algorithm state, allocated on first use and reused
    eg_buf rank, rank_p, rank_q, contrib0, contrib1, pr_part, pr_stats, mp_carry, errflag;
    eg_buf pr_acc;  // PageRank over source blocks: the row sums of the blocks before the last
    eg_buf level, parent, dist, label, spmv_x, spmv_y, spmv_vals;
    eg_buf level_s[EG_OUT_SLOTS - 1], parent_s[EG_OUT_SLOTS - 1];  // output slots 1.. of eg_bfs_batch
    eg_buf first_in;                  // BFS pull: each vertex's first in-neighbour (0xffffffff: none)
    const void *first_in_src = nullptr;  // the in-list column array first_in was taken from
    // WCC: the vertices with an edge (out- or in-list not empty), listed once
    // per layout so that the hooking rounds give no thread to an isolated one
    eg_buf wcc_list;
    uint32_t wcc_list_n = 0;
    const void *wcc_list_src = nullptr;  // the CSR row pointers the list was taken from
    uint64_t spmv_vals_seed;
    int spmv_vals_kind;
    eg_sblocks sb;   // source-blocked copy of the CSC (fp32 SpMV over an x larger than L2)
    eg_sblocks sbp;  // the same of the relabelled CSC (PageRank)
    eg_pcols pcol;   // the relabelled CSC by destination partition and source (PageRank)
    int pr_kernel = 0;  // PageRank's one-pass kernel: 0 the row kernel (row_cfg), 1 the partition kernel
    eg_buf bfs_work;  // bitmaps, queues, counters
    eg_buf msbfs_work;
    eg_buf sssp_work;
    eg_buf ppr_work;
    eg_bfs_graph bfsg[2 * EG_OUT_SLOTS];  // [slot * 2 + with parents]
    eg_bfs_graph prg;      // PageRank iterations (key: options and buffers)
    eg_bfs_graph msg;      // multi-source BFS level loop
    eg_bfs_graph ssg;      // batched SSSP round loop
    eg_bfs_graph ppg;      // batched personalised PageRank sweep loop
    int row_cfg = 0;       // row-kernel schedule (entries per warp tile, per lane)
    int bfs_host_loop = 0; // BFS level-loop form eg_bfs uses by default (eg_graph_tune)
    double bfs_divisor = 40.0;  // push/pull switch divisor eg_bfs uses by default (the reference's rule; eg_graph_tune)
    // SSSP edge weights of the CSR entries for one rule, materialised on first
    // use (the reference stores them in its edge records, init_all.c:661-686)
    eg_buf wts;
    uint64_t wts_key[3] = {~0ull, ~0ull, ~0ull};
    uint64_t prk[16] = {};
};

// ---------------------------------------------------------------- helpers
static inline uint32_t eg_div_up(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

// device scan: out[i] = sum_{j<i} in[j] for i in [0, len]; out has len+1
// entries (the last is the total).  in may equal out only if len+1 fits.
int eg_exscan_u32(eg_ctx *ctx, const uint32_t *in, uint32_t *out, uint64_t len);
// histogram of keys (values < n) into zeroed hist[n]
int eg_histogram(eg_ctx *ctx, const uint32_t *keys, uint64_t len, uint32_t *hist);
// stable LSD radix sort of (key, value) pairs by the low `bits` bits of key.
// Sorted data ends in (k_out, v_out); the input arrays are overwritten.
int eg_radix_sort(eg_ctx *ctx, uint32_t *k_in, uint32_t *v_in, uint32_t *k_tmp, uint32_t *v_tmp, uint64_t len,
                  int bits, uint32_t **k_out, uint32_t **v_out);
// builds g->csc_p / perm / deg_p from the CSC and out-degrees (once)
int eg_build_relabeled_csc(eg_graph *g);
// builds g->pcol with partitions of 2^shift rows from g->csc_p (once per shift)
int eg_build_pcols(eg_graph *g, uint32_t shift);

// ---------------------------------------------------------------- device utils
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t eg_lanemask_lt() {
    uint32_t r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t eg_ldg_nc(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
// SplitMix64 output function (Steele, Lea & Flood, OOPSLA 2014); the same
// counter scheme as the CPU generator.
__host__ __device__ __forceinline__ uint64_t eg_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t eg_key(uint64_t seed, uint64_t idx) {
    return eg_mix64(eg_mix64(seed) ^ idx);
}
__host__ __device__ __forceinline__ uint64_t eg_draw(uint64_t key, uint64_t j) {
    return eg_mix64(key + j * 0x632BE59BD9B4E019ull);
}
// Symmetric per-edge hash of the endpoints, for weight and value rules.
__host__ __device__ __forceinline__ uint64_t eg_edge_hash(uint64_t seed, uint32_t u, uint32_t v) {
    uint32_t a = u < v ? u : v, b = u < v ? v : u;
    return eg_draw(eg_key(seed, ((uint64_t)a << 32) | b), 0);
}

// Two running sums (e.g. a residual and a dangling mass) kept by one thread
// as fp32 (sum, error) pairs (Knuth's TwoSum) and widened to FP64 once per
// thread before the FP64 block reduction.  FP64 instructions issue at a small
// fraction of the fp32 rate on this GPU, and per-row sums often run in
// divergent code (one lane per finished row), so per-row FP64 adds would
// dominate the kernels that carry them.
struct eg_red2 {
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
    __device__ __forceinline__ static void two_sum(float &s, float &c, float x) {
        const float t = s + x;
        const float bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
    }
    __device__ __forceinline__ void add(float2 d) {
        two_sum(s0, c0, d.x);
        two_sum(s1, c1, d.y);
    }
    __device__ __forceinline__ double2 wide() const {
        return make_double2((double)s0 + (double)c0, (double)s1 + (double)c1);
    }
};

// SSSP edge weights computed from the endpoints (no weight array), and the
// extension of a path distance by one edge in the rule's encoding: u32 sums
// saturating at EG_SSSP_INF, or fp32 sums (bit patterns, which order like
// the values for non-negative floats; unreached = +inf).
#define EG_SSSP_INF 0xfffffffeu
#define EG_SSSP_INF_F32 0x7f800000u
struct eg_wrule {
    int rule;
    uint64_t seed;
    uint32_t lo;
    uint64_t span;
    __host__ __device__ __forceinline__ uint32_t inf() const {
        return rule == EG_W_HASH_F32 ? EG_SSSP_INF_F32 : EG_SSSP_INF;
    }
    // the edge's weight in the rule's encoding (fp32 bits for EG_W_HASH_F32)
    __device__ __forceinline__ uint32_t weight(uint32_t u, uint32_t v) const {
        if (rule == EG_W_HASH_F32)
            return __float_as_uint((float)((eg_edge_hash(seed, u, v) >> 40) + 1) * (1.0f / 16777216.0f));
        if (rule == EG_W_REF) return (u % 10u) + (v % 10u);
        if (rule == EG_W_UNIT) return 1u;
        return lo + (uint32_t)(((eg_edge_hash(seed, u, v) >> 32) * span) >> 32);
    }
    // path distance du extended by an edge of weight w
    __device__ __forceinline__ uint32_t add(uint32_t du, uint32_t w) const {
        if (rule == EG_W_HASH_F32) return __float_as_uint(__fadd_rn(__uint_as_float(du), __uint_as_float(w)));
        const uint64_t nd = (uint64_t)du + w;
        return nd < EG_SSSP_INF ? (uint32_t)nd : EG_SSSP_INF;
    }
    __device__ __forceinline__ uint32_t extend(uint32_t du, uint32_t u, uint32_t v) const { return add(du, weight(u, v)); }
};
struct eg_graph;
// Times eg_bfs's two level-loop forms on a few sampled roots (eg_bfs.cu).
int eg_bfs_tune(eg_graph *g, float *ms_graph, float *ms_host, int *host_loop, double *divisor);
// SpMV / PageRank over the 2-D grid layout (eg_grid.cu).
int eg_grid_spmv(eg_graph *g, int kind, uint64_t value_seed, int unit_values, const void *d_x, void *d_y);
int eg_grid_pagerank(eg_graph *g, const eg_pr_opts &o, float *rank_out, eg_pr_stats *stats);
// The CSR-order weight array of rule w, computed once per rule and kept in
// the graph (replaced when another rule is asked for).
int eg_edge_weights(eg_graph *g, const eg_wrule &w, const uint32_t **out);
// Writes rule w's CSR-order weights to out[m] on the context's stream.
int eg_fill_weights(eg_graph *g, const eg_wrule &w, uint32_t *out);
static inline eg_wrule eg_make_wrule(const eg_weights *w) {
    eg_wrule r;
    r.rule = w ? w->rule : EG_W_REF;
    r.seed = w ? w->seed : 0;
    r.lo = w ? w->lo : 0;
    r.span = w ? (uint64_t)w->hi - w->lo + 1 : 1;
    return r;
}
#endif
