// Pull PageRank, personalised PageRank (one query) and SpMV as row
// reductions over the CSC (or CSR), plus the row-schedule autotuner.
//
// Replaces pr_algo_pull and its iterator (pagerank_simple.c:72-84,110-133),
// the grid PR loop (prgrid_cilk.c:62-76,111-141) whose per-destination sum
// order equals the CSC order (the grid-cell form is eg_grid.cu), and the SpMV
// loops (spmv.c:98-135).
//
// PageRank runs on a copy of the CSC whose vertices are relabelled by
// descending out-degree (built once, eg_build_relabeled_csc): the most
// gathered contrib entries are then contiguous, so they share cache sectors
// and stay in L1; ranks are mapped back to the original ids at the end.
// Vertices without in-edges come last in that order, so the rows without
// entries are one range that needs no row-pointer scan.
// Per PageRank iteration the device runs:
//   k_coov_rows<PrOp>      rank[v] = base + d * sum_{u in in(v)} contrib[u],
//                          contrib'[v] = rank[v] / deg[v] (fused into the write);
//                          warp tiles of row-id/column pairs (eg_mp.cuh)
//   k_coo_empty_range, k_coo_fixup  rows without entries, rows split between tiles
//   k_pr_residual          (with a tolerance) the L1 change, coalesced
//   k_pr_reduce            FP64 residual / dangling mass -> next base, stop flag
// contrib[u] = prev[u] / (float)deg[u] is the reference's per-edge quotient
// (pagerank_simple.c:78), computed once per vertex instead of once per edge.
// Algorithmic bytes per iteration: 8 per entry (row id + column) and 16 per
// vertex (gathered contribution, degree, rank write, contribution write).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "eg_mp.cuh"
#include "eg_pcol.cuh"

// ============================================================== merge-path schedule (eg_noalloc.cu)
__global__ void k_mp_schedule(const uint32_t *__restrict__ ptr, uint32_t n, uint32_t m, uint32_t items,
                              uint32_t ntiles, uint2 *__restrict__ coord) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > ntiles) return;
    uint64_t total = (uint64_t)n + m;
    uint64_t diag = (uint64_t)c * items;
    if (diag > total) diag = total;
    // merge-path search: first row index i such that ptr[i+1] > diag - i - 1
    uint64_t lo = diag > m ? diag - m : 0, hi = diag < n ? diag : n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if ((uint64_t)ptr[mid + 1] <= diag - mid - 1) lo = mid + 1;
        else hi = mid;
    }
    coord[c] = make_uint2((uint32_t)lo, (uint32_t)(diag - lo));
}

// ============================================================== PR state
struct eg_pr_dev {
    float base;   // (1-d)/n (+ d * dangling / n)
    int done;     // converged: remaining launches return at once
    int iters;    // iterations that ran
    int pad;
    double residual;
    double dangling;
};

// Teleport set of a single personalised PageRank query: up to
// EG_PPR1_SEEDS distinct vertices (relabelled ids) with their multiplicity.
#define EG_PPR1_SEEDS 8
struct PprSeeds {
    uint32_t count;  // distinct seeds; 0 = uniform teleport (plain PageRank)
    uint32_t id[EG_PPR1_SEEDS];
    float mult[EG_PPR1_SEEDS];
    __device__ __forceinline__ float weight(uint32_t v) const {
        float w = 0.f;
#pragma unroll
        for (int i = 0; i < EG_PPR1_SEEDS; i++)
            if (i < (int)count && v == id[i]) w = mult[i];
        return w;
    }
};

template <bool COMP>
struct PrOp {
    using V = float;
    using A = typename std::conditional<COMP, float2, float>::type;
    const float *__restrict__ cin;
    float *__restrict__ rank;
    float *__restrict__ cout;
    const uint32_t *__restrict__ deg;
    const eg_pr_dev *st;
    uint32_t mult;
    float damping;
    float base;
    PprSeeds seeds;
    const float *__restrict__ acc_in;  // source blocks: the earlier blocks' row sums (else NULL)
    __device__ __forceinline__ bool active() const { return st->done == 0; }
    __device__ __forceinline__ void setup() { base = st->base; }
    __device__ __forceinline__ V gather(uint32_t, uint32_t u) const { return __ldg(cin + u); }
    __device__ __forceinline__ A zero() const {
        if constexpr (COMP) return make_float2(0.f, 0.f);
        else return 0.f;
    }
    __device__ __forceinline__ A add(A a, V x) const {
        if constexpr (COMP) return eg_f2sum::add(a, x);
        else return a + x;
    }
    __device__ __forceinline__ A merge(A a, A b) const {
        if constexpr (COMP) return eg_f2sum::merge(a, b);
        else return a + b;
    }
    __device__ __forceinline__ float2 emit(uint32_t v, A s) const {
        float sum;
        if constexpr (COMP) sum = s.x + s.y;
        else sum = s;
        if (acc_in) sum = acc_in[v] + sum;
        // teleport: base on every vertex, or base x multiplicity on the seeds
        const float b = seeds.count ? base * seeds.weight(v) : base;
        float r = fmaf(damping, sum, b);
        rank[v] = r;
        uint32_t d = deg[v] * mult;
        cout[v] = d ? __fdiv_rn(r, (float)d) : 0.f;
        return make_float2(0.f, d ? 0.f : r);  // (residual: k_pr_residual, dangling mass)
    }
};

// PageRank's row sums over the source blocks before the last one: acc[v] =
// the sum of contrib[u] over v's entries in the blocks so far.
struct PrAccOp {
    using V = float;
    using A = float;
    const float *__restrict__ cin;
    float *__restrict__ acc;
    const eg_pr_dev *st;
    int accum;  // 1: add to acc (blocks after the first)
    __device__ __forceinline__ bool active() const { return st->done == 0; }
    __device__ __forceinline__ void setup() {}
    __device__ __forceinline__ V gather(uint32_t, uint32_t u) const { return __ldg(cin + u); }
    __device__ __forceinline__ A zero() const { return 0.f; }
    __device__ __forceinline__ A add(A a, V x) const { return a + x; }
    __device__ __forceinline__ A merge(A a, A b) const { return a + b; }
    __device__ __forceinline__ float2 emit(uint32_t v, A s) const {
        acc[v] = accum ? acc[v] + s : s;
        return make_float2(0.f, 0.f);
    }
};

// rank = prev_init, contrib = prev_init / deg; partial dangling mass
__global__ void k_pr_init(uint32_t n, float prev_init, const uint32_t *__restrict__ deg, uint32_t mult,
                          float *__restrict__ rank, float *__restrict__ contrib, double2 *__restrict__ part) {
    __shared__ double s_red[8];
    double dang = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        uint32_t d = deg[v] * mult;
        rank[v] = prev_init;
        contrib[v] = d ? __fdiv_rn(prev_init, (float)d) : 0.f;
        if (!d) dang += (double)prev_init;
    }
    for (int o = 16; o > 0; o >>= 1) dang += __shfl_down_sync(EG_FULL_MASK, dang, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = dang;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += s_red[w];
        part[blockIdx.x] = make_double2(0.0, s);
    }
}

// Personalised start vector: multiplicity / total seeds on the seeds, 0 elsewhere.
__global__ void k_ppr1_init(uint32_t n, PprSeeds seeds, float inv_total, const uint32_t *__restrict__ deg,
                            float *__restrict__ rank, float *__restrict__ contrib, double2 *__restrict__ part) {
    __shared__ double s_red[8];
    double dang = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = deg[v];
        const float r = seeds.weight(v) * inv_total;
        rank[v] = r;
        contrib[v] = d ? __fdiv_rn(r, (float)d) : 0.f;
        if (!d) dang += (double)r;
    }
    for (int o = 16; o > 0; o >>= 1) dang += __shfl_down_sync(EG_FULL_MASK, dang, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = dang;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
        part[blockIdx.x] = make_double2(0.0, t);
    }
}

// L1 change between two rank vectors, per-block FP64 partials in .x (the
// stop test's residual); skipped once the run has converged.
__global__ void k_pr_residual(const float *__restrict__ cur, const float *__restrict__ prev, uint32_t n,
                              const eg_pr_dev *st, double2 *__restrict__ part) {
    __shared__ double s_red[8];
    if (st->done) return;
    eg_red2 acc;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        acc.add(make_float2(fabsf(__ldg(cur + v) - __ldg(prev + v)), 0.f));
    double r = acc.wide().x;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(EG_FULL_MASK, r, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
        part[blockIdx.x] = make_double2(t, 0.0);
    }
}

__global__ void k_map_ids(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ in, uint32_t k,
                          uint32_t *__restrict__ out) {
    for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) out[i] = perm[in[i]];
}

// Iteration `it` writes its ranks to buffer B when `it` is even and to A when
// it is odd (the start vector is in A), so the last iteration that ran (the
// stop test may end the run early) left its ranks in B if st->iters is odd.
__global__ void k_pr_unpermute(const float *__restrict__ rank_a, const float *__restrict__ rank_b,
                               const eg_pr_dev *st, const uint32_t *__restrict__ perm, uint32_t n,
                               float *__restrict__ rank) {
    const float *src = (st->iters & 1) ? rank_b : rank_a;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) rank[v] = src[perm[v]];
}

// One block: deterministic FP64 sum of the partials, next base, stop test.
__global__ void k_pr_reduce(const double2 *__restrict__ part, uint32_t nparts, eg_pr_dev *st, double tele_div,
                            float damping, int dangling, double tol, int count_iter) {
    __shared__ double2 s[256];
    if (st->done) return;
    double2 acc = make_double2(0.0, 0.0);
    for (uint32_t i = threadIdx.x; i < nparts; i += blockDim.x) {
        acc.x += part[i].x;
        acc.y += part[i].y;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s[threadIdx.x].x += s[threadIdx.x + w].x;
            s[threadIdx.x].y += s[threadIdx.x + w].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double res = s[0].x, dang = s[0].y;
        st->residual = res;
        st->dangling = dang;
        double b = (1.0 - (double)damping) / tele_div;
        if (dangling) b += (double)damping * dang / tele_div;
        st->base = (float)b;
        if (count_iter) {
            st->iters += 1;
            if (tol > 0.0 && res < tol) st->done = 1;
        }
    }
}

// Row-id stream kernel (k_coov_rows): one warp per TILE entries, U entries
// per lane.  part[] receives per-CTA partials of the main kernel, then of the
// empty-row kernel, then of the fix-up; returns their count.  The schedule
// (TILE, U, ...) is the graph's row_cfg, picked by eg_graph_tune; `hint`
// keeps the streamed row ids and columns out of L1 and first in line for L2
// eviction.
#define EG_COO_TILE_MIN 512
#define EG_ALL_ENTRIES (~0ull)
#define EG_NO_RANGE 0xffffffffu  // coo_launch: rows without entries found from the row pointers
#define EG_SB_LOG2 24  // source-block size by default: 2^24 vertices, a 64 MB slice of x
#define EG_PR_CHECK 4  // iterations between reads of the stop flag
#define EG_PR_RES_BLOCKS 1024
#define EG_ROW_CFGS 12
struct RowCfg {
    int tile, u, pf, minb, hint;
};
// pf: 0 no prefetch, 1 next chunk's words loaded ahead, 2 also its gathers
// issued before the current chunk's scan.  min_blocks bounds the registers:
// 6 resident CTAs of 256 threads leave 42 registers per thread, 5 leave 51,
// 4 leave 64, 8 leave 32.
static const RowCfg kRowCfg[EG_ROW_CFGS] = {
    {1024, 4, 1, 5, 0}, {2048, 4, 0, 6, 0}, {2048, 4, 1, 5, 0}, {1024, 4, 1, 6, 0}, {512, 4, 1, 5, 0},
    {1024, 8, 1, 4, 0}, {1024, 4, 0, 8, 0}, {2048, 8, 0, 5, 0}, {1024, 4, 1, 5, 1}, {2048, 4, 1, 5, 1},
    {1024, 4, 2, 4, 0}, {2048, 4, 2, 4, 0}};

template <class Op, int TILE, int U, bool REDUCE, int PF, int MINB, int HINT = 0, bool MK = false>
static int coo_launch_t(eg_graph *g, eg_adj &adj, eg_buf &carry_buf, double2 *part, const Op &op, uint32_t *nparts,
                        cudaEvent_t ev_begin, cudaEvent_t ev_end, uint64_t m_entries, bool empty_rows,
                        uint32_t empty_from) {
    static_assert(!MK || TILE % EG_TROW_SPAN == 0, "masked tiles start at a row sample");
    eg_ctx *ctx = g->ctx;
    using A = typename Op::A;
    const uint32_t m = (uint32_t)(m_entries == EG_ALL_ENTRIES ? g->m : m_entries);
    const uint32_t ntiles = m ? eg_div_up(m, TILE) : 0;
    EG_TRY(eg_buf_ensure(ctx, carry_buf, ((uint64_t)ntiles + 1) * sizeof(eg_mp_carry<A>)));
    const uint32_t g1 = ntiles ? eg_div_up((uint64_t)ntiles * 32, 256) : 0;  // one warp per tile
    const uint32_t gf = ntiles ? eg_div_up(ntiles, 256) : 0;                 // one thread per tile
    // rows without entries: the range [empty_from, n) when the layout keeps
    // them last, else found from the row pointers
    const bool ranged = empty_from <= g->n;
    const uint32_t empty_n = ranged ? g->n - empty_from : g->n;
    uint32_t g2 = empty_rows ? eg_div_up(empty_n, 256) : 0;
    if (g2 > (uint32_t)ctx->sm_count * 8) g2 = (uint32_t)ctx->sm_count * 8;
    const uint32_t g1_parts = g1;
    if (g1) {
        if (ev_begin) EG_CUDA(cudaEventRecord(ev_begin, ctx->stream));
        // MK: the relabelled CSC's row-start bits stand in for its row ids
        k_coov_rows<Op, TILE, U, REDUCE, PF, MINB, HINT, MK><<<g1, 256, 0, ctx->stream>>>(
            bp<uint32_t>(adj.rid), bp<uint32_t>(adj.col), m, ntiles, bp<eg_mp_carry<A>>(carry_buf), part, op,
            MK ? bp<uint32_t>(g->csc_p_starts) : nullptr, MK ? bp<uint32_t>(g->csc_p_trow) : nullptr);
        EG_LAUNCHED(ctx);
        if (ev_end) EG_CUDA(cudaEventRecord(ev_end, ctx->stream));
    }
    if (g2 && ranged) {
        k_coo_empty_range<Op, REDUCE><<<g2, 256, 0, ctx->stream>>>(empty_from, g->n, part ? part + g1_parts : nullptr,
                                                                   op);
        EG_LAUNCHED(ctx);
    } else if (g2) {
        k_coo_empty_rows<Op, REDUCE><<<g2, 256, 0, ctx->stream>>>(bp<uint32_t>(adj.ptr), g->n,
                                                                  part ? part + g1_parts : nullptr, op);
        EG_LAUNCHED(ctx);
    }
    if (gf) {
        k_coo_fixup<Op, TILE, REDUCE><<<gf, 256, 0, ctx->stream>>>(
            bp<uint32_t>(adj.ptr), ntiles, bp<eg_mp_carry<A>>(carry_buf), part ? part + g1_parts + g2 : nullptr, op);
        EG_LAUNCHED(ctx);
    }
    *nparts = g1_parts + g2 + gf;
    return EG_OK;
}

// m_entries: the entries of `adj` (EG_ALL_ENTRIES: the graph's m); without
// empty_rows the rows that have no entries in `adj` are left as they are.
// empty_from <= n: the rows without entries are exactly [empty_from, n).
// MK: `adj` is the relabelled CSC, read through its row-start bits.
template <class Op, bool REDUCE, bool MK = false>
static int coo_launch(eg_graph *g, eg_adj &adj, eg_buf &carry_buf, double2 *part, const Op &op, uint32_t *nparts,
                      cudaEvent_t ev_begin = nullptr, cudaEvent_t ev_end = nullptr,
                      uint64_t m_entries = EG_ALL_ENTRIES, bool empty_rows = true, uint32_t empty_from = EG_NO_RANGE) {
#define EG_ROW_CASE(i, T, U, PF, MB, H)                                                                             \
    case i:                                                                                                         \
        return coo_launch_t<Op, T, U, REDUCE, PF, MB, H, MK>(g, adj, carry_buf, part, op, nparts, ev_begin, ev_end, \
                                                              m_entries, empty_rows, empty_from);
    switch (g->row_cfg) {
        EG_ROW_CASE(1, 2048, 4, false, 6, 0)
        EG_ROW_CASE(2, 2048, 4, true, 5, 0)
        EG_ROW_CASE(3, 1024, 4, true, 6, 0)
        EG_ROW_CASE(4, 512, 4, true, 5, 0)
        EG_ROW_CASE(5, 1024, 8, true, 4, 0)
        EG_ROW_CASE(6, 1024, 4, false, 8, 0)
        EG_ROW_CASE(7, 2048, 8, false, 5, 0)
        EG_ROW_CASE(8, 1024, 4, true, 5, 1)
        EG_ROW_CASE(9, 2048, 4, true, 5, 1)
        EG_ROW_CASE(10, 1024, 4, 2, 4, 0)
        EG_ROW_CASE(11, 2048, 4, 2, 4, 0)
        default:
            return coo_launch_t<Op, 1024, 4, REDUCE, true, 5, 0, MK>(g, adj, carry_buf, part, op, nparts, ev_begin,
                                                                     ev_end, m_entries, empty_rows, empty_from);
    }
#undef EG_ROW_CASE
}

// PageRank's one-pass iteration over the destination-partition layout
// (k_pcol_rows, eg_pcol.cuh), then the rows without entries as in
// coo_launch.  `mass` bounds the rank mass, and so every row sum: the
// fixed-point unit is 2^-S with S at most 62 - E, 2 * mass < 2^E, so that
// sums stay below 2^61 units.
#ifndef EG_PC_SHIFT
// 8K rows per partition (64 KB of 64-bit sums in shared memory); measured on
// directed RMAT-24 / RMAT-22 per row pass with the finest unit: 2^14 rows
// 0.525 / 0.179 ms, 2^13 0.505 / 0.144, 2^12 0.546 / 0.151, 2^11 0.617 /
// 0.160; with the coarser unit (RMAT-24): 2^14 0.503, 2^13 0.484, 2^12 0.521
#define EG_PC_SHIFT 13
#endif
#define EG_PR_CANDS (EG_ROW_CFGS + 1)  // the tuner's candidates: the row schedules, then the partition kernel
template <bool REDUCE>
static int pcol_launch(eg_graph *g, const PrOp<false> &op, double2 *part, uint32_t *nparts, cudaEvent_t ev_begin,
                       cudaEvent_t ev_end, bool empty_rows, double mass) {
    eg_ctx *ctx = g->ctx;
    eg_pcols &pc = g->pcol;
    int E = 0, Em = 0, Lm = 0, Eb = 0;
    frexp(2.0 * (mass > 1.0 ? mass : 1.0), &E);
    frexp(mass, &Em);                       // mass < 2^Em
    frexp((double)(g->m ? g->m : 1), &Lm);  // m < 2^Lm
    // 2^-S with S = 62 - E keeps every sum below 2^61 units.  A coarser unit
    // leaves most entries' high words alone: S_mean puts the mean
    // contribution (at most mass / m) below 2^28 units, so that a row's high
    // word takes a carry about every 16th add.  S_rank keeps the unit below
    // 2^-27 of b = (1 - d) / n, the least rank any vertex gets, so that the
    // rounding of a row of k entries (half a unit each) moves its rank by at
    // most k * 2^-28 of it, 1/16 of the bound for a serial fp32 sum of the
    // row.  No rank floor (d = 1): the finest unit.
    const double b = (1.0 - (double)op.damping) / (double)(g->n ? g->n : 1);
    int S = 62 - E;
    if (b > 0.0) {
        frexp(b, &Eb);  // b >= 2^(Eb - 1)
        const int s_mean = 27 + Lm - Em, s_rank = 28 - Eb;
        const int s = s_mean > s_rank ? s_mean : s_rank;
        if (s < S) S = s;
    }
    const float fx = ldexpf(1.f, S), fx_inv = ldexpf(1.f, -S);
    const size_t smem = eg_pc_smem<EG_PC_SHIFT>::bytes;  // allowed by pcol_prepare
    auto kern = k_pcol_rows<PrOp<false>, EG_PC_SHIFT, REDUCE>;
    const uint32_t gmax = (uint32_t)ctx->sm_count * EG_PC_CTAS;
    const uint32_t g1 = pc.segs < gmax ? pc.segs : gmax;  // the resident CTAs
    if (g1) {
        if (ev_begin) EG_CUDA(cudaEventRecord(ev_begin, ctx->stream));
        kern<<<g1, EG_PC_THREADS, smem, ctx->stream>>>(
            bp<uint4>(pc.seg), pc.segs, bp<uint32_t>(pc.dst), bp<uint32_t>(pc.ridx), bp<uint32_t>(pc.crun),
            bp<uint32_t>(pc.rsrc), bp<unsigned long long>(pc.acc), bp<uint32_t>(pc.ticket), pc.parts, g->csc_p_rows,
            part, op, fx, fx_inv);
        EG_LAUNCHED(ctx);
        if (ev_end) EG_CUDA(cudaEventRecord(ev_end, ctx->stream));
    }
    uint32_t g2 = 0;
    if (empty_rows && g->csc_p_rows < g->n) {
        g2 = eg_div_up(g->n - g->csc_p_rows, 256);
        if (g2 > (uint32_t)ctx->sm_count * 8) g2 = (uint32_t)ctx->sm_count * 8;
        k_coo_empty_range<PrOp<false>, REDUCE><<<g2, 256, 0, ctx->stream>>>(g->csc_p_rows, g->n,
                                                                          part ? part + g1 : nullptr, op);
        EG_LAUNCHED(ctx);
    }
    *nparts = g1 + g2;
    return EG_OK;
}

// The partition layout, and the kernels' shared-memory allowance (set
// outside any stream capture).
static int pcol_prepare(eg_graph *g) {
    EG_TRY(eg_build_pcols(g, EG_PC_SHIFT));
    const int smem = (int)eg_pc_smem<EG_PC_SHIFT>::bytes;
    EG_CUDA(cudaFuncSetAttribute(k_pcol_rows<PrOp<false>, EG_PC_SHIFT, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    EG_CUDA(cudaFuncSetAttribute(k_pcol_rows<PrOp<false>, EG_PC_SHIFT, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    return EG_OK;
}

extern "C" void eg_pr_opts_default(eg_pr_opts *o) {
    if (!o) return;
    o->iterations = 10;
    o->damping = 0.85f;
    o->prev_init = -1.0f;
    o->swap = 1;
    o->deg_multiplier = 1;
    o->dangling = 0;
    o->compensated = 0;
    o->tolerance = 0.0;
    o->use_graph = 0;
    o->grid = 0;
    o->source_block_log2 = 0;
}

static int sb_prepare(eg_graph *g, eg_sblocks &sb, const eg_adj &adj, uint32_t shift);

// PageRank's source-block size for these options, 0 when it runs in one pass
static uint32_t pr_block_log2(const eg_graph *g, const eg_pr_opts &o) {
    const uint32_t k = o.source_block_log2 > 0 ? (uint32_t)o.source_block_log2 : EG_SB_LOG2;
    if (o.compensated || o.grid || k >= 32 || (uint64_t)g->n <= (1ull << k)) return 0;
    return k;
}

// Launches every iteration; with `timed`, the row kernels of the first
// EG_KEV iterations are bracketed by the context's kernel events.
template <bool COMP, bool REDUCE>
static int pr_iterations(eg_graph *g, const eg_pr_opts &o, const PprSeeds &ps, double tele_div, eg_pr_dev *st,
                         double2 *part, eg_buf &carry, bool timed, int it0, int it1) {
    eg_ctx *ctx = g->ctx;
    for (int it = it0; it < it1; it++) {
        PrOp<COMP> op;
        bool odd = o.swap && (it & 1);
        op.cin = odd ? bp<float>(g->contrib1) : bp<float>(g->contrib0);
        op.cout = odd ? bp<float>(g->contrib0) : bp<float>(g->contrib1);
        float *rank_new = (it & 1) ? bp<float>(g->rank_p) : bp<float>(g->rank_q);
        const float *rank_old = (it & 1) ? bp<float>(g->rank_q) : bp<float>(g->rank_p);
        op.rank = rank_new;
        op.deg = bp<uint32_t>(g->deg_p);
        op.st = st;
        op.mult = o.deg_multiplier;
        op.damping = o.damping;
        op.base = 0.f;
        op.seeds = ps;
        op.acc_in = nullptr;
        uint32_t nparts = 0;
        const bool t = timed && it < EG_KEV;
        const eg_sblocks &sb = g->sbp;
        const uint32_t kb = pr_block_log2(g, o);
        if (!COMP && kb && sb.blocks > 1 && sb.shift == kb) {
            // contributions beyond L2: one pass per source block (eg_sblocks),
            // the earlier blocks' row sums into pr_acc, the last block's
            // pass finishing the ranks from them
            if (t) EG_CUDA(cudaEventRecord(ctx->evk[2 * it], ctx->stream));
            const uint32_t n1 = g->n + 1;
            for (uint32_t b = 0; b < sb.blocks; b++) {
                eg_adj view;  // pointers into the blocked arrays (owned by the graph)
                view.ptr.p = bp<uint32_t>(sb.ptr) + (uint64_t)b * n1;
                view.col.p = bp<uint32_t>(sb.col) + sb.start[b];
                view.rid.p = bp<uint32_t>(sb.rid) + sb.start[b];
                if (b + 1 < sb.blocks) {
                    uint32_t np = 0;
                    PrAccOp aop{op.cin, bp<float>(g->pr_acc), st, b > 0 ? 1 : 0};
                    EG_TRY((coo_launch<PrAccOp, false>(g, view, carry, nullptr, aop, &np, nullptr, nullptr,
                                                        sb.len[b], b == 0)));
                } else {
                    op.acc_in = bp<float>(g->pr_acc);
                    EG_TRY((coo_launch<PrOp<COMP>, REDUCE>(g, view, carry, part, op, &nparts, nullptr, nullptr,
                                                            sb.len[b], true)));
                }
            }
            // after the last pass (a block may have no entries, and so no row kernel)
            if (t) EG_CUDA(cudaEventRecord(ctx->evk[2 * it + 1], ctx->stream));
        } else {
            // rows without in-edges get base (the teleport) alone: with no
            // dangling mass or seed weights moving it, base is the same every
            // iteration, so once both rank buffers and the contribution
            // buffer(s) hold it (iterations 0 and 1) those rows stay written
            const bool fixed_base = !o.dangling && ps.count == 0;
            bool done = false;
            if constexpr (!COMP) {
                if (g->pr_kernel == 1 && ps.count == 0 && g->pcol.shift == EG_PC_SHIFT) {
                    // the rank mass bound: the start vector's, or 1 (an
                    // iteration maps mass B to at most (1 - d) + d B)
                    const double mass = o.prev_init < 0.f ? 1.0 : (double)o.prev_init * (double)g->n;
                    EG_TRY(pcol_launch<REDUCE>(g, op, part, &nparts, t ? ctx->evk[2 * it] : nullptr,
                                               t ? ctx->evk[2 * it + 1] : nullptr, !fixed_base || it < 2, mass));
                    done = true;
                }
            }
            if (!done)
                EG_TRY((coo_launch<PrOp<COMP>, REDUCE, true>(g, g->csc_p, carry, part, op, &nparts,
                                                              t ? ctx->evk[2 * it] : nullptr,
                                                              t ? ctx->evk[2 * it + 1] : nullptr, EG_ALL_ENTRIES,
                                                              !fixed_base || it < 2, g->csc_p_rows)));
        }
        if (o.tolerance > 0.0) {  // the L1 change, after the row kernels (coalesced, 8 bytes per vertex)
            k_pr_residual<<<EG_PR_RES_BLOCKS, 256, 0, ctx->stream>>>(rank_new, rank_old, g->n, st, part + nparts);
            EG_LAUNCHED(ctx);
            nparts += EG_PR_RES_BLOCKS;
        }
        k_pr_reduce<<<1, 256, 0, ctx->stream>>>(part, REDUCE ? nparts : 0, st, tele_div, o.damping, o.dangling,
                                                o.tolerance, 1);
        EG_LAUNCHED(ctx);
    }
    return EG_OK;
}

// Iterations [it0, it1).
static int pr_dispatch(eg_graph *g, const eg_pr_opts &o, const PprSeeds &ps, double tele_div, bool reduce,
                       eg_pr_dev *st, double2 *part, eg_buf &carry, bool timed, int it0, int it1) {
    if (o.compensated) {
        if (reduce) return pr_iterations<true, true>(g, o, ps, tele_div, st, part, carry, timed, it0, it1);
        return pr_iterations<true, false>(g, o, ps, tele_div, st, part, carry, timed, it0, it1);
    }
    if (reduce) return pr_iterations<false, true>(g, o, ps, tele_div, st, part, carry, timed, it0, it1);
    return pr_iterations<false, false>(g, o, ps, tele_div, st, part, carry, timed, it0, it1);
}

// The iteration loop of plain PageRank captured once as a CUDA graph and
// replayed while the options and the buffers it was captured with stay the same.
static int pr_graph(eg_graph *g, const eg_pr_opts &o, bool reduce, eg_pr_dev *st, double2 *part, eg_buf &carry) {
    eg_ctx *ctx = g->ctx;
    uint64_t key[16] = {};
    key[0] = (uint32_t)o.iterations | ((uint64_t)g->csc_p_rows << 32);
    key[1] = (uint64_t)o.swap | ((uint64_t)o.compensated << 1) | ((uint64_t)reduce << 2) | ((uint64_t)o.dangling << 3);
    uint32_t dbits;
    memcpy(&dbits, &o.damping, 4);
    key[2] = dbits | ((uint64_t)o.deg_multiplier << 32);
    memcpy(&key[3], &o.tolerance, 8);
    key[4] = (uint64_t)(uintptr_t)g->contrib0.p;
    key[5] = (uint64_t)(uintptr_t)g->contrib1.p;
    key[6] = (uint64_t)(uintptr_t)g->rank_p.p ^ ((uint64_t)(uintptr_t)g->rank_q.p << 1);
    key[7] = (uint64_t)(uintptr_t)g->deg_p.p;
    key[8] = (uint64_t)(uintptr_t)st;
    key[9] = (uint64_t)(uintptr_t)part;
    key[10] = (uint64_t)(uintptr_t)carry.p;
    key[11] = (uint64_t)(uintptr_t)g->csc_p.rid.p ^ ((uint64_t)(uintptr_t)g->csc_p_starts.p << 17);
    key[12] = (uint64_t)(uintptr_t)g->csc_p.col.p ^ ((uint64_t)(uintptr_t)g->csc_p_trow.p << 17);
    key[13] = (uint64_t)(uintptr_t)g->csc_p.ptr.p ^ ((uint64_t)(uintptr_t)g->pcol.seg.p << 7) ^
              ((uint64_t)(uintptr_t)g->pcol.rsrc.p << 13) ^ ((uint64_t)(uintptr_t)g->pcol.dst.p << 19) ^
              ((uint64_t)(uintptr_t)g->pcol.ridx.p << 25) ^ ((uint64_t)(uintptr_t)g->pcol.crun.p << 31);
    key[14] = g->m ^ ((uint64_t)g->row_cfg << 56) ^ ((uint64_t)pr_block_log2(g, o) << 48) ^
              ((uint64_t)g->pr_kernel << 44) ^ ((uint64_t)g->pcol.shift << 36);
    key[15] = (uint64_t)ctx->stream ^ 0x5052ull;
    if (g->prg.exec && !memcmp(key, g->prk, sizeof(key))) return EG_OK;
    if (g->prg.exec) cudaGraphExecDestroy(g->prg.exec);
    if (g->prg.graph) cudaGraphDestroy(g->prg.graph);
    g->prg.exec = nullptr;
    g->prg.graph = nullptr;
    // the carries must be allocated before capture (no allocation inside it)
    EG_TRY(eg_buf_ensure(ctx, carry,
                         ((uint64_t)(g->m ? eg_div_up(g->m, EG_COO_TILE_MIN) : 0) + 1) * sizeof(eg_mp_carry<double>)));
    key[10] = (uint64_t)(uintptr_t)carry.p;
    PprSeeds none;
    memset(&none, 0, sizeof(none));
    EG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = pr_dispatch(g, o, none, (double)g->n, reduce, st, part, carry, false, 0, o.iterations);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &gr);
    if (rc != EG_OK) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
    }
    if (e != cudaSuccess) return eg_fail(EG_ECUDA, "PageRank capture: %s", cudaGetErrorString(e));
    g->prg.graph = gr;
    EG_CUDA(cudaGraphInstantiate(&g->prg.exec, gr, 0));
    memcpy(g->prk, key, sizeof(key));
    return EG_OK;
}

// Shared by eg_pagerank and eg_ppr: the iterations over the relabelled CSC,
// then the ranks back in the original vertex order.  `ps` (in relabelled
// ids) selects the personalised teleport; its total multiplicity divides it.
static int pr_run(eg_graph *g, const eg_pr_opts &o, const PprSeeds &ps, uint32_t seed_total, float *rank_out,
                  eg_pr_stats *stats) {
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    const uint32_t coo_tiles = g->m ? eg_div_up(g->m, EG_COO_TILE_MIN) : 0;  // the most tiles of any schedule
    const uint32_t nparts = 2 * eg_div_up((uint64_t)coo_tiles * 32, 256) + (uint32_t)ctx->sm_count * 8 + EG_PR_RES_BLOCKS;
    EG_TRY(eg_buf_ensure(ctx, g->rank, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->rank_p, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->rank_q, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->contrib0, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->contrib1, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->pr_part, ((uint64_t)nparts + 1024) * sizeof(double2)));
    eg_buf &carry = g->mp_carry;
    eg_pr_dev *st = bp<eg_pr_dev>(g->pr_stats);
    double2 *part = bp<double2>(g->pr_part);
    EG_CUDA(cudaMemsetAsync(st, 0, sizeof(eg_pr_dev), ctx->stream));
    EG_CUDA(cudaMemsetAsync(part, 0, ((uint64_t)nparts + 1024) * sizeof(double2), ctx->stream));
    const bool ppr = ps.count > 0;
    const double tele_div = ppr ? (double)seed_total : (double)n;
    const bool reduce = o.tolerance > 0.0 || o.dangling;
    uint32_t ib = eg_div_up(n, 256);
    if (ib > 1024) ib = 1024;
    if (ppr) {
        k_ppr1_init<<<ib, 256, 0, ctx->stream>>>(n, ps, (float)(1.0 / (double)seed_total), bp<uint32_t>(g->deg_p),
                                                bp<float>(g->rank_p), bp<float>(g->contrib0), part);
    } else {
        const float prev_init = o.prev_init < 0.f ? 1.0f / (float)n : o.prev_init;
        k_pr_init<<<ib, 256, 0, ctx->stream>>>(n, prev_init, bp<uint32_t>(g->deg_p), o.deg_multiplier,
                                              bp<float>(g->rank_p), bp<float>(g->contrib0), part);
    }
    EG_LAUNCHED(ctx);
    k_pr_reduce<<<1, 256, 0, ctx->stream>>>(part, ib, st, tele_div, o.damping, o.dangling, 0.0, 0);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemsetAsync(part, 0, ((uint64_t)nparts + 1024) * sizeof(double2), ctx->stream));
    const bool graph = o.use_graph && !ppr;
    if (graph) EG_TRY(pr_graph(g, o, reduce, st, part, carry));
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    if (graph) {
        if (o.iterations > 0) EG_CUDA(cudaGraphLaunch(g->prg.exec, ctx->stream));
    } else {
        // with a tolerance, the stop flag is read every EG_PR_CHECK iterations so
        // that converged runs do not keep launching no-op iterations
        const int chunk = o.tolerance > 0.0 ? EG_PR_CHECK : (o.iterations > 0 ? o.iterations : 1);
        int *hdone = (int *)ctx->h_pinned;
        for (int it0 = 0; it0 < o.iterations; it0 += chunk) {
            const int it1 = it0 + chunk < o.iterations ? it0 + chunk : o.iterations;
            EG_TRY(pr_dispatch(g, o, ps, tele_div, reduce, st, part, carry, true, it0, it1));
            if (o.tolerance > 0.0 && it1 < o.iterations) {
                EG_TRY(eg_readback_wait(ctx, hdone, &st->done, sizeof(int), ctx->stream));
                if (*hdone) break;
            }
        }
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    // ranks back to the original vertex ids
    k_pr_unpermute<<<ib, 256, 0, ctx->stream>>>(bp<float>(g->rank_p), bp<float>(g->rank_q), st, bp<uint32_t>(g->perm),
                                                n, bp<float>(g->rank));
    EG_LAUNCHED(ctx);
    eg_pr_dev hst;
    EG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, ctx->stream));
    if (rank_out) EG_CUDA(cudaMemcpyAsync(rank_out, g->rank.p, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->iterations_run = hst.iters;
        stats->residual = hst.residual;
        stats->dangling_mass = hst.dangling;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
        stats->row_kernel_ms = 0.f;
        int timed = graph || !g->m ? 0 : (o.iterations < EG_KEV ? o.iterations : EG_KEV);
        if (timed > hst.iters) timed = hst.iters;  // converged launches return at once
        for (int i = 0; i < timed; i++) {
            float t = 0.f;
            EG_CUDA(cudaEventElapsedTime(&t, ctx->evk[2 * i], ctx->evk[2 * i + 1]));
            stats->row_kernel_ms += t / (float)timed;
        }
    }
    return EG_OK;
}

static int pr_prepare(eg_graph *g, const eg_pr_opts *o = nullptr) {
    if (!(g->built & EG_LAYOUT_CSC) || !(g->built & EG_LAYOUT_CSR))
        return eg_fail(EG_ENOTBUILT, "PageRank needs the CSC (in-lists) and CSR (out-degrees)");
    EG_CUDA(cudaSetDevice(g->ctx->device));
    EG_TRY(eg_build_relabeled_csc(g));
    EG_TRY(eg_buf_ensure(g->ctx, g->pr_stats, 512));
    eg_pr_opts d;
    eg_pr_opts_default(&d);
    const uint32_t kb = pr_block_log2(g, o ? *o : d);
    if (kb) {  // contributions beyond L2: the source-blocked copy
        EG_TRY(sb_prepare(g, g->sbp, g->csc_p, kb));
        EG_TRY(eg_buf_ensure(g->ctx, g->pr_acc, (uint64_t)g->n * 4));
    }
    if (g->pr_kernel == 1) EG_TRY(pcol_prepare(g));
    return EG_OK;
}

extern "C" int eg_pagerank(eg_graph *g, const eg_pr_opts *opts, float *rank_out, eg_pr_stats *stats) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    eg_pr_opts o;
    if (opts) o = *opts;
    else eg_pr_opts_default(&o);
    if (o.iterations < 0 || o.deg_multiplier == 0) return eg_fail(EG_EINVAL, "bad PageRank options");
    if (o.grid) {
        if (!(g->built & EG_LAYOUT_GRID)) return eg_fail(EG_ENOTBUILT, "grid PageRank needs the grid");
        // grid = 1 with the CSC built: the row kernel over the CSC, whose
        // per-destination order (ascending source) is the order in which
        // prgrid's iterator visits the cells of a destination (rows of cells
        // in turn, each cell in source order; prgrid_cilk.c:62-76, 111-141);
        // grid = 2, or no CSC: the cell kernel with atomic adds
        if (o.grid == 1 && (g->built & EG_LAYOUT_CSC) && (g->built & EG_LAYOUT_CSR)) {
            o.grid = 0;
        } else {
            EG_CUDA(cudaSetDevice(g->ctx->device));
            return eg_grid_pagerank(g, o, rank_out, stats);
        }
    }
    EG_TRY(pr_prepare(g, &o));
    PprSeeds none;
    memset(&none, 0, sizeof(none));
    return pr_run(g, o, none, 0, rank_out, stats);
}

// ============================================================== autotuner
extern "C" int eg_graph_set_row_schedule(eg_graph *g, int index) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (index < 0 || index >= EG_PR_CANDS) return eg_fail(EG_EINVAL, "row schedule %d of %d", index, EG_PR_CANDS);
    if (index < EG_ROW_CFGS) {
        g->row_cfg = index;
        g->pr_kernel = 0;
    } else {
        g->pr_kernel = 1;  // PageRank's partition kernel; the row kernels keep their schedule
    }
    return EG_OK;
}

extern "C" int eg_graph_tune(eg_graph *g, eg_tune_result *out) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    EG_TRY(pr_prepare(g));
    eg_pr_opts o;
    eg_pr_opts_default(&o);
    o.iterations = 6;
    PprSeeds none;
    memset(&none, 0, sizeof(none));
    eg_tune_result r;
    memset(&r, 0, sizeof(r));
    r.ncand = EG_PR_CANDS;
    int best = 0;
    g->pr_kernel = 0;
    for (int c = 0; c < EG_ROW_CFGS; c++) {
        g->row_cfg = c;
        eg_pr_stats st;
        EG_TRY(pr_run(g, o, none, 0, nullptr, &st));  // warm-up (caches, carries)
        EG_TRY(pr_run(g, o, none, 0, nullptr, &st));
        r.tile_entries[c] = kRowCfg[c].tile;
        r.entries_per_lane[c] = kRowCfg[c].u;
        r.prefetch[c] = kRowCfg[c].pf;
        r.min_blocks[c] = kRowCfg[c].minb;
        r.cache_hint[c] = kRowCfg[c].hint;
        r.ms[c] = st.row_kernel_ms;
        if (st.row_kernel_ms < r.ms[best]) best = c;
    }
    g->row_cfg = best;
    r.chosen = best;
    {  // the partition kernel (PageRank only; SpMV keeps the row schedule)
        const int c = EG_ROW_CFGS;
        r.tile_entries[c] = EG_PC_CHUNK;
        r.entries_per_lane[c] = 8;
        r.prefetch[c] = 1;
        r.min_blocks[c] = 1;
        r.cache_hint[c] = 1;
        r.partition_log2[c] = EG_PC_SHIFT;
        r.ms[c] = -1.f;  // not timed: its layout does not fit the context's budget
        const int prc = pcol_prepare(g);
        if (prc == EG_ENOMEM) {
            eg_clear_error();
            goto tuned;
        }
        EG_TRY(prc);
        g->pr_kernel = 1;
        eg_pr_stats st;
        EG_TRY(pr_run(g, o, none, 0, nullptr, &st));
        EG_TRY(pr_run(g, o, none, 0, nullptr, &st));
        r.ms[c] = st.row_kernel_ms;
        if (st.row_kernel_ms < r.ms[best]) {
            r.chosen = c;
        } else {
            g->pr_kernel = 0;
        }
    }
tuned:
    if (g->built & EG_LAYOUT_CSR)
        EG_TRY(eg_bfs_tune(g, &r.bfs_graph_ms, &r.bfs_host_ms, &r.bfs_host_loop, &r.bfs_switch_divisor));
    if (out) *out = r;
    return EG_OK;
}

extern "C" int eg_ppr(eg_graph *g, const uint32_t *seeds, uint32_t nseeds, const eg_ppr_opts *opts, float *rank_out,
                      eg_ppr_stats *stats) {
    if (!g || !seeds) return eg_fail(EG_EINVAL, "NULL argument");
    if (nseeds < 1) return eg_fail(EG_EINVAL, "a query needs a seed");
    eg_ppr_opts po;
    if (opts) po = *opts;
    else {
        po.damping = 0.85f;
        po.max_iters = 50;
        for (int q = 0; q < 32; q++) po.tolerance[q] = 1e-6f;
    }
    if (po.max_iters < 1 || !(po.damping > 0.f && po.damping < 1.f)) return eg_fail(EG_EINVAL, "bad PPR options");
    // distinct seeds with their multiplicity
    PprSeeds ps;
    memset(&ps, 0, sizeof(ps));
    for (uint32_t i = 0; i < nseeds; i++) {
        if (seeds[i] >= g->n) return eg_fail(EG_EINVAL, "seed %u >= n", seeds[i]);
        uint32_t j = 0;
        while (j < ps.count && ps.id[j] != seeds[i]) j++;
        if (j == ps.count) {
            if (ps.count == EG_PPR1_SEEDS) return eg_fail(EG_EINVAL, "at most %d distinct seeds", EG_PPR1_SEEDS);
            ps.id[ps.count++] = seeds[i];
        }
        ps.mult[j] += 1.f;
    }
    EG_TRY(pr_prepare(g));
    eg_ctx *ctx = g->ctx;
    // seed ids into the relabelled order
    uint32_t *d_ids = reinterpret_cast<uint32_t *>(static_cast<char *>(g->pr_stats.p) + 256);
    uint32_t *h = (uint32_t *)ctx->h_pinned;
    memcpy(h, ps.id, sizeof(ps.id));
    EG_CUDA(cudaMemcpyAsync(d_ids, h, sizeof(ps.id), cudaMemcpyHostToDevice, ctx->stream));
    k_map_ids<<<1, 32, 0, ctx->stream>>>(bp<uint32_t>(g->perm), d_ids, ps.count, d_ids + EG_PPR1_SEEDS);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaMemcpyAsync(h, d_ids + EG_PPR1_SEEDS, sizeof(ps.id), cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    memcpy(ps.id, h, ps.count * sizeof(uint32_t));
    eg_pr_opts o;
    eg_pr_opts_default(&o);
    o.iterations = po.max_iters;
    o.damping = po.damping;
    o.swap = 1;
    o.dangling = 1;  // the mass on out-degree-0 vertices returns to the seeds
    o.tolerance = po.tolerance[0] > 0.f ? (double)po.tolerance[0] : 0.0;
    eg_pr_stats s;
    EG_TRY(pr_run(g, o, ps, nseeds, rank_out, &s));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations[0] = s.iterations_run;
        stats->residual[0] = s.residual;
        stats->sweeps = s.iterations_run;
        stats->ms = s.ms;
    }
    return EG_OK;
}

// ============================================================== SpMV
template <int MODE>  // 0: x/1000 (reference 0.001 scale), 1: x
struct SpmvU32Op {
    using V = uint32_t;
    using A = uint32_t;
    const uint32_t *__restrict__ x;
    uint32_t *__restrict__ y;
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void setup() {}
    __device__ __forceinline__ V gather(uint32_t, uint32_t u) const {
        uint32_t xv = __ldg(x + u);
        return MODE == 0 ? xv / 1000u : xv;
    }
    __device__ __forceinline__ A zero() const { return 0u; }
    __device__ __forceinline__ A add(A a, V v) const { return a + v; }
    __device__ __forceinline__ A merge(A a, A b) const { return a + b; }
    __device__ __forceinline__ float2 emit(uint32_t v, A s) const {
        y[v] = s;
        return make_float2(0.f, 0.f);
    }
};

template <bool COMP>
struct SpmvF32Op {
    using V = float;
    using A = typename std::conditional<COMP, float2, float>::type;
    const float *__restrict__ x;
    const float *__restrict__ vals;
    float *__restrict__ y;
    int accum;     // 1: y[v] += the row sum (source blocks after the first)
    uint64_t pol;  // L2 evict-first for the streamed values
    float *yerr;   // COMP over source blocks: the rows' error terms between passes
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void setup() { pol = eg_l2_evict_first_policy(); }
    __device__ __forceinline__ V gather(uint32_t j, uint32_t u) const {
        return __fmul_rn(eg_stream_ldf(vals + j, pol), __ldg(x + u));
    }
    __device__ __forceinline__ A zero() const {
        if constexpr (COMP) return make_float2(0.f, 0.f);
        else return 0.f;
    }
    __device__ __forceinline__ A add(A a, V v) const {
        if constexpr (COMP) return eg_f2sum::add(a, v);
        else return a + v;
    }
    __device__ __forceinline__ A merge(A a, A b) const {
        if constexpr (COMP) return eg_f2sum::merge(a, b);
        else return a + b;
    }
    __device__ __forceinline__ float2 emit(uint32_t v, A s) const {
        if constexpr (COMP) {
            float2 t = s;
            if (accum) t = eg_f2sum::merge(make_float2(y[v], yerr[v]), t);
            if (yerr) {  // the pair goes on to the next block (k_pair_finish adds it up)
                y[v] = t.x;
                yerr[v] = t.y;
            } else {
                y[v] = t.x + t.y;
            }
        } else {
            y[v] = accum ? y[v] + s : s;
        }
        return make_float2(0.f, 0.f);
    }
};

struct SpmvF64Op {
    using V = double;
    using A = double;
    const float *__restrict__ x;
    const float *__restrict__ vals;
    double *__restrict__ y;
    uint64_t pol;  // L2 evict-first for the streamed values
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void setup() { pol = eg_l2_evict_first_policy(); }
    __device__ __forceinline__ V gather(uint32_t j, uint32_t u) const {
        return __dmul_rn((double)eg_stream_ldf(vals + j, pol), (double)__ldg(x + u));
    }
    __device__ __forceinline__ A zero() const { return 0.0; }
    __device__ __forceinline__ A add(A a, V v) const { return __dadd_rn(a, v); }
    __device__ __forceinline__ A merge(A a, A b) const { return __dadd_rn(a, b); }
    __device__ __forceinline__ float2 emit(uint32_t v, A s) const {
        y[v] = s;
        return make_float2(0.f, 0.f);
    }
};

// Edge value of CSC entry p (row v, column u): U[0,1) hashed from the
// unordered endpoint pair, or 1.
__global__ void k_csc_values(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col, uint32_t n,
                             uint64_t seed, int unit, float *__restrict__ vals) {
    uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps)
        for (uint32_t p = ptr[v] + lane; p < ptr[v + 1]; p += 32) {
            if (unit) vals[p] = 1.0f;
            else vals[p] = (float)(eg_edge_hash(seed, col[p], v) >> 40) * (1.0f / 16777216.0f);
        }
}

// ---- source-blocked CSC for fp32 SpMV over an x larger than L2
// With x beyond L2 (ER 2^25: 134 MB) every gather that misses goes to DRAM at
// random.  The CSC's entries are split by source block (a stable sort on
// source >> shift keeps CSC order inside a block), each block with its own
// row pointers; one row-kernel pass per block then gathers from an x slice
// that L2 holds: the first pass writes y, the others add to it.
namespace {
__global__ void k_sb_keys(const uint32_t *__restrict__ col, uint64_t M, uint32_t shift, uint32_t *keys,
                          uint32_t *idx) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
        keys[i] = col[i] >> shift;
        idx[i] = (uint32_t)i;
    }
}
__global__ void k_sb_gather(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ rid,
                            const uint32_t *__restrict__ col, uint64_t M, uint32_t *orid, uint32_t *ocol) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = perm[i];
        orid[i] = rid[e];
        ocol[i] = col[e];
    }
}
__global__ void k_pair_finish(float *y, const float *__restrict__ err, uint32_t n) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) y[v] = y[v] + err[v];
}
__global__ void k_sb_vals(const uint32_t *__restrict__ perm, const float *__restrict__ vals, uint64_t M,
                          float *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = vals[perm[i]];
}
}  // namespace

static uint32_t sb_grid(eg_ctx *ctx, uint64_t work) {
    uint64_t b = (work + 255) / 256;
    const uint64_t cap = (uint64_t)ctx->sm_count * 8;
    return (uint32_t)(b > cap ? cap : (b ? b : 1));
}

static int sb_prepare(eg_graph *g, eg_sblocks &sb, const eg_adj &adj, uint32_t shift) {
    if (sb.blocks && sb.shift == shift) return EG_OK;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    const uint64_t M = g->m;
    const uint32_t B = (uint32_t)(((uint64_t)n + (1ull << shift) - 1) >> shift);
    if (B > EG_SB_MAX) return eg_fail(EG_EINVAL, "source blocks of 2^%u vertices: %u blocks, at most %d", shift, B, EG_SB_MAX);
    sb.blocks = 0;
    eg_buf ka, va, kb, vb, cnt;
    int rc = EG_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        eg_buf_free(ctx, ka);
        eg_buf_free(ctx, va);
        eg_buf_free(ctx, kb);
        eg_buf_free(ctx, vb);
        eg_buf_free(ctx, cnt);
    };
#define STRY(x)            \
    do {                   \
        rc = (x);          \
        if (rc != EG_OK) { \
            cleanup();     \
            return rc;     \
        }                  \
    } while (0)
    STRY(eg_buf_ensure(ctx, ka, (M + 1) * 4));
    STRY(eg_buf_ensure(ctx, va, (M + 1) * 4));
    STRY(eg_buf_ensure(ctx, kb, (M + 1) * 4));
    STRY(eg_buf_ensure(ctx, vb, (M + 1) * 4));
    STRY(eg_buf_ensure(ctx, cnt, ((uint64_t)n + EG_SB_MAX + 1) * 4));
    const uint64_t MP = M + 4ull * EG_SB_MAX;  // room for the blocks' alignment padding
    STRY(eg_buf_ensure(ctx, sb.rid, MP * 4 + 16));
    STRY(eg_buf_ensure(ctx, sb.col, MP * 4 + 16));
    STRY(eg_buf_ensure(ctx, sb.perm, MP * 4 + 16));
    STRY(eg_buf_ensure(ctx, sb.ptr, (uint64_t)B * ((uint64_t)n + 1) * 4));
    uint32_t *ks = bp<uint32_t>(ka), *vs = bp<uint32_t>(va);
    if (M) {
        k_sb_keys<<<sb_grid(ctx, M), 256, 0, ctx->stream>>>(bp<uint32_t>(adj.col), M, shift, bp<uint32_t>(ka),
                                                            bp<uint32_t>(va));
        EG_LAUNCHED(ctx);
        const int bits = B <= 1 ? 1 : 32 - __builtin_clz(B - 1);
        STRY(eg_radix_sort(ctx, bp<uint32_t>(ka), bp<uint32_t>(va), bp<uint32_t>(kb), bp<uint32_t>(vb), M, bits, &ks,
                           &vs));
    }
    // entries per block (sorted by block: block b is vs[s_b, s_b + len_b))
    uint32_t *bcnt = bp<uint32_t>(cnt) + n;
    if (cudaMemsetAsync(bcnt, 0, (EG_SB_MAX + 1) * 4, ctx->stream) != cudaSuccess) STRY(eg_fail(EG_ECUDA, "memset"));
    STRY(eg_histogram(ctx, ks, M, bcnt));
    uint32_t hc[EG_SB_MAX + 1];
    if (cudaMemcpyAsync(hc, bcnt, (EG_SB_MAX + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        STRY(eg_fail(EG_ECUDA, "source-block counts"));
    uint64_t sorted_at = 0, placed_at = 0;
    for (uint32_t b = 0; b < B; b++) {
        const uint64_t len = hc[b];
        sb.start[b] = placed_at;  // a multiple of 4 entries
        sb.len[b] = len;
        if (len) {
            k_sb_gather<<<sb_grid(ctx, len), 256, 0, ctx->stream>>>(
                vs + sorted_at, bp<uint32_t>(adj.rid), bp<uint32_t>(adj.col), len,
                bp<uint32_t>(sb.rid) + placed_at, bp<uint32_t>(sb.col) + placed_at);
            EG_LAUNCHED(ctx);
            if (cudaMemcpyAsync(bp<uint32_t>(sb.perm) + placed_at, vs + sorted_at, len * 4, cudaMemcpyDeviceToDevice,
                                ctx->stream) != cudaSuccess)
                STRY(eg_fail(EG_ECUDA, "source-block copy"));
        }
        // the block's row pointers: histogram of its rows, exclusive scan
        if (cudaMemsetAsync(cnt.p, 0, (uint64_t)n * 4, ctx->stream) != cudaSuccess) STRY(eg_fail(EG_ECUDA, "memset"));
        STRY(eg_histogram(ctx, bp<uint32_t>(sb.rid) + placed_at, len, bp<uint32_t>(cnt)));
        STRY(eg_exscan_u32(ctx, bp<uint32_t>(cnt), bp<uint32_t>(sb.ptr) + (uint64_t)b * ((uint64_t)n + 1), n));
        sorted_at += len;
        placed_at = (placed_at + len + 3) & ~3ull;
    }
    cleanup();
#undef STRY
    sb.shift = shift;
    sb.blocks = B;
    sb.vals_kind = 0;
    return EG_OK;
}

// fp32 SpMV over the source blocks (values already in g->spmv_vals, CSC
// order): one pass per block, the first writing y, the others adding to it
// (EG_SPMV_F32_COMP carries each row's (sum, error) pair between passes).
static int sb_spmv(eg_graph *g, int kind, int vk, uint64_t seed) {
    eg_sblocks &sb = g->sb;
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    const uint64_t M = g->m;
    if (sb.vals_kind != vk || (vk == 2 && sb.vals_seed != seed)) {
        EG_TRY(eg_buf_ensure(ctx, sb.vals, (M + 4ull * EG_SB_MAX) * 4 + 16));
        for (uint32_t b = 0; b < sb.blocks; b++) {
            const uint64_t s0 = sb.start[b], len = sb.len[b];
            if (!len) continue;
            k_sb_vals<<<sb_grid(ctx, len), 256, 0, ctx->stream>>>(bp<uint32_t>(sb.perm) + s0,
                                                                  bp<float>(g->spmv_vals), len,
                                                                  bp<float>(sb.vals) + s0);
            EG_LAUNCHED(ctx);
        }
        sb.vals_kind = vk;
        sb.vals_seed = seed;
    }
    if (kind == EG_SPMV_F32_COMP) EG_TRY(eg_buf_ensure(ctx, sb.yerr, (uint64_t)n * 4));
    uint32_t np = 0;
    for (uint32_t b = 0; b < sb.blocks; b++) {
        const uint64_t s0 = sb.start[b], len = sb.len[b];
        eg_adj view;  // pointers into the blocked arrays (owned by the graph)
        view.ptr.p = bp<uint32_t>(sb.ptr) + (uint64_t)b * ((uint64_t)n + 1);
        view.col.p = bp<uint32_t>(sb.col) + s0;
        view.rid.p = bp<uint32_t>(sb.rid) + s0;
        const int acc = b > 0 ? 1 : 0;
        if (kind == EG_SPMV_F32) {
            SpmvF32Op<false> op{bp<float>(g->spmv_x), bp<float>(sb.vals) + s0, bp<float>(g->spmv_y), acc, 0, nullptr};
            EG_TRY((coo_launch<SpmvF32Op<false>, false>(g, view, g->mp_carry, nullptr, op, &np, nullptr, nullptr, len,
                                                         b == 0)));
        } else {
            SpmvF32Op<true> op{bp<float>(g->spmv_x), bp<float>(sb.vals) + s0, bp<float>(g->spmv_y), acc, 0,
                               bp<float>(sb.yerr)};
            EG_TRY((coo_launch<SpmvF32Op<true>, false>(g, view, g->mp_carry, nullptr, op, &np, nullptr, nullptr, len,
                                                        b == 0)));
        }
    }
    if (kind == EG_SPMV_F32_COMP) {
        k_pair_finish<<<sb_grid(ctx, n), 256, 0, ctx->stream>>>(bp<float>(g->spmv_y), bp<float>(sb.yerr), n);
        EG_LAUNCHED(ctx);
    }
    return EG_OK;
}

extern "C" int eg_spmv(eg_graph *g, const eg_spmv_opts *opts, const void *x, void *y, float *ms) {
    if (!g || !opts || !x) return eg_fail(EG_EINVAL, "NULL argument");
    const int kind = opts->kind;
    if (kind < EG_SPMV_U32_PULL || kind > EG_SPMV_F64) return eg_fail(EG_EINVAL, "unknown SpMV kind %d", kind);
    const bool pull = kind == EG_SPMV_U32_PULL || kind >= EG_SPMV_F32;
    const unsigned need = opts->grid ? EG_LAYOUT_GRID : (pull ? EG_LAYOUT_CSC : EG_LAYOUT_CSR);
    if (!(g->built & need)) return eg_fail(EG_ENOTBUILT, "SpMV kind %d needs layout %u", kind, need);
    // grid = 1 with the adjacency built: its rows carry the grid's
    // per-destination (pull) or per-source (push, edge) order, so the fixed-
    // order row kernel runs; grid = 2, or no adjacency: the cell kernel
    const bool cells = opts->grid == 2 || (opts->grid && !(g->built & (pull ? EG_LAYOUT_CSC : EG_LAYOUT_CSR)));
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    eg_adj &adj = pull ? g->csc : g->csr;
    const size_t ysz = kind == EG_SPMV_F64 ? 8 : 4;
    EG_TRY(eg_buf_ensure(ctx, g->spmv_x, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->spmv_y, (uint64_t)n * ysz));
    EG_CUDA(cudaMemcpyAsync(g->spmv_x.p, x, (uint64_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (cells) {
        EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
        EG_TRY(eg_grid_spmv(g, kind, opts->value_seed, opts->unit_values, g->spmv_x.p, g->spmv_y.p));
        EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
        if (y) EG_CUDA(cudaMemcpyAsync(y, g->spmv_y.p, (uint64_t)n * ysz, cudaMemcpyDeviceToHost, ctx->stream));
        EG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ms) EG_CUDA(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
        return EG_OK;
    }
    if (kind >= EG_SPMV_F32) {
        int vk = opts->unit_values ? 1 : 2;
        if (!g->spmv_vals.p || g->spmv_vals_kind != vk || (vk == 2 && g->spmv_vals_seed != opts->value_seed)) {
            EG_TRY(eg_buf_ensure(ctx, g->spmv_vals, g->m * 4 + 16));
            k_csc_values<<<eg_div_up((uint64_t)n * 32, 256) > 65535 ? 65535 : eg_div_up((uint64_t)n * 32, 256), 256, 0,
                           ctx->stream>>>(bp<uint32_t>(g->csc.ptr), bp<uint32_t>(g->csc.col), n, opts->value_seed,
                                          opts->unit_values, bp<float>(g->spmv_vals));
            EG_LAUNCHED(ctx);
            g->spmv_vals_kind = vk;
            g->spmv_vals_seed = opts->value_seed;
        }
    }
    // fp32 kinds over x beyond the source-block size: the source-blocked CSC
    const uint32_t sb_log2 = opts->source_block_log2 ? (uint32_t)opts->source_block_log2 : EG_SB_LOG2;
    // (not FP64: its time is in the FP64 arithmetic, which a second pass only adds to)
    const bool blocked = (kind == EG_SPMV_F32 || kind == EG_SPMV_F32_COMP) && sb_log2 < 32 &&
                         (uint64_t)n > (1ull << sb_log2);
    if (blocked) EG_TRY(sb_prepare(g, g->sb, g->csc, sb_log2));
    eg_buf &carry = g->mp_carry;
    uint32_t np = 0;
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    switch (kind) {
        case EG_SPMV_U32_PULL:
        case EG_SPMV_U32_PUSH: {
            SpmvU32Op<0> op{bp<uint32_t>(g->spmv_x), bp<uint32_t>(g->spmv_y)};
            EG_TRY((coo_launch<SpmvU32Op<0>, false>(g, adj, carry, nullptr, op, &np)));
            break;
        }
        case EG_SPMV_U32_EDGE: {
            SpmvU32Op<1> op{bp<uint32_t>(g->spmv_x), bp<uint32_t>(g->spmv_y)};
            EG_TRY((coo_launch<SpmvU32Op<1>, false>(g, adj, carry, nullptr, op, &np)));
            break;
        }
        case EG_SPMV_F32: {
            if (blocked) {
                EG_TRY(sb_spmv(g, kind, opts->unit_values ? 1 : 2, opts->value_seed));
                break;
            }
            SpmvF32Op<false> op{bp<float>(g->spmv_x), bp<float>(g->spmv_vals), bp<float>(g->spmv_y), 0, 0, nullptr};
            EG_TRY((coo_launch<SpmvF32Op<false>, false>(g, adj, carry, nullptr, op, &np)));
            break;
        }
        case EG_SPMV_F32_COMP: {
            if (blocked) {
                EG_TRY(sb_spmv(g, kind, opts->unit_values ? 1 : 2, opts->value_seed));
                break;
            }
            SpmvF32Op<true> op{bp<float>(g->spmv_x), bp<float>(g->spmv_vals), bp<float>(g->spmv_y), 0, 0, nullptr};
            EG_TRY((coo_launch<SpmvF32Op<true>, false>(g, adj, carry, nullptr, op, &np)));
            break;
        }
        case EG_SPMV_F64: {
            SpmvF64Op op{bp<float>(g->spmv_x), bp<float>(g->spmv_vals), bp<double>(g->spmv_y), 0};
            EG_TRY((coo_launch<SpmvF64Op, false>(g, adj, carry, nullptr, op, &np)));
            break;
        }
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (y) EG_CUDA(cudaMemcpyAsync(y, g->spmv_y.p, (uint64_t)n * ysz, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ms) EG_CUDA(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return EG_OK;
}
