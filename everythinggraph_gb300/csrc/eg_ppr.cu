// Batched personalised PageRank: up to 32 queries advance together, one
// warp lane per query.
//
// No reference counterpart (the reference runs one global PageRank); the
// per-query iteration is pr_numa's correct pull PR (pr_numa.c:245-277,396)
// with the teleport and dangling mass sent to the query's seed set:
//   x'[v] = d * sum_{u->v} x[u]/deg[u] + (1 - d + d * dangling(x)) * t[v]
// where t is uniform over the query's seeds.  Each query stops when the FP64
// L1 change of its vector drops below its tolerance or after max_iters.
//
// Layout: vertex-major [n][32] fp32 rows (128 bytes per vertex), so for an
// entry u->v a warp reads x[u][0..31] with one coalesced 128-byte load.  Each
// warp owns a fixed range of CSC entries and walks it entry by entry (the
// entry's row and column are loaded 32 at a time and broadcast); the lane's
// sum for the current row is written when the row changes.  Rows split
// between warps are joined by a fix-up (head/tail partials, warp order).  A
// lane only ever combines its own query's values, in an order fixed by the
// graph, so each query's result is bit-identical whether it runs alone or in
// a batch.
#include <stdlib.h>
#include <string.h>

#include "eg_ppr.cuh"


namespace {
// Sweep-loop state of the batched PageRank graph.
struct PprLoop {
    int sweeps;
    int max_sweeps;
    int nq;
    int pad;
};

__global__ void k_ppr_loop_init(PprLoop *st, int max_sweeps, int nq) {
    st->sweeps = 0;
    st->max_sweeps = max_sweeps;
    st->nq = nq;
}

// Sweep end: the while node runs another sweep while a query of the batch is
// still running (and fewer than max_iters sweeps ran).
__global__ void k_ppr_loop_end(PprLoop *st, const PprQ *qs, cudaGraphConditionalHandle handle) {
    st->sweeps += 1;
    bool all = true;
    for (int q = 0; q < st->nq; q++) all &= qs[q].done != 0;
    cudaGraphSetConditional(handle, (!all && st->sweeps < st->max_sweeps) ? 1u : 0u);
}

// The sweep loop of eg_ppr_multi as one CUDA graph: a while node whose body
// is one sweep (row sums of the 32 lanes, fix-up of rows split between
// warps, rows without entries, seeds' teleport, finish and the per-query
// FP64 reductions) and the loop test.  Valid while the buffers, nq and the
// options it was captured with (key) stay the same.
int ppr_graph_build(eg_graph *g, const void *const key[8], uint32_t ntiles, uint32_t row_blocks, uint32_t fin_blocks,
                    const eg_ppr_opts &o, int nq, float *R, float *X, float *Y, float *hv, float *tvv, uint32_t *hr,
                    double2 *part, const uint32_t *d_seeds, const uint32_t *d_soff, PprQ *qs, PprLoop *lst) {
    eg_ctx *ctx = g->ctx;
    eg_bfs_graph &bg = g->ppg;
    if (bg.exec) cudaGraphExecDestroy(bg.exec);
    if (bg.graph) cudaGraphDestroy(bg.graph);
    bg.exec = nullptr;
    bg.graph = nullptr;
    const uint32_t n = g->n, m = (uint32_t)g->m;
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
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
    EG_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    if (row_blocks) {
        k_ppr_rows<<<row_blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.rid), bp<uint32_t>(g->csc.col), m, ntiles,
                                                        X, Y, hv, tvv, hr);
        k_ppr_fixup<<<row_blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.ptr), ntiles, hr, hv, tvv, Y);
    }
    k_ppr_empty<<<(uint32_t)ctx->sm_count * 8, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.ptr), n, Y);
    k_ppr_seeds<<<1, EG_PPR_LANES, 0, ctx->stream>>>(d_seeds, d_soff, d_soff + 1, nq, qs, o.damping, Y);
    k_ppr_finish<<<fin_blocks, 256, 0, ctx->stream>>>(Y, deg, n, o.damping, qs, R, X, part);
    k_ppr_reduce<<<1, EG_PPR_LANES, 0, ctx->stream>>>(part, fin_blocks, qs, 1);
    k_ppr_loop_end<<<1, 1, 0, ctx->stream>>>(lst, qs, handle);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &body);
    if (ce != cudaSuccess) return eg_fail(EG_ECUDA, "batched PageRank capture: %s", cudaGetErrorString(ce));
    cudaGraphExec_t exec = nullptr;
    EG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    bg.exec = exec;
    for (int i = 0; i < 8; i++) bg.key[i] = key[i];
    return EG_OK;
}
}  // namespace

extern "C" int eg_ppr_multi(eg_graph *g, const uint32_t *seeds, const uint32_t *seed_offsets, int nq,
                            const eg_ppr_opts *opts, float *ranks_out, eg_ppr_stats *stats) {
    if (!g || !seeds || !seed_offsets) return eg_fail(EG_EINVAL, "NULL argument");
    if (nq < 1 || nq > EG_PPR_LANES) return eg_fail(EG_EINVAL, "nq=%d: a batch holds 1..32 queries", nq);
    if (!(g->built & EG_LAYOUT_CSC) || !(g->built & EG_LAYOUT_CSR))
        return eg_fail(EG_ENOTBUILT, "personalised PageRank needs the CSC and the out-degrees");
    eg_ppr_opts o;
    if (opts) o = *opts;
    else {
        o.damping = 0.85f;
        o.max_iters = 50;
        for (int q = 0; q < EG_PPR_LANES; q++) o.tolerance[q] = 1e-6f;
    }
    if (o.max_iters < 1 || !(o.damping > 0.f && o.damping < 1.f)) return eg_fail(EG_EINVAL, "bad PPR options");
    const uint32_t n = g->n;
    for (int q = 0; q < nq; q++) {
        if (seed_offsets[q + 1] <= seed_offsets[q]) return eg_fail(EG_EINVAL, "query %d has no seed", q);
        for (uint32_t i = seed_offsets[q]; i < seed_offsets[q + 1]; i++)
            if (seeds[i] >= n) return eg_fail(EG_EINVAL, "seed %u >= n", seeds[i]);
    }
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t m = (uint32_t)g->m;
    const uint32_t ntiles = m ? eg_div_up(m, EG_PPR_TILE) : 0;
    const uint32_t nseeds_total = seed_offsets[nq];
    const uint32_t fin_blocks = (uint32_t)ctx->sm_count * 4;
    // work: R, X, Y [n*32 f32] | head/tail vals [ntiles*32 f32] | head rows | parts | seeds | offsets | queries
    const uint64_t vec = (uint64_t)n * EG_PPR_LANES;
    const uint64_t tv = (uint64_t)ntiles * EG_PPR_LANES;
    const uint64_t off_X = vec, off_Y = 2 * vec, off_hv = 3 * vec, off_tv = off_hv + tv, off_hr = off_tv + tv,
                   off_part = (off_hr + ntiles + 63) & ~63ull, off_seeds = off_part + (uint64_t)fin_blocks * 32 * 4,
                   off_soff = off_seeds + nseeds_total + 8, off_q = (off_soff + 40 + 63) & ~63ull,
                   off_loop = off_q + 32 * sizeof(PprQ) / 4;
    EG_TRY(eg_buf_ensure(ctx, g->ppr_work, (off_loop + 64) * 4));
    float *W = bp<float>(g->ppr_work);
    float *R = W, *X = W + off_X, *Y = W + off_Y, *hv = W + off_hv, *tvv = W + off_tv;
    uint32_t *hr = reinterpret_cast<uint32_t *>(W + off_hr);
    double2 *part = reinterpret_cast<double2 *>(W + off_part);
    uint32_t *d_seeds = reinterpret_cast<uint32_t *>(W + off_seeds);
    uint32_t *d_soff = reinterpret_cast<uint32_t *>(W + off_soff);
    PprQ *qs = reinterpret_cast<PprQ *>(W + off_q);
    PprLoop *lst = reinterpret_cast<PprLoop *>(W + off_loop);
    PprQ hq[EG_PPR_LANES];
    memset(hq, 0, sizeof(hq));
    for (int q = 0; q < nq; q++) {
        hq[q].active = 1;
        hq[q].tol = o.tolerance[q];
        hq[q].max_iters = o.max_iters;
        hq[q].nseeds = (int)(seed_offsets[q + 1] - seed_offsets[q]);
    }
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    EG_CUDA(cudaMemcpyAsync(d_seeds, seeds, (uint64_t)nseeds_total * 4, cudaMemcpyHostToDevice, ctx->stream));
    EG_CUDA(cudaMemcpyAsync(d_soff, seed_offsets, ((uint64_t)nq + 1) * 4, cudaMemcpyHostToDevice, ctx->stream));
    EG_CUDA(cudaMemcpyAsync(qs, hq, sizeof(hq), cudaMemcpyHostToDevice, ctx->stream));
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    const uint32_t lanes = nq == 32 ? 0xffffffffu : ((1u << nq) - 1u);
    k_ppr_init<<<(uint32_t)ctx->sm_count * 8, 256, 0, ctx->stream>>>(n, 0xffffffffu, R, X);
    EG_LAUNCHED(ctx);
    k_ppr_init_seeds<<<1, EG_PPR_LANES, 0, ctx->stream>>>(d_seeds, d_soff, d_soff + 1, lanes, qs, deg, R, X);
    EG_LAUNCHED(ctx);
    k_ppr_init_dangling<<<1, EG_PPR_LANES, 0, ctx->stream>>>(d_seeds, d_soff, d_soff + 1, lanes, deg, R, qs);
    EG_LAUNCHED(ctx);
    PprQ *hqs = (PprQ *)ctx->h_pinned;
    const uint32_t row_blocks = ntiles ? eg_div_up((uint64_t)ntiles * 32, 256) : 0;
    // the sweeps: one CUDA graph launch (a while node over one sweep)
    k_ppr_loop_init<<<1, 1, 0, ctx->stream>>>(lst, o.max_iters, nq);
    EG_LAUNCHED(ctx);
    uint32_t dmg;
    memcpy(&dmg, &o.damping, 4);
    // n and m are the graph's own; the seed offsets' place follows the seed count
    const void *key[8] = {W, g->csc.col.p, g->csc.rid.p, (const void *)(uintptr_t)nq,
                          (const void *)(uintptr_t)dmg, d_soff, g->csc.ptr.p, g->out_deg.p};
    eg_bfs_graph &bg = g->ppg;
    bool same = bg.exec != nullptr;
    for (int i = 0; i < 8 && same; i++) same = bg.key[i] == key[i];
    if (!same)
        EG_TRY(ppr_graph_build(g, key, ntiles, row_blocks, fin_blocks, o, nq, R, X, Y, hv, tvv, hr, part, d_seeds,
                               d_soff, qs, lst));
    EG_CUDA(cudaGraphLaunch(bg.exec, ctx->stream));
    ctx->launches += 1;
    PprLoop *hl = reinterpret_cast<PprLoop *>(hqs + EG_PPR_LANES);
    EG_TRY(eg_readback(ctx, hl, lst, sizeof(PprLoop), ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    const int it = hl->sweeps;
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (ranks_out) {
        EG_TRY(eg_buf_ensure(ctx, g->rank, (uint64_t)n * 4));
        for (int q = 0; q < nq; q++) {
            k_ppr_extract<<<(uint32_t)ctx->sm_count * 4, 256, 0, ctx->stream>>>(R, n, q, bp<float>(g->rank));
            EG_LAUNCHED(ctx);
            EG_CUDA(cudaMemcpyAsync(ranks_out + (uint64_t)q * n, g->rank.p, (uint64_t)n * 4, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        }
    }
    EG_CUDA(cudaMemcpyAsync(hqs, qs, sizeof(PprQ) * EG_PPR_LANES, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        for (int q = 0; q < nq; q++) {
            stats->iterations[q] = hqs[q].iters;
            stats->residual[q] = hqs[q].residual;
        }
        stats->sweeps = it;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}
