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

#include "eg_internal.cuh"

#define EG_PPR_LANES 32
#define EG_PPR_TILE 1024
#define EG_PPR_NONE 0xffffffffu

namespace {

struct PprQ {  // per-query state (device)
    double residual;
    double dangling;
    float tol;
    int iters;
    int max_iters;
    int done;
    int nseeds;
    int active;  // lane in use
};

// Y[v][q] = sum over CSC entries of row v of X[u][q], for the rows whose
// entries lie in this warp's tile; rows open at the tile ends go to carries.
__global__ void __launch_bounds__(256) k_ppr_rows(const uint32_t *__restrict__ rid, const uint32_t *__restrict__ col,
                                                  uint32_t m, uint32_t ntiles, const float *__restrict__ X,
                                                  float *__restrict__ Y, float *__restrict__ head_val,
                                                  float *__restrict__ tail_val, uint32_t *__restrict__ head_row) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= ntiles) return;
    const uint32_t E0 = t * EG_PPR_TILE, E1 = min(E0 + EG_PPR_TILE, m);
    const uint32_t first = __ldg(rid + E0);
    const uint32_t hrow = (E0 > 0 && __ldg(rid + E0 - 1) == first) ? first : EG_PPR_NONE;
    const uint32_t tnext = E1 < m ? __ldg(rid + E1) : EG_PPR_NONE;
    float acc = 0.f;
    uint32_t cur = first;
    bool hdone = false;
    float hval = 0.f;
    for (uint32_t base = E0; base < E1; base += 32) {
        const uint32_t e = base + lane;
        const uint32_t my_r = e < E1 ? __ldg(rid + e) : EG_PPR_NONE;
        const uint32_t my_c = e < E1 ? __ldg(col + e) : 0u;
        const uint32_t cnt = min(32u, E1 - base);
        for (uint32_t j = 0; j < cnt; j++) {
            const uint32_t r = __shfl_sync(EG_FULL_MASK, my_r, j);
            const uint32_t u = __shfl_sync(EG_FULL_MASK, my_c, j);
            if (r != cur) {  // row `cur` ended inside the tile
                if (cur == hrow) {
                    hdone = true;
                    hval = acc;
                } else {
                    Y[(uint64_t)cur * EG_PPR_LANES + lane] = acc;
                }
                acc = 0.f;
                cur = r;
            }
            acc += __ldg(X + (uint64_t)u * EG_PPR_LANES + lane);
        }
    }
    // the last row: complete if the next tile starts another row
    if (tnext != cur) {
        if (cur == hrow) {
            hdone = true;
            hval = acc;
        } else {
            Y[(uint64_t)cur * EG_PPR_LANES + lane] = acc;
        }
        tail_val[(uint64_t)t * EG_PPR_LANES + lane] = 0.f;
    } else {
        tail_val[(uint64_t)t * EG_PPR_LANES + lane] = acc;
    }
    if (lane == 0) head_row[t] = hdone ? hrow : EG_PPR_NONE;
    if (hdone) head_val[(uint64_t)t * EG_PPR_LANES + lane] = hval;
}

// Rows split between tiles: a warp per tile with a head row adds the tails of
// the preceding tiles (nearest first is irrelevant: the order is fixed).
__global__ void k_ppr_fixup(const uint32_t *__restrict__ ptr, uint32_t ntiles, const uint32_t *__restrict__ head_row,
                            const float *__restrict__ head_val, const float *__restrict__ tail_val,
                            float *__restrict__ Y) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= ntiles) return;
    const uint32_t row = head_row[t];
    if (row == EG_PPR_NONE) return;
    const uint32_t rstart = ptr[row];
    float tot = 0.f;
    for (int k = (int)t - 1; k >= 0; k--) {
        tot += tail_val[(uint64_t)k * EG_PPR_LANES + lane];
        if (rstart >= (uint32_t)k * EG_PPR_TILE) break;  // the row begins in tile k
    }
    tot += head_val[(uint64_t)t * EG_PPR_LANES + lane];
    Y[(uint64_t)row * EG_PPR_LANES + lane] = tot;
}

// Rows without in-edges sum to zero.
__global__ void k_ppr_empty(const uint32_t *__restrict__ ptr, uint32_t n, float *__restrict__ Y) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps)
        if (ptr[v] == ptr[v + 1]) Y[(uint64_t)v * EG_PPR_LANES + lane] = 0.f;
}

// Teleport plus returned dangling mass at the seeds: Y[s][q] += c_q / d so that
// d * Y carries (1 - d + d * dangling_q) / nseeds_q at every seed occurrence.
__global__ void k_ppr_seeds(const uint32_t *__restrict__ seeds, const uint32_t *__restrict__ soff, int nq,
                            const PprQ *__restrict__ qs, float d, float *__restrict__ Y) {
    const int q = threadIdx.x;
    if (q >= nq || !qs[q].active || qs[q].done) return;
    const float c = (float)(((1.0 - (double)d) + (double)d * qs[q].dangling) / ((double)qs[q].nseeds * (double)d));
    for (uint32_t i = soff[q]; i < soff[q + 1]; i++) Y[(uint64_t)seeds[i] * EG_PPR_LANES + q] += c;
}

// R = d * Y, X = R / deg; per-block FP64 partials of |R - R_old| and of the
// mass on out-degree-0 vertices, per query.
__global__ void __launch_bounds__(256) k_ppr_finish(const float *__restrict__ Y, const uint32_t *__restrict__ deg,
                                                    uint32_t n, float d, const PprQ *__restrict__ qs,
                                                    float *__restrict__ R, float *__restrict__ X,
                                                    double2 *__restrict__ part) {
    __shared__ double2 s_part[8][EG_PPR_LANES];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool live = qs[lane].active && !qs[lane].done;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    double res = 0.0, dang = 0.0;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        if (!live) continue;
        const uint64_t i = (uint64_t)v * EG_PPR_LANES + lane;
        const float r = d * Y[i];
        res += fabs((double)r - (double)R[i]);
        R[i] = r;
        const uint32_t dv = deg[v];
        X[i] = dv ? __fdiv_rn(r, (float)dv) : 0.f;
        if (!dv) dang += (double)r;
    }
    s_part[warp][lane] = make_double2(res, dang);
    __syncthreads();
    if (warp == 0) {
        double2 s = make_double2(0.0, 0.0);
        for (int w = 0; w < 8; w++) {
            s.x += s_part[w][lane].x;
            s.y += s_part[w][lane].y;
        }
        part[(uint64_t)blockIdx.x * EG_PPR_LANES + lane] = s;
    }
}

// Per query: fixed-order FP64 sum of the block partials, stop test.
__global__ void k_ppr_reduce(const double2 *__restrict__ part, uint32_t nblocks, PprQ *qs, int count_iter) {
    const int q = threadIdx.x;
    if (q >= EG_PPR_LANES) return;
    PprQ &s = qs[q];
    if (!s.active || s.done) return;
    double res = 0.0, dang = 0.0;
    for (uint32_t b = 0; b < nblocks; b++) {
        res += part[(uint64_t)b * EG_PPR_LANES + q].x;
        dang += part[(uint64_t)b * EG_PPR_LANES + q].y;
    }
    s.dangling = dang;
    if (count_iter) {
        s.residual = res;
        s.iters += 1;
        if (res < (double)s.tol || s.iters >= s.max_iters) s.done = 1;
    }
}

// Initial vectors: R = t (teleport over the seeds), X = R / deg.
__global__ void k_ppr_init(uint32_t n, float *R, float *X) {
    const uint64_t total = (uint64_t)n * EG_PPR_LANES;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        R[i] = 0.f;
        X[i] = 0.f;
    }
}
__global__ void k_ppr_init_seeds(const uint32_t *__restrict__ seeds, const uint32_t *__restrict__ soff, int nq,
                                 const PprQ *qs, const uint32_t *__restrict__ deg, float *R, float *X) {
    const int q = threadIdx.x;
    if (q >= nq || !qs[q].active) return;
    const float w = 1.0f / (float)qs[q].nseeds;
    for (uint32_t i = soff[q]; i < soff[q + 1]; i++) R[(uint64_t)seeds[i] * EG_PPR_LANES + q] += w;
    for (uint32_t i = soff[q]; i < soff[q + 1]; i++) {
        const uint32_t s = seeds[i];
        const uint32_t dv = deg[s];
        X[(uint64_t)s * EG_PPR_LANES + q] = dv ? __fdiv_rn(R[(uint64_t)s * EG_PPR_LANES + q], (float)dv) : 0.f;
    }
}
__global__ void k_ppr_init_dangling(const uint32_t *__restrict__ seeds, const uint32_t *__restrict__ soff, int nq,
                                    const uint32_t *__restrict__ deg, const float *R, PprQ *qs) {
    const int q = threadIdx.x;
    if (q >= nq || !qs[q].active) return;
    double dang = 0.0;
    for (uint32_t i = soff[q]; i < soff[q + 1]; i++) {
        const uint32_t s = seeds[i];
        bool first = true;  // count each distinct seed once
        for (uint32_t j = soff[q]; j < i; j++) first &= seeds[j] != s;
        if (first && deg[s] == 0) dang += (double)R[(uint64_t)s * EG_PPR_LANES + q];
    }
    qs[q].dangling = dang;
}

__global__ void k_ppr_extract(const float *__restrict__ R, uint32_t n, int q, float *__restrict__ out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        out[v] = R[(uint64_t)v * EG_PPR_LANES + q];
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
                   off_soff = off_seeds + nseeds_total + 8, off_q = (off_soff + 40 + 63) & ~63ull;
    EG_TRY(eg_buf_ensure(ctx, g->ppr_work, (off_q + 32 * sizeof(PprQ) / 4 + 64) * 4));
    float *W = bp<float>(g->ppr_work);
    float *R = W, *X = W + off_X, *Y = W + off_Y, *hv = W + off_hv, *tvv = W + off_tv;
    uint32_t *hr = reinterpret_cast<uint32_t *>(W + off_hr);
    double2 *part = reinterpret_cast<double2 *>(W + off_part);
    uint32_t *d_seeds = reinterpret_cast<uint32_t *>(W + off_seeds);
    uint32_t *d_soff = reinterpret_cast<uint32_t *>(W + off_soff);
    PprQ *qs = reinterpret_cast<PprQ *>(W + off_q);
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
    k_ppr_init<<<(uint32_t)ctx->sm_count * 8, 256, 0, ctx->stream>>>(n, R, X);
    EG_LAUNCHED(ctx);
    k_ppr_init_seeds<<<1, EG_PPR_LANES, 0, ctx->stream>>>(d_seeds, d_soff, nq, qs, deg, R, X);
    EG_LAUNCHED(ctx);
    k_ppr_init_dangling<<<1, EG_PPR_LANES, 0, ctx->stream>>>(d_seeds, d_soff, nq, deg, R, qs);
    EG_LAUNCHED(ctx);
    PprQ *hqs = (PprQ *)ctx->h_pinned;
    const uint32_t row_blocks = ntiles ? eg_div_up((uint64_t)ntiles * 32, 256) : 0;
    const uint32_t empty_blocks = (uint32_t)ctx->sm_count * 8;
    int it;
    for (it = 0; it < o.max_iters; it++) {
        if (row_blocks) {
            k_ppr_rows<<<row_blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.rid), bp<uint32_t>(g->csc.col), m, ntiles,
                                                            X, Y, hv, tvv, hr);
            EG_LAUNCHED(ctx);
            k_ppr_fixup<<<row_blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.ptr), ntiles, hr, hv, tvv, Y);
            EG_LAUNCHED(ctx);
        }
        k_ppr_empty<<<empty_blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.ptr), n, Y);
        EG_LAUNCHED(ctx);
        k_ppr_seeds<<<1, EG_PPR_LANES, 0, ctx->stream>>>(d_seeds, d_soff, nq, qs, o.damping, Y);
        EG_LAUNCHED(ctx);
        k_ppr_finish<<<fin_blocks, 256, 0, ctx->stream>>>(Y, deg, n, o.damping, qs, R, X, part);
        EG_LAUNCHED(ctx);
        k_ppr_reduce<<<1, EG_PPR_LANES, 0, ctx->stream>>>(part, fin_blocks, qs, 1);
        EG_LAUNCHED(ctx);
        // every 4 iterations: stop once every query is done
        if ((it & 3) == 3 || it + 1 == o.max_iters) {
            EG_CUDA(cudaMemcpyAsync(hqs, qs, sizeof(PprQ) * EG_PPR_LANES, cudaMemcpyDeviceToHost, ctx->stream));
            EG_CUDA(cudaStreamSynchronize(ctx->stream));
            bool all = true;
            for (int q = 0; q < nq; q++) all &= hqs[q].done != 0;
            if (all) {
                it++;
                break;
            }
        }
    }
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
