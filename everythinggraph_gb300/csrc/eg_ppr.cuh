// Kernels of the batched personalised PageRank (see eg_ppr.cu), shared with
// the query server.  Internal linkage: each translation unit has its copy.
#pragma once
#include "eg_internal.cuh"

#define EG_PPR_LANES 32
#ifndef EG_PPR_TILE
#define EG_PPR_TILE 1024
#endif
#define EG_PPR_NONE 0xffffffffu
#ifndef EG_PPR_INFLIGHT
#define EG_PPR_INFLIGHT 8  // row loads in flight per lane in k_ppr_rows
#endif
#ifndef EG_PPR_MINB
#define EG_PPR_MINB 4      // resident CTAs per SM asked of the compiler (64 registers)
#endif

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

__device__ __forceinline__ float4 eg_f4add(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 eg_f4shfl(unsigned mask, float4 v, int src) {
    return make_float4(__shfl_sync(mask, v.x, src), __shfl_sync(mask, v.y, src), __shfl_sync(mask, v.z, src),
                       __shfl_sync(mask, v.w, src));
}

// Y[v][q] = sum over CSC entries of row v of X[u][q], for the rows whose
// entries lie in this warp's tile; rows open at the tile ends go to carries.
//
// The warp is four groups of 8 lanes; lane s of a group holds queries
// 4s..4s+3 (one 16-byte load brings a group a whole 128-byte row of X), and
// group g walks quarter g of the tile on its own, 8 entries per step with
// their 8 row loads in flight.  A row is summed in entry order inside a
// group; a row crossing quarter boundaries is completed by the merge at the
// end, which adds the groups' parts in quarter order.  EG_PPR_INFLIGHT rows
// (8 or 4) are loaded before any of them is added.
__global__ void __launch_bounds__(256, EG_PPR_MINB) k_ppr_rows(const uint32_t *__restrict__ rid,
                                                     const uint32_t *__restrict__ col, uint32_t m, uint32_t ntiles,
                                                     const float *__restrict__ X, float *__restrict__ Y,
                                                     float *__restrict__ head_val, float *__restrict__ tail_val,
                                                     uint32_t *__restrict__ head_row) {
    constexpr uint32_t SUB = EG_PPR_TILE / 4;
    const uint32_t lane = threadIdx.x & 31, grp = lane >> 3, sl = lane & 7;
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= ntiles) return;
    const float4 *__restrict__ X4 = reinterpret_cast<const float4 *>(X);
    float4 *__restrict__ Y4 = reinterpret_cast<float4 *>(Y);
    const uint32_t E0 = t * EG_PPR_TILE, E1 = min(E0 + EG_PPR_TILE, m);
    const uint32_t hrow = (E0 > 0 && __ldg(rid + E0 - 1) == __ldg(rid + E0)) ? __ldg(rid + E0) : EG_PPR_NONE;
    const uint32_t tnext = E1 < m ? __ldg(rid + E1) : EG_PPR_NONE;
    const uint32_t S0 = min(E0 + grp * SUB, E1), S1 = min(S0 + SUB, E1);
    const unsigned gmask = 0xffu << (grp * 8);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    // group state: its first row (and that row's sum if it ended inside the
    // quarter), its open last row and partial sum
    const uint32_t first = S0 < S1 ? __ldg(rid + S0) : EG_PPR_NONE;
    bool fclosed = false;
    float4 fval = zero, acc = zero;
    uint32_t cur = first;
    constexpr uint32_t NB = EG_PPR_INFLIGHT;
    static_assert(NB == 4 || NB == 8, "a group's 8 lanes load 8 entries' ids at once");
    for (uint32_t base = S0; base < S1; base += 8) {
        const uint32_t e = base + sl;
        const uint32_t my_r = e < S1 ? __ldg(rid + e) : EG_PPR_NONE;
        const uint32_t my_c = e < S1 ? __ldg(col + e) : 0u;
        const uint32_t cnt = min(8u, S1 - base);
#pragma unroll
        for (uint32_t h = 0; h < 8; h += NB) {
        uint32_t rr[NB];
        float4 xv[NB];
#pragma unroll
        for (uint32_t q = 0; q < NB; q++) {
            rr[q] = __shfl_sync(gmask, my_r, h + q, 8);
            const uint32_t u = __shfl_sync(gmask, my_c, h + q, 8);
            xv[q] = h + q < cnt ? __ldg(X4 + (uint64_t)u * (EG_PPR_LANES / 4) + sl) : zero;
        }
#pragma unroll
        for (uint32_t q = 0; q < NB; q++) {
            if (h + q >= cnt) break;
            if (rr[q] != cur) {  // row `cur` ended inside the quarter
                if (cur == first) {
                    fclosed = true;
                    fval = acc;
                } else {
                    Y4[(uint64_t)cur * (EG_PPR_LANES / 4) + sl] = acc;
                }
                acc = zero;
                cur = rr[q];
            }
            acc = eg_f4add(acc, xv[q]);
        }
        }
    }
    // merge the quarters in order: (orow, oval) is the row open so far
    uint32_t orow = EG_PPR_NONE;
    float4 oval = zero;
    bool hdone = false;
    float4 hval = zero;
    auto emit = [&](uint32_t row, float4 v) {  // every group holds the merged values: group 0 writes
        if (row == hrow) {
            hdone = true;
            hval = v;
        } else if (lane < 8) {
            Y4[(uint64_t)row * (EG_PPR_LANES / 4) + sl] = v;
        }
    };
#pragma unroll
    for (uint32_t gq = 0; gq < 4; gq++) {
        const int src = (int)(gq * 8 + sl);
        const uint32_t f = __shfl_sync(EG_FULL_MASK, first, src);
        if (f == EG_PPR_NONE) continue;  // empty quarter (short last tile)
        const bool fc = __shfl_sync(EG_FULL_MASK, fclosed, src);
        const uint32_t c = __shfl_sync(EG_FULL_MASK, cur, src);
        const float4 fv = eg_f4shfl(EG_FULL_MASK, fval, src);
        const float4 av = eg_f4shfl(EG_FULL_MASK, acc, src);
        if (fc) {  // the quarter's first row ended inside it
            if (orow == f) {
                emit(f, eg_f4add(oval, fv));
            } else {
                if (orow != EG_PPR_NONE) emit(orow, oval);
                emit(f, fv);
            }
            orow = c;
            oval = av;
        } else if (orow == f) {  // one row through the whole quarter
            oval = eg_f4add(oval, av);
        } else {
            if (orow != EG_PPR_NONE) emit(orow, oval);
            orow = f;
            oval = av;
        }
    }
    float4 *tv = reinterpret_cast<float4 *>(tail_val) + (uint64_t)t * (EG_PPR_LANES / 4);
    // the last row: complete if the next tile starts another row
    if (tnext != orow) {
        emit(orow, oval);
        if (lane < 8) tv[sl] = zero;
    } else if (lane < 8) {
        tv[sl] = oval;
    }
    if (lane == 0) head_row[t] = hdone ? hrow : EG_PPR_NONE;
    if (hdone && lane < 8) reinterpret_cast<float4 *>(head_val)[(uint64_t)t * (EG_PPR_LANES / 4) + sl] = hval;
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
// Query q's seeds are seeds[sbeg[q] .. send[q]).
__global__ void k_ppr_seeds(const uint32_t *__restrict__ seeds, const uint32_t *__restrict__ sbeg,
                            const uint32_t *__restrict__ send, int nq, const PprQ *__restrict__ qs, float d,
                            float *__restrict__ Y) {
    const int q = threadIdx.x;
    if (q >= nq || !qs[q].active || qs[q].done) return;
    const float c = (float)(((1.0 - (double)d) + (double)d * qs[q].dangling) / ((double)qs[q].nseeds * (double)d));
    for (uint32_t i = sbeg[q]; i < send[q]; i++) Y[(uint64_t)seeds[i] * EG_PPR_LANES + q] += c;
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
    eg_red2 acc;  // fp32 TwoSum pairs per lane, widened once (FP64 issues slowly)
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        if (!live) continue;
        const uint64_t i = (uint64_t)v * EG_PPR_LANES + lane;
        const float r = d * Y[i];
        const float old = R[i];
        R[i] = r;
        const uint32_t dv = deg[v];
        X[i] = dv ? __fdiv_rn(r, (float)dv) : 0.f;
        acc.add(make_float2(fabsf(r - old), dv ? 0.f : r));
    }
    s_part[warp][lane] = acc.wide();
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

// Zero the columns of the lanes in `mask` (every lane: mask = ~0).
__global__ void k_ppr_init(uint32_t n, uint32_t mask, float *R, float *X) {
    const uint64_t total = (uint64_t)n * EG_PPR_LANES;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!((mask >> (i & 31)) & 1u)) continue;
        R[i] = 0.f;
        X[i] = 0.f;
    }
}
// Lanes in `mask` start from R = t: their columns must be zero on entry.
__global__ void k_ppr_init_seeds(const uint32_t *__restrict__ seeds, const uint32_t *__restrict__ sbeg,
                                 const uint32_t *__restrict__ send, uint32_t mask, const PprQ *qs,
                                 const uint32_t *__restrict__ deg, float *R, float *X) {
    const int q = threadIdx.x;
    if (q >= EG_PPR_LANES || !((mask >> q) & 1u) || !qs[q].active) return;
    const float w = 1.0f / (float)qs[q].nseeds;
    for (uint32_t i = sbeg[q]; i < send[q]; i++) R[(uint64_t)seeds[i] * EG_PPR_LANES + q] += w;
    for (uint32_t i = sbeg[q]; i < send[q]; i++) {
        const uint32_t s = seeds[i];
        const uint32_t dv = deg[s];
        X[(uint64_t)s * EG_PPR_LANES + q] = dv ? __fdiv_rn(R[(uint64_t)s * EG_PPR_LANES + q], (float)dv) : 0.f;
    }
}
__global__ void k_ppr_init_dangling(const uint32_t *__restrict__ seeds, const uint32_t *__restrict__ sbeg,
                                    const uint32_t *__restrict__ send, uint32_t mask,
                                    const uint32_t *__restrict__ deg, const float *R, PprQ *qs) {
    const int q = threadIdx.x;
    if (q >= EG_PPR_LANES || !((mask >> q) & 1u) || !qs[q].active) return;
    double dang = 0.0;
    for (uint32_t i = sbeg[q]; i < send[q]; i++) {
        const uint32_t s = seeds[i];
        bool first = true;  // count each distinct seed once
        for (uint32_t j = sbeg[q]; j < i; j++) first &= seeds[j] != s;
        if (first && deg[s] == 0) dang += (double)R[(uint64_t)s * EG_PPR_LANES + q];
    }
    qs[q].dangling = dang;
}

__global__ void k_ppr_extract(const float *__restrict__ R, uint32_t n, int q, float *__restrict__ out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        out[v] = R[(uint64_t)v * EG_PPR_LANES + q];
}

}  // namespace
