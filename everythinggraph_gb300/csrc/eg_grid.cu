// SpMV and PageRank over the 2-D grid layout (eg_graph_build_grid): the
// reference's prgrid_algo / iterator (prgrid_cilk.c:62-141) and the grid
// modes of spmv.c, which walk the P x P cells of init_grid_sort
// (init_all.c:252-361).
//
// A cell (i, j) holds the edges from source partition i to destination
// partition j.  The cells are visited in B x B blocks (block-row-major), so
// the CTAs running at one time read the x values of B source partitions and
// add into the y values of B destination partitions: with B chosen so that
// those 2B slices fit in a fraction of the 126 MB L2, the gathers of x and
// the additions into y hit L2, and HBM streams only the cells' (src, dst,
// value) words plus each slice once per block.  Work units are chunks of
// EG_GRID_CHUNK edges of a cell (the RMAT cells are very unequal), shared
// out over the grid by an exclusive prefix of the cells' chunk counts.
//
// y is accumulated with atomic adds, so fp32/fp64 sums are not in a fixed
// order (results agree within rounding, not bit for bit); u32 sums are exact.
// PageRank runs its iteration as: zero the accumulators, one grid pass adding
// contributions, one coalesced pass turning them into ranks and the next
// contributions (with the FP64 residual and dangling partials).
#include <stdlib.h>
#include <string.h>

#include "eg_bigwork.cuh"
#include "eg_internal.cuh"

#define EG_GRID_CHUNK 8192u
#define EG_GRID_L2_SLICES (24u << 20)  // bytes of x and y slices kept in L2 per block

namespace {

// Cell visiting order: t -> cell id for B x B blocks, and each cell's count of
// work units.
__global__ void k_grid_order(const uint32_t *__restrict__ cell_ptr, uint32_t P, uint32_t B, uint32_t *order,
                             uint32_t *units) {
    const uint64_t cells = (uint64_t)P * P;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < cells; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t I = (uint32_t)(t / ((uint64_t)B * P));
        const uint32_t rI = min(B, P - I * B);  // rows in this block-row
        const uint32_t t1 = (uint32_t)(t - (uint64_t)I * B * P);
        const uint32_t J = t1 / (rI * B);
        const uint32_t cJ = min(B, P - J * B);  // columns in this block
        const uint32_t t2 = t1 - J * rI * B;
        const uint32_t i = I * B + t2 / cJ, j = J * B + t2 % cJ;
        const uint32_t c = i * P + j;
        order[t] = c;
        units[t] = (cell_ptr[c + 1] - cell_ptr[c] + EG_GRID_CHUNK - 1) / EG_GRID_CHUNK;
    }
}

// Edge values of the grid entries (U[0,1) hashed from the endpoints, or 1).
__global__ void k_grid_values(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                              uint64_t seed, int unit, float *__restrict__ vals) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x)
        vals[e] = unit ? 1.0f : (float)(eg_edge_hash(seed, src[e], dst[e]) >> 40) * (1.0f / 16777216.0f);
}

// One pass over the cells: for every edge (s, d), op.add(s, d, e).
template <class Op>
__global__ void __launch_bounds__(256) k_grid_pass(const uint32_t *__restrict__ cell_ptr,
                                                   const uint32_t *__restrict__ order, const uint32_t *__restrict__ off,
                                                   uint32_t ncells, const uint32_t *__restrict__ src,
                                                   const uint32_t *__restrict__ dst, Op op) {
    if (!op.active()) return;
    const uint32_t total = off[ncells];
    for (uint32_t unit = blockIdx.x; unit < total; unit += gridDim.x) {
        const uint32_t t = eg_big_item(off, ncells, unit);
        const uint32_t c = order[t];
        const uint32_t b = cell_ptr[c] + (unit - off[t]) * EG_GRID_CHUNK;
        const uint32_t e = min(cell_ptr[c + 1], b + EG_GRID_CHUNK);
        for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) op.add(__ldg(src + p), __ldg(dst + p), p);
    }
}

template <int MODE>  // 0: y[dst] += x[src] / 1000, 1: y[src] += x[dst] / 1000, 2: y[src] += x[dst]
struct GridU32Op {
    const uint32_t *__restrict__ x;
    uint32_t *y;
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void add(uint32_t s, uint32_t d, uint32_t) const {
        if (MODE == 0) atomicAdd(y + d, __ldg(x + s) / 1000u);
        else if (MODE == 1) atomicAdd(y + s, __ldg(x + d) / 1000u);
        else atomicAdd(y + s, __ldg(x + d));
    }
};

struct GridF32Op {
    const float *__restrict__ x, *__restrict__ vals;
    float *y;
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void add(uint32_t s, uint32_t d, uint32_t p) const {
        atomicAdd(y + d, __fmul_rn(__ldg(vals + p), __ldg(x + s)));
    }
};

struct GridF64Op {
    const float *__restrict__ x, *__restrict__ vals;
    double *y;
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void add(uint32_t s, uint32_t d, uint32_t p) const {
        atomicAdd(y + d, __dmul_rn((double)__ldg(vals + p), (double)__ldg(x + s)));
    }
};

// PageRank state shared with the finish pass (the layout of eg_pr.cu's state).
struct GridPrDev {
    float base;
    int done;
    int iters;
    int pad;
    double residual;
    double dangling;
};

struct GridPrOp {
    const float *__restrict__ cin;
    float *acc;
    const GridPrDev *st;
    __device__ __forceinline__ bool active() const { return st->done == 0; }
    __device__ __forceinline__ void add(uint32_t s, uint32_t d, uint32_t) const { atomicAdd(acc + d, __ldg(cin + s)); }
};

__global__ void k_grid_zero(float *acc, uint32_t n, const GridPrDev *st) {
    if (st->done) return;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) acc[v] = 0.f;
}

// rank = base + d * acc, next contribution = rank / (deg * mult); per-block
// FP64 partials of |rank - old rank| and of the mass on out-degree-0 vertices.
__global__ void k_grid_pr_finish(const float *__restrict__ acc, const uint32_t *__restrict__ deg, uint32_t mult,
                                 uint32_t n, float damping, const GridPrDev *st, float *rank, float *cout,
                                 double2 *part) {
    __shared__ double2 s_red[8];
    if (st->done) return;
    const float base = st->base;
    eg_red2 red;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const float r = fmaf(damping, acc[v], base);
        const float old = rank[v];
        rank[v] = r;
        const uint32_t d = deg[v] * mult;
        cout[v] = d ? __fdiv_rn(r, (float)d) : 0.f;
        red.add(make_float2(fabsf(r - old), d ? 0.f : r));
    }
    double2 w = red.wide();
    for (int o = 16; o > 0; o >>= 1) {
        w.x += __shfl_down_sync(EG_FULL_MASK, w.x, o);
        w.y += __shfl_down_sync(EG_FULL_MASK, w.y, o);
    }
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = make_double2(0.0, 0.0);
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            t.x += s_red[k].x;
            t.y += s_red[k].y;
        }
        part[blockIdx.x] = t;
    }
}

__global__ void k_grid_pr_init(uint32_t n, float prev_init, const uint32_t *__restrict__ deg, uint32_t mult,
                               float *rank, float *contrib, double2 *part) {
    __shared__ double s_red[8];
    double dang = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = deg[v] * mult;
        rank[v] = prev_init;
        contrib[v] = d ? __fdiv_rn(prev_init, (float)d) : 0.f;
        if (!d) dang += (double)prev_init;
    }
    for (int o = 16; o > 0; o >>= 1) dang += __shfl_down_sync(EG_FULL_MASK, dang, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = dang;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s_red[k];
        part[blockIdx.x] = make_double2(0.0, t);
    }
}

// One block: FP64 sums of the partials, the next teleport base, the stop test.
__global__ void k_grid_pr_reduce(const double2 *__restrict__ part, uint32_t nparts, GridPrDev *st, uint32_t n,
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
        st->residual = s[0].x;
        st->dangling = s[0].y;
        double b = (1.0 - (double)damping) / (double)n;
        if (dangling) b += (double)damping * s[0].y / (double)n;
        st->base = (float)b;
        if (count_iter) {
            st->iters += 1;
            if (tol > 0.0 && s[0].x < tol) st->done = 1;
        }
    }
}

uint32_t grid_blocks(eg_ctx *ctx, uint64_t threads) {
    uint64_t b = (threads + 255) / 256;
    const uint64_t cap = (uint64_t)ctx->sm_count * 8;
    return (uint32_t)(b > cap ? cap : (b ? b : 1));
}

// Visiting order and work-unit offsets of the grid's cells (once per grid).
int grid_prepare(eg_graph *g) {
    if (!(g->built & EG_LAYOUT_GRID)) return eg_fail(EG_ENOTBUILT, "the 2-D grid is not built (eg_graph_build_grid)");
    if (g->grid_order_p == g->grid_p && g->grid_order.p) return EG_OK;
    eg_ctx *ctx = g->ctx;
    const uint32_t P = g->grid_p, n = g->n;
    const uint64_t cells = (uint64_t)P * P;
    const uint64_t slice = (uint64_t)(n / P + 1) * 8;  // x and y bytes of one partition pair
    uint64_t B = EG_GRID_L2_SLICES / (slice ? slice : 1);
    if (B < 1) B = 1;
    if (B > P) B = P;
    EG_TRY(eg_buf_ensure(ctx, g->grid_order, cells * 4));
    EG_TRY(eg_buf_ensure(ctx, g->grid_units, (cells + 1) * 4));
    EG_TRY(eg_buf_ensure(ctx, g->grid_off, (cells + 1) * 4));
    k_grid_order<<<grid_blocks(ctx, cells), 256, 0, ctx->stream>>>(bp<uint32_t>(g->cell_ptr), P, (uint32_t)B,
                                                                   bp<uint32_t>(g->grid_order),
                                                                   bp<uint32_t>(g->grid_units));
    EG_LAUNCHED(ctx);
    EG_TRY(eg_exscan_u32(ctx, bp<uint32_t>(g->grid_units), bp<uint32_t>(g->grid_off), cells));
    g->grid_order_p = P;
    g->grid_block = (uint32_t)B;
    return EG_OK;
}

int grid_values(eg_graph *g, uint64_t seed, int unit) {
    const int vk = unit ? 1 : 2;
    if (g->grid_vals.p && g->grid_vals_kind == vk && (vk == 1 || g->grid_vals_seed == seed)) return EG_OK;
    eg_ctx *ctx = g->ctx;
    EG_TRY(eg_buf_ensure(ctx, g->grid_vals, g->m * 4 + 16));
    k_grid_values<<<grid_blocks(ctx, g->m), 256, 0, ctx->stream>>>(bp<uint32_t>(g->gsrc), bp<uint32_t>(g->gdst), g->m,
                                                                   seed, unit, bp<float>(g->grid_vals));
    EG_LAUNCHED(ctx);
    g->grid_vals_kind = vk;
    g->grid_vals_seed = seed;
    return EG_OK;
}

template <class Op>
int grid_launch(eg_graph *g, const Op &op) {
    eg_ctx *ctx = g->ctx;
    const uint64_t cells = (uint64_t)g->grid_p * g->grid_p;
    k_grid_pass<Op><<<(uint32_t)ctx->sm_count * 8, 256, 0, ctx->stream>>>(
        bp<uint32_t>(g->cell_ptr), bp<uint32_t>(g->grid_order), bp<uint32_t>(g->grid_off), (uint32_t)cells,
        bp<uint32_t>(g->gsrc), bp<uint32_t>(g->gdst), op);
    EG_LAUNCHED(ctx);
    return EG_OK;
}

}  // namespace

// SpMV over the grid (called by eg_spmv when opts->grid is set): x and y are
// device arrays of n, y zeroed here.
int eg_grid_spmv(eg_graph *g, int kind, uint64_t value_seed, int unit_values, const void *d_x, void *d_y) {
    EG_TRY(grid_prepare(g));
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    EG_CUDA(cudaMemsetAsync(d_y, 0, (uint64_t)n * (kind == EG_SPMV_F64 ? 8 : 4), ctx->stream));
    switch (kind) {
        case EG_SPMV_U32_PULL:
            return grid_launch(g, GridU32Op<0>{(const uint32_t *)d_x, (uint32_t *)d_y});
        case EG_SPMV_U32_PUSH:
            return grid_launch(g, GridU32Op<1>{(const uint32_t *)d_x, (uint32_t *)d_y});
        case EG_SPMV_U32_EDGE:
            return grid_launch(g, GridU32Op<2>{(const uint32_t *)d_x, (uint32_t *)d_y});
        case EG_SPMV_F32:
            EG_TRY(grid_values(g, value_seed, unit_values));
            return grid_launch(g, GridF32Op{(const float *)d_x, bp<float>(g->grid_vals), (float *)d_y});
        case EG_SPMV_F64:
            EG_TRY(grid_values(g, value_seed, unit_values));
            return grid_launch(g, GridF64Op{(const float *)d_x, bp<float>(g->grid_vals), (double *)d_y});
        default:
            return eg_fail(EG_EINVAL, "SpMV kind %d is not available over the grid (compensated sums need a fixed "
                                      "order: use the CSC)", kind);
    }
}

// PageRank over the grid (called by eg_pagerank when opts->grid is set).
int eg_grid_pagerank(eg_graph *g, const eg_pr_opts &o, float *rank_out, eg_pr_stats *stats) {
    EG_TRY(grid_prepare(g));
    if (!(g->built & EG_LAYOUT_CSR)) return eg_fail(EG_ENOTBUILT, "grid PageRank needs the out-degrees (CSR)");
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    const uint32_t fb = grid_blocks(ctx, n);
    EG_TRY(eg_buf_ensure(ctx, g->rank, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->contrib0, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->contrib1, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->grid_acc, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->pr_part, ((uint64_t)fb + 64) * sizeof(double2)));
    EG_TRY(eg_buf_ensure(ctx, g->pr_stats, 512));
    GridPrDev *st = bp<GridPrDev>(g->pr_stats);
    double2 *part = bp<double2>(g->pr_part);
    const uint32_t *deg = bp<uint32_t>(g->out_deg);
    EG_CUDA(cudaMemsetAsync(st, 0, sizeof(GridPrDev), ctx->stream));
    const float prev_init = o.prev_init < 0.f ? 1.0f / (float)n : o.prev_init;
    k_grid_pr_init<<<fb, 256, 0, ctx->stream>>>(n, prev_init, deg, o.deg_multiplier, bp<float>(g->rank),
                                                bp<float>(g->contrib0), part);
    EG_LAUNCHED(ctx);
    k_grid_pr_reduce<<<1, 256, 0, ctx->stream>>>(part, fb, st, n, o.damping, o.dangling, 0.0, 0);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    for (int it = 0; it < o.iterations; it++) {
        const bool odd = o.swap && (it & 1);
        float *cin = odd ? bp<float>(g->contrib1) : bp<float>(g->contrib0);
        float *cout = odd ? bp<float>(g->contrib0) : bp<float>(g->contrib1);
        k_grid_zero<<<fb, 256, 0, ctx->stream>>>(bp<float>(g->grid_acc), n, st);
        EG_LAUNCHED(ctx);
        EG_TRY(grid_launch(g, GridPrOp{cin, bp<float>(g->grid_acc), st}));
        k_grid_pr_finish<<<fb, 256, 0, ctx->stream>>>(bp<float>(g->grid_acc), deg, o.deg_multiplier, n, o.damping, st,
                                                      bp<float>(g->rank), cout, part);
        EG_LAUNCHED(ctx);
        k_grid_pr_reduce<<<1, 256, 0, ctx->stream>>>(part, fb, st, n, o.damping, o.dangling, o.tolerance, 1);
        EG_LAUNCHED(ctx);
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    GridPrDev hst;
    EG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, ctx->stream));
    if (rank_out) EG_CUDA(cudaMemcpyAsync(rank_out, g->rank.p, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->iterations_run = hst.iters;
        stats->residual = hst.residual;
        stats->dangling_mass = hst.dangling;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
        stats->row_kernel_ms = 0.f;
    }
    return EG_OK;
}
