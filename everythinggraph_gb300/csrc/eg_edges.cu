// Edge-array load modes and the edge-centric algorithms that stream them.
//
// Replaces the reference's edge-list loader init_edgelist (init_all.c:573-628,
// load modes 7, 8 and 9) and the loops that run over that array instead of an
// adjacency: bfs_edgecentric (bfs_simple.c:58-103), pr_algo_edgecentric
// (pagerank_simple.c:40-61) and prgrid_algo_col (prgrid_cilk.c:79-88), and
// the SpMV edge loop (spmv.c:130-135).  The WCC edge loop (wcc.c:235-261) is
// eg_wcc's hooking over the input edges, which needs no adjacency either.
//
// No CSR or CSC is built.  The array is the input's edges (with the reversed
// copies after them for an undirected graph, as preload_graph lays out
// memblock, init_all.c:81-110) in one of three orders:
//   mode 9  file order, no sort;
//   mode 7  a stable sort by source (one LSD radix sort);
//   mode 8  by source, then destination (two stable radix sorts).
// It is kept as two u32 arrays, sources and destinations, so that a BFS level
// whose frontier holds few vertices reads 4 bytes per edge: the destination
// is loaded only for edges whose source is in the frontier.
//
// The kernels stream the arrays with 16-byte loads, evict-first (each byte is
// read once per pass), from a grid of resident CTAs.  Per edge:
//   BFS level   4 B source + a frontier-bitmap bit (L1/L2) [+ 4 B destination
//               + a visited-bitmap word atomic when the source is active];
//   PageRank    8 B + a contribution gather (L2) + one fp32 atomic add in L2
//               (the reference's write_add, pagerank_simple.c:51);
//   SpMV (u32)  8 B + an x gather + one atomic add per run of equal sources.
#include "eg_internal.cuh"

#define EG_EDGES_T 256

namespace {

struct EdgeCounters {
    uint32_t claimed;  // vertices a BFS level reached
    uint32_t pad[3];
};

// PageRank over the edge array: the FP64 sums of the last finished iterate.
struct EdgePrDev {
    double dangling;  // mass on vertices without out-edges
    double residual;  // L1 change from the iterate before
};

__global__ void k_edges_unpack(const uint32_t *__restrict__ pairs, uint64_t m_in, int undirected, uint32_t n,
                               uint32_t *__restrict__ src, uint32_t *__restrict__ dst, uint32_t *bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t M = undirected ? 2 * m_in : m_in;
    uint32_t anybad = 0;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < M; k += stride) {
        const uint64_t e = k < m_in ? k : k - m_in;
        const uint2 p = __ldcs(reinterpret_cast<const uint2 *>(pairs) + e);
        const uint32_t s = k < m_in ? p.x : p.y;
        const uint32_t d = k < m_in ? p.y : p.x;
        anybad |= (s >= n) | (d >= n);
        src[k] = s;
        dst[k] = d;
    }
    if (__any_sync(EG_FULL_MASK, anybad) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(EG_FULL_MASK, v, o);
    return v;
}

__global__ void k_eb_init(uint32_t n, uint32_t nw, uint32_t root, int32_t *level, int32_t *parent, uint32_t *visited,
                          uint32_t *front, uint32_t *next) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        level[v] = v == root ? 1 : 0;
        if (parent) parent[v] = v == root ? (int32_t)root : -1;
    }
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += stride) {
        const uint32_t bit = (root >> 5) == w ? 1u << (root & 31) : 0u;
        visited[w] = bit;
        front[w] = bit;
        next[w] = 0u;
    }
}

// Edge (s, d) with s in the frontier: d joins the next level unless another
// edge got it first (the CAS on dist[dst] of bfs_simple.c:69, here the
// visited bit).  Returns 1 when this edge claimed d.
__device__ __forceinline__ uint32_t eb_claim(uint32_t s, uint32_t d, uint32_t *visited, uint32_t *next, int32_t *level,
                                             int32_t *parent, int32_t lvl) {
    const uint32_t bit = 1u << (d & 31);
    if (__ldcg(visited + (d >> 5)) & bit) return 0u;
    if (atomicOr(visited + (d >> 5), bit) & bit) return 0u;
    level[d] = lvl;
    if (parent) parent[d] = (int32_t)s;
    atomicOr(next + (d >> 5), bit);
    return 1u;
}

__device__ __forceinline__ bool in_front(const uint32_t *__restrict__ front, uint32_t s) {
    return (__ldg(front + (s >> 5)) >> (s & 31)) & 1u;
}

// One BFS level over the whole edge array (bfs_edgecentric's parallel_for,
// bfs_simple.c:64-74): 4 edges per thread per step.
__global__ void __launch_bounds__(EG_EDGES_T) k_eb_level(const uint32_t *__restrict__ esrc,
                                                         const uint32_t *__restrict__ edst, uint64_t m,
                                                         const uint32_t *__restrict__ front, uint32_t *next,
                                                         uint32_t *visited, int32_t *level, int32_t *parent,
                                                         int32_t lvl, EdgeCounters *cnt) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nq = m >> 2;
    uint32_t c = 0;
    for (uint64_t q = t0; q < nq; q += stride) {
        const uint4 s = __ldcs(reinterpret_cast<const uint4 *>(esrc) + q);
        const bool a0 = in_front(front, s.x), a1 = in_front(front, s.y), a2 = in_front(front, s.z),
                   a3 = in_front(front, s.w);
        if (a0 | a1 | a2 | a3) {
            const uint32_t *dp = edst + 4 * q;
            if (a0) c += eb_claim(s.x, __ldcs(dp + 0), visited, next, level, parent, lvl);
            if (a1) c += eb_claim(s.y, __ldcs(dp + 1), visited, next, level, parent, lvl);
            if (a2) c += eb_claim(s.z, __ldcs(dp + 2), visited, next, level, parent, lvl);
            if (a3) c += eb_claim(s.w, __ldcs(dp + 3), visited, next, level, parent, lvl);
        }
    }
    for (uint64_t e = 4 * nq + t0; e < m; e += stride) {
        const uint32_t s = esrc[e];
        if (in_front(front, s)) c += eb_claim(s, edst[e], visited, next, level, parent, lvl);
    }
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&cnt->claimed, c);
}

// Sum of the out-degrees of the reached vertices and their count.
__global__ void k_eb_reach(const int32_t *__restrict__ level, const uint32_t *__restrict__ deg, uint32_t n,
                           unsigned long long *out) {
    unsigned long long e = 0, r = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (level[v] > 0) {
            e += deg[v];
            r++;
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_down_sync(EG_FULL_MASK, e, o);
        r += __shfl_down_sync(EG_FULL_MASK, r, o);
    }
    if ((threadIdx.x & 31) == 0 && (e || r)) {
        atomicAdd(out, e);
        atomicAdd(out + 1, r);
    }
}

// Block sums of two FP64 values into st (one atomic per block each).
__device__ __forceinline__ void block_add2(double a, double b, double *out_a, double *out_b) {
    __shared__ double s_a[EG_EDGES_T / 32], s_b[EG_EDGES_T / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(EG_FULL_MASK, a, o);
        b += __shfl_down_sync(EG_FULL_MASK, b, o);
    }
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_a[w] = a;
        s_b[w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (uint32_t i = 0; i < blockDim.x / 32; i++) {
            ta += s_a[i];
            tb += s_b[i];
        }
        if (ta != 0.0) atomicAdd(out_a, ta);
        if (tb != 0.0) atomicAdd(out_b, tb);
    }
}

// prev = p0 everywhere, contributions p0 / deg, accumulators zero; the
// dangling mass of the start vector into st.
__global__ void __launch_bounds__(EG_EDGES_T) k_ep_init(uint32_t n, float p0, const uint32_t *__restrict__ deg,
                                                        uint32_t mult, float *rank, float *contrib, float *acc,
                                                        EdgePrDev *st) {
    float dang = 0.f;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = deg[v] * mult;
        rank[v] = p0;
        contrib[v] = d ? __fdiv_rn(p0, (float)d) : 0.f;
        acc[v] = 0.f;
        if (!d) dang += p0;
    }
    block_add2((double)dang, 0.0, &st->dangling, &st->residual);
}

// rank[dst] += contrib[src] for every edge (write_add, pagerank_simple.c:51
// and prgrid_cilk.c:85), 4 edges per thread per step.
__global__ void __launch_bounds__(EG_EDGES_T) k_ep_scatter(const uint32_t *__restrict__ esrc,
                                                           const uint32_t *__restrict__ edst, uint64_t m,
                                                           const float *__restrict__ contrib, float *acc) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nq = m >> 2;
    for (uint64_t q = t0; q < nq; q += stride) {
        const uint4 s = __ldcs(reinterpret_cast<const uint4 *>(esrc) + q);
        const uint4 d = __ldcs(reinterpret_cast<const uint4 *>(edst) + q);
        atomicAdd(acc + d.x, __ldg(contrib + s.x));
        atomicAdd(acc + d.y, __ldg(contrib + s.y));
        atomicAdd(acc + d.z, __ldg(contrib + s.z));
        atomicAdd(acc + d.w, __ldg(contrib + s.w));
    }
    for (uint64_t e = 4 * nq + t0; e < m; e += stride) atomicAdd(acc + edst[e], __ldg(contrib + esrc[e]));
}

// rank = base + d * acc (base = (1-d)/n, plus d * dangling / n when the
// dangling mass is spread); next contributions (swap: prev = rank, as
// prgrid's iterator, prgrid_cilk.c:131-135); acc cleared for the next
// iteration; the new iterate's residual and dangling mass into st_out.
__global__ void __launch_bounds__(EG_EDGES_T) k_ep_finish(uint32_t n, float *acc, float *rank, float *contrib,
                                                          const uint32_t *__restrict__ deg, uint32_t mult,
                                                          float damping, int dangling, int swap, float p0,
                                                          const EdgePrDev *st_in, EdgePrDev *st_out) {
    double b = (1.0 - (double)damping) / (double)n;
    if (dangling) b += (double)damping * st_in->dangling / (double)n;
    const float base = (float)b;
    float res = 0.f, dang = 0.f;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const float r = fmaf(damping, acc[v], base);
        acc[v] = 0.f;
        res += fabsf(r - rank[v]);
        rank[v] = r;
        const uint32_t d = deg[v] * mult;
        if (swap) contrib[v] = d ? __fdiv_rn(r, (float)d) : 0.f;
        if (!d) dang += swap ? r : p0;  // without swap prev stays at its start value
    }
    block_add2((double)res, (double)dang, &st_out->residual, &st_out->dangling);
}

// y[src] += x[dst] over every edge (spmv.c:130-135, u32 wrapping adds): each
// thread takes 8 consecutive edges and adds once per run of equal sources,
// so a source-sorted array (modes 7, 8) costs one atomic per source per
// thread; sums of u32 are exact in any order.
__global__ void __launch_bounds__(EG_EDGES_T) k_es_spmv(const uint32_t *__restrict__ esrc,
                                                        const uint32_t *__restrict__ edst, uint64_t m,
                                                        const uint32_t *__restrict__ x, uint32_t *y) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t no = m >> 3;
    for (uint64_t o = t0; o < no; o += stride) {
        const uint4 s0 = __ldcs(reinterpret_cast<const uint4 *>(esrc) + 2 * o);
        const uint4 s1 = __ldcs(reinterpret_cast<const uint4 *>(esrc) + 2 * o + 1);
        const uint4 d0 = __ldcs(reinterpret_cast<const uint4 *>(edst) + 2 * o);
        const uint4 d1 = __ldcs(reinterpret_cast<const uint4 *>(edst) + 2 * o + 1);
        const uint32_t s[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
        const uint32_t d[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
        uint32_t run = s[0], sum = __ldg(x + d[0]);
#pragma unroll
        for (int k = 1; k < 8; k++) {
            const uint32_t xv = __ldg(x + d[k]);
            if (s[k] == run) {
                sum += xv;
            } else {
                atomicAdd(y + run, sum);
                run = s[k];
                sum = xv;
            }
        }
        atomicAdd(y + run, sum);
    }
    for (uint64_t e = 8 * no + t0; e < m; e += stride) atomicAdd(y + esrc[e], __ldg(x + edst[e]));
}

uint32_t edge_grid(eg_ctx *ctx, uint64_t work) {
    uint64_t b = (work + EG_EDGES_T - 1) / EG_EDGES_T;
    const uint64_t cap = (uint64_t)ctx->sm_count * 8;  // 8 resident CTAs of 256 threads per SM
    if (b > cap) b = cap;
    return (uint32_t)(b ? b : 1);
}

int bits_for_n(uint32_t n) {
    int b = 0;
    for (uint32_t x = n > 1 ? n - 1 : 1; x; x >>= 1) b++;
    return b;
}

int need_edges(eg_graph *g) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (!(g->built & EG_LAYOUT_EDGES)) return eg_fail(EG_ENOTBUILT, "edge array not built (eg_graph_build_edges)");
    return EG_OK;
}

}  // namespace

extern "C" int eg_graph_build_edges(eg_graph *g, int order) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (order != EG_EDGES_FILE_ORDER && order != EG_EDGES_BY_SRC && order != EG_EDGES_BY_SRC_DST)
        return eg_fail(EG_EINVAL, "edge order %d", order);
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint64_t M = g->m;
    const uint32_t n = g->n;
    if (M >= 0xffffffffull) return eg_fail(EG_EINVAL, "m=%llu: 32-bit offsets hold < 2^32", (unsigned long long)M);
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    // four arrays: the sort ping-pongs between the pairs (a, b) and keeps the
    // two that hold its result as the edge array
    eg_buf ka, va, kb, vb;
    int rc = EG_OK;
    auto fail = [&](int code) {
        cudaStreamSynchronize(ctx->stream);
        eg_buf_free(ctx, ka);
        eg_buf_free(ctx, va);
        eg_buf_free(ctx, kb);
        eg_buf_free(ctx, vb);
        return code;
    };
#define ETRY(x)                             \
    do {                                    \
        rc = (x);                           \
        if (rc != EG_OK) return fail(rc);   \
    } while (0)
    ETRY(eg_buf_ensure(ctx, ka, M * 4 + 16));
    ETRY(eg_buf_ensure(ctx, va, M * 4 + 16));
    if (order != EG_EDGES_FILE_ORDER) {
        ETRY(eg_buf_ensure(ctx, kb, M * 4 + 16));
        ETRY(eg_buf_ensure(ctx, vb, M * 4 + 16));
    }
    uint32_t *hbad = (uint32_t *)ctx->h_pinned;
    uint32_t *dbad = bp<uint32_t>(ka) + M;  // a spare word past the data
    ETRY(eg_zero(ctx, dbad, 4, ctx->stream));
    if (M) {
        k_edges_unpack<<<edge_grid(ctx, M), EG_EDGES_T, 0, ctx->stream>>>(
            bp<uint32_t>(g->pairs), g->m_in, (g->flags & EG_UNDIRECTED) != 0, n, bp<uint32_t>(ka), bp<uint32_t>(va),
            dbad);
        ctx->launches++;
    }
    ETRY(eg_readback(ctx, hbad, dbad, 4, ctx->stream));
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return fail(eg_fail(EG_ECUDA, "edge unpack: %s", cudaGetErrorString(cudaGetLastError())));
    if (*hbad) return fail(eg_fail(EG_ERANGE, "an edge endpoint is >= n=%u", n));
    uint32_t *src = bp<uint32_t>(ka), *dst = bp<uint32_t>(va);
    const int bits = bits_for_n(n);
    if (order == EG_EDGES_BY_SRC_DST) {
        // LSD: by destination first, then a stable sort by source
        uint32_t *k1, *v1;
        ETRY(eg_radix_sort(ctx, dst, src, bp<uint32_t>(kb), bp<uint32_t>(vb), M, bits, &k1, &v1));
        uint32_t *kt = k1 == bp<uint32_t>(ka) || k1 == bp<uint32_t>(va) ? bp<uint32_t>(kb) : bp<uint32_t>(ka);
        uint32_t *vt = kt == bp<uint32_t>(kb) ? bp<uint32_t>(vb) : bp<uint32_t>(va);
        // (k1, v1) = (dst, src) sorted by dst; the free pair is (kt, vt)
        ETRY(eg_radix_sort(ctx, v1, k1, kt, vt, M, bits, &src, &dst));
    } else if (order == EG_EDGES_BY_SRC) {
        ETRY(eg_radix_sort(ctx, src, dst, bp<uint32_t>(kb), bp<uint32_t>(vb), M, bits, &src, &dst));
    }
    // keep the two buffers holding the result, free the others
    eg_buf *all[4] = {&ka, &va, &kb, &vb};
    eg_buf keep_s, keep_d;
    for (eg_buf *b : all) {
        if (b->p && b->p == src) {
            keep_s = *b;
            *b = eg_buf();
        } else if (b->p && b->p == dst) {
            keep_d = *b;
            *b = eg_buf();
        }
    }
    if (!keep_s.p || !keep_d.p) return fail(eg_fail(EG_ECUDA, "edge build: result buffers not found"));
    eg_buf_free(ctx, g->esrc);
    eg_buf_free(ctx, g->edst);
    g->esrc = keep_s;
    g->edst = keep_d;
    g->edge_order = order;
    // degrees (count_degree, init_all.c:425-443)
    ETRY(eg_buf_ensure(ctx, g->out_deg, (uint64_t)n * 4));
    ETRY(eg_buf_ensure(ctx, g->in_deg, (uint64_t)n * 4));
    ETRY(eg_zero(ctx, g->out_deg.p, (uint64_t)n * 4, ctx->stream));
    ETRY(eg_zero(ctx, g->in_deg.p, (uint64_t)n * 4, ctx->stream));
    ETRY(eg_histogram(ctx, bp<uint32_t>(g->esrc), M, bp<uint32_t>(g->out_deg)));
    ETRY(eg_histogram(ctx, bp<uint32_t>(g->edst), M, bp<uint32_t>(g->in_deg)));
    g->built |= EG_LAYOUT_EDGES;
    if (cudaEventRecord(ctx->ev1, ctx->stream) != cudaSuccess || cudaEventSynchronize(ctx->ev1) != cudaSuccess)
        return fail(eg_fail(EG_ECUDA, "edge build: %s", cudaGetErrorString(cudaGetLastError())));
    cudaEventElapsedTime(&g->build_ms, ctx->ev0, ctx->ev1);
#undef ETRY
    return fail(EG_OK);
}

extern "C" int eg_graph_copy_edges(eg_graph *g, uint32_t *src, uint32_t *dst) {
    EG_TRY(need_edges(g));
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    if (src) EG_CUDA(cudaMemcpyAsync(src, g->esrc.p, g->m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (dst) EG_CUDA(cudaMemcpyAsync(dst, g->edst.p, g->m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    return EG_OK;
}

extern "C" int eg_edges_bfs(eg_graph *g, uint32_t root, int32_t *level_out, int32_t *parent_out,
                            eg_bfs_stats *stats) {
    EG_TRY(need_edges(g));
    if (root >= g->n) return eg_fail(EG_EINVAL, "root %u >= n %u", root, g->n);
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    const uint32_t nw = (n + 31) / 32;
    EG_TRY(eg_buf_ensure(ctx, g->level, (uint64_t)n * 4));
    if (parent_out) EG_TRY(eg_buf_ensure(ctx, g->parent, (uint64_t)n * 4));
    // work: visited | front | next bitmaps | counters (16-byte aligned)
    const uint64_t nw4 = (nw + 3ull) & ~3ull;
    EG_TRY(eg_buf_ensure(ctx, g->edge_work, (3 * nw4 + 8) * 4));
    uint32_t *visited = bp<uint32_t>(g->edge_work);
    uint32_t *bm[2] = {visited + nw4, visited + 2 * nw4};
    EdgeCounters *cnt = reinterpret_cast<EdgeCounters *>(visited + 3 * nw4);
    unsigned long long *reach = reinterpret_cast<unsigned long long *>(visited + 3 * nw4 + 4);
    int32_t *level = bp<int32_t>(g->level);
    int32_t *parent = parent_out ? bp<int32_t>(g->parent) : nullptr;
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    EG_TRY(eg_zero(ctx, cnt, 32, ctx->stream));
    k_eb_init<<<edge_grid(ctx, n), EG_EDGES_T, 0, ctx->stream>>>(n, nw, root, level, parent, visited, bm[0], bm[1]);
    EG_LAUNCHED(ctx);
    EdgeCounters *h = (EdgeCounters *)ctx->h_pinned;
    int cur = 0;
    int32_t lvl = 1;
    const uint32_t grid = edge_grid(ctx, (g->m + 3) / 4);
    for (;; lvl++) {
        if ((uint64_t)lvl > (uint64_t)n + 1) return eg_fail(EG_ETIMEOUT, "edge BFS did not terminate");
        k_eb_level<<<grid, EG_EDGES_T, 0, ctx->stream>>>(bp<uint32_t>(g->esrc), bp<uint32_t>(g->edst), g->m, bm[cur],
                                                          bm[cur ^ 1], visited, level, parent, lvl + 1, cnt);
        EG_LAUNCHED(ctx);
        EG_TRY(eg_readback_wait(ctx, h, cnt, sizeof(EdgeCounters), ctx->stream, true));  // and clears them
        if (h->claimed == 0) break;
        // the old frontier becomes the level after next's bitmap
        EG_TRY(eg_zero(ctx, bm[cur], (uint64_t)nw * 4, ctx->stream));
        cur ^= 1;
    }
    k_eb_reach<<<edge_grid(ctx, n), EG_EDGES_T, 0, ctx->stream>>>(level, bp<uint32_t>(g->out_deg), n, reach);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (level_out) EG_CUDA(cudaMemcpyAsync(level_out, level, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (parent_out) EG_CUDA(cudaMemcpyAsync(parent_out, parent, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    unsigned long long *hr = (unsigned long long *)((char *)ctx->h_pinned + 64);
    EG_TRY(eg_readback(ctx, hr, reach, 16, ctx->stream, true));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->levels = lvl;
        stats->reached = (uint32_t)hr[1];
        stats->edges_traversed = hr[0];
        stats->pull_levels = 0;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}

extern "C" int eg_edges_pagerank(eg_graph *g, const eg_pr_opts *opts, float *rank_out, eg_pr_stats *stats) {
    EG_TRY(need_edges(g));
    eg_pr_opts o;
    eg_pr_opts_default(&o);
    if (opts) o = *opts;
    if (o.iterations < 0) return eg_fail(EG_EINVAL, "iterations %d", o.iterations);
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    if (n == 0) return EG_OK;
    const uint32_t mult = o.deg_multiplier ? o.deg_multiplier : 1u;
    const float p0 = o.prev_init < 0.f ? 1.0f / (float)n : o.prev_init;
    EG_TRY(eg_buf_ensure(ctx, g->rank, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->contrib0, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->pr_acc, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->pr_stats, 4 * sizeof(EdgePrDev)));
    EdgePrDev *st = bp<EdgePrDev>(g->pr_stats);
    float *rank = bp<float>(g->rank), *contrib = bp<float>(g->contrib0), *acc = bp<float>(g->pr_acc);
    const uint32_t vgrid = edge_grid(ctx, n), egrid = edge_grid(ctx, (g->m + 3) / 4);
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    EG_TRY(eg_zero(ctx, st, 2 * sizeof(EdgePrDev), ctx->stream));
    k_ep_init<<<vgrid, EG_EDGES_T, 0, ctx->stream>>>(n, p0, bp<uint32_t>(g->out_deg), mult, rank, contrib, acc, st);
    EG_LAUNCHED(ctx);
    EdgePrDev *h = (EdgePrDev *)ctx->h_pinned;
    int it = 0;
    double residual = 0.0;
    for (; it < o.iterations; it++) {
        EdgePrDev *sin = st + (it & 1), *sout = st + ((it + 1) & 1);
        EG_TRY(eg_zero(ctx, sout, sizeof(EdgePrDev), ctx->stream));
        k_ep_scatter<<<egrid, EG_EDGES_T, 0, ctx->stream>>>(bp<uint32_t>(g->esrc), bp<uint32_t>(g->edst), g->m, contrib,
                                                             acc);
        EG_LAUNCHED(ctx);
        k_ep_finish<<<vgrid, EG_EDGES_T, 0, ctx->stream>>>(n, acc, rank, contrib, bp<uint32_t>(g->out_deg), mult,
                                                            o.damping, o.dangling, o.swap, p0, sin, sout);
        EG_LAUNCHED(ctx);
        if (o.tolerance > 0.0) {
            EG_TRY(eg_readback_wait(ctx, h, sout, sizeof(EdgePrDev), ctx->stream));
            residual = h->residual;
            if (residual < o.tolerance) {
                it++;
                break;
            }
        }
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (rank_out) EG_CUDA(cudaMemcpyAsync(rank_out, rank, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_TRY(eg_readback(ctx, h, st + (it & 1), sizeof(EdgePrDev), ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->iterations_run = it;
        stats->residual = it ? h->residual : 0.0;
        stats->dangling_mass = h->dangling;
        stats->row_kernel_ms = 0.f;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}

extern "C" int eg_edges_spmv_u32(eg_graph *g, const uint32_t *x, uint32_t *y, float *ms) {
    EG_TRY(need_edges(g));
    if (!x) return eg_fail(EG_EINVAL, "x is NULL");
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    EG_TRY(eg_buf_ensure(ctx, g->spmv_x, (uint64_t)n * 4));
    EG_TRY(eg_buf_ensure(ctx, g->spmv_y, (uint64_t)n * 4));
    if (n) EG_CUDA(cudaMemcpyAsync(g->spmv_x.p, x, (uint64_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    EG_TRY(eg_zero(ctx, g->spmv_y.p, (uint64_t)n * 4, ctx->stream));
    if (g->m) {
        k_es_spmv<<<edge_grid(ctx, (g->m + 7) / 8), EG_EDGES_T, 0, ctx->stream>>>(
            bp<uint32_t>(g->esrc), bp<uint32_t>(g->edst), g->m, bp<uint32_t>(g->spmv_x), bp<uint32_t>(g->spmv_y));
        EG_LAUNCHED(ctx);
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (y && n) EG_CUDA(cudaMemcpyAsync(y, g->spmv_y.p, (uint64_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ms) EG_CUDA(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return EG_OK;
}
