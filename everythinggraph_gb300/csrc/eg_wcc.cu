// Weakly connected components with min-id labels.
//
// Replaces wcc.c: min-label propagation over adjacency lists (wcc_algo,
// 30-42, with its pthread worklist 44-90) and over the grid and edge array
// (193-261), whose fixed point labels every vertex with the minimum vertex id
// of its component.
//
// GPU form: label propagation on component roots with pointer jumping.  Every
// edge hooks the larger of its two roots under the smaller one (atomicCAS on
// the root's parent word), so a root is always the minimum id of its tree;
// finds use path halving (pointer jumping), and a final pass jumps every
// vertex to its root.  The result equals the reference's fixed point bit for
// bit, independent of scheduling.
//
// With the adjacency built, edges are hooked in two rounds (the sampling idea
// of Sutton et al., "Optimizing parallel graph connectivity computation via
// subgraph sampling", IPDPS 2018): first the first two entries of every list,
// then, after a compression, the remaining entries of only those vertices
// whose root is not the largest component's root (sampled), which on
// power-law graphs skips most of the edges.
#include <stdlib.h>

#include "eg_internal.cuh"

#define EG_WCC_NONE 0xffffffffu

namespace {

__device__ __forceinline__ uint32_t uf_find(uint32_t *par, uint32_t x) {
    uint32_t p = __ldcg(par + x);
    while (p != x) {
        const uint32_t gp = __ldcg(par + p);
        if (gp != p) par[x] = gp;  // halve the path; parents only ever decrease
        x = p;
        p = gp;
    }
    return x;
}

__device__ __forceinline__ void uf_link(uint32_t *par, uint32_t x, uint32_t y) {
    uint32_t a = uf_find(par, x), b = uf_find(par, y);
    while (a != b) {
        if (a > b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        const uint32_t old = atomicCAS(par + b, b, a);
        if (old == b) break;
        b = uf_find(par, old);
        a = uf_find(par, a);
    }
}

// Hooks entries [lo, hi) of every list (first round: lo=0, hi=2) or, with
// skip_root set, entries [lo, end) of vertices whose root is not skip_root;
// the vertices are list[0 .. count) (those with an edge).
__global__ void k_wcc_lists(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                            const uint32_t *__restrict__ list, uint32_t count, uint32_t lo, uint32_t hi,
                            uint32_t skip_root, uint32_t *par) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t u = __ldg(list + i);
        if (skip_root != EG_WCC_NONE && uf_find(par, u) == skip_root) continue;
        const uint32_t b = ptr[u], e = ptr[u + 1];
        const uint32_t pe = (hi == EG_WCC_NONE || b + hi > e) ? e : b + hi;
        for (uint32_t p = b + lo; p < pe; p++) uf_link(par, u, col[p]);
    }
}

// Roots of 1024 vertices picked by a fixed hash (the largest component is the
// most frequent root among them).
__global__ void k_wcc_sample(const uint32_t *__restrict__ par, uint32_t n, uint32_t *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 1024) out[i] = par[(uint32_t)(((eg_mix64((uint64_t)i + 0x51ed) >> 32) * (uint64_t)n) >> 32)];
}

// The vertices with a non-empty out-list (or in-list), in id order: a
// flag per vertex, then each warp's ballot placed at its exclusive prefix.
__global__ void k_wcc_has_edge(const uint32_t *__restrict__ optr, const uint32_t *__restrict__ iptr, uint32_t n,
                               uint32_t *flag) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        flag[v] = (optr[v + 1] > optr[v]) || (iptr && iptr[v + 1] > iptr[v]);
}
__global__ void k_wcc_place(const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos, uint32_t n,
                            uint32_t *list) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (flag[v]) list[pos[v]] = v;
}

__global__ void k_wcc_flatten(uint32_t n, uint32_t *par) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) par[v] = uf_find(par, v);
}

__global__ void k_wcc_init(uint32_t n, uint32_t *par) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) par[v] = v;
}

__global__ void k_wcc_hook(const uint32_t *__restrict__ pairs, uint64_t m, uint32_t *par, uint32_t *retries) {
    uint32_t tries = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 p = reinterpret_cast<const uint2 *>(pairs)[e];
        uint32_t a = uf_find(par, p.x), b = uf_find(par, p.y);
        while (a != b) {
            if (a > b) {
                uint32_t t = a;
                a = b;
                b = t;
            }
            // link root b (larger) under root a (smaller)
            const uint32_t old = atomicCAS(par + b, b, a);
            if (old == b) break;
            tries++;
            b = uf_find(par, old);
            a = uf_find(par, a);
        }
    }
    if (tries) atomicAdd(retries, tries);
}

__global__ void k_wcc_compress(uint32_t n, uint32_t *par, uint32_t *label, unsigned long long *roots) {
    unsigned long long c = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t r = uf_find(par, v);
        label[v] = r;
        c += r == v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(EG_FULL_MASK, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(roots, c);
}

__global__ void k_widen(const uint32_t *__restrict__ in, uint32_t n, long long *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) out[v] = in[v];
}

}  // namespace

extern "C" int eg_wcc(eg_graph *g, int64_t *labels_out, eg_wcc_stats *stats) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    const uint32_t n = g->n;
    EG_TRY(eg_buf_ensure(ctx, g->label, (uint64_t)n * 4));
    // work: parent[n] | counters | int64 staging for the host copy
    const uint64_t off_cnt = ((uint64_t)n + 3) & ~3ull;
    const uint64_t off_sample = off_cnt + 8;
    const uint64_t off_wide = off_sample + 1024;
    EG_TRY(eg_buf_ensure(ctx, g->bfs_work, (off_wide + (labels_out ? 2ull * n : 0)) * 4));
    uint32_t *par = bp<uint32_t>(g->bfs_work);
    uint32_t *retries = par + off_cnt;
    unsigned long long *roots = reinterpret_cast<unsigned long long *>(par + off_cnt + 2);
    long long *wide = reinterpret_cast<long long *>(par + off_wide);
    uint32_t blocks = (uint32_t)(ctx->sm_count * 8);
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    EG_CUDA(cudaMemsetAsync(retries, 0, 32, ctx->stream));
    k_wcc_init<<<blocks, 256, 0, ctx->stream>>>(n, par);
    EG_LAUNCHED(ctx);
    const bool have_csr = (g->built & EG_LAYOUT_CSR) != 0;
    const bool sym = (g->flags & EG_UNDIRECTED) != 0;
    const bool have_csc = (g->built & EG_LAYOUT_CSC) != 0;
    int rounds = 1;
    if (have_csr && (sym || have_csc) && n >= 1024 && g->wcc_list_src != g->csr.ptr.p) {
        // once per layout: the vertices with an edge (flags, scan, placement)
        EG_TRY(eg_buf_ensure(ctx, g->wcc_list, ((uint64_t)n + 1) * 4 * 3));
        uint32_t *flag = bp<uint32_t>(g->wcc_list) + (uint64_t)n + 1, *pos = flag + (uint64_t)n + 1;
        k_wcc_has_edge<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), sym ? nullptr : bp<uint32_t>(g->csc.ptr),
                                                        n, flag);
        EG_LAUNCHED(ctx);
        EG_TRY(eg_exscan_u32(ctx, flag, pos, n));
        k_wcc_place<<<blocks, 256, 0, ctx->stream>>>(flag, pos, n, bp<uint32_t>(g->wcc_list));
        EG_LAUNCHED(ctx);
        uint32_t cnt = 0;
        EG_CUDA(cudaMemcpyAsync(&cnt, pos + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
        EG_CUDA(cudaStreamSynchronize(ctx->stream));
        g->wcc_list_n = cnt;
        g->wcc_list_src = g->csr.ptr.p;
    }
    const uint32_t *wl = bp<uint32_t>(g->wcc_list);
    const uint32_t wn = g->wcc_list_n;
    if (have_csr && (sym || have_csc) && n >= 1024) {
        // round 1: two entries per list (both directions for a directed graph)
        k_wcc_lists<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), wl, wn, 0, 2,
                                                     EG_WCC_NONE, par);
        EG_LAUNCHED(ctx);
        if (!sym) {
            k_wcc_lists<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.ptr), bp<uint32_t>(g->csc.col), wl, wn, 0,
                                                         2, EG_WCC_NONE, par);
            EG_LAUNCHED(ctx);
        }
        k_wcc_flatten<<<blocks, 256, 0, ctx->stream>>>(n, par);
        EG_LAUNCHED(ctx);
        // the most frequent root among 1024 sampled vertices
        uint32_t *dsample = par + off_sample;
        k_wcc_sample<<<4, 256, 0, ctx->stream>>>(par, n, dsample);
        EG_LAUNCHED(ctx);
        uint32_t *hs = (uint32_t *)ctx->h_pinned;
        EG_CUDA(cudaMemcpyAsync(hs, dsample, 1024 * 4, cudaMemcpyDeviceToHost, ctx->stream));
        EG_CUDA(cudaStreamSynchronize(ctx->stream));
        qsort(hs, 1024, 4, [](const void *a, const void *b) -> int {
            const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
            return x < y ? -1 : x > y;
        });
        uint32_t best = hs[0], best_cnt = 0;
        for (int i = 0; i < 1024;) {
            int j = i;
            while (j < 1024 && hs[j] == hs[i]) j++;
            if ((uint32_t)(j - i) > best_cnt) {
                best_cnt = (uint32_t)(j - i);
                best = hs[i];
            }
            i = j;
        }
        // round 2: remaining entries of vertices outside the sampled component
        k_wcc_lists<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), wl, wn, 2,
                                                     EG_WCC_NONE, best, par);
        EG_LAUNCHED(ctx);
        if (!sym) {
            k_wcc_lists<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.ptr), bp<uint32_t>(g->csc.col), wl, wn, 2,
                                                         EG_WCC_NONE, best, par);
            EG_LAUNCHED(ctx);
        }
        rounds = 2;
    } else if (g->m_in) {
        k_wcc_hook<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->pairs), g->m_in, par, retries);
        EG_LAUNCHED(ctx);
    }
    k_wcc_compress<<<blocks, 256, 0, ctx->stream>>>(n, par, bp<uint32_t>(g->label), roots);
    EG_LAUNCHED(ctx);
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    if (labels_out) {
        k_widen<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->label), n, wide);
        EG_LAUNCHED(ctx);
        EG_CUDA(cudaMemcpyAsync(labels_out, wide, (uint64_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    }
    unsigned long long *h = (unsigned long long *)ctx->h_pinned;
    EG_CUDA(cudaMemcpyAsync(h, roots, 8, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        stats->components = (uint32_t)*h;
        stats->rounds = rounds;
        EG_CUDA(cudaEventElapsedTime(&stats->ms, ctx->ev0, ctx->ev1));
    }
    return EG_OK;
}
