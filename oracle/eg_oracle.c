/*
 * CPU oracle for the EverythingGraph edge-traversal hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, what the
 * reference computes on each step of the path, so that the CUDA library can be
 * checked against it.  Only the test suite, the smoke check and the CPU
 * baseline leg of the benchmark load it; the product library never links it,
 * and no product code path falls back to it.
 *
 * Parity is pinned: tests/golden/ holds result dumps of the unmodified
 * reference binaries (built by oracle/build_ref.sh from the reference sources
 * with an OpenMP shim for Cilk) on seeded RMAT inputs, and the CPU tests check
 * every function below against them.
 *
 * Each function names the reference lines it restates.  File paths are
 * relative to the reference project root.
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off -shared).
 * -ffp-contract=off keeps the float arithmetic identical to the x86-64 build
 * of the reference, where no fused multiply-add is formed.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_UNREACHED_SSSP (UINT32_MAX - 1u) /* sssp_pushpull.c:8 (MAX) */

/* ------------------------------------------------------------------------ */
/* Synthetic input generators (not part of the reference; the reference reads
 * a binary [src][dst] file).  The same counter-based scheme is implemented in
 * the CUDA generator; tests check that both produce identical edges.
 *
 * mix64 is the SplitMix64 output function (Steele, Lea & Flood, OOPSLA 2014).
 */
static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t or_key(uint64_t seed, uint64_t idx) { return mix64(mix64(seed) ^ idx); }
static inline uint64_t or_draw(uint64_t key, uint64_t j) { return mix64(key + j * 0x632BE59BD9B4E019ull); }

/* RMAT quadrant thresholds: floor(p * 2^32) for p = a, a+b, a+b+c with
 * a=0.57, b=0.19, c=0.19 (d=0.05). */
#define RMAT_TA   2448131358u
#define RMAT_TAB  3264175144u
#define RMAT_TABC 4080218931u

void or_rmat_edges(int scale, uint64_t m, uint64_t seed, uint32_t *pairs) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)m; e++) {
        uint64_t key = or_key(seed, (uint64_t)e);
        uint32_t s = 0, d = 0;
        uint64_t w = 0;
        for (int l = 0; l < scale; l++) {
            if ((l & 1) == 0) w = or_draw(key, (uint64_t)(l >> 1));
            uint32_t r = (l & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
            uint32_t bit = 1u << (scale - 1 - l);
            if (r < RMAT_TA) {
            } else if (r < RMAT_TAB) {
                d |= bit;
            } else if (r < RMAT_TABC) {
                s |= bit;
            } else {
                s |= bit;
                d |= bit;
            }
        }
        pairs[2 * e] = s;
        pairs[2 * e + 1] = d;
    }
}

void or_er_edges(uint32_t n, uint64_t m, uint64_t seed, uint32_t *pairs) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)m; e++) {
        uint64_t w = or_draw(or_key(seed, (uint64_t)e), 0);
        pairs[2 * e] = (uint32_t)(((w & 0xffffffffull) * (uint64_t)n) >> 32);
        pairs[2 * e + 1] = (uint32_t)(((w >> 32) * (uint64_t)n) >> 32);
    }
}

/* fp32 uniform [0,1) with 24 random bits, one per index. */
void or_uniform_f32(uint64_t count, uint64_t seed, float *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++) {
        uint64_t w = or_draw(or_key(seed, (uint64_t)i), 0);
        out[i] = (float)(w >> 40) * (1.0f / 16777216.0f);
    }
}

/* u32 uniform in [lo, hi], one per index. */
void or_uniform_u32(uint64_t count, uint64_t seed, uint32_t lo, uint32_t hi, uint32_t *out) {
    uint64_t span = (uint64_t)hi - lo + 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++) {
        uint64_t w = or_draw(or_key(seed, (uint64_t)i), 0);
        out[i] = lo + (uint32_t)(((w >> 32) * span) >> 32);
    }
}

/* k roots drawn uniformly from vertices with deg[v] > 0 (rejection sampling). */
int or_sample_roots(uint32_t n, const uint32_t *deg, int k, uint64_t seed, uint32_t *roots) {
    for (int i = 0; i < k; i++) {
        uint64_t key = or_key(seed, (uint64_t)i);
        int found = 0;
        for (uint64_t a = 0; a < (1u << 20); a++) {
            uint32_t v = (uint32_t)(((or_draw(key, a) >> 32) * (uint64_t)n) >> 32);
            if (deg[v] > 0) { roots[i] = v; found = 1; break; }
        }
        if (!found) return -1;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Layout builders.
 *
 * or_build_adj restates init_adj_sort (init_all.c:629-790) with the loader in
 * front of it (preload_graph, init_all.c:81-110):
 *  - memblock holds the file's edges in file order; with `undirected` the
 *    reversed copies follow at positions m..2m-1 (init_all.c:102-106) and the
 *    edge count doubles (init_all.c:636);
 *  - the out-lists (CSR) are a stable sort of memblock by src (init_all.c:640),
 *    so a list keeps memblock order;
 *  - the in-lists (CSC) are a stable sort of that array by dst
 *    (init_all.c:722), so an in-list is in ascending src order, ties in
 *    memblock order; each in-entry stores the src (init_all.c:747).
 * eid arrays give the memblock position of every entry (for edge values).
 * Returns -1 when an endpoint is >= n (the reference would write out of bounds).
 */
int or_build_adj(uint32_t n, uint64_t m, const uint32_t *pairs, int undirected,
                 uint32_t *out_ptr, uint32_t *out_col, uint64_t *out_eid,
                 uint32_t *in_ptr, uint32_t *in_col, uint64_t *in_eid) {
    uint64_t M = undirected ? 2 * m : m;
    for (uint64_t e = 0; e < m; e++)
        if (pairs[2 * e] >= n || pairs[2 * e + 1] >= n) return -1;
    uint64_t *cnt = (uint64_t *)calloc((size_t)n + 1, sizeof(uint64_t));
    if (!cnt) return -2;
    for (uint64_t k = 0; k < M; k++) {
        uint64_t e = k < m ? k : k - m;
        uint32_t s = k < m ? pairs[2 * e] : pairs[2 * e + 1];
        cnt[s + 1]++;
    }
    for (uint32_t v = 0; v < n; v++) cnt[v + 1] += cnt[v];
    for (uint32_t v = 0; v <= n; v++) out_ptr[v] = (uint32_t)cnt[v];
    for (uint64_t k = 0; k < M; k++) {
        uint64_t e = k < m ? k : k - m;
        uint32_t s = k < m ? pairs[2 * e] : pairs[2 * e + 1];
        uint32_t d = k < m ? pairs[2 * e + 1] : pairs[2 * e];
        uint64_t pos = cnt[s]++;
        out_col[pos] = d;
        if (out_eid) out_eid[pos] = k;
    }
    if (in_ptr) {
        memset(cnt, 0, ((size_t)n + 1) * sizeof(uint64_t));
        for (uint64_t p = 0; p < M; p++) cnt[out_col[p] + 1]++;
        for (uint32_t v = 0; v < n; v++) cnt[v + 1] += cnt[v];
        for (uint32_t v = 0; v <= n; v++) in_ptr[v] = (uint32_t)cnt[v];
        for (uint32_t s = 0; s < n; s++) {
            for (uint32_t p = out_ptr[s]; p < out_ptr[s + 1]; p++) {
                uint64_t pos = cnt[out_col[p]]++;
                in_col[pos] = s;
                if (in_eid) in_eid[pos] = out_eid ? out_eid[p] : 0;
            }
        }
    }
    free(cnt);
    return 0;
}

/* Grid partitioning, restating get_partition_id (init_all.c:54-60) with the
 * partition sizes set in init (init_all.c:838-842): the first n mod P
 * partitions hold ceil(n/P) vertices, the rest floor(n/P). */
static inline uint32_t or_part(uint32_t v, uint32_t n, uint32_t P) {
    uint32_t mod = n % P;
    uint32_t psz = mod ? n / P + 1 : n / P;
    uint32_t split = mod * psz;
    if (mod == 0) return v / psz;
    return v < split ? v / psz : (v - split) / (psz - 1) + mod;
}
uint32_t or_partition_id(uint32_t v, uint32_t n, uint32_t P) { return or_part(v, n, P); }

/* P chosen by the driver from -n (random.c:69-71). */
uint32_t or_default_p(uint32_t n) {
    uint32_t P = (uint32_t)((n * 8u / 1024u) / 20u);
    if (P > 2000) P = 256;
    if (P == 0) P = 4;
    return P;
}

/* or_build_grid restates init_grid_sort (init_all.c:252-361, load mode 0):
 * stable sort by src, then a stable sort of each src-partition row by dst
 * partition.  Cells are laid out row-major (src partition i, dst partition j);
 * inside a cell edges are in ascending src, ties in file order.
 * cell_ptr has P*P+1 entries (absolute offsets; the reference keeps
 * row_offsets[i] + offsets[i][j], which is the same number). */
int or_build_grid(uint32_t n, uint64_t m, const uint32_t *pairs, uint32_t P,
                  uint32_t *cell_ptr, uint32_t *gsrc, uint32_t *gdst) {
    uint64_t cells = (uint64_t)P * P;
    for (uint64_t e = 0; e < m; e++)
        if (pairs[2 * e] >= n || pairs[2 * e + 1] >= n) return -1;
    /* stable counting sort by src */
    uint64_t *cnt = (uint64_t *)calloc((size_t)n + 1, sizeof(uint64_t));
    uint64_t *ord = (uint64_t *)malloc((size_t)m * sizeof(uint64_t));
    uint64_t *ccnt = (uint64_t *)calloc((size_t)cells + 1, sizeof(uint64_t));
    if (!cnt || !ord || !ccnt) { free(cnt); free(ord); free(ccnt); return -2; }
    for (uint64_t e = 0; e < m; e++) cnt[pairs[2 * e] + 1]++;
    for (uint32_t v = 0; v < n; v++) cnt[v + 1] += cnt[v];
    for (uint64_t e = 0; e < m; e++) ord[cnt[pairs[2 * e]]++] = e;
    /* stable counting sort of that order by cell id (row is fixed by src) */
    for (uint64_t e = 0; e < m; e++) {
        uint64_t c = (uint64_t)or_part(pairs[2 * e], n, P) * P + or_part(pairs[2 * e + 1], n, P);
        ccnt[c + 1]++;
    }
    for (uint64_t c = 0; c < cells; c++) ccnt[c + 1] += ccnt[c];
    for (uint64_t c = 0; c <= cells; c++) cell_ptr[c] = (uint32_t)ccnt[c];
    for (uint64_t i = 0; i < m; i++) {
        uint64_t e = ord[i];
        uint64_t c = (uint64_t)or_part(pairs[2 * e], n, P) * P + or_part(pairs[2 * e + 1], n, P);
        uint64_t pos = ccnt[c]++;
        gsrc[pos] = pairs[2 * e];
        gdst[pos] = pairs[2 * e + 1];
    }
    free(cnt); free(ord); free(ccnt);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* PageRank.
 *
 * or_pagerank_f32 restates the fp32 arithmetic of the pull loop
 * (pagerank_simple.c:72-84):
 *     rank[i] = 0; for u in in(i): rank[i] += (float)prev[u] / (float)deg[u];
 *     rank[i] = adding_constant + DAMPING_FACTOR * rank[i];
 * with adding_constant = (1 - 0.85) * 1 / (float)n stored as float
 * (pagerank_simple.c:88) and the last line evaluated in double
 * (DAMPING_FACTOR is the double literal 0.85, pagerank_simple.c:4).
 * In-lists are summed serially in CSC order.
 *  - swap=0 is pagerank_simple's PULL mode: prev is never updated
 *    (pagerank_simple.c:110-133), so every iteration recomputes one step;
 *  - swap=1 copies rank into prev after each iteration, as prgrid_cilk
 *    (prgrid_cilk.c:131-135) and pr_numa (pr_numa.c:396) do.
 * deg is the per-vertex divisor (degree[] in pagerank_simple.c:97, or
 * nodes[].nb_out_edges doubled by the second degree count in grid modes,
 * init_all.c:851-852).  prev starts at prev_init (0.15 in the reference,
 * pagerank_simple.c:95).  Dangling mass is dropped, as in the reference.
 */
void or_pagerank_f32(uint32_t n, const uint32_t *in_ptr, const uint32_t *in_col,
                     const uint32_t *deg, float prev_init, int iters, int swap, float *out) {
    float ac = (float)((1 - 0.85) * 1 / (double)(float)n);
    float *prev = (float *)malloc((size_t)n * sizeof(float));
    for (uint32_t i = 0; i < n; i++) prev[i] = prev_init;
    for (int it = 0; it < iters; it++) {
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t i = 0; i < (int64_t)n; i++) {
            float r = 0.0f;
            for (uint32_t p = in_ptr[i]; p < in_ptr[i + 1]; p++) {
                uint32_t u = in_col[p];
                r += (float)prev[u] / (float)deg[u];
            }
            out[i] = (float)((double)ac + 0.85 * (double)r);
        }
        if (swap) memcpy(prev, out, (size_t)n * sizeof(float));
    }
    free(prev);
}

/* or_pagerank_grid_f32 restates prgrid_algo over the grid (prgrid_cilk.c:62-76)
 * and its iterator (prgrid_cilk.c:111-141): rows of cells in order, each cell
 * streamed in order, rank[dst] += prev[src] / (float)deg[src]; then
 * rank = ac + 0.85*rank, prev = rank, rank = 0.  Output is prev. */
void or_pagerank_grid_f32(uint32_t n, uint32_t P, const uint32_t *cell_ptr, const uint32_t *gsrc,
                          const uint32_t *gdst, const uint32_t *deg, float prev_init, int iters,
                          float *out) {
    float ac = (float)((1 - 0.85) * 1 / (double)(float)n);
    float *rank = (float *)calloc(n, sizeof(float));
    for (uint32_t i = 0; i < n; i++) out[i] = prev_init;
    for (int it = 0; it < iters; it++) {
        for (uint32_t i = 0; i < P; i++) {
#pragma omp parallel for schedule(dynamic, 1)
            for (int64_t j = 0; j < (int64_t)P; j++) {
                uint64_t c = (uint64_t)i * P + (uint64_t)j;
                for (uint32_t p = cell_ptr[c]; p < cell_ptr[c + 1]; p++)
                    rank[gdst[p]] += (out[gsrc[p]] / (float)deg[gsrc[p]]);
            }
        }
        for (uint32_t v = 0; v < n; v++) {
            rank[v] = (float)((double)ac + 0.85 * (double)rank[v]);
            out[v] = rank[v];
            rank[v] = 0.0f;
        }
    }
    free(rank);
}

/* FP64 PageRank (the error reference): x_{k+1}[v] = (1-d)/n + d*dang_k/n*[dangling]
 * + d * sum_{u->v} x_k[u]/deg[u].  dangling=0 drops the mass of vertices with
 * deg 0 (reference behaviour); dangling=1 spreads it uniformly. */
void or_pagerank_f64(uint32_t n, const uint32_t *in_ptr, const uint32_t *in_col,
                     const uint32_t *deg, double prev_init, int iters, int dangling, double damping,
                     double *out) {
    double *prev = (double *)malloc((size_t)n * sizeof(double));
    for (uint32_t i = 0; i < n; i++) prev[i] = prev_init;
    for (int it = 0; it < iters; it++) {
        double dang = 0.0;
        if (dangling)
            for (uint32_t i = 0; i < n; i++)
                if (deg[i] == 0) dang += prev[i];
        double base = (1.0 - damping) / (double)n + damping * dang / (double)n;
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t i = 0; i < (int64_t)n; i++) {
            double s = 0.0;
            for (uint32_t p = in_ptr[i]; p < in_ptr[i + 1]; p++) s += prev[in_col[p]] / (double)deg[in_col[p]];
            out[i] = base + damping * s;
        }
        memcpy(prev, out, (size_t)n * sizeof(double));
    }
    free(prev);
}

/* Personalised PageRank in FP64: the teleport mass (1-d) goes to the seed set
 * (uniformly over nseeds seeds) and dangling mass returns to the seeds too.
 * Starts from the seed distribution; iterates until the L1 change is below tol
 * or max_iters.  Returns the iteration count. */
int or_ppr_f64(uint32_t n, const uint32_t *in_ptr, const uint32_t *in_col, const uint32_t *deg,
               const uint32_t *seeds, int nseeds, double damping, double tol, int max_iters,
               double *out) {
    double *prev = (double *)calloc(n, sizeof(double));
    double *tele = (double *)calloc(n, sizeof(double));
    for (int s = 0; s < nseeds; s++) tele[seeds[s]] += 1.0 / nseeds;
    memcpy(prev, tele, (size_t)n * sizeof(double));
    int it;
    for (it = 0; it < max_iters; it++) {
        double dang = 0.0;
        for (uint32_t i = 0; i < n; i++)
            if (deg[i] == 0) dang += prev[i];
        double res = 0.0;
        for (uint32_t i = 0; i < n; i++) {
            double s = 0.0;
            for (uint32_t p = in_ptr[i]; p < in_ptr[i + 1]; p++) s += prev[in_col[p]] / (double)deg[in_col[p]];
            out[i] = ((1.0 - damping) + damping * dang) * tele[i] + damping * s;
            res += fabs(out[i] - prev[i]);
        }
        memcpy(prev, out, (size_t)n * sizeof(double));
        if (res < tol) { it++; break; }
    }
    free(prev); free(tele);
    return it;
}

/* ------------------------------------------------------------------------ */
/* SpMV.
 *
 * Integer SpMV restates spmv.c: x[i] = i as u32 (spmv.c:125-128), y u32.
 *  - mode 0 (pull, spmv.c:98-106): for each in-edge u->v,
 *        y[v] = (u32)((double)y[v] + 0.001 * x[u])
 *    summed in CSC order; the double-to-u32 conversion is taken modulo 2^32
 *    (the x86-64 code converts through a 64-bit integer);
 *  - mode 1 (push, spmv.c:110-118): for each out-edge v->u,
 *        y[v] += (u32)(0.001 * x[u])  (wrapping add)
 *  - mode 2 (edge array, spmv.c:130-135): y[src] += x[dst] (wrapping add).
 * For pull the caller passes the CSC, for push and edge array the CSR.
 */
static inline uint32_t or_d2u32(double v) { return (uint32_t)(uint64_t)(int64_t)v; }
void or_spmv_u32(uint32_t n, const uint32_t *ptr, const uint32_t *col, const uint32_t *x, int mode,
                 uint32_t *y) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; v++) {
        uint32_t acc = 0;
        for (uint32_t p = ptr[v]; p < ptr[v + 1]; p++) {
            uint32_t xv = x[col[p]];
            if (mode == 0) acc = or_d2u32((double)acc + 0.001 * (double)xv);
            else if (mode == 1) acc += or_d2u32(0.001 * (double)xv);
            else acc += xv;
        }
        y[v] = acc;
    }
}

/* fp64 SpMV with edge values: y[v] = sum over in-entries p of row v of vals[p] * x[col[p]]. */
void or_spmv_f64(uint32_t n, const uint32_t *ptr, const uint32_t *col, const float *vals,
                 const float *x, double *y) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; v++) {
        double acc = 0.0;
        for (uint32_t p = ptr[v]; p < ptr[v + 1]; p++) acc += (double)vals[p] * (double)x[col[p]];
        y[v] = acc;
    }
}

/* ------------------------------------------------------------------------ */
/* BFS levels, restating the level-synchronous sweep of bfsgrid_cilk.c:48-65
 * and bfs_simple.c:58-103: dist[root] = 1, a vertex reached from a frontier
 * vertex at level L gets L+1, unreached vertices keep 0.  Edges are the CSR
 * out-lists.  Also fills a parent array (parent[root] = root, -1 unreached)
 * with the first frontier vertex that reached each vertex in CSR order. */
int or_bfs_levels(uint32_t n, const uint32_t *ptr, const uint32_t *col, uint32_t root,
                  int32_t *level, int32_t *parent) {
    if (root >= n) return -1;
    uint32_t *q = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; i++) { level[i] = 0; if (parent) parent[i] = -1; }
    uint64_t head = 0, tail = 0;
    level[root] = 1;
    if (parent) parent[root] = (int32_t)root;
    q[tail++] = root;
    while (head < tail) {
        uint32_t u = q[head++];
        for (uint32_t p = ptr[u]; p < ptr[u + 1]; p++) {
            uint32_t v = col[p];
            if (level[v] == 0) {
                level[v] = level[u] + 1;
                if (parent) parent[v] = (int32_t)u;
                q[tail++] = v;
            }
        }
    }
    free(q);
    return 0;
}

/* SSSP: the reference's pull-only run (sssp_pushpull.c:69-98 with -a 1 -r)
 * is frontier Bellman-Ford run to a fixed point, i.e. exact shortest-path
 * distances over the directed out-edges, unreached = UINT32_MAX-1, root 0.
 * Weights are per CSR entry (the reference's CREATE_WEIGHT rule
 * src%10 + dst%10, init_all.c:661-686, is built by the caller).
 * Restated here as Dijkstra with a binary heap (same fixed point). */
typedef struct { uint32_t d, v; } or_hitem;
static void or_heap_push(or_hitem *h, uint64_t *sz, or_hitem it) {
    uint64_t i = (*sz)++;
    while (i > 0) {
        uint64_t p = (i - 1) / 2;
        if (h[p].d <= it.d) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = it;
}
static or_hitem or_heap_pop(or_hitem *h, uint64_t *sz) {
    or_hitem top = h[0], last = h[--(*sz)];
    uint64_t i = 0;
    for (;;) {
        uint64_t c = 2 * i + 1;
        if (c >= *sz) break;
        if (c + 1 < *sz && h[c + 1].d < h[c].d) c++;
        if (h[c].d >= last.d) break;
        h[i] = h[c];
        i = c;
    }
    h[i] = last;
    return top;
}
int or_sssp(uint32_t n, const uint32_t *ptr, const uint32_t *col, const uint32_t *w, uint32_t root,
            uint32_t *dist) {
    if (root >= n) return -1;
    uint64_t m = ptr[n];
    or_hitem *h = (or_hitem *)malloc((size_t)(m + 1) * sizeof(or_hitem));
    uint64_t sz = 0;
    for (uint32_t i = 0; i < n; i++) dist[i] = OR_UNREACHED_SSSP;
    dist[root] = 0;
    or_heap_push(h, &sz, (or_hitem){0, root});
    while (sz) {
        or_hitem it = or_heap_pop(h, &sz);
        if (it.d != dist[it.v]) continue;
        for (uint32_t p = ptr[it.v]; p < ptr[it.v + 1]; p++) {
            uint32_t v = col[p];
            if (v == it.v) continue; /* self-loops skipped, sssp_pushpull.c:80 */
            uint64_t nd = (uint64_t)it.d + w[p];
            if (nd < dist[v]) {
                dist[v] = (uint32_t)nd;
                or_heap_push(h, &sz, (or_hitem){(uint32_t)nd, v});
            }
        }
    }
    free(h);
    return 0;
}

/* SSSP with fp32 weights and fp32 path sums (the reference's pull relax adds
 * in float, sssp_pushpull.c:81): Dijkstra where extending a path rounds
 * d[u] + w to fp32.  Rounded addition of w >= 0 is monotone and never
 * decreases d, so Dijkstra and Bellman-Ford reach the same least fixed point.
 * Distances are returned as fp32 bit patterns (unreached = +inf), which order
 * like the floats for non-negative values. */
int or_sssp_f32(uint32_t n, const uint32_t *ptr, const uint32_t *col, const float *w, uint32_t root,
                uint32_t *dist_bits) {
    if (root >= n) return -1;
    uint64_t m = ptr[n];
    or_hitem *h = (or_hitem *)malloc((size_t)(m + 1) * sizeof(or_hitem));
    uint64_t sz = 0;
    const uint32_t inf = 0x7f800000u;
    for (uint32_t i = 0; i < n; i++) dist_bits[i] = inf;
    dist_bits[root] = 0;
    or_heap_push(h, &sz, (or_hitem){0, root});
    while (sz) {
        or_hitem it = or_heap_pop(h, &sz);
        if (it.d != dist_bits[it.v]) continue;
        float du;
        memcpy(&du, &it.d, 4);
        for (uint32_t p = ptr[it.v]; p < ptr[it.v + 1]; p++) {
            uint32_t v = col[p];
            if (v == it.v) continue;
            float ndv = du + w[p];
            uint32_t nb;
            memcpy(&nb, &ndv, 4);
            if (nb < dist_bits[v]) {
                dist_bits[v] = nb;
                or_heap_push(h, &sz, (or_hitem){nb, v});
            }
        }
    }
    free(h);
    return 0;
}

/* WCC: min-label propagation (wcc.c:30-42 on -u adjacency lists, and the grid
 * and edge-array sweeps wcc.c:193-261 that relax both endpoints) converges to
 * the minimum vertex id of each weakly connected component.  Restated with
 * union-find where the larger root is always linked under the smaller. */
static uint32_t or_find(uint32_t *p, uint32_t x) {
    while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
    return x;
}
int or_wcc(uint32_t n, uint64_t m, const uint32_t *pairs, int64_t *labels) {
    uint32_t *p = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; i++) p[i] = i;
    for (uint64_t e = 0; e < m; e++) {
        uint32_t a = pairs[2 * e], b = pairs[2 * e + 1];
        if (a >= n || b >= n) { free(p); return -1; }
        a = or_find(p, a);
        b = or_find(p, b);
        if (a < b) p[b] = a;
        else if (b < a) p[a] = b;
    }
    for (uint32_t i = 0; i < n; i++) labels[i] = or_find(p, i);
    free(p);
    return 0;
}

/* Degree histogram of the file's edges (preload_graph's count,
 * init_all.c:91-94). */
void or_degrees(uint32_t n, uint64_t m, const uint32_t *pairs, uint32_t *out_deg, uint32_t *in_deg) {
    memset(out_deg, 0, (size_t)n * sizeof(uint32_t));
    if (in_deg) memset(in_deg, 0, (size_t)n * sizeof(uint32_t));
    for (uint64_t e = 0; e < m; e++) {
        out_deg[pairs[2 * e]]++;
        if (in_deg) in_deg[pairs[2 * e + 1]]++;
    }
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void or_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

/* Per-edge attributes hashed from the unordered endpoint pair (the weight and
 * value rules of the CUDA library, restated for the checker). */
static inline uint64_t or_edge_hash(uint64_t seed, uint32_t u, uint32_t v) {
    uint32_t a = u < v ? u : v, b = u < v ? v : u;
    return or_draw(or_key(seed, ((uint64_t)a << 32) | b), 0);
}
void or_hash_weights(uint64_t count, const uint32_t *u, const uint32_t *v, uint64_t seed, uint32_t lo,
                     uint32_t hi, uint32_t *out) {
    uint64_t span = (uint64_t)hi - lo + 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++)
        out[i] = lo + (uint32_t)(((or_edge_hash(seed, u[i], v[i]) >> 32) * span) >> 32);
}
/* fp32 weights in (0, 1]: (top 24 hash bits + 1) / 2^24, exact in fp32. */
void or_hash_weights_f32(uint64_t count, const uint32_t *u, const uint32_t *v, uint64_t seed, float *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++)
        out[i] = (float)((or_edge_hash(seed, u[i], v[i]) >> 40) + 1) * (1.0f / 16777216.0f);
}
void or_hash_values(uint64_t count, const uint32_t *u, const uint32_t *v, uint64_t seed, float *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++)
        out[i] = (float)(or_edge_hash(seed, u[i], v[i]) >> 40) * (1.0f / 16777216.0f);
}

/* fp64 SpMV whose edge values follow the rule of or_hash_values, computed per
 * entry instead of stored: y[v] = sum over in-entries p of row v of
 * val(col[p], v) * x[col[p]] (the FP64 error reference for graphs whose value
 * array would not fit beside the CSC in host memory). */
void or_spmv_f64_hval(uint32_t n, const uint32_t *ptr, const uint32_t *col, uint64_t seed, const float *x,
                      double *y) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; v++) {
        double acc = 0.0;
        for (uint32_t p = ptr[v]; p < ptr[v + 1]; p++) {
            const float val = (float)(or_edge_hash(seed, col[p], (uint32_t)v) >> 40) * (1.0f / 16777216.0f);
            acc += (double)val * (double)x[col[p]];
        }
        y[v] = acc;
    }
}

/* BFS tree check for a parent array (the parents that bfs_numa's top-down
 * step records with a CAS, bfs_numa.c:234-278), against levels in the root = 1
 * convention, in O(n + m):
 *   parent[root] = root and level[root] = 1;
 *   an unreached vertex (level 0) has parent -1;
 *   every other reached v has a parent p with level[p] = level[v] - 1 and an
 *   out-entry p -> v in the CSR.
 * The edge test marks, for every CSR entry u -> w with parent[w] = u, that w's
 * tree edge exists.  Returns 0 when the tree is valid, else a negative code
 * naming the first rule that failed (-1 root, -2 unreached, -3 level, -4 edge). */
int or_bfs_tree_check(uint32_t n, const uint32_t *ptr, const uint32_t *col, uint32_t root, const int32_t *level,
                      const int32_t *parent) {
    if (root >= n || parent[root] != (int32_t)root || level[root] != 1) return -1;
    int bad2 = 0, bad3 = 0, bad4 = 0;
#pragma omp parallel for schedule(static) reduction(| : bad2, bad3)
    for (int64_t v = 0; v < (int64_t)n; v++) {
        if (level[v] == 0) {
            if (parent[v] != -1) bad2 = 1;
        } else if (v != (int64_t)root) {
            const int32_t p = parent[v];
            if (p < 0 || (uint32_t)p >= n || level[p] != level[v] - 1) bad3 = 1;
        }
    }
    if (bad2) return -2;
    if (bad3) return -3;
    uint8_t *found = (uint8_t *)calloc(n, 1);
    if (!found) return -5;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < (int64_t)n; u++)
        for (uint32_t p = ptr[u]; p < ptr[u + 1]; p++)
            if (parent[col[p]] == (int32_t)u) found[col[p]] = 1;
#pragma omp parallel for schedule(static) reduction(| : bad4)
    for (int64_t v = 0; v < (int64_t)n; v++)
        if (level[v] > 0 && v != (int64_t)root && !found[v]) bad4 = 1;
    free(found);
    return bad4 ? -4 : 0;
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded restatements of the reference's CPU loops, used as the
 * timed CPU baseline (the reference binaries themselves need the reference
 * sources, which are not shipped).
 *
 * or_bfs_do restates bfs_simple.c's iterator (136-229): push steps over the
 * frontier's out-lists with a CAS on the next-frontier flag (bfs_push,
 * 121-134), pull steps over unvisited vertices that stop at the first
 * in-neighbour in the frontier (bfs_pull, 104-120), and the switch rule
 * "pull iff items + degree_in_frontier > m/20" (191-197), where
 * degree_in_frontier is the work queue's nb_cleaning, 2 * deg + 1 per
 * frontier vertex (thread_add_task, buffer.c:272-282): pull iff
 * 2 * (items + frontier out-degree) > m/20.  Frontiers are byte maps as in
 * random.c:74-77.  Writes levels (root = 1). */
int or_bfs_do(uint32_t n, const uint32_t *out_ptr, const uint32_t *out_col, const uint32_t *in_ptr,
              const uint32_t *in_col, uint32_t root, int32_t *level) {
    if (root >= n) return -1;
    uint64_t m = out_ptr[n];
    unsigned char *cur = (unsigned char *)calloc(n, 1), *nxt = (unsigned char *)calloc(n, 1);
    uint32_t *q = (uint32_t *)malloc((size_t)n * 4), *q2 = (uint32_t *)malloc((size_t)n * 4);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) level[i] = 0;
    level[root] = 1;
    cur[root] = 1;
    q[0] = root;
    uint64_t qn = 1, items = 1, fdeg = out_ptr[root + 1] - out_ptr[root];
    int pull = 0, have_q = 1;
    int32_t lvl = 1;
    while (items) {
        pull = 2.0 * ((double)items + (double)fdeg) > (double)m / 20.0;
        uint64_t cnt = 0, deg = 0, qn2 = 0;
        if (!pull) {
            if (!have_q) {
                qn = 0;
                for (uint32_t v = 0; v < n; v++)
                    if (cur[v]) q[qn++] = v;
            }
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : cnt, deg)
            for (int64_t i = 0; i < (int64_t)qn; i++) {
                uint32_t u = q[i];
                for (uint32_t p = out_ptr[u]; p < out_ptr[u + 1]; p++) {
                    uint32_t v = out_col[p];
                    if (level[v] == 0 && __sync_bool_compare_and_swap(&level[v], 0, lvl + 1)) {
                        nxt[v] = 1;
                        uint64_t pos = __sync_fetch_and_add(&qn2, 1);
                        q2[pos] = v;
                        cnt++;
                        deg += out_ptr[v + 1] - out_ptr[v];
                    }
                }
            }
            uint32_t *t = q; q = q2; q2 = t;
            qn = qn2;
            have_q = 1;
        } else {
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : cnt, deg)
            for (int64_t v = 0; v < (int64_t)n; v++) {
                if (level[v] != 0) continue;
                for (uint32_t p = in_ptr[v]; p < in_ptr[v + 1]; p++) {
                    if (cur[in_col[p]]) {
                        level[v] = lvl + 1;
                        nxt[v] = 1;
                        cnt++;
                        deg += out_ptr[v + 1] - out_ptr[v];
                        break;
                    }
                }
            }
            have_q = 0;
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) cur[i] = 0;
        unsigned char *t = cur; cur = nxt; nxt = t;
        items = cnt;
        fdeg = deg;
        lvl++;
    }
    free(cur); free(nxt); free(q); free(q2);
    return 0;
}

/* or_wcc_lp restates wcc.c's adjacency-list mode (wcc.c:30-90, 262-277):
 * every vertex starts active with its own id (wcc_reset, 128-135); each round
 * relaxes the out-lists of the active vertices with writeMin and activates
 * the vertices whose label dropped, until no vertex is active.  On a
 * symmetric (-u) adjacency this is the min-id WCC labelling.  Returns rounds. */
int or_wcc_lp(uint32_t n, const uint32_t *out_ptr, const uint32_t *out_col, int64_t *comp) {
    unsigned char *act = (unsigned char *)malloc(n), *nact = (unsigned char *)calloc(n, 1);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) { comp[i] = i; act[i] = 1; }
    int rounds = 0;
    uint64_t active = n;
    while (active) {
        uint64_t nxt = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : nxt)
        for (int64_t u = 0; u < (int64_t)n; u++) {
            if (!act[u]) continue;
            int64_t cu = comp[u];
            for (uint32_t p = out_ptr[u]; p < out_ptr[u + 1]; p++) {
                uint32_t v = out_col[p];
                int64_t c;
                int changed = 0;
                while ((c = comp[v]) > cu) {
                    if (__sync_bool_compare_and_swap(&comp[v], c, cu)) { changed = 1; break; }
                }
                if (changed && __sync_bool_compare_and_swap(&nact[v], 0, 1)) nxt++;
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) { act[i] = nact[i]; nact[i] = 0; }
        active = nxt;
        rounds++;
    }
    free(act); free(nact);
    return rounds;
}
