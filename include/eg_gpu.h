/*
 * eg_gpu.h - C ABI of the GB300 (sm_103a) edge-traversal library.
 *
 * Plain C types only: pointers, sizes, small option structs.  Every call
 * returns an int status (EG_OK = 0, negative on error); eg_last_error()
 * gives the message of the calling thread's last failure.  One context owns
 * one CUDA stream on one device; calls on a context are not thread-safe.
 * Host output arrays are caller-owned; a NULL host output leaves the result
 * on the device (see eg_graph_device_ptr).
 *
 * Each entry point names the reference interface it replaces.  The reference
 * is one process in shared memory whose loader fills globals
 * (init_all.h:36-60) and whose algorithms are `struct algo_func` plug-ins
 * (random.h:64-69) called construct -> reset -> main -> destruct
 * (random.c:128-143).
 */
#ifndef EG_GPU_H
#define EG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define EG_OK 0
#define EG_EINVAL (-1)    /* bad argument */
#define EG_ECUDA (-2)     /* CUDA runtime error */
#define EG_ENOMEM (-3)    /* device allocation failed or over the HBM budget */
#define EG_EIO (-4)       /* input file unreadable or of odd size */
#define EG_ETIMEOUT (-5)  /* a device-side wait hit its iteration limit */
#define EG_ENOTBUILT (-6) /* the layout an algorithm needs was not built */
#define EG_ERANGE (-7)    /* an edge endpoint is >= n */

typedef struct eg_ctx eg_ctx;
typedef struct eg_graph eg_graph;

/* Message of the calling thread's last error ("" if none). */
const char *eg_last_error(void);

/* Library version string. */
const char *eg_version(void);

/* ---- context ------------------------------------------------------------ */
/* Opens device `device` with one stream.  hbm_budget_bytes caps the bytes
 * the context may allocate (0 = no cap).  Replaces the reference's thread
 * setup (setWorkers, random.c:123 and parallel_ligra.h:49-57). */
int eg_open(int device, uint64_t hbm_budget_bytes, eg_ctx **out);
int eg_close(eg_ctx *ctx); /* EG_EINVAL (context kept) while graphs are open:
                              free every graph (and server) first */
/* The context's cudaStream_t, as void*. */
void *eg_stream(eg_ctx *ctx);
int eg_sync(eg_ctx *ctx);
uint64_t eg_bytes_in_use(eg_ctx *ctx);
/* Number of kernels this context has launched so far. */
uint64_t eg_kernel_launches(eg_ctx *ctx);

/* Page-locked host memory for the *_out buffers of the calls below: a
 * device-to-host copy into it runs at the full host-link rate (NVLink-C2C on
 * GB300) instead of being staged through the driver.  Freed by eg_host_free;
 * independent of any context. */
int eg_host_alloc(uint64_t bytes, void **out);
int eg_host_free(void *p);

/* ---- graph input (replaces init(): init_all.c:791-893) ----------------- */
#define EG_UNDIRECTED 1u /* -u: append reversed copies of every edge
                            (init_all.c:102-106), doubling m (init_all.c:636) */
#define EG_WEIGHTED_FILE 2u /* -w: the file holds 12-byte [src][dst][f32 weight]
                               records (struct input, init_all.h:8-14;
                               item_size, init_all.c:43-49).  The weights are
                               skipped: the adjacency build overwrites them
                               with the CREATE_WEIGHT rule (init_all.c:661-686),
                               which the SSSP weight rules restate. */

/* From host pairs: 2*m uint32 values [src][dst] in file order. */
int eg_graph_from_pairs(eg_ctx *ctx, const uint32_t *pairs, uint64_t m, uint32_t n, unsigned flags,
                        eg_graph **out);
/* From device pairs (copied; the caller keeps ownership). */
int eg_graph_from_device_pairs(eg_ctx *ctx, const uint32_t *d_pairs, uint64_t m, uint32_t n,
                               unsigned flags, eg_graph **out);
/* From a binary [src][dst] uint32 file (init_all.c:812-822, 8-byte records). */
int eg_graph_from_file(eg_ctx *ctx, const char *path, uint32_t n, unsigned flags, eg_graph **out);
/* Synthetic graphs generated on the device (seeded, counter-based):
 * RMAT(scale, a=.57,b=.19,c=.19,d=.05) with m edges, and Erdos-Renyi with n
 * vertices and m uniform (src,dst) pairs. */
int eg_graph_generate_rmat(eg_ctx *ctx, int scale, uint64_t m, uint64_t seed, unsigned flags,
                           eg_graph **out);
int eg_graph_generate_er(eg_ctx *ctx, uint32_t n, uint64_t m, uint64_t seed, unsigned flags,
                         eg_graph **out);
void eg_graph_free(eg_graph *g);

/* ---- layouts (replaces init_adj_sort, init_all.c:629-790, and
 * init_grid_sort, init_all.c:252-361) ------------------------------------ */
#define EG_LAYOUT_CSR 1u /* out-lists, stable by src: each list in file order */
#define EG_LAYOUT_CSC 2u /* in-lists: ascending src, ties in file order */
#define EG_LAYOUT_GRID 4u
#define EG_LAYOUT_EDGES 8u /* the edge array of eg_graph_build_edges */

int eg_graph_build(eg_graph *g, unsigned layouts);
/* 2-D grid of P x P cells (reference partitioning, init_all.c:54-60):
 * cells row-major by (src partition, dst partition), ascending src inside. */
int eg_graph_build_grid(eg_graph *g, uint32_t P);

typedef struct {
    uint32_t n;
    uint64_t m_input; /* edges in the input */
    uint64_t m;       /* adjacency entries (2*m_input with EG_UNDIRECTED) */
    unsigned layouts; /* EG_LAYOUT_* built so far */
    uint32_t grid_p;
    uint64_t device_bytes;
    float build_ms; /* device time of the last eg_graph_build */
} eg_graph_info;
int eg_graph_get_info(eg_graph *g, eg_graph_info *info);
/* Copies a built adjacency to the host: ptr has n+1 entries, col has m. */
int eg_graph_copy_adj(eg_graph *g, unsigned layout, uint32_t *ptr, uint32_t *col);
/* Grid copy: cell_ptr has P*P+1 entries, src/dst have m. */
int eg_graph_copy_grid(eg_graph *g, uint32_t *cell_ptr, uint32_t *src, uint32_t *dst);
/* Out-degree (CSR list lengths) and in-degree; either pointer may be NULL. */
int eg_graph_copy_degrees(eg_graph *g, uint32_t *out_deg, uint32_t *in_deg);

/* Device pointers of graph arrays and of the last result of each algorithm. */
#define EG_DEV_CSR_PTR 1
#define EG_DEV_CSR_COL 2
#define EG_DEV_CSC_PTR 3
#define EG_DEV_CSC_COL 4
#define EG_DEV_OUT_DEG 5
#define EG_DEV_EDGE_SRC 6 /* uint32[m], the edge array's sources (eg_graph_build_edges) */
#define EG_DEV_EDGE_DST 7 /* uint32[m], its destinations */
#define EG_DEV_RANK 10   /* float[n], last eg_pagerank */
#define EG_DEV_LEVEL 11  /* int32[n], last eg_bfs */
#define EG_DEV_PARENT 12 /* int32[n], last eg_bfs with parents */
#define EG_DEV_DIST 13   /* uint32[n], last eg_sssp */
#define EG_DEV_LABEL 14  /* uint32[n], last eg_wcc */
#define EG_DEV_SPMV_Y 15 /* last eg_spmv output */
void *eg_graph_device_ptr(eg_graph *g, int which);

/* ---- PageRank (replaces pagerank_simple.c:72-84,110-133 and
 * prgrid_cilk.c:62-76,111-141) --------------------------------------------
 * Pull over the CSC: rank[v] = base + damping * sum_{u->v} prev[u]/deg[u],
 * fp32 values, fp32 row sums (two-sum compensated when `compensated`).
 * swap=1: prev = rank after every iteration (prgrid, pr_numa).  swap=0
 * reproduces pagerank_simple's pull mode, where prev is never updated.
 * deg_multiplier=2 reproduces the doubled degrees of the grid load modes
 * (init_all.c:851-852).  prev_init < 0 means 1/n (the reference uses 0.15).
 * dangling=1 spreads the mass of out-degree-0 vertices uniformly (FP64
 * reduction on the device); 0 drops it like the reference.
 * tolerance > 0 stops once the FP64 L1 change between iterates is below it. */
typedef struct {
    int iterations;
    float damping;
    float prev_init;
    int swap;
    uint32_t deg_multiplier;
    int dangling;
    int compensated;
    double tolerance;
    int use_graph; /* 1: replay the iteration as a captured CUDA graph */
    int grid;      /* the grid load modes (prgrid_cilk.c:62-141); need
                      eg_graph_build_grid.  1: with the CSR and CSC built,
                      the row kernel over the CSC, whose per-destination
                      order is the order in which prgrid visits a
                      destination's cells (fixed-order sums, source blocks
                      when n > 2^24); otherwise as 2.  2: the cell kernel:
                      cells in L2-sized blocks, sums by atomic adds (not in
                      a fixed order) */
    int source_block_log2; /* not compensated, n > 2^k (k = this, 0: 24): the
                      contributions are gathered one source block of 2^k
                      vertices per pass (a copy of the relabelled CSC split by
                      source, built once), each pass from a slice that L2
                      holds; the earlier blocks' row sums feed the last pass */
} eg_pr_opts;
typedef struct {
    int iterations_run;
    double residual;      /* FP64 L1 change of the last iteration (if computed) */
    double dangling_mass; /* FP64 mass on out-degree-0 vertices, last iterate */
    float ms;             /* device time of the iterations */
    float row_kernel_ms;  /* mean device time of one row-sum kernel launch (up to
                             the first 8 iterations; 0 when use_graph) */
} eg_pr_stats;
void eg_pr_opts_default(eg_pr_opts *o);
int eg_pagerank(eg_graph *g, const eg_pr_opts *opts, float *rank_out, eg_pr_stats *stats);

/* ---- row-kernel autotuner (no reference counterpart) ---------------------
 * The PageRank/SpMV row kernel walks the CSC as warp tiles of 512, 1024 or
 * 2048 entries with 4 or 8 entries per lane, optionally loading the next
 * chunk's indices ahead (prefetch), with min_blocks resident CTAs per SM
 * bounding its registers.
 * eg_graph_tune times every schedule on this graph (two 6-iteration PageRank
 * runs each, CUDA events around the row kernel) and keeps the fastest for
 * eg_pagerank, eg_ppr and eg_spmv on this graph; eg_graph_set_row_schedule
 * picks one by index (0 = 1024 x 4 with prefetch, the default).  cache_hint
 * keeps the streamed row ids and columns out of L1 and first in line for L2
 * eviction.  Schedules change only how rows are split between warps, i.e.
 * the fp32 summation order.
 * The last candidate (index 12) is PageRank's partition kernel: the
 * relabelled CSC cut into partitions of 2^13 rows whose entries are ordered
 * by source, so each source's contribution is gathered once per partition,
 * with 64-bit fixed-point row sums in shared memory (the same bits in any
 * order of addition).  It is kept for eg_pagerank only when it is the
 * fastest; eg_ppr and eg_spmv keep the fastest row schedule.  Its ms is -1
 * when its layout did not fit the context's HBM budget (it is then skipped). */
#define EG_ROW_SCHEDULES_MAX 16
typedef struct {
    int ncand;
    int chosen;               /* index of the schedule kept */
    int tile_entries[EG_ROW_SCHEDULES_MAX];
    int entries_per_lane[EG_ROW_SCHEDULES_MAX];
    int prefetch[EG_ROW_SCHEDULES_MAX];
    int min_blocks[EG_ROW_SCHEDULES_MAX];
    int cache_hint[EG_ROW_SCHEDULES_MAX];
    float ms[EG_ROW_SCHEDULES_MAX]; /* mean row-kernel time per iteration */
    /* 0: a row-kernel schedule; k > 0: PageRank's partition kernel over
     * partitions of 2^k rows (the last candidate) */
    int partition_log2[EG_ROW_SCHEDULES_MAX];
    /* BFS level loop (when the graph has a CSR): mean ms per BFS over 48
     * sampled roots for the CUDA-graph and the host-driven loop (each at its
     * best switch divisor of 20, 40, 80, 160, 320), and the form and the
     * divisor kept for eg_bfs's host_loop = -1 and switch_divisor < 0 */
    float bfs_graph_ms, bfs_host_ms;
    int bfs_host_loop;
    double bfs_switch_divisor; /* the push/pull switch divisor kept */
} eg_tune_result;
int eg_graph_tune(eg_graph *g, eg_tune_result *out);
int eg_graph_set_row_schedule(eg_graph *g, int index);

/* ---- SpMV (replaces spmv.c:98-135) ---------------------------------------
 * Row reductions over a built adjacency:
 *  EG_SPMV_U32_PULL  y[v] = sum over in-edges u->v of x[u]/1000 (u32, wraps);
 *                    the reference's pull mode with its 0.001 scale
 *  EG_SPMV_U32_PUSH  y[u] = sum over out-edges u->v of x[v]/1000 (push mode)
 *  EG_SPMV_U32_EDGE  y[u] = sum over out-edges u->v of x[v] (edge-array mode 8)
 *  EG_SPMV_F32       y[v] = sum over in-edges of val(e)*x[u], fp32
 *  EG_SPMV_F32_COMP  same with two-sum compensated row sums
 *  EG_SPMV_F64       same in fp64 (the error reference on the device)
 * val(e) is the edge value rule below (EG_SPMV_F* only). */
#define EG_SPMV_U32_PULL 0
#define EG_SPMV_U32_PUSH 1
#define EG_SPMV_U32_EDGE 2
#define EG_SPMV_F32 3
#define EG_SPMV_F32_COMP 4
#define EG_SPMV_F64 5
typedef struct {
    int kind;
    uint64_t value_seed; /* val(e) = U[0,1) hashed from (seed, min(u,v), max(u,v)) */
    int unit_values;     /* 1: val(e) = 1 */
    int grid;            /* spmv.c's grid modes; need the grid.  1: with the
                            adjacency the kind reads (CSC for pull and fp
                            kinds, CSR for push and edge) built, its fixed-
                            order row kernel, which sums in the grid's
                            per-row order; otherwise as 2.  2: the cell
                            kernel: cells in L2-sized blocks, y by atomic
                            adds (u32 exact; f32/f64 not in a fixed order;
                            no F32_COMP) */
    int source_block_log2; /* EG_SPMV_F32(_COMP) with n > 2^k (k = this, 0: 24):
                            the entries are split by source block of 2^k
                            vertices (a copy of the CSC built once) and summed
                            one block per pass, so each pass gathers from an
                            x slice that L2 holds; a fixed order */
} eg_spmv_opts;
/* x: host array of n (u32 for U32 kinds, f32 otherwise); y: host array of n
 * (u32, f32 or f64 for EG_SPMV_F64), or NULL to keep y on the device. */
int eg_spmv(eg_graph *g, const eg_spmv_opts *opts, const void *x, void *y, float *ms);

/* ---- BFS (replaces bfs_simple.c:104-229 and bfsgrid_cilk.c:48-168) -------
 * Direction-optimising BFS from `root` over the out-lists.  Levels follow
 * the reference: level[root] = 1, reached vertices level+1 of their parent,
 * unreached 0.  parent_out (optional): a BFS tree, parent[root] = root,
 * -1 unreached.  Pull steps read the in-lists (CSC) of directed graphs and
 * the CSR of undirected ones. */
#define EG_BFS_AUTO 0
#define EG_BFS_PUSH_ONLY 1
#define EG_BFS_PULL_ONLY 2
typedef struct {
    int direction;
    /* auto switches to pull when frontier size + frontier out-degree
     * > m / switch_divisor.  The reference's rule (bfs_simple.c:191-197)
     * counts 2 * deg + 1 per frontier vertex against m / 20
     * (nb_cleaning, buffer.c:272-282), which is divisor 40 here.
     * The direction changes how a level is computed, never its levels.
     * < 0 (default): the graph's divisor, which eg_graph_tune picks by
     * timing (40 until then) */
    double switch_divisor;
    /* 1: compute parents on the device even when parent_out is NULL (read
     * them later through eg_graph_device_ptr(g, EG_DEV_PARENT)) */
    int device_parents;
    /* 0: the level loop runs on the device as one CUDA graph with a
     * conditional while node (no host round trip per level); 1: the host
     * launches and synchronises every level, each kernel on a grid sized to
     * its frontier; -1 (default): the form eg_graph_tune found faster on
     * this graph, else the graph */
    int host_loop;
} eg_bfs_opts;
typedef struct {
    int levels;
    uint32_t reached;
    uint64_t edges_traversed; /* sum of out-degrees of reached vertices */
    int pull_levels;
    float ms;
} eg_bfs_stats;
void eg_bfs_opts_default(eg_bfs_opts *o);
int eg_bfs(eg_graph *g, uint32_t root, const eg_bfs_opts *opts, int32_t *level_out, int32_t *parent_out,
           eg_bfs_stats *stats);
/* eg_bfs from each of k roots in turn (the reference's per-root benchmark
 * loop, bfs_simple.c's main): root i's levels go to level_out + i*n and its
 * parents to parent_out + i*n (either may be NULL); stats, if given, holds k
 * entries.  The copies of root i run on a second stream while root i+1 is
 * traversed, so with page-locked outputs (eg_host_alloc) they overlap the
 * traversals. */
int eg_bfs_batch(eg_graph *g, const uint32_t *roots, uint32_t k, const eg_bfs_opts *opts, int32_t *level_out,
                 int32_t *parent_out, eg_bfs_stats *stats);

/* Multi-source BFS, bit-sliced: up to 64 sources per 64-bit word per vertex,
 * all advanced by one level per sweep.  levels_out: k*n int32, row s holds
 * source s's levels (same convention as eg_bfs), or NULL. */
int eg_bfs_multi(eg_graph *g, const uint32_t *roots, int k, int32_t *levels_out, eg_bfs_stats *stats);

/* ---- SSSP (replaces sssp_pushpull.c:39-190) ------------------------------
 * Exact shortest paths over the out-lists; dist[root] = 0, unreached =
 * UINT32_MAX-1 (sssp_pushpull.c:8).  Weight rules, computed from the edge's
 * endpoints like the reference's CREATE_WEIGHT path:
 *   EG_W_REF   src%10 + dst%10 (init_all.c:661-686)
 *   EG_W_HASH  lo + H(seed, min(u,v), max(u,v)) mod (hi-lo+1), symmetric
 *   EG_W_UNIT  1 (hop counts)
 *   EG_W_HASH_F32  fp32 weights in (0,1]: ((H >> 40) + 1) / 2^24; the path
 *              sums are rounded to fp32 like the reference's float add
 *              (sssp_pushpull.c:81), and dist_out holds fp32 bit patterns
 *              (unreached = +inf, 0x7f800000).  Not accepted by the server. */
#define EG_W_REF 0
#define EG_W_HASH 1
#define EG_W_UNIT 2
#define EG_W_HASH_F32 3
typedef struct {
    int rule;
    uint64_t seed;
    uint32_t lo, hi;
} eg_weights;
typedef struct {
    int rounds;
    uint32_t reached;
    uint64_t relaxations;
    float ms;
} eg_sssp_stats;
int eg_sssp(eg_graph *g, uint32_t root, const eg_weights *w, uint32_t *dist_out, eg_sssp_stats *stats);
/* k sources in one batch; dist_out: k*n uint32 (row s for source s) or NULL. */
int eg_sssp_multi(eg_graph *g, const uint32_t *roots, int k, const eg_weights *w, uint32_t *dist_out,
                  eg_sssp_stats *stats);

/* ---- WCC (replaces wcc.c:30-90,186-286) ----------------------------------
 * Weakly connected components; label = the minimum vertex id of the
 * component (the fixed point of the reference's min-label propagation). */
typedef struct {
    int rounds;
    uint32_t components;
    float ms;
} eg_wcc_stats;
int eg_wcc(eg_graph *g, int64_t *labels_out, eg_wcc_stats *stats);

/* ---- edge array (replaces init_edgelist, init_all.c:573-628: load modes
 * 7, 8, 9) ------------------------------------------------------------------
 * Builds the device edge array without any CSR or CSC: the input's edges
 * (reversed copies after them with EG_UNDIRECTED) as two uint32 arrays,
 * sources and destinations, in one of three orders, plus the out- and
 * in-degree counts (count_degree, init_all.c:425-443).  The edge-centric
 * calls below stream it; eg_wcc on a graph without a CSR hooks the input
 * edges directly (the WCC edge loop, wcc.c:235-261). */
#define EG_EDGES_FILE_ORDER 0  /* mode 9: input order, no sort */
#define EG_EDGES_BY_SRC 1      /* mode 7: stable sort by source */
#define EG_EDGES_BY_SRC_DST 2  /* mode 8: by source, then by destination */
int eg_graph_build_edges(eg_graph *g, int order);
/* Copies the edge array to the host (src and dst have m entries; either may
 * be NULL). */
int eg_graph_copy_edges(eg_graph *g, uint32_t *src, uint32_t *dst);
/* Edge-centric BFS (bfs_edgecentric, bfs_simple.c:58-103): every level
 * streams the whole edge array and each edge whose source is in the frontier
 * claims its unvisited destination.  Same levels (root 1, unreached 0) and
 * parent convention as eg_bfs. */
int eg_edges_bfs(eg_graph *g, uint32_t root, int32_t *level_out, int32_t *parent_out, eg_bfs_stats *stats);
/* Edge-centric PageRank (pr_algo_edgecentric, pagerank_simple.c:40-61, and
 * prgrid_algo_col, prgrid_cilk.c:79-88): every iteration adds
 * prev[src]/deg[src] into rank[dst] for every edge with fp32 atomic adds
 * (not in a fixed order), then rank = (1-d)/n + d * sum.  Uses iterations,
 * damping, prev_init, swap, deg_multiplier, dangling and tolerance of the
 * options (swap = 0 keeps prev at prev_init).  stats->row_kernel_ms is 0. */
int eg_edges_pagerank(eg_graph *g, const eg_pr_opts *opts, float *rank_out, eg_pr_stats *stats);
/* The SpMV edge loop (spmv.c:130-135): y[src] += x[dst] over every edge,
 * u32 wrapping adds (exact in any order).  x: host array of n; y: host array
 * of n or NULL (kept on the device, EG_DEV_SPMV_Y). */
int eg_edges_spmv_u32(eg_graph *g, const uint32_t *x, uint32_t *y, float *ms);

/* ---- layout cache (no working counterpart: the reference's pre-processed
 * file path, random.c:6 and init_all.c:823-824, is dead code) --------------
 * eg_graph_save_layouts writes every layout the graph has built (CSR and CSC
 * with their row ids, the grid, the edge array, the degree arrays) to `path`
 * behind a header naming the input: n, the input edge count, the flags and a
 * 64-bit digest of the input edges computed on the device.  The file is
 * written under path + ".tmp" and renamed.  eg_graph_load_layouts fills a
 * graph loaded from the same input from such a file instead of sorting:
 * *hit = 1 when it did; *hit = 0 (and EG_OK) when the file is absent or
 * belongs to another input; EG_EIO when a matching file is truncated. */
int eg_graph_save_layouts(eg_graph *g, const char *path);
int eg_graph_load_layouts(eg_graph *g, const char *path, int *hit);

/* ---- personalised PageRank, batched ---------------------------------------
 * No counterpart in the reference (which runs one global PageRank; the
 * iteration is pr_numa.c:245-277,396 with teleport to a seed set).  Up to 32
 * queries per call, query q seeded by seeds[seed_offsets[q] ..
 * seed_offsets[q+1]): x' = d * A^T D^-1 x + (1 - d + d * dangling(x)) * t,
 * t uniform over the seeds, x0 = t.  Query q stops when the FP64 L1 change
 * of its vector is below tolerance[q] or after max_iters.  Each query's
 * result is bit-identical alone or in any batch.  ranks_out: nq*n floats
 * (row q for query q) or NULL. */
typedef struct {
    float damping;
    int max_iters;
    float tolerance[32];
} eg_ppr_opts;
typedef struct {
    int iterations[32];
    double residual[32];
    int sweeps; /* batch iterations run */
    float ms;
} eg_ppr_stats;
int eg_ppr_multi(eg_graph *g, const uint32_t *seeds, const uint32_t *seed_offsets, int nq, const eg_ppr_opts *opts,
                 float *ranks_out, eg_ppr_stats *stats);
/* One personalised PageRank query on the plain PageRank row kernel (the
 * one-query-at-a-time path): the same iteration with the teleport and the
 * dangling mass sent to at most 8 distinct seeds (repeats count with their
 * multiplicity); stops on opts->tolerance[0] or max_iters.  Fills
 * iterations[0], residual[0], sweeps and ms of the stats. */
int eg_ppr(eg_graph *g, const uint32_t *seeds, uint32_t nseeds, const eg_ppr_opts *opts, float *rank_out,
           eg_ppr_stats *stats);

/* ---- query server (continuous batching) ----------------------------------
 * No counterpart in the reference (one algorithm per process).  A server
 * keeps the graph and every admitted query's state in HBM.  eg_serve_step is
 * one scheduler pass.  The three engines (64 BFS slots, 64 SSSP slots, 32
 * PPR lanes at most; fewer when hbm_budget cannot hold their state) run on
 * their own CUDA streams; an engine whose step (one BFS level, one
 * Bellman-Ford round, one PPR iteration over all its live slots) has
 * finished retires its finished queries, admits queued ones into the freed
 * slots and launches its next step, without waiting for the other engines.
 * Queries join and leave between ticks; a slot's arithmetic never reads
 * another slot's values, so results do not depend on the mix.  Results stay
 * on the device; eg_serve_poll returns a summary per finished query, and
 * with keep_results the full result (levels, distances, or fp32 ranks as
 * u32 words) is kept in host memory in completion order. */
#define EG_Q_BFS 1
#define EG_Q_SSSP 2
#define EG_Q_PPR 3
typedef struct eg_server eg_server;
typedef struct {
    int kind;
    uint32_t source;   /* BFS / SSSP */
    uint32_t nseeds;   /* PPR: 1..8 */
    uint32_t seeds[8];
    float tol;         /* PPR tolerance (<= 0: 1e-6) */
    double arrival_s;  /* arrival time on the server clock (<= 0: now) */
} eg_query;
typedef struct {
    uint64_t id;
    int kind;
    double arrival_s, admit_s, done_s; /* server clock, seconds */
    uint32_t reached;                  /* BFS/SSSP: vertices reached */
    uint32_t depth;                    /* BFS: deepest level; SSSP: largest distance */
    int iterations;                    /* levels / rounds / PPR iterations */
    double value;                      /* PPR: sum of the rank vector */
} eg_query_result;
typedef struct {
    uint64_t hbm_budget; /* bytes of per-query state the server may hold */
    int max_bfs, max_sssp, max_ppr;
    eg_weights weights;  /* SSSP weight rule */
    float ppr_damping;
    int ppr_max_iters;
    int keep_results;
    int exclusive;       /* 1: one engine step on the GPU at a time (engines
                            take turns, each step gets the whole GPU and L2);
                            0 (default): the engines' steps overlap */
    int gang;            /* 1 (default): SSSP queries enter in gangs: a word
                            of 32 source slots is refilled only once all of
                            its sources have finished, so the sources that
                            share a word stay in step and relax dense rows;
                            BFS queries enter only while no BFS slot is live,
                            so that the 64 bit-sliced sources advance level
                            by level together;
                            0: a free slot takes the next query at once
                            (lower latency under light load) */
} eg_serve_opts;
void eg_serve_opts_default(eg_serve_opts *o);
int eg_serve_open(eg_graph *g, const eg_serve_opts *opts, eg_server **out);
int eg_serve_submit(eg_server *s, const eg_query *q, uint64_t *id_out);
/* active_out: queries admitted or queued after the tick */
int eg_serve_step(eg_server *s, int *active_out);
int eg_serve_poll(eg_server *s, eg_query_result *out, int max, int *count);
/* next kept full result (n u32 words), in completion order */
int eg_serve_take_result(eg_server *s, uint32_t *out, uint32_t n);
int eg_serve_info(eg_server *s, int *bfs_slots, int *sssp_slots, int *ppr_slots, double *clock_s);
/* Per-engine counters since eg_serve_open: index 0 BFS, 1 SSSP, 2 PPR.
 * engine_ms is the device time of the engine's steps (CUDA events on the
 * engine's stream; engines overlap, so the three can sum past wall time). */
typedef struct {
    uint64_t ticks;
    uint64_t queued;
    double engine_ms[3];
    uint64_t engine_steps[3];
    uint64_t admitted[3];
    uint64_t completed[3];
} eg_serve_stats_t;
int eg_serve_stats(eg_server *s, eg_serve_stats_t *out);
int eg_serve_close(eg_server *s);

/* ---- allocation-free SpMV ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (a host callback, a plug-in inside a process whose allocator it does
 * not own, a service that has handed HBM to its own pool): y[v] = sum over
 * entries p of row v of vals[p] * x[col[p]] (fp32, vals NULL = all ones)
 * over a caller-owned CSR-shaped array pair in device memory.  All pointers
 * are device pointers; stream is a cudaStream_t (NULL = legacy default).
 * The call allocates nothing: its scratch is a fixed 1.5 MiB array compiled
 * into the library, held by every GPU that loads it until the process exits,
 * which limits n + m to EG_NOALLOC_MAX_ITEMS (larger inputs are rejected
 * with EG_EINVAL).  The first call on a device looks that array up with
 * cudaGetSymbolAddress; make that first call before any stream capture.
 * Every call on a device shares the array (it keeps the last call's
 * contents; each call writes all it reads), so calls that overlap on the GPU
 * race: serialise them on one stream.  Rows are summed over merge-path
 * tiles of 2048 items (row ends + entries), a different fp32 summation order
 * from eg_spmv's EG_SPMV_F32, so the two agree within fp32 rounding (relative
 * L1 <= 1e-6 in the tests), not bit for bit. */
#define EG_NOALLOC_MAX_ITEMS (65536ull * 2048ull)
int eg_spmv_f32_noalloc(const uint32_t *d_ptr, const uint32_t *d_col, const float *d_vals, const float *d_x,
                        float *d_y, uint32_t n, uint64_t m, void *stream);

/* Samples k roots uniformly from vertices with out-degree > 0 (the same
 * counter-based rule as the CPU generator). */
int eg_sample_roots(eg_graph *g, int k, uint64_t seed, uint32_t *roots_out);

#ifdef __cplusplus
}
#endif
#endif /* EG_GPU_H */
