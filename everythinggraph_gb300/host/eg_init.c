/*
 * Loader: replaces init() (init_all.c:791-893).  The file's [src][dst]
 * records go to HBM and the layout selected by load_mode is built there:
 *   0, 6      2-D grid (init_grid_sort) - plus CSR/CSC for the degree arrays
 *   1         grid without sort: same device grid (the reference's
 *             per-cell realloc lists are a host-side construction method)
 *   2, 3      CSR + CSC by stable device radix sort (init_adj_sort)
 *   4, 5      count sort / dynamic lists: the same device CSR + CSC
 *   7, 8, 9   edge array only, no adjacency (init_edgelist,
 *             init_all.c:573-628): 7 sorted by src, 8 by src then dst,
 *             9 in file order (eg_graph_build_edges)
 * -u appends the reversed edges for the adjacency modes only, as in the
 * reference (init_all.c:636 doubles nb_edges only in init_adj_sort).
 * With EG_LAYOUT_CACHE=<directory> set, the built layouts are kept in
 * <directory>/<file name>.m<mode>[u][P].eglayout and a later run on the same
 * input fills them from there instead of sorting (the file's header carries
 * a digest of the input edges, so a changed input is rebuilt).
 */
#include <string.h>

#include "eg_host.h"

/* <EG_LAYOUT_CACHE>/<base name of the input>.m<mode>[u]p<P>.eglayout, or ""
 * without the variable. */
static void cache_path(char *out, size_t len) {
    const char *dir = getenv("EG_LAYOUT_CACHE");
    out[0] = 0;
    if (!dir || !*dir) return;
    const char *base = strrchr(filename, '/');
    base = base ? base + 1 : filename;
    snprintf(out, len, "%s/%s.m%d%sp%u.eglayout", dir, base, load_mode, createUndir ? "u" : "", (unsigned)P);
}

void init(int full) {
    (void)full;
    if (eg_open(0, 0, &eg_context) != EG_OK) eg_die("eg_open");
    unsigned flags = 0;
    int adjacency_mode = load_mode >= 2 && load_mode <= 5;
    if (createUndir && adjacency_mode) flags |= EG_UNDIRECTED;
    if (weighted_graph) flags |= EG_WEIGHTED_FILE;  // 12-byte records, weights skipped
    printf("Load start");
    if (eg_graph_from_file(eg_context, filename, NB_NODES, flags, &eg_g) != EG_OK) eg_die("load");
    eg_graph_info info;
    eg_graph_get_info(eg_g, &info);
    nb_edges = info.m;
    printf("#NB edges = %llu\n", (unsigned long long)info.m_input);
    char cpath[4096];
    cache_path(cpath, sizeof(cpath));
    if (cpath[0]) {
        int hit = 0;
        double t0 = eg_now();
        if (eg_graph_load_layouts(eg_g, cpath, &hit) != EG_OK) eg_die("layout cache");
        if (hit) {
            printf("#Layout cache hit %s ( %f s )\n", cpath, eg_now() - t0);
            return;
        }
    }
    if (load_mode >= 7 && load_mode <= 9) {
        const int order = load_mode == 7 ? EG_EDGES_BY_SRC : load_mode == 8 ? EG_EDGES_BY_SRC_DST : EG_EDGES_FILE_ORDER;
        if (eg_graph_build_edges(eg_g, order) != EG_OK) eg_die("edge array build");
        eg_graph_get_info(eg_g, &info);
        printf("#Device edge array build time ( %f s )\n", info.build_ms / 1000.0);
        if (cpath[0] && eg_graph_save_layouts(eg_g, cpath) != EG_OK) eg_die("layout cache save");
        return;
    }
    unsigned layouts = EG_LAYOUT_CSR | EG_LAYOUT_CSC;
    if (isSymmetric && adjacency_mode) layouts = EG_LAYOUT_CSR;
    if (eg_graph_build(eg_g, layouts) != EG_OK) eg_die("build");
    if (load_mode == 0 || load_mode == 1 || load_mode == 6) {
        if (eg_graph_build_grid(eg_g, P) != EG_OK) eg_die("grid build");
    }
    eg_graph_get_info(eg_g, &info);
    printf("#Device layout build time ( %f s )\n", info.build_ms / 1000.0);
    if (cpath[0] && eg_graph_save_layouts(eg_g, cpath) != EG_OK) eg_die("layout cache save");
}

void eg_need_adjacency(unsigned layouts) {
    eg_graph_info info;
    eg_graph_get_info(eg_g, &info);
    if ((info.layouts & layouts) == layouts) return;
    if (eg_graph_build(eg_g, layouts) != EG_OK) eg_die("adjacency build");
}
