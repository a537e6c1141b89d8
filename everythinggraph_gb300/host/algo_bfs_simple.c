/*
 * BFS plug-in, replacing bfs_simple.c (current_algo, 298-300).  Root 0
 * (bfs_simple.c:6).  Grid modes are refused as in bfs_simple.c:256-259; the
 * edge-array modes (> 6) run the edge-centric BFS (bfs_simple.c:260-261).
 * dist[] holds BFS levels with the root at 1 and 0 for unreached vertices
 * (the edge-centric mode's values; the push/pull modes of the reference
 * store 1 for every visited vertex, i.e. dist != 0 marks the same set).
 */
#include "eg_host.h"

static int32_t *dist_h;
static void b_construct(void) { dist_h = calloc(NB_NODES, sizeof(int32_t)); }
static void b_reset(struct node *n) { (void)n; }
static void b_main(struct node *n) {
    (void)n;
    if (load_mode < 2 || load_mode == 6) {
        printf("Use the BFS grid file, don't know how to run BFS here with this layout\n");
        exit(1);
    }
    eg_bfs_stats st;
    if (load_mode > 6) {
        if (eg_edges_bfs(eg_g, 0, dist_h, NULL, &st) != EG_OK) eg_die("bfs");
    } else {
        eg_bfs_opts o;
        eg_bfs_opts_default(&o);
        if (!switch_mode) o.direction = mode == PULL ? EG_BFS_PULL_ONLY : EG_BFS_PUSH_ONLY;
        if (eg_bfs(eg_g, 0, &o, dist_h, NULL, &st) != EG_OK) eg_die("bfs");
    }
    printf("Done in %d iterations and found %u nodes\n", st.levels, st.reached);
    printf("#Algo time ( %.3f sec) \n", st.ms / 1000.0);
}
static void b_destruct(void) {
    uint64_t found = 0;
    for (uint32_t i = 0; i < NB_NODES; i++) found += dist_h[i] != 0;
    printf("Total nodes discovered:: %llu\n", (unsigned long long)found);
    eg_dump(dist_h, sizeof(int32_t), NB_NODES);
    free(dist_h);
}
struct algo_func current_algo = {.reset = b_reset, .main = b_main, .construct = b_construct, .destruct = b_destruct};
