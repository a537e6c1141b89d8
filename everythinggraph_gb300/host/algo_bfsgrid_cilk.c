/*
 * Grid BFS plug-in, replacing bfsgrid_cilk.c (current_algo, 221-223): only
 * the grid load modes are accepted (bfsgrid_cilk.c:94-97), the root comes
 * from -p, dist[] holds levels with the root at 1 (bfsgrid_cilk.c:59,188).
 */
#include "eg_host.h"

static int32_t *dist_h;
static void g_construct(void) {
    if (load_mode != 0 && load_mode != 1 && load_mode != 6) {
        printf("To run this, you need to give grid as the data layout, otherwise work with pagerank_simple\n");
        exit(1);
    }
    dist_h = calloc(NB_NODES, sizeof(int32_t));
}
static void g_reset(struct node *n) { (void)n; }
static void g_main(struct node *n) {
    (void)n;
    eg_bfs_stats st;
    if (eg_bfs(eg_g, BFS_ROOT, NULL, dist_h, NULL, &st) != EG_OK) eg_die("bfs");
    printf("#Algo time ( %.3f sec) \n", st.ms / 1000.0);
}
static void g_destruct(void) {
    uint64_t found = 0;
    for (uint32_t i = 0; i < NB_NODES; i++) found += dist_h[i] != 0;
    printf("Total nodes discovered:: %llu\n", (unsigned long long)found);
    eg_dump(dist_h, sizeof(int32_t), NB_NODES);
    free(dist_h);
}
struct algo_func current_algo = {.reset = g_reset, .main = g_main, .construct = g_construct, .destruct = g_destruct};
