/*
 * SSSP plug-in, replacing sssp_pushpull.c (current_algo, 240-242).  Root
 * from -p, weights src%10 + dst%10 (the CREATE_WEIGHT rule,
 * init_all.c:661-686), distances exact (the fixed point of the weighted pull
 * relax, sssp_pushpull.c:69-98).  -a 0 -r runs the reference's push relax,
 * which adds 1 per edge (sssp_pushpull.c:46): hop counts.
 */
#include "eg_host.h"

static uint32_t *dist_h;
static void s_construct(void) { dist_h = malloc((size_t)NB_NODES * sizeof(uint32_t)); }
static void s_reset(struct node *n) { (void)n; }
static void s_main(struct node *n) {
    (void)n;
    eg_weights w = {EG_W_REF, 0, 0, 0};
    if (!switch_mode && mode == PUSH) w.rule = EG_W_UNIT;
    eg_sssp_stats st;
    eg_need_adjacency(EG_LAYOUT_CSR);  // the edge-array modes build none
    if (eg_sssp(eg_g, BFS_ROOT, &w, dist_h, &st) != EG_OK) eg_die("sssp");
    printf("#Algo time ( %.3f sec) \n", st.ms / 1000.0);
    uint32_t t = 0;
    for (uint32_t i = 0; i < NB_NODES; i++)
        if (dist_h[i] != UINT32_MAX - 1 && dist_h[i] > t) t = dist_h[i];
    printf("Max dist = %d and dist[1] is %d\n", (int)t, NB_NODES > 1 ? (int)dist_h[1] : 0);
}
static void s_destruct(void) {
    uint64_t found = 0;
    for (uint32_t i = 0; i < NB_NODES; i++) found += dist_h[i] != UINT32_MAX - 1;
    printf("Total nodes discovered:: %llu\n", (unsigned long long)found);
    eg_dump(dist_h, sizeof(uint32_t), NB_NODES);
    free(dist_h);
}
struct algo_func current_algo = {.reset = s_reset, .main = s_main, .construct = s_construct, .destruct = s_destruct};
