/*
 * WCC plug-in, replacing wcc.c (current_algo, 295-297): labels are the
 * minimum vertex id of each weakly connected component (long components[],
 * wcc.c:12), supported load modes 0, 8 and 2/3/4 (wcc.c:192-281), and the
 * validate() summary line (wcc.c:138-182).
 */
#include "eg_host.h"

static int64_t *comp;
static void w_construct(void) { comp = malloc((size_t)NB_NODES * sizeof(int64_t)); }
static void w_reset(struct node *n) { (void)n; }
static void w_main(struct node *n) {
    (void)n;
    if (!(load_mode == 0 || load_mode == 8 || (load_mode >= 2 && load_mode <= 4))) {
        printf("Don't know how to run with this layout\n");
        exit(1);
    }
    eg_wcc_stats st;
    if (eg_wcc(eg_g, comp, &st) != EG_OK) eg_die("wcc");
    printf("Algo time %f \n", st.ms / 1000.0);
    uint32_t *cnt = calloc(NB_NODES, sizeof(uint32_t));
    uint32_t total = 0, mx = 0;
    for (uint32_t i = 0; i < NB_NODES; i++) cnt[comp[i]]++;
    for (uint32_t i = 0; i < NB_NODES; i++) {
        if (cnt[i] > mx) mx = cnt[i];
        if (cnt[i]) total++;
    }
    free(cnt);
    printf("Total comp %d , max comp %d \n", (int)total, (int)mx);
}
static void w_destruct(void) {
    eg_dump(comp, sizeof(int64_t), NB_NODES);
    free(comp);
}
struct algo_func current_algo = {.reset = w_reset, .main = w_main, .construct = w_construct, .destruct = w_destruct};
