/*
 * SpMV plug-in, replacing spmv.c (current_algo, 161-163): x[i] = i
 * (spmv.c:125-128), u32 y; pull (-a 1) and push (-a 0) scale x by 0.001
 * (spmv.c:98-118), the edge-array mode 8 adds x[dst] into y[src]
 * (spmv.c:130-135) over the device edge array; modes 7 and 9 (which the
 * reference runs on adjacency arrays it never built) run the same edge loop.
 */
#include "eg_host.h"

static uint32_t *x, *y;
static void s_construct(void) {
    x = malloc((size_t)NB_NODES * sizeof(uint32_t));
    y = malloc((size_t)NB_NODES * sizeof(uint32_t));
}
static void s_reset(struct node *n) { (void)n; }
static void s_main(struct node *n) {
    (void)n;
    for (uint32_t i = 0; i < NB_NODES; i++) x[i] = i;
    float ms = 0;
    if (load_mode > 6) {
        if (eg_edges_spmv_u32(eg_g, x, y, &ms) != EG_OK) eg_die("spmv");
    } else {
        eg_spmv_opts o = {.kind = EG_SPMV_U32_PUSH}; /* the other fields 0: CSR/CSC path, u32 x */
        if (mode == PULL) o.kind = EG_SPMV_U32_PULL;
        if (eg_spmv(eg_g, &o, x, y, &ms) != EG_OK) eg_die("spmv");
    }
    printf("#Algo time ( %.3f sec) \n", ms / 1000.0);
}
static void s_destruct(void) {
    eg_dump(y, sizeof(uint32_t), NB_NODES);
    free(x);
    free(y);
}
struct algo_func current_algo = {.reset = s_reset, .main = s_main, .construct = s_construct, .destruct = s_destruct};
