/*
 * PageRank plug-in, replacing pagerank_simple.c (current_algo, 177-179).
 * PULL (-a 1) keeps the reference's pull semantics: prev stays at 0.15 and
 * the ten iterations recompute one step (pagerank_simple.c:110-133).  PUSH
 * and the edge-centric modes (> 6) iterate with prev = rank, which is what
 * their loops intend (pagerank_simple.c:40-70, 119-123).  The printed
 * Rank[0..9] are prev, as in pagerank_simple.c:159-161.
 */
#include "eg_host.h"

static float *rank_h;
static float *prev_h;

static void pr_construct(void) {
    rank_h = malloc((size_t)NB_NODES * sizeof(float));
    prev_h = malloc((size_t)NB_NODES * sizeof(float));
}
static void pr_reset(struct node *n) { (void)n; }
static void pr_main(struct node *n) {
    (void)n;
    eg_pr_opts o;
    eg_pr_opts_default(&o);
    o.prev_init = 0.15f;
    o.swap = !(mode == PULL && load_mode <= 6);
    eg_pr_stats st;
    if (load_mode > 6) {  // pr_algo_edgecentric over the edge array (pagerank_simple.c:40-61)
        if (eg_edges_pagerank(eg_g, &o, rank_h, &st) != EG_OK) eg_die("pagerank");
    } else if (eg_pagerank(eg_g, &o, rank_h, &st) != EG_OK) {
        eg_die("pagerank");
    }
    printf("#Algo time ( %.3f sec) \n", st.ms / 1000.0);
    for (uint32_t i = 0; i < NB_NODES; i++) prev_h[i] = o.swap ? rank_h[i] : 0.15f;
    for (int i = 0; i < 10 && i < (int)NB_NODES; i++) printf("Rank[%d] = %.5f\n", i, prev_h[i]);
    eg_dump(rank_h, sizeof(float), NB_NODES);
}
static void pr_destruct(void) {
    free(rank_h);
    free(prev_h);
}
struct algo_func current_algo = {.reset = pr_reset, .main = pr_main, .construct = pr_construct, .destruct = pr_destruct};
