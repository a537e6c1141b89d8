/*
 * Grid PageRank plug-in, replacing prgrid_cilk.c (current_algo, 188-190):
 * ten iterations with prev = rank (prgrid_cilk.c:111-141), prev starting at
 * 0.15 (98).  Modes 0, 1, 6 and 9 count degrees twice (init_all.c:91-94
 * and 851-852; modes 7 and 8 rewrite them from the sorted edge array,
 * init_all.c:605-609), so the divisor is doubled there, as in the
 * reference.  In the grid modes (0, 1, 6) the iterations run over the device
 * grid's cells, like prgrid_algo's tile loops (prgrid_cilk.c:62-76); in the
 * edge-array modes (7, 8, 9) over the edge array, like prgrid_algo_col
 * (prgrid_cilk.c:79-88); otherwise over the CSC, whose per-destination
 * order equals the grid's.
 */
#include "eg_host.h"

static float *rank_h;

static void g_construct(void) { rank_h = malloc((size_t)NB_NODES * sizeof(float)); }
static void g_reset(struct node *n) { (void)n; }
static void g_main(struct node *n) {
    (void)n;
    eg_pr_opts o;
    eg_pr_opts_default(&o);
    o.prev_init = 0.15f;
    o.swap = 1;
    o.deg_multiplier = (load_mode < 2 || load_mode == 6 || load_mode == 9) ? 2 : 1;
    o.grid = load_mode == 0 || load_mode == 1 || load_mode == 6;
    eg_pr_stats st;
    if (load_mode > 6) {
        if (eg_edges_pagerank(eg_g, &o, rank_h, &st) != EG_OK) eg_die("pagerank");
    } else if (eg_pagerank(eg_g, &o, rank_h, &st) != EG_OK) {
        eg_die("pagerank");
    }
    printf("Iter %d time %f \n", st.iterations_run, st.ms / 1000.0);
    eg_dump(rank_h, sizeof(float), NB_NODES);
}
static void g_destruct(void) { free(rank_h); }
struct algo_func current_algo = {.reset = g_reset, .main = g_main, .construct = g_construct, .destruct = g_destruct};
