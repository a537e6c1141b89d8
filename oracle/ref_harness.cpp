/*
 * Result-dump harness for the unmodified reference binaries (test
 * infrastructure only).  The reference's random.c is compiled a second time
 * with -Dmain=ref_main; this main swaps current_algo.destruct for a hook that
 * writes the algorithm's result array to the file named by $EG_DUMP, then
 * calls the original destruct.  The plug-in struct and its call order come
 * from random.h:64-69 and random.c:128-143.
 *
 * Compiled once per algorithm with -DEG_DUMP_<KIND>:
 *   PR_RANK   float rank[n]    (pagerank_simple.c: result of the pull loop)
 *   PR_PREV   float prev[n]    (prgrid_cilk.c: prev holds the last iterate)
 *   DIST      uint32 dist[n]   (bfs_simple.c, bfsgrid_cilk.c, sssp_pushpull.c)
 *   COMP      int64 components[n] (wcc.c)
 *   SPMV      uint32 value_out[n] (spmv.c)
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>

struct node;
struct algo_func {
    void (*reset)(struct node *);
    void (*main)(struct node *);
    void (*construct)(void);
    void (*destruct)(void);
};
extern struct algo_func current_algo;
extern uint32_t NB_NODES;

#if defined(EG_DUMP_PR_RANK)
extern float *rank;
#define EG_PTR rank
#define EG_ELEM sizeof(float)
#elif defined(EG_DUMP_PR_PREV)
extern float *prev;
#define EG_PTR prev
#define EG_ELEM sizeof(float)
#elif defined(EG_DUMP_DIST)
extern uint32_t *dist;
#define EG_PTR dist
#define EG_ELEM sizeof(uint32_t)
#elif defined(EG_DUMP_COMP)
extern long *components;
#define EG_PTR components
#define EG_ELEM sizeof(long)
#elif defined(EG_DUMP_SPMV)
extern uint32_t *value_out;
#define EG_PTR value_out
#define EG_ELEM sizeof(uint32_t)
#else
#error "define one EG_DUMP_<KIND>"
#endif

static void (*orig_destruct)(void);

static void dump_then_destruct(void) {
    const char *path = getenv("EG_DUMP");
    if (path) {
        FILE *f = fopen(path, "wb");
        if (!f || fwrite((const void *)EG_PTR, EG_ELEM, NB_NODES, f) != NB_NODES) {
            fprintf(stderr, "dump to %s failed\n", path);
            exit(3);
        }
        fclose(f);
    }
    orig_destruct();
}

int ref_main(int argc, char **argv);

int main(int argc, char **argv) {
    orig_destruct = current_algo.destruct;
    current_algo.destruct = dump_then_destruct;
    return ref_main(argc, argv);
}
