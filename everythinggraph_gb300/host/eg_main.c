/*
 * Drop-in driver: the reference's command line (random.c:50-145) over the
 * GPU library.  Same flags (-f -n -m -u -w -a -p -s -r -N -h), same plug-in
 * call order (construct, reset, main, destruct) and the same timing lines.
 */
#define _GNU_SOURCE
#include <getopt.h>
#include <locale.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "eg_host.h"

char *filename;
uint32_t NB_NODES;
uint64_t nb_edges;
uint32_t P;
uint32_t BFS_ROOT;
int load_mode = 2;
int createUndir = 0;
int isSymmetric = 0;
int weighted_graph = 0;
int switch_mode = 1;
algo_mode mode = PUSH;
struct node *nodes = NULL;
eg_ctx *eg_context;
eg_graph *eg_g;

double eg_now(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

void eg_die(const char *what) {
    fprintf(stderr, "%s: %s\n", what, eg_last_error());
    exit(1);
}

void eg_dump(const void *p, size_t sz, size_t n) {
    const char *path = getenv("EG_DUMP");
    if (!path) return;
    FILE *f = fopen(path, "wb");
    if (!f || fwrite(p, sz, n, f) != n) {
        fprintf(stderr, "dump to %s failed\n", path);
        exit(3);
    }
    fclose(f);
}

static void usage(void) {
    printf("Usage: %s -f <graph file> -n <nb_nodes> [-m mode -u -w -a mode -p root -s -r]\n", "eg_<algo>");
    printf("\t-u: create undirected on load\n");
    printf("\t-r: do not switch between PUSH and PULL\n");
    printf("\t-a [mode]: 0 PUSH, 1 PULL\n");
    printf("\t-p [root]: BFS & SSSP root\n");
    printf("\t-s: symmetric graph, no in-edges created\n");
    printf("\t-m [0..9]: 0/6 grid, 1 grid nosort, 2/3 adjacency (sort), 4 count sort, 5 dynamic, 7/8/9 edge array;\n"
           "\t           every mode builds its layout on the GPU\n");
    fflush(stdout);
    _exit(255);
}

int main(int argc, char **argv) {
    setlocale(LC_NUMERIC, "");
    int c;
    while ((c = getopt(argc, argv, "f:n:m:uwLa:p:srNh")) != -1) {
        switch (c) {
            case 'f': filename = optarg; break;
            case 'm':
                load_mode = atoi(optarg);
                printf("Load mode = %d\n", load_mode);
                break;
            case 'n':
                NB_NODES = (uint32_t)atol(optarg);
                P = (NB_NODES * 8u / 1024u) / 20u; /* random.c:69-71 */
                if (P > 2000) P = 256;
                if (P == 0) P = 4;
                printf("P = %d\n", P);
                break;
            case 'u':
                createUndir = 1;
                printf("#Creating Undir\n");
                break;
            case 'r': switch_mode = 0; break;
            case 's':
                isSymmetric = 1;
                printf(" no in-edges created\n");
                break;
            case 'a': mode = atoi(optarg) == 0 ? PUSH : PULL; break;
            case 'w': weighted_graph = 1; break;
            case 'p': BFS_ROOT = (uint32_t)atol(optarg); break;
            case 'N': break;
            case 'h':
            default: usage();
        }
    }
    if (!NB_NODES || !filename) usage();
    printf("#Running on the GPU (%s)\n", eg_version());
    double start = eg_now();
    init(0);
    double stop = eg_now();
    printf("#Total loading time ( %fs )\n", stop - start);
    current_algo.construct();
    start = eg_now();
    double ls = eg_now();
    current_algo.reset(nodes);
    printf("#Total reset  time ( %fs )\n", eg_now() - ls);
    current_algo.main(nodes);
    stop = eg_now();
    printf("#Total algo time ( %fs )\n", stop - start);
    current_algo.destruct();
    eg_graph_free(eg_g);
    eg_close(eg_context);
    return 0;
}
