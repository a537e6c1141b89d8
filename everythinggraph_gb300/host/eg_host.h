/*
 * Host side of the drop-in: the reference's driver globals and plug-in
 * interface, with the graph living on the GPU behind include/eg_gpu.h.
 *
 * struct algo_func and its call order are those of random.h:64-69 and
 * random.c:128-143; the load-mode numbers and the globals are those of
 * init_all.h:32-60 and random.c:3-24.
 */
#ifndef EG_HOST_H
#define EG_HOST_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "eg_gpu.h"

struct node; /* opaque: vertex state lives on the device */

struct algo_func {
    void (*reset)(struct node *);
    void (*main)(struct node *);
    void (*construct)(void);
    void (*destruct)(void);
};
extern struct algo_func current_algo;

typedef enum { PUSH, PULL } algo_mode;

/* driver globals (random.c:3-24, init_all.c:75-92) */
extern char *filename;
extern uint32_t NB_NODES;
extern uint64_t nb_edges;
extern uint32_t P;
extern uint32_t BFS_ROOT;
extern int load_mode;
extern int createUndir;
extern int isSymmetric;
extern int weighted_graph;
extern int switch_mode;
extern algo_mode mode;
extern struct node *nodes;

/* device handles */
extern eg_ctx *eg_context;
extern eg_graph *eg_g;

/* loader: mmap-free read of the [src][dst] file into HBM, then the device
 * layout builder selected by load_mode (init_all.c:855-888). */
void init(int full);
/* Builds the adjacency layouts an algorithm needs when the load mode did not
 * (the edge-array modes 7, 8, 9 build none). */
void eg_need_adjacency(unsigned layouts);

double eg_now(void);
void eg_die(const char *what);
/* writes n elements of size sz to $EG_DUMP if set (result dump for tests) */
void eg_dump(const void *p, size_t sz, size_t n);

#endif
