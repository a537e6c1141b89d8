/* Minimal stand-in for <numa.h>: one node, plain malloc.  The reference
 * includes it everywhere; only pr_numa/bfs_numa call into it. */
#ifndef EG_SHIM_NUMA_H
#define EG_SHIM_NUMA_H
#include <stdlib.h>
static inline int numa_num_configured_nodes(void) { return 1; }
static inline int numa_node_of_cpu(int cpu) { (void)cpu; return 0; }
static inline void numa_tonode_memory(void *p, size_t s, int n) { (void)p; (void)s; (void)n; }
static inline void *numa_alloc_onnode(size_t s, int n) { (void)n; return malloc(s); }
static inline void numa_free(void *p, size_t s) { (void)s; free(p); }
static inline int numa_available(void) { return 0; }
#endif
