/* Minimal stand-in for <cilk/cilk_api.h>, mapped onto OpenMP. */
#ifndef EG_SHIM_CILK_API_H
#define EG_SHIM_CILK_API_H
#include <omp.h>
#include <stdlib.h>
static inline int __cilkrts_get_worker_number(void) { return omp_get_thread_num(); }
static inline int __cilkrts_get_nworkers(void) { return omp_get_max_threads(); }
static inline void __cilkrts_end_cilk(void) {}
static inline int __cilkrts_set_param(const char *name, const char *value) {
    (void)name;
    omp_set_num_threads(atoi(value));
    return 0;
}
#endif
