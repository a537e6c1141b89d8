/* Minimal stand-in for <cilk/cilk.h> so the reference sources build with GCC,
 * which dropped Cilk Plus: cilk_for becomes an OpenMP dynamic loop and
 * spawn/sync run inline.  Used only to build the reference for golden dumps. */
#ifndef EG_SHIM_CILK_H
#define EG_SHIM_CILK_H
#include <omp.h>
#define cilk_for _Pragma("omp parallel for schedule(dynamic,1024)") for
#define cilk_spawn
#define cilk_sync
#endif
