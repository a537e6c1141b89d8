#!/usr/bin/env bash
# Builds the unmodified reference algorithm binaries, with the result-dump
# harness, into oracle/_ref/ (test infrastructure only; x86-64 or aarch64 host).
# Reads the sources where they lie (default /root/reference, or $EG_REF_SRC);
# nothing is copied.  Cilk and libnuma are replaced by the headers in
# oracle/shim/ (OpenMP dynamic loops).  Exits 0 without building when the
# sources are absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
SRC="${EG_REF_SRC:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$SRC/random.c" ]; then
    echo "reference sources not found at $SRC; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
FLAGS="-O2 -fopenmp -pthread -fms-extensions -w -ffp-contract=off -I$HERE/shim -I$SRC -include $HERE/shim/pre.h"
# algorithm : dump kind
ALGOS="pagerank_simple:PR_RANK prgrid_cilk:PR_PREV bfs_simple:DIST bfsgrid_cilk:DIST sssp_pushpull:DIST wcc:COMP spmv:SPMV"
build_one() {
    local algo="${1%%:*}" kind="${1##*:}"
    local o="$OUT/obj/$algo"
    mkdir -p "$o"
    local hdr="-DALGO_H=\"$algo.h\""
    for f in utils buffer init_all; do
        $CXX $FLAGS "$hdr" -x c++ -c "$SRC/$f.c" -o "$o/$f.o"
    done
    $CXX $FLAGS "$hdr" -x c++ -Dmain=ref_main -c "$SRC/random.c" -o "$o/random.o"
    $CXX $FLAGS "$hdr" -x c++ -c "$SRC/$algo.c" -o "$o/$algo.o"
    $CXX $FLAGS -DEG_DUMP_$kind -c "$HERE/ref_harness.cpp" -o "$o/harness.o"
    $CXX -fopenmp -pthread "$o"/*.o -o "$OUT/$algo" -lm
}
pids=()
for a in $ALGOS; do build_one "$a" & pids+=($!); done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
