"""CPU oracle for the edge-traversal hot path (test infrastructure only).

Thin numpy wrappers over ``oracle/_build/libeg_oracle.so`` (``eg_oracle.c``),
which restates the reference algorithms in plain C.  Only the tests, the smoke
check and the benchmark's CPU-baseline leg import this module; the product
library never does.

``build()`` compiles the C file with the committed Makefile.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libeg_oracle.so")
_lib = None

UNREACHED_SSSP = 0xFFFFFFFE


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.or_sample_roots.restype = ctypes.c_int
        _lib.or_partition_id.restype = ctypes.c_uint32
        _lib.or_default_p.restype = ctypes.c_uint32
        _lib.or_ppr_f64.restype = ctypes.c_int
        _lib.or_bfs_tree_check.restype = ctypes.c_int
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


u32, u64, i32, i64, f32, f64 = (ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32,
                                ctypes.c_int64, ctypes.c_float, ctypes.c_double)


def set_threads(t):
    lib().or_set_threads(ctypes.c_int(int(t)))


def num_threads():
    return lib().or_num_threads()


# ---------------------------------------------------------------- generators
def rmat_edges(scale, m, seed):
    pairs = np.empty(2 * m, dtype=np.uint32)
    lib().or_rmat_edges(ctypes.c_int(scale), u64(m), u64(seed), _p(pairs))
    return pairs


def er_edges(n, m, seed):
    pairs = np.empty(2 * m, dtype=np.uint32)
    lib().or_er_edges(u32(n), u64(m), u64(seed), _p(pairs))
    return pairs


def uniform_f32(count, seed):
    out = np.empty(count, dtype=np.float32)
    lib().or_uniform_f32(u64(count), u64(seed), _p(out))
    return out


def uniform_u32(count, seed, lo, hi):
    out = np.empty(count, dtype=np.uint32)
    lib().or_uniform_u32(u64(count), u64(seed), u32(lo), u32(hi), _p(out))
    return out


def sample_roots(deg, k, seed):
    deg = np.ascontiguousarray(deg, dtype=np.uint32)
    roots = np.empty(k, dtype=np.uint32)
    rc = lib().or_sample_roots(u32(len(deg)), _p(deg), ctypes.c_int(k), u64(seed), _p(roots))
    if rc != 0:
        raise ValueError("no vertex with positive degree")
    return roots


# ---------------------------------------------------------------- layouts
class Adj:
    """CSR (out-lists) and CSC (in-lists) with the reference's entry order."""

    def __init__(self, n, out_ptr, out_col, out_eid, in_ptr, in_col, in_eid):
        self.n = n
        self.out_ptr, self.out_col, self.out_eid = out_ptr, out_col, out_eid
        self.in_ptr, self.in_col, self.in_eid = in_ptr, in_col, in_eid

    @property
    def m(self):
        return int(self.out_ptr[-1])

    def out_deg(self):
        return np.diff(self.out_ptr.astype(np.int64)).astype(np.uint32)

    def in_deg(self):
        return np.diff(self.in_ptr.astype(np.int64)).astype(np.uint32)

    def out_src(self):
        return np.repeat(np.arange(self.n, dtype=np.uint32), self.out_deg())

    def in_dst(self):
        return np.repeat(np.arange(self.n, dtype=np.uint32), self.in_deg())


def build_csr(n, pairs, undirected=False):
    """The CSR (out-lists) of build_adj alone: (ptr, col), without the CSC and
    the entry ids (for graphs of 10^8-10^9 entries)."""
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1)
    m = len(pairs) // 2
    M = 2 * m if undirected else m
    ptr = np.empty(n + 1, dtype=np.uint32)
    col = np.empty(M, dtype=np.uint32)
    rc = lib().or_build_adj(u32(n), u64(m), _p(pairs), ctypes.c_int(int(undirected)), _p(ptr), _p(col),
                            None, None, None, None)
    if rc != 0:
        raise ValueError("edge endpoint out of range" if rc == -1 else "allocation failed")
    return ptr, col


def build_adj(n, pairs, undirected=False):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    m = len(pairs) // 2
    M = 2 * m if undirected else m
    out_ptr = np.empty(n + 1, dtype=np.uint32)
    in_ptr = np.empty(n + 1, dtype=np.uint32)
    out_col = np.empty(M, dtype=np.uint32)
    in_col = np.empty(M, dtype=np.uint32)
    out_eid = np.empty(M, dtype=np.uint64)
    in_eid = np.empty(M, dtype=np.uint64)
    rc = lib().or_build_adj(u32(n), u64(m), _p(pairs), ctypes.c_int(int(undirected)),
                            _p(out_ptr), _p(out_col), _p(out_eid), _p(in_ptr), _p(in_col), _p(in_eid))
    if rc != 0:
        raise ValueError("edge endpoint out of range" if rc == -1 else "allocation failed")
    return Adj(n, out_ptr, out_col, out_eid, in_ptr, in_col, in_eid)


def default_p(n):
    return lib().or_default_p(u32(n))


def partition_id(v, n, P):
    return lib().or_partition_id(u32(v), u32(n), u32(P))


def build_grid(n, pairs, P):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    m = len(pairs) // 2
    cell_ptr = np.empty(P * P + 1, dtype=np.uint32)
    gsrc = np.empty(m, dtype=np.uint32)
    gdst = np.empty(m, dtype=np.uint32)
    rc = lib().or_build_grid(u32(n), u64(m), _p(pairs), u32(P), _p(cell_ptr), _p(gsrc), _p(gdst))
    if rc != 0:
        raise ValueError("edge endpoint out of range")
    return cell_ptr, gsrc, gdst


def degrees(n, pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    od = np.empty(n, dtype=np.uint32)
    idg = np.empty(n, dtype=np.uint32)
    lib().or_degrees(u32(n), u64(len(pairs) // 2), _p(pairs), _p(od), _p(idg))
    return od, idg


# ---------------------------------------------------------------- algorithms
def pagerank_f32(adj, deg, prev_init, iters, swap):
    deg = np.ascontiguousarray(deg, dtype=np.uint32)
    out = np.empty(adj.n, dtype=np.float32)
    lib().or_pagerank_f32(u32(adj.n), _p(adj.in_ptr), _p(adj.in_col), _p(deg), f32(prev_init),
                          ctypes.c_int(iters), ctypes.c_int(int(swap)), _p(out))
    return out


def pagerank_grid_f32(n, P, cell_ptr, gsrc, gdst, deg, prev_init, iters):
    deg = np.ascontiguousarray(deg, dtype=np.uint32)
    out = np.empty(n, dtype=np.float32)
    lib().or_pagerank_grid_f32(u32(n), u32(P), _p(cell_ptr), _p(gsrc), _p(gdst), _p(deg),
                               f32(prev_init), ctypes.c_int(iters), _p(out))
    return out


def pagerank_f64(adj, deg, prev_init, iters, dangling=False, damping=0.85):
    deg = np.ascontiguousarray(deg, dtype=np.uint32)
    out = np.empty(adj.n, dtype=np.float64)
    lib().or_pagerank_f64(u32(adj.n), _p(adj.in_ptr), _p(adj.in_col), _p(deg), f64(prev_init),
                          ctypes.c_int(iters), ctypes.c_int(int(dangling)), f64(damping), _p(out))
    return out


def ppr_f64(adj, deg, seeds, damping=0.85, tol=1e-10, max_iters=50):
    deg = np.ascontiguousarray(deg, dtype=np.uint32)
    seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
    out = np.empty(adj.n, dtype=np.float64)
    it = lib().or_ppr_f64(u32(adj.n), _p(adj.in_ptr), _p(adj.in_col), _p(deg), _p(seeds),
                          ctypes.c_int(len(seeds)), f64(damping), f64(tol), ctypes.c_int(max_iters), _p(out))
    return out, it


SPMV_PULL, SPMV_PUSH, SPMV_EDGE = 0, 1, 2


def spmv_f64_hashed(n, ptr, col, value_seed, x):
    """fp64 SpMV with the edge values of hash_values(col, row, value_seed),
    computed per entry (no value array)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(n, dtype=np.float64)
    lib().or_spmv_f64_hval(u32(n), _p(ptr), _p(col), u64(value_seed), _p(x), _p(y))
    return y


def spmv_u32(n, ptr, col, x, mode):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    y = np.empty(n, dtype=np.uint32)
    lib().or_spmv_u32(u32(n), _p(ptr), _p(col), _p(x), ctypes.c_int(mode), _p(y))
    return y


def spmv_f64(n, ptr, col, vals, x):
    vals = np.ascontiguousarray(vals, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(n, dtype=np.float64)
    lib().or_spmv_f64(u32(n), _p(ptr), _p(col), _p(vals), _p(x), _p(y))
    return y


def bfs_levels(n, ptr, col, root, parents=False):
    level = np.empty(n, dtype=np.int32)
    parent = np.empty(n, dtype=np.int32) if parents else None
    rc = lib().or_bfs_levels(u32(n), _p(ptr), _p(col), u32(root), _p(level), _p(parent))
    if rc != 0:
        raise ValueError("root out of range")
    return (level, parent) if parents else level


def sssp(n, ptr, col, w, root):
    w = np.ascontiguousarray(w, dtype=np.uint32)
    dist = np.empty(n, dtype=np.uint32)
    rc = lib().or_sssp(u32(n), _p(ptr), _p(col), _p(w), u32(root), _p(dist))
    if rc != 0:
        raise ValueError("root out of range")
    return dist


def sssp_f32(n, ptr, col, w, root):
    """fp32-weight SSSP; returns the fp32 distances (unreached = +inf)."""
    w = np.ascontiguousarray(w, dtype=np.float32)
    dist = np.empty(n, dtype=np.uint32)
    rc = lib().or_sssp_f32(u32(n), _p(ptr), _p(col), _p(w), u32(root), _p(dist))
    if rc != 0:
        raise ValueError("root out of range")
    return dist.view(np.float32)


def wcc(n, pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    labels = np.empty(n, dtype=np.int64)
    rc = lib().or_wcc(u32(n), u64(len(pairs) // 2), _p(pairs), _p(labels))
    if rc != 0:
        raise ValueError("edge endpoint out of range")
    return labels


def ref_weights(adj, which="out"):
    """The reference's CREATE_WEIGHT rule src%10 + dst%10 (init_all.c:661-686,
    734-757) for every CSR (which='out') or CSC (which='in') entry."""
    if which == "out":
        s, d = adj.out_src(), adj.out_col
    else:
        s, d = adj.in_col, adj.in_dst()
    return (s % 10 + d % 10).astype(np.uint32)


def bfs_tree_check(n, out_ptr, out_col, root, level, parent):
    """0 when `parent` is a BFS tree for `level` (root = 1 convention) over the
    CSR out-lists: the root is its own parent, unreached vertices have parent
    -1, every other reached vertex has a parent one level up with an edge
    parent -> v.  Else the negative code of the first rule that failed
    (-1 root, -2 unreached, -3 level, -4 edge)."""
    out_ptr = np.ascontiguousarray(out_ptr, dtype=np.uint32)
    out_col = np.ascontiguousarray(out_col, dtype=np.uint32)
    level = np.ascontiguousarray(level, dtype=np.int32)
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    if len(level) != n or len(parent) != n:
        raise ValueError("level and parent need n entries")
    return lib().or_bfs_tree_check(u32(n), _p(out_ptr), _p(out_col), u32(root), _p(level), _p(parent))


def bfs_tree_ok(n, out_ptr, out_col, root, level, parent):
    """True when `parent` is a BFS tree for `level` (see bfs_tree_check)."""
    return bfs_tree_check(n, out_ptr, out_col, root, level, parent) == 0


def hash_weights(u, v, seed, lo, hi):
    """u32 weights in [lo, hi] hashed from each (u, v) endpoint pair."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    out = np.empty(len(u), dtype=np.uint32)
    lib().or_hash_weights(u64(len(u)), _p(u), _p(v), u64(seed), u32(lo), u32(hi), _p(out))
    return out


def hash_weights_f32(u, v, seed):
    """fp32 weights in (0, 1] hashed from each (u, v) endpoint pair."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    out = np.empty(len(u), dtype=np.float32)
    lib().or_hash_weights_f32(u64(len(u)), _p(u), _p(v), u64(seed), _p(out))
    return out


def hash_values(u, v, seed):
    """fp32 values in [0, 1) hashed from each (u, v) endpoint pair."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    out = np.empty(len(u), dtype=np.float32)
    lib().or_hash_values(u64(len(u)), _p(u), _p(v), u64(seed), _p(out))
    return out


def bfs_do(adj_out_ptr, adj_out_col, adj_in_ptr, adj_in_col, root):
    """Multi-threaded direction-optimising BFS (levels, root = 1)."""
    n = len(adj_out_ptr) - 1
    level = np.empty(n, dtype=np.int32)
    rc = lib().or_bfs_do(u32(n), _p(adj_out_ptr), _p(adj_out_col), _p(adj_in_ptr), _p(adj_in_col), u32(root),
                         _p(level))
    if rc != 0:
        raise ValueError("root out of range")
    return level


def wcc_lp(out_ptr, out_col):
    """Multi-threaded min-label propagation (wcc.c adjacency mode)."""
    n = len(out_ptr) - 1
    comp = np.empty(n, dtype=np.int64)
    rounds = lib().or_wcc_lp(u32(n), _p(out_ptr), _p(out_col), _p(comp))
    return comp, rounds
