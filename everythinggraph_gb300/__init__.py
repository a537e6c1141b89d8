"""EverythingGraph edge-traversal hot path on GB300 (sm_103a).

Python view of the C ABI in include/eg_gpu.h (libeg_gpu.so).  The C ABI is
the product boundary; this module is a thin convenience layer used by the
tests and the benchmark.  Every call runs CUDA kernels; there is no CPU path.

    ctx = Context()
    g = ctx.rmat(scale=20, m=16 << 20, seed=1)      # or ctx.from_pairs / from_file
    g.build(CSR | CSC)
    rank, st = g.pagerank(iterations=10)
"""
import ctypes
import weakref

import numpy as np

from . import _lib as L
from ._lib import EGError  # noqa: F401

CSR, CSC, GRID, EDGES = L.EG_LAYOUT_CSR, L.EG_LAYOUT_CSC, L.EG_LAYOUT_GRID, L.EG_LAYOUT_EDGES
EDGE_ORDERS = {"file": L.EG_EDGES_FILE_ORDER, "src": L.EG_EDGES_BY_SRC, "src_dst": L.EG_EDGES_BY_SRC_DST}
UNDIRECTED = L.EG_UNDIRECTED
UNREACHED_SSSP = 0xFFFFFFFE

SPMV_KINDS = {"u32_pull": L.EG_SPMV_U32_PULL, "u32_push": L.EG_SPMV_U32_PUSH, "u32_edge": L.EG_SPMV_U32_EDGE,
              "f32": L.EG_SPMV_F32, "f32_comp": L.EG_SPMV_F32_COMP, "f64": L.EG_SPMV_F64}


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def lib():
    return L.load()


class _PinnedOwner:
    """Frees one eg_host_alloc block when the last array over it goes."""

    def __init__(self, p):
        self.p = p

    def __del__(self):
        try:
            lib().eg_host_free(ctypes.c_void_p(self.p))
        except Exception:
            pass


def pinned_empty(shape, dtype):
    """Uninitialised numpy array in page-locked host memory (eg_host_alloc):
    the *_out copies of the graph calls land in it at the full host-link rate.
    Reuse it across calls; it is freed with the last array that views it."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    nbytes = max(count * dt.itemsize, 1)
    p = ctypes.c_void_p()
    L.check(lib().eg_host_alloc(nbytes, ctypes.byref(p)))
    buf = (ctypes.c_char * nbytes).from_address(p.value)
    buf._eg_owner = _PinnedOwner(p.value)
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


def _out(a, n, dtype, name):
    """A caller-supplied output array: n elements of dtype, C-contiguous."""
    if a.dtype != np.dtype(dtype) or a.size != n or not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
        raise ValueError("%s must be a writeable C-contiguous %s array of %d elements" % (name, np.dtype(dtype), n))
    return a


def _grid_mode(grid):
    """grid option: False (0), True (1: the fixed-order row kernel in the
    grid's order when the adjacency is built) or "cells" (2: the cell kernel
    with atomic adds)."""
    return 2 if grid == "cells" else int(bool(grid))


def weights(rule="ref", seed=0, lo=1, hi=255):
    """SSSP weight rule: "ref" (src%10+dst%10), "hash" (u32 in [lo, hi]),
    "unit", or "f32" (fp32 in (0, 1]; distances come back as float32)."""
    r = {"ref": L.EG_W_REF, "hash": L.EG_W_HASH, "unit": L.EG_W_UNIT, "f32": L.EG_W_HASH_F32}[rule]
    return L.Weights(r, seed, lo, hi)


class Context:
    """One device, one stream (eg_open)."""

    def __init__(self, device=0, hbm_budget=0):
        self._h = ctypes.c_void_p()
        self._children = weakref.WeakSet()  # graphs and servers, freed before the context
        L.check(lib().eg_open(device, hbm_budget, ctypes.byref(self._h)))

    def _adopt(self, obj):
        self._children.add(obj)
        return obj

    def close(self):
        if self._h:
            kids = list(self._children)
            for k in kids:
                if isinstance(k, Server):
                    k.close()
            for k in kids:
                if isinstance(k, Graph):
                    k.free()
            L.check(lib().eg_close(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return lib().eg_stream(self._h)

    def sync(self):
        L.check(lib().eg_sync(self._h))

    @property
    def bytes_in_use(self):
        return lib().eg_bytes_in_use(self._h)

    @property
    def kernel_launches(self):
        return lib().eg_kernel_launches(self._h)

    def from_pairs(self, n, pairs, undirected=False):
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
        h = ctypes.c_void_p()
        L.check(lib().eg_graph_from_pairs(self._h, _ptr(pairs), len(pairs) // 2, n,
                                          UNDIRECTED if undirected else 0, ctypes.byref(h)))
        return Graph(self, h)

    def from_device_pairs(self, n, dptr, m, undirected=False):
        h = ctypes.c_void_p()
        L.check(lib().eg_graph_from_device_pairs(self._h, ctypes.c_void_p(dptr), m, n,
                                                 UNDIRECTED if undirected else 0, ctypes.byref(h)))
        return Graph(self, h)

    def from_file(self, path, n, undirected=False, weighted=False):
        """Binary [src][dst] u32 records, or 12-byte [src][dst][f32 weight]
        records with weighted=True (-w; the weights are skipped)."""
        h = ctypes.c_void_p()
        flags = (UNDIRECTED if undirected else 0) | (L.EG_WEIGHTED_FILE if weighted else 0)
        L.check(lib().eg_graph_from_file(self._h, path.encode(), n, flags, ctypes.byref(h)))
        return Graph(self, h)

    def rmat(self, scale, m, seed, undirected=False):
        h = ctypes.c_void_p()
        L.check(lib().eg_graph_generate_rmat(self._h, scale, m, seed, UNDIRECTED if undirected else 0,
                                             ctypes.byref(h)))
        return Graph(self, h)

    def er(self, n, m, seed, undirected=False):
        h = ctypes.c_void_p()
        L.check(lib().eg_graph_generate_er(self._h, n, m, seed, UNDIRECTED if undirected else 0, ctypes.byref(h)))
        return Graph(self, h)


class Graph:
    def __init__(self, ctx, h):
        self.ctx = ctx
        self._h = h
        ctx._adopt(self)

    def free(self):
        if self._h:
            lib().eg_graph_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # ---------------------------------------------------------------- layout
    def build(self, layouts=CSR | CSC):
        L.check(lib().eg_graph_build(self._h, layouts))
        return self

    def build_grid(self, P):
        L.check(lib().eg_graph_build_grid(self._h, P))
        return self

    def build_edges(self, order="src"):
        """The edge array of load modes 9 ("file": input order), 7 ("src":
        stable by source) or 8 ("src_dst": by source, then destination),
        without any CSR or CSC."""
        L.check(lib().eg_graph_build_edges(self._h, EDGE_ORDERS[order]))
        return self

    def save_layouts(self, path):
        """Writes the built layouts to an on-disk cache file (eg_graph_save_layouts)."""
        L.check(lib().eg_graph_save_layouts(self._h, path.encode()))

    def load_layouts(self, path):
        """Fills the layouts from a cache file written for the same input;
        True on a hit, False when the file is absent or for another input."""
        hit = ctypes.c_int()
        L.check(lib().eg_graph_load_layouts(self._h, path.encode(), ctypes.byref(hit)))
        return bool(hit.value)

    def edges(self):
        """(src, dst) of the edge array, m entries each."""
        m = self.m
        s = np.empty(m, dtype=np.uint32)
        d = np.empty(m, dtype=np.uint32)
        L.check(lib().eg_graph_copy_edges(self._h, _ptr(s), _ptr(d)))
        return s, d

    def edges_bfs(self, root, parents=False, copy_out=True):
        n = self.n
        lv = np.empty(n, dtype=np.int32) if copy_out else None
        par = np.empty(n, dtype=np.int32) if (copy_out and parents) else None
        st = L.BfsStats()
        L.check(lib().eg_edges_bfs(self._h, root, _ptr(lv), _ptr(par), ctypes.byref(st)))
        return (lv, par, st) if parents else (lv, st)

    def edges_pagerank(self, iterations=10, damping=0.85, prev_init=-1.0, swap=True, deg_multiplier=1,
                       dangling=False, tolerance=0.0, copy_out=True):
        o = L.PrOpts()
        lib().eg_pr_opts_default(ctypes.byref(o))
        o.iterations, o.damping, o.prev_init, o.swap = iterations, damping, prev_init, int(swap)
        o.deg_multiplier, o.dangling, o.tolerance = deg_multiplier, int(dangling), tolerance
        st = L.PrStats()
        out = np.empty(self.n, dtype=np.float32) if copy_out else None
        L.check(lib().eg_edges_pagerank(self._h, ctypes.byref(o), _ptr(out), ctypes.byref(st)))
        return out, st

    def edges_spmv(self, x, copy_out=True):
        x = np.ascontiguousarray(x, dtype=np.uint32)
        y = np.empty(self.n, dtype=np.uint32) if copy_out else None
        ms = ctypes.c_float()
        L.check(lib().eg_edges_spmv_u32(self._h, _ptr(x), _ptr(y), ctypes.byref(ms)))
        return y, ms.value

    def info(self):
        i = L.GraphInfo()
        L.check(lib().eg_graph_get_info(self._h, ctypes.byref(i)))
        return i

    @property
    def n(self):
        return self.info().n

    @property
    def m(self):
        return self.info().m

    def adj(self, layout):
        i = self.info()
        ptr = np.empty(i.n + 1, dtype=np.uint32)
        col = np.empty(i.m, dtype=np.uint32)
        L.check(lib().eg_graph_copy_adj(self._h, layout, _ptr(ptr), _ptr(col)))
        return ptr, col

    def grid(self):
        i = self.info()
        cp = np.empty(i.grid_p * i.grid_p + 1, dtype=np.uint32)
        s = np.empty(i.m, dtype=np.uint32)
        d = np.empty(i.m, dtype=np.uint32)
        L.check(lib().eg_graph_copy_grid(self._h, _ptr(cp), _ptr(s), _ptr(d)))
        return cp, s, d

    def degrees(self, out=True, inn=False):
        n = self.n
        od = np.empty(n, dtype=np.uint32) if out else None
        idg = np.empty(n, dtype=np.uint32) if inn else None
        L.check(lib().eg_graph_copy_degrees(self._h, _ptr(od), _ptr(idg)))
        return od, idg

    def device_ptr(self, which):
        return lib().eg_graph_device_ptr(self._h, which)

    def tune(self):
        """Times the row-kernel schedules on this graph and keeps the fastest;
        returns [{tile, per_lane, prefetch, min_blocks, cache_hint, ms}] and
        the chosen index."""
        r = L.TuneResult()
        L.check(lib().eg_graph_tune(self._h, ctypes.byref(r)))
        cands = [{"tile": r.tile_entries[i], "per_lane": r.entries_per_lane[i], "prefetch": r.prefetch[i],
                  "min_blocks": r.min_blocks[i], "cache_hint": r.cache_hint[i],
                  "partition_log2": r.partition_log2[i], "ms": r.ms[i]} for i in range(r.ncand)]
        self.bfs_tuning = {"graph_ms": r.bfs_graph_ms, "host_ms": r.bfs_host_ms, "host_loop": r.bfs_host_loop,
                           "switch_divisor": r.bfs_switch_divisor}
        return cands, r.chosen

    def set_row_schedule(self, index):
        L.check(lib().eg_graph_set_row_schedule(self._h, index))

    def sample_roots(self, k, seed):
        r = np.empty(k, dtype=np.uint32)
        L.check(lib().eg_sample_roots(self._h, k, seed, _ptr(r)))
        return r

    # ---------------------------------------------------------------- algorithms
    def pagerank(self, iterations=10, damping=0.85, prev_init=-1.0, swap=True, deg_multiplier=1, dangling=False,
                 compensated=False, tolerance=0.0, copy_out=True, use_graph=False, grid=False, source_block_log2=0):
        o = L.PrOpts()
        lib().eg_pr_opts_default(ctypes.byref(o))
        o.iterations, o.damping, o.prev_init, o.swap = iterations, damping, prev_init, int(swap)
        o.deg_multiplier, o.dangling, o.compensated, o.tolerance = deg_multiplier, int(dangling), int(compensated), tolerance
        o.use_graph = int(use_graph)
        o.grid = _grid_mode(grid)
        o.source_block_log2 = int(source_block_log2)
        st = L.PrStats()
        out = np.empty(self.n, dtype=np.float32) if copy_out else None
        L.check(lib().eg_pagerank(self._h, ctypes.byref(o), _ptr(out), ctypes.byref(st)))
        return out, st

    def spmv(self, x, kind="u32_pull", value_seed=0, unit_values=False, copy_out=True, grid=False,
             source_block_log2=0):
        """source_block_log2: fp32 over graphs with more vertices than 2^k
        runs one pass per source block of 2^k vertices (0: k = 24)."""
        k = SPMV_KINDS[kind]
        xd = np.uint32 if kind.startswith("u32") else np.float32
        x = np.ascontiguousarray(x, dtype=xd)
        yd = np.float64 if kind == "f64" else xd
        y = np.empty(self.n, dtype=yd) if copy_out else None
        o = L.SpmvOpts(k, value_seed, int(unit_values), _grid_mode(grid), int(source_block_log2))
        ms = ctypes.c_float()
        L.check(lib().eg_spmv(self._h, ctypes.byref(o), _ptr(x), _ptr(y), ctypes.byref(ms)))
        return y, ms.value

    def bfs(self, root, direction="auto", switch_divisor=None, parents=False, copy_out=True, host_loop=None,
            level_out=None, parent_out=None):
        """host_loop: None = the form eg_graph_tune kept (else the CUDA graph),
        False = CUDA-graph level loop, True = host-driven level loop.
        switch_divisor: None = the divisor eg_graph_tune kept (else 40, the
        reference's).
        level_out / parent_out: int32 arrays of n elements to fill (e.g. from
        pinned_empty) instead of new ones."""
        hl = -1 if host_loop is None else int(bool(host_loop))
        o = L.BfsOpts({"auto": L.EG_BFS_AUTO, "push": L.EG_BFS_PUSH_ONLY, "pull": L.EG_BFS_PULL_ONLY}[direction],
                      -1.0 if switch_divisor is None else switch_divisor, int(parents), hl)
        n = self.n
        lv = par = None
        if copy_out:
            lv = _out(level_out, n, np.int32, "level_out") if level_out is not None else np.empty(n, dtype=np.int32)
            if parents:
                par = (_out(parent_out, n, np.int32, "parent_out") if parent_out is not None
                       else np.empty(n, dtype=np.int32))
        st = L.BfsStats()
        L.check(lib().eg_bfs(self._h, root, ctypes.byref(o), _ptr(lv), _ptr(par), ctypes.byref(st)))
        return (lv, par, st) if parents else (lv, st)

    def bfs_batch(self, roots, direction="auto", switch_divisor=None, parents=False, host_loop=None,
                  level_out=None, parent_out=None):
        """eg_bfs from each root in turn with the copies of one root overlapped
        with the next traversal; returns (levels[k, n], parents[k, n] or None,
        [BfsStats] * k).  level_out / parent_out: int32 arrays of k * n
        elements to fill (pinned_empty for full-rate copies)."""
        roots = np.ascontiguousarray(roots, dtype=np.uint32)
        k, n = len(roots), self.n
        hl = -1 if host_loop is None else int(bool(host_loop))
        o = L.BfsOpts({"auto": L.EG_BFS_AUTO, "push": L.EG_BFS_PUSH_ONLY, "pull": L.EG_BFS_PULL_ONLY}[direction],
                      -1.0 if switch_divisor is None else switch_divisor, int(parents), hl)
        lv = (_out(level_out, k * n, np.int32, "level_out") if level_out is not None
              else np.empty(k * n, dtype=np.int32)).reshape(k, n)
        par = None
        if parents:
            par = (_out(parent_out, k * n, np.int32, "parent_out") if parent_out is not None
                   else np.empty(k * n, dtype=np.int32)).reshape(k, n)
        st = (L.BfsStats * max(k, 1))()
        L.check(lib().eg_bfs_batch(self._h, _ptr(roots), k, ctypes.byref(o), _ptr(lv), _ptr(par), st))
        return lv, par, [st[i] for i in range(k)]

    def bfs_multi(self, roots, copy_out=True):
        roots = np.ascontiguousarray(roots, dtype=np.uint32)
        n = self.n
        out = np.empty((len(roots), n), dtype=np.int32) if copy_out else None
        st = L.BfsStats()
        L.check(lib().eg_bfs_multi(self._h, _ptr(roots), len(roots), _ptr(out), ctypes.byref(st)))
        return out, st

    def sssp(self, root, w=None, copy_out=True):
        w = w or weights("ref")
        out = np.empty(self.n, dtype=np.uint32) if copy_out else None
        st = L.SsspStats()
        L.check(lib().eg_sssp(self._h, root, ctypes.byref(w), _ptr(out), ctypes.byref(st)))
        if out is not None and w.rule == L.EG_W_HASH_F32:
            out = out.view(np.float32)
        return out, st

    def sssp_multi(self, roots, w=None, copy_out=True):
        w = w or weights("ref")
        roots = np.ascontiguousarray(roots, dtype=np.uint32)
        out = np.empty((len(roots), self.n), dtype=np.uint32) if copy_out else None
        st = L.SsspStats()
        L.check(lib().eg_sssp_multi(self._h, _ptr(roots), len(roots), ctypes.byref(w), _ptr(out), ctypes.byref(st)))
        if out is not None and w.rule == L.EG_W_HASH_F32:
            out = out.view(np.float32)
        return out, st

    def ppr(self, seed_lists, damping=0.85, tolerance=1e-6, max_iters=50, copy_out=True):
        """Personalised PageRank for up to 32 queries (one seed list each)."""
        nq = len(seed_lists)
        offs = np.zeros(nq + 1, dtype=np.uint32)
        offs[1:] = np.cumsum([len(s) for s in seed_lists])
        seeds = np.ascontiguousarray(np.concatenate([np.asarray(s, dtype=np.uint32) for s in seed_lists]))
        o = L.PprOpts()
        o.damping, o.max_iters = damping, max_iters
        tols = tolerance if isinstance(tolerance, (list, tuple, np.ndarray)) else [tolerance] * nq
        for q in range(32):
            o.tolerance[q] = float(tols[q]) if q < nq else 1.0
        out = np.empty((nq, self.n), dtype=np.float32) if copy_out else None
        st = L.PprStats()
        L.check(lib().eg_ppr_multi(self._h, _ptr(seeds), _ptr(offs), nq, ctypes.byref(o), _ptr(out), ctypes.byref(st)))
        return out, st

    def ppr_single(self, seeds, damping=0.85, tolerance=1e-6, max_iters=50, copy_out=True):
        """One personalised PageRank query on the plain PageRank row kernel."""
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        o = L.PprOpts()
        o.damping, o.max_iters = damping, max_iters
        for q in range(32):
            o.tolerance[q] = tolerance
        out = np.empty(self.n, dtype=np.float32) if copy_out else None
        st = L.PprStats()
        L.check(lib().eg_ppr(self._h, _ptr(seeds), len(seeds), ctypes.byref(o), _ptr(out), ctypes.byref(st)))
        return out, st

    def wcc(self, copy_out=True, out=None):
        if copy_out:
            out = _out(out, self.n, np.int64, "out") if out is not None else np.empty(self.n, dtype=np.int64)
        else:
            out = None
        st = L.WccStats()
        L.check(lib().eg_wcc(self._h, _ptr(out), ctypes.byref(st)))
        return out, st


class Server:
    """Continuous-batching query server over a resident graph (eg_serve_*)."""

    KINDS = {"bfs": L.EG_Q_BFS, "sssp": L.EG_Q_SSSP, "ppr": L.EG_Q_PPR}

    def __init__(self, graph, hbm_budget=64 << 30, weights_=None, keep_results=False, max_bfs=64, max_sssp=64,
                 max_ppr=32, ppr_max_iters=50, exclusive=False, gang=True):
        self.graph = graph
        o = L.ServeOpts()
        lib().eg_serve_opts_default(ctypes.byref(o))
        o.hbm_budget, o.keep_results = hbm_budget, int(keep_results)
        o.max_bfs, o.max_sssp, o.max_ppr, o.ppr_max_iters = max_bfs, max_sssp, max_ppr, ppr_max_iters
        o.exclusive, o.gang = int(exclusive), int(gang)
        if weights_ is not None:
            o.weights = weights_
        self._h = ctypes.c_void_p()
        L.check(lib().eg_serve_open(graph._h, ctypes.byref(o), ctypes.byref(self._h)))
        graph.ctx._adopt(self)

    def close(self):
        if self._h:
            lib().eg_serve_close(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, kind, source=0, seeds=(), tol=1e-6, arrival=0.0):
        q = L.Query()
        q.kind = self.KINDS[kind]
        q.source = source
        q.nseeds = len(seeds)
        for i, s_ in enumerate(seeds):
            q.seeds[i] = int(s_)
        q.tol, q.arrival_s = tol, arrival
        qid = ctypes.c_uint64()
        L.check(lib().eg_serve_submit(self._h, ctypes.byref(q), ctypes.byref(qid)))
        return qid.value

    def step(self):
        a = ctypes.c_int()
        L.check(lib().eg_serve_step(self._h, ctypes.byref(a)))
        return a.value

    def poll(self, max_results=4096):
        buf = (L.QueryResult * max_results)()
        c = ctypes.c_int()
        L.check(lib().eg_serve_poll(self._h, buf, max_results, ctypes.byref(c)))
        return [buf[i] for i in range(c.value)]

    def take_result(self):
        n = self.graph.n
        out = np.empty(n, dtype=np.uint32)
        L.check(lib().eg_serve_take_result(self._h, _ptr(out), n))
        return out

    def stats(self):
        st = L.ServeStats()
        L.check(lib().eg_serve_stats(self._h, ctypes.byref(st)))
        names = ("bfs", "sssp", "ppr")
        return {"ticks": st.ticks, "queued": st.queued,
                "engines": {names[e]: {"device_ms": st.engine_ms[e], "steps": st.engine_steps[e],
                                       "admitted": st.admitted[e], "completed": st.completed[e]} for e in range(3)}}

    def info(self):
        b, s_, p, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        L.check(lib().eg_serve_info(self._h, ctypes.byref(b), ctypes.byref(s_), ctypes.byref(p), ctypes.byref(t)))
        return {"bfs_slots": b.value, "sssp_slots": s_.value, "ppr_slots": p.value, "clock_s": t.value}
