"""ctypes binding of libeg_gpu.so (the C ABI declared in include/eg_gpu.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback for any call.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libeg_gpu.so")

c_u32, c_u64, c_i32, c_f32, c_f64, c_int, c_void_p, c_char_p = (
    ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_float, ctypes.c_double, ctypes.c_int,
    ctypes.c_void_p, ctypes.c_char_p)

EG_OK, EG_EINVAL, EG_ECUDA, EG_ENOMEM, EG_EIO, EG_ETIMEOUT, EG_ENOTBUILT, EG_ERANGE = 0, -1, -2, -3, -4, -5, -6, -7
EG_UNDIRECTED = 1
EG_LAYOUT_CSR, EG_LAYOUT_CSC, EG_LAYOUT_GRID, EG_LAYOUT_EDGES = 1, 2, 4, 8
EG_EDGES_FILE_ORDER, EG_EDGES_BY_SRC, EG_EDGES_BY_SRC_DST = 0, 1, 2
EG_DEV_CSR_PTR, EG_DEV_CSR_COL, EG_DEV_CSC_PTR, EG_DEV_CSC_COL, EG_DEV_OUT_DEG = 1, 2, 3, 4, 5
EG_DEV_EDGE_SRC, EG_DEV_EDGE_DST = 6, 7
EG_DEV_RANK, EG_DEV_LEVEL, EG_DEV_PARENT, EG_DEV_DIST, EG_DEV_LABEL, EG_DEV_SPMV_Y = 10, 11, 12, 13, 14, 15
EG_SPMV_U32_PULL, EG_SPMV_U32_PUSH, EG_SPMV_U32_EDGE, EG_SPMV_F32, EG_SPMV_F32_COMP, EG_SPMV_F64 = 0, 1, 2, 3, 4, 5
EG_BFS_AUTO, EG_BFS_PUSH_ONLY, EG_BFS_PULL_ONLY = 0, 1, 2
EG_W_REF, EG_W_HASH, EG_W_UNIT, EG_W_HASH_F32 = 0, 1, 2, 3
EG_WEIGHTED_FILE = 2
EG_Q_BFS, EG_Q_SSSP, EG_Q_PPR = 1, 2, 3


class GraphInfo(ctypes.Structure):
    _fields_ = [("n", c_u32), ("m_input", c_u64), ("m", c_u64), ("layouts", ctypes.c_uint), ("grid_p", c_u32),
                ("device_bytes", c_u64), ("build_ms", c_f32)]


class PrOpts(ctypes.Structure):
    _fields_ = [("iterations", c_int), ("damping", c_f32), ("prev_init", c_f32), ("swap", c_int),
                ("deg_multiplier", c_u32), ("dangling", c_int), ("compensated", c_int), ("tolerance", c_f64),
                ("use_graph", c_int), ("grid", c_int), ("source_block_log2", c_int)]


class PrStats(ctypes.Structure):
    _fields_ = [("iterations_run", c_int), ("residual", c_f64), ("dangling_mass", c_f64), ("ms", c_f32),
                ("row_kernel_ms", c_f32)]


class ServeStats(ctypes.Structure):
    _fields_ = [("ticks", c_u64), ("queued", c_u64), ("engine_ms", c_f64 * 3), ("engine_steps", c_u64 * 3),
                ("admitted", c_u64 * 3), ("completed", c_u64 * 3)]


class TuneResult(ctypes.Structure):
    _fields_ = [("ncand", c_int), ("chosen", c_int), ("tile_entries", c_int * 16), ("entries_per_lane", c_int * 16),
                ("prefetch", c_int * 16), ("min_blocks", c_int * 16), ("cache_hint", c_int * 16), ("ms", c_f32 * 16),
                ("partition_log2", c_int * 16), ("bfs_graph_ms", c_f32),
                ("bfs_host_ms", c_f32), ("bfs_host_loop", c_int), ("bfs_switch_divisor", c_f64)]


class SpmvOpts(ctypes.Structure):
    _fields_ = [("kind", c_int), ("value_seed", c_u64), ("unit_values", c_int), ("grid", c_int),
                ("source_block_log2", c_int)]


class BfsOpts(ctypes.Structure):
    _fields_ = [("direction", c_int), ("switch_divisor", c_f64), ("device_parents", c_int), ("host_loop", c_int)]


class BfsStats(ctypes.Structure):
    _fields_ = [("levels", c_int), ("reached", c_u32), ("edges_traversed", c_u64), ("pull_levels", c_int),
                ("ms", c_f32)]


class Weights(ctypes.Structure):
    _fields_ = [("rule", c_int), ("seed", c_u64), ("lo", c_u32), ("hi", c_u32)]


class SsspStats(ctypes.Structure):
    _fields_ = [("rounds", c_int), ("reached", c_u32), ("relaxations", c_u64), ("ms", c_f32)]


class PprOpts(ctypes.Structure):
    _fields_ = [("damping", c_f32), ("max_iters", c_int), ("tolerance", c_f32 * 32)]


class PprStats(ctypes.Structure):
    _fields_ = [("iterations", c_int * 32), ("residual", c_f64 * 32), ("sweeps", c_int), ("ms", c_f32)]


class Query(ctypes.Structure):
    _fields_ = [("kind", c_int), ("source", c_u32), ("nseeds", c_u32), ("seeds", c_u32 * 8), ("tol", c_f32),
                ("arrival_s", c_f64)]


class QueryResult(ctypes.Structure):
    _fields_ = [("id", c_u64), ("kind", c_int), ("arrival_s", c_f64), ("admit_s", c_f64), ("done_s", c_f64),
                ("reached", c_u32), ("depth", c_u32), ("iterations", c_int), ("value", c_f64)]


class ServeOpts(ctypes.Structure):
    _fields_ = [("hbm_budget", c_u64), ("max_bfs", c_int), ("max_sssp", c_int), ("max_ppr", c_int),
                ("weights", Weights), ("ppr_damping", c_f32), ("ppr_max_iters", c_int), ("keep_results", c_int),
                ("exclusive", c_int), ("gang", c_int)]


class WccStats(ctypes.Structure):
    _fields_ = [("rounds", c_int), ("components", c_u32), ("ms", c_f32)]


P = ctypes.POINTER
# name -> (restype, argtypes)
SIGNATURES = {
    "eg_last_error": (c_char_p, []),
    "eg_version": (c_char_p, []),
    "eg_open": (c_int, [c_int, c_u64, P(c_void_p)]),
    "eg_close": (c_int, [c_void_p]),
    "eg_host_alloc": (c_int, [c_u64, P(c_void_p)]),
    "eg_host_free": (c_int, [c_void_p]),
    "eg_stream": (c_void_p, [c_void_p]),
    "eg_sync": (c_int, [c_void_p]),
    "eg_bytes_in_use": (c_u64, [c_void_p]),
    "eg_kernel_launches": (c_u64, [c_void_p]),
    "eg_graph_from_pairs": (c_int, [c_void_p, c_void_p, c_u64, c_u32, ctypes.c_uint, P(c_void_p)]),
    "eg_graph_from_device_pairs": (c_int, [c_void_p, c_void_p, c_u64, c_u32, ctypes.c_uint, P(c_void_p)]),
    "eg_graph_from_file": (c_int, [c_void_p, c_char_p, c_u32, ctypes.c_uint, P(c_void_p)]),
    "eg_graph_generate_rmat": (c_int, [c_void_p, c_int, c_u64, c_u64, ctypes.c_uint, P(c_void_p)]),
    "eg_graph_generate_er": (c_int, [c_void_p, c_u32, c_u64, c_u64, ctypes.c_uint, P(c_void_p)]),
    "eg_graph_free": (None, [c_void_p]),
    "eg_graph_build": (c_int, [c_void_p, ctypes.c_uint]),
    "eg_graph_build_grid": (c_int, [c_void_p, c_u32]),
    "eg_graph_get_info": (c_int, [c_void_p, P(GraphInfo)]),
    "eg_graph_copy_adj": (c_int, [c_void_p, ctypes.c_uint, c_void_p, c_void_p]),
    "eg_graph_copy_grid": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "eg_graph_copy_degrees": (c_int, [c_void_p, c_void_p, c_void_p]),
    "eg_graph_device_ptr": (c_void_p, [c_void_p, c_int]),
    "eg_pr_opts_default": (None, [P(PrOpts)]),
    "eg_pagerank": (c_int, [c_void_p, P(PrOpts), c_void_p, P(PrStats)]),
    "eg_spmv": (c_int, [c_void_p, P(SpmvOpts), c_void_p, c_void_p, P(c_f32)]),
    "eg_bfs_opts_default": (None, [P(BfsOpts)]),
    "eg_bfs": (c_int, [c_void_p, c_u32, P(BfsOpts), c_void_p, c_void_p, P(BfsStats)]),
    "eg_bfs_batch": (c_int, [c_void_p, c_void_p, c_u32, P(BfsOpts), c_void_p, c_void_p, c_void_p]),
    "eg_bfs_multi": (c_int, [c_void_p, c_void_p, c_int, c_void_p, P(BfsStats)]),
    "eg_sssp": (c_int, [c_void_p, c_u32, P(Weights), c_void_p, P(SsspStats)]),
    "eg_sssp_multi": (c_int, [c_void_p, c_void_p, c_int, P(Weights), c_void_p, P(SsspStats)]),
    "eg_wcc": (c_int, [c_void_p, c_void_p, P(WccStats)]),
    "eg_sample_roots": (c_int, [c_void_p, c_int, c_u64, c_void_p]),
    "eg_ppr_multi": (c_int, [c_void_p, c_void_p, c_void_p, c_int, P(PprOpts), c_void_p, P(PprStats)]),
    "eg_graph_tune": (c_int, [c_void_p, P(TuneResult)]),
    "eg_graph_set_row_schedule": (c_int, [c_void_p, c_int]),
    "eg_ppr": (c_int, [c_void_p, c_void_p, c_u32, P(PprOpts), c_void_p, P(PprStats)]),
    "eg_serve_opts_default": (None, [P(ServeOpts)]),
    "eg_serve_stats": (c_int, [c_void_p, P(ServeStats)]),
    "eg_serve_open": (c_int, [c_void_p, P(ServeOpts), P(c_void_p)]),
    "eg_serve_submit": (c_int, [c_void_p, P(Query), P(c_u64)]),
    "eg_serve_step": (c_int, [c_void_p, P(c_int)]),
    "eg_serve_poll": (c_int, [c_void_p, c_void_p, c_int, P(c_int)]),
    "eg_serve_take_result": (c_int, [c_void_p, c_void_p, c_u32]),
    "eg_serve_info": (c_int, [c_void_p, P(c_int), P(c_int), P(c_int), P(c_f64)]),
    "eg_serve_close": (c_int, [c_void_p]),
    "eg_spmv_f32_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_u32, c_u64, c_void_p]),
    "eg_graph_build_edges": (c_int, [c_void_p, c_int]),
    "eg_graph_save_layouts": (c_int, [c_void_p, c_char_p]),
    "eg_graph_load_layouts": (c_int, [c_void_p, c_char_p, c_void_p]),
    "eg_graph_copy_edges": (c_int, [c_void_p, c_void_p, c_void_p]),
    "eg_edges_bfs": (c_int, [c_void_p, c_u32, c_void_p, c_void_p, c_void_p]),
    "eg_edges_pagerank": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "eg_edges_spmv_u32": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
}

_lib = None


def load(path=LIB_PATH):
    """Loads libeg_gpu.so; raises if it is missing (build it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libeg_gpu.so not built (%s); run everythinggraph_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class EGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("eg error %d: %s" % (code, msg))
        self.code = code


def check(rc):
    if rc != EG_OK:
        raise EGError(rc, load().eg_last_error().decode(errors="replace"))
    return rc
