"""The host's poll of a readback flag gives up after a second and falls back
to a stream synchronisation (eg_readback_wait).  The stream is held up on the
host, not on the device: a host function queued on the library's stream
sleeps past the poll's limit, so the first readback of a host-driven BFS
level loop and of an SSSP round loop takes the stream-synchronisation branch.
The results must still be right.  Nothing here waits on the device.
"""
import ctypes
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HOLD_S = 1.4  # longer than the poll's one-second limit


def hold_stream(stream):
    """Queues a host function that sleeps HOLD_S seconds on `stream`
    (cuLaunchHostFunc); returns the callback, which must outlive the wait."""
    cuda = ctypes.CDLL("libcuda.so.1")
    fn_t = ctypes.CFUNCTYPE(None, ctypes.c_void_p)
    cb = fn_t(lambda _: time.sleep(HOLD_S))
    cuda.cuLaunchHostFunc.argtypes = [ctypes.c_void_p, fn_t, ctypes.c_void_p]
    rc = cuda.cuLaunchHostFunc(ctypes.c_void_p(stream), cb, None)
    assert rc == 0, rc
    return cb


def test_readback_wait_falls_back_to_stream_sync():
    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import build
    build.build_lib()
    ctx = eg.Context(0)
    scale = 12
    n = 1 << scale
    pairs = oracle.rmat_edges(scale, 16 * n, 1)
    adj = oracle.build_adj(n, pairs, undirected=True)
    g = ctx.from_pairs(n, pairs, undirected=True).build(eg.CSR | eg.CSC)
    root = int(g.sample_roots(1, 3)[0])
    ref_lv = oracle.bfs_levels(n, adj.out_ptr, adj.out_col, root)
    w = eg.weights("ref")
    ref_d = oracle.sssp(n, adj.out_ptr, adj.out_col, oracle.ref_weights(adj), root)
    # warm: the host loop's launches and buffers exist before the timed calls
    g.bfs(root, host_loop=True)
    g.sssp(root, w)
    ctx.sync()

    cb = hold_stream(ctx.stream)
    t0 = time.perf_counter()
    lv, st = g.bfs(root, host_loop=True)
    dt = time.perf_counter() - t0
    assert dt >= 1.0, dt  # the flag poll ran out; the stream synchronisation waited for the host function
    np.testing.assert_array_equal(lv, ref_lv)

    cb2 = hold_stream(ctx.stream)
    t0 = time.perf_counter()
    d, st = g.sssp(root, w)
    dt = time.perf_counter() - t0
    assert dt >= 1.0, dt
    np.testing.assert_array_equal(d, ref_d)
    ctx.sync()
    del cb, cb2
    g.free()
    ctx.close()
