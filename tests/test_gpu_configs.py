"""GPU results at the benchmark configurations' own sizes, against the CPU
oracle (which the golden tests pin to the reference's dumps).

* undirected RMAT-24 (seed 2): CSR bit-exact, BFS levels bit-exact and
  parents a valid BFS tree for sampled roots (seed 3) through eg_bfs,
  eg_bfs_batch and the bit-sliced eg_bfs_multi; WCC labels bit-exact;
* directed RMAT-23 (seed 5): SSSP distances with u32 weights in [1, 255]
  (seed 6) bit-exact for sampled sources through eg_sssp and one 256-source
  eg_sssp_multi batch; fp32 weights bit-exact too;
* directed RMAT-20 (seed 1): 10 PageRank iterations from 1/n within relative
  L1 1e-6 and max relative 1e-5 of FP64; the reference's pull quirk
  (prev = 0.15, never swapped) within the same bounds of FP64 and within
  2e-5 (plus the serial sum's own error) of the fp32 restatement;
* directed RMAT-24 (seed 1): the headline PageRank within the same FP64
  bounds;
* Erdos-Renyi 2^25 x 32 (seed 4): fp32 and fp32 two-sum SpMV with hashed
  values within the FP64 bounds, and the 64 x 64 grid kernels.

The oracle runs several roots at once in threads (its C calls release the
interpreter lock).
"""
import threading

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL_L1 = 1e-6
MAX_REL = 1e-5
VS_REF32_MAX_REL = 2e-5
GRID_MAX_REL = 5e-5
INF = oracle.UNREACHED_SSSP


class _Csc:
    """The in-lists the FP64 PageRank oracle reads (n, in_ptr, in_col)."""

    def __init__(self, n, ptr, col):
        self.n, self.in_ptr, self.in_col = n, ptr, col


def parallel(fn, args):
    out = [None] * len(args)

    def run(i):
        out[i] = fn(*args[i])

    ts = [threading.Thread(target=run, args=(i,)) for i in range(len(args))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out


def rel_errors(got, ref):
    got = got.astype(np.float64)
    ref = ref.astype(np.float64)
    d = np.abs(got - ref)
    nz = ref != 0
    return d.sum() / np.abs(ref).sum(), (d[nz] / np.abs(ref[nz])).max(), nz


@pytest.fixture(scope="module")
def ctx():
    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import build
    build.build_lib()
    oracle.build()
    c = eg.Context(0)
    yield c
    c.close()


def test_rmat24_undirected_bfs_wcc_bit_exact(ctx):
    import everythinggraph_gb300 as eg
    scale, n = 24, 1 << 24
    pairs = oracle.rmat_edges(scale, 16 * n, 2)
    ptr, col = oracle.build_csr(n, pairs, undirected=True)
    g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
    gptr, gcol = g.adj(eg.CSR)
    np.testing.assert_array_equal(gptr, ptr)
    assert np.array_equal(gcol, col)  # file order inside every list
    del gptr, gcol
    roots = g.sample_roots(64, 3)
    np.testing.assert_array_equal(roots, oracle.sample_roots(np.diff(ptr.astype(np.int64)).astype(np.uint32), 64, 3))
    check = [int(r) for r in roots[[0, 1, 2, 3, 31, 63]]]
    ref = parallel(lambda r: oracle.bfs_levels(n, ptr, col, r), [(r,) for r in check])
    for r, lr in zip(check, ref):
        lv, par, st = g.bfs(r, parents=True)
        np.testing.assert_array_equal(lv, lr)
        assert oracle.bfs_tree_check(n, ptr, col, r, lv, par) == 0, r
        assert st.reached == int((lr > 0).sum())
    # the end-to-end batch call (output copies overlapped with the traversals)
    lvb, parb, sts = g.bfs_batch(check[:4], parents=True)
    for i, r in enumerate(check[:4]):
        np.testing.assert_array_equal(lvb[i], ref[i])
        assert oracle.bfs_tree_check(n, ptr, col, r, lvb[i], parb[i]) == 0, r
    del lvb, parb
    # all 64 roots bit-sliced in one batch
    lvm, _ = g.bfs_multi(roots)
    for i, r in enumerate(check):
        np.testing.assert_array_equal(lvm[list(roots).index(r)], ref[i])
    del lvm
    lab, st = g.wcc()
    np.testing.assert_array_equal(lab, oracle.wcc(n, pairs))
    g.free()


def test_rmat23_sssp_bit_exact(ctx):
    import everythinggraph_gb300 as eg
    scale, n = 23, 1 << 23
    pairs = oracle.rmat_edges(scale, 16 * n, 5)
    ptr, col = oracle.build_csr(n, pairs)
    del pairs
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(ptr.astype(np.int64)))
    wh = oracle.hash_weights(src, col, 6, 1, 255)
    g = ctx.rmat(scale, 16 * n, 5).build(eg.CSR)
    roots = g.sample_roots(256, 6)
    check = [int(r) for r in roots[[0, 1, 2, 3, 128, 255]]]
    ref = parallel(lambda r: oracle.sssp(n, ptr, col, wh, r), [(r,) for r in check])
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    for r, dr in zip(check[:3], ref):
        d, st = g.sssp(r, w)
        np.testing.assert_array_equal(d, dr)
        assert st.reached == int((dr != INF).sum())
    D, st = g.sssp_multi(roots, w)  # one 256-source batch
    idx = {int(r): i for i, r in enumerate(roots)}
    for r, dr in zip(check, ref):
        np.testing.assert_array_equal(D[idx[r]], dr)
    del D
    # fp32 weights in (0, 1]: fp32 path sums, also exact
    wf = oracle.hash_weights_f32(src, col, 6)
    reff = parallel(lambda r: oracle.sssp_f32(n, ptr, col, wf, r), [(r,) for r in check[:2]])
    Df, _ = g.sssp_multi(roots[:64], eg.weights("f32", seed=6))
    for r, dr in zip(check[:2], reff):
        np.testing.assert_array_equal(Df[idx[r]].view(np.uint32), dr.view(np.uint32))
    g.free()


def test_rmat20_pagerank_config(ctx):
    import everythinggraph_gb300 as eg
    scale, n = 20, 1 << 20
    pairs = oracle.rmat_edges(scale, 16 * n, 1)
    adj = oracle.build_adj(n, pairs)
    g = ctx.rmat(scale, 16 * n, 1).build(eg.CSR | eg.CSC)
    g.tune()
    ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10)
    rank, st = g.pagerank(iterations=10)
    l1, mx, _ = rel_errors(rank, ref)
    assert l1 <= REL_L1 and mx <= MAX_REL, (l1, mx)
    # the reference's pull mode: prev = 0.15, never swapped (one effective
    # step).  Against FP64 within the bounds above; against the reference's
    # serial fp32 row sums within 2e-5 plus that serial sum's own error (a
    # hub row of 10^5 terms summed serially in fp32 is off FP64 by more
    # than 2e-5 itself)
    r64 = oracle.pagerank_f64(adj, adj.out_deg(), 0.15, 1)
    r32 = oracle.pagerank_f32(adj, adj.out_deg(), 0.15, 10, swap=False)
    got, _ = g.pagerank(iterations=10, prev_init=0.15, swap=False)
    l1, mx, _ = rel_errors(got, r64)
    assert l1 <= REL_L1 and mx <= MAX_REL, ("quirk vs fp64", l1, mx)
    own = np.abs(r32.astype(np.float64) - r64)
    assert np.all(np.abs(got.astype(np.float64) - r32) <= own + VS_REF32_MAX_REL * np.abs(r64))
    g.free()


def test_rmat24_pagerank_headline(ctx):
    import everythinggraph_gb300 as eg
    scale, n = 24, 1 << 24
    pairs = oracle.rmat_edges(scale, 16 * n, 1)
    out_deg, _ = oracle.degrees(n, pairs)
    # in-lists: the CSR of the reversed edges (list order does not matter in FP64)
    iptr, icol = oracle.build_csr(n, np.ascontiguousarray(pairs.reshape(-1, 2)[:, ::-1]).reshape(-1))
    del pairs
    ref = oracle.pagerank_f64(_Csc(n, iptr, icol), out_deg, 1.0 / n, 10)
    g = ctx.rmat(scale, 16 * n, 1).build(eg.CSR | eg.CSC)
    g.tune()
    rank, st = g.pagerank(iterations=10)
    l1, mx, _ = rel_errors(rank, ref)
    assert l1 <= REL_L1 and mx <= MAX_REL, (l1, mx)
    rank_g, _ = g.pagerank(iterations=10, use_graph=True)  # graph replay: the same bits
    np.testing.assert_array_equal(rank_g.view(np.uint32), rank.view(np.uint32))
    g.free()


def test_er25_spmv_vs_fp64(ctx):
    import everythinggraph_gb300 as eg
    log_n, n = 25, 1 << 25
    g = ctx.er(n, 32 * n, 4).build(eg.CSR | eg.CSC)
    x = oracle.uniform_f32(n, 11)
    ptr, col = g.adj(eg.CSC)
    ref = oracle.spmv_f64_hashed(n, ptr, col, 9, x)
    del ptr, col
    for kind in ("f32", "f32_comp"):
        y, _ = g.spmv(x, kind, value_seed=9)
        l1, mx, nz = rel_errors(y, ref)
        assert l1 <= REL_L1 and mx <= MAX_REL, (kind, l1, mx)
        assert np.all(y[~nz] == 0)
    g.build_grid(64)
    y, _ = g.spmv(x, "f32", value_seed=9, grid=True)
    l1, mx, _ = rel_errors(y, ref)
    assert l1 <= REL_L1 and mx <= GRID_MAX_REL, ("grid", l1, mx)
    g.free()
