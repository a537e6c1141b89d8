"""The edge-array load modes (7, 8, 9) and the edge-centric algorithms over
them, through the C ABI, against the oracle and the reference's dumps.

Layouts are bit-exact: mode 9 is the input order, mode 7 the stable sort by
source (the CSR's entry order), mode 8 sorted by (source, destination).
BFS levels, WCC labels and the u32 SpMV edge loop are bit-exact; parents form
a BFS tree.  Edge-centric PageRank adds contributions with fp32 atomics in no
fixed order: relative L1 <= 1e-6 and max relative <= 5e-5 against FP64, and
max relative <= 5e-5 against the reference's own prgrid dumps over the edge
array (prgrid_cilk -m 7/8/9, whose atomic adds are not ordered either).
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["tiny", "rmat10", "rmat12", "rmat16"]
ORDERS = ["file", "src", "src_dst"]
REL_L1 = 1e-6
ATOMIC_MAX_REL = 5e-5


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    rec = {k: z[k] for k in z.files}
    n = int(rec["n"])
    pairs = rec["pairs"] if "pairs" in rec else oracle.rmat_edges(int(np.log2(n)), 16 * n, 1)
    return n, pairs, rec


@pytest.fixture(scope="module")
def ctx():
    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import build
    build.build_lib()
    c = eg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module", params=CASES)
def case(request, ctx):
    n, pairs, rec = load(request.param)
    adj = oracle.build_adj(n, pairs)
    yield request.param, n, pairs, rec, adj


def rel(got, ref):
    got = got.astype(np.float64)
    ref = ref.astype(np.float64)
    d = np.abs(got - ref)
    nz = ref != 0
    return d.sum() / max(np.abs(ref).sum(), 1e-300), (d[nz] / np.abs(ref[nz])).max() if nz.any() else 0.0


@pytest.mark.parametrize("order", ORDERS)
def test_edge_array_layout_and_algorithms(ctx, case, order):
    import everythinggraph_gb300 as eg
    name, n, pairs, rec, adj = case
    g = ctx.from_pairs(n, pairs).build_edges(order)
    info = g.info()
    assert info.layouts & eg.EDGES and not info.layouts & (eg.CSR | eg.CSC)  # no adjacency was built
    s, d = g.edges()
    ps, pd = pairs[0::2], pairs[1::2]
    if order == "file":
        np.testing.assert_array_equal(s, ps)
        np.testing.assert_array_equal(d, pd)
    elif order == "src":
        np.testing.assert_array_equal(s, adj.out_src())  # stable: the CSR's order
        np.testing.assert_array_equal(d, adj.out_col)
    else:
        idx = np.lexsort((pd, ps))
        np.testing.assert_array_equal(s, ps[idx])
        np.testing.assert_array_equal(d, pd[idx])
    od, _ = g.degrees(True, False)
    np.testing.assert_array_equal(od, adj.out_deg())
    # BFS: the reference's edge-centric levels (bfs_simple -m 8, root 0) and
    # any root against the oracle, parents a BFS tree
    lv, par, st = g.edges_bfs(0, parents=True)
    np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfs_simple_m8"])
    assert oracle.bfs_tree_ok(n, adj.out_ptr, adj.out_col, 0, lv, par)
    assert st.reached == int((lv > 0).sum()) and st.edges_traversed == int(adj.out_deg()[lv > 0].sum())
    for r in rec["roots"]:
        lv, st = g.edges_bfs(int(r))
        np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
    # WCC over the input edges (no adjacency): the reference's edge-array labels
    lab, _ = g.wcc()
    np.testing.assert_array_equal(lab, rec["wcc_m8"])
    # the SpMV edge loop, x[i] = i (spmv -m 8) and random x with wrap-around
    y, _ = g.edges_spmv(np.arange(n, dtype=np.uint32))
    np.testing.assert_array_equal(y, rec["spmv_m8"])
    xr = np.random.default_rng(5).integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    y, _ = g.edges_spmv(xr)
    np.testing.assert_array_equal(y, oracle.spmv_u32(n, adj.out_ptr, adj.out_col, xr, oracle.SPMV_EDGE))
    # PageRank over the edges: FP64 and the reference's prgrid dumps
    ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10)
    rank, st = g.edges_pagerank(iterations=10)
    l1, mx = rel(rank, ref)
    assert l1 <= REL_L1 and mx <= ATOMIC_MAX_REL, (l1, mx)
    assert st.iterations_run == 10
    mode = {"file": 9, "src": 7, "src_dst": 8}[order]
    key = "prgrid_m%d" % mode
    if key in rec:
        pr, _ = g.edges_pagerank(iterations=10, prev_init=0.15, deg_multiplier=2 if mode == 9 else 1)
        _, mx = rel(pr, rec[key])
        assert mx <= ATOMIC_MAX_REL, (key, mx)
    g.free()


def test_edge_pagerank_tolerance_and_dangling(ctx):
    n, pairs, rec = load("rmat12")
    adj = oracle.build_adj(n, pairs)
    g = ctx.from_pairs(n, pairs).build_edges("file")
    ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 30, dangling=True)
    rank, st = g.edges_pagerank(iterations=30, dangling=True)
    l1, mx = rel(rank, ref)
    assert l1 <= REL_L1 and mx <= ATOMIC_MAX_REL, (l1, mx)
    assert abs(rank.astype(np.float64).sum() - 1.0) < 1e-4  # the mass is kept with dangling spread
    rank, st = g.edges_pagerank(iterations=100, tolerance=1e-6)
    assert st.iterations_run < 100 and st.residual < 1e-6
    g.free()


def test_edge_array_undirected_and_errors(ctx):
    import everythinggraph_gb300 as eg
    n, pairs, rec = load("rmat10")
    adju = oracle.build_adj(n, pairs, undirected=True)
    g = ctx.from_pairs(n, pairs, undirected=True).build_edges("src")
    s, d = g.edges()
    np.testing.assert_array_equal(s, adju.out_src())
    np.testing.assert_array_equal(d, adju.out_col)
    lv, _ = g.edges_bfs(0)
    np.testing.assert_array_equal(lv, oracle.bfs_levels(n, adju.out_ptr, adju.out_col, 0))
    with pytest.raises(RuntimeError):
        g.edges_bfs(n)  # root out of range
    g.free()
    g = ctx.from_pairs(n, pairs)
    with pytest.raises(eg.EGError) as e:
        g.edges_bfs(0)
    assert e.value.code == -6  # edge array not built
    assert eg.lib().eg_graph_build_edges(g._h, 7) == -1  # no such order
    g.free()
    g = ctx.from_pairs(4, np.array([0, 1, 1, 9], np.uint32))
    with pytest.raises(eg.EGError) as e:
        g.build_edges("file")
    assert e.value.code == -7  # EG_ERANGE: endpoint >= n
    g.free()
