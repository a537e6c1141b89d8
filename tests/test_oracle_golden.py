"""Pins the CPU oracle to the reference: every oracle function is checked
against result dumps of the unmodified reference binaries (tests/golden/,
made by tests/golden/make_golden.py).  No GPU needed."""
import hashlib
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["tiny", "rmat10", "rmat12", "rmat16"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    rec = {k: z[k] for k in z.files}
    n = int(rec["n"])
    if "pairs" in rec:
        pairs = rec["pairs"]
    else:
        scale = int(np.log2(n))
        pairs = oracle.rmat_edges(scale, 16 * n, 1)
    assert hashlib.sha256(pairs.tobytes()).hexdigest() == rec["pairs_sha256"].item().decode()
    return n, pairs, rec


@pytest.fixture(scope="module", params=CASES)
def case(request):
    n, pairs, rec = load(request.param)
    return request.param, n, pairs, rec


def test_generator_matches_stored_edges():
    # the scale-16 fixture stores only a digest; load() regenerates and checks it
    for name in CASES:
        load(name)


def test_pagerank_pull_quirk(case):
    # pagerank_simple -m 2 -a 1: prev fixed at 0.15, serial fp32 sums in CSC order
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    got = oracle.pagerank_f32(adj, adj.out_deg(), 0.15, 10, swap=False)
    np.testing.assert_array_equal(got.view(np.uint32), rec["pr_simple_pull"].view(np.uint32))


def test_prgrid(case):
    # prgrid_cilk -m 0: 10 iterations with swap, degrees counted twice
    name, n, pairs, rec = case
    P = oracle.default_p(n)
    cell_ptr, gsrc, gdst = oracle.build_grid(n, pairs, P)
    od, _ = oracle.degrees(n, pairs)
    got = oracle.pagerank_grid_f32(n, P, cell_ptr, gsrc, gdst, 2 * od, 0.15, 10)
    np.testing.assert_array_equal(got.view(np.uint32), rec["prgrid_m0"].view(np.uint32))
    # the grid sum order equals the CSC order, so the CSR/CSC oracle agrees too
    adj = oracle.build_adj(n, pairs)
    got2 = oracle.pagerank_f32(adj, 2 * od, 0.15, 10, swap=True)
    np.testing.assert_array_equal(got2.view(np.uint32), rec["prgrid_m0"].view(np.uint32))


def test_prgrid_edge_array(case):
    # prgrid_cilk -m 7/8/9: prgrid_algo_col over the edge array with atomic
    # fp32 adds (no fixed order, so a tolerance, as for the GPU), degrees
    # counted once in modes 7/8 (init_edgelist rewrites them) and twice in 9
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    for mode, mult in ((7, 1), (8, 1), (9, 2)):
        ref = oracle.pagerank_f64(adj, mult * adj.out_deg(), 0.15, 10)
        got = rec["prgrid_m%d" % mode].astype(np.float64)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)) <= 5e-5, mode


def test_bfs(case):
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    for r in rec["roots"]:
        lv = oracle.bfs_levels(n, adj.out_ptr, adj.out_col, int(r))
        np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
    # bfs_simple -m 8 (edge-centric): levels from root 0
    lv0 = oracle.bfs_levels(n, adj.out_ptr, adj.out_col, 0)
    np.testing.assert_array_equal(lv0.astype(np.uint32), rec["bfs_simple_m8"])
    np.testing.assert_array_equal(lv0.astype(np.uint32), rec["bfs_simple_m7"])
    np.testing.assert_array_equal(lv0.astype(np.uint32), rec["bfs_simple_m9"])
    # bfs_simple -m 2 -u: visited counters; the visited set is the -u BFS reach
    adju = oracle.build_adj(n, pairs, undirected=True)
    lvu = oracle.bfs_levels(n, adju.out_ptr, adju.out_col, 0)
    np.testing.assert_array_equal(lvu > 0, rec["bfs_simple_m2u"] > 0)


def test_bfs_parents_form_tree(case):
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    for r in rec["roots"]:
        lv, par = oracle.bfs_levels(n, adj.out_ptr, adj.out_col, int(r), parents=True)
        assert oracle.bfs_tree_ok(n, adj.out_ptr, adj.out_col, int(r), lv, par)


def test_bfs_tree_check_rejects_planted_mistakes(case):
    # mistakes planted in the oracle's own tree (CPU): each rule must fire
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    r = int(rec["roots"][0])
    lv, par = oracle.bfs_levels(n, adj.out_ptr, adj.out_col, r, parents=True)
    assert oracle.bfs_tree_check(n, adj.out_ptr, adj.out_col, r, lv, par) == 0
    deep = np.nonzero(lv > 2)[0]
    if len(deep) == 0:
        pytest.skip("tree too shallow")
    v = int(deep[0])
    bad = par.copy()
    bad[r] = -1
    assert oracle.bfs_tree_check(n, adj.out_ptr, adj.out_col, r, lv, bad) == -1
    unreached = np.nonzero(lv == 0)[0]
    if len(unreached):
        bad = par.copy()
        bad[unreached[0]] = r
        assert oracle.bfs_tree_check(n, adj.out_ptr, adj.out_col, r, lv, bad) == -2
    bad = par.copy()
    bad[v] = r  # root is two or more levels up
    assert oracle.bfs_tree_check(n, adj.out_ptr, adj.out_col, r, lv, bad) == -3
    # a parent one level up that has no edge to v
    same = np.nonzero(lv == lv[v] - 1)[0]
    src = adj.out_src()
    into_v = set(src[adj.out_col == v].tolist())
    cand = [int(p) for p in same if int(p) not in into_v]
    if cand:
        bad = par.copy()
        bad[v] = cand[0]
        assert oracle.bfs_tree_check(n, adj.out_ptr, adj.out_col, r, lv, bad) == -4


def test_spmv_f64_hashed_equals_stored_values(case):
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    x = oracle.uniform_f32(n, 11)
    vals = oracle.hash_values(adj.in_col, adj.in_dst(), 9)
    np.testing.assert_array_equal(oracle.spmv_f64_hashed(n, adj.in_ptr, adj.in_col, 9, x),
                                  oracle.spmv_f64(n, adj.in_ptr, adj.in_col, vals, x))


def test_sssp(case):
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    w = oracle.ref_weights(adj, "out")
    for r in rec["roots"]:
        d = oracle.sssp(n, adj.out_ptr, adj.out_col, w, int(r))
        np.testing.assert_array_equal(d, rec["sssp_pull_p%d" % r])


def test_sssp_f32(case):
    # (1) with the reference's integer weights as floats the fp32 path sums are
    # exact, so the fp32 Dijkstra must reproduce the reference's dumps (its pull
    # relax adds in float); (2) with hashed fp32 weights it must equal an
    # independent float32 Bellman-Ford fixed point
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    w = oracle.ref_weights(adj, "out").astype(np.float32)
    for r in rec["roots"]:
        d = oracle.sssp_f32(n, adj.out_ptr, adj.out_col, w, int(r))
        ref = rec["sssp_pull_p%d" % r]
        np.testing.assert_array_equal(np.isinf(d), ref == 0xFFFFFFFE)
        np.testing.assert_array_equal(d[~np.isinf(d)], ref[ref != 0xFFFFFFFE].astype(np.float32))
    if n > 5000:
        return
    wf = oracle.hash_weights_f32(adj.out_src(), adj.out_col, 6)
    assert wf.min() > 0 and wf.max() <= 1
    src, dst = adj.out_src(), adj.out_col
    keep = src != dst
    src, dst, wf = src[keep], dst[keep], wf[keep]
    for r in rec["roots"]:
        d = np.full(n, np.inf, dtype=np.float32)
        d[int(r)] = 0
        while True:
            cand = (d[src] + wf).astype(np.float32)
            nd = d.copy()
            np.minimum.at(nd, dst, cand)
            if np.array_equal(nd, d):
                break
            d = nd
        got = oracle.sssp_f32(n, adj.out_ptr, adj.out_col, oracle.hash_weights_f32(adj.out_src(), adj.out_col, 6), int(r))
        np.testing.assert_array_equal(got.view(np.uint32), d.view(np.uint32))


def test_wcc(case):
    name, n, pairs, rec = case
    lab = oracle.wcc(n, pairs)
    np.testing.assert_array_equal(lab, rec["wcc_m2u"])
    np.testing.assert_array_equal(lab, rec["wcc_m0"])
    np.testing.assert_array_equal(lab, rec["wcc_m8"])


def test_spmv_u32(case):
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    x = np.arange(n, dtype=np.uint32)
    np.testing.assert_array_equal(oracle.spmv_u32(n, adj.in_ptr, adj.in_col, x, oracle.SPMV_PULL), rec["spmv_pull"])
    np.testing.assert_array_equal(oracle.spmv_u32(n, adj.out_ptr, adj.out_col, x, oracle.SPMV_PUSH), rec["spmv_push"])
    np.testing.assert_array_equal(oracle.spmv_u32(n, adj.out_ptr, adj.out_col, x, oracle.SPMV_EDGE), rec["spmv_m8"])


def test_milli_floor_equals_integer_division():
    # The reference scales x by the double 0.001 and truncates; for every u32 x
    # that equals x // 1000 (the CUDA kernels use the integer form).  Checked on
    # all multiples of 1000 and their neighbours plus a random sample.
    k = np.arange(0, 4294968, dtype=np.uint64) * 1000
    xs = np.concatenate([k, k + 1, k[1:] - 1, np.random.default_rng(0).integers(0, 2**32, 2_000_000)])
    xs = xs[xs < 2**32].astype(np.uint64)
    scaled = np.floor(0.001 * xs.astype(np.float64)).astype(np.uint64)
    np.testing.assert_array_equal(scaled, xs // 1000)


def test_parallel_ports(case):
    # the multi-threaded ports used as the timed CPU baseline agree with the
    # reference dumps too
    name, n, pairs, rec = case
    adj = oracle.build_adj(n, pairs)
    for r in rec["roots"]:
        lv = oracle.bfs_do(adj.out_ptr, adj.out_col, adj.in_ptr, adj.in_col, int(r))
        np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
    adju = oracle.build_adj(n, pairs, undirected=True)
    comp, rounds = oracle.wcc_lp(adju.out_ptr, adju.out_col)
    np.testing.assert_array_equal(comp, rec["wcc_m2u"])
