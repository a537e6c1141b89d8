"""GPU parity: the CUDA path, called through the C ABI, against the oracle
and the reference's own dumps (tests/golden/).

Integer outputs (layouts, BFS levels, SSSP distances, WCC labels, integer
SpMV) must be bit-exact.  Floating-point outputs use the tolerances written
below: against FP64, relative L1 error <= 1e-6 and max relative error <= 1e-5;
against the reference's fp32 dumps (a different summation order), max
relative error <= 2e-5.
"""
import hashlib
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["tiny", "rmat10", "rmat12", "rmat16"]
PR_REL_L1 = 1e-6
PR_MAX_REL = 1e-5
PR_VS_REF32_MAX_REL = 2e-5
# the grid-layout kernels add fp32 contributions with atomics in arbitrary
# order and without compensation: the rel L1 bound is the same, the largest
# single-row error (a hub row of 10^4 terms, ~sqrt(terms) * 2^-24) is looser
GRID_MAX_REL = 5e-5


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    rec = {k: z[k] for k in z.files}
    n = int(rec["n"])
    pairs = rec["pairs"] if "pairs" in rec else oracle.rmat_edges(int(np.log2(n)), 16 * n, 1)
    assert hashlib.sha256(pairs.tobytes()).hexdigest() == rec["pairs_sha256"].item().decode()
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
    import everythinggraph_gb300 as eg
    n, pairs, rec = load(request.param)
    g = ctx.from_pairs(n, pairs).build(eg.CSR | eg.CSC)
    gu = ctx.from_pairs(n, pairs, undirected=True).build(eg.CSR | eg.CSC)
    adj = oracle.build_adj(n, pairs)
    adju = oracle.build_adj(n, pairs, undirected=True)
    yield request.param, n, pairs, rec, g, gu, adj, adju
    g.free()
    gu.free()


def rel_errors(got, ref):
    got = got.astype(np.float64)
    ref = ref.astype(np.float64)
    l1 = np.abs(got - ref).sum() / max(np.abs(ref).sum(), 1e-300)
    mx = (np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)).max() if len(ref) else 0.0
    return l1, mx


# ------------------------------------------------------------------ layouts
def test_layouts_bit_exact(case):
    import everythinggraph_gb300 as eg
    name, n, pairs, rec, g, gu, adj, adju = case
    for graph, a in ((g, adj), (gu, adju)):
        ptr, col = graph.adj(eg.CSR)
        np.testing.assert_array_equal(ptr, a.out_ptr)
        np.testing.assert_array_equal(col, a.out_col)  # file order inside each list
        ptr, col = graph.adj(eg.CSC)
        np.testing.assert_array_equal(ptr, a.in_ptr)
        np.testing.assert_array_equal(col, a.in_col)  # ascending src inside each list
        od, idg = graph.degrees(True, True)
        np.testing.assert_array_equal(od, a.out_deg())
        np.testing.assert_array_equal(idg, a.in_deg())


def test_grid_layout_bit_exact(case, ctx):
    name, n, pairs, rec, g, gu, adj, adju = case
    for P in sorted({oracle.default_p(n), 3, 7}):
        if P > n:
            continue
        gg = ctx.from_pairs(n, pairs)
        gg.build_grid(P)
        cp, s, d = gg.grid()
        rcp, rs, rd = oracle.build_grid(n, pairs, P)
        np.testing.assert_array_equal(cp, rcp)
        np.testing.assert_array_equal(s, rs)
        np.testing.assert_array_equal(d, rd)
        gg.free()


def test_device_generators_match_cpu(ctx):
    import everythinggraph_gb300 as eg
    for scale, seed in ((10, 1), (12, 7)):
        n = 1 << scale
        g = ctx.rmat(scale, 16 * n, seed).build(eg.CSR)
        a = oracle.build_adj(n, oracle.rmat_edges(scale, 16 * n, seed))
        ptr, col = g.adj(eg.CSR)
        np.testing.assert_array_equal(ptr, a.out_ptr)
        np.testing.assert_array_equal(col, a.out_col)
        g.free()
    n, m = 5000, 40000
    g = ctx.er(n, m, 4).build(eg.CSR)
    a = oracle.build_adj(n, oracle.er_edges(n, m, 4))
    ptr, col = g.adj(eg.CSR)
    np.testing.assert_array_equal(col, a.out_col)
    g.free()


# ------------------------------------------------------------------ PageRank
def test_pagerank_reference_pull_quirk(case):
    # pagerank_simple -m 2 -a 1: prev stays 0.15, 10 identical iterations
    name, n, pairs, rec, g, gu, adj, adju = case
    got, st = g.pagerank(iterations=10, prev_init=0.15, swap=False)
    l1, mx = rel_errors(got, rec["pr_simple_pull"])
    assert mx <= PR_VS_REF32_MAX_REL, (l1, mx)


def test_pagerank_prgrid_semantics(case):
    # prgrid_cilk -m 0: 10 iterations with swap, degrees counted twice
    name, n, pairs, rec, g, gu, adj, adju = case
    for comp in (False, True):
        got, st = g.pagerank(iterations=10, prev_init=0.15, swap=True, deg_multiplier=2, compensated=comp)
        l1, mx = rel_errors(got, rec["prgrid_m0"])
        assert mx <= PR_VS_REF32_MAX_REL, (comp, l1, mx)


def test_pagerank_vs_fp64(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    for dangling in (False, True):
        ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=dangling)
        for comp in (False, True):
            got, st = g.pagerank(iterations=10, dangling=dangling, compensated=comp)
            l1, mx = rel_errors(got, ref)
            assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (dangling, comp, l1, mx)
            assert st.iterations_run == 10


def test_pagerank_graph_replay_matches_stream(case):
    # the captured iteration loop gives the same bits as the launched one,
    # on a first capture, a replay, and a re-capture after the options change
    name, n, pairs, rec, g, gu, adj, adju = case
    for comp, dangling in ((False, False), (False, False), (True, True), (False, False)):
        a, sa = g.pagerank(iterations=7, compensated=comp, dangling=dangling)
        b, sb = g.pagerank(iterations=7, compensated=comp, dangling=dangling, use_graph=True)
        np.testing.assert_array_equal(a, b)
        assert sb.iterations_run == 7
        assert sa.row_kernel_ms > 0 and sb.row_kernel_ms == 0


def test_row_schedules_and_autotuner(case):
    # every row-kernel schedule stays within the FP64 tolerance, for PageRank
    # and the fp32 SpMV; the tuner keeps the fastest of them
    name, n, pairs, rec, g, gu, adj, adju = case
    ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=True)
    x = oracle.uniform_f32(n, 11)
    vals = oracle.hash_values(adj.in_col, adj.in_dst(), 9)
    y_ref = oracle.spmv_f64(n, adj.in_ptr, adj.in_col, vals, x)
    cands, chosen = g.tune()
    assert len(cands) == 13 and 0 <= chosen < 13
    assert g.bfs_tuning["switch_divisor"] in (20.0, 40.0, 80.0, 160.0, 320.0)
    assert sum(c["cache_hint"] for c in cands) == 3
    assert [c["partition_log2"] for c in cands] == [0] * 12 + [13]
    if n > 1000:
        assert all(c["ms"] > 0 for c in cands)
    assert cands[chosen]["ms"] == min(c["ms"] for c in cands)
    for idx in range(len(cands)):
        g.set_row_schedule(idx)
        got, st = g.pagerank(iterations=10, dangling=True)
        l1, mx = rel_errors(got, ref)
        assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (cands[idx], l1, mx)
        y, _ = g.spmv(x, "f32_comp", value_seed=9)
        l1, mx = rel_errors(y, y_ref)
        assert l1 <= PR_REL_L1, (cands[idx], l1)
    with pytest.raises(RuntimeError):
        g.set_row_schedule(len(cands))
    g.set_row_schedule(0)


def test_pagerank_partition_kernel(case):
    # schedule 12: the relabelled CSC by destination partition and source,
    # 64-bit fixed-point row sums (the same bits in any order of addition)
    name, n, pairs, rec, g, gu, adj, adju = case
    g.set_row_schedule(12)
    try:
        for dangling in (False, True):
            ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=dangling)
            got, st = g.pagerank(iterations=10, dangling=dangling)
            l1, mx = rel_errors(got, ref)
            assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (dangling, l1, mx)
            assert st.iterations_run == 10 and st.row_kernel_ms > 0
            again, _ = g.pagerank(iterations=10, dangling=dangling)
            np.testing.assert_array_equal(got, again)  # run to run
            replay, _ = g.pagerank(iterations=10, dangling=dangling, use_graph=True)
            np.testing.assert_array_equal(got, replay)  # captured loop
        # the reference's own semantics: pull mode (prev stays 0.15, rank mass
        # 0.15 n) and prgrid (degrees counted twice)
        got, _ = g.pagerank(iterations=10, prev_init=0.15, swap=False)
        _, mx = rel_errors(got, rec["pr_simple_pull"])
        assert mx <= PR_VS_REF32_MAX_REL, mx
        got, _ = g.pagerank(iterations=10, prev_init=0.15, swap=True, deg_multiplier=2)
        _, mx = rel_errors(got, rec["prgrid_m0"])
        assert mx <= PR_VS_REF32_MAX_REL, mx
        # the fixed-point unit follows the least rank (1 - d) / n: other
        # dampings, and d = 1 (no rank floor: the finest unit)
        for d in (0.5, 0.99, 1.0):
            ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=True, damping=d)
            got, _ = g.pagerank(iterations=10, dangling=True, damping=d)
            l1, mx = rel_errors(got, ref)
            assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (d, l1, mx)
        # the tolerance stop
        ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 50, dangling=True)
        got, st = g.pagerank(iterations=50, dangling=True, tolerance=1e-9)
        assert st.iterations_run <= 50
        l1, _ = rel_errors(got, ref)
        assert l1 <= 1e-5, l1
    finally:
        g.set_row_schedule(0)


def test_pagerank_partition_kernel_hub_rows(ctx):
    # one row with most of the entries (its 64-bit sums carry out of the low
    # words many times and its partition spans many segments), rows spread
    # over several partitions, an undirected copy: partition kernel against
    # FP64, bit-identical from run to run and with the graph replay
    import everythinggraph_gb300 as eg
    rng = np.random.default_rng(21)
    n = 40000
    m_star, m_rand = 300000, 200000
    pairs = np.empty(2 * (m_star + m_rand), dtype=np.uint32)
    pairs[0:2 * m_star:2] = rng.integers(1, n, m_star)
    pairs[1:2 * m_star:2] = 0  # everything points at vertex 0
    pairs[2 * m_star::2] = rng.integers(0, n, m_rand)
    pairs[2 * m_star + 1::2] = rng.integers(0, n, m_rand)
    for undirected in (False, True):
        g = ctx.from_pairs(n, pairs, undirected=undirected).build(eg.CSR | eg.CSC)
        adj = oracle.build_adj(n, pairs, undirected=undirected)
        g.set_row_schedule(12)
        for dangling in (False, True):
            ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=dangling)
            got, st = g.pagerank(iterations=10, dangling=dangling)
            l1, mx = rel_errors(got, ref)
            assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (undirected, dangling, l1, mx)
            again, _ = g.pagerank(iterations=10, dangling=dangling, use_graph=True)
            np.testing.assert_array_equal(got, again)
        g.free()


def test_pagerank_source_blocks(case):
    # PageRank gathering its contributions one source block per pass (blocks
    # of 2^k vertices; the default 2^24 only splits larger graphs): within the
    # FP64 tolerance, graph replay = stream launch, the tolerance stop works
    name, n, pairs, rec, g, gu, adj, adju = case
    ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=True)
    ran = 0
    for k in (10, 8, 3):
        if n > (64 << k) or n <= (1 << k):
            continue
        ran += 1
        got, st = g.pagerank(iterations=10, dangling=True, source_block_log2=k)
        l1, mx = rel_errors(got, ref)
        assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (k, l1, mx)
        assert st.row_kernel_ms > 0  # timed over all passes, also when a block has no entries
        a, _ = g.pagerank(iterations=7, source_block_log2=k)
        b, _ = g.pagerank(iterations=7, source_block_log2=k, use_graph=True)
        np.testing.assert_array_equal(a, b)
        got, st = g.pagerank(iterations=200, tolerance=1e-6, dangling=True, source_block_log2=k)
        assert 1 <= st.iterations_run < 200 and st.residual < 1e-6
    assert ran >= 1
    # back to one pass on the same graph
    got, _ = g.pagerank(iterations=10, dangling=True)
    l1, mx = rel_errors(got, ref)
    assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL


def test_pagerank_rows_without_in_edges(ctx):
    # vertices without in-edges (a quarter of them, plus isolated ones) are
    # the rows PageRank writes apart from the row kernel: their ranks, the
    # dangling mass of the isolated ones, and a personalised seed among them
    import everythinggraph_gb300 as eg
    n = 6000
    rng = np.random.default_rng(5)
    m = 60000
    src = rng.integers(0, 4000, size=m)
    dst = rng.integers(1500, 4000, size=m)  # [0, 1500) and [4000, n) have no in-edges
    src[:50] = 4500  # one out-only vertex above the isolated range [4000, 4500), (4500, n)
    pairs = np.stack([src, dst], axis=1).astype(np.uint32).reshape(-1)
    g = ctx.from_pairs(n, pairs).build(eg.CSR | eg.CSC)
    adj = oracle.build_adj(n, pairs)
    try:
        for dangling in (False, True):
            ref = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=dangling)
            got, st = g.pagerank(iterations=10, dangling=dangling)
            l1, mx = rel_errors(got, ref)
            assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (dangling, l1, mx)
            a, _ = g.pagerank(iterations=7, dangling=dangling)
            b, _ = g.pagerank(iterations=7, dangling=dangling, use_graph=True)
            np.testing.assert_array_equal(a, b)
        for seeds in (np.array([4500], np.uint32), np.array([10, 2000, 10], np.uint32)):
            ref, it_ref = oracle.ppr_f64(adj, adj.out_deg(), seeds, tol=1e-7, max_iters=50)
            got, st = g.ppr_single(seeds, tolerance=1e-7, max_iters=50)
            l1 = np.abs(got - ref).sum() / np.abs(ref).sum()
            assert l1 <= 1e-5, (seeds, l1)
            assert abs(st.iterations[0] - it_ref) <= 1
    finally:
        g.free()


def test_pagerank_tolerance_stops_early(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    got, st = g.pagerank(iterations=200, tolerance=1e-6, dangling=True)
    assert 1 <= st.iterations_run < 200
    assert st.residual < 1e-6
    assert abs(float(got.astype(np.float64).sum()) - 1.0) < 1e-4  # mass conserved with dangling redistribution


def test_grid_spmv_and_pagerank(case):
    # grid modes: grid=True runs the fixed-order row kernel (the grid's
    # per-destination order is the CSC's), bit-identical to the plain call;
    # grid="cells" the cell kernel (cells in L2-sized blocks, atomic sums):
    # integer SpMV exact, float within tolerance, prgrid's PageRank against
    # the reference's own dumps and FP64
    name, n, pairs, rec, g, gu, adj, adju = case
    P = oracle.default_p(n) if n > 100 else 3
    g.build_grid(P)
    x = np.arange(n, dtype=np.uint32)
    xf = oracle.uniform_f32(n, 11)
    vals = oracle.hash_values(adj.in_col, adj.in_dst(), 9)
    ref = oracle.spmv_f64(n, adj.in_ptr, adj.in_col, vals, xf)
    for mode in (True, "cells"):
        y, _ = g.spmv(x, "u32_pull", grid=mode)
        np.testing.assert_array_equal(y, rec["spmv_pull"])
        y, _ = g.spmv(x, "u32_push", grid=mode)
        np.testing.assert_array_equal(y, rec["spmv_push"])
        y, _ = g.spmv(x, "u32_edge", grid=mode)
        np.testing.assert_array_equal(y, rec["spmv_m8"])
        y64, _ = g.spmv(xf, "f64", value_seed=9, grid=mode)
        np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-300)
        y32, _ = g.spmv(xf, "f32", value_seed=9, grid=mode)
        l1, mx = rel_errors(y32, ref)
        assert l1 <= PR_REL_L1 and mx <= GRID_MAX_REL, (mode, l1, mx)
        got, st = g.pagerank(iterations=10, prev_init=0.15, swap=True, deg_multiplier=2, grid=mode)
        l1, mx = rel_errors(got, rec["prgrid_m0"])
        assert mx <= PR_VS_REF32_MAX_REL, (mode, l1, mx)
        ref_pr = oracle.pagerank_f64(adj, adj.out_deg(), 1.0 / n, 10, dangling=True)
        got, st = g.pagerank(iterations=10, dangling=True, grid=mode)
        l1, mx = rel_errors(got, ref_pr)
        assert l1 <= PR_REL_L1 and mx <= GRID_MAX_REL, (mode, l1, mx)
        got, st = g.pagerank(iterations=200, tolerance=1e-6, dangling=True, grid=mode)
        assert 1 <= st.iterations_run < 200 and st.residual < 1e-6
    with pytest.raises(RuntimeError):
        g.spmv(xf, "f32_comp", grid="cells")
    # the fixed-order grid path is the row kernel itself: the same bits
    y1, _ = g.spmv(xf, "f32", value_seed=9, grid=True)
    y0, _ = g.spmv(xf, "f32", value_seed=9)
    np.testing.assert_array_equal(y1.view(np.uint32), y0.view(np.uint32))
    yc, _ = g.spmv(xf, "f32_comp", value_seed=9, grid=True)
    l1, mx = rel_errors(yc, ref)
    assert l1 <= PR_REL_L1 and mx <= PR_MAX_REL, (l1, mx)


# ------------------------------------------------------------------ SpMV
def test_spmv_u32_bit_exact(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    x = np.arange(n, dtype=np.uint32)
    y, _ = g.spmv(x, "u32_pull")
    np.testing.assert_array_equal(y, rec["spmv_pull"])
    y, _ = g.spmv(x, "u32_push")
    np.testing.assert_array_equal(y, rec["spmv_push"])
    y, _ = g.spmv(x, "u32_edge")
    np.testing.assert_array_equal(y, rec["spmv_m8"])
    # random x with wrap-around
    xr = np.random.default_rng(5).integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    y, _ = g.spmv(xr, "u32_edge")
    np.testing.assert_array_equal(y, oracle.spmv_u32(n, adj.out_ptr, adj.out_col, xr, oracle.SPMV_EDGE))


def test_spmv_float_vs_fp64(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    x = oracle.uniform_f32(n, 11)
    # edge values are hashed from the endpoints; the oracle recomputes them
    vals = oracle.hash_values(adj.in_col, adj.in_dst(), 9)
    ref = oracle.spmv_f64(n, adj.in_ptr, adj.in_col, vals, x)
    y64, _ = g.spmv(x, "f64", value_seed=9)
    assert y64.dtype == np.float64
    np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-300)
    ones64 = oracle.spmv_f64(n, adj.in_ptr, adj.in_col, np.ones(adj.m, np.float32), x)
    y1, _ = g.spmv(x, "f64", unit_values=True)
    np.testing.assert_allclose(y1, ones64, rtol=1e-12, atol=1e-300)
    nz = ref != 0
    for kind in ("f32", "f32_comp"):
        y, _ = g.spmv(x, kind, value_seed=9)
        l1, mx = rel_errors(y[nz], ref[nz])
        assert l1 <= 1e-6 and mx <= 1e-5, (kind, l1, mx)
        assert np.all(y[~nz] == 0)


def test_spmv_source_blocks(case):
    # fp32 SpMV one source block per pass (blocks of 2^k vertices; the default
    # 2^24 only splits larger graphs): within the FP64 tolerance, rows without
    # entries zero, values re-gathered when the seed or the rule changes
    name, n, pairs, rec, g, gu, adj, adju = case
    x = oracle.uniform_f32(n, 11)
    for seed in (9, 3):
        vals = oracle.hash_values(adj.in_col, adj.in_dst(), seed)
        ref = oracle.spmv_f64(n, adj.in_ptr, adj.in_col, vals, x)
        nz = ref != 0
        y_one, _ = g.spmv(x, "f32", value_seed=seed)
        for k in (10, 3, 2):
            if n > (64 << k):  # at most 64 blocks
                continue
            y, _ = g.spmv(x, "f32", value_seed=seed, source_block_log2=k)
            l1, mx = rel_errors(y[nz], ref[nz])
            assert l1 <= 1e-6 and mx <= 1e-5, (k, l1, mx)
            assert np.all(y[~nz] == 0)
            if n <= (1 << k):  # one block: the same pass as without blocks
                np.testing.assert_array_equal(y, y_one)
            y2, _ = g.spmv(x, "f32", value_seed=seed, source_block_log2=k)
            np.testing.assert_array_equal(y, y2)  # a fixed order
            yc, _ = g.spmv(x, "f32_comp", value_seed=seed, source_block_log2=k)
            l1, mx = rel_errors(yc[nz], ref[nz])
            assert l1 <= 1e-6 and mx <= 1e-5, ("comp", k, l1, mx)
            assert np.all(yc[~nz] == 0)
    ones = oracle.spmv_f64(n, adj.in_ptr, adj.in_col, np.ones(adj.m, np.float32), x)
    k = max(2, int(np.ceil(np.log2(max(n, 2)))) - 2)
    y, _ = g.spmv(x, "f32", unit_values=True, source_block_log2=k)
    nz = ones != 0
    l1, mx = rel_errors(y[nz], ones[nz])
    assert l1 <= 1e-6 and mx <= 1e-5, (l1, mx)


# ------------------------------------------------------------------ BFS
def test_bfs_levels_bit_exact(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    for r in rec["roots"]:
        for direction in ("auto", "push", "pull"):
            for host_loop in (False, True):  # device-driven graph loop and host-driven loop
                lv, par, st = g.bfs(int(r), direction=direction, parents=True, host_loop=host_loop)
                np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
                assert oracle.bfs_tree_ok(n, adj.out_ptr, adj.out_col, int(r), lv, par)
                assert st.reached == int((lv > 0).sum())
    # the push/pull switch point changes how levels are computed, not them
    r = int(rec["roots"][0])
    for div in (2.0, 80.0, 320.0, 1e9):
        lv, par, st = g.bfs(r, switch_divisor=div, parents=True)
        np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
        assert oracle.bfs_tree_ok(n, adj.out_ptr, adj.out_col, r, lv, par)
    lv, st = g.bfs(0)
    np.testing.assert_array_equal(lv.astype(np.uint32), rec["bfs_simple_m8"])
    lvu, st = gu.bfs(0)
    np.testing.assert_array_equal(lvu > 0, rec["bfs_simple_m2u"] > 0)
    assert st.reached == int((lvu > 0).sum())


def test_outputs_into_pinned_buffers(case):
    # caller-supplied page-locked outputs, reused across calls, hold the same
    # results as freshly allocated ones
    import everythinggraph_gb300 as eg
    name, n, pairs, rec, g, gu, adj, adju = case
    lv_h = eg.pinned_empty(n, np.int32)
    par_h = eg.pinned_empty(n, np.int32)
    lab_h = eg.pinned_empty(n, np.int64)
    for r in rec["roots"][:2]:
        lv, par, st = g.bfs(int(r), parents=True, level_out=lv_h, parent_out=par_h)
        assert lv is lv_h and par is par_h
        np.testing.assert_array_equal(lv_h.astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
        assert oracle.bfs_tree_ok(n, adj.out_ptr, adj.out_col, int(r), lv_h, par_h)
    lab, _ = g.wcc(out=lab_h)
    np.testing.assert_array_equal(lab_h, g.wcc()[0])
    # batched roots: copies of one root overlap the next traversal, results
    # equal root-by-root BFS; both level-loop forms
    roots = np.array(list(rec["roots"]) * 3, dtype=np.uint32)
    k = len(roots)
    lvb = eg.pinned_empty(k * n, np.int32)
    pab = eg.pinned_empty(k * n, np.int32)
    for host_loop in (False, True):
        lvs, pas, sts = g.bfs_batch(roots, parents=True, host_loop=host_loop, level_out=lvb, parent_out=pab)
        for i, r in enumerate(roots):
            np.testing.assert_array_equal(lvs[i].astype(np.uint32), rec["bfsgrid_m0_p%d" % r])
            assert oracle.bfs_tree_ok(n, adj.out_ptr, adj.out_col, int(r), lvs[i], pas[i])
            assert sts[i].reached == int((lvs[i] > 0).sum())
    lvs, pas, sts = g.bfs_batch(roots[:3])
    assert pas is None and lvs.shape == (3, n)
    with pytest.raises(ValueError):
        g.bfs(0, level_out=np.empty(n, dtype=np.int64))


def test_bfs_multi_matches_single(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    od = adju.out_deg()
    for k in (1, 5, 64):
        roots = oracle.sample_roots(od, k, 3)
        lv, st = gu.bfs_multi(roots)
        for s, r in enumerate(roots):
            ref = oracle.bfs_levels(n, adju.out_ptr, adju.out_col, int(r))
            np.testing.assert_array_equal(lv[s], ref)


# ------------------------------------------------------------------ SSSP
def test_sssp_bit_exact(case):
    import everythinggraph_gb300 as eg
    name, n, pairs, rec, g, gu, adj, adju = case
    for r in rec["roots"]:
        d, st = g.sssp(int(r), eg.weights("ref"))
        np.testing.assert_array_equal(d, rec["sssp_pull_p%d" % r])


def test_sssp_hash_weights_and_batch(case):
    import everythinggraph_gb300 as eg
    name, n, pairs, rec, g, gu, adj, adju = case
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    # the oracle gets the same per-entry weights (hash of the endpoints)
    wa = oracle.hash_weights(adj.out_src(), adj.out_col, 6, 1, 255)
    roots = oracle.sample_roots(adj.out_deg(), 7, 5)
    dm, st = g.sssp_multi(roots, w)
    for s, r in enumerate(roots):
        ref = oracle.sssp(n, adj.out_ptr, adj.out_col, wa, int(r))
        d1, _ = g.sssp(int(r), w)
        np.testing.assert_array_equal(d1, ref)
        np.testing.assert_array_equal(dm[s], ref)


def test_sssp_f32_weights_bit_exact(case):
    # fp32 weights in (0, 1] with fp32 path sums: the least fixed point is
    # unique, so the GPU's relaxation order cannot change a bit
    import everythinggraph_gb300 as eg
    name, n, pairs, rec, g, gu, adj, adju = case
    w = eg.weights("f32", seed=6)
    wa = oracle.hash_weights_f32(adj.out_src(), adj.out_col, 6)
    assert wa.min() > 0 and wa.max() <= 1
    roots = oracle.sample_roots(adj.out_deg(), 5, 9)
    dm, st = g.sssp_multi(roots, w)
    assert dm.dtype == np.float32
    for s, r in enumerate(roots):
        ref = oracle.sssp_f32(n, adj.out_ptr, adj.out_col, wa, int(r))
        d1, st1 = g.sssp(int(r), w)
        np.testing.assert_array_equal(d1.view(np.uint32), ref.view(np.uint32))
        np.testing.assert_array_equal(dm[s].view(np.uint32), ref.view(np.uint32))
        assert st1.reached == int(np.isfinite(ref).sum())


# ------------------------------------------------------------------ WCC
def test_wcc_bit_exact(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    lab, st = g.wcc()
    np.testing.assert_array_equal(lab, rec["wcc_m2u"])
    lab2, st2 = gu.wcc()
    np.testing.assert_array_equal(lab2, rec["wcc_m0"])
    assert st.components == len(np.unique(lab))


# ------------------------------------------------------------------ edge cases
def test_empty_and_tiny_graphs(ctx):
    import everythinggraph_gb300 as eg
    g = ctx.from_pairs(5, np.zeros(0, np.uint32)).build(eg.CSR | eg.CSC)
    lv, st = g.bfs(3)
    assert list(lv) == [0, 0, 0, 1, 0]
    r, _ = g.pagerank(iterations=3)
    np.testing.assert_allclose(r, np.full(5, 0.15 / 5, np.float32), rtol=1e-6)
    lab, _ = g.wcc()
    assert list(lab) == [0, 1, 2, 3, 4]
    d, _ = g.sssp(2)
    assert d[2] == 0 and (d[[0, 1, 3, 4]] == 0xFFFFFFFE).all()
    g.free()
    g1 = ctx.from_pairs(1, np.array([0, 0], np.uint32)).build(eg.CSR | eg.CSC)
    lv, st = g1.bfs(0)
    assert list(lv) == [1]
    g1.free()


def test_errors_are_reported(ctx):
    import everythinggraph_gb300 as eg
    g = ctx.from_pairs(4, np.array([0, 1, 1, 9], np.uint32))
    with pytest.raises(eg.EGError) as e:
        g.build()
    assert e.value.code == -7  # EG_ERANGE: endpoint >= n
    g.free()
    g = ctx.from_pairs(4, np.array([0, 1, 1, 2], np.uint32))
    with pytest.raises(eg.EGError) as e:
        g.bfs(0)
    assert e.value.code == -6  # layout not built
    g.build()
    with pytest.raises(eg.EGError) as e:
        g.bfs(4)
    assert e.value.code == -1
    g.free()
    small = eg.Context(0, hbm_budget=1 << 20)
    with pytest.raises(eg.EGError) as e:
        small.rmat(16, 1 << 20, 1)
    assert e.value.code == -3  # over the HBM budget
    small.close()


# ------------------------------------------------------------------ larger, property checks
@pytest.fixture(scope="module")
def big(ctx):
    import everythinggraph_gb300 as eg
    g = ctx.rmat(20, 16 << 20, 2, undirected=True).build(eg.CSR | eg.CSC)
    yield g
    g.free()


def test_big_bfs_properties(big):
    import everythinggraph_gb300 as eg
    ptr, col = big.adj(eg.CSR)
    src = np.repeat(np.arange(len(ptr) - 1, dtype=np.int64), np.diff(ptr.astype(np.int64)))
    roots = big.sample_roots(4, 3)
    lvm, _ = big.bfs_multi(roots)
    for s, r in enumerate(roots):
        lv, par, st = big.bfs(int(r), parents=True)
        np.testing.assert_array_equal(lv, lvm[s])
        lvh, sth = big.bfs(int(r), host_loop=True)
        np.testing.assert_array_equal(lv, lvh)
        assert (st.levels, st.reached, st.edges_traversed) == (sth.levels, sth.reached, sth.edges_traversed)
        # every edge from a reached vertex reaches a vertex at most one level deeper
        ls, ld = lv[src], lv[col]
        assert np.all(ld[ls > 0] > 0) and np.all(ld[ls > 0] <= ls[ls > 0] + 1)
        reached = np.nonzero(lv > 0)[0]
        reached = reached[reached != r]
        assert np.all(lv[par[reached]] == lv[reached] - 1)


def test_big_wcc_and_sssp_properties(big):
    import everythinggraph_gb300 as eg
    ptr, col = big.adj(eg.CSR)
    n = len(ptr) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(ptr.astype(np.int64)))
    lab, st = big.wcc()
    assert np.all(lab[src] == lab[col])
    assert np.all(lab <= np.arange(len(lab))) and np.all(lab[lab] == lab)
    # the labels are the oracle's min-id labels (a merge of two components
    # under the smaller id would pass the closure checks above)
    np.testing.assert_array_equal(lab, oracle.wcc(n, oracle.rmat_edges(20, 16 << 20, 2)))
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    wa = oracle.hash_weights(src.astype(np.uint32), col, 6, 1, 255).astype(np.int64)
    r = int(big.sample_roots(1, 5)[0])
    d, st = big.sssp(r, w)
    d = d.astype(np.int64)
    INF = 0xFFFFFFFE
    ok = (d[src] != INF) & (src != col)
    assert np.all(d[col][ok] <= d[src][ok] + wa[ok])  # no edge can still be relaxed
    assert d[r] == 0
    # every reached vertex's distance is attained by an in-edge (too-small
    # distances would pass the relaxation check above)
    attained = np.zeros(n, dtype=bool)
    attained[col[ok & (d[src] + wa == d[col])]] = True
    reached = np.nonzero(d != INF)[0]
    assert np.all(attained[reached[reached != r]])
    np.testing.assert_array_equal(d.astype(np.uint32), oracle.sssp(n, ptr, col, wa.astype(np.uint32), r))


# ------------------------------------------------------------------ personalised PageRank
def test_ppr_batch_vs_fp64_and_alone(case):
    name, n, pairs, rec, g, gu, adj, adju = case
    rng = np.random.default_rng(7)
    nz = np.nonzero(adj.out_deg() > 0)[0]
    seed_lists = [rng.choice(nz, size=int(rng.integers(1, 9))).astype(np.uint32) for _ in range(12)]
    tols = [1e-4, 1e-5, 1e-6, 1e-7] * 3
    R, st = g.ppr(seed_lists, tolerance=tols, max_iters=50)
    for q, seeds in enumerate(seed_lists):
        ref, it_ref = oracle.ppr_f64(adj, adj.out_deg(), seeds, tol=tols[q], max_iters=50)
        l1 = np.abs(R[q] - ref).sum() / np.abs(ref).sum()
        assert l1 <= 1e-5, (q, l1)
        assert abs(st.iterations[q] - it_ref) <= 1, (q, st.iterations[q], it_ref)
    # each query alone gives the same bits as in the batch
    for q in (0, 5, 11):
        Ra, sta = g.ppr([seed_lists[q]], tolerance=[tols[q]], max_iters=50)
        np.testing.assert_array_equal(Ra[0].view(np.uint32), R[q].view(np.uint32))
        assert sta.iterations[0] == st.iterations[q]


def test_ppr_single_query_path(case):
    # the plain one-query path (PageRank row kernel with a seed teleport)
    # against FP64, with repeated seeds counted by multiplicity
    name, n, pairs, rec, g, gu, adj, adju = case
    rng = np.random.default_rng(11)
    nz = np.nonzero(adj.out_deg() > 0)[0]
    for k, tol in ((1, 1e-4), (3, 1e-6), (8, 1e-7)):
        seeds = rng.choice(nz, size=k).astype(np.uint32)
        if k == 3:
            seeds[2] = seeds[0]
        ref, it_ref = oracle.ppr_f64(adj, adj.out_deg(), seeds, tol=tol, max_iters=50)
        got, st = g.ppr_single(seeds, tolerance=tol, max_iters=50)
        l1 = np.abs(got - ref).sum() / np.abs(ref).sum()
        assert l1 <= 1e-5, (k, l1)
        assert abs(st.iterations[0] - it_ref) <= 1, (k, st.iterations[0], it_ref)
    with pytest.raises(RuntimeError):
        g.ppr_single(np.arange(9, dtype=np.uint32))  # more than 8 distinct seeds


# ------------------------------------------------------------------ query server
@pytest.mark.parametrize("budget_slots,exclusive,gang", [(64, False, True), (3, False, True), (64, True, True),
                                                         (64, False, False)])
def test_server_results_equal_standalone(ctx, budget_slots, exclusive, gang):
    """Mixed BFS/SSSP/PPR queries arriving over several ticks: every result
    equals the same query run alone by the plain kernels."""
    import everythinggraph_gb300 as eg
    n, pairs, rec = load("rmat12")
    g = ctx.from_pairs(n, pairs, undirected=True).build(eg.CSR | eg.CSC)
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    per_slot = n * 4 * 3
    budget = 0 if budget_slots == 64 else (n * 8 * 4 + n * 8 * 2 + (n // 32) * 8 + n * 12 + n * 16 + 3 * budget_slots * per_slot)
    srv = eg.Server(g, hbm_budget=budget, weights_=w, keep_results=True, exclusive=exclusive, gang=gang)
    info = srv.info()
    if budget_slots != 64:
        assert info["bfs_slots"] < 64 and info["ppr_slots"] < 32
    rng = np.random.default_rng(11)
    nz = np.nonzero(np.diff(g.adj(eg.CSR)[0].astype(np.int64)) > 0)[0]
    queries = {}
    results = {}
    for wave in range(6):
        for _ in range(int(rng.integers(3, 9))):
            r = float(rng.random())
            if r < 0.6:
                src = int(rng.choice(nz))
                queries[srv.submit("bfs", source=src)] = ("bfs", src)
            elif r < 0.85:
                src = int(rng.choice(nz))
                queries[srv.submit("sssp", source=src)] = ("sssp", src)
            else:
                seeds = [int(x) for x in rng.choice(nz, size=int(rng.integers(1, 9)))]
                queries[srv.submit("ppr", seeds=seeds, tol=1e-6)] = ("ppr", seeds)
        for _ in range(int(rng.integers(1, 4))):
            srv.step()
            for res in srv.poll():
                results[res.id] = (res, srv.take_result())
    for _ in range(500):
        if srv.step() == 0:
            break
        for res in srv.poll():
            results[res.id] = (res, srv.take_result())
    for res in srv.poll():
        results[res.id] = (res, srv.take_result())
    assert set(results) == set(queries)
    for qid, (kind, arg) in queries.items():
        res, full = results[qid]
        if kind == "bfs":
            lv, st = g.bfs(arg)
            np.testing.assert_array_equal(full.view(np.int32), lv)
            assert res.reached == st.reached
        elif kind == "sssp":
            d, st = g.sssp(arg, w)
            np.testing.assert_array_equal(full, d)
            assert res.reached == st.reached
        else:
            R, st = g.ppr([arg], tolerance=1e-6)
            np.testing.assert_array_equal(full, R[0].view(np.uint32))
            assert res.iterations == st.iterations[0]
        assert res.arrival_s <= res.admit_s <= res.done_s
    srv.close()
    g.free()
