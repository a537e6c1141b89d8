"""Benchmark of the edge-traversal hot path on one GB300 (or N replicas).

Default workload (the BFS/WCC configuration): undirected RMAT scale 24,
edgefactor 16 (a=.57 b=.19 c=.19, seed 2), 16,777,216 vertices and
536,870,912 adjacency entries after symmetrisation; one step = BFS from 64
roots drawn uniformly from vertices with degree > 0 (seed 3), with int32
levels and parents, plus min-id WCC.  value = GTEPS = (sum over roots of the
out-degrees of reached vertices + input edges scanned by WCC) / step time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Inputs are larger than L2 (the CSR alone is
2.1 GB), so no L2 flush is done between steps.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"workload": "bfs64+wcc rmat24 undirected", "scale": 24, "edgefactor": 16, "seed": 2, "roots": 64,
            "root_seed": 3, "undirected": True}
METRIC, UNIT = "GTEPS", "GTEPS"
# DRAM bytes (read + write) of one row-kernel launch per CSC entry, from an
# ncu capture of PageRank on directed RMAT-22 (the kernel's traffic grows with
# the entries); the summary and its command are in
# profiles/k_coov_rows_pagerank_rmat22.md.
PR_ROWS_DRAM_BYTES_PER_ENTRY = (294.009e6 + 3.622e6) / 67108864


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.samples = []
        self.stop = threading.Event()
        self.index = index
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) == 6:
                    self.samples.append(f)
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


E2E_BATCH = 32  # roots per eg_bfs_batch call in the end-to-end step


def rank_reduce(x, op="max", device=None):
    """x reduced over the ranks of the default process group ("max" or
    "sum"); x itself without a group or with one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def replica_throughput(units, seconds, device=None):
    """Whole-job rate of independent replicas: the units every rank processed
    over the slowest rank's time, in 10^9 units per second; and that time."""
    total = rank_reduce(units, "sum", device)
    slowest = rank_reduce(seconds, "max", device)
    return total / slowest / 1e9, slowest


def run_ours(args):
    import torch

    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import build

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    build.build_lib()
    ctx = eg.Context(local)
    W = dict(WORKLOAD)
    if args.scale:
        W["scale"] = args.scale
    scale, ef = W["scale"], W["edgefactor"]
    n = 1 << scale
    m_in = ef * n
    # ---- load: host pairs -> device -> CSR/CSC (timed separately, like init())
    g = ctx.rmat(scale, m_in, W["seed"], undirected=True)
    t0 = time.perf_counter()
    g.build(eg.CSR | eg.CSC)
    build_ms = g.info().build_ms
    g.tune()  # row schedule and BFS level-loop form for this graph (untimed setup)
    roots = g.sample_roots(W["roots"], W["root_seed"])
    stream = torch.cuda.ExternalStream(ctx.stream)
    # the BFS level-loop form: the tuner's (default), or fixed (a profiler
    # slows per-level host round trips, so its own tuning would differ)
    bfs_form = {"auto": None, "graph": False, "host": True}[args.bfs_form]

    # host outputs of the end-to-end step: page-locked, allocated once and
    # reused by every call (what a serving process holds); eg_bfs_batch takes
    # E2E_BATCH roots per call and copies one root's levels and parents out
    # while it traverses the next
    lv_h = eg.pinned_empty(E2E_BATCH * n, np.int32)
    par_h = eg.pinned_empty(E2E_BATCH * n, np.int32)
    lab_h = eg.pinned_empty(n, np.int64)

    def step(copy_out):
        traversed = 0
        if copy_out:
            for c in range(0, len(roots), E2E_BATCH):
                _, _, sts = g.bfs_batch(roots[c:c + E2E_BATCH], parents=True, level_out=lv_h, parent_out=par_h,
                                        host_loop=bfs_form)
                traversed += sum(st.edges_traversed for st in sts)
        else:
            for r in roots:
                lv, par, st = g.bfs(int(r), parents=True, copy_out=False, host_loop=bfs_form)
                traversed += st.edges_traversed
        lab, wst = g.wcc(copy_out=copy_out, out=lab_h)
        return traversed + m_in, wst

    for _ in range(max(args.warmup, 0)):
        step(False)
    # ---- device-resident timed region
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    edges = 0
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            te, _ = step(False)
            edges += te
        e1.record(stream)
        torch.cuda.synchronize()
    launches = ctx.kernel_launches - l0
    # all ranks' edges over the slowest rank's device time
    value, slowest_s = replica_throughput(edges, e0.elapsed_time(e1) / 1e3, device="cuda")
    ms_step = slowest_s * 1e3 / args.steps
    # ---- end-to-end through the C ABI with host outputs (levels, parents, labels),
    # after one untimed step of its own (first use of the output slots and of
    # the page-locked buffers)
    step(True)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    te0 = time.perf_counter()
    e_edges = 0
    for _ in range(args.steps):
        te, _ = step(True)
        e_edges += te
    torch.cuda.synchronize()
    e2e_value, e2e_s = replica_throughput(e_edges, time.perf_counter() - te0, device="cuda")
    d2h = (W["roots"] * 2 * 4 * n + 8 * n)
    h2d = W["roots"] * 4
    # ---- per-kernel reports on the same graph size
    kernels = {}
    if not args.no_extras:
        try:
            kernels["msbfs_64_roots"] = msbfs_report(g, roots)
        except Exception as ex:  # reported, not fatal for the headline
            kernels["msbfs_64_roots"] = {"error": str(ex)}
        try:
            kernels["serve"] = serve_report(ctx, eg, scale, args.rate, args.queries, g=g, exclusive=args.serve_exclusive, gang=not args.serve_no_gang)
        except Exception as ex:
            kernels["serve"] = {"error": str(ex)}
        kernels.update(kernel_reports(ctx, eg, scale, args))
        for name, fn in (("spmv_er25", lambda: spmv_report(ctx, eg, 25 if scale >= 24 else scale, 32)),
                         ("sssp_rmat23_256", lambda: sssp_report(ctx, eg, 23 if scale >= 24 else scale - 1)),
                         ("ppr_32_queries", lambda: ppr_report(ctx, eg, scale))):
            try:
                kernels[name] = fn()
            except Exception as ex:
                kernels[name] = {"error": str(ex)}
    hbm, src = peaks()
    dom = kernels.get("pagerank_pull_rmat%d" % scale)
    roof = None
    if dom:
        roof = {"bound": "hbm", "achieved": dom["row_kernel_gbps"], "peak": hbm, "unit": "GB/s",
                "frac": dom["row_kernel_gbps"] / hbm,
                "traffic": PR_ROWS_DRAM_BYTES_PER_ENTRY * dom["m"] if PR_ROWS_DRAM_BYTES_PER_ENTRY else None,
                "kernel": "k_coov_rows<PrOp<0>, %d, %d> prefetch=%d min_blocks=%d (PageRank pull, RMAT-%d directed)"
                          % (dom["schedule"]["tile"], dom["schedule"]["per_lane"], dom["schedule"]["prefetch"],
                             dom["schedule"]["min_blocks"], scale),
                "algorithmic_bytes": dom["bytes_per_iter"], "peak_source": src}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (device RMAT generator)",
        "config": dict(W, n=n, m_adjacency=2 * m_in, l2="inputs larger than L2 (CSR 2.1 GB)",
                       parallelism="replicas" if world > 1 else "single"),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3 / args.steps, "host_buffers": "page-locked (eg_host_alloc), reused by every call",
                "api": "eg_bfs_batch (%d roots per call, copies overlapped with the next traversal) + eg_wcc" % E2E_BATCH},
        "gpu_launches": launches,
        "load": {"build_ms": build_ms, "bfs_tuning": g.bfs_tuning},
        "roofline": roof,
        "clocks": clk.summary(),
        "kernels": kernels,
    }
    if not args.no_cpu and rank == 0:
        out["cpu_baseline"] = cpu_baseline(g, eg, roots, n, m_in, args)
    g.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(out))


def kernel_reports(ctx, eg, scale, args):
    """PageRank pull on the directed RMAT graph of the same scale (10 iterations)."""
    import torch
    rep = {}
    n = 1 << scale
    m = 16 * n
    g = ctx.rmat(scale, m, 1).build(eg.CSR | eg.CSC)
    cands, chosen = g.tune()  # row-kernel schedule for this graph
    g.pagerank(iterations=3, copy_out=False)
    torch.cuda.synchronize()
    _, st = g.pagerank(iterations=10, copy_out=False)
    _, stg = g.pagerank(iterations=10, copy_out=False, use_graph=True)
    _, stg = g.pagerank(iterations=10, copy_out=False, use_graph=True)
    it_ms = st.ms / 10
    bytes_it = 8 * m + 16 * n
    rep["pagerank_pull_rmat%d" % scale] = {
        "ms_per_iter": it_ms, "gbps": bytes_it / (it_ms / 1e3) / 1e9, "gteps": m / (it_ms / 1e3) / 1e9,
        "row_kernel_ms": st.row_kernel_ms, "row_kernel_gbps": bytes_it / (st.row_kernel_ms / 1e3) / 1e9,
        "ms_per_iter_graph_replay": stg.ms / 10, "bytes_per_iter": bytes_it,
        "bytes_rule": "8 per CSC entry (column + gathered contribution) + 16 per vertex (row start, degree, rank and next-contribution writes)",
        "build_ms": g.info().build_ms, "m": m,
        "schedule": dict(cands[chosen], candidates=cands)}
    g.free()
    return rep


def spmv_report(ctx, eg, log_n=25, degree=32):
    """SpMV over an Erdos-Renyi graph (2^25 vertices, 32 out-edges each, seed 4):
    fp32 values U[0,1) hashed from the endpoints, x U[0,1) (seed 11); fp32,
    fp32 two-sum and fp64, with max-relative and L1 error against fp64 (x is
    larger than 2^24 vertices, so the source-blocked CSC is used: two passes
    over x slices L2 holds; its build is timed apart); the 64x64 grid layout
    built on the device beside it."""
    import oracle
    n = 1 << log_n
    m = degree * n
    g = ctx.er(n, m, 4).build(eg.CSR | eg.CSC)
    g.tune()  # row-kernel schedule for this graph (untimed setup)
    x = oracle.uniform_f32(n, 11)
    y64, _ = g.spmv(x, "f64", value_seed=9)
    out = {"workload": "ER n=2^%d m=%d" % (log_n, m), "build_ms": g.info().build_ms}
    nz = y64 != 0
    for kind in ("f32", "f32_comp", "f64"):
        g.spmv(x, kind, value_seed=9, copy_out=False)
        y, ms = g.spmv(x, kind, value_seed=9)
        bytes_ = 12 * m + (16 if kind == "f64" else 12) * n
        rec = {"ms": ms, "gbps": bytes_ / (ms / 1e3) / 1e9, "gflops": 2 * m / (ms / 1e3) / 1e9}
        if kind != "f64":
            d = np.abs(y.astype(np.float64) - y64)
            rec["max_rel_err"] = float((d[nz] / np.abs(y64[nz])).max())
            rec["l1_rel_err"] = float(d.sum() / np.abs(y64).sum())
        out[kind] = rec
    # PageRank over the same graph, 10 iterations
    _, st = g.pagerank(iterations=10, copy_out=False)
    out["pagerank_ms_per_iter"] = st.ms / 10
    # the 64 x 64 grid layout and the grid kernels (cells in L2-sized blocks)
    import time as _t
    t0 = _t.perf_counter()
    g.build_grid(64)
    out["grid64_build_s"] = _t.perf_counter() - t0
    grid = {}
    for kind in ("f32", "f64"):
        g.spmv(x, kind, value_seed=9, copy_out=False, grid=True)
        y, ms = g.spmv(x, kind, value_seed=9, grid=True)
        bytes_ = 12 * m + (16 if kind == "f64" else 12) * n
        rec = {"ms": ms, "gbps": bytes_ / (ms / 1e3) / 1e9}
        if kind == "f32":
            d = np.abs(y.astype(np.float64) - y64)
            rec["max_rel_err"] = float((d[nz] / np.abs(y64[nz])).max())
            rec["l1_rel_err"] = float(d.sum() / np.abs(y64).sum())
        grid[kind] = rec
    _, st = g.pagerank(iterations=10, copy_out=False, grid=True)
    grid["pagerank_ms_per_iter"] = st.ms / 10
    out["grid64"] = grid
    g.free()
    return out


def sssp_report(ctx, eg, scale=23, k=256, singles=16):
    """Batched SSSP on RMAT-23 (seed 5), u32 weights U[1,255] hashed from the
    endpoints: k sources in one batch versus single-source launches (a sample
    of `singles`, scaled to k)."""
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 5).build(eg.CSR)
    roots = g.sample_roots(k, 6)
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    g.sssp_multi(roots[:8], w, copy_out=False)
    _, stb = g.sssp_multi(roots, w, copy_out=False)
    t1 = 0.0
    for r in roots[:singles]:
        _, st = g.sssp(int(r), w, copy_out=False)
        t1 += st.ms
    per_single = t1 / singles
    wf = eg.weights("f32", seed=6)
    _, stf = g.sssp_multi(roots, wf, copy_out=False)
    g.free()
    return {"workload": "rmat%d, %d sources" % (scale, k), "batched_ms": stb.ms, "single_ms_each": per_single,
            "runs_per_s_batched": k / (stb.ms / 1e3), "runs_per_s_single": 1e3 / per_single,
            "speedup": per_single * k / stb.ms, "rounds_batched": stb.rounds,
            "gteps_batched": stb.relaxations / (stb.ms / 1e3) / 1e9,
            "f32_weights_batched_ms": stf.ms, "f32_rounds_batched": stf.rounds}


def msbfs_report(g, roots):
    """Bit-sliced BFS of all roots in one batch versus the same roots one by one."""
    g.bfs_multi(roots[:4], copy_out=False)
    _, stm = g.bfs_multi(roots, copy_out=False)
    t1 = 0.0
    for r in roots[:16]:
        _, st = g.bfs(int(r), copy_out=False)
        t1 += st.ms
    per_single = t1 / 16
    return {"batched_ms": stm.ms, "single_ms_each": per_single, "gteps_batched": stm.edges_traversed / (stm.ms / 1e3) / 1e9,
            "speedup": per_single * len(roots) / stm.ms}


def serve_report(ctx, eg, scale, rate, nq, seed=7, plain_sample=40, g=None, exclusive=False, gang=True):
    """Serving workload: Poisson arrivals at `rate` qps of 60% BFS, 25% SSSP
    (u32 weights U[1,255]), 15% personalised PageRank (1-8 seeds, tolerance
    10^U(-7,-4), <= 50 iterations) on the resident undirected RMAT graph;
    p50/p99 latency (arrival -> completion) and QPS, next to the QPS of the
    plain one-query-at-a-time kernels on a sample of the same queries (BFS:
    the direction-optimising BFS; SSSP: the single-source frontier
    Bellman-Ford; PPR: the PageRank row kernel with a seed teleport)."""
    import torch
    n = 1 << scale
    own = g is None
    if own:
        g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
    od, _ = g.degrees(True, False)
    nz = np.nonzero(od > 0)[0].astype(np.uint32)
    rng = np.random.default_rng(seed)
    kinds = rng.choice(3, size=nq, p=[0.60, 0.25, 0.15])
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=nq))
    qs = []
    for i in range(nq):
        if kinds[i] == 0:
            qs.append(("bfs", int(rng.choice(nz)), None, 0.0))
        elif kinds[i] == 1:
            qs.append(("sssp", int(rng.choice(nz)), None, 0.0))
        else:
            k = int(rng.integers(1, 9))
            qs.append(("ppr", 0, [int(x) for x in rng.choice(nz, size=k)], float(10 ** rng.uniform(-7, -4))))
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    srv = eg.Server(g, hbm_budget=64 << 30, weights_=w, exclusive=exclusive, gang=gang)
    torch.cuda.synchronize()
    t_start = srv.info()["clock_s"]
    arrivals = arrivals + t_start
    done = []
    i = 0
    while len(done) < nq:
        now = srv.info()["clock_s"]
        while i < nq and arrivals[i] <= now:
            kind, src, seeds, tol = qs[i]
            if kind == "ppr":
                srv.submit("ppr", seeds=seeds, tol=tol, arrival=float(arrivals[i]))
            else:
                srv.submit(kind, source=src, arrival=float(arrivals[i]))
            i += 1
        active = srv.step()
        done.extend(srv.poll())
        if active == 0 and i < nq:  # idle: wait for the next arrival
            time.sleep(max(0.0, min(0.001, arrivals[i] - srv.info()["clock_s"])))
    info = srv.info()
    info["stats"] = srv.stats()
    srv.close()
    lat = np.array([r.done_s - r.arrival_s for r in done]) * 1e3
    span = max(r.done_s for r in done) - arrivals[0]
    # plain kernels, one query at a time, on a sample of the same mix
    samp = list(range(min(plain_sample, nq)))
    t0 = time.perf_counter()
    for j in samp:
        kind, src, seeds, tol = qs[j]
        if kind == "bfs":
            g.bfs(src, copy_out=False)
        elif kind == "sssp":
            g.sssp(src, w, copy_out=False)
        else:
            g.ppr_single(seeds, tolerance=tol, copy_out=False)
    plain_qps = len(samp) / (time.perf_counter() - t0)
    if own:
        g.free()
    qps = nq / span
    return {"workload": "serve rmat%d undirected, %d queries, Poisson %g qps offered" % (scale, nq, rate),
            "engines": "exclusive" if exclusive else "concurrent", "sssp_gang": gang,
            "qps": qps, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "plain_qps": plain_qps, "speedup_vs_plain": qps / plain_qps, "slots": info}


def cpu_baseline(g, eg, roots, n, m_in, args):
    """The multi-threaded CPU port of the reference loops (bfs_simple's
    direction-optimising iterator, wcc's label propagation) on a bounded
    sample of the same step: the first roots that fit in ~15 s plus one WCC,
    on the same graph copied to the host."""
    import oracle
    oracle.build()
    ptr, col = g.adj(eg.CSR)
    return cpu_sample(oracle, ptr, col, roots, m_in, budget_s=15.0)


def cpu_sample(oracle, ptr, col, roots, m_in, budget_s):
    od = np.diff(ptr.astype(np.int64))
    t0 = time.perf_counter()
    comp, rounds = oracle.wcc_lp(ptr, col)
    edges = m_in
    k = 0
    for r in roots:
        lv = oracle.bfs_do(ptr, col, ptr, col, int(r))
        edges += int(od[lv > 0].sum())
        k += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": edges / dt / 1e9, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": "WCC + %d of %d BFS roots on the same graph (OpenMP port of bfs_simple/wcc loops), %.1f s"
                      % (k, len(roots), dt)}


def run_reference(args):
    """CPU arm: the reference's loops (OpenMP port; the reference sources are
    not available on the GPU host) on the same workload, all host threads.
    Each step is a bounded sample: WCC plus the first roots that fit ~20 s."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    W = dict(WORKLOAD)
    if args.scale:
        W["scale"] = args.scale
    scale = W["scale"]
    n = 1 << scale
    m_in = W["edgefactor"] * n
    pairs = oracle.rmat_edges(scale, m_in, W["seed"])
    adj = oracle.build_adj(n, pairs, undirected=True)
    del pairs
    roots = oracle.sample_roots(adj.out_deg(), W["roots"], W["root_seed"])
    for _ in range(max(args.warmup, 0)):
        cpu_sample(oracle, adj.out_ptr, adj.out_col, roots[:1], m_in, budget_s=0.0)
    vals, samples = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = cpu_sample(oracle, adj.out_ptr, adj.out_col, roots, m_in, budget_s=20.0)
        vals.append(r["value"])
        samples.append(r["sample"])
    dt = time.perf_counter() - t0
    value = float(np.mean(vals))
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / max(args.steps, 1) * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
           "data": "synthetic (CPU RMAT generator, same edges as the GPU arm)",
           "config": dict(W, n=n, m_adjacency=2 * m_in),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                            "sample": samples[-1] if samples else ""},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def ppr_report(ctx, eg, scale=24, nq=32, seed=7):
    """Personalised PageRank on the undirected RMAT graph: nq queries (1-8
    seeds, tolerance 1e-6, <= 50 iterations) in one 32-lane batch versus the
    same queries one at a time on the PageRank row kernel."""
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
    od, _ = g.degrees(True, False)
    nz = np.nonzero(od > 0)[0]
    rng = np.random.default_rng(seed)
    seeds = [rng.choice(nz, int(rng.integers(1, 9))).astype(np.uint32) for _ in range(nq)]
    g.ppr(seeds[:2], tolerance=1e-6, copy_out=False)
    _, stb = g.ppr(seeds, tolerance=1e-6, max_iters=50, copy_out=False)
    t1, its = 0.0, 0
    for sd in seeds[:8]:
        _, st = g.ppr_single(sd, tolerance=1e-6, max_iters=50, copy_out=False)
        t1 += st.ms
        its += st.sweeps
    g.free()
    per_single = t1 / 8
    return {"workload": "ppr rmat%d undirected, %d queries" % (scale, nq), "batched_ms": stb.ms,
            "sweeps": stb.sweeps, "ms_per_sweep": stb.ms / max(stb.sweeps, 1), "single_ms_each": per_single,
            "single_iters_each": its / 8, "speedup": per_single * nq / stb.ms}


def bfs_report(ctx, eg, scale=24, roots=16):
    """Single-source BFS (levels + parents) on the undirected RMAT graph: the
    CUDA-graph level loop and the host-driven loop (the same kernels launched
    level by level, which a profiler can capture one by one), plus WCC."""
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
    rs = g.sample_roots(roots, 3)
    out = {"workload": "bfs rmat%d undirected, %d roots" % (scale, roots)}
    for name, host_loop in (("graph_loop", False), ("host_loop", True)):
        g.bfs(int(rs[0]), parents=True, copy_out=False, host_loop=host_loop)
        ms, te, lv, pl = 0.0, 0, 0, 0
        for r in rs:
            _, _, st = g.bfs(int(r), parents=True, copy_out=False, host_loop=host_loop)
            ms += st.ms
            te += st.edges_traversed
            lv += st.levels
            pl += st.pull_levels
        out[name] = {"ms_per_bfs": ms / roots, "gteps": te / (ms / 1e3) / 1e9, "levels": lv / roots,
                     "pull_levels": pl / roots}
    g.wcc(copy_out=False)
    _, st = g.wcc(copy_out=False)
    out["wcc"] = {"ms": st.ms, "components": st.components, "rounds": st.rounds}
    g.free()
    return out


def only_report(name, args):
    """One report alone (profiling and quick checks)."""
    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import build
    build.build_lib()
    ctx = eg.Context(0)
    scale = args.scale or 24
    if name == "serve":
        out = serve_report(ctx, eg, scale, args.rate, args.queries, exclusive=args.serve_exclusive, gang=not args.serve_no_gang)
    elif name == "pr":
        out = kernel_reports(ctx, eg, scale, args)
    elif name == "spmv":
        out = spmv_report(ctx, eg, args.scale or 25, 32)
    elif name == "sssp":
        out = sssp_report(ctx, eg, args.scale or 23)
    elif name == "ppr":
        out = ppr_report(ctx, eg, scale)
    elif name == "bfs":
        out = bfs_report(ctx, eg, scale)
    else:  # msbfs
        n = 1 << scale
        g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
        out = msbfs_report(g, g.sample_roots(64, 3))
        g.free()
    print(json.dumps(out))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=0)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--bfs-form", choices=["auto", "graph", "host"], default="auto",
                    help="BFS level loop: the form eg_graph_tune keeps (auto), or a fixed one")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--pr-only", action="store_true", help="only the PageRank pull report (profiling)")
    ap.add_argument("--serve-only", action="store_true", help="only the serving report")
    ap.add_argument("--only", choices=["pr", "spmv", "sssp", "msbfs", "ppr", "bfs", "serve"],
                    help="only one kernel report (profiling)")
    ap.add_argument("--rate", type=float, default=20000.0)
    ap.add_argument("--queries", type=int, default=1000)
    ap.add_argument("--serve-no-gang", action="store_true",
                    help="query server admits SSSP queries into any free slot instead of 32-source gangs")
    ap.add_argument("--serve-exclusive", action="store_true",
                    help="query server runs one engine step at a time instead of overlapping them")
    args = ap.parse_args()
    if args.only or args.serve_only or args.pr_only:
        only_report(args.only or ("serve" if args.serve_only else "pr"), args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
