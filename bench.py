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
# the entries).
PR_ROWS_DRAM_BYTES_PER_ENTRY = (294.009e6 + 3.622e6) / 67108864
# the same for the partition kernel (k_pcol_rows), from a one-pass capture
# on directed RMAT-24 itself
PR_PCOL_DRAM_BYTES_PER_ENTRY = (1290.110208e6 + 41.027584e6) / 268435456


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
    eb = args.e2e_batch
    lv_h = eg.pinned_empty(eb * n, np.int32)
    par_h = eg.pinned_empty(eb * n, np.int32)
    lab_h = eg.pinned_empty(n, np.int64)

    def step(copy_out):
        traversed = 0
        if copy_out:
            for c in range(0, len(roots), eb):
                _, _, sts = g.bfs_batch(roots[c:c + eb], parents=True, level_out=lv_h, parent_out=par_h,
                                        host_loop=bfs_form)
                traversed += sum(st.edges_traversed for st in sts)
        else:
            for r in roots:
                lv, par, st = g.bfs(int(r), parents=True, copy_out=False, host_loop=bfs_form)
                traversed += st.edges_traversed
        lab, wst = g.wcc(copy_out=copy_out, out=lab_h)
        return traversed + m_in, traversed

    for _ in range(max(args.warmup, 0)):
        step(False)
    # ---- device-resident timed region
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    edges = bfs_entries = 0
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            te, tb = step(False)
            edges += te
            bfs_entries += tb
        e1.record(stream)
        torch.cuda.synchronize()
    launches = ctx.kernel_launches - l0
    # all ranks' edges over the slowest rank's device time
    value, slowest_s = replica_throughput(edges, e0.elapsed_time(e1) / 1e3, device="cuda")
    ms_step = slowest_s * 1e3 / args.steps
    # Graph500 counts each undirected edge of the traversed component once:
    # half the adjacency entries the BFS runs traverse (+ WCC's input edges)
    g500 = (bfs_entries / 2 + (edges - bfs_entries)) / (edges / value) if edges else 0.0
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
        # run in this order; printed with the serving and PageRank reports last
        # (the end of the line is what a log tail keeps)
        for name, fn in (("msbfs64", lambda: msbfs_report(g, roots)),
                         ("serve", lambda: serve_sweep(ctx, eg, scale, args, g)),
                         ("pr", lambda: kernel_reports(ctx, eg, scale, args)),
                         ("spmv_er25", lambda: spmv_report(ctx, eg, 25 if scale >= 24 else scale, 32)),
                         ("sssp_rmat23_256", lambda: sssp_report(ctx, eg, 23 if scale >= 24 else scale - 1)),
                         ("ppr32", lambda: ppr_report(ctx, eg, scale))):
            try:
                kernels[name] = fn()
            except Exception as ex:  # reported, not fatal for the headline
                kernels[name] = {"error": str(ex)[:200]}
        if "pr" in kernels and "error" not in kernels["pr"]:
            kernels.update(kernels.pop("pr"))
        order = ["spmv_er25", "sssp_rmat23_256", "ppr32", "msbfs64", "pr_rmat%d" % scale, "serve"]
        kernels = {k: kernels[k] for k in order + [k for k in kernels if k not in order] if k in kernels}
    hbm, src = peaks()
    dom = kernels.get("pr_rmat%d" % scale)
    roof = None
    if dom and "row_ms" in dom:
        gbps = dom["bytes"] / (dom["row_ms"] / 1e3) / 1e9
        pcol = dom["sched"].startswith("partitions")
        per_entry = PR_PCOL_DRAM_BYTES_PER_ENTRY if pcol else PR_ROWS_DRAM_BYTES_PER_ENTRY
        kname = ("k_pcol_rows<PrOp<0>,%s>" % dom["sched"].split()[1].rstrip(",").split("^")[1] if pcol
                 else "k_coov_rows<PrOp<0>,%s>" % dom["sched"])
        roof = {"bound": "hbm", "achieved": r4(gbps), "peak": hbm, "unit": "GB/s", "frac": r4(gbps / hbm),
                "traffic": r4(per_entry * dom["m"]) if per_entry else None,
                "kernel": "%s (PageRank pull, RMAT-%d directed)" % (kname, scale),
                "algorithmic_bytes": dom["bytes"], "peak_source": src}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (device RMAT generator)",
        "config": dict(W, n=n, m_adjacency=2 * m_in, l2="inputs larger than L2 (CSR 2.1 GB)",
                       parallelism="replicas" if world > 1 else "single",
                       edges_counted="BFS: out-degrees of reached vertices; WCC: the input edges"),
        "graph500_gteps": r4(g500),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3 / args.steps,
                "api": "eg_bfs_batch x%d roots/call into page-locked buffers + eg_wcc" % eb},
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clk.summary(),
    }
    if not args.no_cpu and rank == 0:
        cb, parity = cpu_baseline(g, eg, roots, n, m_in, args, lv_h, par_h, lab_h, eb)
        out["cpu_baseline"] = cb
        out["parity"] = parity
    out["load_build_ms"] = r4(build_ms)
    out["kernels"] = kernels
    g.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(out, separators=(",", ":")))


def r4(x):
    """x to 4 significant digits (keeps the JSON line short)."""
    return float("%.4g" % x) if x is not None else None


class _Csc:
    """The in-lists the FP64 PageRank oracle reads (n, in_ptr, in_col)."""

    def __init__(self, n, ptr, col):
        self.n, self.in_ptr, self.in_col = n, ptr, col


def rel_errors(got, ref):
    """(relative L1, max relative) error of got against the FP64 ref."""
    got = got.astype(np.float64)
    d = np.abs(got - ref)
    nz = ref != 0
    return r4(d.sum() / np.abs(ref).sum()), r4((d[nz] / np.abs(ref[nz])).max())


def kernel_reports(ctx, eg, scale, args):
    """PageRank pull on the directed RMAT graph of the same scale (seed 1):
    10 iterations from 1/n after eg_graph_tune; relative L1 and max relative
    error of the ranks against the CPU FP64 oracle run on the same in-lists."""
    import oracle
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
    rank, _ = g.pagerank(iterations=10)
    it_ms = st.ms / 10
    bytes_it = 8 * m + 16 * n
    c = cands[chosen]
    rec = {"ms_iter": r4(it_ms), "ms_iter_graph": r4(stg.ms / 10), "row_ms": r4(st.row_kernel_ms),
           "row_gbps": r4(bytes_it / (st.row_kernel_ms / 1e3) / 1e9), "gteps": r4(m / (it_ms / 1e3) / 1e9),
           "bytes": bytes_it, "m": m,
           "sched": ("partitions 2^%d, %d-entry chunks" % (c["partition_log2"], c["tile"]) if c["partition_log2"]
                     else "%d,%d pf%d mb%d ch%d" % (c["tile"], c["per_lane"], c["prefetch"], c["min_blocks"],
                                                    c["cache_hint"])),
           "cand_ms": [round(x["ms"], 3) for x in cands]}
    try:
        oracle.build()
        ptr, col = g.adj(eg.CSC)
        od, _ = g.degrees(True, False)
        ref = oracle.pagerank_f64(_Csc(n, ptr, col), od, 1.0 / n, 10)
        rec["l1_err"], rec["max_rel_err"] = rel_errors(rank, ref)
        rec["err_vs"] = "CPU FP64 oracle"
    except Exception as ex:
        rec["err"] = str(ex)[:120]
    g.free()
    rep["pr_rmat%d" % scale] = rec
    return rep


def spmv_report(ctx, eg, log_n=25, degree=32):
    """SpMV over an Erdos-Renyi graph (2^25 vertices, 32 out-edges each, seed 4):
    fp32 values U[0,1) hashed from the endpoints, x U[0,1) (seed 11); fp32,
    fp32 two-sum and fp64, with max-relative and L1 error against the CPU
    FP64 oracle over the same in-lists (x is larger than 2^24 vertices, so the
    source-blocked CSC is used: two passes over x slices L2 holds); PageRank
    over the same graph; the 64x64 grid layout built on the device beside it."""
    import oracle
    n = 1 << log_n
    m = degree * n
    g = ctx.er(n, m, 4).build(eg.CSR | eg.CSC)
    g.tune()  # row-kernel schedule for this graph (untimed setup)
    x = oracle.uniform_f32(n, 11)
    oracle.build()
    ptr, col = g.adj(eg.CSC)
    y64 = oracle.spmv_f64_hashed(n, ptr, col, 9, x)
    del ptr, col
    out = {}
    for kind in ("f32", "f32_comp", "f64"):
        g.spmv(x, kind, value_seed=9, copy_out=False)
        y, ms = g.spmv(x, kind, value_seed=9)
        bytes_ = 12 * m + (16 if kind == "f64" else 12) * n
        rec = {"ms": r4(ms), "gbps": r4(bytes_ / (ms / 1e3) / 1e9)}
        if kind != "f64":  # (the fp64 path is the FP64 oracle's own arithmetic)
            rec["l1_err"], rec["max_rel_err"] = rel_errors(y, y64)
        out[kind] = rec
    _, st = g.pagerank(iterations=10, copy_out=False)
    out["pr_ms_iter"] = r4(st.ms / 10)
    # the 64 x 64 grid layout and the grid kernels
    t0 = time.perf_counter()
    g.build_grid(64)
    out["grid64_build_s"] = r4(time.perf_counter() - t0)
    gr = {}
    for mode, tag in ((True, ""), ("cells", "cells_")):  # fixed-order row kernel; cell kernel (atomics)
        g.spmv(x, "f32", value_seed=9, copy_out=False, grid=mode)
        y, ms = g.spmv(x, "f32", value_seed=9, grid=mode)
        gr[tag + "f32_ms"] = r4(ms)
        gr[tag + "f32_gbps"] = r4((12 * m + 12 * n) / (ms / 1e3) / 1e9)
        gr[tag + "l1_err"], gr[tag + "max_rel_err"] = rel_errors(y, y64)
        _, st = g.pagerank(iterations=10, copy_out=False, grid=mode, deg_multiplier=2, prev_init=0.15)
        gr[tag + "pr_ms_iter"] = r4(st.ms / 10)
    out["grid64"] = gr
    g.free()
    return out


def sssp_report(ctx, eg, scale=23, k=256, singles=16):
    """Batched SSSP on RMAT-23 (seed 5), u32 weights U[1,255] hashed from the
    endpoints: k sources in one batch versus single-source launches (a sample
    of `singles`, scaled to k); fp32 weights batched."""
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
    return {"batch_ms": r4(stb.ms), "single_ms": r4(per_single), "speedup": r4(per_single * k / stb.ms),
            "rounds": stb.rounds, "f32_batch_ms": r4(stf.ms)}


def msbfs_report(g, roots):
    """Bit-sliced BFS of all roots in one batch versus the same roots one by one."""
    g.bfs_multi(roots[:4], copy_out=False)
    _, stm = g.bfs_multi(roots, copy_out=False)
    t1 = 0.0
    for r in roots[:16]:
        _, st = g.bfs(int(r), copy_out=False)
        t1 += st.ms
    per_single = t1 / 16
    return {"batch_ms": r4(stm.ms), "single_ms": r4(per_single), "speedup": r4(per_single * len(roots) / stm.ms)}


def serve_queries(nz, nq, rate, seed):
    """The serving mix: arrival times (Poisson at `rate`) and queries, 60% BFS,
    25% SSSP, 15% personalised PageRank (1-8 seeds, tolerance 10^U(-7,-4))."""
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
    return arrivals, qs


def serve_run(eg, g, w, arrivals, qs, exclusive=False, gang=True):
    """Offers the queries at their arrival times to a fresh server; returns
    (latencies in ms, span in s from the first arrival to the last completion)."""
    import torch
    nq = len(qs)
    srv = eg.Server(g, hbm_budget=64 << 30, weights_=w, exclusive=exclusive, gang=gang)
    torch.cuda.synchronize()
    t_start = srv.info()["clock_s"]
    arr = arrivals - arrivals[0] + t_start
    done = []
    i = 0
    while len(done) < nq:
        now = srv.info()["clock_s"]
        while i < nq and arr[i] <= now:
            kind, src, seeds, tol = qs[i]
            if kind == "ppr":
                srv.submit("ppr", seeds=seeds, tol=tol, arrival=float(arr[i]))
            else:
                srv.submit(kind, source=src, arrival=float(arr[i]))
            i += 1
        active = srv.step()
        done.extend(srv.poll())
        if active == 0 and i < nq:  # idle: wait for the next arrival
            time.sleep(max(0.0, min(0.001, arr[i] - srv.info()["clock_s"])))
    srv.close()
    lat = np.array([r.done_s - r.arrival_s for r in done]) * 1e3
    kinds = np.array([r.kind for r in done])
    return lat, max(r.done_s for r in done) - arr[0], kinds


def plain_qps(g, w, qs):
    """The plain one-query-at-a-time kernels on the same queries: BFS (the
    direction-optimising BFS), SSSP (single-source frontier Bellman-Ford),
    PPR (the PageRank row kernel with a seed teleport)."""
    t0 = time.perf_counter()
    for kind, src, seeds, tol in qs:
        if kind == "bfs":
            g.bfs(src, copy_out=False)
        elif kind == "sssp":
            g.sssp(src, w, copy_out=False)
        else:
            g.ppr_single(seeds, tolerance=tol, copy_out=False)
    return len(qs) / (time.perf_counter() - t0)


def serve_sweep(ctx, eg, scale, args, g):
    """The serving workload on the resident undirected RMAT graph at several
    offered Poisson rates (seed 7): per rate QPS achieved and p50/p99 latency
    (arrival to completion); the plain one-query-at-a-time kernels' QPS on
    a sample of the same queries."""
    od, _ = g.degrees(True, False)
    nz = np.nonzero(od > 0)[0].astype(np.uint32)
    w = eg.weights("hash", seed=6, lo=1, hi=255)
    rates = [float(r) for r in args.rates.split(",")] if args.rates else [args.rate]
    out = {"rates": []}
    for rate in rates:
        nq = int(min(args.queries, max(200, rate * args.serve_seconds)))
        arrivals, qs = serve_queries(nz, nq, rate, 7)
        lat, span, kinds = serve_run(eg, g, w, arrivals, qs, exclusive=args.serve_exclusive,
                                     gang=not args.serve_no_gang)
        # p50 per query kind: BFS, SSSP, PPR
        p50k = [r4(np.percentile(lat[kinds == k], 50)) if np.any(kinds == k) else None for k in (1, 2, 3)]
        out["rates"].append({"offered": rate, "n": nq, "qps": r4(nq / span), "p50_ms": r4(np.percentile(lat, 50)),
                             "p99_ms": r4(np.percentile(lat, 99)), "p50_bfs_sssp_ppr": p50k})
    _, qs = serve_queries(nz, args.plain_sample, 1000.0, 7)
    out["plain_qps"] = r4(plain_qps(g, w, qs))
    best = max(r["qps"] for r in out["rates"])
    out["max_qps_vs_plain"] = r4(best / out["plain_qps"])
    return out


def cpu_baseline(g, eg, roots, n, m_in, args, lv_h=None, par_h=None, lab_h=None, eb=E2E_BATCH):
    """The multi-threaded CPU port of the reference loops (bfs_simple's
    direction-optimising iterator, wcc's label propagation) on a bounded
    sample of the same step: the first roots that fit in ~15 s plus one WCC,
    on the same graph copied to the host.  Outside the CPU timing, the GPU's
    last end-to-end outputs (levels and parents of the last `eb` roots,
    WCC labels, in the page-locked buffers) are compared with the port's:
    levels and labels bit for bit, parents as a BFS tree."""
    import oracle
    oracle.build()
    ptr, col = g.adj(eg.CSR)
    first = len(roots) - eb
    par = {"bfs_roots_checked": 0, "bfs_levels_bit_exact": True, "bfs_trees_valid": True}

    def check(i, r, lv):
        if lv_h is None or i < first:
            return
        j = i - first
        par["bfs_roots_checked"] += 1
        par["bfs_levels_bit_exact"] &= bool(np.array_equal(lv, lv_h[j * n:(j + 1) * n]))
        if par["bfs_roots_checked"] <= 4:
            par["bfs_trees_valid"] &= oracle.bfs_tree_check(n, ptr, col, int(r), lv_h[j * n:(j + 1) * n],
                                                            par_h[j * n:(j + 1) * n]) == 0

    cb, comp = cpu_sample(oracle, ptr, col, roots, m_in, budget_s=15.0, check=check)
    if lab_h is not None:
        par["wcc_bit_exact"] = bool(np.array_equal(comp, lab_h))
    par["vs"] = "CPU port (bfs_do, wcc_lp) on the GPU's CSR"
    return cb, par


def cpu_sample(oracle, ptr, col, roots, m_in, budget_s, check=None):
    """WCC plus BFS from the roots in turn until budget_s of CPU time; only the
    oracle calls are timed.  Returns (the cpu_baseline record, WCC labels)."""
    od = np.diff(ptr.astype(np.int64))
    t0 = time.perf_counter()
    comp, rounds = oracle.wcc_lp(ptr, col)
    dt = time.perf_counter() - t0
    edges = m_in
    k = 0
    for i, r in enumerate(roots):
        t0 = time.perf_counter()
        lv = oracle.bfs_do(ptr, col, ptr, col, int(r))
        dt += time.perf_counter() - t0
        edges += int(od[lv > 0].sum())
        k += 1
        if check:
            check(i, r, lv)
        if dt > budget_s:
            break
    return ({"value": edges / dt / 1e9, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
             "sample": "WCC + %d of %d BFS roots on the same graph (OpenMP port of bfs_simple/wcc loops), %.1f s"
                       % (k, len(roots), dt)}, comp)


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
        r, _ = cpu_sample(oracle, adj.out_ptr, adj.out_col, roots, m_in, budget_s=20.0)
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
    return {"batch_ms": r4(stb.ms), "sweeps": stb.sweeps, "single_ms": r4(per_single),
            "single_iters": r4(its / 8), "speedup": r4(per_single * nq / stb.ms)}


def cache_report(ctx, eg, scale=24, path=None):
    """The layout cache on the undirected RMAT graph: device build (CSR +
    CSC) against writing the layouts to a file and filling a fresh graph
    from it."""
    import tempfile
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
    build_ms = g.info().build_ms
    d = tempfile.mkdtemp()
    path = path or os.path.join(d, "g.eglayout")
    t0 = time.perf_counter()
    g.save_layouts(path)
    save_s = time.perf_counter() - t0
    size = os.path.getsize(path)
    h = ctx.rmat(scale, 16 * n, 2, undirected=True)
    t0 = time.perf_counter()
    hit = h.load_layouts(path)
    load_s = time.perf_counter() - t0
    same = bool(np.array_equal(g.adj(eg.CSR)[1], h.adj(eg.CSR)[1]))
    g.free()
    h.free()
    os.remove(path)
    os.rmdir(d)
    return {"build_ms": r4(build_ms), "file_gb": r4(size / 1e9), "save_s": r4(save_s), "load_s": r4(load_s),
            "hit": hit, "same_csr": same}


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
        n = 1 << scale
        g = ctx.rmat(scale, 16 * n, 2, undirected=True).build(eg.CSR | eg.CSC)
        g.tune()
        out = serve_sweep(ctx, eg, scale, args, g)
        g.free()
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
    elif name == "cache":
        out = cache_report(ctx, eg, scale)
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
    ap.add_argument("--e2e-batch", type=int, default=E2E_BATCH, help="roots per eg_bfs_batch call in the end-to-end step")
    ap.add_argument("--pr-only", action="store_true", help="only the PageRank pull report (profiling)")
    ap.add_argument("--serve-only", action="store_true", help="only the serving report")
    ap.add_argument("--only", choices=["pr", "spmv", "sssp", "msbfs", "ppr", "bfs", "serve", "cache"],
                    help="only one kernel report (profiling)")
    ap.add_argument("--rate", type=float, default=20000.0, help="offered rate when --rates is empty")
    ap.add_argument("--rates", default="100,250,1000,5000,50000",
                    help="comma-separated offered Poisson rates (qps) of the serving sweep")
    ap.add_argument("--serve-seconds", type=float, default=2.0,
                    help="offered arrival span per rate (queries = rate x seconds, 200..--queries)")
    ap.add_argument("--queries", type=int, default=1500, help="most queries per offered rate")
    ap.add_argument("--plain-sample", type=int, default=40,
                    help="queries of the same mix run one at a time on the plain kernels")
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
