"""Host logic of the N-replica bench (one process per GPU, no data-path
collective) on CPU: two gloo ranks, as torchrun would launch them.

The whole-job rate is every rank's units over the slowest rank's time; only
rank 0 runs the CPU reference arm.  No GPU is used."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["EG_ROOT"])
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"])
dist.init_process_group("gloo", init_method="env://")
# rank r processed (r + 1) * 10^9 units in (1 + r) seconds
value, slowest = bench.replica_throughput((rank + 1) * 1e9, 1.0 + rank)
mx = bench.rank_reduce(5.0 * (rank + 1), "max")
sm = bench.rank_reduce(5.0 * (rank + 1), "sum")
print(json.dumps({"rank": rank, "value": value, "slowest": slowest, "max": mx, "sum": sm}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_throughput_two_gloo_ranks():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), EG_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        # 3e9 units over the slowest rank's 2 s
        assert o["value"] == pytest.approx(1.5)
        assert o["slowest"] == pytest.approx(2.0)
        assert o["max"] == pytest.approx(10.0) and o["sum"] == pytest.approx(15.0)


def test_single_rank_needs_no_group():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    value, slowest = bench.replica_throughput(4e9, 2.0)
    assert value == pytest.approx(2.0) and slowest == 2.0
    assert bench.rank_reduce(3.0, "sum") == 3.0


def test_reference_arm_runs_on_rank_zero_only(tmp_path):
    # rank 1 of a torchrun launch exits 0 at once, printing nothing
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
