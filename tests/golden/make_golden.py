"""Generates the golden fixtures in tests/golden/ from the unmodified reference.

Run in a container that has the reference sources (default /root/reference,
or $EG_REF_SRC):

    python tests/golden/make_golden.py

It builds the reference binaries with the dump harness (oracle/build_ref.sh),
writes seeded synthetic graphs as binary uint32 [src][dst] files, runs each
reference binary on them with the flags listed below and stores the dumped
result arrays.  Small graphs keep their edge arrays in the fixture; the
scale-16 graph stores only a SHA-256 of its edges, and the tests regenerate it
with the oracle's generator and check the digest first.
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def run_ref(binary, args, dtype, n, tmp):
    out = os.path.join(tmp, "dump.bin")
    if os.path.exists(out):
        os.remove(out)
    env = dict(os.environ, EG_DUMP=out, OMP_NUM_THREADS="8")
    subprocess.run([os.path.join(REF, binary)] + args, env=env, check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=600)
    a = np.fromfile(out, dtype=dtype)
    assert a.size == n, (binary, args, a.size, n)
    return a


def tiny_graph():
    # 10 vertices: a path 0-1-2-3, a star around 5, a self-loop on 7, a
    # duplicated edge 8->9, vertex 4 and 6 isolated on the out side.
    e = [(0, 1), (1, 2), (2, 3), (5, 0), (5, 6), (5, 7), (5, 8), (7, 7), (8, 9), (8, 9), (9, 5), (3, 1)]
    return 10, np.array(e, dtype=np.uint32).reshape(-1)


def make(name, n, pairs, store_pairs, roots, tmp):
    path = os.path.join(tmp, name + ".bin")
    pairs.astype(np.uint32).tofile(path)
    N = str(n)
    rec = {"n": np.int64(n), "pairs_sha256": np.bytes_(hashlib.sha256(pairs.astype(np.uint32).tobytes()).hexdigest())}
    if store_pairs:
        rec["pairs"] = pairs.astype(np.uint32)
    rec["roots"] = np.array(roots, dtype=np.uint32)
    f = ["-f", path, "-n", N]
    rec["pr_simple_pull"] = run_ref("pagerank_simple", f + ["-m", "2", "-a", "1"], np.float32, n, tmp)
    rec["prgrid_m0"] = run_ref("prgrid_cilk", f + ["-m", "0"], np.float32, n, tmp)
    rec["bfs_simple_m2u"] = run_ref("bfs_simple", f + ["-m", "2", "-u"], np.uint32, n, tmp)
    rec["bfs_simple_m8"] = run_ref("bfs_simple", f + ["-m", "8"], np.uint32, n, tmp)
    # the edge-array load modes: 7 (sorted by src), 9 (file order); prgrid's
    # column loop over the edge array (degrees counted twice in mode 9)
    rec["bfs_simple_m7"] = run_ref("bfs_simple", f + ["-m", "7"], np.uint32, n, tmp)
    rec["bfs_simple_m9"] = run_ref("bfs_simple", f + ["-m", "9"], np.uint32, n, tmp)
    for mode in ("7", "8", "9"):
        rec["prgrid_m" + mode] = run_ref("prgrid_cilk", f + ["-m", mode], np.float32, n, tmp)
    for r in roots:
        rec["bfsgrid_m0_p%d" % r] = run_ref("bfsgrid_cilk", f + ["-m", "0", "-p", str(r)], np.uint32, n, tmp)
        rec["sssp_pull_p%d" % r] = run_ref("sssp_pushpull", f + ["-m", "2", "-a", "1", "-r", "-p", str(r)],
                                           np.uint32, n, tmp)
    rec["wcc_m2u"] = run_ref("wcc", f + ["-m", "2", "-u"], np.int64, n, tmp)
    rec["wcc_m0"] = run_ref("wcc", f + ["-m", "0"], np.int64, n, tmp)
    rec["wcc_m8"] = run_ref("wcc", f + ["-m", "8"], np.int64, n, tmp)
    rec["spmv_pull"] = run_ref("spmv", f + ["-m", "2", "-a", "1"], np.uint32, n, tmp)
    rec["spmv_push"] = run_ref("spmv", f + ["-m", "2", "-a", "0"], np.uint32, n, tmp)
    rec["spmv_m8"] = run_ref("spmv", f + ["-m", "8"], np.uint32, n, tmp)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print("wrote", name, {k: v.shape for k, v in rec.items()})


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    oracle.build()
    with tempfile.TemporaryDirectory() as tmp:
        n, pairs = tiny_graph()
        make("tiny", n, pairs, True, [0, 5, 8], tmp)
        for scale, store in ((10, True), (12, True), (16, False)):
            n = 1 << scale
            pairs = oracle.rmat_edges(scale, 16 * n, 1)
            od, _ = oracle.degrees(n, pairs)
            roots = [0] + [int(r) for r in oracle.sample_roots(od, 2, 3)]
            make("rmat%d" % scale, n, pairs, store, roots, tmp)


if __name__ == "__main__":
    main()
