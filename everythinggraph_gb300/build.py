"""Builds the CUDA library (libeg_gpu.so) and the C drop-in driver binaries.

Every .cu file under csrc/ is compiled for sm_103a in parallel and linked
into everythinggraph_gb300/_build/libeg_gpu.so; the C host driver under
host/ is compiled with gcc and linked against it.  No CMake, one -gencode.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libeg_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_lib(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    cus = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(INCLUDE, "eg_gpu.h"))
    objs = []
    jobs = []
    for f in cus:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f[:-3] + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + hdrs):
            jobs.append([nvcc()] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                            "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj] + list(extra))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not _newer(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_host(force=False):
    """C drop-in driver: one binary per algorithm plug-in, like the reference."""
    if not os.path.isdir(HOST):
        return []
    srcs = [os.path.join(HOST, f) for f in ("eg_main.c", "eg_init.c")]
    plugins = sorted(f for f in os.listdir(HOST) if f.startswith("algo_") and f.endswith(".c"))
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [os.path.join(INCLUDE, "eg_gpu.h")]
    outs = []
    jobs = []
    for p in plugins:
        name = "eg_" + p[len("algo_"):-2]
        exe = os.path.join(OUT, name)
        outs.append(exe)
        deps = srcs + [os.path.join(HOST, p), LIB] + hdrs
        if force or not _newer(exe, deps):
            jobs.append(["gcc", "-O2", "-std=gnu11", "-Wall", "-I", INCLUDE, "-I", HOST] + srcs +
                        [os.path.join(HOST, p), "-o", exe, "-L", OUT, "-leg_gpu", "-Wl,-rpath,$ORIGIN", "-lm"])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), 8))) as ex:
        list(ex.map(_run, jobs))
    return outs


def build(force=False, verbose=False):
    lib = build_lib(force=force, verbose=verbose)
    build_host(force=force)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
