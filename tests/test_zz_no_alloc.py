"""The allocation-free SpMV entry point, called through the C ABI.

eg_spmv_f32_noalloc exists for callers that cannot allocate device memory:
it takes device pointers to the caller's CSR-shaped arrays, x and y, and
keeps its own scratch in a fixed array compiled into the library.  Its rows
are summed over merge-path tiles, so it agrees with eg_spmv's EG_SPMV_F32
within fp32 rounding; both are also checked against the CPU FP64 oracle.
This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL_L1 = 1e-6
MAX_REL = 1e-5
TILE_ITEMS = 2048  # row ends + entries per merge-path tile


def errors(y, ref):
    ref = ref.astype(np.float64)
    y = y.astype(np.float64)
    nz = ref != 0
    l1 = np.abs(y - ref).sum() / max(np.abs(ref).sum(), 1e-300)
    mx = (np.abs(y[nz] - ref[nz]) / np.abs(ref[nz])).max() if nz.any() else 0.0
    return l1, mx, nz


@pytest.fixture(scope="module")
def env():
    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import _lib, build

    build.build_lib()
    lib = _lib.load()
    ctx = eg.Context(0)
    yield eg, _lib, lib, ctx
    ctx.close()


def call(lib, ctx, ptr, col, vals, x, y, n, m):
    vp = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    rc = lib.eg_spmv_f32_noalloc(vp(ptr) if not isinstance(ptr, ctypes.c_void_p) else ptr,
                                 vp(col) if not isinstance(col, ctypes.c_void_p) else col, vp(vals), vp(x), vp(y),
                                 n, m, ctypes.c_void_p(ctx.stream))
    assert rc == 0, lib.eg_last_error()
    ctx.sync()


def test_noalloc_spmv_matches_eg_spmv_twice(env):
    import torch
    eg, _lib, lib, ctx = env
    scale = 16
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 1).build(eg.CSC)
    m = g.m
    x = np.random.default_rng(3).random(n, dtype=np.float32)
    y_ref, _ = g.spmv(x, "f32", unit_values=True)  # the existing entry point
    hptr, hcol = g.adj(eg.CSC)
    y64 = oracle.spmv_f64(n, hptr, hcol, np.ones(m, dtype=np.float32), x)
    xd = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    ptr = ctypes.c_void_p(g.device_ptr(_lib.EG_DEV_CSC_PTR))
    col = ctypes.c_void_p(g.device_ptr(_lib.EG_DEV_CSC_COL))
    used = ctx.bytes_in_use
    for c in range(2):
        yd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        call(lib, ctx, ptr, col, None, xd, yd, n, m)
        y = yd.cpu().numpy()
        l1, mx, nz = errors(y, y_ref)
        assert l1 <= REL_L1 and mx <= MAX_REL, (c, l1, mx)
        assert np.all(y[~nz] == 0)
        l1, mx, _ = errors(y, y64)
        assert l1 <= REL_L1 and mx <= MAX_REL, ("vs fp64", c, l1, mx)
    assert ctx.bytes_in_use == used  # nothing was allocated through the context
    # sizes past the fixed scratch are refused before any device work
    big = 1 << 31
    rc = lib.eg_spmv_f32_noalloc(ptr, col, None, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(xd.data_ptr()),
                                 big, big, ctypes.c_void_p(ctx.stream))
    assert rc == -1 and b"exceeds the fixed scratch limit" in lib.eg_last_error()
    g.free()


def test_noalloc_spmv_edge_values_vs_fp64(env):
    """Explicit per-entry values (vals[p] * x[col[p]]) against the CPU FP64
    oracle and against eg_spmv run on the same values, two calls in a row."""
    import torch
    eg, _lib, lib, ctx = env
    scale = 14
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 2).build(eg.CSC)
    m = g.m
    hptr, hcol = g.adj(eg.CSC)
    rows = np.repeat(np.arange(n, dtype=np.uint32), np.diff(hptr.astype(np.int64)))
    vals = oracle.hash_values(hcol, rows, 9)  # the same value rule eg_spmv uses with value_seed=9
    x = oracle.uniform_f32(n, 11)
    y64 = oracle.spmv_f64(n, hptr, hcol, vals, x)
    y_ref, _ = g.spmv(x, "f32", value_seed=9)
    l1, mx, _ = errors(y_ref, y64)
    assert l1 <= REL_L1 and mx <= MAX_REL, ("eg_spmv vs fp64", l1, mx)
    ptr = torch.from_numpy(hptr.view(np.int32)).cuda()
    col = torch.from_numpy(hcol.view(np.int32)).cuda()
    vd = torch.from_numpy(vals).cuda()
    xd = torch.from_numpy(x).cuda()
    for c in range(2):
        yd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        call(lib, ctx, ptr, col, vd, xd, yd, n, m)
        y = yd.cpu().numpy()
        l1, mx, _ = errors(y, y64)
        assert l1 <= REL_L1 and mx <= MAX_REL, (c, l1, mx)
        l1, mx, _ = errors(y, y_ref)
        assert l1 <= REL_L1 and mx <= MAX_REL, ("vs eg_spmv", c, l1, mx)
    g.free()


def test_noalloc_spmv_no_entries_and_full_last_tile(env):
    """m = 0 with a NULL column array (every row sums to 0), and a graph whose
    n + m fills its last merge-path tile exactly."""
    import torch
    eg, _lib, lib, ctx = env
    n = 1000
    ptr = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    xd = torch.ones(n, dtype=torch.float32, device="cuda")
    for c in range(2):
        yd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        call(lib, ctx, ptr, ctypes.c_void_p(0), None, xd, yd, n, 0)
        assert torch.all(yd == 0).item(), c
    # n + m = 3 tiles exactly: rows of ragged lengths, some empty
    n = 1500
    m = 3 * TILE_ITEMS - n
    rng = np.random.default_rng(5)
    pairs = np.empty(2 * m, dtype=np.uint32)
    pairs[0::2] = rng.integers(0, n, m)
    pairs[1::2] = (rng.integers(0, 40, m) ** 2) % n  # a few heavy rows
    g = ctx.from_pairs(n, pairs).build(eg.CSC)
    assert g.m == m and (n + m) % TILE_ITEMS == 0
    hptr, hcol = g.adj(eg.CSC)
    x = oracle.uniform_f32(n, 4)
    y64 = oracle.spmv_f64(n, hptr, hcol, np.ones(m, dtype=np.float32), x)
    xd = torch.from_numpy(x).cuda()
    ptr = ctypes.c_void_p(g.device_ptr(_lib.EG_DEV_CSC_PTR))
    col = ctypes.c_void_p(g.device_ptr(_lib.EG_DEV_CSC_COL))
    for c in range(2):
        yd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        call(lib, ctx, ptr, col, None, xd, yd, n, m)
        y = yd.cpu().numpy()
        l1, mx, nz = errors(y, y64)
        assert l1 <= REL_L1 and mx <= MAX_REL, (c, l1, mx)
        assert np.all(y[~nz] == 0)
    g.free()
