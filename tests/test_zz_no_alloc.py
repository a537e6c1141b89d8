"""The allocation-free SpMV entry point, called through the C ABI.

eg_spmv_f32_noalloc exists for callers that cannot allocate device memory:
it takes device pointers to the caller's CSR-shaped arrays, x and y, and
keeps its own scratch in a fixed array compiled into the library.  This file
is collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_L1 = 1e-6
MAX_REL = 1e-5


def test_noalloc_spmv_matches_eg_spmv_twice():
    import torch

    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import _lib, build

    build.build_lib()
    lib = _lib.load()
    ctx = eg.Context(0)
    scale = 16
    n = 1 << scale
    g = ctx.rmat(scale, 16 * n, 1).build(eg.CSC)
    m = g.m
    x = np.random.default_rng(3).random(n, dtype=np.float32)
    y_ref, _ = g.spmv(x, "f32", unit_values=True)  # the existing entry point
    xd = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    ptr = ctypes.c_void_p(g.device_ptr(_lib.EG_DEV_CSC_PTR))
    col = ctypes.c_void_p(g.device_ptr(_lib.EG_DEV_CSC_COL))
    used = ctx.bytes_in_use
    for call in range(2):
        yd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.eg_spmv_f32_noalloc(ptr, col, None, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()),
                                     n, m, ctypes.c_void_p(ctx.stream))
        assert rc == 0, lib.eg_last_error()
        ctx.sync()
        y = yd.cpu().numpy()
        nz = y_ref != 0
        l1 = np.abs(y - y_ref).sum() / np.abs(y_ref).sum()
        mx = (np.abs(y[nz] - y_ref[nz]) / np.abs(y_ref[nz])).max()
        assert l1 <= REL_L1 and mx <= MAX_REL, (call, l1, mx)
        assert np.all(y[~nz] == 0)
    assert ctx.bytes_in_use == used  # nothing was allocated through the context
    # sizes past the fixed scratch are refused before any device work
    big = 1 << 31
    rc = lib.eg_spmv_f32_noalloc(ptr, col, None, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(xd.data_ptr()),
                                 big, big, ctypes.c_void_p(ctx.stream))
    assert rc == -1 and b"exceeds the fixed scratch limit" in lib.eg_last_error()
    g.free()
    ctx.close()
