"""CPU checks of the drop-in boundary: the C-ABI library builds, loads and
exports every entry point that include/eg_gpu.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "eg_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(eg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from everythinggraph_gb300 import build
    path = build.build_lib()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "eg_pagerank" in names and "eg_bfs" in names and len(names) > 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from everythinggraph_gb300 import _lib
    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_no_device_call_needed_for_errors(lib):
    lib.eg_last_error.restype = ctypes.c_char_p
    lib.eg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.eg_version()
    # NULL arguments are rejected before any CUDA call
    lib.eg_graph_build.restype = ctypes.c_int
    assert lib.eg_graph_build(None, 1) == -1
    assert b"NULL" in lib.eg_last_error()


def test_product_refuses_to_run_without_library(tmp_path):
    from everythinggraph_gb300 import _lib
    saved = _lib._lib
    _lib._lib = None
    try:
        with pytest.raises(RuntimeError, match="not built"):
            _lib.load(str(tmp_path / "missing.so"))
    finally:
        _lib._lib = saved
