"""The on-disk layout cache (eg_graph_save_layouts / eg_graph_load_layouts)
through the C ABI: a graph filled from the cache holds the same layouts,
bit for bit, as one that built them, and gives the same results; another
input is a miss; a truncated file is an error."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def ctx():
    import everythinggraph_gb300 as eg
    from everythinggraph_gb300 import build
    build.build_lib()
    c = eg.Context(0)
    yield c
    c.close()


def test_cache_round_trip_adjacency_and_grid(ctx, tmp_path):
    import everythinggraph_gb300 as eg
    z = np.load(os.path.join(GOLDEN, "rmat12.npz"))
    n, pairs = int(z["n"]), z["pairs"]
    path = str(tmp_path / "g.eglayout")
    # the grid is built from directed input (its load modes take no -u)
    g = ctx.from_pairs(n, pairs).build(eg.CSR | eg.CSC).build_grid(17)
    g.save_layouts(path)
    assert os.path.exists(path) and not os.path.exists(path + ".tmp")
    h = ctx.from_pairs(n, pairs)
    assert h.load_layouts(path)
    info = h.info()
    assert info.layouts & (eg.CSR | eg.CSC | eg.GRID) == eg.CSR | eg.CSC | eg.GRID and info.grid_p == 17
    for lay in (eg.CSR, eg.CSC):
        for a, b in zip(g.adj(lay), h.adj(lay)):
            np.testing.assert_array_equal(a, b)
    for a, b in zip(g.grid(), h.grid()):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(g.degrees(True, True)[0], h.degrees(True, True)[0])
    r = int(z["roots"][1])
    np.testing.assert_array_equal(g.bfs(r)[0], h.bfs(r)[0])
    np.testing.assert_array_equal(g.pagerank()[0].view(np.uint32), h.pagerank()[0].view(np.uint32))
    np.testing.assert_array_equal(g.wcc()[0], h.wcc()[0])
    # another input of the same size is a miss (the digest differs)
    other = pairs.copy()
    other[5] = (other[5] + 1) % n
    assert not ctx.from_pairs(n, other).load_layouts(path)
    assert not ctx.from_pairs(n, pairs, undirected=True).load_layouts(path)  # other flags
    assert not ctx.from_pairs(n, pairs).load_layouts(str(tmp_path / "absent"))
    # a truncated file that matches the header is an error, not a miss
    with open(path, "rb") as f:
        head = f.read(os.path.getsize(path) // 2)
    cut = str(tmp_path / "cut.eglayout")
    with open(cut, "wb") as f:
        f.write(head)
    with pytest.raises(eg.EGError) as e:
        ctx.from_pairs(n, pairs).load_layouts(cut)
    assert e.value.code == -4
    g.free()
    h.free()
    # undirected adjacency
    g = ctx.from_pairs(n, pairs, undirected=True).build(eg.CSR)
    g.save_layouts(path)
    h = ctx.from_pairs(n, pairs, undirected=True)
    assert h.load_layouts(path)
    for a, b in zip(g.adj(eg.CSR), h.adj(eg.CSR)):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(g.wcc()[0], h.wcc()[0])
    g.free()
    h.free()


def test_cache_round_trip_edge_array(ctx, tmp_path):
    import everythinggraph_gb300 as eg
    z = np.load(os.path.join(GOLDEN, "rmat10.npz"))
    n, pairs = int(z["n"]), z["pairs"]
    path = str(tmp_path / "e.eglayout")
    g = ctx.from_pairs(n, pairs).build_edges("src_dst")
    g.save_layouts(path)
    h = ctx.from_pairs(n, pairs)
    assert h.load_layouts(path)
    assert h.info().layouts & eg.EDGES and not h.info().layouts & eg.CSR
    for a, b in zip(g.edges(), h.edges()):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(h.edges_bfs(0)[0].astype(np.uint32), z["bfs_simple_m8"])
    g.free()
    h.free()


def test_driver_layout_cache(tmp_path):
    from everythinggraph_gb300 import build
    build.build_lib()
    build.build_host()
    z = np.load(os.path.join(GOLDEN, "rmat12.npz"))
    n = int(z["n"])
    path = str(tmp_path / "g.bin")
    z["pairs"].tofile(path)
    cache = tmp_path / "cache"
    cache.mkdir()
    outs = []
    for run in range(2):
        dump = str(tmp_path / ("wcc%d.bin" % run))
        env = dict(os.environ, EG_DUMP=dump, EG_LAYOUT_CACHE=str(cache))
        r = subprocess.run([os.path.join(ROOT, "everythinggraph_gb300", "_build", "eg_wcc"), "-f", path, "-n", str(n),
                            "-m", "2", "-u"], env=env, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert ("Layout cache hit" in r.stdout) == (run == 1)
        outs.append(np.fromfile(dump, dtype=np.int64))
    np.testing.assert_array_equal(outs[0], z["wcc_m2u"])
    np.testing.assert_array_equal(outs[1], z["wcc_m2u"])
    assert len(os.listdir(cache)) == 1
