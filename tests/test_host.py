"""Host-side layer without a GPU: the C ABI library loads and exports every
declared symbol, the MatrixMarket reader, the partitioner, the boundary /
reorder step, argument validation, and the multi-rank sharding logic."""
import re

import numpy as np
import pytest
from conftest import GOLDEN, ROOT, load_golden

from fastapsp_gb300 import graphs


def declared_symbols():
    text = (ROOT / "include" / "fastapsp.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fap_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(fap_lib):
    import ctypes

    lib = ctypes.CDLL(str(fap_lib._lib.LIB_PATH))
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_cpp_dropin_symbols_exported(fap_lib):
    import subprocess

    out = subprocess.run(["nm", "-DC", str(fap_lib._lib.LIB_PATH)], capture_output=True, text=True).stdout
    for m in ("fap::fapGraph::solve(bool)", "fap::fapGraph::solveSubGraph(int, bool)",
              "fap::fapGraph::preCondition()", "fap::fapGraph::isSplit()",
              "fap::fapGraph::getSubGraphDistance(int)", "fap::fapGraph::getMapping()"):
        assert m in out, m


def test_no_device_is_reported_not_faked(fap_lib):
    if fap_lib.device_count() > 0:
        pytest.skip("a GPU is present")
    g = graphs.grid_graph(4, 4)
    with pytest.raises(fap_lib.FapError) as ex:
        fap_lib.Engine(g.n, g.row_offset, g.col_val, g.weight, 2)
    assert ex.value.status == -7


def test_invalid_arguments_rejected(fap_lib):
    g = graphs.grid_graph(4, 4)
    bad = g.col_val.copy()
    bad[0] = g.n + 5
    with pytest.raises(fap_lib.FapError) as ex:
        fap_lib.Engine(g.n, g.row_offset, bad, g.weight, 2)
    assert ex.value.status == -1
    w = g.weight.copy()
    w[0] = 0.5
    with pytest.raises(fap_lib.FapError) as ex:
        fap_lib.Engine(g.n, g.row_offset, g.col_val, w, 2, dtype=fap_lib.DTYPE_I32)
    assert ex.value.status == -8
    with pytest.raises(fap_lib.FapError):
        fap_lib.partition(g.row_offset, g.col_val, 0)


def test_mtx_reader_matches_oracle(fap_lib, oracle_lib, tmp_path):
    for name in GOLDEN:
        z, g = load_golden(name)
        path = tmp_path / f"{name}.mtx"
        graphs.write_mtx(g, str(path))
        ro, col, w = fap_lib.mtx_read(str(path), g.directed, g.weighted)
        ro2, col2, w2 = oracle_lib.mtx_read(path, g.directed, g.weighted)
        assert np.array_equal(ro, ro2) and np.array_equal(col, col2) and np.array_equal(w, w2)
        assert np.array_equal(ro, g.row_offset)


def test_mtx_reader_shipped_graph_header(fap_lib, tmp_path):
    p = tmp_path / "h.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n% c\n3 3 2\n1 2\n2 3\n")
    ro, col, w = fap_lib.mtx_read(str(p), False, False)
    assert ro.tolist() == [0, 1, 3, 4]
    assert col.tolist() == [1, 2, 0, 1]  # newest entry first in each row
    assert w.tolist() == [1, 1, 1, 1]


@pytest.mark.parametrize("name", GOLDEN)
def test_preprocess_matches_oracle_and_reference(fap_lib, oracle_lib, name):
    z, g = load_golden(name)
    K = int(z["K"])
    a = fap_lib.preprocess(K, z["graph_id"], g.row_offset, g.col_val)
    b = oracle_lib.preprocess(K, z["graph_id"], g.row_offset, g.col_val)
    for k in ("st2ed", "ed2st", "ver_num", "ver_offset", "bdy_num", "bdy_offset"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["st2ed"], z["mapping"])


@pytest.mark.parametrize("K", [2, 7, 16])
def test_partition_balanced_and_complete(fap_lib, K):
    g = graphs.grid_graph(64, 64, seed=4)
    gid, cut = fap_lib.partition(g.row_offset, g.col_val, K)
    counts = np.bincount(gid, minlength=K + 1)[1:]
    assert gid.min() >= 1 and gid.max() <= K
    assert counts.min() > 0
    assert counts.max() <= np.ceil(1.03 * g.n / K) + 1
    # cut = number of undirected grid edges across parts
    src = np.repeat(np.arange(g.n), np.diff(g.row_offset))
    cross = (gid[src] != gid[g.col_val]) & (g.col_val > src)
    assert cut == int(cross.sum())
    # a grid cut far below the random-partition cut
    assert cut < 0.2 * (g.row_offset[-1] / 2)


def test_partition_deterministic(fap_lib):
    g = graphs.geometric_knn(3000, seed=2)
    a, _ = fap_lib.partition(g.row_offset, g.col_val, 8, seed=5)
    b, _ = fap_lib.partition(g.row_offset, g.col_val, 8, seed=5)
    assert np.array_equal(a, b)


def test_workload_shapes():
    g1 = graphs.grid_graph()
    assert g1.n == 16384 and not g1.directed and not g1.weighted
    assert 0.6 * 2 * 127 * 128 < g1.lines_src.shape[0] < 0.9 * 2 * 127 * 128
    g4 = graphs.road_like()
    assert g4.n == 114599
    assert 235_000 < g4.m < 245_000
    assert abs(g4.m / g4.n - 2.09) < 0.03
    assert g4.weight.min() >= 0.1 and g4.weight.max() <= 10.0
    g5 = graphs.regular_digraph(300, rng=np.random.default_rng(1))
    assert np.all(np.diff(g5.row_offset) == 4)
    assert np.all(np.bincount(g5.col_val, minlength=300) == 4)
