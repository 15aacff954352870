"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference's fap.cpp) and known answers."""
import numpy as np
import pytest
from conftest import GOLDEN, load_golden

from fastapsp_gb300 import graphs


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_matches_reference_bit_for_bit(oracle_lib, name):
    z, g = load_golden(name)
    D, P, pre = oracle_lib.solve(int(z["K"]), g.row_offset, g.col_val, g.weight, z["graph_id"])
    assert np.array_equal(pre["st2ed"], z["mapping"])
    assert np.array_equal(D.view(np.int32), z["dist"].view(np.int32))
    assert np.array_equal(P, z["path"])


def test_oracle_sub_graph_rows_match_reference(oracle_lib):
    z, g = load_golden("grid16_sub")
    pre = oracle_lib.preprocess(int(z["K"]), z["graph_id"], g.row_offset, g.col_val)
    for p in (1, int(z["K"])):
        d, pth, _ = oracle_lib.run_part(p, g.row_offset, g.col_val, g.weight, z["graph_id"], pre)
        assert np.array_equal(d.view(np.int32), z[f"sub{p}_dist"].view(np.int32))
        assert np.array_equal(pth, z[f"sub{p}_path"])
        off, sub = int(pre["ver_offset"][p]), int(pre["ver_num"][p])
        assert np.array_equal(pre["st2ed"][off:off + sub], z[f"sub{p}_index"])


def test_full_grid_manhattan_total(oracle_lib):
    """8x8 full grid: the sum of all hop distances is 2 * 8^2 * (8^2-1)/3 * ... = 21504."""
    z, _ = load_golden("grid8_full")
    assert float(z["dist"].sum()) == 21504.0


def test_oracle_mtx_reader_matches_generator(oracle_lib, tmp_path):
    for g in (graphs.grid_graph(6, 7, seed=3),
              graphs.small_random_graph(30, 70, True, True, seed=5),
              graphs.small_random_graph(30, 70, False, True, seed=6, integer=False)):
        path = tmp_path / "g.mtx"
        graphs.write_mtx(g, str(path))
        ro, col, w = oracle_lib.mtx_read(path, g.directed, g.weighted)
        assert np.array_equal(ro, g.row_offset)
        assert np.array_equal(col, g.col_val)
        assert np.array_equal(w, g.weight)


def test_dijkstra_f32_close_to_f64(oracle_lib):
    g = graphs.road_like(2000, seed=3)
    d32, _ = oracle_lib.dijkstra_path(0, g.row_offset, g.col_val, g.weight)
    d64 = oracle_lib.dijkstra_f64(0, g.row_offset, g.col_val, g.weight)
    fin = d64 < 1e299
    rel = np.abs(d32[fin] - d64[fin]) / np.maximum(d64[fin], 1e-30)
    assert rel.max() < 1e-5
