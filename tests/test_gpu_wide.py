"""The int32 engine's wide form (separate values and steps) of the FW and the
min-plus, used when a plan cannot prove every finite result below 2^24 - 1
(the packed keys' range).  The reference computes in FP32 for any weights
(fap/fap.h:52, fap/utils/readMatFile.h:124,140), so the int32 engine must
stay exact where packed keys cannot:

* a 300-vertex directed graph with integer weights up to 3.5e6 (its fixture
  made by the reference's own binary, tests/golden/make_golden.py): distances
  equal FP64 Dijkstra (exact for integers) in every row, and equal the
  reference wherever the reference is exact (below 2^24; above it the
  reference's FP32 sums round, and the rows agree within 1e-6 relative);
* a 16,384-vertex geometric graph in parts of about 1,024 vertices (17 FW
  rounds) solved with the wide form forced: the same distances and
  predecessors as the packed form."""
import numpy as np
import pytest
import torch
from conftest import load_golden
from helpers import MAXV, check_pred_tight, to_ref_float

from fastapsp_gb300 import graphs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [1, 0])
def test_large_integer_weights_exact(gpu, oracle_lib, mode):
    z, g = load_golden("bigw300_dir_wide")
    n, K = g.n, int(z["K"])
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, K, graph_id=z["graph_id"],
                    dtype=gpu.DTYPE_I32) as eng:
        assert np.array_equal(eng.mapping(), z["mapping"])
        d = torch.empty((n, n), dtype=torch.int32, device="cuda")
        p = torch.empty((n, n), dtype=torch.int32, device="cuda")
        eng.solve(d, p, mode)
        torch.cuda.synchronize()
        d, p = d.cpu().numpy(), p.cpu().numpy()
    mapping = z["mapping"]
    fin = d < (1 << 30)
    assert (d[fin] > (1 << 24)).mean() > 0.05, "the case must reach past the packed range"
    for r in range(n):
        d64 = oracle_lib.dijkstra_f64(int(mapping[r]), g.row_offset, g.col_val, g.weight)
        ref = np.where(d64 < 1e299, d64, float(1 << 30)).astype(np.int64)
        assert np.array_equal(d[r].astype(np.int64), ref), f"row {r} differs from exact Dijkstra"
    ref = z["dist"]
    exact = ref < (1 << 24)
    got = to_ref_float(d)
    assert np.array_equal(got[exact], ref[exact])
    big = ~exact & (ref < MAXV)
    assert np.all(np.abs(d[big].astype(np.float64) - ref[big]) <= 1e-6 * ref[big])
    check_pred_tight(d, p, mapping, n, g.row_offset, g.col_val, g.weight, unreached=1 << 30)


def test_wide_form_forced_matches_packed_form(gpu, oracle_lib):
    g = graphs.geometric_knn(16384, seed=31)
    K = 16
    gid, _ = gpu.partition(g.row_offset, g.col_val, K)
    outs = []
    for form in (0, 1):
        with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, K, graph_id=gid, dtype=gpu.DTYPE_I32) as eng:
            eng.set_option(gpu._lib.OPT_INT32_FORM, form)
            assert eng.get_option(gpu._lib.OPT_INT32_FORM) == form
            d = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
            p = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
            eng.solve(d, p, gpu.MODE_BATCHED)
            eng.solve(d, p, gpu.MODE_BATCHED)  # the captured graph
            torch.cuda.synchronize()
            mapping = eng.mapping()
            outs.append((d.cpu(), p.cpu()))
            del d, p
    assert torch.equal(outs[0][0], outs[1][0]), "distances differ between packed and wide forms"
    assert torch.equal(outs[0][1], outs[1][1]), "predecessors differ between packed and wide forms"
    dd = outs[1][0].numpy()
    for r in np.random.default_rng(2).choice(g.n, size=24, replace=False):
        rd, _ = oracle_lib.dijkstra_path(int(mapping[r]), g.row_offset, g.col_val, g.weight)
        ref = np.where(rd >= 1e8, 1 << 30, rd).astype(np.int64)
        assert np.array_equal(dd[r].astype(np.int64), ref), f"row {r}"
