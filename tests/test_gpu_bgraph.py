"""The boundary SSSP through the boundary graph (FAP_OPT_SSSP_METHOD = 2,
csrc/bgraph.cu) against the whole-graph search (FAP_OPT_SSSP_METHOD = 1),
whose rows equal the reference's Dijkstra (fap/kernel/batch_sssp.h:79-114)
bit for bit: whole solves must agree bit for bit -- distances and
predecessors -- on int32 graphs and on FP32 graphs with the FP64 option whose
weights fit the fixed point (there the FP64 search's sums are exact too).
Graphs cover directed and undirected inputs, parallel edges and self loops,
one part, parts without boundary vertices and many small parts; both solve
forms and single-part solves; the automatic choice (0) picks one of them on
the first run and reports it."""
import numpy as np
import pytest
import torch

from fastapsp_gb300 import graphs

pytestmark = pytest.mark.gpu


def _solve(gpu, g, K, gid, dtype, method, mode, fp64=0):
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, K, graph_id=gid, dtype=dtype) as eng:
        eng.set_option(gpu._lib.OPT_SSSP_METHOD, method)
        if dtype == gpu.DTYPE_F32:
            eng.set_option(gpu._lib.OPT_SSSP_FP64, fp64)
        tdt = torch.int32 if dtype == gpu.DTYPE_I32 else torch.float32
        d = torch.full((g.n, g.n), 7, dtype=tdt, device="cuda")
        p = torch.full((g.n, g.n), 7, dtype=torch.int32, device="cuda")
        eng.solve(d, p, mode)
        eng.solve(d, p, mode)  # second run: the captured graph (batched) or the cached plan
        torch.cuda.synchronize()
        stats = eng.sssp_stats()
        parts = []
        for part in (1, K):
            sub, _, _ = eng.part_info(part)
            dp = torch.full((max(sub, 1), g.n), 7, dtype=tdt, device="cuda")
            pp = torch.full((max(sub, 1), g.n), 7, dtype=torch.int32, device="cuda")
            if sub:
                eng.solve_part(part, dp, pp)
            torch.cuda.synchronize()
            parts.append((dp[:sub].cpu(), pp[:sub].cpu()))
    return d.cpu(), p.cpu(), stats, parts


def _case(name):
    if name == "grid_i32":
        g = graphs.grid_graph(48, 48, seed=5)
        return g, 9, None, 1
    if name == "knn_dir_i32":
        g = graphs.geometric_knn(4000, seed=6)
        return g, 12, None, 1
    if name == "rand_dir_par_i32":  # parallel edges and self loops
        g = graphs.small_random_graph(600, 2400, True, True, seed=7)
        return g, 7, None, 1
    if name == "one_part_i32":
        g = graphs.grid_graph(20, 20, seed=8)
        return g, 1, None, 1
    if name == "many_parts_i32":  # parts of a handful of vertices, some without boundary
        g = graphs.small_random_graph(300, 500, False, True, seed=9)
        return g, 60, None, 1
    if name == "road_f32":
        g = graphs.road_like(5000, seed=10)
        return g, 10, None, 0
    raise KeyError(name)


@pytest.mark.parametrize("name", ["grid_i32", "knn_dir_i32", "rand_dir_par_i32", "one_part_i32",
                                  "many_parts_i32", "road_f32"])
@pytest.mark.parametrize("mode", [1, 0])
def test_boundary_graph_equals_whole_graph_search(gpu, name, mode):
    g, K, gid, is_int = _case(name)
    if gid is None:
        gid, _ = gpu.partition(g.row_offset, g.col_val, K)
    dtype = gpu.DTYPE_I32 if is_int else gpu.DTYPE_F32
    fp64 = 0 if is_int else 1
    d0, p0, st0, parts0 = _solve(gpu, g, K, gid, dtype, 2, mode, fp64)
    d1, p1, st1, parts1 = _solve(gpu, g, K, gid, dtype, 1, mode, fp64)
    da, pa, _, _ = _solve(gpu, g, K, gid, dtype, 0, mode, fp64)
    # the boundary graph ran (no search batches) unless the graph has no boundary
    assert st1["batches"] > 0 or st1["steps"] == 0
    if K > 1:
        assert st0["batches"] == 0, st0
    assert torch.equal(d0, d1), "distances differ between the two SSSP methods"
    assert torch.equal(p0, p1), "predecessors differ between the two SSSP methods"
    assert torch.equal(da, d1) and torch.equal(pa, p1), "the automatic choice differs"
    for (a, b), (c, e) in zip(parts0, parts1):
        assert torch.equal(a, c) and torch.equal(b, e), "single-part solves differ"


def test_fp32_without_fixed_point_falls_back_to_the_search(gpu):
    """Weights spread over many binades with full mantissas: no 64-bit fixed
    point holds every path, so the engine keeps the whole-graph search."""
    g = graphs.road_like(3000, seed=11)
    rng = np.random.default_rng(3)
    g.weight[:] = (10.0 ** rng.uniform(-7, 7, size=g.m)).astype(np.float32)
    gid, _ = gpu.partition(g.row_offset, g.col_val, 6)
    d0, p0, st0, _ = _solve(gpu, g, 6, gid, gpu.DTYPE_F32, 2, 1, fp64=1)
    d1, p1, st1, _ = _solve(gpu, g, 6, gid, gpu.DTYPE_F32, 1, 1, fp64=1)
    assert st0["batches"] > 0  # the search ran
    assert torch.equal(d0, d1) and torch.equal(p0, p1)


def test_sssp_method_option_values(gpu):
    g = graphs.grid_graph(32, 32, seed=1)
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, 4, dtype=gpu.DTYPE_I32) as eng:
        assert eng.get_option(gpu._lib.OPT_SSSP_METHOD) == 0  # automatic, not tuned yet
        d = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
        eng.solve(d, None)
        assert eng.get_option(gpu._lib.OPT_SSSP_METHOD) in (1, 2)  # the trial's choice
        eng.set_option(gpu._lib.OPT_SSSP_METHOD, 1)
        assert eng.get_option(gpu._lib.OPT_SSSP_METHOD) == 1
        with pytest.raises(gpu._lib.FapError):
            eng.set_option(gpu._lib.OPT_SSSP_METHOD, 3)
        assert eng.get_option(gpu._lib.OPT_SSSP_METHOD) == 1
