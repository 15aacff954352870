"""Full Fast-APSP solves through the C ABI against the reference's own outputs
(golden fixtures) and the CPU oracle."""
import numpy as np
import pytest
import torch
from conftest import GOLDEN, load_golden
from helpers import MAXV, check_pred_tight, has_parallel_edges, to_ref_float

pytestmark = pytest.mark.gpu

# *_wide fixtures hold distances above 2^24, where the reference's FP32
# arithmetic is inexact; tests/test_gpu_wide.py checks them
INT_CASES = [n for n in GOLDEN if not n.endswith("f32") and not n.endswith("wide")]
F32_CASES = [n for n in GOLDEN if n.endswith("f32")]


def solve_engine(gpu, z, g, dtype, mode, on_device):
    n = g.n
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, int(z["K"]), graph_id=z["graph_id"],
                    dtype=dtype) as eng:
        assert np.array_equal(eng.mapping(), z["mapping"])
        npdt = np.int32 if dtype == gpu.DTYPE_I32 else np.float32
        if on_device:
            d = torch.empty((n, n), dtype=torch.int32 if dtype == gpu.DTYPE_I32 else torch.float32, device="cuda")
            p = torch.empty((n, n), dtype=torch.int32, device="cuda")
            eng.solve(d, p, mode)
            torch.cuda.synchronize()
            d, p = d.cpu().numpy(), p.cpu().numpy()
        else:
            d = np.empty((n, n), npdt)
            p = np.empty((n, n), np.int32)
            eng.solve(d, p, mode)
        # second call reuses the cached plan / graph
        if not on_device:
            d2 = np.empty_like(d)
            p2 = np.empty_like(p)
            eng.solve(d2, p2, mode)
            assert np.array_equal(d, d2) and np.array_equal(p, p2)
    return to_ref_float(d), p


def out_of_part_mask(z):
    gid = z["graph_id"]
    rows_part = gid[z["mapping"]]
    return rows_part[:, None] != gid[None, :]


@pytest.mark.parametrize("name", INT_CASES)
@pytest.mark.parametrize("dtype_name", ["i32", "f32"])
@pytest.mark.parametrize("mode", [0, 1])
def test_solve_integer_graphs_bit_exact(gpu, name, dtype_name, mode):
    z, g = load_golden(name)
    dtype = gpu.DTYPE_I32 if dtype_name == "i32" else gpu.DTYPE_F32
    d, p = solve_engine(gpu, z, g, dtype, mode, on_device=(mode == 1))
    assert np.array_equal(d.view(np.int32), z["dist"].view(np.int32))
    # predecessors: identical to the reference outside each part's own columns
    # (SSSP and min-plus region); tight shortest-path edges everywhere
    m = out_of_part_mask(z)
    assert np.array_equal(p[m], z["path"][m])
    check_pred_tight(d, p, z["mapping"], g.n, g.row_offset, g.col_val, g.weight)


@pytest.mark.parametrize("name", F32_CASES)
@pytest.mark.parametrize("mode", [0, 1])
def test_solve_f32_graphs_within_tolerance(gpu, oracle_lib, name, mode):
    z, g = load_golden(name)
    d, p = solve_engine(gpu, z, g, gpu.DTYPE_F32, mode, on_device=False)
    ref = z["dist"]
    fin = ref < MAXV
    assert np.array_equal(fin, d < MAXV)
    rel = np.abs(d[fin] - ref[fin]) / np.maximum(ref[fin], 1e-30)
    assert rel.max() <= 1e-6
    # against FP64 Dijkstra.  Not with parallel edges: the reference's part
    # matrix keeps the last CSR entry of parallel edges, not the lightest
    # (util_Myalgorithm.h:54-63), and the engine reproduces that.
    rows = [] if has_parallel_edges(g.n, g.row_offset, g.col_val) else range(0, g.n, max(1, g.n // 20))
    for r in rows:
        s = int(z["mapping"][r])
        d64 = oracle_lib.dijkstra_f64(s, g.row_offset, g.col_val, g.weight)
        f = d64 < 1e299
        assert np.all((d[r] < MAXV) == f)
        assert np.max(np.abs(d[r][f] - d64[f]) / np.maximum(d64[f], 1e-30)) <= 1e-6
    check_pred_tight(d, p, z["mapping"], g.n, g.row_offset, g.col_val, g.weight, rtol=1e-6)


def test_solve_part_matches_reference_sub_graph(gpu):
    z, g = load_golden("grid16_sub")
    K = int(z["K"])
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, K, graph_id=z["graph_id"],
                    dtype=gpu.DTYPE_I32) as eng:
        for part in (1, K):
            sub, bdy, off = eng.part_info(part)
            d = np.empty((sub, g.n), np.int32)
            p = np.empty((sub, g.n), np.int32)
            eng.solve_part(part, d, p)
            assert np.array_equal(to_ref_float(d), z[f"sub{part}_dist"])
            assert np.array_equal(eng.mapping()[off:off + sub], z[f"sub{part}_index"])


def test_fapgraph_mirror_solve_and_split(gpu):
    z, g = load_golden("knn300_dir_int")
    G = gpu.FapGraph(g.n, g.m, g.row_offset, g.col_val, g.weight, int(z["K"]), graph_id=z["graph_id"])
    G.preCondition()
    assert not G.isSplit()
    assert G.solve() == 0
    assert np.array_equal(G.getAllDistance(), z["dist"])
    assert np.array_equal(G.getMapping(), z["mapping"])
    assert G.solveSubGraph(2) == 0
    assert G.solveSubGraph(2) == 0  # already processed: warning, no work
    off = int(G.C_BlockVer_offset[2])
    sub = int(G.C_BlockVer_num[2])
    assert np.array_equal(G.getSubGraphDistance(2), z["dist"][off:off + sub])
    assert np.array_equal(G.getSubGraphIndex(2), z["mapping"][off:off + sub])
    G.close()


@pytest.mark.parametrize("name", INT_CASES[:4] + F32_CASES[:1])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("with_pred", [True, False])
@pytest.mark.parametrize("direct", [0, 1])
def test_solve_into_page_locked_host_rows(gpu, name, mode, with_pred, direct):
    """Page-locked host results, staged (a device copy moved by the copy
    engines) or direct (inner rows written by the kernels into host memory,
    boundary rows copied out): same rows as a device-resident solve, on two
    calls in a row."""
    z, g = load_golden(name)
    n = g.n
    dtype = gpu.DTYPE_F32 if name.endswith("f32") else gpu.DTYPE_I32
    tdt = torch.float32 if dtype == gpu.DTYPE_F32 else torch.int32
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, int(z["K"]), graph_id=z["graph_id"],
                    dtype=dtype) as eng:
        eng.set_option(gpu._lib.OPT_HOST_RESULTS, direct)
        dd = torch.empty((n, n), dtype=tdt, device="cuda")
        pd = torch.empty((n, n), dtype=torch.int32, device="cuda") if with_pred else None
        eng.solve(dd, pd, mode)
        torch.cuda.synchronize()
        for _ in range(2):
            dh = torch.full((n, n), 7, dtype=tdt).pin_memory()
            ph = torch.full((n, n), 7, dtype=torch.int32).pin_memory() if with_pred else None
            eng.solve(dh, ph, mode)
            assert torch.equal(dh, dd.cpu())
            if with_pred:
                assert torch.equal(ph, pd.cpu())


@pytest.mark.parametrize("f32", [True, False])
@pytest.mark.parametrize("with_pred", [True, False])
def test_host_rows_in_groups_and_slots(gpu, f32, with_pred):
    """Batched solves into page-locked host rows in many groups (about 1 MB
    of rows each, capped at 8): the FP32 engine then stages the rows in two
    slots that the groups take in turn, the int32 engine at their own
    offsets.  Same rows as a device-resident solve, on the first run of the
    plan and on a replay of its captured graph."""
    from fastapsp_gb300 import graphs

    if f32:
        g, dtype, tdt = graphs.road_like(6000, seed=8), gpu.DTYPE_F32, torch.float32
    else:
        g, dtype, tdt = graphs.geometric_knn(n=6000, k=3, seed=8), gpu.DTYPE_I32, torch.int32
    n = g.n
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, 9, dtype=dtype) as eng:
        dd = torch.empty((n, n), dtype=tdt, device="cuda")
        pd = torch.empty((n, n), dtype=torch.int32, device="cuda") if with_pred else None
        eng.solve(dd, pd, 1)
        torch.cuda.synchronize()
        eng.set_option(gpu._lib.OPT_HOST_GROUP_MB, 1)
        assert eng.get_option(gpu._lib.OPT_HOST_GROUP_MB) == 1
        dh = torch.full((n, n), 7, dtype=tdt).pin_memory()
        ph = torch.full((n, n), 7, dtype=torch.int32).pin_memory() if with_pred else None
        for _ in range(2):
            dh.fill_(7)
            if with_pred:
                ph.fill_(7)
            eng.solve(dh, ph, 1)
            assert torch.equal(dh, dd.cpu())
            if with_pred:
                assert torch.equal(ph, pd.cpu())
        with pytest.raises(gpu.FapError):
            eng.set_option(gpu._lib.OPT_HOST_GROUP_MB, 0.5)


def test_batched_solve_repeats_bit_for_bit(gpu):
    """The batched form's overlapped launches (FW lookahead on two streams)
    give the same distances and predecessors on every replay of the captured
    graph, and the same as the plain form."""
    from fastapsp_gb300 import graphs

    g = graphs.geometric_knn(n=6144, k=3, seed=11)
    n = g.n
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, 6, dtype=gpu.DTYPE_I32) as eng:
        outs = []
        for mode in (1, 1, 1, 0):
            d = torch.empty((n, n), dtype=torch.int32, device="cuda")
            p = torch.empty((n, n), dtype=torch.int32, device="cuda")
            eng.solve(d, p, mode)
            torch.cuda.synchronize()
            outs.append((d.cpu(), p.cpu()))
    for d, p in outs[1:]:
        assert torch.equal(d, outs[0][0]) and torch.equal(p, outs[0][1])


@pytest.mark.parametrize("cols", [64, 128])
@pytest.mark.parametrize("name", INT_CASES)
def test_solve_bit_exact_with_either_tile_width(gpu, name, cols):
    """The min-plus tile width (forced instead of tuned) changes no output."""
    z, g = load_golden(name)
    n = g.n
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, int(z["K"]), graph_id=z["graph_id"],
                    dtype=gpu.DTYPE_I32) as eng:
        eng.set_option(gpu._lib.OPT_TILE_COLS, cols)
        assert eng.get_option(gpu._lib.OPT_TILE_COLS) == cols
        d = torch.empty((n, n), dtype=torch.int32, device="cuda")
        p = torch.empty((n, n), dtype=torch.int32, device="cuda")
        eng.solve(d, p, 1)
        torch.cuda.synchronize()
        d, p = d.cpu().numpy(), p.cpu().numpy()
    assert np.array_equal(to_ref_float(d).view(np.int32), z["dist"].view(np.int32))
    m = out_of_part_mask(z)
    assert np.array_equal(p[m], z["path"][m])


def test_autotuners_keep_results(gpu):
    """Tuned, 64-column and 128-column min-plus tiles give the same rows, in
    both forms, on graphs whose parts fall in both K classes of the strip form
    (the tuner's trial launches rewrite the rows of the first run), and the
    same as an engine with the autotuners off; the SSSP tuner of the
    whole-graph search (which the boundary-graph method does not need)
    reports the batch width it chose."""
    from fastapsp_gb300 import graphs

    for g, K in ((graphs.geometric_knn(n=6144, k=3, seed=11), 6), (graphs.grid_graph(64, 64, seed=3), 4)):
        n = g.n
        outs = []
        for tune in (1, 0):
            with gpu.Engine(n, g.row_offset, g.col_val, g.weight, K, dtype=gpu.DTYPE_I32) as eng:
                eng.set_option(gpu._lib.OPT_AUTOTUNE, tune)
                eng.set_option(gpu._lib.OPT_SSSP_METHOD, 1)
                runs = ((0, 1), (64, 1), (128, 1), (0, 0)) if tune else ((0, 1),)
                for cols, mode in runs:
                    eng.set_option(gpu._lib.OPT_TILE_COLS, cols)
                    d = torch.empty((n, n), dtype=torch.int32, device="cuda")
                    p = torch.empty((n, n), dtype=torch.int32, device="cuda")
                    eng.solve(d, p, mode)
                    eng.solve(d, p, mode)  # the second run uses the tuned widths
                    torch.cuda.synchronize()
                    outs.append((d.cpu(), p.cpu()))
                lanes = eng.get_option(gpu._lib.OPT_SSSP_LANES)
                assert lanes in ((8, 16, 32) if tune else (0,))
        for d, p in outs[1:]:
            assert torch.equal(d, outs[0][0]) and torch.equal(p, outs[0][1])


def test_set_partition_matches_a_fresh_engine(gpu):
    """fap_set_partition on a solved engine gives the mapping and the rows of
    an engine created with that partition; fap_precondition keeps them;
    fap_solve_all / fap_solve_batched are fap_solve in each mode."""
    from fastapsp_gb300 import graphs
    from fastapsp_gb300._lib import check, ptr

    g = graphs.geometric_knn(n=4096, k=3, seed=5)
    n, K = g.n, 4
    gid_a, _ = gpu.partition(g.row_offset, g.col_val, K)
    gid_b = (np.arange(n) * K // n + 1).astype(np.int32)  # contiguous id blocks
    outs = []
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, K, graph_id=gid_a, dtype=gpu.DTYPE_I32) as eng:
        d = torch.empty((n, n), dtype=torch.int32, device="cuda")
        p = torch.empty((n, n), dtype=torch.int32, device="cuda")
        eng.solve(d, p, 1)
        eng.set_partition(gid_b)
        assert np.array_equal(eng.graph_id(), gid_b)
        mapping = eng.mapping()
        eng.precondition()
        assert np.array_equal(eng.mapping(), mapping)
        for fn in ("fap_solve_batched", "fap_solve_all"):
            check(getattr(gpu.lib(), fn)(eng._h, ptr(d), ptr(p), None), fn)
            torch.cuda.synchronize()
            outs.append((d.cpu(), p.cpu()))
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, K, graph_id=gid_b, dtype=gpu.DTYPE_I32) as ref:
        assert np.array_equal(ref.mapping(), mapping)
        d2 = torch.empty((n, n), dtype=torch.int32, device="cuda")
        p2 = torch.empty((n, n), dtype=torch.int32, device="cuda")
        ref.solve(d2, p2, 1)
        torch.cuda.synchronize()
        d2, p2 = d2.cpu(), p2.cpu()
    for d, p in outs:
        assert torch.equal(d, d2) and torch.equal(p, p2)
