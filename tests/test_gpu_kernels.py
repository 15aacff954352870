"""Parity of the standalone sm_103a kernels against the CPU oracle, called
through the C ABI on device memory."""
import numpy as np
import pytest
import torch
from helpers import INF_I32, MAXV, check_pred_tight

from fastapsp_gb300 import graphs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu):
    c = gpu.Context(0)
    yield c
    c.close()


def rand_dist(rng, shape, inf_frac, f32):
    if f32:
        a = rng.uniform(0.1, 50.0, size=shape).astype(np.float32)
        a[rng.random(shape) < inf_frac] = MAXV
    else:
        a = rng.integers(0, 1000, size=shape).astype(np.int32)
        a[rng.random(shape) < inf_frac] = INF_I32
    return a


def as_oracle(a):
    if a.dtype == np.int32:
        o = a.astype(np.float32)
        o[a >= INF_I32] = MAXV
        return o
    return a


@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (31, 33, 7), (64, 64, 64), (65, 129, 33), (200, 300, 130),
                                   (130, 70, 0), (5, 1000, 257), (300, 2100, 29), (129, 2053, 48),
                                   (257, 4100, 49), (150, 700, 100), (70, 300, 101), (200, 2200, 32),
                                   (131, 1100, 33)])
def test_minplus_matches_oracle(ctx, oracle_lib, f32, M, N, K):
    rng = np.random.default_rng(M * 1000 + N * 10 + K)
    A = rand_dist(rng, (M, K), 0.2, f32)
    B = rand_dist(rng, (K, N), 0.2, f32)
    # ties: force duplicate minima so the first-k rule matters, within a group
    # of four steps (k = 0, 1) and across groups (k = 2, 6)
    if K > 3:
        B[1] = B[0]
        A[:, 1] = A[:, 0]
    if K > 6:
        B[6] = B[2]
        A[:, 6] = A[:, 2]
    Bp = rng.integers(0, 10**6, size=(K, N)).astype(np.int32)
    ref_c, ref_p = oracle_lib.min_plus(as_oracle(A), as_oracle(B), Bp)
    dt = torch.float32 if f32 else torch.int32
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dBp = torch.from_numpy(Bp).cuda()
    dC = torch.full((M, N), 7, dtype=dt, device="cuda")
    dCp = torch.full((M, N), 7, dtype=torch.int32, device="cuda")
    ctx.minplus(0 if f32 else 1, dA, dB, dC, dBp, dCp, M=M, N=N, K=K,
                lda=max(K, 1), ldb=N, ldc=N)
    torch.cuda.synchronize()
    c = dC.cpu().numpy()
    assert np.array_equal(as_oracle(c).view(np.int32), ref_c.view(np.int32))
    assert np.array_equal(dCp.cpu().numpy(), ref_p)


def make_dense(rng, n, density, f32):
    W = rand_dist(rng, (n, n), 1.0 - density, f32)
    if f32:
        W = np.where(W < MAXV, W, MAXV).astype(np.float32)
    np.fill_diagonal(W, 0)
    P = np.where(as_oracle(W) < MAXV, np.arange(n)[:, None], -1).astype(np.int32)
    return W, P


@pytest.mark.parametrize("f32", [False, True])
def test_floyd_batched_matches_oracle(ctx, oracle_lib, f32):
    rng = np.random.default_rng(7 + f32)
    # (sizes that are multiples of 4 have 16-byte rows: their remaining tiles
    # are staged by bulk tensor copies, boxes past the edge included)
    sizes = [1, 5, 63, 64, 65, 130, 132, 200, 257, 260]
    mats, preds, dev_d, dev_p = [], [], [], []
    for n in sizes:
        W, P = make_dense(rng, n, 0.08, f32)
        mats.append(W)
        preds.append(P)
        dev_d.append(torch.from_numpy(W).cuda())
        dev_p.append(torch.from_numpy(P).cuda())
    ctx.floyd_batched(0 if f32 else 1, dev_d, dev_p)
    torch.cuda.synchronize()
    for W, P, dd, dp in zip(mats, preds, dev_d, dev_p):
        n = W.shape[0]
        ref_d, _ = oracle_lib.floyd_path(as_oracle(W), P)
        got = as_oracle(dd.cpu().numpy())
        gp = dp.cpu().numpy()
        if f32:
            fin = ref_d < MAXV
            assert np.array_equal(fin, got < MAXV)
            assert np.allclose(got[fin], ref_d[fin], rtol=1e-6, atol=0)
        else:
            assert np.array_equal(got, ref_d)
        # predecessors: tight edges of the input matrix
        Wf = as_oracle(W).astype(np.float64)
        Wf[Wf >= MAXV] = np.inf
        np.fill_diagonal(Wf, np.inf)
        ro = np.zeros(n + 1, np.int64)
        rows, cols = np.nonzero(np.isfinite(Wf))
        np.add.at(ro, rows + 1, 1)
        ro = np.cumsum(ro)
        check_pred_tight(got, gp, np.arange(n), n, ro, cols, Wf[rows, cols],
                         rtol=1e-6 if f32 else 0.0)


@pytest.mark.parametrize("kind", ["grid", "knn_int", "road_f32", "rand_dir_int"])
def test_sssp_matches_dijkstra_bit_for_bit(gpu, oracle_lib, kind):
    if kind == "grid":
        g, dtype = graphs.grid_graph(40, 40, seed=1), gpu.DTYPE_I32
    elif kind == "knn_int":
        g, dtype = graphs.geometric_knn(3000, seed=2), gpu.DTYPE_I32
    elif kind == "road_f32":
        g, dtype = graphs.road_like(5000, seed=3), gpu.DTYPE_F32
    else:
        g, dtype = graphs.small_random_graph(500, 1500, True, True, seed=4), gpu.DTYPE_I32
    rng = np.random.default_rng(0)
    src = rng.choice(g.n, size=min(70, g.n), replace=False).astype(np.int32)
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, 2, dtype=dtype) as eng:
        dt = torch.int32 if dtype == gpu.DTYPE_I32 else torch.float32
        d = torch.empty((len(src), g.n), dtype=dt, device="cuda")
        p = torch.empty((len(src), g.n), dtype=torch.int32, device="cuda")
        eng.sssp(src, d, p)
        torch.cuda.synchronize()
        d = as_oracle(d.cpu().numpy())
        p = p.cpu().numpy()
    for i, s in enumerate(src):
        rd, rp = oracle_lib.dijkstra_path(int(s), g.row_offset, g.col_val, g.weight)
        assert np.array_equal(d[i].view(np.int32), rd.view(np.int32)), f"row {i}"
        assert np.array_equal(p[i], rp), f"pred row {i}"


@pytest.mark.parametrize("kind", ["grid", "road_f32"])
def test_sssp_result_independent_of_near_far_step(gpu, oracle_lib, kind):
    """The near-far step and the batch width only order the work: any of
    them gives the reference Dijkstra's distances and predecessors."""
    if kind == "grid":
        g, dtype = graphs.grid_graph(30, 30, seed=2), gpu.DTYPE_I32
    else:
        g, dtype = graphs.road_like(3000, seed=5), gpu.DTYPE_F32
    src = np.random.default_rng(3).choice(g.n, size=40, replace=False).astype(np.int32)
    dt = torch.int32 if dtype == gpu.DTYPE_I32 else torch.float32
    outs = []
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, 2, dtype=dtype) as eng:
        lo = 1e-3 if dtype == gpu.DTYPE_F32 else 1
        for delta, lanes in ((lo, 0), (0.0, 0), (1e9, 0), (0.0, 8), (0.0, 16), (0.0, 32)):
            eng.set_option(gpu._lib.OPT_SSSP_DELTA, delta)
            eng.set_option(gpu._lib.OPT_SSSP_LANES, lanes)
            d = torch.empty((len(src), g.n), dtype=dt, device="cuda")
            p = torch.empty((len(src), g.n), dtype=torch.int32, device="cuda")
            eng.sssp(src, d, p)
            torch.cuda.synchronize()
            outs.append((d.cpu().numpy(), p.cpu().numpy()))
    for d, p in outs[1:]:
        assert np.array_equal(d, outs[0][0]) and np.array_equal(p, outs[0][1])
    for i, s in enumerate(src):
        rd, rp = oracle_lib.dijkstra_path(int(s), g.row_offset, g.col_val, g.weight)
        assert np.array_equal(as_oracle(outs[0][0][i]).view(np.int32), rd.view(np.int32))
        assert np.array_equal(outs[0][1][i], rp)


def test_sssp_large_graph_bitmaps_in_global_memory(gpu, oracle_lib):
    """n = 450,000: the frontier bitmaps (3 x n bits) exceed the shared-memory
    budget and live in device memory; results stay bit-exact."""
    g = graphs.road_like(450_000, seed=21)
    n = g.n
    gid = np.where(np.arange(n) < n // 2, 1, 2).astype(np.int32)
    src = np.random.default_rng(9).choice(n, size=24, replace=False).astype(np.int32)
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, 2, graph_id=gid, dtype=gpu.DTYPE_F32) as eng:
        d = torch.empty((len(src), n), dtype=torch.float32, device="cuda")
        p = torch.empty((len(src), n), dtype=torch.int32, device="cuda")
        eng.sssp(src, d, p)
        torch.cuda.synchronize()
        d = d.cpu().numpy()
        p = p.cpu().numpy()
    for i in (0, 7, 23):
        rd, rp = oracle_lib.dijkstra_path(int(src[i]), g.row_offset, g.col_val, g.weight)
        assert np.array_equal(d[i].view(np.int32), rd.view(np.int32)), f"row {i}"
        assert np.array_equal(p[i], rp), f"pred row {i}"


@pytest.mark.parametrize("lanes", [0, 32])
def test_sssp_fp64_option_rounds_once(gpu, oracle_lib, lanes):
    """With FP64 search the FP32 output is the FP64 distance rounded once
    (16-source batches by default, 32-source batches forced)."""
    g = graphs.road_like(4000, seed=8)
    src = np.random.default_rng(2).choice(g.n, size=33, replace=False).astype(np.int32)
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, 2, dtype=gpu.DTYPE_F32) as eng:
        eng.set_option(gpu._lib.OPT_SSSP_FP64, 1)
        eng.set_option(gpu._lib.OPT_SSSP_LANES, lanes)
        d = torch.empty((len(src), g.n), dtype=torch.float32, device="cuda")
        p = torch.empty((len(src), g.n), dtype=torch.int32, device="cuda")
        eng.sssp(src, d, p)
        torch.cuda.synchronize()
        d = d.cpu().numpy()
        p = p.cpu().numpy()
    for i, s in enumerate(src):
        d64 = oracle_lib.dijkstra_f64(int(s), g.row_offset, g.col_val, g.weight)
        f = d64 < 1e299
        assert np.array_equal(f, d[i] < 1e8)
        assert np.array_equal(d[i][f], d64[f].astype(np.float32))  # round-to-nearest of FP64
    n = g.n
    check_pred_tight(d.astype(np.float64), p, src, n, g.row_offset, g.col_val, g.weight, rtol=1e-6)


@pytest.mark.parametrize("lanes", [0, 32])
def test_engine_fp64_sssp_option_meets_1e6_on_road_graph(gpu, oracle_lib, lanes):
    g = graphs.road_like(6000, seed=12)
    K = 8
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, K, dtype=gpu.DTYPE_F32) as eng:
        eng.set_option(gpu._lib.OPT_SSSP_FP64, 1)
        eng.set_option(gpu._lib.OPT_SSSP_LANES, lanes)
        n = g.n
        d = torch.empty((n, n), dtype=torch.float32, device="cuda")
        p = torch.empty((n, n), dtype=torch.int32, device="cuda")
        eng.solve(d, p, gpu.MODE_BATCHED)
        torch.cuda.synchronize()
        mapping = eng.mapping()
        rows = np.arange(0, n, 97)
        dd = d[torch.from_numpy(rows).cuda()].cpu().numpy()
    worst = 0.0
    for i, r in enumerate(rows):
        d64 = oracle_lib.dijkstra_f64(int(mapping[r]), g.row_offset, g.col_val, g.weight)
        f = d64 < 1e299
        assert np.array_equal(f, dd[i] < 1e8)
        worst = max(worst, float(np.max(np.abs(dd[i][f] - d64[f]) / np.maximum(d64[f], 1e-30))))
    assert worst <= 1e-6, worst


def test_speed_options_reject_unsupported_widths(gpu):
    """Batch and tile widths are limited to the kernels that exist; a rejected
    value leaves the option as it was."""
    g = graphs.grid_graph(16, 16, seed=4)
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, 2, dtype=gpu.DTYPE_I32) as eng:
        for opt, bad, good in ((gpu._lib.OPT_SSSP_LANES, 12, 8), (gpu._lib.OPT_TILE_COLS, 48, 128)):
            eng.set_option(opt, good)
            with pytest.raises(gpu._lib.FapError):
                eng.set_option(opt, bad)
            assert eng.get_option(opt) == good


def test_addmin_peak_probe_modes(ctx):
    """The register-only add-min probe (the roofline denominator) runs every
    form and rejects unknown ones; the DPX form outruns the forms that keep
    an index beside each value."""
    rates = {m: ctx.addmin_peak(m) for m in range(13)}
    assert all(r > 1e11 for r in rates.values()), rates
    assert rates[0] > rates[3] and rates[12] > rates[3]
    from fastapsp_gb300._lib import FapError
    with pytest.raises(FapError):
        ctx.addmin_peak(13)
