"""The adjoint (dLoss/dw along argmin paths) against path-count gradients from
CPU Dijkstra and against central finite differences of an FP64 oracle, with a
torch.autograd.Function over the C ABI as the harness (test-only)."""
import numpy as np
import pytest
import torch

from fastapsp_gb300 import graphs

pytestmark = pytest.mark.gpu

MAXV = 1e8


def dense_from_graph(g):
    n = g.n
    W = np.full((n, n), MAXV, np.float32)
    src = np.repeat(np.arange(n), np.diff(g.row_offset))
    W[src, g.col_val] = g.weight
    np.fill_diagonal(W, 0)
    P = np.where(W < MAXV, np.arange(n)[:, None], -1).astype(np.int32)
    return W, P


class APSPPairs(torch.autograd.Function):
    """loss-side view: D[b][s][t] for the given pairs; weights are the edge
    weight vectors of the graphs (CSR order).  Forward = batched FW with
    predecessors through fap_floyd_batched, backward = fap_backward_dense."""

    @staticmethod
    def forward(ctx, ctx_handle, gs, b, s, t, *weights):
        mats, preds = [], []
        for g, w in zip(gs, weights):
            n = g.n
            W = torch.full((n, n), MAXV, dtype=torch.float32, device="cuda")
            src = torch.repeat_interleave(torch.arange(n, device="cuda"),
                                          torch.from_numpy(np.diff(g.row_offset)).cuda())
            col = torch.from_numpy(g.col_val.astype(np.int64)).cuda()
            W[src, col] = w
            W.fill_diagonal_(0)
            P = torch.where(W < MAXV, torch.arange(n, device="cuda", dtype=torch.int32)[:, None],
                            torch.full((1, 1), -1, dtype=torch.int32, device="cuda")).contiguous()
            mats.append(W)
            preds.append(P)
        ctx_handle.floyd_batched(0, mats, preds)
        out = torch.stack([mats[bi][si, ti] for bi, si, ti in zip(b.tolist(), s.tolist(), t.tolist())])
        ctx.save_for_backward(b, s, t)
        ctx.handle, ctx.gs, ctx.preds = ctx_handle, gs, preds
        return out

    @staticmethod
    def backward(ctx, grad):
        b, s, t = ctx.saved_tensors
        dWs = [torch.zeros((g.n, g.n), dtype=torch.float32, device="cuda") for g in ctx.gs]
        ctx.handle.backward_dense(ctx.preds, dWs, b.int().cuda(), s.int().cuda(), t.int().cuda(),
                                  grad.float().contiguous().cuda())
        torch.cuda.synchronize()
        gw = []
        for g, dW in zip(ctx.gs, dWs):
            src = torch.repeat_interleave(torch.arange(g.n, device="cuda"),
                                          torch.from_numpy(np.diff(g.row_offset)).cuda())
            col = torch.from_numpy(g.col_val.astype(np.int64)).cuda()
            gw.append(dW[src, col])
        return (None, None, None, None, None, *gw)


def path_counts(oracle_lib, gs, b, s, t):
    """dLoss/dw for loss = sum of D[s,t]: edges on each Dijkstra path, counted."""
    grads = [np.zeros(g.m, np.float64) for g in gs]
    cache = {}
    for bi, si, ti in zip(b, s, t):
        g = gs[bi]
        key = (bi, si)
        if key not in cache:
            cache[key] = oracle_lib.dijkstra_path(si, g.row_offset, g.col_val, g.weight)
        d, p = cache[key]
        v = ti
        if p[v] < 0:
            continue
        while v != si:
            u = p[v]
            es = np.arange(g.row_offset[u], g.row_offset[u + 1])
            es = es[g.col_val[es] == v]
            e = es[np.argmin(g.weight[es])]
            grads[bi][e] += 1.0
            v = u
    return grads


def fp64_loss(oracle_lib, gs, b, s, t, weights):
    tot = 0.0
    cache = {}
    for bi, si, ti in zip(b, s, t):
        key = (bi, si)
        if key not in cache:
            g = gs[bi]
            cache[key] = oracle_lib.dijkstra_f64(si, g.row_offset, g.col_val, weights[bi])
        d = cache[key][ti]
        if d < 1e299:
            tot += d
    return tot


def test_adjoint_matches_path_counts_and_finite_differences(gpu, oracle_lib):
    rng = np.random.default_rng(5)
    gs = [graphs.regular_digraph(int(n), rng=rng) for n in rng.integers(40, 140, size=6)]
    npairs = 400
    b = rng.integers(0, len(gs), size=npairs)
    s = np.array([rng.integers(0, gs[i].n) for i in b])
    t = np.array([rng.integers(0, gs[i].n) for i in b])
    ctx = gpu.Context(0)
    ws = [torch.tensor(g.weight, device="cuda", requires_grad=True) for g in gs]
    out = APSPPairs.apply(ctx, gs, torch.from_numpy(b), torch.from_numpy(s), torch.from_numpy(t), *ws)
    loss = out.sum()
    loss.backward()
    got = [w.grad.cpu().numpy().astype(np.float64) for w in ws]
    ref = path_counts(oracle_lib, gs, b, s, t)
    for gi, (a, r) in enumerate(zip(got, ref)):
        assert np.array_equal(a, r), f"graph {gi}"
    # forward values against FP64 Dijkstra
    d = out.detach().cpu().numpy()
    for k in range(0, npairs, 37):
        g = gs[b[k]]
        d64 = oracle_lib.dijkstra_f64(int(s[k]), g.row_offset, g.col_val, g.weight)[t[k]]
        assert abs(d[k] - d64) <= 1e-6 * max(d64, 1.0)
    # central finite differences (h = 1e-3) in FP64 on a few edges
    h = 1e-3
    base_w = [g.weight.astype(np.float64) for g in gs]
    for gi in range(2):
        for e in rng.choice(gs[gi].m, size=5, replace=False):
            wp = [w.copy() for w in base_w]
            wm = [w.copy() for w in base_w]
            wp[gi][e] += h
            wm[gi][e] -= h
            fd = (fp64_loss(oracle_lib, gs, b, s, t, wp) - fp64_loss(oracle_lib, gs, b, s, t, wm)) / (2 * h)
            assert abs(fd - got[gi][e]) < 1e-6, (gi, e, fd, got[gi][e])
    ctx.close()


def test_graph_backward_matches_path_counts(gpu, oracle_lib):
    g = graphs.road_like(1500, seed=9)
    K = 6
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, K, dtype=gpu.DTYPE_F32) as eng:
        n = g.n
        dist = torch.empty((n, n), dtype=torch.float32, device="cuda")
        pred = torch.empty((n, n), dtype=torch.int32, device="cuda")
        eng.solve(dist, pred, gpu.MODE_BATCHED)
        rng = np.random.default_rng(1)
        s = rng.integers(0, n, size=300).astype(np.int32)
        t = rng.integers(0, n, size=300).astype(np.int32)
        gw = torch.ones(300, dtype=torch.float32, device="cuda")
        dw = torch.zeros(g.m, dtype=torch.float32, device="cuda")
        eng.backward(pred, torch.from_numpy(s).cuda(), torch.from_numpy(t).cuda(), gw, dw)
        torch.cuda.synchronize()
        got = dw.cpu().numpy().astype(np.float64)
    ref = path_counts(oracle_lib, [g], np.zeros(300, np.int64), s, t)[0]
    assert np.array_equal(got, ref)
