"""Result consumers: point-to-point distances and paths, and solves of a
subset of the parts.

* fap::fapGraph::getDistanceP2P / getPathP2P (source, target) of the drop-in
  class -- the reference declares them without bodies (fap/fap.cpp:674-680)
  -- after solve() and after solveSubGraph(), and the same getters of the
  Python mirror;
* fap_query on device-resident solve() rows (no copy of the n x n rows to
  the host): distances equal the rows, paths are walks of tight edges from s
  to t that match the predecessor rows, unreached pairs have no path, and
  paths longer than the caller's slots only report their length;
* fap_solve_parts with each rank's share of a cost-balanced assignment
  (the part-sharded multi-GPU run, emulated one share after another on the
  one GPU): the shares' rows are the full solve's rows.

Distances are checked against the oracle's Dijkstra."""
import subprocess

import numpy as np
import pytest
import torch
from conftest import ROOT, load_golden

from fastapsp_gb300 import graphs
from fastapsp_gb300.sharding import assign_parts

pytestmark = pytest.mark.gpu
LIB = ROOT / "fastapsp_gb300"


def _edge_weights(g):
    src = np.repeat(np.arange(g.n), np.diff(g.row_offset))
    W = {}
    for u, v, w in zip(src.tolist(), g.col_val.tolist(), g.weight.tolist()):
        W.setdefault((u, v), []).append(w)
    return W


def _check_path(path, s, t, d, W, tol):
    assert path[0] == s and path[-1] == t
    tot = 0.0
    for u, v in zip(path[:-1], path[1:]):
        assert (u, v) in W, f"{u}->{v} is not an edge"
        tot += min(W[(u, v)])
    assert abs(tot - d) <= tol * max(1.0, d), (tot, d)


@pytest.mark.parametrize("split", [False, True])
def test_cpp_p2p_getters(gpu, oracle_lib, tmp_path, split):
    z, g = load_golden("knn300_dir_int")
    K = int(z["K"])
    rng = np.random.default_rng(3)
    pairs = rng.integers(0, g.n, size=(60, 2)).astype(np.int32)
    pairs[:5, 1] = pairs[:5, 0]  # s == t
    gid, _ = gpu.partition(g.row_offset, g.col_val, K)  # the class partitions the same way (seed 1)
    pairs = pairs[np.argsort(gid[pairs[:, 0]], kind="stable")]  # one solveSubGraph per source part
    g.row_offset.astype("<i4").tofile(tmp_path / "ro.i32")
    g.col_val.astype("<i4").tofile(tmp_path / "col.i32")
    g.weight.astype("<f4").tofile(tmp_path / "w.f32")
    pairs.astype("<i4").tofile(tmp_path / "queries.i32")
    exe = tmp_path / "p2p_check"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests" / "p2p_check.cpp"),
                        "-L", str(LIB), "-lfastapsp", f"-Wl,-rpath,{LIB}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path), str(K)] + (["split"] if split else []),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    W = _edge_weights(g)
    lines = r.stdout.strip().splitlines()
    assert len(lines) == len(pairs)
    for line in lines:
        f = line.split()
        s, t, d, ln = int(f[0]), int(f[1]), float(f[2]), int(f[3])
        path = [int(x) for x in f[4:]]
        rd, _ = oracle_lib.dijkstra_path(s, g.row_offset, g.col_val, g.weight)
        assert d == float(rd[t]), (s, t, d, rd[t])
        if rd[t] >= 1e8:
            assert ln == 0
        else:
            assert ln == len(path) >= 1
            _check_path(path, s, t, d, W, 0.0)


def test_python_mirror_p2p_getters(gpu, oracle_lib):
    z, g = load_golden("road300_f32")
    G = gpu.FapGraph(g.n, g.m, g.row_offset, g.col_val, g.weight, int(z["K"]), graph_id=z["graph_id"])
    G.preCondition()
    G.solve()
    W = _edge_weights(g)
    for s, t in np.random.default_rng(4).integers(0, g.n, size=(40, 2)):
        d = G.getDistanceP2P(int(s), int(t))
        d64 = oracle_lib.dijkstra_f64(int(s), g.row_offset, g.col_val, g.weight)[t]
        assert abs(d - d64) <= 1e-6 * max(1.0, d64)
        _check_path(G.getPathP2P(int(s), int(t)), int(s), int(t), d, W, 1e-6)
    G.close()


@pytest.mark.parametrize("kind", ["grid_i32", "knn_dir_i32", "road_f32"])
def test_device_queries(gpu, oracle_lib, kind):
    if kind == "grid_i32":
        g, K, dtype = graphs.grid_graph(64, 64, seed=2), 8, gpu.DTYPE_I32
    elif kind == "knn_dir_i32":
        g, K, dtype = graphs.geometric_knn(5000, seed=3), 8, gpu.DTYPE_I32
    else:
        g, K, dtype = graphs.road_like(6000, seed=4), 8, gpu.DTYPE_F32
    n = g.n
    tdt = torch.int32 if dtype == gpu.DTYPE_I32 else torch.float32
    rng = np.random.default_rng(5)
    nq = 3000
    s = rng.integers(0, n, size=nq).astype(np.int32)
    t = rng.integers(0, n, size=nq).astype(np.int32)
    t[:10] = s[:10]
    max_len = 400
    with gpu.Engine(n, g.row_offset, g.col_val, g.weight, K, dtype=dtype) as eng:
        d = torch.empty((n, n), dtype=tdt, device="cuda")
        p = torch.empty((n, n), dtype=torch.int32, device="cuda")
        eng.solve(d, p)
        sd, td = torch.from_numpy(s).cuda(), torch.from_numpy(t).cuda()
        od = torch.empty(nq, dtype=tdt, device="cuda")
        ol = torch.empty(nq, dtype=torch.int32, device="cuda")
        op = torch.full((nq, max_len), -7, dtype=torch.int32, device="cuda")
        eng.query(d, p, sd, td, od, ol, op, max_len)
        torch.cuda.synchronize()
        mapping = eng.mapping()
        inv = np.empty(n, np.int64)
        inv[mapping] = np.arange(n)
        rows = torch.from_numpy(inv[s]).cuda()
        want_d = d[rows, td.long()].cpu().numpy()
        prows = p[rows].cpu().numpy()
        od, ol, op = od.cpu().numpy(), ol.cpu().numpy(), op.cpu().numpy()
        # a path too long for its slots reports its length and writes nothing
        short = torch.full((nq, 2), -7, dtype=torch.int32, device="cuda")
        ol2 = torch.empty(nq, dtype=torch.int32, device="cuda")
        eng.query(d, p, sd, td, torch.empty(nq, dtype=tdt, device="cuda"), ol2, short, 2)
        torch.cuda.synchronize()
        assert np.array_equal(ol2.cpu().numpy(), ol)
        assert np.all(short.cpu().numpy()[ol > 2] == -7)
        bad = torch.tensor([n + 3], dtype=torch.int32, device="cuda")
        with pytest.raises(gpu._lib.FapError):
            eng.query(d, p, bad, bad, torch.empty(1, dtype=tdt, device="cuda"),
                      torch.empty(1, dtype=torch.int32, device="cuda"))
    assert np.array_equal(od, want_d)
    inf = (1 << 30) if dtype == gpu.DTYPE_I32 else 1e8
    W = _edge_weights(g)
    tol = 2e-6 if dtype == gpu.DTYPE_F32 else 0.0
    checked = 0
    for q in range(nq):
        if od[q] >= inf:
            assert ol[q] == 0
            continue
        ln = int(ol[q])
        assert ln >= 1
        walk, v = [int(t[q])], int(t[q])  # the path the predecessor row gives, walked on the host
        while v != s[q]:
            v = int(prows[q][v])
            walk.append(v)
        assert len(walk) == ln
        if ln <= max_len:
            assert walk[::-1] == list(op[q][:ln])
            if checked < 300:
                _check_path(walk[::-1], int(s[q]), int(t[q]), float(od[q]), W, tol)
                checked += 1
    assert checked > 50
    for q in range(0, nq, 300):  # distances against Dijkstra
        rd, _ = oracle_lib.dijkstra_path(int(s[q]), g.row_offset, g.col_val, g.weight)
        if dtype == gpu.DTYPE_I32:
            assert od[q] == (rd[t[q]] if rd[t[q]] < 1e8 else 1 << 30)
        else:
            assert abs(float(od[q]) - float(rd[t[q]])) <= 1e-6 * max(1.0, float(rd[t[q]]))


@pytest.mark.parametrize("world", [2, 3])
def test_part_shares_equal_the_full_solve(gpu, world):
    g = graphs.geometric_knn(6144, seed=8)
    K = 12
    gid, _ = gpu.partition(g.row_offset, g.col_val, K)
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, K, graph_id=gid, dtype=gpu.DTYPE_I32) as eng:
        d = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
        p = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
        eng.solve(d, p)
        ver = [0] + [eng.part_info(q)[0] for q in range(1, K + 1)]
        bdy = [0] + [eng.part_info(q)[1] for q in range(1, K + 1)]
        shares = assign_parts(ver, bdy, g.n, g.m, world)
        assert sorted(x for sh in shares for x in sh) == list(range(1, K + 1))
        for sh in shares:
            rows = sum(ver[q] for q in sh)
            dd = torch.empty((rows, g.n), dtype=torch.int32, device="cuda")
            pp = torch.empty((rows, g.n), dtype=torch.int32, device="cuda")
            eng.solve_parts(sh[::-1], dd, pp)  # any order: rows follow the list
            r0 = 0
            for q in sh[::-1]:
                sub, _, off = eng.part_info(q)
                assert torch.equal(dd[r0:r0 + sub], d[off:off + sub]), f"part {q}"
                assert torch.equal(pp[r0:r0 + sub], p[off:off + sub]), f"part {q} predecessors"
                r0 += sub
        with pytest.raises(gpu._lib.FapError):
            eng.solve_parts([1, 1], d, p)
