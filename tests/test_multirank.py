"""Multi-rank path on CPU (gloo, world size 2): every rank takes its parts
from the cost-balanced assignment, solves them (with the CPU oracle standing
in for the per-rank GPU engine, since this container has no GPU), and the
gathered rows equal the single-process solve.  No collective touches the
distance data in the product; the gather here is only the test's check."""
import os

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from fastapsp_gb300 import graphs
from fastapsp_gb300.sharding import assign_parts


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root), str(root / "oracle")]
    import oracle

    from fastapsp_gb300.engine import partition

    g = graphs.grid_graph(20, 20, seed=3)
    K = 6
    gid, _ = partition(g.row_offset, g.col_val, K)
    pre = oracle.preprocess(K, gid, g.row_offset, g.col_val)
    mine = assign_parts(pre["ver_num"], pre["bdy_num"], g.n, g.m, world)[rank]
    rows = {}
    for p in mine:
        d, _, _ = oracle.run_part(p, g.row_offset, g.col_val, g.weight, gid, pre)
        rows[p] = d
    gathered = [None] * world
    dist.all_gather_object(gathered, rows)
    if rank == 0:
        full = {}
        for r in gathered:
            full.update(r)
        D, _, _ = oracle.solve(K, g.row_offset, g.col_val, g.weight, gid)
        ok = sorted(full) == list(range(1, K + 1))
        for p, d in full.items():
            off, sub = int(pre["ver_offset"][p]), int(pre["ver_num"][p])
            ok = ok and np.array_equal(d, D[off:off + sub])
        out.put(bool(ok))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_solve_matches_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert ok
    assert all(p.exitcode == 0 for p in procs)


def test_assignment_balanced_and_complete():
    rng = np.random.default_rng(0)
    K = 64
    ver = np.concatenate([[0], rng.integers(900, 1100, K)])
    bdy = np.concatenate([[0], rng.integers(10, 60, K)])
    for world in (1, 2, 3, 8):
        a = assign_parts(ver, bdy, 65536, 200000, world)
        flat = sorted(p for r in a for p in r)
        assert flat == list(range(1, K + 1))
        from fastapsp_gb300.sharding import part_costs

        c = part_costs(ver, bdy, 65536, 200000)
        loads = [sum(c[p - 1] for p in r) for r in a]
        assert max(loads) <= sum(c) / world + max(c)
