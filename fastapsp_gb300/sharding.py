"""Assignment of parts to GPUs for multi-process runs.

Parts are independent once every rank holds the CSR (the reference's MPI
layer broadcasts metadata and never gathers results,
fap/fap_more_task_mpi.cpp:34-91, and balances by a random shuffle, :39).
Here parts go to ranks by longest-processing-time first on an estimated cost
per part:  sub^3 (Floyd-Warshall) + inner * n * bdy (min-plus)
+ bdy * (n + m) (SSSP rows).  Each rank then solves its own parts with
fap_solve_part; no collective touches the distance data.
"""
from __future__ import annotations

import heapq

import numpy as np


def part_costs(ver_num, bdy_num, n: int, m: int) -> np.ndarray:
    """Estimated work of parts 1..K (index 0 of the K+1 arrays is unused)."""
    sub = np.asarray(ver_num[1:], np.float64)
    bdy = np.asarray(bdy_num[1:], np.float64)
    return sub ** 3 + (sub - bdy) * n * bdy + bdy * (n + m)


def assign_parts(ver_num, bdy_num, n: int, m: int, world: int):
    """Part ids (1-based) per rank, LPT on part_costs; deterministic."""
    costs = part_costs(ver_num, bdy_num, n, m)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i + 1)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(x) for x in out]
