"""Seeded synthetic graphs of the shapes the Fast-APSP workloads are quoted on.

Every generator returns a :class:`Graph`: a CSR built with the same rules as
the reference's MatrixMarket reader (``fap/utils/readMatFile.h:66-173``):
undirected input lines become two directed entries, and each CSR row lists
its entries in reverse input order (the reader prepends to per-vertex linked
lists).  ``write_mtx`` writes the input lines so that the reference's reader
rebuilds exactly the same CSR from the file.

Workload shapes:
  * ``grid_graph``        128x128 grid, random spanning tree + each other grid
                          edge kept with p=0.6, unweighted, undirected.
  * ``geometric_knn``     65,536 points in the unit square, each joined to its 3
                          nearest neighbours (directed), integer weights
                          U[1,1000].
  * ``road_like``         perturbed planar grid thinned to a near-tree and
                          subdivided by degree-2 chains to 114,599 vertices and
                          ~239k directed entries; FP32 weights U[0.1,10].
  * ``dense_instances``   dense int32 adjacency matrices, sizes log-uniform.
  * ``regular_digraphs``  random 4-regular directed graphs, FP32 weights.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Graph:
    n: int
    row_offset: np.ndarray  # int32 [n+1]
    col_val: np.ndarray  # int32 [m]
    weight: np.ndarray  # float32 [m]
    directed: bool
    weighted: bool
    # The input lines (0-based ids) the CSR was built from, for write_mtx.
    lines_src: np.ndarray
    lines_dst: np.ndarray
    lines_w: np.ndarray
    integer_weights: bool = True
    # Planar coordinates of the vertices where the generator has them (n x 2;
    # None otherwise): the input of geometric partitioning baselines.
    coords: np.ndarray = None

    @property
    def m(self) -> int:
        return int(self.col_val.shape[0])

    @property
    def adj_size(self) -> np.ndarray:
        return np.diff(self.row_offset).astype(np.int32)


def csr_from_lines(n, src, dst, w, directed, weighted, integer_weights=True) -> Graph:
    """CSR with the reference reader's entry order (see module docstring)."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    w = np.abs(np.asarray(w, dtype=np.float64)).astype(np.float32)
    if not weighted:
        w = np.ones_like(w, dtype=np.float32)
    nl = src.shape[0]
    if directed:
        rows, cols, ws = src, dst, w
        seq = np.arange(nl, dtype=np.int64)
    else:
        rows = np.empty(2 * nl, dtype=np.int64)
        cols = np.empty(2 * nl, dtype=np.int64)
        rows[0::2], rows[1::2] = src, dst
        cols[0::2], cols[1::2] = dst, src
        ws = np.repeat(w, 2)
        seq = np.arange(2 * nl, dtype=np.int64)
    # Row-major, and inside a row the newest entry first.
    order = np.lexsort((-seq, rows))
    col_val = cols[order].astype(np.int32)
    weight = ws[order].astype(np.float32)
    counts = np.bincount(rows, minlength=n)[:n]
    row_offset = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=row_offset[1:])
    return Graph(n=int(n), row_offset=row_offset.astype(np.int32), col_val=col_val,
                 weight=weight, directed=bool(directed), weighted=bool(weighted),
                 lines_src=src.astype(np.int32), lines_dst=dst.astype(np.int32),
                 lines_w=w.astype(np.float32), integer_weights=bool(integer_weights))


def write_mtx(g: Graph, path: str) -> None:
    """MatrixMarket file whose reference-reader CSR equals ``g``'s CSR."""
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{g.n} {g.n} {g.lines_src.shape[0]}\n")
        a = g.lines_src.astype(np.int64) + 1
        b = g.lines_dst.astype(np.int64) + 1
        if g.weighted:
            ws = g.lines_w
            body = "\n".join(f"{x} {y} {float(v):.9g}" for x, y, v in zip(a.tolist(), b.tolist(), ws.tolist()))
        else:
            body = "\n".join(f"{x} {y}" for x, y in zip(a.tolist(), b.tolist()))
        f.write(body)
        f.write("\n")


def _spanning_tree_mask(n, eu, ev, rng):
    """Random spanning forest (Kruskal over a random edge order)."""
    parent = np.arange(n)

    def find(x):
        root = x
        while parent[root] != root:
            root = parent[root]
        while parent[x] != root:
            parent[x], x = root, parent[x]
        return root

    order = rng.permutation(eu.shape[0])
    mask = np.zeros(eu.shape[0], dtype=bool)
    for e in order.tolist():
        a, b = find(int(eu[e])), find(int(ev[e]))
        if a != b:
            parent[a] = b
            mask[e] = True
    return mask


def _grid_edges(rows, cols):
    idx = np.arange(rows * cols).reshape(rows, cols)
    h = np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1)
    v = np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], 1)
    e = np.concatenate([h, v], 0)
    return e[:, 0], e[:, 1]


def grid_graph(rows=128, cols=128, p=0.6, seed=20261204) -> Graph:
    """Undirected unweighted grid: random spanning tree + each other edge w.p. p."""
    rng = np.random.default_rng(seed)
    eu, ev = _grid_edges(rows, cols)
    tree = _spanning_tree_mask(rows * cols, eu, ev, rng)
    keep = tree | (rng.random(eu.shape[0]) < p)
    sel = np.nonzero(keep)[0]
    sel = sel[rng.permutation(sel.shape[0])]  # input line order
    w = np.ones(sel.shape[0], dtype=np.float32)
    g = csr_from_lines(rows * cols, eu[sel], ev[sel], w, directed=False, weighted=False)
    g.coords = np.stack(np.divmod(np.arange(rows * cols), cols), 1).astype(np.float64)
    return g


def geometric_knn(n=65536, k=3, wmin=1, wmax=1000, seed=20261205) -> Graph:
    """Directed k-nearest-neighbour graph of uniform points, integer weights."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    tree = cKDTree(pts)
    _, nn = tree.query(pts, k=k + 1)
    src = np.repeat(np.arange(n), k)
    dst = nn[:, 1:].reshape(-1)
    w = rng.integers(wmin, wmax + 1, size=src.shape[0]).astype(np.float32)
    g = csr_from_lines(n, src, dst, w, directed=True, weighted=True)
    g.coords = pts
    return g


def road_like(n_target=114599, extra_ratio=0.0442, wmin=0.1, wmax=10.0, seed=20261207) -> Graph:
    """Near-tree planar road network: thinned perturbed grid + degree-2 chains.

    A grid of about n/6 junctions keeps a random spanning tree plus
    ``extra_ratio * n`` further grid edges (the cycles of a road net); the
    remaining vertices are inserted as degree-2 chain vertices on random edges
    until the graph has ``n_target`` vertices.  Undirected, FP32 weights.
    """
    rng = np.random.default_rng(seed)
    side = int(math.sqrt(n_target / 5.5))
    rows, cols = side, side
    n0 = rows * cols
    eu, ev = _grid_edges(rows, cols)
    tree = _spanning_tree_mask(n0, eu, ev, rng)
    extra_n = int(round(extra_ratio * n_target))
    non_tree = np.nonzero(~tree)[0]
    extra = rng.choice(non_tree, size=min(extra_n, non_tree.shape[0]), replace=False)
    sel = np.concatenate([np.nonzero(tree)[0], extra])
    bu, bv = eu[sel], ev[sel]
    n_chain = n_target - n0
    # distribute chain vertices over the base edges
    per_edge = np.bincount(rng.integers(0, bu.shape[0], size=n_chain), minlength=bu.shape[0])
    src, dst = [], []
    xy = np.zeros((n_target, 2))
    xy[:n0] = np.stack(np.divmod(np.arange(n0), cols), 1)
    nxt = n0
    for a, b, c in zip(bu.tolist(), bv.tolist(), per_edge.tolist()):
        prev = a
        for i in range(c):  # chain vertices evenly along the junctions' segment
            xy[nxt] = xy[a] + (xy[b] - xy[a]) * (i + 1) / (c + 1)
            src.append(prev)
            dst.append(nxt)
            prev = nxt
            nxt += 1
        src.append(prev)
        dst.append(b)
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    # relabel so chain vertices are not all at the end (the road file is unordered)
    perm = rng.permutation(n_target)
    src, dst = perm[src], perm[dst]
    order = rng.permutation(src.shape[0])
    src, dst = src[order], dst[order]
    w = rng.uniform(wmin, wmax, size=src.shape[0]).astype(np.float32)
    g = csr_from_lines(n_target, src, dst, w, directed=False, weighted=True, integer_weights=False)
    coords = np.empty_like(xy)
    coords[perm] = xy
    g.coords = coords
    return g


def regular_digraph(n, degree=4, wlo=0.5, whi=2.0, rng=None) -> Graph:
    """Random ``degree``-regular digraph: union of permutations, no self loops
    or parallel edges (rejection on a per-permutation basis)."""
    rng = rng if rng is not None else np.random.default_rng(0)
    src_l, dst_l = [], []
    used = set()
    for _ in range(degree):
        for _attempt in range(1000):
            perm = rng.permutation(n)
            if np.any(perm == np.arange(n)):
                continue
            pairs = set(zip(range(n), perm.tolist()))
            if pairs & used:
                continue
            used |= pairs
            src_l.append(np.arange(n))
            dst_l.append(perm)
            break
        else:
            raise RuntimeError("could not draw a regular digraph")
    src = np.concatenate(src_l)
    dst = np.concatenate(dst_l)
    w = rng.uniform(wlo, whi, size=src.shape[0]).astype(np.float32)
    w = np.maximum(w, np.nextafter(np.float32(wlo), np.float32(whi)))
    return csr_from_lines(n, src, dst, w, directed=True, weighted=True, integer_weights=False)


def regular_digraphs(count=256, nmin=256, nmax=1024, seed=20261208):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=count)
    return [regular_digraph(int(s), rng=rng) for s in sizes]


INF_I32 = 1 << 30


def dense_instances(count=512, nmin=32, nmax=2048, density=0.05, wmin=1, wmax=100,
                    seed=20261206):
    """Dense int32 adjacency matrices (INF = 2^30 off-edge, 0 on the diagonal).
    Sizes log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=count)).astype(np.int64)
    sizes = np.clip(sizes, nmin, nmax)
    mats = []
    for s in sizes.tolist():
        a = np.full((s, s), INF_I32, dtype=np.int32)
        mask = rng.random((s, s)) < density
        a[mask] = rng.integers(wmin, wmax + 1, size=int(mask.sum()), dtype=np.int32)
        np.fill_diagonal(a, 0)
        mats.append(a)
    return mats


def small_random_graph(n, m_lines, directed, weighted, seed, integer=True, wmax=20):
    """Small random graph for parity tests (may be disconnected, may contain
    self loops and parallel edges, like arbitrary MatrixMarket input)."""
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, size=m_lines)
    dst = rng.integers(0, n, size=m_lines)
    if integer:
        w = rng.integers(1, wmax + 1, size=m_lines).astype(np.float32)
    else:
        w = rng.uniform(0.1, 10.0, size=m_lines).astype(np.float32)
    return csr_from_lines(n, src, dst, w, directed=directed, weighted=weighted,
                          integer_weights=integer or not weighted)
