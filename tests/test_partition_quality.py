"""Quality of the engine's multilevel partitioner (the stand-in for the
reference's METIS front end, fap/utils/readIdFile.h:200-283) on the three
benchmark graphs, against recursive coordinate bisection (a geometric
partitioner on the generators' vertex coordinates, balanced medians along the
longer axis) and against contiguous vertex-id blocks.  What the partition
decides is the boundary: the SSSP runs from every boundary vertex and the
min-plus costs sum over parts of inner * n * boundary add-mins, so the test
compares edge cut, boundary vertices and that min-plus work.  No GPU."""
import numpy as np
import pytest

from fastapsp_gb300 import graphs


def part_stats(g, gid, K):
    src = np.repeat(np.arange(g.n), np.diff(g.row_offset))
    cut = gid[src] != gid[g.col_val]
    bnd = np.zeros(g.n, bool)
    bnd[src[cut]] = True
    bnd[g.col_val[cut]] = True
    sub = np.bincount(gid, minlength=K + 1)[1:].astype(np.float64)
    bdy = np.bincount(gid[bnd], minlength=K + 1)[1:].astype(np.float64)
    return dict(cut=int(cut.sum()), boundary=int(bnd.sum()), minplus=float(((sub - bdy) * bdy).sum() * g.n),
                largest=int(sub.max()))


def coordinate_bisection(coords, K):
    gid = np.zeros(coords.shape[0], np.int32)

    def split(idx, k, base):
        if k == 1:
            gid[idx] = base
            return
        c = coords[idx]
        ax = 0 if np.ptp(c[:, 0]) >= np.ptp(c[:, 1]) else 1
        order = idx[np.argsort(c[:, ax], kind="stable")]
        h = order.shape[0] * (k // 2) // k
        split(order[:h], k // 2, base)
        split(order[h:], k - k // 2, base + k // 2)

    split(np.arange(coords.shape[0]), K, 1)
    return gid


@pytest.mark.parametrize("gen,K,margin", [("grid_graph", 16, 0.95), ("geometric_knn", 64, 0.6),
                                          ("road_like", 128, 0.7)])
def test_partitioner_beats_coordinate_bisection(fap_lib, gen, K, margin, record_property):
    g = getattr(graphs, gen)()
    ours = part_stats(g, fap_lib.partition(g.row_offset, g.col_val, K)[0], K)
    rcb = part_stats(g, coordinate_bisection(g.coords, K), K)
    ids = part_stats(g, (np.arange(g.n) * K // g.n + 1).astype(np.int32), K)
    for name, st in (("ours", ours), ("coordinate_bisection", rcb), ("id_blocks", ids)):
        record_property(f"{gen}_{name}", st)
    print(gen, "ours", ours, "coordinate bisection", rcb, "vertex-id blocks", ids)
    assert ours["boundary"] <= margin * rcb["boundary"]
    assert ours["minplus"] <= margin * rcb["minplus"]
    assert ours["boundary"] < ids["boundary"]
    # balance: the largest part stays within 3% of n / K
    assert ours["largest"] <= 1.03 * g.n / K + 1
