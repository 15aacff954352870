"""Generates the golden fixtures of tests/golden/ by running the reference's
own fapGraph (compiled from its sources by `make -C oracle ref`).

For each case: a seeded graph is written as a MatrixMarket file under a
scratch working directory (graph/<type>/<name>.mtx, the path the reference's
reader expects), partitioned by the engine's partitioner, and solved by the
reference binary with that partition (solve() for every case, plus
solveSubGraph() for two parts of the last case).  The fixture stores the input
lines, the partition, the reference's mapping and its dist/path outputs.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle  # noqa: E402
from fastapsp_gb300 import graphs  # noqa: E402
from fastapsp_gb300.engine import partition  # noqa: E402

OUT = Path(__file__).resolve().parent


def cases():
    yield "grid8_full", graphs.grid_graph(8, 8, p=1.0, seed=1), 4
    yield "grid12_tree", graphs.grid_graph(12, 12, p=0.6, seed=2), 4
    yield "rand50_dir_int", graphs.small_random_graph(50, 160, True, True, seed=3), 3
    yield "rand60_undir_f32", graphs.small_random_graph(60, 120, False, True, seed=4, integer=False), 4
    yield "knn300_dir_int", graphs.geometric_knn(300, seed=5), 5
    yield "road300_f32", graphs.road_like(300, seed=6), 6
    yield "rand40_k1", graphs.small_random_graph(40, 90, True, True, seed=7), 1
    yield "tiny10_k3", graphs.small_random_graph(10, 12, False, False, seed=8), 3
    yield "grid16_sub", graphs.grid_graph(16, 16, p=0.6, seed=9), 5
    # integer weights up to 3.5e6 on 300 vertices: (n - 1) * max weight stays
    # below 2^30 (the int32 engine's limit) while many distances exceed
    # 2^24 - 1, where the engine must leave its packed keys for the wide form
    # and where the reference's FP32 arithmetic is no longer exact
    yield "bigw300_dir_wide", graphs.small_random_graph(300, 650, True, True, seed=10, wmax=3_500_000), 4
    # rows of n = 301 and 303 entries are not 16-byte aligned: the min-plus
    # stores them with its realigned form
    yield "knn301_dir_int", graphs.geometric_knn(301, seed=12), 5
    yield "road303_f32", graphs.road_like(303, seed=13), 6


def main():
    only = set(sys.argv[1:])  # case names to (re)generate; all when empty
    oracle.build(ref=True)
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        for name, g, K in cases():
            if only and name not in only:
                continue
            typ = ("weight-" if g.weighted else "unweight-") + ("directed" if g.directed else "undirected")
            (tmp / "graph" / typ).mkdir(parents=True, exist_ok=True)
            graphs.write_mtx(g, str(tmp / "graph" / typ / f"{name}.mtx"))
            gid, _ = partition(g.row_offset, g.col_val, K)
            pfile = tmp / f"{name}.part"
            gid.astype("<i4").tofile(pfile)
            outdir = tmp / name
            outdir.mkdir()
            parts = [1, K] if name == "grid16_sub" else None
            oracle.run_reference(tmp, name, g.directed, g.weighted, K, pfile, outdir)
            n = g.n
            rec = dict(
                n=np.int32(n), K=np.int32(K), directed=np.int8(g.directed),
                weighted=np.int8(g.weighted), lines_src=g.lines_src, lines_dst=g.lines_dst,
                lines_w=g.lines_w, graph_id=gid,
                mapping=np.fromfile(outdir / "mapping.i32", "<i4"),
                dist=np.fromfile(outdir / "dist.f32", "<f4").reshape(n, n),
                path=np.fromfile(outdir / "path.i32", "<i4").reshape(n, n),
            )
            if parts:
                sub_out = tmp / (name + "_sub")
                sub_out.mkdir()
                oracle.run_reference(tmp, name, g.directed, g.weighted, K, pfile, sub_out, parts)
                for p in parts:
                    rec[f"sub{p}_dist"] = np.fromfile(sub_out / f"dist_{p}.f32", "<f4").reshape(-1, n)
                    rec[f"sub{p}_path"] = np.fromfile(sub_out / f"path_{p}.i32", "<i4").reshape(-1, n)
                    rec[f"sub{p}_index"] = np.fromfile(sub_out / f"index_{p}.i32", "<i4")
            np.savez_compressed(OUT / f"{name}.npz", **rec)
            print(name, n, K, "ok")


if __name__ == "__main__":
    main()
