"""Times the reference's own CPU path (oracle/_ref/fap_ref, built from the
reference's fap.cpp by `make ref`) against the oracle restatement on the same
parts of the same graph, with the same host threads.  TEST INFRASTRUCTURE
ONLY: it checks that the CPU baseline the benchmark reports (the
restatement, kind "port") runs at the reference's own speed.  It needs the
reference sources (the x86 build container), so it is not part of the
benchmark.

  python oracle/time_ref_vs_port.py [--config c2] [--parts 1 2] [--threads 8]

Per part it prints the phase times (SSSP, Floyd-Warshall, min-plus, data)
that the reference's fapGraph records (getTime*, fap/fap.cpp:622-639) and the
restatement's own, and checks that the two produce the same rows.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import bench  # noqa: E402  (workload generators and committed partitions)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2", choices=list(bench.WORKLOADS))
    ap.add_argument("--parts", type=int, nargs="*", default=[1])
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    args = ap.parse_args()
    oracle.build(ref=True)
    g, K, gid, _ = bench.load_workload(args.config)
    oracle.set_threads(args.threads)
    res = {"config": args.config, "n": g.n, "K": K, "threads": args.threads, "parts": []}
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        typ = ("weight-" if g.weighted else "unweight-") + ("directed" if g.directed else "undirected")
        (tmp / "graph" / typ).mkdir(parents=True)
        mtx = tmp / "graph" / typ / "g.mtx"
        bench.load_graphs_module().write_mtx(g, str(mtx))
        pfile = tmp / "g.part"
        gid.astype("<i4").tofile(pfile)
        # the reference reads the file itself; the restatement gets the CSR the
        # reference's reader builds from it (the restated reader, pinned to it)
        ro, col, w = oracle.mtx_read(mtx, g.directed, g.weighted)
        pre = oracle.preprocess(K, gid, ro, col)
        for part in args.parts:
            out = tmp / f"out{part}"
            out.mkdir()
            os.environ["OMP_NUM_THREADS"] = str(args.threads)
            t0 = time.perf_counter()
            oracle.run_reference(tmp, "g", g.directed, g.weighted, K, pfile, out, parts=[part])
            wall = time.perf_counter() - t0
            times = dict(line.split() for line in (out / "times.txt").read_text().splitlines())
            ref = {k: float(v) for k, v in times.items()}
            d_ref = np.fromfile(out / f"dist_{part}.f32", "<f4")
            t1 = time.perf_counter()
            d, p, t = oracle.run_part(part, ro, col, w, gid, pre)
            port_wall = time.perf_counter() - t1
            same = bool(np.array_equal(d.reshape(-1), d_ref))
            res["parts"].append({"part": part, "reference_s": ref, "reference_wall_s": wall,
                                 "port_s": t, "port_wall_s": port_wall, "rows_equal": same})
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
