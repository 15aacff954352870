"""Writes the part assignments of the benchmark graphs (partition_*.npz).

The benchmark's two arms -- the engine on the GPU and the reference's CPU
algorithm on the host cores -- must solve the same parts of the same graph,
and the reference arm must not load the engine's library to get them.  So the
engine's multilevel partitioner runs once here and its output is committed:
graph_id (1..K, uint8 or uint16), the graph's size and a CRC of its CSR, and
the edge cut.  bench.py checks the CRC against the graph it generates.

  python tests/golden/partitions/make_partitions.py
"""
from __future__ import annotations

import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[2]
sys.path.insert(0, str(ROOT))

CASES = {
    # name: (generator, K)
    "grid_n16384_K16": ("grid_graph", 16),
    "geometric_knn_n65536_K64": ("geometric_knn", 64),
    "road_like_n114599_K128": ("road_like", 128),
}


def csr_crc(g) -> int:
    crc = zlib.crc32(np.ascontiguousarray(g.row_offset, np.int32).tobytes())
    crc = zlib.crc32(np.ascontiguousarray(g.col_val, np.int32).tobytes(), crc)
    return zlib.crc32(np.ascontiguousarray(g.weight, np.float32).tobytes(), crc)


def main() -> None:
    import fastapsp_gb300 as fap
    from fastapsp_gb300 import graphs

    for name, (gen, K) in CASES.items():
        g = getattr(graphs, gen)()
        gid, cut = fap.partition(g.row_offset, g.col_val, K)
        dt = np.uint8 if K < 256 else np.uint16
        np.savez_compressed(HERE / f"partition_{name}.npz", graph_id=gid.astype(dt), n=g.n, m=g.m, K=K,
                            csr_crc=csr_crc(g), edge_cut=cut)
        print(name, g.n, g.m, K, "cut", cut)


if __name__ == "__main__":
    main()
