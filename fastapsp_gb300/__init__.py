"""GB300-native Fast-APSP engine.

All-pairs shortest paths by the divide-and-conquer method of
TomerHaham/FastAPSP (partition -> boundary SSSP -> per-part Floyd-Warshall ->
min-plus), with the hot path in hand-written sm_103a CUDA kernels behind the C
ABI in ``include/fastapsp.h`` and the drop-in C++ class in
``include/fap/fap.h``.  This package holds the kernels and the C ABI
(``csrc/``), the in-tree build (``build.py``), a ctypes host layer
(``engine.py``) and the seeded workload generators (``graphs.py``).
"""
from ._lib import FapError, lib  # noqa: F401
from .engine import (  # noqa: F401
    DTYPE_F32,
    DTYPE_I32,
    MODE_BATCHED,
    MODE_PLAIN,
    Context,
    Engine,
    FapGraph,
    device_count,
    mtx_read,
    partition,
    preprocess,
)
