"""Python host side of the engine: thin classes over the C ABI.

``Engine`` wraps one graph on one GPU (``fap_create``); ``Context`` wraps a
graph-less handle for the standalone kernels (``fap_minplus``,
``fap_floyd_batched``, ``fap_backward_dense``); ``FapGraph`` mirrors the
reference's ``fap::fapGraph`` interface (fap/fap.h:97-161) on top of an
``Engine`` with the same method names, argument meaning and error behaviour.

Buffers are numpy arrays (host memory) or torch tensors (host or CUDA); the
engine detects where they live.  Nothing here computes a distance in Python.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check, lib, ptr

DTYPE_F32 = _lib.DTYPE_F32
DTYPE_I32 = _lib.DTYPE_I32
MODE_PLAIN = _lib.MODE_PLAIN
MODE_BATCHED = _lib.MODE_BATCHED


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def device_count() -> int:
    c = C.c_int32(0)
    check(lib().fap_device_count(C.byref(c)), "fap_device_count")
    return int(c.value)


def mtx_read(path: str, directed: bool, weighted: bool):
    """CSR of a MatrixMarket file with the reference reader's semantics."""
    n = C.c_int32(0)
    m = C.c_int64(0)
    p = os.fsencode(path)
    check(lib().fap_mtx_counts(p, int(directed), int(weighted), C.byref(n), C.byref(m)), "fap_mtx_counts")
    adj = np.zeros(n.value, np.int32)
    ro = np.zeros(n.value + 1, np.int32)
    col = np.zeros(m.value, np.int32)
    w = np.zeros(m.value, np.float32)
    check(lib().fap_mtx_read(p, int(directed), int(weighted), n.value, m.value, ptr(adj), ptr(ro),
                             ptr(col), ptr(w)), "fap_mtx_read")
    mm = int(ro[-1])
    return ro, col[:mm].copy(), w[:mm].copy()


def partition(row_offset, col_val, K: int, seed: int = 1):
    """1-based part ids from the engine's multilevel partitioner, and the cut."""
    ro = _i32(row_offset)
    col = _i32(col_val)
    n = ro.shape[0] - 1
    gid = np.zeros(n, np.int32)
    cut = C.c_int64(0)
    check(lib().fap_partition(n, ptr(ro), ptr(col), int(K), int(seed), ptr(gid), C.byref(cut)),
          "fap_partition")
    return gid, int(cut.value)


def preprocess(K: int, graph_id, row_offset, col_val):
    """Boundary detection and vertex order (findBoundry + sort_and_encode)."""
    ro = _i32(row_offset)
    col = _i32(col_val)
    gid = _i32(graph_id)
    n = ro.shape[0] - 1
    st2ed = np.zeros(n, np.int32)
    ed2st = np.zeros(n, np.int32)
    arrs = [np.zeros(K + 1, np.int32) for _ in range(4)]
    check(lib().fap_preprocess(K, n, ptr(gid), ptr(ro), ptr(col), ptr(st2ed), ptr(ed2st),
                               *[ptr(a) for a in arrs]), "fap_preprocess")
    return dict(st2ed=st2ed, ed2st=ed2st, ver_num=arrs[0], ver_offset=arrs[1], bdy_num=arrs[2],
                bdy_offset=arrs[3])


class Engine:
    """One graph resident on one GPU (``fap_create``)."""

    def __init__(self, n, row_offset, col_val, weight, K, graph_id=None, dtype=DTYPE_F32, device=0):
        self._h = C.c_void_p()
        self._ro = _i32(row_offset)
        self._col = _i32(col_val)
        self._w = _f32(weight)
        self.n = int(n)
        self.m = int(self._col.shape[0])
        self.K = int(K)
        self.dtype = int(dtype)
        gid = None if graph_id is None else _i32(graph_id)
        check(lib().fap_create(self.n, self.m, ptr(self._ro), ptr(self._col), ptr(self._w), self.K,
                               ptr(gid), self.dtype, int(device), C.byref(self._h)), "fap_create")

    def close(self):
        if self._h:
            lib().fap_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def mapping(self):
        out = np.zeros(self.n, np.int32)
        check(lib().fap_mapping(self._h, ptr(out)), "fap_mapping")
        return out

    def graph_id(self):
        out = np.zeros(self.n, np.int32)
        check(lib().fap_graph_id(self._h, ptr(out)), "fap_graph_id")
        return out

    def part_info(self, part: int):
        sub, bdy, off = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().fap_part_info(self._h, int(part), C.byref(sub), C.byref(bdy), C.byref(off)),
              "fap_part_info")
        return int(sub.value), int(bdy.value), int(off.value)

    def solve(self, dist, pred=None, mode=MODE_BATCHED, stream=None):
        check(lib().fap_solve(self._h, ptr(dist), ptr(pred), int(mode), stream), "fap_solve")

    def solve_parts(self, parts, dist, pred=None, mode=MODE_BATCHED, stream=None):
        """Rows of the listed parts, one part after another (fap_solve_parts)."""
        pl = _i32(parts)
        check(lib().fap_solve_parts(self._h, ptr(pl), int(pl.shape[0]), ptr(dist), ptr(pred), int(mode), stream),
              "fap_solve_parts")

    def solve_part(self, part: int, dist, pred=None, stream=None):
        check(lib().fap_solve_part(self._h, int(part), ptr(dist), ptr(pred), stream), "fap_solve_part")

    def set_partition(self, graph_id):
        """New partition (n part ids, 1..K) for this graph; boundary and
        vertex order are recomputed, later solves use the new parts."""
        gid = np.ascontiguousarray(graph_id, dtype=np.int32)
        if gid.shape != (self.n,):
            raise ValueError("graph_id needs one part id per vertex")
        check(lib().fap_set_partition(self._h, ptr(gid)), "fap_set_partition")

    def precondition(self):
        check(lib().fap_precondition(self._h), "fap_precondition")

    def last_times(self):
        t = (C.c_double * 5)()
        check(lib().fap_last_times(self._h, t), "fap_last_times")
        return dict(zip(["sssp", "floyd", "min_plus", "data", "total"], list(t)))

    def last_launches(self) -> int:
        """Kernels the last solve launched."""
        v = C.c_int64(0)
        check(lib().fap_last_launches(self._h, C.byref(v)), "fap_last_launches")
        return int(v.value)

    def minplus_counters(self, reset: bool = True):
        """Strip min-plus work counters since the last reset: tiles, tiles with
        no active k-step, add-mins executed (active k-steps x tile outputs)."""
        v = (C.c_uint64 * 3)()
        check(lib().fap_minplus_counters(self._h, v, int(bool(reset))), "fap_minplus_counters")
        return dict(zip(["tiles", "empty_tiles", "executed_addmins"], list(v)))

    def query(self, dist, pred, src, dst, out_dist, out_len, out_path=None, max_len=0, stream=None):
        """Point-to-point distances and paths from device-resident solve()
        rows (fap_query); every argument is a device buffer."""
        n = int(src.numel()) if hasattr(src, "numel") else len(src)
        check(lib().fap_query(self._h, ptr(dist), ptr(pred), n, ptr(src), ptr(dst), ptr(out_dist),
                              ptr(out_len), ptr(out_path), int(max_len), stream), "fap_query")

    def fw_counters(self, reset: bool = True):
        """FW add-mins since the last reset: executed by the remaining-tile
        strips (device counter) and by the other FW launches (block count)."""
        v = (C.c_uint64 * 2)()
        check(lib().fap_fw_counters(self._h, v, int(bool(reset))), "fap_fw_counters")
        return dict(zip(["strip_addmins", "other_addmins"], list(v)))

    def sssp_stats(self):
        """Counters of the last solve's SSSP phase."""
        v = (C.c_uint64 * 5)()
        check(lib().fap_sssp_stats(self._h, v), "fap_sssp_stats")
        return dict(zip(["steps", "far_splits", "relaxed", "far_scanned", "batches"], list(v)))

    def set_option(self, option: int, value: float):
        check(lib().fap_set_option(self._h, int(option), float(value)), "fap_set_option")

    def get_option(self, option: int) -> float:
        v = C.c_double(0)
        check(lib().fap_get_option(self._h, int(option), C.byref(v)), "fap_get_option")
        return float(v.value)

    def sssp(self, sources, dist, pred=None, ld=None, stream=None):
        src = _i32(sources)
        check(lib().fap_sssp(self._h, ptr(src), int(src.shape[0]), ptr(dist), ptr(pred),
                             int(ld if ld is not None else self.n), stream), "fap_sssp")

    def backward(self, pred, s, t, g, dw, stream=None):
        check(lib().fap_backward(self._h, ptr(pred), int(s.shape[0]), ptr(s), ptr(t), ptr(g), ptr(dw),
                                 stream), "fap_backward")


class Context:
    """A handle without a graph, for the standalone batched kernels."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        check(lib().fap_create_context(int(device), C.byref(self._h)), "fap_create_context")

    def close(self):
        if self._h:
            lib().fap_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def minplus(self, dtype, A, B, C_out, Bp=None, Cp=None, M=None, N=None, K=None, lda=None,
                ldb=None, ldc=None, stream=None):
        """C_out = A (x) B (and Cp from Bp) on device tensors (2-D, row-major)."""
        M = A.shape[0] if M is None else M
        K = A.shape[1] if K is None else K
        N = B.shape[1] if N is None else N
        lda = A.stride(0) if lda is None else lda
        ldb = B.stride(0) if ldb is None else ldb
        ldc = C_out.stride(0) if ldc is None else ldc
        ldbp = Bp.stride(0) if Bp is not None else 0
        ldcp = Cp.stride(0) if Cp is not None else 0
        check(lib().fap_minplus(self._h, int(dtype), int(M), int(N), int(K), ptr(A), int(lda), ptr(B),
                                int(ldb), ptr(Bp), int(ldbp), ptr(C_out), int(ldc), ptr(Cp), int(ldcp),
                                stream), "fap_minplus")

    def floyd_batched(self, dtype, mats, preds=None, stream=None):
        """In-place FW of a list of square device tensors (optionally with preds)."""
        cnt = len(mats)
        sizes = np.array([m.shape[0] for m in mats], np.int32)
        lds = np.array([m.stride(0) for m in mats], np.int64)
        D = (C.c_void_p * cnt)(*[m.data_ptr() for m in mats])
        P = None
        if preds is not None:
            P = (C.c_void_p * cnt)(*[p.data_ptr() for p in preds])
        check(lib().fap_floyd_batched(self._h, int(dtype), cnt, ptr(sizes), D, ptr(lds), P, stream),
              "fap_floyd_batched")

    def addmin_peak(self, mode: int) -> float:
        """Add-min ops/s issued from registers (0: int32 DPX, 1: FP32,
        2: int32 with argmin, 3: FP32 with argmin)."""
        v = C.c_double(0)
        check(lib().fap_addmin_peak(self._h, int(mode), C.byref(v)), "fap_addmin_peak")
        return float(v.value)

    def backward_dense(self, preds, dWs, b, s, t, g, stream=None):
        cnt = len(preds)
        sizes = np.array([p.shape[0] for p in preds], np.int32)
        lds = np.array([p.stride(0) for p in preds], np.int64)
        P = (C.c_void_p * cnt)(*[p.data_ptr() for p in preds])
        W = (C.c_void_p * cnt)(*[w.data_ptr() for w in dWs])
        check(lib().fap_backward_dense(self._h, cnt, ptr(sizes), P, W, ptr(lds), int(b.shape[0]), ptr(b),
                                       ptr(s), ptr(t), ptr(g), stream), "fap_backward_dense")


class FapGraph:
    """Python mirror of ``fap::fapGraph`` (fap/fap.h:97-161) over the engine.

    Constructed from a CSR (the metadata constructor, fap/fap.h:102-104) or
    from a MatrixMarket file with :meth:`from_file`.  Results are numpy arrays
    in the reference's conventions: float32 distances with 1e8 for
    unreached, int32 predecessors with -1 for unreached; rows of part i are
    the part's vertices in mapping order, columns are vertex ids.
    """

    max_vertexs_num_limit = 20000

    def __init__(self, num_vertexs, num_edges, row_offset, col_val, weight, K, version=True,
                 graph_id=None, device=0):
        self.num_vertexs = int(num_vertexs)
        self.num_edges = int(num_edges)
        self.row_offset = _i32(row_offset)
        self.col_val = _i32(col_val)
        self.weight = _f32(weight)
        self.adj_size = np.diff(self.row_offset).astype(np.int32)
        self.K = int(K)
        self.version = bool(version)
        self.device = device
        if graph_id is None:
            graph_id, cut = partition(self.row_offset, self.col_val, self.K)
        else:
            cut = None
        self._graph_id = _i32(graph_id)
        self.edge_cut = cut
        w = self.weight
        integer = bool(np.all(w == np.floor(w))) and bool(np.all(w >= 0))
        wmax = float(w.max()) if w.size else 0.0
        self.int_mode = integer and wmax * max(self.num_vertexs - 1, 1) < (1 << 24)
        self._engine = None
        self.is_split = False
        self.current_subgraph_id = 0
        self.dist = None
        self.path = None
        self.subgraph_dist = None
        self.subgraph_path = None
        self._processed = set()
        self.times = dict(sssp=0.0, floyd=0.0, min_plus=0.0, data=0.0)

    @classmethod
    def from_file(cls, path, directed, weighted, K, **kw):
        ro, col, w = mtx_read(path, directed, weighted)
        return cls(ro.shape[0] - 1, col.shape[0], ro, col, w, K, **kw)

    # -- fap/fap.cpp:100-122
    def preCondition(self):
        pre = preprocess(self.K, self._graph_id, self.row_offset, self.col_val)
        self.st2ed = pre["st2ed"]
        self.ed2st = pre["ed2st"]
        self.C_BlockVer_num = pre["ver_num"]
        self.C_BlockVer_offset = pre["ver_offset"]
        self.C_BlockBdy_num = pre["bdy_num"]
        self.C_BlockBdy_offset = pre["bdy_offset"]
        self.is_split = self.num_vertexs > self.max_vertexs_num_limit

    def isSplit(self):
        return self.is_split

    def getGraphId(self):
        return self._graph_id.copy()

    def _eng(self):
        if self._engine is None:
            if not hasattr(self, "st2ed"):
                self.preCondition()
            self._engine = Engine(self.num_vertexs, self.row_offset, self.col_val, self.weight, self.K,
                                  graph_id=self._graph_id,
                                  dtype=DTYPE_I32 if self.int_mode else DTYPE_F32, device=self.device)
        return self._engine

    def _to_float(self, buf):
        if not self.int_mode:
            return buf
        iv = buf.view(np.int32)
        out = iv.astype(np.float32)
        out[iv >= _lib.INF_I32] = _lib.MAXVALUE_F32
        return out

    def _account(self):
        t = self._eng().last_times()
        for k in ("sssp", "floyd", "min_plus", "data"):
            self.times[k] += t[k] / 1e3

    # -- fap/fap.cpp:507-545
    def solve(self, is_path_needed=False):
        eng = self._eng()
        n = self.num_vertexs
        d = np.empty((n, n), np.float32)
        p = np.empty((n, n), np.int32)
        eng.solve(d, p, MODE_BATCHED if self.version else MODE_PLAIN)
        self.dist = self._to_float(d)
        self.path = p
        self._account()
        return 0

    def solveSubGraph(self, sub_graph_id, is_path_needed=False):
        if sub_graph_id in self._processed:
            print(f"Warning: Subgraph {sub_graph_id} has already been processed, skipping.")
            return 0
        eng = self._eng()
        sub = int(self.C_BlockVer_num[sub_graph_id])
        d = np.empty((sub, self.num_vertexs), np.float32)
        p = np.empty((sub, self.num_vertexs), np.int32)
        self.current_subgraph_id = sub_graph_id
        self._processed.add(sub_graph_id)
        eng.solve_part(sub_graph_id, d, p)
        self.subgraph_dist = self._to_float(d)
        self.subgraph_path = p
        self._account()
        return 0

    # -- getters, fap/fap.cpp:546-670
    def getMapping(self):
        return self.st2ed.copy()

    def getAllDistance(self):
        assert not self.is_split
        return self.dist

    def getAllPath(self):
        assert not self.is_split
        return self.path

    def getCurrentSubGraphId(self):
        return self.current_subgraph_id

    def getSubGraphIndex(self, sub_graph_id):
        off = int(self.C_BlockVer_offset[sub_graph_id])
        return self.st2ed[off: off + int(self.C_BlockVer_num[sub_graph_id])].copy()

    def getSubGraphDistance(self, sub_graph_id):
        assert self.current_subgraph_id == sub_graph_id
        return self.subgraph_dist

    def getSubGraphPath(self, sub_graph_id):
        assert self.current_subgraph_id == sub_graph_id
        return self.subgraph_path

    def _row_of(self, s):
        """(distance row, predecessor row) of vertex s from the last solve()
        or, after solveSubGraph, from the current part."""
        if self.dist is not None and not self.is_split:
            r = int(self.ed2st[s])
            return self.dist[r], self.path[r]
        off = int(self.C_BlockVer_offset[self.current_subgraph_id])
        r = int(self.ed2st[s]) - off
        if not 0 <= r < self.subgraph_dist.shape[0]:
            raise ValueError("vertex not in the current subgraph")
        return self.subgraph_dist[r], self.subgraph_path[r]

    def getDistanceP2P(self, source, target):
        """Distance from source to target (1e8 when unreached); declared by
        the reference without a body (fap/fap.cpp:674-680)."""
        if not (0 <= source < self.num_vertexs and 0 <= target < self.num_vertexs):
            raise IndexError("vertex id")
        return float(self._row_of(source)[0][target])

    def getPathP2P(self, source, target):
        """Vertices from source to target along the predecessors ([] when
        unreached)."""
        if not (0 <= source < self.num_vertexs and 0 <= target < self.num_vertexs):
            raise IndexError("vertex id")
        prow = self._row_of(source)[1]
        out, v = [], int(target)
        for _ in range(self.num_vertexs + 1):
            if v < 0:
                return []
            out.append(v)
            if v == source:
                return out[::-1]
            v = int(prow[v])
        return []

    def getTimeSSSP(self):
        return self.times["sssp"]

    def getTimeFloyd(self):
        return self.times["floyd"]

    def getTimeMinPlus(self):
        return self.times["min_plus"]

    def getTimeData(self):
        return self.times["data"]

    def getBoundaryNum(self):
        return int(self.C_BlockBdy_num.sum())

    def getInnerNum(self):
        return int((self.C_BlockVer_num - self.C_BlockBdy_num).sum())

    def getEdgeCut(self):
        return self.edge_cut

    def close(self):
        if self._engine is not None:
            self._engine.close()
            self._engine = None
