"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the engine.  See fap_oracle.h for what
each function restates from the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_BIN = HERE / "_ref" / "fap_ref"
MAXVALUE = np.float32(1e8)

_lib = None


def build(ref: bool = False) -> None:
    """Builds liboracle.so (and the reference binary if `ref` and its
    sources are present)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    if ref and Path(os.environ.get("FAP_REFERENCE_DIR", "/root/reference")).exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref",
                        "REF=" + os.environ.get("FAP_REFERENCE_DIR", "/root/reference")], check=True)


class _times(C.Structure):
    _fields_ = [("sssp", C.c_double), ("floyd", C.c_double), ("min_plus", C.c_double),
                ("data", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        _lib.oracle_run_part.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 12 + [
            C.c_int32, C.POINTER(_times)]
        _lib.oracle_dijkstra_path.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 6
        _lib.oracle_dijkstra_f64.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 4
        _lib.oracle_floyd_path.argtypes = [C.c_int32, C.c_void_p, C.c_void_p]
        _lib.oracle_min_plus_path_advanced.argtypes = [C.c_void_p] * 5 + [C.c_int32] * 3
        _lib.oracle_preprocess.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 11
        _lib.oracle_mtx_counts.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_int32),
                                           C.POINTER(C.c_int64)]
        _lib.oracle_mtx_read.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int32, C.c_int64] + [
            C.c_void_p] * 4
        _lib.oracle_set_threads.argtypes = [C.c_int32]
        _lib.oracle_get_threads.restype = C.c_int32
    return _lib


def _p(a):
    return a.ctypes.data


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def mtx_read(path, directed, weighted):
    n = C.c_int32()
    m = C.c_int64()
    if lib().oracle_mtx_counts(os.fsencode(str(path)), int(directed), int(weighted), C.byref(n),
                               C.byref(m)) != 0:
        raise IOError(path)
    adj = np.zeros(n.value, np.int32)
    ro = np.zeros(n.value + 1, np.int32)
    col = np.zeros(m.value, np.int32)
    w = np.zeros(m.value, np.float32)
    lib().oracle_mtx_read(os.fsencode(str(path)), int(directed), int(weighted), n.value, m.value,
                          _p(adj), _p(ro), _p(col), _p(w))
    mm = int(ro[-1])
    return ro, col[:mm].copy(), w[:mm].copy()


def dijkstra_path(u, ro, col, w):
    ro, col = _i32(ro), _i32(col)
    w = np.ascontiguousarray(w, np.float32)
    n = ro.shape[0] - 1
    adj = np.diff(ro).astype(np.int32)
    d = np.empty(n, np.float32)
    p = np.empty(n, np.int32)
    lib().oracle_dijkstra_path(int(u), n, _p(adj), _p(ro), _p(col), _p(w), _p(d), _p(p))
    return d, p


def dijkstra_f64(u, ro, col, w):
    ro, col = _i32(ro), _i32(col)
    w = np.ascontiguousarray(w, np.float64)
    n = ro.shape[0] - 1
    d = np.empty(n, np.float64)
    lib().oracle_dijkstra_f64(int(u), n, _p(ro), _p(col), _p(w), _p(d))
    return d


def floyd_path(mat, path):
    mat = np.ascontiguousarray(mat, np.float32).copy()
    path = np.ascontiguousarray(path, np.int32).copy()
    lib().oracle_floyd_path(mat.shape[0], _p(mat), _p(path))
    return mat, path


def min_plus(mat1, mat2, mat2_path):
    mat1 = np.ascontiguousarray(mat1, np.float32)
    mat2 = np.ascontiguousarray(mat2, np.float32)
    mat2_path = np.ascontiguousarray(mat2_path, np.int32)
    M, K = mat1.shape
    N = mat2.shape[1]
    res = np.empty((M, N), np.float32)
    path = np.empty((M, N), np.int32)
    lib().oracle_min_plus_path_advanced(_p(mat1), _p(mat2), _p(mat2_path), _p(res), _p(path), M, N, K)
    return res, path


def preprocess(K, graph_id, ro, col):
    ro, col, gid = _i32(ro), _i32(col), _i32(graph_id)
    n = ro.shape[0] - 1
    adj = np.diff(ro).astype(np.int32)
    st2ed = np.empty(n, np.int32)
    ed2st = np.empty(n, np.int32)
    arr = [np.zeros(K + 1, np.int32) for _ in range(4)]
    isb = np.empty(n, np.int32)
    lib().oracle_preprocess(K, n, _p(gid), _p(adj), _p(ro), _p(col), _p(st2ed), _p(ed2st),
                            *[_p(a) for a in arr], _p(isb))
    return dict(st2ed=st2ed, ed2st=ed2st, ver_num=arr[0], ver_offset=arr[1], bdy_num=arr[2],
                bdy_offset=arr[3], is_boundary=isb)


def set_threads(t):
    lib().oracle_set_threads(int(t))


def get_threads():
    return int(lib().oracle_get_threads())


def run_part(part, ro, col, w, graph_id, pre, mp_rows=-1, out=None):
    """fapGraph::run (CPU branch) for one part: (dist, path, phase times)."""
    ro, col, gid = _i32(ro), _i32(col), _i32(graph_id)
    w = np.ascontiguousarray(w, np.float32)
    n = ro.shape[0] - 1
    adj = np.diff(ro).astype(np.int32)
    sub = int(pre["ver_num"][part])
    if out is None:
        d = np.zeros((sub, n), np.float32)
        p = np.zeros((sub, n), np.int32)
    else:
        d, p = out
    # written through before the timed call, as the reference's rows are
    # (std::vector::resize zero-fills them before fapGraph::run,
    # fap/fap.cpp:532-534): the phase times then hold no first-touch faults
    d.fill(0)
    p.fill(0)
    t = _times()
    lib().oracle_run_part(int(part), n, _p(adj), _p(ro), _p(col), _p(w), _p(gid), _p(pre["st2ed"]),
                          _p(pre["ed2st"]), _p(pre["ver_num"]), _p(pre["ver_offset"]),
                          _p(pre["bdy_num"]), _p(d), _p(p), int(mp_rows), C.byref(t))
    return d, p, dict(sssp=t.sssp, floyd=t.floyd, min_plus=t.min_plus, data=t.data)


def solve(K, ro, col, w, graph_id):
    """fapGraph::solve (CPU branch): full n x n dist/path in solve() layout."""
    pre = preprocess(K, graph_id, ro, col)
    n = len(ro) - 1
    D = np.zeros((n, n), np.float32)
    P = np.zeros((n, n), np.int32)
    for part in range(1, K + 1):
        off = int(pre["ver_offset"][part])
        sub = int(pre["ver_num"][part])
        if sub == 0:
            continue
        run_part(part, ro, col, w, graph_id, pre, out=(D[off:off + sub], P[off:off + sub]))
    return D, P, pre


def run_reference(workdir, name, directed, weighted, K, partition_file, outdir, parts=None):
    """Runs the reference's own fapGraph (oracle/_ref/fap_ref) on
    workdir/graph/<type>/<name>.mtx; returns the output directory."""
    if not REF_BIN.exists():
        raise FileNotFoundError(REF_BIN)
    env = dict(os.environ, FAP_REF_PARTITION=str(partition_file))
    cmd = [str(REF_BIN), str(workdir), name, str(int(directed)), str(int(weighted)), str(K),
           str(outdir)] + ([str(p) for p in parts] if parts else [])
    subprocess.run(cmd, check=True, env=env, stdout=subprocess.DEVNULL)
    return Path(outdir)
