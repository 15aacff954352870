"""ctypes binding of ``libfastapsp.so`` (the C ABI declared in include/fastapsp.h).

The library is built in-tree by :mod:`fastapsp_gb300.build`.  Loading fails
loudly when it is missing: there is no Python or CPU fallback for any kernel.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfastapsp.so"

FAP_OK = 0
FAP_ERR_INVALID = -1
FAP_ERR_CUDA = -2
FAP_ERR_NOMEM = -3
FAP_ERR_STATE = -4
FAP_ERR_NOT_CONVERGED = -5
FAP_ERR_IO = -6
FAP_ERR_NO_DEVICE = -7
FAP_ERR_RANGE = -8

DTYPE_F32 = 0
DTYPE_I32 = 1
MODE_PLAIN = 0
MODE_BATCHED = 1
MAXVALUE_F32 = 1e8
OPT_SSSP_FP64 = 1
OPT_SSSP_DELTA = 2
OPT_AUTOTUNE = 3
OPT_SSSP_LANES = 4
OPT_TILE_COLS = 5
OPT_SSSP_METHOD = 6
OPT_HOST_RESULTS = 7
OPT_INT32_FORM = 8
OPT_HOST_GROUP_MB = 9
INF_I32 = 1 << 30

_i32 = C.c_int32
_i64 = C.c_int64
_p = C.c_void_p
_pi32 = C.POINTER(C.c_int32)
_pi64 = C.POINTER(C.c_int64)
_pf = C.POINTER(C.c_float)

# name -> (restype, argtypes); every function returns int status unless noted.
SIGNATURES = {
    "fap_version": (C.c_char_p, []),
    "fap_status_string": (C.c_char_p, [C.c_int]),
    "fap_last_error": (C.c_char_p, []),
    "fap_device_count": (C.c_int, [_pi32]),
    "fap_mtx_counts": (C.c_int, [C.c_char_p, _i32, _i32, _pi32, _pi64]),
    "fap_mtx_read": (C.c_int, [C.c_char_p, _i32, _i32, _i32, _i64, _p, _p, _p, _p]),
    "fap_partition": (C.c_int, [_i32, _p, _p, _i32, C.c_uint64, _p, _pi64]),
    "fap_preprocess": (C.c_int, [_i32, _i32, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "fap_create": (C.c_int, [_i32, _i64, _p, _p, _p, _i32, _p, _i32, _i32, C.POINTER(_p)]),
    "fap_create_context": (C.c_int, [_i32, C.POINTER(_p)]),
    "fap_destroy": (C.c_int, [_p]),
    "fap_num_vertices": (C.c_int, [_p, _pi32, _pi32]),
    "fap_mapping": (C.c_int, [_p, _p]),
    "fap_graph_id": (C.c_int, [_p, _p]),
    "fap_part_info": (C.c_int, [_p, _i32, _pi32, _pi32, _pi32]),
    "fap_solve_part": (C.c_int, [_p, _i32, _p, _p, _p]),
    "fap_solve": (C.c_int, [_p, _p, _p, _i32, _p]),
    "fap_solve_parts": (C.c_int, [_p, _p, _i32, _p, _p, _i32, _p]),
    "fap_solve_all": (C.c_int, [_p, _p, _p, _p]),
    "fap_solve_batched": (C.c_int, [_p, _p, _p, _p]),
    "fap_set_partition": (C.c_int, [_p, _p]),
    "fap_precondition": (C.c_int, [_p]),
    "fap_last_times": (C.c_int, [_p, C.POINTER(C.c_double)]),
    "fap_last_launches": (C.c_int, [_p, C.POINTER(C.c_int64)]),
    "fap_minplus_counters": (C.c_int, [_p, C.POINTER(C.c_uint64), _i32]),
    "fap_fw_counters": (C.c_int, [_p, C.POINTER(C.c_uint64), _i32]),
    "fap_query": (C.c_int, [_p, _p, _p, _i32, _p, _p, _p, _p, _p, _i32, _p]),
    "fap_minplus": (C.c_int, [_p, _i32, _i32, _i32, _i32, _p, _i64, _p, _i64, _p, _i64, _p, _i64,
                              _p, _i64, _p]),
    "fap_floyd_batched": (C.c_int, [_p, _i32, _i32, _p, _p, _p, _p, _p]),
    "fap_fw_batched": (C.c_int, [_p, _i32, _i32, _p, _p, _p, _p, _p]),
    "fap_sssp": (C.c_int, [_p, _p, _i32, _p, _p, _i64, _p]),
    "fap_backward": (C.c_int, [_p, _p, _i32, _p, _p, _p, _p, _p]),
    "fap_backward_dense": (C.c_int, [_p, _i32, _p, _p, _p, _p, _i32, _p, _p, _p, _p, _p]),
    "fap_addmin_peak": (C.c_int, [_p, _i32, C.POINTER(C.c_double)]),
    "fap_set_option": (C.c_int, [_p, _i32, C.c_double]),
    "fap_sssp_stats": (C.c_int, [_p, C.POINTER(C.c_uint64)]),
    "fap_get_option": (C.c_int, [_p, _i32, C.POINTER(C.c_double)]),
    "fap_sssp_noalloc": (C.c_int, [_i32, _i32, _i64, _p, _p, _p, _p, _p, _p, _p, _i32, _p, _p, _i64,
                                   _p]),
}

_lib = None


class FapError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {message} (status {status})")
        self.status = status


def lib() -> C.CDLL:
    """The loaded library (built on first use if the sources are present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FapError(FAP_ERR_STATE, "load",
                       f"{LIB_PATH} is missing; run `python -m fastapsp_gb300.build` first")
    handle = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return _lib


def check(status: int, where: str) -> None:
    if status != FAP_OK:
        L = lib()
        msg = L.fap_last_error().decode() or L.fap_status_string(status).decode()
        raise FapError(status, where, msg)


def ptr(x) -> int | None:
    """Raw address of a numpy array or torch tensor (None passes NULL)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    if isinstance(x, int):
        return x
    raise TypeError(f"cannot take the address of {type(x)}")
