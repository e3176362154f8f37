"""ctypes binding of libmdsgpu (the C ABI declared in include/mdsgpu.h).

The library is loaded from ``mdsctk_gb300/lib/libmdsgpu.so`` (built in-tree by
``mdsctk_gb300/build.py``). There is no fallback: if the library is missing
or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmdsgpu.so")

MDS_OK = 0
MDS_ERR_ARG = -1
MDS_ERR_CUDA = -2
MDS_ERR_NOMEM = -3
MDS_ERR_UNSUPPORTED = -4
MDS_ERR_TIMEOUT = -5
MDS_ERR_INTERNAL = -6

MDS_NOFIT = 0x1
MDS_FULL = 0x2
MDS_DEVICE_IO = 0x4
MDS_CORRELATION = 0x8
MDS_PREC_FP32 = 0x00
MDS_PREC_BF16X3 = 0x10
MDS_PREC_FP16X3 = 0x20
MDS_NO_SKIP = 0x100
MDS_INJECT_SCREEN_STALL = 0x1

PRECISIONS = {"fp32": MDS_PREC_FP32, "bf16x3": MDS_PREC_BF16X3, "fp16x3": MDS_PREC_FP16X3}


class MdsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mdsgpu error {code}: {msg}")
        self.code = code


class KnnStats(ctypes.Structure):
    _fields_ = [("prep_ms", ctypes.c_double), ("screen_ms", ctypes.c_double),
                ("recheck_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("pairs", ctypes.c_longlong), ("kprime", ctypes.c_int),
                ("rows_flagged", ctypes.c_int), ("passes", ctypes.c_int),
                ("screen_launches", ctypes.c_int), ("launches", ctypes.c_int),
                ("screen_pairs", ctypes.c_longlong), ("recheck_pairs", ctypes.c_longlong),
                ("guard_violations", ctypes.c_int), ("screen_err_max", ctypes.c_float),
                ("guard_coef", ctypes.c_float), ("rows_audit_flagged", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("k", ctypes.c_int), ("sigma", ctypes.c_double),
                ("nev", ctypes.c_int), ("ncv", ctypes.c_int), ("tol", ctypes.c_double),
                ("maxiter", ctypes.c_int), ("flags", ctypes.c_uint), ("max_batch_frames", ctypes.c_int),
                ("slots", ctypes.c_int), ("hbm_budget", ctypes.c_size_t), ("use_graphs", ctypes.c_int)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("batch", ctypes.c_int),
                ("batch_frames", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int), ("slot_bytes", ctypes.c_longlong),
                ("requests_submitted", ctypes.c_longlong), ("requests_done", ctypes.c_longlong),
                ("batches", ctypes.c_longlong), ("frames", ctypes.c_longlong),
                ("graph_launches", ctypes.c_longlong), ("graphs_captured", ctypes.c_longlong),
                ("rows_flagged", ctypes.c_longlong), ("model_knn_ms", ctypes.c_double),
                ("model_decomp_ms", ctypes.c_double), ("model_nconv", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# Exported symbols and their signatures (kept in step with include/mdsgpu.h).
_vp, _i, _u, _sz, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint, ctypes.c_size_t, ctypes.c_double
_ip = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)
SIGNATURES = {
    "mds_version": ([], ctypes.c_char_p),
    "mds_create": ([_i, _sz, ctypes.POINTER(_vp)], _i),
    "mds_destroy": ([_vp], _i),
    "mds_last_error": ([_vp], ctypes.c_char_p),
    "mds_test_inject": ([_vp, _u], _i),
    "mds_get_knn_stats": ([_vp, ctypes.POINTER(KnnStats)], _i),
    "mds_knn_rms": ([_vp, _vp, _i, _vp, _i, _i, _vp, _i, _u, _vp, _vp, _ip], _i),
    "mds_knn_rms_screen": ([_vp, _vp, _i, _vp, _i, _i, _vp, _i, _u, _vp, _vp], _i),
    "mds_knn_rms_superpose": ([_vp, _vp, _i, _i, _vp, _u, _vp, _vp], _i),
    "mds_knn_data": ([_vp, _vp, _i, _vp, _i, _i, _i, _u, _vp, _vp, _ip], _i),
    "mds_knn_data_noalloc": ([_vp, _vp, _i, _vp, _i, _i, _i, _u, _vp, _vp, _ip], _i),
    "mds_knn_data_sparse": ([_vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _i, _u, _vp, _vp, _ip], _i),
    "mds_contact_profile": ([_vp, _vp, _i, _i, _vp, _i, _vp, _i, _d, _vp, _vp, ctypes.c_int64], _i),
    "mds_sysparse": ([_vp, _vp, _vp, _i, _i, _i, _u, _vp, _vp, _vp, ctypes.c_int64, _i64p], _i),
    "mds_gesparse": ([_vp, _vp, _vp, _i, _i, _i, _i, _u, _vp, _vp, _vp, ctypes.c_int64, _i64p], _i),
    "mds_decomp_sparse": ([_vp, _i, _vp, _vp, _vp, _d, _i, _i, _d, _i, _u, _vp, _vp, _vp, _ip], _i),
    "mds_server_create": ([ctypes.POINTER(ServerConfig), _vp, _i, _i, _vp, ctypes.POINTER(_vp)], _i),
    "mds_server_destroy": ([_vp], _i),
    "mds_server_last_error": ([_vp], ctypes.c_char_p),
    "mds_server_model": ([_vp, _vp, _vp], _i),
    "mds_server_submit": ([_vp, _vp, _i, _i64p], _i),
    "mds_server_wait": ([_vp, ctypes.c_int64, _i, _vp, _vp, _vp, ctypes.POINTER(RequestInfo)], _i),
    "mds_server_get_stats": ([_vp, ctypes.POINTER(ServerStats)], _i),
    "mds_server_hold": ([_vp, _i], _i),
    "mds_decomp_sparse_nystrom": ([_vp, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _d, _i, _i, _d, _i, _u, _vp, _vp,
                                   _vp, _vp, _ip], _i),
    "mds_xtc_index": ([_vp, _sz, _vp, _i, _ip, _ip], _i),
    "mds_xtc_decode": ([_vp, _vp, _sz, _vp, _i, _i, _u, _vp, _vp, _vp, _vp], _i),
    "mds_auto_decomp_sparse": ([_vp, _i, _vp, _vp, _vp, _i, _d, _i, _i, _d, _i, _u, _vp, _vp, _vp, _ip, _vp], _i),
    "mds_auto_decomp_sparse_nystrom": ([_vp, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _d, _i, _i, _d, _i, _u,
                                        _vp, _vp, _vp, _vp, _ip, _vp], _i),
}

_lib = None


def lib():
    """Load libmdsgpu (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libmdsgpu is not built ({LIB_PATH} missing); run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(ctx, code: int):
    if code != MDS_OK:
        msg = lib().mds_last_error(ctx)
        raise MdsError(code, msg.decode() if msg else "")
