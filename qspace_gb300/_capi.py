"""ctypes binding of libqsgpu.so (the C-ABI of include/qsgpu.h).

The library is built in-tree (``qspace_gb300/_build.py``).  There is no CPU
fallback: if the shared library is missing or a CUDA device is absent, calls
fail loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

from . import _build

c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)
c_double_p = C.POINTER(C.c_double)


class QSpaceView(C.Structure):
    _fields_ = [("rank", C.c_int32), ("qdim", C.c_int32), ("nblk", C.c_int64),
                ("q", c_int32_p), ("dims", c_int64_p), ("offs", c_int64_p),
                ("data", c_double_p), ("is_complex", C.c_int32), ("itags", C.c_char_p)]


class Opts(C.Structure):
    _fields_ = [("prec", C.c_int32), ("nslices", C.c_int32), ("tol", C.c_double),
                ("flags", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("flops", C.c_double), ("bytes", C.c_double), ("device_ms", C.c_double),
                ("npairs", C.c_int64), ("nblk_out", C.c_int64), ("nslices", C.c_int32),
                ("digit_bits", C.c_int32), ("err_bound", C.c_double), ("launches", C.c_int32),
                ("pad_", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


class PairList(C.Structure):
    _fields_ = [("npairs", C.c_int64), ("M", c_int32_p), ("N", c_int32_p), ("K", c_int32_p),
                ("a_off", c_int64_p), ("b_off", c_int64_p), ("c_off", c_int64_p),
                ("lda", c_int32_p), ("ldb", c_int32_p), ("ldc", c_int32_p),
                ("trans", c_int32_p), ("afac", c_double_p), ("c_blk", c_int32_p),
                ("is_complex", C.c_int32)]


class ServerCfg(C.Structure):
    _fields_ = [("nslots", C.c_int32), ("max_batch", C.c_int32), ("hbm_budget", C.c_int64)]


QS_PREC_FP64 = 0
QS_PREC_SPLIT = 1
QS_FLAG_NO_GRAPH = 1
QS_FLAG_AUTOTUNE = 4

STATUS = {0: "QS_OK", 1: "QS_ERR_ARG", 2: "QS_ERR_SHAPE", 3: "QS_ERR_LABEL", 4: "QS_ERR_CUDA",
          5: "QS_ERR_OOM", 6: "QS_ERR_TIMEOUT", 7: "QS_ERR_UNSUPPORTED", 8: "QS_ERR_INTERNAL",
          9: "QS_ERR_CANCELLED", 10: "QS_ERR_NUMERIC"}


class QSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


# Every symbol declared in include/qsgpu.h with (restype, argtypes).
_V = None
SIGNATURES = {
    "qs_last_error": (C.c_char_p, []),
    "qs_version": (C.c_char_p, []),
    "qs_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "qs_ctx_destroy": (_V, [C.c_void_p]),
    "qs_ctx_stream": (C.c_void_p, [C.c_void_p]),
    "qs_ctx_sync": (C.c_int, [C.c_void_p]),
    "qs_ctx_launches": (C.c_int64, [C.c_void_p]),
    "qs_ctx_set_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "qs_ctx_phase_ms": (C.c_int, [C.c_void_p, c_double_p, c_double_p]),
    "qs_contractQS": (C.c_int, [C.c_void_p, C.POINTER(QSpaceView), C.c_char_p, C.POINTER(QSpaceView),
                                C.c_char_p, c_int32_p, C.c_int32, C.POINTER(Opts),
                                C.POINTER(C.c_void_p), C.POINTER(Stats)]),
    "qs_result_info": (C.c_int, [C.c_void_p, c_int32_p, c_int32_p, c_int64_p, c_int64_p, c_int32_p]),
    "qs_result_copy": (C.c_int, [C.c_void_p, c_int32_p, c_int64_p, c_int64_p, c_double_p]),
    "qs_result_free": (_V, [C.c_void_p]),
    "qs_result_itags": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "qs_tensor_itags": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "qs_tensor_upload": (C.c_int, [C.c_void_p, C.POINTER(QSpaceView), C.POINTER(C.c_void_p)]),
    "qs_tensor_info": (C.c_int, [C.c_void_p, c_int32_p, c_int32_p, c_int64_p, c_int64_p, c_int32_p]),
    "qs_tensor_download": (C.c_int, [C.c_void_p, C.c_void_p, c_int32_p, c_int64_p, c_int64_p,
                                     c_double_p]),
    "qs_tensor_data": (C.c_void_p, [C.c_void_p]),
    "qs_tensor_free": (_V, [C.c_void_p]),
    "qs_tensor_meta": (C.c_int, [C.c_void_p, c_int32_p, c_int64_p, c_int64_p]),
    "qs_svd_keep": (C.c_int, [C.c_int64, c_int64_p, c_double_p, C.c_int64, C.c_int64, C.c_double,
                              C.POINTER(C.c_uint8), C.POINTER(C.c_int64), C.POINTER(C.c_double),
                              C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "qs_plus_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.POINTER(C.c_void_p)]),
    "qs_eigQS_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.POINTER(C.c_void_p),
                               C.POINTER(C.c_void_p), c_double_p, C.POINTER(C.c_uint8), C.POINTER(C.c_int64),
                               C.POINTER(C.c_double)]),
    "qs_wire_size": (C.c_int, [C.POINTER(QSpaceView), C.POINTER(C.c_int64)]),
    "qs_wire_pack": (C.c_int, [C.POINTER(QSpaceView), C.c_void_p, C.c_int64]),
    "qs_wire_view": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(QSpaceView)]),
    "qs_tensor_from_wire": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    "qs_tensor_wire_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "qs_tensor_to_wire": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]),
    "qs_contract_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_char_p, C.c_void_p, C.c_char_p,
                                  c_int32_p, C.c_int32, C.POINTER(Opts), C.POINTER(C.c_void_p),
                                  C.POINTER(Stats)]),
    "qs_permuteQS": (C.c_int, [C.c_void_p, C.POINTER(QSpaceView), c_int32_p, C.c_int32, C.c_int32,
                               C.POINTER(C.c_void_p)]),
    "qs_permute_dev": (C.c_int, [C.c_void_p, C.c_void_p, c_int32_p, C.c_int32, C.c_int32,
                                 C.POINTER(C.c_void_p)]),
    "qs_contract_batch": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_char_p),
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_char_p), C.POINTER(c_int32_p), c_int32_p,
                                    C.POINTER(Opts), C.POINTER(C.c_void_p)]),
    "qs_contract_itags": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), c_int32_p, c_int32_p,
                                    C.c_int32, C.POINTER(Opts), C.POINTER(C.c_void_p)]),
    "qs_grouped_gemm": (C.c_int, [C.c_void_p, C.POINTER(PairList), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.POINTER(Opts), C.POINTER(Stats)]),
    "qs_grouped_plan_create": (C.c_int, [C.c_void_p, C.POINTER(PairList), C.POINTER(Opts),
                                         C.POINTER(C.c_void_p)]),
    "qs_grouped_plan_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Stats)]),
    "qs_grouped_plan_destroy": (None, [C.c_void_p]),
    "qs_grouped_gemm_split_static": (C.c_int, [C.c_void_p, C.POINTER(PairList), C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.POINTER(Opts), C.POINTER(Stats)]),
    "qs_xcache_create": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    "qs_xcache_destroy": (None, [C.c_void_p]),
    "qs_xcache_put": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "qs_xcache_get": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "qs_xcache_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "qs_grouped_gemm_keyed": (C.c_int, [C.c_void_p, C.POINTER(PairList), C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.POINTER(Opts), C.POINTER(Stats)]),
    "qs_grouped_gemm_host": (C.c_int, [C.c_void_p, C.POINTER(PairList), c_double_p, C.c_int64,
                                       c_double_p, C.c_int64, c_double_p, C.c_int64,
                                       C.POINTER(Opts), C.POINTER(Stats)]),
    "qs_eig_blocks": (C.c_int, [C.c_void_p, C.c_int64, c_int64_p, c_int64_p, c_int64_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_int32]),
    "qs_mark_keep": (C.c_int, [C.c_int64, c_int64_p, c_double_p, c_double_p, C.c_int64, C.c_double,
                               C.c_double, C.POINTER(C.c_uint8), c_int64_p, c_double_p]),
    "qs_average_levels": (C.c_int, [C.c_int64, c_int64_p, c_double_p, C.c_double, c_double_p]),
    "qs_mark_keep_dev": (C.c_int, [C.c_void_p, C.c_int64, c_int64_p, C.c_void_p, C.c_int64, C.c_double,
                                   C.c_double, C.c_void_p, c_int64_p, c_double_p]),
    "qs_svd_blocks": (C.c_int, [C.c_void_p, C.c_int64, c_int64_p, c_int64_p, c_int64_p, c_int64_p,
                                c_int64_p, c_int64_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p]),
    "qs_svd_blocks_ex": (C.c_int, [C.c_void_p, C.c_int64, c_int64_p, c_int64_p, c_int64_p, c_int64_p,
                                   c_int64_p, c_int64_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_int32, C.c_double]),
    "qs_gs_reortho": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                c_double_p]),
    "qs_server_create": (C.c_int, [C.c_void_p, C.POINTER(ServerCfg), C.POINTER(C.c_void_p)]),
    "qs_server_destroy": (_V, [C.c_void_p]),
    "qs_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_char_p, C.c_void_p, C.c_char_p,
                                   c_int32_p, C.c_int32, C.POINTER(Opts), c_int64_p]),
    "qs_server_poll": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, c_int32_p,
                                 C.POINTER(C.c_void_p), c_double_p]),
    "qs_server_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "qs_server_submit_eig": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double,
                                       c_int64_p]),
    "qs_server_submit_eig_from": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_double,
                                            C.c_double, c_int64_p]),
    "qs_server_submit_from": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_void_p,
                                        C.c_char_p, c_int32_p, C.c_int32, C.POINTER(Opts), c_int64_p]),
    "qs_server_poll_eig": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), c_double_p,
                                     C.POINTER(C.c_uint8), c_int64_p, c_double_p, c_double_p]),
}

_lib = None
_lock = threading.Lock()


def lib_file() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libqsgpu.so (building it in-tree first when absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_file()
        if not path.exists():
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run qspace_gb300._build.build()")
            _build.build()
        lib = C.CDLL(str(path), mode=os.RTLD_NOW | C.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(code: int) -> None:
    if code != 0:
        msg = load().qs_last_error()
        raise QSError(code, msg.decode() if msg else "")
