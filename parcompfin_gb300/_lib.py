"""ctypes binding of libpcf.so (include/pcf.h).

The library is loaded from the package's own _lib/ directory, where
parcompfin_gb300.build puts it. There is no fallback: if the library is
missing or cannot be loaded, every call raises, so no pricing path can run
anywhere but through the CUDA engine.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

PCF_OK = 0
PCF_EINVAL = -1
PCF_ENOMEM = -2
PCF_ESINGULAR = -3
PCF_ETIMEOUT = -4
PCF_ECUDA = -5
PCF_ENODEV = -6
PCF_PENDING = 1


class PcfError(RuntimeError):
    """A libpcf call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class McResult(C.Structure):
    _fields_ = [
        ("price", C.c_double),
        ("std_error", C.c_double),
        ("price_plain", C.c_double),
        ("std_error_plain", C.c_double),
        ("price_cv", C.c_double),
        ("std_error_cv", C.c_double),
        ("cv_beta", C.c_double),
        ("cv_mean", C.c_double),
        ("discount", C.c_double),
        ("sums", C.c_double * 5),
        ("n_paths", C.c_longlong),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "sums"}
        d["sums"] = list(self.sums)
        return d


METHOD_EUR, METHOD_ASIA, METHOD_BASKET, METHOD_AMER = 0, 1, 2, 3
TUNE_MC, TUNE_LSM, TUNE_SAVE = 1, 2, 4


class McRequest(C.Structure):
    _fields_ = [
        ("method", C.c_int),
        ("payoff_fun", C.c_int),
        ("S0", C.c_double),
        ("E", C.c_double),
        ("r", C.c_double),
        ("sigma", C.c_double),
        ("T", C.c_double),
        ("N", C.c_longlong),
        ("M", C.c_int),
        ("mode", C.c_int),
        ("use_cv", C.c_int),
        ("assets", C.c_int),
        ("rho", C.c_double),
        ("basket_S0", C.POINTER(C.c_double)),
        ("basket_sigma", C.POINTER(C.c_double)),
        ("corr", C.POINTER(C.c_double)),
        ("scale_by_sqrt_T", C.c_int),
        ("seed", C.c_ulonglong),
        ("stream", C.c_uint),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("target_rel_se", C.c_double), ("pilot_paths", C.c_longlong),
                ("max_paths", C.c_longlong), ("max_amer_paths", C.c_longlong),
                ("max_batch", C.c_int), ("slots", C.c_int), ("hbm_fraction", C.c_double)]


class ServedResult(C.Structure):
    _fields_ = [("result", McResult), ("arrival_s", C.c_double), ("admit_s", C.c_double),
                ("done_s", C.c_double), ("paths", C.c_longlong), ("status", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int), ("batches", C.c_int), ("wall_s", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("max_ms", C.c_double), ("contracts_per_s", C.c_double),
                ("paths_per_s", C.c_double), ("paths", C.c_longlong),
                ("reserved_bytes", C.c_size_t)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BinomContract(C.Structure):
    _fields_ = [("S0", C.c_double), ("E", C.c_double), ("r", C.c_double),
                ("sigma", C.c_double), ("T", C.c_double), ("N", C.c_int),
                ("payoff_fun", C.c_int)]


_D = C.c_double
_LL = C.c_longlong
_ULL = C.c_ulonglong
_I = C.c_int
_P = C.c_void_p
_PD = C.POINTER(C.c_double)

# name -> (restype, argtypes). Mirrors include/pcf.h.
SIGNATURES = {
    "pcf_version": (C.c_char_p, []),
    "pcf_strerror": (C.c_char_p, [_I]),
    "pcf_last_error": (C.c_char_p, []),
    "pcf_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "pcf_ctx_destroy": (_I, [_P]),
    "pcf_ctx_stream": (_P, [_P]),
    "pcf_ctx_launch_count": (_LL, [_P]),
    "pcf_ctx_release": (_I, [_P]),
    "pcf_ctx_set_memory_limit": (_I, [_P, C.c_ulonglong]),
    "pcf_mc_eur": (_I, [_P, _D, _D, _D, _D, _D, _LL, _I, _ULL, _I, C.POINTER(McResult)]),
    "pcf_mc_asia": (_I, [_P, _D, _D, _D, _D, _D, _LL, _I, _I, _I, _ULL, _I,
                         C.POINTER(McResult)]),
    "pcf_mc_eur_multi": (_I, [_P, _D, _D, _D, _D, _D, _LL, _I, _I, _D, _ULL, _I,
                              C.POINTER(McResult)]),
    "pcf_mc_basket": (_I, [_P, _I, _PD, _PD, _PD, _D, _D, _D, _LL, _I, _I, _ULL, _I,
                           C.POINTER(McResult)]),
    "pcf_mc_amer": (_I, [_P, _D, _D, _D, _D, _D, _LL, _I, _I, _I, _ULL, _I,
                         C.POINTER(McResult)]),
    "pcf_mc_amer_audit": (_I, [_P, _D, _D, _D, _D, _D, _LL, _I, _I, _I, _ULL,
                               C.POINTER(McResult), C.POINTER(C.c_float), _PD,
                               C.POINTER(C.c_ushort), C.POINTER(C.c_float)]),
    "pcf_ctx_set_test_barrier": (_I, [_P, C.c_uint, C.c_uint]),
    "pcf_autotune": (_I, [_P, _I, C.c_char_p, _I]),
    "pcf_autotune_batch": (_I, [_P, _I, _I, C.POINTER(McRequest), C.c_char_p, _I]),
    "pcf_tune_report": (_I, [_P, C.c_char_p, _I]),
    "pcf_tune_reset": (_I, [_P]),
    "pcf_mc_eur_noalloc": (_I, [_D, _D, _D, _D, _D, _LL, _I, _ULL, _P, _P]),
    "pcf_binom_embar": (_I, [_P, _D, _D, _D, _D, _D, _I, _I, _I, _PD]),
    "pcf_binom_embar_batch": (_I, [_P, _I, C.POINTER(BinomContract), _I, _PD]),
    "pcf_binom_vanilla": (_I, [_P, _D, _D, _D, _D, _D, _I, _I, _I, _PD]),
    "pcf_plan_create": (_I, [_P, _I, C.POINTER(McRequest), C.POINTER(_P)]),
    "pcf_plan_launch": (_I, [_P]),
    "pcf_plan_set_graph": (_I, [_P, _I]),
    "pcf_plan_uses_graph": (_I, [_P]),
    "pcf_plan_results": (_I, [_P, C.POINTER(McResult)]),
    "pcf_plan_kernel_count": (_I, [_P]),
    "pcf_plan_destroy": (_I, [_P]),
    "pcf_price_batch": (_I, [_P, _I, C.POINTER(McRequest), C.POINTER(McResult)]),
    "pcf_server_start": (_I, [_P, C.POINTER(ServerConfig), C.POINTER(_P)]),
    "pcf_server_submit": (_I, [_P, C.POINTER(McRequest), C.POINTER(C.c_longlong)]),
    "pcf_server_poll": (_I, [_P, C.c_longlong, C.POINTER(ServedResult)]),
    "pcf_server_wait": (_I, [_P, C.c_longlong, _D, C.POINTER(ServedResult)]),
    "pcf_server_stop": (_I, [_P, C.POINTER(ServerStats)]),
    "pcf_serve_trace": (_I, [_P, C.POINTER(ServerConfig), _I, C.POINTER(McRequest), _PD,
                             C.POINTER(ServedResult), C.POINTER(ServerStats)]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libpcf.so (building it first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise PcfError(PCF_ENODEV, f"libpcf.so not found at {path}; run parcompfin_gb300.build")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int) -> None:
    if status == PCF_OK:
        return
    lib = load()
    msg = lib.pcf_last_error().decode() or lib.pcf_strerror(status).decode()
    if status == PCF_EINVAL:
        raise ValueError(msg)
    raise PcfError(status, msg)
