"""ctypes binding of libuvatrmm.so (the C ABI declared in include/uvatrmm.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when libuvatrmm.so has not been built (``uvatrmm_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libuvatrmm.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "uvatrmm.h")

_lib = None

i32, i64, u32, u64, dbl, vp = C.c_int, C.c_int64, C.c_uint32, C.c_uint64, C.c_double, C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "cblas_dtrmm": (None, [i32, i32, i32, i32, i32, i32, i32, dbl, vp, i32, vp, i32]),
    "uvatrmm_create": (i32, [C.POINTER(vp)]),
    "uvatrmm_destroy": (i32, [vp]),
    "uvatrmm_set_stream": (i32, [vp, vp]),
    "uvatrmm_set_option": (i32, [vp, i32, i32]),
    "uvatrmm_dtrmm": (i32, [vp, i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64]),
    "uvatrmm_dtrmm_async": (i32, [vp, i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64]),
    "uvatrmm_dtrmm_device": (i32, [vp, i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64]),
    "uvatrmm_dtrmm_device_oop": (i32, [vp, i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64, vp, i64]),
    "uvatrmm_sync": (i32, [vp]),
    "uvatrmm_dtrmm_device_noalloc": (i32, [i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64, vp]),
    "uvatrmm_ozaki_dtrmm_device": (i32, [vp, i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64, i32,
                                         C.POINTER(dbl), C.POINTER(i32)]),
    "uvatrmm_ozaki_dtrmm": (i32, [vp, i32, i32, i32, i32, i32, i64, i64, dbl, vp, i64, vp, i64, i32,
                                  C.POINTER(dbl), C.POINTER(i32)]),
    "uvatrmm_ozaki_plan": (i32, [i64, i32, C.POINTER(i32), C.POINTER(i32)]),
    "uvatrmm_stage_times": (i32, [vp, C.POINTER(dbl)]),
    "uvatrmm_map_rows": (i32, [i32, u64, u32, u32, C.POINTER(u64), C.POINTER(u64)]),
    "uvatrmm_product": (i32, [vp, i64, i32, i32, vp, vp, vp, C.POINTER(dbl)]),
    "uvatrmm_gen_consecutive": (i32, [vp, i64, i32, vp]),
    "uvatrmm_gen_uniform": (i32, [vp, u64, u64, i64, i64, vp, i64, i64, i32, dbl, i32]),
    "uvatrmm_inf_norm": (i32, [vp, i64, i64, vp, i64, C.POINTER(dbl)]),
    "uvatrmm_device_alloc": (i32, [C.c_size_t, C.POINTER(vp)]),
    "uvatrmm_device_free": (i32, [vp]),
    "uvatrmm_copy": (i32, [vp, vp, vp, C.c_size_t, i32]),
    "uvatrmm_host_alloc": (i32, [C.c_size_t, C.POINTER(vp)]),
    "uvatrmm_host_free": (i32, [vp]),
    "uvatrmm_last_error": (C.c_char_p, []),
    "uvatrmm_last_status": (i32, []),
    "uvatrmm_version": (C.c_char_p, []),
}


class TrmmProblem(C.Structure):
    """uvatrmm_trmm_problem (include/uvatrmm.h)."""
    _fields_ = [("layout", i32), ("side", i32), ("uplo", i32), ("transa", i32), ("diag", i32),
                ("m", i64), ("n", i64), ("alpha", dbl), ("A", vp), ("lda", i64), ("B", vp), ("ldb", i64),
                ("tier", i32), ("moduli", i32)]


class ServerConfig(C.Structure):
    """uvatrmm_server_config (include/uvatrmm.h)."""
    _fields_ = [("hbm_budget_bytes", i64), ("max_active", i32), ("tick_fp64_gflop", dbl),
                ("tick_ozaki_gflop", dbl)]


class ServerStats(C.Structure):
    """uvatrmm_server_stats (include/uvatrmm.h)."""
    _fields_ = [("submitted", i64), ("completed", i64), ("failed", i64), ("cancelled", i64), ("refused", i64),
                ("ticks", i64), ("p50_ms", dbl), ("p99_ms", dbl), ("mean_ms", dbl), ("max_ms", dbl),
                ("served_flops", dbl), ("first_submit_s", dbl), ("last_done_s", dbl), ("peak_bytes", i64)]


SIGNATURES.update({
    "uvatrmm_server_create": (i32, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
    "uvatrmm_server_submit": (i32, [vp, C.POINTER(TrmmProblem), i32, C.POINTER(i64)]),
    "uvatrmm_server_wait": (i32, [vp, i64, dbl]),
    "uvatrmm_server_cancel": (i32, [vp, i64]),
    "uvatrmm_server_get_stats": (i32, [vp, C.POINTER(ServerStats)]),
    "uvatrmm_server_latency": (i32, [vp, i64, C.POINTER(dbl)]),
    "uvatrmm_server_destroy": (i32, [vp]),
    "uvatrmm_group_create": (i32, [vp, C.POINTER(TrmmProblem), i32, C.POINTER(vp)]),
    "uvatrmm_group_run": (i32, [vp]),
    "uvatrmm_group_stats": (i32, [vp, C.POINTER(dbl), C.POINTER(i32), C.POINTER(i64), C.POINTER(i64),
                                  C.POINTER(i32), C.POINTER(i64)]),
    "uvatrmm_group_destroy": (i32, [vp]),
    "uvatrmm_tune": (i32, [vp, i32, i32, i64, i64, C.POINTER(i32)]),
    "cblas_dgemm": (None, [i32, i32, i32, i32, i32, i32, dbl, vp, i32, vp, i32, dbl, vp, i32]),
    "uvatrmm_dgemm": (i32, [vp, i32, i32, i32, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64]),
    "uvatrmm_dgemm_device": (i32, [vp, i32, i32, i32, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64]),
    "uvatrmm_stage": (i32, [vp, i64, i64, i64, i64, vp, i64, vp, i64, vp, i64]),
    "uvatrmm_write_result": (i32, [C.c_char_p, i32, i32, i32, i32, i32, i32, vp, i64]),
    "uvatrmm_read_result": (i32, [C.c_char_p, C.POINTER(i32), vp, i64]),
    "uvatrmm_numroc": (i64, [i64, i64, i32, i32, i32]),
    "uvatrmm_bc_gather": (i32, [vp, i64, i64, i64, i64, i32, i32, C.POINTER(vp), C.POINTER(i64), vp, i64]),
    "uvatrmm_bc_scatter": (i32, [vp, i64, i64, i64, i64, i32, i32, vp, i64, C.POINTER(vp), C.POINTER(i64)]),
})


class UvatrmmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"uvatrmm status {status}: {msg}")
        self.status = status


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"UVATRMM_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def lib() -> C.CDLL:
    """Load libuvatrmm.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m uvatrmm_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            if hasattr(L, name):
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise UvatrmmError(status, lib().uvatrmm_last_error().decode())
