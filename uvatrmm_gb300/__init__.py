"""uvatrmm_gb300: FP64 triangular matrix multiply (TRMM) on one NVIDIA GB300.

The product is the C ABI of ``libuvatrmm.so`` (``include/uvatrmm.h``) and the
``uvatrmm.x`` command line built on it.  This package only builds them and
binds the ABI for Python callers (tests and the benchmark): every call goes
through the CUDA library, and nothing here computes a result on the CPU.
"""
from __future__ import annotations

import ctypes as C

from ._lib import UvatrmmError, check, header_symbols, lib  # noqa: F401

# CBLAS enumerations (same values as cblas.h).
ROW, COL = 101, 102
NOTRANS, TRANS, CONJTRANS = 111, 112, 113
UPPER, LOWER = 121, 122
NONUNIT, UNIT = 131, 132
LEFT, RIGHT = 141, 142

OPT_ENGINE, OPT_SCHEDULE, OPT_SHAPE, OPT_TILE = 1, 2, 3, 4
ENGINE_DFMA, ENGINE_DMMA = 0, 1
SCHED_DYNAMIC, SCHED_REG, SCHED_BALANCED = 0, 1, 2
SHAPE_TRAPEZOID, SHAPE_BOXES = 0, 1

OK, EINVAL, ENOMEM, EDEVICE, ETIMEOUT, EUNSUPPORTED, EBUSY, ENOTREADY = 0, -1, -2, -3, -4, -5, -6, -7


def _ptr(x) -> int:
    """Address of a numpy array or torch tensor."""
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


class Handle:
    """Owns a uvatrmm handle on the current CUDA device."""

    def __init__(self, stream=None, **options):
        h = C.c_void_p()
        check(lib().uvatrmm_create(C.byref(h)))
        self.h = h
        if stream is not None:
            self.set_stream(stream)
        for k, v in options.items():
            self.set_option(k, v)

    def close(self) -> None:
        if self.h:
            lib().uvatrmm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream) -> None:
        s = getattr(stream, "cuda_stream", stream)
        check(lib().uvatrmm_set_stream(self.h, C.c_void_p(int(s) if s else 0)))

    def set_option(self, name: str, value: int) -> None:
        key = {"engine": OPT_ENGINE, "schedule": OPT_SCHEDULE, "shape": OPT_SHAPE, "tile": OPT_TILE,
               "ozaki_scratch_mb": 5, "stage_timing": 6, "autotune": 7, "ozaki_raster": 8,
               "host_stage_kb": 9, "wait_expiry_test": 10, "ozaki_err_host": 11}[name]
        check(lib().uvatrmm_set_option(self.h, key, int(value)))

    def stage_times(self):
        """(scaling, slicing, GEMMs, reassembly) GPU ms of the last Ozaki call."""
        buf = (C.c_double * 4)()
        check(lib().uvatrmm_stage_times(self.h, buf))
        return tuple(buf)

    # -- TRMM ------------------------------------------------------------
    def dtrmm(self, layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb) -> None:
        """Host buffers (numpy float64), in place on B."""
        check(lib().uvatrmm_dtrmm(self.h, layout, side, uplo, transa, diag, m, n, alpha,
                                  _ptr(A), lda, _ptr(B), ldb))

    def dtrmm_async(self, layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb) -> None:
        """Host buffers from host_empty(), in place on B; enqueued on the
        handle's stream, complete after sync()."""
        check(lib().uvatrmm_dtrmm_async(self.h, layout, side, uplo, transa, diag, m, n, alpha,
                                        _ptr(A), lda, _ptr(B), ldb))

    def dtrmm_device(self, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb) -> None:
        """Device buffers (torch float64 CUDA tensors), in place on dB."""
        check(lib().uvatrmm_dtrmm_device(self.h, layout, side, uplo, transa, diag, m, n, alpha,
                                         _ptr(dA), lda, _ptr(dB), ldb))

    def dtrmm_device_oop(self, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, dC, ldc) -> None:
        check(lib().uvatrmm_dtrmm_device_oop(self.h, layout, side, uplo, transa, diag, m, n, alpha,
                                             _ptr(dA), lda, _ptr(dB), ldb, _ptr(dC), ldc))

    def sync(self) -> None:
        check(lib().uvatrmm_sync(self.h))

    # -- GEMM, the product loop's stage, block-cyclic layouts -------------------
    def dgemm(self, layout, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C_, ldc) -> None:
        """Host buffers (numpy float64): C := alpha*op(A)*op(B) + beta*C."""
        check(lib().uvatrmm_dgemm(self.h, layout, transa, transb, m, n, k, alpha, _ptr(A), lda, _ptr(B), ldb,
                                  beta, _ptr(C_), ldc))

    def dgemm_device(self, layout, transa, transb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc) -> None:
        check(lib().uvatrmm_dgemm_device(self.h, layout, transa, transb, m, n, k, alpha, _ptr(dA), lda,
                                         _ptr(dB), ldb, beta, _ptr(dC), ldc))

    def stage(self, n, w, b, h, dAblk, lda, dB, ldb, dC, ldc) -> None:
        """One step of the row-block product loop (row-major device buffers)."""
        check(lib().uvatrmm_stage(self.h, n, w, b, h, _ptr(dAblk), lda, _ptr(dB), ldb, _ptr(dC), ldc))

    def bc_gather(self, m, n, mb, nb, nprow, npcol, locals_, llds, dglobal, ldg) -> None:
        """Block-cyclic local blocks (device, column-major, process (p,q) at p*npcol+q) -> global."""
        ptrs = (C.c_void_p * len(locals_))(*[_ptr(x) for x in locals_])
        ld = (C.c_int64 * len(llds))(*llds)
        check(lib().uvatrmm_bc_gather(self.h, m, n, mb, nb, nprow, npcol, ptrs, ld, _ptr(dglobal), ldg))

    def bc_scatter(self, m, n, mb, nb, nprow, npcol, dglobal, ldg, locals_, llds) -> None:
        ptrs = (C.c_void_p * len(locals_))(*[_ptr(x) for x in locals_])
        ld = (C.c_int64 * len(llds))(*llds)
        check(lib().uvatrmm_bc_scatter(self.h, m, n, mb, nb, nprow, npcol, _ptr(dglobal), ldg, ptrs, ld))

    # -- Ozaki (emulated FP64) --------------------------------------------------
    def ozaki_device(self, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, moduli=0,
                     want_err=False):
        """Device buffers, in place on dB.  Returns (relerr or None, bits)."""
        err, bits = C.c_double(), C.c_int()
        check(lib().uvatrmm_ozaki_dtrmm_device(self.h, layout, side, uplo, transa, diag, m, n, alpha,
                                               _ptr(dA), lda, _ptr(dB), ldb, moduli,
                                               C.byref(err) if want_err else None, C.byref(bits)))
        return (err.value if want_err else None), bits.value

    def ozaki(self, layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, moduli=0, want_err=False):
        """Host buffers, in place on B.  Returns (relerr or None, bits)."""
        err, bits = C.c_double(), C.c_int()
        check(lib().uvatrmm_ozaki_dtrmm(self.h, layout, side, uplo, transa, diag, m, n, alpha,
                                        _ptr(A), lda, _ptr(B), ldb, moduli,
                                        C.byref(err) if want_err else None, C.byref(bits)))
        return (err.value if want_err else None), bits.value

    def product(self, n, schedule, shape, dA, dB, dC) -> float:
        secs = C.c_double()
        check(lib().uvatrmm_product(self.h, n, schedule, shape, _ptr(dA), _ptr(dB), _ptr(dC), C.byref(secs)))
        return secs.value

    # -- generators and norms -------------------------------------------------
    def gen_consecutive(self, n, triangular, d) -> None:
        check(lib().uvatrmm_gen_consecutive(self.h, n, int(triangular), _ptr(d)))

    def gen_uniform(self, seed, stream, rows, cols, d, rs, cs, tri=None, fill=0.0, spread=0) -> None:
        t = 0 if tri is None else ord(tri)
        check(lib().uvatrmm_gen_uniform(self.h, seed, stream, rows, cols, _ptr(d), rs, cs, t, fill, spread))

    def inf_norm(self, rows, cols, dC, ldc) -> float:
        v = C.c_double()
        check(lib().uvatrmm_inf_norm(self.h, rows, cols, _ptr(dC), ldc, C.byref(v)))
        return v.value


TIER_FP64, TIER_OZAKI = 0, 1


class Group:
    """A grouped batch of device TRMMs captured in a CUDA graph.

    `problems` is a list of dicts with keys layout, side, uplo, transa, diag,
    m, n, alpha, A (tensor), lda, B (tensor), ldb, tier, moduli."""

    def __init__(self, handle: "Handle", problems):
        from ._lib import TrmmProblem
        arr = (TrmmProblem * max(1, len(problems)))()
        for i, p in enumerate(problems):
            arr[i] = TrmmProblem(p["layout"], p["side"], p["uplo"], p["transa"], p["diag"], p["m"], p["n"],
                                 p.get("alpha", 1.0), _ptr(p["A"]), p["lda"], _ptr(p["B"]), p["ldb"],
                                 p.get("tier", TIER_FP64), p.get("moduli", 0))
        g = C.c_void_p()
        check(lib().uvatrmm_group_create(handle.h, arr, len(problems), C.byref(g)))
        self.g, self.handle = g, handle

    def run(self) -> None:
        check(lib().uvatrmm_group_run(self.g))

    def stats(self) -> dict:
        f, la, wv = C.c_double(), C.c_int(), C.c_int()
        t64, toz, ab = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().uvatrmm_group_stats(self.g, C.byref(f), C.byref(la), C.byref(t64), C.byref(toz), C.byref(wv),
                                        C.byref(ab)))
        return {"flops": f.value, "launches": la.value, "fp64_tiles": t64.value, "ozaki_tiles": toz.value,
                "ozaki_waves": wv.value, "arena_bytes": ab.value}

    def close(self) -> None:
        if self.g:
            lib().uvatrmm_group_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _problem(p):
    from ._lib import TrmmProblem
    return TrmmProblem(p["layout"], p["side"], p["uplo"], p["transa"], p["diag"], p["m"], p["n"],
                       p.get("alpha", 1.0), _ptr(p["A"]), p["lda"], _ptr(p["B"]), p["ldb"],
                       p.get("tier", TIER_FP64), p.get("moduli", 0))


class Server:
    """The request loop with continuous batching (uvatrmm_server_*)."""

    def __init__(self, handle: "Handle", hbm_budget_bytes=0, max_active=0, tick_fp64_gflop=0.0,
                 tick_ozaki_gflop=0.0):
        from ._lib import ServerConfig
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_active), float(tick_fp64_gflop), float(tick_ozaki_gflop))
        s = C.c_void_p()
        check(lib().uvatrmm_server_create(handle.h, C.byref(cfg), C.byref(s)))
        self.s = s

    def submit(self, problem: dict, on_device: bool = True) -> int:
        rid = C.c_int64()
        pr = _problem(problem)
        check(lib().uvatrmm_server_submit(self.s, C.byref(pr), int(on_device), C.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout_s: float = 300.0) -> int:
        return lib().uvatrmm_server_wait(self.s, rid, timeout_s)

    def cancel(self, rid: int) -> int:
        return lib().uvatrmm_server_cancel(self.s, rid)

    def latency_ms(self, rid: int):
        """Submit -> result-ready ms of a completed request (None while in flight or failed)."""
        v = C.c_double()
        return v.value if lib().uvatrmm_server_latency(self.s, rid, C.byref(v)) == 0 else None

    def stats(self) -> dict:
        from ._lib import ServerStats
        st = ServerStats()
        check(lib().uvatrmm_server_get_stats(self.s, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self.s:
            lib().uvatrmm_server_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def host_empty(count: int, dtype="float64"):
    """A numpy array of `count` elements in page-locked, huge-page-backed host
    memory from uvatrmm_host_alloc (zeroed); freed when the array is collected.
    Operands of the host entry points keep their full copy rate in it."""
    import weakref

    import numpy as np
    dt = np.dtype(dtype)
    p = C.c_void_p()
    check(lib().uvatrmm_host_alloc(max(1, count) * dt.itemsize, C.byref(p)))
    buf = (C.c_char * (max(1, count) * dt.itemsize)).from_address(p.value)
    weakref.finalize(buf, lib().uvatrmm_host_free, p.value)
    return np.frombuffer(buf, dtype=dt, count=count)


def tune(handle: "Handle", tier: int, side: int, m: int, n: int) -> int:
    c = C.c_int()
    check(lib().uvatrmm_tune(handle.h, tier, side, m, n, C.byref(c)))
    return c.value


def ozaki_plan(k: int, moduli: int = 0):
    """(moduli, bits per scaled entry) the Ozaki path uses for inner dimension k."""
    mo, bi = C.c_int(), C.c_int()
    check(lib().uvatrmm_ozaki_plan(k, moduli, C.byref(mo), C.byref(bi)))
    return mo.value, bi.value


def map_rows(schedule: int, n: int, nblocks: int, idx: int):
    """The reference's map_regular / map_balanced; None where it aborts."""
    b, s = C.c_uint64(), C.c_uint64()
    rc = lib().uvatrmm_map_rows(schedule, n, nblocks, idx, C.byref(b), C.byref(s))
    return None if rc else (b.value, s.value)


def numroc(n: int, nb: int, iproc: int, isrcproc: int, nprocs: int) -> int:
    """Rows (or columns) of an n-long block-cyclic dimension held by process iproc."""
    return lib().uvatrmm_numroc(n, nb, iproc, isrcproc, nprocs)


def write_result(path: str, rows: int, cols: int, row_begin: int, nrows: int, col_begin: int, ncols: int,
                 block, ld: int) -> None:
    """Writes one rank's result block in the reference's binary result-file format."""
    check(lib().uvatrmm_write_result(path.encode(), rows, cols, row_begin, nrows, col_begin, ncols,
                                     _ptr(block) if block is not None else None, ld))


def read_result(path: str, out=None):
    """Reads a result file: (header of 6 ints, block as a flat float64 numpy array)."""
    import numpy as np
    import sys
    hdr = (C.c_int * 6)()
    try:
        with open(path, "rb") as f:  # sizes the buffer; the library parses and checks the file
            raw = f.read(24)
    except OSError as e:
        raise UvatrmmError(EINVAL, f"cannot open {path}: {e}") from None
    if len(raw) != 24:
        raise UvatrmmError(EINVAL, f"malformed result file: {path}")
    nr = int.from_bytes(raw[12:16], sys.byteorder, signed=True)
    nc = int.from_bytes(raw[20:24], sys.byteorder, signed=True)
    buf = np.empty(max(nr, 0) * max(nc, 0), dtype=np.float64) if out is None else out
    check(lib().uvatrmm_read_result(path.encode(), hdr, buf.ctypes.data if buf.size else None, buf.size))
    return list(hdr), buf
