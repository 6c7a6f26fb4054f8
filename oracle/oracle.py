"""Python face of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker or as the timed CPU baseline.  The
product (``uvatrmm_gb300``) never imports it.

It wraps oracle/_build/liboracle.so (oracle/trmm_oracle.c, built by
oracle/Makefile) with numpy-facing helpers.  Each helper names the reference
lines that the C function restates.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

ROW, COL = 101, 102
NOTRANS, TRANS = 111, 112
UPPER, LOWER = 121, 122
NONUNIT, UNIT = 131, 132
LEFT, RIGHT = 141, 142

_lib = None
_blas_loaded = False


def build() -> None:
    """Compile oracle/trmm_oracle.c (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        u64, i64, u32, i32, dbl = C.c_uint64, C.c_int64, C.c_uint32, C.c_int, C.c_double
        P = C.c_void_p
        L.orc_map_regular.argtypes = [u64, u32, u32, C.POINTER(u64), C.POINTER(u64)]
        L.orc_map_balanced.argtypes = [u64, u32, u32, C.POINTER(u64), C.POINTER(u64)]
        L.orc_gen_consecutive.argtypes = [i64, i64, i64, i64, i64, i32, i32, P]
        L.orc_gen_consecutive.restype = None
        L.orc_fill_uniform.argtypes = [u64, u64, i64, i64, P, i64, i64, i32, dbl]
        L.orc_fill_uniform.restype = None
        L.orc_fill_wide.argtypes = [u64, u64, i64, i64, P, i64, i64, i32, dbl, i32]
        L.orc_fill_wide.restype = None
        L.orc_dtrmm_naive.argtypes = [i32, i32, i32, i32, i32, i64, i64, dbl, P, i64, P, i64]
        L.orc_dtrmm_dd.argtypes = [i32, i32, i32, i32, i32, i64, i64, dbl, P, i64, P, i64,
                                   i64, i64, i64, i64, P, i64]
        L.orc_blas_load.argtypes = [C.c_char_p]
        L.orc_blas_threads.argtypes = [i32]
        L.orc_blas_threads.restype = None
        L.orc_blas_dtrmm.argtypes = [i32, i32, i32, i32, i32, i32, i32, dbl, P, i32, P, i32]
        L.orc_blas_dgemm.argtypes = [i32, i32, i32, i32, i32, i32, dbl, P, i32, P, i32, dbl, P, i32]
        L.orc_uvatrmm_product.argtypes = [i64, u32, i32, P, P, P]
        L.orc_uvatrmm_ranks.argtypes = [i64, u32, i32, u32, u32, P, P, P]
        L.orc_inf_norm.argtypes = [i64, i64, P, i64]
        L.orc_inf_norm.restype = dbl
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ---------------------------------------------------------------- mappings

def map_regular(n: int, P: int, idx: int):
    """UVaTRMM/src/mm_mapping.c:27-67.  (begin, size) or None where it aborts."""
    b, s = C.c_uint64(), C.c_uint64()
    rc = lib().orc_map_regular(n, P, idx, C.byref(b), C.byref(s))
    return None if rc else (b.value, s.value)


def map_balanced(n: int, P: int, idx: int):
    """UVaTRMM/src/mm_mapping.c:319-366.  (begin, size) or None where it aborts."""
    b, s = C.c_uint64(), C.c_uint64()
    rc = lib().orc_map_balanced(n, P, idx, C.byref(b), C.byref(s))
    return None if rc else (b.value, s.value)


# ---------------------------------------------------------------- generators

def gen_consecutive(n: int, rows_begin: int, rows: int, cols_begin: int, cols: int,
                    triangular: bool, mininums: bool = True) -> np.ndarray:
    """UVaTRMM/src/mm_triangular_common.c:1782-1805 (row-major block)."""
    out = np.empty((rows, cols), dtype=np.float64)
    lib().orc_gen_consecutive(n, rows_begin, rows, cols_begin, cols, int(triangular), int(mininums), _ptr(out))
    return out


def fill_uniform(seed: int, stream: int, rows: int, cols: int, tri: str | None = None,
                 fill: float = 0.0) -> np.ndarray:
    """Seeded uniform[-1,1) matrix; element (i,j) from logical index i*cols+j."""
    out = np.empty((rows, cols), dtype=np.float64)
    t = 0 if tri is None else ord(tri)
    lib().orc_fill_uniform(seed, stream, rows, cols, _ptr(out), cols, 1, t, fill)
    return out


def fill_wide(seed: int, stream: int, rows: int, cols: int, spread: int = 20, tri: str | None = None,
              fill: float = 0.0) -> np.ndarray:
    """As fill_uniform, each element times 2^k, k uniform in [-spread, spread]."""
    out = np.empty((rows, cols), dtype=np.float64)
    t = 0 if tri is None else ord(tri)
    lib().orc_fill_wide(seed, stream, rows, cols, _ptr(out), cols, 1, t, fill, spread)
    return out


# ---------------------------------------------------------------- TRMM

def dtrmm_naive(layout, side, uplo, transa, diag, m, n, alpha, A: np.ndarray, lda, B: np.ndarray, ldb) -> None:
    """cblas_dtrmm semantics, naive FP64 loops, in place on B (flat buffers)."""
    assert A.dtype == np.float64 and B.dtype == np.float64
    rc = lib().orc_dtrmm_naive(layout, side, uplo, transa, diag, m, n, alpha, _ptr(A), lda, _ptr(B), ldb)
    assert rc == 0


def dtrmm_dd(layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb,
             rows=None, cols=None) -> np.ndarray:
    """Double-double reference of the column-major-normalised result.

    Returns the block [rows) x [cols) of the result as a column-major
    (Fortran-ordered) array; the normalised problem is M x N with
    (M, N) = (m, n) for column-major and (n, m) for row-major calls.
    """
    M, N = (m, n) if layout == COL else (n, m)
    r0, r1 = rows if rows is not None else (0, M)
    c0, c1 = cols if cols is not None else (0, N)
    out = np.zeros((r1 - r0, c1 - c0), dtype=np.float64, order="F")
    lib().orc_dtrmm_dd(layout, side, uplo, transa, diag, m, n, alpha, _ptr(A), lda, _ptr(B), ldb,
                       r0, r1, c0, c1, _ptr(out), max(r1 - r0, 1))
    return out


def openblas_path() -> str:
    import scipy
    c = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs",
                                      "libscipy_openblas*.so")))
    if not c:
        raise RuntimeError("scipy-bundled OpenBLAS not found")
    return os.path.realpath(c[0])


def blas_ready(threads: int | None = None) -> None:
    global _blas_loaded
    if not _blas_loaded:
        rc = lib().orc_blas_load(openblas_path().encode())
        if rc:
            raise RuntimeError(f"could not load OpenBLAS CBLAS symbols (rc={rc})")
        _blas_loaded = True
    if threads is not None:
        lib().orc_blas_threads(threads)


def blas_dtrmm(layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb) -> None:
    """OpenBLAS cblas_dtrmm in place on B (the reference links MKL's)."""
    blas_ready()
    rc = lib().orc_blas_dtrmm(layout, side, uplo, transa, diag, m, n, alpha, _ptr(A), lda, _ptr(B), ldb)
    assert rc == 0


def blas_dgemm(layout, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc) -> None:
    """OpenBLAS cblas_dgemm (the local GEMM of UVaTRMM/src/mm_triangular.c:347-360), in place on Cm."""
    blas_ready()
    rc = lib().orc_blas_dgemm(layout, ta, tb, m, n, k, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(Cm), ldc)
    assert rc == 0


def uvatrmm_product(n: int, P: int, balanced: bool, A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """UVaTRMM/src/mm_triangular.c:319-403 for all P ranks; row-major n x n."""
    blas_ready()
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    Cm = np.zeros((n, n), dtype=np.float64)
    rc = lib().orc_uvatrmm_product(n, P, int(balanced), _ptr(A), _ptr(B), _ptr(Cm))
    if rc:
        raise ValueError(f"reference decomposition aborts for n={n} P={P} (rc={rc})")
    return Cm


def uvatrmm_ranks(n: int, P: int, balanced: bool, r0: int, r1: int, A: np.ndarray, B: np.ndarray,
                  Cm: np.ndarray) -> None:
    """Ranks [r0, r1) of UVaTRMM/src/mm_triangular.c:319-403 (their column slices of Cm)."""
    blas_ready()
    rc = lib().orc_uvatrmm_ranks(n, P, int(balanced), r0, r1, _ptr(A), _ptr(B), _ptr(Cm))
    if rc:
        raise ValueError(f"reference decomposition aborts for n={n} P={P} (rc={rc})")


def inf_norm(Cm: np.ndarray) -> float:
    """UVaTRMM/src/mm_triangular_common.c:2936-2991 (row-major)."""
    Cm = np.ascontiguousarray(Cm, dtype=np.float64)
    return lib().orc_inf_norm(Cm.shape[0], Cm.shape[1], _ptr(Cm), Cm.shape[1])


def ref_binary(name: str) -> str | None:
    """Path of a program built by oracle/build_ref.sh, or None."""
    p = os.path.join(REF_DIR, name)
    return p if os.path.exists(p) else None


# ---------------------------------------------------------------- result files

def result_file_bytes(rows: int, cols: int, row_begin: int, nrows: int, col_begin: int, ncols: int,
                      block: np.ndarray) -> bytes:
    """The bytes print_output_results_generic writes
    (UVaTRMM/src/mm_triangular_common.c:2134-2163): the ints rows, cols,
    row_begin, nrows, col_begin, ncols in native order, then the nrows x ncols
    row-major block of doubles.  print_output_results (:2103-2131) is the
    special case row_begin = 0, nrows = rows."""
    hdr = np.array([rows, cols, row_begin, nrows, col_begin, ncols], dtype=np.intc)
    body = np.ascontiguousarray(np.asarray(block, dtype=np.float64).reshape(nrows, ncols))
    return hdr.tobytes() + body.tobytes()


# ---------------------------------------------------------------- ScaLAPACK block-cyclic layout

def numroc(n: int, nb: int, iproc: int, isrcproc: int, nprocs: int) -> int:
    """ScaLAPACK's NUMROC (TOOLS/numroc.f, ScaLAPACK 2.x; the library is not part
    of the reference, which calls it at ScaLAPACK/scalapack_sample_trmm.c:66-67
    and scalapack_sample_gemm.c:60-61): how many of the n rows (or columns),
    dealt out in blocks of nb round-robin from process isrcproc, process iproc
    holds.  Restated from the published algorithm."""
    mydist = (nprocs + iproc - isrcproc) % nprocs
    nblocks = n // nb
    r = (nblocks // nprocs) * nb
    extra = nblocks % nprocs
    if mydist < extra:
        r += nb
    elif mydist == extra:
        r += n % nb
    return r


def _local_to_global(nloc: int, nb: int, me: int, nprocs: int) -> np.ndarray:
    """Global index of each local index (ScaLAPACK/scalapack_sample_trmm.c:77-86)."""
    i = np.arange(nloc)
    return ((i // nb) * nprocs + me) * nb + i % nb


def sample_locals(kind: str, n: int, nb: int, nprow: int, npcol: int) -> dict:
    """Local column-major blocks (mpA x nqA, ld mpA) of the ScaLAPACK samples, in
    BLACS rank order iam = myrow*npcol + mycol (row-major grid, layout 'R').

    kind "trmm": ScaLAPACK/scalapack_sample_trmm.c:74-96 -- A[k] = 9*iam + counter
    on and below the diagonal (0 above), B = 1 on and below, 2 above.
    kind "gemm": ScaLAPACK/scalapack_sample_gemm.c:64-85 -- A[k] = 9*iam + counter
    everywhere, B = 2 on the diagonal (0 elsewhere), C = 0."""
    out = {"A": [], "B": [], "C": []}
    for iam in range(nprow * npcol):
        myrow, mycol = iam // npcol, iam % npcol
        mp, nq = numroc(n, nb, myrow, 0, nprow), numroc(n, nb, mycol, 0, npcol)
        I = _local_to_global(mp, nb, myrow, nprow)[:, None]
        J = _local_to_global(nq, nb, mycol, npcol)[None, :]
        # counter runs over local columns, then local rows (k = i + j*mp)
        k = (np.arange(mp)[:, None] + np.arange(nq)[None, :] * mp).astype(np.float64)
        if kind == "trmm":
            low = I >= J
            A = np.where(low, 9.0 * iam + np.cumsum(low.T.ravel()).reshape(nq, mp).T - 1.0, 0.0)
            B = np.where(low, 1.0, 2.0)
        else:
            A = 9.0 * iam + k
            B = np.where(I == J, 2.0, 0.0)
        out["A"].append(np.asfortranarray(A))
        out["B"].append(np.asfortranarray(B))
        out["C"].append(np.zeros((mp, nq), order="F"))
    return out


def bc_to_global(locals_: list, m: int, n: int, mb: int, nb: int, nprow: int, npcol: int) -> np.ndarray:
    """The global m x n matrix whose block-cyclic pieces are locals_ (ordered p*npcol + q)."""
    G = np.zeros((m, n))
    for pq, L in enumerate(locals_):
        p, q = pq // npcol, pq % npcol
        I = _local_to_global(L.shape[0], mb, p, nprow)
        J = _local_to_global(L.shape[1], nb, q, npcol)
        G[np.ix_(I, J)] = L
    return G


def bc_from_global(G: np.ndarray, mb: int, nb: int, nprow: int, npcol: int) -> list:
    """Block-cyclic pieces of G, ordered p*npcol + q (inverse of bc_to_global)."""
    m, n = G.shape
    out = []
    for pq in range(nprow * npcol):
        p, q = pq // npcol, pq % npcol
        I = _local_to_global(numroc(m, mb, p, 0, nprow), mb, p, nprow)
        J = _local_to_global(numroc(n, nb, q, 0, npcol), nb, q, npcol)
        out.append(np.asfortranarray(G[np.ix_(I, J)]))
    return out
