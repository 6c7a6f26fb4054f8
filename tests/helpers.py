"""Shared test helpers: seeded problems in flat column/row-major buffers."""
from __future__ import annotations

import numpy as np

from oracle import oracle as orc

ROW, COL = 101, 102
NOTRANS, TRANS = 111, 112
UPPER, LOWER = 121, 122
NONUNIT, UNIT = 131, 132
LEFT, RIGHT = 141, 142

EPS = np.finfo(np.float64).eps


def dims(layout, side, m, n):
    """(ka, rows_of_B_storage, cols_of_B_storage) for a CBLAS call."""
    ka = m if side == LEFT else n
    if layout == COL:
        return ka, m, n
    return ka, n, m  # row-major B: m rows of n -> as storage: n contiguous


def make_problem(layout, side, uplo, m, n, lda_pad=0, ldb_pad=0, seed=7, garbage=np.nan):
    """Flat A (ka x ka, ld lda) and B buffers; the unreferenced triangle of A
    holds `garbage`.  Storage is column-major for COL and row-major for ROW.
    Returns A, lda, B, ldb."""
    ka = m if side == LEFT else n
    lda = max(ka, 1) + lda_pad
    Am = orc.fill_uniform(seed, 0, ka, ka)  # logical matrix (i, j)
    keep = np.tril(np.ones((ka, ka), bool)) if uplo == LOWER else np.triu(np.ones((ka, ka), bool))
    Am = np.where(keep, Am, garbage)
    Bm = orc.fill_uniform(seed, 1, m, n)
    A = np.full(lda * max(ka, 1), 1e300)
    if layout == COL:
        ldb = max(m, 1) + ldb_pad
        B = np.full(ldb * max(n, 1), -7.0)
        for j in range(ka):
            A[j * lda:j * lda + ka] = Am[:, j]
        for j in range(n):
            B[j * ldb:j * ldb + m] = Bm[:, j]
    else:
        ldb = max(n, 1) + ldb_pad
        B = np.full(ldb * max(m, 1), -7.0)
        for i in range(ka):
            A[i * lda:i * lda + ka] = Am[i, :]
        for i in range(m):
            B[i * ldb:i * ldb + n] = Bm[i, :]
    return A, lda, B, ldb


def view(buf, layout, rows, cols, ld):
    """Logical rows x cols matrix of a flat buffer."""
    if layout == COL:
        return np.lib.stride_tricks.as_strided(buf, (rows, cols), (8, 8 * ld)).copy()
    return np.lib.stride_tricks.as_strided(buf, (rows, cols), (8 * ld, 8)).copy()


def rel_fro(x, ref):
    d = np.linalg.norm(ref)
    return np.linalg.norm(x - ref) / (d if d > 0 else 1.0)


def oracle_result(p):
    """The oracle's logical m x n result for a problem dict (layout, side, uplo,
    transa, diag, m, n, alpha, A (host array or CUDA tensor), lda, B0 (the host
    input buffer), ldb, tier) and the tolerance of its tier: FP64 against the
    naive FP64 loops at 8 k eps, Ozaki against the double-double oracle at
    1e-14 (relative Frobenius)."""
    A = p["A"].cpu().numpy() if hasattr(p["A"], "cpu") else p["A"]
    layout, m, n = p["layout"], p["m"], p["n"]
    args = (layout, p["side"], p["uplo"], p["transa"], p["diag"], m, n, p["alpha"])
    if p.get("tier", 0) == 1:
        R = orc.dtrmm_dd(*args, A, p["lda"], p["B0"].copy(), p["ldb"])
        return (R if layout == COL else R.T), 1e-14
    ref = p["B0"].copy()
    orc.dtrmm_naive(*args, A, p["lda"], ref, p["ldb"])
    k = m if p["side"] == LEFT else n
    return view(ref, layout, m, n, p["ldb"]), 8 * max(k, 1) * EPS


def assert_matches_oracle(p, got_buf, what=""):
    """Asserts that the flat result buffer of problem p is within its tier's
    tolerance of the oracle (see oracle_result)."""
    if p["m"] == 0 or p["n"] == 0:
        return
    ref, tol = oracle_result(p)
    got = view(got_buf, p["layout"], p["m"], p["n"], p["ldb"])
    err = rel_fro(got, ref)
    assert err <= tol, (what, p.get("tier"), p["m"], p["n"], err, tol)
