"""Self-consistency of the oracle: naive loops, double-double, OpenBLAS."""
import itertools

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import (COL, LEFT, LOWER, NONUNIT, NOTRANS, RIGHT, ROW, TRANS, UNIT, UPPER, make_problem,
                           rel_fro)

VARIANTS = list(itertools.product((COL, ROW), (LEFT, RIGHT), (LOWER, UPPER), (NOTRANS, TRANS), (NONUNIT, UNIT)))


@pytest.mark.parametrize("layout,side,uplo,trans,diag", VARIANTS)
def test_naive_matches_openblas(built, layout, side, uplo, trans, diag):
    m, n = 13, 9
    A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=3, ldb_pad=2, garbage=123.0)
    B1, B2 = B.copy(), B.copy()
    orc.dtrmm_naive(layout, side, uplo, trans, diag, m, n, -1.5, A, lda, B1, ldb)
    orc.blas_dtrmm(layout, side, uplo, trans, diag, m, n, -1.5, A, lda, B2, ldb)
    assert np.abs(B1 - B2).max() < 1e-13
    # padding between columns (rows) is untouched
    assert np.array_equal(B1 == -7.0, B == -7.0)


def test_double_double_reference_is_more_accurate(built):
    m, n = 200, 7
    A, lda, B, ldb = make_problem(COL, LEFT, LOWER, m, n, garbage=0.0)
    ref = orc.dtrmm_dd(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, B, ldb)
    Am = A.reshape(m, lda).T[:m, :m]
    Bm = B.reshape(n, ldb).T[:m, :n]
    exact = np.tril(Am).astype(np.longdouble) @ Bm.astype(np.longdouble)
    assert rel_fro(ref, exact.astype(np.float64)) < 1e-16
    B2 = B.copy()
    orc.dtrmm_naive(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, B2, ldb)
    assert rel_fro(B2.reshape(n, ldb).T[:m], ref) < 1e-14


def test_uniform_and_wide_generators(built):
    a = orc.fill_uniform(1, 0, 300, 200)
    assert a.min() >= -1.0 and a.max() < 1.0 and abs(a.mean()) < 0.02
    assert np.array_equal(a, orc.fill_uniform(1, 0, 300, 200))
    assert not np.array_equal(a, orc.fill_uniform(2, 0, 300, 200))
    w = orc.fill_wide(2, 0, 200, 200, spread=20)
    e = np.frexp(w[w != 0])[1]
    assert e.min() >= -20 - 60 and e.max() <= 21
    ratio = w / orc.fill_uniform(2, 0, 200, 200)
    k = np.log2(np.abs(ratio[np.isfinite(ratio) & (ratio != 0)]))
    assert np.all(k == np.round(k)) and k.min() == -20 and k.max() == 20
    t = orc.fill_uniform(3, 0, 5, 5, tri="L", fill=np.nan)
    assert np.isnan(t[0, 1]) and not np.isnan(t[1, 0])


def test_product_decomposition_equals_plain_trmm(built):
    n = 300
    A = orc.fill_uniform(0, 0, n, n, tri="L")
    B = orc.fill_uniform(0, 1, n, n)
    ref = np.tril(A) @ B
    for P in (1, 2, 3, 5):
        for bal in (False, True):
            C = orc.uvatrmm_product(n, P, bal, A, B)
            assert rel_fro(C, ref) < 4 * n * np.finfo(float).eps
