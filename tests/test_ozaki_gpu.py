"""Ozaki-style emulated FP64 TRMM on the GPU, through the C ABI.

Bars: bit-exact where the exact product is representable (integer inputs);
relative Frobenius error <= 1e-14 against the oracle's double-double TRMM
otherwise (the accuracy target of the emulated tier).
"""
import itertools

import numpy as np
import pytest

import uvatrmm_gb300 as u
from oracle import oracle as orc
from tests.helpers import (COL, LEFT, LOWER, NONUNIT, NOTRANS, RIGHT, ROW, TRANS, UNIT, UPPER, make_problem,
                           rel_fro)

pytestmark = pytest.mark.gpu
VARIANTS = list(itertools.product((COL, ROW), (LEFT, RIGHT), (LOWER, UPPER), (NOTRANS, TRANS), (NONUNIT, UNIT)))
TOL = 1e-14


def dd_reference(layout, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb):
    """Double-double result written back into a copy of B's storage."""
    ref_cm = orc.dtrmm_dd(layout, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb)
    out = B.copy()
    M, N = ref_cm.shape
    for j in range(N):
        out[j * ldb:j * ldb + M] = ref_cm[:, j]
    return out


@pytest.mark.parametrize("layout,side,uplo,trans,diag", VARIANTS)
def test_ozaki_all_variants_vs_double_double(handle, layout, side, uplo, trans, diag):
    m, n = 70, 90
    A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=1, ldb_pad=2)
    ref = dd_reference(layout, side, uplo, trans, diag, m, n, -0.5, A, lda, B, ldb)
    got = B.copy()
    err, bits = handle.ozaki(layout, side, uplo, trans, diag, m, n, -0.5, A, lda, got, ldb, want_err=True)
    pad = B == -7.0
    assert np.array_equal(got[pad], B[pad])
    assert rel_fro(got[~pad], ref[~pad]) <= TOL
    assert bits >= 52 and err <= TOL


@pytest.mark.parametrize("K", [513, 1100, 2500])
@pytest.mark.parametrize("side", [LEFT, RIGHT])
def test_ozaki_exact_on_integer_inputs(handle, K, side):
    """Integer operands: the emulated product is exact, across several
    512-wide K chunks (exercising the in-TMEM modular folds)."""
    rng = np.random.default_rng(K)
    m, n = (K, 37) if side == LEFT else (37, K)
    Af = rng.integers(-1024, 1025, size=(K, K)).astype(np.float64)
    Bf = rng.integers(-1024, 1025, size=(m, n)).astype(np.float64)
    exact = (np.tril(Af).astype(np.int64) @ Bf.astype(np.int64)) if side == LEFT else \
        (Bf.astype(np.int64) @ np.tril(Af).astype(np.int64))
    A = np.asfortranarray(Af).ravel(order="F").copy()
    B = np.asfortranarray(Bf).ravel(order="F").copy()
    handle.ozaki(COL, side, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, K, B, m)
    got = B.reshape(n, m).T
    assert np.array_equal(got, exact.astype(np.float64))


def test_ozaki_device_in_place_matches_host(handle):
    import torch
    m, n = 300, 200
    A, lda, B, ldb = make_problem(COL, LEFT, UPPER, m, n)
    host = B.copy()
    handle.ozaki(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, 1.0, A, lda, host, ldb)
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B.copy()).cuda()
    handle.ozaki_device(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, 1.0, dA, lda, dB, ldb)
    handle.sync()
    assert np.array_equal(dB.cpu().numpy(), host)


def test_ozaki_raster_group_does_not_change_the_result(handle):
    """The raster group only reorders the residue GEMM's tiles: bit-identical results."""
    m, n = 1100, 700
    for side in (LEFT, RIGHT):
        A, lda, B, ldb = make_problem(COL, side, LOWER, m, n)
        want = B.copy()
        handle.ozaki(COL, side, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, want, ldb)
        try:
            for g in (1, 3, 16):
                handle.set_option("ozaki_raster", g)
                got = B.copy()
                handle.ozaki(COL, side, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, got, ldb)
                assert np.array_equal(got, want), g
        finally:
            handle.set_option("ozaki_raster", 0)
    with pytest.raises(u.UvatrmmError):
        handle.set_option("ozaki_raster", 65)


def test_ozaki_passes_do_not_change_the_result(handle):
    m, n = 640, 300
    A, lda, B, ldb = make_problem(COL, RIGHT, LOWER, m, n)
    one = B.copy()
    handle.ozaki(COL, RIGHT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, one, ldb, moduli=16)
    handle.set_option("tile", 0)
    try:
        u.check(u.lib().uvatrmm_set_option(handle.h, 5, 64))  # 64 MiB of residue planes per pass
        many = B.copy()
        handle.ozaki(COL, RIGHT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, many, ldb, moduli=16)
    finally:
        u.check(u.lib().uvatrmm_set_option(handle.h, 5, 49152))
    assert np.array_equal(one, many)


@pytest.mark.parametrize("moduli", [2, 3, 5, 8, 12, 16, 20])
def test_ozaki_exact_forced_slice_counts(handle, moduli):
    """Integer operands that fit the slice count's bits give the exact product
    for every slice count: the 64-bit slicing path (bits <= 63), the wide
    path (20 slices: more than 63 bits), and the CRT reconstruction from one
    to six 32-bit limbs."""
    K = 1100 if moduli >= 5 else 64
    _, bits = u.ozaki_plan(K, moduli)
    hi = 2 ** min(bits - 1, 11) - 1
    rng = np.random.default_rng(moduli)
    m, n = K, 29
    Af = rng.integers(-hi, hi + 1, size=(K, K)).astype(np.float64)
    Bf = rng.integers(-hi, hi + 1, size=(m, n)).astype(np.float64)
    exact = np.tril(Af).astype(np.int64) @ Bf.astype(np.int64)
    A = np.asfortranarray(Af).ravel(order="F").copy()
    B = np.asfortranarray(Bf).ravel(order="F").copy()
    _, got_bits = handle.ozaki(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, K, B, m, moduli=moduli)
    assert got_bits == bits
    assert np.array_equal(B.reshape(n, m).T, exact.astype(np.float64))


def test_ozaki_wide_exponent_sweep(handle):
    """Entries uniform[-1,1) * 2^k, k in [-20, 20] (the precision config's
    distribution): error falls with the slice count and meets 1e-14 with the
    automatic choice."""
    m = n = 384
    Am = orc.fill_wide(2, 0, m, m, spread=20)
    Bm = orc.fill_wide(2, 1, m, n, spread=20)
    A = np.asfortranarray(np.triu(Am)).ravel(order="F").copy()
    B = np.asfortranarray(Bm).ravel(order="F").copy()
    ref = orc.dtrmm_dd(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, 1.0, A, m, B, m)
    errs = {}
    for mo in (10, 12, 14, 16, 18, 20):
        got = B.copy()
        est, bits = handle.ozaki(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, 1.0, A, m, got, m, moduli=mo,
                                 want_err=True)
        errs[mo] = rel_fro(got.reshape(n, m).T, ref)
    assert errs[20] <= errs[10]
    got = B.copy()
    handle.ozaki(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, 1.0, A, m, got, m)
    assert rel_fro(got.reshape(n, m).T, ref) <= TOL, errs


@pytest.mark.parametrize("m,n", [(0, 4), (4, 0), (1, 1), (1, 300), (300, 1), (129, 257)])
def test_ozaki_edge_sizes(handle, m, n):
    for side in (LEFT, RIGHT):
        A, lda, B, ldb = make_problem(COL, side, LOWER, m, n)
        ref = dd_reference(COL, side, LOWER, NOTRANS, UNIT, m, n, 3.0, A, lda, B, ldb) if m and n else B.copy()
        got = B.copy()
        handle.ozaki(COL, side, LOWER, NOTRANS, UNIT, m, n, 3.0, A, lda, got, ldb)
        pad = B == -7.0
        assert rel_fro(got[~pad], ref[~pad]) <= TOL


def test_ozaki_zero_rows_and_alpha_zero(handle):
    m, n = 50, 40
    A, lda, B, ldb = make_problem(COL, LEFT, LOWER, m, n)
    B2 = B.copy()
    B2[5 * ldb:5 * ldb + m] = 0.0  # one zero column of B
    ref = dd_reference(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, B2, ldb)
    got = B2.copy()
    handle.ozaki(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, got, ldb)
    assert np.all(got[5 * ldb:5 * ldb + m] == 0.0)
    assert rel_fro(got, ref) <= TOL
    got = B.copy()
    handle.ozaki(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 0.0, A, lda, got, ldb)
    assert np.all(got.reshape(n, ldb)[:, :m] == 0.0)


def _sampled_relerr(layout, side, m, n, got, ldb, ref_cm, S=8):
    """Relative Frobenius error over the error report's samples: S evenly
    spaced columns (side Left of the column-major-normalised call) or rows
    (side Right) of the result."""
    M, N = ref_cm.shape
    nside = side if layout == COL else (RIGHT if side == LEFT else LEFT)
    g = np.lib.stride_tricks.as_strided(got, (M, N), (8, 8 * ldb))
    cnt = N if nside == LEFT else M
    S = min(S, cnt)
    idx = [(cnt - 1) * s // (S - 1) if S > 1 else 0 for s in range(S)]
    if nside == LEFT:
        return rel_fro(g[:, idx], ref_cm[:, idx])
    return rel_fro(g[idx, :], ref_cm[idx, :])


@pytest.mark.parametrize("layout,side,uplo,trans,diag", [(COL, LEFT, LOWER, NOTRANS, UNIT),
                                                         (ROW, RIGHT, UPPER, TRANS, NONUNIT),
                                                         (COL, RIGHT, LOWER, NOTRANS, NONUNIT),
                                                         (ROW, LEFT, UPPER, TRANS, UNIT),
                                                         (COL, LEFT, UPPER, TRANS, NONUNIT),
                                                         (COL, RIGHT, UPPER, TRANS, UNIT)])
def test_error_report_against_the_host_fp64_reference(handle, layout, side, uplo, trans, diag):
    """relerr_out of the host entry point is measured against FP64 on the host
    (compensated dot products from the caller's own A and B).  With 6 moduli
    the emulated result is deliberately coarse (about 21 bits), so the report
    must equal the error against the double-double oracle over the same
    sampled vectors; the device entry point with UVATRMM_OPT_OZAKI_ERR_HOST
    reports the same number."""
    import torch
    m, n = 70, 45
    A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=1, ldb_pad=2, seed=31)
    ref_cm = orc.dtrmm_dd(layout, side, uplo, trans, diag, m, n, 1.5, A, lda, B, ldb)
    got = B.copy()
    err, bits = handle.ozaki(layout, side, uplo, trans, diag, m, n, 1.5, A, lda, got, ldb, moduli=6, want_err=True)
    expect = _sampled_relerr(layout, side, m, n, got, ldb, ref_cm)
    assert 1e-9 < expect < 1e-3, expect
    assert abs(err - expect) <= 1e-6 * expect, (err, expect)
    h = u.Handle()
    try:
        h.set_option("ozaki_err_host", 1)
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B.copy()).cuda()
        derr, _ = h.ozaki_device(layout, side, uplo, trans, diag, m, n, 1.5, dA, lda, dB, ldb, moduli=6,
                                 want_err=True)
        assert np.array_equal(dB.cpu().numpy(), got)
        assert derr == err
    finally:
        h.close()


def test_error_report_is_zero_for_exact_products(handle):
    """Integer operands give an exact emulated product and an exact host
    reference (every partial sum is an integer below 2^53): the report is 0."""
    rng = np.random.default_rng(5)
    K, n = 700, 33
    Af = rng.integers(-1024, 1025, size=(K, K)).astype(np.float64)
    Bf = rng.integers(-1024, 1025, size=(K, n)).astype(np.float64)
    A = np.asfortranarray(Af).ravel(order="F").copy()
    B = np.asfortranarray(Bf).ravel(order="F").copy()
    err, _ = handle.ozaki(COL, LEFT, UPPER, TRANS, NONUNIT, K, n, 1.0, A, K, B, K, want_err=True)
    assert err == 0.0


@pytest.mark.parametrize("side,uplo,trans", [(LEFT, UPPER, TRANS), (LEFT, LOWER, NOTRANS),
                                             (RIGHT, LOWER, NOTRANS), (RIGHT, UPPER, TRANS)])
def test_ozaki_large_wide_exponents_sampled_vs_double_double(handle, side, uplo, trans):
    """m = n = 6144 on the device with entries uniform[-1,1) * 2^k, k in [-20, 20]
    (the precision configuration's distribution) and NaN in the unreferenced
    triangle: sampled result columns (side Left) or rows (side Right) within
    1e-14 of the double-double oracle."""
    import torch
    m = n = 6144
    ka = m
    dA = torch.empty(ka * ka, dtype=torch.float64, device="cuda")
    dB = torch.empty(m * n, dtype=torch.float64, device="cuda")
    handle.gen_uniform(7, 0, ka, ka, dA, 1, ka, tri="L" if uplo == LOWER else "U", fill=float("nan"), spread=20)
    handle.gen_uniform(7, 1, m, n, dB, 1, m, spread=20)
    handle.sync()
    A = dA.cpu().numpy()
    B0 = dB.cpu().numpy()
    handle.ozaki_device(COL, side, uplo, trans, NONUNIT, m, n, 1.0, dA, ka, dB, m)
    handle.sync()
    got_all = dB.cpu().numpy()
    sel = [0, 1, 2047, 4096, 6143]
    got, ref = [], []
    for j in sel:
        if side == LEFT:
            ref.append(orc.dtrmm_dd(COL, side, uplo, trans, NONUNIT, m, n, 1.0, A, ka, B0, m, cols=(j, j + 1))[:, 0])
            got.append(got_all[j * m:(j + 1) * m])
        else:
            ref.append(orc.dtrmm_dd(COL, side, uplo, trans, NONUNIT, m, n, 1.0, A, ka, B0, m, rows=(j, j + 1))[0, :])
            got.append(got_all[j::m])
    assert rel_fro(np.concatenate(got), np.concatenate(ref)) <= TOL
