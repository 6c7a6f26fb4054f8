"""Plain FP64 TRMM on the GPU, through the C ABI, against the oracle.

Tolerance: relative Frobenius error <= 8 * k * eps against the oracle's
naive FP64 loops (k = order of the triangular matrix), or bitwise where the
arithmetic order makes it exact (generators).
"""
import itertools
import json
import os
import subprocess

import numpy as np
import pytest

import uvatrmm_gb300 as u
from oracle import oracle as orc
from tests.helpers import (COL, EPS, LEFT, LOWER, NONUNIT, NOTRANS, RIGHT, ROW, TRANS, UNIT, UPPER, make_problem,
                           rel_fro)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
VARIANTS = list(itertools.product((COL, ROW), (LEFT, RIGHT), (LOWER, UPPER), (NOTRANS, TRANS), (NONUNIT, UNIT)))


def torch_dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def oracle_result(layout, side, uplo, trans, diag, m, n, alpha, A, lda, B, ldb):
    ref = B.copy()
    orc.dtrmm_naive(layout, side, uplo, trans, diag, m, n, alpha, A, lda, ref, ldb)
    return ref


def check_close(got, ref, B_orig, k, tol_mult=8):
    pad = B_orig == -7.0
    assert np.array_equal(got[pad], B_orig[pad]), "padding was written"
    assert rel_fro(got[~pad], ref[~pad]) <= tol_mult * max(k, 1) * EPS


@pytest.mark.parametrize("engine", [u.ENGINE_DFMA, u.ENGINE_DMMA])
@pytest.mark.parametrize("layout,side,uplo,trans,diag", VARIANTS)
def test_host_api_all_variants(handle, engine, layout, side, uplo, trans, diag):
    handle.set_option("engine", engine)
    try:
        for (m, n) in ((37, 21), (70, 131)):
            A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=1, ldb_pad=3)
            ref = oracle_result(layout, side, uplo, trans, diag, m, n, 0.75, A, lda, B, ldb)
            got = B.copy()
            handle.dtrmm(layout, side, uplo, trans, diag, m, n, 0.75, A, lda, got, ldb)
            check_close(got, ref, B, m if side == LEFT else n)
    finally:
        handle.set_option("engine", u.ENGINE_DFMA)


@pytest.mark.parametrize("tile", [64, 128])
@pytest.mark.parametrize("schedule", [u.SCHED_DYNAMIC, u.SCHED_REG, u.SCHED_BALANCED])
@pytest.mark.parametrize("shape", [u.SHAPE_TRAPEZOID, u.SHAPE_BOXES])
def test_schedules_shapes_tiles(handle, tile, schedule, shape):
    handle.set_option("tile", tile)
    handle.set_option("schedule", schedule)
    handle.set_option("shape", shape)
    try:
        for (layout, side, uplo, trans) in ((COL, LEFT, LOWER, NOTRANS), (COL, RIGHT, UPPER, TRANS),
                                            (ROW, LEFT, UPPER, TRANS)):
            m, n = 300, 260
            A, lda, B, ldb = make_problem(layout, side, uplo, m, n)
            ref = oracle_result(layout, side, uplo, trans, NONUNIT, m, n, 1.0, A, lda, B, ldb)
            got = B.copy()
            handle.dtrmm(layout, side, uplo, trans, NONUNIT, m, n, 1.0, A, lda, got, ldb)
            check_close(got, ref, B, m if side == LEFT else n)
    finally:
        handle.set_option("tile", 0)
        handle.set_option("schedule", u.SCHED_DYNAMIC)
        handle.set_option("shape", u.SHAPE_TRAPEZOID)


@pytest.mark.parametrize("engine", [u.ENGINE_DFMA, u.ENGINE_DMMA])
@pytest.mark.parametrize("tile", [64, 128])
@pytest.mark.parametrize("shape", [u.SHAPE_TRAPEZOID, u.SHAPE_BOXES])
def test_partial_and_diagonal_tiles_every_variant(handle, engine, tile, shape):
    """Tiles that overhang the matrix compute only their valid register rows
    (DFMA) or fragments (DMMA) and column blocks, and trapezoid diagonal
    slabs skip the rows or column blocks in the zero half: sizes that leave
    every row-range case of the skipping (partial last tiles of 1-63 rows,
    triangles of 1-3 tiles) for all 16 column-major variants, NaN in the
    unreferenced triangle."""
    handle.set_option("engine", engine)
    handle.set_option("tile", tile)
    handle.set_option("shape", shape)
    try:
        for side, uplo, trans, diag in itertools.product((LEFT, RIGHT), (LOWER, UPPER), (NOTRANS, TRANS),
                                                         (NONUNIT, UNIT)):
            for (m, n) in ((50, 33), (111, 70), (200, 17), (18, 145)):
                A, lda, B, ldb = make_problem(COL, side, uplo, m, n, ldb_pad=2)
                ref = oracle_result(COL, side, uplo, trans, diag, m, n, -1.5, A, lda, B, ldb)
                got = B.copy()
                handle.dtrmm(COL, side, uplo, trans, diag, m, n, -1.5, A, lda, got, ldb)
                check_close(got, ref, B, m if side == LEFT else n)
    finally:
        handle.set_option("engine", u.ENGINE_DFMA)
        handle.set_option("tile", 0)
        handle.set_option("shape", u.SHAPE_TRAPEZOID)


@pytest.mark.parametrize("m,n", [(0, 5), (5, 0), (1, 1), (1, 17), (17, 1), (2, 3), (63, 65), (129, 2)])
def test_edge_sizes(handle, m, n):
    for side in (LEFT, RIGHT):
        A, lda, B, ldb = make_problem(COL, side, LOWER, m, n)
        ref = oracle_result(COL, side, LOWER, NOTRANS, NONUNIT, m, n, 2.0, A, lda, B, ldb)
        got = B.copy()
        handle.dtrmm(COL, side, LOWER, NOTRANS, NONUNIT, m, n, 2.0, A, lda, got, ldb)
        check_close(got, ref, B, max(m, n))


def test_alpha_zero_does_not_read_A(handle):
    m, n = 40, 30
    A, lda, B, ldb = make_problem(COL, LEFT, LOWER, m, n)
    A[:] = np.nan
    got = B.copy()
    got[0] = np.nan
    handle.dtrmm(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 0.0, A, lda, got, ldb)
    assert np.all(got.reshape(n, ldb)[:, :m] == 0.0)


def test_device_in_place_and_out_of_place(handle):
    import torch
    for (layout, side, uplo, trans) in ((COL, LEFT, LOWER, NOTRANS), (ROW, RIGHT, UPPER, TRANS)):
        m, n = 200, 150
        A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=1, ldb_pad=1)  # odd ld: staging path
        ref = oracle_result(layout, side, uplo, trans, UNIT, m, n, -1.25, A, lda, B, ldb)
        dA, dB = torch_dev(A), torch_dev(B)
        handle.dtrmm_device(layout, side, uplo, trans, UNIT, m, n, -1.25, dA, lda, dB, ldb)
        handle.sync()
        check_close(dB.cpu().numpy(), ref, B, m if side == LEFT else n)
        dB2 = torch_dev(B)
        dC = torch.full_like(dB2, -7.0)
        handle.dtrmm_device_oop(layout, side, uplo, trans, UNIT, m, n, -1.25, dA, lda, dB2, ldb, dC, ldb)
        handle.sync()
        check_close(dC.cpu().numpy(), ref, B, m if side == LEFT else n)
        assert np.array_equal(dB2.cpu().numpy(), B)


def test_cblas_drop_in(handle):
    import ctypes as C
    m, n = 90, 45
    A, lda, B, ldb = make_problem(ROW, LEFT, LOWER, m, n)
    ref = oracle_result(ROW, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, B, ldb)
    got = B.copy()
    u.lib().cblas_dtrmm(ROW, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A.ctypes.data, lda, got.ctypes.data, ldb)
    assert u.lib().uvatrmm_last_status() == 0
    check_close(got, ref, B, m)


def test_reference_call_site_submatrix_view(handle):
    """The reference calls dtrmm on a sub-matrix view: A + n + (b+1), lda = n
    (UVaTRMM/src/mm_triangular.c:374-387)."""
    n, b, h, w = 96, 30, 41, 24
    Afull = orc.gen_consecutive(n, 0, n, 0, n, True)
    Bl = orc.gen_consecutive(n, 0, n, 0, w, False)
    tri = h - 1
    Aview = Afull.ravel()[(b + 1) * n + (b + 1):]
    ref = Bl.ravel().copy()
    orc.blas_dtrmm(ROW, LEFT, LOWER, NOTRANS, NONUNIT, tri, w, 1.0, Aview, n, ref[(b + 1) * w:], w)
    got = Bl.ravel().copy()
    sub = got[(b + 1) * w:]
    handle.dtrmm(ROW, LEFT, LOWER, NOTRANS, NONUNIT, tri, w, 1.0, Aview, n, sub, w)
    got[(b + 1) * w:] = sub
    assert rel_fro(got, ref) <= 8 * tri * EPS


def test_generators_bit_identical_to_oracle(handle):
    import torch
    for (rows, cols, spread, tri) in ((33, 17, 0, None), (64, 80, 20, None), (50, 50, 0, "U")):
        d = torch.empty(rows * cols, dtype=torch.float64, device="cuda")
        handle.gen_uniform(5, 3, rows, cols, d, cols, 1, tri=tri, fill=-2.0, spread=spread)
        handle.sync()
        ref = orc.fill_wide(5, 3, rows, cols, spread=spread, tri=tri, fill=-2.0) if spread else \
            orc.fill_uniform(5, 3, rows, cols, tri=tri, fill=-2.0)
        assert np.array_equal(d.cpu().numpy().reshape(rows, cols), ref)
        dc = torch.empty(rows * cols, dtype=torch.float64, device="cuda")  # column-major storage
        handle.gen_uniform(5, 3, rows, cols, dc, 1, rows, tri=tri, fill=-2.0, spread=spread)
        handle.sync()
        assert np.array_equal(dc.cpu().numpy().reshape(cols, rows).T, ref)
    for n in (8, 13, 300):
        d = torch.empty(n * n, dtype=torch.float64, device="cuda")
        handle.gen_consecutive(n, True, d)
        handle.sync()
        assert np.array_equal(d.cpu().numpy().reshape(n, n), orc.gen_consecutive(n, 0, n, 0, n, True))


@pytest.mark.parametrize("n", [8, 17, 64, 100, 512, 1000, 2048])
def test_product_norms_match_reference(handle, n):
    import torch
    norms = json.load(open(os.path.join(GOLD, "norms.json")))["norms"][str(n)]
    dA = torch.empty(n * n, dtype=torch.float64, device="cuda")
    dB = torch.empty_like(dA)
    dC = torch.empty_like(dA)
    handle.gen_consecutive(n, True, dA)
    handle.gen_consecutive(n, False, dB)
    A = orc.gen_consecutive(n, 0, n, 0, n, True)
    B = orc.gen_consecutive(n, 0, n, 0, n, False)
    ref = orc.uvatrmm_product(n, min(4, n), True, A, B)
    for sched, sname in ((u.SCHED_REG, "reg"), (u.SCHED_BALANCED, "balanced")):
        for shape, shname in ((u.SHAPE_BOXES, "boxes"), (u.SHAPE_TRAPEZOID, "trapezoid")):
            handle.product(n, sched, shape, dA, dB, dC)
            norm = handle.inf_norm(n, n, dC, n)
            assert "%.3f" % norm == norms[f"{sname}/{shname}"]
            assert rel_fro(dC.cpu().numpy().reshape(n, n), ref) <= 8 * n * EPS


def test_cli_matches_reference(handle, tmp_path):
    from uvatrmm_gb300 import build
    norms = json.load(open(os.path.join(GOLD, "norms.json")))["norms"]
    for n in ("64", "1000"):
        for mp in ("reg", "balanced"):
            for shape in ("boxes", "trapezoid"):
                r = subprocess.run([build.CLI, n, mp, shape], capture_output=True, text=True, cwd=tmp_path)
                assert r.returncode == 0, r.stderr
                lines = r.stdout.split("\n")
                assert lines[0] == "" and lines[1].startswith("Total t: ") and lines[2] == "Total mpis: 1"
                assert lines[3].startswith("Mult t: ") and lines[4] == ""
                assert lines[5] == "Norm: " + norms[n][f"{mp}/{shape}"]
                assert (tmp_path / "norm_ff.txt").read_text() == norms[n][f"{mp}/{shape}"]


@pytest.mark.parametrize("side,uplo,trans", [(LEFT, LOWER, NOTRANS), (LEFT, UPPER, TRANS), (RIGHT, LOWER, TRANS)])
def test_large_sampled_columns(handle, side, uplo, trans):
    """m = n = 4096 on the device; sampled columns (side Left) or rows (side
    Right) of the result checked against OpenBLAS on the same inputs."""
    import torch
    m = n = 4096
    dA = torch.empty(m * m, dtype=torch.float64, device="cuda")
    dB = torch.empty(m * n, dtype=torch.float64, device="cuda")
    handle.gen_uniform(1, 0, m, m, dA, 1, m)   # column-major, full (other triangle unreferenced)
    handle.gen_uniform(1, 1, m, n, dB, 1, m)
    dC = torch.empty_like(dB)
    handle.dtrmm_device_oop(COL, side, uplo, trans, NONUNIT, m, n, 1.0, dA, m, dB, m, dC, m)
    handle.sync()
    A = dA.cpu().numpy()
    B = dB.cpu().numpy().reshape(n, m).T
    C = dC.cpu().numpy().reshape(n, m).T
    sel = np.random.default_rng(0).choice(n, 8, replace=False)
    if side == LEFT:
        Bs = np.asfortranarray(B[:, sel]).ravel(order="F").copy()
        orc.blas_dtrmm(COL, side, uplo, trans, NONUNIT, m, 8, 1.0, A, m, Bs, m)
        ref, got = Bs.reshape(8, m).T, C[:, sel]
    else:
        Bs = np.asfortranarray(B[sel, :]).ravel(order="F").copy()
        orc.blas_dtrmm(COL, side, uplo, trans, NONUNIT, 8, n, 1.0, A, m, Bs, 8)
        ref, got = Bs.reshape(n, 8).T, C[sel, :]
    assert rel_fro(got, ref) <= 8 * m * EPS


@pytest.mark.parametrize("schedule,shape", [(u.SCHED_BALANCED, u.SHAPE_BOXES), (u.SCHED_REG, u.SHAPE_TRAPEZOID),
                                            (u.SCHED_DYNAMIC, u.SHAPE_TRAPEZOID)])
def test_skinny_16384x256_sampled_columns(handle, schedule, shape):
    """The skinny case of the plain-path configuration (m = 16384, n = 256,
    uplo U) under the reference's balanced / reg row mappings and both message
    shapes, the mapped product of UVaTRMM/src/mm_triangular.c:88-99,319-410;
    eight sampled columns against OpenBLAS cblas_dtrmm."""
    import torch
    m, n = 16384, 256
    dA = torch.empty(m * m, dtype=torch.float64, device="cuda")
    dB = torch.empty(m * n, dtype=torch.float64, device="cuda")
    handle.gen_uniform(1, 0, m, m, dA, 1, m, tri="U", fill=float("nan"))  # NaN in the unreferenced triangle
    handle.gen_uniform(1, 1, m, n, dB, 1, m)
    dC = torch.empty_like(dB)
    handle.set_option("schedule", schedule)
    handle.set_option("shape", shape)
    try:
        handle.dtrmm_device_oop(COL, LEFT, UPPER, NOTRANS, NONUNIT, m, n, 1.0, dA, m, dB, m, dC, m)
        handle.sync()
    finally:
        handle.set_option("schedule", u.SCHED_DYNAMIC)
        handle.set_option("shape", u.SHAPE_TRAPEZOID)
    A = dA.cpu().numpy()
    sel = [0, 1, 77, 128, 129, 200, 254, 255]
    Bs = np.concatenate([dB[j * m:(j + 1) * m].cpu().numpy() for j in sel])
    orc.blas_dtrmm(COL, LEFT, UPPER, NOTRANS, NONUNIT, m, len(sel), 1.0, A, m, Bs, m)
    got = np.concatenate([dC[j * m:(j + 1) * m].cpu().numpy() for j in sel])
    assert rel_fro(got, Bs) <= 8 * m * EPS


def test_wait_expiry_reports_etimeout_and_the_handle_recovers(handle):
    """The kernel's bounded waits: with the test option set, the consumers wait
    on a barrier that nothing completes, give up after the set number of
    polls, record the timeout flag and return (the producer drains its copies
    in flight first).  The host reads UVATRMM_ETIMEOUT at the next sync; the
    same handle then computes the next call correctly."""
    import torch
    h = u.Handle()
    try:
        m, n = 1024, 512
        A, lda, B, ldb = make_problem(COL, LEFT, LOWER, m, n, seed=5)
        dA = torch_dev(A)
        ref = oracle_result(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, B, ldb)
        for engine in (u.ENGINE_DFMA, u.ENGINE_DMMA):
            h.set_option("engine", engine)
            h.set_option("wait_expiry_test", 1000)
            dB = torch_dev(B.copy())
            h.dtrmm_device(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, dA, lda, dB, ldb)
            with pytest.raises(u.UvatrmmError) as ei:
                h.sync()
            assert ei.value.status == u.ETIMEOUT
            h.set_option("wait_expiry_test", 0)
            dB = torch_dev(B.copy())
            h.dtrmm_device(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, dA, lda, dB, ldb)
            h.sync()
            check_close(dB.cpu().numpy(), ref, B, m)
    finally:
        h.close()


def test_allocation_failure_is_reported_and_the_next_calls_run(handle):
    """An allocation the device cannot hold fails with UVATRMM_ENOMEM, both
    for the library's allocator and for a server whose HBM budget exceeds the
    device; the failure leaves nothing behind, so the next calls on the same
    thread (a TRMM and its kernel launch) still run and are correct."""
    import ctypes as C

    import torch
    p = C.c_void_p()
    assert u.lib().uvatrmm_device_alloc(1 << 50, C.byref(p)) == u.ENOMEM
    assert b"cudaMalloc" in u.lib().uvatrmm_last_error()
    with pytest.raises(u.UvatrmmError) as ei:
        u.Server(handle, hbm_budget_bytes=1 << 50)
    assert ei.value.status == u.ENOMEM
    m, n = 200, 150
    A, lda, B, ldb = make_problem(COL, LEFT, UPPER, m, n, seed=9)
    ref = oracle_result(COL, LEFT, UPPER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, B, ldb)
    dA, dB = torch_dev(A), torch_dev(B.copy())
    handle.dtrmm_device(COL, LEFT, UPPER, NOTRANS, NONUNIT, m, n, 1.0, dA, lda, dB, ldb)
    handle.sync()
    check_close(dB.cpu().numpy(), ref, B, m)
