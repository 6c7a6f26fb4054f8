"""uvatrmm_host_alloc / uvatrmm_host_free: page-locked, huge-page-aligned host
memory for the operands of the host entry points."""
import ctypes as C
import gc

import numpy as np
import pytest

import uvatrmm_gb300 as u
from oracle import oracle as orc
from tests.helpers import COL, LEFT, LOWER, NONUNIT, NOTRANS, RIGHT, TRANS, UPPER, rel_fro


def _gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_host_free_rejects_foreign_pointers(built):
    L = u.lib()
    assert L.uvatrmm_host_free(None) == 0
    x = np.zeros(16)
    assert L.uvatrmm_host_free(x.ctypes.data) == u.EINVAL
    assert "uvatrmm_host_alloc" in L.uvatrmm_last_error().decode()


def test_host_alloc_needs_a_device(built):
    """Without a CUDA device the allocation fails loudly (no unpinned fallback)."""
    if _gpu():
        pytest.skip("a CUDA device is present")
    p = C.c_void_p()
    rc = u.lib().uvatrmm_host_alloc(1 << 20, C.byref(p))
    assert rc != 0 and not p.value


def _hpage():
    try:
        return int(open("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size").read())
    except OSError:
        return 2 << 20


@pytest.mark.gpu
def test_host_alloc_aligned_zeroed_and_freed(handle):
    a = u.host_empty(1000)
    assert a.ctypes.data % _hpage() == 0
    assert not a.any()
    a[:] = 3.0
    assert a.sum() == 3000.0
    p = a.ctypes.data
    del a
    gc.collect()
    # freed by the finaliser: a second free of the same pointer is refused
    assert u.lib().uvatrmm_host_free(p) == u.EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("side,uplo,trans", [(LEFT, LOWER, NOTRANS), (RIGHT, UPPER, TRANS)])
def test_dtrmm_on_host_alloc_buffers(handle, side, uplo, trans):
    """uvatrmm_dtrmm on operands in uvatrmm_host_alloc memory equals OpenBLAS."""
    m, n = 300, 170
    ka = m if side == LEFT else n
    rng = np.random.default_rng(11)
    A = u.host_empty(ka * ka)
    B = u.host_empty(m * n)
    A[:] = rng.uniform(-1, 1, ka * ka)
    B[:] = rng.uniform(-1, 1, m * n)
    ref = np.array(B)
    orc.blas_dtrmm(COL, side, uplo, trans, NONUNIT, m, n, 1.5, np.array(A), ka, ref, m)
    handle.dtrmm(COL, side, uplo, trans, NONUNIT, m, n, 1.5, A, ka, B, m)
    assert rel_fro(B, ref) <= 8 * ka * np.finfo(np.float64).eps


@pytest.fixture
def small_stage_handle(built):
    if not _gpu():
        pytest.skip("no CUDA device")
    h = u.Handle()
    h.set_option("host_stage_kb", 64)  # many staging chunks on small operands
    return h


@pytest.mark.gpu
@pytest.mark.parametrize("pad", [0, 13])
def test_staged_host_copies_dtrmm(small_stage_handle, pad):
    """malloc'd operands go through the staging pipeline (64 KiB chunks here):
    flat (pad 0) and strided (pad 13) copies in both directions."""
    m, n = 600, 410
    lda, ldb = m + pad, m + pad
    rng = np.random.default_rng(5)
    A = rng.uniform(-1, 1, lda * m)
    B = rng.uniform(-1, 1, ldb * n)
    ref = B.copy()
    orc.blas_dtrmm(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, -0.5, A, lda, ref, ldb)
    got = B.copy()
    small_stage_handle.dtrmm(COL, LEFT, UPPER, TRANS, NONUNIT, m, n, -0.5, A, lda, got, ldb)
    G, R = got.reshape(n, ldb)[:, :m], ref.reshape(n, ldb)[:, :m]
    assert rel_fro(G, R) <= 8 * m * np.finfo(np.float64).eps
    if pad:  # rows beyond m untouched
        assert np.array_equal(got.reshape(n, ldb)[:, m:], B.reshape(n, ldb)[:, m:])


@pytest.mark.gpu
def test_staged_host_copies_dgemm_and_ozaki(small_stage_handle):
    m, n, k = 520, 300, 450
    rng = np.random.default_rng(6)
    A = rng.uniform(-1, 1, m * k)
    B = rng.uniform(-1, 1, k * n)
    C = rng.uniform(-1, 1, m * n)
    got = C.copy()
    small_stage_handle.dgemm(COL, NOTRANS, NOTRANS, m, n, k, 1.25, A, m, B, k, 0.5, got, m)
    ref = 1.25 * (A.reshape(k, m).T @ B.reshape(n, k).T) + 0.5 * C.reshape(n, m).T
    assert rel_fro(got.reshape(n, m).T, ref) <= 8 * k * np.finfo(np.float64).eps
    T = rng.uniform(-1, 1, m * m)
    Bo = rng.uniform(-1, 1, m * n)
    refo = Bo.copy()
    orc.blas_dtrmm(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, T, m, refo, m)
    goto = Bo.copy()
    small_stage_handle.ozaki(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, T, m, goto, m)
    assert rel_fro(goto, refo) <= 1e-14


@pytest.mark.gpu
def test_dtrmm_async_two_handles(handle):
    """uvatrmm_dtrmm_async on two handles: both results equal OpenBLAS after sync."""
    h2 = u.Handle()
    rng = np.random.default_rng(8)
    cases = [(LEFT, LOWER, NOTRANS, 700, 333), (RIGHT, UPPER, TRANS, 290, 512)]
    hs, bufs, refs = [handle, h2], [], []
    for (side, uplo, trans, m, n), hh in zip(cases, hs):
        ka = m if side == LEFT else n
        A = u.host_empty(ka * ka)
        B = u.host_empty(m * n)
        A[:] = rng.uniform(-1, 1, ka * ka)
        B[:] = rng.uniform(-1, 1, m * n)
        ref = np.array(B)
        orc.blas_dtrmm(COL, side, uplo, trans, NONUNIT, m, n, 0.75, np.array(A), ka, ref, m)
        hh.dtrmm_async(COL, side, uplo, trans, NONUNIT, m, n, 0.75, A, ka, B, m)
        bufs.append((A, B, ka))
        refs.append(ref)
    for hh in hs:
        hh.sync()
    for (A, B, ka), ref in zip(bufs, refs):
        assert rel_fro(B, ref) <= 8 * ka * np.finfo(np.float64).eps


@pytest.mark.gpu
def test_dtrmm_async_requires_host_alloc_memory(handle):
    A = np.zeros(64 * 64)
    B = np.zeros(64 * 8)
    with pytest.raises(u.UvatrmmError) as ei:
        handle.dtrmm_async(COL, LEFT, LOWER, NOTRANS, NONUNIT, 64, 8, 1.0, A, 64, B, 64)
    assert ei.value.status == u.EINVAL
