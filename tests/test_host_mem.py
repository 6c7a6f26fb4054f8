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
