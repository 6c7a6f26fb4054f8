"""uvatrmm_dtrmm_device_noalloc against uvatrmm_dtrmm_device.

The no-allocation entry point serves callers that cannot allocate device
memory (all of it belongs to their own pool, or their loop must not take the
synchronisation of cudaMalloc/cudaFree): its scratch is a fixed device array.
This file is collected last so that a run stopping at the first failure has
already run every other test; it passes alone in a fresh process too.
"""
import numpy as np
import pytest

import uvatrmm_gb300 as u
from tests.helpers import (COL, EPS, LEFT, LOWER, NONUNIT, NOTRANS, RIGHT, ROW, TRANS, UNIT, UPPER,
                           assert_matches_oracle, make_problem, rel_fro)

pytestmark = pytest.mark.gpu

CASES = [  # layout, side, uplo, trans, diag, m, n, lda_pad, ldb_pad
    (COL, LEFT, LOWER, NOTRANS, NONUNIT, 300, 200, 0, 0),
    (ROW, RIGHT, UPPER, TRANS, UNIT, 130, 257, 1, 3),   # odd lda: A staged in the fixed array
    (COL, RIGHT, LOWER, TRANS, NONUNIT, 64, 1000, 0, 2),
]


def test_noalloc_matches_allocating_entry_point(handle):
    import torch
    L = u.lib()
    for call in range(2):  # two calls in a row share (and reuse) the fixed scratch
        for (layout, side, uplo, trans, diag, m, n, lp, bp) in CASES:
            A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=lp, ldb_pad=bp, seed=11 + call)
            dA = torch.from_numpy(A).cuda()
            ref = torch.from_numpy(B.copy()).cuda()
            handle.dtrmm_device(layout, side, uplo, trans, diag, m, n, -1.5, dA, lda, ref, ldb)
            handle.sync()
            got = torch.from_numpy(B.copy()).cuda()
            rc = L.uvatrmm_dtrmm_device_noalloc(layout, side, uplo, trans, diag, m, n, -1.5, dA.data_ptr(), lda,
                                                got.data_ptr(), ldb, None)
            assert rc == 0, L.uvatrmm_last_error()
            r, g = ref.cpu().numpy(), got.cpu().numpy()
            pad = B == -7.0
            assert np.array_equal(g[pad], B[pad])
            k = m if side == LEFT else n
            assert rel_fro(g[~pad], r[~pad]) <= 8 * k * EPS
            # and against the oracle (naive FP64 cblas_dtrmm loops), same tolerance
            assert_matches_oracle(dict(layout=layout, side=side, uplo=uplo, transa=trans, diag=diag, m=m, n=n,
                                       alpha=-1.5, A=A, lda=lda, B0=B, ldb=ldb, tier=u.TIER_FP64), g, "no-alloc")


def test_noalloc_rejects_problems_beyond_its_scratch(handle):
    import torch
    L = u.lib()
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    m = n = 4096  # staged B alone is 128 MiB
    rc = L.uvatrmm_dtrmm_device_noalloc(COL, LEFT, LOWER, NOTRANS, NONUNIT, m, n, 1.0, d.data_ptr(), m,
                                        d.data_ptr(), m, None)
    assert rc == u.EINVAL
    assert b"no-allocation" in L.uvatrmm_last_error()
    # sizes whose scratch products would overflow 64-bit arithmetic are refused
    # too, before any device memory is touched
    for (mm, nn) in ((1 << 40, 1 << 40), (16, 1 << 60), (1 << 61, 4)):
        rc = L.uvatrmm_dtrmm_device_noalloc(COL, LEFT, LOWER, NOTRANS, NONUNIT, mm, nn, 1.0, d.data_ptr(), mm,
                                            d.data_ptr(), mm, None)
        assert rc == u.EINVAL, (mm, nn)
        assert b"no-allocation" in L.uvatrmm_last_error()
