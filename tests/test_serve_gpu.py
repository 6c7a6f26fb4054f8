"""The request loop with continuous batching: results are bitwise the same
served alone and served in a mix of concurrently active requests, and every
served result is within its tier's tolerance of the oracle (naive FP64 loops
at 8 k eps; double-double at 1e-14 for the Ozaki tier); admission respects
the HBM budget; refusal and cancellation."""
import threading
import time

import numpy as np
import pytest

import uvatrmm_gb300 as u
from tests.helpers import COL, LEFT, LOWER, NONUNIT, NOTRANS, UPPER, assert_matches_oracle, make_problem
from tests.test_group_gpu import mixed_problems

pytestmark = pytest.mark.gpu


def reset(p):
    import torch
    p["B"].copy_(torch.from_numpy(p["B0"]))


def test_each_result_is_the_same_alone_and_in_the_mix(handle):
    probs = mixed_problems(36, seed=21, max_dim=900)
    srv = u.Server(handle, hbm_budget_bytes=8 << 30)
    try:
        alone = []
        for p in probs:  # one request in the server at a time
            reset(p)
            rid = srv.submit(p)
            assert srv.wait(rid) == 0
            alone.append(p["B"].cpu().numpy())
        for p in probs:
            reset(p)
        ids = []
        for k, p in enumerate(probs):  # all at once: they share every tick
            ids.append(srv.submit(p))
            if k % 7 == 3:
                time.sleep(0.002)  # some arrive while others run
        for rid in ids:
            assert srv.wait(rid) == 0
        for p, a in zip(probs, alone):
            got = p["B"].cpu().numpy()
            assert np.array_equal(got, a)
            assert_matches_oracle(p, got, "served in the mix")
        st = srv.stats()
        assert st["completed"] == 2 * len(probs) and st["failed"] == 0
        assert st["p99_ms"] >= st["p50_ms"] > 0
    finally:
        srv.close()
    # and the same as the direct entry points
    for p, a in zip(probs, alone):
        reset(p)
        args = (p["layout"], p["side"], p["uplo"], p["transa"], p["diag"], p["m"], p["n"], p["alpha"], p["A"],
                p["lda"], p["B"], p["ldb"])
        (handle.ozaki_device if p["tier"] == u.TIER_OZAKI else handle.dtrmm_device)(*args)
        handle.sync()
        assert np.array_equal(p["B"].cpu().numpy(), a)


def test_admission_under_a_small_budget(handle):
    probs = mixed_problems(16, seed=22, max_dim=700, min_dim=300)
    budget = 96 << 20
    srv = u.Server(handle, hbm_budget_bytes=budget, max_active=4)
    try:
        ids = [srv.submit(p) for p in probs]
        for rid in ids:
            assert srv.wait(rid, 60.0) == 0
        st = srv.stats()
        assert st["completed"] == len(probs)
        assert 0 < st["peak_bytes"] <= budget
    finally:
        srv.close()


def test_host_operands_round_trip(handle):
    srv = u.Server(handle, hbm_budget_bytes=1 << 30)
    try:
        for tier in (u.TIER_FP64, u.TIER_OZAKI):
            m, n = 150, 90
            A, lda, B, ldb = make_problem(COL, LEFT, UPPER, m, n)
            ref = B.copy()
            if tier == u.TIER_OZAKI:
                handle.ozaki(COL, LEFT, UPPER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, ref, ldb)
            else:
                handle.dtrmm(COL, LEFT, UPPER, NOTRANS, NONUNIT, m, n, 1.0, A, lda, ref, ldb)
            got = B.copy()
            p = dict(layout=COL, side=LEFT, uplo=UPPER, transa=NOTRANS, diag=NONUNIT, m=m, n=n, alpha=1.0,
                     A=A, lda=lda, B=got, ldb=ldb, tier=tier, B0=B)
            rid = srv.submit(p, on_device=False)
            assert srv.wait(rid) == 0
            assert np.array_equal(got, ref)
            assert_matches_oracle(p, got, "served from host operands")
    finally:
        srv.close()


def test_refusal_and_cancellation(handle):
    import torch
    srv = u.Server(handle, hbm_budget_bytes=64 << 20, max_active=1)
    try:
        big = torch.zeros(4096 * 4096, dtype=torch.float64, device="cuda")
        p = dict(layout=COL, side=LEFT, uplo=LOWER, transa=NOTRANS, diag=NONUNIT, m=4096, n=4096, alpha=1.0,
                 A=big, lda=4096, B=big, ldb=4096, tier=u.TIER_FP64)
        with pytest.raises(u.UvatrmmError, match="HBM budget"):
            srv.submit(p)
        # a queue of requests behind a single slot held by a ~12 ms FP64
        # request: cancel the last one before it is admitted
        n0 = 2500
        a0 = torch.rand(n0 * n0, dtype=torch.float64, device="cuda")
        b0 = torch.rand(n0 * n0, dtype=torch.float64, device="cuda")
        first = dict(p, m=n0, n=n0, A=a0, lda=n0, B=b0, ldb=n0)
        small = mixed_problems(5, seed=23, max_dim=500, min_dim=400)
        ids = [srv.submit(first)] + [srv.submit(q) for q in small]
        assert srv.cancel(ids[-1]) == 0
        assert srv.wait(ids[-1]) == u.EINVAL  # cancelled
        for rid in ids[:-1]:
            assert srv.wait(rid) == 0
        assert srv.stats()["cancelled"] == 1 and srv.stats()["refused"] == 1
    finally:
        srv.close()


def test_submitters_on_several_threads(handle):
    probs = mixed_problems(24, seed=24, max_dim=400)
    srv = u.Server(handle, hbm_budget_bytes=2 << 30)
    errors = []

    def client(chunk):
        try:
            ids = [srv.submit(p) for p in chunk]
            for rid in ids:
                if srv.wait(rid) != 0:
                    errors.append(rid)
        except Exception as e:  # noqa: BLE001
            errors.append(e)

    try:
        threads = [threading.Thread(target=client, args=(probs[k::3],)) for k in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors
        assert srv.stats()["completed"] == len(probs)
    finally:
        srv.close()


def test_latency_of_each_request(handle):
    """uvatrmm_server_latency: every completed request has a submit-to-result
    latency within the server's own bounds; an unknown id is refused."""
    import ctypes as C
    probs = mixed_problems(10, seed=25, max_dim=300)
    srv = u.Server(handle, hbm_budget_bytes=1 << 30)
    try:
        ids = [srv.submit(p) for p in probs]
        for rid in ids:
            assert srv.wait(rid) == 0
        lats = [srv.latency_ms(rid) for rid in ids]
        st = srv.stats()
        assert all(x is not None and 0.0 < x <= st["max_ms"] + 1e-9 for x in lats)
        assert abs(max(lats) - st["max_ms"]) < 1e-6
        v = C.c_double()
        assert u.lib().uvatrmm_server_latency(srv.s, 10 ** 9, C.byref(v)) == u.EINVAL
    finally:
        srv.close()
