"""Grouped batches (one CUDA graph of grouped persistent launches) against
the single-problem entry points: bitwise identical results, because every
output element accumulates in the same order (FP64 tier) or exactly (Ozaki
tier) however the problems are grouped.  Every grouped result is also
checked against the oracle: FP64-tier results against the naive FP64 loops
at 8 k eps, Ozaki-tier results against the double-double oracle at 1e-14
(cblas_dtrmm semantics, as the reference calls it at
UVaTRMM/src/mm_triangular.c:374-387)."""
import os

import numpy as np
import pytest

import uvatrmm_gb300 as u
from tests.helpers import (COL, LEFT, LOWER, NONUNIT, NOTRANS, RIGHT, ROW, TRANS, UNIT, UPPER, assert_matches_oracle,
                           make_problem)

pytestmark = pytest.mark.gpu


def mixed_problems(count, seed, max_dim=600, min_dim=8):
    import torch
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        layout = [COL, ROW][rng.integers(2)]
        side = [LEFT, RIGHT][rng.integers(2)]
        uplo = [LOWER, UPPER][rng.integers(2)]
        trans = [NOTRANS, TRANS][rng.integers(2)]
        diag = [NONUNIT, UNIT][rng.integers(2)]
        m = int(np.exp(rng.uniform(np.log(min_dim), np.log(max_dim))))
        n = int(np.exp(rng.uniform(np.log(max(4, min_dim // 2)), np.log(max_dim))))
        tier = u.TIER_OZAKI if rng.random() < 0.3 else u.TIER_FP64
        A, lda, B, ldb = make_problem(layout, side, uplo, m, n, lda_pad=int(rng.integers(2)),
                                      ldb_pad=int(rng.integers(3)), seed=seed * 1000 + i)
        out.append(dict(layout=layout, side=side, uplo=uplo, transa=trans, diag=diag, m=m, n=n,
                        alpha=float(rng.choice([1.0, -0.5, 2.0])), A=torch.from_numpy(A).cuda(), lda=lda,
                        B=torch.from_numpy(B).cuda(), ldb=ldb, tier=tier, moduli=0, B0=B))
    return out


def single_reference(handle, p):
    import torch
    B = torch.from_numpy(p["B0"].copy()).cuda()
    args = (p["layout"], p["side"], p["uplo"], p["transa"], p["diag"], p["m"], p["n"], p["alpha"], p["A"],
            p["lda"], B, p["ldb"])
    if p["tier"] == u.TIER_OZAKI:
        handle.ozaki_device(*args)
    else:
        handle.dtrmm_device(*args)
    handle.sync()
    return B.cpu().numpy()


def test_group_matches_single_calls_bitwise(handle):
    import torch
    probs = mixed_problems(48, seed=3)
    probs.append(dict(probs[0], m=0))  # empty problem
    z = dict(probs[1])
    z["B"] = torch.from_numpy(z["B0"].copy()).cuda()
    z["alpha"] = 0.0
    probs.append(z)
    refs = [single_reference(handle, p) for p in probs[:-2]]
    g = u.Group(handle, probs)
    st = g.stats()
    assert st["fp64_tiles"] > 0 and st["ozaki_tiles"] > 0 and st["ozaki_waves"] >= 1
    for rep in range(2):  # the graph replays: reset the in-place buffers each run
        for p in probs:
            p["B"].copy_(torch.from_numpy(p["B0"]))
        g.run()
        handle.sync()
        for p, r in zip(probs, refs):
            got = p["B"].cpu().numpy()
            assert np.array_equal(got, r), (rep, p["tier"], p["m"], p["n"])
            if rep == 0:
                assert_matches_oracle(p, got, "grouped")
        zb = probs[-1]["B"].cpu().numpy()
        m, n, ldb, layout = z["m"], z["n"], z["ldb"], z["layout"]
        rows, cols = (m, n) if layout == COL else (n, m)
        assert np.all(zb.reshape(cols, ldb)[:, :rows] == 0.0)
    g.close()


def test_group_ozaki_waves_under_a_small_budget(handle):
    import torch
    # each problem needs > 64 MiB of residue planes at these sizes
    probs = [dict(p, tier=u.TIER_OZAKI) for p in mixed_problems(5, seed=5, max_dim=1100, min_dim=800)]
    refs = [single_reference(handle, p) for p in probs]
    u.check(u.lib().uvatrmm_set_option(handle.h, 5, 64))  # 64 MiB of Ozaki scratch per wave
    try:
        g = u.Group(handle, probs)
    finally:
        u.check(u.lib().uvatrmm_set_option(handle.h, 5, 49152))
    assert g.stats()["ozaki_waves"] > 1
    g.run()
    handle.sync()
    for p, r in zip(probs, refs):
        got = p["B"].cpu().numpy()
        assert np.array_equal(got, r)
        assert_matches_oracle(p, got, "grouped, several waves")
    g.close()


def test_autotuner_choices_and_cache(handle):
    for tier, allowed in ((u.TIER_FP64, (64, 128)), (u.TIER_OZAKI, (1, 2, 3))):
        for side in (LEFT, RIGHT):
            c = u.tune(handle, tier, side, 300, 700)
            assert c in allowed
            assert u.tune(handle, tier, side, 290, 600) == c  # same bucket: cached
    path = os.environ["UVATRMM_TUNE_CACHE"]
    lines = open(path).read().split("\n")
    assert any(line.startswith("0 0 9 10 ") for line in lines)


def test_group_rejects_bad_problems(handle):
    import torch
    d = torch.zeros(64, dtype=torch.float64, device="cuda")
    bad = dict(layout=COL, side=LEFT, uplo=LOWER, transa=NOTRANS, diag=NONUNIT, m=8, n=8, alpha=1.0, A=d, lda=4,
               B=d, ldb=8, tier=u.TIER_FP64, moduli=0)
    with pytest.raises(u.UvatrmmError, match="problem 0: parameter 10"):
        u.Group(handle, [bad])
    with pytest.raises(u.UvatrmmError, match="unknown tier"):
        u.Group(handle, [dict(bad, lda=8, tier=7)])
