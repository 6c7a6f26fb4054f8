"""GEMM, the product loop's stage and the block-cyclic adapters on the GPU,
through the C ABI, against the oracle.

Tolerance: relative Frobenius error <= 8 * k * eps against OpenBLAS (k = inner
dimension); bitwise where every product and partial sum is an exactly
representable integer (the ScaLAPACK sample fills, consecutive values).
"""
import ctypes as C
import itertools
import json
import os

import numpy as np
import pytest

import uvatrmm_gb300 as u
from oracle import oracle as orc
from tests.helpers import COL, EPS, NOTRANS, ROW, TRANS, rel_fro

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x).ravel()).cuda()


def gemm_operands(layout, ta, tb, m, n, k, pad, seed):
    """Flat operand buffers (padded leading dimensions, -7 sentinels in the padding of C)."""
    rng = np.random.default_rng(seed)
    col = layout == COL
    ar, ac = (m, k) if ta == NOTRANS else (k, m)
    br, bc = (k, n) if tb == NOTRANS else (n, k)
    # Storage dims: column-major rows x cols, row-major the transpose.
    sa = (ar, ac) if col else (ac, ar)
    sb = (br, bc) if col else (bc, br)
    sc = (m, n) if col else (n, m)
    lda, ldb, ldc = sa[0] + pad, sb[0] + pad, sc[0] + pad
    A = rng.uniform(-1, 1, size=max(lda * sa[1], 1))
    B = rng.uniform(-1, 1, size=max(ldb * sb[1], 1))
    Cm = np.full(max(ldc * sc[1], 1), -7.0)
    for j in range(sc[1]):
        Cm[j * ldc:j * ldc + sc[0]] = rng.uniform(-1, 1, size=sc[0])
    return A, max(lda, 1), B, max(ldb, 1), Cm, max(ldc, 1)


def ref_gemm(layout, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    out = Cm.copy()
    orc.blas_dgemm(layout, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, out, ldc)
    return out


@pytest.mark.parametrize("layout,ta,tb", list(itertools.product((COL, ROW), (NOTRANS, TRANS), (NOTRANS, TRANS))))
def test_dgemm_all_variants(handle, layout, ta, tb):
    for (m, n, k, pad) in ((37, 53, 129, 3), (130, 70, 64, 0), (1, 17, 5, 1)):
        for (alpha, beta) in ((1.0, 0.0), (0.5, 1.0), (-1.25, -0.5)):
            A, lda, B, ldb, Cm, ldc = gemm_operands(layout, ta, tb, m, n, k, pad, seed=m + n + k)
            ref = ref_gemm(layout, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc)
            got = Cm.copy()
            handle.dgemm(layout, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, got, ldc)
            pad_mask = Cm == -7.0
            assert np.array_equal(got[pad_mask], Cm[pad_mask]), "padding was written"
            assert rel_fro(got[~pad_mask], ref[~pad_mask]) <= 8 * k * EPS
            dC = dev(Cm)
            handle.dgemm_device(layout, ta, tb, m, n, k, alpha, dev(A), lda, dev(B), ldb, beta, dC, ldc)
            handle.sync()
            assert np.array_equal(dC.cpu().numpy(), got), "device and host entry points disagree"


@pytest.mark.parametrize("engine,tile", [(u.ENGINE_DMMA, 64), (u.ENGINE_DFMA, 128), (u.ENGINE_DMMA, 128)])
def test_dgemm_engines_and_tiles(handle, engine, tile):
    handle.set_option("engine", engine)
    handle.set_option("tile", tile)
    try:
        for (layout, ta, tb) in ((COL, NOTRANS, TRANS), (ROW, TRANS, NOTRANS)):
            m, n, k = 150, 97, 211
            A, lda, B, ldb, Cm, ldc = gemm_operands(layout, ta, tb, m, n, k, 1, seed=13)
            ref = ref_gemm(layout, ta, tb, m, n, k, 0.75, A, lda, B, ldb, -1.0, Cm, ldc)
            got = Cm.copy()
            handle.dgemm(layout, ta, tb, m, n, k, 0.75, A, lda, B, ldb, -1.0, got, ldc)
            mask = Cm == -7.0
            assert np.array_equal(got[mask], Cm[mask])
            assert rel_fro(got[~mask], ref[~mask]) <= 8 * k * EPS
    finally:
        handle.set_option("engine", u.ENGINE_DFMA)
        handle.set_option("tile", 0)


def test_dgemm_misaligned_device_operands(handle):
    import torch
    m, n, k = 67, 45, 99
    A, lda, B, ldb, Cm, ldc = gemm_operands(COL, NOTRANS, TRANS, m, n, k, 1, seed=5)
    ref = ref_gemm(COL, NOTRANS, TRANS, m, n, k, 2.0, A, lda, B, ldb, 1.0, Cm, ldc)
    # Every operand starts 8 bytes past a 16-byte boundary, with odd leading dimensions.
    bufs = [torch.zeros(x.size + 1, dtype=torch.float64, device="cuda") for x in (A, B, Cm)]
    for b, x in zip(bufs, (A, B, Cm)):
        b[1:] = torch.from_numpy(x).cuda()
    views = [b[1:] for b in bufs]
    assert all(v.data_ptr() % 16 == 8 for v in views)
    handle.dgemm_device(COL, NOTRANS, TRANS, m, n, k, 2.0, views[0], lda, views[1], ldb, 1.0, views[2], ldc)
    handle.sync()
    got = views[2].cpu().numpy()
    mask = Cm == -7.0
    assert np.array_equal(got[mask], Cm[mask])
    assert rel_fro(got[~mask], ref[~mask]) <= 8 * k * EPS


@pytest.mark.parametrize("m,n,k", [(0, 5, 3), (5, 0, 3), (4, 6, 0), (1, 1, 1), (65, 63, 1), (2, 3, 300)])
def test_dgemm_edge_sizes(handle, m, n, k):
    A, lda, B, ldb, Cm, ldc = gemm_operands(ROW, NOTRANS, NOTRANS, m, n, k, 2, seed=11)
    ref = ref_gemm(ROW, NOTRANS, NOTRANS, m, n, k, 1.5, A, lda, B, ldb, 0.25, Cm, ldc)
    got = Cm.copy()
    handle.dgemm(ROW, NOTRANS, NOTRANS, m, n, k, 1.5, A, lda, B, ldb, 0.25, got, ldc)
    assert rel_fro(got, ref) <= 8 * max(k, 1) * EPS


def test_dgemm_alpha_zero_scales_c_without_reading_ab(handle):
    m, n, k = 20, 30, 40
    A, lda, B, ldb, Cm, ldc = gemm_operands(COL, NOTRANS, NOTRANS, m, n, k, 0, seed=2)
    A[:] = np.nan
    B[:] = np.nan
    for beta, want in ((0.0, np.zeros_like(Cm)), (-2.0, -2.0 * Cm)):
        got = Cm.copy()
        handle.dgemm(COL, NOTRANS, NOTRANS, m, n, k, 0.0, A, lda, B, ldb, beta, got, ldc)
        assert np.array_equal(got, want)


def test_cblas_dgemm_drop_in(built, handle):
    L = u.lib()
    m, n, k = 33, 47, 61
    A, lda, B, ldb, Cm, ldc = gemm_operands(ROW, TRANS, NOTRANS, m, n, k, 0, seed=9)
    ref = ref_gemm(ROW, TRANS, NOTRANS, m, n, k, 0.5, A, lda, B, ldb, 2.0, Cm, ldc)
    got = Cm.copy()
    L.cblas_dgemm(ROW, TRANS, NOTRANS, m, n, k, 0.5, A.ctypes.data, lda, B.ctypes.data, ldb, 2.0,
                  got.ctypes.data, ldc)
    assert rel_fro(got, ref) <= 8 * k * EPS


def _stage_loop(handle, n, P, sched, dA, dBl, dCl, w):
    for s in range(P):
        b, h = u.map_rows(sched, n, P, s)
        if h:
            handle.stage(n, w, b, h, dA[b * n:], n, dBl, w, dCl, w)


@pytest.mark.parametrize("n,P", [(8, 1), (17, 3), (64, 4), (100, 7), (512, 4), (1000, 4), (2048, 8)])
def test_stage_loop_matches_reference_product(handle, n, P):
    """UVaTRMM/src/mm_triangular.c:319-403 driven stage by stage, rank by rank."""
    import torch
    A = orc.gen_consecutive(n, 0, n, 0, n, True)
    B = orc.gen_consecutive(n, 0, n, 0, n, False)
    norms = json.load(open(os.path.join(GOLD, "norms.json")))["norms"][str(n)]
    dA = dev(A)
    for sched, sname, balanced in ((u.SCHED_REG, "reg", False), (u.SCHED_BALANCED, "balanced", True)):
        ref = orc.uvatrmm_product(n, P, balanced, A, B)
        got = np.zeros((n, n))
        for r in range(P):  # rank r's column slice of B and C
            cb, w = u.map_rows(u.SCHED_REG, n, P, r)
            dBl = dev(B[:, cb:cb + w])
            dCl = torch.zeros(n * w, dtype=torch.float64, device="cuda")
            _stage_loop(handle, n, P, sched, dA, dBl, dCl, w)
            handle.sync()
            got[:, cb:cb + w] = dCl.cpu().numpy().reshape(n, w)
            assert np.array_equal(dBl.cpu().numpy().reshape(n, w), B[:, cb:cb + w]), "B was modified"
        assert rel_fro(got, ref) <= 8 * n * EPS
        if P == 4 and f"{sname}/trapezoid" in norms:
            assert "%.3f" % orc.inf_norm(got) == norms[f"{sname}/trapezoid"]


def test_stage_argument_errors(handle):
    import torch
    d = torch.zeros(64, dtype=torch.float64, device="cuda")
    for (n, w, b, h) in ((8, 4, 6, 3), (8, 4, 0, 0), (0, 4, 0, 1), (8, -1, 0, 2)):
        with pytest.raises(u.UvatrmmError):
            handle.stage(n, w, b, h, d, 8, d, 4, d, 4)


def _to_dev_locals(locals_):
    arrs = [dev(np.asfortranarray(x).ravel(order="F")) if x.size else None for x in locals_]
    import torch
    arrs = [a if a is not None else torch.zeros(1, dtype=torch.float64, device="cuda") for a in arrs]
    lld = [max(x.shape[0], 1) for x in locals_]
    return arrs, lld


def _from_dev_locals(arrs, like):
    return [a.cpu().numpy()[:x.size].reshape(x.shape, order="F") for a, x in zip(arrs, like)]


@pytest.mark.parametrize("n,nb,pr,pc", [(1000, 256, 2, 2), (333, 32, 3, 2), (10, 3, 2, 2), (5, 8, 1, 3), (64, 64, 1, 1)])
def test_scalapack_trmm_sample_through_block_cyclic_adapters(handle, n, nb, pr, pc):
    """ScaLAPACK/scalapack_sample_trmm.c: pdtrmm('L','L','N','N') on its own fill,
    as gather -> TRMM -> scatter."""
    import torch
    L = orc.sample_locals("trmm", n, nb, pr, pc)
    dA, lldA = _to_dev_locals(L["A"])
    dB, lldB = _to_dev_locals(L["B"])
    gA = torch.empty(n * n, dtype=torch.float64, device="cuda")
    gB = torch.empty_like(gA)
    handle.bc_gather(n, n, nb, nb, pr, pc, dA, lldA, gA, n)
    handle.bc_gather(n, n, nb, nb, pr, pc, dB, lldB, gB, n)
    GA = orc.bc_to_global(L["A"], n, n, nb, nb, pr, pc)
    GB = orc.bc_to_global(L["B"], n, n, nb, nb, pr, pc)
    assert np.array_equal(gA.cpu().numpy().reshape(n, n).T, GA)
    handle.dtrmm_device(COL, u.LEFT, u.LOWER, NOTRANS, u.NONUNIT, n, n, 1.0, gA, n, gB, n)
    handle.bc_scatter(n, n, nb, nb, pr, pc, gB, n, dB, lldB)
    ref = np.asfortranarray(GB).ravel(order="F").copy()
    orc.dtrmm_naive(COL, u.LEFT, u.LOWER, NOTRANS, u.NONUNIT, n, n, 1.0,
                    np.asfortranarray(GA).ravel(order="F").copy(), n, ref, n)
    want = orc.bc_from_global(ref.reshape(n, n, order="F"), nb, nb, pr, pc)
    for got, w in zip(_from_dev_locals(dB, L["B"]), want):
        assert np.array_equal(got, w)


@pytest.mark.parametrize("n,nb,pr,pc", [(1000, 256, 2, 2), (77, 16, 2, 3)])
def test_scalapack_gemm_sample_through_block_cyclic_adapters(handle, n, nb, pr, pc):
    """ScaLAPACK/scalapack_sample_gemm.c: pdgemm('N','N') with B = 2I gives C = 2A."""
    import torch
    L = orc.sample_locals("gemm", n, nb, pr, pc)
    dA, lld = _to_dev_locals(L["A"])
    dB, _ = _to_dev_locals(L["B"])
    dC, _ = _to_dev_locals(L["C"])
    g = [torch.empty(n * n, dtype=torch.float64, device="cuda") for _ in range(3)]
    handle.bc_gather(n, n, nb, nb, pr, pc, dA, lld, g[0], n)
    handle.bc_gather(n, n, nb, nb, pr, pc, dB, lld, g[1], n)
    handle.dgemm_device(COL, NOTRANS, NOTRANS, n, n, n, 1.0, g[0], n, g[1], n, 0.0, g[2], n)
    handle.bc_scatter(n, n, nb, nb, pr, pc, g[2], n, dC, lld)
    for got, a in zip(_from_dev_locals(dC, L["C"]), L["A"]):
        assert np.array_equal(got, 2.0 * a)


def test_block_cyclic_round_trip_rectangular(handle):
    import torch
    m, n, mb, nb, pr, pc = 131, 77, 16, 9, 3, 4
    G = np.random.default_rng(1).uniform(-1, 1, size=(m, n))
    want = orc.bc_from_global(G, mb, nb, pr, pc)
    locs, lld = _to_dev_locals([np.zeros_like(w) for w in want])
    lld = [x + 2 for x in lld]  # padded local leading dimensions
    locs = [torch.zeros(max(l * w.shape[1], 1), dtype=torch.float64, device="cuda") for l, w in zip(lld, want)]
    ldg = m + 5
    dG = torch.full((ldg * n,), -7.0, dtype=torch.float64, device="cuda")
    dG.view(n, ldg)[:, :m] = torch.from_numpy(G.T.copy()).cuda()
    handle.bc_scatter(m, n, mb, nb, pr, pc, dG, ldg, locs, lld)
    for a, l, w in zip(locs, lld, want):
        if w.size:
            got = a.cpu().numpy()[:l * w.shape[1]].reshape(w.shape[1], l).T[:w.shape[0]]
            assert np.array_equal(got, w)
    dG2 = torch.full_like(dG, -7.0)
    handle.bc_gather(m, n, mb, nb, pr, pc, locs, lld, dG2, ldg)
    assert torch.equal(dG2, dG)
    with pytest.raises(u.UvatrmmError):
        handle.bc_gather(m, n, mb, nb, pr, pc, locs, [1] * len(locs), dG2, ldg)  # lld too small
