"""Host-side parts of the GEMM / result-file / block-cyclic entry points (no GPU).

Result files are pinned to bytes written by the reference's own
print_output_results_generic (UVaTRMM/src/mm_triangular_common.c:2134-2163);
NUMROC follows ScaLAPACK's published algorithm (called at
ScaLAPACK/scalapack_sample_trmm.c:66-67).
"""
import json
import os

import numpy as np
import pytest

import uvatrmm_gb300 as u
from oracle import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _golden_results():
    return json.load(open(os.path.join(GOLD, "result_files.json")))["files"]


def _golden_block(nr, nc):
    return (0.25 * np.arange(nr * nc) + 1.0 / 3.0).reshape(nr, nc)


def test_oracle_result_bytes_match_reference_writer():
    for f in _golden_results():
        rows, cols, rb, nr, cb, nc, _, _ = f["args"]
        assert oracle.result_file_bytes(rows, cols, rb, nr, cb, nc, _golden_block(nr, nc)) == bytes.fromhex(f["hex"])


def test_write_result_byte_identical_to_reference(built, tmp_path):
    for i, f in enumerate(_golden_results()):
        rows, cols, rb, nr, cb, nc, _, _ = f["args"]
        block = _golden_block(nr, nc)
        path = str(tmp_path / f"r{i}.dat")
        u.write_result(path, rows, cols, rb, nr, cb, nc, block if block.size else None, max(nc, 1))
        assert open(path, "rb").read() == bytes.fromhex(f["hex"])
        hdr, data = u.read_result(path)
        assert hdr == [rows, cols, rb, nr, cb, nc]
        assert np.array_equal(data, block.ravel())


def test_write_result_strided_block(built, tmp_path):
    big = np.arange(6 * 10, dtype=np.float64).reshape(6, 10)
    path = str(tmp_path / "s.dat")
    u.write_result(path, 6, 10, 1, 4, 3, 5, big[1:5, 3:8].copy(order="C"), 5)
    a = open(path, "rb").read()
    u.write_result(path, 6, 10, 1, 4, 3, 5, big[1:, 3:], 10)  # same block read with ld 10
    assert open(path, "rb").read() == a == oracle.result_file_bytes(6, 10, 1, 4, 3, 5, big[1:5, 3:8])


def test_result_file_errors(built, tmp_path):
    path = str(tmp_path / "t.dat")
    with pytest.raises(u.UvatrmmError):
        u.read_result(str(tmp_path / "missing.dat"))
    open(path, "wb").write(oracle.result_file_bytes(3, 3, 0, 3, 0, 3, np.ones((3, 3)))[:-8])
    with pytest.raises(u.UvatrmmError):
        u.read_result(path)  # truncated body
    with pytest.raises(u.UvatrmmError):
        u.read_result(path, out=np.empty(4))  # capacity below nrows*ncols
    with pytest.raises(u.UvatrmmError):
        u.write_result(path, 3, 3, 0, 3, 0, 3, np.ones(9), 2)  # ld < ncols


def test_numroc_matches_oracle(built):
    for n in (0, 1, 2, 7, 100, 1000, 1023, 4096):
        for nb in (1, 3, 32, 256, 5000):
            for nprocs in (1, 2, 3, 4, 7):
                for src in range(nprocs):
                    got = [u.numroc(n, nb, p, src, nprocs) for p in range(nprocs)]
                    assert got == [oracle.numroc(n, nb, p, src, nprocs) for p in range(nprocs)]
                    assert sum(got) == n


def test_sample_layouts_round_trip():
    for (n, nb, pr, pc) in [(1000, 256, 2, 2), (10, 3, 2, 2), (333, 32, 3, 2), (5, 8, 1, 3)]:
        for kind in ("trmm", "gemm"):
            L = oracle.sample_locals(kind, n, nb, pr, pc)
            for pq, A in enumerate(L["A"]):
                assert A.shape == (oracle.numroc(n, nb, pq // pc, 0, pr), oracle.numroc(n, nb, pq % pc, 0, pc))
            G = oracle.bc_to_global(L["A"], n, n, nb, nb, pr, pc)
            back = oracle.bc_from_global(G, nb, nb, pr, pc)
            assert all(np.array_equal(x, y) for x, y in zip(back, L["A"]))
            if kind == "trmm":
                assert np.array_equal(np.triu(G, 1), np.zeros_like(G))


def test_gemm_argument_errors(built):
    # Invalid arguments are refused before any device work, numbered as CBLAS numbers them.
    lib = u.lib()
    for args, bad in [((0, u.NOTRANS, u.NOTRANS, 2, 2, 2, 2, 2, 2), 1),
                      ((u.COL, 7, u.NOTRANS, 2, 2, 2, 2, 2, 2), 2),
                      ((u.COL, u.NOTRANS, 0, 2, 2, 2, 2, 2, 2), 3),
                      ((u.COL, u.NOTRANS, u.NOTRANS, -1, 2, 2, 2, 2, 2), 4),
                      ((u.COL, u.NOTRANS, u.NOTRANS, 2, -2, 2, 2, 2, 2), 5),
                      ((u.COL, u.NOTRANS, u.NOTRANS, 2, 2, -1, 2, 2, 2), 6),
                      ((u.COL, u.NOTRANS, u.NOTRANS, 4, 2, 2, 3, 2, 4), 9),
                      ((u.ROW, u.NOTRANS, u.NOTRANS, 2, 4, 3, 3, 3, 4), 11),
                      ((u.COL, u.TRANS, u.NOTRANS, 5, 2, 3, 3, 3, 4), 14)]:
        layout, ta, tb, m, n, k, lda, ldb, ldc = args
        for fn in (lib.uvatrmm_dgemm_device, lib.uvatrmm_dgemm):
            rc = fn(None, layout, ta, tb, m, n, k, 1.0, None, lda, None, ldb, 0.0, None, ldc)
            assert rc == u.EINVAL, bad
            assert f"parameter {bad} " in lib.uvatrmm_last_error().decode()
