"""The CPU oracle pinned against the reference itself (committed fixtures)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_mappings_match_reference(built):
    cases = load("mappings.json")["cases"]
    assert len(cases) > 100
    for c in cases:
        n, P = c["n"], c["P"]
        for mode, fn in (("reg", orc.map_regular), ("balanced", orc.map_balanced)):
            ref = c[mode]
            for p in range(P):
                got = fn(n, P, p)
                if p < len(ref):
                    assert got == tuple(ref[p]), (mode, n, P, p, got, ref[p])
                else:
                    # the reference aborted at block p (exit code recorded)
                    assert c[mode + "_exit"] != 0
                    assert got is None, (mode, n, P, p, got)
                    break
            else:
                assert c[mode + "_exit"] == 0


def test_consecutive_generator_matches_reference(built):
    for b in load("consecutive.json")["blocks"]:
        got = orc.gen_consecutive(b["n"], b["rows_begin"], b["rows"], b["cols_begin"], b["cols"],
                                  bool(b["triangular"]))
        ref = np.array(b["values"]).reshape(b["rows"], b["cols"])
        assert np.array_equal(got, ref), b["n"]


@pytest.mark.parametrize("n", [1, 2, 3, 8, 17, 64, 100, 512, 1000])
def test_product_norm_matches_reference(built, n):
    norms = load("norms.json")["norms"][str(n)]
    A = orc.gen_consecutive(n, 0, n, 0, n, True)
    B = orc.gen_consecutive(n, 0, n, 0, n, False)
    for P in range(1, min(n, 4) + 1):
        for bal in (False, True):
            key = f"{'balanced' if bal else 'reg'}/trapezoid"
            try:
                C = orc.uvatrmm_product(n, P, bal, A, B)
            except ValueError:
                continue  # the reference aborts for this (n, P, mapping)
            assert "%.3f" % orc.inf_norm(C) == norms[key], (n, P, bal)
            ref = np.tril(A) @ B
            assert np.abs(C - ref).max() <= 64 * n * np.finfo(float).eps * np.abs(ref).max()


def test_norms_identical_across_mappings_and_shapes():
    for n, d in load("norms.json")["norms"].items():
        assert len(set(d.values())) == 1, n


def test_cli_stdout_format_pinned():
    text = open(os.path.join(GOLD, "cli_stdout.txt")).read()
    assert text == "\nTotal t: T\nTotal mpis: 1\nMult t: T\n\nNorm: 4.744\n"
