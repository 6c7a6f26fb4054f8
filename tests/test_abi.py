"""The C ABI library: loads, exports what the header declares, host logic."""
import ctypes as C
import json
import os
import subprocess

import pytest

import uvatrmm_gb300 as u
from uvatrmm_gb300 import build

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_library_exports_every_header_symbol(built):
    syms = u.header_symbols()
    assert "cblas_dtrmm" in syms and "uvatrmm_dtrmm" in syms
    out = subprocess.run(["nm", "-D", "--defined-only", u._lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    L = u.lib()
    for s in syms:
        assert hasattr(L, s)


def test_built_for_sm103a(built):
    out = subprocess.run(["strings", u._lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "sm_103a" in out or "sm_103" in out


def test_map_rows_matches_reference_golden(built):
    cases = json.load(open(os.path.join(GOLD, "mappings.json")))["cases"]
    for c in cases:
        for mode, sched in (("reg", u.SCHED_REG), ("balanced", u.SCHED_BALANCED)):
            for p, ref in enumerate(c[mode]):
                assert u.map_rows(sched, c["n"], c["P"], p) == tuple(ref)
            if c[mode + "_exit"] != 0:
                assert u.map_rows(sched, c["n"], c["P"], len(c[mode])) is None


def test_map_rows_rejects_bad_arguments(built):
    assert u.map_rows(u.SCHED_DYNAMIC, 10, 2, 0) is None
    assert u.map_rows(u.SCHED_REG, 10, 0, 0) is None
    assert u.map_rows(u.SCHED_REG, 10, 2, 2) is None
    assert u.map_rows(u.SCHED_REG, 3, 4, 0) is None  # reference: too few rows


def test_cblas_dtrmm_rejects_bad_arguments_without_gpu(built):
    # argument checking happens before any device call
    L = u.lib()
    buf = (C.c_double * 4)()
    L.cblas_dtrmm(102, 141, 121, 111, 131, -1, 2, 1.0, buf, 2, buf, 2)
    assert L.uvatrmm_last_status() == u.EINVAL
    assert b"parameter 6" in L.uvatrmm_last_error()
    L.cblas_dtrmm(102, 141, 121, 111, 131, 4, 2, 1.0, buf, 2, buf, 4)
    assert L.uvatrmm_last_status() == u.EINVAL
    assert b"parameter 10" in L.uvatrmm_last_error()
    L.cblas_dtrmm(99, 141, 121, 111, 131, 1, 1, 1.0, buf, 1, buf, 1)
    assert b"parameter 1" in L.uvatrmm_last_error()


def test_cli_usage_errors(built):
    exe = build.CLI
    for args, msg in ((["8", "reg"], "Number of arguments"), (["8", "foo", "boxes"], "Unknown name of mapping"),
                      (["8", "reg", "full"], "Unknown name of communication shape"),
                      (["0", "reg", "boxes"], "Number of rows")):
        r = subprocess.run([exe] + args, capture_output=True, text=True)
        assert r.returncode == 3, (args, r.returncode)
        assert msg in r.stderr
        assert "Usage:" in r.stderr


def test_no_gpu_reports_device_error(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = u.lib().uvatrmm_create(C.byref(h))
    assert rc in (u.EDEVICE, u.EUNSUPPORTED)


def test_ozaki_plan_is_monotonic(built):
    prev = 0
    for mo in range(2, 21):
        n, bits = u.ozaki_plan(4096, mo)
        assert n == mo and bits >= prev
        prev = bits
    auto, bits = u.ozaki_plan(32768)
    assert bits >= 52 and 14 <= auto <= 20
    with pytest.raises(u.UvatrmmError):
        u.ozaki_plan(100, 1)


def test_noalloc_refuses_oversized_problems_without_touching_the_device(built):
    """The no-allocation entry point bounds every dimension before it
    multiplies sizes out: problems whose scratch would exceed the fixed array
    (including sizes whose byte counts overflow 64 bits) are refused with
    UVATRMM_EINVAL before any CUDA call, so this runs without a GPU."""
    L = u.lib()
    for (m, n) in ((4096, 4096), (1 << 40, 1 << 40), (16, 1 << 60), (1 << 61, 4)):
        rc = L.uvatrmm_dtrmm_device_noalloc(102, 141, 122, 111, 131, m, n, 1.0, 16, m, 16, m, None)
        assert rc == u.EINVAL, (m, n)
        assert b"no-allocation" in L.uvatrmm_last_error()
