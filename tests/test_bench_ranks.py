"""The bench's multi-rank plumbing on CPU (gloo, two ranks on 127.0.0.1).

One process per GPU is the bench's N > 1 layout: every rank runs an
independent replica, the timed region is the maximum over ranks, and only
rank 0 prints.  The GPU arm needs GPUs; these tests cover what does not.
"""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.max_over_ranks(10.0 * (rank + 1) + 0.25, world)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 20.25, 1: 20.25}


def test_max_over_ranks_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_reference_arm_under_torchrun_prints_once():
    """`--impl reference` launched as two ranks: rank 0 times the CPU
    implementation and prints one JSON line, rank 1 exits 0 without output."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "1", "--cpu-n", "512"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")


def test_single_gpu_sections_run_only_on_one_rank(monkeypatch):
    """With more than one rank the bench runs the headline replica only: the
    Ozaki, variant, next-row, batch and serving sections are never called and
    the line names them as skipped.  With one rank all of them run."""
    import argparse

    sys.path.insert(0, ROOT)
    import bench
    import uvatrmm_gb300

    called = []
    for name in ("run_ozaki", "run_variants", "run_next_rows", "run_batch", "run_serving"):
        monkeypatch.setattr(bench, name, lambda *a, _n=name, **k: called.append(_n) or {"stub": _n})

    class FakeHandle:
        def __init__(self, *a, **k):
            pass

        def close(self):
            pass

    monkeypatch.setattr(uvatrmm_gb300, "Handle", FakeHandle)
    args = argparse.Namespace(no_ozaki=False, variants=True, next_n=8, batch=5, serve=5)
    out = bench.run_sections(args, 2, 0, None, None, None, 1.0, 1.0)
    assert called == []
    assert set(out) == {"sections_skipped"}
    assert set(out["sections_skipped"]["sections"]) == {"ozaki", "variants", "next_rows", "batch", "serving"}
    out = bench.run_sections(args, 1, 0, None, None, None, 1.0, 1.0)
    assert called == ["run_ozaki", "run_variants", "run_next_rows", "run_batch", "run_serving"]
    assert set(out) == {"ozaki", "variants", "next_rows", "batch", "serving"}


def test_summary_closes_the_line():
    """The compact summary (checks, Ozaki, serving) is the last key of the line,
    so a reader of the line's tail sees it."""
    sys.path.insert(0, ROOT)
    import bench

    out = {"value": 1.0, "check": {"sampled_rel_fro_err_vs_openblas": 1.23456e-16, "tol": 3e-11},
           "variants": {"cases": [{"uplo": "L", "schedule/shape": "reg/boxes", "rel_err": 2e-16}],
                        "skinny": {"rel_err": 3e-16}, "large": {"rel_err": 4e-16}},
           "ozaki": {"value": 80.0, "speedup_vs_plain_fp64": 64.0, "moduli": 15, "bits": 54,
                     "rel_fro_err_vs_dd_oracle": 2.2e-16, "library_relerr_vs_host_fp64": 2.1e-16,
                     "roofline": {"achieved": 1500.0, "frac": 0.88}, "clocks": {"sm_mhz": 1700, "reasons": []},
                     "slice_sweep": [{"int8_slices": 5, "moduli": 11, "bits": 37, "rel_fro_err_vs_dd_oracle": 1e-9}]},
           "serving": {"max_steady_rate_req_per_s": 150.0, "max_rate_p99_within_2x_alone": 50.0, "alone_p99_ms": 139.0,
                       "rates": [{"rate_req_per_s": 50.0, "p50_ms": 1.0, "p99_ms": 100.0, "p99_first_half_ms": 90.0,
                                  "p99_second_half_ms": 95.0, "sustained_tflops": 1.2}]},
           "cpu_baseline": {"value": 0.5}}
    out["summary"] = bench.summary(out)
    line = json.dumps(out)
    assert line.rindex('"summary"') > line.rindex('"cpu_baseline"')
    s = out["summary"]
    assert s["check"]["headline_rel_err"] == 1.23e-16
    assert s["check"]["variants_rel_err"] == {"L reg/boxes": 2e-16, "skinny": 3e-16, "large": 4e-16}
    assert s["ozaki"]["moduli"] == 15 and s["ozaki"]["int8_sweep"] == [[5, 11, 37, 1e-9]]
    assert s["serving"]["max_steady_rate"] == 150.0 and s["serving"]["max_rate_p99_2x_alone"] == 50.0
    assert len(json.dumps(s)) < 1400


def test_reference_arm_reports_the_headline_config():
    sys.path.insert(0, ROOT)
    import bench
    c = bench.headline_config(16384, 16384, 1)
    assert c["m"] == c["n"] == 16384 and "seed 1" in c["workload"]


def test_a_failing_section_is_recorded_and_the_line_still_prints(monkeypatch):
    """An exception in one diagnostic section becomes an `error` entry of that
    section; the other sections still run and the summary names the failure."""
    import argparse

    sys.path.insert(0, ROOT)
    import bench
    import uvatrmm_gb300

    def boom(*a, **k):
        raise RuntimeError("device said no")

    monkeypatch.setattr(bench, "run_ozaki", boom)
    for name in ("run_variants", "run_next_rows", "run_batch", "run_serving"):
        monkeypatch.setattr(bench, name, lambda *a, **k: {"ok": True})

    class FakeHandle:
        def __init__(self, *a, **k):
            pass

        def close(self):
            pass

    monkeypatch.setattr(uvatrmm_gb300, "Handle", FakeHandle)
    args = argparse.Namespace(no_ozaki=False, variants=True, next_n=8, batch=5, serve=5)
    out = bench.run_sections(args, 1, 0, None, None, None, 1.0, 1.0)
    assert out["ozaki"] == {"error": "RuntimeError: device said no"}
    assert out["batch"] == {"ok": True} and out["serving"] == {"ok": True}
    s = bench.summary(dict(out, check={}))
    assert s["errors"] == {"ozaki": "RuntimeError: device said no"}
    json.dumps(s)
