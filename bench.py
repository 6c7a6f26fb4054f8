"""Benchmark of the FP64 TRMM hot path on GB300 (one JSON line on rank 0).

Workload (headline, `value`): plain FP64 TRMM B := alpha*op(A)*B with
m = n = 16384, side=Left, uplo=Lower, trans=N, diag=NonUnit, alpha=1.0, A and B
i.i.d. uniform[-1,1) from seed 1 (the GPU configuration of the reference's
metric), dynamic tile schedule, trapezoid diagonal tiles.  A step is one TRMM.
Inputs (2 GiB per matrix) are far larger than L2 (129 MB), so no flush is
needed between steps.  TFLOP/s counts m^2*n flops.

  value     device-resident operands, out-of-place kernel, CUDA events on the
            handle's stream, max over ranks
  e2e       the same TRMM through the host C ABI (uvatrmm_dtrmm: pinned host A
            and B copied in, B copied back, every step)
  roofline  FP64 pipe bound: achieved = m^2*n / mean kernel time; peak = the
            FP64 issue limit (2 DFMA per clock per SM) at the SM clock sampled
            during the timed region
  cpu_baseline  the reference's per-rank decomposition (cblas_dgemm + cblas_dtrmm
            + add per row block, UVaTRMM/src/mm_triangular.c:319-403) restated in
            oracle/ over OpenBLAS, one rank's column slice of the P=4 balanced
            run, all host cores
After the headline the line carries single-GPU sections (Ozaki precision
sweep, the plain-path variants with their checks, GEMM / stage / layout
rows, grouped batch, serving sweep) and ends with a compact `summary`
(checks, Ozaki, serving).
--impl reference: the same CPU implementation timed per step on that sample.
N>1 (torchrun): independent replicas of the headline TRMM, one per GPU (the
reference's column split makes replicas the natural scaling; there is no
data exchange); the single-GPU sections are skipped and the line says so.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TRMM TFLOP/s, FP64 DMMA vs Ozaki at <=1e-14 rel err; served p50/p99 latency"
NOMINAL_FP64_TFLOPS = 1.25
FP64_FLOP_PER_CLK_SM = 4.0
# DRAM bytes (read + write) of one launch of the FP64 kernel (m = n, side L,
# lower, no transpose), measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum, first launch, cold L2) with the banded tile order:
# 1.73x, 4.23x and 8.67x the algorithmic bytes 8 (m(m+1)/2 + 2 m n).
TRAFFIC_MEASURED = {4096: 0.5810e9, 8192: 5.6793e9, 16384: 46.5478e9}
TRAFFIC_SOURCE = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum -k regex:trmm_fp64_kernel -c 1 "
                  "python -m uvatrmm_gb300.run_case --tier fp64 --m M --reps 1 (one pass), per launch")


def tri_copy_elems(ka, block=256):
    """Elements of A the host entry points copy to the device: the referenced
    (here lower) triangle in blocks of 256 columns, each block the rectangle
    from its first column's diagonal down."""
    return sum((ka - j0) * min(block, ka - j0) for j0 in range(0, ka, block))


def headline_config(m, n, ws):
    """The headline workload; both arms report this same config."""
    return {"workload": f"plain FP64 TRMM m=n={m}, side=L uplo=L trans=N diag=N alpha=1, "
                        "A and B uniform[-1,1) seed 1", "m": m, "n": n,
            "l2": "inputs larger than L2 (no flush needed)", "parallelism": f"replicas{ws}"}


def _sig(x, d=3):
    return None if x is None else float(f"{x:.{d}g}")


def summary(out):
    """Compact end of the JSON line: the checks, the Ozaki figures and the serving result
    (a section that failed shows its error instead)."""
    s = {}
    for k in ("ozaki", "variants", "serving", "next_rows", "batch"):
        if isinstance(out.get(k), dict) and "error" in out[k]:
            s.setdefault("errors", {})[k] = out[k]["error"][:120]
    chk = {"headline_rel_err": _sig(out.get("check", {}).get("sampled_rel_fro_err_vs_openblas"))}
    var = out.get("variants")
    if var and "cases" in var:
        cases = {f'{c["uplo"]} {c["schedule/shape"]}': _sig(c.get("rel_err")) for c in var["cases"]}
        for k in ("dmma_engine", "skinny", "large"):
            if k in var:
                cases[k] = _sig(var[k].get("rel_err"))
        chk["variants_rel_err"] = cases
    chk["tol_8_k_eps"] = _sig(out.get("check", {}).get("tol"))
    s["check"] = chk
    oz = out.get("ozaki")
    if oz and "slice_sweep" in oz:
        s["ozaki"] = {"tflops": oz["value"], "x_plain": oz["speedup_vs_plain_fp64"], "moduli": oz["moduli"],
                      "bits": oz["bits"], "rel_err_dd": _sig(oz["rel_fro_err_vs_dd_oracle"]),
                      "lib_rel_err_host_fp64": _sig(oz.get("library_relerr_vs_host_fp64")),
                      "gemm_tflops": oz["roofline"]["achieved"], "gemm_frac": oz["roofline"]["frac"],
                      "sm_mhz": oz["clocks"].get("sm_mhz"), "reasons": oz["clocks"].get("reasons"),
                      "int8_sweep": [[e.get("int8_slices"), e["moduli"], e["bits"], _sig(e["rel_fro_err_vs_dd_oracle"])]
                                     for e in oz["slice_sweep"]]}
    sv = out.get("serving")
    if sv and "rates" in sv:
        s["serving"] = {"max_steady_rate": sv["max_steady_rate_req_per_s"],
                        "max_rate_p99_2x_alone": sv.get("max_rate_p99_within_2x_alone"),
                        "alone_p99_ms": sv["alone_p99_ms"],
                        "rate_p50_p99_p99h1_p99h2_tflops": [
                            [r["rate_req_per_s"], _sig(r["p50_ms"]), _sig(r["p99_ms"]), _sig(r["p99_first_half_ms"]),
                             _sig(r["p99_second_half_ms"]), r["sustained_tflops"]] for r in sv["rates"]]}
    return s


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device=None) -> float:
    """The maximum of x over all ranks of the process group (x itself for one rank)."""
    if ws <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.item()


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# --------------------------------------------------------------------- CPU arm

def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_reference_sample(n: int, steps: int, warmup: int, threads: int):
    """Time the reference's per-rank product (restated in oracle/ over
    OpenBLAS) for rank 0 of `mpirun -np 4 uvatrmm.x n balanced trapezoid`:
    columns [0, n/4) of C = tril(A) B for all four row blocks."""
    import numpy as np
    from oracle import oracle as orc
    orc.blas_ready(threads)
    P = 4
    A = orc.fill_uniform(1, 0, n, n, tri="L")
    B = orc.fill_uniform(1, 1, n, n)
    C = np.zeros((n, n))
    w = orc.map_regular(n, P, 0)[1]
    times = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        orc.uvatrmm_ranks(n, P, True, 0, 1, A, B, C)
        dt = time.perf_counter() - t0
        if it >= warmup:
            times.append(dt)
    flops = float(n) * n * w
    t = statistics.mean(times)
    return {"value": flops / t / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port", "cpu": cpu_model(),
            "sample": f"rank 0 of 4 (balanced map): C[:, 0:{w}] = tril(A) B[:, 0:{w}], n={n}, "
                      f"per-row-block cblas_dgemm+cblas_dtrmm+add over OpenBLAS, {threads} threads, "
                      f"mean of {len(times)} runs ({t:.2f} s each)"}


# --------------------------------------------------------------------- GPU arm

def run_gpu(args, ws, rank, local):
    import numpy as np
    import torch

    import uvatrmm_gb300 as u

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    h = u.Handle(stream=stream)
    m = n = args.n
    L, Lo, NT, NU = u.COL, u.LOWER, u.NOTRANS, u.NONUNIT

    dA = torch.empty(m * m, dtype=torch.float64, device=dev)
    dB = torch.empty(m * n, dtype=torch.float64, device=dev)
    dC = torch.empty(m * n, dtype=torch.float64, device=dev)
    h.gen_uniform(1, 0, m, m, dA, 1, m, tri="L")
    h.gen_uniform(1, 1, m, n, dB, 1, m)
    h.sync()

    def step():
        h.dtrmm_device_oop(L, u.LEFT, Lo, NT, NU, m, n, 1.0, dA, m, dB, m, dC, m)

    for _ in range(args.warmup):
        step()
    h.sync()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        t_end.record(stream)
        h.sync()
    torch.cuda.synchronize(dev)
    total_ms = t_start.elapsed_time(t_end)
    per_launch = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(total_ms, ws, dev)
    flops = float(m) * m * n
    value = ws * flops * args.steps / (total_ms * 1e-3) / 1e12
    achieved = flops / (statistics.mean(per_launch) * 1e-3) / 1e12
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    n_sms = torch.cuda.get_device_properties(dev).multi_processor_count
    # FP64 issue limit: 2 DFMA (4 flop) per clock per SM at the sampled clock.
    peak = FP64_FLOP_PER_CLK_SM * n_sms * sm_mhz * 1e6 / 1e12

    # correctness spot check of the timed output: 4 sampled columns vs OpenBLAS (rank 0 only)
    relerr = None
    if rank == 0 and args.check:
        from oracle import oracle as orc
        sel = [0, n // 3, n // 2, n - 1]
        A = dA.cpu().numpy()
        Bs = np.concatenate([dB[j * m:(j + 1) * m].cpu().numpy() for j in sel])
        Cs = np.concatenate([dC[j * m:(j + 1) * m].cpu().numpy() for j in sel])
        orc.blas_dtrmm(L, u.LEFT, Lo, NT, NU, m, len(sel), 1.0, A, m, Bs, m)
        relerr = float(np.linalg.norm(Cs - Bs) / np.linalg.norm(Bs))

    # e2e through the host C ABI, operands in the library's page-locked host
    # memory (uvatrmm_host_alloc: huge-page backed)
    del dC
    hA = u.host_empty(m * m)
    hBs = [u.host_empty(m * n), u.host_empty(m * n)]
    hA[:] = dA.cpu().numpy()
    hB0 = dB.cpu().numpy()
    del dA, dB
    torch.cuda.empty_cache()
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    for b in hBs:
        b[:] = hB0
    # Pipelined: a stream of independent products through uvatrmm_dtrmm_async
    # on two handles (double-buffered B), so one step's copies overlap the
    # other's product; every step still copies its A (the referenced triangle)
    # and B in and B out.
    # The second handle gets its own non-blocking stream: on the legacy default
    # stream the same loop ran 1.1 % slower (36.37 against 35.96 s for 10 steps).
    h2 = u.Handle(stream=torch.cuda.Stream(dev))
    hs = [h, h2]
    for hh, b in zip(hs, hBs):  # warm-up (allocates each handle's workspace)
        hh.dtrmm_async(L, u.LEFT, Lo, NT, NU, m, n, 1.0, hA, m, b, m)
        hh.sync()
    if ws > 1:
        torch.distributed.barrier()
    with ClockSampler(local) as clk_e2e:
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            hs[k % 2].dtrmm_async(L, u.LEFT, Lo, NT, NU, m, n, 1.0, hA, m, hBs[k % 2], m)
        for hh in hs:
            hh.sync()
        e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, ws, dev)
    e2e_value = ws * flops * e2e_steps / e2e_s / 1e12
    # One call at a time: the synchronous uvatrmm_dtrmm, copies not overlapped.
    step_ms = []
    sync_steps = min(3, e2e_steps)
    t0 = time.perf_counter()
    for _ in range(sync_steps):
        ts = time.perf_counter()
        h.dtrmm(L, u.LEFT, Lo, NT, NU, m, n, 1.0, hA, m, hBs[0], m)
        step_ms.append(round(1e3 * (time.perf_counter() - ts), 1))
    sync_s = max_over_ranks(time.perf_counter() - t0, ws, dev)
    sync_value = ws * flops * sync_steps / sync_s / 1e12
    h2.close()

    out = {
        "metric": METRIC, "value": round(value, 4), "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform[-1,1), seed 1)",
        "config": headline_config(m, n, ws),
        "kernel": {"engine": "DFMA", "schedule": "dynamic", "shape": "trapezoid"},
        "e2e": {"value": round(e2e_value, 4), "unit": "TFLOP/s", "h2d_bytes_per_step": 8 * (tri_copy_elems(m) + m * n),
                "d2h_bytes_per_step": 8 * m * n, "api": "uvatrmm_dtrmm_async on two handles (host operands from uvatrmm_host_alloc, B "
                       "double-buffered), every step copying A's triangle and B in and B out",
                "steps": e2e_steps, "clocks": clk_e2e.summary(),
                "sync_value": round(sync_value, 4), "sync_api": "uvatrmm_dtrmm, one call at a time",
                "sync_step_ms": step_ms},
        "roofline": {"bound": "tensor", "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": TRAFFIC_MEASURED.get(m) if m == n else None,
                     "traffic_measured": {f"m=n={k}": v for k, v in TRAFFIC_MEASURED.items()},
                     "peak_source": f"FP64 issue limit {FP64_FLOP_PER_CLK_SM} flop/clk/SM x {n_sms} SMs x "
                                    f"{sm_mhz:.0f} MHz (sampled); MEASURED_PEAKS.json has no FP64 figure; "
                                    f"nominal GB300 FP64 {NOMINAL_FP64_TFLOPS}",
                     "frac_of_nominal": round(achieved / NOMINAL_FP64_TFLOPS, 4),
                     "traffic_source": TRAFFIC_SOURCE},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "check": {"sampled_rel_fro_err_vs_openblas": relerr, "tol": 8 * m * 2.0 ** -52},
    }
    del hA, hBs, hB0
    out.update(run_sections(args, ws, rank, h, dev, stream, achieved, peak))
    return out


SINGLE_GPU_SECTIONS = ("ozaki", "variants", "next_rows", "batch", "serving")


def _guarded(fn, *a):
    """A section's result, or its error: a failure in one diagnostic section
    is recorded in the line instead of ending the run before the line prints."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001
        return {"error": f"{type(e).__name__}: {e}"[:400]}


def run_sections(args, ws, rank, h, dev, stream, plain_tflops, fp64_peak):
    """The sections after the headline.  They are single-GPU measurements:
    under torchrun (ws > 1) every rank runs the headline replica only and the
    line records which sections were skipped."""
    import uvatrmm_gb300 as u
    out = {}
    if ws > 1:
        out["sections_skipped"] = {"sections": list(SINGLE_GPU_SECTIONS),
                                   "why": "single-GPU sections; at N > 1 each rank runs the plain FP64 replica only"}
        return out
    if not args.no_ozaki:
        out["ozaki"] = _guarded(run_ozaki, args, h, dev, stream, rank, plain_tflops)
    if args.variants:
        out["variants"] = _guarded(run_variants, args, h, dev, stream, fp64_peak)
    if args.next_n > 0:
        out["next_rows"] = _guarded(run_next_rows, args, h, dev, stream, fp64_peak)
    if args.batch > 0:
        hb = u.Handle(stream=stream)  # its own workspace for the one-call-per-problem comparison
        out["batch"] = _guarded(run_batch, args, hb, dev, stream)
        hb.close()
    if args.serve > 0:
        hs = u.Handle(stream=stream)
        out["serving"] = _guarded(run_serving, args, hs, dev, stream)
        hs.close()
    return out


def serve_requests(count, seed, dev, h):
    """The serving configuration's request mix: m log-uniform [128, 8192], n
    log-uniform [32, 8192], half exact FP64 / half <= 1e-14 Ozaki, side /
    uplo / trans uniform, entries uniform[-1,1), seed 4."""
    import numpy as np
    import torch

    import uvatrmm_gb300 as u
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        m = int(round(np.exp(rng.uniform(np.log(128), np.log(8192)))))
        n = int(round(np.exp(rng.uniform(np.log(32), np.log(8192)))))
        side = [u.LEFT, u.RIGHT][rng.integers(2)]
        uplo = [u.LOWER, u.UPPER][rng.integers(2)]
        trans = [u.NOTRANS, u.TRANS][rng.integers(2)]
        tier = u.TIER_OZAKI if rng.random() < 0.5 else u.TIER_FP64
        ka = m if side == u.LEFT else n
        A = torch.empty(ka * ka, dtype=torch.float64, device=dev)
        B = torch.empty(m * n, dtype=torch.float64, device=dev)
        h.gen_uniform(seed, 2 * i, ka, ka, A, 1, ka)
        h.gen_uniform(seed, 2 * i + 1, m, n, B, 1, m)
        reqs.append(dict(layout=u.COL, side=side, uplo=uplo, transa=trans, diag=u.NONUNIT, m=m, n=n, alpha=1.0,
                         A=A, lda=ka, B=B, ldb=m, tier=tier, moduli=0))
    h.sync()
    return reqs, rng


def _pct(v, q):
    import numpy as np
    return round(float(np.percentile(v, q)), 3) if len(v) else None


def run_serving(args, h, dev, stream):
    """Poisson arrivals into the server (device-resident operands, 120 GB
    budget) at rates up to about the device's capacity, each for
    `serve_seconds` of arrivals; requests cycle through a pool of distinct
    operand sets (a set is reused once its previous request is done).
    Per-request latencies give p50 / p99 over the stream and p99 over each
    half of it: a queue that grows shows as a second half slower than the
    first.  Beside them, the same requests one at a time through the direct
    entry points."""
    import numpy as np
    import torch

    import uvatrmm_gb300 as u
    reqs, rng = serve_requests(args.serve, 4, dev, h)
    flops = [(p["m"] ** 2 * p["n"] if p["side"] == u.LEFT else p["n"] ** 2 * p["m"]) for p in reqs]
    # one at a time through the direct entry points (the unbatched reference point)
    alone_ms = []
    for p in reqs[: min(len(reqs), 200)]:
        a = (p["layout"], p["side"], p["uplo"], p["transa"], p["diag"], p["m"], p["n"], 1.0, p["A"], p["lda"],
             p["B"], p["ldb"])
        t0 = time.perf_counter()
        (h.ozaki_device if p["tier"] == u.TIER_OZAKI else h.dtrmm_device)(*a)
        h.sync()
        alone_ms.append((time.perf_counter() - t0) * 1e3)
    alone_p99 = _pct(alone_ms, 99)
    alone_tier = [reqs[i]["tier"] for i in range(len(alone_ms))]

    def by_tier(lats, tiers):
        """p50 / p99 per accuracy tier."""
        out = {}
        for t, name in ((u.TIER_FP64, "fp64"), (u.TIER_OZAKI, "ozaki")):
            v = [x for x, k in zip(lats, tiers) if k == t]
            out[name] = {"n": len(v), "p50_ms": _pct(v, 50), "p99_ms": _pct(v, 99)}
        return out
    rates = []
    for rate in args.serve_rates:
        count = max(1, int(round(rate * args.serve_seconds)))
        srv = u.Server(h, hbm_budget_bytes=int(120e9))
        gaps = rng.exponential(1.0 / rate, size=count)
        ids, last = [], {}
        t_next = time.perf_counter()
        for i in range(count):
            k = i % len(reqs)
            if k in last:
                srv.wait(last[k])
            t_next += gaps[i]
            while True:
                d = t_next - time.perf_counter()
                if d <= 0:
                    break
                time.sleep(min(d, 0.001) if d > 0.0002 else 0)
            last[k] = srv.submit(reqs[k])
            ids.append(last[k])
        bad = sum(srv.wait(r) != 0 for r in ids)
        pairs = [(srv.latency_ms(r), reqs[i % len(reqs)]["tier"]) for i, r in enumerate(ids)]
        lat = [x for x, _ in pairs if x is not None]
        tiers = [t for x, t in pairs if x is not None]
        st = srv.stats()
        srv.close()
        span = st["last_done_s"] - st["first_submit_s"]
        half = len(lat) // 2
        served = sum(flops[i % len(reqs)] for i in range(count))
        rates.append({"rate_req_per_s": rate, "requests": count, "failed": bad,
                      "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
                      "p99_first_half_ms": _pct(lat[:half], 99), "p99_second_half_ms": _pct(lat[half:], 99),
                      "mean_ms": round(float(np.mean(lat)), 3) if lat else None, "max_ms": round(max(lat), 3),
                      "offered_tflops": round(served / (count / rate) / 1e12, 4),
                      "sustained_tflops": round(st["served_flops"] / span / 1e12, 4), "ticks": st["ticks"],
                      "peak_pool_gib": round(st["peak_bytes"] / 2 ** 30, 2), "by_tier": by_tier(lat, tiers)})
    # Highest rate served in steady state (no failures, the second half's p99
    # within 1.5x the first half's: the queue does not grow), and the highest
    # of those whose p99 also stays within 2x the one-at-a-time p99.
    steady = [r for r in rates if r["failed"] == 0 and r["p99_second_half_ms"] <= 1.5 * r["p99_first_half_ms"]]
    tight = [r for r in steady if r["p99_ms"] <= 2.0 * alone_p99]
    del reqs
    torch.cuda.empty_cache()
    return {"workload": f"Poisson arrivals for {args.serve_seconds:g} s per rate over a pool of {args.serve} "
                        "request operand sets, m logU[128,8192], n logU[32,8192], 50% FP64 / 50% Ozaki (<=1e-14), "
                        "side/uplo/trans uniform, 120 GB budget, device-resident operands, seed 4",
            "alone_p50_ms": _pct(alone_ms, 50), "alone_p99_ms": alone_p99,
            "alone_requests": len(alone_ms), "alone_by_tier": by_tier(alone_ms, alone_tier),
            "alone_capacity_req_per_s": round(1e3 / float(np.mean(alone_ms)), 1),
            "mean_gflop_per_request": round(sum(flops) / len(flops) / 1e9, 2),
            "max_steady_rate_req_per_s": max((r["rate_req_per_s"] for r in steady), default=None),
            "max_rate_p99_within_2x_alone": max((r["rate_req_per_s"] for r in tight), default=None),
            "steady_rule": "no failures and second-half p99 <= 1.5x first-half p99 (no queue growth)",
            "rates": rates}


def batch_problems(count, seed, dev, h):
    """The batching configuration: m log-uniform [64, 4096], n log-uniform
    [16, 4096], side/uplo/trans uniform, 70 % FP64 / 30 % Ozaki, entries
    uniform[-1,1), seed 3 (sizes drawn with numpy's PCG64 from the seed)."""
    import numpy as np
    import torch

    import uvatrmm_gb300 as u
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        m = int(round(np.exp(rng.uniform(np.log(64), np.log(4096)))))
        n = int(round(np.exp(rng.uniform(np.log(16), np.log(4096)))))
        side = [u.LEFT, u.RIGHT][rng.integers(2)]
        uplo = [u.LOWER, u.UPPER][rng.integers(2)]
        trans = [u.NOTRANS, u.TRANS][rng.integers(2)]
        tier = u.TIER_OZAKI if rng.random() < 0.3 else u.TIER_FP64
        ka = m if side == u.LEFT else n
        A = torch.empty(ka * ka, dtype=torch.float64, device=dev)
        B = torch.empty(m * n, dtype=torch.float64, device=dev)
        h.gen_uniform(seed, 2 * i, ka, ka, A, 1, ka)
        h.gen_uniform(seed, 2 * i + 1, m, n, B, 1, m)
        probs.append(dict(layout=u.COL, side=side, uplo=uplo, transa=trans, diag=u.NONUNIT, m=m, n=n, alpha=1.0,
                          A=A, lda=ka, B=B, ldb=m, tier=tier, moduli=0))
    h.sync()
    return probs


def run_batch(args, h, dev, stream):
    """Grouped persistent launches in one CUDA graph vs one call per problem."""
    import torch

    import uvatrmm_gb300 as u
    probs = batch_problems(args.batch, 3, dev, h)
    t0 = time.perf_counter()
    g = u.Group(h, probs)
    plan_s = time.perf_counter() - t0
    st = g.stats()
    g.run()  # warm-up
    h.sync()
    times = []
    for _ in range(args.batch_steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.run()
        e1.record(stream)
        h.sync()
        times.append(e0.elapsed_time(e1))
    ms = statistics.mean(times)
    # The same problems one call at a time (FP64: uvatrmm_dtrmm_device; Ozaki: uvatrmm_ozaki_dtrmm_device).
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for p in probs:
        a = (p["layout"], p["side"], p["uplo"], p["transa"], p["diag"], p["m"], p["n"], 1.0, p["A"], p["lda"],
             p["B"], p["ldb"])
        if p["tier"] == u.TIER_OZAKI:
            h.ozaki_device(*a)
        else:
            h.dtrmm_device(*a)
    e1.record(stream)
    h.sync()
    seq_ms = e0.elapsed_time(e1)
    g.close()
    n_oz = sum(p["tier"] == u.TIER_OZAKI for p in probs)
    del probs
    torch.cuda.empty_cache()
    return {"workload": f"{args.batch} TRMMs, m logU[64,4096], n logU[16,4096], side/uplo/trans uniform, "
                        f"{args.batch - n_oz} FP64 + {n_oz} Ozaki, seed 3",
            "value": round(st["flops"] / (ms * 1e-3) / 1e12, 4), "unit": "TFLOP/s (sum of m^2 n)",
            "ms_per_batch": round(ms, 3), "runs": len(times), "graph_kernel_launches": st["launches"],
            "fp64_tiles": st["fp64_tiles"], "ozaki_tiles": st["ozaki_tiles"], "ozaki_waves": st["ozaki_waves"],
            "arena_gib": round(st["arena_bytes"] / 2 ** 30, 2), "plan_and_capture_s": round(plan_s, 2),
            "one_call_per_problem_ms": round(seq_ms, 3),
            "speedup_vs_one_call_per_problem": round(seq_ms / ms, 3)}


def _timed(stream, fn, steps, warm=True):
    """Mean CUDA-event ms of fn() over `steps` calls on `stream` (after one warm-up call if `warm`)."""
    import torch
    if warm:
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.mean(times)


def _sample_cols(d, rows, ld, cols):
    """Columns `cols` of a column-major device matrix as a host (rows x len(cols)) array."""
    import numpy as np
    return np.stack([d[j * ld:j * ld + rows].cpu().numpy() for j in cols], axis=1)


def _openblas_cols(A, m, uplo, Bcols):
    """OpenBLAS cblas_dtrmm (left, no-trans, non-unit, alpha 1) of sampled B
    columns (an m x k host array); A is the flat column-major m x m operand."""
    import numpy as np

    import uvatrmm_gb300 as u
    from oracle import oracle as orc
    k = Bcols.shape[1]
    flat = np.ascontiguousarray(Bcols.T).ravel()  # column-major m x k, ld m
    orc.blas_dtrmm(u.COL, u.LEFT, uplo, u.NOTRANS, u.NONUNIT, m, k, 1.0, A, m, flat, m)
    return flat.reshape(k, m).T


def _rel(got, ref):
    import numpy as np
    return float(np.linalg.norm(got - ref) / np.linalg.norm(ref))


def run_variants(args, h, dev, stream, fp64_peak):
    """The plain FP64 configuration's other cases: both uplo under every schedule and
    message shape at m = n = 16384, the skinny m = 16384, n = 256 case, and m = n = 32768.
    Every case's output is checked on four sampled columns against OpenBLAS
    cblas_dtrmm (tolerance 8 k eps relative Frobenius)."""
    import torch

    import uvatrmm_gb300 as u
    hbm, _ = hbm_peak()
    out = {"cases": [], "tol": 8 * args.n * 2.0 ** -52}
    m = args.n
    sel = [0, m // 3, m // 2, m - 1]
    dA = torch.empty(m * m, dtype=torch.float64, device=dev)
    dB = torch.empty(m * m, dtype=torch.float64, device=dev)
    dC = torch.empty_like(dB)
    h.gen_uniform(1, 1, m, m, dB, 1, m)
    h.sync()
    Bs = _sample_cols(dB, m, m, sel)
    combos = [(u.SCHED_DYNAMIC, u.SHAPE_TRAPEZOID, "dynamic/trapezoid"), (u.SCHED_REG, u.SHAPE_BOXES, "reg/boxes"),
              (u.SCHED_REG, u.SHAPE_TRAPEZOID, "reg/trapezoid"), (u.SCHED_BALANCED, u.SHAPE_BOXES, "balanced/boxes"),
              (u.SCHED_BALANCED, u.SHAPE_TRAPEZOID, "balanced/trapezoid")]
    ref = None
    for uplo, uname in ((u.LOWER, "L"), (u.UPPER, "U")):
        h.gen_uniform(1, 0, m, m, dA, 1, m, tri=uname)
        h.sync()
        if args.check:
            ref = _openblas_cols(dA.cpu().numpy(), m, uplo, Bs)
        for sched, shape, name in combos:
            h.set_option("schedule", sched)
            h.set_option("shape", shape)
            ms = _timed(stream, lambda: h.dtrmm_device_oop(u.COL, u.LEFT, uplo, u.NOTRANS, u.NONUNIT, m, m, 1.0,
                                                           dA, m, dB, m, dC, m), 1, warm=False)
            tf = float(m) ** 3 / (ms * 1e-3) / 1e12
            case = {"m": m, "n": m, "uplo": uname, "schedule/shape": name, "tflops": round(tf, 4),
                    "frac_of_fp64_issue_limit": round(tf / fp64_peak, 4), "ms": round(ms, 2)}
            if ref is not None:
                case["rel_err"] = _rel(_sample_cols(dC, m, m, sel), ref)
            out["cases"].append(case)
    h.set_option("schedule", u.SCHED_DYNAMIC)
    h.set_option("shape", u.SHAPE_TRAPEZOID)
    # the FP64 tensor-core engine (DMMA, mma.sync m8n8k4) on the last uplo's operands
    h.set_option("engine", u.ENGINE_DMMA)
    ms = _timed(stream, lambda: h.dtrmm_device_oop(u.COL, u.LEFT, u.UPPER, u.NOTRANS, u.NONUNIT, m, m, 1.0,
                                                   dA, m, dB, m, dC, m), 1)
    h.set_option("engine", u.ENGINE_DFMA)
    tf = float(m) ** 3 / (ms * 1e-3) / 1e12
    out["dmma_engine"] = {"m": m, "n": m, "uplo": "U", "schedule/shape": "dynamic/trapezoid",
                          "tflops": round(tf, 4), "frac_of_fp64_issue_limit": round(tf / fp64_peak, 4),
                          "ms": round(ms, 2)}
    if ref is not None:
        out["dmma_engine"]["rel_err"] = _rel(_sample_cols(dC, m, m, sel), ref)
    # skinny: B is m x 256; bytes = A triangle + B read + C written
    ns = 256
    h.gen_uniform(1, 0, m, m, dA, 1, m, tri="L")
    h.sync()
    ms = _timed(stream, lambda: h.dtrmm_device_oop(u.COL, u.LEFT, u.LOWER, u.NOTRANS, u.NONUNIT, m, ns, 1.0,
                                                   dA, m, dB, m, dC, m), 3)
    tf = float(m) * m * ns / (ms * 1e-3) / 1e12
    gbs = 8.0 * (m * (m + 1) / 2 + 2 * m * ns) / (ms * 1e-3) / 1e9
    out["skinny"] = {"m": m, "n": ns, "tflops": round(tf, 4), "frac_of_fp64_issue_limit": round(tf / fp64_peak, 4),
                     "algorithmic_gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / hbm, 4),
                     "ms": round(ms, 3),
                     "note": "arithmetic intensity n/4 = 64 flop/B, far above the FP64 ridge (~0.19 flop/B): "
                             "still bound by the FP64 pipe"}
    if args.check:
        ssel = [0, ns // 3, ns // 2, ns - 1]
        out["skinny"]["rel_err"] = _rel(_sample_cols(dC, m, m, ssel),
                                        _openblas_cols(dA.cpu().numpy(), m, u.LOWER, _sample_cols(dB, m, m, ssel)))
    del dA, dB, dC
    torch.cuda.empty_cache()
    if args.big_n > 0:
        M = args.big_n
        dA = torch.empty(M * M, dtype=torch.float64, device=dev)
        dB = torch.empty_like(dA)
        dC = torch.empty_like(dA)
        h.gen_uniform(1, 0, M, M, dA, 1, M, tri="L")
        h.gen_uniform(1, 1, M, M, dB, 1, M)
        h.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.dtrmm_device_oop(u.COL, u.LEFT, u.LOWER, u.NOTRANS, u.NONUNIT, M, M, 1.0, dA, M, dB, M, dC, M)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        tf = float(M) ** 3 / (ms * 1e-3) / 1e12
        out["large"] = {"m": M, "n": M, "tflops": round(tf, 4), "frac_of_fp64_issue_limit": round(tf / fp64_peak, 4),
                        "ms": round(ms, 1), "runs": 1, "note": "one timed call after the 16384 runs (warm kernel)"}
        if args.check:
            bsel = [0, M // 3, M // 2, M - 1]
            out["large"]["rel_err"] = _rel(_sample_cols(dC, M, M, bsel),
                                           _openblas_cols(dA.cpu().numpy(), M, u.LOWER, _sample_cols(dB, M, M, bsel)))
            out["large"]["tol"] = 8 * M * 2.0 ** -52
        del dA, dB, dC
        torch.cuda.empty_cache()
    return out


def run_next_rows(args, h, dev, stream, fp64_peak):
    """The entry points either side of the TRMM: GEMM, the reference's product
    loop driven stage by stage, and the ScaLAPACK block-cyclic adapters."""
    import numpy as np
    import torch

    import uvatrmm_gb300 as u
    n = args.next_n
    out = {}
    dA = torch.empty(n * n, dtype=torch.float64, device=dev)
    dB = torch.empty_like(dA)
    dC = torch.empty_like(dA)
    h.gen_uniform(5, 0, n, n, dA, 1, n)
    h.gen_uniform(5, 1, n, n, dB, 1, n)
    h.sync()
    # DGEMM n^3 (2 n^3 flop)
    ms = _timed(stream, lambda: h.dgemm_device(u.COL, u.NOTRANS, u.NOTRANS, n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n),
                args.next_steps)
    tf = 2.0 * n ** 3 / (ms * 1e-3) / 1e12
    out["dgemm"] = {"workload": f"uvatrmm_dgemm_device m=n=k={n} NN alpha=1 beta=0", "value": round(tf, 4),
                    "unit": "TFLOP/s", "ms": round(ms, 3), "frac_of_fp64_issue_limit": round(tf / fp64_peak, 4)}
    # The reference's product loop (4 balanced row blocks, one rank owning all columns), stage by stage.
    h.gen_uniform(5, 2, n, n, dA, 1, n, tri="U")  # row-major lower triangle = column-major upper
    h.sync()
    torch.cuda.synchronize()
    P = 4
    blocks = [u.map_rows(u.SCHED_BALANCED, n, P, s) for s in range(P)]

    def loop():
        for b, hh in blocks:
            h.stage(n, n, b, hh, dA[b * n:], n, dB, n, dC, n)
    ms = _timed(stream, loop, args.next_steps)
    tf = float(n) ** 3 / (ms * 1e-3) / 1e12
    # parity: the same product through one plain TRMM call (row-major left lower), sampled columns
    dR = dB.clone()
    torch.cuda.synchronize()  # the clone ran on torch's stream, the library runs on `stream`
    h.dtrmm_device(u.ROW, u.LEFT, u.LOWER, u.NOTRANS, u.NONUNIT, n, n, 1.0, dA, n, dR, n)
    h.sync()
    cols = torch.tensor([0, n // 3, n - 1], device=dev)
    got = dC.view(n, n)[:, cols].cpu().numpy()
    ref = dR.view(n, n)[:, cols].cpu().numpy()
    del dR
    out["stage_loop"] = {"workload": f"uvatrmm_stage x {P} balanced row blocks, n={n}, one rank (all columns)",
                         "value": round(tf, 4), "unit": "TFLOP/s (n^3)", "ms": round(ms, 3),
                         "gpu_launches": 2 * P,
                         "rel_fro_vs_single_trmm_call": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
    # Block-cyclic gather + scatter of one n x n matrix (2x2 grid, 256 x 256 blocks): 2 reads + 2 writes of 8n^2 bytes.
    nb, pr, pc = 256, 2, 2
    loc = []
    lld = []
    for pq in range(pr * pc):
        mp, nq = u.numroc(n, nb, pq // pc, 0, pr), u.numroc(n, nb, pq % pc, 0, pc)
        loc.append(torch.empty(mp * nq, dtype=torch.float64, device=dev))
        lld.append(max(mp, 1))
    h.bc_scatter(n, n, nb, nb, pr, pc, dB, n, loc, lld)
    ms = _timed(stream, lambda: (h.bc_scatter(n, n, nb, nb, pr, pc, dB, n, loc, lld),
                                 h.bc_gather(n, n, nb, nb, pr, pc, loc, lld, dC, n)), args.next_steps)
    gbs = 4 * 8 * n * n / (ms * 1e-3) / 1e9
    hbm, _ = hbm_peak()
    out["block_cyclic"] = {"workload": f"uvatrmm_bc_scatter + uvatrmm_bc_gather, {n}x{n}, nb={nb}, {pr}x{pc} grid",
                           "value": round(gbs, 1), "unit": "GB/s", "ms": round(ms, 3),
                           "frac_of_measured_hbm": round(gbs / hbm, 4),
                           "round_trip_exact": bool(torch.equal(dB, dC))}
    del dA, dB, dC, loc
    torch.cuda.empty_cache()
    return out


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except Exception:
        return 6800.0, "fallback (profiling recipe)"


def bf16_peak():
    """Sustained cuBLAS bf16 TFLOP/s from MEASURED_PEAKS.json (driver-measured), else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops_sustained"]), "measured (MEASURED_PEAKS.json, sustained)"
    except Exception:
        return 1700.0, "fallback (profiling recipe, sustained)"


def ozaki_mma_flops(m, n, moduli, side_left=True, lower=True):
    """bf16 MMA flops the residue GEMM issues for one call (tile-exact): CTA pairs
    cover 256 rows x 256 columns over one K range (for a triangular left operand,
    the union of both 128-row tiles' ranges), in slabs of 128."""
    BM, BN, BK, PAIR = 128, 256, 128, 2
    Mp, Np = -(-m // (PAIR * BM)) * PAIR * BM, -(-n // BN) * BN
    K = m if side_left else n
    total = 0
    if side_left:
        for tp in range(Mp // (PAIR * BM)):
            i0 = tp * PAIR * BM
            kb, ke = (0, min(i0 + PAIR * BM, K)) if lower else (i0, K)
            total += PAIR * (Np // BN) * ((ke + BK - 1) // BK - kb // BK) * BK
    else:
        for tj in range(Np // BN):
            j0 = tj * BN
            kb, ke = (j0, K) if lower else (0, min(j0 + BN, K))
            total += (Mp // BM) * ((ke + BK - 1) // BK - kb // BK) * BK
    return 2.0 * BM * BN * total * moduli


def int8_slice_map(k):
    """INT8 digit-slice counts 5-9 (7 bits per signed 8-bit slice) mapped to the
    fewest CRT moduli whose bits per scaled entry reach the same budget at
    inner dimension k."""
    import uvatrmm_gb300 as u
    out = []
    for sl in range(5, 10):
        for mo in range(2, 21):
            _, b = u.ozaki_plan(k, mo)
            if b >= 7 * sl:
                out.append({"int8_slices": sl, "int8_bits": 7 * sl, "int8_products": sl * (sl + 1) // 2,
                            "moduli": mo})
                break
    return out


def run_ozaki(args, h, dev, stream, rank, plain_tflops):
    """Ozaki emulated FP64 TRMM at the precision configuration: m = n = 32768,
    side=L, uplo=U, trans=T, entries uniform[-1,1) * 2^k, k uniform in
    [-20, 20], seed 2; automatic slice count timed, slice counts swept for
    the error against the double-double oracle on sampled columns."""
    import numpy as np
    import torch

    import uvatrmm_gb300 as u
    m = n = args.ozaki_n
    C_, Le, Up, Tr, NU = u.COL, u.LEFT, u.UPPER, u.TRANS, u.NONUNIT
    dA = torch.empty(m * m, dtype=torch.float64, device=dev)
    dB0 = torch.empty(m * n, dtype=torch.float64, device=dev)
    dB = torch.empty(m * n, dtype=torch.float64, device=dev)
    h.gen_uniform(2, 0, m, m, dA, 1, m, tri="U", spread=20)
    h.gen_uniform(2, 1, m, n, dB0, 1, m, spread=20)
    h.sync()
    h.set_option("stage_timing", 1)
    h.set_option("ozaki_raster", args.ozaki_raster)
    moduli, bits = u.ozaki_plan(m)

    def step(mo=0, want_err=False):
        with torch.cuda.stream(stream):  # ordered before the library's work on the same stream
            dB.copy_(dB0)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        err, b = h.ozaki_device(C_, Le, Up, Tr, NU, m, n, 1.0, dA, m, dB, m, moduli=mo, want_err=want_err)
        ev1.record(stream)
        h.sync()
        return ev0.elapsed_time(ev1), err, b

    for _ in range(max(1, args.warmup - 2)):
        step()
    times, stages = [], []
    with ClockSampler(dev.index or 0) as clk:
        for _ in range(args.ozaki_steps):
            ms, _, _ = step()
            times.append(ms)
            stages.append(h.stage_times())
    t_ms = statistics.mean(times)
    tflops = float(m) * m * n / (t_ms * 1e-3) / 1e12
    st = [statistics.mean(s[k] for s in stages) for k in range(4)]
    gemm_flops = ozaki_mma_flops(m, n, moduli, True, True)
    peak, peak_src = bf16_peak()
    gemm_tflops = gemm_flops / (st[2] * 1e-3) / 1e12

    # The precision configuration sweeps INT8 digit-slice counts 5-9.  Signed
    # 8-bit slices hold 7 bits each, so s slices keep 7s bits of a scaled
    # entry (and need s(s+1)/2 INT8 products); the CRT form keeps t bits with
    # N residue products.  Each s maps to the fewest moduli N with t >= 7s at
    # this K; the automatic count and the widest set (20) are timed too.
    slice_map = int8_slice_map(m)
    settings = sorted({e["moduli"] for e in slice_map} | {moduli, 20})
    sweep = []
    lib_err = None
    if rank == 0 and args.check:
        from oracle import oracle as orc
        sel = [1, n // 3, (2 * n) // 3, n - 2]
        A = dA.cpu().numpy()
        B = dB0.cpu().numpy()
        Bs = np.concatenate([B[j * m:(j + 1) * m] for j in sel])
        orc.lib()
        ref = orc.dtrmm_dd(C_, Le, Up, Tr, NU, m, len(sel), 1.0, A, m, Bs, m)
        del A
        for mo in settings:
            ms, _, b = step(mo)
            got = np.stack([dB[j * m:(j + 1) * m].cpu().numpy() for j in sel], axis=1)
            e = {"moduli": mo, "bits": b, "ms": round(ms, 2),
                 "rel_fro_err_vs_dd_oracle": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
            e.update({k: v for x in slice_map if x["moduli"] == mo for k, v in x.items() if k != "moduli"})
            sweep.append(e)
        # The library's own error report against its host FP64 reference (Dot2
        # over 8 sampled columns), at the automatic count.
        h.set_option("ozaki_err_host", 1)
        _, lib_err, _ = step(0, want_err=True)
        h.set_option("ozaki_err_host", 0)
    h.set_option("stage_timing", 0)
    h.set_option("ozaki_raster", 0)
    del dA, dB0, dB
    torch.cuda.empty_cache()
    auto = next((s for s in sweep if s["moduli"] == moduli), None)
    return {
        "workload": f"Ozaki emulated FP64 TRMM m=n={m}, side=L uplo=U trans=T diag=N alpha=1, "
                    "entries uniform[-1,1)*2^k, k in [-20,20], seed 2",
        "value": round(tflops, 3), "unit": "TFLOP/s (m^2 n FP64-equivalent flops)", "steps": len(times),
        "ms_per_step": round(t_ms, 3), "moduli": moduli, "bits": bits,
        "rel_fro_err_vs_dd_oracle": auto["rel_fro_err_vs_dd_oracle"] if auto else None,
        "library_relerr_vs_host_fp64": lib_err,
        "speedup_vs_plain_fp64": round(tflops / plain_tflops, 2),
        "stage_ms": {"scaling": round(st[0], 3), "slicing": round(st[1], 3), "residue_gemm": round(st[2], 3),
                     "reassembly": round(st[3], 3)},
        "roofline": {"bound": "tensor", "kernel": "oz_gemm_kernel (tcgen05 kind::f16, bf16 -> fp32)",
                     "achieved": round(gemm_tflops, 2), "peak": peak, "unit": "TFLOP/s",
                     "frac": round(gemm_tflops / peak, 4), "peak_source": peak_src,
                     "flops": "bf16 MMA flops issued (tile-exact) / residue-GEMM GPU time"},
        "slice_sweep": sweep,
        "clocks": clk.summary(),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="uvatrmm", choices=["uvatrmm", "reference"])
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-n", type=int, default=16384)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-check", dest="check", action="store_false")
    ap.add_argument("--no-ozaki", action="store_true")
    ap.add_argument("--ozaki-n", type=int, default=32768)
    ap.add_argument("--ozaki-steps", type=int, default=3)
    ap.add_argument("--ozaki-raster", type=int, default=0,
                    help="residue-GEMM raster group (pair rows per group; 0 = library default)")
    ap.add_argument("--no-variants", dest="variants", action="store_false")
    ap.add_argument("--big-n", type=int, default=32768)
    ap.add_argument("--next-n", type=int, default=8192)
    ap.add_argument("--next-steps", type=int, default=3)
    ap.add_argument("--batch", type=int, default=2000)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--serve", type=int, default=300, help="distinct request operand sets (0: no serving run)")
    ap.add_argument("--serve-seconds", type=float, default=20.0, help="seconds of arrivals per rate")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[50.0, 100.0, 150.0, 200.0])
    args = ap.parse_args()
    ws, rank, local = dist_env()
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_reference_sample(args.cpu_n, args.steps, args.warmup, threads)
        line = {"impl": "reference", "metric": METRIC, "value": round(cb["value"], 5), "unit": "TFLOP/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform[-1,1))",
                "config": headline_config(args.n, args.n, ws),
                "cpu_baseline": cb,
                "e2e": {"value": round(cb["value"], 5), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    if ws > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_gpu(args, ws, rank, local)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = _guarded(cpu_reference_sample, args.cpu_n, 1, 1, threads)
    if rank == 0:
        out["summary"] = summary(out)
    if ws > 1:
        import torch
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
