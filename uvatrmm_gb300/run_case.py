"""Runs one TRMM configuration a few times through the C ABI (for profilers).

    python -m uvatrmm_gb300.run_case --tier fp64 --engine dmma --m 4096 --n 4096 --reps 2
    python -m uvatrmm_gb300.run_case --tier ozaki --m 6144 --reps 2

Operands are seeded uniform[-1,1) (column-major, device-resident, generated
by the library); the product is B := op(A) B (side Left) or B op(A) (side
Right), out of place for the FP64 tier and in place for the Ozaki tier.
Prints the mean wall time per call after one untimed call; the kernels'
own time is what a profiler reads.
"""
from __future__ import annotations

import argparse
import time


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--tier", choices=["fp64", "ozaki"], default="fp64")
    ap.add_argument("--engine", choices=["dfma", "dmma"], default="dfma")
    ap.add_argument("--m", type=int, default=4096)
    ap.add_argument("--n", type=int, default=0, help="0: same as m")
    ap.add_argument("--side", choices=["L", "R"], default="L")
    ap.add_argument("--uplo", choices=["L", "U"], default="L")
    ap.add_argument("--trans", choices=["N", "T"], default="N")
    ap.add_argument("--moduli", type=int, default=0)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()

    import torch

    import uvatrmm_gb300 as u
    m, n = a.m, a.n or a.m
    side = u.LEFT if a.side == "L" else u.RIGHT
    uplo = u.LOWER if a.uplo == "L" else u.UPPER
    trans = u.NOTRANS if a.trans == "N" else u.TRANS
    ka = m if side == u.LEFT else n
    h = u.Handle()
    h.set_option("engine", u.ENGINE_DMMA if a.engine == "dmma" else u.ENGINE_DFMA)
    dA = torch.empty(ka * ka, dtype=torch.float64, device="cuda")
    dB = torch.empty(m * n, dtype=torch.float64, device="cuda")
    h.gen_uniform(1, 0, ka, ka, dA, 1, ka, tri=a.uplo)
    h.gen_uniform(1, 1, m, n, dB, 1, m)
    dC = torch.empty_like(dB) if a.tier == "fp64" else None
    h.sync()

    def call():
        if a.tier == "fp64":
            h.dtrmm_device_oop(u.COL, side, uplo, trans, u.NONUNIT, m, n, 1.0, dA, ka, dB, m, dC, m)
        else:
            h.ozaki_device(u.COL, side, uplo, trans, u.NONUNIT, m, n, 1.0, dA, ka, dB, m, moduli=a.moduli)
        h.sync()

    call()
    t0 = time.perf_counter()
    for _ in range(a.reps):
        call()
    dt = (time.perf_counter() - t0) / max(a.reps, 1)
    flops = float(ka) * ka * (n if side == u.LEFT else m)
    print(f"{a.tier} {a.engine} m={m} n={n}: {dt * 1e3:.2f} ms per call, {flops / dt / 1e12:.3f} TFLOP/s (wall)")
    h.close()


if __name__ == "__main__":
    main()
