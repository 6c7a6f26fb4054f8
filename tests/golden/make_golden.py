"""Writes the golden fixtures in this folder by running the reference itself.

Needs oracle/_ref/ (built from the reference sources by oracle/build_ref.sh);
the committed JSON files are what the tests read, so the GPU machine never needs
the reference.

  norms.json        ||C||_inf printed by `uvatrmm.x <n> <reg|balanced> <boxes|trapezoid>`
                    (UVaTRMM/src/mm_triangular_common.c:2986-2988), one rank
  mappings.json     (begin, size) of map_regular / map_balanced for many (n, P)
                    (UVaTRMM/src/mm_mapping.c:27-67, :319-366), via oracle/_ref/ref_harness
  consecutive.json  blocks made by mat_consecutive_values
                    (UVaTRMM/src/mm_triangular_common.c:1782-1805), via ref_harness
  cli_stdout.txt    one full stdout of `uvatrmm.x 64 balanced trapezoid` (format pin)
  result_files.json bytes of result files written by print_output_results_generic
                    (UVaTRMM/src/mm_triangular_common.c:2134-2163), via ref_harness

Usage: python tests/golden/make_golden.py   (after oracle/build_ref.sh)
"""
import json
import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "..", "..", "oracle", "_ref")
UVATRMM = os.path.join(REF, "uvatrmm.x")
HARNESS = os.path.join(REF, "ref_harness")


def run(args, cwd=None):
    return subprocess.run(args, check=True, capture_output=True, text=True, cwd=cwd).stdout


def main():
    if not (os.path.exists(UVATRMM) and os.path.exists(HARNESS)):
        raise SystemExit("run oracle/build_ref.sh first")
    norms = {}
    with tempfile.TemporaryDirectory() as tmp:
        for n in (1, 2, 3, 8, 17, 64, 100, 512, 1000, 2048, 4096):
            norms[str(n)] = {}
            for mp in ("reg", "balanced"):
                for shape in ("boxes", "trapezoid"):
                    if n == 4096 and (mp, shape) != ("balanced", "trapezoid"):
                        continue
                    out = run([UVATRMM, str(n), mp, shape], cwd=tmp)
                    m = re.search(r"Norm: ([0-9.]+)", out)
                    norms[str(n)][f"{mp}/{shape}"] = m.group(1)
                    with open(os.path.join(tmp, "norm_ff.txt")) as f:
                        assert f.read() == m.group(1)
        stdout = run([UVATRMM, "64", "balanced", "trapezoid"], cwd=tmp)
    with open(os.path.join(HERE, "norms.json"), "w") as f:
        json.dump({"source": "oracle/_ref/uvatrmm.x (reference, one rank)", "norms": norms}, f, indent=1)
    with open(os.path.join(HERE, "cli_stdout.txt"), "w") as f:
        f.write(re.sub(r"[0-9]+\.[0-9]{6}", "T", stdout))

    maps = []
    for n in (1, 2, 3, 4, 5, 7, 8, 10, 16, 17, 64, 100, 1000, 4096, 16384, 32768, 65536):
        for P in (1, 2, 3, 4, 5, 6, 7, 8, 16, 76, 152, 304):
            if P > n:
                continue
            entry = {"n": n, "P": P}
            for mode in ("reg", "balanced"):
                r = subprocess.run([HARNESS, "maps", str(n), str(P), mode], capture_output=True, text=True)
                entry[mode] = [[int(x) for x in line.split()[1:]] for line in r.stdout.split("\n") if line.strip()]
                entry[mode + "_exit"] = r.returncode
            maps.append(entry)
    with open(os.path.join(HERE, "mappings.json"), "w") as f:
        json.dump({"source": "reference map_regular/map_balanced via oracle/_ref/ref_harness",
                   "cases": maps}, f)

    blocks = []
    for (n, rb, rows, cb, cols, tri) in [(8, 0, 8, 0, 8, 1), (8, 0, 8, 0, 8, 0), (13, 3, 5, 0, 13, 1),
                                         (13, 0, 13, 4, 3, 0), (50, 10, 7, 0, 50, 1), (3000, 2990, 2, 0, 3000, 1)]:
        vals = run([HARNESS, "gen", str(n), str(rb), str(rows), str(cb), str(cols), str(tri)]).split()
        blocks.append({"n": n, "rows_begin": rb, "rows": rows, "cols_begin": cb, "cols": cols,
                       "triangular": tri, "values": [float.fromhex(float(v).hex()) for v in vals]})
    with open(os.path.join(HERE, "consecutive.json"), "w") as f:
        json.dump({"source": "reference mat_consecutive_values (-DMININUMS=1) via oracle/_ref/ref_harness",
                   "blocks": blocks}, f)

    # Result files written by the reference's own print_output_results_generic.
    results = []
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "tests", "outputs"))
        for (rows, cols, rb, nr, cb, nc, rank, procs) in [(5, 7, 0, 5, 2, 3, 1, 4), (6, 6, 2, 3, 0, 6, 0, 2),
                                                           (4, 9, 0, 4, 0, 0, 3, 4), (1, 1, 0, 1, 0, 1, 0, 1)]:
            run([HARNESS, "result", str(rows), str(cols), str(rb), str(nr), str(cb), str(nc), str(rank),
                 str(procs)], cwd=tmp)
            path = os.path.join(tmp, "tests", "outputs", f"output_golden.{rows}.{procs}.{rank}.dat")
            with open(path, "rb") as f:
                results.append({"args": [rows, cols, rb, nr, cb, nc, rank, procs], "hex": f.read().hex()})
    with open(os.path.join(HERE, "result_files.json"), "w") as f:
        json.dump({"source": "reference print_output_results_generic via oracle/_ref/ref_harness; "
                   "block entries 0.25*k + 1/3 row-major", "files": results}, f, indent=1)
    print("wrote norms.json, mappings.json, consecutive.json, cli_stdout.txt, result_files.json")


if __name__ == "__main__":
    main()
