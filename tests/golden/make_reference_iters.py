#!/usr/bin/env python3
"""Record the reference's own BiCGSTAB iteration counts on a bench workload.

Runs the reference harness (oracle/build_ref.py, native flavour) with FULL solves to
relative residual 1e-8 (Jacobi-scaled CSR rows, the workload's solver) for --steps steps
and writes reference_iters_<workload>.json beside this file: iterations per step and the
reference's own per-step wall times.  bench.py evaluates the reference's CPU throughput
at these counts from a bounded timing sample (one full C2 step takes ~5 min on 4 cores).
The case's solver and tolerance are its own (bench.WORKLOADS: Jacobi-BiCGSTAB to 1e-8, or
the reference's default SPE-BiCGSTAB to 1e-3 on its stretched grid for `ref`).

    python tests/golden/make_reference_iters.py --workload c2 --steps 13 --threads 6
    python tests/golden/make_reference_iters.py --workload c2 --from-stats <run dir>/stats.txt
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def main():
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--from-stats", default=None, help="reuse a finished harness run's stats.txt")
    a = ap.parse_args()
    cfg = bench.WORKLOADS[a.workload]
    exe, hsolver, tol = bench.reference_build(a.workload)
    if a.from_stats:
        text = Path(a.from_stats).read_text()
    else:
        with tempfile.TemporaryDirectory() as td:
            env = dict(os.environ, OMP_NUM_THREADS=str(a.threads), OMP_PROC_BIND="close")
            subprocess.run([str(exe), "run", str(a.steps), repr(cfg["Re"]), repr(cfg["dt"]), repr(tol), hsolver,
                            "1.7", "0", "0", td], check=True, env=env, cwd=td, stdout=subprocess.DEVNULL)
            text = (Path(td) / "stats.txt").read_text()
    rows = [l.split() for l in text.splitlines() if l and not l.startswith("#")]
    iters = [int(r[2]) for r in rows]
    out = {"workload": a.workload,
           "solver": {"csr": "csr (Jacobi-scaled) bicgstabRe2", "spe": "spe bicgstabRe2"}[hsolver], "tol": tol,
           "steps": len(rows), "iters": iters, "relres": [float(r[3]) for r in rows],
           "t_step_s": [float(r[6]) for r in rows], "t_solve_s": [float(r[7]) for r in rows],
           "threads": a.threads, "host": platform.machine(),
           "note": "index 0 is step 1 (no pressure solve, RUN_CPU.cpp:303)"}
    (HERE / f"reference_iters_{a.workload}.json").write_text(json.dumps(out, indent=1) + "\n")
    print(out["iters"])


if __name__ == "__main__":
    main()
