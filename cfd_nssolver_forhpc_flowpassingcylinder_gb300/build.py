"""Build libcfdgb.so in-tree: every CUDA translation unit compiled for sm_103a in
parallel, then linked with nvcc.  No torch, no cmake; a minute at most."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcfdgb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", str(ROOT / "include"), "-I", str(CSRC)]
# Per-file flags.  step_exact.cu reproduces the reference's FP64 arithmetic bit for bit:
# no fused multiply-add contraction, IEEE division and square root.
PER_FILE = {
    "step_exact.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    # the adjoint re-derives the forward branch decisions with the same arithmetic
    "adjoint.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
}
SOURCES = ["api.cu", "step_exact.cu", "step_fast.cu", "solver.cu", "multigrid.cu", "adjoint.cu", "noalloc.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "cfdgb.h"]
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        if force or _stale(o, [s, *headers, Path(__file__)]):
            cmd = [nvcc(), *ARCH, *COMMON, *PER_FILE.get(src, []), *extra_flags, "-c", str(s), "-o", str(o)]
            jobs.append((src, cmd))
    objs = [BUILD / (s + ".o") for s in SOURCES]

    def run(job):
        name, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr[-6000:]}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return name

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(tmp, LIB)
    cli = PKG / "cfdgb_run"
    cli_src = CSRC / "cfdgb_run.cpp"
    if force or _stale(cli, [cli_src, LIB, ROOT / "include" / "cfdgb.hpp"]):
        cmd = ["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(cli_src), "-L", str(PKG), "-lcfdgb",
               "-Wl,-rpath,$ORIGIN", "-o", str(cli)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cfdgb_run build failed:\n" + r.stderr[-4000:])
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    build(force="--force" in sys.argv, verbose=v,
          extra_flags=["-Xptxas", "-v"] if v else [])
    print(LIB)
