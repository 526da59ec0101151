#!/usr/bin/env python3
"""Recipe that builds the UNMODIFIED reference solver functions as an oracle binary.

Test infrastructure only: nothing in the shipped library imports or links this.

The reference (jimmy3769tw/CFD_NSsolver_forHPC_flowPassingCylinder) fixes its grid,
domain and cylinder position as compile-time ``const`` members, so every grid needs
its own compile.  This recipe

1. copies the reference's ``inc/`` tree into ``oracle/_ref/src/inc`` (git-ignored build
   output; the repository never holds reference sources),
2. rewrites exactly five literals so they read from ``-D`` macros instead:
   ``inc/grid/structureGrid.hpp:20`` (Gridder), ``:28`` (lx, ly, lz),
   ``:38-40`` (nxCal, nyCal, nzCal) and ``inc/dfib/setEta.hpp:145`` (center_x);
   puts the convection switch ``#define CONVECTION_DIFUSSION_QUICK``
   (``inc/0_General.hpp:114``) under ``#ifndef ORACLE_SCHEME_SET`` so that a build can
   name LUD or UD; turns the v entries of the y-wall rows of the boundary table
   (``inc/BoundaryCondition/FLOWpassing.hpp:25,29``) into a macro, so that a build can
   take the free-slip rows the reference leaves commented out (``:14-21``); and corrects
   the one misspelt token (``auot``) that keeps the
   Smagorinsky model (``inc/source/SmagorinskyModel.hpp:61``) from compiling, for the
   builds that switch it on.  Every other line is the reference's own,
3. compiles ``oracle/ref_harness.cpp`` (our driver, which calls the reference's own
   functions in the order of ``src/RUN_CPU.cpp:257-436``) once per grid into
   ``oracle/_ref/bin/ref_<nx>x<ny>x<nz>_<tag>``.

Two flavours are built per grid:

* ``parity``: ``-O3 -fopenmp -ffp-contract=off`` so that its arithmetic is the plain
  IEEE order of the source (the C restatement in ``oracle/cfd_oracle.c`` is built the
  same way and matches it bit for bit at one OpenMP thread);
* ``native``: the reference's own ``Makefile:7,24`` flags (``-O3 -fopenmp
  -march=native``), used only to time the reference CPU path.

When the reference tree is absent (the GPU host), the patched copy already under
``oracle/_ref/src`` is compiled instead, if present.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference tree this recipe reads: --reference-root, else CFD_REFERENCE_ROOT, else the
# location where this build's container mounts it (read-only).  Nothing but this recipe and
# the fixture scripts beside the goldens reads it; the GPU host uses the staged copy.
DEFAULT_REF_ROOT = "/root/reference"
REF_ROOT = Path(os.environ.get("CFD_REFERENCE_ROOT", DEFAULT_REF_ROOT))


def set_reference_root(path) -> None:
    """Read the reference tree from `path` instead (the --reference-root option)."""
    global REF_ROOT
    REF_ROOT = Path(path)
OUT = HERE / "_ref"
SRC = OUT / "src"
BIN = OUT / "bin"

# (file, literal in the reference, replacement)
PATCHES = [
    ("inc/grid/structureGrid.hpp",
     'const std::string Gridder = "non_uniform-SML";',
     "const std::string Gridder = ORACLE_GRIDDER;"),
    ("inc/grid/structureGrid.hpp",
     "const double  lx = 17.0 ,      ly = 12.0 ,      lz = 3.0 ;",
     "const double  lx = ORACLE_LX ,      ly = ORACLE_LY ,      lz = ORACLE_LZ ;"),
    ("inc/grid/structureGrid.hpp",
     "const int       nxCal = 190,     // nx should > 40",
     "const int       nxCal = ORACLE_NX,"),
    ("inc/grid/structureGrid.hpp",
     "                        nyCal = 210,\n                        nzCal = 40;",
     "                        nyCal = ORACLE_NY,\n                        nzCal = ORACLE_NZ;"),
    ("inc/dfib/setEta.hpp",
     "double  center_x    = 6.5, ",
     "double  center_x    = ORACLE_CX, "),
    # the convection switch: QUICK unless the build names another scheme
    ("inc/0_General.hpp",
     "\n#define CONVECTION_DIFUSSION_QUICK\n",
     "\n#ifndef ORACLE_SCHEME_SET\n#define CONVECTION_DIFUSSION_QUICK\n#endif\n"),
    # the y-wall rows of the boundary table: v zero-gradient (active) or, for the builds
    # with the free-slip rows the reference leaves commented out, Dirichlet 0
    ("inc/BoundaryCondition/FLOWpassing.hpp",
     "Dir[2][1] = 0.;/* 2 */Num[2][1] = 1.;",
     "Dir[2][1] = 0.;/* 2 */Num[2][1] = ORACLE_WALL_NUM_V;"),
    ("inc/BoundaryCondition/FLOWpassing.hpp",
     "Dir[3][1] = 0.;/* 3 */Num[3][1] = 1.;",
     "Dir[3][1] = 0.;/* 3 */Num[3][1] = ORACLE_WALL_NUM_V;"),
    # the Smagorinsky model does not compile as published (a misspelt `auto`); this one
    # token is the whole fix, and it only matters to builds with TERBULENCE_SMAGORINSKY
    ("inc/source/SmagorinskyModel.hpp",
     "const auot icelCal",
     "const auto icelCal"),
]
# the staged copy is redone whenever the patch list changes
PATCH_SIGNATURE = repr(PATCHES)


def stage_sources(force: bool = False) -> Path:
    """Copy + patch the reference headers into oracle/_ref/src (idempotent)."""
    stamp = SRC / ".patched"
    if stamp.exists() and not force and stamp.read_text() == PATCH_SIGNATURE:
        return SRC
    if not (REF_ROOT / "inc").is_dir():
        if stamp.exists():
            return SRC
        raise FileNotFoundError(
            f"reference tree not found at {REF_ROOT} and no staged copy in {SRC}")
    if SRC.exists():
        shutil.rmtree(SRC)
    SRC.mkdir(parents=True)
    # amgcl / yakutat are never included by the live path; skip them to keep the copy small
    def _ignore(d, names):
        if Path(d).resolve() == (REF_ROOT / "inc").resolve():
            return [n for n in names if n in ("amgcl", "yakutat")]
        return []
    shutil.copytree(REF_ROOT / "inc", SRC / "inc", ignore=_ignore)
    for rel, old, new in PATCHES:
        f = SRC / rel
        text = f.read_text()
        n = text.count(old)
        if n != 1:
            raise RuntimeError(f"patch anchor found {n} times in {rel}: {old!r}")
        f.write_text(text.replace(old, new))
    stamp.write_text(PATCH_SIGNATURE)
    return SRC


GRIDDERS = {"uniform": "uniform", "sml": "non_uniform-SML"}  # structureGrid.hpp:19-20


SCHEMES = {"quick": "CONVECTION_DIFUSSION_QUICK", "lud": "CONVECTION_DIFUSSION_LUD",
           "ud": "CONVECTION_DIFUSSION_UD"}  # 0_General.hpp:114-118


def binary_name(nx: int, ny: int, nz: int, flavour: str, gridder: str = "uniform", scheme: str = "quick",
                les: bool = False, walls: str = "zero_gradient") -> Path:
    tag = "" if gridder == "uniform" else f"_{gridder}"
    tag += "" if scheme == "quick" else f"_{scheme}"
    tag += "_les" if les else ""
    tag += "" if walls == "zero_gradient" else "_freeslip"
    return BIN / f"ref_{nx}x{ny}x{nz}{tag}_{flavour}"


def build(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float, cx: float,
          flavour: str = "parity", force: bool = False, gridder: str = "uniform", scheme: str = "quick",
          les: bool = False, walls: str = "zero_gradient") -> Path:
    """Compile the harness for one grid; returns the binary path.  gridder: "uniform" or
    "sml" (the reference's own default, non_uniform-SML); scheme: "quick", "lud" or "ud"
    (the convection switch); les: TERBULENCE_SMAGORINSKY; walls: "zero_gradient" (the
    active boundary rows) or "free_slip" (the rows left commented out)."""
    src = stage_sources()
    BIN.mkdir(parents=True, exist_ok=True)
    exe = binary_name(nx, ny, nz, flavour, gridder, scheme, les, walls)
    # the domain is part of the name only through a sidecar, so check it too
    sidecar = exe.with_suffix(".cfg")
    cfg = f"{nx} {ny} {nz} {lx!r} {ly!r} {lz!r} {cx!r} {gridder} {scheme} {int(les)} {walls}\n"
    harness = HERE / "ref_harness.cpp"
    if (exe.exists() and not force and sidecar.exists() and sidecar.read_text() == cfg
            and exe.stat().st_mtime >= harness.stat().st_mtime):
        return exe
    if flavour == "parity":
        flags = ["-O3", "-fopenmp", "-ffp-contract=off"]
    elif flavour == "native":
        flags = ["-O3", "-fopenmp", "-march=native"]
    else:
        raise ValueError(flavour)
    defs = [f"-DORACLE_NX={nx}", f"-DORACLE_NY={ny}", f"-DORACLE_NZ={nz}",
            f"-DORACLE_LX={lx!r}", f"-DORACLE_LY={ly!r}", f"-DORACLE_LZ={lz!r}",
            f"-DORACLE_CX={cx!r}", f'-DORACLE_GRIDDER="{GRIDDERS[gridder]}"']
    if scheme != "quick":
        defs += ["-DORACLE_SCHEME_SET", f"-D{SCHEMES[scheme]}"]
    if les:
        defs += ["-DTERBULENCE_SMAGORINSKY"]
    defs += [f"-DORACLE_WALL_NUM_V={'0.' if walls == 'free_slip' else '1.'}"]
    cmd = (["g++", "-std=c++17", "-w"] + flags + defs +
           ["-I", str(src / "inc"), str(harness), "-o", str(exe)])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and flavour == "native":
        # e.g. a compiler without -march=native support: fall back to portable flags
        cmd = [c for c in cmd if c != "-march=native"]
        r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference harness build failed:\n" + r.stderr[-4000:])
    sidecar.write_text(cfg)
    return exe


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--grid", nargs=3, type=int, default=[96, 48, 4])
    ap.add_argument("--domain", nargs=3, type=float, default=[24.0, 12.0, 1.0])
    ap.add_argument("--cx", type=float, default=6.0)
    ap.add_argument("--flavour", default="parity", choices=["parity", "native"])
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--reference-root", default=None,
                    help="the reference project's root (default: $CFD_REFERENCE_ROOT or " + DEFAULT_REF_ROOT + ")")
    a = ap.parse_args(argv)
    if a.reference_root:
        set_reference_root(a.reference_root)
    exe = build(*a.grid, *a.domain, a.cx, flavour=a.flavour, force=a.force)
    print(exe)


if __name__ == "__main__":
    sys.exit(main())
