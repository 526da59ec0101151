#!/usr/bin/env python3
"""Regenerate the golden vectors from the reference's OWN code.

Builds the reference harness (oracle/build_ref.py: the reference's headers with only the
grid/domain/cylinder literals turned into -D macros, driven by oracle/ref_harness.cpp)
and runs it at ONE OpenMP thread, so that its in-place loops run in the sequential
order.  Needs the reference tree (this container), not a GPU.

Fixtures written next to this file:
  unit_<grid>.npz   every hot-path function once on seeded random fields
                    (inputs and outputs, padded layout), the CFL diagnostic, the
                    bytes of the reference's Plot3D .x and .q files and what its
                    reader (QfileRead) makes of the .q file
  unit_<grid>_variants.npz
                    ConvectionDifussion of the same fields with the LUD scheme and with
                    the Smagorinsky model (its eddy viscosity too); the ghost fill and copy
                    with the free-slip wall rows of the boundary table
  run_<case>.npz    whole runs of the 96x48x4 flow-past-cylinder case (reference BCs,
                    Re 100, dt 0.005; also with LUD, with the Smagorinsky model and with
                    free-slip walls) and of
                    the stretched SML grid: interior of the final u, v, w, p and the
                    per-step iterations, residual, Cd and Cl.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
from oracle import build_ref  # noqa: E402

UNIT_GRIDS = {
    # name: (nxc, nyc, nzc, lx, ly, lz, cx)
    "g10x8x6_h025": (10, 8, 6, 2.5, 2.0, 1.5, 1.25),
    "g10x8x6_h030": (10, 8, 6, 3.0, 2.4, 1.8, 1.5),
}
C1 = (96, 48, 4, 24.0, 12.0, 1.0, 6.0)
RUNS = {
    # name: (steps, Re, dt, tol, solver, omega)
    "c1_spe_tol1e-8_200": (200, 100.0, 0.005, 1e-8, "spe", 1.8),
    "c1_spe_tol1e-13_20": (20, 100.0, 0.005, 1e-13, "spe", 1.8),
    "c1_csr_tol1e-13_20": (20, 100.0, 0.005, 1e-13, "csr", 1.8),
    "c1_sor_tol1e-3_4": (4, 100.0, 0.005, 1e-3, "sor", 1.8),
}
# the reference's default stretched grid (non_uniform-SML) at the smallest sizes its
# unit_SML accepts (100 fine cells per x/y axis), on its default domain 17 x 12 x 3 with
# the cylinder at (6.5, 6); tol 1e-3, the tolerance the reference's default case runs at
# (with its zero-gradient boundaries the stretched Neumann problem is not consistent, and
# its own BiCGSTAB hits the cap from step 3 at 1e-6 and tighter)
SML = (120, 110, 4, 17.0, 12.0, 3.0, 6.5)
SML_RUNS = {
    # name: (steps, Re, dt, tol, solver, omega, fields stored)
    "sml_spe_tol1e-3_10": (10, 100.0, 0.005, 1e-3, "spe", 1.8, ("u", "v", "w", "p")),
    "sml_csr_tol1e-3_10": (10, 100.0, 0.005, 1e-3, "csr", 1.8, ("p",)),
}
UNIT_SEED = 7
UNIT_RE, UNIT_DT = 100.0, 0.005


def _env():
    e = dict(os.environ)
    e["OMP_NUM_THREADS"] = "1"
    return e


def _load_dir(d: Path) -> dict:
    out = {}
    for f in sorted(d.glob("*.f64")):
        out[f.stem] = np.fromfile(f, dtype="<f8")
    for f in sorted(d.glob("*.bin")):  # files the reference writes itself (Plot3D)
        out[f.stem] = np.fromfile(f, dtype=np.uint8)
    return out


def make_unit(name, spec):
    nxc, nyc, nzc, lx, ly, lz, cx = spec
    exe = build_ref.build(nxc, nyc, nzc, lx, ly, lz, cx, "parity")
    with tempfile.TemporaryDirectory() as td:
        # the reference's Plot3D writers use ./mx_out and ../mx_out: run one level down
        wd = Path(td) / "run"
        wd.mkdir()
        subprocess.run([str(exe), "unit", str(UNIT_SEED), repr(UNIT_RE), repr(UNIT_DT), td],
                       check=True, env=_env(), stdout=subprocess.DEVNULL, cwd=wd)
        arrs = _load_dir(Path(td))
    meta = np.array([nxc, nyc, nzc, lx, ly, lz, cx, UNIT_RE, UNIT_DT, UNIT_SEED], dtype=np.float64)
    np.savez_compressed(HERE / f"unit_{name}.npz", meta=meta, **arrs)


# builds of the reference with its other convection scheme (LUD) and with its Smagorinsky
# model switched on; UD does not compile as published (the uniform-grid variant's UdUnit
# calls, Convection_Difussion.uniformGrid.hpp:143-144, match no overload)
VARIANTS = {"lud": dict(scheme="lud"), "les": dict(les=True), "freeslip": dict(walls="free_slip")}


def make_unit_variants(name, spec):
    """unit_<grid>_variants.npz: ConvectionDifussion of the same seeded fields under LUD
    (cd_lud_*) and with the Smagorinsky eddy viscosity (les_nut, cd_les_*)."""
    nxc, nyc, nzc, lx, ly, lz, cx = spec
    base = np.load(HERE / f"unit_{name}.npz")
    out = {}
    for tag, kw in VARIANTS.items():
        exe = build_ref.build(nxc, nyc, nzc, lx, ly, lz, cx, "parity", **kw)
        with tempfile.TemporaryDirectory() as td:
            wd = Path(td) / "run"
            wd.mkdir()
            subprocess.run([str(exe), "unit", str(UNIT_SEED), repr(UNIT_RE), repr(UNIT_DT), td],
                           check=True, env=_env(), stdout=subprocess.DEVNULL, cwd=wd)
            arrs = _load_dir(Path(td))
        for k in ("in_u", "in_v", "in_w"):  # the same seeded inputs as the QUICK fixture
            assert np.array_equal(arrs[k], base[k]), k
        if tag == "freeslip":  # the boundary rows change the ghost fill only
            for k in ("bc_u", "bc_v", "bc_w", "bc_p", "bcc_u", "bcc_v", "bcc_w"):
                out[f"{tag}_{k}"] = arrs[k]
            continue
        for c in ("u", "v", "w"):
            out[f"cd_{tag}_{c}"] = arrs[f"cd_{c}"]
        if "les_nut" in arrs:
            out["les_nut"] = arrs["les_nut"]
    np.savez_compressed(HERE / f"unit_{name}_variants.npz", **out)


# whole runs of the 96x48x4 case with LUD and with the Smagorinsky model
VARIANT_RUNS = {
    # name: (steps, Re, dt, tol, solver, omega, scheme, les)
    "c1_lud_spe_tol1e-13_20": (20, 100.0, 0.005, 1e-13, "spe", 1.8, "lud", False),
    "c1_les_spe_tol1e-13_20": (20, 100.0, 0.005, 1e-13, "spe", 1.8, "quick", True),
    "c1_freeslip_spe_tol1e-13_20": (20, 100.0, 0.005, 1e-13, "spe", 1.8, "quick", False, "free_slip"),
}


def make_run(name, spec, grid=C1, gridder="uniform", keep=("u", "v", "w", "p"), scheme="quick", les=False,
             walls="zero_gradient"):
    nxc, nyc, nzc, lx, ly, lz, cx = grid
    steps, Re, dt, tol, solver, omega = spec
    exe = build_ref.build(nxc, nyc, nzc, lx, ly, lz, cx, "parity", gridder=gridder, scheme=scheme, les=les,
                          walls=walls)
    with tempfile.TemporaryDirectory() as td:
        subprocess.run([str(exe), "run", str(steps), repr(Re), repr(dt), repr(tol), solver,
                        repr(omega), "0", "0", td], check=True, env=_env(),
                       stdout=subprocess.DEVNULL, cwd=td)
        shape = (nxc + 4, nyc + 4, nzc + 4)
        fields = {k: np.fromfile(Path(td) / f"{k}.f64").reshape(shape)[2:-2, 2:-2, 2:-2].copy()
                  for k in keep}
        stats = np.loadtxt(Path(td) / "stats.txt")
    meta = np.array([nxc, nyc, nzc, lx, ly, lz, cx, steps, Re, dt, tol, omega], dtype=np.float64)
    np.savez_compressed(HERE / f"run_{name}.npz", meta=meta, solver=np.array(solver),
                        scheme=np.array(scheme), les=np.array(int(les)), walls=np.array(walls),
                        iters=stats[:, 2].astype(np.int64), err=stats[:, 3], cd=stats[:, 4],
                        cl=stats[:, 5], **fields)


def main():
    for n, s in UNIT_GRIDS.items():
        make_unit(n, s)
        make_unit_variants(n, s)
        print("unit", n)
    for n, s in RUNS.items():
        make_run(n, s)
        print("run", n)
    for n, s in SML_RUNS.items():
        make_run(n, s[:6], grid=SML, gridder="sml", keep=s[6])
        print("run", n)
    for n, s in VARIANT_RUNS.items():
        make_run(n, s[:6], scheme=s[6], les=s[7], walls=s[8] if len(s) > 8 else "zero_gradient")
        print("run", n)


if __name__ == "__main__":
    main()
