"""The C++ shim (include/cfdgb.hpp) and the command-line driver on the GPU: a driver written
in the reference's call shapes (tests/shim_driver.cpp) against the oracle, and cfdgb_run
with a Plot3D restart."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
PKG = Path(cg.__file__).resolve().parent


def test_reference_shaped_driver_matches_oracle(tmp_path):
    exe = tmp_path / "shim_driver"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "shim_driver.cpp"),
                    "-o", str(exe), "-L", str(PKG), "-lcfdgb", f"-Wl,-rpath,{PKG}"], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], check=True, capture_output=True, text=True).stdout.split("\n")
    vals = {}
    for line in out:
        f = line.split()
        if f:
            vals.setdefault(f[0], []).append(f[1:])
    cd = np.array([float(x[1]) for x in vals["cd"]])
    g = O.Grid(96, 48, 4, 24.0, 12.0, 1.0, 6.0)
    ref = O.run(g, 3, 100.0, 0.005, 1e-12, "spe")
    np.testing.assert_allclose(cd, ref["cd"], rtol=1e-10)
    assert 0.0 < float(vals["cfl"][0][0]) < 1.0
    assert float(vals["viseff_max"][0][0]) > 0.0
    nb, reyn, time, n = vals["qfile"][0]
    assert (int(nb), float(reyn), float(time), int(n)) == (1, 100.0, 0.5, 100 * 52 * 8)


def test_cli_run_and_restart(tmp_path):
    cli = PKG / "cfdgb_run"
    base = ["nx=96", "ny=48", "nz=4", "lx=24", "ly=12", "lz=1", "cx=6", "cy=6", "Re=100", "dt=0.005", "tol=1e-12"]
    subprocess.run([str(cli), *base, "steps=4", "p3d=2", f"out={tmp_path}/a"], check=True, capture_output=True)
    cd_a = np.loadtxt(tmp_path / "a" / "Time_cDcL.dat", skiprows=3)
    g = O.Grid(96, 48, 4, 24.0, 12.0, 1.0, 6.0)
    ref = O.run(g, 4, 100.0, 0.005, 1e-12, "spe")
    np.testing.assert_allclose(cd_a[:, 1], ref["cd"], rtol=1e-10)
    q = tmp_path / "a" / "P3D02.q"
    assert q.stat().st_size == 32 + 5 * 4 * 96 * 48 * 4
    # restart from the step-4 file: the simulated time continues from its header
    subprocess.run([str(cli), *base, "steps=1", f"restart={q}", f"out={tmp_path}/b"], check=True, capture_output=True)
    cd_b = np.loadtxt(tmp_path / "b" / "Time_cDcL.dat", skiprows=3, ndmin=2)
    assert abs(cd_b[0, 0] - 0.02) < 1e-9 and np.isfinite(cd_b[0, 1])
