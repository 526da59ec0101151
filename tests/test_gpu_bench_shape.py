"""Parity on the launch shape of the 512x256x64 benchmark grid.

The grid-stride kernels pick their k-block width from nz (32 lanes for nz = 64), and the
FP32 bulk-copy pipeline tiles tj = 256 / (nz / 4) = 16 rows per block there.  The other
whole-step tests use nz <= 13, so this file runs nz = 64 with the benchmark's spacing
(1/16), Reynolds number and time step: 128x64x64 cells over [0,8]x[0,4]x[0,4], the D=1
cylinder at (2,2), Re 200, dt 0.002, Jacobi-scaled BiCGSTAB (the benchmark's solver).

FP64 against the oracle run live, both solving to 1e-13: u, v, w and mean-free p within
1e-10 relative, drag within 1e-10.  The FP32+FP64-refined paths that the benchmark times
(BiCGSTAB sweeps, CG sweeps and the multigrid-preconditioned sweeps, all on the bulk-copy
pipeline at this shape) against the FP64 GPU run: every solve below its 1e-10 tolerance,
velocity within 1e-8 and mean-free p within 1e-6 of FP64."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASE = dict(nx=128, ny=64, nz=64, lx=8.0, ly=4.0, lz=4.0, cx=2.0, cy=2.0, Re=200.0, dt=0.002)
BSET = dict(walls="free_slip", bc_z="periodic", outflow="convective")
STEPS = 3


def vel_err(f, ref):
    core = (slice(2, -2),) * 3
    scale = np.sqrt(sum(np.linalg.norm(ref[k][core]) ** 2 for k in "uvw"))
    return {k: float(np.linalg.norm(f[k][core] - ref[k][core]) / scale) for k in "uvw"}


def p_err(a, b):
    a, b = a[2:-2, 2:-2, 2:-2], b[2:-2, 2:-2, 2:-2]
    a, b = a - a.mean(), b - b.mean()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def fp64_run():
    with cg.Solver(solver="jacobi", tol=1e-13, **CASE) as s:
        s.init_fields()
        st = s.step(STEPS)
        f = s.get_fields()
    return st, f


def test_fp64_matches_oracle_at_nz64(fp64_run):
    st, f = fp64_run
    g = O.Grid(CASE["nx"], CASE["ny"], CASE["nz"], CASE["lx"], CASE["ly"], CASE["lz"], CASE["cx"])
    ref = O.run(g, STEPS, CASE["Re"], CASE["dt"], 1e-13, "csr")
    assert [r.status for r in st] == [0] * STEPS
    assert all(r.relres < 1e-13 for r in st[1:]), [r.relres for r in st]
    for k, e in vel_err(f, ref).items():
        assert e <= 1e-10, (k, e)
    assert p_err(f["p"], ref["p"]) <= 1e-10
    np.testing.assert_allclose([r.cd for r in st], ref["cd"], rtol=1e-10)
    np.testing.assert_allclose([r.cl for r in st], ref["cl"], rtol=1e-10, atol=1e-12)
    # iteration counts: two correct solvers near the rounding floor agree to a few percent
    it, rit = np.array([r.iters for r in st]), np.asarray(ref["iters"])
    assert np.all(np.abs(it[1:] - rit[1:]) <= 0.1 * rit[1:]), (it, rit)


@pytest.fixture(scope="module")
def fp64_set_run():
    with cg.Solver(solver="jacobi", tol=1e-12, amp=1e-3, seed=5, **BSET, **CASE) as s:
        s.init_fields()
        st = s.step(STEPS)
        f = s.get_fields()
    return st, f


@pytest.mark.parametrize("kw", [dict(solver="jacobi"), dict(solver="cg"),
                                dict(solver="jacobi", precond="multigrid")],
                         ids=["bicgstab", "cg", "multigrid"])
def test_mixed_paths_on_the_boundary_set_at_nz64(fp64_set_run, kw):
    """The boundary set (convective outflow, free-slip walls, periodic z) at this shape: the
    bulk-copy and quad kernels take the cells across the wrap at each line's ends (16 quads
    a line, two lines a warp).  Every FP64 solve reaches 1e-12 (the flux-corrected problem
    is consistent); the MIXED runs end below 1e-10 and agree with FP64 as above."""
    st64, f64 = fp64_set_run
    assert [r.status for r in st64] == [0] * STEPS
    assert all(r.relres < 1e-12 for r in st64[1:]), [r.relres for r in st64]
    with cg.Solver(precision="mixed", tol=1e-10, amp=1e-3, seed=5, **kw, **BSET, **CASE) as s:
        s.init_fields()
        st = s.step(STEPS)
        f = s.get_fields()
    assert [r.status for r in st] == [0] * STEPS
    assert all(r.relres < 1e-10 for r in st[1:]), [r.relres for r in st]
    for k, e in vel_err(f, f64).items():
        assert e <= 1e-8, (kw, k, e)
    assert p_err(f["p"], f64["p"]) <= 1e-6, kw
    np.testing.assert_allclose([r.cd for r in st], [r.cd for r in st64], rtol=1e-8)


@pytest.mark.parametrize("kw", [dict(solver="jacobi"), dict(solver="cg"),
                                dict(solver="jacobi", precond="multigrid")],
                         ids=["bicgstab", "cg", "multigrid"])
def test_mixed_paths_match_fp64_at_nz64(fp64_run, kw):
    st64, f64 = fp64_run
    with cg.Solver(precision="mixed", tol=1e-10, **kw, **CASE) as s:
        s.init_fields()
        st = s.step(STEPS)
        f = s.get_fields()
    assert [r.status for r in st] == [0] * STEPS
    assert all(r.relres < 1e-10 for r in st[1:]), [r.relres for r in st]
    for k, e in vel_err(f, f64).items():
        assert e <= 1e-8, (kw, k, e)
    assert p_err(f["p"], f64["p"]) <= 1e-6, kw
    np.testing.assert_allclose([r.cd for r in st], [r.cd for r in st64], rtol=1e-8)
