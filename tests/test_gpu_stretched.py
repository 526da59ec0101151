"""The reference's default stretched grid (non_uniform-SML, structureGrid.hpp:250-329) on
the GPU: operator and right-hand side bit-exact against the oracle (itself pinned to the
reference's runs on this grid), and whole runs against the reference's own golden runs.

The grid is the smallest unit_SML accepts (120 x 110 x 4 on the reference's default
17 x 12 x 3 domain).  The runs use the reference's working tolerance 1e-3: with its
zero-gradient boundaries the stretched Neumann problem is not consistent and the
reference's own BiCGSTAB hits its cap from step 3 at 1e-6 and tighter."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu
SML = dict(nx=120, ny=110, nz=4, lx=17.0, ly=12.0, lz=3.0, cx=6.5, cy=6.0, grid="sml", Re=100.0, dt=0.005)


@pytest.fixture(scope="module")
def pair():
    g = O.Grid(120, 110, 4, 17.0, 12.0, 3.0, 6.5, gridder="sml")
    s = cg.Solver(**SML)
    yield g, s
    s.close()


def test_operators_bit_exact(pair):
    g, s = pair
    x = np.random.default_rng(3).standard_normal(s.cells)
    np.testing.assert_array_equal(s.spmv(x), O.spe_multiply(g, x))
    np.testing.assert_array_equal(s.spmv(x, jacobi=True), O.csr_multiply(g, x))


def test_rhs_and_solid_fraction_bit_exact(pair):
    g, s = pair
    rng = np.random.default_rng(4)
    us, vs, ws = (rng.standard_normal(s.shape) for _ in range(3))
    np.testing.assert_array_equal(s.rhs(us, vs, ws), O.rhs(g, 0.005, us, vs, ws))
    np.testing.assert_array_equal(s.rhs(us, vs, ws, jacobi=True), O.rhs(g, 0.005, us, vs, ws, O.jacobi_scale(g)))
    np.testing.assert_array_equal(s.solid_fraction(), O.dfib_cylinder_z(g))


def _vel_err(f, ref):
    core = (slice(2, -2),) * 3
    get = lambda a: a[core] if a.shape == f["u"].shape else a
    scale = np.sqrt(sum(np.linalg.norm(get(ref[k])) ** 2 for k in "uvw"))
    return {k: float(np.linalg.norm(f[k][core] - get(ref[k])) / scale) for k in "uvw"}


def _p_err(p, q):
    core = (slice(2, -2),) * 3
    p = p[core]
    q = q[core] if q.shape != p.shape else q
    return float(np.linalg.norm((p - p.mean()) - (q - q.mean())) / np.linalg.norm(q - q.mean()))


@pytest.mark.parametrize("solver,osolver", [("bicgstab", "spe"), ("jacobi", "csr")])
def test_two_steps_match_oracle_at_tight_tolerance(solver, osolver):
    """Step 2 carries the only solve that converges to 1e-12 on this grid: the GPU step
    against the oracle there, to 1e-10."""
    g = O.Grid(120, 110, 4, 17.0, 12.0, 3.0, 6.5, gridder="sml")
    ref = O.run(g, 2, 100.0, 0.005, 1e-12, osolver)
    with cg.Solver(solver=solver, tol=1e-12, **SML) as s:
        s.init_fields()
        st = s.step(2)
        f = s.get_fields()
    assert st[1].status == 0 and st[1].relres < 1e-12
    for k, e in _vel_err(f, ref).items():
        assert e <= 1e-10, (k, e)
    assert _p_err(f["p"], ref["p"]) <= 1e-10
    np.testing.assert_allclose([r.cd for r in st], ref["cd"], rtol=1e-10)


@pytest.mark.parametrize("case,solver", [("sml_spe_tol1e-3_10", "bicgstab"), ("sml_csr_tol1e-3_10", "jacobi")])
def test_run_tracks_reference_at_its_tolerance(case, solver, golden):
    """Ten steps at the reference's tolerance 1e-3 against its own runs.  Two correct
    solvers stop at different iterates within that tolerance (the counts differ), so the
    bar is the solve tolerance's scale: Cd and the velocity within 1e-2.  The pressure is
    not compared: at a 1e-3 residual its smoothest modes are barely resolved, and two
    such solves differ there by 5-10 % while the velocity they produce agrees."""
    z = golden(f"run_{case}.npz")
    with cg.Solver(solver=solver, tol=1e-3, **SML) as s:
        s.init_fields()
        st = s.step(10)
        f = s.get_fields()
    assert all(r.status == 0 and r.relres < 1e-3 for r in st[1:])
    cd = np.array([r.cd for r in st])
    assert np.abs(cd - z["cd"]).max() <= 1e-2 * np.abs(z["cd"]).max(), (cd, z["cd"])
    if "u" in z:
        for k, e in _vel_err(f, {k: z[k] for k in "uvw"}).items():
            assert e <= 1e-2, (k, e)


@pytest.mark.parametrize("solver", ["bicgstab", "jacobi"])
def test_mixed_on_the_stretched_grid_reaches_fp64(solver):
    """MIXED precision on the stretched grid (FP32 sweeps on the stored rows rounded to
    FP32, FP64 refinement): at the tight tolerance step 2 allows, every solve ends below it
    in the FP64 residual and the fields agree with the FP64 run; over ten steps at the
    reference's 1e-3 the drag tracks the FP64 run's at that tolerance's scale."""
    runs = {}
    for prec in ("fp64", "mixed"):
        with cg.Solver(solver=solver, precision=prec, tol=1e-10, **SML) as s:
            s.init_fields()
            st = s.step(2)
            runs[prec] = (s.get_fields(), st)
    f, st = runs["mixed"]
    assert st[1].status == 0 and st[1].relres < 1e-10, (st[1].status, st[1].relres)
    for k, e in _vel_err(f, runs["fp64"][0]).items():
        assert e <= 1e-8, (k, e)
    assert _p_err(f["p"], runs["fp64"][0]["p"]) <= 1e-6
    cds = {}
    for prec in ("fp64", "mixed"):
        with cg.Solver(solver=solver, precision=prec, tol=1e-3, **SML) as s:
            s.init_fields()
            st = s.step(10)
            assert all(r.status == 0 and r.relres < 1e-3 for r in st[1:]), (prec, [r.relres for r in st])
            cds[prec] = np.array([r.cd for r in st])
    assert np.abs(cds["mixed"] - cds["fp64"]).max() <= 1e-2 * np.abs(cds["fp64"]).max()
