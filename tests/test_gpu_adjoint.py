"""Discrete adjoint of the projection step (cfdgb_forward / cfdgb_backward) against
central finite differences: of the CUDA forward step itself, and of the reference
restatement on the CPU (the oracle, same parameters injected).

Objective: drag averaged over steps 8..12 of a 12-step run on a 32x16x4 grid (checkpoint
every 5 steps, so one window is partial), Poisson solved to 1e-12 so that the FD
quotients (eps = 1e-6) resolve the derivative to ~1e-6 of its size.

The runs remove the Poisson rhs's mean before each solve (project_rhs).  With the
reference's zero-gradient outflow and walls, any change of the inflow or of the body breaks
the Neumann problem's solvability by about the size of the change: the reference's own
BiCGSTAB then runs to its cap and diverges to NaN at the first perturbed step, so the
unprojected step has no derivative to check.  The adjoint solve already works on the
mean-free subspace, so it is the exact adjoint of the projected step."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASE = dict(nx=32, ny=16, nz=4, lx=8.0, ly=4.0, lz=1.0, cx=2.0, cy=2.0, Re=100.0, dt=0.005)
PROJECT = 1
NSTEPS, FIRST, LAST, K = 12, 8, 12, 5
TOL = 1e-12
EPS = 1e-6


def _J(s, inlet=None, eta=None):
    # the inlet also feeds the initial ghost fill: set it before init_fields
    s.set_inlet(inlet)
    if eta is not None:
        s.set_eta(eta)
    s.init_fields()
    return s.forward(NSTEPS, FIRST, LAST, K)


@pytest.fixture(scope="module")
def adj():
    s = cg.Solver(tol=TOL, project_rhs=PROJECT, **CASE)
    eta0 = s.get_eta()
    J0 = _J(s, eta=eta0)
    g_in, g_eta = s.backward()
    yield s, eta0, J0, g_in, g_eta
    s.close()


def _fd(s, base_inlet, eta0, d_in=None, d_eta=None):
    ip = None if d_in is None else base_inlet + EPS * d_in
    im = None if d_in is None else base_inlet - EPS * d_in
    ep = eta0 if d_eta is None else eta0 + EPS * d_eta
    em = eta0 if d_eta is None else eta0 - EPS * d_eta
    return (_J(s, ip, ep) - _J(s, im, em)) / (2 * EPS)


def test_gradients_are_finite_and_nonzero(adj):
    s, eta0, J0, g_in, g_eta = adj
    assert np.isfinite(J0) and J0 > 0
    assert np.all(np.isfinite(g_in)) and np.abs(g_in).max() > 0
    assert np.all(np.isfinite(g_eta)) and np.abs(g_eta).max() > 0
    # eta enters only through interior faces
    assert np.abs(g_eta[:2]).max() == 0 and np.abs(g_eta[-2:]).max() == 0


@pytest.mark.parametrize("seed", range(4))
def test_inlet_gradient_matches_central_fd(adj, seed):
    s, eta0, J0, g_in, g_eta = adj
    d = np.random.default_rng(seed).standard_normal(g_in.shape)
    fd = _fd(s, np.ones(g_in.shape), eta0, d_in=d)
    ad = float(np.sum(g_in * d))
    assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-9, (ad, fd)


@pytest.mark.parametrize("seed", range(8))
def test_eta_gradient_matches_central_fd(adj, seed):
    s, eta0, J0, g_in, g_eta = adj
    band = (eta0 > 0) & (eta0 < 1)
    band[:2] = band[-2:] = False
    band[:, :2] = band[:, -2:] = False
    band[:, :, :2] = band[:, :, -2:] = False
    d = np.where(band, np.random.default_rng(100 + seed).standard_normal(eta0.shape), 0.0)
    fd = _fd(s, None, eta0, d_eta=d)
    ad = float(np.sum(g_eta * d))
    assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-9, (ad, fd)


def test_against_fd_of_the_cpu_reference_restatement(adj):
    """The same objective computed by the oracle (reference restatement, CPU), finite-
    differenced in one inlet and one eta direction, against the GPU adjoint."""
    s, eta0, J0, g_in, g_eta = adj
    g = O.Grid(CASE["nx"], CASE["ny"], CASE["nz"], CASE["lx"], CASE["ly"], CASE["lz"], CASE["cx"])

    def J_cpu(inlet=None, eta=None):
        r = O.run(g, NSTEPS, CASE["Re"], CASE["dt"], TOL, "spe", eta_in=eta, inlet=inlet, project=PROJECT)
        return float(np.mean(r["cd"][FIRST - 1:LAST]))

    assert abs(J_cpu() - J0) <= 1e-10 * abs(J0)
    rng = np.random.default_rng(7)
    d = rng.standard_normal(g_in.shape)
    one = np.ones(g_in.shape)
    fd = (J_cpu(inlet=one + EPS * d) - J_cpu(inlet=one - EPS * d)) / (2 * EPS)
    assert abs(float(np.sum(g_in * d)) - fd) <= 1e-4 * abs(fd) + 1e-9
    band = (eta0 > 0) & (eta0 < 1)
    de = np.where(band, rng.standard_normal(eta0.shape), 0.0)
    de[:2] = de[-2:] = 0
    fd = (J_cpu(eta=eta0 + EPS * de) - J_cpu(eta=eta0 - EPS * de)) / (2 * EPS)
    assert abs(float(np.sum(g_eta * de)) - fd) <= 1e-4 * abs(fd) + 1e-9


def test_backward_is_repeatable(adj):
    """The transposed stencil scatters with atomics, so two sweeps differ in rounding,
    which the adjoint Poisson solves (tolerance 1e-12) carry to ~1e-9 relative."""
    s, eta0, J0, g_in, g_eta = adj
    _J(s, eta=eta0)
    g_in2, g_eta2 = s.backward()
    np.testing.assert_allclose(g_in2, g_in, rtol=1e-7, atol=1e-9 * np.abs(g_in).max())
    np.testing.assert_allclose(g_eta2, g_eta, rtol=1e-7, atol=1e-9 * np.abs(g_eta).max())


def test_free_slip_walls_gradients_match_central_fd():
    """With the free-slip wall rows of the boundary table the adjoint's transposed ghost
    fill takes the same table: one inlet and one eta direction against central FD."""
    s = cg.Solver(tol=TOL, project_rhs=PROJECT, walls="free_slip", **CASE)
    try:
        eta0 = s.get_eta()
        _J(s, eta=eta0)
        g_in, g_eta = s.backward()
        rng = np.random.default_rng(11)
        d = rng.standard_normal(g_in.shape)
        fd = _fd(s, np.ones(g_in.shape), eta0, d_in=d)
        assert abs(float(np.sum(g_in * d)) - fd) <= 1e-4 * abs(fd) + 1e-9
        band = (eta0 > 0) & (eta0 < 1)
        band[:2] = band[-2:] = False
        de = np.where(band, rng.standard_normal(eta0.shape), 0.0)
        fd = _fd(s, None, eta0, d_eta=de)
        assert abs(float(np.sum(g_eta * de)) - fd) <= 1e-4 * abs(fd) + 1e-9
    finally:
        s.close()


@pytest.mark.parametrize("kw", [dict(precond="multigrid"), dict(precision="mixed", precond="multigrid"),
                                dict(precision="mixed", solver="cg")],
                         ids=["fp64_multigrid", "mixed_multigrid", "mixed_cg"])
def test_adjoint_of_other_contexts_matches_fp64(adj, kw):
    """The adjoint from a context whose forward runs the multigrid-preconditioned FP64
    solver (its transposed solve with the FP64 V-cycle), or MIXED precision (FP32 sweeps in
    FP64 refinement, forward and transposed solves alike, to the same FP64 tolerance): the
    same objective and gradients as the plain FP64 context's, which the finite-difference
    tests above check.  The MIXED runs differ from FP64 by their FP32 rounding."""
    s0, eta0, J0, g_in0, g_eta0 = adj
    with cg.Solver(tol=TOL, project_rhs=PROJECT, **kw, **CASE) as s:
        s.set_inlet(None)
        s.init_fields()
        J = s.forward(NSTEPS, FIRST, LAST, K)
        g_in, g_eta = s.backward()
    bar = 1e-9 if "precision" not in kw else 1e-6
    assert abs(J - J0) <= bar * abs(J0), (J, J0)
    assert np.linalg.norm(g_in - g_in0) <= 1e2 * bar * np.linalg.norm(g_in0)
    assert np.linalg.norm(g_eta - g_eta0) <= 1e2 * bar * np.linalg.norm(g_eta0)
