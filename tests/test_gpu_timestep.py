"""The CFL number computed inside the convection-diffusion kernel and the adaptive time
step it feeds, through the C ABI.

- FP64: the CFL number a step reports is get_Cfl (inc/analyses/cfl.hpp:3) of that step's
  u*, bit for bit: the same u* from the per-function convection-diffusion entry point and
  the separate CFL entry point (itself bit-exact against the reference's goldens).
- MIXED: the FP32 sweep's CFL number agrees with FP64's on the same state to FP32 rounding.
- CFDGB_DT_REFERENCE: the reference's timestepper (0_1_SimulationVariable.hpp:172-185,
  restated in the oracle) on the extremes get_Cfl keeps since init, applied at the next
  step as finishloop does; in a flow without z motion w's minimum is 0 and dt drops to
  the 1e-12 floor, as the reference's formula gives.
- CFDGB_DT_CFL: each step's dt is cfl_target over the previous step's per-cell maximum,
  capped at dt_max, and time is the sum of the steps' dt.""" 
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _ustar(s, f):
    """u*, v*, w* of the state f by the per-function convection-diffusion entry point."""
    us, vs, ws = f["u"].copy(), f["v"].copy(), f["w"].copy()
    s.convection_diffusion(f["u"], f["v"], f["w"], us, vs, ws)
    return us, vs, ws


def test_step_cfl_is_get_cfl_of_its_ustar():
    with cg.Solver(tol=1e-12) as s:
        s.init_fields()
        for _ in range(3):
            f = s.get_fields()
            ref = s.cfl(*_ustar(s, f))
            st = s.step(1)[0]
            assert st.cfl == ref[0], (st.step, st.cfl, ref[0])


def test_mixed_cfl_matches_fp64():
    with cg.Solver(tol=1e-10) as a, cg.Solver(tol=1e-10, precision="mixed", solver="cg") as b:
        a.init_fields()
        b.init_fields()
        sa, sb = a.step(3), b.step(3)
    for x, y in zip(sa, sb):
        assert abs(x.cfl - y.cfl) <= 1e-6 * x.cfl, (x.cfl, y.cfl)


@pytest.mark.parametrize("amp", [0.0, 1e-3], ids=["quasi2d", "perturbed"])
def test_reference_timestepper(amp):
    kw = dict(tol=1e-12, dt_mode="reference", amp=amp, seed=1234, project_rhs=1 if amp else 0)
    with cg.Solver(**kw) as s:
        s.init_fields()
        umax, umin = np.full(3, -1e10), np.full(3, 1e10)
        dt_expect = s.cfg.dt
        t = 0.0
        for n in range(3):
            # the per-function entry points use the configured dt: give them this step's
            # (set_dt writes the value the rule has already put on the device)
            s.set_dt(dt_expect)
            f = s.get_fields()
            ext = s.cfl(*_ustar(s, f))  # this step's u*: cfl, U_max[3], U_min[3]
            st = s.step(1)[0]
            assert st.dt == dt_expect, (n, st.dt, dt_expect)
            t += st.dt
            assert st.time == t
            umax, umin = np.maximum(umax, ext[1:4]), np.minimum(umin, ext[4:7])
            dt_expect = O.timestepper(s.cfg.Re, umax, umin)
            if amp == 0.0 and n == 0:
                assert umax[2] == 0.0 and umin[2] == 0.0 and dt_expect == 1e-12


def test_cfl_target_timestep():
    target, dt_max = 0.03, 0.01
    with cg.Solver(tol=1e-10, dt_mode="cfl", cfl_target=target, dt_max=dt_max) as s:
        s.init_fields()
        st = s.step(6)
    assert st[0].dt == s.cfg.dt
    for a, b in zip(st, st[1:]):
        cmax = a.cfl / a.dt  # the per-cell maximum of u/Dxs + v/Dys + w/Dzs
        assert b.dt == pytest.approx(min(target / cmax, dt_max), rel=1e-14), (b.step, b.dt, target / cmax)
    assert st[-1].time == pytest.approx(sum(r.dt for r in st), rel=1e-15)


@pytest.mark.parametrize("order", [2, 3])
def test_adams_bashforth_matches_the_oracle(order):
    """Adams-Bashforth time stepping (not in the reference: its 2nd/3rd-order branch does not
    compile): 10 steps on 48x24x4 against the oracle's restatement of the same formulas,
    both solving to 1e-13; the same 1e-10 bar as the Euler runs.  The Euler run differs."""
    dom = dict(nx=48, ny=24, nz=4, lx=12.0, ly=6.0, lz=1.0, cx=3.0, cy=3.0)
    g = O.Grid(48, 24, 4, 12.0, 6.0, 1.0, 3.0, time_order=order)
    ref = O.run(g, 10, 100.0, 0.005, 1e-13, "spe")
    with cg.Solver(tol=1e-13, time_order=order, **dom) as s:
        s.init_fields()
        st = s.step(10)
        f = s.get_fields()
    core = (slice(2, -2),) * 3
    scale = np.sqrt(sum(np.linalg.norm(ref[k][core]) ** 2 for k in "uvw"))
    for k in "uvw":
        assert np.linalg.norm(f[k][core] - ref[k][core]) / scale <= 1e-10, k
    np.testing.assert_allclose([r.cd for r in st], ref["cd"], rtol=1e-10)
    euler = O.run(O.Grid(48, 24, 4, 12.0, 6.0, 1.0, 3.0), 10, 100.0, 0.005, 1e-13, "spe")
    assert abs(euler["cd"][-1] - ref["cd"][-1]) > 1e-6 * abs(ref["cd"][-1])


def test_adams_bashforth_variable_step():
    """Second order with the CFL rule changing dt every step: runs, every solve converges,
    and the steps' dt follow the rule (the variable-step coefficients use dt_n / dt_(n-1))."""
    with cg.Solver(tol=1e-10, time_order=2, dt_mode="cfl", cfl_target=0.03, dt_max=0.01) as s:
        s.init_fields()
        st = s.step(6)
    assert all(r.status == 0 for r in st)
    assert len({r.dt for r in st}) > 2
