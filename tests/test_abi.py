"""CPU checks of the C-ABI library: it loads, exports every entry point include/cfdgb.h
declares, and its host-side logic (defaults, validation, perturbation generator) is
right.  No kernel runs here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    text = (ROOT / "include" / "cfdgb.h").read_text()
    return sorted(set(re.findall(r"\b(cfdgb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not cg.LIB_PATH.exists():
        from cfd_nssolver_forhpc_flowpassingcylinder_gb300 import build as B
        B.build()
    return cg.load_library()


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # and the binding covers exactly the declared surface
    assert set(names) == set(cg.EXPORTS)


def test_defaults_are_the_reference_case(lib):
    cfg = cg.default_config()
    assert (cfg.nx, cfg.ny, cfg.nz) == (96, 48, 4)
    assert (cfg.lx, cfg.ly, cfg.lz, cfg.cx, cfg.cy, cfg.radius) == (24.0, 12.0, 1.0, 6.0, 6.0, 0.5)
    assert (cfg.Re, cfg.dt, cfg.maxit) == (100.0, 0.005, 5000)
    assert cfg.solver == cg.BICGSTAB and cfg.precision == cg.FP64
    assert lib.cfdgb_abi_version() == cg.ABI_VERSION == 9
    assert cfg.scheme == cg.QUICK and cfg.les == 0 and cfg.walls == cg.WALLS_ZERO_GRADIENT
    assert cfg.dt_mode == cg.DT_FIXED and cfg.cfl_target == 0.5 and cfg.dt_max == 0.0 and cfg.time_order == 1
    assert cfg.bc_z == cg.Z_ZERO_GRADIENT and cfg.outflow == cg.OUTFLOW_ZERO_GRADIENT


@pytest.mark.parametrize("field,value", [("nx", 2), ("dt", 0.0), ("Re", -1.0), ("solver", 7),
                                         ("precision", 3), ("tol", 0.0), ("maxit", 0), ("scheme", 3),
                                         ("scheme", -1), ("les", 2), ("walls", 2), ("dt_mode", 3),
                                         ("dt_mode", -1), ("time_order", 4), ("bc_z", 2), ("bc_z", -1),
                                         ("outflow", 2), ("outflow", -1)])
def test_invalid_config_is_rejected_before_any_device_work(lib, field, value):
    cfg = cg.default_config()
    setattr(cfg, field, value)
    h = C.c_void_p()
    rc = lib.cfdgb_create(C.byref(cfg), C.byref(h))
    assert rc == cg.EINVAL
    assert h.value is None
    assert lib.cfdgb_last_error()


def test_cfl_timestep_needs_a_positive_target(lib):
    cfg = cg.default_config(dt_mode="cfl", cfl_target=0.0)
    h = C.c_void_p()
    assert lib.cfdgb_create(C.byref(cfg), C.byref(h)) == cg.EINVAL


def test_timestepper_restatement():
    """The oracle's timestepper (0_1_SimulationVariable.hpp:172-185): the CFL limit of each
    component's maximum, the grid-Fourier limit of its minimum, the 1e-12 floor."""
    assert O.timestepper(100.0, [1.0, 0.5, 0.0], [0.5, -0.5, -0.3]) == min(0.05 / 100.0, 0.075 * 100 * 0.09)
    assert O.timestepper(100.0, [1.0, 0.5, 0.0], [0.5, -0.5, 0.0]) == 1e-12


def test_mixed_sor_combination_rejected(lib):
    cfg = cg.default_config(solver="rbsor", precision="mixed")
    h = C.c_void_p()
    assert lib.cfdgb_create(C.byref(cfg), C.byref(h)) == cg.EINVAL


@pytest.mark.parametrize("kw", [dict(precond="multigrid", precision="mixed", nz=6), dict(precond="multigrid", nz=6),
                                dict(solver="rbsor", nz=5)])
def test_periodic_z_limits_rejected(lib, kw):
    """Periodic z: red-black smoothing and red-black SOR need the cells across the wrap to
    differ in colour, so an even nz on the grid and on every multigrid level (6 coarsens to
    3)."""
    base = dict(nx=32, ny=16, nz=8, lx=8.0, ly=4.0, lz=2.0, cx=2.0, cy=2.0, bc_z="periodic")
    cfg = cg.default_config(**{**base, **kw})
    h = C.c_void_p()
    assert lib.cfdgb_create(C.byref(cfg), C.byref(h)) == cg.EINVAL
    assert h.value is None


def test_null_arguments_are_errors(lib):
    assert lib.cfdgb_create(None, None) == cg.EINVAL
    assert lib.cfdgb_step(None, 1, None) == cg.EINVAL
    assert lib.cfdgb_get_fields(None, None, None, None, None) == cg.EINVAL


def test_perturbation_generator_matches_oracle():
    g = O.Grid(10, 8, 6, 2.5, 2.0, 1.5, 1.25)
    u, v, w = np.ones(g.shape), g.zeros(), g.zeros()
    O.perturb(g, u, v, w, 1234, 1e-3)
    du, dv, dw = cg.perturbation(g.shape, 1234, 1e-3)
    np.testing.assert_array_equal(u, 1.0 + du)
    np.testing.assert_array_equal(v, dv)
    np.testing.assert_array_equal(w, dw)


@pytest.mark.parametrize("kw", [dict(nx=96, ny=110), dict(nx=121, ny=110), dict(nx=120, ny=100),
                                dict(solver="cg"), dict(solver="rbsor"), dict(precision="mixed", solver="cg"),
                                dict(precision="mixed", precond="multigrid"), dict(project_rhs=1)])
def test_stretched_grid_limits_rejected(lib, kw):
    """The SML grid needs unit_SML's sizes and runs the BiCGSTAB solvers (FP64 or MIXED,
    unpreconditioned): its operator is not symmetric and the V-cycle is the uniform grid's."""
    base = dict(nx=120, ny=110, nz=4, lx=17.0, ly=12.0, lz=3.0, cx=6.5, cy=6.0, grid="sml")
    base.update(kw)
    cfg = cg.default_config(**base)
    h = C.c_void_p()
    assert lib.cfdgb_create(C.byref(cfg), C.byref(h)) == cg.EINVAL
    assert h.value is None
