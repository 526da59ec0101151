"""ctypes binding of the C restatement (oracle/cfd_oracle.c).

TEST INFRASTRUCTURE ONLY -- imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker; the library under test never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libcfd_oracle.so"
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> Path:
    """Compile the restatement with the flags that keep IEEE source order."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "cfd_oracle.c"
    hdr = HERE / "cfd_oracle.h"
    newest = max(src.stat().st_mtime, hdr.stat().st_mtime)
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class _Grid(C.Structure):
    _fields_ = [("nxc", C.c_int), ("nyc", C.c_int), ("nzc", C.c_int),
                ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double)] + [
        (n, C.POINTER(C.c_double)) for n in
        ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs")] + [
        ("scheme", C.c_int), ("les", C.c_int), ("walls", C.c_int), ("time_order", C.c_int),
        ("periodic_z", C.c_int), ("outflow", C.c_int)]


# the reference's compile-time convection switch (0_General.hpp:114-118)
SCHEMES = {"quick": 0, "lud": 1, "ud": 2}
# the y-wall rows of its boundary table (FLOWpassing.hpp: active, and the commented-out ones)
WALLS = {"zero_gradient": 0, "free_slip": 1}
# the z faces and the outlet (neither option is in the reference)
BC_Z = {"zero_gradient": 0, "periodic": 1}
OUTFLOWS = {"zero_gradient": 0, "convective": 1}


class _Bicg(C.Structure):
    _fields_ = [("n", C.c_long), ("timestep", C.c_int), ("iters_max", C.c_int),
                ("tol", C.c_double), ("restart_factor", C.c_double)] + [
        (n, C.POINTER(C.c_double)) for n in
        ("r0", "r1", "p1", "s1", "ap", "as_", "px1", "px2")] + [
        ("kind", C.c_int), ("g", C.c_void_p), ("val7", C.POINTER(C.c_double)),
        ("jp", C.POINTER(C.c_double))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        gp = C.POINTER(_Grid)
        L.og_grid_init_uniform.argtypes = [gp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 6
        L.og_grid_init_sml.argtypes = [gp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 6
        L.og_grid_free.argtypes = [gp]
        L.og_perturb.argtypes = [gp, _dp, _dp, _dp, C.c_uint64, C.c_double]
        L.og_convection_diffusion.argtypes = [gp, C.c_double, C.c_double] + [_dp] * 6
        L.og_bc_main.argtypes = [gp] + [_dp] * 4
        L.og_bc_copy.argtypes = [gp] + [_dp] * 6
        L.og_rhs.argtypes = [gp, C.c_double, _dp, _dp, _dp, C.c_void_p, _dp]
        L.og_jacobi_scale.argtypes = [gp, _dp]
        L.og_spe_setup.argtypes = [gp, _dp]
        L.og_spe_multiply.argtypes = [gp, _dp, _dp, _dp]
        L.og_csr_multiply.argtypes = [gp, _dp, _dp, _dp]
        bp = C.POINTER(_Bicg)
        L.og_bicg_init.argtypes = [bp, gp, C.c_int, C.c_double]
        L.og_bicg_free.argtypes = [bp]
        L.og_bicg_solve.argtypes = [bp, _dp, _dp, C.POINTER(C.c_double)]
        L.og_sor.argtypes = [gp, C.c_double, C.c_double, C.c_double, C.c_int,
                             _dp, _dp, _dp, _dp, C.POINTER(C.c_double)]
        L.og_transform.argtypes = [gp, _dp, _dp]
        L.og_update_uf.argtypes = [gp, C.c_double] + [_dp] * 9
        L.og_dfib_cylinder_z.argtypes = [gp, _dp]
        L.og_force_sum.argtypes = [gp, _dp, C.c_int]
        L.og_force_sum.restype = C.c_double
        L.og_run.argtypes = [gp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                             C.c_double, _dp, _dp, _dp, _dp, _dp, C.c_void_p]
        L.og_run_ex.argtypes = L.og_run.argtypes + [C.c_void_p, C.c_void_p, C.c_int]
        _lib = L
    return _lib


class Grid:
    """Uniform MAC grid of the reference (structureGrid.hpp:336), cylinder at (cx, ly/2)."""

    def __init__(self, nxc, nyc, nzc, lx, ly, lz, cx, radius=0.5, gridder="uniform", scheme="quick",
                 les=False, walls="zero_gradient", time_order=1, bc_z="zero_gradient", outflow="zero_gradient"):
        """gridder: "uniform" (init_uniform) or "sml" (the reference's default stretched
        non_uniform-SML grid); scheme: "quick", "lud" or "ud" (the convection switch);
        les: the Smagorinsky eddy viscosity in run(); walls: the y walls' boundary rows;
        time_order: run()'s time stepping, 1 the reference's Euler step, 2 or 3
        Adams-Bashforth (constant dt; not in the reference); bc_z: "periodic" wraps z;
        outflow: "convective" (with the flux correction) in place of the zero-gradient
        outlet."""
        self._g = _Grid()
        init = {"uniform": lib().og_grid_init_uniform, "sml": lib().og_grid_init_sml}[gridder]
        rc = init(C.byref(self._g), nxc, nyc, nzc, lx, ly, lz, cx, ly / 2.0, radius)
        if rc != 0:
            raise ValueError("grid too small")
        self._g.scheme = SCHEMES[scheme]
        self._g.les = 1 if les else 0
        self._g.walls = WALLS[walls]
        self._g.time_order = int(time_order)
        self._g.periodic_z = BC_Z[bc_z]
        self._g.outflow = OUTFLOWS[outflow]
        self.shape = (nxc + 4, nyc + 4, nzc + 4)
        self.cells = nxc * nyc * nzc

    @property
    def ptr(self):
        return C.byref(self._g)

    def __del__(self):
        try:
            lib().og_grid_free(C.byref(self._g))
        except Exception:
            pass

    def zeros(self):
        return np.zeros(self.shape, dtype=np.float64)

    def coords(self):
        g = self._g
        return (np.ctypeslib.as_array(g.X, (g.nx + 1,)).copy(),
                np.ctypeslib.as_array(g.Y, (g.ny + 1,)).copy(),
                np.ctypeslib.as_array(g.Z, (g.nz + 1,)).copy())


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def convection_diffusion(g: Grid, dt, nu, u, v, w, us, vs, ws, nut=None):
    """ConvectionDifussion with the grid's scheme; nut (compact): the eddy viscosity."""
    L = lib()
    L.og_convection_diffusion_ex.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p] + [_dp] * 6
    L.og_convection_diffusion_ex(g.ptr, dt, nu, None if nut is None else _c(nut).ctypes.data_as(C.c_void_p),
                                 _c(u), _c(v), _c(w), us, vs, ws)


def smagorinsky(g: Grid, u, v, w):
    """SmagorinskyModel (SmagorinskyModel.hpp:30): compact eddy viscosity of u, v, w."""
    L = lib()
    L.og_smagorinsky.argtypes = [C.c_void_p] + [_dp] * 4
    nut = np.zeros(g.cells)
    L.og_smagorinsky(g.ptr, _c(u), _c(v), _c(w), nut)
    return nut


def bc_main(g, u, v, w, p):
    lib().og_bc_main(g.ptr, u, v, w, p)


def bc_main_ex(g, u, v, w, p, inlet=None, us=None, vs=None, ws=None, dt=0.0):
    """The ghost fill of a time step (us, vs, ws: the last step's copies; None at init)."""
    L = lib()
    vp = C.c_void_p
    L.og_bc_main_ex.argtypes = [vp] + [_dp] * 4 + [vp] * 4 + [C.c_double]
    keep = [None if a is None else _c(a) for a in (inlet, us, vs, ws)]
    L.og_bc_main_ex(g.ptr, u, v, w, p, *[None if a is None else a.ctypes.data_as(vp) for a in keep], dt)


def inlet_mean(g, inlet=None):
    L = lib()
    L.og_inlet_mean.argtypes = [C.c_void_p, C.c_void_p]
    L.og_inlet_mean.restype = C.c_double
    a = None if inlet is None else _c(inlet).reshape(-1)
    return L.og_inlet_mean(g.ptr, None if a is None else a.ctypes.data_as(C.c_void_p))


def bc_copy(g, u, v, w, us, vs, ws):
    lib().og_bc_copy(g.ptr, _c(u), _c(v), _c(w), us, vs, ws)


def rhs(g, dt, us, vs, ws, jp=None):
    b = np.zeros(g.cells)
    jpp = None if jp is None else _c(jp).ctypes.data_as(C.c_void_p)
    lib().og_rhs(g.ptr, dt, _c(us), _c(vs), _c(ws), jpp, b)
    return b


def jacobi_scale(g):
    jp = np.zeros(g.cells)
    lib().og_jacobi_scale(g.ptr, jp)
    return jp


def spe_multiply(g, x):
    val = np.zeros(7 * g.cells)
    lib().og_spe_setup(g.ptr, val)
    y = np.zeros(g.cells)
    lib().og_spe_multiply(g.ptr, val, _c(x), y)
    return y


def csr_multiply(g, x):
    y = np.zeros(g.cells)
    lib().og_csr_multiply(g.ptr, jacobi_scale(g), _c(x), y)
    return y


class BiCGSTAB:
    """bicgstabRe2 (inc/solver/bicgstabRe2.hpp) with kind 0 = SPE, 1 = Jacobi-scaled CSR."""

    def __init__(self, g: Grid, kind: int, tol: float):
        self._s = _Bicg()
        self._g = g
        lib().og_bicg_init(C.byref(self._s), g.ptr, kind, tol)

    def solve(self, rhs_, x):
        rr = C.c_double()
        it = lib().og_bicg_solve(C.byref(self._s), _c(rhs_), x, C.byref(rr))
        return it, rr.value

    def __del__(self):
        try:
            lib().og_bicg_free(C.byref(self._s))
        except Exception:
            pass


def cfl(g, dt, us, vs, ws):
    """get_Cfl (cfl.hpp:3): [cfl, U_max x3, U_min x3]."""
    out = np.zeros(7)
    L = lib()
    L.og_cfl.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.og_cfl(g.ptr, dt, _c(us).ctypes.data_as(C.c_void_p), _c(vs).ctypes.data_as(C.c_void_p),
             _c(ws).ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
    return out


def timestepper(Re, U_max, U_min, dt_min=1e-12, cfl_factor=0.05, grid_fo_factor=0.15):
    """simpulationVariable::timestepper (inc/0_1_SimulationVariable.hpp:172-185) with its
    factors (:270-272): dt_next from the velocity extremes get_Cfl keeps, each product in
    the reference's left-to-right order, std::min as (b < a ? b : a)."""
    d = 1e10
    for x in U_max:
        lim = cfl_factor / (Re * x * x) if Re * x * x != 0.0 else float("inf")
        d = lim if lim < d else d
    for x in U_min:
        lim = grid_fo_factor * 0.5 * Re * x * x
        d = lim if lim < d else d
    return dt_min if d < dt_min else d


def plot3d(g, p, u, v, w, eta, Re, time, qpath, xpath):
    """The reference's Plot3D .q and .x files (qfile.hpp, xfileWrite.hpp)."""
    L = lib()
    L.og_plot3d_x.argtypes = [C.c_void_p, C.c_char_p]
    L.og_plot3d_q.argtypes = [C.c_void_p] + [C.c_void_p] * 5 + [C.c_double, C.c_double, C.c_char_p]
    arrs = [_c(a) for a in (p, u, v, w, eta)]
    if L.og_plot3d_x(g.ptr, str(xpath).encode()) or L.og_plot3d_q(
            g.ptr, *[a.ctypes.data_as(C.c_void_p) for a in arrs], Re, time, str(qpath).encode()):
        raise OSError("plot3d write failed")


def plot3d_read(g, qpath):
    """QfileRead (qfileRead.hpp:6): (head = [blocks, mach, alpha, Re, time], p, u, v, w, eta)
    as padded arrays rebuilt from the cell-centred .q file."""
    L = lib()
    L.og_plot3d_read.argtypes = [C.c_void_p, C.c_char_p] + [C.c_void_p] * 6
    head = np.zeros(5)
    out = [g.zeros() for _ in range(5)]
    if L.og_plot3d_read(g.ptr, str(qpath).encode(), head.ctypes.data_as(C.c_void_p),
                        *[a.ctypes.data_as(C.c_void_p) for a in out]):
        raise OSError(f"cannot read {qpath} as a Plot3D solution of this grid")
    return (head, *out)


def sor(g, dt, omega, tol, itmax, us, vs, ws, p):
    err = C.c_double()
    it = lib().og_sor(g.ptr, dt, omega, tol, itmax, _c(us), _c(vs), _c(ws), p, C.byref(err))
    return it, err.value


def update_uf(g, dt, eta, p, us, vs, ws, u3, v3, w3, f):
    lib().og_update_uf(g.ptr, dt, _c(eta), _c(p), _c(us), _c(vs), _c(ws), u3, v3, w3, f)


def dfib_cylinder_z(g):
    eta = g.zeros()
    lib().og_dfib_cylinder_z(g.ptr, eta)
    return eta


def force_sum(g, f, d):
    return lib().og_force_sum(g.ptr, _c(f), d)


def perturb(g, u, v, w, seed, amp):
    lib().og_perturb(g.ptr, u, v, w, seed, amp)


SOLVERS = {"spe": 0, "bicgstab": 0, "jacobi": 1, "csr": 1, "sor": 2, "cg": 3}


def run(g: Grid, steps, Re, dt, tol, solver="spe", omega=1.8, seed=0, amp=0.0, eta_in=None,
        inlet=None, project=False, init=None):
    """Whole run (src/RUN_CPU.cpp:257-436 order); returns dict of final fields + stats.
    eta_in (padded) replaces the cylinder's solid fraction, inlet (ny, nz) the inlet u;
    project removes the Poisson rhs's mean before each BiCGSTAB solve (not in the reference);
    init: padded (u, v, w) to start from in place of u = 1, v = w = 0 (+ the perturbation)."""
    u = np.ones(g.shape)
    v = g.zeros()
    w = g.zeros()
    if init is not None:
        u, v, w = (np.array(a, dtype=np.float64, copy=True) for a in init)
    elif amp:
        perturb(g, u, v, w, seed, amp)
    p = g.zeros()
    eta = g.zeros()
    stats = np.zeros((steps, 4))
    ein = None if eta_in is None else _c(eta_in)
    inl = None if inlet is None else _c(inlet).reshape(-1)
    lib().og_run_ex(g.ptr, steps, Re, dt, tol, SOLVERS[solver], omega, u, v, w, p, eta,
                    stats.ctypes.data_as(C.c_void_p),
                    None if ein is None else ein.ctypes.data_as(C.c_void_p),
                    None if inl is None else inl.ctypes.data_as(C.c_void_p), int(bool(project)))
    return {"u": u, "v": v, "w": w, "p": p, "eta": eta, "iters": stats[:, 0].astype(int),
            "err": stats[:, 1], "cd": stats[:, 2], "cl": stats[:, 3]}
