"""GB300-native projection time step for flow past a cylinder (cfdgb).

Python binding of the C ABI in include/cfdgb.h through ctypes: plain pointers and
sizes, numpy arrays in the reference's padded layout.  The CUDA library
(libcfdgb.so, built in-tree by build.py) is the only compute path; importing this
module never falls back to anything else, and every call raises CfdgbError when the
library returns a non-zero status.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libcfdgb.so"

ABI_VERSION = 9  # CFDGB_ABI_VERSION
OK, EINVAL, ECUDA, ENOCONV, ENAN, ENOMEM, ESTATE = 0, -1, -2, -3, -4, -5, -6
BICGSTAB, BICGSTAB_JACOBI, RBSOR, CG = 0, 1, 2, 3
FP64, MIXED = 0, 1
SOLVERS = {"bicgstab": BICGSTAB, "spe": BICGSTAB, "jacobi": BICGSTAB_JACOBI, "csr": BICGSTAB_JACOBI,
           "rbsor": RBSOR, "sor": RBSOR, "cg": CG}
PRECISIONS = {"fp64": FP64, "mixed": MIXED}
GRID_UNIFORM, GRID_SML = 0, 1
GRIDS = {"uniform": GRID_UNIFORM, "sml": GRID_SML}
QUICK, LUD, UD = 0, 1, 2
SCHEMES = {"quick": QUICK, "lud": LUD, "ud": UD}
WALLS_ZERO_GRADIENT, WALLS_FREE_SLIP = 0, 1
WALLS = {"zero_gradient": WALLS_ZERO_GRADIENT, "free_slip": WALLS_FREE_SLIP}
PRECOND_NONE, PRECOND_MULTIGRID = 0, 1
PRECONDS = {"none": PRECOND_NONE, "multigrid": PRECOND_MULTIGRID}
DT_FIXED, DT_REFERENCE, DT_CFL = 0, 1, 2
DT_MODES = {"fixed": DT_FIXED, "reference": DT_REFERENCE, "cfl": DT_CFL}
Z_ZERO_GRADIENT, Z_PERIODIC = 0, 1
BC_Z = {"zero_gradient": Z_ZERO_GRADIENT, "periodic": Z_PERIODIC}
OUTFLOW_ZERO_GRADIENT, OUTFLOW_CONVECTIVE = 0, 1
OUTFLOWS = {"zero_gradient": OUTFLOW_ZERO_GRADIENT, "convective": OUTFLOW_CONVECTIVE}
# the boundary set of the plain FP64 cylinder case (uniform inflow, convective outflow,
# free-slip y walls, periodic z): default_config(**BOUNDARY_SET) or Solver(**BOUNDARY_SET, ...)
BOUNDARY_SET = {"walls": "free_slip", "bc_z": "periodic", "outflow": "convective"}


class CfdgbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"cfdgb status {status}: {msg}")
        self.status = status


class Config(C.Structure):
    """cfdgb_config (field meanings in include/cfdgb.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double),
                ("Re", C.c_double), ("dt", C.c_double),
                ("solver", C.c_int), ("precision", C.c_int),
                ("tol", C.c_double), ("maxit", C.c_int), ("omega", C.c_double),
                ("inner_tol", C.c_double), ("max_outer", C.c_int), ("check_every", C.c_int),
                ("dfib", C.c_int), ("seed", C.c_uint64), ("amp", C.c_double), ("project_rhs", C.c_int),
                ("grid", C.c_int), ("scheme", C.c_int), ("les", C.c_int), ("walls", C.c_int),
                ("precond", C.c_int), ("dt_mode", C.c_int), ("cfl_target", C.c_double), ("dt_max", C.c_double),
                ("time_order", C.c_int), ("bc_z", C.c_int), ("outflow", C.c_int)]


class Objective(C.Structure):
    """cfdgb_objective: mean drag over steps first..last of an nsteps run."""
    _fields_ = [("nsteps", C.c_int), ("first", C.c_int), ("last", C.c_int), ("ckpt_every", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("step", C.c_int), ("iters", C.c_int), ("outer", C.c_int), ("status", C.c_int),
                ("relres", C.c_double), ("cd", C.c_double), ("cl", C.c_double), ("cfl", C.c_double),
                ("dt", C.c_double), ("time", C.c_double)]


_dp = C.POINTER(C.c_double)
_lib = None

EXPORTS = {
    # name: (restype, argtypes)
    "cfdgb_abi_version": (C.c_int, []),
    "cfdgb_check_division": (C.c_int, [C.c_longlong, C.c_uint64, C.c_double, C.POINTER(C.c_ulonglong)]),
    "cfdgb_last_error": (C.c_char_p, []),
    "cfdgb_config_default": (C.c_int, [C.POINTER(Config)]),
    "cfdgb_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "cfdgb_destroy": (C.c_int, [C.c_void_p]),
    "cfdgb_padded_dims": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 3),
    "cfdgb_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "cfdgb_init_fields": (C.c_int, [C.c_void_p] + [_dp] * 4),
    "cfdgb_set_fields": (C.c_int, [C.c_void_p] + [_dp] * 4),
    "cfdgb_get_fields": (C.c_int, [C.c_void_p] + [_dp] * 4),
    "cfdgb_get_eta": (C.c_int, [C.c_void_p, _dp]),
    "cfdgb_set_eta": (C.c_int, [C.c_void_p, _dp]),
    "cfdgb_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(StepStats)]),
    "cfdgb_pressure_solve": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), _dp]),
    "cfdgb_set_inlet": (C.c_int, [C.c_void_p, _dp]),
    "cfdgb_forward": (C.c_int, [C.c_void_p, C.c_void_p, _dp]),
    "cfdgb_backward": (C.c_int, [C.c_void_p, _dp, _dp]),
    "cfdgb_poisson_solve_static": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                             C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.POINTER(C.c_int), _dp]),
    "cfdgb_set_kernel_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "cfdgb_reset_counters": (C.c_int, [C.c_void_p]),
    "cfdgb_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "cfdgb_kernel_stat": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_char_p), _dp,
                                    C.POINTER(C.c_longlong)]),
    "cfdgb_op_convection_diffusion": (C.c_int, [C.c_void_p] + [_dp] * 6),
    "cfdgb_op_bc_main": (C.c_int, [C.c_void_p] + [_dp] * 4),
    "cfdgb_op_bc_copy": (C.c_int, [C.c_void_p] + [_dp] * 6),
    "cfdgb_op_rhs": (C.c_int, [C.c_void_p, C.c_int] + [_dp] * 4),
    "cfdgb_op_spmv": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "cfdgb_op_bicgstab": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, _dp, _dp,
                                    C.POINTER(C.c_int), _dp]),
    "cfdgb_op_update_uf": (C.c_int, [C.c_void_p] + [_dp] * 11),
    "cfdgb_op_solid_fraction": (C.c_int, [C.c_void_p, _dp]),
    "cfdgb_op_cfl": (C.c_int, [C.c_void_p] + [_dp] * 4),
    "cfdgb_op_smagorinsky": (C.c_int, [C.c_void_p] + [_dp] * 4),
    "cfdgb_set_dt": (C.c_int, [C.c_void_p, C.c_double]),
    "cfdgb_write_plot3d": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_double]),
    "cfdgb_read_plot3d": (C.c_int, [C.c_void_p, C.c_char_p, _dp]),
    "cfdgb_op_plot3d_read": (C.c_int, [C.c_void_p, C.c_void_p] + [_dp] * 5),
}


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Load libcfdgb.so; raises if it is missing (there is no other compute path)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                          "or `python cfd_nssolver_forhpc_flowpassingcylinder_gb300/build.py`")
    L = C.CDLL(str(p))
    for name, (res, args) in EXPORTS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if L.cfdgb_abi_version() != ABI_VERSION:
        raise ImportError("libcfdgb ABI version mismatch")
    if path is None:
        _lib = L
    return L


def _check(rc, allow=()):
    if rc != 0 and rc not in allow:
        raise CfdgbError(rc, load_library().cfdgb_last_error().decode())
    return rc


def _ptr(a):
    if a is None:
        return None
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_dp)


def check_division(n: int, seed: int, b: float) -> int:
    """cfdgb_check_division: results of the step kernels' reciprocal division that differ
    from IEEE division over n seeded dividends for divisor b (0 expected)."""
    out = C.c_ulonglong(0)
    _check(load_library().cfdgb_check_division(n, seed, b, C.byref(out)))
    return int(out.value)


def default_config(**kw) -> Config:
    cfg = Config()
    _check(load_library().cfdgb_config_default(C.byref(cfg)))
    for k, v in kw.items():
        if k == "solver" and isinstance(v, str):
            v = SOLVERS[v]
        if k == "precision" and isinstance(v, str):
            v = PRECISIONS[v]
        if k == "grid" and isinstance(v, str):
            v = GRIDS[v]
        if k == "scheme" and isinstance(v, str):
            v = SCHEMES[v]
        if k == "walls" and isinstance(v, str):
            v = WALLS[v]
        if k == "precond" and isinstance(v, str):
            v = PRECONDS[v]
        if k == "dt_mode" and isinstance(v, str):
            v = DT_MODES[v]
        if k == "bc_z" and isinstance(v, str):
            v = BC_Z[v]
        if k == "outflow" and isinstance(v, str):
            v = OUTFLOWS[v]
        if k == "les":
            v = int(bool(v))
        setattr(cfg, k, v)
    return cfg


@dataclass
class StepResult:
    step: int
    iters: int
    outer: int
    status: int
    relres: float
    cd: float
    cl: float
    cfl: float = 0.0
    dt: float = 0.0
    time: float = 0.0


class Solver:
    """One simulation context on the current CUDA device (cfdgb_create)."""

    def __init__(self, cfg: Config | None = None, **kw):
        self._L = load_library()
        self.cfg = cfg if cfg is not None else default_config(**kw)
        h = C.c_void_p()
        _check(self._L.cfdgb_create(C.byref(self.cfg), C.byref(h)))
        self._h = h
        nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
        _check(self._L.cfdgb_padded_dims(h, C.byref(nx), C.byref(ny), C.byref(nz)))
        self.shape = (nx.value, ny.value, nz.value)
        self.cells = self.cfg.nx * self.cfg.ny * self.cfg.nz

    def close(self):
        if getattr(self, "_h", None):
            self._L.cfdgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(self._L.cfdgb_stream(self._h, C.byref(s)))
        return s.value or 0

    def zeros(self):
        return np.zeros(self.shape, dtype=np.float64)

    # ---- state ----
    def init_fields(self, u=None, v=None, w=None, p=None):
        _check(self._L.cfdgb_init_fields(self._h, _ptr(u), _ptr(v), _ptr(w), _ptr(p)))

    def set_fields(self, u=None, v=None, w=None, p=None):
        _check(self._L.cfdgb_set_fields(self._h, _ptr(u), _ptr(v), _ptr(w), _ptr(p)))

    def get_fields(self, out=None):
        out = out or {k: self.zeros() for k in "uvwp"}
        _check(self._L.cfdgb_get_fields(self._h, *(_ptr(out.get(k)) for k in "uvwp")))
        return out

    def get_eta(self):
        e = self.zeros()
        _check(self._L.cfdgb_get_eta(self._h, _ptr(e)))
        return e

    def set_eta(self, eta):
        _check(self._L.cfdgb_set_eta(self._h, _ptr(np.ascontiguousarray(eta, dtype=np.float64))))

    def step(self, n=1, allow_noconv=False):
        st = (StepStats * max(n, 1))()
        rc = self._L.cfdgb_step(self._h, n, st)
        _check(rc, allow=(ENOCONV,) if allow_noconv else ())
        return [StepResult(s.step, s.iters, s.outer, s.status, s.relres, s.cd, s.cl, s.cfl, s.dt, s.time)
                for s in st[:n]]

    def pressure_solve(self):
        it, rr = C.c_int(), C.c_double()
        _check(self._L.cfdgb_pressure_solve(self._h, C.byref(it), C.byref(rr)))
        return it.value, rr.value

    # ---- discrete adjoint ----
    def set_inlet(self, u_in=None):
        """Inlet u per (j, k) of the inlet face, shape (ny, nz); None: the constant 1."""
        a = None if u_in is None else np.ascontiguousarray(u_in, dtype=np.float64).reshape(-1)
        if a is not None and a.size != self.cfg.ny * self.cfg.nz:
            raise ValueError("inlet profile must have ny*nz values")
        _check(self._L.cfdgb_set_inlet(self._h, _ptr(a)))

    def forward(self, nsteps, first, last, ckpt_every):
        """Run nsteps from the initial state; J = mean Cd over steps first..last."""
        obj = Objective(nsteps, first, last, ckpt_every)
        J = C.c_double()
        _check(self._L.cfdgb_forward(self._h, C.byref(obj), C.byref(J)), allow=(ENOCONV,))
        return J.value

    def backward(self):
        """(dJ/d inlet profile (ny, nz), dJ/d eta (padded)) for the last forward()."""
        g_in = np.zeros((self.cfg.ny, self.cfg.nz))
        g_eta = self.zeros()
        _check(self._L.cfdgb_backward(self._h, _ptr(g_in), _ptr(g_eta)), allow=(ENOCONV,))
        return g_in, g_eta

    # ---- instrumentation ----
    def set_kernel_timing(self, on: bool):
        _check(self._L.cfdgb_set_kernel_timing(self._h, int(on)))

    def reset_counters(self):
        _check(self._L.cfdgb_reset_counters(self._h))

    def launch_count(self) -> int:
        n = C.c_longlong()
        _check(self._L.cfdgb_launch_count(self._h, C.byref(n)))
        return n.value

    def kernel_stats(self) -> dict:
        """{kernel name: (total device ms, launches)} since the last reset."""
        out, idx = {}, 0
        name, ms, n = C.c_char_p(), C.c_double(), C.c_longlong()
        while self._L.cfdgb_kernel_stat(self._h, idx, C.byref(name), C.byref(ms), C.byref(n)) == 0:
            out[name.value.decode()] = (ms.value, n.value)
            idx += 1
        return out

    # ---- per-function entry points (host arrays) ----
    def convection_diffusion(self, u, v, w, us, vs, ws):
        _check(self._L.cfdgb_op_convection_diffusion(self._h, *map(_ptr, (u, v, w, us, vs, ws))))

    def smagorinsky(self, u, v, w):
        """SmagorinskyModel: the compact eddy viscosity of padded u, v, w."""
        nut = np.zeros(self.cells)
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w)]
        _check(self._L.cfdgb_op_smagorinsky(self._h, *[_ptr(x) for x in a], _ptr(nut)))
        return nut

    def bc_main(self, u, v, w, p):
        _check(self._L.cfdgb_op_bc_main(self._h, *map(_ptr, (u, v, w, p))))

    def bc_copy(self, u, v, w, us, vs, ws):
        _check(self._L.cfdgb_op_bc_copy(self._h, *map(_ptr, (u, v, w, us, vs, ws))))

    def rhs(self, us, vs, ws, jacobi=False):
        b = np.zeros(self.cells)
        _check(self._L.cfdgb_op_rhs(self._h, int(jacobi), *map(_ptr, (us, vs, ws, b))))
        return b

    def spmv(self, x, jacobi=False):
        y = np.zeros(self.cells)
        _check(self._L.cfdgb_op_spmv(self._h, int(jacobi), _ptr(np.ascontiguousarray(x, dtype=np.float64)), _ptr(y)))
        return y

    def bicgstab(self, rhs, x, tol, maxit=5000, jacobi=False):
        it, rr = C.c_int(), C.c_double()
        rc = self._L.cfdgb_op_bicgstab(self._h, BICGSTAB_JACOBI if jacobi else BICGSTAB, tol, maxit,
                                       _ptr(np.ascontiguousarray(rhs, dtype=np.float64)), _ptr(x),
                                       C.byref(it), C.byref(rr))
        _check(rc, allow=(ENOCONV,))
        return it.value, rr.value, rc

    def update_uf(self, eta, p, us, vs, ws, u3, v3, w3, f=None):
        cd, cl = C.c_double(), C.c_double()
        _check(self._L.cfdgb_op_update_uf(self._h, *map(_ptr, (eta, p, us, vs, ws, u3, v3, w3, f)),
                                          C.byref(cd), C.byref(cl)))
        return cd.value, cl.value

    def solid_fraction(self):
        e = self.zeros()
        _check(self._L.cfdgb_op_solid_fraction(self._h, _ptr(e)))
        return e

    def cfl(self, us, vs, ws):
        """get_Cfl on padded u*: [cfl, U_max x3, U_min x3]."""
        out = np.zeros(7)
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (us, vs, ws)]
        _check(self._L.cfdgb_op_cfl(self._h, *[_ptr(x) for x in a], _ptr(out)))
        return out

    def set_dt(self, dt):
        _check(self._L.cfdgb_set_dt(self._h, float(dt)))
        self.cfg.dt = float(dt)

    def write_plot3d(self, xpath=None, qpath=None, time=0.0):
        """The reference's Plot3D grid (.x) and solution (.q) files of the current state."""
        enc = lambda p: None if p is None else str(p).encode()
        _check(self._L.cfdgb_write_plot3d(self._h, enc(xpath), enc(qpath), float(time)))

    def read_plot3d(self, qpath):
        """Restart from a Plot3D solution file of this grid (QfileRead): it becomes the state,
        as init_fields would set it.  Returns the header [blocks, mach, alpha, Re, time]."""
        head = np.zeros(5)
        _check(self._L.cfdgb_read_plot3d(self._h, str(qpath).encode(), _ptr(head)))
        return head

    def plot3d_read_arrays(self, q):
        """QfileRead's padded p, u, v, w, eta from the float32 arrays of a .q file (after its
        header)."""
        q = np.ascontiguousarray(q, dtype=np.float32)
        out = [self.zeros() for _ in range(5)]
        _check(self._L.cfdgb_op_plot3d_read(self._h, q.ctypes.data_as(C.c_void_p), *map(_ptr, out)))
        return out


def perturbation(shape, seed, amp):
    """The seeded interior perturbation (splitmix64, uniform(-amp, amp)) that
    cfdgb_init_fields adds to u, v, w; returned as three padded arrays."""
    nx, ny, nz = shape
    n = (nx - 4) * (ny - 4) * (nz - 4)
    s = np.uint64(seed)
    with np.errstate(over="ignore"):
        idx = np.arange(1, 3 * n + 1, dtype=np.uint64)
        z = s + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    r = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    d = amp * (2.0 * r - 1.0)
    out = []
    for c in range(3):
        a = np.zeros(shape)
        a[2:-2, 2:-2, 2:-2] = d[c * n:(c + 1) * n].reshape(nx - 4, ny - 4, nz - 4)
        out.append(a)
    return out
