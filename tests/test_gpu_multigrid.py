"""MIXED precision with the multigrid-preconditioned FP32 BiCGSTAB sweeps, through the
C ABI.  The preconditioner changes the path to the solution, not the solution: every solve
must end below the FP64 tolerance in the FP64 residual, and the fields must agree with the
plain FP64 BiCGSTAB run of the same case (relative L2 1e-6 over 5 steps, 1e-4 over 20
seeded steps, the bars of the other MIXED solvers)."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg

pytestmark = pytest.mark.gpu


def vel_err(f, ref):
    get = lambda a: a[2:-2, 2:-2, 2:-2]
    scale = np.sqrt(sum(np.linalg.norm(get(ref[k])) ** 2 for k in "uvw"))
    return {k: float(np.linalg.norm(get(f[k]) - get(ref[k])) / scale) for k in "uvw"}


CASES = {
    "96x48x4": dict(),
    "48x24x6": dict(nx=48, ny=24, nz=6, lx=12.0, ly=6.0, lz=1.5, cx=3.0, cy=3.0),
    "128x64x16": dict(nx=128, ny=64, nz=16, lx=32.0, ly=16.0, lz=4.0, cx=8.0, cy=8.0),
    "120x40x12": dict(nx=120, ny=40, nz=12, lx=30.0, ly=10.0, lz=3.0, cx=7.5, cy=5.0),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("solver", ["bicgstab", "jacobi"])
def test_multigrid_sweeps_reach_the_fp64_solution(solver, case):
    dom = CASES[case]
    with cg.Solver(solver=solver, precision="mixed", precond="multigrid", **dom) as a, \
            cg.Solver(solver=solver, **dom) as b:
        a.init_fields()
        b.init_fields()
        sa, sb = a.step(5), b.step(5)
        fa, fb = a.get_fields(), b.get_fields()
    assert all(r.status == 0 and r.relres < 1e-8 for r in sa[1:]), [(r.status, r.relres) for r in sa]
    # a few dozen preconditioned iterations where the plain sweeps take hundreds
    assert all(r.iters <= 200 for r in sa[1:]), [r.iters for r in sa]
    for k, e in vel_err(fa, fb).items():
        assert e <= 1e-6, (solver, case, k, e)


@pytest.mark.parametrize("env", [{}, {"CFDGB_SCALAR_FP32": "1"}], ids=["quads", "scalar"])
def test_multigrid_quad_and_scalar_kernels_agree(env, monkeypatch):
    """The preconditioned iteration's quad kernels (nz a multiple of 4) and its scalar ones
    (any nz; forced here) on the same grid: both reach the FP64 run's fields."""
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    dom = CASES["128x64x16"]
    with cg.Solver(precision="mixed", precond="multigrid", **dom) as a, cg.Solver(**dom) as b:
        a.init_fields()
        b.init_fields()
        sa, sb = a.step(4), b.step(4)
        fa, fb = a.get_fields(), b.get_fields()
    assert all(r.status == 0 and r.relres < 1e-8 for r in sa[1:])
    for k, e in vel_err(fa, fb).items():
        assert e <= 1e-6, (env, k, e)


MARCH_CASES = {
    # levels 128x64x16 and 64x32x8 above the one-block tail: nz / 4 = 4 and 2
    "128x64x16": CASES["128x64x16"],
    # four marching levels (nz / 4 = 16, 8, 4, 2), several bands and segments on each
    "256x128x64": dict(nx=256, ny=128, nz=64, lx=32.0, ly=16.0, lz=4.0, cx=8.0, cy=8.0),
    # a ragged band on level 0 (40 rows: bands of 32 and 8), one band on level 1
    "64x40x32": dict(nx=64, ny=40, nz=32, lx=16.0, ly=10.0, lz=8.0, cx=4.0, cy=5.0, project_rhs=1),
    # level 0 on the per-pass kernels (nz / 4 = 32), level 1 marching: the two paths meet
    "64x32x128": dict(nx=64, ny=32, nz=128, lx=16.0, ly=8.0, lz=32.0, cx=4.0, cy=4.0, project_rhs=1),
    # the stated boundary set: periodic z on every level, the seeded perturbation
    "set 128x64x16": dict(CASES["128x64x16"], seed=7, amp=1e-3, **cg.BOUNDARY_SET),
}


@pytest.mark.parametrize("case", sorted(MARCH_CASES))
@pytest.mark.parametrize("solver", ["bicgstab", "jacobi"])
def test_multigrid_marching_kernels_match_the_per_pass_kernels(solver, case, monkeypatch):
    """The two marching kernels a level (pre-smoothing + restriction, prolongation +
    post-smoothing) form every value by the per-pass kernels' expressions in their order:
    the whole run, fields and iteration counts, is identical bit for bit."""
    dom = MARCH_CASES[case]
    runs = []
    for per_pass in (False, True):
        if per_pass:
            monkeypatch.setenv("CFDGB_MG_PER_PASS", "1")
        else:
            monkeypatch.delenv("CFDGB_MG_PER_PASS", raising=False)
        with cg.Solver(solver=solver, precision="mixed", precond="multigrid", **dom) as s:
            s.init_fields()
            st = s.step(3)
            runs.append((s.get_fields(), [(r.iters, r.outer, r.relres) for r in st]))
    (fa, sa), (fb, sb) = runs
    assert sa == sb, (sa, sb)
    assert all(r[2] < 1e-8 for r in sa[1:]), sa
    for k in "uvwp":
        assert np.array_equal(fa[k], fb[k]), (case, k, float(np.abs(fa[k] - fb[k]).max()))


def test_multigrid_with_perturbation_and_projection():
    """The seeded-perturbation case over 20 steps."""
    res = {}
    for prec, extra in (("fp64", {}), ("mixed", {"precond": "multigrid"})):
        with cg.Solver(precision=prec, tol=1e-8, seed=1234, amp=1e-3, project_rhs=1, **extra) as s:
            s.init_fields()
            st = s.step(20)
            res[prec] = (s.get_fields(), st)
    assert all(r.relres < 1e-8 and r.status == 0 for r in res["mixed"][1][1:])
    assert all(r.outer >= 1 for r in res["mixed"][1][1:])
    for k, e in vel_err(res["mixed"][0], res["fp64"][0]).items():
        assert e < 1e-4, (k, e)


@pytest.mark.parametrize("shape", [(3, 3, 3), (5, 4, 3), (7, 5, 9), (12, 6, 13), (16, 10, 7)])
def test_multigrid_small_and_ragged_grids(shape):
    """Grids of a single level (all extents odd, or at most 64 cells) and ragged ones that
    halve along some axes only; right-hand side projected as for the other small-grid runs."""
    nx, ny, nz = shape
    dom = dict(nx=nx, ny=ny, nz=nz, lx=float(nx), ly=float(ny), lz=float(nz), cx=nx / 2.0, cy=ny / 2.0, radius=0.75,
               project_rhs=1)
    with cg.Solver(precision="mixed", precond="multigrid", tol=1e-8, **dom) as s:
        s.init_fields()
        st = s.step(3)
    assert all(r.status == 0 and r.relres < 1e-8 for r in st[1:]), (shape, st)


@pytest.mark.parametrize("case", ["96x48x4", "128x64x16"])
@pytest.mark.parametrize("solver", ["bicgstab", "jacobi"])
def test_fp64_multigrid_reaches_the_fp64_solution(solver, case):
    """The FP64 BiCGSTAB preconditioned by the same V-cycle in FP64 (the like-for-like FP64
    counterpart of the MIXED multigrid sweep): every solve below the tolerance in a few
    dozen iterations, fields within 1e-6 of the plain FP64 BiCGSTAB, and the MIXED multigrid
    run within 1e-6 of it."""
    dom = CASES[case]
    runs = {}
    for key, kw in (("mg64", dict(precond="multigrid")), ("plain", {}),
                    ("mg32", dict(precond="multigrid", precision="mixed"))):
        with cg.Solver(solver=solver, **kw, **dom) as s:
            s.init_fields()
            st = s.step(5)
            runs[key] = (s.get_fields(), st)
    st = runs["mg64"][1]
    assert all(r.status == 0 and r.relres < 1e-8 for r in st[1:]), [(r.status, r.relres) for r in st]
    assert all(r.iters <= 100 for r in st[1:]), [r.iters for r in st]
    for ref in ("plain", "mg32"):
        for k, e in vel_err(runs["mg64"][0], runs[ref][0]).items():
            assert e <= 1e-6, (solver, case, ref, k, e)


@pytest.mark.parametrize("bad", [
    dict(precond="multigrid", solver="cg"),                         # not BiCGSTAB (FP64)
    dict(precond="multigrid", precision="mixed", solver="cg"),      # not BiCGSTAB
    dict(precond="multigrid", precision="mixed", solver="rbsor"),
    dict(precond=7, precision="mixed"),                             # unknown value
    dict(precond="multigrid", precision="mixed", nx=99, ny=45, nz=33, lx=33.0, ly=15.0, lz=11.0),  # no coarsening
])
def test_multigrid_rejects_what_it_does_not_cover(bad):
    with pytest.raises(cg.CfdgbError) as e:
        cg.Solver(**bad)
    assert e.value.status == cg.EINVAL
