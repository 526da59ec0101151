"""One CUDA graph per time step: after the first step, an FP64 Krylov step (convection-
diffusion with its CFL reduction, right-hand side, the solver's set-up, its convergence
loop as a conditional WHILE node, NaN recovery, transform, correction, ghost fill and a
record of the step's scalars) is a single graph launch, and cfdgb_step reads the records
back once.  The graph path must give the host-driven path's results bit for bit (same
kernels, same order), and its launch count must be the kernels it ran."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg

pytestmark = pytest.mark.gpu

CASE = dict(nx=128, ny=64, nz=16, lx=32.0, ly=16.0, lz=4.0, cx=8.0, cy=8.0)


def _run(monkeypatch, graph, **kw):
    if graph:
        monkeypatch.delenv("CFDGB_NO_STEP_GRAPH", raising=False)
    else:
        monkeypatch.setenv("CFDGB_NO_STEP_GRAPH", "1")
    with cg.Solver(**CASE, **kw) as s:
        s.init_fields()
        s.step(1)
        s.step(3)  # the graph is captured here
        s.init_fields()  # a restart clears the solver scalars; the graph must not depend on them
        st = s.step(1) + s.step(5)  # the second call runs as graphs
        s.reset_counters()
        st += s.step(2)
        n = s.launch_count()
        f = s.get_fields()
    return st, f, n


@pytest.mark.parametrize("kw", [dict(solver="jacobi"), dict(solver="bicgstab"), dict(solver="cg"),
                                dict(solver="jacobi", precond="multigrid"),
                                dict(solver="jacobi", dt_mode="cfl", cfl_target=0.2)],
                         ids=["jacobi", "spe", "cg", "multigrid64", "cfl_dt"])
def test_step_graph_matches_host_driven_step(monkeypatch, kw):
    sg, fg, ng = _run(monkeypatch, True, **kw)
    sh, fh, nh = _run(monkeypatch, False, **kw)
    for a, b in zip(sg, sh):
        assert (a.step, a.iters, a.status, a.relres, a.cd, a.cl, a.cfl, a.dt, a.time) == \
               (b.step, b.iters, b.status, b.relres, b.cd, b.cl, b.cfl, b.dt, b.time)
    for k in "uvwp":
        np.testing.assert_array_equal(fg[k], fh[k])
    # the host path counts every launch of its captured chunks; the graph path counts the
    # WHILE bodies it ran (one condition kernel each) and its record kernel, so it is at
    # least the host path's count and at most a chunk of iterations more per step
    assert nh <= ng <= nh + 2 * 64 * 8
