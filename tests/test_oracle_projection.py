"""The Poisson right-hand side projection (project_rhs), on the oracle (CPU).

With the reference's boundary table (zero-gradient outflow and walls), a non-uniform
inflow leaves the Neumann problem without a solution: its BiCGSTAB runs to the 5000
iteration cap and the fields blow up.  Removing the right-hand side's mean before each
solve makes the system consistent; the unperturbed case, already consistent, is unchanged
to the solver tolerance."""
import numpy as np

from oracle import oracle as O

GRID = (32, 16, 4, 8.0, 4.0, 1.0, 2.0)


def test_reference_diverges_on_a_nonuniform_inflow_and_projection_fixes_it():
    g = O.Grid(*GRID)
    d = np.random.default_rng(7).standard_normal((16, 4))
    inlet = 1.0 + 1e-6 * d
    raw = O.run(g, 3, 100.0, 0.005, 1e-12, "spe", inlet=inlet)
    assert raw["iters"][1] == 5000 and abs(raw["cd"][2]) > 1e100
    for solver in ("spe", "csr"):
        r = O.run(g, 3, 100.0, 0.005, 1e-12, solver, inlet=inlet, project=True)
        assert np.all(r["iters"][1:] < 500) and np.all(r["err"][1:] < 1e-12)
        assert np.all(np.isfinite(r["cd"]))


def test_projection_leaves_a_consistent_problem_unchanged():
    g = O.Grid(*GRID)
    a = O.run(g, 4, 100.0, 0.005, 1e-12, "spe")
    b = O.run(g, 4, 100.0, 0.005, 1e-12, "spe", project=True)
    np.testing.assert_allclose(b["cd"], a["cd"], rtol=1e-9)
    for k in ("u", "v", "w"):
        assert np.abs(b[k] - a[k]).max() <= 1e-9 * np.abs(a["u"]).max()


def test_cg_restatement_converges_to_the_bicgstab_solution():
    """The CG restatement (inc/solver/cg.hpp's method) reaches the same fields as the
    reference's BiCGSTAB at a tight tolerance."""
    g = O.Grid(*GRID)
    a = O.run(g, 4, 100.0, 0.005, 1e-13, "spe")
    b = O.run(g, 4, 100.0, 0.005, 1e-13, "cg")
    assert np.all(b["err"][1:] < 1e-13) and np.all(b["iters"][1:] > 0)
    np.testing.assert_allclose(b["cd"], a["cd"], rtol=1e-11)
    for k in ("u", "v", "w"):
        assert np.abs(b[k] - a[k]).max() <= 1e-11 * np.abs(a["u"]).max()
