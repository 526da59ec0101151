"""Per-function parity of the CUDA kernels, called through the C ABI, against the golden
vectors made by the reference's own functions (tests/golden/make_golden.py).

The FP64 step kernels are compiled without FMA contraction and follow the reference's
operation order, so the bar is bit-exact.  Reductions (drag sum, BiCGSTAB dots) are
tree-ordered on the GPU and serial in the reference: relative tolerance 1e-12 there."""
import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu
UNITS = ["unit_g10x8x6_h025.npz", "unit_g10x8x6_h030.npz"]


def _solver_for(meta, **kw):
    nxc, nyc, nzc = (int(x) for x in meta[:3])
    lx, ly, lz, cx, Re, dt = meta[3], meta[4], meta[5], meta[6], meta[7], meta[8]
    return cg.Solver(nx=nxc, ny=nyc, nz=nzc, lx=lx, ly=ly, lz=lz, cx=cx, cy=ly / 2.0, Re=Re, dt=dt, **kw)


@pytest.fixture(params=UNITS, scope="module")
def unit(request):
    from conftest import load_golden
    z = load_golden(request.param)
    s = _solver_for(z["meta"])
    P = {k: v.reshape(s.shape) for k, v in z.items() if v.size == np.prod(s.shape)}
    yield z, s, P
    s.close()


def test_convection_diffusion_bit_exact(unit):
    z, s, P = unit
    us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
    s.convection_diffusion(P["in_u"], P["in_v"], P["in_w"], us, vs, ws)
    np.testing.assert_array_equal(us, P["cd_u"])
    np.testing.assert_array_equal(vs, P["cd_v"])
    np.testing.assert_array_equal(ws, P["cd_w"])


@pytest.mark.parametrize("name", UNITS)
def test_lud_ud_and_smagorinsky_kernels(name):
    """ConvectionDifussion with LUD (bit-exact against the reference built with it), the
    Smagorinsky eddy viscosity and the conv-diff using it (against the reference built
    with TERBULENCE_SMAGORINSKY; its length scale pow(Dx Dy Dz, 1/3) comes from the host's
    libm, which may round one ulp apart between machines, hence 1e-15 there), and UD
    (against the oracle: no reference build compiles it)."""
    from conftest import load_golden
    z = load_golden(name)
    zv = load_golden(name.replace(".npz", "_variants.npz"))
    meta = z["meta"]
    nxc, nyc, nzc = (int(x) for x in meta[:3])
    shape = (nxc + 4, nyc + 4, nzc + 4)
    P = {k: z[k].reshape(shape) for k in ("in_u", "in_v", "in_w", "in_us", "in_vs", "in_ws")}

    def cd(s):
        out = [P[k].copy() for k in ("in_us", "in_vs", "in_ws")]
        s.convection_diffusion(P["in_u"], P["in_v"], P["in_w"], *out)
        return out

    with _solver_for(meta, scheme="lud") as s:
        for a, c in zip(cd(s), "uvw"):
            np.testing.assert_array_equal(a.ravel(), zv["cd_lud_" + c])
    with _solver_for(meta, les=True) as s:
        np.testing.assert_allclose(s.smagorinsky(P["in_u"], P["in_v"], P["in_w"]), zv["les_nut"], rtol=1e-15)
        for a, c in zip(cd(s), "uvw"):
            np.testing.assert_allclose(a.ravel(), zv["cd_les_" + c], rtol=1e-15)
    g = O.Grid(nxc, nyc, nzc, *meta[3:7], scheme="ud")
    ref = [P[k].copy() for k in ("in_us", "in_vs", "in_ws")]
    O.convection_diffusion(g, meta[8], 1.0 / meta[7], P["in_u"], P["in_v"], P["in_w"], *ref)
    with _solver_for(meta, scheme="ud") as s:
        for a, b in zip(cd(s), ref):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", UNITS)
def test_free_slip_walls_bit_exact(name):
    """The free-slip y-wall rows of the boundary table (FLOWpassing.hpp:14-21): ghost fill
    and copy bit-exact against the reference built with them."""
    from conftest import load_golden
    z = load_golden(name)
    zv = load_golden(name.replace(".npz", "_variants.npz"))
    meta = z["meta"]
    with _solver_for(meta, walls="free_slip") as s:
        P = {k: z[k].reshape(s.shape).copy() for k in ("in_u", "in_v", "in_w", "in_p", "in_us", "in_vs", "in_ws")}
        u, v, w, p = P["in_u"], P["in_v"], P["in_w"], P["in_p"]
        s.bc_main(u, v, w, p)
        for a, k in ((u, "bc_u"), (v, "bc_v"), (w, "bc_w"), (p, "bc_p")):
            np.testing.assert_array_equal(a.ravel(), zv["freeslip_" + k])
        us, vs, ws = P["in_us"], P["in_vs"], P["in_ws"]
        s.bc_copy(u, v, w, us, vs, ws)
        for a, k in ((us, "bcc_u"), (vs, "bcc_v"), (ws, "bcc_w")):
            np.testing.assert_array_equal(a.ravel(), zv["freeslip_" + k])


def test_bc_main_and_copy_bit_exact(unit):
    z, s, P = unit
    u, v, w, p = (P[k].copy() for k in ("in_u", "in_v", "in_w", "in_p"))
    s.bc_main(u, v, w, p)
    for a, k in ((u, "bc_u"), (v, "bc_v"), (w, "bc_w"), (p, "bc_p")):
        np.testing.assert_array_equal(a, P[k])
    us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
    s.bc_copy(u, v, w, us, vs, ws)
    for a, k in ((us, "bcc_u"), (vs, "bcc_v"), (ws, "bcc_w")):
        np.testing.assert_array_equal(a, P[k])


def test_rhs_bit_exact(unit):
    z, s, P = unit
    np.testing.assert_array_equal(s.rhs(P["in_us"], P["in_vs"], P["in_ws"]), z["b_spe"])
    np.testing.assert_array_equal(s.rhs(P["in_us"], P["in_vs"], P["in_ws"], jacobi=True), z["b_jac"])


def test_spmv_bit_exact(unit):
    z, s, P = unit
    np.testing.assert_array_equal(s.spmv(z["in_x"]), z["y_spe"])
    np.testing.assert_array_equal(s.spmv(z["in_x"], jacobi=True), z["y_csr"])


def test_update_uf_bit_exact_and_drag(unit):
    z, s, P = unit
    u3, v3, w3 = P["in_u3"].copy(), P["in_v3"].copy(), P["in_w3"].copy()
    f = np.zeros(3 * int(np.prod(s.shape)))
    cd, cl = s.update_uf(P["in_eta"], P["in_p"], P["in_us"], P["in_vs"], P["in_ws"], u3, v3, w3, f)
    np.testing.assert_array_equal(u3, P["uf_u"])
    np.testing.assert_array_equal(v3, P["uf_v"])
    np.testing.assert_array_equal(w3, P["uf_w"])
    np.testing.assert_array_equal(f, z["uf_f"])
    np.testing.assert_allclose([cd, cl], z["cdcl"], rtol=1e-12, atol=0)


def test_solid_fraction_bit_exact(unit):
    z, s, P = unit
    np.testing.assert_array_equal(s.solid_fraction(), P["eta_cyl"])
    np.testing.assert_array_equal(s.get_eta(), P["eta_cyl"])


def test_bicgstab_matches_reference_solution(unit):
    z, s, P = unit
    x = np.zeros(s.cells)
    it, rr, rc = s.bicgstab(z["bicg_rhs"], x, 1e-10)
    assert rc == 0 and rr < 1e-10
    # same algorithm, different dot-product rounding: iteration count within a few,
    # solutions agree to the solve tolerance (singular operator: compare mean-free parts)
    assert abs(it - int(z["bicg_it"][0])) <= 3
    a, b = x - x.mean(), z["bicg_x"] - z["bicg_x"].mean()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-8


def test_mixed_stencil_sweep_within_fp32_error(unit):
    z, s0, P = unit
    with _solver_for(z["meta"], precision="mixed") as s:
        us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
        s.convection_diffusion(P["in_u"], P["in_v"], P["in_w"], us, vs, ws)
        dt = z["meta"][8]
        for a, k, src in ((us, "cd_u", "in_u"), (vs, "cd_v", "in_v"), (ws, "cd_w", "in_w")):
            # the FP32 part is the increment dt*(conv + diff); bound its error relative to
            # the increment's own scale
            inc_ref = P[k] - P[src]
            err = np.abs((a - P[src]) - inc_ref).max()
            assert err <= 1e-5 * np.abs(inc_ref).max() + 1e-7 * dt, (k, err)


def test_fp32_operator_matches_fp64(unit):
    z, s, P = unit
    y64 = O.spe_multiply(O.Grid(*(int(v) for v in z["meta"][:3]), *z["meta"][3:7]), z["in_x"])
    np.testing.assert_array_equal(s.spmv(z["in_x"]), y64)


def test_cfl_bit_exact(unit):
    """get_Cfl (cfl.hpp:3) on u*: CFL number (divisions in the reference's order, exact
    maxima) and velocity extremes, against the reference's own values."""
    z, s, P = unit
    np.testing.assert_array_equal(s.cfl(P["in_us"], P["in_vs"], P["in_ws"]), z["cfl"])


def test_plot3d_files_byte_identical(unit, tmp_path):
    """The reference's Plot3D .x and .q files of a state (T3, p, eta at time 0), byte for
    byte; the solution arrays are packed on the GPU."""
    z, s, P = unit
    s.init_fields()
    s.set_fields(u=P["in_u3"], v=P["in_v3"], w=P["in_w3"], p=P["in_p"])
    s.set_eta(P["in_eta"])
    q, x = tmp_path / "P3D00.q", tmp_path / "P3D.x"
    s.write_plot3d(x, q, 0.0)
    np.testing.assert_array_equal(np.fromfile(x, dtype=np.uint8), z["p3d_x"])
    np.testing.assert_array_equal(np.fromfile(q, dtype=np.uint8), z["p3d_q"])


def test_plot3d_read_arrays_bit_exact(unit):
    """QfileRead's padded p, u, v, w, eta rebuilt on the GPU from the reference's own .q
    file: bit-exact against what the reference's reader returned."""
    z, s, P = unit
    q = z["p3d_q"][32:].view("<f4")  # after the 4 int + 4 float header
    for name, f in zip(("p", "u", "v", "w", "eta"), s.plot3d_read_arrays(q)):
        np.testing.assert_array_equal(f, P["p3d_read_" + name])


def test_plot3d_restart_sets_the_state(unit, tmp_path):
    """cfdgb_read_plot3d: the file's fields become the state, with the ghost fill a run
    starts with (BC_staggered_main on the reader's arrays), and the header comes back."""
    z, s, P = unit
    q = tmp_path / "P3D00.q"
    z["p3d_q"].tofile(q)
    head = s.read_plot3d(q)
    np.testing.assert_array_equal(head, z["p3d_read_head"])
    g = O.Grid(*(int(x) for x in z["meta"][:3]), *z["meta"][3:7])
    ref = {k: P["p3d_read_" + k].copy() for k in "uvwp"}
    O.bc_main(g, ref["u"], ref["v"], ref["w"], ref["p"])
    got = s.get_fields()
    for k in "uvwp":
        np.testing.assert_array_equal(got[k], ref[k])
    bad = tmp_path / "short.q"
    z["p3d_q"][:100].tofile(bad)
    with pytest.raises(RuntimeError):
        s.read_plot3d(bad)
