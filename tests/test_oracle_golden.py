"""Pins the C restatement (oracle/cfd_oracle.c) to golden vectors produced by the
reference's own functions (tests/golden/make_golden.py).  The bar is bit-exact: both are
compiled with -ffp-contract=off and the reference ran at one OpenMP thread."""
import numpy as np
import pytest

from oracle import oracle as O

UNITS = ["unit_g10x8x6_h025.npz", "unit_g10x8x6_h030.npz"]


def _grid(meta):
    nxc, nyc, nzc = (int(x) for x in meta[:3])
    lx, ly, lz, cx = meta[3:7]
    return O.Grid(nxc, nyc, nzc, lx, ly, lz, cx)


@pytest.fixture(params=UNITS)
def unit(request, golden):
    z = golden(request.param)
    g = _grid(z["meta"])
    sh = g.shape
    padded = {k: v.reshape(sh) for k, v in z.items()
              if v.size == g.shape[0] * g.shape[1] * g.shape[2]}
    return z, g, padded


def test_convection_diffusion_bit_exact(unit):
    z, g, P = unit
    Re, dt = z["meta"][7], z["meta"][8]
    us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
    O.convection_diffusion(g, dt, 1.0 / Re, P["in_u"], P["in_v"], P["in_w"], us, vs, ws)
    np.testing.assert_array_equal(us, P["cd_u"])
    np.testing.assert_array_equal(vs, P["cd_v"])
    np.testing.assert_array_equal(ws, P["cd_w"])


@pytest.mark.parametrize("name", UNITS)
def test_lud_and_smagorinsky_bit_exact(name, golden):
    """The reference's other convection scheme (LUD) and its Smagorinsky model, from builds
    of the reference with those switched on: eddy viscosity and ConvectionDifussion."""
    z = golden(name)
    zv = golden(name.replace(".npz", "_variants.npz"))
    meta = z["meta"]
    Re, dt = meta[7], meta[8]
    args = (int(meta[0]), int(meta[1]), int(meta[2]), *meta[3:7])
    g = O.Grid(*args, scheme="lud")
    P = {k: z[k].reshape(g.shape) for k in ("in_u", "in_v", "in_w", "in_us", "in_vs", "in_ws")}
    us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
    O.convection_diffusion(g, dt, 1.0 / Re, P["in_u"], P["in_v"], P["in_w"], us, vs, ws)
    for a, c in ((us, "u"), (vs, "v"), (ws, "w")):
        np.testing.assert_array_equal(a.ravel(), zv["cd_lud_" + c])
    g = O.Grid(*args, les=True)
    nut = O.smagorinsky(g, P["in_u"], P["in_v"], P["in_w"])
    np.testing.assert_array_equal(nut, zv["les_nut"])
    us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
    O.convection_diffusion(g, dt, 1.0 / Re, P["in_u"], P["in_v"], P["in_w"], us, vs, ws, nut=nut)
    for a, c in ((us, "u"), (vs, "v"), (ws, "w")):
        np.testing.assert_array_equal(a.ravel(), zv["cd_les_" + c])


@pytest.mark.parametrize("name", UNITS)
def test_free_slip_walls_bit_exact(name, golden):
    """The free-slip rows of the boundary table (FLOWpassing.hpp:14-21, commented out in the
    reference; a build of the reference with them): BC_staggered_main and the copy."""
    z = golden(name)
    zv = golden(name.replace(".npz", "_variants.npz"))
    meta = z["meta"]
    g = O.Grid(int(meta[0]), int(meta[1]), int(meta[2]), *meta[3:7], walls="free_slip")
    P = {k: z[k].reshape(g.shape).copy() for k in ("in_u", "in_v", "in_w", "in_p", "in_us", "in_vs", "in_ws")}
    u, v, w, p = P["in_u"], P["in_v"], P["in_w"], P["in_p"]
    O.bc_main(g, u, v, w, p)
    for a, k in ((u, "bc_u"), (v, "bc_v"), (w, "bc_w"), (p, "bc_p")):
        np.testing.assert_array_equal(a.ravel(), zv["freeslip_" + k])
    us, vs, ws = P["in_us"], P["in_vs"], P["in_ws"]
    O.bc_copy(g, u, v, w, us, vs, ws)
    for a, k in ((us, "bcc_u"), (vs, "bcc_v"), (ws, "bcc_w")):
        np.testing.assert_array_equal(a.ravel(), zv["freeslip_" + k])


def test_upwind_scheme_is_the_upwind_cell():
    """UD (UdUnit, Convection_Difussion.hpp:150): no reference build compiles it, so its
    restatement is checked by its definition: every face value is the upwind cell's, so a
    flow along +x with v = w = 0 and nu = 0 gives u* - u = -dt (u_i^2 - u_{i-1}^2)/dx."""
    g = O.Grid(12, 8, 6, 3.0, 2.0, 1.5, 1.5, scheme="ud")
    rng = np.random.default_rng(3)
    u = 1.0 + 0.1 * rng.random(g.shape)
    v = np.zeros(g.shape)
    w = np.zeros(g.shape)
    us, vs, ws = u.copy(), v.copy(), w.copy()
    dt = 0.01
    O.convection_diffusion(g, dt, 0.0, u, v, w, us, vs, ws)
    dx = 3.0 / 12
    i, j, k = 5, 4, 3
    upwind = u[i, j, k] - dt * (u[i, j, k] ** 2 - u[i - 1, j, k] ** 2) / dx
    assert us[i, j, k] == pytest.approx(upwind, rel=1e-14)


def test_bc_main_and_copy_bit_exact(unit):
    z, g, P = unit
    u, v, w, p = (P[k].copy() for k in ("in_u", "in_v", "in_w", "in_p"))
    O.bc_main(g, u, v, w, p)
    for a, k in ((u, "bc_u"), (v, "bc_v"), (w, "bc_w"), (p, "bc_p")):
        np.testing.assert_array_equal(a, P[k])
    us, vs, ws = P["in_us"].copy(), P["in_vs"].copy(), P["in_ws"].copy()
    O.bc_copy(g, u, v, w, us, vs, ws)
    for a, k in ((us, "bcc_u"), (vs, "bcc_v"), (ws, "bcc_w")):
        np.testing.assert_array_equal(a, P[k])


def test_rhs_and_jacobi_bit_exact(unit):
    z, g, P = unit
    dt = z["meta"][8]
    np.testing.assert_array_equal(O.rhs(g, dt, P["in_us"], P["in_vs"], P["in_ws"]), z["b_spe"])
    jp = O.jacobi_scale(g)
    np.testing.assert_array_equal(jp, z["jp"])
    np.testing.assert_array_equal(O.rhs(g, dt, P["in_us"], P["in_vs"], P["in_ws"], jp), z["b_jac"])


def test_operators_bit_exact(unit):
    z, g, P = unit
    np.testing.assert_array_equal(O.spe_multiply(g, z["in_x"]), z["y_spe"])
    np.testing.assert_array_equal(O.csr_multiply(g, z["in_x"]), z["y_csr"])


def test_update_uf_and_drag_bit_exact(unit):
    z, g, P = unit
    dt = z["meta"][8]
    u3, v3, w3 = P["in_u3"].copy(), P["in_v3"].copy(), P["in_w3"].copy()
    f = np.zeros(3 * g.shape[0] * g.shape[1] * g.shape[2])
    O.update_uf(g, dt, P["in_eta"], P["in_p"], P["in_us"], P["in_vs"], P["in_ws"], u3, v3, w3, f)
    np.testing.assert_array_equal(u3, P["uf_u"])
    np.testing.assert_array_equal(v3, P["uf_v"])
    np.testing.assert_array_equal(w3, P["uf_w"])
    np.testing.assert_array_equal(f, z["uf_f"])
    cd = -2.0 * O.force_sum(g, f, 0) / g._g.lz
    cl = -2.0 * O.force_sum(g, f, 1) / g._g.lz
    np.testing.assert_array_equal(np.array([cd, cl]), z["cdcl"])


def test_solid_fraction_bit_exact(unit):
    z, g, P = unit
    eta = O.dfib_cylinder_z(g)
    np.testing.assert_array_equal(eta, P["eta_cyl"])
    assert 0 < eta.max() <= 1.0 and eta.min() == 0.0


def test_bicgstab_bit_exact(unit):
    z, g, P = unit
    s = O.BiCGSTAB(g, 0, 1e-10)
    x = np.zeros(g.cells)
    it, err = s.solve(z["bicg_rhs"], x)
    np.testing.assert_array_equal(x, z["bicg_x"])
    assert (it, err) == (int(z["bicg_it"][0]), z["bicg_it"][1])


def test_sor_bit_exact(unit):
    z, g, P = unit
    dt = z["meta"][8]
    p = P["in_p"].copy()
    it, err = O.sor(g, dt, 1.7, 1e-30, 7, P["in_us"], P["in_vs"], P["in_ws"], p)
    np.testing.assert_array_equal(p, P["sor_p"])
    assert (it, err) == (int(z["sor_it"][0]), z["sor_it"][1])


@pytest.mark.parametrize("case", ["c1_spe_tol1e-13_20", "c1_csr_tol1e-13_20",
                                  "c1_sor_tol1e-3_4", "c1_spe_tol1e-8_200",
                                  "c1_lud_spe_tol1e-13_20", "c1_les_spe_tol1e-13_20",
                                  "c1_freeslip_spe_tol1e-13_20"])
def test_whole_run_bit_exact(case, golden):
    z = golden(f"run_{case}.npz")
    m = z["meta"]
    nxc, nyc, nzc = (int(x) for x in m[:3])
    extra = {}
    if "scheme" in z:  # runs of the reference built with LUD, its Smagorinsky model or free slip
        extra = dict(scheme=str(z["scheme"]), les=bool(z["les"]))
        if "walls" in z:
            extra["walls"] = str(z["walls"])
    g = O.Grid(nxc, nyc, nzc, *m[3:7], **extra)
    steps, Re, dt, tol, omega = int(m[7]), m[8], m[9], m[10], m[11]
    r = O.run(g, steps, Re, dt, tol, str(z["solver"]), omega)
    np.testing.assert_array_equal(r["iters"], z["iters"])
    np.testing.assert_array_equal(r["cd"], z["cd"])
    np.testing.assert_array_equal(r["cl"], z["cl"])
    for k in ("u", "v", "w", "p"):
        np.testing.assert_array_equal(r[k][2:-2, 2:-2, 2:-2], z[k])


def test_cfl_bit_exact(unit):
    """get_Cfl (cfl.hpp:3) on u*: the CFL number and the velocity extremes."""
    z, g, P = unit
    dt = z["meta"][8]
    out = O.cfl(g, dt, P["in_us"], P["in_vs"], P["in_ws"])
    np.testing.assert_array_equal(out, z["cfl"])


def test_plot3d_files_byte_identical(unit, tmp_path):
    """The reference's Plot3D grid (.x) and solution (.q) files, byte for byte: T3, p and
    eta of the unit fields at time 0."""
    z, g, P = unit
    Re = z["meta"][7]
    q, x = tmp_path / "P3D00.q", tmp_path / "P3D.x"
    O.plot3d(g, P["in_p"], P["in_u3"], P["in_v3"], P["in_w3"], P["in_eta"], Re, 0.0, q, x)
    np.testing.assert_array_equal(np.fromfile(x, dtype=np.uint8), z["p3d_x"])
    np.testing.assert_array_equal(np.fromfile(q, dtype=np.uint8), z["p3d_q"])


def test_plot3d_read_bit_exact(unit, tmp_path):
    """QfileRead (qfileRead.hpp:6) of the reference's own .q file: header and the padded
    p, u, v, w, eta it rebuilds from the cell-centred values."""
    z, g, P = unit
    q = tmp_path / "P3D00.q"
    z["p3d_q"].tofile(q)
    head, *fields = O.plot3d_read(g, q)
    np.testing.assert_array_equal(head, z["p3d_read_head"])
    for name, f in zip(("p", "u", "v", "w", "eta"), fields):
        np.testing.assert_array_equal(f, P["p3d_read_" + name])


def test_plot3d_read_rejects_another_grid(unit, tmp_path):
    z, g, P = unit
    q = tmp_path / "P3D00.q"
    z["p3d_q"].tofile(q)
    other = O.Grid(g.shape[0] - 3, g.shape[1] - 4, g.shape[2] - 4, 1.0, 1.0, 1.0, 0.5)
    with pytest.raises(OSError):
        O.plot3d_read(other, q)


@pytest.mark.parametrize("case", ["sml_spe_tol1e-3_10", "sml_csr_tol1e-3_10"])
def test_stretched_grid_run_bit_exact(case, golden):
    """The reference's default stretched grid (non_uniform-SML): the restated grid generator
    and the whole step on it, SPE and CSR-Jacobi, against the reference's own runs."""
    z = golden(f"run_{case}.npz")
    m = z["meta"]
    nxc, nyc, nzc = (int(x) for x in m[:3])
    g = O.Grid(nxc, nyc, nzc, m[3], m[4], m[5], m[6], gridder="sml")
    steps, Re, dt, tol, omega = int(m[7]), m[8], m[9], m[10], m[11]
    r = O.run(g, steps, Re, dt, tol, str(z["solver"]), omega)
    np.testing.assert_array_equal(r["iters"], z["iters"])
    np.testing.assert_array_equal(r["cd"], z["cd"])
    np.testing.assert_array_equal(r["cl"], z["cl"])
    for k in ("u", "v", "w", "p"):
        if k in z:
            np.testing.assert_array_equal(r[k][2:-2, 2:-2, 2:-2], z[k])
