"""cfdgb_poisson_solve_static: the Poisson solve for callers that cannot allocate device
memory (hosts whose framework owns all device memory through its own pool, services that
must not allocate after start-up).  It keeps every work vector in a static device array;
here it is called through the C ABI on device buffers the test owns, twice in a row (the
array keeps the previous call's contents), and its solution is compared with the
context-based entry point cfdgb_op_bicgstab on the same right-hand side and warm start.
Two grids: nz = 16 and nz = 40, where the k-block width (8) is not the next power of two.

Collected last on purpose: if it fails, a run that stops at the first failure has already
run every other test."""
import ctypes as C

import numpy as np
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg

pytestmark = pytest.mark.gpu

H = 0.25
TOL = 1e-10


def _static_solve(L, torch, dims, rhs, x0, solver):
    d_rhs = torch.from_numpy(rhs).cuda()
    d_x = torch.from_numpy(x0).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    it, rr = C.c_int(), C.c_double()
    torch.cuda.synchronize()
    rc = L.cfdgb_poisson_solve_static(*dims, H, H, H, solver, TOL, 5000, C.c_void_p(d_rhs.data_ptr()),
                                      C.c_void_p(d_x.data_ptr()), C.c_void_p(stream), C.byref(it), C.byref(rr))
    torch.cuda.synchronize()
    return rc, it.value, rr.value, d_x.cpu().numpy()


@pytest.mark.parametrize("dims", [(40, 24, 16), (24, 20, 40)], ids=["nz16", "nz40"])
def test_static_solve_matches_context_solve_on_two_calls_in_a_row(dims):
    torch = pytest.importorskip("torch")
    L = cg.load_library()
    nx, ny, nz = dims
    with cg.Solver(nx=nx, ny=ny, nz=nz, lx=nx * H, ly=ny * H, lz=nz * H, cx=nx * H / 2, cy=ny * H / 2,
                   dfib=0) as s:
        for call, solver in enumerate((cg.BICGSTAB, cg.BICGSTAB_JACOBI)):
            rng = np.random.default_rng(call)
            rhs = s.spmv(rng.standard_normal(s.cells), jacobi=solver == cg.BICGSTAB_JACOBI)  # consistent
            x0 = 0.1 * rng.standard_normal(s.cells)
            x_ref = x0.copy()
            it_ref, rr_ref, rc_ref = s.bicgstab(rhs, x_ref, TOL, jacobi=solver == cg.BICGSTAB_JACOBI)
            rc, it, rr, x = _static_solve(L, torch, dims, rhs, x0, solver)
            assert rc == rc_ref == 0
            assert rr < TOL
            # same kernels and launch shape: same iterations, solutions equal to roundoff
            assert it == it_ref
            np.testing.assert_allclose(x, x_ref, rtol=0, atol=1e-12 * np.abs(x_ref).max())


def test_static_solve_rejects_grids_beyond_its_array():
    L = cg.load_library()
    it, rr = C.c_int(), C.c_double()
    # 65 x 64 x 64 > 2^18 unknowns: rejected before any device work
    rc = L.cfdgb_poisson_solve_static(65, 64, 64, H, H, H, cg.BICGSTAB, TOL, 10, C.c_void_p(16), C.c_void_p(16),
                                      None, C.byref(it), C.byref(rr))
    assert rc == cg.EINVAL


def test_static_solve_rejects_a_capturing_stream():
    """The call waits on its stream to poll convergence; on a stream that is capturing into
    a graph it returns CFDGB_EINVAL before enqueuing anything."""
    torch = pytest.importorskip("torch")
    L = cg.load_library()
    n = 8 * 8 * 8
    d_rhs = torch.zeros(n, dtype=torch.float64, device="cuda")
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
    y = torch.zeros(4, device="cuda")
    it, rr = C.c_int(), C.c_double()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        y.add_(1.0)
        rc = L.cfdgb_poisson_solve_static(8, 8, 8, H, H, H, cg.BICGSTAB, TOL, 10, C.c_void_p(d_rhs.data_ptr()),
                                          C.c_void_p(d_x.data_ptr()), C.c_void_p(side.cuda_stream), C.byref(it),
                                          C.byref(rr))
    graph.replay()
    torch.cuda.synchronize()
    assert rc == cg.EINVAL
    assert float(y[0]) == 1.0  # the caller's capture is intact
