"""The step kernels (convection-diffusion, right-hand side, velocity correction, CFL) divide
by a metric or by dt through its reciprocal with Markstein's FMA correction, which must give
IEEE division's result bit for bit.  Markstein's theorem proves the single correction for a
divisor b whose reciprocal y = RN(1/b) has |b y - 1| < 2^-54; a context with any other
divisor applies the correction twice (proven for every divisor).  Checked on the GPU over
seeded dividends for every divisor the workloads use: all spacings and centre spacings of
the uniform grids of the benchmark cases and of the reference's stretched grids, and the
time steps, each in the form the library would use for it."""
from fractions import Fraction

import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRIDS = [(96, 48, 4, 24.0, 12.0, 1.0, 6.0, "uniform"), (512, 256, 64, 32.0, 16.0, 4.0, 8.0, "uniform"),
         (1024, 512, 128, 32.0, 16.0, 4.0, 8.0, "uniform"), (256, 128, 32, 24.0, 12.0, 2.0, 6.0, "uniform"),
         (1536, 768, 96, 48.0, 24.0, 3.0, 12.0, "uniform"), (190, 210, 40, 17.0, 12.0, 3.0, 6.5, "sml"),
         (120, 110, 4, 17.0, 12.0, 3.0, 6.5, "sml")]
DTS = [0.005, 0.002, 0.001, 0.004]


def _divisors():
    out = set(DTS)
    for nx, ny, nz, lx, ly, lz, cx, gridder in GRIDS:
        grid = O.Grid(nx, ny, nz, lx, ly, lz, cx, gridder=gridder)  # holds the arrays
        g = grid._g
        for name, n in (("Dx", g.nx), ("Dy", g.ny), ("Dz", g.nz), ("Dxs", g.nx), ("Dys", g.ny), ("Dzs", g.nz)):
            arr = getattr(g, name)
            out.update(arr[i] for i in range(n))
    return sorted(out)


def certified(b):
    """Markstein's condition for the single correction, in exact arithmetic."""
    return abs(Fraction(b) * Fraction(1.0 / b) - 1) < Fraction(1, 2 ** 54)


def test_every_workload_divisor_gives_ieee_division():
    divs = _divisors()
    assert len(divs) > 40
    for b in divs:
        # the uncertified ones (double correction) get more dividends
        n = 400_000 if certified(b) else 4_000_000
        assert cg.check_division(n, 1234, b) == 0, b


@pytest.mark.parametrize("b", [0.25, 1.0 / 3.0, 3.0, 7.0e-3, 0.123456789, 1e-7, 0.09375, 0.75])
def test_reciprocal_division_other_divisors(b):
    assert cg.check_division(4_000_000, 4321, b) == 0
