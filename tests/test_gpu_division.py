"""The step kernels (right-hand side, velocity correction, CFL) divide by a metric or by dt
through its reciprocal with Markstein's FMA correction, which must give IEEE division's
result bit for bit: checked on the GPU over seeded dividends for the divisors the
workloads use (the spacings of the uniform and stretched grids, their half spacings, the
time steps).  The whole-step parity tests check the same kernels against the oracle."""
import pytest

import cfd_nssolver_forhpc_flowpassingcylinder_gb300 as cg

pytestmark = pytest.mark.gpu

DIVISORS = [0.25, 0.0625, 0.03125, 24.0 / 256, 12.0 / 128, 17.0 / 190 * 0.7, 0.1 / 3.0, 0.005, 0.002, 0.001,
            0.004, 1.0 / 3.0, 3.0, 7.0e-3, 0.123456789, 1e-7]


@pytest.mark.parametrize("b", DIVISORS)
def test_reciprocal_division_is_ieee_division(b):
    assert cg.check_division(4_000_000, 1234, b) == 0
