"""The roofline's FLOP model (bench.py) against the per-product counts the profiles state:
slice pairs x 2 M N K, the Coulomb product's lower half over the half spectrum."""
import pytest

import bench


def test_c2_flops():
    # P 21 x 2 x 256 x 110,592 x 32; zeta 21 x 2 x 256^2 x 110,592; M 15 x 256^2 x 115,200.
    f = bench.sliced_gemm_flops(110592, 32, 256, (48, 48, 48), False, 0)
    p, z, m = 21 * 2 * 256 * 110592 * 32, 21 * 2 * 256 ** 2 * 110592, 15 * 256 ** 2 * 115200
    assert f == pytest.approx(p + z + m, rel=1e-12)
    assert f == pytest.approx(4.557e11, rel=1e-3)


def test_c3_adds_the_inverse_product():
    ng, no, nmu = 373248, 256, 2048
    f = bench.sliced_gemm_flops(ng, no, nmu, (72, 72, 72), False, 0)
    nc2 = 2 * 72 * 72 * 37
    expect = (21 * 2 * nmu * ng * no + 21 * 2 * nmu * nmu * ng + 15 * nmu * nmu * nc2
              + 21 * 2 * nmu ** 3)
    assert f == pytest.approx(expect, rel=1e-12)


def test_c5_shifted_solve_with_refinement():
    ng, no, nmu = 1259712, 864, 5184
    f = bench.sliced_gemm_flops(ng, no, nmu, (108, 108, 108), True, 1)
    unshifted = bench.sliced_gemm_flops(ng, no, nmu, (108, 108, 108), False, 0)
    # The shifted solve adds the second N_g-long product and G plus one Horner step, and
    # drops the explicit inverse.
    extra = 21 * 2 * nmu * ng * nmu + 21 * 2 * nmu ** 3 * 2 - 21 * 2 * nmu ** 3
    assert f - unshifted == pytest.approx(extra, rel=1e-12)
    assert f == pytest.approx(3.61e15, rel=2e-3)
