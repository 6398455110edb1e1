"""The offset-polynomial oracle against known answers (no GPU)."""
import numpy as np
import pytest

from oracle.offsetpoly_oracle import TERMS, basis, evaluate, offsetpoly


def test_basis_order_follows_poly_funcs():
    # poly_funcs.f90: cf(1) + x (cf(2) + x (cf(5) + x cf(9))) + y (cf(3) + y (cf(6) + y cf(10)))
    #                 + x y (cf(4) + y cf(7) + x cf(8))
    x, y = np.array([2.0]), np.array([3.0])
    assert basis(x, y, 10)[0].tolist() == [1, 2, 3, 6, 4, 9, 18, 12, 8, 27]
    assert TERMS == ["1", "x", "y", "xy", "x2", "y2", "xy2", "x2y", "x3", "y3"]


@pytest.mark.parametrize("ma", [1, 3, 6])
def test_exact_polynomial_is_recovered(ma):
    rng = np.random.default_rng(ma)
    x, y = rng.uniform(0, 400, 500), rng.uniform(0, 300, 500)
    true = np.array([0.5, 2e-3, -1e-3, 1e-6, 2e-6, -3e-6])[:ma]
    z = evaluate(true, x, y)
    c = offsetpoly(x, y, z, rng.uniform(1, 20, 500), ma)
    assert np.allclose(evaluate(c, x, y), z, atol=1e-9)
    assert np.allclose(c, true, rtol=1e-6, atol=1e-12)


def test_weights_are_one_over_one_plus_inverse_snr():
    rng = np.random.default_rng(9)
    x, y = rng.uniform(0, 100, 300), rng.uniform(0, 100, 300)
    z = 1 + 0.01 * x + rng.normal(0, 0.1, 300)
    snr = rng.uniform(0.5, 10, 300)
    c = offsetpoly(x, y, z, snr, 3)
    w = 1 / (1 + 1 / snr)
    A = basis(x, y, 3) * w[:, None]
    assert np.allclose(c, np.linalg.lstsq(A, z * w, rcond=None)[0], rtol=1e-10)


def test_single_row_keeps_the_minimum_norm_fit():
    # every offset on one down location: y and 1 are dependent columns; the
    # SVD threshold drops the zero singular value
    x = np.linspace(0, 1000, 200)
    y = np.full(200, 50.0)
    z = 0.3 + 1e-3 * x
    c = offsetpoly(x, y, z, np.full(200, 10.0), 3)
    assert np.allclose(evaluate(c, x, y), z, atol=1e-10)
    # minimum norm: the constant / y split is c0 : c2 = 1 : 50
    assert abs(c[2] / c[0] - 50.0) < 1e-6


def test_coefficient_count_is_checked():
    with pytest.raises(ValueError):
        offsetpoly([1.0], [1.0], [1.0], [1.0], 11)


def test_offsetpoly_interface_checks_lengths_before_the_gpu():
    from isce2_gb300.offsets import Offsetpoly

    o = Offsetpoly()
    o.setLocationAcross([1.0, 2.0])
    o.setLocationDown([1.0])
    o.setOffset([0.5, 0.6])
    o.setSNR([3.0, 4.0])
    with pytest.raises(ValueError, match="locationDown"):
        o.offsetpoly()
    assert o.numberFitCoefficients == 6  # Offsetpoly.py default
