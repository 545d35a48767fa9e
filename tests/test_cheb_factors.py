"""The polynomial preconditioner's coefficients (host code of the library,
no GPU): the factors the solver applies multiply out to the polynomial of the
Chebyshev iteration, restated here independently with numpy's polynomial
class, and every factor is positive on the whole spectrum [0, lambda_max]."""
import numpy as np
import pytest
from numpy.polynomial import Polynomial as Poly

import xflow_gb300 as xf


def chebyshev_iteration_poly(ratio, degree):
    """z_d(mu) with z = p(A) r after `degree` steps of the Chebyshev iteration
    for A z = r over [1/ratio, 1] (mu = lambda / lambda_max), from z_0 = r /
    theta: d_0 = z_0, d_{k+1} = rho_{k+1} rho_k d_k + (2 rho_{k+1} / delta)
    (1 - mu z_k), z_{k+1} = z_k + d_{k+1} (Saad, Iterative Methods for Sparse
    Linear Systems, Algorithm 12.1).  Scaled so that p(0) = 1."""
    lo, hi = 1.0 / ratio, 1.0
    theta, delta = (hi + lo) / 2, (hi - lo) / 2
    sigma = theta / delta
    rho = 1 / sigma
    mu = Poly([0.0, 1.0])
    z = Poly([1 / theta])
    d = z
    for _ in range(degree):
        rho_next = 1 / (2 * sigma - rho)
        d = rho_next * rho * d + (2 * rho_next / delta) * (1 - mu * z)
        z = z + d
        rho = rho_next
    return z / z.coef[0]


@pytest.mark.parametrize("degree", [2, 4, 6, 8, 10, 12])
@pytest.mark.parametrize("ratio", [30, 120, 250])
@pytest.mark.parametrize("lmax", [12.0, 4.0 * 3 * 256.0 ** 2])
def test_factors_multiply_out_to_the_chebyshev_polynomial(degree, ratio, lmax):
    f = xf.cheb_factors(lmax, ratio, degree)
    assert f.shape == (1 if degree == 2 else degree // 2, 3)
    want = chebyshev_iteration_poly(ratio, degree)           # in mu = lambda / lmax
    got = Poly([1.0])
    for row in f:
        got = got * Poly(row * lmax ** np.arange(3))        # back to mu units
    assert got.degree() == degree
    scale = np.abs(want.coef).max()
    assert np.abs(got.coef - want.coef).max() <= 1e-5 * scale   # float32 factors
    # positive on the spectrum: p(A) is SPD, each factor on its own as well
    mu = np.linspace(0.0, 1.0, 20001)
    assert (got(mu) > 0).all()
    for row in f:
        assert (Poly(row * lmax ** np.arange(3))(mu) > 0).all()


def test_degree_limits():
    with pytest.raises(xf.XFError):
        xf.cheb_factors(12.0, 120, 16)
    with pytest.raises(xf.XFError):
        xf.cheb_factors(12.0, 120, 5)
