"""Host-side method parameters (no GPU)."""
import math

import numpy as np
import pytest
import scipy.special as sps

from gpumatfun_gb300 import params


def test_polynomial_coeffs_known():
    np.testing.assert_allclose(params.polynomial_coeffs(0, 2), [1.0])
    g = params.polynomial_coeffs(3, 2)
    np.testing.assert_allclose(g, [-0.125, 2.25, -13.5, 30.0], rtol=1e-14)


@pytest.mark.parametrize("degree", [1, 2, 4, 8])
def test_polynomial_is_inverse_approximation(degree):
    """x p(x) (p the Jacobi least-squares approximation of 1/x, scaled by
    3 + 2 degree in polynomial_coeffs.m:28) stays positive on (0, 4 prob_dim]
    and is much better conditioned there than x itself."""
    pd = 2.0
    g = params.polynomial_coeffs(degree, pd)
    a = 4 * pd * 1e-3
    x = np.geomspace(a, 4 * pd, 4000)
    xp = x * np.polyval(g, x)
    assert np.all(xp > 0)
    assert xp.max() / xp.min() < 0.5 * (4 * pd / a)


def test_ellipkkp_and_ellipjc():
    L = 0.3
    K, Kp = params.ellipkkp(L)
    k = math.exp(-math.pi * L)
    assert abs(K - sps.ellipk(k * k)) < 1e-13
    assert abs(Kp - sps.ellipk(1 - k * k)) < 1e-13
    u = np.array([0.3 + 0.4j, -0.7 + 0.2j])
    sn, cn, dn = params.ellipjc(u, L)
    np.testing.assert_allclose(sn ** 2 + cn ** 2, 1, atol=1e-13)
    np.testing.assert_allclose(dn ** 2 + k * k * sn ** 2, 1, atol=1e-13)


@pytest.mark.parametrize("f", [params.frac_exp(1e-2, 1.5), params.frac_power(-0.8), params.frac_phi(1e-2, 1.5)])
def test_contour_reproduces_scalar_function(f):
    """The quadrature Im sum_j w_j (xi_j - x)^-1 reproduces f(x) on [l1, lN]."""
    l1, lN = 2.0, 3000.0
    con = params.hht_contour(l1, lN, 40)
    w = con.weights(f)
    x = np.geomspace(l1, lN, 50)
    approx = np.imag((w[None, :] / (con.xi[None, :] - x[:, None])).sum(1))
    np.testing.assert_allclose(approx, f(x), rtol=1e-9)


def test_shifted_coeffs_synthetic_division():
    g = params.polynomial_coeffs(3, 2)
    xi = np.array([1.5 + 0.5j, 3 - 1j])
    gs, sigma = params.shifted_poly_coeffs(g, xi)
    np.testing.assert_allclose(sigma, xi * np.polyval(g, xi))
    x = 0.7
    for j in range(2):
        q = np.polyval(gs[:, j], x)
        np.testing.assert_allclose(q, (sigma[j] - x * np.polyval(g, x)) / (xi[j] - x))


def test_krylov_dim_rule():
    m = params.krylov_dim([1.0], 1.0, 100.0, 1e-8)
    kp = (10 - 1) / (10 + 1)
    assert m == math.ceil(math.log(0.5e-8) / math.log(kp))


def test_shifts_layout():
    s = params.shifts_vector(np.array([1 + 2j, 3 - 4j]), 3, 2)
    assert s.size == 4 * 3 * 2
    np.testing.assert_allclose(s[:6], [1, 2, 1, 2, 1, 2])
    np.testing.assert_allclose(s[6:12], [3, -4, 3, -4, 3, -4])
    np.testing.assert_allclose(s[12:], s[:12])
