"""Host-side method parameters for the contour-integral f(A)b method.

These are the inputs the reference computes in MATLAB before it calls
``lanczos_create``: the Jacobi least-squares polynomial preconditioner, the
Hale-Higham-Trefethen (HHT) conformal-map quadrature nodes and weights, the
shifted (synthetic-division) polynomial coefficients, the shift layout the
engine consumes and the Krylov-dimension rule.

Reference statements restated here (file:line):

* ``polynomial_coeffs``      -- polynomial_coeffs.m:11-28
* ``hht_contour``            -- startup_nicksmethod_GPU.m:159-179
* ``shifted_poly_coeffs``    -- startup_nicksmethod_GPU.m:189-200
* ``krylov_dim``             -- startup_nicksmethod_GPU.m:202-213
* ``shifts_vector``          -- startup_nicksmethod_GPU.m:214-218
* ``contour_size_from_bound``-- startup_nicksmethod_GPU.m:164-168,
                                bound_M_val.m:1-18, func_for_bound.m:1-25

The complete elliptic integrals K, K' and the complex Jacobi functions
sn/cn/dn (Driscoll's ``ellipkkp``/``ellipjc`` in the reference, which are not
vendored there) are rebuilt from scipy's real ``ellipk``/``ellipj`` with the
imaginary-argument addition formulas (Abramowitz & Stegun 16.21.1-4).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Sequence

import numpy as np
import scipy.special as sps

__all__ = [
    "polynomial_coeffs", "ellipkkp", "ellipjc", "hht_contour",
    "shifted_poly_coeffs", "krylov_dim", "shifts_vector", "Contour",
    "frac_exp", "frac_phi", "frac_power", "contour_size_from_bound",
]


def polynomial_coeffs(degree: int, prob_dim: float) -> np.ndarray:
    """Coefficients of the Jacobi (mu=1/2, nu=-1/2) least-squares polynomial.

    Returns gamma (highest power first, length degree+1) such that
    p(x) = sum_i gamma[i] x^(degree-i) approximates 1/x on [0, 4*prob_dim].
    Restates polynomial_coeffs.m:11-28 (the residual polynomial R built term
    by term from binomial rows and kappa_j, then s(x) = (1-R(x))/x rescaled).
    """
    degree = int(degree)
    if degree < 0:
        raise ValueError("degree must be >= 0")
    R = np.zeros(degree + 2)
    for j in range(1, degree + 3):
        L = degree - j + 3
        bin_coeff = np.array([math.comb(degree - j + 2, i) for i in range(L)], dtype=np.float64)
        q = np.arange(j - 1, dtype=np.float64)
        kappaj = math.comb(degree + 1, j - 1) * float(np.prod((degree + 1 - 0.5 - q) / (q + 1.5)))
        R[j - 1:] += (1.0 / 4.0 ** (j - 1)) * (-1.0) ** (j - 1) * kappaj * bin_coeff * (-4.0) ** (-np.arange(L, dtype=np.float64))
    pw = float(prob_dim) ** np.arange(degree, -1, -1, dtype=np.float64)
    return -R[::-1][:-1] * (3 + 2 * degree) / pw


def ellipkkp(L: float) -> tuple[float, float]:
    """K(k) and K'(k) for modulus k = exp(-pi*L) (Driscoll's ``ellipkkp``).

    Uses the parameter m = k^2 and its complement computed without
    cancellation as 1-k^2 = (1-k)(1+k).
    """
    k = math.exp(-math.pi * L)
    m = k * k
    m1 = -math.expm1(-2.0 * math.pi * L)  # 1 - k^2
    K = float(sps.ellipkm1(m1))  # K(m) = ellipkm1(1-m)
    Kp = float(sps.ellipkm1(m))  # K(1-m)
    return K, Kp


def ellipjc(u: np.ndarray, L: float) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Jacobi sn, cn, dn of complex argument u, parameter m = exp(-2*pi*L).

    Abramowitz & Stegun 16.21.1-4: with s,c,d = sn,cn,dn(x|m) and
    s1,c1,d1 = sn,cn,dn(y|1-m), delta = c1^2 + m s^2 s1^2,
    sn(x+iy) = (s d1 + i c d s1 c1)/delta,
    cn(x+iy) = (c c1 - i s d s1 d1)/delta,
    dn(x+iy) = (d c1 d1 - i m s c s1)/delta.
    """
    u = np.asarray(u, dtype=np.complex128)
    m = math.exp(-2.0 * math.pi * L)
    m1 = -math.expm1(-2.0 * math.pi * L)
    s, c, d, _ = sps.ellipj(u.real, m)
    s1, c1, d1, _ = sps.ellipj(u.imag, m1)
    delta = c1 * c1 + m * s * s * s1 * s1
    sn = (s * d1 + 1j * c * d * s1 * c1) / delta
    cn = (c * c1 - 1j * s * d * s1 * d1) / delta
    dn = (d * c1 * d1 - 1j * m * s * c * s1) / delta
    return sn, cn, dn


def frac_exp(eta: float, alpha: float) -> Callable[[np.ndarray], np.ndarray]:
    """f1(x) = exp(-eta x^(alpha/2)) (startup_nicksmethod_GPU.m:71)."""
    return lambda x: np.exp(-eta * np.power(x, alpha / 2.0))


def frac_phi(eta: float, alpha: float) -> Callable[[np.ndarray], np.ndarray]:
    """f2(x) = phi(-eta x^(alpha/2)), phi(z) = (e^z-1)/z (startup_nicksmethod_GPU.m:70-72)."""
    def f(x):
        z = -eta * np.power(x, alpha / 2.0)
        return np.expm1(z) / z
    return f


def frac_power(p: float) -> Callable[[np.ndarray], np.ndarray]:
    """f(x) = x^p (fractional power, e.g. p = -alpha/2)."""
    return lambda x: np.power(x, p)


@dataclass
class Contour:
    """HHT quadrature on the spectrum interval [l1, lN] with n nodes."""
    l1: float
    lN: float
    n: int
    k: float
    K: float
    Kp: float
    xi: np.ndarray        # (n,) complex nodes
    dxidt: np.ndarray     # (n,) complex map derivative
    s: float              # real scale -4 K sqrt(l1 lN)/(k pi n)

    def weights(self, f: Callable[[np.ndarray], np.ndarray]) -> np.ndarray:
        """w_j = s f(xi_j) dxi/dt_j (startup_nicksmethod_GPU.m:176-177)."""
        return self.s * f(self.xi) * self.dxidt

    def weights_mat(self, f) -> np.ndarray:
        """(n, 2) [real, imag] layout of ``wts1mat``/``wts2mat`` (:178-179)."""
        w = self.weights(f)
        return np.stack([w.real, w.imag], axis=1)


def hht_contour(l1: float, lN: float, n: int) -> Contour:
    """Conformal-map nodes of startup_nicksmethod_GPU.m:159-175.

    k = (sqrt(lN/l1)-1)/(sqrt(lN/l1)+1); midpoint points
    t = i K'/2 - K + (n-1/2, n-3/2, ..., 1/2) 2K/n;
    xi = sqrt(l1 lN)(1/k + sn)/(1/k - sn); dxi/dt = cn dn/(1/k - sn)^2.
    """
    if not (0 < l1 < lN):
        raise ValueError("need 0 < l1 < lN")
    n = int(n)
    if n < 1:
        raise ValueError("need n >= 1")
    r = math.sqrt(lN / l1)
    k = (r - 1.0) / (r + 1.0)
    L = -math.log(k) / math.pi
    K, Kp = ellipkkp(L)
    t = 0.5j * Kp - K + (n - 0.5 - np.arange(n, dtype=np.float64)) * 2.0 * K / n
    sn, cn, dn = ellipjc(t, L)
    g = math.sqrt(l1 * lN)
    xi = g * (1.0 / k + sn) / (1.0 / k - sn)
    dxidt = cn * dn / (1.0 / k - sn) ** 2
    s = -4.0 * K * g / (k * math.pi * n)
    return Contour(l1=l1, lN=lN, n=n, k=k, K=K, Kp=Kp, xi=xi, dxidt=dxidt, s=s)


def shifted_poly_coeffs(gamma: Sequence[float], xi: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """gammas (d+1, n) and sigma = xi * gammas[-1] (startup_nicksmethod_GPU.m:189-200).

    gammas[0] = gamma[0]; gammas[i] = gamma[i] + xi * gammas[i-1]; these are the
    synthetic-division coefficients of q_xi(x) = (xi p(xi) - x p(x))/(xi - x).
    """
    gamma = np.asarray(gamma, dtype=np.float64)
    xi = np.asarray(xi, dtype=np.complex128)
    gs = np.zeros((gamma.size, xi.size), dtype=np.complex128)
    gs[0, :] = gamma[0]
    for i in range(1, gamma.size):
        gs[i, :] = gamma[i] + xi * gs[i - 1, :]
    return gs, xi * gs[-1, :]


def krylov_dim(gamma: Sequence[float], l1: float, lN: float, tol: float) -> int:
    """Krylov dimension rule of startup_nicksmethod_GPU.m:202-213.

    Bounds of x p(x) on [l1, lN] (endpoints and interior critical points),
    kpoly = (sqrt(Lmax/Lmin)-1)/(sqrt(Lmax/Lmin)+1), m = ceil(log(tol/2)/log(kpoly)).
    """
    gamma = np.asarray(gamma, dtype=np.float64)
    d = gamma.size - 1
    xp = np.append(gamma, 0.0)  # coefficients of x p(x)
    cand = [np.polyval(xp, l1), np.polyval(xp, lN)]
    if d >= 1:
        y = np.roots(gamma * np.arange(d + 1, 0, -1))
        y = y[np.abs(y.imag) < 1e-12].real
        y = y[(y > l1) & (y < lN)]
        cand.extend(np.polyval(xp, y).tolist())
    Lmin, Lmax = min(cand), max(cand)
    kp = (math.sqrt(Lmax / Lmin) - 1.0) / (math.sqrt(Lmax / Lmin) + 1.0)
    return int(math.ceil(math.log(tol / 2.0) / math.log(kp)))


def shifts_vector(sigma: np.ndarray, m: int, nrhs: int = 2) -> np.ndarray:
    """Per-diagonal shift array of length 2*m*C*nrhs (4mC for the reference's 2 RHS).

    Layout of startup_nicksmethod_GPU.m:214-218: for RHS r and node j, block
    (r*C + j) holds (Re sigma_j, Im sigma_j) repeated m times.
    """
    sigma = np.asarray(sigma, dtype=np.complex128)
    C = sigma.size
    blk = np.empty((C, m, 2))
    blk[:, :, 0] = sigma.real[:, None]
    blk[:, :, 1] = sigma.imag[:, None]
    return np.tile(blk.reshape(-1), nrhs)


def _bound_M_val(K, Kp, a, f):
    """Max |f| on the rectangle |Re x| <= K, |Im x - Kp/2| <= a (bound_M_val.m:1-18)."""
    import scipy.optimize as so
    corners = [f(-K + 1j * (Kp / 2 - a)), f(K + 1j * (Kp / 2 - a)),
               f(-K + 1j * (Kp / 2 + a)), f(K + 1j * (Kp / 2 + a))]
    vals = [abs(v) for v in corners]
    for sgn in (+1, -1):
        res = so.minimize_scalar(lambda x: -abs(f(x + 1j * (Kp / 2 + sgn * a))),
                                 bounds=(-K, K), method="bounded")
        vals.append(-res.fun)
    return max(vals)


def contour_size_from_bound(l1: float, lN: float, fs, tol: float) -> int:
    """Contour size n from the HHT error bound (startup_nicksmethod_GPU.m:164-168).

    n = min over a in (0, K'/2) of ceil(log(4 K M(a)/tol + 1) K/(pi a)), with
    M(a) from bound_M_val.m over func_for_bound.m's integrand bound.
    """
    import scipy.optimize as so
    r = math.sqrt(lN / l1)
    k = (r - 1.0) / (r + 1.0)
    L = -math.log(k) / math.pi
    K, Kp = ellipkkp(L)
    g = math.sqrt(l1 * lN)

    def integrand_bound(x):
        sn, cn, dn = ellipjc(np.array([x]), L)
        sn, cn, dn = sn[0], cn[0], dn[0]
        z = g * (1 / k + sn) / (1 / k - sn)
        F = max(abs(fj(z) * cn * dn / (1 / k - sn) ** 2) for fj in fs)
        c = z.real
        if l1 <= c <= lN:
            dd = 1.0 / abs(z.imag)
        else:
            dd = max(abs(1 / (z - l1)), abs(1 / (z - lN)))
        return 2 * g / (k * math.pi) * F * dd

    def n_of_a(a):
        M = _bound_M_val(K, Kp, a, integrand_bound)
        return math.ceil(math.log(4 * K * M / tol + 1) * K / (math.pi * a))

    res = so.minimize_scalar(n_of_a, bounds=(1e-6, Kp / 2), method="bounded")
    return int(n_of_a(res.x))
