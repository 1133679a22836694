"""The FP64 closed-form oracles: Heston (characteristic function, little-trap
form, adaptive Gauss-Kronrod) against a second, independent formulation
(Lewis 2000 single integral with scipy quadrature), and Black-Scholes anchors."""
import cmath
import math
import os

import numpy as np
import pytest

import oracle

scipy_integrate = pytest.importorskip("scipy.integrate")


def heston_cf(u, T, v0, kappa, theta, xi, rho):
    """E[exp(i u ln(S_T / F))] in the little-trap form."""
    d = cmath.sqrt((rho * xi * 1j * u - kappa) ** 2 + xi * xi * (1j * u + u * u))
    g = (kappa - rho * xi * 1j * u - d) / (kappa - rho * xi * 1j * u + d)
    e = cmath.exp(-d * T)
    C = kappa * theta / xi ** 2 * ((kappa - rho * xi * 1j * u - d) * T - 2 * cmath.log((1 - g * e) / (1 - g)))
    D = (kappa - rho * xi * 1j * u - d) / xi ** 2 * (1 - e) / (1 - g * e)
    return cmath.exp(C + D * v0)


def lewis_call(S, K, T, r, q, v0, kappa, theta, xi, rho):
    F = S * math.exp((r - q) * T)
    k = math.log(F / K)

    def f(u):
        return (cmath.exp(1j * u * k) * heston_cf(u - 0.5j, T, v0, kappa, theta, xi, rho)).real / (u * u + 0.25)

    val, _ = scipy_integrate.quad(f, 0, np.inf, limit=500, epsabs=1e-13, epsrel=1e-12)
    return math.exp(-r * T) * (F - math.sqrt(F * K) / math.pi * val)


def test_heston_oracle_against_30_digit_fixture():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "heston_cf.npz"))
    for args, ref in zip(g["args"], g["call"]):
        got = oracle.heston_price(*args, True)
        assert abs(got - ref) <= 1e-10 * abs(ref) + 1e-12, (args, got, ref)


@pytest.mark.parametrize("K", [80.0, 90.0, 100.0, 110.0, 120.0])
@pytest.mark.parametrize("T", [1 / 12.0, 0.5, 2.0])
def test_heston_second_rules_agree(K, T):
    p = dict(v0=0.04, kappa=1.5, theta=0.04, xi=0.6, rho=-0.7)
    a = oracle.heston_price(100.0, K, T, 0.03, 0.0, p["v0"], p["kappa"], p["theta"], p["xi"], p["rho"], True)
    b = lewis_call(100.0, K, T, 0.03, 0.0, **p)            # scipy quadrature of the same integral
    assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (a, b)
    c = oracle.heston_price_p12(100.0, K, T, 0.03, 0.0, p["v0"], p["kappa"], p["theta"], p["xi"], p["rho"], True)
    assert abs(a - c) <= 5e-8, (a, c)                     # reference's P1/P2 form (weaker: F P1 - K P2 cancels)


def test_heston_put_call_parity_and_bs_limit():
    S, K, T, r = 100.0, 105.0, 1.0, 0.03
    c = oracle.heston_price(S, K, T, r, 0.0, 0.04, 1.5, 0.04, 0.6, -0.7, True)
    p = oracle.heston_price(S, K, T, r, 0.0, 0.04, 1.5, 0.04, 0.6, -0.7, False)
    assert abs((c - p) - (S - K * math.exp(-r * T))) < 1e-10
    # vanishing vol-of-vol with v0 = theta: Black-Scholes at sqrt(theta)
    h = oracle.heston_price(S, K, T, r, 0.0, 0.04, 1.5, 0.04, 1e-4, 0.0, True)
    bs = oracle.bs_price(S * math.exp(r * T), K, T, 0.2, math.exp(-r * T))
    assert abs(h - bs) < 1e-5


def test_black_scholes_anchors():
    # simple_call sample: S = K = 100, vol 30 %, r 8 %, 1y -> 15.71 (README of the reference)
    assert abs(oracle.bs_price(100 * math.exp(0.08), 100, 1.0, 0.3, math.exp(-0.08)) - 15.7113) < 1e-3
    c = oracle.bs_price(110, 100, 0.5, 0.2, 0.97, True)
    p = oracle.bs_price(110, 100, 0.5, 0.2, 0.97, False)
    assert abs((c - p) - 0.97 * 10) < 1e-12
    # pathwise formulas used by the GPU tests
    h = 1e-5
    d = (oracle.bs_price(100 * (1 + h) * math.exp(0.02), 100, 1, 0.25, math.exp(-0.03)) -
         oracle.bs_price(100 * (1 - h) * math.exp(0.02), 100, 1, 0.25, math.exp(-0.03))) / (200 * h)
    assert abs(d - oracle.bs_delta(100, 100, 1, 0.25, 0.03, 0.01)) < 1e-6
