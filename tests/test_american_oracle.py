"""The Longstaff-Schwartz oracle (oracle/american.py), pinned to the reference's own code.

* golden vectors (tests/golden/american.npz, from the reference's fit and apply loops around
  its own LeastSquares, made by tests/golden/make_american.py): same regression dates, same
  coefficients up to the summation order, same premium;
* the reference's LeastSquares and loops live (oracle/_ref, where it was built);
* the exact sums: order-independent, within n 2^-64 of the exact real sum;
* the reference's tests (pricer/tests/test_american.cpp) on exact-GBM paths, with a binomial
  tree as the continuous-exercise value.
"""
import math
import os
import random
from fractions import Fraction

import numpy as np
import pytest

import oracle
from oracle import american as am

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "american.npz")
need_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


@pytest.mark.parametrize("name,call", [("put", False), ("call", True)])
def test_fit_matches_the_reference_golden_vectors(g, name, call):
    tau = g["days"] / 365.0
    K = float(g[name + "_strike"])
    o = am.fit(g[name + "_paths"], tau, g[name + "_rates"], K, call, K, int(g["min_itm"]))
    has = g[name + "_has_fit"]
    np.testing.assert_array_equal(o["has_fit"], has)
    assert has[1:-1].sum() >= 5
    # the normal equations amplify the summation-order difference; the decisions agree
    np.testing.assert_allclose(o["beta"][has], g[name + "_beta"][has], rtol=1e-7, atol=1e-7)
    assert o["premium"] == pytest.approx(float(g[name + "_premium"]), rel=1e-13)
    assert o["trust"] == pytest.approx(float(g[name + "_trust"]), rel=1e-10)


def test_frozen_apply_matches_the_reference_golden_vectors(g):
    tau = g["days"] / 365.0
    o = am.fit(g["put_paths"], tau, g["put_rates"], 100.0, False, 100.0, int(g["min_itm"]))
    a = am.apply(g["bump_paths"], tau, g["put_rates"], 100.0, False, 100.0, g["put_beta"], g["put_has_fit"])
    assert a["premium"] == pytest.approx(float(g["bump_premium"]), rel=1e-13)
    # the oracle's own policy gives the same value (same decisions)
    b = am.apply(g["bump_paths"], tau, g["put_rates"], 100.0, False, 100.0, o["beta"], o["has_fit"])
    assert b["premium"] == pytest.approx(a["premium"], rel=1e-13)


def test_apply_on_the_fitting_paths_is_the_fit_value(g):
    tau = g["days"] / 365.0
    o = am.fit(g["call_paths"], tau, g["call_rates"], 95.0, True, 95.0)
    a = am.apply(g["call_paths"], tau, g["call_rates"], 95.0, True, 95.0, o["beta"], o["has_fit"])
    assert a["premium"] == o["premium"] and a["trust"] == o["trust"]


@need_ref
def test_solve_matches_the_reference_least_squares():
    rng = np.random.default_rng(5)
    for n in (60, 500, 4000):
        m = rng.uniform(0.3, 1.0, n)
        y = np.maximum(1.0 - m, 0.0) * rng.uniform(0.5, 1.5, n)
        X = np.stack([np.ones(n), m, m * m], axis=1)
        ref = oracle.ref_least_squares(X, y)
        m2 = m * m
        sums = [am.exact_sum(v) for v in (m, m2, m2 * m, m2 * m2, y, m * y, m2 * y)]
        b = am.solve3(n, sums)
        np.testing.assert_allclose(b, ref, rtol=1e-8, atol=1e-10)
    # a singular design (one moneyness value): both decline
    X = np.stack([np.ones(80), np.full(80, 0.9), np.full(80, 0.81)], axis=1)
    assert oracle.ref_least_squares(X, np.ones(80)) is None
    s = [am.exact_sum(np.full(80, v)) for v in (0.9, 0.81, 0.81 * 0.9, 0.81 * 0.81, 1.0, 0.9, 0.81)]
    assert am.solve3(80, s) is None


@need_ref
@pytest.mark.parametrize("seed,call", [(3, False), (4, True)])
def test_fit_matches_the_reference_loop_live(seed, call):
    days = list(range(0, 181, 7)) + [182]
    S = am.gbm_paths(100.0, 0.25, 0.05, 0.07 if call else 0.0, days, 8000, seed)
    tau = np.asarray(days) / 365.0
    rates = 0.02 + 0.03 * tau
    K = 98.0 if call else 102.0
    o = am.fit(S, tau, rates, K, call, K)
    r = oracle.ref_lsm(S, tau, rates, K, call, K)
    np.testing.assert_array_equal(o["has_fit"], r["has_fit"])
    assert o["premium"] == pytest.approx(r["premium"], rel=1e-13)


def test_exact_sum_is_order_independent_and_exact():
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.uniform(0, 1, 5000) ** 6, rng.uniform(0, 3e4, 50), [0.0, 1e-30, 2.0 ** -64]])
    s = am.exact_sum(x)
    assert am.exact_sum(rng.permutation(x)) == s
    exact = sum(Fraction(float(v)) for v in x)
    assert abs(Fraction(s) - exact) <= len(x) * Fraction(1, 2 ** 64) + Fraction(s) * Fraction(1, 2 ** 52)
    with pytest.raises(ValueError):
        am.exact_sum(np.array([2.0 ** 40]))
    # ties round to even like the device's conversion: 1 + 2^-53 sits halfway
    assert am.exact_sum(np.array([1.0, 2.0 ** -53])) == 1.0
    assert am.exact_sum(np.array([1.0, 2.0 ** -53, 2.0 ** -60])) == 1.0 + 2.0 ** -52


def test_reference_properties_on_exact_gbm_paths():
    """test_american.cpp:8-44 at 100 000 paths: the call equals Black-Scholes within MC error,
    the put lies between the European put and (about) the continuous-exercise tree."""
    days = list(range(0, 361, 30)) + [365]
    tau = np.asarray(days) / 365.0
    rates = np.full(len(days), 0.08)
    S = am.gbm_paths(100.0, 0.30, 0.08, 0.0, days, 100000, 21)
    c = am.fit(S, tau, rates, 100.0, True, 100.0)
    bs_call = oracle.bs_price(100.0 * math.exp(0.08), 100.0, 1.0, 0.30, math.exp(-0.08), True)
    assert abs(c["premium"] - bs_call) <= 6.0 * c["trust"] + 5e-2
    p = am.fit(S, tau, rates, 100.0, False, 100.0)
    euro = oracle.bs_price(100.0 * math.exp(0.08), 100.0, 1.0, 0.30, math.exp(-0.08), False)
    tree = am.binomial(100.0, 100.0, 1.0, 0.08, 0.0, 0.30, call=False)
    assert euro < p["premium"] <= tree + 6.0 * p["trust"] + 5e-2
    assert p["premium"] >= 0.95 * tree
    # the tree itself: European limit and early-exercise premium
    assert am.binomial(100.0, 100.0, 1.0, 0.08, 0.0, 0.30, call=False, american=False) == pytest.approx(euro, abs=1e-2)
    assert am.binomial(60.0, 100.0, 1.0, 0.08, 0.0, 0.30, call=False) == pytest.approx(40.0, abs=1e-9)


def _fma32(a, b, c):
    """Single-precision fused multiply-add: the product of two floats is exact in double,
    one rounding to double of the sum, then to float (within the screen's bound either way)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def _screen32(s, K, norm, b, call):
    """The apply kernel's single-precision screen of the exercise test (american.cu,
    exercise_screened), restated in numpy float32: +1 exercise, -1 hold, 0 left to double."""
    f = np.float32
    sf = s.astype(f)
    Kf = f(K)
    inv = f(1.0 / norm)
    m = sf * inv
    iv = (sf - Kf) if call else (Kf - sf)
    b0, b1, b2 = (x.astype(f) for x in b)
    c = _fma32(_fma32(b2, m, b1), m, b0)
    d = iv - c
    am_ = np.abs(m)
    mag = _fma32(np.abs(b2) * am_, am_, _fma32(np.abs(b1), am_, np.abs(b0))) + (abs(Kf) + np.abs(sf))
    e = _fma32(mag, np.full_like(mag, f(2.0 ** -19)), np.full_like(mag, f(1e-30)))
    return np.where(d > e, 1, np.where(d < -e, -1, 0))


@pytest.mark.parametrize("call", [False, True])
def test_single_precision_screen_never_contradicts_the_double_test(call):
    """Wherever the screen decides, it decides as the reference's double-precision test
    iv >= (b0 + b1 m) + (b2 m) m does; it leaves only a thin band around the boundary."""
    rng = np.random.default_rng(7 + call)
    n = 400000
    K = 100.0
    s = (K * np.exp(0.25 * rng.standard_normal(n))).astype(np.float32)
    sd = s.astype(np.float64)
    iv = (sd - K) if call else (K - sd)
    m = sd / K
    b1 = 60.0 * rng.standard_normal(n)
    b2 = 30.0 * rng.standard_normal(n)
    # b0 puts the continuation a signed distance from the intrinsic value, from 1e-14 to 10
    gap = np.sign(rng.standard_normal(n)) * 10.0 ** rng.uniform(-14, 1, n)
    b0 = iv - (b1 * m + (b2 * m) * m) - gap
    cont = (b0 + b1 * m) + (b2 * m) * m
    exact = np.where(iv >= cont, 1, -1)
    sc = _screen32(s, K, K, (b0, b1, b2), call)
    decided = sc != 0
    assert np.array_equal(sc[decided], exact[decided])
    # gaps above the bound are decided: the band is at most 2^-19 mag wide
    mag = np.abs(K) + np.abs(sd) + np.abs(b0) + np.abs(b1 * m) + np.abs(b2) * m * m
    assert decided[np.abs(gap) > 2.0 ** -18 * mag].all()
    # on generic policies the band is rare
    sg = _screen32(s, K, K, (iv - 5.0 * rng.standard_normal(n), b1 * 0.0, b2 * 0.0), call)
    assert np.mean(sg == 0) < 1e-3
