"""Bump-and-revalue Greeks on common random numbers (thoth_gpu_bump_greeks).

Oracle: the same bumped books (spot x 1.01 and x (1 +/- 0.1) per asset, vol level
+1 point, rates +1bp, today + 1 day, Heston parameters + 0.01), built here with the
definitions of pricer_mcl_greeks.cpp:43-299 / pricer.cpp:144-193, priced by the CPU
oracle on the same Sobol paths, and turned into the same finite differences. The GPU
and oracle prices of one scenario agree to FP32 path precision, so the Greeks agree
to that precision divided by the bump. A GBM call is also checked against the
Black-Scholes finite differences of the same bumps.
"""
import math

import numpy as np
import pytest

import oracle
from thoth_gb300 import abi

pytestmark = pytest.mark.gpu

PARAMS = abi.PARAMS


def bumped(book, kind, a=None, h=None, k=None):
    b = book.copy()
    if kind == "spot":
        b.assets[a]["spot"] *= 1 + h
    elif kind == "vol":
        for A in b.assets:
            if A["model"] == abi.MODEL_GBM:
                A["vol"] += 0.01
            else:
                A["v0"] = (math.sqrt(A["v0"]) + 0.01) ** 2
                A["theta"] = (math.sqrt(A["theta"]) + 0.01) ** 2
    elif kind == "rate":
        for A in b.assets:
            A["carry"] = A["carry"] + 1e-4
        for P in b.products:
            P["zero_rate"] += 1e-4
    elif kind == "param":
        for A in b.assets:
            if A["model"] != abi.MODEL_GBM:
                A[PARAMS[k]] += 0.01
    elif kind == "roll":                      # date 1 is today + 1: it becomes today
        assert b.days[1] == b.days[0] + 1
        t_old = b.t.copy()
        b.days = np.ascontiguousarray(b.days[1:] - b.days[1], dtype=np.int32)
        b.t = b.days.astype(np.float64) / 365.0
        b.n_dates = len(b.t)
        for A in b.assets:
            c = A["carry"]
            new = np.empty(b.n_dates)
            new[0] = c[1]
            new[1:] = (c[2:] * t_old[2:] - c[1] * t_old[1]) / b.t[1:]
            A["carry"] = new
            if A["model"] == abi.MODEL_LSV:
                A["lev_ln_step"] = A["lev_ln_step"][1:].copy()
                A["lev_offset"] = A["lev_offset"][1:].copy()
                A["lev_values"] = A["lev_values"][1:].copy()
        for P in b.products:
            P["maturity"] = max(P["maturity"] - 1, 0)
            if "monitor" in P:
                P["monitor"] = np.ascontiguousarray([m - 1 for m in P["monitor"] if m >= 1], dtype=np.int32)
            if "obs" in P:
                P["obs"] = np.ascontiguousarray([o - 1 for o in P["obs"] if o >= 2], dtype=np.int32)
    return b


def oracle_greeks(book):
    P = lambda b: oracle.price_book(b, threads=16)
    base = P(book)
    p0, b0 = base["premium"], base["book_premium"]
    g = {"premium": p0}
    d = np.zeros_like(p0)
    gm = np.zeros_like(p0)
    for a, A in enumerate(book.assets):
        s = A["spot"]
        up = P(bumped(book, "spot", a, 0.01))
        d += (up["premium"] - p0) / (0.01 * s)
        gu, gd = P(bumped(book, "spot", a, 0.1)), P(bumped(book, "spot", a, -0.1))
        gm += (gu["premium"] - 2 * p0 + gd["premium"]) / (0.1 * s) ** 2
    g["delta"], g["gamma"] = d, gm
    g["vega"] = P(bumped(book, "vol"))["premium"] - p0
    g["rho"] = (P(bumped(book, "rate"))["premium"] - p0) / 1e-4 * 0.01
    g["theta"] = P(bumped(book, "roll"))["premium"] - p0
    for k, name in enumerate(PARAMS):
        g["vega_" + name] = (P(bumped(book, "param", k=k))["premium"] - p0) / 0.01
    return g, b0


# denominators of the finite differences (how far a price error moves the Greek)
SCALE = {"delta": 1.0, "gamma": 100.0, "vega": 1.0, "rho": 0.01, "theta": 1.0}


def heston_book(paths):
    b = abi.Book(days=np.arange(0, 91), paths=paths)
    h = b.add_heston(100.0, 0.04, 1.5, 0.04, 0.6, -0.7, 0.02)
    b.add_vanilla(h, 100.0, 90, abi.CALL, zero_rate=0.03)
    b.add_vanilla(h, 90.0, 60, abi.PUT, zero_rate=0.03)
    b.add_barrier(h, 100.0, 90, 85.0, up=False, knock_in=False, monitor=np.arange(1, 91), zero_rate=0.03)
    b.add_variance(h, 90, strike_variance=0.04, notional=100.0, zero_rate=0.03)
    return b


def test_bump_greeks_match_the_oracle(gpu):
    b = heston_book((1 << 12) + 3)
    g = gpu.bump_greeks(b)
    ref, _ = oracle_greeks(b)
    assert g["n_scenarios"] == 1 + 3 + 1 + 1 + 1 + 5
    p0 = np.abs(ref["premium"])
    np.testing.assert_allclose(g["premium"], ref["premium"], rtol=1e-4, atol=1e-5)
    for k in ("delta", "gamma", "vega", "rho", "theta") + tuple("vega_" + p for p in PARAMS):
        s = SCALE.get(k, 0.01)
        err = np.abs(g[k] - ref[k])
        # four scenario prices at most, each within FP32 path precision of the oracle's
        tol = 4 * 1e-5 * (p0 + 1.0) / s + 5e-3 * np.abs(ref[k])
        assert np.all(err <= tol), (k, g[k], ref[k])
    assert np.isfinite(g["book"]["delta"]) and g["note"] == ""


def test_bump_greeks_black_scholes(gpu):
    """GBM call, 1 year daily: every Greek against the same finite difference of BS."""
    S, K, vol, r, q = 100.0, 100.0, 0.25, 0.03, 0.01
    b = abi.Book(days=np.arange(0, 366), paths=1 << 18)
    a = b.add_gbm(S, vol, r - q)
    b.add_vanilla(a, K, 365, abi.CALL, zero_rate=r)
    g = gpu.bump_greeks(b, abi.BUMP_ALL)

    def bs(S=S, vol=vol, r=r, T=1.0):
        F = S * math.exp((r - q) * T)
        return oracle.bs_price(F, K, T, vol, math.exp(-r * T))

    p = bs()
    want = {"delta": (bs(S=1.01 * S) - p) / (0.01 * S),
            "gamma": (bs(S=1.1 * S) - 2 * p + bs(S=0.9 * S)) / (0.1 * S) ** 2,
            "vega": bs(vol=vol + 0.01) - p,
            "rho": (bs(r=r + 1e-4) - p) / 1e-4 * 0.01,
            "theta": bs(T=1.0 - 1 / 365.0) - p}
    for k, w in want.items():
        assert abs(g[k][0] - w) <= 0.02 * abs(w), (k, g[k][0], w)
    assert np.isnan(g["vega_v0"][0])                 # no Heston asset: no parameter Greeks


def test_bump_greeks_without_calendar_days(gpu):
    b = abi.Book(times=np.arange(0, 64) / 252.0, paths=1 << 12)
    h = b.add_heston(100.0, 0.04, 1.5, 0.04, 0.6, -0.7, 0.0)
    b.add_vanilla(h, 100.0, 63, abi.CALL, zero_rate=0.0)
    g = gpu.bump_greeks(b, abi.BUMP_DELTA | abi.BUMP_THETA)
    assert np.isfinite(g["delta"][0]) and np.isnan(g["theta"][0]) and np.isnan(g["gamma"][0])
    assert "days" in g["note"]
