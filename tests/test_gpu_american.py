"""American exercise (thoth_gpu_price_american) against the Longstaff-Schwartz oracle.

The engine's regression and premium sums are exact fixed-point sums, and oracle/american.py
sums the same way, so on the stored paths of the same book (thoth_gpu_simulate_paths) the
engine's coefficients, exercise decisions, premium and trust equal the oracle's bit for bit.
The frozen-policy Greeks value the fitted policy on the stored paths of each bumped book
(theta refits on the rolled book), checked the same way. The reference's own tests
(pricer/tests/test_american.cpp) fix the behaviour against its PDE engine; those checks run
here at the reference's path counts, with a binomial tree as the continuous-exercise value.
"""
import math

import numpy as np
import pytest

import oracle
from oracle import american as am
from thoth_gb300 import abi

pytestmark = pytest.mark.gpu

# one year, at most 30 days a step: the diffusion grid of the reference's tests
DAYS = list(range(0, 361, 30)) + [365]


def vanilla_book(S=100.0, K=100.0, vol=0.30, r=0.08, typ=abi.PUT, paths=1 << 16, days=DAYS, model="gbm"):
    b = abi.Book(days=np.asarray(days), paths=paths)
    if model == "gbm":
        a = b.add_gbm(S, vol, r)
    else:
        a = b.add_heston(S, 0.09, 1.5, 0.09, 0.5, -0.6, r)
    b.add_vanilla(a, K, len(days) - 1, typ, zero_rate=r)
    return b


def rates_of(b, zero_rates=None):
    return np.asarray(zero_rates if zero_rates is not None else np.full(b.n_dates, b.products[0]["zero_rate"]))


def oracle_pass(gpu, b, zero_rates=None, policy=None):
    P = b.products[0]
    S, _ = gpu.simulate_paths(b, P["asset"])
    M = P["maturity"] + 1
    K, call = P["strike"], P["option_type"] == abi.CALL
    z = rates_of(b, zero_rates)
    if policy is None:
        return am.fit(S[:M], b.t, z, K, call, K)
    return am.apply(S[:M], b.t, z, K, call, K, policy["beta"], policy["has_fit"])


def assert_same_fit(r, o, M):
    assert r["premium"] == o["premium"], (r["premium"], o["premium"])
    assert r["trust"] == o["trust"]
    assert r["european"] == o["european"]
    has = o["has_fit"]
    assert r["fitted_dates"] == int(has.sum()) > 0
    np.testing.assert_array_equal(r["beta"][:M][has], o["beta"][has])
    assert np.all(np.isnan(r["beta"][:M][~has])) and np.all(np.isnan(r["beta"][M:]))


@pytest.mark.parametrize("typ,model,paths", [(abi.PUT, "gbm", (1 << 16) + 77), (abi.CALL, "gbm", 50000),
                                             (abi.PUT, "heston", (1 << 15) + 5)])
def test_fit_equals_the_oracle_bit_for_bit(gpu, typ, model, paths):
    b = vanilla_book(typ=typ, model=model, paths=paths, K=100.0 if typ == abi.PUT else 95.0, r=0.08 if typ == abi.PUT else 0.02)
    if typ == abi.CALL:                       # a dividend yield makes early exercise of a call pay
        b.assets[0]["carry"] = b.assets[0]["carry"] - 0.06
    r = gpu.price_american(b, 0)
    o = oracle_pass(gpu, b)
    assert_same_fit(r, o, b.n_dates)
    assert r["premium"] > r["european"] - 3 * r["trust"]


def test_daily_exercise_on_a_sloped_curve(gpu):
    days = np.arange(0, 181)
    b = vanilla_book(paths=20000, days=days, K=105.0)
    z = 0.01 + 0.04 * b.t                      # zero rates rising with maturity
    r = gpu.price_american(b, 0, zero_rates=z)
    o = oracle_pass(gpu, b, zero_rates=z)
    assert_same_fit(r, o, b.n_dates)
    flat = gpu.price_american(b, 0)
    assert flat["premium"] != r["premium"]


def test_min_itm_above_the_path_count_keeps_no_regression(gpu):
    b = vanilla_book(paths=4000)
    r = gpu.price_american(b, 0, min_itm=5000)
    assert r["fitted_dates"] == 0 and np.all(np.isnan(r["beta"]))
    assert r["premium"] == max(r["european"], 0.0)


def roll(b):
    """The book rolled one day: today + 1 becomes date 0 (the engine's theta book)."""
    r = b.copy()
    d = np.asarray(b.days)
    drop = len(d) >= 3 and d[1] == d[0] + 1
    sh = 1 if drop else 0
    nd = len(d) - sh
    new_days = np.array([0] + [d[i + sh] - d[0] - 1 for i in range(1, nd)], dtype=np.int32)
    r.days = new_days
    r.t = new_days.astype(np.float64) / 365.0
    r.n_dates = nd
    for A in r.assets:
        c = np.asarray(A["carry"])
        new = np.empty(nd)
        new[0] = c[1]
        for i in range(1, nd):
            o = i + sh
            new[i] = (c[o] * b.t[o] - c[1] * (1.0 / 365.0)) / r.t[i]
        A["carry"] = new
    for P in r.products:
        P["maturity"] = max(P["maturity"] - sh, 0)
    return r, sh


def test_frozen_policy_greeks_equal_the_oracle(gpu):
    b = vanilla_book(paths=(1 << 15) + 11)
    S0 = b.assets[0]["spot"]
    g = gpu.price_american(b, 0, flags=abi.BUMP_DELTA | abi.BUMP_GAMMA | abi.BUMP_VEGA | abi.BUMP_RHO |
                           abi.BUMP_THETA)
    base = oracle_pass(gpu, b)
    A0 = base["premium"]
    assert g["premium"] == A0

    def frozen(book, z=None):
        return oracle_pass(gpu, book, zero_rates=z, policy=base)["premium"]

    def spot(h):
        c = b.copy()
        c.assets[0]["spot"] *= 1 + h
        return frozen(c)

    want = {"delta": (spot(0.01) - A0) / (0.01 * S0),
            "gamma": (spot(0.1) - 2.0 * A0 + spot(-0.1)) / ((0.1 * S0) * (0.1 * S0))}
    v = b.copy()
    v.assets[0]["vol"] += 0.01
    want["vega"] = frozen(v) - A0
    rb = b.copy()
    rb.assets[0]["carry"] = np.asarray(rb.assets[0]["carry"]) + 1e-4
    rb.products[0]["zero_rate"] += 1e-4
    want["rho"] = (frozen(rb, rates_of(b) + 1e-4) - A0) / 1e-4 * 0.01
    tb, sh = roll(b)
    zt = rates_of(b)[sh:] if sh else rates_of(b)
    want["theta"] = oracle_pass(gpu, tb, zero_rates=zt)["premium"] - A0
    for k, w in want.items():
        assert g[k] == pytest.approx(w, rel=1e-12, abs=1e-13), (k, g[k], w)


def test_frozen_policy_on_daily_dates_equals_the_oracle(gpu):
    """The apply walk on many dates and paths: single-precision screening of each exercise
    test, double precision near the boundary; the bumped premiums equal the oracle's."""
    days = np.arange(0, 151)
    b = vanilla_book(paths=(1 << 16) + 3, days=days, K=104.0, model="heston")
    S0 = b.assets[0]["spot"]
    g = gpu.price_american(b, 0, flags=abi.BUMP_DELTA | abi.BUMP_GAMMA)
    base = oracle_pass(gpu, b)
    A0 = base["premium"]
    assert g["premium"] == A0

    def frozen(book):
        return oracle_pass(gpu, book, policy=base)["premium"]

    def spot(h):
        c = b.copy()
        c.assets[0]["spot"] *= 1 + h
        return frozen(c)

    want = {"delta": (spot(0.01) - A0) / (0.01 * S0),
            "gamma": (spot(0.1) - 2.0 * A0 + spot(-0.1)) / ((0.1 * S0) * (0.1 * S0))}
    for k, w in want.items():
        assert g[k] == pytest.approx(w, rel=1e-12, abs=1e-13), (k, g[k], w)


def test_reference_american_call_equals_the_european_call(gpu):
    """test_american.cpp:8-20: no dividend, so never exercised early (200 000 paths)."""
    b = vanilla_book(typ=abi.CALL, paths=200000)
    r = gpu.price_american(b, 0)
    bs = oracle.bs_price(100.0 * math.exp(0.08), 100.0, 1.0, 0.30, math.exp(-0.08), True)
    assert abs(r["premium"] - bs) <= 6.0 * r["trust"] + 5e-2


def test_reference_american_put_against_the_tree(gpu):
    """test_american.cpp:22-44 (300 000 paths): above the European put, close to and not
    much above the continuous-exercise value."""
    b = vanilla_book(paths=300000)
    r = gpu.price_american(b, 0)
    euro = oracle.bs_price(100.0 * math.exp(0.08), 100.0, 1.0, 0.30, math.exp(-0.08), False)
    tree = am.binomial(100.0, 100.0, 1.0, 0.08, 0.0, 0.30, call=False)
    assert tree > euro
    assert r["premium"] > euro
    assert r["premium"] <= tree + 6.0 * r["trust"] + 5e-2
    assert r["premium"] >= 0.95 * tree


def test_reference_american_put_greeks_track_the_tree(gpu):
    """test_american.cpp:46-97: frozen-policy delta, vega, theta close to the continuous-
    exercise Greeks of the same bumps; gamma positive, rho negative."""
    b = vanilla_book(paths=300000)
    g = gpu.price_american(b, 0, flags=abi.BUMP_DELTA | abi.BUMP_GAMMA | abi.BUMP_VEGA | abi.BUMP_RHO |
                           abi.BUMP_THETA)

    def tree(S=100.0, vol=0.30, T=1.0, r=0.08):
        return am.binomial(S, 100.0, T, r, 0.0, vol, call=False)

    p = tree()
    t_delta = (tree(S=101.0) - p) / 1.0
    t_vega = tree(vol=0.31) - p
    t_theta = tree(T=1.0 - 1.0 / 365.0) - p
    assert g["delta"] < 0 and abs(g["delta"] - t_delta) <= 0.03, (g["delta"], t_delta)
    assert g["vega"] > 0 and abs(g["vega"] - t_vega) <= 0.05, (g["vega"], t_vega)
    assert g["theta"] < 0 and abs(g["theta"] - t_theta) <= 0.01, (g["theta"], t_theta)
    assert g["gamma"] > 0
    assert g["rho"] < 0


def test_deep_in_the_money_put_is_near_intrinsic(gpu):
    """test_american.cpp:99-106 (there on the PDE engine; here on the exercise fit)."""
    b = vanilla_book(S=60.0, paths=100000)
    r = gpu.price_american(b, 0)
    assert 40.0 - 1e-2 <= r["premium"] <= 42.0


def test_errors_and_maturity_today(gpu):
    b = vanilla_book(paths=4096)
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.price_american(b, 3)
    assert e.value.code == abi.THOTH_GPU_E_INVALID
    q = vanilla_book(paths=4096)
    q.products[0]["quanto"] = 0.01
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.price_american(q, 0)
    assert e.value.code == abi.THOTH_GPU_E_UNSUPPORTED
    br = abi.Book(days=np.asarray(DAYS), paths=4096)
    a = br.add_gbm(100.0, 0.3, 0.0)
    br.add_barrier(a, 100.0, len(DAYS) - 1, 80.0, up=False, knock_in=False, monitor=np.arange(1, len(DAYS)))
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.price_american(br, 0)
    assert e.value.code == abi.THOTH_GPU_E_UNSUPPORTED
    t0 = vanilla_book(paths=4096)
    t0.products[0]["maturity"] = 0
    r = gpu.price_american(t0, 0)
    assert r["premium"] == 0.0 and r["fitted_dates"] == 0


def test_book_call_equals_contract_by_contract(gpu):
    """thoth_gpu_price_american_book: one simulation per asset and scenario, the same
    numbers as pricing each contract alone."""
    b = abi.Book(days=np.asarray(DAYS), paths=20000)
    g = b.add_gbm(100.0, 0.30, 0.05)
    h = b.add_heston(50.0, 0.05, 1.5, 0.05, 0.5, -0.6, 0.03)
    b.add_vanilla(g, 100.0, 13, abi.PUT, zero_rate=0.05)
    b.add_vanilla(g, 90.0, 6, abi.PUT, zero_rate=0.05)
    b.add_variance(g, 13, strike_variance=0.09, notional=1.0, zero_rate=0.05)   # not American: skipped
    b.add_vanilla(h, 55.0, 13, abi.PUT, zero_rate=0.03)
    b.add_vanilla(h, 45.0, 9, abi.CALL, zero_rate=0.03)
    am = [0, 1, 3, 4]
    flags = abi.BUMP_DELTA | abi.BUMP_GAMMA | abi.BUMP_VEGA | abi.BUMP_RHO | abi.BUMP_THETA
    together = gpu.price_american_book(b, am, flags=flags)
    for r, p in zip(together, am):
        alone = gpu.price_american(b, p, flags=flags)
        for k in ("premium", "trust", "european", "delta", "gamma", "vega", "rho", "theta", "fitted_dates"):
            assert r[k] == alone[k], (p, k, r[k], alone[k])
        np.testing.assert_array_equal(r["beta"], alone["beta"])


def test_american_on_a_calibrated_lsv_name(gpu):
    """Leverage calibrated on the device, LSV paths stored, the exercise fit on them: the fit
    equals the oracle's on the same stored paths."""
    from thoth_gb300 import workloads as W
    c = W.lsv_calibration(horizon_days=182, particles=8192)
    lev, _ = gpu.calibrate_leverage(c)
    h = c.heston
    b = abi.Book(days=c.days, paths=30000)
    a = b.add_heston(100.0, h["v0"], h["kappa"], h["theta"], h["xi"], h["rho"], 0.02,
                     leverage=(c.ln_step, c.offset, lev))
    b.add_vanilla(a, 100.0, 182, abi.PUT, zero_rate=0.03)
    r = gpu.price_american(b, 0)
    o = oracle_pass(gpu, b)
    assert_same_fit(r, o, b.n_dates)


def test_book_call_past_one_fit_launch(gpu):
    """70 contracts on one name: two fit launches (64 + 6), each contract as if alone."""
    b = abi.Book(days=np.asarray(DAYS), paths=4096)
    a = b.add_gbm(100.0, 0.30, 0.06)
    for k in range(70):
        b.add_vanilla(a, 70.0 + k, 13 if k % 3 else 7, abi.PUT if k % 2 else abi.CALL, zero_rate=0.06)
    together = gpu.price_american_book(b, list(range(70)))
    for p in (0, 1, 63, 64, 69):
        alone = gpu.price_american(b, p)
        assert together[p]["premium"] == alone["premium"], p
        np.testing.assert_array_equal(together[p]["beta"], alone["beta"])


def test_zero_strike_normalises_by_the_initial_spot(gpu):
    """Vanilla::LsmBasisNorm (vanilla.hpp:38-41): a non-positive strike regresses on S / S0,
    S0 the paths' spot at date 0 (stored in single precision)."""
    b = vanilla_book(typ=abi.CALL, K=0.0, paths=20000, r=0.02)
    b.assets[0]["carry"] = b.assets[0]["carry"] - 0.05
    r = gpu.price_american(b, 0)
    S, _ = gpu.simulate_paths(b, 0)
    o = am.fit(S, b.t, rates_of(b), 0.0, True, float(np.float32(100.0)))
    assert r["premium"] == o["premium"] and r["fitted_dates"] == int(o["has_fit"].sum())
