"""Seeded synthetic books with the shapes of the engine's benchmark workloads.

The reference publishes no dataset; every input here is synthetic and seeded,
with the shapes, sizes and parameter ranges of the workloads it is measured on:

  gbm_call            1 asset GBM European call, 1 step
  heston_grid         Heston vanilla grid, 9 strikes x 7 maturities x call/put
  lsv_book            5 LSV names, 20 down-and-out calls, 10 variance swaps, 20 baskets
  ragged_books        256 books of uneven path and step counts (GBM / Heston / LSV mix)
  lsv_calibration     leverage calibration inputs: daily dates, layer grids sized as the
                      reference sizes them, a skewed target local-vol surface
  american_put        1 asset American put, Heston daily exercise or the reference tests'
                      GBM case (30-day exercise grid)
"""
import math

import numpy as np

from .abi import Book, CALL, PUT, GREEK_DELTA, GREEK_VEGA

MONTHS = (1, 2, 3, 4, 5, 12, 24)
STRIKES = tuple(range(80, 121, 5))
HESTON = dict(kappa=1.5, theta=0.04, xi=0.6, rho=-0.7, v0=0.04)


def gbm_call(paths=1 << 18, greeks=True):
    """S0 = K = 100, T = 365 days, sigma 0.25, r 0.03, q 0.01; delta and vega pathwise."""
    b = Book(days=[0, 365], paths=paths, greeks=(GREEK_DELTA | GREEK_VEGA) if greeks else 0)
    a = b.add_gbm(100.0, 0.25, 0.03 - 0.01)
    b.add_vanilla(a, 100.0, 1, CALL, zero_rate=0.03)
    return b


def heston_grid(paths=1 << 20, steps_per_year=252, calendar=False, months=MONTHS, strikes=STRIKES, greeks=False):
    """Heston grid: kappa 1.5, theta 0.04, xi 0.6, rho -0.7, v0 0.04, S0 100, r 0.03, q 0.

    steps_per_year grid (t = k / steps_per_year, maturity m months at k = m * steps_per_year / 12),
    or, with calendar=True, the reference's daily ACT/365 grid (max_day_step 1) with
    maturities at round(365 m / 12) days.
    """
    r = 0.03
    if calendar:
        mat_days = [int(round(365 * m / 12.0)) for m in months]
        days = np.arange(0, max(mat_days) + 1)
        b = Book(days=days, paths=paths)
        mats = mat_days
    else:
        n = int(round(max(months) * steps_per_year / 12.0))
        b = Book(times=np.arange(n + 1) / float(steps_per_year), paths=paths)
        mats = [int(round(m * steps_per_year / 12.0)) for m in months]
    if greeks:
        b.greeks = GREEK_DELTA
    a = b.add_heston(100.0, HESTON["v0"], HESTON["kappa"], HESTON["theta"], HESTON["xi"], HESTON["rho"], r)
    for mi in mats:
        for K in strikes:
            for typ in (CALL, PUT):
                b.add_vanilla(a, float(K), mi, typ, zero_rate=r)
    return b


def _smooth(x, passes=2):
    for _ in range(passes):
        p = np.pad(x, 1, mode="edge")
        x = sum(p[i:i + x.shape[0], j:j + x.shape[1]] for i in range(3) for j in range(3)) / 9.0
    return x


def _repair_correlation(rng, n):
    A = rng.normal(size=(n, n + 2))
    C = A @ A.T
    d = np.sqrt(np.diag(C))
    C = C / np.outer(d, d)
    w, V = np.linalg.eigh(C)
    w = np.maximum(w, 1e-3)
    C = (V * w) @ V.T
    d = np.sqrt(np.diag(C))
    return C / np.outer(d, d)


def lsv_book(paths=1 << 20, seed=20260101, horizon_days=365, n_lev_strikes=50, n_lev_times=40, greeks=False):
    """5 LSV names (Heston base + 50 x 40 leverage surface), 3 currencies, EUR quanto;
    20 down-and-out calls (daily monitoring, H in 70-90% S0), 10 variance swaps,
    20 basket calls; daily calendar grid over one year."""
    rng = np.random.default_rng(seed)
    days = np.arange(0, horizon_days + 1)
    nd = len(days)
    b = Book(days=days, paths=paths, greeks=GREEK_DELTA if greeks else 0)
    rates = rng.uniform(0.0, 0.05, size=3)           # USD (book), EUR, JPY
    ccy = [0, 1, 1, 2, 0]
    fx_spot = [1.0, 1.1, 0.007]
    S0 = rng.uniform(50, 200, size=5)
    corr = _repair_correlation(rng, 5)
    assets = []
    for k in range(5):
        kappa = rng.uniform(0.5, 3)
        theta = rng.uniform(0.02, 0.09)
        xi = rng.uniform(0.2, 0.8)
        rho = rng.uniform(-0.9, -0.3)
        v0 = rng.uniform(0.02, 0.09)
        # leverage: 50 absolute log-spot knots x 40 time knots, values U[0.7,1.3] smoothed twice (3x3 box)
        surf = _smooth(rng.uniform(0.7, 1.3, size=(n_lev_times, n_lev_strikes)))
        ln_lo, ln_hi = math.log(S0[k] * 0.3), math.log(S0[k] * 2.5)
        ln_step = (ln_hi - ln_lo) / (n_lev_strikes - 1)
        offset = int(math.floor(ln_lo / ln_step))
        layer_of_date = np.minimum((np.arange(nd) * n_lev_times) // nd, n_lev_times - 1)
        values = surf[layer_of_date]
        lev = (np.full(nd, ln_step), np.full(nd, offset, dtype=np.int64), values)
        assets.append(b.add_heston(S0[k], v0, kappa, theta, xi, rho, rates[ccy[k]], leverage=lev))
    b.set_cholesky(np.linalg.cholesky(corr))
    sigma_fx, rho_fx = 0.1, rng.uniform(-0.5, 0.5, size=5)
    mats = [91, 182, 365]

    def settle(k):
        # EUR names pay in USD as quantos (no FX conversion); others convert at spot
        if ccy[k] == 1:
            q = math.sqrt(b.assets[k]["v0"]) * sigma_fx * rho_fx[k]
            return 1.0, q, rates[0]
        return fx_spot[ccy[k]], 0.0, rates[ccy[k]]

    for j in range(20):
        k = j % 5
        fx, q, r = settle(k)
        m = mats[j % 3]
        H = rng.uniform(0.7, 0.9) * S0[k]
        b.add_barrier(k, S0[k] * rng.uniform(0.9, 1.1), m, H, up=False, knock_in=False,
                      monitor=np.arange(1, m + 1), option_type=CALL, zero_rate=r, fx=fx, quanto=q)
    for j in range(10):
        k = j % 5
        fx, q, r = settle(k)
        m = mats[j % 3]
        b.add_variance(k, m, strike_variance=rng.uniform(0.15, 0.3) ** 2, notional=100.0, zero_rate=r, fx=fx, quanto=q)
    for j in range(20):
        comps = rng.choice(5, size=int(rng.integers(2, 6)), replace=False)
        w = rng.uniform(0.5, 1.5, size=len(comps))
        w = 100.0 * w / w.sum() / S0[comps]          # rebased-100 index weights
        m = mats[j % 3]
        b.add_basket(comps, w, rng.uniform(90, 110), m, CALL, zero_rate=rates[0], fx=1.0)
    return b


LSV_GRID_POINTS = 201          # single.cpp:179
LSV_GRID_SIGMA_FACTOR = 8.0    # single.cpp:177


def layer_grids(days, spot, atm_vol):
    """Each date's leverage grid as Single::CalibrateLeverage sizes it (single.cpp:428-443):
    +-8 ATM standard deviations around ln S0 in 201 points (today uses T = 1 day)."""
    ln_step, offset = [], []
    for d in days:
        T = d / 365.0
        if T <= 0:
            T = 1.0 / 365.0
        hw = LSV_GRID_SIGMA_FACTOR * atm_vol * math.sqrt(T)
        st = 2.0 * hw / (LSV_GRID_POINTS - 1)
        if st <= 0:
            st = 1e-4
        ln_step.append(st)
        offset.append(int(math.floor((math.log(spot) - hw) / st)))
    return np.asarray(ln_step), np.asarray(offset, dtype=np.int64)


def skew_local_vol(S, t, atm=0.22, skew=-0.35, term=0.15):
    """A smooth skewed local-vol surface: atm (S/100)^skew, rising slowly with t, floored."""
    return np.maximum(atm * (np.asarray(S) / 100.0) ** skew * (1.0 + term * np.sqrt(t)), 0.05)


def lsv_calibration(horizon_days=365, spot=100.0, particles=0, local_vol=skew_local_vol, carry=0.02,
                    heston=None, seed=None):
    """Leverage calibration inputs for one LSV name: daily dates to the horizon, the
    reference's layer grids, and the target local vol on them."""
    from .abi import LeverageCalibration, LSV_CALIB_SEED
    days = np.arange(0, horizon_days + 1)
    h = heston or dict(v0=0.0324, kappa=2.0, theta=0.0676, xi=0.5, rho=-0.6)
    ln_step, offset = layer_grids(days, spot, 0.22)
    x = (offset[:, None] + np.arange(LSV_GRID_POINTS)[None, :]) * ln_step[:, None]
    sig = local_vol(np.exp(x), (days / 365.0)[:, None])
    return LeverageCalibration(days, carry, spot, h, ln_step, offset, sig, particles=particles,
                               seed=LSV_CALIB_SEED if seed is None else seed)


def american_put(paths=1 << 20, heston=True, days=None):
    """American put K=100 on one asset S0=100: Heston (the grid's parameters, r=3%) with a
    year of daily exercise dates, or GBM vol 30% r=8% on the reference tests' grid (one
    year, 30-day steps: pricer/tests/test_american.cpp). Product 0 is the put."""
    if days is None:
        days = range(0, 366) if heston else list(range(0, 361, 30)) + [365]
    b = Book(days=np.asarray(days), paths=paths)
    if heston:
        h = HESTON
        a = b.add_heston(100.0, h["v0"], h["kappa"], h["theta"], h["xi"], h["rho"], 0.03)
    else:
        a = b.add_gbm(100.0, 0.30, 0.08)
    b.add_vanilla(a, 100.0, len(b.t) - 1, PUT, zero_rate=0.03 if heston else 0.08)
    return b


def ragged_books(n_books=256, seed=7, min_paths=1 << 14, max_paths=1 << 22, min_steps=12, max_steps=730,
                 path_scale=1.0, model_mix=(0.4, 0.4, 0.2), payoffs=(0, 1, 2)):
    """Batched ragged workload: path counts log-uniform in [min, max], step counts uniform,
    model mix 40% GBM / 40% Heston / 20% LSV, payoff mix vanilla / barrier / variance.
    model_mix (GBM, Heston, LSV shares) and payoffs (0 vanilla, 1 barrier, 2 variance) narrow
    the mix; at their defaults the draws are those of the ragged-book workload."""
    rng = np.random.default_rng(seed)
    books = []
    for _ in range(n_books):
        paths = int(round(math.exp(rng.uniform(math.log(min_paths), math.log(max_paths))) * path_scale))
        paths = max(paths, 2)
        steps = int(rng.integers(min_steps, max_steps + 1))
        days = np.arange(0, steps + 1)
        b = Book(days=days, paths=paths)
        u = rng.random()
        r = 0.03
        if u < model_mix[0]:
            a = b.add_gbm(100.0, 0.25, r - 0.01)
        else:
            lev = None
            if u >= model_mix[0] + model_mix[1]:
                nd = steps + 1
                ln_step = (math.log(250.0) - math.log(30.0)) / 49
                offset = int(math.floor(math.log(30.0) / ln_step))
                vals = _smooth(rng.uniform(0.7, 1.3, size=(8, 50)))[np.minimum(np.arange(nd) * 8 // nd, 7)]
                lev = (np.full(nd, ln_step), np.full(nd, offset, dtype=np.int64), vals)
            a = b.add_heston(100.0, HESTON["v0"], HESTON["kappa"], HESTON["theta"], HESTON["xi"], HESTON["rho"], r,
                             leverage=lev)
        kind = payoffs[int(rng.integers(0, len(payoffs)))]
        mat = steps
        if kind == 0:
            for K in (90.0, 100.0, 110.0):
                b.add_vanilla(a, K, mat, CALL, zero_rate=r)
                b.add_vanilla(a, K, mat, PUT, zero_rate=r)
        elif kind == 1:
            b.add_barrier(a, 100.0, mat, 80.0, up=False, knock_in=False, monitor=np.arange(1, mat + 1), zero_rate=r)
            b.add_barrier(a, 100.0, mat, 120.0, up=True, knock_in=True, monitor=np.arange(1, mat + 1),
                          option_type=PUT, zero_rate=r)
        else:
            b.add_variance(a, mat, strike_variance=0.04, notional=100.0, zero_rate=r)
        books.append(b)
    return books
