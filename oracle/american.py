"""TEST INFRASTRUCTURE: Longstaff-Schwartz exercise restated in numpy.

The algorithm of PricerMCL::FitAmericanPolicy / ApplyAmericanPolicy
(pricer/src/tasks/pricer_mcl_american.cpp:263-447), with the normal equations and the
Cholesky solve of pricer/src/helpers/maths.cpp:354-381 and 419-470, on date-major
single-precision spot paths S[date][path] as the engine stores them.

Every sum is exact: each addend is truncated to a multiple of 2^-64, the addends are
added as integers and the total is rounded once to the nearest double. That is the
engine's summation (thoth_gb300/csrc/exact.cuh), so on the same paths the engine's
regression coefficients, exercise decisions and premium equal this restatement's bit
for bit. The reference sums in path order; ``ref_lsm`` in oracle/_ref runs the
reference's loop that way around its own LeastSquares and pins this restatement to it.
Only tests/ and bench.py's CPU leg use this module.
"""
import math

import numpy as np

TWO64 = 2.0 ** 64
MAX_ADDEND = 2.0 ** 36


def exact_sum(x):
    """Sum of non-negative doubles, each truncated to a multiple of 2^-64, rounded once."""
    x = np.asarray(x, dtype=np.float64).ravel()
    if x.size == 0:
        return 0.0
    if not np.all(x < MAX_ADDEND):
        raise ValueError("addend out of range of the exact accumulator")
    ip = np.floor(x)
    f = np.floor((x - ip) * TWO64).astype(np.uint64)
    lo32 = (f & np.uint64(0xFFFFFFFF)).sum(dtype=np.uint64)
    hi32 = (f >> np.uint64(32)).sum(dtype=np.uint64)
    total = (int(ip.astype(np.int64).sum()) << 64) + (int(hi32) << 32) + int(lo32)
    return math.ldexp(float(total), -64)


def intrinsic(s, strike, call):
    """payoff_vanilla floored at 0 (helpers/finance.cpp:9-32): max(phi (S - K), 0)."""
    v = (s - strike) if call else (strike - s)
    return np.where(v < 0.0, 0.0, v)


def discounts(tau, rates, M):
    """df[t] rolls a cashflow from date t+1 back to t, disc[t] values date t today."""
    df = [math.exp(rates[t] * tau[t] - rates[t + 1] * tau[t + 1]) if t + 1 < M else 1.0 for t in range(M)]
    disc = [math.exp(-rates[t] * (tau[t] - tau[0])) for t in range(M)]
    return df, disc


def solve3(n, s):
    """(X^T X) beta = X^T y for X = {1, m, m^2} from the sums s = [m, m^2, m^3, m^4, y, y m, y m^2]:
    Cholesky in place, forward and back substitution; None where a pivot is not positive."""
    n = float(n)
    A = [[n, s[0], s[1]], [s[0], s[1], s[2]], [s[1], s[2], s[3]]]
    g = [s[4], s[5], s[6]]
    for i in range(3):
        for j in range(i + 1):
            acc = A[i][j]
            for k in range(j):
                acc -= A[i][k] * A[j][k]
            if i == j:
                if acc <= 0.0:
                    return None
                A[i][j] = math.sqrt(acc)
            else:
                A[i][j] = acc / A[j][j]
    z = [0.0] * 3
    for i in range(3):
        acc = g[i]
        for k in range(i):
            acc -= A[i][k] * z[k]
        z[i] = acc / A[i][i]
    b = [0.0] * 3
    for i in range(2, -1, -1):
        acc = z[i]
        for k in range(i + 1, 3):
            acc -= A[k][i] * b[k]
        b[i] = acc / A[i][i]
    return b


def _finish(val, S, strike, call):
    n = val.size
    total, total2 = exact_sum(val), exact_sum(val * val)
    mean = total / n
    trust = math.sqrt((total2 / n - mean * mean) / (n - 1.0)) if n > 1 else 0.0
    s0 = float(S[0, 0])
    premium = max(mean, float(intrinsic(s0, strike, call)))
    return premium, trust


def fit(S, tau, rates, strike, call, norm, min_itm=50):
    """Fit the policy on paths S[M][n] (M = maturity + 1 dates) and value it on them.
    Returns dict(premium, trust, european, beta [M][3] (0 where no fit), has_fit [M])."""
    S = np.asarray(S, dtype=np.float32)
    M, n = S.shape
    beta = np.zeros((M, 3))
    has = np.zeros(M, dtype=bool)
    if M < 2:
        return dict(premium=0.0, trust=0.0, european=0.0, beta=beta, has_fit=has)
    df, disc = discounts(tau, rates, M)
    iv = intrinsic(S[M - 1].astype(np.float64), strike, call)
    cf = iv.copy()
    val = iv * disc[M - 1]
    european = exact_sum(val) / n
    for t in range(M - 2, 0, -1):
        cf = cf * df[t]
        s = S[t].astype(np.float64)
        iv = intrinsic(s, strike, call)
        itm = np.nonzero(iv > 0.0)[0]
        if itm.size < min_itm:
            continue
        m = s[itm] / norm
        m2 = m * m
        y = cf[itm]
        sums = [exact_sum(m), exact_sum(m2), exact_sum(m2 * m), exact_sum(m2 * m2),
                exact_sum(y), exact_sum(m * y), exact_sum(m2 * y)]
        b = solve3(itm.size, sums)
        if b is None:
            continue
        beta[t] = b
        has[t] = True
        cont = (b[0] + b[1] * m) + (b[2] * m) * m
        ex = itm[iv[itm] >= cont]
        cf[ex] = iv[ex]
        val[ex] = iv[ex] * disc[t]
    premium, trust = _finish(val, S, strike, call)
    return dict(premium=premium, trust=trust, european=european, beta=beta, has_fit=has)


def apply(S, tau, rates, strike, call, norm, beta, has_fit):
    """Value a frozen policy on paths S[M][n]: exercise at the first date with a positive
    intrinsic value at least the fitted continuation, else at maturity."""
    S = np.asarray(S, dtype=np.float32)
    M, n = S.shape
    if M < 2:
        return dict(premium=0.0, trust=0.0)
    _, disc = discounts(tau, rates, M)
    val = np.zeros(n)
    alive = np.ones(n, dtype=bool)
    for t in range(1, M - 1):
        if not has_fit[t]:
            continue
        s = S[t].astype(np.float64)
        iv = intrinsic(s, strike, call)
        m = s / norm
        b = beta[t]
        cont = (b[0] + b[1] * m) + (b[2] * m) * m
        ex = alive & (iv > 0.0) & (iv >= cont)
        val[ex] = iv[ex] * disc[t]
        alive &= ~ex
    last = intrinsic(S[M - 1].astype(np.float64), strike, call) * disc[M - 1]
    val[alive] = last[alive]
    premium, trust = _finish(val, S, strike, call)
    return dict(premium=premium, trust=trust)


def gbm_paths(S0, vol, r, q, days, n, seed):
    """Exact GBM spot paths at the given calendar days (ACT/365), float32 [dates][n]."""
    rng = np.random.default_rng(seed)
    t = np.asarray(days, dtype=np.float64) / 365.0
    dt = np.diff(t)
    z = rng.standard_normal((dt.size, n))
    inc = ((r - q) - 0.5 * vol * vol) * dt[:, None] + vol * np.sqrt(dt)[:, None] * z
    logs = np.vstack([np.zeros((1, n)), np.cumsum(inc, axis=0)])
    return (S0 * np.exp(logs)).astype(np.float32)


def binomial(S0, K, T, r, q, vol, call, steps=2000, american=True):
    """Cox-Ross-Rubinstein tree with exercise at every step: the continuous-exercise
    value the reference's tests take from its PDE engine (tests/test_american.cpp)."""
    dt = T / steps
    u = math.exp(vol * math.sqrt(dt))
    d = 1.0 / u
    p = (math.exp((r - q) * dt) - d) / (u - d)
    disc = math.exp(-r * dt)
    j = np.arange(steps + 1)
    s = S0 * u ** (steps - 2 * j)
    v = np.maximum(s - K, 0.0) if call else np.maximum(K - s, 0.0)
    for i in range(steps - 1, -1, -1):
        v = disc * (p * v[:-1] + (1.0 - p) * v[1:])
        if american:
            s = S0 * u ** (i - 2 * np.arange(i + 1))
            v = np.maximum(v, (s - K) if call else (K - s))
    return float(v[0])
