"""Learned Heston surrogate: data from the GPU Monte-Carlo engine, training and
serving on the tensor-core kernels, and the MC judge / fallback around it.

Inputs (7): log-moneyness ln(K/S) in [-0.5, 0.5], maturity T in [1/12, 3] years,
kappa in [0.5, 5], theta in [0.01, 0.16], xi in [0.1, 1.0], rho in [-0.95, 0],
v0 in [0.01, 0.16]; r = q = 0. Output: the call price in units of spot.

Accuracy metric of a cell: |price - reference| / max(reference, 0.01) (relative
error with a floor at 1% of spot); the target is 1e-3.
"""
import ctypes as C
import math
import time

import numpy as np

from . import abi
from .abi import Book, CALL

BOX_LO = np.array([-0.5, 1 / 12.0, 0.5, 0.01, 0.1, -0.95, 0.01])
BOX_HI = np.array([0.5, 3.0, 5.0, 0.16, 1.0, 0.0, 0.16])
FEATURES = ("log_moneyness", "T", "kappa", "theta", "xi", "rho", "v0")
LATTICE_LM = np.round(np.linspace(-0.5, 0.5, 21), 10)
LATTICE_T = np.array([1, 2, 3, 6, 9, 12, 15, 18, 24, 27, 30, 36]) / 12.0
STEPS_PER_YEAR = 252
FLOOR = 0.01
TOL = 1e-3


def _ndtr(x):
    from scipy.special import ndtr
    return ndtr(x)


def bs_effective(X):
    """Black-Scholes call price (S = 1, r = q = 0) at the expected average Heston
    variance over [0, T]: the closed-form estimate the network corrects."""
    X = np.asarray(X, dtype=np.float64)
    lm, T, kappa, theta, v0 = X[:, 0], X[:, 1], X[:, 2], X[:, 3], X[:, 6]
    kt = kappa * T
    var = theta + (v0 - theta) * (1.0 - np.exp(-kt)) / kt
    sd = np.sqrt(np.maximum(var, 1e-8) * T)
    K = np.exp(lm)
    d1 = -lm / sd + 0.5 * sd
    return _ndtr(d1) - K * _ndtr(d1 - sd)


def price_scale(X):
    """bs_effective with a smooth floor at 1% of spot, sqrt(BS^2 + 0.01^2): the
    network learns price / scale, an O(1) correction, so its absolute precision
    is relative price precision. The floor is smooth because a kink (max) in the
    scale is a kink in the target, which a SiLU network fits badly."""
    c = bs_effective(X)
    return np.sqrt(c * c + FLOOR * FLOOR)


def normalise(x):
    return (2.0 * (np.asarray(x, dtype=np.float64) - BOX_LO) / (BOX_HI - BOX_LO) - 1.0).astype(np.float32)


def in_box(x):
    x = np.asarray(x)
    return np.all((x >= BOX_LO - 1e-12) & (x <= BOX_HI + 1e-12), axis=1)


def cell_error(price, ref):
    return np.abs(np.asarray(price) - np.asarray(ref)) / np.maximum(np.abs(ref), FLOOR)


def sobol_params(n, skip=0):
    """Heston parameter sets (kappa, theta, xi, rho, v0) from the first 5 Sobol dimensions."""
    from . import sobol_points
    u = (sobol_points(5, skip, n).astype(np.float64) + 0.5) / 2.0 ** 32
    return BOX_LO[2:] + u * (BOX_HI[2:] - BOX_LO[2:])


def lattice_book(params, paths, lms=LATTICE_LM, Ts=LATTICE_T, skip=0):
    """One Heston book pricing every (log-moneyness, maturity) call of the lattice on shared paths."""
    kappa, theta, xi, rho, v0 = (float(v) for v in params)
    n = int(round(max(Ts) * STEPS_PER_YEAR))
    b = Book(times=np.arange(n + 1) / float(STEPS_PER_YEAR), paths=paths, sobol_skip=skip)
    a = b.add_heston(1.0, v0, kappa, theta, xi, rho, 0.0)
    for T in Ts:
        mi = int(round(T * STEPS_PER_YEAR))
        for lm in lms:
            b.add_vanilla(a, float(math.exp(lm)), mi, CALL, zero_rate=0.0)
    return b


def lattice_features(params, lms=LATTICE_LM, Ts=LATTICE_T):
    rows = []
    for T in Ts:
        for lm in lms:
            rows.append([lm, T] + list(params))
    return np.array(rows)


def mc_labels(param_sets, paths, lms=LATTICE_LM, Ts=LATTICE_T, distinct=False):
    """Price each parameter set's lattice with the GPU MC engine: (features, prices, trusts, seconds).

    distinct=True gives set i its own block of Sobol points (skip = i * paths), so
    label errors are independent across sets and the fit averages them out;
    with shared points they are a smooth function of the parameters, which the
    network would learn as if it were the price."""
    from . import price_book
    X, Y, S = [], [], []
    t0 = time.perf_counter()
    for i, p in enumerate(param_sets):
        r = price_book(lattice_book(p, paths, lms, Ts, skip=i * paths if distinct else 0))
        X.append(lattice_features(p, lms, Ts))
        Y.append(r["premium"])
        S.append(r["trust"])
    return np.concatenate(X), np.concatenate(Y), np.concatenate(S), time.perf_counter() - t0


def train_targets(X, Y):
    """(normalised inputs, targets price / scale, loss scales) for thoth_gpu_surrogate_train."""
    sc = price_scale(X)
    return normalise(X), (Y / sc).astype(np.float32), (np.maximum(np.abs(Y), FLOOR) / sc).astype(np.float32)


def predict_prices(model, X):
    """Surrogate prices (units of spot) of raw feature rows X [n][7]."""
    X = np.asarray(X, dtype=np.float64)
    r, ms = model.predict(normalise(X))
    return r.astype(np.float64) * price_scale(X), ms


class Surrogate:
    """The MLP on the GPU (thoth_gpu_surrogate_*)."""

    def __init__(self, seed=0):
        from . import lib
        self.L = lib()
        L = self.L
        L.thoth_gpu_surrogate_create.argtypes = [C.POINTER(C.c_void_p), C.c_uint64]
        L.thoth_gpu_surrogate_destroy.argtypes = [C.c_void_p]
        L.thoth_gpu_surrogate_get_params.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        L.thoth_gpu_surrogate_set_params.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        L.thoth_gpu_surrogate_train.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                                C.POINTER(C.c_float), C.c_int64, C.c_int32, C.c_int32, C.c_double,
                                                C.c_uint64, C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_gradient.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                                   C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                                                   C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_predict.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float),
                                                  C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_last_error.restype = C.c_char_p
        self.n_params = L.thoth_gpu_surrogate_n_params()
        self.h = C.c_void_p()
        self._check(L.thoth_gpu_surrogate_create(C.byref(self.h), seed))

    def _check(self, rc):
        if rc != 0:
            from . import ThothGpuError
            raise ThothGpuError(rc, self.L.thoth_gpu_surrogate_last_error().decode())

    @staticmethod
    def _f(a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        return a, a.ctypes.data_as(C.POINTER(C.c_float))

    def params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.L.thoth_gpu_surrogate_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p, pp = self._f(p)
        self._check(self.L.thoth_gpu_surrogate_set_params(self.h, pp))

    def gradient(self, xn, y, scale):
        xn, px = self._f(xn)
        y, py = self._f(y)
        sc, ps = self._f(scale)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_double()
        self._check(self.L.thoth_gpu_surrogate_gradient(self.h, px, py, ps, len(y),
                                                        g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return g, loss.value

    def train(self, xn, y, scale, epochs=20, batch=8192, lr=2e-3, seed=1):
        xn, px = self._f(xn)
        y, py = self._f(y)
        sc, ps = self._f(scale)
        loss = C.c_double()
        self._check(self.L.thoth_gpu_surrogate_train(self.h, px, py, ps, len(y), epochs, batch, lr, seed,
                                                     C.byref(loss)))
        return loss.value

    def predict(self, xn):
        xn, px = self._f(xn)
        y = np.zeros(len(xn), dtype=np.float32)
        ms = C.c_double()
        self._check(self.L.thoth_gpu_surrogate_predict(self.h, px, len(xn), y.ctypes.data_as(C.POINTER(C.c_float)),
                                                       C.byref(ms)))
        return y, ms.value

    def close(self):
        if self.h:
            self.L.thoth_gpu_surrogate_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _mc_subset(param_sets, paths, lms, Ts):
    """MC prices of the (lms x Ts) sub-lattice of each set: (prices [sets][len(Ts)*len(lms)], seconds)."""
    if len(param_sets) == 0:
        return np.zeros((0, len(lms) * len(Ts))), 0.0
    _, y, _, secs = mc_labels(param_sets, paths, lms, Ts)
    return y.reshape(len(param_sets), -1), secs


POLICIES = ("bucket", "grid")


def choose_fallback(jerr, tol=TOL, policy="bucket", margin=1.0, n_T=None):
    """Buckets (columns of jerr [judged sets][buckets], the surrogate's judged cell
    errors, maturity-major with n_T maturities) that MC takes over; see judge().
    The grid policy is cost-aware: an MC fallback book runs to its longest
    maturity, so it looks for the shortest maturity horizon within which taking
    over the worst buckets (worst first) brings the grid to the target."""
    jerr = np.asarray(jerr, dtype=np.float64)
    bucket = np.quantile(jerr, 0.9, axis=0)
    if policy == "bucket":
        return bucket > tol
    if policy != "grid":
        raise ValueError("policy must be one of %s" % (POLICIES,))
    nb = bucket.size
    n_T = n_T or nb
    mat = np.arange(nb) // (nb // n_T)        # maturity index of each bucket
    if np.quantile(jerr, 0.9) <= margin * tol:
        return np.zeros(nb, dtype=bool)
    best = None
    for h in range(n_T):                       # horizon: maturities 0 .. h may fall back
        bad = np.zeros(nb, dtype=bool)
        e = jerr.copy()
        for b in np.argsort(-bucket, kind="stable"):
            if mat[b] > h or bucket[b] <= 0.5 * tol:
                continue
            bad[b] = True
            e[:, b] = 0.5 * tol
            if np.quantile(e, 0.9) <= margin * tol:
                break
        if np.quantile(e, 0.9) <= margin * tol:
            return bad
        best = bad
    return best | (bucket > tol)               # the target is out of reach: every bucket above tol too


def judge(model, param_sets, judge_frac=0.01, judge_paths=1 << 20, tol=TOL, seed=0, lms=LATTICE_LM, Ts=LATTICE_T,
          policy="bucket", margin=1.0):
    """MC judge: re-price a random judge_frac of the sets with judge_paths (whose Sobol
    error is below tol) and choose the lattice buckets (maturity, log-moneyness) that
    MC takes over.

    policy "bucket": every bucket whose 90th-percentile surrogate error on the judged
    sets exceeds tol (each bucket meets the target on its own).
    policy "grid": buckets, worst first and within the shortest maturity horizon
    that suffices, such that the judged grid's 90th-percentile error, with the
    taken-over cells counted at tol / 2 (the MC fallback's own accuracy,
    calibrated to stay below tol), is at most margin * tol (the grid as a whole
    meets the target). The judge's own MC error adds to the measured one (the
    measured error is an upper estimate), so judge_paths should be well above the
    plain-MC count."""
    rng = np.random.default_rng(seed)
    n_judge = max(1, int(round(judge_frac * len(param_sets))))
    judged = np.sort(rng.choice(len(param_sets), size=n_judge, replace=False))
    Xj = np.concatenate([lattice_features(p, lms, Ts) for p in param_sets[judged]])
    t0 = time.perf_counter()
    _, jy, js, t_mc = mc_labels(param_sets[judged], judge_paths, lms, Ts)
    pj, _ = predict_prices(model, Xj)
    t_judge = time.perf_counter() - t0
    jerr = cell_error(pj, jy).reshape(n_judge, -1)
    bad = choose_fallback(jerr, tol, policy, margin, n_T=len(Ts))
    return dict(judged=judged, bad=bad.reshape(len(Ts), len(lms)), judge_s=t_judge,
                judge_mc_seconds_per_set=t_mc / n_judge, judged_p90=float(np.quantile(jerr, 0.9)))


def price_grid(model, param_sets, mc_paths, judge_frac=0.01, judge_paths=1 << 20, fallback_sample=None, seed=0,
               tol=TOL, lms=LATTICE_LM, Ts=LATTICE_T, policy="bucket"):
    """Price a grid of (parameter set x lattice) cells with the surrogate, judged by MC.

    1. inference for every cell (out-of-box features are clipped, then re-priced by MC);
    2. the MC judge (see judge(), with its policy) marks the lattice buckets MC takes over;
    3. the failing buckets of every set, and every set with out-of-box cells, are
       re-priced by MC with mc_paths (the plain-MC path count for the same accuracy),
       on books cut to the failing maturities and strikes. With fallback_sample = k only k sets are
       re-priced and the fallback time is scaled to all sets (used by the benchmark).
    Returns (prices [cells], info dict with timings and counts).
    """
    n_sets = len(param_sets)
    ncell = len(lms) * len(Ts)
    X = np.concatenate([lattice_features(p, lms, Ts) for p in param_sets])
    t0 = time.perf_counter()
    inside = in_box(X)
    price, dev_ms = predict_prices(model, np.clip(X, BOX_LO, BOX_HI))
    t_inf = time.perf_counter() - t0
    J = judge(model, param_sets, judge_frac, judge_paths, tol, seed, lms, Ts, policy=policy)
    bad2 = J["bad"]
    t2 = time.perf_counter()
    fb_T = np.nonzero(bad2.any(axis=1))[0]
    fb_lm = np.nonzero(bad2.any(axis=0))[0]
    fb_sets = np.arange(n_sets)
    if fallback_sample is not None and fallback_sample < n_sets:
        fb_sets = np.linspace(0, n_sets - 1, fallback_sample).astype(int)
    n_fb = 0
    if len(fb_T):
        fy, _ = _mc_subset(param_sets[fb_sets], mc_paths, lms[fb_lm], Ts[fb_T])
        fy = fy.reshape(len(fb_sets), len(fb_T), len(fb_lm))
        for a, ti in enumerate(fb_T):
            for b, li in enumerate(fb_lm):
                if bad2[ti, li]:
                    price[fb_sets * ncell + ti * len(lms) + li] = fy[:, a, b]
                    n_fb += len(fb_sets)
    out_sets = np.unique(np.nonzero(~inside)[0] // ncell)
    if len(out_sets):
        oy, _ = _mc_subset(param_sets[out_sets], mc_paths, lms, Ts)
        for j, k in enumerate(out_sets):
            sel = ~inside[k * ncell:(k + 1) * ncell]
            price[k * ncell:(k + 1) * ncell][sel] = oy[j][sel]
            n_fb += int(sel.sum())
    t_fb = time.perf_counter() - t2
    scale_fb = n_sets / len(fb_sets) if len(fb_T) else 1.0
    total = t_inf + J["judge_s"] + t_fb * scale_fb
    return price, dict(cells=len(X), seconds=total, inference_s=t_inf, inference_device_ms=dev_ms,
                       judge_s=J["judge_s"], judge_sets=len(J["judged"]), judge_paths=judge_paths,
                       fallback_s=t_fb * scale_fb, fallback_sets_run=int(len(fb_sets)) if len(fb_T) else 0,
                       fallback_cells=int(bad2.sum()) * n_sets + int((~inside).sum()),
                       failing_buckets=int(bad2.sum()), mc_paths=mc_paths, cells_per_sec=len(X) / total,
                       policy=policy, judged_p90=J["judged_p90"])


def calibrate_plain_mc(param_sets, cf, tol=TOL, lo=10, hi=24):
    """Smallest power-of-two path count whose 90th-percentile cell error against the
    closed form cf is at most tol, with the measured per-set seconds at that count.
    (Sobol + bridge errors fall faster than the MC standard error suggests, so the
    count is found by measurement, not from the trust.)"""
    for k in range(lo, hi + 1):
        X, y, _, secs = mc_labels(param_sets, 1 << k)
        e = cell_error(y, cf)
        if np.quantile(e, 0.9) <= tol:
            return 1 << k, secs / len(param_sets), e
    return 1 << hi, secs / len(param_sets), e


def benchmark(n_train=4096, n_eval=4096, train_paths=1 << 18, epochs=3000, lr=2e-3, batch=8192, cf_sets=16, seed=1,
              fallback_sample=16, judge_factor=8):
    """Train on MC labels, then price an n_eval x 252-cell grid at the same accuracy
    target (90th-percentile cell error <= 1e-3 against the FP64 closed form):
      plain MC   — every cell by MC at the path count calibrated on cf_sets sets;
      surrogate  — inference + 1% MC judge (judge_factor x the plain-MC path count)
                   + MC fallback, once per judge policy ("grid": the grid meets
                   the target; "bucket": every bucket does).
    The fallback runs on fallback_sample sets and is scaled to the grid. Errors are
    measured against the closed form on cf_sets sets spread over the grid."""
    import oracle  # the FP64 closed form, as the checker only
    t0 = time.perf_counter()
    X, Y, _, t_labels = mc_labels(sobol_params(n_train, 0), train_paths, distinct=True)
    model = Surrogate(seed=seed)
    xn, yt, st = train_targets(X, Y)
    t1 = time.perf_counter()
    loss = model.train(xn, yt, st, epochs=epochs, batch=batch, lr=lr)
    t_train = time.perf_counter() - t1
    ev = sobol_params(n_eval, n_train)
    ncell = len(LATTICE_LM) * len(LATTICE_T)
    pick = np.linspace(0, n_eval - 1, cf_sets).astype(int)
    Xs = np.concatenate([lattice_features(ev[k]) for k in pick])
    t2 = time.perf_counter()
    cf = oracle.heston_prices(1.0, np.exp(Xs[:, 0]), Xs[:, 1], 0, 0, Xs[:, 6], Xs[:, 2], Xs[:, 3], Xs[:, 4], Xs[:, 5])
    t_cf = time.perf_counter() - t2
    mc_paths, mc_set_s, e_mc = calibrate_plain_mc(ev[pick], cf)
    plain = ncell / mc_set_s
    raw, _ = predict_prices(model, Xs)
    q = lambda e: {"median": float(np.median(e)), "p90": float(np.quantile(e, 0.9)),
                   "p99": float(np.quantile(e, 0.99)), "max": float(e.max()), "frac_above_tol": float(np.mean(e > TOL))}
    policies = {}
    for policy in POLICIES:
        price, pinfo = price_grid(model, ev, mc_paths, judge_paths=judge_factor * mc_paths,
                                  fallback_sample=fallback_sample, policy=policy)
        pipe = np.concatenate([price[k * ncell:(k + 1) * ncell] for k in pick])
        pinfo.update(error_pipeline=q(cell_error(pipe, cf)), speedup=pinfo["cells_per_sec"] / plain)
        policies[policy] = pinfo
    info = dict(policies["grid"])
    info.update(train_sets=n_train, train_labels=len(Y), train_paths=train_paths, label_seconds=t_labels,
                train_seconds=t_train, epochs=epochs, final_loss=loss, cf_cells=len(cf), cf_seconds=t_cf,
                plain_mc_paths=mc_paths, plain_mc_seconds_per_set=mc_set_s, plain_mc_cells_per_sec=plain,
                inference_cells_per_sec=info["cells"] / info["inference_s"],
                error_surrogate_raw=q(cell_error(raw, cf)), error_surrogate_pipeline=info["error_pipeline"],
                error_plain_mc=q(e_mc), policies=policies, total_seconds=time.perf_counter() - t0)
    model.close()
    return info
