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
    """Feature rows of one set's lattice, maturity-major: [len(Ts) * len(lms)][7]."""
    return grid_features(np.asarray(params, dtype=np.float64)[None, :], lms, Ts)


def grid_features(param_sets, lms=LATTICE_LM, Ts=LATTICE_T):
    """Feature rows of every set's lattice, set-major then maturity-major:
    [n_sets * len(Ts) * len(lms)][7] (log-moneyness, T, kappa, theta, xi, rho, v0)."""
    P = np.asarray(param_sets, dtype=np.float64).reshape(-1, 5)
    lms, Ts = np.asarray(lms, dtype=np.float64), np.asarray(Ts, dtype=np.float64)
    n, nT, nl = len(P), len(Ts), len(lms)
    X = np.empty((n, nT, nl, 7))
    X[..., 0] = lms[None, None, :]
    X[..., 1] = Ts[None, :, None]
    X[..., 2:] = P[:, None, None, :]
    return X.reshape(n * nT * nl, 7)


def mc_labels(param_sets, paths, lms=LATTICE_LM, Ts=LATTICE_T, distinct=False, skip=0):
    """Price each parameter set's lattice with the GPU MC engine: (features, prices, trusts, seconds).

    distinct=True gives set i its own block of Sobol points (skip = i * paths), so
    label errors are independent across sets and the fit averages them out;
    with shared points they are a smooth function of the parameters, which the
    network would learn as if it were the price. skip offsets every set's points."""
    from . import price_batch
    Y, S = [], []
    t0 = time.perf_counter()
    chunk = 256  # books per batch call (one CUDA graph each)
    for c0 in range(0, len(param_sets), chunk):
        sets = param_sets[c0:c0 + chunk]
        books = [lattice_book(p, paths, lms, Ts, skip=skip + ((c0 + i) * paths if distinct else 0))
                 for i, p in enumerate(sets)]
        for r in price_batch(books):
            Y.append(r["premium"])
            S.append(r["trust"])
    secs = time.perf_counter() - t0
    return grid_features(param_sets, lms, Ts), np.concatenate(Y), np.concatenate(S), secs


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
        L.thoth_gpu_surrogate_train_avg.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                                    C.POINTER(C.c_float), C.c_int64, C.c_int32, C.c_int32, C.c_double,
                                                    C.c_uint64, C.c_int32, C.c_double, C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_gradient.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                                   C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                                                   C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_predict.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float),
                                                  C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_price_lattice.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int32,
                                                        C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double),
                                                        C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                        C.c_double, C.POINTER(C.c_float), C.POINTER(C.c_double)]
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

    def train(self, xn, y, scale, epochs=20, batch=8192, lr=2e-3, seed=1, avg_epochs=0, lr_avg=0.0):
        """Adam with a cosine learning-rate decay; with avg_epochs > 0 the decay ends at lr_avg
        before the last avg_epochs epochs, whose end-of-epoch weights are averaged into the model."""
        xn, px = self._f(xn)
        y, py = self._f(y)
        sc, ps = self._f(scale)
        loss = C.c_double()
        self._check(self.L.thoth_gpu_surrogate_train_avg(self.h, px, py, ps, len(y), epochs, batch, lr, seed,
                                                         int(avg_epochs), float(lr_avg), C.byref(loss)))
        return loss.value

    def predict(self, xn):
        xn, px = self._f(xn)
        y = np.zeros(len(xn), dtype=np.float32)
        ms = C.c_double()
        self._check(self.L.thoth_gpu_surrogate_predict(self.h, px, len(xn), y.ctypes.data_as(C.POINTER(C.c_float)),
                                                       C.byref(ms)))
        return y, ms.value

    def price_lattice(self, param_sets, lms=LATTICE_LM, Ts=LATTICE_T):
        """Prices (units of spot) of every (set, maturity, log-moneyness) cell, features,
        clipping, normalisation and price scale on the device: the same cells and order as
        lattice_features and the same prices as predict_prices of the clipped features."""
        d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        P, lm, T, lo, hi = d(param_sets), d(lms), d(Ts), d(BOX_LO), d(BOX_HI)
        if P.ndim != 2 or P.shape[1] != 5:
            raise ValueError("param_sets must be [n][5] (kappa, theta, xi, rho, v0)")
        out = np.zeros(len(P) * len(lm) * len(T), dtype=np.float32)
        ms = C.c_double()
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._check(self.L.thoth_gpu_surrogate_price_lattice(self.h, ptr(P), len(P), ptr(lm), len(lm), ptr(T), len(T),
                                                             ptr(lo), ptr(hi), FLOOR,
                                                             out.ctypes.data_as(C.POINTER(C.c_float)), C.byref(ms)))
        return out, ms.value

    def close(self):
        if self.h:
            self.L.thoth_gpu_surrogate_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """k networks of the surrogate's architecture, each from its own initialisation and data
    order, trained side by side (thoth_gpu_surrogate_train_members) and served as the mean of
    their outputs (thoth_gpu_surrogate_price_lattice_mean). Trained on MC labels, one network's
    fit carries part of the labels' noise, differently for each initialisation; the mean keeps
    the common fit and averages that part out."""

    def __init__(self, members=4, seed=1):
        if members < 1:
            raise ValueError("an ensemble needs at least one member")
        self.members = [Surrogate(seed=seed + j) for j in range(members)]
        self.seed = seed
        L = self.L = self.members[0].L
        L.thoth_gpu_surrogate_train_members.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_float),
                                                        C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                                        C.c_int32, C.c_int32, C.c_double, C.c_uint64, C.c_int32,
                                                        C.c_double, C.POINTER(C.c_double)]
        L.thoth_gpu_surrogate_price_lattice_mean.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_double),
                                                             C.c_int32, C.POINTER(C.c_double), C.c_int32,
                                                             C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double),
                                                             C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_float),
                                                             C.POINTER(C.c_double)]

    def _handles(self):
        return (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])

    def train(self, xn, y, scale, epochs=20, batch=8192, lr=2e-3, seed=None, avg_epochs=0, lr_avg=0.0):
        """Every member on the same labels, member j with data-order seed seed + j; the final
        losses, one a member."""
        seed = self.seed if seed is None else seed
        xn, px = Surrogate._f(xn)
        y, py = Surrogate._f(y)
        sc, ps = Surrogate._f(scale)
        loss = (C.c_double * len(self.members))()
        self.members[0]._check(self.L.thoth_gpu_surrogate_train_members(
            self._handles(), len(self.members), px, py, ps, len(y), epochs, batch, lr, seed, int(avg_epochs),
            float(lr_avg), loss))
        return list(loss)

    def price_lattice(self, param_sets, lms=LATTICE_LM, Ts=LATTICE_T):
        """As Surrogate.price_lattice, for the members' mean."""
        d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        P, lm, T, lo, hi = d(param_sets), d(lms), d(Ts), d(BOX_LO), d(BOX_HI)
        if P.ndim != 2 or P.shape[1] != 5:
            raise ValueError("param_sets must be [n][5] (kappa, theta, xi, rho, v0)")
        out = np.zeros(len(P) * len(lm) * len(T), dtype=np.float32)
        ms = C.c_double()
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self.members[0]._check(self.L.thoth_gpu_surrogate_price_lattice_mean(
            self._handles(), len(self.members), ptr(P), len(P), ptr(lm), len(lm), ptr(T), len(T), ptr(lo), ptr(hi),
            FLOOR, out.ctypes.data_as(C.POINTER(C.c_float)), C.byref(ms)))
        return out, ms.value

    def close(self):
        for m in self.members:
            m.close()


def _mc_subset(param_sets, paths, lms, Ts):
    """MC prices of the (lms x Ts) sub-lattice of each set: (prices [sets][len(Ts)*len(lms)], seconds)."""
    if len(param_sets) == 0:
        return np.zeros((0, len(lms) * len(Ts))), 0.0
    _, y, _, secs = mc_labels(param_sets, paths, lms, Ts)
    return y.reshape(len(param_sets), -1), secs


POLICIES = ("bucket", "grid")
JUDGE_SECOND_BLOCK = 1 << 31  # Sobol skip of the judge's second, independent block


def choose_fallback(jerr, tol=TOL, policy="grid", margin=1.0, n_T=None):
    """Buckets (columns of jerr [judged sets][buckets], the surrogate's judged cell
    errors, maturity-major with n_T maturities) that MC takes over; see judge().
    policy "bucket": every bucket whose 90th-percentile error exceeds tol.
    policy "grid": the grid as a whole meets the target. It is cost-aware: an MC fallback
    book runs to its longest maturity, so it looks for the shortest maturity horizon within
    which taking over the worst buckets (worst first, a taken-over bucket counting at tol / 2,
    the plain MC's accuracy) brings the grid's 90th percentile to margin * tol."""
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


def noise_corrected(r, noise):
    """Judged cell errors with the judge's own noise taken out: the 90th percentile of |e|
    (e the surrogate's error) is estimated by quantile subtraction in quadrature,
    p90(|e|)^2 = p90(|r|)^2 - p90(|n|)^2 (r = e + the judge's noise, n a sample of that
    noise), which makes no assumption on the shape of e's distribution; the cells' errors are
    then scaled by p90(|e|) / p90(|r|), keeping their ranking. Returns (scaled errors,
    estimated p90, p90 of |r|, p90 of |n|)."""
    r, noise = np.abs(np.asarray(r, dtype=np.float64)), np.abs(np.asarray(noise, dtype=np.float64))
    qr, qn = float(np.quantile(r, 0.9)), float(np.quantile(noise, 0.9))
    est = math.sqrt(max(qr * qr - qn * qn, 0.0))
    k = est / qr if qr > 0 else 1.0
    return r * k, est, qr, qn


def judge(model, param_sets, judge_frac=0.01, judge_paths=1 << 19, tol=TOL, seed=0, lms=LATTICE_LM, Ts=LATTICE_T,
          policy="grid", margin=1.0):
    """MC judge with its own noise removed: re-price a random judge_frac of the sets by MC,
    measure the surrogate's error against it, and choose the lattice buckets (maturity,
    log-moneyness) that MC takes over.

    The judged sets are priced twice, on two Sobol blocks of judge_paths / 2 points far
    apart in the sequence (the first points, and points from 2^31 on), whose errors are
    independent; ybar is their mean. (The two halves of one block of judge_paths points
    would not do: their errors partly cancel in the full block, so their difference would
    overstate the error of the mean.) r = (s - ybar) / w is the surrogate's judged cell error
    (w the cell's error floor, max(|ybar|, 1% of spot)), and n = (y1 - y2) / (2 w) has the
    distribution of the judge's own error in r. noise_corrected() takes that error out, so
    the judge can run at the plain-MC path count (1% of the sets costs about 1% of plain MC)
    without its noise flagging healthy buckets; choose_fallback() then picks the buckets."""
    rng = np.random.default_rng(seed)
    n_judge = max(1, int(round(judge_frac * len(param_sets))))
    judged = np.sort(rng.choice(len(param_sets), size=n_judge, replace=False))
    sets = param_sets[judged]
    half = max(1, judge_paths // 2)
    t0 = time.perf_counter()
    _, y1, _, _ = mc_labels(sets, half, lms, Ts)
    _, y2, _, _ = mc_labels(sets, half, lms, Ts, skip=JUDGE_SECOND_BLOCK)
    pj, _ = model.price_lattice(sets, lms, Ts)
    t_judge = time.perf_counter() - t0
    ybar = 0.5 * (y1 + y2)
    w = np.maximum(np.abs(ybar), FLOOR)
    r = ((pj - ybar) / w).reshape(n_judge, -1)
    noise = (0.5 * (y1 - y2) / w).reshape(n_judge, -1)
    jerr, est, qr, qn = noise_corrected(r, noise)
    bad = choose_fallback(jerr, tol, policy, margin, n_T=len(Ts))
    return dict(judged=judged, bad=bad.reshape(len(Ts), len(lms)), judge_s=t_judge,
                judge_mc_seconds_per_set=t_judge / n_judge, judged_p90=qr, estimated_p90=est, judge_noise_p90=qn)


def price_grid(model, param_sets, mc_paths, judge_frac=0.01, judge_paths=None, seed=0, tol=TOL, lms=LATTICE_LM,
               Ts=LATTICE_T, policy="grid"):
    """Price a grid of (parameter set x lattice) cells with the surrogate, judged by MC.

    1. inference for every cell on the device (price_lattice: features, clipping and the
       price scale on the GPU; sets outside the training box are re-priced by MC);
    2. the MC judge (see judge(), at judge_paths, by default the plain-MC count mc_paths)
       marks the lattice buckets MC takes over;
    3. those buckets of every set are re-priced by MC with mc_paths (the plain-MC path
       count for the same accuracy), on books cut to the failing maturities and strikes.
    Every stage runs on every set it concerns and is timed as run.
    Returns (prices [cells], info dict with timings and counts)."""
    n_sets = len(param_sets)
    ncell = len(lms) * len(Ts)
    judge_paths = judge_paths or mc_paths
    t0 = time.perf_counter()
    price, dev_ms = model.price_lattice(param_sets, lms, Ts)
    price = price.astype(np.float64)
    inside = np.all((param_sets >= BOX_LO[2:] - 1e-12) & (param_sets <= BOX_HI[2:] + 1e-12), axis=1)
    t_inf = time.perf_counter() - t0
    J = judge(model, param_sets, judge_frac, judge_paths, tol, seed, lms, Ts, policy=policy)
    bad2 = J["bad"]
    t2 = time.perf_counter()
    fb_T = np.nonzero(bad2.any(axis=1))[0]
    fb_lm = np.nonzero(bad2.any(axis=0))[0]
    in_sets = np.nonzero(inside)[0]
    n_fb = 0
    if len(fb_T) and len(in_sets):
        fy, _ = _mc_subset(param_sets[in_sets], mc_paths, lms[fb_lm], Ts[fb_T])
        fy = fy.reshape(len(in_sets), len(fb_T), len(fb_lm))
        for a, ti in enumerate(fb_T):
            for b, li in enumerate(fb_lm):
                if bad2[ti, li]:
                    price[in_sets * ncell + ti * len(lms) + li] = fy[:, a, b]
                    n_fb += len(in_sets)
    out_sets = np.nonzero(~inside)[0]
    if len(out_sets):
        oy, _ = _mc_subset(param_sets[out_sets], mc_paths, lms, Ts)
        for j, k in enumerate(out_sets):
            price[k * ncell:(k + 1) * ncell] = oy[j]
            n_fb += ncell
    t_fb = time.perf_counter() - t2
    total = t_inf + J["judge_s"] + t_fb
    cells = n_sets * ncell
    return price, dict(cells=cells, seconds=total, inference_s=t_inf, inference_device_ms=dev_ms,
                       judge_s=J["judge_s"], judge_sets=len(J["judged"]), judge_paths=judge_paths,
                       fallback_s=t_fb, fallback_cells=n_fb, failing_buckets=int(bad2.sum()),
                       out_of_box_sets=int(len(out_sets)), mc_paths=mc_paths, cells_per_sec=cells / total,
                       policy=policy, judged_p90=J["judged_p90"], estimated_p90=J["estimated_p90"],
                       judge_noise_p90=J["judge_noise_p90"])


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
