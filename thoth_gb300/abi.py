"""ctypes mirror of include/thoth_gpu.h and a builder for book descriptors.

The structs below must stay field-for-field identical to the C header;
tests/test_host_logic.py compiles a C probe of the header and compares sizes
and offsets.
"""
import ctypes as C

import numpy as np

THOTH_GPU_OK = 0
THOTH_GPU_E_INVALID = -1
THOTH_GPU_E_NODEVICE = -2
THOTH_GPU_E_CUDA = -3
THOTH_GPU_E_UNSUPPORTED = -4
THOTH_GPU_E_CANCELLED = -5
THOTH_GPU_E_NOMEM = -6
THOTH_GPU_E_TOO_LARGE = -7

MODEL_GBM, MODEL_HESTON, MODEL_LSV = 0, 1, 2
VANILLA, BARRIER, VARIANCE, BASKET = 0, 1, 2, 3
CALL, PUT = 0, 1
GREEK_DELTA, GREEK_VEGA = 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


class ThothAsset(C.Structure):
    _fields_ = [
        ("model", C.c_int32),
        ("lev_points", C.c_int32),
        ("spot", C.c_double),
        ("carry", _dp),
        ("vol", C.c_double),
        ("v0", C.c_double),
        ("kappa", C.c_double),
        ("theta", C.c_double),
        ("xi", C.c_double),
        ("rho", C.c_double),
        ("lev_ln_step", _dp),
        ("lev_offset", _i64p),
        ("lev_values", _dp),
    ]


class ThothProduct(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("option_type", C.c_int32),
        ("asset", C.c_int32),
        ("maturity", C.c_int32),
        ("strike", C.c_double),
        ("zero_rate", C.c_double),
        ("fx", C.c_double),
        ("quanto", C.c_double),
        ("barrier_up", C.c_int32),
        ("barrier_in", C.c_int32),
        ("barrier_level", C.c_double),
        ("n_monitor", C.c_int32),
        ("monitor", _ip),
        ("notional", C.c_double),
        ("strike_variance", C.c_double),
        ("total_year_fraction", C.c_double),
        ("past_variance", C.c_double),
        ("n_obs", C.c_int32),
        ("obs", _ip),
        ("n_components", C.c_int32),
        ("components", _ip),
        ("weights", _dp),
    ]


class ThothBookDesc(C.Structure):
    _fields_ = [
        ("n_dates", C.c_int32),
        ("days", _ip),
        ("t", _dp),
        ("n_assets", C.c_int32),
        ("assets", C.POINTER(ThothAsset)),
        ("cholesky", _dp),
        ("n_products", C.c_int32),
        ("products", C.POINTER(ThothProduct)),
        ("paths", C.c_int64),
        ("sobol_skip", C.c_int64),
        ("use_sobol", C.c_int32),
        ("greeks", C.c_int32),
        ("seed", C.c_uint64), ("correlate_all_spots", C.c_int32),
    ]


class ThothBookResult(C.Structure):
    _fields_ = [
        ("book_premium", C.c_double),
        ("book_trust", C.c_double),
        ("premium", _dp),
        ("trust", _dp),
        ("delta", _dp),
        ("delta_trust", _dp),
        ("vega", _dp),
        ("vega_trust", _dp),
        ("device_ms", C.c_double),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
    ]


class ThothGbmResult(C.Structure):
    _fields_ = [("premium", C.c_double), ("trust", C.c_double)]


class ThothTuneResult(C.Structure):
    _fields_ = [("grid", C.c_int32), ("default_grid", C.c_int32), ("candidates", C.c_int32),
                ("streams", C.c_int32), ("policy", C.c_int32), ("shape", C.c_int32), ("threads", C.c_int32),
                ("tile_paths", C.c_int32), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("persistent", C.c_int32)]


BUMP_DELTA, BUMP_GAMMA, BUMP_VEGA, BUMP_RHO, BUMP_THETA, BUMP_PARAMS = 1, 2, 4, 8, 16, 32
BUMP_ALL = 63
PARAMS = ("v0", "kappa", "theta", "xi", "rho")


class ThothBumpGreeks(C.Structure):
    _fields_ = [("flags", C.c_int32), ("n_scenarios", C.c_int32)] + \
               [(k, C.POINTER(C.c_double)) for k in ("premium", "delta", "gamma", "vega", "rho", "theta",
                                                     "vega_param")] + \
               [(k, C.c_double) for k in ("book_premium", "book_delta", "book_gamma", "book_vega", "book_rho",
                                          "book_theta")] + \
               [("book_vega_param", C.c_double * 5), ("device_ms", C.c_double)]


class ThothAmerican(C.Structure):
    _fields_ = [("product", C.c_int32), ("flags", C.c_int32), ("min_itm", C.c_int32), ("fitted_dates", C.c_int32),
                ("zero_rates", C.POINTER(C.c_double)), ("beta", C.POINTER(C.c_double))] + \
               [(k, C.c_double) for k in ("premium", "trust", "european", "delta", "gamma", "vega", "rho", "theta",
                                          "device_ms", "exercise_ms")]


class ThothLeverageCalib(C.Structure):
    _fields_ = [("n_dates", C.c_int32), ("points", C.c_int32), ("days", C.POINTER(C.c_int32)),
                ("carry", C.POINTER(C.c_double)), ("spot", C.c_double), ("v0", C.c_double), ("kappa", C.c_double),
                ("theta", C.c_double), ("xi", C.c_double), ("rho", C.c_double),
                ("ln_step", C.POINTER(C.c_double)), ("offset", C.POINTER(C.c_int64)),
                ("local_vol", C.POINTER(C.c_double)), ("particles", C.c_int32), ("bins", C.c_int32),
                ("min_bin_count", C.c_int32), ("_pad", C.c_int32), ("seed", C.c_uint64),
                ("min_cond_variance", C.c_double), ("lev_min", C.c_double), ("lev_max", C.c_double),
                ("leverage", C.POINTER(C.c_double)), ("device_ms", C.c_double)]


LSV_CALIB_SEED = 20260708  # the reference's fixed calibration seed (single.cpp:246)


class LeverageCalibration:
    """Inputs of one leverage calibration (numpy buffers kept alive) and its C view.

    days: calendar days from today (days[0] = 0); carry: net carry r - q - repo to each
    date; ln_step / offset / local_vol: each layer's log-spot grid and the target local
    vol at its points ([n_dates][points])."""

    def __init__(self, days, carry, spot, heston, ln_step, offset, local_vol, particles=0, bins=0,
                 min_bin_count=0, seed=LSV_CALIB_SEED):
        self.days = np.ascontiguousarray(days, dtype=np.int32)
        n = len(self.days)
        self.carry = np.ascontiguousarray(np.broadcast_to(carry, (n,)), dtype=np.float64)
        self.ln_step = np.ascontiguousarray(ln_step, dtype=np.float64)
        self.offset = np.ascontiguousarray(offset, dtype=np.int64)
        self.local_vol = np.ascontiguousarray(local_vol, dtype=np.float64)
        assert self.local_vol.ndim == 2 and self.local_vol.shape[0] == n
        self.spot = float(spot)
        self.heston = dict(heston)
        self.particles, self.bins, self.min_bin_count, self.seed = particles, bins, min_bin_count, seed
        self.leverage = np.zeros_like(self.local_vol)

    def desc(self):
        d = ThothLeverageCalib()
        d.n_dates = len(self.days)
        d.points = self.local_vol.shape[1]
        d.days = _ptr(self.days, C.c_int32)
        d.carry = _ptr(self.carry, C.c_double)
        d.spot = self.spot
        for k in ("v0", "kappa", "theta", "xi", "rho"):
            setattr(d, k, float(self.heston[k]))
        d.ln_step = _ptr(self.ln_step, C.c_double)
        d.offset = _ptr(self.offset, C.c_int64)
        d.local_vol = _ptr(self.local_vol, C.c_double)
        d.particles, d.bins, d.min_bin_count = int(self.particles), int(self.bins), int(self.min_bin_count)
        d.seed = int(self.seed)
        d.leverage = _ptr(self.leverage, C.c_double)
        return d


def _ptr(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


class Book:
    """Owns the numpy buffers behind one ThothBookDesc (keeps them alive).

    Assets and products are plain dicts; ``desc()`` materialises the C view.
    Dates are calendar days from today (ACT/365) unless ``times`` is given.
    """

    def __init__(self, days=None, times=None, paths=1 << 14, sobol_skip=0, use_sobol=True, seed=0, greeks=0):
        if days is not None:
            self.days = np.ascontiguousarray(days, dtype=np.int32)
            self.t = (self.days - self.days[0]).astype(np.float64) / 365.0
        else:
            self.days = None
            self.t = np.ascontiguousarray(times, dtype=np.float64)
        self.n_dates = len(self.t)
        self.assets = []
        self.products = []
        self.cholesky = None
        # True: the Cholesky factor also drives Heston / LSV spot noises (an extension; the
        # reference correlates only GBM spots)
        self.correlate_all_spots = False
        self.paths = int(paths)
        self.sobol_skip = int(sobol_skip)
        self.use_sobol = bool(use_sobol)
        self.seed = int(seed)
        self.greeks = int(greeks)
        self._keep = []

    # -- assets ---------------------------------------------------------
    def _carry(self, carry):
        if np.isscalar(carry):
            return np.full(self.n_dates, float(carry))
        return np.ascontiguousarray(carry, dtype=np.float64)

    def add_gbm(self, spot, vol, carry):
        self.assets.append(dict(model=MODEL_GBM, spot=spot, vol=vol, carry=self._carry(carry)))
        return len(self.assets) - 1

    def add_heston(self, spot, v0, kappa, theta, xi, rho, carry, leverage=None):
        a = dict(model=MODEL_HESTON, spot=spot, v0=v0, kappa=kappa, theta=theta, xi=xi, rho=rho,
                 carry=self._carry(carry))
        if leverage is not None:
            ln_step, offset, values = leverage
            a["model"] = MODEL_LSV
            a["lev_ln_step"] = np.ascontiguousarray(ln_step, dtype=np.float64)
            a["lev_offset"] = np.ascontiguousarray(offset, dtype=np.int64)
            a["lev_values"] = np.ascontiguousarray(values, dtype=np.float64)
            assert a["lev_values"].shape[0] == self.n_dates
        self.assets.append(a)
        return len(self.assets) - 1

    # -- products -------------------------------------------------------
    def add_vanilla(self, asset, strike, maturity, option_type=CALL, zero_rate=0.0, fx=1.0, quanto=0.0):
        self.products.append(dict(kind=VANILLA, asset=asset, strike=strike, maturity=maturity,
                                  option_type=option_type, zero_rate=zero_rate, fx=fx, quanto=quanto))
        return len(self.products) - 1

    def add_barrier(self, asset, strike, maturity, level, up, knock_in, monitor, option_type=CALL,
                    zero_rate=0.0, fx=1.0, quanto=0.0):
        self.products.append(dict(kind=BARRIER, asset=asset, strike=strike, maturity=maturity,
                                  option_type=option_type, zero_rate=zero_rate, fx=fx, quanto=quanto,
                                  barrier_level=level, barrier_up=int(up), barrier_in=int(knock_in),
                                  monitor=np.ascontiguousarray(monitor, dtype=np.int32)))
        return len(self.products) - 1

    def add_variance(self, asset, maturity, strike_variance, notional=1.0, zero_rate=0.0, fx=1.0,
                     total_year_fraction=0.0, past_variance=0.0, obs=None, quanto=0.0):
        p = dict(kind=VARIANCE, asset=asset, strike=0.0, maturity=maturity, option_type=CALL,
                 zero_rate=zero_rate, fx=fx, quanto=quanto, strike_variance=strike_variance,
                 notional=notional, total_year_fraction=total_year_fraction, past_variance=past_variance)
        if obs is not None:
            p["obs"] = np.ascontiguousarray(obs, dtype=np.int32)
        self.products.append(p)
        return len(self.products) - 1

    def add_basket(self, components, weights, strike, maturity, option_type=CALL, zero_rate=0.0, fx=1.0,
                   quanto=0.0):
        self.products.append(dict(kind=BASKET, asset=-1, strike=strike, maturity=maturity,
                                  option_type=option_type, zero_rate=zero_rate, fx=fx, quanto=quanto,
                                  components=np.ascontiguousarray(components, dtype=np.int32),
                                  weights=np.ascontiguousarray(weights, dtype=np.float64)))
        return len(self.products) - 1

    def set_cholesky(self, L):
        self.cholesky = np.ascontiguousarray(L, dtype=np.float64)

    def copy(self):
        """An independent copy (assets, products and arrays) without the C view."""
        import copy as _copy
        keep, self._keep = self._keep, []
        try:
            return _copy.deepcopy(self)
        finally:
            self._keep = keep

    # -- C view ---------------------------------------------------------
    def desc(self):
        keep = []
        na, npr = len(self.assets), len(self.products)
        A = (ThothAsset * max(na, 1))()
        for i, a in enumerate(self.assets):
            A[i].model = a["model"]
            A[i].spot = a["spot"]
            A[i].carry = _ptr(a["carry"], C.c_double)
            A[i].vol = a.get("vol", 0.0)
            for k in ("v0", "kappa", "theta", "xi", "rho"):
                setattr(A[i], k, a.get(k, 0.0))
            if a["model"] == MODEL_LSV:
                A[i].lev_points = a["lev_values"].shape[1]
                A[i].lev_ln_step = _ptr(a["lev_ln_step"], C.c_double)
                A[i].lev_offset = _ptr(a["lev_offset"], C.c_int64)
                A[i].lev_values = _ptr(a["lev_values"], C.c_double)
        P = (ThothProduct * max(npr, 1))()
        for i, p in enumerate(self.products):
            P[i].kind = p["kind"]
            P[i].option_type = p["option_type"]
            P[i].asset = p["asset"]
            P[i].maturity = p["maturity"]
            P[i].strike = p["strike"]
            P[i].zero_rate = p["zero_rate"]
            P[i].fx = p["fx"]
            P[i].quanto = p["quanto"]
            if p["kind"] == BARRIER:
                P[i].barrier_up = p["barrier_up"]
                P[i].barrier_in = p["barrier_in"]
                P[i].barrier_level = p["barrier_level"]
                P[i].n_monitor = len(p["monitor"])
                P[i].monitor = _ptr(p["monitor"], C.c_int32)
            if p["kind"] == VARIANCE:
                P[i].notional = p["notional"]
                P[i].strike_variance = p["strike_variance"]
                P[i].total_year_fraction = p["total_year_fraction"]
                P[i].past_variance = p["past_variance"]
                if "obs" in p:
                    P[i].n_obs = len(p["obs"])
                    P[i].obs = _ptr(p["obs"], C.c_int32)
            if p["kind"] == BASKET:
                P[i].n_components = len(p["components"])
                P[i].components = _ptr(p["components"], C.c_int32)
                P[i].weights = _ptr(p["weights"], C.c_double)
        d = ThothBookDesc()
        d.n_dates = self.n_dates
        d.days = _ptr(self.days, C.c_int32) if self.days is not None else None
        d.t = _ptr(self.t, C.c_double)
        d.n_assets = na
        d.assets = A
        d.cholesky = _ptr(self.cholesky, C.c_double) if self.cholesky is not None else None
        d.n_products = npr
        d.products = P
        d.paths = self.paths
        d.sobol_skip = self.sobol_skip
        d.use_sobol = int(self.use_sobol)
        d.greeks = self.greeks
        d.seed = self.seed
        d.correlate_all_spots = int(bool(self.correlate_all_spots))
        keep += [A, P]
        self._keep = keep
        return d

    def result(self, greeks=False):
        """Allocate a ThothBookResult with numpy-backed arrays; returns (res, arrays)."""
        n = len(self.products)
        arrs = {k: np.zeros(n) for k in ("premium", "trust", "delta", "delta_trust", "vega", "vega_trust")}
        r = ThothBookResult()
        r.premium = _ptr(arrs["premium"], C.c_double)
        r.trust = _ptr(arrs["trust"], C.c_double)
        if greeks:
            for k in ("delta", "delta_trust", "vega", "vega_trust"):
                setattr(r, k, _ptr(arrs[k], C.c_double))
        return r, arrs
