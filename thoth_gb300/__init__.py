"""thoth_gb300 — GB300 (sm_103a) Monte-Carlo engine behind Thoth's !mcl_pricer.

Python mirror of the reference's GPU interface (pricer/src/tasks/mcl_gpu.hpp:16-48:
``Available``, ``DeviceInfo``, ``PriceEuropeanGbm``) plus the whole-book entry
point, all calling the C ABI of ``libthoth_gpu.so`` (include/thoth_gpu.h).
There is no CPU fallback: without the built library every call raises.
"""
import ctypes as C
import os
import pathlib

import numpy as np

from . import abi
from .abi import Book  # noqa: F401

HERE = pathlib.Path(__file__).resolve().parent
# THOTH_GPU_LIB selects another build of the same library (the sanitized host build)
LIB_PATH = pathlib.Path(os.environ.get("THOTH_GPU_LIB") or HERE / "_build" / "libthoth_gpu.so")

_lib = None


class ThothGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("thoth_gpu error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libthoth_gpu.so (built by thoth_gb300.build); raise if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ThothGpuError(abi.THOTH_GPU_E_NODEVICE,
                                "%s is not built: run `python -m thoth_gb300.build`" % LIB_PATH)
        L = C.CDLL(str(LIB_PATH))
        L.thoth_gpu_available.restype = C.c_int
        L.thoth_gpu_device_info.argtypes = [C.c_char_p, C.c_size_t]
        L.thoth_gpu_price_european_gbm.argtypes = [C.c_double] * 5 + [C.c_int, C.c_int64, C.c_uint64,
                                                                       C.POINTER(abi.ThothGbmResult)]
        L.thoth_gpu_price_book.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBookResult)]
        L.thoth_gpu_price_batch.argtypes = [C.POINTER(abi.ThothBookDesc), C.c_int32, C.POINTER(abi.ThothBookResult)]
        L.thoth_gpu_sobol_points.argtypes = [C.c_int32, C.c_int64, C.c_int64, C.POINTER(C.c_uint32)]
        L.thoth_gpu_bridge_increments.argtypes = [C.POINTER(C.c_double), C.c_int32, C.c_int32, C.c_int64, C.c_int64,
                                                  C.POINTER(C.c_float)]
        L.thoth_gpu_normal_quantiles.argtypes = [C.POINTER(C.c_uint32), C.c_int64, C.POINTER(C.c_float)]
        L.thoth_gpu_bridge_program.argtypes = [C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32),
                                               C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.thoth_gpu_plan_summary.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(C.c_int64)]
        L.thoth_gpu_last_error.restype = C.c_char_p
        L.thoth_gpu_book_create.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(C.c_void_p)]
        L.thoth_gpu_book_run.argtypes = [C.c_void_p, C.POINTER(abi.ThothBookResult)]
        L.thoth_gpu_book_destroy.argtypes = [C.c_void_p]
        L.thoth_gpu_measure_fp32_peak.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.thoth_gpu_measure_mufu_peak.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.thoth_gpu_debug_fail_allocations.argtypes = [C.c_int32]
        L.thoth_gpu_batch_streams.argtypes = [C.c_int32]
        L.thoth_gpu_batch_persistent.argtypes = [C.c_int32]
        L.thoth_gpu_batch_launches.argtypes = []
        L.thoth_gpu_bump_greeks.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBumpGreeks)]
        L.thoth_gpu_bump_greeks_last_error.restype = C.c_char_p
        L.thoth_gpu_calibrate_leverage.argtypes = [C.POINTER(abi.ThothLeverageCalib)]
        L.thoth_gpu_xoshiro_jump.argtypes = [C.POINTER(C.c_uint64), C.c_uint64, C.POINTER(C.c_uint64)]
        L.thoth_gpu_price_american.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothAmerican)]
        L.thoth_gpu_price_american_book.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothAmerican),
                                                    C.c_int32]
        L.thoth_gpu_american_last_error.restype = C.c_char_p
        L.thoth_gpu_simulate_paths.argtypes = [C.POINTER(abi.ThothBookDesc), C.c_int32, C.POINTER(C.c_float),
                                               C.POINTER(C.c_double)]
        L.thoth_gpu_autotune_book.argtypes = [C.POINTER(abi.ThothBookDesc), C.c_int32, C.POINTER(abi.ThothTuneResult)]
        L.thoth_gpu_autotune_batch.argtypes = [C.POINTER(abi.ThothBookDesc), C.c_int32, C.c_int32,
                                               C.POINTER(abi.ThothTuneResult)]
        L.thoth_gpu_autotune_save.argtypes = [C.c_char_p]
        L.thoth_gpu_autotune_load.argtypes = [C.c_char_p]
        L.thoth_gpu_tc_gemm_test.argtypes = [C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), C.c_int32, C.c_int32,
                                             C.POINTER(C.c_float)]
        _lib = L
    return _lib


def _check(rc):
    if rc != abi.THOTH_GPU_OK:
        raise ThothGpuError(rc, lib().thoth_gpu_last_error().decode())


def available():
    """Reference gpu::Available()."""
    return bool(lib().thoth_gpu_available())


def device_info():
    """Reference gpu::DeviceInfo()."""
    buf = C.create_string_buffer(256)
    _check(lib().thoth_gpu_device_info(buf, 256))
    return buf.value.decode()


def price_european_gbm(forward, strike, t, vol, df, is_call, paths, seed=0):
    """Reference gpu::PriceEuropeanGbm -> (premium, trust)."""
    r = abi.ThothGbmResult()
    _check(lib().thoth_gpu_price_european_gbm(forward, strike, t, vol, df, int(bool(is_call)), int(paths), int(seed),
                                              C.byref(r)))
    return r.premium, r.trust


def price_book(book, greeks=False):
    """Price every product of ``book`` (an abi.Book) in one sweep on the GPU."""
    d = book.desc()
    r, arrs = book.result(greeks=greeks)
    _check(lib().thoth_gpu_price_book(C.byref(d), C.byref(r)))
    out = dict(book_premium=r.book_premium, book_trust=r.book_trust, device_ms=r.device_ms,
               h2d_bytes=r.h2d_bytes, d2h_bytes=r.d2h_bytes)
    out.update({k: v.copy() for k, v in arrs.items()})
    return out


def simulate_paths(book, asset=0):
    """Spot of `asset` at every date of every path of `book`: (float32 [n_dates][paths], device ms)."""
    d = book.desc()
    out = np.zeros((d.n_dates, book.paths), dtype=np.float32)
    ms = C.c_double()
    _check(lib().thoth_gpu_simulate_paths(C.byref(d), int(asset), out.ctypes.data_as(C.POINTER(C.c_float)),
                                          C.byref(ms)))
    return out, ms.value


def bump_greeks(book, flags=abi.BUMP_ALL):
    """Bump-and-revalue Greeks on common random numbers (the reference's definitions):
    dict of per-product arrays and book values; NaN where not requested or available."""
    n = len(book.products)
    d = book.desc()
    arrs = {k: np.full(n, np.nan) for k in ("premium", "delta", "gamma", "vega", "rho", "theta")}
    vp = np.full((5, n), np.nan)
    g = abi.ThothBumpGreeks()
    g.flags = int(flags)
    for k, a in arrs.items():
        setattr(g, k, a.ctypes.data_as(C.POINTER(C.c_double)))
    g.vega_param = vp.ctypes.data_as(C.POINTER(C.c_double))
    rc = lib().thoth_gpu_bump_greeks(C.byref(d), C.byref(g))
    if rc != abi.THOTH_GPU_OK:
        raise ThothGpuError(rc, lib().thoth_gpu_bump_greeks_last_error().decode())
    out = dict(arrs)
    out.update({"vega_" + p: vp[k].copy() for k, p in enumerate(abi.PARAMS)})
    out["book"] = {k: getattr(g, "book_" + k) for k in ("premium", "delta", "gamma", "vega", "rho", "theta")}
    out["book"].update({"vega_" + p: g.book_vega_param[k] for k, p in enumerate(abi.PARAMS)})
    out["n_scenarios"] = g.n_scenarios
    out["device_ms"] = g.device_ms
    out["note"] = lib().thoth_gpu_bump_greeks_last_error().decode()
    return out


def calibrate_leverage(calib):
    """LSV leverage calibration (abi.LeverageCalibration) on the device: returns the layers
    [n_dates][points] (the lev_values of an LSV asset on the same grids) and device ms."""
    d = calib.desc()
    _check(lib().thoth_gpu_calibrate_leverage(C.byref(d)))
    return calib.leverage.copy(), d.device_ms


def xoshiro_jump(state, n):
    """The reference Rng's state after n draws from `state` (4 x uint64), by jump-ahead."""
    s = (C.c_uint64 * 4)(*[int(x) for x in state])
    out = (C.c_uint64 * 4)()
    _check(lib().thoth_gpu_xoshiro_jump(s, int(n), out))
    return [int(x) for x in out]


def price_american(book, product, flags=0, min_itm=0, zero_rates=None):
    """American exercise of one vanilla of the book by Longstaff-Schwartz on its asset's
    stored paths, with frozen-policy Greeks (flags: abi.BUMP_DELTA | ... | BUMP_THETA).
    Returns premium, trust, european, the Greeks (NaN where not requested), beta
    [n_dates, 3] (NaN where a date has no regression), fitted_dates and the device times."""
    return price_american_book(book, [product], flags, min_itm, zero_rates)[0]


def price_american_book(book, products, flags=0, min_itm=0, zero_rates=None):
    """Every listed American vanilla of the book in one call (one simulation per asset and
    scenario): a list of dicts as price_american returns. zero_rates: one array for every
    contract, or a list with one per contract (None: the product's zero_rate)."""
    d = book.desc()
    n = len(products)
    arr = (abi.ThothAmerican * max(n, 1))()
    keep = []
    for i, pr in enumerate(products):
        a = arr[i]
        a.product = int(pr)
        a.flags = int(flags)
        a.min_itm = int(min_itm)
        zr = zero_rates[i] if isinstance(zero_rates, (list, tuple)) else zero_rates
        if zr is not None:
            z = np.ascontiguousarray(zr, dtype=np.float64)
            if z.shape != (book.n_dates,):
                raise ValueError("zero_rates needs one rate per date")
            a.zero_rates = z.ctypes.data_as(C.POINTER(C.c_double))
            keep.append(z)
        beta = np.full((book.n_dates, 3), np.nan)
        a.beta = beta.ctypes.data_as(C.POINTER(C.c_double))
        keep.append(beta)
    rc = lib().thoth_gpu_price_american_book(C.byref(d), arr, n)
    if rc != abi.THOTH_GPU_OK:
        raise ThothGpuError(rc, lib().thoth_gpu_american_last_error().decode())
    note = lib().thoth_gpu_american_last_error().decode()
    out = []
    for i in range(n):
        a = arr[i]
        r = {k: getattr(a, k) for k in ("premium", "trust", "european", "delta", "gamma", "vega", "rho", "theta",
                                         "device_ms", "exercise_ms", "fitted_dates")}
        r["beta"] = np.ctypeslib.as_array(a.beta, shape=(book.n_dates, 3)).copy()
        r["note"] = note
        out.append(r)
    return out


def price_batch(books):
    """Price independent books in one CUDA-graph launch; returns one result dict per book."""
    n = len(books)
    descs = (abi.ThothBookDesc * max(n, 1))()
    results = (abi.ThothBookResult * max(n, 1))()
    keep = []
    for i, b in enumerate(books):
        descs[i] = b.desc()
        r, arrs = b.result()
        results[i] = r
        keep.append((b, arrs))
    _check(lib().thoth_gpu_price_batch(descs, n, results))
    out = []
    for i, (b, arrs) in enumerate(keep):
        r = results[i]
        d = dict(book_premium=r.book_premium, book_trust=r.book_trust, device_ms=r.device_ms,
                 h2d_bytes=r.h2d_bytes, d2h_bytes=r.d2h_bytes)
        d.update({k: v.copy() for k, v in arrs.items()})
        out.append(d)
    return out


def batch_graph_replays():
    """Replays of the cached batch graph since its capture."""
    return lib().thoth_gpu_batch_graph_replays()


def set_batch_streams(n):
    _check(lib().thoth_gpu_batch_streams(int(n)))


def set_batch_persistent(on):
    """True (default): a batch's single-asset books in one persistent launch; False: one launch per book."""
    _check(lib().thoth_gpu_batch_persistent(1 if on else 0))


def batch_launches():
    """Kernel launches recorded into the cached batch graph."""
    return lib().thoth_gpu_batch_launches()


def _tune_dict(r):
    return dict(grid=r.grid, default_grid=r.default_grid, candidates=r.candidates, streams=r.streams,
                policy=r.policy, shape=r.shape, threads=r.threads, tile_paths=r.tile_paths, best_ms=r.best_ms,
                default_ms=r.default_ms, persistent=r.persistent)


def autotune_book(book, reps=3):
    """Time the candidate persistent grids for this book's shape; later calls use the fastest."""
    d = book.desc()
    r = abi.ThothTuneResult()
    _check(lib().thoth_gpu_autotune_book(C.byref(d), int(reps), C.byref(r)))
    return _tune_dict(r)


def autotune_batch(books, reps=1):
    """Time the persistent launch and the per-book launches (stream counts, shapes, grid policies)
    of the batch graph; later batches use the fastest."""
    n = len(books)
    descs = (abi.ThothBookDesc * max(n, 1))()
    keep = []
    for i, b in enumerate(books):
        descs[i] = b.desc()
        keep.append(b)
    r = abi.ThothTuneResult()
    _check(lib().thoth_gpu_autotune_batch(descs, n, int(reps), C.byref(r)))
    return _tune_dict(r)


def autotune_save(path):
    _check(lib().thoth_gpu_autotune_save(str(path).encode()))


def autotune_load(path):
    _check(lib().thoth_gpu_autotune_load(str(path).encode()))


def autotune_clear():
    _check(lib().thoth_gpu_autotune_clear())


class ResidentBook:
    """A book whose plan stays on the device (thoth_gpu_book_create / _run / _destroy)."""

    def __init__(self, book, greeks=False):
        self.book = book
        self.greeks = greeks
        self._d = book.desc()
        self.h = C.c_void_p()
        _check(lib().thoth_gpu_book_create(C.byref(self._d), C.byref(self.h)))

    def run(self):
        r, arrs = self.book.result(greeks=self.greeks)
        _check(lib().thoth_gpu_book_run(self.h, C.byref(r)))
        out = dict(book_premium=r.book_premium, book_trust=r.book_trust, device_ms=r.device_ms,
                   h2d_bytes=r.h2d_bytes, d2h_bytes=r.d2h_bytes)
        out.update({k: v.copy() for k, v in arrs.items()})
        return out

    def close(self):
        if self.h:
            lib().thoth_gpu_book_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_fp32_peak():
    """FP32 FMA throughput of the device, TFLOP/s (2 flops per FMA)."""
    tf, ms = C.c_double(), C.c_double()
    _check(lib().thoth_gpu_measure_fp32_peak(C.byref(tf), C.byref(ms)))
    return tf.value


def debug_fail_allocations(n):
    """Test hook: drop the engine's working buffers and make the next n allocations of
    them fail as on a full device (THOTH_GPU_E_NOMEM); n = 0 clears it."""
    _check(lib().thoth_gpu_debug_fail_allocations(int(n)))


def measure_mufu_peak():
    """Special-function-unit throughput of the device (reciprocal square roots), Gop/s."""
    g, ms = C.c_double(), C.c_double()
    _check(lib().thoth_gpu_measure_mufu_peak(C.byref(g), C.byref(ms)))
    return g.value


def to_bf16_bits(x):
    """float32 array -> bf16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32)


def tc_gemm_test(a, b):
    """D = A (128 x K) @ B (N x K)^T on the tensor cores (inputs rounded to bf16)."""
    a16, b16 = to_bf16_bits(a), to_bf16_bits(b)
    n, k = b16.shape
    d = np.zeros((128, n), dtype=np.float32)
    _check(lib().thoth_gpu_tc_gemm_test(a16.ctypes.data_as(C.POINTER(C.c_uint16)),
                                        b16.ctypes.data_as(C.POINTER(C.c_uint16)), n, k,
                                        d.ctypes.data_as(C.POINTER(C.c_float))))
    return d


def sobol_points(dims, skip, n):
    out = np.zeros((n, dims), dtype=np.uint32)
    _check(lib().thoth_gpu_sobol_points(dims, skip, n, out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out


def normal_quantiles(x):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros(x.shape, dtype=np.float32)
    _check(lib().thoth_gpu_normal_quantiles(x.ctypes.data_as(C.POINTER(C.c_uint32)), x.size,
                                            out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def bridge_increments(t, factors, skip, n_paths):
    t = np.ascontiguousarray(t, dtype=np.float64)
    N = len(t) - 1
    out = np.zeros((n_paths, factors, N), dtype=np.float32)
    _check(lib().thoth_gpu_bridge_increments(t.ctypes.data_as(C.POINTER(C.c_double)), len(t), factors, skip, n_paths,
                                             out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def bridge_program(t):
    """Host-only: the time-ordered bridge program (first/count per step, nodes, stack depth)."""
    t = np.ascontiguousarray(t, dtype=np.float64)
    m = len(t) - 1
    fc = np.zeros(2 * m, dtype=np.int32)
    nodes = np.zeros(4 * m, dtype=np.float64)
    nn, depth = C.c_int32(), C.c_int32()
    _check(lib().thoth_gpu_bridge_program(t.ctypes.data_as(C.POINTER(C.c_double)), len(t),
                                          fc.ctypes.data_as(C.POINTER(C.c_int32)),
                                          nodes.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nn), C.byref(depth)))
    return fc.reshape(m, 2), nodes[:4 * nn.value].reshape(nn.value, 4), depth.value


def plan_summary(book):
    """Host-only: validate a book and return its launch plan as a dict."""
    d = book.desc()
    out = np.zeros(11, dtype=np.int64)
    _check(lib().thoth_gpu_plan_summary(C.byref(d), out.ctypes.data_as(C.POINTER(C.c_int64))))
    keys = ("variant", "tile", "smem", "slots", "groups", "stack_depth", "sobol_dims", "tiles", "shape", "threads",
            "few_moments")
    return dict(zip(keys, (int(v) for v in out)))
