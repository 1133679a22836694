"""TEST INFRASTRUCTURE: Python handles on the parity oracles.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package. It loads
  * oracle/_build/liboracle_port.so  — the C restatement (thoth_oracle.c),
  * oracle/_ref/libref_oracle.so     — the reference's own node graph
    (present only where the reference checkout was available to build it).
"""
import ctypes as C
import os
import pathlib
import shutil
import subprocess

import numpy as np

from thoth_gb300 import abi

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
JK_TABLE = ROOT / "thoth_gb300" / "data" / "joe_kuo_6_21201.bin"
PORT_SO = HERE / "_build" / "liboracle_port.so"
REF_SO = HERE / "_ref" / "libref_oracle.so"
REF_GPU_SRC = HERE / "_ref" / "gpu" / "mcl_gpu.cu"
REF_GBM_SO = HERE / "_ref" / "libref_gbm.so"

_port = None
_ref = None


def reference_root(ref=None):
    """The reference checkout (GValas/Thoth): `ref`, else $THOTH_REFERENCE, else a
    directory named `reference` beside this repository. None where none of them holds
    the pricer's sources."""
    for cand in (ref, os.environ.get("THOTH_REFERENCE"), ROOT.parent / "reference"):
        if cand and (pathlib.Path(cand) / "pricer" / "src").is_dir():
            return pathlib.Path(cand)
    return None


def build(ref=None):
    """Compile the port (and the reference build when its sources exist)."""
    targets = ["port"]
    refroot = reference_root(ref)
    if refroot is not None:
        targets += ["ref", "refgpu-src"]
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE)] + (["REF=%s" % refroot] if refroot else []) + targets,
                   check=True)
    # the reference's GPU kernel for the benchmark, where its staged sources and nvcc exist
    if REF_GPU_SRC.exists() and shutil.which("nvcc"):
        subprocess.run(["make", "-s", "-C", str(HERE), "refgpu"], check=True)


_ref_gbm = None


def ref_gbm():
    """The reference's own GPU kernel (gbm_kernel and gpu::PriceEuropeanGbm of
    pricer/src/tasks/mcl_gpu.cu) with its timing harness, oracle/_ref/libref_gbm.so; None
    where it was not built (no staged sources or no nvcc). Benchmark use only."""
    global _ref_gbm
    if _ref_gbm is None and REF_GBM_SO.exists():
        lib = C.CDLL(str(REF_GBM_SO))
        args = [C.c_double] * 5 + [C.c_int, C.c_long, C.c_ulong]
        lib.ref_gbm_call.argtypes = args + [C.POINTER(C.c_double)] * 3
        lib.ref_gbm_kernel.argtypes = args + [C.c_int] + [C.POINTER(C.c_double)] * 3
        _ref_gbm = lib
    return _ref_gbm


def port():
    global _port
    if _port is None:
        if not PORT_SO.exists():
            build()
        lib = C.CDLL(str(PORT_SO))
        lib.oracle_load_direction_numbers.argtypes = [C.c_char_p]
        lib.oracle_sobol_points.argtypes = [C.c_int, C.c_int64, C.c_int64, C.POINTER(C.c_uint32)]
        lib.oracle_normal_cdf_inv.argtypes = [C.c_double]
        lib.oracle_normal_cdf_inv.restype = C.c_double
        lib.oracle_normal_cdf_inv_n.argtypes = [C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double)]
        lib.oracle_bridge_increments.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.c_int64,
                                                 C.c_int64, C.c_uint64, C.POINTER(C.c_double)]
        lib.oracle_price_book.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBookResult), C.c_int,
                                          C.POINTER(C.c_double), C.c_int64]
        for f in ("oracle_bs_price",):
            getattr(lib, f).argtypes = [C.c_double] * 5 + [C.c_int]
            getattr(lib, f).restype = C.c_double
        lib.oracle_bs_delta.argtypes = [C.c_double] * 6 + [C.c_int]
        lib.oracle_bs_delta.restype = C.c_double
        lib.oracle_bs_vega.argtypes = [C.c_double] * 6
        lib.oracle_bs_vega.restype = C.c_double
        for f in ("oracle_heston_price", "oracle_heston_price_p12"):
            getattr(lib, f).argtypes = [C.c_double] * 10 + [C.c_int]
            getattr(lib, f).restype = C.c_double
        lib.oracle_heston_prices.argtypes = [C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        lib.oracle_calibrate_leverage.argtypes = [C.POINTER(abi.ThothLeverageCalib)]
        lib.oracle_xoshiro_draws.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, C.POINTER(C.c_uint64),
                                             C.POINTER(C.c_uint64)]
        rc = lib.oracle_load_direction_numbers(str(JK_TABLE).encode())
        if rc != 0:
            raise RuntimeError("cannot load %s (%d)" % (JK_TABLE, rc))
        _port = lib
    return _port


def ref_available():
    return REF_SO.exists()


def ref():
    global _ref
    if _ref is None:
        lib = C.CDLL(str(REF_SO))
        lib.ref_sobol_points.argtypes = [C.c_int, C.c_int64, C.c_int64, C.POINTER(C.c_uint32)]
        lib.ref_normal_cdf_inv.argtypes = [C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double)]
        lib.ref_bridge_increments.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.c_int64, C.c_int64,
                                              C.c_uint64, C.POINTER(C.c_double)]
        lib.ref_price_book.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBookResult),
                                       C.POINTER(C.c_double), C.c_int64]
        lib.ref_rng_draws.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, C.POINTER(C.c_uint64),
                                      C.POINTER(C.c_double)]
        lib.ref_least_squares.argtypes = [C.POINTER(C.c_double), C.c_int64, C.c_int, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
        lib.ref_lsm.argtypes = [C.POINTER(C.c_float), C.c_int64, C.c_int, C.POINTER(C.c_double),
                                C.POINTER(C.c_double), C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                                C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                C.POINTER(C.c_double)]
        _ref = lib
    return _ref


def _u32(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def sobol_points(dims, skip, n, which="port"):
    out = np.zeros((n, dims), dtype=np.uint32)
    lib = port() if which == "port" else ref()
    f = lib.oracle_sobol_points if which == "port" else lib.ref_sobol_points
    d = f(dims, skip, n, _u32(out))
    return out[:, :d]


def normal_cdf_inv(p, which="port"):
    p = np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros_like(p)
    if which == "port":
        port().oracle_normal_cdf_inv_n(_d(p), p.size, _d(out))
    else:
        ref().ref_normal_cdf_inv(_d(p), p.size, _d(out))
    return out


def bridge_increments(t, factors, skip, n_paths, seed=0, which="port"):
    t = np.ascontiguousarray(t, dtype=np.float64)
    N = len(t) - 1
    out = np.zeros((n_paths, factors, N))
    f = port().oracle_bridge_increments if which == "port" else ref().ref_bridge_increments
    f(_d(t), len(t), factors, skip, n_paths, seed, _d(out))
    return out


def price_book(book, which="port", threads=1, n_per_path=0):
    """Returns dict(book_premium, book_trust, premium, trust, per_path)."""
    d = book.desc()
    r, arrs = book.result()
    per = np.zeros((max(n_per_path, 1), len(book.products)))
    if which == "port":
        rc = port().oracle_price_book(C.byref(d), C.byref(r), threads, _d(per) if n_per_path else None, n_per_path)
    else:
        rc = ref().ref_price_book(C.byref(d), C.byref(r), _d(per) if n_per_path else None, n_per_path)
    if rc != 0:
        raise RuntimeError("%s price_book failed: %d" % (which, rc))
    return dict(book_premium=r.book_premium, book_trust=r.book_trust, premium=arrs["premium"].copy(),
                trust=arrs["trust"].copy(), per_path=per[:n_per_path].copy() if n_per_path else None)


def calibrate_leverage(calib):
    """Single::CalibrateLeverage restated (thoth_oracle.c) on abi.LeverageCalibration inputs:
    the layers [n_dates][points]."""
    d = calib.desc()
    out = np.zeros_like(calib.local_vol)
    d.leverage = _d(out)
    if port().oracle_calibrate_leverage(C.byref(d)) != 0:
        raise RuntimeError("oracle calibration failed")
    return out


def xoshiro_draws(seed, skip, n):
    """(n raw draws of the reference Rng after `skip`, the state after them)."""
    out = np.zeros(max(n, 1), dtype=np.uint64)
    st = (C.c_uint64 * 4)()
    port().oracle_xoshiro_draws(seed, skip, n, out.ctypes.data_as(C.POINTER(C.c_uint64)), st)
    return out[:n], [int(x) for x in st]


def ref_rng_draws(seed, skip, n):
    """The reference Rng: (n raw 64-bit draws, n Gaussians) after skipping `skip` draws."""
    raw = np.zeros(n, dtype=np.uint64)
    g = np.zeros(n)
    ref().ref_rng_draws(seed, skip, n, raw.ctypes.data_as(C.POINTER(C.c_uint64)), _d(g))
    return raw, g


def ref_least_squares(X, y):
    """The reference's LeastSquares on X [n][p], y [n]: beta, or None where it fails."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    beta = np.zeros(X.shape[1])
    ok = ref().ref_least_squares(_d(X), X.shape[0], X.shape[1], _d(y), _d(beta))
    return beta if ok else None


def ref_lsm(S, tau, rates, strike, call, norm, min_itm=50, policy=None):
    """The reference's Longstaff-Schwartz loops (sums in path order) on S [M][n] float32:
    fit and value, or value the frozen policy (beta [M][3], has_fit [M])."""
    S = np.ascontiguousarray(S, dtype=np.float32)
    M, n = S.shape
    tau = np.ascontiguousarray(tau[:M], dtype=np.float64)
    rates = np.ascontiguousarray(rates[:M], dtype=np.float64)
    if policy is None:
        beta, has = np.zeros((M, 3)), np.zeros(M, dtype=np.int32)
    else:
        beta = np.ascontiguousarray(policy[0], dtype=np.float64)
        has = np.ascontiguousarray(policy[1], dtype=np.int32)
    prem, trust = C.c_double(), C.c_double()
    ref().ref_lsm(S.ctypes.data_as(C.POINTER(C.c_float)), n, M, _d(tau), _d(rates), strike, int(call), norm,
                  min_itm, int(policy is None), _d(beta), has.ctypes.data_as(C.POINTER(C.c_int)),
                  C.byref(prem), C.byref(trust))
    return dict(premium=prem.value, trust=trust.value, beta=beta, has_fit=has.astype(bool))


def bs_price(F, K, T, vol, df, is_call=True):
    return port().oracle_bs_price(F, K, T, vol, df, int(is_call))


def bs_delta(S, K, T, vol, r, q, is_call=True):
    return port().oracle_bs_delta(S, K, T, vol, r, q, int(is_call))


def bs_vega(S, K, T, vol, r, q):
    return port().oracle_bs_vega(S, K, T, vol, r, q)


def heston_price(S, K, T, r, q, v0, kappa, theta, xi, rho, is_call=True):
    """FP64 Heston price (Lewis single integral of the little-trap characteristic function)."""
    return port().oracle_heston_price(S, K, T, r, q, v0, kappa, theta, xi, rho, int(is_call))


def heston_price_p12(S, K, T, r, q, v0, kappa, theta, xi, rho, is_call=True):
    """The reference's P1/P2 decomposition of the same price (second rule)."""
    return port().oracle_heston_price_p12(S, K, T, r, q, v0, kappa, theta, xi, rho, int(is_call))


def heston_prices(S, K, T, r, q, v0, kappa, theta, xi, rho, threads=None):
    """Vectorised FP64 Heston call prices (all arguments broadcast), on all host threads."""
    args = np.ascontiguousarray(np.stack(np.broadcast_arrays(*(np.asarray(a, dtype=np.float64) for a in
                                                              (S, K, T, r, q, v0, kappa, theta, xi, rho))), axis=-1)
                                .reshape(-1, 10))
    out = np.zeros(len(args))
    port().oracle_heston_prices(len(args), _d(args), _d(out), int(threads or os.cpu_count() or 1))
    return out
