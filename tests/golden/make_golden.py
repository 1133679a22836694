"""Generate the golden fixtures in this folder from the reference's own code.

Runs the reference's hot-path sources (compiled unmodified into
oracle/_ref/libref_oracle.so by oracle/Makefile from a GValas/Thoth checkout)
on seeded inputs and stores their outputs:

  sobol.npz    uint32 Sobol points (SobolGenerator Skip/Next)
  acklam.npz   NormalCdfInv on a probability grid including the tails
  bridge.npz   PathGenerator::NextPath normalised increments
  books.npz    prices, trusts and the first per-path contract values of the
               books built by books() below, through the reference node graph

Usage: python tests/golden/make_golden.py   (needs oracle/_ref built)
"""
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402
from thoth_gb300 import workloads as W  # noqa: E402
from thoth_gb300.abi import Book, CALL, PUT  # noqa: E402

N_PER_PATH = 64


def mixed_book(paths=1 << 12):
    """GBM + Heston names on a weekly grid: vanilla, barrier (up/down, in/out),
    variance (continuous and discrete), quanto vanilla, correlated basket."""
    days = np.concatenate([np.arange(0, 365, 7), [365]])
    b = Book(days=days, paths=paths)
    g0 = b.add_gbm(100.0, 0.25, 0.02)
    g1 = b.add_gbm(50.0, 0.35, 0.01)
    h = b.add_heston(80.0, 0.05, 2.0, 0.05, 0.5, -0.6, 0.03)
    b.set_cholesky(np.linalg.cholesky(np.array([[1.0, 0.5, 0.2], [0.5, 1.0, 0.3], [0.2, 0.3, 1.0]])))
    last = len(days) - 1
    b.add_vanilla(g0, 105.0, last, CALL, zero_rate=0.03)
    b.add_vanilla(h, 75.0, 26, PUT, zero_rate=0.03)
    b.add_vanilla(g1, 52.0, last, CALL, zero_rate=0.03, quanto=0.25 * 0.1 * 0.3)
    b.add_barrier(g0, 100.0, last, 80.0, up=False, knock_in=False, monitor=np.arange(1, last + 1), zero_rate=0.03)
    b.add_barrier(h, 80.0, last, 100.0, up=True, knock_in=True, monitor=np.arange(4, last + 1, 4), zero_rate=0.03,
                  option_type=PUT)
    b.add_barrier(g1, 50.0, 40, 60.0, up=True, knock_in=False, monitor=np.arange(1, 41), zero_rate=0.02, fx=1.1)
    b.add_variance(h, last, strike_variance=0.05, notional=100.0, zero_rate=0.03)
    b.add_variance(g0, 30, strike_variance=0.06, notional=50.0, zero_rate=0.03, obs=np.arange(2, 31, 2))
    b.add_basket([0, 1, 2], [0.4, 0.8, 0.5], 100.0, last, CALL, zero_rate=0.03)
    return b


def books():
    return {
        "gbm_call": W.gbm_call(paths=1 << 14, greeks=False),
        "heston_calendar": W.heston_grid(paths=1 << 12, calendar=True, months=(1, 3, 12), strikes=(80, 100, 120)),
        "lsv_book": W.lsv_book(paths=1 << 10),
        "mixed_book": mixed_book(),
    }


def main():
    if not oracle.ref_available():
        oracle.build()
    assert oracle.ref_available(), "reference build missing"
    # Sobol
    sob = {}
    for name, (dims, skip, n) in {"a": (16, 0, 1024), "b": (4097, 1000, 8), "c": (1460, 123456, 16),
                                  "d": (3, 4294967000 - 64, 64)}.items():
        sob[name] = oracle.sobol_points(dims, skip, n, "ref")
        sob[name + "_args"] = np.array([dims, skip, n], dtype=np.int64)
    np.savez_compressed(HERE / "sobol.npz", **sob)
    # Acklam
    p = np.concatenate([np.logspace(-12, -1, 200), np.linspace(0.01, 0.99, 199), 1 - np.logspace(-1, -12, 200),
                        np.array([0.02425, 0.97575, 0.5, 2.0 ** -32, 1 - 2.0 ** -32])])
    np.savez_compressed(HERE / "acklam.npz", p=p, z=oracle.normal_cdf_inv(p, "ref"))
    # bridge
    t = np.arange(0, 366) / 365.0
    np.savez_compressed(HERE / "bridge.npz", t=t,
                        inc=oracle.bridge_increments(t, 2, 3, 3, which="ref"),
                        t2=np.arange(0, 505) / 252.0,
                        inc2=oracle.bridge_increments(np.arange(0, 505) / 252.0, 2, 0, 2, which="ref"))
    # books
    out = {}
    for name, b in books().items():
        r = oracle.price_book(b, "ref", n_per_path=N_PER_PATH)
        out[name + "_premium"] = r["premium"]
        out[name + "_trust"] = r["trust"]
        out[name + "_book"] = np.array([r["book_premium"], r["book_trust"]])
        out[name + "_per_path"] = r["per_path"]
    np.savez_compressed(HERE / "books.npz", **out)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
