"""The oracle port against the reference compiled here (oracle/_ref), on more
cases than the committed fixtures. Skipped where the reference build is absent."""
import numpy as np
import pytest

import oracle
from thoth_gb300 import workloads as W
from tests.golden.make_golden import mixed_book

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")


@pytest.mark.parametrize("dims,skip,n", [(1, 0, 5000), (97, 17, 300), (4097, 0, 20), (4097, 2 ** 20 + 3, 5)])
def test_sobol(dims, skip, n):
    assert np.array_equal(oracle.sobol_points(dims, skip, n), oracle.sobol_points(dims, skip, n, "ref"))


def test_acklam_random():
    p = np.random.default_rng(5).random(200000)
    assert np.array_equal(oracle.normal_cdf_inv(p), oracle.normal_cdf_inv(p, "ref"))


@pytest.mark.parametrize("t", [np.array([0.0, 0.5]), np.array([0, .1, .15, .4, .41, 1.0, 2.0]),
                               np.concatenate([[0], np.sort(np.random.default_rng(2).random(80)) * 3])])
def test_bridge(t):
    for f in (1, 3):
        assert np.array_equal(oracle.bridge_increments(t, f, 11, 4), oracle.bridge_increments(t, f, 11, 4, which="ref"))


def test_bridge_beyond_sobol_budget():
    # 2100 steps x 2 factors > 4097 dims: the tail draws come from xoshiro256++ (rng.hpp)
    t = np.arange(0, 2101) / 365.0
    a = oracle.bridge_increments(t, 2, 0, 2, seed=9)
    b = oracle.bridge_increments(t, 2, 0, 2, seed=9, which="ref")
    assert np.array_equal(a, b)


@pytest.mark.parametrize("book", ["heston", "lsv", "mixed", "skip"])
def test_books(book):
    b = {"heston": lambda: W.heston_grid(paths=1 << 11, calendar=True, months=(1, 2, 6)),
         "lsv": lambda: W.lsv_book(paths=1 << 9, seed=3),
         "mixed": lambda: mixed_book(paths=1 << 11),
         "skip": lambda: W.gbm_call(paths=3000, greeks=False)}[book]()
    if book == "skip":
        b.sobol_skip = 12345
    r1 = oracle.price_book(b, n_per_path=32)
    r2 = oracle.price_book(b, "ref", n_per_path=32)
    assert np.array_equal(r1["per_path"], r2["per_path"])
    assert np.array_equal(r1["premium"], r2["premium"])
    assert r1["book_premium"] == r2["book_premium"]


def test_pseudo_random_one_draw_per_path():
    """use_sobol: false on a one-step, one-factor book: one draw per path, so the oracle's
    stream is the reference's, path for path. (Otherwise the reference draws in the order of
    its topological schedule, e.g. a 30-date GBM book's dates last to first, which the
    oracle does not restate.)"""
    b = W.gbm_call(paths=3000, greeks=False)
    b.use_sobol = False
    b.seed = 11
    r1 = oracle.price_book(b, n_per_path=32)
    r2 = oracle.price_book(b, "ref", n_per_path=32)
    assert np.array_equal(r1["per_path"], r2["per_path"])
    assert np.array_equal(r1["premium"], r2["premium"])
