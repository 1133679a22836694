"""The CPU oracle (oracle/thoth_oracle.c) against fixtures generated from the
reference's own code (tests/golden/make_golden.py)."""
import numpy as np

import oracle
from tests.golden.make_golden import books, N_PER_PATH


def test_sobol_points_bit_exact(golden):
    g = golden["sobol"]
    for k in ("a", "b", "c", "d"):
        dims, skip, n = (int(v) for v in g[k + "_args"])
        assert np.array_equal(oracle.sobol_points(dims, skip, n), g[k]), k


def test_first_sobol_points_known_values():
    # the first points printed by the reference generator: all 0.5, then (.75,.25,...), (.25,.75,...)
    p = oracle.sobol_points(4, 0, 4).astype(np.float64) / 2.0 ** 32
    assert np.array_equal(p, [[.5, .5, .5, .5], [.75, .25, .25, .25], [.25, .75, .75, .75], [.375, .375, .625, .875]])


def test_acklam_bit_exact(golden):
    g = golden["acklam"]
    assert np.array_equal(oracle.normal_cdf_inv(g["p"]), g["z"])
    assert abs(oracle.normal_cdf_inv(np.array([0.975]))[0] - 1.959963986120) < 1e-12


def test_bridge_bit_exact(golden):
    g = golden["bridge"]
    assert np.array_equal(oracle.bridge_increments(g["t"], 2, 3, 3), g["inc"])
    assert np.array_equal(oracle.bridge_increments(g["t2"], 2, 0, 2), g["inc2"])


def test_books_match_reference_graph(golden):
    g = golden["books"]
    for name, b in books().items():
        r = oracle.price_book(b, n_per_path=N_PER_PATH)
        # same operation order as the reference: equal up to libm differences between machines
        np.testing.assert_allclose(r["premium"], g[name + "_premium"], rtol=1e-12, atol=1e-12, err_msg=name)
        np.testing.assert_allclose(r["trust"], g[name + "_trust"], rtol=1e-9, atol=1e-12, err_msg=name)
        np.testing.assert_allclose(r["per_path"], g[name + "_per_path"], rtol=1e-12, atol=1e-12, err_msg=name)
        np.testing.assert_allclose([r["book_premium"], r["book_trust"]], g[name + "_book"], rtol=1e-9, err_msg=name)


def test_config1_anchor():
    # 2^18 Sobol paths, 1 step: the reference graph prices 10.761964 +- 0.034004 (BS 10.762395)
    from thoth_gb300 import workloads as W
    r = oracle.price_book(W.gbm_call(paths=1 << 18, greeks=False))
    assert abs(r["premium"][0] - 10.761964) < 5e-7
    assert abs(r["trust"][0] - 0.034004) < 5e-7
    bs = oracle.bs_price(100 * np.exp(0.02), 100, 1.0, 0.25, np.exp(-0.03))
    assert abs(bs - 10.762395) < 5e-7
