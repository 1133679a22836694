"""LSV leverage calibration on the host side: the oracle and the Rng jump-ahead.

* the oracle's Rng (thoth_oracle.c) draws the reference's own stream (helpers/rng.hpp,
  through oracle/_ref where it was built), Gaussians included;
* thoth_gpu_xoshiro_jump, the engine's host jump-ahead (x^n modulo the transition's
  characteristic polynomial), lands on the state sequential stepping reaches;
* the oracle's calibration (Single::CalibrateLeverage restated) in the reference test's
  degenerate limit: a flat 25 % target on a 30 % Heston base with vanishing vol of vol
  gives the flat ratio 25 / 30 (pricer/tests/test_lsv.cpp:77-103);
* the layers clamp, and the first layer uses the ensemble mean v0.
"""
import numpy as np
import pytest

import oracle
from thoth_gb300 import abi, workloads as W

need_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")


@need_ref
def test_oracle_rng_is_the_reference_rng():
    raw_o, _ = oracle.xoshiro_draws(abi.LSV_CALIB_SEED, 1000, 4096)
    raw_r, g_r = oracle.ref_rng_draws(abi.LSV_CALIB_SEED, 1000, 4096)
    np.testing.assert_array_equal(raw_o, raw_r)
    u = (raw_r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    np.testing.assert_array_equal(oracle.normal_cdf_inv(np.where(u > 0, u, 1.0 / 9007199254740992.0)), g_r)


@pytest.mark.parametrize("n", [0, 1, 2, 255, 256, 257, 32766, 99991])
def test_jump_ahead_equals_stepping(n):
    import thoth_gb300 as G
    _, s0 = oracle.xoshiro_draws(12345, 17, 0)
    _, want = oracle.xoshiro_draws(12345, 17 + n, 0)
    assert G.xoshiro_jump(s0, n) == want


def flat_case(days=40, particles=4096, vol=0.25, base=0.30, xi=1e-4):
    h = dict(v0=base * base, kappa=3.0, theta=base * base, xi=xi, rho=0.0)
    return W.lsv_calibration(horizon_days=days, particles=particles, local_vol=lambda S, t: np.full(np.broadcast(S, t).shape, vol),
                             heston=h, carry=0.05)


def test_oracle_degenerate_limit_is_the_flat_ratio():
    L = oracle.calibrate_leverage(flat_case())
    np.testing.assert_allclose(L, 0.25 / 0.30, rtol=2e-3)


def test_oracle_layers_clamp_and_first_layer_uses_v0():
    c = W.lsv_calibration(horizon_days=30, particles=2048)
    L = oracle.calibrate_leverage(c)
    assert L.min() >= 0.05 and L.max() <= 10.0
    np.testing.assert_allclose(L[0], np.clip(c.local_vol[0] / np.sqrt(c.heston["v0"]), 0.05, 10.0), rtol=1e-12)
    tiny = W.lsv_calibration(horizon_days=5, particles=512, local_vol=lambda S, t: np.full(np.broadcast(S, t).shape, 1e-4))
    assert np.all(oracle.calibrate_leverage(tiny) == 0.05)
