"""LSV leverage calibration on the device (thoth_gpu_calibrate_leverage).

* layers against the oracle (Single::CalibrateLeverage restated, on the reference's Rng
  stream): the device draws the same stream, rounds every expression as the reference does
  and sums exactly, so the ensembles differ only where CUDA's exp / log / erfc differ from
  the host libm in the last bit;
* the reference test's degenerate limit (pricer/tests/test_lsv.cpp:77-103): flat 25 % target
  on a 30 % Heston base with vanishing vol of vol gives 25 / 30, and the calibrated LSV call
  prices at Black-Scholes 25 %;
* the defining property (test_lsv.cpp:42-60): LSV with the calibrated leverage reprices the
  target local-vol model's vanillas across strikes, within MC error plus the binned-particle
  bias the reference allows (0.10). The target is priced by the same engine as a local-vol
  model (an LSV asset whose variance stays at 1 and whose leverage is the local vol).
"""
import math

import numpy as np
import pytest

import oracle
from thoth_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


def test_layers_match_the_oracle(gpu):
    c = W.lsv_calibration(horizon_days=90)
    L, ms = gpu.calibrate_leverage(c)
    ref = oracle.calibrate_leverage(c)
    assert ms > 0
    np.testing.assert_allclose(L, ref, rtol=1e-9, atol=0)


def test_layers_match_the_oracle_uneven_dates_and_particles(gpu):
    c = W.lsv_calibration(horizon_days=45, particles=5000)
    c.days = np.ascontiguousarray(np.r_[0, 1, 2, 5, 9, 14, 30, 45], dtype=np.int32)
    ls, off = W.layer_grids(c.days, 100.0, 0.22)
    c.ln_step, c.offset = ls, off
    x = (off[:, None] + np.arange(201)[None, :]) * ls[:, None]
    c.local_vol = np.ascontiguousarray(W.skew_local_vol(np.exp(x), (c.days / 365.0)[:, None]))
    c.carry = np.ascontiguousarray(np.linspace(0.01, 0.03, len(c.days)))
    c.leverage = np.zeros_like(c.local_vol)
    L, _ = gpu.calibrate_leverage(c)
    np.testing.assert_allclose(L, oracle.calibrate_leverage(c), rtol=1e-9, atol=0)


def test_degenerate_limit_prices_black_scholes(gpu):
    h = dict(v0=0.09, kappa=3.0, theta=0.09, xi=1e-4, rho=0.0)
    c = W.lsv_calibration(horizon_days=365, local_vol=lambda S, t: np.full(np.broadcast(S, t).shape, 0.25),
                          heston=h, carry=0.05)
    L, _ = gpu.calibrate_leverage(c)
    np.testing.assert_allclose(L, 0.25 / 0.30, rtol=2e-3)
    b = abi.Book(days=c.days, paths=200000)
    a = b.add_heston(100.0, h["v0"], h["kappa"], h["theta"], h["xi"], h["rho"], 0.05,
                     leverage=(c.ln_step, c.offset, L))
    b.add_vanilla(a, 100.0, 365, abi.CALL, zero_rate=0.05)
    r = gpu.price_book(b)
    bs = oracle.bs_price(100.0 * math.exp(0.05), 100.0, 1.0, 0.25, math.exp(-0.05), True)
    assert abs(r["premium"][0] - bs) <= 6.0 * r["trust"][0] + 0.06


def test_calibrated_lsv_reprices_the_local_vol_model(gpu):
    c = W.lsv_calibration(horizon_days=365)
    L, _ = gpu.calibrate_leverage(c)
    h = c.heston
    strikes = (80.0, 100.0, 120.0)

    def book(local_model):
        b = abi.Book(days=c.days, paths=1 << 18)
        if local_model:      # variance pinned at 1: the leverage is the local vol itself
            a = b.add_heston(100.0, 1.0, 1.0, 1.0, 1e-9, 0.0, 0.02, leverage=(c.ln_step, c.offset, c.local_vol))
        else:
            a = b.add_heston(100.0, h["v0"], h["kappa"], h["theta"], h["xi"], h["rho"], 0.02,
                             leverage=(c.ln_step, c.offset, L))
        for K in strikes:
            b.add_vanilla(a, K, 365, abi.PUT if K < 100 else abi.CALL, zero_rate=0.02)
        return b

    lv = gpu.price_book(book(True))
    lsv = gpu.price_book(book(False))
    for i, K in enumerate(strikes):
        se = math.hypot(lv["trust"][i], lsv["trust"][i])
        assert abs(lsv["premium"][i] - lv["premium"][i]) <= 6.0 * se + 0.10, (K, lsv["premium"][i], lv["premium"][i])
    # and the Heston base alone does not: the leverage is doing the work
    plain = abi.Book(days=c.days, paths=1 << 18)
    a = plain.add_heston(100.0, h["v0"], h["kappa"], h["theta"], h["xi"], h["rho"], 0.02)
    for K in strikes:
        plain.add_vanilla(a, K, 365, abi.PUT if K < 100 else abi.CALL, zero_rate=0.02)
    pr = gpu.price_book(plain)
    miss = [abs(pr["premium"][i] - lv["premium"][i]) - 6.0 * math.hypot(pr["trust"][i], lv["trust"][i]) - 0.10
            for i in range(len(strikes))]
    assert max(miss) > 0.0, miss


def test_invalid_inputs(gpu):
    c = W.lsv_calibration(horizon_days=10, particles=1024)
    c.bins = 500
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.calibrate_leverage(c)
    assert e.value.code == abi.THOTH_GPU_E_INVALID
    c = W.lsv_calibration(horizon_days=10, particles=1024)
    c.days = np.ascontiguousarray(c.days[::-1])
    with pytest.raises(gpu.ThothGpuError):
        gpu.calibrate_leverage(c)


@pytest.mark.parametrize("particles,bins,min_count", [(1000, 30, 20), (700, 12, 100), (4099, 1, 1)])
def test_uneven_ensembles_and_thin_bins_match_the_oracle(gpu, particles, bins, min_count):
    """Particle counts off the warp size, every bin thin (the ensemble mean everywhere), and
    one bin: the device follows the oracle."""
    c = W.lsv_calibration(horizon_days=30, particles=particles)
    c.bins, c.min_bin_count = bins, min_count
    L, _ = gpu.calibrate_leverage(c)
    np.testing.assert_allclose(L, oracle.calibrate_leverage(c), rtol=1e-9, atol=0)
