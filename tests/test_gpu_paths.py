"""Stored paths (thoth_gpu_simulate_paths) against the oracle, path by path.

A vanilla call struck at 1e-9 with zero rates pays S_T: the oracle's per-path
contract values of one such call per date are the reference's spot path, to be
matched by the GPU's stored path (FP32 Kahan-compensated log-spot against FP64:
2e-5 relative). The stored paths also reproduce the GPU's own prices.
"""
import numpy as np
import pytest

import oracle
from thoth_gb300 import abi

pytestmark = pytest.mark.gpu

TINY = 1e-9


def spot_book(paths, lsv_second=False, skip=0):
    days = np.arange(0, 41)
    b = abi.Book(days=days, paths=paths)
    b.sobol_skip = skip
    a = b.add_heston(100.0, 0.04, 1.5, 0.04, 0.6, -0.7, 0.02)
    assets = [a]
    if lsv_second:
        ln_step = (np.log(240.0) - np.log(15.0)) / 39
        offset = int(np.floor(np.log(15.0) / ln_step))
        vals = 0.8 + 0.4 * np.random.default_rng(1).random((len(days), 40))
        assets.append(b.add_heston(60.0, 0.05, 2.0, 0.05, 0.5, -0.5, 0.01,
                                   leverage=(np.full(len(days), ln_step), np.full(len(days), offset, dtype=np.int64),
                                             vals)))
    for k in assets:
        for m in range(1, 41):
            b.add_vanilla(k, TINY, m, abi.CALL, zero_rate=0.0)
    return b, assets


@pytest.mark.parametrize("lsv_second,asset,skip", [(False, 0, 0), (True, 1, 0), (True, 0, 777)])
def test_stored_paths_match_the_oracle_per_path(gpu, lsv_second, asset, skip):
    n = 600
    b, assets = spot_book(n, lsv_second, skip)
    paths, ms = gpu.simulate_paths(b, asset)
    assert paths.shape == (41, n) and ms > 0
    ref = oracle.price_book(b, n_per_path=n)["per_path"]          # [path][product]
    first = 40 * asset
    want = ref[:, first:first + 40].T + TINY                        # [date 1..40][path]
    np.testing.assert_allclose(paths[1:], want, rtol=2e-5)
    assert np.all(paths[0] == b.assets[asset]["spot"])


def test_stored_paths_reproduce_the_prices(gpu):
    days = np.arange(0, 91)
    b = abi.Book(days=days, paths=(1 << 15) + 11)
    a = b.add_gbm(100.0, 0.3, 0.01)
    for K, m in ((95.0, 30), (100.0, 60), (110.0, 90)):
        b.add_vanilla(a, K, m, abi.CALL, zero_rate=0.0)
    paths, _ = gpu.simulate_paths(b, 0)
    r = gpu.price_book(b)
    for p, (K, m) in enumerate(((95.0, 30), (100.0, 60), (110.0, 90))):
        mc = np.mean(np.maximum(paths[m].astype(np.float64) - K, 0.0))
        assert abs(mc - r["premium"][p]) <= 1e-6 * r["premium"][p]


def test_stored_paths_errors(gpu):
    b, _ = spot_book(100)
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.simulate_paths(b, 3)
    assert e.value.code == abi.THOTH_GPU_E_INVALID
