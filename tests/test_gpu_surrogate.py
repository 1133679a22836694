"""The learned surrogate's tensor-core kernels (tcgen05, BF16 operands, FP32
accumulation) against the CPU oracle (oracle/mlp_oracle.py), and what the
trained network gains over the pricing method without it."""
import numpy as np
import pytest

import oracle
from oracle import mlp_oracle as MO
from thoth_gb300 import surrogate as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(16, 16), (128, 16), (128, 128), (256, 64), (32, 256)])
def test_tcgen05_gemm(gpu, n, k):
    rng = np.random.default_rng(n * 1000 + k)
    a = rng.standard_normal((128, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    ref = gpu.from_bf16_bits(gpu.to_bf16_bits(a)).astype(np.float64) @ \
        gpu.from_bf16_bits(gpu.to_bf16_bits(b)).astype(np.float64).T
    d = gpu.tc_gemm_test(a, b)
    assert np.abs(d - ref).max() <= 1e-6 * k * np.abs(ref).max()


def _batch(seed, n=256):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=(n, 7)).astype(np.float32)
    y = rng.uniform(0, 1.5, size=n).astype(np.float32)
    sc = np.maximum(y, 0.05).astype(np.float32)
    return x, y, sc


def test_gradient_matches_cpu_oracle(gpu):
    m = S.Surrogate(seed=3)
    p = m.params().astype(np.float64)
    x, y, sc = _batch(0)
    g, loss = m.gradient(x, y, sc)
    go, lo = MO.gradient(p, x.astype(np.float64), y.astype(np.float64), sc.astype(np.float64))
    assert abs(loss - lo) <= 1e-4 * lo
    for a, b in [(MO.OFF_W1, MO.OFF_B1), (MO.OFF_B1, MO.OFF_W2), (MO.OFF_W2, MO.OFF_W5), (MO.OFF_W5, MO.N_PARAMS)]:
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 2e-3 * np.linalg.norm(go[a:b])
    m.close()


def test_inference_matches_cpu_oracle(gpu):
    m = S.Surrogate(seed=4)
    p = m.params().astype(np.float64)
    x, _, _ = _batch(1, n=1000)           # not a multiple of the 128-row tile
    y, _ = m.predict(x)
    yo, _, _ = MO.forward(p, x.astype(np.float64))
    assert np.abs(y - yo).max() <= 1e-3 * max(1.0, np.abs(yo).max())
    m.close()


def test_lattice_serving_matches_host_features(gpu):
    """Features, clipping, normalisation and price scale built on the device give the prices
    of the host path (predict_prices on the clipped lattice features), and the oracle's
    network with the same scale; sets outside the box are clipped the same way."""
    m = S.Surrogate(seed=6)
    rng = np.random.default_rng(7)
    sets = rng.uniform(S.BOX_LO[2:], S.BOX_HI[2:], size=(37, 5))
    sets[3] = S.BOX_HI[2:] * 1.2                         # outside the box: clipped
    lms, Ts = S.LATTICE_LM[::3], S.LATTICE_T[::2]
    got, ms = m.price_lattice(sets, lms, Ts)
    X = np.concatenate([S.lattice_features(p, lms, Ts) for p in sets])
    Xc = np.clip(X, S.BOX_LO, S.BOX_HI)
    want, _ = S.predict_prices(m, Xc)
    assert got.shape == want.shape and ms > 0
    assert np.abs(got - want).max() <= 1e-6 * max(1.0, np.abs(want).max())
    yo, _, _ = MO.forward(m.params().astype(np.float64), S.normalise(Xc).astype(np.float64))
    assert np.abs(got - yo * S.price_scale(Xc)).max() <= 1e-3 * max(1.0, np.abs(want).max())
    m.close()


def test_adam_step_matches_cpu(gpu):
    m = S.Surrogate(seed=5)
    p0 = m.params().astype(np.float64)
    x, y, sc = _batch(2)
    g, _ = m.gradient(x, y, sc)
    lr = 1e-3
    m.train(x, y, sc, epochs=1, batch=256, lr=lr)       # exactly one step
    p1 = m.params().astype(np.float64)
    g = g.astype(np.float64)
    w1 = g[MO.OFF_W1:MO.OFF_B1].reshape(MO.H, MO.KIN)
    w1[:, :7] += w1[:, 7:14].copy()                     # tied hi/lo input columns
    w1[:, 7:14] = w1[:, :7]
    w1[:, 14:] = 0.0
    m1, v1 = 0.1 * g, 0.001 * g * g
    step = (lr + 1e-6) * (m1 / 0.1) / (np.sqrt(v1 / 0.001) + 1e-8)
    step[MO.OFF_W1:MO.OFF_B1].reshape(MO.H, MO.KIN)[:, 14:] = 0.0
    np.testing.assert_allclose(p1, p0 - step, rtol=1e-4, atol=1e-7)
    m.close()


def test_trained_network_beats_the_method_without_it(gpu):
    # small version of the training setup: 96 parameter sets x 252 lattice cells, 2^14 paths
    X, Y, _, _ = S.mc_labels(S.sobol_params(96, 0), 1 << 14)
    m = S.Surrogate(seed=1)
    before = m.train(*S.train_targets(X, Y), epochs=1, batch=512, lr=1e-6)
    m.close()
    m = S.Surrogate(seed=1)
    after = m.train(*S.train_targets(X, Y), epochs=150, batch=1024, lr=5e-3)
    ev = S.sobol_params(4, 96)
    Xe = np.concatenate([S.lattice_features(p) for p in ev])
    cf = oracle.heston_prices(1.0, np.exp(Xe[:, 0]), Xe[:, 1], 0, 0, Xe[:, 6], Xe[:, 2], Xe[:, 3], Xe[:, 4],
                              Xe[:, 5])
    net, _ = S.predict_prices(m, Xe)
    plain = S.bs_effective(Xe)           # the closed-form estimate the network corrects, on its own
    e_net, e_plain = S.cell_error(net, cf), S.cell_error(plain, cf)
    assert after < 0.05 * before
    # the 2^14-path labels of this small setup carry ~5e-3 error of their own,
    # which bounds the network; it still at least halves the closed-form error
    assert np.median(e_net) < 0.5 * np.median(e_plain)
    assert np.quantile(e_net, 0.9) < 0.5 * np.quantile(e_plain, 0.9)
    m.close()


def test_price_grid_pipeline_small(gpu):
    X, Y, _, _ = S.mc_labels(S.sobol_params(64, 0), 1 << 14)
    m = S.Surrogate(seed=2)
    m.train(*S.train_targets(X, Y), epochs=60, batch=1024, lr=5e-3)
    ev = S.sobol_params(8, 64)
    fails = {}
    for policy in S.POLICIES:
        price, info = S.price_grid(m, ev, mc_paths=1 << 14, judge_frac=0.25, judge_paths=1 << 16, policy=policy)
        assert price.shape == (8 * 252,) and np.isfinite(price).all()
        assert info["judge_sets"] == 2 and info["cells"] == 8 * 252 and info["policy"] == policy
        # every flagged bucket of every in-box set went to MC, timed as run
        assert info["fallback_cells"] == info["failing_buckets"] * 8 + 252 * info["out_of_box_sets"]
        assert info["seconds"] == info["inference_s"] + info["judge_s"] + info["fallback_s"]
        assert 0 <= info["estimated_p90"] <= info["judged_p90"] and info["judge_noise_p90"] > 0
        fails[policy] = info["failing_buckets"]
    # the grid policy never takes over more buckets than the per-bucket one
    assert fails["grid"] <= fails["bucket"]
    m.close()
