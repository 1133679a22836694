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


def test_weight_averaged_training(gpu):
    """Training with tail averaging of the weights: the model keeps the average, its bf16
    operand copies follow (predictions equal the oracle's network on the returned FP32
    weights), the loss falls, and no averaging is the plain training call bit for bit."""
    x, y, sc = _batch(11, n=4096)
    xo = x.astype(np.float64)
    plain, avg0 = S.Surrogate(seed=9), S.Surrogate(seed=9)
    la = plain.train(x, y, sc, epochs=6, batch=1024, lr=2e-3, seed=5)
    lb = avg0.train(x, y, sc, epochs=6, batch=1024, lr=2e-3, seed=5, avg_epochs=0)
    assert la == lb and np.array_equal(plain.params(), avg0.params())
    m = S.Surrogate(seed=9)
    _, l0 = m.gradient(x[:1024], y[:1024], sc[:1024])
    m.train(x, y, sc, epochs=6, batch=1024, lr=2e-3, seed=5, avg_epochs=3, lr_avg=5e-4)
    p = m.params().astype(np.float64)
    assert not np.array_equal(p, plain.params().astype(np.float64))
    W1 = p[MO.OFF_W1:MO.OFF_B1].reshape(MO.H, MO.KIN)
    assert np.array_equal(W1[:, :7], W1[:, 7:14])          # the tied hi / lo input columns
    got, _ = m.predict(x)
    want, _, _ = MO.forward(p, xo)
    assert np.abs(got - want).max() <= 1e-3 * max(1.0, np.abs(want).max())
    _, l1 = m.gradient(x[:1024], y[:1024], sc[:1024])
    assert l1 < 0.9 * l0                                   # random targets: the fit is partial
    with pytest.raises(gpu.ThothGpuError):
        m.train(x, y, sc, epochs=4, batch=1024, lr=2e-3, avg_epochs=4, lr_avg=1e-4)
    with pytest.raises(gpu.ThothGpuError):
        m.train(x, y, sc, epochs=4, batch=1024, lr=2e-3, avg_epochs=2, lr_avg=0.0)
    for s_ in (plain, avg0, m):
        s_.close()


def test_ensemble_trains_members_side_by_side_and_serves_their_mean(gpu):
    """An ensemble's members trained side by side on their own streams end with exactly the
    weights each gets trained alone (same initialisation, data-order seed seed + j); the
    ensemble's lattice prices are the mean of the members' own lattice prices."""
    x, y, sc = _batch(12, n=4096)
    ens = S.Ensemble(members=3, seed=20)
    losses = ens.train(x, y, sc, epochs=3, batch=1024, lr=2e-3, seed=7)
    assert len(losses) == 3 and all(np.isfinite(losses))
    for j, m in enumerate(ens.members):
        alone = S.Surrogate(seed=20 + j)
        alone.train(x, y, sc, epochs=3, batch=1024, lr=2e-3, seed=7 + j)
        assert np.array_equal(alone.params(), m.params()), j
        alone.close()
    rng = np.random.default_rng(3)
    sets = rng.uniform(S.BOX_LO[2:], S.BOX_HI[2:], size=(11, 5))
    got, ms = ens.price_lattice(sets)
    each = np.stack([m.price_lattice(sets)[0] for m in ens.members]).astype(np.float64)
    assert ms > 0 and got.shape == each.shape[1:]
    assert np.abs(got - each.mean(axis=0)).max() <= 1e-6 * max(1.0, np.abs(each).max())
    ens.close()


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
