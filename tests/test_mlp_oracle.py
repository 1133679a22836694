"""The CPU oracle of the surrogate MLP is itself a correct gradient: with the
bf16 roundings switched off it matches central finite differences."""
import numpy as np

from oracle import mlp_oracle as MO


def test_oracle_gradient_finite_differences(monkeypatch):
    monkeypatch.setattr(MO, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(0)
    p = rng.normal(scale=0.1, size=MO.N_PARAMS)
    p[MO.OFF_W1:MO.OFF_B1].reshape(MO.H, MO.KIN)[:, 14:] = 0.0
    x = rng.uniform(-1, 1, size=(8, 7))
    y = rng.uniform(0, 1, size=8)
    sc = np.maximum(y, 0.1)
    g, _ = MO.gradient(p, x, y, sc)
    for j in list(rng.choice(MO.N_PARAMS, size=40, replace=False)) + [MO.OFF_B5, MO.OFF_W5 + 3, MO.OFF_B1 + 7]:
        if MO.OFF_W1 <= j < MO.OFF_B1 and (j % MO.KIN) >= 14:
            continue
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[j] += h
        pm[j] -= h
        fd = (MO.gradient(pp, x, y, sc)[1] - MO.gradient(pm, x, y, sc)[1]) / (2 * h)
        assert abs(fd - g[j]) <= 1e-5 + 1e-4 * abs(fd), (j, fd, g[j])
