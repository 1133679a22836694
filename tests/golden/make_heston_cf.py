"""30-digit Heston call prices (mpmath) pinning the FP64 closed-form oracle.

Lewis (2000) single integral of the little-trap characteristic function,
evaluated with mpmath at 30 significant digits on:
  * the Heston vanilla grid (S0 100, r 0.03, q 0, kappa 1.5, theta 0.04,
    xi 0.6, rho -0.7, v0 0.04): strikes 80..120 step 5, maturities 1,2,3,4,5,12,24 months;
  * 24 seeded parameter sets drawn from the surrogate's training box.
Usage: python tests/golden/make_heston_cf.py
"""
import pathlib

import mpmath as mp
import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
mp.mp.dps = 30


def cf(u, T, v0, kappa, theta, xi, rho):
    d = mp.sqrt((rho * xi * 1j * u - kappa) ** 2 + xi * xi * (1j * u + u * u))
    g = (kappa - rho * xi * 1j * u - d) / (kappa - rho * xi * 1j * u + d)
    e = mp.exp(-d * T)
    C = kappa * theta / xi ** 2 * ((kappa - rho * xi * 1j * u - d) * T - 2 * mp.log((1 - g * e) / (1 - g)))
    D = (kappa - rho * xi * 1j * u - d) / xi ** 2 * (1 - e) / (1 - g * e)
    return mp.exp(C + D * v0)


def lewis_call(S, K, T, r, q, v0, kappa, theta, xi, rho):
    S, K, T, r, q = (mp.mpf(x) for x in (S, K, T, r, q))
    F = S * mp.exp((r - q) * T)
    k = mp.log(F / K)
    f = lambda u: mp.re(mp.exp(1j * u * k) * cf(u - 0.5j, T, v0, kappa, theta, xi, rho)) / (u * u + 0.25)
    val = mp.quad(f, [0, 2, 8, 32, 128, 512, 2048, mp.inf])
    return mp.exp(-r * T) * (F - mp.sqrt(F * K) / mp.pi * val)


def main():
    rows = []
    for m in (1, 2, 3, 4, 5, 12, 24):
        for K in range(80, 121, 5):
            rows.append((100.0, K, m / 12.0, 0.03, 0.0, 0.04, 1.5, 0.04, 0.6, -0.7))
    rng = np.random.default_rng(11)
    for _ in range(24):
        lm = rng.uniform(-0.5, 0.5)
        rows.append((100.0, 100.0 * float(np.exp(lm)), rng.uniform(1 / 12, 3), 0.0, 0.0, rng.uniform(0.01, 0.16),
                     rng.uniform(0.5, 5), rng.uniform(0.01, 0.16), rng.uniform(0.1, 1.0), rng.uniform(-0.95, 0.0)))
    args = np.array(rows, dtype=np.float64)
    price = np.array([float(lewis_call(*r)) for r in rows])
    np.savez_compressed(HERE / "heston_cf.npz", args=args, call=price)
    print("wrote", len(rows), "prices")


if __name__ == "__main__":
    main()
