"""Generator of the inverse-normal coefficients in engine.cuh (quantile_central, quantile_tail).

The engine's FP32 inverse normal follows Giles' change of variable (M. Giles, "Approximating
the erfinv function", GPU Computing Gems Jade Edition, 2011): with q = min(u, 1 - u),
s = 2u - 1 and w = -ln(4 q (1 - q)) = -ln(1 - s^2),

    Phi^-1(u) = s * g(w),   g(w) = sqrt(2) erfinv(s) / s,

and g is smooth in w. It is approximated by two polynomials:
  central  w < 6.25:  a polynomial of degree 9 in v = w - 3.125,
  tail     w >= 6.25: a polynomial of degree 9 in v = sqrt(w) - 3.6479158,
the tail covering q down to 2^-32 (w <= 20.8), the smallest q a 32-bit Sobol word gives.

This script fits both by minimising the largest relative error on a dense set of points
(Lawson's iteratively reweighted least squares: each pass reweights the points by their
error, which converges to the minimax polynomial), with the target computed to 40 digits by
mpmath. The coefficients are rounded to float32 one at a time, the remaining ones refitted after each
rounding, and then polished by one-ulp moves against the error of an FP32 Horner evaluation
with fused multiply-adds (emulated in float64 with one rounding per step). The script prints
that error on a second set of points and the coefficients as engine.cuh writes them,
highest power first.

    python thoth_gb300/csrc/fit_quantile.py
"""
import mpmath
import numpy as np

mpmath.mp.dps = 40
W_SPLIT = 6.25
CENTRAL_SHIFT = 3.125
TAIL_SHIFT = 3.6479158
DEGREE = 9
Q_MIN = 2.0 ** -32


def g_of_w(w):
    """sqrt(2) erfinv(s) / s at s = sqrt(1 - e^-w), to 40 digits."""
    w = mpmath.mpf(w)
    if w == 0:
        return mpmath.sqrt(mpmath.pi / 2)  # the limit s -> 0
    s = mpmath.sqrt(-mpmath.expm1(-w))
    return mpmath.sqrt(2) * mpmath.erfinv(s) / s


def lawson(A, b, passes):
    """Minimax solution of A c ~ b through Lawson's reweighted least squares."""
    weight = np.full(len(b), 1.0 / len(b))
    coef = None
    for _ in range(passes):
        sw = np.sqrt(weight)
        coef, *_ = np.linalg.lstsq(A * sw[:, None], b * sw, rcond=None)
        weight = weight * (np.abs(A @ coef - b) + 1e-300)
        weight /= weight.sum()
    return coef


def fit(v, target, degree, passes=200):
    """Minimax (relative error) polynomial in v, coefficients rounded to float32 one at a
    time from the constant term up, the higher powers refitted after each rounding so that
    they absorb its error. Returns the float32 coefficients, highest power first."""
    A = np.vander(v, degree + 1, increasing=True) / target[:, None]
    b = np.ones_like(target)
    fixed = []  # rounded coefficients, constant term first
    for k in range(degree + 1):
        # fit powers k..degree with the rounded powers below k held
        rhs = b.copy()
        for j, c in enumerate(fixed):
            rhs -= A[:, j] * float(c)
        coef = lawson(A[:, k:], rhs, passes)
        fixed.append(np.float32(coef[0]))
    return fixed[::-1]


def polish(desc32, v, target, rounds=4):
    """Greedy search over one-ulp moves of each float32 coefficient, keeping a move where it
    lowers the largest relative error of the FP32 evaluation on (v, target)."""
    desc32 = list(desc32)
    v32 = v.astype(np.float32)

    def worst(c):
        return float(np.max(np.abs(horner_f32(c, v32) / target - 1.0)))

    best = worst(desc32)
    for _ in range(rounds):
        for i in range(len(desc32)):
            for direction in (np.float32(np.inf), np.float32(-np.inf)):
                trial = list(desc32)
                trial[i] = np.nextafter(desc32[i], direction)
                e = worst(trial)
                if e < best:
                    best, desc32 = e, trial
    return desc32


def horner_f32(coef_desc32, v32):
    """FP32 Horner with fused multiply-adds: each step rounds once to float32."""
    p = np.full_like(v32, coef_desc32[0], dtype=np.float32)
    for c in coef_desc32[1:]:
        p = (p.astype(np.float64) * v32.astype(np.float64) + np.float64(c)).astype(np.float32)
    return p


def main():
    w_max = float(-mpmath.log(4 * mpmath.mpf(Q_MIN) * (1 - mpmath.mpf(Q_MIN))))
    # dense Chebyshev-distributed points on each interval
    n = 3000
    k = np.arange(n)
    cheb = 0.5 * (1 - np.cos(np.pi * (k + 0.5) / n))
    w_c = W_SPLIT * cheb
    r_t = np.sqrt(W_SPLIT) + (np.sqrt(w_max) - np.sqrt(W_SPLIT)) * cheb
    g_c = np.array([float(g_of_w(w)) for w in w_c])
    g_t = np.array([float(g_of_w(r * r)) for r in r_t])
    out = {}
    for name, v, g in (("central", w_c - CENTRAL_SHIFT, g_c), ("tail", r_t - TAIL_SHIFT, g_t)):
        desc32 = polish(fit(v, g, DEGREE), v, g)
        # error of the FP32 evaluation on a second, uniform set of points
        vv = np.linspace(v.min(), v.max(), 2001)
        if name == "central":
            ref = np.array([float(g_of_w(x + CENTRAL_SHIFT)) for x in vv])
        else:
            ref = np.array([float(g_of_w((x + TAIL_SHIFT) ** 2)) for x in vv])
        got = horner_f32(desc32, vv.astype(np.float32))
        out[name] = (desc32, float(np.max(np.abs(got / ref - 1.0))))
    for name, (desc32, err) in out.items():
        print("// %s: max relative error of the FP32 evaluation %.2e" % (name, err))
        for c in desc32:
            print("    %.9e" % c)


if __name__ == "__main__":
    main()
