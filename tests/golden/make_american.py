"""Generate american.npz: golden vectors of the Longstaff-Schwartz exercise from the
reference's own code.

oracle/_ref/libref_oracle.so runs the fit and apply loops of
pricer/src/tasks/pricer_mcl_american.cpp:263-447 around the reference's unmodified
LeastSquares (helpers/maths.cpp) and payoff_vanilla (helpers/finance.cpp), summing in
path order as the reference does. Inputs are seeded exact-GBM spot paths in single
precision, date-major, on the reference tests' grid (one year, 30-day steps):

  put_*    put K=100, S0=100, vol 30 %, r 8 %: the fit (beta, has_fit, premium, trust)
  bump_*   the put's frozen policy applied to paths from S0=101
  call_*   call K=95, S0=100, vol 30 %, r 2 %, dividend yield 6 %: the fit

Usage: python tests/golden/make_american.py   (needs oracle/_ref built)
"""
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402
from oracle import american as am  # noqa: E402

DAYS = np.array(list(range(0, 361, 30)) + [365])
N = 1024
MIN_ITM = 50


def main():
    tau = DAYS / 365.0
    out = dict(days=DAYS, min_itm=MIN_ITM)
    cases = [("put", 100.0, 100.0, 0.08, 0.0, False, 11), ("call", 100.0, 95.0, 0.02, 0.06, True, 12)]
    for name, S0, K, r, q, call, seed in cases:
        S = am.gbm_paths(S0, 0.30, r, q, DAYS, N, seed)
        rates = np.full(len(DAYS), r)
        f = oracle.ref_lsm(S, tau, rates, K, call, K, MIN_ITM)
        out.update({name + "_paths": S, name + "_rates": rates, name + "_strike": K, name + "_beta": f["beta"],
                    name + "_has_fit": f["has_fit"], name + "_premium": f["premium"], name + "_trust": f["trust"]})
        if name == "put":
            Sb = am.gbm_paths(101.0, 0.30, r, q, DAYS, N, seed)
            a = oracle.ref_lsm(Sb, tau, rates, K, call, K, MIN_ITM, policy=(f["beta"], f["has_fit"]))
            out.update(bump_paths=Sb, bump_premium=a["premium"], bump_trust=a["trust"])
    np.savez_compressed(HERE / "american.npz", **out)
    print({k: v for k, v in out.items() if np.ndim(v) == 0})


if __name__ == "__main__":
    main()
