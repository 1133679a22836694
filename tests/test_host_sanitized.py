"""The library's host code under AddressSanitizer and UBSan, without a GPU.

The reference runs its test binary in an ASan + UBSan build. Here the same library is built
with its host code sanitized (thoth_gb300.build.build_sanitized) and loaded in a child
process with the sanitizer runtimes preloaded. The child runs the host-logic tests and
prices nothing: it validates and plans 900 mutated book descriptors (indices,
dates, counts, model parameters and leverage grids out of range or not finite), and checks
300 mutated calibration inputs and 200 American requests. Every descriptor must come back
planned or rejected with an error code, and the sanitizers must report nothing.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _runtime(name):
    p = subprocess.run(["gcc", "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


@pytest.fixture(scope="module")
def sanitized_env(tmp_path_factory):
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not asan or not ubsan:
        pytest.skip("no AddressSanitizer / UBSan runtime for this compiler")
    sys.path.insert(0, ROOT)
    from thoth_gb300 import build as B
    lib = B.build_sanitized(tmp_path_factory.mktemp("build_san"))
    env = dict(os.environ)
    env.update(THOTH_GPU_LIB=str(lib), LD_PRELOAD=asan + " " + ubsan,
               ASAN_OPTIONS="detect_leaks=0:protect_shadow_gap=0:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", PYTHONPATH=ROOT)
    return env


def test_host_logic_under_sanitizers(sanitized_env):
    p = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-m", "not gpu",
                        os.path.join(ROOT, "tests", "test_host_logic.py")],
                       cwd=ROOT, env=sanitized_env, capture_output=True, text=True, timeout=900)
    assert p.returncode == 0, p.stdout[-3000:] + p.stderr[-3000:]
    assert "ERROR: AddressSanitizer" not in p.stderr and "runtime error" not in p.stderr


FUZZ = r'''
import math, random
import numpy as np
import thoth_gb300 as G
from thoth_gb300 import abi, workloads as W


def books():
    yield W.heston_grid(paths=4096)
    yield W.lsv_book(paths=4096)
    b = abi.Book(days=np.arange(0, 40), paths=5000)
    g = b.add_gbm(100.0, 0.2, 0.01)
    h = b.add_heston(50.0, 0.04, 1.5, 0.04, 0.5, -0.6, 0.02)
    b.add_vanilla(g, 100.0, 39)
    b.add_barrier(g, 100.0, 39, 80.0, up=False, knock_in=False, monitor=np.arange(1, 40))
    b.add_variance(h, 30, strike_variance=0.04)
    b.add_basket([0, 1], [0.5, 0.5], 100.0, 20)
    b.set_cholesky(np.eye(2))
    yield b


def mutate(b, rng):
    what = rng.randrange(12)
    P, A = b.products, b.assets
    if what == 0:
        rng.choice(P)["maturity"] = rng.choice([-1, b.n_dates, 10 ** 6])
    elif what == 1:
        rng.choice(P)["asset"] = rng.choice([-5, len(A), 99])
    elif what == 2:
        rng.choice(P)["kind"] = rng.choice([-1, 7, 99])
    elif what == 3:
        rng.choice(P)["strike"] = rng.choice([math.nan, -math.inf, -5.0])
    elif what == 4:
        rng.choice(A)["spot"] = rng.choice([math.nan, 0.0, -1.0, math.inf])
    elif what == 5:
        rng.choice(A)["model"] = rng.choice([-1, 3, 77])
    elif what == 6:
        b.paths = rng.choice([0, 1, -7, 1 << 40])
    elif what == 7:
        v, c = rng.choice([-3, 0, b.n_dates, 10 ** 7]), rng.choice([-1, 50])
        for p in P:
            if "monitor" in p:
                p["monitor"] = np.full(len(p["monitor"]), v, dtype=np.int32)
            if "components" in p:
                p["components"] = np.full(len(p["components"]), c, dtype=np.int32)
    elif what == 8:
        for a in A:
            for k in ("v0", "kappa", "theta", "xi", "rho", "vol"):
                if k in a and rng.random() < 0.3:
                    a[k] = rng.choice([math.nan, -1.0, 1e300, -0.0, 2.0])
    elif what == 9:
        for a in A:
            if "lev_offset" in a:
                a["lev_offset"] = a["lev_offset"] + rng.choice([-10 ** 12, 10 ** 12, -(1 << 62)])
            if "lev_ln_step" in a and rng.random() < 0.5:
                a["lev_ln_step"] = a["lev_ln_step"] * rng.choice([0.0, -1.0, math.nan])
    elif what == 10:
        if b.days is not None:
            b.days = b.days.copy()
            i = rng.randrange(1, len(b.days))
            b.days[i] = b.days[i - 1] - rng.choice([0, 1, 5])
        b.t = b.t.copy()
        b.t[rng.randrange(len(b.t))] = rng.choice([math.nan, -1.0, 1e9])
    else:
        b.sobol_skip = rng.choice([-1, 1 << 62])
        b.seed = rng.randrange(1 << 63)


rng = random.Random(5)
planned = rejected = 0
for base in books():
    for _ in range(300):
        b = base.copy()
        mutate(b, rng)
        try:
            G.plan_summary(b)
            planned += 1
        except G.ThothGpuError as e:
            assert e.code < 0
            rejected += 1
print("planned", planned, "rejected", rejected)
'''


def test_mutated_descriptors_are_planned_or_rejected_under_sanitizers(sanitized_env):
    p = subprocess.run([sys.executable, "-c", FUZZ], cwd=ROOT, env=sanitized_env, capture_output=True, text=True,
                       timeout=900)
    assert p.returncode == 0, p.stdout[-3000:] + p.stderr[-3000:]
    assert "ERROR: AddressSanitizer" not in p.stderr and "runtime error" not in p.stderr
    planned, rejected = (int(x) for x in p.stdout.split()[1::2])
    assert planned + rejected == 900 and rejected > 600


FUZZ_INPUTS = r'''
import copy, math, random
import numpy as np
import thoth_gb300 as G
from thoth_gb300 import abi, workloads as W

rng = random.Random(9)
ok_codes = (abi.THOTH_GPU_E_INVALID, abi.THOTH_GPU_E_UNSUPPORTED, abi.THOTH_GPU_E_TOO_LARGE,
            abi.THOTH_GPU_E_NODEVICE)
seen = 0
base = W.lsv_calibration(horizon_days=20, particles=1024)
for _ in range(300):
    c = copy.deepcopy(base)
    what = rng.randrange(8)
    if what == 0:
        c.days = c.days.copy(); c.days[rng.randrange(1, len(c.days))] = rng.choice([-1, 0, 10 ** 9])
    elif what == 1:
        c.ln_step = c.ln_step * rng.choice([0.0, -1.0, math.nan, 1e300])
    elif what == 2:
        c.offset = c.offset + rng.choice([-(1 << 62), 1 << 62, -10 ** 15])
    elif what == 3:
        c.local_vol = c.local_vol.copy(); c.local_vol.flat[rng.randrange(c.local_vol.size)] = rng.choice([math.nan, -0.1, 0.0, math.inf])
    elif what == 4:
        c.particles, c.bins, c.min_bin_count = rng.choice([(-5, 0, 0), (1, 0, 0), (1 << 30, 0, 0), (0, 1 << 20, 0), (0, -3, 7), (0, 0, 1 << 30)])
    elif what == 5:
        c.heston[rng.choice(["v0", "kappa", "theta", "xi", "rho"])] = rng.choice([math.nan, -1.0, 5.0, 0.0])
    elif what == 6:
        c.spot = rng.choice([0.0, -1.0, math.nan, math.inf])
    else:
        c.carry = c.carry * rng.choice([math.nan, 1e300])
    try:
        G.calibrate_leverage(c)
        raise SystemExit("calibration ran without a device")
    except G.ThothGpuError as e:
        assert e.code in ok_codes, e
        seen += 1
b = W.american_put(4096)
for _ in range(200):
    p = rng.choice([-1, 0, 1, 5, 1 << 20])
    kw = dict(flags=rng.choice([0, 31, 1 << 20]), min_itm=rng.choice([0, -5, 10 ** 9]))
    if rng.random() < 0.3:
        kw["zero_rates"] = np.full(b.n_dates, rng.choice([0.01, math.nan]))
    try:
        G.price_american(b, p, **kw)
        raise SystemExit("American pricing ran without a device")
    except G.ThothGpuError as e:
        assert e.code in ok_codes, e
        seen += 1
    except ValueError:
        seen += 1
print("checked", seen)
'''


def test_calibration_and_american_inputs_are_checked_under_sanitizers(sanitized_env):
    p = subprocess.run([sys.executable, "-c", FUZZ_INPUTS], cwd=ROOT, env=sanitized_env, capture_output=True,
                       text=True, timeout=900)
    assert p.returncode == 0, p.stdout[-3000:] + p.stderr[-3000:]
    assert "ERROR: AddressSanitizer" not in p.stderr and "runtime error" not in p.stderr
    assert p.stdout.split() == ["checked", "500"]
