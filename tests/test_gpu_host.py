"""The C++ drop-in (namespace gpu over the C ABI, thoth_gb300/host) on the GPU:
the reference's PriceEuropeanGbm call shape, a whole book, and the ERR path."""
import math
import os
import subprocess

import pytest

import oracle

pytestmark = pytest.mark.gpu
EXE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "thoth_gb300", "_build", "host_check")


def test_cpp_dropin(gpu):
    out = subprocess.run([EXE], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in out.stdout.splitlines() if ln}
    prem, trust = (float(v) for v in lines["gbm"])
    bs = oracle.bs_price(100 * math.exp(0.02), 100, 1.0, 0.25, math.exp(-0.03))
    assert abs(prem - bs) < 3 * trust
    call, put, book, book_trust = (float(v) for v in lines["book"])
    parity = math.exp(-0.03) * (100 * math.exp(0.02) - 100)                      # df (F - K)
    assert abs((call - put) - parity) < 3 * book_trust + 1e-3
    assert "error" in lines and "paths must be > 1" in out.stdout
    am, euro, delta = (float(v) for v in lines["american"])
    assert am > euro > 0 and -1.0 < delta < 0.0                            # early exercise pays for a put
    lo, hi = (float(v) for v in lines["calib"])
    assert 0.5 < lo <= hi < 3.0                                            # about 0.25 / 0.20


def test_peak_microbenchmarks_are_plausible(gpu):
    """The roofline denominators the benchmark measures in its own run: FP32 FMA and
    special-function throughput of one GB300 (152 SMs, at most 2.07 GHz)."""
    tf = gpu.measure_fp32_peak()
    assert 20.0 < tf < 90.0           # 152 x 128 lanes x 2 flops x clock
    gops = gpu.measure_mufu_peak()
    assert 500.0 < gops < 25000.0     # 152 SMs x (16 .. 64) ops a clock x clock
