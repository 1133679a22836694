"""Host-side fault injection on the GPU: the engine's working-buffer allocations fail as on a
full device (thoth_gpu_debug_fail_allocations). Every entry point returns THOTH_GPU_E_NOMEM,
the engine stays usable, and later calls give the same results as before. Nothing here makes
the device fault: the failures are made on the host, before any allocation reaches CUDA.

After the hook drops the working buffers, each call stops at its first allocation, so k
injected failures fail exactly k calls.
"""
import ctypes as C

import numpy as np
import pytest

from thoth_gb300 import abi, workloads as W
from tests.test_gpu_american import vanilla_book

pytestmark = pytest.mark.gpu


def fails_then_recovers(gpu, call, k):
    gpu.debug_fail_allocations(k)
    try:
        for _ in range(k):
            with pytest.raises(gpu.ThothGpuError) as e:
                call()
            assert e.value.code == abi.THOTH_GPU_E_NOMEM, str(e.value)
        return call()
    finally:
        gpu.debug_fail_allocations(0)


@pytest.mark.parametrize("k", [1, 3])
def test_book_pricing_recovers_from_allocation_failures(gpu, k):
    b = W.heston_grid(paths=1 << 14)
    want = gpu.price_book(b)
    got = fails_then_recovers(gpu, lambda: gpu.price_book(b), k)
    np.testing.assert_array_equal(got["premium"], want["premium"])
    np.testing.assert_array_equal(got["trust"], want["trust"])


def test_american_and_calibration_recover_from_allocation_failures(gpu):
    b = vanilla_book(paths=1 << 14)
    want = gpu.price_american(b, 0, flags=abi.BUMP_DELTA)
    got = fails_then_recovers(gpu, lambda: gpu.price_american(b, 0, flags=abi.BUMP_DELTA), 2)
    assert got["premium"] == want["premium"] and got["delta"] == want["delta"]
    c = W.lsv_calibration(horizon_days=30, particles=2048)
    lev, _ = gpu.calibrate_leverage(c)
    lev2, _ = fails_then_recovers(gpu, lambda: gpu.calibrate_leverage(c), 1)
    np.testing.assert_array_equal(lev2, lev)


def test_batch_recovers_from_allocation_failures(gpu):
    books = [W.heston_grid(paths=1 << 12), W.gbm_call(paths=1 << 13, greeks=False), W.heston_grid(paths=3000)]
    want = gpu.price_batch(books)
    got = fails_then_recovers(gpu, lambda: gpu.price_batch(books), 2)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g["premium"], w["premium"])


def test_allocation_free_entry_point_is_unaffected(gpu):
    """thoth_gpu_price_book_noalloc uses no working buffer: it prices while every engine
    allocation would fail, and equals the allocating entry point."""
    b = W.heston_grid(paths=1 << 13)
    want = gpu.price_book(b)
    lib = gpu.lib()
    lib.thoth_gpu_price_book_noalloc.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBookResult)]
    gpu.debug_fail_allocations(1000)
    try:
        d = b.desc()
        r, arrs = b.result()
        assert lib.thoth_gpu_price_book_noalloc(C.byref(d), C.byref(r)) == abi.THOTH_GPU_OK
        np.testing.assert_allclose(arrs["premium"], want["premium"], rtol=1e-4, atol=1e-5)
        with pytest.raises(gpu.ThothGpuError) as e:
            gpu.price_book(b)
        assert e.value.code == abi.THOTH_GPU_E_NOMEM
    finally:
        gpu.debug_fail_allocations(0)
    np.testing.assert_array_equal(gpu.price_book(b)["premium"], want["premium"])
