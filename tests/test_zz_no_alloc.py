"""The allocation-free entry point, thoth_gpu_price_book_noalloc.

It serves callers that may not allocate device memory, such as a host whose
device memory is budgeted before pricing starts, or a framework that owns
every allocation on the GPU. Its scratch is one static 2 MiB device array, so
these checks call it through the C ABI, twice in a row, and compare each result
with the regular allocating entry point on the same book. The file is named to
be collected last, so a run that stops at the first failure has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from thoth_gb300 import abi, workloads as W
from tests.golden.make_golden import mixed_book

pytestmark = pytest.mark.gpu

# the same tolerance the parity tests use for prices on shared paths
REL, ABS = 1e-4, 1e-5


def _noalloc(G, book):
    lib = G.lib()
    lib.thoth_gpu_price_book_noalloc.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBookResult)]
    d = book.desc()
    r, arrs = book.result()
    rc = lib.thoth_gpu_price_book_noalloc(C.byref(d), C.byref(r))
    if rc != abi.THOTH_GPU_OK:
        raise G.ThothGpuError(rc, lib.thoth_gpu_last_error().decode())
    return dict(book_premium=r.book_premium, book_trust=r.book_trust, premium=arrs["premium"].copy(),
                trust=arrs["trust"].copy())


@pytest.mark.parametrize("make", [lambda: W.heston_grid(paths=1 << 16, calendar=True),
                                  lambda: mixed_book(paths=1 << 13),
                                  lambda: W.gbm_call(paths=1 << 18, greeks=False)])
def test_noalloc_matches_allocating_entry_point_twice(gpu, make):
    book = make()
    ref = gpu.price_book(book)
    for _ in range(2):  # the second call reuses the static array left by the first
        got = _noalloc(gpu, book)
        np.testing.assert_allclose(got["premium"], ref["premium"], rtol=REL, atol=ABS)
        np.testing.assert_allclose(got["trust"], ref["trust"], rtol=1e-3, atol=1e-9)
        assert abs(got["book_premium"] - ref["book_premium"]) <= REL * abs(ref["book_premium"]) + ABS


def test_noalloc_rejects_books_beyond_its_array(gpu):
    # 8 names over 8190 daily steps: 3 MiB of per-step constants alone, more than the 2 MiB array
    book = abi.Book(days=np.arange(0, 8191), paths=1000)
    for k in range(8):
        a = book.add_gbm(100.0 + k, 0.2, 0.0)
        book.add_vanilla(a, 100.0, 8190)
    with pytest.raises(gpu.ThothGpuError) as e:
        _noalloc(gpu, book)
    assert e.value.code == abi.THOTH_GPU_E_TOO_LARGE
    assert "allocation-free" in str(e.value)
