"""The allocation-free entry point, thoth_gpu_price_book_noalloc.

It serves callers that may not allocate device memory, such as a host whose
device memory is budgeted before pricing starts, or a framework that owns
every allocation on the GPU. Its scratch is one static 2 MiB device array, so
these checks call it through the C ABI, twice in a row, and compare each result
with the regular allocating entry point and with the oracle on the same book.
They also price with every allocation of the engine's allocators made to fail,
and make it the first call of a fresh process, before anything has set the
engine up. The file is named to be collected last, so a run that stops at the
first failure has already run every other test; it also passes alone in a fresh
process.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from thoth_gb300 import abi, workloads as W
from tests.golden.make_golden import mixed_book
from tests.test_gpu_parity import assert_shared_path_parity

pytestmark = pytest.mark.gpu

# the same tolerance the parity tests use for prices on shared paths
REL, ABS = 1e-4, 1e-5
THREADS = max(1, min(16, os.cpu_count() or 1))
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


BOOKS = [lambda: W.heston_grid(paths=1 << 16, calendar=True),
         lambda: mixed_book(paths=1 << 13),
         lambda: W.gbm_call(paths=1 << 18, greeks=False)]


@pytest.mark.parametrize("make", BOOKS)
def test_noalloc_matches_allocating_entry_point_and_oracle_twice(gpu, make):
    book = make()
    ref = gpu.price_book(book)
    orc = oracle.price_book(book, threads=THREADS)
    for _ in range(2):  # the second call reuses the static array left by the first
        got = _noalloc(gpu, book)
        np.testing.assert_allclose(got["premium"], ref["premium"], rtol=REL, atol=ABS)
        np.testing.assert_allclose(got["trust"], ref["trust"], rtol=1e-3, atol=1e-9)
        assert abs(got["book_premium"] - ref["book_premium"]) <= REL * abs(ref["book_premium"]) + ABS
        # and directly against the oracle on the same Sobol paths
        assert_shared_path_parity(got, orc["premium"], orc["trust"], "noalloc")
        assert abs(got["book_premium"] - orc["book_premium"]) <= (0.5 * orc["book_trust"] +
                                                                  REL * abs(orc["book_premium"]) + ABS)


def test_noalloc_prices_while_every_engine_allocation_fails(gpu):
    """With the engine's working buffers dropped and every allocation through its
    allocators made to fail, the allocating entry point reports NOMEM and this one still
    prices, with the same results."""
    book = W.heston_grid(paths=1 << 15, calendar=True)
    ref = gpu.price_book(book)
    gpu.debug_fail_allocations(1 << 30)
    try:
        with pytest.raises(gpu.ThothGpuError) as e:
            gpu.price_book(book)
        assert e.value.code == abi.THOTH_GPU_E_NOMEM
        for _ in range(2):
            got = _noalloc(gpu, book)
            np.testing.assert_allclose(got["premium"], ref["premium"], rtol=REL, atol=ABS)
    finally:
        gpu.debug_fail_allocations(0)


FIRST_CALL = r"""
import ctypes as C, json, sys
sys.path.insert(0, %r)
import numpy as np
import thoth_gb300 as G
from thoth_gb300 import abi, workloads as W
book = W.heston_grid(paths=1 << 14, calendar=True, months=(1, 3, 12), strikes=(90, 100, 110))
lib = G.lib()
lib.thoth_gpu_price_book_noalloc.argtypes = [C.POINTER(abi.ThothBookDesc), C.POINTER(abi.ThothBookResult)]
out = []
for _ in range(2):
    d = book.desc()
    r, arrs = book.result()
    rc = lib.thoth_gpu_price_book_noalloc(C.byref(d), C.byref(r))
    out.append(dict(rc=rc, premium=arrs["premium"].tolist(), trust=arrs["trust"].tolist()))
# the engine (which allocates) was never set up by these calls
out.append(dict(cancel_rc=lib.thoth_gpu_request_cancel()))
print(json.dumps(out))
""" % ROOT


def test_noalloc_as_the_first_call_of_a_fresh_process(gpu):
    """In a process that has made no other call into the library (no engine, no arena), the
    first two calls price through the static array alone and match the oracle."""
    p = subprocess.run([sys.executable, "-c", FIRST_CALL], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert p.returncode == 0, p.stderr
    import json
    res = json.loads(p.stdout.strip().splitlines()[-1])
    book = W.heston_grid(paths=1 << 14, calendar=True, months=(1, 3, 12), strikes=(90, 100, 110))
    orc = oracle.price_book(book, threads=THREADS)
    for call in res[:2]:
        assert call["rc"] == abi.THOTH_GPU_OK
        assert_shared_path_parity({"premium": np.array(call["premium"])}, orc["premium"], orc["trust"], "first call")
    assert res[2]["cancel_rc"] == abi.THOTH_GPU_E_NODEVICE


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
