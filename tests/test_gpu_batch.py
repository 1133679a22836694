"""Ragged batches and the autotuner on the GPU.

The batch workload follows the ragged-book mix (40% GBM, 40% Heston, 20% LSV;
vanilla / barrier / variance payoffs; ragged path and step counts) at reduced
path counts, so the oracle prices every book in seconds. Every book is checked
against the oracle on the same Sobol paths (0.5 SE and 1e-4 relative), and the
batch graph against one-at-a-time pricing (bit-identical at equal grids).
"""
import os

import numpy as np
import pytest

import oracle
from thoth_gb300 import abi, workloads as W
from tests.test_gpu_parity import assert_shared_path_parity, leg_scale

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def small_batch(n=32, seed=11):
    return W.ragged_books(n_books=n, seed=seed, min_paths=1 << 9, max_paths=1 << 14, min_steps=12, max_steps=120)


@pytest.fixture(autouse=True)
def untuned(gpu):
    gpu.autotune_clear()
    yield
    gpu.autotune_clear()


def test_every_book_of_a_ragged_batch_vs_oracle(gpu):
    books = small_batch()
    res = gpu.price_batch(books)
    assert len(res) == len(books)
    for i, (b, r) in enumerate(zip(books, res)):
        ref = oracle.price_book(b, threads=THREADS)
        assert_shared_path_parity(r, ref["premium"], ref["trust"], "book %d" % i)
        assert abs(r["book_premium"] - ref["book_premium"]) <= 0.5 * ref["book_trust"] + 1e-4 * abs(ref["book_premium"])


def test_long_books_with_lsv_barriers_vs_oracle(gpu):
    """Step counts up to the workload's 730 daily steps, every model, and LSV books with
    daily-monitored barriers (down-and-out call, up-and-in put) among them: every book of
    the batch against the oracle on the same Sobol paths."""
    books = W.ragged_books(n_books=12, seed=29, min_paths=1 << 10, max_paths=1 << 12, min_steps=600,
                           max_steps=730)
    books += W.ragged_books(n_books=6, seed=31, min_paths=1 << 10, max_paths=1 << 12, min_steps=700,
                            max_steps=730, model_mix=(0.0, 0.0, 1.0), payoffs=(1,))
    assert max(len(b.days) - 1 for b in books) >= 725
    assert sum(b.assets[0]["model"] == abi.MODEL_LSV and b.products[0]["kind"] == abi.BARRIER for b in books) >= 6
    res = gpu.price_batch(books)
    for i, (b, r) in enumerate(zip(books, res)):
        ref = oracle.price_book(b, threads=THREADS)
        sc = leg_scale(b)
        assert_shared_path_parity(r, ref["premium"], ref["trust"], "book %d (%d steps)" % (i, len(b.days) - 1),
                                  scale=sc)
        assert abs(r["book_premium"] - ref["book_premium"]) <= (0.5 * ref["book_trust"] +
                                                                1e-4 * max(abs(ref["book_premium"]), sc.sum()))


@pytest.mark.parametrize("persistent", [True, False])
def test_batch_equals_one_at_a_time(gpu, persistent):
    """Work item r of a book in the persistent launch is CTA r's share of the book's own
    launch: every book's sums are bit for bit those of pricing it alone, in either mode."""
    books = small_batch(n=20, seed=3)
    gpu.set_batch_persistent(persistent)
    try:
        res = gpu.price_batch(books)
        assert gpu.batch_launches() == (3 if persistent else 3 * len(books))
    finally:
        gpu.set_batch_persistent(True)
    for b, r in zip(books, res):
        one = gpu.price_book(b)
        np.testing.assert_array_equal(r["premium"], one["premium"])
        np.testing.assert_array_equal(r["trust"], one["trust"])
        assert r["book_premium"] == one["book_premium"]


def test_persistent_launch_with_books_it_does_not_run(gpu):
    """Multi-asset books (correlated GBM names, LSV and Heston names in turn) beside single-asset
    books of every model: the single-asset books share the persistent launch, the others
    get their own launches meanwhile; every book equals its own pricing bit for bit, and
    long LSV books with daily barriers among them match the oracle on shared paths."""
    books = small_batch(n=14, seed=17)
    books += W.ragged_books(n_books=3, seed=41, min_paths=1 << 10, max_paths=1 << 11, min_steps=400,
                            max_steps=500, model_mix=(0.0, 0.0, 1.0), payoffs=(1,))
    two = abi.Book(days=np.arange(0, 61), paths=3000)   # two independent Heston names: assets in turn
    h0 = two.add_heston(100.0, 0.05, 2.0, 0.05, 0.5, -0.6, 0.02)
    h1 = two.add_heston(80.0, 0.04, 1.5, 0.04, 0.7, -0.7, 0.01)
    two.add_vanilla(h0, 100.0, 60, abi.CALL, zero_rate=0.02)
    two.add_vanilla(h1, 80.0, 40, abi.PUT, zero_rate=0.02)
    pair = abi.Book(days=np.arange(0, 31), paths=2500)  # two correlated GBM names: the mixed kernel
    g0 = pair.add_gbm(100.0, 0.25, 0.02)
    g1 = pair.add_gbm(90.0, 0.30, 0.01)
    pair.set_cholesky(np.linalg.cholesky(np.array([[1.0, 0.5], [0.5, 1.0]])))
    pair.add_basket([g0, g1], [0.5, 0.5], 95.0, 30, zero_rate=0.02)
    multi = [W.lsv_book(paths=2000), pair, two]
    assert [gpu.plan_summary(m)["variant"] for m in multi] == [6, 3, 6]
    books[3:3] = multi
    res = gpu.price_batch(books)
    assert gpu.batch_launches() == 3 + len(multi)
    for i, (b, r) in enumerate(zip(books, res)):
        one = gpu.price_book(b)
        np.testing.assert_array_equal(r["premium"], one["premium"], err_msg="book %d" % i)
        assert r["book_premium"] == one["book_premium"]
    for i in range(len(books) - 3, len(books)):
        ref = oracle.price_book(books[i], threads=THREADS)
        assert_shared_path_parity(res[i], ref["premium"], ref["trust"], "LSV barrier book %d" % i,
                                  scale=leg_scale(books[i]))


def test_graph_is_replayed_while_shapes_repeat(gpu):
    books = small_batch(n=12, seed=5)
    first = gpu.price_batch(books)
    assert gpu.batch_graph_replays() == 0
    again = gpu.price_batch(books)
    assert gpu.batch_graph_replays() == 1
    for a, b in zip(first, again):
        np.testing.assert_array_equal(a["premium"], b["premium"])
    # a changed parameter is a changed kernel argument: the graph is captured again
    i = next(k for k, b in enumerate(books) if b.products[0]["kind"] == abi.VANILLA)
    books[i].assets[0]["spot"] = 105.0
    changed = gpu.price_batch(books)
    assert gpu.batch_graph_replays() == 0
    one = gpu.price_book(books[i])
    np.testing.assert_array_equal(changed[i]["premium"], one["premium"])
    assert not np.array_equal(changed[i]["premium"], first[i]["premium"])


@pytest.mark.parametrize("streams", [1, 3, 16])
def test_stream_count_does_not_change_results(gpu, streams):
    books = small_batch(n=10, seed=9)
    base = gpu.price_batch(books)
    gpu.set_batch_streams(streams)
    other = gpu.price_batch(books)
    for a, b in zip(base, other):
        np.testing.assert_array_equal(a["premium"], b["premium"])


def test_empty_and_invalid_batches(gpu):
    assert gpu.price_batch([]) == []
    books = small_batch(n=4, seed=1)
    books[2].paths = 1                       # invalid: paths must be > 1
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.price_batch(books)
    assert e.value.code == abi.THOTH_GPU_E_INVALID and "book 2" in str(e.value)
    books[2].paths = 1000
    assert len(gpu.price_batch(books)) == 4  # the engine is still usable


@pytest.mark.parametrize("make", [
    lambda: W.heston_grid(paths=1 << 16, calendar=True, months=(1, 3, 6), strikes=(90, 100, 110)),
    lambda: W.gbm_call(paths=1 << 15)])
def test_autotune_book_keeps_parity(gpu, make, tmp_path):
    b = make()
    t = gpu.autotune_book(b, reps=2)
    # every launch shape (paths per thread x tile size) and grid was timed; the default is among them
    assert t["candidates"] >= 8 and 1 <= t["grid"]
    assert t["shape"] in (0, 1, 2, 3, 4) and t["threads"] in (64, 128, 256) and t["tile_paths"] in (128, 256)
    assert t["best_ms"] <= t["default_ms"] * (1 + 1e-9)
    plan = gpu.plan_summary(b)
    assert plan["shape"] == t["shape"] and plan["threads"] == t["threads"] and plan["tile"] == t["tile_paths"]
    r = gpu.price_book(b, greeks=b.greeks != 0)
    ref = oracle.price_book(b, threads=THREADS)
    assert_shared_path_parity(r, ref["premium"], ref["trust"], "tuned shape %d grid %d" % (t["shape"], t["grid"]))
    # the choice survives a save / clear / load round trip
    path = tmp_path / "tune.txt"
    gpu.autotune_save(path)
    assert any(line.startswith("book ") for line in path.read_text().splitlines())
    gpu.autotune_clear()
    assert gpu.plan_summary(b)["shape"] == 0
    gpu.autotune_load(path)
    assert gpu.plan_summary(b)["shape"] == t["shape"]
    again = gpu.price_book(b, greeks=b.greeks != 0)
    np.testing.assert_array_equal(again["premium"], r["premium"])


@pytest.mark.parametrize("variant,shape_paths", [(1, (1 << 13) + 77), (1, 1 << 15), (6, (1 << 12) + 5)])
def test_every_launch_shape_matches_the_oracle(gpu, variant, shape_paths, tmp_path):
    """Force each launch shape through an autotune file and check parity on shared paths:
    variant 1 a Heston calendar grid, variant 6 the multi-asset LSV book (assets in turn)."""
    import math
    if variant == 1:
        b = W.heston_grid(paths=shape_paths, calendar=True, months=(1, 2), strikes=(90, 100, 110))
    else:
        b = W.lsv_book(paths=shape_paths)
    assert gpu.plan_summary(b)["variant"] in (variant, 4)
    n = b.desc().n_dates - 1
    key = "book %d %d %d" % (variant, math.ceil(math.log2(shape_paths)), math.ceil(math.log2(n)))
    base = tmp_path / "base.txt"
    gpu.autotune_save(base)                 # header lines of this device, nothing tuned
    ref = oracle.price_book(b, threads=THREADS)
    for shape in range(5):
        f = tmp_path / ("s%d.txt" % shape)
        f.write_text(base.read_text() + "%s %d 0 0\n" % (key, shape))
        gpu.autotune_clear()
        gpu.autotune_load(f)
        assert gpu.plan_summary(b)["shape"] == shape
        r = gpu.price_book(b)
        assert_shared_path_parity(r, ref["premium"], ref["trust"], "shape %d" % shape)


def test_autotune_batch_save_load(gpu, tmp_path):
    books = small_batch(n=16, seed=21)
    t = gpu.autotune_batch(books, reps=1)
    assert t["streams"] in (1, 2, 4, 8, 16) and t["policy"] in (0, 1, 2) and t["shape"] in (-1, 0, 1, 2, 3, 4)
    assert t["persistent"] in (0, 1) and (t["shape"] == -1 or not t["persistent"])
    assert t["candidates"] >= 13
    assert t["best_ms"] <= t["default_ms"] * (1 + 1e-9)
    path = tmp_path / "tune.txt"
    gpu.autotune_save(path)
    text = path.read_text().splitlines()
    assert text[0] == "thoth-autotune 1"
    assert text[2] == "batch %d %d %d %d" % (t["streams"], t["policy"], t["shape"], t["persistent"])
    tuned = gpu.price_batch(books)
    gpu.autotune_clear()
    gpu.autotune_load(path)
    loaded = gpu.price_batch(books)
    for a, b in zip(tuned, loaded):
        np.testing.assert_array_equal(a["premium"], b["premium"])
    # every book still matches the oracle under the tuned grids
    for i in (0, 7, 15):
        ref = oracle.price_book(books[i], threads=THREADS)
        assert_shared_path_parity(loaded[i], ref["premium"], ref["trust"], "tuned book %d" % i)
    # a file from another device is refused, a malformed one too
    other = tmp_path / "other.txt"
    other.write_text("thoth-autotune 1\ndevice 7 Some Other GPU\nbatch 4 0\n")
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.autotune_load(other)
    assert e.value.code == abi.THOTH_GPU_E_UNSUPPORTED
    bad = tmp_path / "bad.txt"
    bad.write_text("thoth-autotune 1\nbatch -3 9\n")
    with pytest.raises(gpu.ThothGpuError) as e:
        gpu.autotune_load(bad)
    assert e.value.code == abi.THOTH_GPU_E_INVALID
