"""Benchmark: Heston vanilla grid on one GB300.

Workload (the engine's headline configuration): one Heston underlying
(kappa 1.5, theta 0.04, xi 0.6, rho -0.7, v0 0.04, S0 100, r 0.03, q 0), 9 strikes
80..120 x 7 maturities 1,2,3,4,5,12,24 months x call/put = 126 cells priced on
shared paths; 2^20 Sobol paths with Brownian bridge (2 dimensions per step),
252 steps a year (504 steps to 24 months), FP32 path state, FP64 reductions.

metric: path-steps per second (paths x steps / time) of the whole job.
  value  device time of the pricing kernels with the plan resident in HBM
         (CUDA events on the engine's stream; L2 flushed before every step)
  e2e    the reference-facing C-ABI call thoth_gpu_price_book from host
         descriptors: plan build, host->device copy, kernels, device->host copy
Run: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun each rank prices its own disjoint Sobol block (weak scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PATHS = 1 << 20
STEPS_PER_YEAR = 252
FLOPS_PER_PATH_STEP = 96  # algorithmic FP32 flops of a Heston-QE + Andersen path-step (FMA = 2)
MUFU_PER_PATH_STEP = 8  # algorithmic special-function ops of the same path-step (rcp, sqrt, ...)
# DRAM bytes per launch of the book kernel from the ncu capture summarised in
# profiles/book_kernel_heston_grid.md (a 2^18-path capture; the traffic is the
# plan, the Sobol tables and the per-CTA sums, which do not grow with paths)
NCU_DRAM_BYTES_PER_LAUNCH = 1268224


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="thoth", choices=["thoth", "reference"])
    ap.add_argument("--cpu-sample-paths", type=int, default=1 << 18)
    ap.add_argument("--paths", type=int, default=PATHS, help="paths of the headline workload (default 2^20)")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate-vs-plain-MC grid section")
    ap.add_argument("--no-batch", action="store_true", help="skip the ragged-batch (256 books) section")
    ap.add_argument("--no-lsv", action="store_true", help="skip the multi-asset LSV book section")
    ap.add_argument("--no-paths", action="store_true", help="skip the stored-paths (HBM) section")
    ap.add_argument("--no-american", action="store_true", help="skip the American (Longstaff-Schwartz) section")
    ap.add_argument("--no-calibration", action="store_true", help="skip the LSV leverage calibration section")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def workload(rank=0, paths=PATHS):
    from thoth_gb300 import workloads as W
    b = W.heston_grid(paths=paths, steps_per_year=STEPS_PER_YEAR)
    b.sobol_skip = rank * paths  # disjoint Sobol block per rank
    return b


def config(world, paths=PATHS):
    return {"workload": "heston_vanilla_grid", "paths": paths, "steps": 2 * STEPS_PER_YEAR,
            "steps_per_year": STEPS_PER_YEAR, "cells": 126, "strikes": "80..120 step 5",
            "maturities_months": [1, 2, 3, 4, 5, 12, 24], "sobol_dims": 1008, "brownian_bridge": True,
            "parallelism": "dp%d" % world if world > 1 else "single",
            "l2": "flushed (256 MiB write) before every timed step"}


class Clocks:
    """nvidia-smi samples (200 ms) while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once sampling is live (the first sample is in)
            t0 = time.perf_counter()
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def mark(self):
        """The count of samples so far: summary(since=mark()) keeps the later ones."""
        return len(self.lines)

    def summary(self, since=0):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[since:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(sample_paths, threads):
    """The oracle (CPU restatement of the reference's node graph) on a bounded sample."""
    import oracle
    from thoth_gb300 import workloads as W
    b = W.heston_grid(paths=sample_paths, steps_per_year=STEPS_PER_YEAR)
    t0 = time.perf_counter()
    oracle.price_book(b, "port", threads=threads)
    dt = time.perf_counter() - t0
    n_steps = 2 * STEPS_PER_YEAR
    return {"value": sample_paths * n_steps / dt, "unit": "path-steps/s", "cores": threads, "kind": "port",
            "sample": "%d paths x %d steps of the same Heston grid (126 cells), %d threads, %.2f s"
                      % (sample_paths, n_steps, threads, dt)}


def one_core_baseline(sample_paths=1 << 13):
    """The same oracle on one thread: the single-core figure beside the all-core one."""
    c = cpu_baseline(sample_paths, 1)
    return {"value": c["value"], "unit": c["unit"], "cores": 1, "sample": c["sample"]}


def run_reference(args):
    """The reference's CPU Monte-Carlo (its node-graph arithmetic, restated bit for bit in
    oracle/thoth_oracle.c) on all host cores. Every step, warm-up included, prices the whole
    workload of this arm's config: the 126-cell Heston grid on 2^20 paths x 504 steps (--paths),
    about 2 s on 16 Arm cores. ms_per_step is the mean wall time of the timed steps."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    threads = os.cpu_count() or 1
    n_steps = 2 * STEPS_PER_YEAR
    book = workload(0, args.paths)
    for _ in range(args.warmup):
        oracle.price_book(book, "port", threads=threads)
    secs = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.price_book(book, "port", threads=threads)
        secs.append(time.perf_counter() - t0)
    wall = time.perf_counter() - t_all
    ms = 1e3 * sum(secs) / len(secs)
    v = args.paths * n_steps / (ms * 1e-3)
    line = {"metric": "path-steps/sec", "value": v, "unit": "path-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(world, args.paths),
            "cpu_baseline": {"value": v, "unit": "path-steps/s", "cores": threads, "kind": "port",
                             "sample": "the whole workload every step: %d paths x %d steps, 126 cells, %d threads"
                                       % (args.paths, n_steps, threads),
                             "one_core": one_core_baseline()},
            "e2e": {"value": v, "unit": "path-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s_timed_region": wall,
            "note": "the reference's CPU Monte-Carlo restated bit for bit in oracle/thoth_oracle.c (kind port: "
                    "the build of the reference's own sources needs its checkout, which the GPU host does not "
                    "have), all host threads, "
                    "each step the full workload of config"}
    if world > 1:
        line["note"] += "; at N > 1 rank 0 prices one rank's path block (the host's cores do not grow with N)"
    print(json.dumps(line), flush=True)


def lsv_book_section(G, flush, steps):
    """The multi-asset LSV book: 5 correlated-currency LSV names (Heston base + leverage
    surface), 20 daily-monitored down-and-out calls, 10 variance swaps, 20 basket calls,
    2^20 paths x 365 daily steps; plan resident, L2 flushed before every run."""
    import numpy as np
    import torch
    from thoth_gb300 import workloads as W
    book = W.lsv_book(paths=1 << 20)
    n_steps, n_assets = len(book.days) - 1, len(book.assets)
    res = G.ResidentBook(book)
    for _ in range(2):
        res.run()
    ms = []
    for _ in range(max(2, steps // 2)):
        flush.fill_(1)
        torch.cuda.synchronize()
        ms.append(res.run()["device_ms"])
    res.close()
    t0 = time.perf_counter()
    r = G.price_book(book)
    e2e_s = time.perf_counter() - t0
    dev = float(np.mean(ms))
    work = float(book.paths) * n_steps * n_assets
    plan = G.plan_summary(book)
    # the same book with its correlation matrix acting on the LSV spots as well (an extension:
    # the reference correlates only GBM spots); all names in one pass (mixed kernel)
    book.correlate_all_spots = True
    res = G.ResidentBook(book)
    for _ in range(2):
        res.run()
    msc = []
    for _ in range(max(2, steps // 2)):
        flush.fill_(1)
        torch.cuda.synchronize()
        msc.append(res.run()["device_ms"])
    rc = res.run()
    res.close()
    devc = float(np.mean(msc))
    return {"workload": "lsv_book: 5 LSV assets, 50 products (barrier / variance / basket), 2^20 paths x 365 steps",
            "asset_path_steps_per_sec": work / (dev * 1e-3), "device_ms": dev,
            "e2e_asset_path_steps_per_sec": work / e2e_s, "plan": plan,
            "book_premium": r["book_premium"], "book_trust": r["book_trust"],
            "correlated_spots": {"device_ms": devc, "asset_path_steps_per_sec": work / (devc * 1e-3),
                                 "book_premium": rc["book_premium"], "book_trust": rc["book_trust"],
                                 "plan": G.plan_summary(book),
                                 "note": "correlate_all_spots: the Cholesky factor drives the LSV spot noises too "
                                         "(no reference counterpart); the headline entry above is the reference's "
                                         "semantics, independent stochastic-vol spots"}}


def paths_section(G, flush):
    """The path-storing variant: every date's spot of every path written to HBM
    (date-major, coalesced), 2^20 paths; GBM on 252 daily steps and the Heston grid
    (504 steps). Rate against the measured HBM copy bandwidth."""
    import numpy as np
    import torch
    from thoth_gb300 import abi, workloads as W
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    gbm = abi.Book(days=np.arange(0, 253), paths=1 << 20)
    a = gbm.add_gbm(100.0, 0.25, 0.02)
    gbm.add_vanilla(a, 100.0, 252, abi.CALL, zero_rate=0.03)
    out = {}
    for name, book in (("gbm_252", gbm), ("heston_grid_504", W.heston_grid(paths=1 << 20))):
        G.simulate_paths(book, 0)
        ms = []
        for _ in range(3):
            flush.fill_(1)
            torch.cuda.synchronize()
            ms.append(G.simulate_paths(book, 0)[1])
        dev = float(np.median(ms))
        n_dates = book.desc().n_dates
        written = 4.0 * n_dates * book.paths
        out[name] = {"device_ms": dev, "bytes_written": written, "gbs": written / (dev * 1e-3) / 1e9,
                     "frac_of_measured_hbm": written / (dev * 1e-3) / 1e9 / hbm,
                     "path_steps_per_sec": book.paths * (n_dates - 1) / (dev * 1e-3)}
    out["note"] = ("spot of every date of every path stored to HBM by the book kernel; the kernel stays "
                   "FP32-issue bound, so the write rate is the step rate x 4 bytes")
    return out


def american_section(G, flush, steps):
    """American put by Longstaff-Schwartz on Heston paths: 2^20 paths, one year of daily
    exercise dates (365 path rows read by the fit), and the reference tests' size (300 000
    GBM paths, 30-day exercise grid). The fit kernel's rate in path-dates/s, the whole call
    (simulation, fit, copies) per the C ABI, the frozen-policy Greeks, and the oracle's fit
    on a 2^15-path sample of the same stored paths on one host core."""
    import numpy as np
    import torch
    from oracle import american as am
    from thoth_gb300 import abi, workloads as W

    out = {}
    cases = (("heston_daily_2^20", W.american_put(1 << 20)),
             ("gbm_30day_300000", W.american_put(300000, heston=False)))
    for name, book in cases:
        G.price_american(book, 0)
        ex, dev, wall = [], [], []
        for _ in range(max(3, steps // 2)):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = G.price_american(book, 0)
            wall.append(time.perf_counter() - t0)
            ex.append(r["exercise_ms"])
            dev.append(r["device_ms"])
        rows = book.n_dates - 1
        units = float(book.paths) * rows
        fit_ms, e2e_ms = float(np.median(ex)), 1e3 * float(np.median(wall))
        out[name] = {"paths": book.paths, "exercise_dates": rows, "premium": r["premium"], "trust": r["trust"],
                     "european": r["european"], "fitted_dates": r["fitted_dates"],
                     "fit_kernel_ms": fit_ms, "fit_path_dates_per_sec": units / (fit_ms * 1e-3),
                     "simulate_and_fit_device_ms": float(np.median(dev)),
                     "e2e_ms": e2e_ms, "e2e_path_dates_per_sec": units / (e2e_ms * 1e-3),
                     "fit_read_gbs": 4.0 * units / (fit_ms * 1e-3) / 1e9}
    # a grid of 27 American puts on one Heston name (9 strikes x 3 maturities, daily exercise):
    # one batched fit, one regression round a date for all of them, against one call each
    grid = abi.Book(days=np.arange(0, 366), paths=1 << 18)
    hh = grid.add_heston(100.0, 0.04, 1.5, 0.04, 0.6, -0.7, 0.03)
    for K in range(80, 121, 5):
        for mty in (91, 182, 365):
            grid.add_vanilla(hh, float(K), mty, abi.PUT, zero_rate=0.03)
    idx = list(range(len(grid.products)))
    G.price_american_book(grid, idx)
    t0 = time.perf_counter()
    rg = G.price_american_book(grid, idx)
    t_book = time.perf_counter() - t0
    t0 = time.perf_counter()
    for i in idx:
        G.price_american(grid, i)
    t_one = time.perf_counter() - t0
    out["heston_grid_27_puts_2^18"] = {"contracts": len(idx), "book_call_ms": 1e3 * t_book,
                                        "book_call_device_ms": rg[0]["device_ms"],
                                        "one_call_each_ms": 1e3 * t_one, "speedup": t_one / t_book}
    book = cases[0][1]
    t0 = time.perf_counter()
    g = G.price_american(book, 0, flags=abi.BUMP_DELTA | abi.BUMP_GAMMA | abi.BUMP_VEGA | abi.BUMP_RHO |
                         abi.BUMP_THETA)
    out["heston_daily_2^20"]["greeks"] = {k: g[k] for k in ("delta", "gamma", "vega", "rho", "theta")}
    out["heston_daily_2^20"]["greeks_wall_ms"] = 1e3 * (time.perf_counter() - t0)
    out["heston_daily_2^20"]["greeks_device_ms"] = g["device_ms"]
    # CPU: the oracle (numpy, exact sums, one core) on the first 2^15 stored paths
    sample = W.american_put(1 << 15)
    S, _ = G.simulate_paths(sample, 0)
    t0 = time.perf_counter()
    o = am.fit(S, sample.t, np.full(sample.n_dates, 0.03), 100.0, False, 100.0)
    cpu_s = time.perf_counter() - t0
    cpu_rate = float(sample.paths) * (sample.n_dates - 1) / cpu_s
    out["cpu_baseline"] = {"value": cpu_rate, "unit": "path-dates/s", "cores": 1, "kind": "port",
                           "sample": "oracle.american.fit on 2^15 Heston paths x 365 daily exercise dates "
                                     "(%.2f s)" % cpu_s,
                           "gpu_equals_oracle_on_sample": bool(G.price_american(sample, 0)["premium"] == o["premium"])}
    out["note"] = ("fit = one cooperative launch, one publish/reduce/release per exercise date; FP64-issue and "
                   "latency bound (GB300 runs FP64 at 1/64 of FP32): the paths are read once (fit_read_gbs)")
    return out


def calibration_section(G):
    """LSV leverage calibration by the reference's particle method for one name: 365 daily
    layers of 201 points, 16 384 particles (the reference's count) and 2^18; the oracle (C
    restatement of the reference's loop, one host core) on the 16 384-particle case."""
    import numpy as np
    import oracle
    from thoth_gb300 import workloads as W
    out = {}
    L = None
    for P in (16384, 1 << 18):
        c = W.lsv_calibration(horizon_days=365, particles=P)
        G.calibrate_leverage(c)
        dev, wall = [], []
        for _ in range(3):
            t0 = time.perf_counter()
            lev, ms = G.calibrate_leverage(c)
            wall.append(time.perf_counter() - t0)
            dev.append(ms)
        if P == 16384:
            L = lev
        d = float(np.median(dev))
        out["particles_%d" % P] = {"device_ms": d, "e2e_ms": 1e3 * float(np.median(wall)),
                                   "particle_steps_per_sec": P * 365 / (d * 1e-3), "layers": 366, "points": 201}
    c = W.lsv_calibration(horizon_days=365)
    t0 = time.perf_counter()
    ref = oracle.calibrate_leverage(c)
    cpu = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": 16384 * 365 / cpu, "unit": "particle-steps/s", "cores": 1, "kind": "port",
                           "sample": "oracle.calibrate_leverage: 16384 particles x 365 daily layers (%.3f s)" % cpu}
    out["max_rel_diff_vs_oracle"] = float(np.max(np.abs(L / ref - 1.0)))
    out["note"] = ("one cooperative launch, two exact publish-and-release rounds a date (extremes and sum of v, "
                   "then the bins); FP64-latency bound; the Rng stream is the reference's, jumped per particle")
    return out


def _first_paths(book, n):
    """A copy of `book` priced on its first n Sobol points (the same indices as the book's)."""
    import copy
    b = copy.copy(book)
    b.paths = int(n)
    return b


def batch_parity(G, books, check_paths=1 << 16):
    """Every book of a batch against the oracle: each book is re-priced on its first
    min(paths, check_paths) Sobol points, in one batch call together with the full books,
    and those premiums are compared with the oracle's on the same points (all host cores).
    A book fails where any product (or the book value) is further from the oracle than
    0.5 standard errors or 1e-4 relative + 1e-5, the bar of the GPU parity tests; for a
    variance swap the relative part applies to its variance leg, notional * strike variance,
    as its premium is the near-cancelling difference of two legs."""
    import numpy as np
    import oracle
    trunc = [_first_paths(b, min(b.paths, check_paths)) for b in books]
    t0 = time.perf_counter()
    res = G.price_batch(list(books) + trunc)[len(books):]
    gpu_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    failing, worst_se, worst_rel, t0 = [], 0.0, 0.0, time.perf_counter()
    for i, (b, r) in enumerate(zip(trunc, res)):
        ref = oracle.price_book(b, "port", threads=threads)
        g = np.append(r["premium"], r["book_premium"])
        o = np.append(ref["premium"], ref["book_premium"])
        se = np.append(ref["trust"], ref["book_trust"])
        leg = np.array([abs(p["notional"] * p["strike_variance"]) if p["kind"] == 2 else 0.0 for p in b.products])
        size = np.maximum(np.abs(o), np.append(leg, leg.sum()))
        err = np.abs(g - o)
        bad = (err > 0.5 * se + 1e-12) | (err > 1e-4 * size + 1e-5)
        if bad.any():
            failing.append(i)
        worst_se = max(worst_se, float(np.max(err / np.maximum(se, 1e-300))))
        worst_rel = max(worst_rel, float(np.max(err / (np.abs(o) + 1e-300))))
    return {"books_checked": len(books), "books_failing_parity": len(failing), "failing_books": failing[:16],
            "worst_error_in_se": worst_se, "worst_rel_error": worst_rel,
            "paths_per_book": "min(paths, %d): the book's first Sobol points" % check_paths,
            "bar": "every product and the book value within 0.5 SE and 1e-4 relative + 1e-5 of the oracle "
                   "(variance swaps: relative to the variance leg)",
            "path_steps_checked": float(sum(b.paths * (len(b.days) - 1) for b in trunc)),
            "batch_call_s": gpu_s, "oracle_s": time.perf_counter() - t0, "oracle_threads": threads}


def ragged_batch_section(G, steps):
    """256 ragged books (path counts log-uniform in [2^14, 2^22], 12..730 daily steps,
    40% GBM / 40% Heston / 20% LSV) priced as one CUDA graph: the single-asset books in one
    persistent launch (the default), the same batch with one launch per book, after the
    autotuner (which times both), and one book at a time for comparison."""
    import numpy as np
    from thoth_gb300 import workloads as W
    books = W.ragged_books()
    work = float(sum(b.paths * (len(b.days) - 1) for b in books))
    G.autotune_clear()

    def timed(k):
        ms, wall = [], []
        for _ in range(k):
            t0 = time.perf_counter()
            r = G.price_batch(books)
            wall.append(time.perf_counter() - t0)
            ms.append(r[0]["device_ms"])
        return float(np.mean(ms)), float(np.mean(wall)), r

    G.price_batch(books)                       # capture: one persistent launch
    untuned_ms, untuned_wall, pers_res = timed(max(1, steps // 2))
    pers_launches = G.batch_launches()
    G.set_batch_persistent(False)
    G.price_batch(books)                       # capture: one launch per book
    per_book_ms, _, per_res = timed(max(1, steps // 2))
    per_book_launches = G.batch_launches()
    G.set_batch_persistent(True)
    same = all(np.array_equal(a["premium"], b["premium"]) and a["book_premium"] == b["book_premium"]
               for a, b in zip(pers_res, per_res))
    t0 = time.perf_counter()
    tune = G.autotune_batch(books, reps=1)
    tune_s = time.perf_counter() - t0
    G.price_batch(books)                       # capture with the tuned configuration
    tuned_ms, tuned_wall, res = timed(max(2, steps // 2))
    launches = G.batch_launches()
    one_ms = 0.0
    for b in books:
        one_ms += G.price_book(b)["device_ms"]
    parity = batch_parity(G, books)
    G.autotune_clear()
    return {
        "workload": "256 ragged books: paths log-uniform [2^14, 2^22], steps uniform [12, 730], "
                    "40% GBM / 40% Heston / 20% LSV, vanilla / barrier / variance",
        "path_steps": work, "books": len(books),
        "path_steps_per_sec": work / (tuned_ms * 1e-3),
        "device_ms": tuned_ms, "e2e_ms": 1e3 * tuned_wall,
        "e2e_path_steps_per_sec": work / tuned_wall,
        "persistent_launch": {"device_ms": untuned_ms, "e2e_ms": 1e3 * untuned_wall,
                              "path_steps_per_sec": work / (untuned_ms * 1e-3), "gpu_launches": pers_launches,
                              "note": "every single-asset book's work items in one persistent kernel between one "
                                      "gather and one reduction"},
        "one_launch_per_book": {"device_ms": per_book_ms, "gpu_launches": per_book_launches,
                                "note": "gather, book kernel and reduction per book over 8 streams"},
        "modes_bit_identical": bool(same),
        "untuned_device_ms": untuned_ms, "one_book_at_a_time_device_ms": one_ms,
        "autotune": dict(tune, seconds=tune_s,
                         note="persistent launch (grid policy) against one launch per book (stream count, one "
                              "launch shape for the single-asset books, grid policy), timed on the batch graph"),
        "gpu_launches_per_batch": launches,
        "books_nonfinite": int(sum(not np.all(np.isfinite(r["premium"])) for r in res)),
        "parity": parity,
    }


def gbm_section(G, flush):
    """Config 1 (European call under GBM: S0 = K = 100, T = 1, sigma 0.25, r 0.03, q 0.01, one
    step) at 2^18 and 2^24 paths: this engine (Sobol, FP32 path, FP64 sums) beside the
    reference's own GPU kernel (gbm_kernel of pricer/src/tasks/mcl_gpu.cu, Philox, FP64),
    compiled unmodified for sm_103a. Device times by CUDA events (the engine's book kernel and
    reduction; the reference's kernel alone), whole calls by host wall time, and both prices
    against Black-Scholes."""
    import math
    import numpy as np
    import torch
    import oracle
    from thoth_gb300 import workloads as W
    F, K, T, vol, df = 100.0 * math.exp(0.02), 100.0, 1.0, 0.25, math.exp(-0.03)
    bs = oracle.bs_price(F, K, T, vol, df, True)
    ref = oracle.ref_gbm()
    out = {"black_scholes": bs, "reference_kernel": "built" if ref is not None else
           "not built (its staged sources or nvcc absent)"}
    for k in (18, 24):
        n = 1 << k
        res = G.ResidentBook(W.gbm_call(paths=n, greeks=False))
        for _ in range(3):
            res.run()
        dev = []
        for _ in range(10):
            flush.fill_(1)
            torch.cuda.synchronize()
            r = res.run()
            dev.append(r["device_ms"])
        res.close()
        G.price_european_gbm(F, K, T, vol, df, True, n)
        walls = []
        for _ in range(5):
            t0 = time.perf_counter()
            p_, tr = G.price_european_gbm(F, K, T, vol, df, True, n)
            walls.append(1e3 * (time.perf_counter() - t0))
        row = {"thoth": {"device_ms": float(np.median(dev)), "paths_per_sec": n / (np.median(dev) * 1e-3),
                         "call_ms": float(np.median(walls)), "premium": p_, "trust": tr}}
        if ref is not None:
            import ctypes as C
            pr, trr, ms = C.c_double(), C.c_double(), C.c_double()
            rc = ref.ref_gbm_kernel(F, K, T, vol, df, 1, n, 0, 10, C.byref(pr), C.byref(trr), C.byref(ms))
            calls = []
            for _ in range(5):
                cp, ct, cw = C.c_double(), C.c_double(), C.c_double()
                rc |= ref.ref_gbm_call(F, K, T, vol, df, 1, n, 0, C.byref(cp), C.byref(ct), C.byref(cw))
                calls.append(cw.value)
            row["reference"] = {"rc": rc, "kernel_ms": ms.value, "paths_per_sec": n / (ms.value * 1e-3),
                                "call_ms": float(np.median(calls)), "premium": pr.value, "trust": trr.value}
            row["kernel_speedup"] = ms.value / row["thoth"]["device_ms"]
        out["paths_2^%d" % k] = row
    out["note"] = ("the reference draws Philox normals in FP64 (curand_normal_double) and exponentiates in FP64; "
                   "this engine draws Sobol + FP32 inverse normal; both sum in FP64. Its device time covers the "
                   "book kernel and the fixed-order reduction; the reference's, its one kernel")
    return out


def surrogate_section(n_train=4096, n_eval=4096, train_paths=1 << 18, epochs=3000, lr=2e-3, batch=8192, cf_sets=64,
                      seed=1, plain_sets=512, members=4):
    """Learned Heston surrogate against plain GPU MC on a 4096-set x 252-cell grid (1.03M
    cells) at the same accuracy target, 90th-percentile cell error <= 1e-3 against the FP64
    Heston closed form (relative, floor 1% of spot):
      plain MC  every cell by MC (batched books) at the smallest power-of-two path count that
                meets the target on the closed-form sets, timed on plain_sets sets of the grid;
      pipeline  device inference of every cell + the MC judge (1% of the sets at the plain-MC
                path count, its own noise removed) + MC fallback of the buckets it flags, every
                stage run on every set it concerns and timed as run.
    The one-off labelling and training times, and the number of grids after which they are
    paid back, are reported beside the rates. Errors are measured against the closed form on
    cf_sets sets spread over the grid (the oracle's closed form is the checker).
    The surrogate is an ensemble of `members` networks of the configured architecture (each 7 ->
    4 x 128 SiLU -> 1, BF16), trained side by side on the same labels from their own
    initialisations and served as their mean; one member's error is reported beside it."""
    import numpy as np
    import oracle
    from thoth_gb300 import surrogate as S
    t_all = time.perf_counter()
    X, Y, _, t_labels = S.mc_labels(S.sobol_params(n_train, 0), train_paths, distinct=True)
    model = S.Ensemble(members=members, seed=seed)
    xn, yt, st = S.train_targets(X, Y)
    t0 = time.perf_counter()
    loss = model.train(xn, yt, st, epochs=epochs, batch=batch, lr=lr)
    t_train = time.perf_counter() - t0
    ev = S.sobol_params(n_eval, n_train)
    ncell = len(S.LATTICE_LM) * len(S.LATTICE_T)
    pick = np.linspace(0, n_eval - 1, cf_sets).astype(int)
    Xs = S.grid_features(ev[pick])
    cf = oracle.heston_prices(1.0, np.exp(Xs[:, 0]), Xs[:, 1], 0, 0, Xs[:, 6], Xs[:, 2], Xs[:, 3], Xs[:, 4], Xs[:, 5])
    q = lambda e: {"median": float(np.median(e)), "p90": float(np.quantile(e, 0.9)),
                   "p99": float(np.quantile(e, 0.99)), "max": float(e.max()),
                   "frac_above_tol": float(np.mean(e > S.TOL)), "cells": int(e.size)}
    mc_paths, _, e_mc = S.calibrate_plain_mc(ev[pick], cf)
    sample = ev[np.linspace(0, n_eval - 1, plain_sets).astype(int)]
    _, _, _, t_plain = S.mc_labels(sample, mc_paths)
    plain_rate = plain_sets * ncell / t_plain
    raw, _ = model.price_lattice(ev[pick])
    one, _ = model.members[0].price_lattice(ev[pick])
    policies = {}
    for policy in S.POLICIES:
        price, info = S.price_grid(model, ev, mc_paths, policy=policy)
        pipe = np.concatenate([price[k * ncell:(k + 1) * ncell] for k in pick])
        info.update(error_pipeline=q(S.cell_error(pipe, cf)), speedup=info["cells_per_sec"] / plain_rate)
        policies[policy] = info
    g = policies["grid"]
    grid_plain_s = n_eval * ncell / plain_rate
    saved = grid_plain_s - g["seconds"]
    model.close()
    return {
        "target": "90th-percentile cell error <= 1e-3 against the FP64 Heston closed form (relative, floor 1% of "
                  "spot); 4096 parameter sets x 252 lattice cells",
        "surrogate": g["cells_per_sec"], "plain_mc": plain_rate, "speedup": g["speedup"], "judge_policy": "grid",
        "surrogate_inference_only": g["cells"] / g["inference_s"], "plain_mc_paths": mc_paths,
        "plain_mc_sample": "%d sets of the grid priced as batched books in %.2f s" % (plain_sets, t_plain),
        "error_surrogate_raw": q(S.cell_error(raw, cf)), "error_one_member": q(S.cell_error(one, cf)),
        "members": members, "error_surrogate_pipeline": g["error_pipeline"],
        "error_plain_mc": q(e_mc),
        "policies": {k: {f: v[f] for f in ("cells_per_sec", "speedup", "failing_buckets", "fallback_cells",
                                           "fallback_s", "judge_s", "judged_p90", "estimated_p90",
                                           "judge_noise_p90", "error_pipeline")}
                     for k, v in policies.items()},
        "detail": {k: g[k] for k in ("seconds", "inference_s", "inference_device_ms", "judge_s", "judge_sets",
                                     "judge_paths", "fallback_s", "fallback_cells", "failing_buckets",
                                     "out_of_box_sets")},
        "one_off": {"label_seconds": t_labels, "train_seconds": t_train, "train_sets": n_train,
                    "train_labels": int(len(Y)), "train_paths": train_paths, "epochs": epochs, "final_loss": loss,
                    "members_trained_side_by_side": members,
                    "grids_to_break_even": (t_labels + t_train) / saved if saved > 0 else None,
                    "note": "the speed-up holds for grids priced after training; labels and training are paid "
                            "once, and are repaid after grids_to_break_even grids of this size"},
        "cf_sets": cf_sets, "section_seconds": time.perf_counter() - t_all,
    }


def run_gpu(args):
    import torch
    import thoth_gb300 as G
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n_steps = 2 * STEPS_PER_YEAR
    book = workload(rank, args.paths)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    peak_fp32 = G.measure_fp32_peak()
    peak_mufu = G.measure_mufu_peak()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- kernel throughput, plan resident --------------------------------
    res = G.ResidentBook(book)
    for _ in range(max(args.warmup, 3)):
        res.run()
    dev_ms = []
    barrier()
    with Clocks(local) as clk:
        since = clk.mark()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1)          # evict L2 (129 MB) before each timed step
            r = res.run()           # synchronous: kernels timed by CUDA events on the engine stream
            dev_ms.append(r["device_ms"])
        barrier()
        wall = time.perf_counter() - t0
        # a timed region shorter than the 200 ms sampling period: the same steps, untimed,
        # continue until two samples have been taken under this load (at most 2 s)
        t1 = time.perf_counter()
        while clk.proc is not None and clk.mark() - since < 2 and time.perf_counter() - t1 < 2.0:
            flush.fill_(1)
            res.run()
        clocks = clk.summary(since)
    res.close()
    ms = sum(dev_ms) / len(dev_ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.paths * n_steps / (ms * 1e-3)

    # ---- end to end through the C ABI from host descriptors ---------------
    for _ in range(2):
        G.price_book(book)
    barrier()
    e2e_ms, h2d, d2h = [], 0, 0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r = G.price_book(book)  # returns after the device->host copy of the results
        e2e_ms.append(1e3 * (time.perf_counter() - t1))
        h2d, d2h = r["h2d_bytes"], r["d2h_bytes"]
    e_ms = sum(e2e_ms) / len(e2e_ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e_ms = float(t.item())
    e2e = world * args.paths * n_steps / (e_ms * 1e-3)

    if rank == 0:
        achieved = FLOPS_PER_PATH_STEP * args.paths * n_steps / (ms * 1e-3) / 1e12
        mufu = MUFU_PER_PATH_STEP * args.paths * n_steps / (ms * 1e-3) / 1e9
        line = {
            "metric": "path-steps/sec", "value": value, "unit": "path-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(world, args.paths),
            "e2e": {"value": e2e, "unit": "path-steps/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e_ms},
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s",
                         "frac": achieved / peak_fp32, "traffic": NCU_DRAM_BYTES_PER_LAUNCH,
                         "peak_source": "FMA microbenchmark in this run (thoth_gpu_measure_fp32_peak); "
                                        "MEASURED_PEAKS.json records no FP32 figure",
                         "flops_per_unit": FLOPS_PER_PATH_STEP, "unit_of_work": "path-step",
                         "mufu": {"achieved": mufu, "peak": peak_mufu, "unit": "Gop/s", "frac": mufu / peak_mufu,
                                  "ops_per_unit": MUFU_PER_PATH_STEP,
                                  "peak_source": "reciprocal-square-root microbenchmark in this run "
                                                 "(thoth_gpu_measure_mufu_peak)"}},
            "clocks": clocks,
            "wall_s_timed_region": wall,
        }
        # the CPU baseline and the other workloads run at N = 1 only: at N > 1 the line
        # carries the headline, so that the other ranks' GPUs are not held while rank 0 runs them
        solo = world == 1
        if solo:
            line["cpu_baseline"] = cpu_baseline(args.cpu_sample_paths, os.cpu_count() or 1)
            line["cpu_baseline"]["one_core"] = one_core_baseline()
        else:
            line["sections"] = "CPU baseline and single-GPU sections reported at N = 1"
        if solo:
            line["gbm_vs_reference_kernel"] = gbm_section(G, flush)
        if solo and not args.no_lsv:
            line["lsv_book"] = lsv_book_section(G, flush, args.steps)
        if solo and not args.no_paths:
            line["stored_paths"] = paths_section(G, flush)
        if solo and not args.no_american:
            line["american_lsm"] = american_section(G, flush, args.steps)
        if solo and not args.no_calibration:
            line["lsv_calibration"] = calibration_section(G)
        if solo and not args.no_batch:
            line["ragged_batch"] = ragged_batch_section(G, args.steps)
        if solo and not args.no_surrogate:
            line["grid_cells_per_sec"] = surrogate_section()
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
