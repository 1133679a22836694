// american.cuh — Longstaff-Schwartz exercise on stored paths: the kernels' arguments and
// launchers (american.cu), shared with the host pass in thoth_gpu.cu.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "thoth_gpu.h"

#include "exact.cuh"

constexpr int LSM_THREADS = 512;
// regression sums of one date: sum m, m^2, m^3, m^4, y, y m, y m^2 over the in-the-money
// paths (m = S / norm, y = discounted continuation), then the path count
constexpr int LSM_NQ = 7;
constexpr int LSM_PART = LSM_NQ + 1;
// per-CTA result sums: discounted exercise values, their squares, discounted maturity payoffs
constexpr int LSM_NACC = 3;

struct LsmArgs {
    const float* S;       // [n_dates][ld] spot of every date and path, date-major
    int64_t ld;           // row stride of S (the book's path count)
    int64_t n;            // paths
    int M;                // exercise grid: dates 0 .. M-1, maturity M-1
    int call;             // 1 call, 0 put
    double strike, norm;  // strike; moneyness normaliser (m = S / norm)
    double inv_norm;      // 1 / norm, rounded to nearest
    // in the money <=> float bits of S >= itm_bits (call) or <= itm_bits (put): the
    // single-precision threshold of (double) S > K, resp. < K, found on the host
    int32_t itm_bits;
    int min_itm;          // in-the-money paths a date needs for its regression
    const double* df;     // [M] df[t]: discount of a cashflow from date t+1 to date t
    const double* disc;   // [M] disc[t]: discount from date t to today
    double* beta;         // [3M] b0, b1, b2 of each date (written by the fit, read by the apply)
    int* fit;             // [M] 1 where date t has a regression
    double* cf;           // [n] fit scratch: each path's cashflow, valued at the current date
    double* val;          // [n] fit scratch: each path's exercise value discounted to today
    // fit scratch, the in-the-money paths of the current date compacted per warp: warp w
    // owns entries [w seg_len, (w + 1) seg_len), seg_len = 32 ceil(n / threads)
    int64_t seg_len;
    int32_t* c_idx;       // path index
    double* c_m;          // moneyness
    double* c_iv;         // intrinsic value
    Fx128* part;          // [2][grid][LSM_PART] per-CTA regression sums, double-buffered by date
    Fx128* acc;           // [grid][LSM_NACC] per-CTA result sums
    unsigned* bar;        // arrivals of the CTAs' sums, all dates (zero at launch)
    unsigned* done;       // dates whose regression is published (zero at launch)
    int* status;          // 0 ok; 2 a wait timed out; 3 an addend out of range
};

// the fit kernel is a cooperative launch: every CTA must be resident at once
int lsm_fit_max_grid(int sms);
cudaError_t launch_lsm_fit(const LsmArgs& A, int grid, cudaStream_t st);
cudaError_t launch_lsm_apply(const LsmArgs& A, int grid, cudaStream_t st);

// One pass over the stored paths of one asset of a book (thoth_gpu.cu): the book is
// simulated, then a policy is fitted and valued on the same paths (fit), or the given
// frozen policy is valued (apply).
struct LsmPass {
    int asset = 0;                // in: the asset whose paths are stored
    int M = 0;                    // in: exercise dates 0 .. M-1
    int call = 0;                 // in
    double strike = 0, norm = 0;  // in
    int min_itm = 50;             // in
    bool fit = true;              // in
    std::vector<double> df, disc; // in: [M], as in LsmArgs
    std::vector<double> beta;     // [3M]: out when fitting, in otherwise
    std::vector<int32_t> fit_at;  // [M]: out when fitting, in otherwise
    double sum = 0, sum2 = 0;     // out: sums of the discounted exercise values and their squares
    double euro = 0;              // out: sum of the discounted maturity payoffs
    double s0 = 0;                // out: stored spot of path 0 at date 0
    int64_t paths = 0;            // out
    int grid = 0;                 // out: CTAs of the pass's kernel
    double sim_ms = 0, lsm_ms = 0; // out: device time of the simulation and of the exercise kernel
};

// under the engine's lock; errors as the C ABI's, message in thoth_gpu_last_error()
int thoth_lsm_pass(const ThothBookDesc* book, LsmPass& io);
