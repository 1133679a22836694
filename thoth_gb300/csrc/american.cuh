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

// The frozen-policy apply of one contract (lsm_apply_kernel).
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
    Fx128* acc;           // [grid][LSM_NACC] per-CTA result sums
    int* status;          // 0 ok; 3 an addend out of range
    // apply only: the exercise test in single precision first (exercise_screened)
    const float4* screen; // [M] b0, b1, b2 rounded to float; w = 1 where date t has a regression
    float strike_f;       // strike rounded to float
    float inv_norm_f;     // 1 / norm rounded to float
};

// One contract of a batched fit: its exercise grid, payoff, discount tables, outputs and
// scratch on the device.
constexpr int LSM_MAX_CONTRACTS = 64;
struct LsmContract {
    int M, call, min_itm, itm_bits; // as in LsmArgs
    double strike, norm, inv_norm;
    const double* df;               // [M]
    const double* disc;             // [M]
    double* beta;                   // [3M] out
    int* fit;                       // [M] out (zero at launch)
    double *cf, *val;               // [n] scratch
    int32_t* c_idx;                 // [n_list] compacted in-the-money lists, per warp
    double *c_m, *c_iv;             // [n_list]
    unsigned long long* tot;        // [M][LSM_PART][3] per-date regression sums as 42/42/44-bit
                                    // limbs (zero at launch)
    Fx128* acc;                     // [grid][LSM_NACC] per-CTA result sums
};

// The batched fit: every contract fitted on the same stored paths in one launch, each date
// one publish-and-release for all of them.
struct LsmFitArgs {
    const float* S;
    int64_t ld, n;
    int C;                          // contracts, <= LSM_MAX_CONTRACTS
    int Tmax;                       // the largest M
    const LsmContract* ct;          // [C]
    int64_t seg_len;                // list entries of one warp, 32 ceil(n / threads)
    unsigned *bar, *done;           // arrivals and releases, all dates (zero at launch)
    int* status;                    // 0 ok; 2 a wait timed out; 3 an addend out of range
};

// the fit kernel is a cooperative launch: every CTA must be resident at once
int lsm_fit_max_grid(int sms);
cudaError_t launch_lsm_fit(const LsmFitArgs& A, int grid, cudaStream_t st);
cudaError_t launch_lsm_apply(const LsmArgs& A, int grid, cudaStream_t st);

// One pass over the stored paths of one asset of a book (thoth_gpu.cu): a policy fitted and
// valued on the paths (fit), or the given frozen policy valued (apply).
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
    // out: device time of the simulation and of the exercise kernel; passes that share a
    // simulation or a batched fit launch carry its time on the first of them only
    double sim_ms = 0, lsm_ms = 0;
};

// Simulate the book once with the paths of `asset` stored, then run the n passes on them
// (each pass's asset must be `asset`); under the engine's lock; errors as the C ABI's,
// message in thoth_gpu_last_error(). sim_ms is charged to the first pass.
int thoth_lsm_passes(const ThothBookDesc* book, int asset, LsmPass* io, int n);
