/*
 * thoth_oracle.h — TEST INFRASTRUCTURE: CPU restatement of the reference's
 * Monte-Carlo hot path, used only as the parity checker (tests/, the smoke
 * check) and as the timed CPU baseline of bench.py. Never linked into or
 * called by the GPU product path.
 *
 * Parity pin: tests/test_oracle_vs_reference.py checks every function below
 * against the reference's own code compiled into oracle/_ref/ (Sobol integers
 * bit-exact, FP64 prices to 1e-12) and against the committed fixtures in
 * tests/golden/ generated from that build.
 */
#ifndef THOTH_ORACLE_H
#define THOTH_ORACLE_H

#include <stdint.h>

#include "thoth_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Load the Joe-Kuo table (thoth_gb300/data/joe_kuo_6_21201.bin). 0 on success. */
int oracle_load_direction_numbers(const char* path);

/* V[d][32] direction numbers of the first `dims` Sobol dimensions. */
int oracle_direction_numbers(int dims, uint32_t* v);

/* Sobol integer points skip+1 .. skip+n, layout [point][dim]. */
int oracle_sobol_points(int dims, int64_t skip, int64_t n, uint32_t* out);

/* Acklam inverse normal CDF in FP64 (pricer/src/helpers/distributions.cpp:37-81). */
double oracle_normal_cdf_inv(double p);
int oracle_normal_cdf_inv_n(const double* p, int64_t n, double* out);

/* Normalised bridge increments [path][factor][N] (path_generator.cpp:126-198). */
int oracle_bridge_increments(const double* t, int n_dates, int factors, int64_t skip, int64_t n_paths,
                             uint64_t seed, double* out);

/* Price a book like the reference's node graph, on one thread when threads <= 1
 * (bit-for-bit the reference's operation order), else split into `threads`
 * disjoint Sobol blocks pooled as the reference cluster pools slaves
 * (pricer/src/modes/run_cluster.cpp:308-340, 413-445). per_path (optional,
 * single-thread only) receives the discounted contract values of the first
 * n_per_path paths, [path][product]; greeks are not computed by the oracle
 * (the pathwise Greeks are checked against closed forms). */
int oracle_price_book(const ThothBookDesc* d, ThothBookResult* r, int threads, double* per_path,
                      int64_t n_per_path);

/* Closed forms (FP64): Black-Scholes (pricer/src/helpers/finance.cpp:64-85)
 * and the Heston characteristic-function price with the "little Heston trap"
 * characteristic function (finance.cpp:472-568): the Lewis single-integral
 * form as the primary oracle and the reference's P1/P2 form as a cross-check,
 * both integrated by adaptive Gauss-Kronrod 7-15. */
double oracle_bs_price(double forward, double strike, double t, double vol, double df, int is_call);
double oracle_bs_delta(double spot, double strike, double t, double vol, double r, double q, int is_call);
double oracle_bs_vega(double spot, double strike, double t, double vol, double r, double q);
double oracle_heston_price(double spot, double strike, double t, double r, double q, double v0,
                           double kappa, double theta, double xi, double rho, int is_call);
double oracle_heston_price_p12(double spot, double strike, double t, double r, double q, double v0,
                               double kappa, double theta, double xi, double rho, int is_call);

/* batch of Heston calls, args[i] = (S, K, T, r, q, v0, kappa, theta, xi, rho), on `threads` threads */
int oracle_heston_prices(int64_t n, const double* args, double* out, int threads);

/* LSV leverage calibration, Single::CalibrateLeverage (single.cpp:390-473) restated:
 * fills c->leverage; defaults as thoth_gpu_calibrate_leverage */
int oracle_calibrate_leverage(ThothLeverageCalib* c);

/* the reference Rng's raw 64-bit draws: n draws from seed after skipping `skip` */
int oracle_xoshiro_draws(uint64_t seed, uint64_t skip, int64_t n, uint64_t* out, uint64_t state_out[4]);

#ifdef __cplusplus
}
#endif

#endif
