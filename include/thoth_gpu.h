/*
 * thoth_gpu.h — C ABI of the GB300 Monte-Carlo engine behind Thoth's
 * `!mcl_pricer` (allow_gpu: true).
 *
 * Plain C: POD structs, pointers and sizes only, so a C++23 host, a ctypes
 * binding or any other FFI can call it. Every entry point returns an int
 * status (THOTH_GPU_OK or a negative THOTH_GPU_E_* code); no exception or
 * C++ type crosses this boundary. All result memory is caller-owned.
 *
 * Reference interface this replaces (GValas/Thoth):
 *   pricer/src/tasks/mcl_gpu.hpp:16-48   namespace gpu { Available, DeviceInfo,
 *                                        PriceEuropeanGbm }
 *   pricer/src/tasks/pricer_mcl_gpu_gate.cpp:82-126
 *                                        BookIsGpuSupported / PriceContract
 *   pricer/src/tasks/pricer_mcl.cpp:623-644, 677-709
 *                                        the CPU path loop (Tree_Run) and the
 *                                        indicator read-out (Tree_Read) that a
 *                                        whole-book call replaces
 *
 * Threading: every entry point may be called from any host thread (the
 * reference server prices on a per-request std::thread, run_server.cpp:110-116).
 * Calls are serialised by an internal mutex; the device arena and stream are
 * created lazily on the first call and reused.
 *
 * Device: the engine binds to the calling thread's current CUDA device at its
 * first call and sets that device on every later call, from any thread. A
 * process drives one GPU: with one process per GPU, each selects its device
 * (cudaSetDevice) before its first call. A surrogate handle binds to the device
 * current when it is created.
 */
#ifndef THOTH_GPU_H
#define THOTH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define THOTH_GPU_OK 0
#define THOTH_GPU_E_INVALID (-1)     /* bad descriptor / argument            */
#define THOTH_GPU_E_NODEVICE (-2)    /* no usable CUDA device                */
#define THOTH_GPU_E_CUDA (-3)        /* a CUDA runtime call failed           */
#define THOTH_GPU_E_UNSUPPORTED (-4) /* book outside the GPU gate            */
#define THOTH_GPU_E_CANCELLED (-5)   /* thoth_gpu_request_cancel() honoured  */
#define THOTH_GPU_E_NOMEM (-6)       /* device arena could not grow          */
#define THOTH_GPU_E_TOO_LARGE (-7)   /* size above a documented maximum      */

/* ---- enumerations ------------------------------------------------------ */
/* diffusion models (reference: marketdata/single.cpp:65-153) */
#define THOTH_MODEL_GBM 0    /* SpotDiffusionNode, constant vol            */
#define THOTH_MODEL_HESTON 1 /* HestonVarianceNode (QE) + HestonSpotNode   */
#define THOTH_MODEL_LSV 2    /* Heston + LocalVolatilityNode leverage      */

/* payoffs (reference: nodes/vanilla_flow_node.cpp, barrier_flow_node.cpp,
 * variance_flow_node.cpp, absolute_basket_node.cpp) */
#define THOTH_PRODUCT_VANILLA 0
#define THOTH_PRODUCT_BARRIER 1
#define THOTH_PRODUCT_VARIANCE 2
#define THOTH_PRODUCT_BASKET 3 /* vanilla on sum_i w_i S_i */

#define THOTH_CALL 0
#define THOTH_PUT 1

/* pathwise Greeks mask (ThothBookDesc.greeks) */
#define THOTH_GREEK_DELTA 1 /* d premium / d S0 of the product's asset        */
#define THOTH_GREEK_VEGA 2  /* d premium / d sigma (GBM assets), per 1.0 vol  */

/* largest supported sizes (checked; larger books return THOTH_GPU_E_TOO_LARGE) */
#define THOTH_MAX_ASSETS 8
#define THOTH_MAX_SOBOL_DIMS 4097 /* reference SobolGenerator::MaxDimension()  */
#define THOTH_MAX_DATES 8192
#define THOTH_MAX_PRODUCTS 4096
#define THOTH_MAX_LEV_POINTS 65536 /* log-strike points of one leverage layer */

/* ---- book descriptor ---------------------------------------------------- */
typedef struct ThothAsset
{
    int32_t model;      /* THOTH_MODEL_*                                          */
    int32_t lev_points; /* LSV: points per leverage layer (else 0)                */
    double spot;        /* S(0)                                                   */
    /* [n_dates] cumulative carry r - q - repo to each date: the DriftNode value;
     * a step's log-drift is carry[i]*t[i] - carry[i-1]*t[i-1]
     * (spot_diffusion_node.cpp:45-46, heston_spot_node.cpp:54-55)              */
    const double* carry;
    double vol; /* GBM: constant sigma                                           */
    /* Heston / LSV base (heston_variance_node.cpp:8-14, heston_spot_node.cpp:8-14) */
    double v0, kappa, theta, xi, rho;
    /* LSV leverage layers, one per diffusion date: grid point k of layer i sits at
     * log-spot (lev_offset[i] + k) * lev_ln_step[i]; read at S_{i-1} by clamped
     * linear interpolation (local_volatility_node.cpp:19-47).                  */
    const double* lev_ln_step; /* [n_dates]                                      */
    const int64_t* lev_offset; /* [n_dates]                                      */
    const double* lev_values;  /* [n_dates * lev_points]                         */
} ThothAsset;

typedef struct ThothProduct
{
    int32_t kind;        /* THOTH_PRODUCT_*                                        */
    int32_t option_type; /* THOTH_CALL / THOTH_PUT (vanilla, barrier, basket)     */
    int32_t asset;       /* underlying asset index (not used by baskets)          */
    int32_t maturity;    /* flow date index                                       */
    double strike;
    /* discounting: df = exp(-t[maturity] * zero_rate) (contract_node.cpp:16-51)  */
    double zero_rate;
    double fx; /* contract -> book currency factor (book_node.cpp:16-31)       */
    /* quanto: the payoff reads S_i * exp(-quanto * t[i]) with
     * quanto = sigma_S * sigma_FX * rho (quanto_adjustment_node.cpp:20-42); 0 = none */
    double quanto;
    /* barrier (barrier_flow_node.cpp:23-56); level already BGK-shifted if the
     * contract is continuously monitored (contracts/barrier.cpp:151-165)        */
    int32_t barrier_up, barrier_in;
    double barrier_level;
    int32_t n_monitor;
    const int32_t* monitor; /* sorted date indices                               */
    /* variance swap (variance_flow_node.cpp:13-60)                              */
    double notional, strike_variance, total_year_fraction, past_variance;
    int32_t n_obs;
    const int32_t* obs; /* sorted observation indices; NULL = every date 1..maturity */
    /* basket (absolute_basket_node.cpp:15-26): level = sum_k weights[k] * S_{components[k]} */
    int32_t n_components;
    const int32_t* components;
    const double* weights;
} ThothProduct;

typedef struct ThothBookDesc
{
    int32_t n_dates;     /* diffusion dates including today (index 0)              */
    const int32_t* days; /* [n_dates] calendar days from today, or NULL             */
    const double* t;     /* [n_dates] ACT/365 year fractions, t[0] = 0              */
    int32_t n_assets;
    const ThothAsset* assets;
    /* [n_assets*n_assets] row-major lower-triangular Cholesky factor L over the
     * assets' white noises; asset u's GBM Brownian is driven by sum_v L[u][v] n_v
     * (pricer_mcl.cpp:246-314). NULL = independent noises.                      */
    const double* cholesky;
    int32_t n_products;
    const ThothProduct* products;
    int64_t paths;      /* number of Monte-Carlo paths (> 1)                       */
    int64_t sobol_skip; /* leading Sobol points skipped (mcl_configuration sobol_skip) */
    int32_t use_sobol;  /* 1: Sobol + Brownian bridge (dimensions beyond 4097: the
                           reference Rng's stream); 0: counter-based pseudo-random */
    int32_t greeks;     /* THOTH_GREEK_* mask                                       */
    uint64_t seed;      /* the Rng seed: dimensions beyond 4097 (the reference's
                           xoshiro256++ stream), and the counter-based use_sobol = 0 */
    /* 1: the Cholesky factor also drives the spot white noise of Heston and LSV assets
     * (asset u's spot noise = sum_v L[u][v] n_v, as for a GBM Brownian); their variance
     * noises stay independent. An extension with no reference counterpart: the reference
     * correlates only GBM spots (pricer_mcl.cpp:277-283; single.cpp:88). 0: the
     * reference's behaviour. */
    int32_t correlate_all_spots;
} ThothBookDesc;

/* Per-product and book results. Arrays are caller-owned, n_products long;
 * delta / vega arrays may be NULL when not requested. trust = standard error
 * sqrt((S2 - S1^2/n)/(n-1)/n) (monte_carlo_node.cpp:35-40). */
typedef struct ThothBookResult
{
    double book_premium;
    double book_trust;
    double* premium;
    double* trust;
    double* delta;
    double* delta_trust;
    double* vega;
    double* vega_trust;
    double device_ms;  /* device time of the pricing kernels (CUDA events on the engine's stream) */
    int64_t h2d_bytes; /* bytes copied host -> device by this call                           */
    int64_t d2h_bytes; /* bytes copied device -> host by this call                           */
} ThothBookResult;

/* A book whose plan is resident on the device: created once, priced many
 * times (e.g. the reference's bump-and-revalue reprices share one grid and
 * Sobol block, pricer.cpp:273-392), destroyed by the caller. */
typedef struct ThothBookHandle ThothBookHandle;

/* Reference gpu::GbmResult (mcl_gpu.hpp:34-38). */
typedef struct ThothGbmResult
{
    double premium;
    double trust;
} ThothGbmResult;

/* ---- entry points ------------------------------------------------------ */

/* 1 iff a CUDA device of compute capability 10.3 is usable.
 * Replaces gpu::Available() (mcl_gpu.cpp via mcl_gpu.cu:77-82). */
int thoth_gpu_available(void);

/* One-line device description into buf (NUL-terminated, truncated to n).
 * Replaces gpu::DeviceInfo() (mcl_gpu.cu:84-98). */
int thoth_gpu_device_info(char* buf, size_t n);

/* European vanilla under GBM in the forward measure:
 *   F_T = forward * exp(-vol^2 T / 2 + vol sqrt(T) Z),  premium = df * mean(payoff)
 * Z is the first Sobol dimension (point 0 skipped) through the inverse normal,
 * so the result is deterministic and `seed` only selects the pseudo-random
 * stream when paths exceed 2^32 - 1. Replaces gpu::PriceEuropeanGbm
 * (mcl_gpu.hpp:40-46, mcl_gpu.cu:100-154). */
int thoth_gpu_price_european_gbm(double forward, double strike, double t, double vol, double df,
                                 int is_call, int64_t paths, uint64_t seed, ThothGbmResult* out);

/* Price a whole book in one sweep: every product on shared paths, FP64 sums
 * and sums of squares, pathwise Greeks on request. Replaces the reference's
 * per-contract GPU loop (pricer_mcl_gpu_gate.cpp:109-126) and, for the GPU
 * gate's widened model x payoff set, the CPU Tree_Run/Tree_Read
 * (pricer_mcl.cpp:598-709). */
int thoth_gpu_price_book(const ThothBookDesc* book, ThothBookResult* out);

/* Upload a book's plan and keep it resident. *out receives the handle. */
int thoth_gpu_book_create(const ThothBookDesc* book, ThothBookHandle** out);

/* Price a resident book (no host -> device copy of the plan). */
int thoth_gpu_book_run(ThothBookHandle* handle, ThothBookResult* out);

/* Release a resident book's device memory. */
int thoth_gpu_book_destroy(ThothBookHandle* handle);

/* Measurement hook, no reference counterpart: FP32 FMA throughput of the
 * device from a kernel of independent FMA chains; *tflops = 2 flops per FMA
 * over the kernel's CUDA-event time; *ms = that time. */
int thoth_gpu_measure_fp32_peak(double* tflops, double* ms);

/* Test hook, no reference counterpart (host-side fault injection): drops the
 * engine's working buffers (arena, staging, stored paths, exercise and
 * calibration scratch, batch buffers), so that the next calls allocate them
 * afresh, and makes the next n of those allocations fail as on a full device:
 * the calls return THOTH_GPU_E_NOMEM and later calls succeed. n = 0 clears it.
 * Handles (resident books, surrogates) keep their memory. */
int thoth_gpu_debug_fail_allocations(int32_t n);

/* Measurement hook, no reference counterpart: special-function-unit (MUFU)
 * throughput from a kernel of independent reciprocal-square-root chains;
 * *gops = 10^9 operations a second over the kernel's CUDA-event time; *ms = that time. */
int thoth_gpu_measure_mufu_peak(double* gops, double* ms);

/* Capacity of the device array behind thoth_gpu_price_book_noalloc. */
#define THOTH_NOALLOC_SCRATCH_BYTES (2u << 20)

/* Allocation-free variant of thoth_gpu_price_book; no counterpart in the
 * reference. For callers that must not allocate device memory: a host whose
 * memory is budgeted and locked before pricing starts, or code running inside a
 * framework that owns every allocation on the device. It calls no cudaMalloc,
 * cudaFree, cudaHostAlloc or other allocating routine; the plan, the Sobol
 * tables of the book's dimensions (direction numbers and the per-thread
 * low-bit table, 1152 bytes per dimension) and the FP64 partial sums all live
 * in one statically allocated device array of THOTH_NOALLOC_SCRATCH_BYTES
 * (2 MiB), which every GPU that loads the library holds until the process
 * exits. Books that do not fit return THOTH_GPU_E_TOO_LARGE (large books use
 * fewer CTAs before that). The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process; make that first call
 * before any stream capture, and do not reset the device's context (cudaDeviceReset)
 * between calls. The call prices on the device the engine is bound to once any other
 * entry point has run (as they do), else on the calling thread's current device. It
 * honours thoth_gpu_request_cancel once the engine is set up, through the engine's
 * existing mapped cancel word. The call is synchronous on the legacy default stream.
 * Every call reuses the same array and leaves its contents behind; the library
 * serialises its own calls, and work that overlaps one of these calls on the same GPU
 * and touches the array races with it. Same inputs, outputs and results as
 * thoth_gpu_price_book, except device_ms, which is not measured here (NaN). */
int thoth_gpu_price_book_noalloc(const ThothBookDesc* book, ThothBookResult* out);

/* Simulate the book's paths and return the spot of one asset at every date of
 * every path: spots[date * paths + path] (caller-owned, n_dates x paths floats),
 * path p being Sobol index sobol_skip + 1 + p. The book's products are priced on
 * the same paths (not returned). On the device the paths are written
 * date-major, consecutive paths by consecutive threads. *device_ms (may be
 * null) is the kernels' device time. No reference counterpart: the
 * reference's node graph keeps only the current path (nodes/monte_carlo_node.hpp:15-25). */
int thoth_gpu_simulate_paths(const ThothBookDesc* book, int32_t asset, float* spots, double* device_ms);

/* ---- bump-and-revalue Greeks on common random numbers ----------------------
 * The reference's definitions (pricer_mcl_greeks.cpp:43-299, pricer.cpp:144-193;
 * bump sizes pricer.hpp:20-30, constants.hpp:36), per product and for the book:
 *   delta  sum over assets of (P(S_a * 1.01) - P) / (0.01 S_a)
 *   gamma  sum over assets of (P(S_a * 1.1) - 2P + P(S_a * 0.9)) / (0.1 S_a)^2
 *   vega   P(vol + 0.01) - P per vol point: GBM sigma + 0.01, Heston / LSV
 *          v0 and theta -> (sqrt(v) + 0.01)^2 (leverage layers kept as given)
 *   rho    (P(rates + 1bp) - P) / 1bp * 0.01: every carry and zero rate
 *   theta  P(today + 1 day) - P (needs days; carries re-based, flat before
 *          date 1; zero rates kept)
 *   vega_param[k] (P(param_k + 0.01) - P) / 0.01 for k = v0, kappa, theta,
 *          xi, rho on every Heston / LSV asset
 * Every scenario is priced in one batch (one CUDA graph) on the same Sobol
 * paths. Output arrays are caller-owned (n_products, vega_param 5 x
 * n_products, any may be NULL); Greeks not requested or not available are NaN. */
#define THOTH_BUMP_DELTA 1
#define THOTH_BUMP_GAMMA 2
#define THOTH_BUMP_VEGA 4
#define THOTH_BUMP_RHO 8
#define THOTH_BUMP_THETA 16
#define THOTH_BUMP_PARAMS 32

typedef struct ThothBumpGreeks {
    int32_t flags;         /* in: THOTH_BUMP_* mask                                  */
    int32_t n_scenarios;   /* out: scenarios priced, the base included               */
    double* premium;       /* out: base premium per product                          */
    double* delta;
    double* gamma;
    double* vega;
    double* rho;
    double* theta;
    double* vega_param;    /* [5][n_products]                                        */
    double book_premium, book_delta, book_gamma, book_vega, book_rho, book_theta;
    double book_vega_param[5];
    double device_ms;      /* the batch's device time                                */
} ThothBumpGreeks;

int thoth_gpu_bump_greeks(const ThothBookDesc* book, ThothBumpGreeks* out);
/* the message of the last thoth_gpu_bump_greeks failure (or why theta is NaN) */
const char* thoth_gpu_bump_greeks_last_error(void);

/* ---- American exercise by Longstaff-Schwartz --------------------------------
 * Replaces PricerMCL::PriceAmerican (pricer_mcl_american.cpp:137-261) for one
 * vanilla of the book: the spot paths of its asset are stored on every date up
 * to maturity (the recorder, path_recorder.cpp), and the exercise policy is fitted
 * once on them (FitAmericanPolicy, pricer_mcl_american.cpp:263-378): backward over
 * dates maturity-1 .. 1, the discounted continuation of the in-the-money paths is
 * regressed on {1, m, m^2}, m = S / strike (the spot at date 0 when the strike is
 * not positive), at dates with at least min_itm of them, by the normal equations
 * and Cholesky (maths.cpp:354-381, 419-470). The value is the policy applied to
 * the same paths (ApplyAmericanPolicy, :380-447): exercise at the first date whose
 * intrinsic value is positive and at least the fitted continuation, else at
 * maturity, discounted at that date's zero rate; premium = max(mean, intrinsic at
 * the spot of date 0), trust = its standard error.
 * Greeks (flags): delta, gamma, vega and rho apply the FROZEN policy to the paths
 * of the bumped book (spot x 1.01, x 1.1 / x 0.9, vol level + 0.01, carries and
 * zero rates + 1bp: the bumps of thoth_gpu_bump_greeks, rho discounting at the
 * bumped rates); theta refits on the book rolled one day (a full reprice, as the
 * reference's theta pass). Regression and premium sums are exact (fixed point,
 * 2^-64): results do not depend on the launch shape. */
typedef struct ThothAmerican {
    int32_t product;          /* in: a THOTH_PRODUCT_VANILLA of the book, quanto 0   */
    int32_t flags;            /* in: THOTH_BUMP_DELTA|GAMMA|VEGA|RHO|THETA           */
    int32_t min_itm;          /* in: in-the-money paths a regression needs; <= 0: 50 */
    int32_t fitted_dates;     /* out: dates of the policy with a regression          */
    /* in: zero rate of the premium currency at each date (n_dates) for the
     * discounting, or NULL: the product's zero_rate at every date             */
    const double* zero_rates;
    double* beta;             /* out, optional [3 * n_dates]: b0 b1 b2 per date, NaN
                                 where the date has no regression                    */
    double premium, trust;    /* out                                                 */
    double european;          /* out: discounted maturity payoff on the same paths   */
    double delta, gamma, vega, rho, theta; /* out: NaN where not requested          */
    double device_ms;         /* out: every simulation and exercise kernel           */
    double exercise_ms;       /* out: the base fit kernel(s) of the call alone        */
} ThothAmerican;

int thoth_gpu_price_american(const ThothBookDesc* book, ThothAmerican* am);
/* Every American contract of a book in one call, as PriceAmerican prices all of a book's
 * American contracts: am[0..n) as above, one per contract. Each scenario (the base, each
 * asset's spot bumps, the vol, rate and roll scenarios) is simulated once per asset that
 * carries contracts, and all of that asset's contracts are fitted or valued on the same
 * stored paths; the fits of an asset's contracts share one launch, one regression round
 * per date for all of them (the normal equations batched). device_ms and exercise_ms of
 * every entry are the whole call's. */
int thoth_gpu_price_american_book(const ThothBookDesc* book, ThothAmerican* am, int32_t n);
const char* thoth_gpu_american_last_error(void);

/* ---- LSV leverage calibration (binned particle method) ----------------------
 * Replaces Single::CalibrateLeverage (pricer/src/marketdata/single.cpp:390-473):
 * a Heston ensemble is diffused forward over the dates with the leverage being
 * built; before the step into date k, layer k is set from the Dupire condition
 *   L(x_i, t_k) = clamp(sigma_loc(x_i, t_k) / sqrt(max(E[v | ln S = x_i], min_cv)),
 *                       lev_min, lev_max)
 * with E[v | ln S] the binned conditional mean of the current ensemble
 * (equal-width log-spot bins between the ensemble's extremes, thin bins filled
 * from the nearest populated one, linear between bin centres; the ensemble mean
 * while all particles share one spot). The step is the reference's QE variance
 * step and leveraged log-spot step, layer k read at the previous spot. Gaussians
 * are the reference's Rng stream (xoshiro256++ seeded by splitmix64, inverse
 * normal), two per particle and date in particle order, so the layers follow the
 * reference's ensemble.
 * The caller supplies each layer's grid and the target local vol on it (the
 * reference sizes the grid from the ATM implied vol, single.cpp:432-443, and reads
 * sigma_loc from its implied surface): the output is the leverage surface of an
 * LSV ThothAsset (lev_ln_step = ln_step, lev_offset = offset, lev_values). */
typedef struct ThothLeverageCalib {
    int32_t n_dates;          /* in: layers, one per date; date 0 is today             */
    int32_t points;           /* in: grid points per layer (the reference: 201)        */
    const int32_t* days;      /* in: [n_dates] calendar days from today, days[0] = 0   */
    const double* carry;      /* in: [n_dates] net carry r - q - repo to each date     */
    double spot;              /* in: diffusion spot at today                           */
    double v0, kappa, theta, xi, rho; /* in: the Heston base                           */
    const double* ln_step;    /* in: [n_dates] layer grid spacing in log-spot          */
    const int64_t* offset;    /* in: [n_dates] grid point i sits at (offset + i) ln_step */
    const double* local_vol;  /* in: [n_dates][points] target local vol at the points */
    int32_t particles;        /* in: ensemble size; <= 0: 16384                         */
    int32_t bins;             /* in: conditional-mean bins; <= 0: 30                    */
    int32_t min_bin_count;    /* in: a thinner bin takes its neighbour's mean; <= 0: 20 */
    int32_t _pad;
    uint64_t seed;            /* in: Rng seed (the reference's is 20260708)             */
    double min_cond_variance; /* in: <= 0: 1e-6                                         */
    double lev_min, lev_max;  /* in: clamp; <= 0: 0.05 and 10                          */
    double* leverage;         /* out: [n_dates][points] layers                         */
    double device_ms;         /* out                                                    */
} ThothLeverageCalib;

int thoth_gpu_calibrate_leverage(ThothLeverageCalib* c);

/* the reference Rng's state after n draws from the state s (xoshiro256++ is
 * linear over GF(2): a jump is a polynomial in the transition, x^n modulo its
 * characteristic polynomial); host computation, no device needed */
int thoth_gpu_xoshiro_jump(const uint64_t s[4], uint64_t n, uint64_t out[4]);

/* Price n_books independent books (ragged path and step counts) in one CUDA
 * graph launch: all plans in one upload, all sums back in one copy. By default
 * (batches of up to 65535 books; larger ones launch per book) the
 * single-asset books run in ONE persistent kernel launch over a shared work
 * list (item r of a book = the tiles r, r + grid, ... that CTA r of the book's own
 * launch takes, so every book's sums are bit for bit those of its own launch at
 * the same grid; largest items first, taken by resident CTAs from a counter),
 * between one gather of the books' low Sobol words and one fixed-order
 * reduction of every book's rows: three kernel launches for the batch. Books
 * that kernel does not run (several assets, or shared memory beyond what keeps
 * its CTAs resident) get their own launches on side streams meanwhile. With
 * thoth_gpu_batch_persistent(0), every book's gather, kernel and reduction go
 * on one of several streams instead (largest first). The graph is captured on
 * the first call and replayed while the batch's shapes repeat. device_ms of
 * every result is the whole batch's device time. No reference counterpart
 * beyond repeated PriceBook calls (pricer_mcl.cpp:197-240). */
int thoth_gpu_price_batch(const ThothBookDesc* books, int32_t n_books, ThothBookResult* out);

/* ---- autotuner (no reference counterpart) ----------------------------------
 * Times candidate launch configurations on the device with CUDA events and
 * keeps the fastest for later calls in this process:
 *  - per book size, keyed by (kernel variant, ceil(log2 paths), ceil(log2
 *    steps)): the launch shape of single-asset books (paths per tile 256 or
 *    128, paths per thread 1 or 2, so 64 to 256 threads per CTA), and the
 *    persistent grid (k x SMs for k = 1 .. resident CTAs per SM, and the
 *    "balanced" grid of each: same waves, fewest CTAs);
 *  - per batch: the persistent launch or one launch per book; for the
 *    persistent launch the grid policy of its books' work items; for one launch
 *    per book the stream count (1 .. 32), one launch shape for every
 *    single-asset book of the batch (or each book's own), and the grid policy
 *    of the batch graph (0 full, 1 balanced, 2 half).
 * Choices can be saved to and loaded from a small text file, which is tied to
 * the device name and SM count it was measured on (THOTH_GPU_E_UNSUPPORTED
 * when loaded on another device). Step chunking has no knob here: every step
 * of a path runs in registers in one pass. */
typedef struct ThothTuneResult {
    int32_t grid;          /* chosen CTAs (book) */
    int32_t default_grid;  /* untuned grid: default shape, resident CTAs per SM x SMs, capped by tiles */
    int32_t candidates;    /* configurations timed */
    int32_t streams;       /* chosen stream count (batch) */
    int32_t policy;        /* chosen grid policy */
    int32_t shape;         /* chosen launch shape (book; -1 for a batch) */
    int32_t threads;       /* threads per CTA of the chosen shape */
    int32_t tile_paths;    /* paths per tile of the chosen shape */
    double best_ms;        /* mean device time of the chosen configuration */
    double default_ms;     /* the same for the untuned configuration */
    int32_t persistent;    /* batch: 1 the persistent launch was chosen, 0 one launch per book */
} ThothTuneResult;

int thoth_gpu_autotune_book(const ThothBookDesc* book, int32_t reps, ThothTuneResult* out);
int thoth_gpu_autotune_batch(const ThothBookDesc* books, int32_t n_books, int32_t reps, ThothTuneResult* out);
int thoth_gpu_autotune_save(const char* path);
int thoth_gpu_autotune_load(const char* path);
/* forget every tuned choice (back to the untuned defaults) */
int thoth_gpu_autotune_clear(void);

/* Number of streams a batch graph fans out over (default 8): every book in
 * the per-book mode, the books outside the persistent launch otherwise. */
int thoth_gpu_batch_streams(int32_t n);

/* 1 (default): the single-asset books of a batch in one persistent launch;
 * 0: one launch per book. */
int thoth_gpu_batch_persistent(int32_t on);

/* Kernel launches recorded into the cached batch graph (0 before the first batch). */
int thoth_gpu_batch_launches(void);

/* Replays of the cached batch graph since its capture (0 right after a capture). */
int thoth_gpu_batch_graph_replays(void);

/* Sobol integer coordinates x[d] (before the 2^-32 scaling) of points
 * skip+1 .. skip+n_points of the Joe-Kuo sequence, row-major [point][dim].
 * Same numbers as SobolGenerator::Next after Skip(skip)
 * (sobol_generator.cpp:80-121). Test hook for bit-exact parity. */
int thoth_gpu_sobol_points(int32_t dims, int64_t skip, int64_t n_points, uint32_t* out);

/* Normalised Brownian-bridge increments n[f][i] = dW_i / sqrt(dt_i), i = 1..N,
 * of paths skip+1 .. skip+n_paths, FP32, layout [path][factor][N].
 * Same construction as PathGenerator::NextPath (path_generator.cpp:126-198).
 * t: [n_dates] year fractions. Test hook. */
int thoth_gpu_bridge_increments(const double* t, int32_t n_dates, int32_t factors, int64_t skip,
                                int64_t n_paths, float* out);

/* Inverse standard-normal CDF in FP32 of the uniforms x * 2^-32, x given as
 * uint32 Sobol coordinates. Test hook for the device quantile. */
int thoth_gpu_normal_quantiles(const uint32_t* x, int64_t n, float* out);

/* Host-only test hook (no device needed): the time-ordered Brownian-bridge
 * program the kernels execute. first_count[2*(i-1)] / [2*(i-1)+1] = first node
 * and node count of step i (count 0 = pop); nodes[4*k..4*k+3] = (lw, rw, sd,
 * build step) of node k; *n_nodes and *stack_depth are set. Buffers must hold
 * n_dates-1 steps and n_dates-1 nodes. Same schedule as
 * PathGenerator::BuildBridgeSchedule (path_generator.cpp:49-120). */
int thoth_gpu_bridge_program(const double* t, int32_t n_dates, int32_t* first_count, double* nodes,
                             int32_t* n_nodes, int32_t* stack_depth);

/* Host-only test hook: validate a descriptor and report the launch plan.
 * out[0] kernel variant, [1] paths per tile, [2] shared-memory bytes per CTA,
 * [3] observation slots, [4] path groups, [5] bridge stack depth,
 * [6] Sobol dimensions, [7] tiles, [8] launch shape, [9] threads per CTA,
 * [10] moments summed per thread across tiles (books of at most four products;
 * 0: sums reduced per tile) (out holds 11 values). Returns the descriptor's
 * status code. */
int thoth_gpu_plan_summary(const ThothBookDesc* book, int64_t* out);

/* Test hook, no reference counterpart: one tcgen05 BF16 tensor-core GEMM,
 * D (128 x N, FP32) = A (128 x K, bf16 bits) * B (N x K, bf16 bits)^T, all
 * row-major host arrays; N and K multiples of 16, N <= 256, K <= 256. Used to
 * check the tensor-core building blocks of the surrogate against the CPU. */
int thoth_gpu_tc_gemm_test(const uint16_t* a, const uint16_t* b, int32_t n, int32_t k, float* d);

/* ---- learned surrogate (no reference counterpart) ------------------------
 * A 7 -> 4 x 128 SiLU -> 1 MLP of the Heston vanilla price surface, trained
 * and served by BF16 tcgen05 tensor-core kernels with FP32 accumulation and
 * FP32 Adam. Inputs are the 7 features already scaled to [-1, 1] (row-major
 * [n][7]); outputs are the normalised prices the model was trained on. */
typedef struct ThothSurrogate ThothSurrogate;
int thoth_gpu_surrogate_create(ThothSurrogate** out, uint64_t seed);
int thoth_gpu_surrogate_destroy(ThothSurrogate* s);
int thoth_gpu_surrogate_n_params(void);
int thoth_gpu_surrogate_get_params(ThothSurrogate* s, float* params);
int thoth_gpu_surrogate_set_params(ThothSurrogate* s, const float* params);
/* Weighted MSE sum_i ((yhat_i - y_i) / scale_i)^2 / n, Adam with a cosine
 * learning-rate decay over all steps; batch a multiple of 128. */
int thoth_gpu_surrogate_train(ThothSurrogate* s, const float* x, const float* y, const float* scale, int64_t n,
                              int32_t epochs, int32_t batch, double lr, uint64_t seed, double* final_loss);
/* As thoth_gpu_surrogate_train, with tail averaging of the weights: the cosine decay runs
 * from lr to lr_avg over the first epochs - avg_epochs epochs, lr_avg then holds, and the
 * weights at the end of each of the last avg_epochs epochs are averaged on the device; the
 * model keeps that average (one network, whose fit averages out more of the label noise
 * than the last iterate does). avg_epochs = 0 is thoth_gpu_surrogate_train. */
int thoth_gpu_surrogate_train_avg(ThothSurrogate* s, const float* x, const float* y, const float* scale, int64_t n,
                                  int32_t epochs, int32_t batch, double lr, uint64_t seed, int32_t avg_epochs,
                                  double lr_avg, double* final_loss);
/* An ensemble's k members (1 <= k <= 64, distinct handles on one device) trained side by
 * side on the same set: member j as by thoth_gpu_surrogate_train_avg with data-order seed
 * seed + j (its initialisation is its own creation seed); each member replays its own step
 * on its own stream, so their kernels share the device. final_loss (may be null) holds k
 * values. */
int thoth_gpu_surrogate_train_members(ThothSurrogate* const* members, int32_t k, const float* x, const float* y,
                                      const float* scale, int64_t n, int32_t epochs, int32_t batch, double lr,
                                      uint64_t seed, int32_t avg_epochs, double lr_avg, double* final_loss);
/* Gradient of that loss over `rows` rows (multiple of 128) at the current
 * parameters, without updating them; for checks against a CPU oracle. */
int thoth_gpu_surrogate_gradient(ThothSurrogate* s, const float* x, const float* y, const float* scale, int32_t rows,
                                 float* grad, double* loss);
int thoth_gpu_surrogate_predict(ThothSurrogate* s, const float* x, int64_t n, float* y, double* device_ms);
/* Prices of a lattice grid in units of spot, every step on the device: the cells are
 * every (parameter set, maturity, log-moneyness), cell (s, j, k) at index
 * (s * n_T + j) * n_lm + k, with raw features (lms[k], Ts[j], params[s * 5 + 0..4] =
 * kappa, theta, xi, rho, v0). Each cell's features are clipped to the training box
 * [box_lo, box_hi] (7 each, in that feature order) and normalised to [-1, 1], the network
 * is evaluated, and its output is multiplied by the scale it was trained against:
 * sqrt(bs^2 + floor^2), bs the Black-Scholes call (S = 1, r = q = 0) at the expected
 * average Heston variance theta + (v0 - theta)(1 - e^-kT)/(kT) over [0, T]. Only the
 * parameter sets and the lattice axes cross to the device and only the prices come back.
 * *device_ms: the three kernels' device time. */
int thoth_gpu_surrogate_price_lattice(ThothSurrogate* s, const double* params, int32_t n_sets, const double* lms,
                                      int32_t n_lm, const double* Ts, int32_t n_T, const double* box_lo,
                                      const double* box_hi, double floor, float* prices, double* device_ms);
/* As thoth_gpu_surrogate_price_lattice for an ensemble of k networks (1 <= k <= 64, all on
 * one device): the features are built once, every member is evaluated on them, and their
 * normalised outputs are added on the device in member order; the mean is scaled to prices.
 * Member 0's buffers and stream serve the call. */
int thoth_gpu_surrogate_price_lattice_mean(ThothSurrogate* const* members, int32_t k, const double* params,
                                           int32_t n_sets, const double* lms, int32_t n_lm, const double* Ts,
                                           int32_t n_T, const double* box_lo, const double* box_hi, double floor,
                                           float* prices, double* device_ms);
const char* thoth_gpu_surrogate_last_error(void);

/* Cooperative cancellation (reference: helpers/cancellation.hpp:9-15): a
 * running thoth_gpu_price_* call polls a host-mapped word between launches and
 * returns THOTH_GPU_E_CANCELLED. The flag is cleared by thoth_gpu_clear_cancel. */
int thoth_gpu_request_cancel(void);
int thoth_gpu_clear_cancel(void);

/* Text of the last error on this thread (never NULL). */
const char* thoth_gpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* THOTH_GPU_H */
