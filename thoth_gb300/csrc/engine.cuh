// engine.cuh — device side of the GB300 Monte-Carlo engine.
//
// One persistent kernel per book: every CTA walks tiles of 2^TB consecutive
// Sobol indices (two paths per thread for single-asset books, one for mixed
// books), all steps of all factors in registers (log-spot with Kahan
// compensation, variance, bridge anchors; the bridge stack in shared memory),
// and evaluates every product of the book on the tile's paths before moving
// on. FP32 path arithmetic; FP64 only for the per-CTA sums and the cross-CTA
// reduction.
//
// Reference semantics restated here (GValas/Thoth, pricer/src/...):
//   Sobol Gray-code points          nodes/sobol_generator.cpp:22-121
//   Brownian bridge increments      nodes/path_generator.cpp:49-198
//   GBM log-Euler step              nodes/spot_diffusion_node.cpp:21-73
//   Heston QE variance              nodes/heston_variance_node.cpp:17-57
//   Andersen log-spot (+ leverage)  nodes/heston_spot_node.cpp:32-94
//   leverage lookup                 nodes/local_volatility_node.cpp:19-47
//   payoffs                         nodes/vanilla_flow_node.cpp, barrier_flow_node.cpp,
//                                   variance_flow_node.cpp, absolute_basket_node.cpp,
//                                   quanto_adjustment_node.cpp
//   discounting / book / indicators nodes/contract_node.cpp, book_node.cpp,
//                                   monte_carlo_node.cpp:26-96
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace thoth {

constexpr int MAX_ASSETS = 8;
constexpr int SOBOL_BITS = 32;
constexpr int SOBOL_LO_ROW = 256; // threads covered by the low-bit table (tiles of up to 2^8 paths)

// M_SEQ: a multi-asset book whose assets are independent path by path (no
// correlated GBM name; the reference correlates only GBM spots), simulated one
// asset after the other with the single-asset state and a two-factor bridge
enum : int { M_GBM = 0, M_HESTON = 1, M_LSV = 2, M_MIXED = 3, M_SEQ = 4 };

// per-step, per-asset constants (12 floats, three 16-byte loads)
//  GBM:    c[0] = carry_drift - sigma^2 dt / 2, c[1] = sigma sqrt(dt) (Brownian scale), c[2] = sqrt(dt)
//  Heston: c[0] = e = exp(-kappa dt), c[1] = theta (1 - e), c[2] = A, c[3] = B   (s2 = A v + B)
//          c[4] = carry_drift, c[5] = k0, c[6] = a1, c[7] = a2, c[8] = k3, c[9] = r = rho/xi
//          step(L) = c4 + L (k0 + a1 s + r (vc - vp) + sqrt(k3 s) z) - L^2 a2 s, s = vp + vc
//          degenerate xi: c[10] = dt (step = c4 - L^2 vp dt / 2 + L sqrt(vp dt) z)
struct alignas(16) AssetStep {
    float c[12];
};

// time-ordered Brownian-bridge program node: W_new = lw * W_{i-1} + rw * W_top + sd * z(bstep)
struct alignas(16) BridgeNode {
    float lw, rw, sd;
    int bstep;
};

// per-step program: bridge nodes [first, first + count); count == 0 pops the stack
struct StepProg {
    int first, count;
};

// per-step record read once per step (prefetched one step ahead): the first
// bridge node inline, the node count (0 = pop), the remaining nodes' start,
// 1/sqrt(dt) of the path generator, and whether any asset has events this date
struct alignas(16) StepRec {
    float lw, rw, sd;
    int dim;   // reference dimension of the first node for factor 0: bstep * F
    float isd;
    int count;
    int first; // index of the second node in nodes[] (when count > 1)
    int ev;    // 1: events on this date
};

// path events, applied after the state at date i is known
enum : int {
    EV_SNAP_S = 0,     // slot = S0 exp(x)
    EV_SNAP_W = 1,     // slot = Brownian W (GBM vega)
    EV_SNAP_Y = 2,     // slot = tangent dX/dX0 (LSV delta)
    EV_GRP_MIN = 3,    // grp = min(grp, x - p)
    EV_GRP_MAX = 4,    // grp = max(grp, x - p)
    EV_GRP_SQ_STEP = 5,// grp += (step - p)^2   (continuous variance observation)
    EV_GRP_SQ_OBS = 6, // grp += (x - last - p)^2, last = x  (discrete observation; pad = row of last)
    EV_SNAP_G = 7,     // slot = grp[pad]  (a running group seen by a product that ends before it)
};
struct Event {
    int type, a; // a = slot or group
    float p;
    int pad;
};

enum : int { P_VANILLA = 0, P_BARRIER = 1, P_VARIANCE = 2, P_BASKET = 3 };

struct DevProduct {
    int kind, call, slot_s, slot_g; // slot_g: group (barrier extreme, variance sum)
    float K, df, fx, qfac;
    float level;
    int up, knock_in;
    float notional, kvar, inv_T, past;
    int comp_first, comp_n;
    int slot_y, slot_w; // greek observables (-1: none)
    float inv_s0, vol_t;
    int greek_mask;     // bit 0 delta supported, bit 1 vega supported
    int g_snap;         // 1: slot_g is a snapshot slot of a running group, 0: the group itself
};

struct Comp {
    int slot;
    float w;   // weight * quanto factor
    int slot_y;
    float inv_s0;
};

struct DevPlan {
    // sizes
    int n_steps, n_assets, n_slots_used, n_groups;
    int n_last;           // discretely observed variance groups (rows of the previous observation)
    int n_factors_active; // active factors of the book
    int stack_factors;    // factors held in the bridge stack (n_factors_active, or 2 when assets run one by one)
    int sobol_dims;       // dims served by Sobol (<= 4097)
    int ref_factors;      // F in the reference dimension layout dim = bstep * F + f
    int use_sobol;
    int stack_depth;
    int n_products;
    int greeks;
    int corr;             // 1: GBM noises correlated with chol
    int64_t skip, paths;  // Sobol index range [skip + 1, skip + paths]
    int64_t tile_first, n_tiles;
    uint64_t seed;
    // per asset (uniform)
    int model[MAX_ASSETS];
    int degenerate[MAX_ASSETS];
    int lev_points[MAX_ASSETS];
    float s0[MAX_ASSETS];
    float vol[MAX_ASSETS];
    float v0[MAX_ASSETS];
    int fid_spot[MAX_ASSETS];   // reference factor index of the spot noise
    int fid_var[MAX_ASSETS];    // reference factor index of the variance noise (-1: none)
    int cidx_spot[MAX_ASSETS];  // compact stack index
    int cidx_var[MAX_ASSETS];
    float chol[MAX_ASSETS * MAX_ASSETS];
    // device arrays
    const AssetStep* steps;      // [n_steps][n_assets]   (index i-1 for step i)
    const float* inv_sqrt_dt;    // [n_steps] path-generator 1/sqrt(t_i - t_{i-1})
    const StepProg* prog;        // [n_steps]
    const StepRec* recs;         // [n_steps]
    int uniform_steps;           // 1: every step's AssetStep equals step 1's
    const BridgeNode* nodes;     // time-ordered program
    const int2* ev_range;        // [(n_steps + 1)][n_assets] (first, count) into events; row 0 = date 0
    const Event* events;
    const int* lev_layer;        // [n_assets][n_steps + 1] layer of date i
    const float2* lev_map;       // [n_assets][layers] (1/ln_step, lnS0/ln_step - offset)
    const float* lev_values;     // [n_assets][layers][lev_row_stride]
    int lev_layers_stride;       // layers per asset (max)
    int lev_row_stride;          // floats per leverage layer (max points over the assets)
    const float* grp_init;       // [n_groups] +inf (min), -inf (max), 0 (sums)
    const DevProduct* products;
    const Comp* comps;
    const uint32_t* sobol_v;     // [4097][32] direction numbers
    const int* sobol_order;      // [n_sobol] Sobol dimensions in the order the step loop consumes them
    const uint32_t* sobol_lo;    // [n_sobol][T] low-bit words of those dimensions, in that order
    int n_sobol;
    double* acc;                 // [gridDim][n_acc] per-CTA FP64 sums
    int n_acc;
    float* path_out;             // [n_steps + 1][path_ld] spot of asset path_asset at every date (null: not stored)
    int64_t path_ld;             // paths per stored date (the book's path count)
    int path_asset;
    volatile int* cancel;        // host-mapped cancel word (may be null)
    int* status;                 // device status word
};

// ---------------------------------------------------------------------------
// Inverse normal CDF in FP32 for a uniform u = x * 2^-32, x a nonzero uint32.
// Method: Giles (2010, "Approximating the erfinv function") change of variable
// w = -ln(4 q (1 - q)), q = min(u, 1 - u), with polynomials in w (central) and
// sqrt(w) (tail) whose coefficients were fitted for this project by weighted
// least squares against 40-digit reference values; max relative error of the
// FP32 evaluation 2.2e-7 over the full uint32 range. Both q and 2u - 1 are
// formed from the integer (q = min(x, 2^32 - x), 2u - 1 = (x - 2^31) 2^-31),
// so the tails keep their relative accuracy.
// ---------------------------------------------------------------------------
// the pieces of quantile_u32: s = 2u - 1 and lg = log2(4 q (1 - q)) <= 0
__device__ __forceinline__ void quantile_prep(uint32_t x, float& s, float& lg)
{
    const uint32_t qi = min(x, 0u - x);                                     // q * 2^32 in [1, 2^31]
    s = __int2float_rn((int)(x ^ 0x80000000u)) * 4.656612873077393e-10f;    // 2u - 1
    const float qf = __uint2float_rn(qi);
    const float one_m_q = fmaf(qf, -2.3283064365386963e-10f, 1.0f);         // 1 - q
    // at q = 1/2 the MUFU result is clamped (fminf drops a NaN operand)
    lg = fminf(__log2f(qf * 9.313225746154785e-10f * one_m_q), 0.0f);
}

constexpr float QUANTILE_TAIL_LG = -9.016844005556021f; // w = -ln2 lg = 6.25

// central polynomial in w - 3.125, valid for lg > QUANTILE_TAIL_LG
__device__ __forceinline__ float quantile_central(float lg)
{
    const float v = fmaf(lg, -0.6931471805599453f, -3.125f);
    float p = -7.202387403e-09f;
    p = fmaf(p, v, -1.226470401e-08f);
    p = fmaf(p, v, 6.170809376e-07f);
    p = fmaf(p, v, -2.155695626e-06f);
    p = fmaf(p, v, -1.975007828e-05f);
    p = fmaf(p, v, 2.648245696e-04f);
    p = fmaf(p, v, -1.047204452e-03f);
    p = fmaf(p, v, -8.533770903e-03f);
    p = fmaf(p, v, 3.396347351e-01f);
    p = fmaf(p, v, 2.338620874e+00f);
    return p;
}

// tail polynomial in sqrt(w) - 3.6479158, for lg <= QUANTILE_TAIL_LG
__device__ __forceinline__ float quantile_tail(float lg)
{
    const float v = sqrtf(lg * -0.6931471805599453f) - 3.6479158f;
    float p = 6.598971903e-06f;
    p = fmaf(p, v, 5.795662157e-05f);
    p = fmaf(p, v, -2.423309240e-04f);
    p = fmaf(p, v, 3.854843299e-04f);
    p = fmaf(p, v, -5.190533957e-04f);
    p = fmaf(p, v, 9.818501131e-04f);
    p = fmaf(p, v, -2.186479756e-03f);
    p = fmaf(p, v, 3.518813816e-03f);
    p = fmaf(p, v, 1.425832630e+00f);
    p = fmaf(p, v, 4.927907588e+00f);
    return p;
}

__device__ __forceinline__ float quantile_u32(uint32_t x)
{
    float s, lg;
    quantile_prep(x, s, lg);
    const float p = lg > QUANTILE_TAIL_LG ? quantile_central(lg) : quantile_tail(lg);
    return p * s;
}

// N quantiles at once: the central polynomials as one straight-line block, the
// rare tail afterwards (same expressions as quantile_u32, same results)
template <int N>
__device__ __forceinline__ void quantile_n(const uint32_t (&x)[N], float (&z)[N])
{
    float s[N], lg[N];
    bool tail = false;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        quantile_prep(x[i], s[i], lg[i]);
        z[i] = quantile_central(lg[i]);
        tail |= !(lg[i] > QUANTILE_TAIL_LG);
    }
    if (tail) {
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (!(lg[i] > QUANTILE_TAIL_LG)) z[i] = quantile_tail(lg[i]);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) z[i] *= s[i];
}

// counter-based uint32 for dimensions beyond the Sobol budget and use_sobol = 0
// (splitmix64 finaliser of a Weyl combination of seed, point index and dimension)
__device__ __forceinline__ uint32_t hash_u32(uint64_t seed, uint64_t n, uint32_t dim)
{
    uint64_t z = seed + n * 0x9E3779B97F4A7C15ull + (uint64_t)dim * 0xD1B54A32D192ED03ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint32_t r = (uint32_t)(z >> 32);
    return r ? r : 1u;
}

// sqrt for x >= 0 on the MUFU rsqrt path (x * rsqrt(x); 0 maps to 0)
__device__ __forceinline__ float fast_sqrt(float x)
{
    return x * rsqrtf(fmaxf(x, 1e-30f));
}

// Phi(-z) = erfc(z / sqrt 2) / 2 with the Chebyshev-fitted erfc of Press et al.
// (Numerical Recipes in C, 2nd ed., section 6.2, "erfcc"; fractional error
// below 1.2e-7 everywhere), so the exponential QE branch keeps its accuracy in
// the upper tail without a library call.
__device__ __forceinline__ float phi_neg(float z)
{
    const float y = z * 0.7071067811865476f;
    const float a = fabsf(y);
    const float t = __fdividef(1.0f, fmaf(0.5f, a, 1.0f));
    float p = 0.17087277f;
    p = fmaf(p, t, -0.82215223f);
    p = fmaf(p, t, 1.48851587f);
    p = fmaf(p, t, -1.13520398f);
    p = fmaf(p, t, 0.27886807f);
    p = fmaf(p, t, -0.18628806f);
    p = fmaf(p, t, 0.09678418f);
    p = fmaf(p, t, 0.37409196f);
    p = fmaf(p, t, 1.00002368f);
    p = fmaf(p, t, -1.26551223f);
    const float e = t * __expf(fmaf(-a, a, p));
    return 0.5f * (y >= 0.f ? e : 2.0f - e);
}

// Andersen QE variance step in FP32 (heston_variance_node.cpp:17-57).
// c = {e, theta (1 - e), A, B}: m = theta + (v - theta) e, s2 = A v + B.
// psi = s2 / m^2 <= 1.5 is tested as s2 <= 1.5 m^2; the exponential branch
// uses 1 - u = Phi(-z) and 1 - p = 2 m^2 / (s2 + m^2). Both branches are
// evaluated and one is selected: the paths of a warp nearly always take both,
// so this costs no more issue slots than divergence and schedules as one block.
// The guards on the quadratic branch only act when it is not selected.
__device__ __forceinline__ float qe_step(float v, float z, float e, float th1e, float A, float B)
{
    const float m = fmaf(v, e, th1e);
    const float s2 = fmaf(v, A, B);
    const float m2 = m * m;
    // quadratic branch; c is capped at 1e18 (psi >= 2e-18, where the step's random part is
    // below single precision) so that c (c - 1) stays finite for a vanishing vol of vol
    const float c = fminf(__fdividef(2.0f * m2, s2), 1e18f);
    const float b2 = c - 1.0f + fast_sqrt(fmaxf(c * (c - 1.0f), 0.0f));
    const float a = __fdividef(m, 1.0f + b2);
    const float bz = fast_sqrt(fmaxf(b2, 0.0f)) + z;
    const float vq = a * bz * bz;
    // exponential branch
    const float num = s2 + m2;
    const float one_m_p = __fdividef(2.0f * m2, num);
    const float uc = phi_neg(z);
    const float ve = (uc >= one_m_p) ? 0.0f : __fdividef(num, 2.0f * m) * __logf(__fdividef(one_m_p, uc));
    return (s2 <= 1.5f * m2) ? vq : ve;
}

} // namespace thoth
