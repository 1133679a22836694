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

// per-step, per-asset constants (16 floats: three 16-byte loads, a fourth for LSV)
//  GBM:    c[0] = carry_drift - sigma^2 dt / 2, c[1] = sigma sqrt(dt) (Brownian scale), c[2] = sqrt(dt)
//  Heston: c[0] = e = exp(-kappa dt), c[1] = theta (1 - e), c[2] = A, c[3] = B   (s2 = A v + B)
//          c[4] = carry_drift, c[5] = k0, c[6] = a1, c[7] = a2, c[8] = k3, c[9] = r = rho/xi
//          step(L) = c4 + L (k0 + a1 s + r (vc - vp) + sqrt(k3 s) z) - L^2 a2 s, s = vp + vc
//          degenerate xi: c[10] = dt (step = c4 - L^2 vp dt / 2 + L sqrt(vp dt) z)
//  LSV:    the Heston constants, and the leverage layer of the date the step ends on:
//          c[12] = 1/ln_step, c[13] = ln S0 / ln_step - offset (the grid coordinate is
//          x c[12] + c[13], x = ln(S/S0)), c[14] = the layer's first value in lev_values
//          (an int), so the lookup needs no dependent load of the layer index or its map
struct alignas(16) AssetStep {
    float c[16];
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

// per-step record read once per step (at the step, or one step ahead): the first
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

// a vanilla product in the lean form used when every product of a book is a vanilla and no
// pathwise Greek is asked: discounted flow f = max(a S + b, 0) with a = phi qfac df and
// b = -phi K df (phi = +1 call, -1 put; df > 0), its weight in the book value w = fx, and
// the observation slot of S at maturity
struct alignas(16) VanTerm {
    float a, b, w;
    int slot;
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
    int corr_all;         // 1: Heston / LSV spot noises correlated with chol as well
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
    const StepRec* recs;         // [n_steps + 1] (the last is padding for a load one step ahead)
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
    const VanTerm* vterms;       // [n_products] lean vanilla terms (vanilla_only)
    int vanilla_only;            // 1: every product a vanilla and no pathwise Greek
    const Comp* comps;
    const uint32_t* sobol_v;     // [4097][32] direction numbers
    const int* sobol_order;      // [n_sobol] Sobol dimensions in the order the step loop consumes them
    const uint32_t* sobol_lo;    // [n_sobol][T] low-bit words of those dimensions, in that order
    int n_sobol;
    int n_tail;                  // reference dimensions beyond the Sobol budget (Sobol mode): n_steps F - sobol_dims
    const float* tail;           // [n_tail][tail_ld] their Gaussians, the reference Rng's stream (path-major)
    int64_t tail_ld;             // paths per tail dimension (the book's path count)
    double* acc;                 // [gridDim][n_acc] per-CTA FP64 sums
    int n_acc;
    int few_m;                   // > 0: few-product accumulation over few_m moments (see book_kernel)
    float* path_out;             // [n_steps + 1][path_ld] spot of asset path_asset at every date (null: not stored)
    int64_t path_ld;             // paths per stored date (the book's path count)
    int path_asset;
    volatile int* cancel;        // host-mapped cancel word (may be null)
    int* status;                 // device status word
};

// ragged batches in one persistent launch (batch_kernel): a book of the work list, its
// items r = 0 .. grid - 1 being what CTAs r of the book's own launch do
struct alignas(16) BatchBook {
    int plan;    // index into the plans
    int variant; // 0 GBM, 1 Heston, 2 LSV, 4 Heston with uniform steps, 5 GBM with uniform steps
    int grid;    // the book's own grid: its work items and the stride between an item's tiles
    int first;   // list index of the book's item 0
};

// the variants the batch kernel runs (single-asset books in the (8, 2) launch shape)
__host__ __device__ constexpr bool batch_variant(int v) { return v == 0 || v == 1 || v == 2 || v == 4 || v == 5; }

// a plan whose single-asset passes run the fast pair pass: Sobol mode with every dimension a
// Sobol dimension, no stored paths
__host__ __device__ inline bool fast_pass(const DevPlan& P)
{
    return P.use_sobol && P.sobol_dims >= P.n_steps * P.ref_factors && !P.path_out;
}

// one book's fixed-order reduction of its rows, and its gather of low Sobol words, in a batch
struct alignas(16) BatchReduce {
    const double* acc;
    double* out;
    int rows, n_acc;
};
struct alignas(16) BatchGather {
    const int* order;
    uint32_t* out;
    int n, T;
};

// ---------------------------------------------------------------------------
// Inverse normal CDF in FP32 for a uniform u = x * 2^-32, x a nonzero uint32.
// Method: Giles (2010, "Approximating the erfinv function") change of variable
// w = -ln(4 q (1 - q)), q = min(u, 1 - u), with polynomials in w (central) and
// sqrt(w) (tail) whose coefficients are fitted for this project: minimax in
// relative error against 40-digit values, rounded to float32 with refits and a
// one-ulp polish; thoth_gb300/csrc/fit_quantile.py prints them. The polynomials'
// FP32 evaluation is within 1.5e-7 (central) and 1.1e-7 (tail) of the target. Both q and 2u - 1 are
// formed from the integer (q = min(x, 2^32 - x), 2u - 1 = (x - 2^31) 2^-31),
// so the tails keep their relative accuracy.
// ---------------------------------------------------------------------------
// the pieces of quantile_u32: s = 2u - 1 and lg = log2(4 q (1 - q)) <= 0, with
// 4 q (1 - q) = qf (2^-30 - qf 2^-62) for qf = q 2^32
__device__ __forceinline__ void quantile_prep(uint32_t x, float& s, float& lg)
{
    const uint32_t qi = min(x, 0u - x);                                     // q * 2^32 in [1, 2^31]
    s = __int2float_rn((int)(x ^ 0x80000000u)) * 4.656612873077393e-10f;    // 2u - 1
    const float qf = __uint2float_rn(qi);
    // the MUFU result at q = 1/2 (argument 1) is clamped: fminf drops a NaN operand
    lg = fminf(__log2f(qf * fmaf(qf, -2.168404344971009e-19f, 9.313225746154785e-10f)), 0.0f);
}

constexpr float QUANTILE_TAIL_LG = -9.016844005556021f; // w = -ln2 lg = 6.25

// central polynomial in w - 3.125, valid for lg > QUANTILE_TAIL_LG
__device__ __forceinline__ float quantile_central(float lg)
{
    const float v = fmaf(lg, -0.6931471805599453f, -3.125f);
    float p = -7.086651266e-09f;
    p = fmaf(p, v, -1.266508587e-08f);
    p = fmaf(p, v, 6.137755690e-07f);
    p = fmaf(p, v, -2.147811756e-06f);
    p = fmaf(p, v, -1.971671372e-05f);
    p = fmaf(p, v, 2.647771616e-04f);
    p = fmaf(p, v, -1.047342434e-03f);
    p = fmaf(p, v, -8.533691987e-03f);
    p = fmaf(p, v, 3.396349251e-01f);
    p = fmaf(p, v, 2.338620901e+00f);
    return p;
}

// tail polynomial in sqrt(w) - 3.6479158, for lg <= QUANTILE_TAIL_LG
__device__ __forceinline__ float quantile_tail(float lg)
{
    const float v = sqrtf(lg * -0.6931471805599453f) - 3.6479158f;
    float p = 3.439537977e-05f;
    p = fmaf(p, v, 1.085241311e-04f);
    p = fmaf(p, v, -2.765924437e-04f);
    p = fmaf(p, v, 2.949863265e-04f);
    p = fmaf(p, v, -5.131622893e-04f);
    p = fmaf(p, v, 1.033666427e-03f);
    p = fmaf(p, v, -2.182901371e-03f);
    p = fmaf(p, v, 3.508982947e-03f);
    p = fmaf(p, v, 1.425832033e+00f);
    p = fmaf(p, v, 4.927907944e+00f);
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

// ---- two lanes in one instruction (sm_100 and later) --------------------------------
// A thread's two paths run the same arithmetic, so the FP32 fused multiply-adds, multiplies
// and adds of the per-path polynomials are issued as packed pairs. Each lane rounds exactly as
// the scalar fmaf / multiply / add, so the results are bit-identical to the scalar forms.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }

__device__ __forceinline__ float2 quantile_central2(float2 lg)
{
    const float2 v = __ffma2_rn(lg, f2s(-0.6931471805599453f), f2s(-3.125f));
    float2 p = f2s(-7.086651266e-09f);
    p = __ffma2_rn(p, v, f2s(-1.266508587e-08f));
    p = __ffma2_rn(p, v, f2s(6.137755690e-07f));
    p = __ffma2_rn(p, v, f2s(-2.147811756e-06f));
    p = __ffma2_rn(p, v, f2s(-1.971671372e-05f));
    p = __ffma2_rn(p, v, f2s(2.647771616e-04f));
    p = __ffma2_rn(p, v, f2s(-1.047342434e-03f));
    p = __ffma2_rn(p, v, f2s(-8.533691987e-03f));
    p = __ffma2_rn(p, v, f2s(3.396349251e-01f));
    p = __ffma2_rn(p, v, f2s(2.338620901e+00f));
    return p;
}

// quantiles of two words, quantile_prep and the central polynomial paired
__device__ __forceinline__ void quantile_pair(uint32_t x0, uint32_t x1, float& z0, float& z1)
{
    const uint32_t q0 = min(x0, 0u - x0), q1 = min(x1, 0u - x1);
    const float2 sv = __fmul2_rn(f2(__int2float_rn((int)(x0 ^ 0x80000000u)), __int2float_rn((int)(x1 ^ 0x80000000u))),
                                 f2s(4.656612873077393e-10f));
    const float2 qf = f2(__uint2float_rn(q0), __uint2float_rn(q1));
    const float2 arg = __fmul2_rn(qf, __ffma2_rn(qf, f2s(-2.168404344971009e-19f), f2s(9.313225746154785e-10f)));
    const float lg0 = fminf(__log2f(arg.x), 0.0f), lg1 = fminf(__log2f(arg.y), 0.0f);
    float2 zz = quantile_central2(f2(lg0, lg1));
    if (!(fminf(lg0, lg1) > QUANTILE_TAIL_LG)) {
        if (!(lg0 > QUANTILE_TAIL_LG)) zz.x = quantile_tail(lg0);
        if (!(lg1 > QUANTILE_TAIL_LG)) zz.y = quantile_tail(lg1);
    }
    zz = __fmul2_rn(zz, sv);
    z0 = zz.x;
    z1 = zz.y;
}

// quantile_n for an even number of paths a thread: their quantiles in pairs
template <>
__device__ __forceinline__ void quantile_n<2>(const uint32_t (&x)[2], float (&z)[2])
{
    quantile_pair(x[0], x[1], z[0], z[1]);
}

template <>
__device__ __forceinline__ void quantile_n<4>(const uint32_t (&x)[4], float (&z)[4])
{
    quantile_pair(x[0], x[1], z[0], z[1]);
    quantile_pair(x[2], x[3], z[2], z[3]);
}

// counter-based uint32 for use_sobol = 0 (and beyond the Sobol budget where a plan has no tail
// table: the bridge test hook)
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

// The special-function unit's approximate square root (one MUFU instruction, sqrt(0) = 0)
// and reciprocal, for x >= 0 and x > 0 respectively. a * rcp_approx(b) is the same
// computation as __fdividef(a, b) in the range used here.
__device__ __forceinline__ float fast_sqrt(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float2 sqrt2_approx(float2 x) { return make_float2(fast_sqrt(x.x), fast_sqrt(x.y)); }
__device__ __forceinline__ float2 rcp2_approx(float2 x) { return make_float2(rcp_approx(x.x), rcp_approx(x.y)); }

// a - b as one fused multiply-add (b * -1 + a: the product is exact, so this rounds as the
// subtraction does); for pairs it avoids forming -b lane by lane
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

constexpr float LN2 = 0.6931471805599453f, LOG2E = 1.4426950408889634f;

__device__ __forceinline__ float exp2f_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float log2f_approx(float x)
{
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Phi(-z) = erfc(z / sqrt 2) / 2 with the Chebyshev-fitted erfc of Press et al.
// (Numerical Recipes in C, 2nd ed., section 6.2, "erfcc"; fractional error
// below 1.2e-7 everywhere), so the exponential QE branch keeps its accuracy in
// the upper tail without a library call. That fit is erfc(a) = t exp(-a^2 + P(t)),
// t = 1 / (1 + a / 2), a = |z| / sqrt 2; here it is taken in base 2 with the factor 1/2
// folded into the exponent: h = erfc(a) / 2 = t 2^(Q(t) - z^2 log2(e) / 2), where
// Q = log2(e) P - 1 (phi_q: Press's coefficients times log2 e, the constant term less 1).
constexpr float HALF_LOG2E = 0.7213475108146667f;

__device__ __forceinline__ float phi_q(float t)
{
    float p = 0.24651730060577393f;
    p = fmaf(p, t, -1.1861149072647095f);
    p = fmaf(p, t, 2.147474527359009f);
    p = fmaf(p, t, -1.6377531290054321f);
    p = fmaf(p, t, 0.40232157707214355f);
    p = fmaf(p, t, -0.2687568664550781f);
    p = fmaf(p, t, 0.1396300494670868f);
    p = fmaf(p, t, 0.5397006273269653f);
    p = fmaf(p, t, 1.4427292346954346f);
    p = fmaf(p, t, -2.8257482051849365f);
    return p;
}

__device__ __forceinline__ float2 phi_q2(float2 t)
{
    float2 p = f2s(0.24651730060577393f);
    p = __ffma2_rn(p, t, f2s(-1.1861149072647095f));
    p = __ffma2_rn(p, t, f2s(2.147474527359009f));
    p = __ffma2_rn(p, t, f2s(-1.6377531290054321f));
    p = __ffma2_rn(p, t, f2s(0.40232157707214355f));
    p = __ffma2_rn(p, t, f2s(-0.2687568664550781f));
    p = __ffma2_rn(p, t, f2s(0.1396300494670868f));
    p = __ffma2_rn(p, t, f2s(0.5397006273269653f));
    p = __ffma2_rn(p, t, f2s(1.4427292346954346f));
    p = __ffma2_rn(p, t, f2s(-2.8257482051849365f));
    return p;
}

__device__ __forceinline__ float phi_neg(float z)
{
    const float t = rcp_approx(fmaf(0.3535533845424652f, fabsf(z), 1.0f));
    const float p = phi_q(t);
    const float h = t * exp2f_approx(fmaf(z * z, -HALF_LOG2E, p));
    // Phi(-z) = h for z >= 0 (sign bit clear), 1 - h otherwise, as sg h + off with sg = +-1,
    // off = 0 or 1 (at z = -0, h = 1/2 and both forms give 1/2)
    const float sg = copysignf(1.0f, z);
    return fmaf(sg, h, fmaf(sg, -0.5f, 0.5f));
}

// Andersen QE variance step in FP32 (heston_variance_node.cpp:17-57).
// c = {e, theta (1 - e), A, B}: m = theta + (v - theta) e, s2 = A v + B.
// psi = s2 / m^2 <= 1.5 is tested as s2 <= 1.5 m^2; the exponential branch
// uses 1 - u = Phi(-z) and 1 - p = 2 m^2 / (s2 + m^2), and 1/beta = (s2 + m^2) / (2 m).
// Both branches are evaluated and one is selected: the paths of a warp nearly always take
// both, so this costs no more issue slots than divergence and schedules as one block. The
// quadratic branch's square roots need no guard: where c (c - 1) or b^2 is negative (c < 1,
// psi > 2) the branch is not selected, and its NaN is dropped by the selection.
__device__ __forceinline__ float qe_step(float v, float z, float e, float th1e, float A, float B)
{
    const float m = fmaf(v, e, th1e);
    const float s2 = fmaf(v, A, B);
    const float m2 = m * m;
    const float tm2 = 2.0f * m2;
    // quadratic branch; c is capped at 1e18 (psi >= 2e-18, where the step's random part is
    // below single precision) so that c (c - 1) stays finite for a vanishing vol of vol
    const float c = fminf(tm2 * rcp_approx(s2), 1e18f);
    const float cm1 = c - 1.0f;
    const float b2 = cm1 + fast_sqrt(c * cm1);
    const float a = m * rcp_approx(1.0f + b2);
    const float bz = fast_sqrt(b2) + z;
    const float vq = (a * bz) * bz;
    // exponential branch
    const float num = s2 + m2;
    const float one_m_p = tm2 * rcp_approx(num);
    const float uc = phi_neg(z);
    const float r = (num * rcp_approx(m)) * (log2f_approx(one_m_p * rcp_approx(uc)) * (0.5f * LN2));
    const float ve = (uc >= one_m_p) ? 0.0f : r;
    return (s2 <= 1.5f * m2) ? vq : ve;
}

// phi_neg for a thread's two paths (same expressions, paired)
__device__ __forceinline__ float2 phi_neg2(float2 z)
{
    const float2 t = rcp2_approx(__ffma2_rn(f2s(0.3535533845424652f), f2(fabsf(z.x), fabsf(z.y)), f2s(1.0f)));
    const float2 p = phi_q2(t);
    const float2 g = __ffma2_rn(__fmul2_rn(z, z), f2s(-HALF_LOG2E), p);
    const float2 h = __fmul2_rn(t, f2(exp2f_approx(g.x), exp2f_approx(g.y)));
    const float2 sg = f2(copysignf(1.0f, z.x), copysignf(1.0f, z.y));
    return __ffma2_rn(sg, h, __ffma2_rn(sg, f2s(-0.5f), f2s(0.5f)));
}

// qe_step for a thread's two paths (same expressions, paired)
__device__ __forceinline__ float2 qe_step2(float2 v, float2 z, float e, float th1e, float A, float B)
{
    const float2 m = __ffma2_rn(v, f2s(e), f2s(th1e));
    const float2 s2 = __ffma2_rn(v, f2s(A), f2s(B));
    const float2 m2 = __fmul2_rn(m, m);
    const float2 tm2 = __fmul2_rn(f2s(2.0f), m2);
    const float2 cr = __fmul2_rn(tm2, rcp2_approx(s2));
    const float2 c = f2(fminf(cr.x, 1e18f), fminf(cr.y, 1e18f));
    const float2 cm1 = __fadd2_rn(c, f2s(-1.0f));
    const float2 b2 = __fadd2_rn(cm1, sqrt2_approx(__fmul2_rn(c, cm1)));
    const float2 a = __fmul2_rn(m, rcp2_approx(__fadd2_rn(f2s(1.0f), b2)));
    const float2 bz = __fadd2_rn(sqrt2_approx(b2), z);
    const float2 vq = __fmul2_rn(__fmul2_rn(a, bz), bz);
    const float2 num = __fadd2_rn(s2, m2);
    const float2 one_m_p = __fmul2_rn(tm2, rcp2_approx(num));
    const float2 uc = phi_neg2(z);
    const float2 q = __fmul2_rn(one_m_p, rcp2_approx(uc));
    const float2 r = __fmul2_rn(__fmul2_rn(num, rcp2_approx(m)),
                                __fmul2_rn(f2(log2f_approx(q.x), log2f_approx(q.y)), f2s(0.5f * LN2)));
    const float2 ve = f2(uc.x >= one_m_p.x ? 0.0f : r.x, uc.y >= one_m_p.y ? 0.0f : r.y);
    const float2 lim = __fmul2_rn(f2s(1.5f), m2);
    return f2(s2.x <= lim.x ? vq.x : ve.x, s2.y <= lim.y ? vq.y : ve.y);
}

} // namespace thoth
