// american.cu — Longstaff-Schwartz exercise of a vanilla on its asset's stored paths, the
// algorithm of pricer_mcl_american.cpp:263-447 (FitAmericanPolicy / ApplyAmericanPolicy)
// with the normal-equation solve of helpers/maths.cpp:354-381 and 419-470.
//
// Fit: one cooperative, persistent launch fits every contract of an asset on the same stored
// paths, walking the exercise dates backwards. At each date, for each contract whose grid
// reaches the date, every CTA discounts its paths' cashflows, queues the in-the-money paths so
// that full warps do the FP64 work, and adds the regression moments into the contract's
// per-date totals (exact 128-bit integer atomics). The last CTA to publish solves every
// contract's 3x3 system, one thread each, and releases the others with a flag; every CTA then
// rolls its paths' cashflows back through each contract's exercise decision. The dates are
// sequential and the contracts share them, so one launch with one publish-and-release per
// date replaces a launch per contract and date. The exercise decisions of the backward pass
// are the frozen policy's decisions on the same paths (the same test at the same dates), so
// the earliest exercise the pass records per path is the value the reference's apply step
// finds: the premium comes out of the fit without a second walk over the paths.
//
// Apply: the frozen policy on another path set (the bumped scenarios of the Greeks), one
// forward walk per path that stops at the first exercise.
//
// Sums are exact (exact.cuh), so the regressions, the decisions and the premium do not
// depend on the grid; the arithmetic of each addend, of the solve and of the decision is
// the reference's, operation for operation, in round-to-nearest double with no fused
// multiply-adds (those inside the moneyness quotient give its correctly rounded value).
// GB300 runs FP64 at a small fraction of its FP32 rate, so the per-path work keeps FP64
// to what the result depends on: the in-the-money test is an integer compare on the
// spot's bits, and the quotient S / norm is one multiply and four fused multiply-adds. In
// the apply the exercise test runs in FP32 wherever a proven margin shows that it decides as
// the FP64 test (screen_exercise), which then runs only in a thin band around the boundary.
// (The fit's test, on its compacted lists of full warps, measured faster in FP64.)
#include "american.cuh"

namespace {

constexpr int LSM_WARPS = LSM_THREADS / 32;
static_assert(LSM_WARPS >= LSM_PART, "one warp per regression sum in the cross-CTA reduction");
constexpr int LSM_QCAP = 64; // per-warp queue of in-the-money paths waiting for a full warp
constexpr unsigned long long BARRIER_LIMIT_NS = 2000000000ull; // 2 s

// max(phi (S - K), 0): payoff_vanilla with a floor at 0 (helpers/finance.cpp:9-32)
__device__ __forceinline__ double intrinsic(double s, double k, int call)
{
    const double v = call ? __dsub_rn(s, k) : __dsub_rn(k, s);
    return v < 0.0 ? 0.0 : v;
}

// intrinsic(S) > 0, decided on the single-precision bits of S (integer compare; the
// threshold is exact, see itm_bits)
template <class K>
__device__ __forceinline__ bool in_the_money(float s, const K& A)
{
    const int b = __float_as_int(s);
    return A.call ? b >= A.itm_bits : b <= A.itm_bits;
}

// S / norm rounded to nearest, from y = 1 / norm rounded to nearest. q0 = RN(S y) may be
// more than one ulp off near a power of two; one correction step q1 = RN(q0 + RN(S - norm q0) y)
// brings it within one ulp, and then the remainder S - norm q1 is exact and the second step
// q1 + r y rounded once is the correctly rounded quotient (P. Markstein, IBM J. Res. Dev.
// 34(1), 1990: y within half an ulp of 1 / norm, q1 within one ulp of S / norm).
// Five FP64 operations in place of a full division.
template <class K>
__device__ __forceinline__ double moneyness(double s, const K& A)
{
    const double y = A.inv_norm, b = A.norm;
    const double q0 = __dmul_rn(s, y);
    const double q1 = __fma_rn(__fma_rn(-q0, b, s), y, q0);
    return __fma_rn(__fma_rn(-q1, b, s), y, q1);
}

// b0 + b1 m + b2 m m, evaluated left to right
__device__ __forceinline__ double continuation(double b0, double b1, double b2, double m)
{
    return __dadd_rn(__dadd_rn(b0, __dmul_rn(b1, m)), __dmul_rn(__dmul_rn(b2, m), m));
}

__device__ __forceinline__ void warp_sum(Fx128& a)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long lo = __shfl_xor_sync(0xffffffffu, (unsigned long long)a.lo, o);
        const unsigned long long hi = __shfl_xor_sync(0xffffffffu, (unsigned long long)a.hi, o);
        fx_add(a, (uint64_t)lo, (uint64_t)hi);
    }
}

__device__ __forceinline__ unsigned long long now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void prefetch_l2(const void* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// wait until *flag >= want; false (status 2) after 2 s, or at once when another CTA
// has failed: the caller returns, so no wait outlives the limit
__device__ bool wait_for(const unsigned* flag, unsigned want, int* status)
{
    const unsigned long long t0 = now_ns();
    while (ld_acquire(flag) < want) {
        if (*(volatile int*)status != 0) return false;
        if (now_ns() - t0 > BARRIER_LIMIT_NS) {
            atomicExch(status, 2);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}

// (X^T X) beta = X^T y for X = {1, m, m^2}: Cholesky A = L L^T in place of the lower
// triangle, forward then back substitution (maths.cpp:354-381, 419-470). False when a pivot
// is not positive (the date keeps no regression).
__device__ bool solve3(const double* tot, double* beta)
{
    const double n = tot[LSM_NQ];
    const double s1 = tot[0], s2 = tot[1], s3 = tot[2], s4 = tot[3];
    double A[3][3] = {{n, s1, s2}, {s1, s2, s3}, {s2, s3, s4}};
    const double g[3] = {tot[4], tot[5], tot[6]};
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j <= i; j++) {
            double sum = A[i][j];
            for (int k = 0; k < j; k++) sum = __dsub_rn(sum, __dmul_rn(A[i][k], A[j][k]));
            if (i == j) {
                if (sum <= 0.0) return false;
                A[i][j] = __dsqrt_rn(sum);
            } else {
                A[i][j] = __ddiv_rn(sum, A[j][j]);
            }
        }
    }
    double z[3];
    for (int i = 0; i < 3; i++) {
        double s = g[i];
        for (int k = 0; k < i; k++) s = __dsub_rn(s, __dmul_rn(A[i][k], z[k]));
        z[i] = __ddiv_rn(s, A[i][i]);
    }
    for (int i = 2; i >= 0; i--) {
        double s = z[i];
        for (int k = i + 1; k < 3; k++) s = __dsub_rn(s, __dmul_rn(A[k][i], beta[k]));
        beta[i] = __ddiv_rn(s, A[i][i]);
    }
    return true;
}

// An exact 128-bit sum split into three limbs of 42, 42 and 44 bits, each added into its own
// 64-bit word by a reduction that returns nothing (no round trip for a carry). The limbs of a
// per-CTA sum are below 2^44, so fewer than 2^20 CTAs cannot overflow a word; the solving CTA
// reassembles the exact value.
constexpr uint64_t LIMB42 = (1ull << 42) - 1;

__device__ __forceinline__ void fx_red3(unsigned long long* dst, const Fx128& a)
{
    atomicAdd(dst, (unsigned long long)(a.lo & LIMB42));
    atomicAdd(dst + 1, (unsigned long long)((a.lo >> 42) | ((a.hi & ((1ull << 20) - 1)) << 22)));
    atomicAdd(dst + 2, (unsigned long long)(a.hi >> 20));
}

__device__ __forceinline__ Fx128 fx_from3(const unsigned long long* src)
{
    const uint64_t l0 = __ldcg(src), l1 = __ldcg(src + 1), l2 = __ldcg(src + 2);
    Fx128 r = {l0, 0};
    fx_add(r, l1 << 42, l1 >> 22);
    fx_add(r, 0, l2 << 20);
    return r;
}

// The exercise test iv >= b0 + b1 m + b2 m^2 (iv = phi (S - K), m = S / norm) of an
// in-the-money spot sf, in single precision: 1 exercise, 0 hold, -1 too close to call.
// With u = 2^-24 and mag = |K| + |S| + |b0| + |b1 m| + |b2| m^2, the single-precision
// difference d = iv - c (the inputs rounded to float, then five rounded operations) is within
// 8 u mag of the real iv - c, and the reference's double-precision operands are within
// 6 * 2^-53 mag of it. So |d| > 2^-19 mag (four times that bound, computed from the rounded
// inputs) fixes the sign of the double-precision difference and hence the reference's test;
// an absolute floor keeps underflow out of the bound. Inputs too large for single precision
// give an infinite or NaN d or bound and come back undecided, as does the thin band around
// the exercise boundary: the caller then runs the double-precision test.
template <class K>
__device__ __forceinline__ int screen_exercise(float sf, float b0, float b1, float b2, const K& A)
{
    const float m = sf * A.inv_norm_f;
    const float iv = A.call ? sf - A.strike_f : A.strike_f - sf;
    const float c = fmaf(fmaf(b2, m, b1), m, b0);
    const float d = iv - c;
    const float am = fabsf(m);
    const float mag = fmaf(fabsf(b2) * am, am, fmaf(fabsf(b1), am, fabsf(b0))) + (fabsf(A.strike_f) + fabsf(sf));
    const float e = fmaf(mag, 0x1p-19f, 1e-30f);
    return d > e ? 1 : (d < -e ? 0 : -1);
}

// phi (S - K) in double precision, the reference's intrinsic value of an in-the-money spot
template <class K>
__device__ __forceinline__ double itm_value(float sf, const K& A)
{
    const double s = (double)sf;
    return A.call ? __dsub_rn(s, A.strike) : __dsub_rn(A.strike, s);
}

// one in-the-money path of contract K at the current date: its regression terms into the
// lane's sums, its moneyness and intrinsic value into the warp's compacted list at entry o
__device__ __forceinline__ void itm_item(int p, float sf, double y, const LsmContract& K, Fx128* q, int64_t o,
                                         bool& bad)
{
    const double s = (double)sf;
    const double iv = K.call ? __dsub_rn(s, K.strike) : __dsub_rn(K.strike, s);
    const double m = moneyness(s, K), m2 = __dmul_rn(m, m);
    K.c_idx[o] = p;
    K.c_m[o] = m;
    K.c_iv[o] = iv;
    fx_add_checked(q[0], m, bad);
    fx_add_checked(q[1], m2, bad);
    fx_add_checked(q[2], __dmul_rn(m2, m), bad);
    fx_add_checked(q[3], __dmul_rn(m2, m2), bad);
    fx_add_checked(q[4], y, bad);
    fx_add_checked(q[5], __dmul_rn(m, y), bad);
    fx_add_checked(q[6], __dmul_rn(m2, y), bad);
}

// CTA-wide exact sum of one accumulator per thread into out (thread 0 writes)
__device__ void block_sum(Fx128 a, Fx128 (*s_w)[LSM_PART], int slot, Fx128* out)
{
    warp_sum(a);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_w[warp][slot] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        Fx128 s = {0, 0};
        for (int w = 0; w < LSM_WARPS; w++) fx_add(s, s_w[w][slot]);
        *out = s;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(LSM_THREADS, 1) lsm_fit_kernel(const LsmFitArgs A)
{
    __shared__ Fx128 s_w[LSM_WARPS][LSM_PART];
    __shared__ int q_idx[LSM_WARPS][LSM_QCAP];
    __shared__ float q_s[LSM_WARPS][LSM_QCAP];
    __shared__ double q_y[LSM_WARPS][LSM_QCAP];
    __shared__ LsmContract s_ct[LSM_MAX_CONTRACTS];
    __shared__ int s_nout[LSM_WARPS][LSM_MAX_CONTRACTS];
    __shared__ double s_b[LSM_MAX_CONTRACTS][3];
    __shared__ double s_tot[LSM_MAX_CONTRACTS][LSM_PART];
    __shared__ int s_fit[LSM_MAX_CONTRACTS];
    __shared__ int s_ok, s_last;
    const int G = gridDim.x;
    const int C = A.C;
    const int64_t T = (int64_t)G * LSM_THREADS;
    const int64_t g0 = (int64_t)blockIdx.x * LSM_THREADS + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t gw = (int64_t)blockIdx.x * LSM_WARPS + warp; // global warp: paths gw 32 + lane + k T
    const int64_t seg = gw * A.seg_len;
    const unsigned below = (1u << lane) - 1u;
    bool bad = false;
    for (int c = threadIdx.x; c < C; c += LSM_THREADS) s_ct[c] = A.ct[c];
    __syncthreads();

    // maturity: each contract's cashflow is its payoff, and its value if never exercised earlier
    for (int c = 0; c < C; ++c) {
        const LsmContract K = s_ct[c];
        Fx128 eu = {0, 0};
        const float* row = A.S + (int64_t)(K.M - 1) * A.ld;
        const double dT = K.disc[K.M - 1];
        for (int64_t p = g0; p < A.n; p += T) {
            const double iv = intrinsic((double)row[p], K.strike, K.call);
            const double v = __dmul_rn(iv, dT);
            K.cf[p] = iv;
            K.val[p] = v;
            fx_add_checked(eu, v, bad);
        }
        block_sum(eu, s_w, 2, K.acc + (size_t)blockIdx.x * LSM_NACC + 2);
    }

    unsigned phase = 0; // dates done
    for (int t = A.Tmax - 2; t >= 1; --t) {
        const float* row = A.S + (int64_t)t * A.ld;
        // every contract whose exercise grid reaches date t: discount, queue, sum, publish
        for (int c = 0; c < C; ++c) {
            const LsmContract K = s_ct[c];
            if (t > K.M - 2) continue;
            const double d = K.df[t];
            Fx128 q[LSM_NQ];
#pragma unroll
            for (int i = 0; i < LSM_NQ; i++) q[i] = Fx128{0, 0};
            // in-the-money paths queue until a full warp of them does the FP64 work (the
            // warp's count qn and list length nout are uniform)
            int qn = 0, nout = 0;
            // each lane's next cashflow and spot are loaded one iteration ahead
            double cf_next = gw * 32 + lane < A.n ? K.cf[gw * 32 + lane] : 0.0;
            float s_next = gw * 32 + lane < A.n ? row[gw * 32 + lane] : 0.0f;
            for (int64_t base = gw * 32; base < A.n; base += T) {
                const int64_t p = base + lane;
                const double cf_p = cf_next;
                const float s_p = s_next;
                if (p + T < A.n) {
                    cf_next = K.cf[p + T];
                    s_next = row[p + T];
                }
                bool itm = false;
                float sf = 0.0f;
                double y = 0.0;
                if (p < A.n) {
                    y = __dmul_rn(cf_p, d);
                    K.cf[p] = y;
                    sf = s_p;
                    itm = in_the_money(sf, K);
                }
                const unsigned mk = __ballot_sync(0xffffffffu, itm);
                if (itm) {
                    const int k = qn + __popc(mk & below);
                    q_idx[warp][k] = (int)p;
                    q_s[warp][k] = sf;
                    q_y[warp][k] = y;
                }
                qn += __popc(mk);
                __syncwarp();
                if (qn >= 32) {
                    qn -= 32;
                    const int k = qn + lane;
                    itm_item(q_idx[warp][k], q_s[warp][k], q_y[warp][k], K, q, seg + nout + lane, bad);
                    nout += 32;
                    __syncwarp();
                }
            }
            if (lane < qn) itm_item(q_idx[warp][lane], q_s[warp][lane], q_y[warp][lane], K, q, seg + nout + lane, bad);
            nout += qn;
#pragma unroll
            for (int i = 0; i < LSM_NQ; i++) warp_sum(q[i]);
            if (lane == 0) {
#pragma unroll
                for (int i = 0; i < LSM_NQ; i++) s_w[warp][i] = q[i];
                s_w[warp][LSM_NQ] = Fx128{(uint64_t)nout, 0};
                s_nout[warp][c] = nout;
            }
            __syncthreads();
            if (threadIdx.x < LSM_PART) {
                Fx128 sm = {0, 0};
                for (int w = 0; w < LSM_WARPS; w++) fx_add(sm, s_w[w][threadIdx.x]);
                fx_red3(K.tot + ((size_t)t * LSM_PART + threadIdx.x) * 3, sm);
                __threadfence();
            }
            __syncthreads();
        }
        if (bad) atomicExch(A.status, 3);
        ++phase;
        if (threadIdx.x == 0) s_last = atomicAdd(A.bar, 1u) == phase * (unsigned)G - 1;
        // while the regressions are solved: pull the next date's spots of this warp's paths
        // into L2 (lane k takes the warp's k-th, (k+32)-th, ... line of 32 paths)
        if (t > 1) {
            const float* next = A.S + (int64_t)(t - 1) * A.ld;
            for (int64_t pp = gw * 32 + (int64_t)lane * T; pp < A.n; pp += 32 * T) prefetch_l2(next + pp);
        }
        __syncthreads();
        if (s_last) {
            // the last CTA to publish rounds every active contract's sums (one thread a sum)
            // and solves every contract's system (one thread a contract)
            __threadfence();
            for (int x = threadIdx.x; x < C * LSM_PART; x += LSM_THREADS) {
                const int c = x / LSM_PART, i = x - c * LSM_PART;
                if (t > s_ct[c].M - 2) continue;
                const Fx128 v = fx_from3(s_ct[c].tot + ((size_t)t * LSM_PART + i) * 3);
                s_tot[c][i] = i == LSM_NQ ? (double)v.lo : fx_to_double(v);
            }
            __syncthreads();
            for (int c = threadIdx.x; c < C; c += LSM_THREADS) {
                const LsmContract K = s_ct[c];
                if (t > K.M - 2) continue;
                double b[3] = {0.0, 0.0, 0.0};
                const int f = s_tot[c][LSM_NQ] >= (double)K.min_itm && solve3(s_tot[c], b);
                K.fit[t] = f;
                K.beta[3 * t] = b[0];
                K.beta[3 * t + 1] = b[1];
                K.beta[3 * t + 2] = b[2];
                s_fit[c] = f;
                s_b[c][0] = b[0];
                s_b[c][1] = b[1];
                s_b[c][2] = b[2];
                __threadfence();
            }
            __syncthreads();
            if (threadIdx.x == 0) st_release(A.done, phase);
        } else {
            if (threadIdx.x == 0) s_ok = wait_for(A.done, phase, A.status);
            __syncthreads();
            if (!s_ok) return;
            for (int c = threadIdx.x; c < C; c += LSM_THREADS) {
                const LsmContract K = s_ct[c];
                if (t > K.M - 2) continue;
                s_fit[c] = __ldcg(K.fit + t);
                s_b[c][0] = __ldcg(K.beta + 3 * t);
                s_b[c][1] = __ldcg(K.beta + 3 * t + 1);
                s_b[c][2] = __ldcg(K.beta + 3 * t + 2);
            }
        }
        __syncthreads();
        // every active contract's exercise decision on its list
        for (int c = 0; c < C; ++c) {
            const LsmContract K = s_ct[c];
            if (t > K.M - 2 || !s_fit[c]) continue;
            const double b0 = s_b[c][0], b1 = s_b[c][1], b2 = s_b[c][2];
            const double dt = K.disc[t];
            const int nout = s_nout[warp][c];
            // two entries a lane per pass, their loads issued together
            for (int j = lane; j < nout; j += 64) {
                const int64_t o0 = seg + j, o1 = o0 + 32;
                const bool h1 = j + 32 < nout;
                const double iv0 = K.c_iv[o0], m0 = K.c_m[o0];
                const double iv1 = h1 ? K.c_iv[o1] : 0.0, m1 = h1 ? K.c_m[o1] : 0.0;
                if (iv0 >= continuation(b0, b1, b2, m0)) {
                    const int p = K.c_idx[o0];
                    K.cf[p] = iv0;
                    K.val[p] = __dmul_rn(iv0, dt);
                }
                if (h1 && iv1 >= continuation(b0, b1, b2, m1)) {
                    const int p = K.c_idx[o1];
                    K.cf[p] = iv1;
                    K.val[p] = __dmul_rn(iv1, dt);
                }
            }
        }
        __syncthreads();
    }

    for (int c = 0; c < C; ++c) {
        const LsmContract K = s_ct[c];
        Fx128 v = {0, 0}, v2 = {0, 0};
        for (int64_t p = g0; p < A.n; p += T) {
            const double x = K.val[p];
            fx_add_checked(v, x, bad);
            fx_add_checked(v2, __dmul_rn(x, x), bad);
        }
        Fx128* acc = K.acc + (size_t)blockIdx.x * LSM_NACC;
        block_sum(v, s_w, 0, acc);
        block_sum(v2, s_w, 1, acc + 1);
    }
    if (bad) atomicExch(A.status, 3);
}

constexpr int APPLY_UNROLL = 8; // dates whose spots one thread loads together

__global__ void __launch_bounds__(LSM_THREADS) lsm_apply_kernel(const LsmArgs A)
{
    __shared__ Fx128 s_w[LSM_WARPS][LSM_PART];
    const int64_t T = (int64_t)gridDim.x * LSM_THREADS;
    const int64_t g0 = (int64_t)blockIdx.x * LSM_THREADS + threadIdx.x;
    bool bad = false;
    Fx128 v = {0, 0}, v2 = {0, 0}, eu = {0, 0};
    const float* last = A.S + (int64_t)(A.M - 1) * A.ld;
    const double dT = A.disc[A.M - 1];
    const int tend = A.M - 1; // exercise dates 1 .. M-2; the maturity pays the European payoff
    for (int64_t p = g0; p < A.n; p += T) {
        double x = -1.0;
        // forward walk to the first exercise, APPLY_UNROLL dates at a time so that their
        // loads are in flight together (row t + u of the date-major paths: coalesced in p)
        for (int t = 1; t < tend && x < 0.0; t += APPLY_UNROLL) {
            float sv[APPLY_UNROLL];
#pragma unroll
            for (int u = 0; u < APPLY_UNROLL; ++u)
                sv[u] = t + u < tend ? __ldg(A.S + (int64_t)(t + u) * A.ld + p) : 0.f;
#pragma unroll
            for (int u = 0; u < APPLY_UNROLL; ++u) {
                const int tu = t + u;
                if (tu >= tend) break;
                const float4 b = __ldg(A.screen + tu);
                if (b.w == 0.f || !in_the_money(sv[u], A)) continue;
                int ex = screen_exercise(sv[u], b.x, b.y, b.z, A);
                if (ex < 0)
                    ex = itm_value(sv[u], A) >= continuation(A.beta[3 * tu], A.beta[3 * tu + 1], A.beta[3 * tu + 2],
                                                             moneyness((double)sv[u], A));
                if (ex) {
                    x = __dmul_rn(itm_value(sv[u], A), A.disc[tu]);
                    break;
                }
            }
        }
        const double e = __dmul_rn(intrinsic((double)last[p], A.strike, A.call), dT);
        if (x < 0.0) x = e;
        fx_add_checked(v, x, bad);
        fx_add_checked(v2, __dmul_rn(x, x), bad);
        fx_add_checked(eu, e, bad);
    }
    if (bad) atomicExch(A.status, 3);
    Fx128* acc = A.acc + (size_t)blockIdx.x * LSM_NACC;
    block_sum(v, s_w, 0, acc);
    block_sum(v2, s_w, 1, acc + 1);
    block_sum(eu, s_w, 2, acc + 2);
}

} // namespace

int lsm_fit_max_grid(int sms)
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lsm_fit_kernel, LSM_THREADS, 0) != cudaSuccess) return 0;
    return per * sms;
}

cudaError_t launch_lsm_fit(const LsmFitArgs& A, int grid, cudaStream_t st)
{
    LsmFitArgs a = A;
    void* args[] = {&a};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(lsm_fit_kernel), dim3(grid), dim3(LSM_THREADS),
                                       args, 0, st);
}

cudaError_t launch_lsm_apply(const LsmArgs& A, int grid, cudaStream_t st)
{
    lsm_apply_kernel<<<grid, LSM_THREADS, 0, st>>>(A);
    return cudaGetLastError();
}
