// calib.cu — LSV leverage calibration by the binned particle method, the algorithm of
// Single::CalibrateLeverage and its helpers (pricer/src/marketdata/single.cpp:240-473) with
// the reference Rng (helpers/rng.hpp) and inverse normal (helpers/distributions.cpp:37-81).
//
// One cooperative launch walks the dates. Per date, two publish-and-release rounds build
// the conditional variance of the current ensemble: (A) the extremes of ln S and the sum of
// v, (B) per-bin counts and sums of v between those extremes. The last CTA to publish in a
// round adds every CTA's contribution (exact integer sums), and after round B computes the
// bin means, fills thin bins and writes layer k of the surface; the others wait for its
// release flag. Every CTA then steps its particles into date k with layer k, read from
// shared memory.
//
// The Gaussians are the reference's stream: xoshiro256++ seeded by splitmix64, one 64-bit
// draw per Gaussian through Acklam's inverse normal, two per particle per date in particle
// order. Each particle keeps its own generator state: it starts 2p draws into the stream and
// jumps 2P - 2 draws after each date. The generator is linear over GF(2), so a jump by d
// draws is the polynomial x^d mod chi (chi the characteristic polynomial of the transition)
// evaluated at the transition: 256 transitions and XORs (F. Haramoto et al., "Efficient jump
// ahead for F2-linear random number generators", INFORMS J. Computing 20(3), 2008).
//
// Compiled without FMA contraction: every expression rounds as the reference's does, so the
// ensemble differs from the reference's only where CUDA's exp, log and erfc differ from the
// host's in the last bit. The sums of v are exact (exact.cuh), independent of the grid.
#include "calib.cuh"

#include <mutex>
#include <vector>

namespace {

constexpr int CALIB_WARPS = CALIB_THREADS / 32;
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull; // 2 s

__host__ __device__ __forceinline__ uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

// xoshiro256++: output, then the state transition (helpers/rng.hpp:50-62)
__host__ __device__ __forceinline__ uint64_t xo_next(uint64_t* s)
{
    const uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

__host__ __device__ __forceinline__ void xo_step(uint64_t* s)
{
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
}

// s <- q(A) s for q = sum_i poly_i x^i: the state sum_i poly_i A^i s
__host__ __device__ void xo_jump(const uint64_t* poly, uint64_t* s)
{
    uint64_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    for (int w = 0; w < 4; w++) {
        uint64_t bits = poly[w];
        for (int b = 0; b < 64; b++) {
            if (bits & 1u) {
                r0 ^= s[0];
                r1 ^= s[1];
                r2 ^= s[2];
                r3 ^= s[3];
            }
            bits >>= 1;
            xo_step(s);
        }
    }
    s[0] = r0;
    s[1] = r1;
    s[2] = r2;
    s[3] = r3;
}

// the fixed date-to-date jump by its nibble table in shared memory: the XOR of the table
// rows the state's 64 nibbles select (the matrix-vector product over GF(2))
__device__ __forceinline__ void xo_jump_tab(const uint64_t* tab, uint64_t* s)
{
    uint64_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
#pragma unroll
    for (int w = 0; w < 4; w++) {
        uint64_t x = s[w];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const ulonglong2* t = reinterpret_cast<const ulonglong2*>(tab + ((w * 16 + k) * 16 + (int)(x & 15u)) * 4);
            const ulonglong2 a = t[0], b = t[1];
            r0 ^= a.x;
            r1 ^= a.y;
            r2 ^= b.x;
            r3 ^= b.y;
            x >>= 4;
        }
    }
    s[0] = r0;
    s[1] = r1;
    s[2] = r2;
    s[3] = r3;
}

// Acklam's inverse normal as the reference evaluates it (NormalCdfInv). Both the tail and
// the central rational are evaluated and one is selected: the selected value is the same
// expression the reference evaluates, and without branches the compiler can interleave the
// particle's independent FP64 chains (two Gaussians, the layer lookup).
__device__ double normal_cdf_inv(double P)
{
    const double a0 = -3.969683028665376e+01, a1 = 2.209460984245205e+02, a2 = -2.759285104469687e+02,
                 a3 = 1.383577518672690e+02, a4 = -3.066479806614716e+01, a5 = 2.506628277459239e+00;
    const double b0 = -5.447609879822406e+01, b1 = 1.615858368580409e+02, b2 = -1.556989798598866e+02,
                 b3 = 6.680131188771972e+01, b4 = -1.328068155288572e+01;
    const double c0 = -7.784894002430293e-03, c1 = -3.223964580411365e-01, c2 = -2.400758277161838e+00,
                 c3 = -2.549732539343734e+00, c4 = 4.374664141464968e+00, c5 = 2.938163982698783e+00;
    const double d0 = 7.784695709041462e-03, d1 = 3.224671290700398e-01, d2 = 2.445134137142996e+00,
                 d3 = 3.754408661907416e+00;
    const double p_low = 0.02425, p_high = 1.0 - p_low;
    const bool lower = P < p_low, upper = !(P <= p_high);
    // tail: q = sqrt(-2 ln P) below, sqrt(-2 ln(1 - P)) above (1 - P is exact where it is used)
    const double qt = sqrt(-2.0 * log(lower ? P : 1.0 - P));
    const double tn = ((((c0 * qt + c1) * qt + c2) * qt + c3) * qt + c4) * qt + c5;
    const double td = (((d0 * qt + d1) * qt + d2) * qt + d3) * qt + 1.0;
    const double q = P - 0.5;
    const double r = q * q;
    const double cn = (((((a0 * r + a1) * r + a2) * r + a3) * r + a4) * r + a5) * q;
    const double cd = ((((b0 * r + b1) * r + b2) * r + b3) * r + b4) * r + 1.0;
    const double num = lower ? tn : (upper ? -tn : cn);
    const double den = (lower || upper) ? td : cd;
    return num / den;
}

// Rng::Gaussian: a 53-bit uniform in (0, 1) through the inverse normal
__device__ __forceinline__ double gaussian(uint64_t* s)
{
    const double u0 = (double)(xo_next(s) >> 11) * (1.0 / 9007199254740992.0);
    return normal_cdf_inv(u0 > 0.0 ? u0 : (1.0 / 9007199254740992.0));
}

// QeVarianceStep (single.cpp:344-368) with e = exp(-kappa Dt) rounded on the host
__device__ double qe_step(double V, double Z, double e, const CalibArgs& A)
{
    const double m = A.theta + (V - A.theta) * e;
    const double s2 = V * A.xi * A.xi * e / A.kappa * (1 - e) + A.theta * A.xi * A.xi / (2 * A.kappa) * (1 - e) * (1 - e);
    const double psi = (m > 0) ? s2 / (m * m) : 0;
    if (psi <= 1.5) {
        const double c = 2.0 / psi;
        const double b2 = c - 1.0 + sqrt(c) * sqrt(c - 1.0);
        const double a = m / (1.0 + b2);
        const double bz = sqrt(b2) + Z;
        return a * bz * bz;
    }
    const double p = (psi - 1.0) / (psi + 1.0);
    const double beta = (1.0 - p) / m;
    const double u = 0.5 * erfc(-Z / sqrt(2.0));
    return (u <= p) ? 0.0 : log((1.0 - p) / (1.0 - u)) / beta;
}

// LeveragedLogSpotStep (single.cpp:370-388)
__device__ double spot_step(double Vp, double Vc, double Dt, double Carry, double L, double Z, const CalibArgs& A)
{
    if (A.xi > 1e-12) {
        const double g = 0.5;
        const double k0 = -L * A.rho * A.kappa * A.theta / A.xi * Dt;
        const double a = g * Dt * (L * A.kappa * A.rho / A.xi - 0.5 * L * L);
        const double k1 = a - L * A.rho / A.xi;
        const double k2 = a + L * A.rho / A.xi;
        const double k3 = g * Dt * (1.0 - A.rho * A.rho) * L * L;
        double var = k3 * (Vp + Vc);
        if (var < 0) var = 0;
        return Carry + k0 + k1 * Vp + k2 * Vc + sqrt(var) * Z;
    }
    return Carry - 0.5 * L * L * Vp * Dt + L * sqrt(Vp * Dt) * Z;
}

// LeverageSurface::LayerAt (leverage_surface.cpp:19-40) on a layer in shared memory: the
// clamps select instead of branching (the interpolation index is clamped to the layer, and
// its value is only selected where the reference interpolates)
__device__ __forceinline__ double layer_at(const double* lev, int points, double ln_step, int64_t offset, double S)
{
    const double f = log(S) / ln_step - (double)offset;
    const int last = points - 1;
    const bool inside = f > 0.0 && f < (double)last;
    const int i = inside ? (int)f : 0;
    const double w = f - (double)i;
    const double mid = (1.0 - w) * lev[i] + w * lev[i + 1];
    return !(f > 0.0) ? lev[0] : (f >= (double)last ? lev[last] : mid);
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

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// wait until *flag >= want; false (status 2) after 2 s, or at once when another CTA failed
__device__ bool wait_for(const unsigned* flag, unsigned want, int* status)
{
    const unsigned long long t0 = now_ns();
    while (ld_acquire(flag) < want) {
        if (*(volatile int*)status != 0) return false;
        if (now_ns() - t0 > WAIT_LIMIT_NS) {
            atomicExch(status, 2);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}

// a double's bit pattern as a signed integer with the same order
__device__ __forceinline__ long long order_key(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

__device__ __forceinline__ double from_key(long long k)
{
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

// exact 128-bit add into global memory: the low word's returned old value gives the carry
__device__ __forceinline__ void fx_atomic_add(Fx128* dst, const Fx128& a)
{
    unsigned long long* w = reinterpret_cast<unsigned long long*>(dst);
    const unsigned long long old = atomicAdd(w, (unsigned long long)a.lo);
    const unsigned long long carry = (old + (unsigned long long)a.lo < old) ? 1ull : 0ull;
    if (a.hi + carry) atomicAdd(w + 1, (unsigned long long)(a.hi + carry));
}

__device__ __forceinline__ Fx128 fx_load_cg(const Fx128* p)
{
    const unsigned long long* w = reinterpret_cast<const unsigned long long*>(p);
    return Fx128{(uint64_t)__ldcg(w), (uint64_t)__ldcg(w + 1)};
}

// the two 64-bit words x adds to an Fx128 (x >= 0, truncated to 2^-64); bad when out of range
__device__ __forceinline__ void fx_words(double x, uint64_t& lo, uint64_t& hi, bool& bad)
{
    Fx128 t = {0, 0};
    fx_add_checked(t, x, bad);
    lo = t.lo;
    hi = t.hi;
}

// layer k from the conditional variance cv(x) of the published bins (all threads of the CTA)
__device__ void build_layer(const CalibArgs& A, int k, bool flat, double fallback, double x0, double dx,
                            const double* mean)
{
    const double ls = A.ln_step[k];
    const int64_t off = A.offset[k];
    for (int i = threadIdx.x; i < A.points; i += CALIB_THREADS) {
        const double x = (double)(off + i) * ls;
        double ev;
        if (flat) {
            ev = fallback;
        } else {
            const double f = (x - x0) / dx;
            const double last = (double)(A.bins - 1);
            if (f <= 0) {
                ev = mean[0];
            } else if (f >= last) {
                ev = mean[A.bins - 1];
            } else {
                const int j = (int)f;
                const double w = f - (double)j;
                ev = (1.0 - w) * mean[j] + w * mean[j + 1];
            }
        }
        if (ev < A.min_cv) ev = A.min_cv;
        const double L = A.local_vol[(size_t)k * A.points + i] / sqrt(ev);
        A.lev[(size_t)k * A.points + i] = L < A.lmin ? A.lmin : (L > A.lmax ? A.lmax : L);
    }
}

__global__ void __launch_bounds__(CALIB_THREADS) lsv_calib_kernel(const CalibArgs A)
{
    extern __shared__ __align__(16) unsigned char s_dyn[]; // the jump table, then the layer [points]
    uint64_t* s_jtab = reinterpret_cast<uint64_t*>(s_dyn);
    double* s_layer = reinterpret_cast<double*>(s_dyn + sizeof(uint64_t) * CALIB_JTAB_WORDS);
    __shared__ double s_min[CALIB_WARPS], s_max[CALIB_WARPS];
    __shared__ Fx128 s_sum[CALIB_WARPS];
    __shared__ unsigned s_cnt[CALIB_MAX_BINS];
    __shared__ unsigned long long s_blo[CALIB_MAX_BINS], s_bhi[CALIB_MAX_BINS];
    __shared__ double s_bsum[CALIB_MAX_BINS], s_mean[CALIB_MAX_BINS];
    __shared__ double s_bc[4];
    __shared__ int s_last, s_ok;
    const int G = gridDim.x;
    const int T = G * CALIB_THREADS;
    const int gt = blockIdx.x * CALIB_THREADS + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int P = A.P, bins = A.bins;
    bool bad = false;

    for (int i = threadIdx.x; i < (int)CALIB_JTAB_WORDS; i += CALIB_THREADS) s_jtab[i] = A.jtab[i];
    __syncthreads();
    // the ensemble at today; particle p's generator at draw 2p of the stream
    for (int p = gt; p < P; p += T) {
        A.spot[p] = A.s0;
        A.var[p] = A.v0;
        A.lns[p] = A.ln_s0;
        uint64_t s[4] = {A.seed_state[0], A.seed_state[1], A.seed_state[2], A.seed_state[3]};
        const uint64_t off = 2ull * (uint64_t)p;
        for (int i = 0; i < CALIB_JUMP_BITS; i++)
            if ((off >> i) & 1u) xo_jump(A.jpow + 4 * i, s);
        for (int w = 0; w < 4; w++) A.rng[(size_t)w * P + p] = s[w];
    }

    unsigned round = 0;
    for (int k = 0; k < A.n; k++) {
        // ---- round A: extremes of ln S, sum of v ----
        double mn = INFINITY, mx = -INFINITY;
        Fx128 sv = {0, 0};
        for (int p = gt; p < P; p += T) {
            const double x = A.lns[p];
            mn = fmin(mn, x);
            mx = fmax(mx, x);
            fx_add_checked(sv, A.var[p], bad);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        warp_sum(sv);
        if (lane == 0) {
            s_min[warp] = mn;
            s_max[warp] = mx;
            s_sum[warp] = sv;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double cm = s_min[0], cx = s_max[0];
            Fx128 cs = s_sum[0];
            for (int w = 1; w < CALIB_WARPS; w++) {
                cm = fmin(cm, s_min[w]);
                cx = fmax(cx, s_max[w]);
                fx_add(cs, s_sum[w]);
            }
            if (cm <= cx) { // a CTA without particles adds nothing
                atomicMin(A.kmin + k, order_key(cm));
                atomicMax(A.kmax + k, order_key(cx));
                fx_atomic_add(A.vsum + k, cs);
            }
            __threadfence();
        }
        if (bad) atomicExch(A.status, 3);
        ++round;
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(A.bar, 1u) == round * (unsigned)G - 1;
        __syncthreads();
        if (s_last) {
            if (threadIdx.x == 0) {
                __threadfence();
                const double gmn = from_key((long long)__ldcg((const unsigned long long*)(A.kmin + k)));
                const double gmx = from_key((long long)__ldcg((const unsigned long long*)(A.kmax + k)));
                s_bc[0] = gmn;
                s_bc[1] = (gmx - gmn) / bins;
                s_bc[2] = fx_to_double(fx_load_cg(A.vsum + k)) / (double)P;
                s_bc[3] = (gmx - gmn < 1e-10) ? 1.0 : 0.0;
                for (int j = 0; j < 4; j++) A.bc[j] = s_bc[j];
            }
            __syncthreads();
            if (s_bc[3] != 0.0) build_layer(A, k, true, s_bc[2], 0.0, 1.0, s_mean);
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                st_release(A.done, round);
            }
        } else if (threadIdx.x == 0) {
            const bool ok = wait_for(A.done, round, A.status);
            if (ok)
                for (int j = 0; j < 4; j++) s_bc[j] = __ldcg(A.bc + j);
            s_ok = ok;
        }
        __syncthreads();
        if (!s_last && !s_ok) return;

        if (s_bc[3] == 0.0) {
            // ---- round B: per-bin counts and sums of v ----
            const double bmn = s_bc[0], width = s_bc[1];
            for (int b = threadIdx.x; b < bins; b += CALIB_THREADS) {
                s_cnt[b] = 0;
                s_blo[b] = 0;
                s_bhi[b] = 0;
            }
            __syncthreads();
            for (int p = gt; p < P; p += T) {
                int b = (int)((A.lns[p] - bmn) / width);
                b = b < 0 ? 0 : (b > bins - 1 ? bins - 1 : b);
                uint64_t lo, hi;
                fx_words(A.var[p], lo, hi, bad);
                atomicAdd(&s_cnt[b], 1u);
                const unsigned long long old = atomicAdd(&s_blo[b], (unsigned long long)lo);
                atomicAdd(&s_bhi[b], (unsigned long long)(hi + ((uint64_t)old + lo < lo ? 1u : 0u)));
            }
            __syncthreads();
            for (int b = threadIdx.x; b < bins; b += CALIB_THREADS) {
                if (s_cnt[b]) {
                    atomicAdd(A.bcnt + (size_t)k * bins + b, s_cnt[b]);
                    fx_atomic_add(A.bsum + (size_t)k * bins + b, Fx128{s_blo[b], s_bhi[b]});
                }
                __threadfence();
            }
            if (bad) atomicExch(A.status, 3);
            ++round;
            __syncthreads();
            if (threadIdx.x == 0) s_last = atomicAdd(A.bar, 1u) == round * (unsigned)G - 1;
            __syncthreads();
            if (s_last) {
                __threadfence();
                for (int b = threadIdx.x; b < bins; b += CALIB_THREADS) {
                    s_bsum[b] = fx_to_double(fx_load_cg(A.bsum + (size_t)k * bins + b));
                    s_cnt[b] = __ldcg(A.bcnt + (size_t)k * bins + b);
                }
                __syncthreads();
                __syncthreads();
                // populated bins, then each thin bin from its nearest populated one, left first
                // (one thread a bin: the fill reads only populated bins)
                const unsigned mc = (unsigned)A.min_count;
                for (int b = threadIdx.x; b < bins; b += CALIB_THREADS) {
                    double mv = s_bc[2];
                    if (s_cnt[b] >= mc) {
                        mv = s_bsum[b] / s_cnt[b];
                    } else {
                        for (int d = 1; d < bins; d++) {
                            if (b - d >= 0 && s_cnt[b - d] >= mc) {
                                mv = s_bsum[b - d] / s_cnt[b - d];
                                break;
                            }
                            if (b + d < bins && s_cnt[b + d] >= mc) {
                                mv = s_bsum[b + d] / s_cnt[b + d];
                                break;
                            }
                        }
                    }
                    s_mean[b] = mv;
                }
                __syncthreads();
                build_layer(A, k, false, s_bc[2], bmn + 0.5 * width, width, s_mean);
                __syncthreads();
                if (threadIdx.x == 0) {
                    __threadfence();
                    st_release(A.done, round);
                }
            } else if (threadIdx.x == 0) {
                s_ok = wait_for(A.done, round, A.status);
            }
            __syncthreads();
            if (!s_last && !s_ok) return;
        }
        if (k == 0) continue;

        // ---- the step into date k with layer k ----
        for (int i = threadIdx.x; i < A.points; i += CALIB_THREADS) s_layer[i] = __ldcg(A.lev + (size_t)k * A.points + i);
        __syncthreads();
        const double dt = A.dt[k], carry = A.carry[k], e = A.qe_e[k], ls = A.ln_step[k];
        const int64_t off = A.offset[k];
        for (int p = gt; p < P; p += T) {
            uint64_t s[4];
            for (int w = 0; w < 4; w++) s[w] = A.rng[(size_t)w * P + p];
            // both Gaussians in draw order (the variance's first) and the layer lookup before
            // the branched QE step: three independent chains in one block
            const double z1 = gaussian(s);
            const double z2 = gaussian(s);
            const double lp = layer_at(s_layer, A.points, ls, off, A.spot[p]);
            const double vp = A.var[p];
            const double vc = qe_step(vp, z1, e, A);
            const double step = spot_step(vp, vc, dt, carry, lp, z2, A);
            A.var[p] = vc;
            A.spot[p] *= exp(step);
            A.lns[p] += step;
            xo_jump_tab(s_jtab, s);
            for (int w = 0; w < 4; w++) A.rng[(size_t)w * P + p] = s[w];
        }
        __syncthreads();
    }
}

// ---- host: GF(2) polynomials of degree < 256 as 4 words, bit i = coefficient of x^i ----
struct Poly {
    uint64_t w[4];
};

std::mutex g_chi_mu;
bool g_chi_ready = false;
Poly g_chi;                           // chi - x^256
Poly g_pow2[CALIB_JUMP_BITS + 24];    // x^(2^i) mod chi

bool bit(const Poly& p, int i) { return (p.w[i >> 6] >> (i & 63)) & 1u; }

// a b mod chi (Horner over the bits of b, high to low)
Poly mulmod(const Poly& a, const Poly& b)
{
    Poly r = {{0, 0, 0, 0}};
    for (int i = 255; i >= 0; i--) {
        const bool top = (r.w[3] >> 63) & 1u; // r x overflows into x^256 = chi - x^256
        r.w[3] = (r.w[3] << 1) | (r.w[2] >> 63);
        r.w[2] = (r.w[2] << 1) | (r.w[1] >> 63);
        r.w[1] = (r.w[1] << 1) | (r.w[0] >> 63);
        r.w[0] <<= 1;
        if (top)
            for (int j = 0; j < 4; j++) r.w[j] ^= g_chi.w[j];
        if (bit(b, i))
            for (int j = 0; j < 4; j++) r.w[j] ^= a.w[j];
    }
    return r;
}

// chi from the minimal polynomial of one state bit's sequence (Berlekamp-Massey over GF(2));
// the transition's characteristic polynomial is primitive of degree 256, so any nonzero
// sequence has it as its minimal polynomial
bool find_chi()
{
    const int N = 512;
    std::vector<uint8_t> s(N);
    uint64_t st[4];
    xo_seed_state(1, st);
    for (int i = 0; i < N; i++) {
        s[i] = (uint8_t)(st[0] & 1u);
        xo_advance(st);
    }
    std::vector<uint8_t> C(N + 1, 0), B(N + 1, 0), Tm;
    C[0] = B[0] = 1;
    int L = 0, m = 1;
    for (int n = 0; n < N; n++) {
        uint8_t d = s[n];
        for (int i = 1; i <= L; i++) d ^= (uint8_t)(C[i] & s[n - i]);
        if (!d) {
            m++;
        } else if (2 * L <= n) {
            Tm = C;
            for (int i = 0; i + m <= N; i++) C[i + m] ^= B[i];
            L = n + 1 - L;
            B = Tm;
            m = 1;
        } else {
            for (int i = 0; i + m <= N; i++) C[i + m] ^= B[i];
            m++;
        }
    }
    if (L != 256) return false;
    // chi(x) = x^256 C(1/x): the coefficient of x^(256 - i) is C[i]
    Poly c = {{0, 0, 0, 0}};
    for (int i = 1; i <= 256; i++)
        if (C[i]) {
            const int e = 256 - i;
            c.w[e >> 6] |= 1ull << (e & 63);
        }
    g_chi = c;
    Poly x = {{2, 0, 0, 0}};
    g_pow2[0] = x;
    for (int i = 1; i < CALIB_JUMP_BITS + 24; i++) g_pow2[i] = mulmod(g_pow2[i - 1], g_pow2[i - 1]);
    return true;
}

// ---- the reference Rng's stream for the book kernel's tail dimensions -------------------
__constant__ uint64_t c_xo_pow2[64 * 4]; // x^(2^i) mod chi for i < 64

struct TailSeed {
    uint64_t s[4];
};

constexpr int TAIL_THREADS = 128;
constexpr int TAIL_WARPS = TAIL_THREADS / 32;
constexpr int TAIL_PATHS_PER_THREAD = 16;
constexpr double ACKLAM_P_LOW = 0.02425;

// normal_cdf_inv's two branches apart, each the same expression the reference evaluates there
__device__ __forceinline__ double acklam_central(double P) // P in [p_low, 1 - p_low]
{
    const double a0 = -3.969683028665376e+01, a1 = 2.209460984245205e+02, a2 = -2.759285104469687e+02,
                 a3 = 1.383577518672690e+02, a4 = -3.066479806614716e+01, a5 = 2.506628277459239e+00;
    const double b0 = -5.447609879822406e+01, b1 = 1.615858368580409e+02, b2 = -1.556989798598866e+02,
                 b3 = 6.680131188771972e+01, b4 = -1.328068155288572e+01;
    const double q = P - 0.5;
    const double r = q * q;
    const double cn = (((((a0 * r + a1) * r + a2) * r + a3) * r + a4) * r + a5) * q;
    const double cd = ((((b0 * r + b1) * r + b2) * r + b3) * r + b4) * r + 1.0;
    return cn / cd;
}

__device__ __forceinline__ double acklam_tail(double P) // P < p_low or P > 1 - p_low
{
    const double c0 = -7.784894002430293e-03, c1 = -3.223964580411365e-01, c2 = -2.400758277161838e+00,
                 c3 = -2.549732539343734e+00, c4 = 4.374664141464968e+00, c5 = 2.938163982698783e+00;
    const double d0 = 7.784695709041462e-03, d1 = 3.224671290700398e-01, d2 = 2.445134137142996e+00,
                 d3 = 3.754408661907416e+00;
    const bool lower = P < ACKLAM_P_LOW;
    const double qt = sqrt(-2.0 * log(lower ? P : 1.0 - P));
    const double tn = ((((c0 * qt + c1) * qt + c2) * qt + c3) * qt + c4) * qt + c5;
    const double td = (((d0 * qt + d1) * qt + d2) * qt + d3) * qt + 1.0;
    return (lower ? tn : -tn) / td;
}

// thread k draws the tail Gaussians of paths [16 k, 16 k + 16): one jump to its first path's
// place in the stream (p dt draws in: the binary powers of x), then its paths' draws in stream
// order, as the reference's NextPath draws them. A draw in the central region is inverted at
// once; one in a tail (4.85 % of them) waits in its warp's queue in shared memory, and 32
// queued draws are inverted at once on the warp's 32 lanes, so the logarithm runs on full
// warps instead of on most warps' iterations.
__global__ void __launch_bounds__(TAIL_THREADS) tail_normals_kernel(const TailSeed s0, int dt, int64_t paths,
                                                                    float* __restrict__ out)
{
    __shared__ double q_u[TAIL_WARPS][64];
    __shared__ uint32_t q_i[TAIL_WARPS][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t p0 = ((int64_t)blockIdx.x * TAIL_THREADS + threadIdx.x) * TAIL_PATHS_PER_THREAD;
    const bool live = p0 < paths;
    if (__all_sync(0xffffffffu, !live)) return; // warp-uniform
    const int np = live ? (int)(paths - p0 < TAIL_PATHS_PER_THREAD ? paths - p0 : TAIL_PATHS_PER_THREAD) : 0;
    uint64_t s[4] = {s0.s[0], s0.s[1], s0.s[2], s0.s[3]};
    if (live) {
        const uint64_t pos = (uint64_t)p0 * (uint64_t)dt;
        for (int i = 0; i < 64; i++)
            if ((pos >> i) & 1u) xo_jump(c_xo_pow2 + 4 * i, s);
    }
    int qn = 0; // the warp's queue length (the same on every lane)
    for (int pl = 0; pl < TAIL_PATHS_PER_THREAD; pl++) {
        const bool act = pl < np;
        for (int d = 0; d < dt; d++) {
            double u = 0.0;
            uint32_t idx = 0;
            bool tail = false;
            if (act) {
                const double u0 = (double)(xo_next(s) >> 11) * (1.0 / 9007199254740992.0);
                u = u0 > 0.0 ? u0 : (1.0 / 9007199254740992.0);
                idx = (uint32_t)((size_t)d * (size_t)paths + (size_t)(p0 + pl)); // < 2^31: the table's size limit
                tail = u < ACKLAM_P_LOW || !(u <= 1.0 - ACKLAM_P_LOW);
                if (!tail) out[idx] = (float)acklam_central(u);
            }
            const unsigned m = __ballot_sync(0xffffffffu, tail);
            if (tail) {
                const int slot = qn + __popc(m & ((1u << lane) - 1u)); // < 63
                q_u[w][slot] = u;
                q_i[w][slot] = idx;
            }
            qn += __popc(m);
            if (qn >= 32) { // 32 to 63 entries: invert the first 32, keep the rest
                __syncwarp();
                out[q_i[w][lane]] = (float)acklam_tail(q_u[w][lane]);
                const int rest = qn - 32;
                double mu = 0.0;
                uint32_t mi = 0;
                if (lane < rest) {
                    mu = q_u[w][32 + lane];
                    mi = q_i[w][32 + lane];
                }
                __syncwarp();
                if (lane < rest) {
                    q_u[w][lane] = mu;
                    q_i[w][lane] = mi;
                }
                __syncwarp();
                qn = rest;
            }
        }
    }
    __syncwarp();
    if (lane < qn) out[q_i[w][lane]] = (float)acklam_tail(q_u[w][lane]);
}

} // namespace

void xo_seed_state(uint64_t seed, uint64_t s[4])
{
    uint64_t z = seed;
    for (int i = 0; i < 4; i++) {
        z += 0x9e3779b97f4a7c15ULL;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
        s[i] = x ^ (x >> 31);
    }
}

void xo_advance(uint64_t s[4]) { xo_step(s); }

bool xo_jump_poly(uint64_t d, uint64_t out[4])
{
    {
        std::lock_guard<std::mutex> lk(g_chi_mu);
        if (!g_chi_ready) {
            if (!find_chi()) return false;
            g_chi_ready = true;
        }
    }
    Poly r = {{1, 0, 0, 0}};
    for (int i = 0; i < 64; i++)
        if ((d >> i) & 1u) {
            if (i >= CALIB_JUMP_BITS + 24) return false;
            r = mulmod(r, g_pow2[i]);
        }
    for (int j = 0; j < 4; j++) out[j] = r.w[j];
    return true;
}

void xo_apply_jump(const uint64_t poly[4], uint64_t s[4]) { xo_jump(poly, s); }

void xo_jump_table(const uint64_t poly[4], uint64_t* tab)
{
    // column i of the jump matrix: the jump of the state with only bit i set
    std::vector<uint64_t> col(256 * 4);
    for (int i = 0; i < 256; i++) {
        uint64_t e[4] = {0, 0, 0, 0};
        e[i >> 6] = 1ull << (i & 63);
        xo_jump(poly, e);
        for (int w = 0; w < 4; w++) col[i * 4 + w] = e[w];
    }
    for (int n = 0; n < 64; n++)
        for (int v = 0; v < 16; v++) {
            uint64_t r[4] = {0, 0, 0, 0};
            for (int b = 0; b < 4; b++)
                if ((v >> b) & 1)
                    for (int w = 0; w < 4; w++) r[w] ^= col[(4 * n + b) * 4 + w];
            for (int w = 0; w < 4; w++) tab[(n * 16 + v) * 4 + w] = r[w];
        }
}

int calib_max_grid(int sms, size_t smem)
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lsv_calib_kernel, CALIB_THREADS, smem) != cudaSuccess)
        return 0;
    return per * sms;
}

cudaError_t launch_calib(const CalibArgs& A, int grid, size_t smem, cudaStream_t st)
{
    CalibArgs a = A;
    void* args[] = {&a};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(lsv_calib_kernel), dim3(grid),
                                       dim3(CALIB_THREADS), args, smem, st);
}

cudaError_t tail_normals_prepare()
{
    static std::mutex mu;
    static bool ready[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && ready[dev]) return cudaSuccess;
    std::vector<uint64_t> pw(64 * 4);
    for (int i = 0; i < 64; i++)
        if (!xo_jump_poly(1ull << i, pw.data() + 4 * i)) return cudaErrorUnknown;
    e = cudaMemcpyToSymbol(c_xo_pow2, pw.data(), sizeof(uint64_t) * pw.size());
    if (e == cudaSuccess && dev >= 0 && dev < 64) ready[dev] = true;
    return e;
}

cudaError_t launch_tail_normals(uint64_t seed, int dt, int64_t paths, float* out, cudaStream_t st)
{
    if (dt <= 0 || paths <= 0) return cudaSuccess;
    TailSeed s0;
    xo_seed_state(seed, s0.s);
    const int64_t threads = (paths + TAIL_PATHS_PER_THREAD - 1) / TAIL_PATHS_PER_THREAD;
    const unsigned blocks = (unsigned)((threads + TAIL_THREADS - 1) / TAIL_THREADS);
    tail_normals_kernel<<<blocks, TAIL_THREADS, 0, st>>>(s0, dt, paths, out);
    return cudaGetLastError();
}
