// book.cuh — the persistent book kernel (book_kernel) and its launch templates,
// instantiated per model by book_gbm.cu, book_heston.cu, book_lsv.cu and
// book_multi.cu, so that the variants compile as separate translation units.
// The host-side sizing (smem_bytes) is shared with kernels.cu and the plan builder.
#pragma once

#include "engine.cuh"

#include <cuda_runtime.h>

namespace thoth {

// ---------------------------------------------------------------------------
// shared-memory carve-up (host and device compute the same sizes)
// ---------------------------------------------------------------------------
struct Smem {
    uint2* hs;      // [min(sobol_dims, HS_CHUNK)] tile parts of the current chunk of Sobol entries,
                    // for tile columns t and t + T/2 (see tile_high_bits)
    float* stk;     // [stack_depth][stack_factors][T]; after the time loop, the product partials
    float* slots;   // [n_slots][T + 1]
    float* grp;     // [n_groups][T + 1]
    float* last;    // [n_last][T + 1] previous observation of each discretely observed variance group
    float* part;    // [T * 6] product partials: the bridge stack's space, free once the paths are built
    double* red;    // [2 * warps]
    float* fa;      // few-product mode: [few_m][T] per-thread FP32 moment sums since the last flush
    float* fw;      // few-product mode: [T / 32][few_m][2] per-warp Kahan (sum, compensation)
    float* fshift;  // few-product mode: [few_m / 2] the CTA's shift of each quantity
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ constexpr int log2i(int x) { return x <= 1 ? 0 : 1 + log2i(x / 2); }

// Sobol entries whose tile parts are held in shared memory at a time
constexpr int HS_CHUNK = 512;
__host__ __device__ inline int hs_words(int sobol_dims) { return sobol_dims < HS_CHUNK ? sobol_dims : HS_CHUNK; }

// the bridge stack, or the product partials that reuse its space after the time loop
__host__ __device__ inline size_t stack_part_bytes(int T, int stack_depth, int nfa)
{
    const size_t stk = sizeof(float) * (size_t)stack_depth * nfa * T, part = sizeof(float) * (size_t)T * 6;
    return align16(stk > part ? stk : part);
}

// the few-product mode's accumulators (few_m moments; sized for T threads, the widest shape)
__host__ __device__ inline size_t few_bytes(int T, int few_m)
{
    if (few_m <= 0) return 0;
    return align16(sizeof(float) * (size_t)few_m * T) + align16(sizeof(float) * 2 * (size_t)few_m * (T / 32)) +
           align16(sizeof(float) * (size_t)(few_m / 2));
}

__host__ __device__ inline size_t smem_bytes(int T, int sobol_dims, int stack_depth, int nfa, int n_slots,
                                             int n_groups, int n_last, int few_m)
{
    size_t b = 0;
    b += align16(sizeof(uint2) * (size_t)hs_words(sobol_dims));
    b += stack_part_bytes(T, stack_depth, nfa);
    b += align16(sizeof(float) * (size_t)n_slots * (T + 1));
    b += align16(sizeof(float) * (size_t)n_groups * (T + 1));
    b += align16(sizeof(float) * (size_t)n_last * (T + 1));
    b += align16(sizeof(double) * 2 * (T / 32));
    b += few_bytes(T, few_m);
    return b;
}

__device__ inline Smem carve(unsigned char* base, const DevPlan& P, int T)
{
    Smem s;
    size_t o = 0;
    s.hs = reinterpret_cast<uint2*>(base + o);
    o += align16(sizeof(uint2) * (size_t)hs_words(P.sobol_dims));
    s.stk = reinterpret_cast<float*>(base + o);
    s.part = s.stk;
    o += stack_part_bytes(T, P.stack_depth, P.stack_factors);
    s.slots = reinterpret_cast<float*>(base + o);
    o += align16(sizeof(float) * (size_t)P.n_slots_used * (T + 1));
    s.grp = reinterpret_cast<float*>(base + o);
    o += align16(sizeof(float) * (size_t)P.n_groups * (T + 1));
    s.last = reinterpret_cast<float*>(base + o);
    o += align16(sizeof(float) * (size_t)P.n_last * (T + 1));
    s.red = reinterpret_cast<double*>(base + o);
    o += align16(sizeof(double) * 2 * (T / 32));
    s.fa = s.fw = s.fshift = nullptr;
    if (P.few_m > 0) {
        s.fa = reinterpret_cast<float*>(base + o);
        o += align16(sizeof(float) * (size_t)P.few_m * T);
        s.fw = reinterpret_cast<float*>(base + o);
        o += align16(sizeof(float) * 2 * (size_t)P.few_m * (T / 32));
        s.fshift = reinterpret_cast<float*>(base + o);
    }
    return s;
}

// ---------------------------------------------------------------------------
// Sobol for the current tile. Path n = m * T + t (T = 2^TB). gray(n) splits
// into bits >= TB, shared by the whole tile, and the thread's low TB bits
// gray(t) ^ ((m & 1) << (TB - 1)). The XOR of V[d][j] over the bits of gray(t)
// depends on the thread only: a fixed word lo[d][t]. Every Sobol dimension is
// used once per path, in an order fixed by the bridge program, so the book's
// low words are laid out in that order (sobol_lo[j][t], j the j-th dimension
// consumed) and the tile part likewise (hs[j], computed per tile in chunks of
// HS_CHUNK entries). The step loop then reads both sequentially:
// x = hs[j] ^ lo[j][t], with the coalesced load of entry j + 2 in flight while
// entry j is used. Every thread of the CTA consumes the same entries in the
// same order, so all of them reach a chunk boundary at the same call, where
// the next chunk is computed between two barriers.
//
// Columns t and t + T/2 (t < T/2) differ in their low bits by gray(T/2) =
// 3 << (TB - 2), so lo[d][t + T/2] = lo[d][t] ^ V[d][TB-1] ^ V[d][TB-2], a word
// shared by the tile. The tile part is therefore kept as a pair, hs[j] and
// hs[j] ^ V[d][TB-1] ^ V[d][TB-2]: a thread with two paths (columns t and
// t + T/2) reads one low word per entry, and one 8-byte broadcast of the pair.
// ---------------------------------------------------------------------------
template <int TB>
__device__ inline void tile_high_bits(const DevPlan& P, uint2* hs, int64_t m, int j0)
{
    const uint64_t g = (uint64_t)m ^ ((uint64_t)m >> 1);
    const int j1 = min(j0 + HS_CHUNK, P.n_sobol);
    for (int j = j0 + (int)threadIdx.x; j < j1; j += blockDim.x) {
        const uint32_t* V = P.sobol_v + __ldg(P.sobol_order + j) * SOBOL_BITS;
        uint32_t acc = (m & 1) ? __ldg(V + TB - 1) : 0u;
        uint64_t gg = g;
        for (int k = 0; gg != 0 && k < SOBOL_BITS - TB; ++k, gg >>= 1)
            if (gg & 1u) acc ^= __ldg(V + TB + k);
        hs[j - j0] = make_uint2(acc, acc ^ __ldg(V + TB - 1) ^ __ldg(V + TB - 2));
    }
}

// low words a thread loads per Sobol entry: with an even number of paths, one for each pair
// of columns t + k T/PP and t + k T/PP + T/2 (k < PP/2), through the tile-part pair; else
// one per path
template <int PP>
struct LoadsPerEntry {
    static constexpr int value = PP % 2 == 0 ? PP / 2 : PP;
};

template <int T, int PP>
struct SobolLane {
    static constexpr int LW = LoadsPerEntry<PP>::value;
    uint2* hs;             // tile parts of entries [jend - HS_CHUNK, jend), smem
    const uint32_t* lo;    // column threadIdx.x of the book's low words
    int64_t m;             // tile index
    int j, jend;           // next entry; end of the chunk in shared memory
    uint32_t cur[LW], nxt[LW]; // low words of entries j and j + 1
};

// path p of a thread is tile column threadIdx.x + p * (T / PP); the first chunk
// of tile parts must already be in hs
template <int TB, int PP>
__device__ __forceinline__ SobolLane<1 << TB, PP> sobol_lane(const DevPlan& P, uint2* hs, int64_t m)
{
    constexpr int T = 1 << TB, TH = T / PP, LW = LoadsPerEntry<PP>::value;
    SobolLane<T, PP> L;
    L.hs = hs;
    L.lo = P.sobol_lo + threadIdx.x;
    L.m = m;
    L.j = 0;
    L.jend = HS_CHUNK;
#pragma unroll
    for (int p = 0; p < LW; ++p) {
        L.cur[p] = P.n_sobol > 0 ? __ldg(L.lo + p * TH) : 0u;
        L.nxt[p] = P.n_sobol > 1 ? __ldg(L.lo + T + p * TH) : 0u;
    }
    return L;
}

// the Gaussian of tail dimension dim (>= sobol_dims) of the path with Sobol index n, from the
// book's tail table (0 for a column outside the book's paths)
__device__ __forceinline__ float tail_gauss(const DevPlan& P, uint64_t n, int dim)
{
    const uint64_t k = n - (uint64_t)P.skip - 1; // the path's place in the book
    return k < (uint64_t)P.paths ? __ldg(P.tail + (size_t)(dim - P.sobol_dims) * (size_t)P.tail_ld + k) : 0.f;
}

// Gaussians of reference dimension `dim` for the thread's PP paths (Sobol
// indices n[p]); a Sobol dimension is the lane's next entry
template <int T, int PP>
__device__ __forceinline__ void gauss(const DevPlan& P, SobolLane<T, PP>& L, const uint64_t (&n)[PP], int dim,
                                      float (&z)[PP])
{
    constexpr int TH = T / PP, LW = LoadsPerEntry<PP>::value;
    uint32_t x[PP];
    if (dim < P.sobol_dims) {
        if (L.j == L.jend) { // next chunk of tile parts (uniform across the CTA, see above)
            __syncthreads();
            tile_high_bits<log2i(T)>(P, L.hs, L.m, L.j);
            __syncthreads();
            L.jend += HS_CHUNK;
        }
        const uint2 h = L.hs[L.j - (L.jend - HS_CHUNK)];
        const int jn = L.j + 2;
        const bool more = jn < P.n_sobol;
        if constexpr (PP % 2 == 0) {
            // path k is column t + k TH; path k + PP/2 is column t + k TH + T/2
#pragma unroll
            for (int k = 0; k < PP / 2; ++k) {
                x[k] = h.x ^ L.cur[k];
                x[k + PP / 2] = h.y ^ L.cur[k];
            }
        } else {
#pragma unroll
            for (int p = 0; p < PP; ++p) x[p] = h.x ^ L.cur[p];
        }
#pragma unroll
        for (int p = 0; p < LW; ++p) {
            L.cur[p] = L.nxt[p];
            L.nxt[p] = more ? __ldg(L.lo + jn * T + p * TH) : 0u;
        }
        ++L.j;
    } else if (P.tail) {
        // beyond the Sobol budget: the reference Rng's Gaussians of this path (tail_normals)
#pragma unroll
        for (int p = 0; p < PP; ++p) z[p] = tail_gauss(P, n[p], dim);
        return;
    } else {
#pragma unroll
        for (int p = 0; p < PP; ++p) x[p] = hash_u32(P.seed, n[p], (uint32_t)dim);
    }
    quantile_n<PP>(x, z);
}

// lw W_prev + (rw W_top + sd z) for a thread's two paths, paired (same roundings as the
// scalar fmaf form)
__device__ __forceinline__ float2 bridge_comb2(float lw, float rw, float sd, float wp0, float wp1, float tp0, float tp1,
                                               float z0, float z1)
{
    return __ffma2_rn(f2s(lw), f2(wp0, wp1), __ffma2_rn(f2s(rw), f2(tp0, tp1), __fmul2_rn(f2s(sd), f2(z0, z1))));
}

// ---------------------------------------------------------------------------
// One time step of the bridge for every active factor slot of the thread's PP
// paths: fills nz[][] with the normalised increments
// n_i = (W_i - W_{i-1}) / sqrt(t_i - t_{i-1}). Stack entry of path column k:
// stk[(level * nfa + factor) * T + k].
// ---------------------------------------------------------------------------
// SEQ: one asset, a0, per pass; its spot and variance factors are stack rows 0 and 1
template <int NA, int T, int PP, bool SEQ>
__device__ __forceinline__ void bridge_step(const DevPlan& P, const Smem& S, const StepRec& rec, int& sp,
                                            SobolLane<T, PP>& L, const uint64_t (&n)[PP],
                                            float (&Wprev)[PP][2 * NA], float (&top)[PP][2 * NA],
                                            float (&nz)[PP][2 * NA], int a0)
{
    constexpr int FS = 2 * NA, TH = T / PP;
    const int t = threadIdx.x;
    const int nfa = P.stack_factors;
    // asset and stack row of factor slot f (stack row < 0: slot inactive)
    auto slot = [&](int f, int& a, int& ci) {
        const int s_ = f < NA ? f : f - NA;
        a = SEQ ? a0 : s_;
        const int c = f < NA ? P.cidx_spot[a] : P.cidx_var[a];
        ci = (a < P.n_assets && c >= 0) ? (SEQ ? (f < NA ? 0 : 1) : c) : -1;
    };
    float Wi[PP][FS];
#pragma unroll
    for (int p = 0; p < PP; ++p)
#pragma unroll
        for (int f = 0; f < FS; ++f) Wi[p][f] = 0.f;
    if (rec.count == 0) {
        const int base = (sp - 1) * nfa * T + t;
#pragma unroll
        for (int f = 0; f < FS; ++f) {
            int a, ci;
            slot(f, a, ci);
            if (ci >= 0) {
#pragma unroll
                for (int p = 0; p < PP; ++p) {
                    Wi[p][f] = top[p][f];
                    top[p][f] = S.stk[base + ci * T + p * TH];
                }
            }
        }
        --sp;
    } else if (rec.count == 1) {
        // a single node ending at this date (about a quarter of the steps): no push
#pragma unroll
        for (int f = 0; f < FS; ++f) {
            int a, ci;
            slot(f, a, ci);
            if (ci >= 0) {
                const int fid = f < NA ? P.fid_spot[a] : P.fid_var[a];
                float z[PP];
                gauss(P, L, n, rec.dim + fid, z);
                if constexpr (PP % 2 == 0) {
#pragma unroll
                    for (int h = 0; h < PP; h += 2) {
                        const float2 w = bridge_comb2(rec.lw, rec.rw, rec.sd, Wprev[h][f], Wprev[h + 1][f], top[h][f],
                                                      top[h + 1][f], z[h], z[h + 1]);
                        Wi[h][f] = w.x;
                        Wi[h + 1][f] = w.y;
                    }
                } else {
#pragma unroll
                    for (int p = 0; p < PP; ++p)
                        Wi[p][f] = fmaf(rec.lw, Wprev[p][f], fmaf(rec.rw, top[p][f], rec.sd * z[p]));
                }
            }
        }
    } else {
        float lw = rec.lw, rw = rec.rw, sd = rec.sd;
        int dim = rec.dim;
        BridgeNode nd = P.nodes[rec.first]; // node 1 of the chain, loaded one node ahead
        for (int k = 0; k < rec.count; ++k) {
            if (k > 0) {
                lw = nd.lw;
                rw = nd.rw;
                sd = nd.sd;
                dim = nd.bstep * P.ref_factors;
                if (k + 1 < rec.count) nd = P.nodes[rec.first + k];
            }
            const bool push = k + 1 < rec.count;
            const int base = sp * nfa * T + t;
#pragma unroll
            for (int f = 0; f < FS; ++f) {
                int a, ci;
                slot(f, a, ci);
                if (ci >= 0) {
                    const int fid = f < NA ? P.fid_spot[a] : P.fid_var[a];
                    float z[PP];
                    gauss(P, L, n, dim + fid, z);
                    float Wns[PP];
                    if constexpr (PP % 2 == 0) {
#pragma unroll
                        for (int h = 0; h < PP; h += 2) {
                            const float2 w = bridge_comb2(lw, rw, sd, Wprev[h][f], Wprev[h + 1][f], top[h][f],
                                                          top[h + 1][f], z[h], z[h + 1]);
                            Wns[h] = w.x;
                            Wns[h + 1] = w.y;
                        }
                    } else {
#pragma unroll
                        for (int p = 0; p < PP; ++p) Wns[p] = fmaf(lw, Wprev[p][f], fmaf(rw, top[p][f], sd * z[p]));
                    }
#pragma unroll
                    for (int p = 0; p < PP; ++p) {
                        const float Wn = Wns[p];
                        if (push) {
                            S.stk[base + ci * T + p * TH] = top[p][f];
                            top[p][f] = Wn;
                        } else {
                            Wi[p][f] = Wn;
                        }
                    }
                }
            }
            if (push) ++sp;
        }
    }
    if constexpr (PP % 2 == 0) {
#pragma unroll
        for (int h = 0; h < PP; h += 2)
#pragma unroll
            for (int f = 0; f < FS; ++f) {
                const float2 d =
                    __fmul2_rn(sub2(f2(Wi[h][f], Wi[h + 1][f]), f2(Wprev[h][f], Wprev[h + 1][f])), f2s(rec.isd));
                nz[h][f] = d.x;
                nz[h + 1][f] = d.y;
                Wprev[h][f] = Wi[h][f];
                Wprev[h + 1][f] = Wi[h + 1][f];
            }
    } else {
#pragma unroll
        for (int p = 0; p < PP; ++p)
#pragma unroll
            for (int f = 0; f < FS; ++f) {
                nz[p][f] = (Wi[p][f] - Wprev[p][f]) * rec.isd;
                Wprev[p][f] = Wi[p][f];
            }
    }
}

// leverage L(X_{i-1}) and dL/dX (local_volatility_node.cpp:19-47) on the layer the
// step's record names (c3 = {1/ln_step, grid offset, first value as int bits}): the
// layer's rows are uniform across the CTA and stay in L1 (staging the current layer in
// shared memory measured slower)
__device__ __forceinline__ void leverage(const DevPlan& P, int a, float4 c3, float x, float& L, float& dL)
{
    const float2 mp = make_float2(c3.x, c3.y);
    const float* v = P.lev_values + __float_as_int(c3.z);
    const int npts = P.lev_points[a];
    const float f = fmaf(x, mp.x, mp.y);
    const int last = npts - 1;
    if (f <= 0.f) {
        L = __ldg(v);
        dL = 0.f;
    } else if (f >= (float)last) {
        L = __ldg(v + last);
        dL = 0.f;
    } else {
        const int k = (int)f;
        const float w = f - (float)k;
        const float v0 = __ldg(v + k), v1 = __ldg(v + k + 1);
        L = fmaf(w, v1 - v0, v0);
        dL = (v1 - v0) * mp.x;
    }
}

__device__ __forceinline__ float intrinsic(const DevProduct& pr, float s)
{
    const float iv = pr.call ? s - pr.K : pr.K - s;
    return fmaxf(iv, 0.f);
}

// discounted flow of product pr on tile path k (contract_node.cpp:16-51)
__device__ __forceinline__ float payoff(const DevPlan& P, const DevProduct& pr, const float* slots, const float* grp,
                                       int stride, int k)
{
    float s;
    switch (pr.kind) {
    case P_VARIANCE: {
        const float sum2 = (pr.g_snap ? slots : grp)[pr.slot_g * stride + k];
        return pr.notional * ((pr.past + sum2) * pr.inv_T - pr.kvar) * pr.df;
    }
    case P_BARRIER: {
        const float ext = (pr.g_snap ? slots : grp)[pr.slot_g * stride + k];
        const bool hit = pr.up ? (ext >= pr.level) : (ext <= pr.level);
        const bool alive = pr.knock_in ? hit : !hit;
        if (!alive) return 0.f;
        s = slots[pr.slot_s * stride + k] * pr.qfac;
        break;
    }
    case P_BASKET: {
        s = 0.f;
        for (int c = 0; c < pr.comp_n; ++c) {
            const Comp cp = P.comps[pr.comp_first + c];
            s = fmaf(slots[cp.slot * stride + k], cp.w, s);
        }
        break;
    }
    default:
        s = slots[pr.slot_s * stride + k] * pr.qfac;
    }
    return intrinsic(pr, s) * pr.df;
}

// pathwise delta and vega of product pr on tile path k
__device__ __forceinline__ void greeks_of(const DevPlan& P, const DevProduct& pr, const float* slots, int stride,
                                          int k, float& d, float& g)
{
    d = 0.f;
    g = 0.f;
    const float sgn = pr.call ? 1.f : -1.f;
    if (pr.kind == P_VANILLA) {
        const float sT = slots[pr.slot_s * stride + k];
        const float s = sT * pr.qfac;
        if (intrinsic(pr, s) > 0.f) {
            const float y = pr.slot_y >= 0 ? slots[pr.slot_y * stride + k] : 1.f;
            d = sgn * s * pr.inv_s0 * y * pr.df;
            if (pr.slot_w >= 0) g = sgn * s * (slots[pr.slot_w * stride + k] - pr.vol_t) * pr.df;
        }
    } else if (pr.kind == P_BASKET) {
        float s = 0.f, ds = 0.f;
        for (int c = 0; c < pr.comp_n; ++c) {
            const Comp cp = P.comps[pr.comp_first + c];
            const float sc = slots[cp.slot * stride + k] * cp.w;
            s += sc;
            const float y = cp.slot_y >= 0 ? slots[cp.slot_y * stride + k] : 1.f;
            ds = fmaf(sc * cp.inv_s0, y, ds);
        }
        if (intrinsic(pr, s) > 0.f) d = sgn * ds * pr.df;
    }
}

// ---------------------------------------------------------------------------
// Few-product mode (books of at most FEW_PRODUCTS products; few_m > 0). Every
// thread adds its own paths' values into per-thread FP32 sums in shared memory,
// so a tile ends with no cross-thread work and no FP64 (an FP64 warp
// instruction holds GB300's narrow FP64 pipe for tens of cycles whatever the
// active lanes, which made the per-tile reduction the whole cost of short
// books). Every FEW_FLUSH tiles, and at the end, the per-thread sums are
// folded by FP32 warp shuffles into per-warp Kahan-compensated FP32 totals;
// the CTA's row of FP64 sums is formed once, after its last tile.
// Quantities, in order: the book value, then per product its flow (and, with
// pathwise Greeks, its delta and vega); moments 2q and 2q + 1 hold the sum of
// x - c_q and of (x - c_q)^2, with c_q the quantity's value on the first valid
// path of the CTA's first tile (the same shift for every thread of the CTA).
// ---------------------------------------------------------------------------
constexpr int FEW_PRODUCTS = 4;
constexpr int FEW_Q_MAX = 1 + 3 * FEW_PRODUCTS;
constexpr int FEW_FLUSH = 16; // tiles between folds: a per-thread FP32 sum holds at most 16 x PP paths

// quantity q of the few-product layout on tile column k
__device__ __forceinline__ float few_value(const DevPlan& P, const float* slots, const float* grp, int stride, int k,
                                           int q)
{
    const bool gk = P.greeks != 0;
    if (q == 0) {
        float b = 0.f;
        for (int j = 0; j < P.n_products; ++j) {
            if (P.vanilla_only) {
                const VanTerm vt = P.vterms[j];
                b = fmaf(vt.w, fmaxf(fmaf(vt.a, slots[vt.slot * stride + k], vt.b), 0.f), b);
            } else {
                const DevProduct pr = P.products[j];
                b = fmaf(payoff(P, pr, slots, grp, stride, k), pr.fx, b);
            }
        }
        return b;
    }
    const int j = gk ? (q - 1) / 3 : q - 1, kind = gk ? (q - 1) % 3 : 0;
    if (P.vanilla_only) {
        const VanTerm vt = P.vterms[j];
        return fmaxf(fmaf(vt.a, slots[vt.slot * stride + k], vt.b), 0.f);
    }
    const DevProduct pr = P.products[j];
    if (kind == 0) return payoff(P, pr, slots, grp, stride, k);
    float d, g;
    greeks_of(P, pr, slots, stride, k, d, g);
    return kind == 1 ? d : g;
}

__device__ __forceinline__ void few_add(float (&am)[2 * FEW_Q_MAX], const float (&cs)[FEW_Q_MAX], int q, float x)
{
    const float y = x - cs[q];
    am[2 * q] += y;
    am[2 * q + 1] = fmaf(y, y, am[2 * q + 1]);
}

// fold the per-thread sums of the calling thread's warp into the warp's Kahan totals
__device__ __forceinline__ void few_fold(const Smem& S, int M, int T)
{
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int m = 0; m < M; ++m) {
        float v = S.fa[m * T + t];
        S.fa[m * T + t] = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
            float* k = S.fw + 2 * (w * M + m);
            const float y = v - k[1];
            const float tt = k[0] + y;
            k[1] = (tt - k[0]) - y;
            k[0] = tt;
        }
    }
}

__device__ __forceinline__ StepRec load_rec(const DevPlan& P, int i)
{
    const float4* r = reinterpret_cast<const float4*>(P.recs + (i - 1));
    const float4 a = __ldg(r), b = __ldg(r + 1);
    StepRec s;
    s.lw = a.x;
    s.rw = a.y;
    s.sd = a.z;
    s.dim = __float_as_int(a.w);
    s.isd = b.x;
    s.count = __float_as_int(b.y);
    s.first = __float_as_int(b.z);
    s.ev = __float_as_int(b.w);
    return s;
}

// ---------------------------------------------------------------------------
// One asset's pass over a tile for two paths a thread (tile columns t and t + T/2), held as
// packed pairs: the paths' state is float2 throughout, the bridge stack holds one float2 per
// thread and row (one 8-byte shared access per stack entry for both paths), and every FP32
// operation on the paths issues as one FFMA2 / FMUL2 / FADD2. The operations and their order
// are those of the generic loop in book_kernel, lane by lane.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 comb2(float lw, float rw, float sd, float2 wp, float2 tp, float2 z)
{
    return __ffma2_rn(f2s(lw), wp, __ffma2_rn(f2s(rw), tp, __fmul2_rn(f2s(sd), z)));
}

// The Sobol lane of a thread with two paths: a running pointer into the tile parts in shared
// memory (refilled HS_CHUNK entries at a time, uniformly across the CTA as in gauss) and a
// running pointer into the book's low words, whose table carries two rows of padding so that
// the load two entries ahead needs no bounds test.
struct PairLane {
    const uint2* hs;      // tile part of the next entry
    const uint2* hs_end;  // end of the chunk in shared memory
    const uint32_t* lo;   // low word of the entry two ahead (this thread's column)
    uint32_t cur, nxt;    // low words of the next two entries
    int jc;               // first entry of the chunk in shared memory
    int64_t m;            // tile index
};

template <int T>
__device__ __forceinline__ PairLane pair_lane(const DevPlan& P, const uint2* hs, int64_t m)
{
    PairLane L;
    L.hs = hs;
    L.hs_end = hs + HS_CHUNK;
    L.lo = P.sobol_lo + 2 * T + threadIdx.x;
    L.cur = __ldg(P.sobol_lo + threadIdx.x);
    L.nxt = __ldg(P.sobol_lo + T + threadIdx.x);
    L.jc = 0;
    L.m = m;
    return L;
}

// ALL: every dimension of the book is a Sobol dimension (the bound test is dropped)
template <int TB, bool ALL>
__device__ __forceinline__ float2 pair_gauss(const DevPlan& P, uint2* hs_base, PairLane& L, const uint64_t (&n)[2],
                                             int dim)
{
    constexpr int T = 1 << TB;
    uint32_t x0, x1;
    if (ALL || dim < P.sobol_dims) {
        if (L.hs == L.hs_end) { // next chunk of tile parts (uniform across the CTA)
            L.jc += HS_CHUNK;
            __syncthreads();
            tile_high_bits<TB>(P, hs_base, L.m, L.jc);
            __syncthreads();
            L.hs = hs_base;
        }
        const uint2 h = *L.hs++;
        x0 = h.x ^ L.cur; // columns t and t + T/2 share the low word through the tile-part pair
        x1 = h.y ^ L.cur;
        L.cur = L.nxt;
        L.nxt = __ldg(L.lo);
        L.lo += T;
    } else if (P.tail) {
        return f2(tail_gauss(P, n[0], dim), tail_gauss(P, n[1], dim));
    } else {
        x0 = hash_u32(P.seed, n[0], (uint32_t)dim);
        x1 = hash_u32(P.seed, n[1], (uint32_t)dim);
    }
    float z0, z1;
    quantile_pair(x0, x1, z0, z1);
    return f2(z0, z1);
}

// The path events of date i for asset a on both tile columns of a thread (t and t + TH), each
// event read once and applied to column t, then to column t + TH: per column the operations and
// their order are those of apply_events in book_body.
template <int TH>
__device__ __forceinline__ void pair_events(const DevPlan& P, const Smem& S, int i, int a, float2 x, float2 step,
                                            float2 w, float2 y)
{
    const int stride = 2 * TH + 1;
    const int t = threadIdx.x;
    const int2 r = P.ev_range[i * P.n_assets + a];
    for (int e = r.x; e < r.x + r.y; ++e) {
        const Event ev = P.events[e];
        const int k = ev.a * stride + t; // the event's row (slot or group), column t
        switch (ev.type) {
        case EV_SNAP_S:
            S.slots[k] = P.s0[a] * expf(x.x);
            S.slots[k + TH] = P.s0[a] * expf(x.y);
            break;
        case EV_SNAP_W:
            S.slots[k] = w.x;
            S.slots[k + TH] = w.y;
            break;
        case EV_SNAP_Y:
            S.slots[k] = y.x;
            S.slots[k + TH] = y.y;
            break;
        case EV_GRP_MIN:
            S.grp[k] = fminf(S.grp[k], x.x - ev.p);
            S.grp[k + TH] = fminf(S.grp[k + TH], x.y - ev.p);
            break;
        case EV_GRP_MAX:
            S.grp[k] = fmaxf(S.grp[k], x.x - ev.p);
            S.grp[k + TH] = fmaxf(S.grp[k + TH], x.y - ev.p);
            break;
        case EV_GRP_SQ_STEP: {
            const float d0 = step.x - ev.p, d1 = step.y - ev.p;
            S.grp[k] = fmaf(d0, d0, S.grp[k]);
            S.grp[k + TH] = fmaf(d1, d1, S.grp[k + TH]);
            break;
        }
        case EV_SNAP_G: {
            const int kg = ev.pad * stride + t;
            S.slots[k] = S.grp[kg];
            S.slots[k + TH] = S.grp[kg + TH];
            break;
        }
        default: { // EV_GRP_SQ_OBS
            const int kl = ev.pad * stride + t; // pad: the group's row of last
            const float d0 = x.x - S.last[kl] - ev.p;
            S.grp[k] = fmaf(d0, d0, S.grp[k]);
            S.last[kl] = x.x;
            const float d1 = x.y - S.last[kl + TH] - ev.p;
            S.grp[k + TH] = fmaf(d1, d1, S.grp[k + TH]);
            S.last[kl + TH] = x.y;
        }
        }
    }
}

// FAST: the book is in Sobol mode with every dimension a Sobol dimension, and stores no paths.
// There each step's record is loaded at the step: loading it one step ahead holds eight more
// registers across the step and measured slower (2.93 against 2.75 ms for the 2^20-path Heston
// grid). The other pass loads it one step ahead, which measured faster where the paths are
// stored (GBM, 2^20 paths x 252 steps: 1.11 against 1.23 ms).
template <int TB, int MODEL, bool UNIFORM, bool FAST>
__device__ __forceinline__ void pair_pass(const DevPlan& P, const Smem& S, PairLane& L,
                                          const uint64_t (&n)[2], const bool (&valid)[2], int a0, float4 u0,
                                          float4 u1, float4 u2)
{
    constexpr int T = 1 << TB, TH = T / 2;
    constexpr bool SEQ = MODEL == M_SEQ;
    const int t = threadIdx.x;
    const int aid = SEQ ? a0 : 0;
    const int model = SEQ ? P.model[aid] : MODEL;
    // the spot factor, and the variance factor where the model has one: compact stack row and
    // reference factor index (the dimension of a node is its bridge step * F + that index)
    // A single-asset book's spot factor is reference factor 0 and stack row 0; a Heston or LSV
    // asset adds its variance factor as factor 1 and row 1. A pass of a multi-asset book uses
    // rows 0 and 1 of a two-row stack and the asset's own factors.
    const bool act1 = MODEL == M_GBM ? false : (SEQ ? model != M_GBM : true);
    constexpr int ci0 = 0, ci1 = 1;
    const int fid0 = SEQ ? P.fid_spot[aid] : 0, fid1 = SEQ ? P.fid_var[aid] : 1;
    constexpr int nfa = MODEL == M_GBM ? 1 : 2;
    float2* const stk = reinterpret_cast<float2*>(S.stk) + t; // this thread's column of the stack
    const bool degenerate = P.degenerate[aid] != 0;

    float2 X = f2s(0.f), CP = f2s(0.f), V = f2s(P.v0[aid]), WB = f2s(0.f), Y = f2s(1.f);
    float2 Wp0 = f2s(0.f), Wp1 = f2s(0.f), T0 = f2s(0.f), T1 = f2s(0.f);
    int sp = 0;
    pair_events<TH>(P, S, 0, aid, f2s(0.f), f2s(0.f), f2s(0.f), f2s(1.f));
    const bool store = !FAST && P.path_out && aid == P.path_asset;
    if (store)
#pragma unroll
        for (int p = 0; p < 2; ++p)
            if (valid[p]) P.path_out[n[p] - (uint64_t)P.skip - 1] = P.s0[aid];

    StepRec rec;
    if constexpr (!FAST) rec = load_rec(P, 1);
    for (int i = 1; i <= P.n_steps; ++i) {
        StepRec cur;
        if constexpr (FAST) {
            cur = load_rec(P, i);
        } else {
            cur = rec;
            rec = load_rec(P, i + 1); // the record past the last step is padding
        }
        // this step's constants, requested before the bridge work that covers their latency
        float4 c0 = u0, c1 = u1, c2 = u2, c3 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!UNIFORM) {
            const float4* cs = reinterpret_cast<const float4*>(P.steps[(i - 1) * P.n_assets + aid].c);
            c0 = __ldg(cs);
            c1 = __ldg(cs + 1);
            c2 = __ldg(cs + 2);
            if (MODEL == M_LSV || (SEQ && model == M_LSV)) c3 = __ldg(cs + 3);
        }
        // LSV: the leverage at the step's start, requested before the bridge work (see book_kernel)
        float lvL[2] = {1.f, 1.f}, lvD[2] = {0.f, 0.f};
        if (MODEL == M_LSV || (SEQ && model == M_LSV)) {
            leverage(P, aid, c3, X.x, lvL[0], lvD[0]);
            leverage(P, aid, c3, X.y, lvL[1], lvD[1]);
        }
        // ---- Brownian bridge: normalised increments nz0 (spot), nz1 (variance) ----
        float2 nz0, nz1 = f2s(0.f);
        if (FAST || P.use_sobol) {
            float2 Wi0 = f2s(0.f), Wi1 = f2s(0.f);
            if (cur.count == 0) {
                const int base = (sp - 1) * nfa;
                Wi0 = T0;
                T0 = stk[(base + ci0) * TH];
                if (act1) {
                    Wi1 = T1;
                    T1 = stk[(base + ci1) * TH];
                }
                --sp;
            } else if (cur.count == 1) {
                Wi0 = comb2(cur.lw, cur.rw, cur.sd, Wp0, T0, pair_gauss<TB, FAST>(P, S.hs, L, n, cur.dim + fid0));
                if (act1) Wi1 = comb2(cur.lw, cur.rw, cur.sd, Wp1, T1, pair_gauss<TB, FAST>(P, S.hs, L, n, cur.dim + fid1));
            } else {
                float lw = cur.lw, rw = cur.rw, sd = cur.sd;
                int dim = cur.dim;
                BridgeNode nd = P.nodes[cur.first]; // node 1 of the chain, loaded one node ahead
                for (int k = 0; k < cur.count; ++k) {
                    if (k > 0) {
                        lw = nd.lw;
                        rw = nd.rw;
                        sd = nd.sd;
                        dim = nd.bstep * P.ref_factors;
                        if (k + 1 < cur.count) nd = P.nodes[cur.first + k];
                    }
                    const float2 w0 = comb2(lw, rw, sd, Wp0, T0, pair_gauss<TB, FAST>(P, S.hs, L, n, dim + fid0));
                    float2 w1 = f2s(0.f);
                    if (act1) w1 = comb2(lw, rw, sd, Wp1, T1, pair_gauss<TB, FAST>(P, S.hs, L, n, dim + fid1));
                    if (k + 1 < cur.count) {
                        const int base = sp * nfa;
                        stk[(base + ci0) * TH] = T0;
                        T0 = w0;
                        if (act1) {
                            stk[(base + ci1) * TH] = T1;
                            T1 = w1;
                        }
                        ++sp;
                    } else {
                        Wi0 = w0;
                        Wi1 = w1;
                    }
                }
            }
            nz0 = __fmul2_rn(sub2(Wi0, Wp0), f2s(cur.isd));
            Wp0 = Wi0;
            if (act1) {
                nz1 = __fmul2_rn(sub2(Wi1, Wp1), f2s(cur.isd));
                Wp1 = Wi1;
            }
        } else {
            const uint32_t d0 = (uint32_t)((i - 1) * P.ref_factors + fid0);
            nz0 = f2(quantile_u32(hash_u32(P.seed, n[0], d0)), quantile_u32(hash_u32(P.seed, n[1], d0)));
            if (act1) {
                const uint32_t d1 = (uint32_t)((i - 1) * P.ref_factors + fid1);
                nz1 = f2(quantile_u32(hash_u32(P.seed, n[0], d1)), quantile_u32(hash_u32(P.seed, n[1], d1)));
            }
        }
        // ---- the model's step of the log-spot (relative to S0) ----------------------
        float2 step;
        if (MODEL == M_GBM || (SEQ && model == M_GBM)) {
            step = __ffma2_rn(f2s(c0.y), nz0, f2s(c0.x));
            WB = __ffma2_rn(f2s(c0.z), nz0, WB);
        } else {
            const float2 vc = qe_step2(V, nz1, c0.x, c0.y, c0.z, c0.w);
            if ((MODEL == M_HESTON || (SEQ && model == M_HESTON)) && !degenerate) {
                const float2 s2 = __fadd2_rn(V, vc);
                const float2 F = __ffma2_rn(f2s(c2.y), sub2(vc, V), __ffma2_rn(f2s(c1.z), s2, f2s(c1.y)));
                const float2 qr = sqrt2_approx(__fmul2_rn(f2s(c2.x), s2));
                const float2 B = __ffma2_rn(qr, nz0, F);
                step = __ffma2_rn(f2s(-c1.w), s2, __fadd2_rn(f2s(c1.x), B));
            } else {
                float sl[2];
                const float vpl[2] = {V.x, V.y}, vcl[2] = {vc.x, vc.y}, zl[2] = {nz0.x, nz0.y};
                float yl[2] = {Y.x, Y.y};
#pragma unroll
                for (int p = 0; p < 2; ++p) {
                    const float vp = vpl[p], vcp = vcl[p];
                    const float Lv = lvL[p], dL = lvD[p];
                    const float s = vp + vcp;
                    if (!degenerate) {
                        const float B = fmaf(c2.y, vcp - vp, fmaf(c1.z, s, c1.y)) + fast_sqrt(c2.x * s) * zl[p];
                        if (model == M_LSV) {
                            sl[p] = fmaf(Lv, B, c1.x) - Lv * Lv * c1.w * s;
                            yl[p] *= fmaf(B - 2.f * Lv * c1.w * s, dL, 1.f);
                        } else {
                            sl[p] = c1.x + B - c1.w * s;
                        }
                    } else {
                        const float sq = fast_sqrt(vp * c2.z) * zl[p];
                        sl[p] = c1.x - 0.5f * Lv * Lv * vp * c2.z + Lv * sq;
                        if (model == M_LSV) yl[p] *= fmaf(-Lv * vp * c2.z + sq, dL, 1.f);
                    }
                }
                step = f2(sl[0], sl[1]);
                Y = f2(yl[0], yl[1]);
            }
            V = vc;
        }
        // ---- Kahan-compensated log-spot ------------------------------------------
        {
            const float2 yy = sub2(step, CP);
            const float2 tt = __fadd2_rn(X, yy);
            CP = sub2(sub2(tt, X), yy);
            X = tt;
        }
        if (cur.ev) pair_events<TH>(P, S, i, aid, X, step, WB, Y);
        if (store) {
            if (valid[0]) P.path_out[(size_t)i * P.path_ld + (n[0] - (uint64_t)P.skip - 1)] = P.s0[aid] * expf(X.x);
            if (valid[1]) P.path_out[(size_t)i * P.path_ld + (n[1] - (uint64_t)P.skip - 1)] = P.s0[aid] * expf(X.y);
        }
    }
}

// ---------------------------------------------------------------------------
// The book kernel. Template parameters:
//   TB      log2 paths per tile (= threads per CTA)
//   NA      compile-time asset slots (1 = single-asset fast path)
//   MODEL   M_GBM / M_HESTON / M_LSV for single-model books, M_MIXED for books
//           with correlated GBM names, M_SEQ for other multi-asset books
//   UNIFORM every step has the same per-asset constants (kept in registers)
// ---------------------------------------------------------------------------
// resident CTAs per SM the registers are bounded for: 768 threads per SM worth for one or two
// paths a thread, 7 CTAs of 64 threads (146 registers each) for four, 3 for the mixed kernel
template <int TB, int NA, int PP>
struct MinBlocks {
    static constexpr int value = NA != 1 ? 3 : (PP == 4 ? 7 : 768 / ((1 << TB) / PP));
};

// The work of one CTA of a book: tiles tile0, tile0 + tile_step, ... below P.n_tiles, every
// product evaluated on each tile's paths, the FP64 sums in the row acc (zeroed here). A book's
// own launch runs it with tile0 = blockIdx.x and tile_step = gridDim.x; the batch kernel runs
// the same work items from a shared work list. Returns false when the cancel word stopped it.
template <int TB, int NA, int MODEL, bool UNIFORM, int PP>
__device__ __forceinline__ bool book_body(const DevPlan& P, unsigned char* smem_raw, int64_t tile0, int64_t tile_step,
                                          double* acc)
{
    constexpr int T = 1 << TB;  // paths per tile
    constexpr int TH = T / PP;  // threads per CTA; path p of thread t is tile column t + p * TH
    constexpr int FS = 2 * NA;
    const Smem S = carve(smem_raw, P, T);
    const int t = threadIdx.x;
    const int stride = T + 1;
    __shared__ int s_cancel;

    for (int j = t; j < P.n_acc; j += TH) acc[j] = 0.0;

    // uniform step constants (UNIFORM: step 1's for every step)
    float4 u0[NA], u1[NA], u2[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        if (UNIFORM && a < P.n_assets) {
            const float4* cs = reinterpret_cast<const float4*>(P.steps[a].c);
            u0[a] = __ldg(cs);
            u1[a] = __ldg(cs + 1);
            u2[a] = __ldg(cs + 2);
        } else {
            u0[a] = u1[a] = u2[a] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }

    // thread 0 reads the host-mapped cancel word one tile ahead, so its latency is not on the path
    int cancel_ahead = (t == 0 && P.cancel != nullptr) ? *P.cancel : 0;
    int ntile = 0;        // tiles done by this CTA
    int64_t nvalid = 0;   // valid paths of those tiles (few-product mode)
    for (int64_t tile = tile0; tile < P.n_tiles; tile += tile_step) {
        const int64_t m = P.tile_first + tile;
        uint64_t n[PP];
        bool valid[PP];
#pragma unroll
        for (int p = 0; p < PP; ++p) {
            n[p] = (uint64_t)m * T + (uint64_t)(t + p * TH);
            valid[p] = n[p] >= (uint64_t)P.skip + 1 && n[p] <= (uint64_t)(P.skip + P.paths);
        }
        __syncthreads(); // previous tile fully evaluated
        if (t == 0) {
            s_cancel = cancel_ahead;
            if (P.cancel != nullptr) cancel_ahead = *P.cancel;
        }
        if (P.use_sobol) tile_high_bits<TB>(P, S.hs, m, 0);
        __syncthreads();
        if (s_cancel) {
            if (t == 0) atomicExch(P.status, 1);
            return false;
        }
        SobolLane<T, PP> L = sobol_lane<TB, PP>(P, S.hs, m);

        for (int g = 0; g < P.n_groups; ++g)
#pragma unroll
            for (int p = 0; p < PP; ++p) S.grp[g * stride + t + p * TH] = P.grp_init[g];
        for (int g = 0; g < P.n_last; ++g)
#pragma unroll
            for (int p = 0; p < PP; ++p) S.last[g * stride + t + p * TH] = 0.f;

        // events on date index i for asset a of tile column k (after the state at date i is known)
        auto apply_events = [&](int i, int a, int k, float xa, float step, float wa, float ya) {
            const int2 r = P.ev_range[i * P.n_assets + a];
            for (int e = r.x; e < r.x + r.y; ++e) {
                const Event ev = P.events[e];
                switch (ev.type) {
                case EV_SNAP_S: S.slots[ev.a * stride + k] = P.s0[a] * expf(xa); break;
                case EV_SNAP_W: S.slots[ev.a * stride + k] = wa; break;
                case EV_SNAP_Y: S.slots[ev.a * stride + k] = ya; break;
                case EV_GRP_MIN: {
                    float* g = S.grp + ev.a * stride + k;
                    *g = fminf(*g, xa - ev.p);
                    break;
                }
                case EV_GRP_MAX: {
                    float* g = S.grp + ev.a * stride + k;
                    *g = fmaxf(*g, xa - ev.p);
                    break;
                }
                case EV_GRP_SQ_STEP: {
                    float* g = S.grp + ev.a * stride + k;
                    const float d = step - ev.p;
                    *g = fmaf(d, d, *g);
                    break;
                }
                case EV_SNAP_G: S.slots[ev.a * stride + k] = S.grp[ev.pad * stride + k]; break;
                default: { // EV_GRP_SQ_OBS
                    float* g = S.grp + ev.a * stride + k;
                    float* l = S.last + ev.pad * stride + k; // pad: the group's row of last
                    const float d = xa - *l - ev.p;
                    *g = fmaf(d, d, *g);
                    *l = xa;
                }
                }
            }
        };

        // one pass per asset for M_SEQ (asset a0), one pass for every asset otherwise
        constexpr bool SEQ = (MODEL == M_SEQ);
        const int n_pass = SEQ ? P.n_assets : 1;
        PairLane PL = pair_lane<T>(P, S.hs, m); // unused (and dropped) unless NA == 1 and PP == 2
        for (int a0 = 0; a0 < n_pass; ++a0) {
            if constexpr (NA == 1 && PP == 2) {
                // both passes in one kernel: the fast pass's own instantiation measured slower
                // (Heston grid 2.91 against 2.75 ms, same box)
                if (fast_pass(P))
                    pair_pass<TB, MODEL, UNIFORM, true>(P, S, PL, n, valid, a0, u0[0], u1[0], u2[0]);
                else
                    pair_pass<TB, MODEL, UNIFORM, false>(P, S, PL, n, valid, a0, u0[0], u1[0], u2[0]);
                continue;
            }
            // ---- path state -------------------------------------------------
            float x[PP][NA], comp[PP][NA], v[PP][NA], Wb[PP][NA], y[PP][NA];
            float Wprev[PP][FS], top[PP][FS], nz[PP][FS];
#pragma unroll
            for (int p = 0; p < PP; ++p) {
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                    x[p][a] = 0.f;
                    comp[p][a] = 0.f;
                    v[p][a] = P.v0[SEQ ? a0 : a];
                    Wb[p][a] = 0.f;
                    y[p][a] = 1.f;
                }
#pragma unroll
                for (int f = 0; f < FS; ++f) {
                    Wprev[p][f] = 0.f;
                    top[p][f] = 0.f;
                    nz[p][f] = 0.f;
                }
            }
            int sp = 0;
#pragma unroll
            for (int a = 0; a < NA; ++a) {
                const int aid = SEQ ? a0 : a;
                if (aid < P.n_assets)
#pragma unroll
                    for (int p = 0; p < PP; ++p) apply_events(0, aid, t + p * TH, 0.f, 0.f, 0.f, 1.f);
                if (P.path_out && aid == P.path_asset)
#pragma unroll
                    for (int p = 0; p < PP; ++p)
                        if (valid[p]) P.path_out[n[p] - (uint64_t)P.skip - 1] = P.s0[aid];
            }

            // ---- time loop ---------------------------------------------------
            for (int i = 1; i <= P.n_steps; ++i) {
                const StepRec cur = load_rec(P, i);
                // one asset a pass: its constants for this step are requested before the bridge
                // work, which covers their latency
                constexpr bool HOIST = !UNIFORM && (NA == 1 || MODEL == M_SEQ);
                float4 h0, h1, h2, h3;
                if constexpr (HOIST) {
                    const int ha = MODEL == M_SEQ ? a0 : 0;
                    const float4* cs = reinterpret_cast<const float4*>(P.steps[(i - 1) * P.n_assets + ha].c);
                    h0 = __ldg(cs);
                    h1 = __ldg(cs + 1);
                    h2 = __ldg(cs + 2);
                    h3 = (MODEL == M_LSV || (MODEL == M_SEQ && P.model[ha] == M_LSV)) ? __ldg(cs + 3)
                                                                                      : make_float4(0.f, 0.f, 0.f, 0.f);
                }
                // LSV: the leverage at the step's start (it depends on the log-spot of the previous
                // date only), requested before the bridge work, which covers its dependent loads
                float lvL[PP], lvD[PP];
#pragma unroll
                for (int p = 0; p < PP; ++p) {
                    lvL[p] = 1.f;
                    lvD[p] = 0.f;
                }
                if constexpr (HOIST) {
                    const int ha = MODEL == M_SEQ ? a0 : 0;
                    if (MODEL == M_LSV || (MODEL == M_SEQ && P.model[ha] == M_LSV))
#pragma unroll
                        for (int p = 0; p < PP; ++p) leverage(P, ha, h3, x[p][0], lvL[p], lvD[p]);
                }
                if (P.use_sobol) {
                    bridge_step<NA, T, PP, SEQ>(P, S, cur, sp, L, n, Wprev, top, nz, a0);
                } else {
#pragma unroll
                    for (int f = 0; f < FS; ++f) {
                        const int sa = f < NA ? f : f - NA;
                        const int aid = SEQ ? a0 : sa;
                        const int fid = f < NA ? P.fid_spot[aid] : P.fid_var[aid];
                        if (aid < P.n_assets && fid >= 0)
#pragma unroll
                            for (int p = 0; p < PP; ++p)
                                nz[p][f] = quantile_u32(
                                    hash_u32(P.seed, n[p], (uint32_t)((i - 1) * P.ref_factors + fid)));
                    }
                }
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                    const int aid = SEQ ? a0 : a; // asset id; a is the register slot
                    if (aid >= P.n_assets) continue;
                    float4 c0, c1, c2, c3 = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (UNIFORM) {
                        c0 = u0[a];
                        c1 = u1[a];
                        c2 = u2[a];
                    } else if constexpr (HOIST) {
                        c0 = h0;
                        c1 = h1;
                        c2 = h2;
                        c3 = h3;
                    } else {
                        const float4* cs = reinterpret_cast<const float4*>(P.steps[(i - 1) * P.n_assets + aid].c);
                        c0 = __ldg(cs);
                        c1 = __ldg(cs + 1);
                        c2 = __ldg(cs + 2);
                        if (P.model[aid] == M_LSV) c3 = __ldg(cs + 3);
                    }
                    const int model = (MODEL == M_MIXED || SEQ) ? P.model[aid] : MODEL;
                    // an even number of paths a thread: the variance step and the log-spot sum paired
                    constexpr bool PAIRED = PP % 2 == 0;
                    float vcs[PP], stp[PP];
                    if (PAIRED && model != M_GBM) {
#pragma unroll
                        for (int h = 0; h < PP; h += 2) {
                            const float2 r = qe_step2(f2(v[h][a], v[h + 1][a]), f2(nz[h][NA + a], nz[h + 1][NA + a]),
                                                      c0.x, c0.y, c0.z, c0.w);
                            vcs[h] = r.x;
                            vcs[h + 1] = r.y;
                        }
                    }
                    // Heston kernels, paired paths: the log-spot step paired as well
                    constexpr bool PAIR_SPOT = PAIRED && MODEL == M_HESTON;
                    if constexpr (PAIR_SPOT) {
                        if (!P.degenerate[aid]) {
#pragma unroll
                            for (int h = 0; h < PP; h += 2) {
                                const float2 vp2 = f2(v[h][a], v[h + 1][a]), vc2 = f2(vcs[h], vcs[h + 1]);
                                const float2 s2 = __fadd2_rn(vp2, vc2);
                                const float2 F =
                                    __ffma2_rn(f2s(c2.y), sub2(vc2, vp2), __ffma2_rn(f2s(c1.z), s2, f2s(c1.y)));
                                const float2 qr = sqrt2_approx(__fmul2_rn(f2s(c2.x), s2));
                                const float2 B = __ffma2_rn(qr, f2(nz[h][a], nz[h + 1][a]), F);
                                const float2 st = __ffma2_rn(f2s(-c1.w), s2, __fadd2_rn(f2s(c1.x), B));
                                stp[h] = st.x;
                                stp[h + 1] = st.y;
                                v[h][a] = vc2.x;
                                v[h + 1][a] = vc2.y;
                            }
                        }
                    }
#pragma unroll
                    for (int p = 0; p < PP; ++p) {
                        float step;
                        if (PAIR_SPOT && !P.degenerate[aid]) {
                            step = stp[p];
                        } else if (model == M_GBM) {
                            float e = nz[p][a];
                            if (MODEL == M_MIXED && P.corr) {
                                e = 0.f;
#pragma unroll
                                for (int u = 0; u < NA; ++u)
                                    if (u < P.n_assets) e = fmaf(P.chol[a * MAX_ASSETS + u], nz[p][u], e);
                            }
                            step = fmaf(c0.y, e, c0.x);
                            Wb[p][a] = fmaf(c0.z, e, Wb[p][a]);
                        } else {
                            const float vp = v[p][a];
                            const float vc = PAIRED ? vcs[p] : qe_step(vp, nz[p][NA + a], c0.x, c0.y, c0.z, c0.w);
                            // the spot's noise: its own, or correlated through chol (correlate_all_spots)
                            float zs = nz[p][a];
                            if (MODEL == M_MIXED && P.corr_all) {
                                zs = 0.f;
#pragma unroll
                                for (int u = 0; u < NA; ++u)
                                    if (u < P.n_assets) zs = fmaf(P.chol[a * MAX_ASSETS + u], nz[p][u], zs);
                            }
                            float Lv = 1.f, dL = 0.f;
                            if (model == M_LSV) {
                                if constexpr (HOIST) {
                                    Lv = lvL[p];
                                    dL = lvD[p];
                                } else {
                                    leverage(P, aid, c3, x[p][a], Lv, dL);
                                }
                            }
                            const float s = vp + vc;
                            if (!P.degenerate[aid]) {
                                const float B =
                                    fmaf(c2.y, vc - vp, fmaf(c1.z, s, c1.y)) + fast_sqrt(c2.x * s) * zs;
                                if (model == M_LSV) {
                                    step = fmaf(Lv, B, c1.x) - Lv * Lv * c1.w * s;
                                    y[p][a] *= fmaf(B - 2.f * Lv * c1.w * s, dL, 1.f);
                                } else {
                                    step = c1.x + B - c1.w * s;
                                }
                            } else {
                                const float sq = fast_sqrt(vp * c2.z) * zs;
                                step = c1.x - 0.5f * Lv * Lv * vp * c2.z + Lv * sq;
                                if (model == M_LSV) y[p][a] *= fmaf(-Lv * vp * c2.z + sq, dL, 1.f);
                            }
                            v[p][a] = vc;
                        }
                        stp[p] = step;
                    }
                    // Kahan-compensated log-spot
                    if constexpr (PAIRED) {
#pragma unroll
                        for (int h = 0; h < PP; h += 2) {
                            const float2 yy = sub2(f2(stp[h], stp[h + 1]), f2(comp[h][a], comp[h + 1][a]));
                            const float2 xx = f2(x[h][a], x[h + 1][a]);
                            const float2 tt = __fadd2_rn(xx, yy);
                            const float2 cp = sub2(sub2(tt, xx), yy);
                            comp[h][a] = cp.x;
                            comp[h + 1][a] = cp.y;
                            x[h][a] = tt.x;
                            x[h + 1][a] = tt.y;
                        }
                    } else {
#pragma unroll
                        for (int p = 0; p < PP; ++p) {
                            const float yy = stp[p] - comp[p][a];
                            const float tt = x[p][a] + yy;
                            comp[p][a] = (tt - x[p][a]) - yy;
                            x[p][a] = tt;
                        }
                    }
#pragma unroll
                    for (int p = 0; p < PP; ++p) {
                        const float step = stp[p];
                        if (cur.ev) apply_events(i, aid, t + p * TH, x[p][a], step, Wb[p][a], y[p][a]);
                        // stored paths: date-major, consecutive paths on consecutive threads
                        if (P.path_out && aid == P.path_asset && valid[p])
                            P.path_out[(size_t)i * P.path_ld + (n[p] - (uint64_t)P.skip - 1)] = P.s0[aid] * expf(x[p][a]);
                    }
                }
            }
        }
        __syncthreads(); // every path of the tile observed

        // ---- product evaluation: thread per product, FP32 tile partials ----
        // The tile's valid paths are the contiguous columns [k0, k0 + nv). Every sum of the tile
        // is shifted by the value at column k0 (payoff, pathwise delta, pathwise vega of the
        // product): the FP32 partials hold f - c and (f - c)^2, and the shift is added back in
        // FP64. So the sum of squares keeps its precision where the payoff's variance is small
        // next to its square (deep in-the-money cells), and the trust with it.
        const int k0 = (int)max((int64_t)0, P.skip + 1 - m * T);
        const int kend = (int)min((int64_t)T, P.skip + P.paths - m * T + 1);
        const int nv = kend - k0;
        const int C = P.n_products;

        // ---- few-product mode: per-thread FP32 sums (see few_value) --------
        if (P.few_m > 0) {
            const int M = P.few_m, NQ = M / 2;
            if (ntile == 0) {
                if (t < NQ) S.fshift[t] = few_value(P, S.slots, S.grp, stride, k0, t);
                for (int j = t; j < M * T; j += TH) S.fa[j] = 0.f;
                for (int j = t; j < 2 * M * (T / 32); j += TH) S.fw[j] = 0.f;
                __syncthreads();
            }
            float cs[FEW_Q_MAX], am[2 * FEW_Q_MAX];
#pragma unroll
            for (int q = 0; q < FEW_Q_MAX; ++q) cs[q] = q < NQ ? S.fshift[q] : 0.f;
#pragma unroll
            for (int q = 0; q < 2 * FEW_Q_MAX; ++q) am[q] = 0.f;
#pragma unroll
            for (int p = 0; p < PP; ++p) {
                if (!valid[p]) continue;
                const int k = t + p * TH;
                float bv = 0.f;
                if (P.vanilla_only) {
#pragma unroll
                    for (int j = 0; j < FEW_PRODUCTS; ++j)
                        if (j < C) {
                            const VanTerm vt = P.vterms[j];
                            const float f = fmaxf(fmaf(vt.a, S.slots[vt.slot * stride + k], vt.b), 0.f);
                            bv = fmaf(vt.w, f, bv);
                            few_add(am, cs, 1 + j, f);
                        }
                } else if (P.greeks) {
#pragma unroll
                    for (int j = 0; j < FEW_PRODUCTS; ++j)
                        if (j < C) {
                            const DevProduct pr = P.products[j];
                            const float f = payoff(P, pr, S.slots, S.grp, stride, k);
                            float d, g;
                            greeks_of(P, pr, S.slots, stride, k, d, g);
                            bv = fmaf(f, pr.fx, bv);
                            few_add(am, cs, 1 + 3 * j, f);
                            few_add(am, cs, 2 + 3 * j, d);
                            few_add(am, cs, 3 + 3 * j, g);
                        }
                } else {
#pragma unroll
                    for (int j = 0; j < FEW_PRODUCTS; ++j)
                        if (j < C) {
                            const DevProduct pr = P.products[j];
                            const float f = payoff(P, pr, S.slots, S.grp, stride, k);
                            bv = fmaf(f, pr.fx, bv);
                            few_add(am, cs, 1 + j, f);
                        }
                }
                few_add(am, cs, 0, bv);
            }
#pragma unroll
            for (int q = 0; q < 2 * FEW_Q_MAX; ++q)
                if (q < M) S.fa[q * T + t] += am[q];
            nvalid += nv;
            if ((++ntile % FEW_FLUSH) == 0) few_fold(S, M, T);
            continue;
        }
        ++ntile;
        for (int pc = 0; pc < C; pc += TH) {
            const int CP = min(C - pc, TH);
            const int G = TH / CP;
            const int pl = t % CP, g = t / CP;
            float a6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (g < G) {
                if (P.vanilla_only) {
                    // lean vanilla loop: f = max(a S + b, 0), no dispatch
                    const VanTerm vt = P.vterms[pc + pl];
                    const float* col = S.slots + vt.slot * stride;
                    const float c0 = fmaxf(fmaf(vt.a, col[k0], vt.b), 0.f);
                    float s1 = 0.f, s2 = 0.f;
#pragma unroll 4
                    for (int k = k0 + g; k < kend; k += G) {
                        const float f = fmaxf(fmaf(vt.a, col[k], vt.b), 0.f) - c0;
                        s1 += f;
                        s2 = fmaf(f, f, s2);
                    }
                    a6[0] = s1;
                    a6[1] = s2;
                } else {
                    const DevProduct pr = P.products[pc + pl];
                    const float c0 = payoff(P, pr, S.slots, S.grp, stride, k0);
                    float cd = 0.f, cg = 0.f;
                    if (P.greeks) greeks_of(P, pr, S.slots, stride, k0, cd, cg);
                    for (int k = k0 + g; k < kend; k += G) {
                        const float f = payoff(P, pr, S.slots, S.grp, stride, k) - c0;
                        a6[0] += f;
                        a6[1] = fmaf(f, f, a6[1]);
                        if (P.greeks) {
                            float d, gg;
                            greeks_of(P, pr, S.slots, stride, k, d, gg);
                            d -= cd;
                            gg -= cg;
                            a6[2] += d;
                            a6[3] = fmaf(d, d, a6[3]);
                            a6[4] += gg;
                            a6[5] = fmaf(gg, gg, a6[5]);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < 6; ++j) S.part[(g * CP + pl) * 6 + j] = a6[j];
            }
            __syncthreads();
            if (t < CP) {
                float cf = 0.f, cd = 0.f, cg = 0.f;
                if (P.vanilla_only) {
                    const VanTerm vt = P.vterms[pc + t];
                    cf = fmaxf(fmaf(vt.a, S.slots[vt.slot * stride + k0], vt.b), 0.f);
                } else {
                    const DevProduct pr = P.products[pc + t];
                    cf = payoff(P, pr, S.slots, S.grp, stride, k0);
                    if (P.greeks) greeks_of(P, pr, S.slots, stride, k0, cd, cg);
                }
                const float c3[3] = {cf, cd, cg};
                // the groups' FP32 partials of the tile are summed in FP32 (each is already a
                // shifted FP32 sum over the tile's columns), then converted once
                float f6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                for (int g2 = 0; g2 < G; ++g2)
#pragma unroll
                    for (int j = 0; j < 6; ++j) f6[j] += S.part[(g2 * CP + t) * 6 + j];
                double s6[6];
#pragma unroll
                for (int j = 0; j < 6; ++j) s6[j] = (double)f6[j];
                // sum f = sum (f - c) + n c;  sum f^2 = sum (f - c)^2 + 2 c sum (f - c) + n c^2
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const double c = c3[q], d1 = s6[2 * q];
                    s6[2 * q + 1] += 2.0 * c * d1 + (double)nv * c * c;
                    s6[2 * q] = d1 + (double)nv * c;
                }
#pragma unroll
                for (int j = 0; j < 6; ++j) acc[(size_t)(pc + t) * 6 + j] += s6[j];
            }
            __syncthreads();
        }
        // ---- book value per path (book_node.cpp:16-31) ---------------------
        double b1 = 0.0, b2 = 0.0;
        float bv[PP];
#pragma unroll
        for (int p = 0; p < PP; ++p) bv[p] = 0.f;
        if (P.vanilla_only) {
            // the thread's paths share each product's terms
            for (int q = 0; q < C; ++q) {
                const VanTerm vt = P.vterms[q];
                const float* col = S.slots + vt.slot * stride + t;
#pragma unroll
                for (int p = 0; p < PP; ++p) bv[p] = fmaf(vt.w, fmaxf(fmaf(vt.a, col[p * TH], vt.b), 0.f), bv[p]);
            }
        } else {
#pragma unroll
            for (int p = 0; p < PP; ++p)
                for (int q = 0; q < C; ++q) {
                    const DevProduct pr = P.products[q];
                    bv[p] = fmaf(payoff(P, pr, S.slots, S.grp, stride, t + p * TH), pr.fx, bv[p]);
                }
        }
#pragma unroll
        for (int p = 0; p < PP; ++p) {
            const float b = valid[p] ? bv[p] : 0.f;
            b1 += b;
            b2 += (double)b * b;
        }
        for (int o = 16; o > 0; o >>= 1) {
            b1 += __shfl_xor_sync(0xffffffffu, b1, o);
            b2 += __shfl_xor_sync(0xffffffffu, b2, o);
        }
        if ((t & 31) == 0) {
            S.red[2 * (t >> 5)] = b1;
            S.red[2 * (t >> 5) + 1] = b2;
        }
        __syncthreads();
        if (t == 0) {
            double s1 = 0, s2 = 0;
            for (int w = 0; w < TH / 32; ++w) {
                s1 += S.red[2 * w];
                s2 += S.red[2 * w + 1];
            }
            acc[(size_t)C * 6] += s1;
            acc[(size_t)C * 6 + 1] += s2;
        }
    }

    // ---- few-product mode: the CTA's row of FP64 sums, once --------------------
    if (P.few_m > 0 && ntile > 0) {
        const int M = P.few_m, NQ = M / 2;
        if (ntile % FEW_FLUSH) few_fold(S, M, T);
        __syncthreads();
        double* tot = reinterpret_cast<double*>(S.part); // the bridge stack's space, free after the paths
        if (t < M) {
            double sm = 0.0;
            for (int w = 0; w < TH / 32; ++w) {
                const float* k = S.fw + 2 * (w * M + t);
                sm += (double)k[0] - (double)k[1];
            }
            tot[t] = sm;
        }
        __syncthreads();
        if (t < NQ) {
            // sum x = sum (x - c) + n c;  sum x^2 = sum (x - c)^2 + 2 c sum (x - c) + n c^2
            const double c = S.fshift[t], d1 = tot[2 * t], d2 = tot[2 * t + 1], n = (double)nvalid;
            int idx;
            if (t == 0) idx = 6 * P.n_products;
            else if (P.greeks) idx = 6 * ((t - 1) / 3) + 2 * ((t - 1) % 3);
            else idx = 6 * (t - 1);
            acc[idx] = d1 + n * c;
            acc[idx + 1] = d2 + 2.0 * c * d1 + n * c * c;
        }
    }
    return true;
}

template <int TB, int NA, int MODEL, bool UNIFORM, int PP>
__global__ void __launch_bounds__((1 << TB) / PP, MinBlocks<TB, NA, PP>::value) book_kernel(const DevPlan P)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    book_body<TB, NA, MODEL, UNIFORM, PP>(P, smem_raw, blockIdx.x, gridDim.x, P.acc + (size_t)blockIdx.x * P.n_acc);
}

// ---------------------------------------------------------------------------
// Ragged batches in one persistent launch. Work item r of a book is what CTA r of
// the book's own launch does (its tiles r, r + grid, ..., its row r of FP64 sums),
// so a batch prices every book bit for bit as its own launch at the same grid
// would. The items sit in one list: books in decreasing item cost, a book's
// items consecutive. Resident CTAs take the next item from a counter in global
// memory, so the largest items go first and the small ones fill the tail; a CTA
// keeps the current book's plan in shared memory while its items follow on.
// ---------------------------------------------------------------------------
template <int TB, int PP>
__global__ void __launch_bounds__((1 << TB) / PP, MinBlocks<TB, 1, PP>::value)
    batch_kernel(const DevPlan* __restrict__ plans, const BatchBook* __restrict__ books, int n_books, int n_items,
                 int* next)
{
    constexpr int TH = (1 << TB) / PP;
    static_assert(sizeof(DevPlan) % 8 == 0, "plans are copied in 8-byte words");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) DevPlan sp;
    __shared__ int s_item, s_book, s_cur; // s_cur: the book whose plan is in sp
    const int t = threadIdx.x;
    if (t == 0) s_cur = -1;
    for (;;) {
        __syncthreads(); // the previous item is done with shared memory
        if (t == 0) {
            const int j = atomicAdd(next, 1);
            int lo = 0;
            if (j < n_items) { // the last book whose first item is at or before j
                int hi = n_books - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (__ldg(&books[mid].first) <= j) lo = mid;
                    else hi = mid - 1;
                }
            }
            s_item = j;
            s_book = lo;
        }
        __syncthreads();
        const int j = s_item, k = s_book;
        if (j >= n_items) break;
        const BatchBook bk = books[k];
        if (k != s_cur) { // nothing but shared memory carries over from one item to the next
            const unsigned long long* src = reinterpret_cast<const unsigned long long*>(plans + bk.plan);
            unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sp);
            for (int w = t; w < (int)(sizeof(DevPlan) / 8); w += TH) dst[w] = __ldg(src + w);
            __syncthreads();
            if (t == 0) s_cur = k;
        }
        const int r = j - bk.first;
        double* acc = sp.acc + (size_t)r * sp.n_acc;
        bool ok = true;
        switch (bk.variant) {
        case 0: ok = book_body<TB, 1, M_GBM, false, PP>(sp, smem_raw, r, bk.grid, acc); break;
        case 1: ok = book_body<TB, 1, M_HESTON, false, PP>(sp, smem_raw, r, bk.grid, acc); break;
        case 2: ok = book_body<TB, 1, M_LSV, false, PP>(sp, smem_raw, r, bk.grid, acc); break;
        case 4: ok = book_body<TB, 1, M_HESTON, true, PP>(sp, smem_raw, r, bk.grid, acc); break;
        default: ok = book_body<TB, 1, M_GBM, true, PP>(sp, smem_raw, r, bk.grid, acc); break;
        }
        if (!ok) break; // the book's cancel word is set: this CTA stops
    }
}

// ---- launch wrappers --------------------------------------------------------
// Launch shapes. Single-asset variants come in five: (log2 paths per tile,
// paths per thread) = (8, 2), (8, 1), (7, 1), (7, 2), (8, 4), i.e. 128, 256, 128, 64
// and 64 threads per CTA, the first four bounded to 768 resident threads per SM
// worth of registers, the last to 7 CTAs of 64 threads; the autotuner picks one per
// book size. The mixed variant has one: (7, 1).
constexpr int N_SHAPES = 5;
constexpr int SHAPE_TB[N_SHAPES] = {8, 8, 7, 7, 8};
constexpr int SHAPE_PP[N_SHAPES] = {2, 1, 1, 2, 4};


template <int TB, int NA, int MODEL, bool UNIFORM, int PP>
static cudaError_t smem_attr_t()
{
    // once per variant: allow the device's opt-in maximum, so that launches of
    // any size (and graph nodes captured earlier) stay valid whatever runs next
    static bool done = false;
    if (done) return cudaSuccess;
    int dev = 0, mx = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, book_kernel<TB, NA, MODEL, UNIFORM, PP>);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(book_kernel<TB, NA, MODEL, UNIFORM, PP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 mx - (int)fa.sharedSizeBytes);
    done = e == cudaSuccess;
    return e;
}

template <int TB, int NA, int MODEL, bool UNIFORM, int PP>
static cudaError_t launch_book_t(const DevPlan& P, int grid, size_t smem, cudaStream_t st)
{
    cudaError_t e = smem_attr_t<TB, NA, MODEL, UNIFORM, PP>();
    if (e != cudaSuccess) return e;
    book_kernel<TB, NA, MODEL, UNIFORM, PP><<<grid, (1 << TB) / PP, smem, st>>>(P);
    return cudaGetLastError();
}

template <int TB, int NA, int MODEL, bool UNIFORM, int PP>
static int occ_t(size_t smem)
{
    auto k = book_kernel<TB, NA, MODEL, UNIFORM, PP>;
    if (smem_attr_t<TB, NA, MODEL, UNIFORM, PP>() != cudaSuccess) return 1;
    int n = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, (1 << TB) / PP, smem) != cudaSuccess) return 1;
    return n < 1 ? 1 : n;
}

// one single-asset model in each of the four shapes: launch (grid > 0) or occupancy (grid == 0)
template <int MODEL, bool UNIFORM>
static int single_t(const DevPlan* P, int shape, int grid, size_t smem, cudaStream_t st, cudaError_t* err)
{
    switch (shape) {
    case 0:
        if (grid) *err = launch_book_t<8, 1, MODEL, UNIFORM, 2>(*P, grid, smem, st);
        return grid ? 0 : occ_t<8, 1, MODEL, UNIFORM, 2>(smem);
    case 1:
        if (grid) *err = launch_book_t<8, 1, MODEL, UNIFORM, 1>(*P, grid, smem, st);
        return grid ? 0 : occ_t<8, 1, MODEL, UNIFORM, 1>(smem);
    case 2:
        if (grid) *err = launch_book_t<7, 1, MODEL, UNIFORM, 1>(*P, grid, smem, st);
        return grid ? 0 : occ_t<7, 1, MODEL, UNIFORM, 1>(smem);
    case 3:
        if (grid) *err = launch_book_t<7, 1, MODEL, UNIFORM, 2>(*P, grid, smem, st);
        return grid ? 0 : occ_t<7, 1, MODEL, UNIFORM, 2>(smem);
    default:
        if (grid) *err = launch_book_t<8, 1, MODEL, UNIFORM, 4>(*P, grid, smem, st);
        return grid ? 0 : occ_t<8, 1, MODEL, UNIFORM, 4>(smem);
    }
}

// per-model dispatch of one translation unit: launch (grid > 0) or occupancy (grid == 0)
int book_dispatch_gbm(const DevPlan* P, bool uniform, int shape, int grid, size_t smem, cudaStream_t st,
                      cudaError_t* err);
int book_dispatch_heston(const DevPlan* P, bool uniform, int shape, int grid, size_t smem, cudaStream_t st,
                         cudaError_t* err);
int book_dispatch_lsv(const DevPlan* P, int shape, int grid, size_t smem, cudaStream_t st, cudaError_t* err);
int book_dispatch_multi(const DevPlan* P, int variant, int shape, int grid, size_t smem, cudaStream_t st,
                        cudaError_t* err);

} // namespace thoth
