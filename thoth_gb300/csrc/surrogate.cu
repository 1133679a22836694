// surrogate.cu — BF16 tensor-core (tcgen05) kernels of the learned Heston
// surrogate: a validation GEMM, the fused MLP inference kernel, the training
// layers (forward with bias + SiLU epilogue, backward for inputs and weights)
// and Adam.
#include "engine.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace thoth {

// ---------------------------------------------------------------------------
// Validation GEMM: one CTA of 128 threads computes D (128 x N, FP32, row-major)
// = A (128 x K) * B (N x K)^T with A, B bf16 row-major in global memory.
// N in {16..256} multiple of 16, K multiple of 16 up to 256.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) tc_gemm_test_kernel(const __nv_bfloat16* __restrict__ A,
                                                           const __nv_bfloat16* __restrict__ B, int N, int K,
                                                           float* __restrict__ D, int* status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t taddr_s;
    unsigned char* sA = sm;
    unsigned char* sB = sm + 128 * K * 2;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    uint32_t ncols = 32;
    while (ncols < (uint32_t)N) ncols <<= 1;
    if (warp == 0) tc::tmem_alloc(&taddr_s, ncols);
    if (t == 0) tc::mbar_init(&mbar, 1);
    // stage A and B into the K-major core-matrix layout (16-byte chunks)
    const int kc = K / 8;
    for (int c = t; c < 128 * kc; c += 128) {
        const int r = c / kc, kb = c % kc;
        *reinterpret_cast<uint4*>(sA + tc::cm_offset(r, kb * 8, 128)) =
            *reinterpret_cast<const uint4*>(A + (size_t)r * K + kb * 8);
    }
    for (int c = t; c < N * kc; c += 128) {
        const int r = c / kc, kb = c % kc;
        *reinterpret_cast<uint4*>(sB + tc::cm_offset(r, kb * 8, N)) =
            *reinterpret_cast<const uint4*>(B + (size_t)r * K + kb * 8);
    }
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = taddr_s;
    if (t == 0) {
        const uint32_t idesc = tc::make_idesc_bf16(128, N);
        const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
        for (int kk = 0; kk < K / 16; ++kk) {
            const uint64_t ad = tc::make_desc(a0 + (uint32_t)(2 * kk) * (128 * 16), 128 * 16, 128);
            const uint64_t bd = tc::make_desc(b0 + (uint32_t)(2 * kk) * (uint32_t)(N * 16), (uint32_t)N * 16, 128);
            tc::mma_bf16(tm, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::mma_commit(&mbar);
    }
    const bool ok = tc::mbar_wait(&mbar, 0);
    if (!ok && lane == 0) atomicExch(status, 1);
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) D[(size_t)row * N + c0 + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, ncols);
}

cudaError_t launch_tc_gemm_test(const void* A, const void* B, int N, int K, float* D, int* status, cudaStream_t st)
{
    // padded far beyond the operands so that every descriptor-generated address stays
    // inside this CTA's shared memory even if an offset field were misread
    const size_t need = (size_t)(128 + N) * K * 2;
    const size_t smem = need > 200 * 1024 ? need : 200 * 1024;
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_test_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    tc_gemm_test_kernel<<<1, 128, smem, st>>>(reinterpret_cast<const __nv_bfloat16*>(A),
                                              reinterpret_cast<const __nv_bfloat16*>(B), N, K, D, status);
    return cudaGetLastError();
}


// ===========================================================================
// The surrogate MLP: 7 inputs (padded to 16) -> 4 x 128 SiLU -> 1.
// Parameters (FP32 master, offsets in floats):
//   W1 [128][16], b1[128], W2..W4 [128][128] + b[128], w5[128], b5[1]
// BF16 copies of W1..W4 are the tensor-core operands.
// ===========================================================================
namespace mlp {

constexpr int H = 128;      // hidden width
constexpr int KIN = 16;     // input features padded to one MMA K slice
constexpr int ROWS = 128;   // rows per tile = MMA M
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + H * KIN;
constexpr int OFF_W2 = OFF_B1 + H;
constexpr int LAYER = H * H + H; // W + b of a hidden layer 2..4
constexpr int OFF_W5 = OFF_W2 + 3 * LAYER;
constexpr int OFF_B5 = OFF_W5 + H;
constexpr int N_PARAMS = OFF_B5 + 1;
constexpr int OFF_BF_W1 = 0;                 // bf16 weights, offsets in elements
constexpr int OFF_BF_W2 = H * KIN;
constexpr int N_BF = H * KIN + 3 * H * H;

__host__ __device__ constexpr int w_off(int l) { return l == 1 ? OFF_W1 : OFF_W2 + (l - 2) * LAYER; }
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + H * (l == 1 ? KIN : H); }
__host__ __device__ constexpr int bf_off(int l) { return l == 1 ? OFF_BF_W1 : OFF_BF_W2 + (l - 2) * H * H; }

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = __fdividef(1.0f, 1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// stage an R x K row-major bf16 global tile (row stride ld elements, rows >= valid
// are zero-filled) into the K-major core-matrix layout
template <int R>
__device__ __forceinline__ void stage(unsigned char* dst, const __nv_bfloat16* src, int ld, int K, int valid)
{
    const int kc = K / 8;
    for (int c = threadIdx.x; c < R * kc; c += blockDim.x) {
        const int r = c / kc, kb = c % kc;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r < valid) v = *reinterpret_cast<const uint4*>(src + (size_t)r * ld + kb * 8);
        *reinterpret_cast<uint4*>(dst + tc::cm_offset(r, kb * 8, R)) = v;
    }
}

// stage the transpose: dst (R x K) element (r, k) = src[k][r], src row-major with
// row stride ld, src rows >= valid_k are zero-filled
template <int R>
__device__ __forceinline__ void stage_t(unsigned char* dst, const __nv_bfloat16* src, int ld, int K, int valid_k)
{
    for (int e = threadIdx.x; e < R * K; e += blockDim.x) {
        const int k = e / R, r = e % R; // consecutive threads read consecutive src columns
        const __nv_bfloat16 v = (k < valid_k) ? src[(size_t)k * ld + r] : __float2bfloat16(0.f);
        *reinterpret_cast<__nv_bfloat16*>(dst + tc::cm_offset(r, k, R)) = v;
    }
}

struct Ctx {
    uint64_t* mbar;
    uint32_t tm;
    uint32_t phase;
    int* status;
};

// issue D (+)= A * B^T over K (single thread), then everyone waits for it
__device__ __forceinline__ bool run_mma(Ctx& c, uint32_t dcol, const unsigned char* sA, int RA, const unsigned char* sB,
                                        int RB, int K, bool accumulate_first)
{
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc::make_idesc_bf16(RA, RB);
        const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
        for (int kk = 0; kk < K / 16; ++kk) {
            const uint64_t ad = tc::make_desc(a0 + (uint32_t)(2 * kk) * (uint32_t)(RA * 16), (uint32_t)RA * 16, 128);
            const uint64_t bd = tc::make_desc(b0 + (uint32_t)(2 * kk) * (uint32_t)(RB * 16), (uint32_t)RB * 16, 128);
            tc::mma_bf16(c.tm + dcol, ad, bd, idesc, (kk > 0 || accumulate_first) ? 1u : 0u);
        }
        tc::mma_commit(c.mbar);
    }
    const bool ok = tc::mbar_wait(c.mbar, c.phase);
    c.phase ^= 1u;
    if (!ok && (threadIdx.x & 31) == 0) atomicExch(c.status, 1);
    tc::fence_after_sync();
    return ok;
}

// 128-column row of this thread's TMEM lane (row = threadIdx.x) starting at col
__device__ __forceinline__ void load_row(const Ctx& c, uint32_t col, int ncols, float* v)
{
    const int warp = threadIdx.x >> 5;
    for (int c0 = 0; c0 < ncols; c0 += 16) {
        float t[16];
        tc::tmem_ld16(c.tm + ((uint32_t)(warp * 32) << 16) + col + (uint32_t)c0, t);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[c0 + j] = t[j];
    }
}

// write this thread's row of 128 bf16 values into a K-major core-matrix tile
__device__ __forceinline__ void put_row(unsigned char* tile, int row, const float* v, int K)
{
    for (int kb = 0; kb < K / 8; ++kb) {
        __align__(16) __nv_bfloat16 h[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) h[j] = __float2bfloat16(v[kb * 8 + j]);
        *reinterpret_cast<uint4*>(tile + tc::cm_offset(row, kb * 8, ROWS)) = *reinterpret_cast<const uint4*>(h);
    }
}

struct TrainSched {
    long long count;           // steps done in this training call
    long long total;           // steps of the call
    long long steps_per_epoch; // batches of one permutation
    long long step0;           // Adam steps before the call
    double lr0;                // peak learning rate
    float lr_t, bc1, bc2;      // this step's learning rate and bias corrections
    int rows;                  // batch rows
    long long decay_steps;     // steps of the cosine decay (after them the rate stays at lr_lo)
    double lr_lo;              // the rate the decay ends at
};

struct TrainArgs {
    int rows;                       // batch rows (multiple of 128)
    const __nv_bfloat16* x;         // [rows][16] normalised inputs
    const float* y;                 // [rows] targets
    const float* inv_w2;            // [rows] loss weights 1 / scale^2
    const float* params;            // FP32 master
    const __nv_bfloat16* wbf;       // bf16 W1..W4
    float* z[5];                    // pre-activations of layers 1..4 ([rows][128]); index by layer
    __nv_bfloat16* a[5];            // a[0] = x (alias), a[l] = SiLU(z[l]) ([rows][128])
    __nv_bfloat16* dz[5];           // dL/dz of layers 1..4 ([rows][128])
    float* part;                    // per-CTA partial gradients, [tiles][N_PARAMS]
    float* loss_part;               // [tiles]
    int* status;
};

// forward of hidden layer l for one 128-row tile; layer 4 also evaluates the head,
// the loss and its gradient back to dz4, plus the head's weight gradients
template <int L>
__global__ void __launch_bounds__(128) fwd_layer_kernel(TrainArgs A)
{
    constexpr int K = (L == 1) ? KIN : H;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tm_s;
    __shared__ float red[4][H + 2];
    unsigned char* sX = sm;                 // 128 x K
    unsigned char* sW = sm + ROWS * K * 2;  // 128 x K
    const int t = threadIdx.x, warp = t >> 5;
    const int tile = blockIdx.x, r0 = tile * ROWS;
    if (warp == 0) tc::tmem_alloc(&tm_s, 128);
    if (t == 0) tc::mbar_init(&mbar, 1);
    const __nv_bfloat16* src = (L == 1) ? A.x + (size_t)r0 * KIN : A.a[L - 1] + (size_t)r0 * H;
    stage<ROWS>(sX, src, K, K, ROWS);
    stage<ROWS>(sW, A.wbf + bf_off(L), K, K, H);
    Ctx c{&mbar, 0, 0, A.status};
    __syncthreads();
    c.tm = tm_s;
    const bool ok = run_mma(c, 0, sX, ROWS, sW, H, K, false);
    float v[H];
    if (ok) load_row(c, 0, H, v);
    else
        for (int j = 0; j < H; ++j) v[j] = 0.f;
    const int row = r0 + t;
    const float* b = A.params + b_off(L);
    float* zr = A.z[L] + (size_t)row * H;
    __nv_bfloat16* ar = A.a[L] + (size_t)row * H;
    for (int j = 0; j < H; ++j) {
        const float z = v[j] + b[j];
        v[j] = z;
        zr[j] = z;
        ar[j] = __float2bfloat16(silu(z));
    }
    if (L == 4) {
        // head y = w5 . a4 + b5, weighted MSE, dL/dy, dL/da4 = dy w5, dz4 = da4 * silu'(z4)
        const float* w5 = A.params + OFF_W5;
        float yhat = A.params[OFF_B5];
        for (int j = 0; j < H; ++j) yhat = fmaf(w5[j], silu(v[j]), yhat);
        const float e = yhat - A.y[row];
        const float w = A.inv_w2[row];
        const float dy = 2.f * e * w / (float)A.rows;
        float* gp = A.part + (size_t)tile * N_PARAMS;
        __nv_bfloat16* dzr = A.dz[4] + (size_t)row * H;
        for (int j = 0; j < H; ++j) {
            const float s = silu(v[j]);
            dzr[j] = __float2bfloat16(dy * w5[j] * dsilu(v[j]));
            v[j] = dy * s; // head weight gradient contribution of this row
        }
        // reduce over the tile's rows: warp shuffles then smem
        const int lane = t & 31;
        for (int j = 0; j < H; ++j) {
            float s = v[j];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) red[warp][j] = s;
        }
        float sdy = dy, sl = e * e * w;
        for (int o = 16; o > 0; o >>= 1) {
            sdy += __shfl_xor_sync(0xffffffffu, sdy, o);
            sl += __shfl_xor_sync(0xffffffffu, sl, o);
        }
        if (lane == 0) {
            red[warp][H] = sdy;
            red[warp][H + 1] = sl;
        }
        __syncthreads();
        gp[OFF_W5 + t] = red[0][t] + red[1][t] + red[2][t] + red[3][t];
        if (t == 0) {
            gp[OFF_B5] = red[0][H] + red[1][H] + red[2][H] + red[3][H];
            A.loss_part[tile] = red[0][H + 1] + red[1][H + 1] + red[2][H + 1] + red[3][H + 1];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(c.tm, 128);
}

// backward of hidden layer l for one tile: partial dW_l = dz_l^T a_{l-1},
// partial db_l = sum dz_l, and for l >= 2 dz_{l-1} = (dz_l W_l) * silu'(z_{l-1})
template <int L>
__global__ void __launch_bounds__(128) bwd_layer_kernel(TrainArgs A)
{
    constexpr int K = (L == 1) ? KIN : H; // input width of layer l
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tm_s;
    unsigned char* sDzT = sm;                      // 128 (out) x 128 (rows): dz^T
    unsigned char* sAT = sDzT + ROWS * H * 2;      // K (in) x 128 (rows): a_{l-1}^T
    unsigned char* sDz = sAT + K * ROWS * 2;       // 128 (rows) x 128 (out): dz
    unsigned char* sWT = sDz + ROWS * H * 2;       // K (in) x 128 (out): W^T
    const int t = threadIdx.x, warp = t >> 5;
    const int tile = blockIdx.x, r0 = tile * ROWS;
    if (warp == 0) tc::tmem_alloc(&tm_s, 256);
    if (t == 0) tc::mbar_init(&mbar, 1);
    const __nv_bfloat16* dz = A.dz[L] + (size_t)r0 * H;
    const __nv_bfloat16* ain = (L == 1) ? A.x + (size_t)r0 * KIN : A.a[L - 1] + (size_t)r0 * H;
    stage_t<H>(sDzT, dz, H, ROWS, ROWS);           // (o, r) = dz[r][o]
    stage_t<K>(sAT, ain, K, ROWS, ROWS);           // (i, r) = a[r][i]
    if (L > 1) {
        stage<ROWS>(sDz, dz, H, H, ROWS);          // (r, o) = dz[r][o]
        stage_t<K>(sWT, A.wbf + bf_off(L), K, H, H); // (i, o) = W[o][i]
    }
    Ctx c{&mbar, 0, 0, A.status};
    __syncthreads();
    c.tm = tm_s;
    // dW (128 out x K in) in TMEM columns [0, K)
    bool ok = run_mma(c, 0, sDzT, H, sAT, K, ROWS, false);
    float* gp = A.part + (size_t)tile * N_PARAMS;
    {
        float v[H];
        if (ok) load_row(c, 0, K, v);
        else
            for (int j = 0; j < K; ++j) v[j] = 0.f;
        float* gw = gp + w_off(L) + t * K; // row o = t
        for (int j = 0; j < K; ++j) gw[j] = v[j];
        // db_o = sum over rows of dz[r][o] (coalesced over o = t)
        float s = 0.f;
        for (int r = 0; r < ROWS; ++r) s += __bfloat162float(dz[(size_t)r * H + t]);
        gp[b_off(L) + t] = s;
    }
    if (L > 1) {
        // da_{l-1} (128 rows x K in) in TMEM columns [128, 128 + K)
        ok = run_mma(c, 128, sDz, ROWS, sWT, K, H, false) && ok;
        float v[H];
        if (ok) load_row(c, 128, K, v);
        else
            for (int j = 0; j < K; ++j) v[j] = 0.f;
        const int row = r0 + t;
        const float* zp = A.z[L - 1] + (size_t)row * H;
        __nv_bfloat16* out = A.dz[L - 1] + (size_t)row * H;
        for (int j = 0; j < K; ++j) out[j] = __float2bfloat16(v[j] * dsilu(zp[j]));
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(c.tm, 256);
}

// the learning-rate schedule (a cosine decay from lr0 to lr_lo over decay_steps steps, then
// lr_lo) and Adam's bias corrections of step `count` of a training call, computed where the
// graph of one step can read them (its kernels' arguments stay the same from step to step)
__host__ __device__ inline void sched_set(TrainSched& s)
{
    const double pi = 3.14159265358979323846;
    const double step = (double)(s.step0 + s.count + 1);
    const double c = (double)(s.count < s.decay_steps ? s.count : s.decay_steps);
    s.lr_t = (float)(s.lr_lo + (s.lr0 - s.lr_lo) * 0.5 * (1.0 + cos(pi * c / (double)s.decay_steps)) + 1e-6);
    s.bc1 = (float)(1.0 - pow(0.9, step));
    s.bc2 = (float)(1.0 - pow(0.999, step));
}

__global__ void sched_advance_kernel(TrainSched* s)
{
    s->count += 1;
    sched_set(*s);
}

// grad[j] = sum over tiles of part[tile][j] (fixed order), then Adam on the FP32
// master and refresh of the bf16 operand copies
__global__ void adam_kernel(float* params, float* m, float* v, const float* part, int tiles, __nv_bfloat16* wbf,
                            float lr, float b1, float b2, float eps, float bc1, float bc2, const TrainSched* sched)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N_PARAMS) return;
    if (sched) { // this step's learning rate and bias corrections, set by sched_advance_kernel
        lr = sched->lr_t;
        bc1 = sched->bc1;
        bc2 = sched->bc2;
    }
    float g = 0.f;
    for (int tl = 0; tl < tiles; ++tl) g += part[(size_t)tl * N_PARAMS + j];
    // W1 columns f and f + 7 carry the hi and lo bf16 parts of feature f with one
    // tied weight: column f's thread applies the summed gradient to both; columns
    // 14 and 15 are padding and stay zero
    if (j < OFF_B1) {
        const int col = j % KIN;
        if (col >= 7) return;
        for (int tl = 0; tl < tiles; ++tl) g += part[(size_t)tl * N_PARAMS + j + 7];
    }
    const float mj = fmaf(b1, m[j], (1.f - b1) * g);
    const float vj = fmaf(b2, v[j], (1.f - b2) * g * g);
    m[j] = mj;
    v[j] = vj;
    const float p = params[j] - lr * (mj / bc1) / (sqrtf(vj / bc2) + eps);
    params[j] = p;
    // bf16 copies of W1..W4
    if (j < OFF_B1) {
        params[j + 7] = p;
        wbf[OFF_BF_W1 + j] = __float2bfloat16(p);
        wbf[OFF_BF_W1 + j + 7] = __float2bfloat16(p);
    } else if (j >= OFF_W2 && j < OFF_W5) {
        const int l = (j - OFF_W2) / LAYER, o = (j - OFF_W2) % LAYER;
        if (o < H * H) wbf[OFF_BF_W2 + l * H * H + o] = __float2bfloat16(p);
    }
}

// tail averaging of the weights: avg = params (k == 0), else avg += (params - avg) / (k + 1)
__global__ void weight_avg_kernel(const float* __restrict__ params, float* __restrict__ avg, int k)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N_PARAMS) return;
    avg[j] = k == 0 ? params[j] : fmaf(params[j] - avg[j], 1.0f / (float)(k + 1), avg[j]);
}

// the model takes the averaged weights, and its bf16 operand copies follow (as in adam_kernel)
__global__ void weight_avg_finish_kernel(float* __restrict__ params, const float* __restrict__ avg,
                                         __nv_bfloat16* __restrict__ wbf)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N_PARAMS) return;
    if (j < OFF_B1 && j % KIN >= 7) return; // the tied hi/lo columns are written by their partner
    const float p = avg[j];
    params[j] = p;
    if (j < OFF_B1) {
        params[j + 7] = p;
        wbf[OFF_BF_W1 + j] = __float2bfloat16(p);
        wbf[OFF_BF_W1 + j + 7] = __float2bfloat16(p);
    } else if (j >= OFF_W2 && j < OFF_W5) {
        const int l = (j - OFF_W2) / LAYER, o = (j - OFF_W2) % LAYER;
        if (o < H * H) wbf[OFF_BF_W2 + l * H * H + o] = __float2bfloat16(p);
    }
}

__global__ void sum_kernel(const float* x, int n, float* out)
{
    __shared__ float s[256];
    float a = 0.f;
    for (int i = threadIdx.x; i < n; i += 256) a += x[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

// fused inference: persistent CTAs of three warpgroups, one CTA per SM. The weights
// are resident in shared memory and shared by all; each warpgroup walks its own
// 128-cell tiles with its own TMEM accumulator (128 columns each), mbarrier and
// named barrier, so the warpgroups' bias + SiLU epilogues overlap one another's
// MMAs. The epilogue streams 16 accumulator columns at a time straight into the
// next layer's A operand (K-major core-matrix layout); the last layer folds the head.
// Three warpgroups: 208 KB of shared memory (the weights and three tiles of
// activations) and 384 of the 512 TMEM columns.
constexpr int INFER_WG = 3;
constexpr int INFER_THREADS = 128 * INFER_WG;
constexpr uint32_t INFER_TMEM_COLS = 512; // a power of two >= 128 x INFER_WG

__device__ __forceinline__ void wg_sync(int wg) { asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory"); }

// SiLU of two columns at once for inference: silu(z) = z sigmoid(z), sigmoid(z) = (1 + tanh(z/2)) / 2,
// with one special-function-unit tanh per value (the exponential and reciprocal form takes two)
// and the arithmetic on packed pairs. tanh.approx is within about 2^-11 of tanh, well inside the
// bf16 rounding (2^-9 relative) the next layer's operand gets anyway.
__device__ __forceinline__ float2 silu2_infer(float2 z)
{
    const float2 h = __fmul2_rn(z, make_float2(0.5f, 0.5f));
    float t0, t1;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t0) : "f"(h.x));
    asm("tanh.approx.f32 %0, %1;" : "=f"(t1) : "f"(h.y));
    return __ffma2_rn(h, make_float2(t0, t1), h); // z/2 (1 + tanh(z/2))
}

__global__ void __launch_bounds__(INFER_THREADS) infer_kernel(const __nv_bfloat16* __restrict__ x, int n,
                                                              const float* params, const __nv_bfloat16* wbf,
                                                              float* __restrict__ y, int* status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar[INFER_WG];
    __shared__ uint32_t tm_s;
    __shared__ __align__(16) float sb[4 * H + H + 1]; // biases of layers 1..4, head weights, head bias (pairs read as float2)
    unsigned char* sW1 = sm;                         // 128 x 16
    unsigned char* sW = sW1 + H * KIN * 2;           // 3 x (128 x 128)
    const int t = threadIdx.x, warp = t >> 5, wg = t >> 7, r = t & 127;
    unsigned char* sX = sW + 3 * H * H * 2 + wg * (ROWS * KIN * 2 + ROWS * H * 2); // this warpgroup's 128 x 16
    unsigned char* sAct = sX + ROWS * KIN * 2;                                    // and 128 x 128
    if (warp == 0) tc::tmem_alloc(&tm_s, INFER_TMEM_COLS);
    if (t == 0)
        for (int w = 0; w < INFER_WG; ++w) tc::mbar_init(&mbar[w], 1);
    stage<H>(sW1, wbf + OFF_BF_W1, KIN, KIN, H);
    for (int l = 0; l < 3; ++l) stage<H>(sW + l * H * H * 2, wbf + OFF_BF_W2 + l * H * H, H, H, H);
    for (int i = t; i < 4 * H; i += INFER_THREADS) sb[i] = params[b_off(1 + i / H) + i % H];
    for (int i = t; i < H; i += INFER_THREADS) sb[4 * H + i] = params[OFF_W5 + i];
    if (t == 0) sb[5 * H] = params[OFF_B5];
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    Ctx c{&mbar[wg], tm_s + (uint32_t)(wg * 128), 0, status};
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16; // TMEM lanes of this warp
    const int tiles = (n + ROWS - 1) / ROWS;
    for (int tile = INFER_WG * blockIdx.x + wg; tile < tiles; tile += INFER_WG * gridDim.x) {
        const int r0 = tile * ROWS;
        const int valid = min(ROWS, n - r0);
        // this warpgroup stages its input tile (row r by thread r: two 16-byte chunks)
        for (int kb = 0; kb < KIN / 8; ++kb) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (r < valid) v = *reinterpret_cast<const uint4*>(x + (size_t)(r0 + r) * KIN + kb * 8);
            *reinterpret_cast<uint4*>(sX + tc::cm_offset(r, kb * 8, ROWS)) = v;
        }
        float o = sb[5 * H];
        for (int l = 1; l <= 4; ++l) {
            const unsigned char* A = (l == 1) ? sX : sAct;
            const unsigned char* W = (l == 1) ? sW1 : sW + (l - 2) * H * H * 2;
            const int K = (l == 1) ? KIN : H;
            // operand writes of every thread of the warpgroup -> visible to the tensor core
            tc::fence_smem_async();
            tc::fence_before_sync();
            wg_sync(wg);
            tc::fence_after_sync();
            if (r == 0) {
                const uint32_t idesc = tc::make_idesc_bf16(ROWS, H);
                const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(W);
                for (int kk = 0; kk < K / 16; ++kk) {
                    const uint64_t ad = tc::make_desc(a0 + (uint32_t)(2 * kk) * (ROWS * 16), ROWS * 16, 128);
                    const uint64_t bd = tc::make_desc(b0 + (uint32_t)(2 * kk) * (H * 16), H * 16, 128);
                    tc::mma_bf16(c.tm, ad, bd, idesc, kk > 0 ? 1u : 0u);
                }
                tc::mma_commit(c.mbar);
            }
            const bool ok = tc::mbar_wait(c.mbar, c.phase);
            c.phase ^= 1u;
            if (!ok && (t & 31) == 0) atomicExch(c.status, 1);
            tc::fence_after_sync();
            const float* bias = sb + (l - 1) * H;
            for (int c0 = 0; c0 < H; c0 += 16) {
                float v[16];
                tc::tmem_ld16(c.tm + lane_base + (uint32_t)c0, v);
                if (!ok) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] = 0.f;
                }
#pragma unroll
                for (int j = 0; j < 16; j += 2) {
                    const float2 z = __fadd2_rn(make_float2(v[j], v[j + 1]),
                                                *reinterpret_cast<const float2*>(bias + c0 + j));
                    const float2 a = silu2_infer(z);
                    v[j] = a.x;
                    v[j + 1] = a.y;
                }
                if (l < 4) {
                    // the MMA that read sAct has completed: overwrite it in place with the next operand
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        __align__(16) __nv_bfloat162 hv[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) hv[j] = __floats2bfloat162_rn(v[h * 8 + 2 * j], v[h * 8 + 2 * j + 1]);
                        *reinterpret_cast<uint4*>(sAct + tc::cm_offset(r, c0 + h * 8, ROWS)) =
                            *reinterpret_cast<const uint4*>(hv);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j) o = fmaf(sb[4 * H + c0 + j], v[j], o);
                }
            }
            // every lane has read the accumulator before the next MMA overwrites it
            tc::fence_before_sync();
        }
        if (r < valid) y[r0 + r] = o;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm_s, INFER_TMEM_COLS);
}

} // namespace mlp

// ---- launchers -----------------------------------------------------------------
constexpr size_t kFwdSmem1 = (size_t)2 * mlp::ROWS * mlp::KIN * 2;
constexpr size_t kFwdSmem = (size_t)2 * mlp::ROWS * mlp::H * 2;

constexpr size_t kBwdSmem = (size_t)(mlp::ROWS * mlp::H + mlp::H * mlp::ROWS + mlp::ROWS * mlp::H + mlp::H * mlp::H) * 2;
constexpr size_t kBwdSmem1 = (size_t)(mlp::ROWS * mlp::H + mlp::KIN * mlp::ROWS) * 2;

// the layer kernels' shared-memory limits, set once per device (not inside a captured step)
static cudaError_t train_attributes()
{
    using namespace mlp;
    static bool set_on[64] = {};
    int dev = 0;
    cudaError_t e0 = cudaGetDevice(&dev);
    if (e0 != cudaSuccess) return e0;
    bool dummy = false;
    bool& done = (dev >= 0 && dev < 64) ? set_on[dev] : dummy;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(fwd_layer_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fwd_layer_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fwd_layer_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fwd_layer_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bwd_layer_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bwd_layer_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bwd_layer_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bwd_layer_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem1);
    done = e == cudaSuccess;
    return e;
}

cudaError_t mlp_train_prepare() { return train_attributes(); }

// one training step: forward and backward layer by layer, Adam. With a schedule (sched not
// null) the learning rate and bias corrections are read on the device, so the step's launches
// have the same arguments every step and can be captured once into a graph.
cudaError_t mlp_train_step(const mlp::TrainArgs& A, float* params, float* m, float* v, __nv_bfloat16* wbf, float lr,
                           float b1, float b2, float eps, float bc1, float bc2, float* loss_out, cudaStream_t st,
                           const mlp::TrainSched* sched)
{
    using namespace mlp;
    const int tiles = A.rows / ROWS;
    cudaError_t e = train_attributes();
    if (e != cudaSuccess) return e;
    fwd_layer_kernel<1><<<tiles, 128, kFwdSmem1, st>>>(A);
    fwd_layer_kernel<2><<<tiles, 128, kFwdSmem, st>>>(A);
    fwd_layer_kernel<3><<<tiles, 128, kFwdSmem, st>>>(A);
    fwd_layer_kernel<4><<<tiles, 128, kFwdSmem, st>>>(A);
    bwd_layer_kernel<4><<<tiles, 128, kBwdSmem, st>>>(A);
    bwd_layer_kernel<3><<<tiles, 128, kBwdSmem, st>>>(A);
    bwd_layer_kernel<2><<<tiles, 128, kBwdSmem, st>>>(A);
    bwd_layer_kernel<1><<<tiles, 128, kBwdSmem1, st>>>(A);
    adam_kernel<<<(N_PARAMS + 255) / 256, 256, 0, st>>>(params, m, v, A.part, tiles, wbf, lr, b1, b2, eps, bc1, bc2,
                                                         sched);
    if (loss_out) sum_kernel<<<1, 256, 0, st>>>(A.loss_part, tiles, loss_out);
    return cudaGetLastError();
}

void mlp_sched_init(mlp::TrainSched& s) { mlp::sched_set(s); }

// sum = y (j == 0) or sum + y; at the last member (j == k - 1) the sum becomes the mean
__global__ void mean_add_kernel(float* __restrict__ sum, const float* __restrict__ y, int64_t n, int j, int k)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a = j == 0 ? y[i] : sum[i] + y[i];
    if (j == k - 1) a *= 1.0f / (float)k;
    sum[i] = a;
}

cudaError_t mlp_mean_add(float* sum, const float* y, int64_t n, int j, int k, cudaStream_t st)
{
    mean_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sum, y, n, j, k);
    return cudaGetLastError();
}

cudaError_t mlp_weight_avg(const float* params, float* avg, int k, cudaStream_t st)
{
    mlp::weight_avg_kernel<<<(mlp::N_PARAMS + 255) / 256, 256, 0, st>>>(params, avg, k);
    return cudaGetLastError();
}

cudaError_t mlp_weight_avg_finish(float* params, const float* avg, __nv_bfloat16* wbf, cudaStream_t st)
{
    mlp::weight_avg_finish_kernel<<<(mlp::N_PARAMS + 255) / 256, 256, 0, st>>>(params, avg, wbf);
    return cudaGetLastError();
}

cudaError_t mlp_sched_advance(mlp::TrainSched* s, cudaStream_t st)
{
    mlp::sched_advance_kernel<<<1, 1, 0, st>>>(s);
    return cudaGetLastError();
}

cudaError_t mlp_infer(const __nv_bfloat16* x, int n, const float* params, const __nv_bfloat16* wbf, float* y,
                      int* status, int grid, cudaStream_t st)
{
    using namespace mlp;
    const size_t smem = (size_t)(H * KIN + 3 * H * H + INFER_WG * (ROWS * KIN + ROWS * H)) * 2;
    cudaError_t e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    infer_kernel<<<grid, INFER_THREADS, smem, st>>>(x, n, params, wbf, y, status);
    return cudaGetLastError();
}

// one training batch from the device-resident set: rows perm[first .. first + rows)
__global__ void gather_batch_kernel(const __nv_bfloat16* __restrict__ X, const float* __restrict__ Y,
                                    const float* __restrict__ W, const int* __restrict__ perm, int64_t first, int rows,
                                    __nv_bfloat16* __restrict__ xb, float* __restrict__ yb, float* __restrict__ wb,
                                    const mlp::TrainSched* sched)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    if (sched) first = (sched->count % sched->steps_per_epoch) * (int64_t)sched->rows; // this step's batch
    const int64_t i = __ldg(perm + first + r);
    const uint4* src = reinterpret_cast<const uint4*>(X + i * mlp::KIN);
    uint4* dst = reinterpret_cast<uint4*>(xb + (int64_t)r * mlp::KIN);
    dst[0] = __ldg(src);
    dst[1] = __ldg(src + 1);
    yb[r] = __ldg(Y + i);
    wb[r] = __ldg(W + i);
}

cudaError_t mlp_gather_batch(const __nv_bfloat16* X, const float* Y, const float* W, const int* perm, int64_t first,
                             int rows, __nv_bfloat16* xb, float* yb, float* wb, cudaStream_t st,
                             const mlp::TrainSched* sched)
{
    gather_batch_kernel<<<(rows + 127) / 128, 128, 0, st>>>(X, Y, W, perm, first, rows, xb, yb, wb, sched);
    return cudaGetLastError();
}

int mlp_n_params() { return mlp::N_PARAMS; }
int mlp_n_bf() { return mlp::N_BF; }

// ---------------------------------------------------------------------------
// Lattice serving: the cells of n_sets parameter sets x n_T maturities x n_lm
// log-moneyness, cell c = (set * n_T + j) * n_lm + k with raw features
// (lm[k], T[j], kappa, theta, xi, rho, v0 of the set), built, clipped to the
// training box and normalised on the device (the network's hi/lo bf16 input
// split), and the network's output scaled back to a price in units of spot.
// ---------------------------------------------------------------------------
struct LatticeArgs {
    const double* params; // [n_sets][5] kappa, theta, xi, rho, v0
    const double* lms;    // [n_lm]
    const double* Ts;     // [n_T]
    double lo[7], hi[7];  // training box
    double floor;         // scale floor (units of spot)
    int64_t n;            // cells
    int n_lm, n_T;
};

__device__ __forceinline__ void lattice_cell(const LatticeArgs& A, int64_t c, double (&f)[7])
{
    const int64_t per = (int64_t)A.n_lm * A.n_T;
    const int64_t set = c / per;
    const int r = (int)(c % per);
    f[0] = A.lms[r % A.n_lm];
    f[1] = A.Ts[r / A.n_lm];
    for (int q = 0; q < 5; ++q) f[2 + q] = A.params[set * 5 + q];
#pragma unroll
    for (int q = 0; q < 7; ++q) f[q] = fmin(fmax(f[q], A.lo[q]), A.hi[q]);
}

__global__ void lattice_features_kernel(const LatticeArgs A, __nv_bfloat16* __restrict__ x)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.n) return;
    double f[7];
    lattice_cell(A, c, f);
    __nv_bfloat16* row = x + c * mlp::KIN;
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        // 2 (f - lo) / (hi - lo) - 1 in FP64, then to FP32, as the host normalisation
        const float v = (float)(2.0 * (f[q] - A.lo[q]) / (A.hi[q] - A.lo[q]) - 1.0);
        const __nv_bfloat16 h = __float2bfloat16(v);
        row[q] = h;
        row[7 + q] = __float2bfloat16(v - __bfloat162float(h));
    }
    row[14] = row[15] = __float2bfloat16(0.f);
}

// y (the network's normalised price) times sqrt(bs^2 + floor^2), bs the Black-Scholes call
// (S = 1, r = q = 0) at the expected average Heston variance over [0, T]
__global__ void lattice_scale_kernel(const LatticeArgs A, const float* __restrict__ y, float* __restrict__ price)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.n) return;
    double f[7];
    lattice_cell(A, c, f);
    const double lm = f[0], T = f[1], kappa = f[2], theta = f[3], v0 = f[6];
    const double kt = kappa * T;
    const double var = theta + (v0 - theta) * (1.0 - exp(-kt)) / kt;
    const double sd = sqrt(fmax(var, 1e-8) * T);
    const double d1 = -lm / sd + 0.5 * sd;
    const double bs = normcdf(d1) - exp(lm) * normcdf(d1 - sd);
    price[c] = (float)((double)y[c] * sqrt(bs * bs + A.floor * A.floor));
}

cudaError_t lattice_features(const LatticeArgs& A, __nv_bfloat16* x, cudaStream_t st)
{
    lattice_features_kernel<<<(unsigned)((A.n + 255) / 256), 256, 0, st>>>(A, x);
    return cudaGetLastError();
}

cudaError_t lattice_scale(const LatticeArgs& A, const float* y, float* price, cudaStream_t st)
{
    lattice_scale_kernel<<<(unsigned)((A.n + 255) / 256), 256, 0, st>>>(A, y, price);
    return cudaGetLastError();
}

} // namespace thoth
