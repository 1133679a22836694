// kernels.cu — sm_103a kernels of the Monte-Carlo engine (see engine.cuh) other
// than the book kernel itself (book.cuh): the fixed-order reduction, the Sobol
// low-word gather, test hooks, peak microbenchmarks and the book launch dispatch.
#include "book.cuh"

#include <cuda_runtime.h>

namespace thoth {

// fixed-order FP64 reduction of the per-CTA rows
// (32 columns per CTA; row group g of REDUCE_GROUPS sums rows g, g + GROUPS, ...
// in order, then the group sums are added in group order: the same order on
// every run, whatever the scheduling)
constexpr int REDUCE_GROUPS = 16;
__global__ void __launch_bounds__(32 * REDUCE_GROUPS)
    reduce_rows(const double* __restrict__ acc, int rows, int n_acc, double* __restrict__ out)
{
    __shared__ double part[REDUCE_GROUPS][33];
    const int c = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + c;
    double s = 0.0;
    if (j < n_acc)
        for (int r = g; r < rows; r += REDUCE_GROUPS) s += acc[(size_t)r * n_acc + j];
    part[g][c] = s;
    __syncthreads();
    if (g == 0 && j < n_acc) {
        double t = 0.0;
        for (int k = 0; k < REDUCE_GROUPS; ++k) t += part[k][c];
        out[j] = t;
    }
}

// the same reduction for every book of a batch at once: block (x, y) sums columns
// 32 x .. 32 x + 31 of book y's rows
__global__ void __launch_bounds__(32 * REDUCE_GROUPS) reduce_rows_batch(const BatchReduce* __restrict__ jobs)
{
    __shared__ double part[REDUCE_GROUPS][33];
    const BatchReduce J = jobs[blockIdx.y];
    if ((int)blockIdx.x * 32 >= J.n_acc) return; // uniform over the block
    const int c = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + c;
    double s = 0.0;
    if (j < J.n_acc)
        for (int r = g; r < J.rows; r += REDUCE_GROUPS) s += J.acc[(size_t)r * J.n_acc + j];
    part[g][c] = s;
    __syncthreads();
    if (g == 0 && j < J.n_acc) {
        double t = 0.0;
        for (int k = 0; k < REDUCE_GROUPS; ++k) t += part[k][c];
        J.out[j] = t;
    }
}

cudaError_t launch_reduce_batch(const void* jobs, int n_books, int max_acc, cudaStream_t st)
{
    if (n_books == 0) return cudaSuccess;
    const dim3 grid((unsigned)((max_acc + 31) / 32), (unsigned)n_books);
    reduce_rows_batch<<<grid, 32 * REDUCE_GROUPS, 0, st>>>(reinterpret_cast<const BatchReduce*>(jobs));
    return cudaGetLastError();
}

// the book's low Sobol words in consumption order: out[j][t] = lo_all[order[j]][t]
__global__ void gather_low_kernel(const uint32_t* __restrict__ lo_all, const int* __restrict__ order, int n, int T,
                                  uint32_t* __restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * T) return;
    const int j = (int)(i / T), t = (int)(i % T);
    out[i] = __ldg(lo_all + (size_t)__ldg(order + j) * SOBOL_LO_ROW + t);
}

cudaError_t launch_gather_low(const uint32_t* lo_all, const int* order, int n, int T, uint32_t* out, cudaStream_t st)
{
    const int64_t total = (int64_t)n * T;
    if (total == 0) return cudaSuccess;
    gather_low_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(lo_all, order, n, T, out);
    return cudaGetLastError();
}

// the same gather for every book of a batch at once: blocks (., y) stride over book y's words
constexpr int GATHER_BATCH_BLOCKS = 32;

__global__ void __launch_bounds__(256) gather_low_batch_kernel(const uint32_t* __restrict__ lo_all,
                                                               const BatchGather* __restrict__ jobs)
{
    const BatchGather J = jobs[blockIdx.y];
    const int64_t total = (int64_t)J.n * J.T;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / J.T), t = (int)(i % J.T);
        J.out[i] = __ldg(lo_all + (size_t)__ldg(J.order + j) * SOBOL_LO_ROW + t);
    }
}

cudaError_t launch_gather_low_batch(const uint32_t* lo_all, const void* jobs, int n_books, cudaStream_t st)
{
    if (n_books == 0) return cudaSuccess;
    gather_low_batch_kernel<<<dim3(GATHER_BATCH_BLOCKS, (unsigned)n_books), 256, 0, st>>>(
        lo_all, reinterpret_cast<const BatchGather*>(jobs));
    return cudaGetLastError();
}

// ---- test hooks -----------------------------------------------------------
__global__ void sobol_points_kernel(const uint32_t* __restrict__ V, int dims, int64_t skip, int64_t n_points,
                                    uint32_t* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_points * dims) return;
    const int64_t p = idx / dims;
    const int d = (int)(idx % dims);
    const uint64_t nn = (uint64_t)(skip + 1 + p);
    const uint64_t g = nn ^ (nn >> 1);
    uint32_t x = 0;
    for (int k = 0; k < SOBOL_BITS; ++k)
        if ((g >> k) & 1u) x ^= __ldg(V + (size_t)d * SOBOL_BITS + k);
    out[idx] = x;
}

__global__ void quantile_kernel(const uint32_t* __restrict__ x, int64_t n, float* __restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = quantile_u32(x[i]);
}

// writes the bridge increments of every valid path: out[path][factor][N]
template <int TB>
__global__ void __launch_bounds__(1 << TB) bridge_kernel(const DevPlan P, float* __restrict__ out)
{
    constexpr int T = 1 << TB;
    constexpr int NA = 1; // factor slots 0..1 carry reference factors 0..1
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Smem S = carve(smem_raw, P, T);
    const int t = threadIdx.x;
    for (int64_t tile = blockIdx.x; tile < P.n_tiles; tile += gridDim.x) {
        const int64_t m = P.tile_first + tile;
        const uint64_t n[1] = {(uint64_t)m * T + (uint64_t)t};
        const bool valid = n[0] >= (uint64_t)P.skip + 1 && n[0] <= (uint64_t)(P.skip + P.paths);
        __syncthreads();
        tile_high_bits<TB>(P, S.hs, m, 0);
        __syncthreads();
        SobolLane<T, 1> L = sobol_lane<TB, 1>(P, S.hs, m);
        float Wprev[1][2] = {{0.f, 0.f}}, top[1][2] = {{0.f, 0.f}}, nz[1][2];
        int sp = 0;
        const int64_t path = (int64_t)n[0] - P.skip - 1;
        for (int i = 1; i <= P.n_steps; ++i) {
            const StepRec rec = load_rec(P, i);
            bridge_step<NA, T, 1, false>(P, S, rec, sp, L, n, Wprev, top, nz, 0);
            if (valid) {
                for (int f = 0; f < P.n_factors_active; ++f)
                    out[((size_t)path * P.n_factors_active + f) * P.n_steps + (i - 1)] = nz[0][f];
            }
        }
    }
}

// ---- FP32 peak microbenchmark: 8 independent FMA chains per thread ----------
__global__ void __launch_bounds__(256) fma_peak_kernel(float* out, int iters, float a, float b)
{
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fmaf(x0, a, b);
            x1 = fmaf(x1, a, b);
            x2 = fmaf(x2, a, b);
            x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b);
            x5 = fmaf(x5, a, b);
            x6 = fmaf(x6, a, b);
            x7 = fmaf(x7, a, b);
        }
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1.2345f) out[blockIdx.x] = s; // keeps the chains alive
}

cudaError_t launch_fma_peak(float* out, int blocks, int iters, cudaStream_t st)
{
    fma_peak_kernel<<<blocks, 256, 0, st>>>(out, iters, 0.999999f, 1e-7f);
    return cudaGetLastError();
}

// ---- MUFU peak microbenchmark: 8 independent reciprocal-square-root chains per thread ----
// x -> 1 / sqrt(x) keeps every chain positive and finite (it converges to 1); with -ftz each
// rsqrtf is one special-function-unit instruction.
__global__ void __launch_bounds__(256) mufu_peak_kernel(float* out, int iters)
{
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1.0f + (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
#pragma unroll
            for (int k = 0; k < 8; ++k) x[k] = rsqrtf(x[k]);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 1.2345f) out[blockIdx.x] = s; // keeps the chains alive
}

cudaError_t launch_mufu_peak(float* out, int blocks, int iters, cudaStream_t st)
{
    mufu_peak_kernel<<<blocks, 256, 0, st>>>(out, iters);
    return cudaGetLastError();
}

int book_shape_count(int variant) { return variant == 3 ? 1 : N_SHAPES; }
int book_shape_tile_bits(int variant, int shape) { return variant == 3 ? 7 : SHAPE_TB[shape]; }
int book_shape_threads(int variant, int shape) { return variant == 3 ? 128 : (1 << SHAPE_TB[shape]) / SHAPE_PP[shape]; }

static int dispatch(const DevPlan* P, int variant, int shape, int grid, size_t smem, cudaStream_t st, cudaError_t* err)
{
    *err = cudaSuccess;
    if (variant != 3 && (shape < 0 || shape >= N_SHAPES)) {
        *err = cudaErrorInvalidValue;
        return 1;
    }
    switch (variant) {
    case 0: return book_dispatch_gbm(P, false, shape, grid, smem, st, err);
    case 1: return book_dispatch_heston(P, false, shape, grid, smem, st, err);
    case 2: return book_dispatch_lsv(P, shape, grid, smem, st, err);
    case 3: return book_dispatch_multi(P, 3, shape, grid, smem, st, err);
    case 4: return book_dispatch_heston(P, true, shape, grid, smem, st, err);
    case 5: return book_dispatch_gbm(P, true, shape, grid, smem, st, err);
    case 6: return book_dispatch_multi(P, 6, shape, grid, smem, st, err);
    default: *err = cudaErrorInvalidValue; return 1;
    }
}

// variants: 0 GBM, 1 Heston, 2 LSV (single asset, per-step constants),
//           3 mixed multi-asset with correlated GBM names, 4 Heston with uniform steps,
//           5 GBM with uniform steps, 6 multi-asset with independent assets (one pass per asset)
cudaError_t launch_book(const DevPlan& P, int variant, int shape, int grid, size_t smem, cudaStream_t st)
{
    if (grid < 1) return cudaErrorInvalidValue;
    cudaError_t e;
    dispatch(&P, variant, shape, grid, smem, st, &e);
    return e;
}

// resident CTAs per SM of a variant and shape at a given dynamic shared-memory size
int book_occupancy(int variant, int shape, size_t smem)
{
    cudaError_t e;
    const int n = dispatch(nullptr, variant, shape, 0, smem, 0, &e);
    return e == cudaSuccess ? n : 1;
}

size_t book_smem_bytes(int T, int sobol_dims, int stack_depth, int nfa, int n_slots, int n_groups, int n_last,
                       int few_m)
{
    return smem_bytes(T, sobol_dims, stack_depth, nfa, n_slots, n_groups, n_last, few_m);
}

cudaError_t launch_reduce(const double* acc, int rows, int n_acc, double* out, cudaStream_t st)
{
    reduce_rows<<<(n_acc + 31) / 32, 32 * REDUCE_GROUPS, 0, st>>>(acc, rows, n_acc, out);
    return cudaGetLastError();
}

cudaError_t launch_sobol_points(const uint32_t* V, int dims, int64_t skip, int64_t n_points, uint32_t* out,
                                cudaStream_t st)
{
    const int64_t total = n_points * dims;
    if (total == 0) return cudaSuccess;
    sobol_points_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(V, dims, skip, n_points, out);
    return cudaGetLastError();
}

cudaError_t launch_quantile(const uint32_t* x, int64_t n, float* out, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    quantile_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, n, out);
    return cudaGetLastError();
}

cudaError_t launch_bridge(const DevPlan& P, int grid, size_t smem, float* out, cudaStream_t st)
{
    auto k = bridge_kernel<8>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, 256, smem, st>>>(P, out);
    return cudaGetLastError();
}

} // namespace thoth
