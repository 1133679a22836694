// TEST INFRASTRUCTURE (benchmark only): the reference's own GPU Monte-Carlo kernel,
// pricer/src/tasks/mcl_gpu.cu (gbm_kernel, lines 25-70, and gpu::PriceEuropeanGbm,
// lines 100-154), compiled unmodified for sm_103a and timed beside this engine.
//
// The reference file is included as a whole, so its kernel, which lives in an anonymous
// namespace, is visible here. oracle/Makefile stages the file and its header from the
// reference checkout into oracle/_ref/gpu/ (never committed); this file only adds timing:
//   ref_gbm_call     the reference's public call PriceEuropeanGbm, host wall time
//                    (its allocations, launch, synchronisation and copies included);
//   ref_gbm_kernel   gbm_kernel alone, launched with the grid the reference's call uses
//                    (SMs x 32 blocks of 256 threads), timed by CUDA events on its stream.
#include "mcl_gpu.cu"

#include <chrono>

extern "C" {

int ref_gbm_call(double forward, double strike, double t, double vol, double df, int is_call, long paths,
                 unsigned long seed, double* premium, double* trust, double* wall_ms)
{
    const auto t0 = std::chrono::steady_clock::now();
    const gpu::GbmResult r = gpu::PriceEuropeanGbm(forward, strike, t, vol, df, is_call != 0, paths, seed);
    const auto t1 = std::chrono::steady_clock::now();
    *premium = r.premium;
    *trust = r.trust;
    *wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int ref_gbm_kernel(double forward, double strike, double t, double vol, double df, int is_call, long paths,
                   unsigned long seed, int reps, double* premium, double* trust, double* kernel_ms)
{
    if (paths <= 0 || reps < 1) return -1;
    const double a = -0.5 * vol * vol * t, b = vol * sqrt(t);
    int device = 0;
    cudaGetDevice(&device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -3;
    const int blocks = prop.multiProcessorCount * 32;
    double* d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(double)) != cudaSuccess) return -6;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float total = 0.f;
    double h[2] = {0, 0};
    for (int k = 0; k < reps; k++) {
        cudaMemset(d, 0, 2 * sizeof(double));
        cudaEventRecord(e0);
        gbm_kernel<<<blocks, BLOCK>>>(forward, strike, a, b, is_call ? 1 : 0, paths, seed, d, d + 1);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
    }
    cudaMemcpy(h, d, 2 * sizeof(double), cudaMemcpyDeviceToHost);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    const double n = (double)paths, mean = h[0] / n;
    const double var = fmax(h[1] / n - mean * mean, 0.0);
    *premium = df * mean;
    *trust = df * sqrt(var / n);
    *kernel_ms = total / reps;
    return err == cudaSuccess ? 0 : -3;
}

} // extern "C"
