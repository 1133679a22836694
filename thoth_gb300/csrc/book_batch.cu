// book_batch.cu — the persistent batch kernel (batch_kernel in book.cuh): the
// single-asset books of a ragged batch, every model, in one launch of the
// (8, 2) shape (256 paths a tile, two paths a thread, 128 threads a CTA).
#include "book.cuh"

namespace thoth {

constexpr int BATCH_TB = 8, BATCH_PP = 2;

static cudaError_t batch_attr()
{
    // once: allow the device's opt-in maximum of dynamic shared memory
    static bool done = false;
    if (done) return cudaSuccess;
    int dev = 0, mx = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, batch_kernel<BATCH_TB, BATCH_PP>);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_kernel<BATCH_TB, BATCH_PP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 mx - (int)fa.sharedSizeBytes);
    done = e == cudaSuccess;
    return e;
}

int batch_threads() { return (1 << BATCH_TB) / BATCH_PP; }
int batch_tile_paths() { return 1 << BATCH_TB; }

// resident CTAs per SM of the batch kernel with smem bytes of dynamic shared memory (0 on error)
int batch_occupancy(size_t smem)
{
    if (batch_attr() != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<BATCH_TB, BATCH_PP>, batch_threads(), smem) !=
        cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_batch_kernel(const DevPlan* plans, const BatchBook* books, int n_books, int n_items, int* next,
                                int grid, size_t smem, cudaStream_t st)
{
    cudaError_t e = batch_attr();
    if (e != cudaSuccess) return e;
    batch_kernel<BATCH_TB, BATCH_PP><<<grid, batch_threads(), smem, st>>>(plans, books, n_books, n_items, next);
    return cudaGetLastError();
}

} // namespace thoth
