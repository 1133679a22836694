// book_gbm.cu — book kernel instantiations for GBM books (per-step and uniform constants), in every launch shape.
#include "book.cuh"

namespace thoth {

int book_dispatch_gbm(const DevPlan* P, bool uniform, int shape, int grid, size_t smem, cudaStream_t st,
                      cudaError_t* err)
{
    return uniform ? single_t<M_GBM, true>(P, shape, grid, smem, st, err)
                   : single_t<M_GBM, false>(P, shape, grid, smem, st, err);
}

} // namespace thoth
