// book_heston.cu — book kernel instantiations for single-asset Heston books (per-step and uniform constants), in every launch shape.
#include "book.cuh"

namespace thoth {

int book_dispatch_heston(const DevPlan* P, bool uniform, int shape, int grid, size_t smem, cudaStream_t st,
                         cudaError_t* err)
{
    return uniform ? single_t<M_HESTON, true>(P, shape, grid, smem, st, err)
                   : single_t<M_HESTON, false>(P, shape, grid, smem, st, err);
}

} // namespace thoth
