// book_lsv.cu — book kernel instantiations for single-asset LSV books, in every launch shape.
#include "book.cuh"

namespace thoth {

int book_dispatch_lsv(const DevPlan* P, int shape, int grid, size_t smem, cudaStream_t st, cudaError_t* err)
{
    return single_t<M_LSV, false>(P, shape, grid, smem, st, err);
}

} // namespace thoth
