// book_multi.cu — book kernel instantiations for multi-asset books: correlated GBM names together (variant 3), independent assets one per pass (variant 6), in every launch shape.
#include "book.cuh"

namespace thoth {

int book_dispatch_multi(const DevPlan* P, int variant, int shape, int grid, size_t smem, cudaStream_t st,
                        cudaError_t* err)
{
    if (variant == 3) {
        if (grid) *err = launch_book_t<7, MAX_ASSETS, M_MIXED, false, 1>(*P, grid, smem, st);
        return grid ? 0 : occ_t<7, MAX_ASSETS, M_MIXED, false, 1>(smem);
    }
    return single_t<M_SEQ, false>(P, shape, grid, smem, st, err);
}

} // namespace thoth
