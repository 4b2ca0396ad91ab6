// Mixed-precision batched refinement, size bin of orders <= 32 (row tile 2 x 16).
#include "refine_bin_impl.cuh"

namespace gsk {
template cudaError_t launch_refine_bin<2>(const RefineArgs&, int, int, int, cudaStream_t);
}  // namespace gsk
