// Mixed-precision batched refinement, size bin of orders <= 64 (row tile 4 x 16).
#include "refine_bin_impl.cuh"

namespace gsk {
template cudaError_t launch_refine_bin<4>(const RefineArgs&, int, int, int, cudaStream_t);
}  // namespace gsk
