// Mixed-precision batched refinement, size bin of orders <= 128 (row tile 8 x 16).
#include "refine_bin_impl.cuh"

namespace gsk {
template cudaError_t launch_refine_bin<8>(const RefineArgs&, int, int, int, cudaStream_t);
}  // namespace gsk
