// Two-warp packed 16-bit banded affine kernels: 64 lanes a pass, C = 28 cells per lane
// (14 words; bands up to 1792 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16w_28(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16w_c<14>(tb, a, grid, block, s);
}
}  // namespace sfk
