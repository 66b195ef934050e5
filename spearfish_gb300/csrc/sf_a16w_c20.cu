// Two-warp packed 16-bit banded affine kernels: 64 lanes a pass, C = 20 cells per lane
// (10 words; bands up to 1280 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16w_20(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16w_c<10>(tb, a, grid, block, s);
}
}  // namespace sfk
