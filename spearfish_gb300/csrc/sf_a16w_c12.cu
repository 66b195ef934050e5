// Two-warp packed 16-bit banded affine kernels: 64 lanes a pass, C = 12 cells per lane
// (6 words; bands up to 768 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16w_12(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16w_c<6>(tb, a, grid, block, s);
}
}  // namespace sfk
