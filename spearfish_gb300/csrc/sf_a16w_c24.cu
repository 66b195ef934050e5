// Two-warp packed 16-bit banded affine kernels: 64 lanes a pass, C = 24 cells per lane
// (12 words; bands up to 1536 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16w_24(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16w_c<12>(tb, a, grid, block, s);
}
}  // namespace sfk
