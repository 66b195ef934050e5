// Packed 16-bit banded affine kernels with C = 20 cells per lane (10 words; bands up to 640 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_20(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<10>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_20(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<10>(a, grid, block, s);
}
}  // namespace sfk
