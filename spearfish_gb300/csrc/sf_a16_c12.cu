// Packed 16-bit banded affine kernels with C = 12 cells per lane (6 words; bands up to 384 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_12(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<6>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_12(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<6>(a, grid, block, s);
}
}  // namespace sfk
