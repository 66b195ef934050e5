// Packed 16-bit banded affine kernels with C = 10 cells per lane (5 words; bands up to 320 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_10(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<5>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_10(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<5>(a, grid, block, s);
}
}  // namespace sfk
