// Packed 16-bit banded affine kernels with C = 4 cells per lane (2 words; bands up to 128 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_4(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<2>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_4(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<2>(a, grid, block, s);
}
}  // namespace sfk
