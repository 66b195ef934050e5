// Packed 16-bit banded affine kernels with C = 6 cells per lane (3 words; bands up to 192 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_6(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<3>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_6(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<3>(a, grid, block, s);
}
}  // namespace sfk
