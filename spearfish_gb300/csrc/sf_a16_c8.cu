// Packed 16-bit banded affine kernels with C = 8 cells per lane (4 words; bands up to 256 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_8(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<4>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_8(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<4>(a, grid, block, s);
}
}  // namespace sfk
