// Packed 16-bit banded affine kernels with C = 16 cells per lane (8 words; bands up to 512 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_16(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<8>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_16(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<8>(a, grid, block, s);
}
}  // namespace sfk
