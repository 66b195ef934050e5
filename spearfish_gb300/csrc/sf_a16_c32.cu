// Packed 16-bit banded affine kernels with C = 32 cells per lane (16 words; bands up to 1024 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_32(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<16>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_32(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<16>(a, grid, block, s);
}
}  // namespace sfk
