// Packed 16-bit banded affine kernels with C = 64 cells per lane (32 words; bands up to 2048 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_64(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<32>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_64(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<32>(a, grid, block, s);
}
}  // namespace sfk
