// Packed 16-bit banded affine kernels with C = 24 cells per lane (12 words; bands up to 768 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_24(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<12>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_24(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<12>(a, grid, block, s);
}
}  // namespace sfk
