// Packed 16-bit banded affine kernels with C = 48 cells per lane (24 words; bands up to 1536 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_48(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<24>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_48(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<24>(a, grid, block, s);
}
}  // namespace sfk
