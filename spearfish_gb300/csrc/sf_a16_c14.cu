// Packed 16-bit banded affine kernels with C = 14 cells per lane (7 words; bands up to 448 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_14(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<7>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_14(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<7>(a, grid, block, s);
}
}  // namespace sfk
