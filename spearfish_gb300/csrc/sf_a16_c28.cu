// Packed 16-bit banded affine kernels with C = 28 cells per lane (14 words; bands up to 896 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_28(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<14>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_28(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<14>(a, grid, block, s);
}
}  // namespace sfk
