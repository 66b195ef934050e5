// Packed 16-bit banded affine kernels with C = 56 cells per lane (28 words; bands up to 1792 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_56(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<28>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_56(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<28>(a, grid, block, s);
}
}  // namespace sfk
