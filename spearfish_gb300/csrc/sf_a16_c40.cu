// Packed 16-bit banded affine kernels with C = 40 cells per lane (20 words; bands up to 1280 cells).
#include "sf_affine16_impl.cuh"

namespace sfk {
cudaError_t launch_affine16_40(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_c<20>(tb, a, grid, block, s);
}
cudaError_t launch_affine16_chain_40(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  return launch_affine16_chain_c<20>(a, grid, block, s);
}
}  // namespace sfk
