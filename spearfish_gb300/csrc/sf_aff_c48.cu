// Register-row banded affine kernels with C = 48 cells per lane (bands up to 1536 cells).
#include "sf_affine_impl.cuh"

namespace sfk {
cudaError_t launch_affine_regs_48(bool tb, bool local, const AffLaunch& a, int grid, int block,
                                  cudaStream_t s) {
  return launch_affine_c<48, false>(tb, local, a, grid, block, s);
}
}  // namespace sfk
