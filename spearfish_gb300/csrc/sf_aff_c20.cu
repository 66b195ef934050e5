// Register-row banded affine kernels with C = 20 cells per lane (bands up to 640 cells).
#include "sf_affine_impl.cuh"

namespace sfk {
cudaError_t launch_affine_regs_20(bool tb, bool local, const AffLaunch& a, int grid, int block,
                                  cudaStream_t s) {
  return launch_affine_c<20, false>(tb, local, a, grid, block, s);
}
}  // namespace sfk
