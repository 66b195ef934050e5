// Register-row banded affine kernels with C = 9 cells per lane (bands up to 288 cells).
#include "sf_affine_impl.cuh"

namespace sfk {
cudaError_t launch_affine_regs_9(bool tb, bool local, const AffLaunch& a, int grid, int block,
                                  cudaStream_t s) {
  return launch_affine_c<9, false>(tb, local, a, grid, block, s);
}
}  // namespace sfk
