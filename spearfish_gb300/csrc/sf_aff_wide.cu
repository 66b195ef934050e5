// Wide-row banded affine kernels: rows of any width in global scratch, 32 * kWideC offsets
// per chunk (unbanded Infix passes, bands wider than the register kernels hold).
#include "sf_affine_impl.cuh"

namespace sfk {
cudaError_t launch_affine_wide(bool tb, bool local, const AffLaunch& a, int grid, int block,
                               cudaStream_t s) {
  return launch_affine_c<kWideC, true>(tb, local, a, grid, block, s);
}
}  // namespace sfk
