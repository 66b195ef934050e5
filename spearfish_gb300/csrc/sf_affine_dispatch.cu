// Dispatcher over the banded affine kernel classes (one translation unit per class).
#include "sf_internal.cuh"

namespace sfk {

cudaError_t launch_affine_regs_4(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_6(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_8(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_9(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_10(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_11(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_12(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_14(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_16(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_20(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_24(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_28(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_32(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_40(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_48(bool, bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_wide(bool, bool, const AffLaunch&, int, int, cudaStream_t);

const int kAffineC[] = {4, 6, 8, 9, 10, 11, 12, 14, 16, 20, 24, 28, 32, 40, 48};
const int kAffineNC = 15;

cudaError_t launch_affine(int c, bool wide, bool tb, bool local, const AffLaunch& a, int grid,
                          int block, cudaStream_t s) {
  if (wide) return launch_affine_wide(tb, local, a, grid, block, s);
  switch (c) {
    case 4: return launch_affine_regs_4(tb, local, a, grid, block, s);
    case 6: return launch_affine_regs_6(tb, local, a, grid, block, s);
    case 8: return launch_affine_regs_8(tb, local, a, grid, block, s);
    case 9: return launch_affine_regs_9(tb, local, a, grid, block, s);
    case 10: return launch_affine_regs_10(tb, local, a, grid, block, s);
    case 11: return launch_affine_regs_11(tb, local, a, grid, block, s);
    case 12: return launch_affine_regs_12(tb, local, a, grid, block, s);
    case 14: return launch_affine_regs_14(tb, local, a, grid, block, s);
    case 16: return launch_affine_regs_16(tb, local, a, grid, block, s);
    case 20: return launch_affine_regs_20(tb, local, a, grid, block, s);
    case 24: return launch_affine_regs_24(tb, local, a, grid, block, s);
    case 28: return launch_affine_regs_28(tb, local, a, grid, block, s);
    case 32: return launch_affine_regs_32(tb, local, a, grid, block, s);
    case 40: return launch_affine_regs_40(tb, local, a, grid, block, s);
    case 48: return launch_affine_regs_48(tb, local, a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sfk
