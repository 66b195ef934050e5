// Dispatcher over the packed 16-bit banded affine kernel classes (one translation unit each).
#include "sf_internal.cuh"

namespace sfk {

cudaError_t launch_affine16_4(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_6(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_8(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_10(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_12(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_14(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_16(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_20(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_24(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_28(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_32(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_40(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_48(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_56(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_64(bool, const AffLaunch&, int, int, cudaStream_t);

const int kAffine16C[] = {4, 6, 8, 10, 12, 14, 16, 20, 24, 28, 32, 40, 48, 56, 64};
const int kAffine16NC = 15;

cudaError_t launch_affine16(int c, bool tb, const AffLaunch& a, int grid, int block,
                            cudaStream_t s) {
  switch (c) {
    case 4: return launch_affine16_4(tb, a, grid, block, s);
    case 6: return launch_affine16_6(tb, a, grid, block, s);
    case 8: return launch_affine16_8(tb, a, grid, block, s);
    case 10: return launch_affine16_10(tb, a, grid, block, s);
    case 12: return launch_affine16_12(tb, a, grid, block, s);
    case 14: return launch_affine16_14(tb, a, grid, block, s);
    case 16: return launch_affine16_16(tb, a, grid, block, s);
    case 20: return launch_affine16_20(tb, a, grid, block, s);
    case 24: return launch_affine16_24(tb, a, grid, block, s);
    case 28: return launch_affine16_28(tb, a, grid, block, s);
    case 32: return launch_affine16_32(tb, a, grid, block, s);
    case 40: return launch_affine16_40(tb, a, grid, block, s);
    case 48: return launch_affine16_48(tb, a, grid, block, s);
    case 56: return launch_affine16_56(tb, a, grid, block, s);
    case 64: return launch_affine16_64(tb, a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_affine16h_8(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_10(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_12(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_14(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_16(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_18(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_20(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16h_24(bool, const AffLaunch&, int, int, cudaStream_t);

const int kAffine16HC[] = {8, 10, 12, 14, 16, 18, 20, 24};
const int kAffine16HNC = 8;

cudaError_t launch_affine16h(int c, bool tb, const AffLaunch& a, int grid, int block,
                             cudaStream_t s) {
  switch (c) {
    case 8: return launch_affine16h_8(tb, a, grid, block, s);
    case 10: return launch_affine16h_10(tb, a, grid, block, s);
    case 12: return launch_affine16h_12(tb, a, grid, block, s);
    case 14: return launch_affine16h_14(tb, a, grid, block, s);
    case 16: return launch_affine16h_16(tb, a, grid, block, s);
    case 18: return launch_affine16h_18(tb, a, grid, block, s);
    case 20: return launch_affine16h_20(tb, a, grid, block, s);
    case 24: return launch_affine16h_24(tb, a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_affine16w_12(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16w_16(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16w_20(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16w_24(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16w_28(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16w_32(bool, const AffLaunch&, int, int, cudaStream_t);

const int kAffine16WC[] = {12, 16, 20, 24, 28, 32};
const int kAffine16WNC = 6;

cudaError_t launch_affine16w(int c, bool tb, const AffLaunch& a, int grid, int block,
                             cudaStream_t s) {
  switch (c) {
    case 12: return launch_affine16w_12(tb, a, grid, block, s);
    case 16: return launch_affine16w_16(tb, a, grid, block, s);
    case 20: return launch_affine16w_20(tb, a, grid, block, s);
    case 24: return launch_affine16w_24(tb, a, grid, block, s);
    case 28: return launch_affine16w_28(tb, a, grid, block, s);
    case 32: return launch_affine16w_32(tb, a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_affine16_chain_4(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_6(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_8(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_10(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_12(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_14(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_16(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_20(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_24(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_28(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_32(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_40(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_48(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_56(const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine16_chain_64(const AffLaunch&, int, int, cudaStream_t);

cudaError_t launch_affine16_chain(int c, const AffLaunch& a, int grid, int block,
                                  cudaStream_t s) {
  switch (c) {
    case 4: return launch_affine16_chain_4(a, grid, block, s);
    case 6: return launch_affine16_chain_6(a, grid, block, s);
    case 8: return launch_affine16_chain_8(a, grid, block, s);
    case 10: return launch_affine16_chain_10(a, grid, block, s);
    case 12: return launch_affine16_chain_12(a, grid, block, s);
    case 14: return launch_affine16_chain_14(a, grid, block, s);
    case 16: return launch_affine16_chain_16(a, grid, block, s);
    case 20: return launch_affine16_chain_20(a, grid, block, s);
    case 24: return launch_affine16_chain_24(a, grid, block, s);
    case 28: return launch_affine16_chain_28(a, grid, block, s);
    case 32: return launch_affine16_chain_32(a, grid, block, s);
    case 40: return launch_affine16_chain_40(a, grid, block, s);
    case 48: return launch_affine16_chain_48(a, grid, block, s);
    case 56: return launch_affine16_chain_56(a, grid, block, s);
    case 64: return launch_affine16_chain_64(a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sfk
