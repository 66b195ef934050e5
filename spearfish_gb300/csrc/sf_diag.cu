// INT32 throughput probe for the roofline of the DP kernels.  The banded Gotoh and Myers
// kernels are bound by the integer ALU pipes, not HBM and not tensor cores; no integer peak
// is published for GB300, so it is measured: independent chains of x = max(x + c, y) --
// the add-then-max that dominates a DP cell -- counted as two int32 ops each.
#include "sf_internal.cuh"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) int_peak_kernel(int32_t* out, int32_t seed) {
  int32_t x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = seed + (int32_t)(threadIdx.x * 7 + c * 13);
  const int32_t k1 = seed & 3, k2 = -(seed & 5);
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = max(x[c] + k1, x[(c + 1) % kChains] + k2);
  }
  int32_t s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s ^= x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

namespace sfk {

cudaError_t run_int_peak(int sms, int32_t* out, float* ms, uint64_t* ops) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int grid = sms * 8, block = 256;
  cudaEventRecord(a, 0);
  int_peak_kernel<<<grid, block>>>(out, 1);
  cudaEventRecord(b, 0);
  cudaError_t e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventElapsedTime(ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  // Per chain step: one add and one max of the chain value, plus the neighbour's add.
  *ops = (uint64_t)grid * block * kIters * kChains * 3;
  return e;
}

}  // namespace sfk
