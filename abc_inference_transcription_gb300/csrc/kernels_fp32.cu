// kernels_fp32.cu — production SSA: FP32 propensities, waiting times and
// channel selection with fast intrinsics; FP64 clock.  Built with FMA
// contraction on.
#include "kernels.h"

namespace abc {

cudaError_t launch_ssa_fp32(const SsaArgs& a, int grid, cudaStream_t s) {
  ssa_kernel<false><<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

int ssa_blocks_per_sm_fp32() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_kernel<false>, 128, 0);
  return n;
}

}  // namespace abc
