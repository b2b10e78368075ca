// Test helper: words of cuRAND's Philox4_32_10 generator, used only to
// cross-check the project's own Philox4x32-10 on the GPU.
#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <stdint.h>

__global__ void words_kernel(unsigned long long seed, unsigned long long subseq, int nblocks, uint4* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  curandStatePhilox4_32_10_t st;
  curand_init(seed, subseq, 0ull, &st);
  for (int i = 0; i < nblocks; ++i) out[i] = curand4(&st);
}

extern "C" int curand_philox_words(unsigned long long seed, unsigned long long subseq, int nblocks,
                                   uint32_t* host_out) {
  uint4* d = nullptr;
  if (cudaMalloc(&d, sizeof(uint4) * nblocks) != cudaSuccess) return -1;
  words_kernel<<<1, 32>>>(seed, subseq, nblocks, d);
  cudaError_t e = cudaMemcpy(host_out, d, sizeof(uint4) * nblocks, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : -2;
}
