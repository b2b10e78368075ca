// Draws from the production mode's FP32 samplers (sampler32.cuh) and, for
// comparison, the FP64 samplers of common.cuh: one draw per thread, each
// from its own Philox stream (cell = low word, particle = high word of the
// draw index), copied to the caller's host array.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../abc_inference_transcription_gb300/csrc/sampler32.cuh"

namespace {

__global__ void draw_kernel(int kind, long long n, double p, float lam, long long count, unsigned long long seed,
                            long long* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    abc::Rng r;
    abc::rng_init(r, seed, 2u, (uint32_t)i, (uint32_t)(i >> 32));
    long long x = 0;
    if (kind == 0) x = abc::binomial32(r, (int)n, (float)p);
    if (kind == 1) x = abc::binomial(r, n, p);
    if (kind == 2) x = abc::poisson32(r, lam);
    if (kind == 3) x = abc::poisson(r, (double)lam);
    out[i] = x;
  }
}

}  // namespace

// kind: 0 binomial32(n, p), 1 FP64 binomial(n, p), 2 poisson32(lam), 3 FP64 poisson(lam)
extern "C" int sampler_draw(int kind, long long n, double p, float lam, long long count, unsigned long long seed,
                            long long* out_host) {
  long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(long long) * (size_t)count) != cudaSuccess) return 1;
  draw_kernel<<<1024, 256>>>(kind, n, p, lam, count, seed, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out_host, d, sizeof(long long) * (size_t)count, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : 2;
}
