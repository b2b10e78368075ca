// Bit-exact check of abc::rn32_bits (FP64 -> FP32 rounding on the bit fields)
// against the conversion instruction on the device.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../abc_inference_transcription_gb300/csrc/distance.cuh"

__device__ __forceinline__ uint64_t mix64r(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void rn32_check_kernel(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                                  unsigned long long* first) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint64_t b = mix64r(i ^ seed);
    if ((i & 3) == 1)  // exponents of the normal float range and just outside it
      b = (b & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(890 + mix64r(i ^ 77) % 268) << 52);
    if ((i & 7) == 2)  // ties and near-ties at the rounding position
      b = (b & ~0x1FFFFFFFull) | 0x10000000ull | ((mix64r(i ^ 5) & 1) ? 0x1ull : 0ull);
    const double x = __longlong_as_double((long long)b);
    const float a = abc::rn32_bits(x), c = (float)x;
    if (__float_as_uint(a) != __float_as_uint(c) && !(a != a && c != c))
      if (atomicAdd(bad, 1ull) == 0ull) *first = b;
  }
}

extern "C" int rn32_check(unsigned long long n, unsigned long long seed, unsigned long long* bad_out,
                          unsigned long long* first_out) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  rn32_check_kernel<<<4096, 256>>>(n, seed, d, d + 1);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(bad_out, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(first_out, d + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : 1;
}
