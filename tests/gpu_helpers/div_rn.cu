// Bit-exact check of abc::div_rn (three-operation division from a correctly
// rounded reciprocal) against the IEEE division a / b on the device.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../abc_inference_transcription_gb300/csrc/distance.cuh"

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// value with the given 52-bit mantissa field and unbiased exponent
__device__ __forceinline__ double make(uint64_t mant, int ex) {
  return __longlong_as_double((long long)(((uint64_t)(ex + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

__global__ void div_check_kernel(uint64_t n, uint64_t seed, unsigned long long* bad, double* first) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed ^ (2 * i)), h2 = mix64(seed ^ (2 * i + 1)), h3 = mix64(h1 ^ h2);
    const int ea = (int)(h3 % 121) - 60, eb = (int)((h3 >> 8) % 41) - 20;
    double a = make(h1, ea), b = make(h2, eb);
    switch (i & 7) {
      case 1: b = make(~0ull, eb); break;                      // divisor significand all ones
      case 2: a = make(~0ull, ea); break;                      // dividend significand all ones
      case 3: b = make(0, eb); break;                          // power of two
      case 4: a = a * a; break;                                // squares, as (d - s)^2
      case 5: b = make(h2 >> 40, 0); break;                    // near one
      case 6: a = make(h1 & 0xF000000000000ull, ea); b = make(h2 & 0xFF00000000000ull, eb); break;
      case 7: a = b * (double)((h1 % 1000) + 1); break;        // exact quotients
      default: break;
    }
    if ((i & 63) == 9) a = make(h1, (int)(h3 % 1800) - 900);   // wide exponent range, both paths
    const double y = 1.0 / b;
    const double q = abc::div_rn(a, b, y);
    const double want = a / b;
    if (__double_as_longlong(q) != __double_as_longlong(want)) {
      if (atomicAdd(bad, 1ull) == 0ull) {
        first[0] = a;
        first[1] = b;
        first[2] = q;
        first[3] = want;
      }
    }
  }
}

extern "C" int div_rn_check(unsigned long long n, unsigned long long seed, unsigned long long* bad_out,
                            double* first_out) {
  unsigned long long* d_bad = nullptr;
  double* d_first = nullptr;
  if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess) return 1;
  if (cudaMalloc(&d_first, 4 * sizeof(double)) != cudaSuccess) return 1;
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  cudaMemset(d_first, 0, 4 * sizeof(double));
  div_check_kernel<<<4096, 256>>>(n, seed, d_bad, d_first);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(bad_out, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(first_out, d_first, 4 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d_bad);
  cudaFree(d_first);
  return e == cudaSuccess ? 0 : 2;
}
