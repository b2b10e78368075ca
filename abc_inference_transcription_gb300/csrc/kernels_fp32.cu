// kernels_fp32.cu — production SSA launch: FP32 propensities, waiting times
// and channel selection with fast intrinsics; compensated FP32 interval clock
// re-anchored at every breakpoint (integer breakpoint grid, or FP64 when the
// configuration's times are not on one).  Built with FMA contraction on.
#include "kernels.h"
#include "ssa_fp32.cuh"

namespace abc {

// Kernel variants the autotuner chooses from: register allocation for 8 or
// 10 resident blocks of 128 threads per SM.
static const int kVariantMinBlocks[kSsaVariants] = {8, 10};

template <bool SPLICE, bool GRID, bool GENSCAL>
static cudaError_t launch_variant(const SsaArgs& b, int variant, int grid, cudaStream_t s) {
  if (variant == 1)
    ssa_kernel_f32<SPLICE, 10, GRID, GENSCAL><<<grid, 128, 0, s>>>(b);
  else
    ssa_kernel_f32<SPLICE, 8, GRID, GENSCAL><<<grid, 128, 0, s>>>(b);
  return cudaGetLastError();
}

template <bool SPLICE, bool GRID>
static cudaError_t launch_scal(const SsaArgs& b, int variant, int grid, cudaStream_t s) {
  // a scaling column in theta gives each particle its own size exponent;
  // without one the exponent is 0 or 1 and the rate is linear in time
  return b.cfg.scaling_column ? launch_variant<SPLICE, GRID, true>(b, variant, grid, s)
                              : launch_variant<SPLICE, GRID, false>(b, variant, grid, s);
}

cudaError_t launch_ssa_fp32(const SsaArgs& a, int grid, cudaStream_t s, int variant) {
  SsaArgs b = a;
  uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
  for (int r = 0; r < 10; ++r) {
    b.rk[2 * r] = k0;
    b.rk[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  // integer breakpoints when the configuration's times lie on a power-of-two grid
  if (a.cfg.grid_ok)
    return a.cfg.splicing ? launch_scal<true, true>(b, variant, grid, s) : launch_scal<false, true>(b, variant, grid, s);
  return a.cfg.splicing ? launch_scal<true, false>(b, variant, grid, s) : launch_scal<false, false>(b, variant, grid, s);
}

int ssa_blocks_per_sm_fp32(int variant) {
  int n = 0;
  if (variant == 1)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_kernel_f32<false, 10, true, false>, 128, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_kernel_f32<false, 8, true, false>, 128, 0);
  return n > 0 ? n : kVariantMinBlocks[variant < 0 || variant >= kSsaVariants ? 0 : variant];
}

// ---------------------------------------------------------------------------
// Work order: particles by expected fired events per trajectory, heaviest
// first (longest-processing-time-first), so the long trajectories start early
// and the end of the persistent kernel is filled with short ones.  64 buckets
// on log2(cost), counting sort; order inside a bucket is arbitrary (it only
// affects scheduling, never results: random streams are keyed by particle).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cost_bucket(double cost) {
  const int e = (int)((__double_as_longlong(cost) >> 52) & 0x7ff) - 1023;
  const int b = e < 0 ? 0 : (e > 63 ? 63 : e);
  return 63 - b;
}

__global__ void order_hist_kernel(const PRec* rec, int64_t P, unsigned int* hist) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&hist[cost_bucket(rec[p].cost)], 1u);
}

__global__ void order_scatter_kernel(const PRec* rec, int64_t P, const unsigned int* hist, unsigned int* cursor,
                                     uint32_t* order) {
  __shared__ unsigned int start[64];
  if (threadIdx.x == 0) {
    unsigned int run = 0;
    for (int b = 0; b < 64; ++b) {
      start[b] = run;
      run += hist[b];
    }
  }
  __syncthreads();
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    const int b = cost_bucket(rec[p].cost);
    order[start[b] + atomicAdd(&cursor[b], 1u)] = (uint32_t)p;
  }
}

cudaError_t launch_work_order(const PRec* rec, int64_t P, unsigned int* hist128, uint32_t* order, cudaStream_t s) {
  if (P <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(hist128, 0, 128 * sizeof(unsigned int), s);
  if (e) return e;
  const int blocks = (int)((P + 255) / 256 < 4096 ? (P + 255) / 256 : 4096);
  order_hist_kernel<<<blocks, 256, 0, s>>>(rec, P, hist128);
  order_scatter_kernel<<<blocks, 256, 0, s>>>(rec, P, hist128, hist128 + 64, order);
  return cudaGetLastError();
}

}  // namespace abc
