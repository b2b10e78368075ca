// datastats.cu — the data side of the distance: the 53 statistics of every
// gene's observed per-cell counts and their bootstrap standard errors
// (scripts/data_summary_statistics.jl:1-216).  Same layout as the simulated
// statistics: [pulse mean (A), pulse FF (A), chase mean (A), chase FF (A),
// ratio (J), mean_corr (J), corr_mean (J)].
//
// One CTA per (gene, resample); resample 0 is the estimate itself, 1..n_boot
// are bootstrap resamples of the cells with replacement, drawn separately for
// the pulse cells, the chase cells and all cells (ratios and correlations), as
// the reference's get_ccp_se / get_ratio_se / get_correlation_se do.  Draw i
// of (gene, resample, family) comes from its own Philox counter, so threads
// draw independently; every statistic is computed from exact integer sums
// (n, sum x, sum x^2, sum u l per group), so the result does not depend on
// the reduction order and is bit-identical to the C oracle.  FP64 formulas
// built with -fmad=false.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "model.cuh"

namespace abc {
namespace {

constexpr int kThreads = 256;

// position in [0, n) of draw i of stream (seed, family, resample, gene):
// floor(x n / 2^52) of a 52-bit uniform integer x, in exact integer arithmetic
__device__ __forceinline__ int64_t draw_pos(uint64_t seed, int fam, int b, int64_t g, int64_t i, int64_t n) {
  U4 c;
  c.x = (uint32_t)(i >> 1);
  c.y = ((uint32_t)((uint64_t)i >> 33) & 0x3fffffffu) | (ST_AUX << 30);
  c.z = (uint32_t)b | ((uint32_t)(fam + 1) << 24);
  c.w = (uint32_t)g;
  const U4 o = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t hi = (i & 1) ? o.z : o.x, lo = (i & 1) ? o.w : o.y;
  const uint64_t x = ((uint64_t)hi << 20) | (uint64_t)(lo >> 12);
  return (int64_t)__umul64hi(x << 12, (uint64_t)n);
}

// exact sample variance / covariance from integer sums: (n sxy - sx sy) / (n (n - 1))
__device__ __forceinline__ double sample_cov(unsigned long long n, unsigned long long sx, unsigned long long sy,
                                             unsigned long long sxy) {
  const __int128 num = (__int128)n * (__int128)sxy - (__int128)sx * (__int128)sy;
  return i128_to_double(num) / ((double)n * (double)(n - 1));
}

__global__ void __launch_bounds__(kThreads) data_stats_kernel(DataStatsArgs a) {
  extern __shared__ unsigned long long sums[];
  const int A = a.cfg.n_ages, J = a.cfg.n_conds, K = 4 * A + 3 * J;
  unsigned long long* Sp = sums;               // pulse cells: per age (n, sx, sxx)
  unsigned long long* Sc = Sp + 3 * A;         // chase cells
  unsigned long long* Sg = Sc + 3 * A;         // all cells: per (condition, age) (n, su, sl, suu, sll, sul)
  const int nsum = 6 * A + 6 * J * A;
  const int64_t g = blockIdx.x;
  const int b = blockIdx.y;
  for (int i = threadIdx.x; i < nsum; i += blockDim.x) sums[i] = 0ull;
  __syncthreads();
  const int32_t* u = a.u + g * a.C;
  const int32_t* l = a.l + g * a.C;
  // pulse and chase cells (contiguous in the group-sorted cell order)
  for (int f = 0; f < 2; ++f) {
    const int cond = f == 0 ? a.cfg.pulse_stat : a.cfg.chase_stat;
    const int64_t base = a.gstart[cond * A], n = a.gstart[(cond + 1) * A] - base;
    unsigned long long* S = f == 0 ? Sp : Sc;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const int64_t cell = base + (b == 0 ? i : draw_pos(a.seed, f, b, g, i, n));
      const int64_t id = a.cell_id[cell];
      const unsigned long long x = (unsigned long long)u[id] + (unsigned long long)l[id];
      const int ag = a.cell_age[cell];
      atomicAdd(&S[3 * ag + 0], 1ull);
      atomicAdd(&S[3 * ag + 1], x);
      atomicAdd(&S[3 * ag + 2], x * x);
    }
  }
  for (int64_t i = threadIdx.x; i < a.C; i += blockDim.x) {
    const int64_t cell = b == 0 ? i : draw_pos(a.seed, 2, b, g, i, a.C);
    const int64_t id = a.cell_id[cell];
    const unsigned long long uu = (unsigned long long)u[id], ll = (unsigned long long)l[id];
    unsigned long long* S = Sg + 6 * (a.cell_cond[cell] * A + a.cell_age[cell]);
    atomicAdd(&S[0], 1ull);
    atomicAdd(&S[1], uu);
    atomicAdd(&S[2], ll);
    atomicAdd(&S[3], uu * uu);
    atomicAdd(&S[4], ll * ll);
    atomicAdd(&S[5], uu * ll);
  }
  __syncthreads();
  // The statistics of one (family, age) cell or one condition are independent
  // FP64 computations: lanes of warp 0 take the (family, age) cells, lanes of
  // warp 1 the conditions (GB300 issues FP64 warp instructions slowly, so one
  // instruction stream per warp serves all of them).
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* st = a.out + (g * (int64_t)(a.n_boot + 1) + b) * K;
  if (warp == 0) {
    // mean and Fano factor of u + l per age cluster (get_mean_ccp_data, get_ff_ccp_data)
    for (int t = lane; t < 2 * A; t += 32) {
      const int f = t / A, ag = t - (t / A) * A;
      const unsigned long long* S = f == 0 ? Sp : Sc;
      const int off = f == 0 ? 0 : 2 * A;
      const unsigned long long n = S[3 * ag];
      double m = 0.0, ff = 0.0;
      if (n > 0) {
        m = (double)S[3 * ag + 1] / (double)n;
        const double v = sample_cov(n, S[3 * ag + 1], S[3 * ag + 1], S[3 * ag + 2]);
        const double eps = (m == 0.0) ? 0.0001 : 0.0;
        ff = v / (m + eps);
      }
      st[off + ag] = m;
      st[off + A + ag] = ff;
    }
    return;
  }
  if (warp != 1) return;
  for (int j = lane; j < J; j += 32) {
    double m1[kMaxAges], m2[kMaxAges], v1[kMaxAges], v2[kMaxAges], c12[kMaxAges], w[kMaxAges];
    unsigned long long nj = 0, suj = 0, slj = 0;
    for (int ag = 0; ag < A; ++ag) {
      const unsigned long long* S = Sg + 6 * (j * A + ag);
      nj += S[0];
      suj += S[1];
      slj += S[2];
      if (S[0] == 0) {
        m1[ag] = m2[ag] = v1[ag] = v2[ag] = c12[ag] = 0.0;
      } else {
        m1[ag] = (double)S[1] / (double)S[0];
        m2[ag] = (double)S[2] / (double)S[0];
        v1[ag] = sample_cov(S[0], S[1], S[1], S[3]);
        v2[ag] = sample_cov(S[0], S[2], S[2], S[4]);
        c12[ag] = sample_cov(S[0], S[1], S[2], S[5]);
      }
    }
    // ratio of means (get_cond_specific_ratios)
    const double mu = (double)suj / (double)nj, ml = (double)slj / (double)nj;
    st[4 * A + j] = (mu + ml > 0.0) ? ml / (mu + ml) : 0.0;
    // age weights: the given distribution for the estimate; for a bootstrap
    // resample the resampled cells' age fractions within the condition
    // (get_correlation_se normalises per condition)
    for (int ag = 0; ag < A; ++ag) {
      if (b == 0) {
        w[ag] = a.age_dist[ag * J + j];
      } else {
        const double x = (double)Sg[6 * (j * A + ag)] / (double)nj;
        w[ag] = x == x ? x : 0.0;
      }
    }
    // get_cond_specific_correlations
    const double tv1 = wsum(w, v1, A) + wcov(m1, m1, w, A);
    const double tv2 = wsum(w, v2, A) + wcov(m2, m2, w, A);
    bool any_cov = false;
    for (int ag = 0; ag < A; ++ag) any_cov = any_cov || (c12[ag] != 0.0);
    const bool tv_ok = tv1 != 0.0 && tv2 != 0.0;
    st[4 * A + J + j] = (any_cov && tv_ok) ? wsum(w, c12, A) / sqrt(fabs(tv1 * tv2)) : 0.0;
    st[4 * A + 2 * J + j] = tv_ok ? wcov(m1, m2, w, A) / sqrt(fabs(tv1 * tv2)) : 0.0;
  }
}

// standard error over the resamples 1..n_boot of each (gene, statistic):
// sqrt(sum (v - mean)^2 / (n_boot - 1)), sums in resample order
__global__ void data_se_kernel(const double* boot, int64_t G, int K, int n_boot, double* se) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= G * K) return;
  const int64_t g = t / K;
  const int k = (int)(t - g * K);
  const double* v = boot + g * (int64_t)(n_boot + 1) * K + k;
  double s = 0.0;
  for (int b = 1; b <= n_boot; ++b) s = s + v[(int64_t)b * K];
  const double m = s / (double)n_boot;
  double q = 0.0;
  for (int b = 1; b <= n_boot; ++b) {
    const double d = v[(int64_t)b * K] - m;
    q = q + d * d;
  }
  se[t] = sqrt((1.0 / (double)(n_boot - 1)) * q);
}

}  // namespace

cudaError_t launch_data_stats(const DataStatsArgs& a, double* se, cudaStream_t s) {
  if (a.G <= 0) return cudaSuccess;
  const int A = a.cfg.n_ages, J = a.cfg.n_conds, K = 4 * A + 3 * J;
  const size_t smem = sizeof(unsigned long long) * (6 * A + 6 * J * A);
  dim3 grid((unsigned)a.G, (unsigned)(a.n_boot + 1));
  data_stats_kernel<<<grid, kThreads, smem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || a.n_boot < 2 || !se) return e;
  const int64_t n = a.G * K;
  data_se_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.out, a.G, K, a.n_boot, se);
  return cudaGetLastError();
}

}  // namespace abc
