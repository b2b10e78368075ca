// datastats.cu — the data side of the distance: the 53 statistics of every
// gene's observed per-cell counts and their bootstrap standard errors
// (scripts/data_summary_statistics.jl:1-216).  Same layout as the simulated
// statistics: [pulse mean (A), pulse FF (A), chase mean (A), chase FF (A),
// ratio (J), mean_corr (J), corr_mean (J)].
//
// Two phases: one CTA per (gene, resample) forms the integer sums, then one
// thread per (gene, resample, statistic group) computes the statistics from
// them.  Resample 0 is the estimate itself, 1..n_boot are bootstrap resamples
// of the cells with replacement, drawn separately for
// the pulse cells, the chase cells and all cells (ratios and correlations), as
// the reference's get_ccp_se / get_ratio_se / get_correlation_se do.  Draw i
// of (gene, resample, family) comes from its own Philox counter, so threads
// draw independently; every statistic is computed from exact integer sums
// (n, sum x, sum x^2, sum u l per group), so the result does not depend on
// the reduction order and is bit-identical to the C oracle.  FP64 formulas
// built with -fmad=false.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "distance.cuh"
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

// the same with the denominator d2 = n (n - 1) and r2 = RN(1 / d2) given: the
// quotient through div_rn (correctly rounded, equal to the IEEE division)
__device__ __forceinline__ double sample_cov_r(unsigned long long n, unsigned long long sx, unsigned long long sy,
                                               unsigned long long sxy, double d2, double r2) {
  const __int128 num = (__int128)n * (__int128)sxy - (__int128)sx * (__int128)sy;
  return div_rn(i128_to_double(num), d2, r2);
}

// Exact 64-bit sums from 32-bit shared-memory atomics (the 64-bit form is far
// slower): the low word takes the addend's low 32 bits, its carry out is read
// from the returned old value, and the high word is touched only for a carry
// or a non-zero high part (rare for counts).
__device__ __forceinline__ void add64(unsigned* lo, unsigned* hi, unsigned long long v) {
  const unsigned vl = (unsigned)v, vh = (unsigned)(v >> 32);
  const unsigned old = atomicAdd(lo, vl);
  const unsigned carry = old + vl < old ? 1u : 0u;
  if (carry | vh) atomicAdd(hi, vh + carry);
}

// Phase 1, one CTA per (gene, resample group): the integer sums of the
// resamples b = blockIdx.y, blockIdx.y + gridDim.y, ...  The gene's cells are
// first copied into shared memory in the group-sorted order, (u, l) and the
// (condition, age) group of each, so that the draws (random cells) read
// shared memory instead of scattered global lines.  Each warp accumulates
// into its own copy of the sums (low and high words), so atomics contend only
// within a warp; after each resample the copies are added and the nsum totals
// written to S_out (integer sums: the order does not matter).
constexpr int kWarps = kThreads / 32;
constexpr size_t data_stats_smem_limit() { return 227 * 1024; }

__global__ void __launch_bounds__(kThreads) data_sums_kernel(DataStatsArgs a, int64_t g0,
                                                             unsigned long long* S_out) {
  extern __shared__ unsigned long long sums[];
  const int A = a.cfg.n_ages, J = a.cfg.n_conds;
  const int nsum = 6 * A + 6 * J * A;
  const int64_t C = a.C;
  unsigned* words = reinterpret_cast<unsigned*>(sums);               // per warp: lo[nsum], hi[nsum]
  int2* T = reinterpret_cast<int2*>(sums + kWarps * nsum);           // (u, l) per sorted cell
  unsigned short* grp = reinterpret_cast<unsigned short*>(T + C);   // condition * A + age
  unsigned* lo = words + (threadIdx.x >> 5) * 2 * nsum;
  unsigned* hi = lo + nsum;
  const int ocs = 6 * A;                                              // offset of the all-cells sums
  const int64_t g = g0 + blockIdx.x;
  const int32_t* u = a.u + g * C;
  const int32_t* l = a.l + g * C;
  for (int64_t i = threadIdx.x; i < C; i += blockDim.x) {
    const int64_t id = a.cell_id[i];
    T[i] = make_int2(u[id], l[id]);
    grp[i] = (unsigned short)(a.cell_cond[i] * A + a.cell_age[i]);
  }
  for (int b = blockIdx.y; b <= a.n_boot; b += gridDim.y) {
    for (int i = threadIdx.x; i < 2 * kWarps * nsum; i += blockDim.x) words[i] = 0u;
    __syncthreads();
    // pulse and chase cells (contiguous in the group-sorted cell order):
    // per age (n, sx, sxx) at 3 A f + 3 ag
    for (int f = 0; f < 2; ++f) {
      const int cond = f == 0 ? a.cfg.pulse_stat : a.cfg.chase_stat;
      const int64_t base = a.gstart[cond * A], n = a.gstart[(cond + 1) * A] - base;
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const int64_t cell = base + (b == 0 ? i : draw_pos(a.seed, f, b, g, i, n));
        const int2 t = T[cell];
        const unsigned long long x = (unsigned long long)t.x + (unsigned long long)t.y;
        const int o = 3 * A * f + 3 * ((int)grp[cell] - cond * A);
        atomicAdd(&lo[o], 1u);
        add64(&lo[o + 1], &hi[o + 1], x);
        add64(&lo[o + 2], &hi[o + 2], x * x);
      }
    }
    // all cells: per (condition, age) (n, su, sl, suu, sll, sul)
    for (int64_t i = threadIdx.x; i < C; i += blockDim.x) {
      const int64_t cell = b == 0 ? i : draw_pos(a.seed, 2, b, g, i, C);
      const int2 t = T[cell];
      const unsigned long long uu = (unsigned long long)t.x, ll = (unsigned long long)t.y;
      const int o = ocs + 6 * (int)grp[cell];
      atomicAdd(&lo[o], 1u);
      add64(&lo[o + 1], &hi[o + 1], uu);
      add64(&lo[o + 2], &hi[o + 2], ll);
      add64(&lo[o + 3], &hi[o + 3], uu * uu);
      add64(&lo[o + 4], &hi[o + 4], ll * ll);
      add64(&lo[o + 5], &hi[o + 5], uu * ll);
    }
    __syncthreads();
    unsigned long long* out = S_out + ((int64_t)blockIdx.x * (a.n_boot + 1) + b) * nsum;
    for (int i = threadIdx.x; i < nsum; i += blockDim.x) {
      unsigned long long t = 0ull;
      for (int w = 0; w < kWarps; ++w)
        t += ((unsigned long long)words[w * 2 * nsum + nsum + i] << 32) | words[w * 2 * nsum + i];
      out[i] = t;
    }
    __syncthreads();
  }
}

// Phase 2, one thread per (gene, resample, item): items 0..2A-1 are the mean
// and Fano factor of one (family, age) cell, items 2A..2A+J-1 the ratio,
// mean_corr and corr_mean of one condition.
__global__ void data_stats_kernel(DataStatsArgs a, int64_t g0, int64_t ng, const unsigned long long* S_in) {
  const int A = a.cfg.n_ages, J = a.cfg.n_conds, K = 4 * A + 3 * J;
  const int nsum = 6 * A + 6 * J * A;
  const int items = 2 * A + J;
  const int64_t total = ng * (a.n_boot + 1) * items;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t gb = t / items;  // (gene - g0) * (n_boot + 1) + resample
    const int it = (int)(t - gb * items);
    const int b = (int)(gb % (a.n_boot + 1));
    const unsigned long long* Sp = S_in + gb * nsum;
    const unsigned long long* Sc = Sp + 3 * A;
    const unsigned long long* Sg = Sc + 3 * A;
    double* st = a.out + (g0 * (int64_t)(a.n_boot + 1) + gb) * K;
    if (it < 2 * A) {
      // mean and Fano factor of u + l per age cluster (get_mean_ccp_data, get_ff_ccp_data)
      const int f = it / A, ag = it - (it / A) * A;
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
      continue;
    }
    const int j = it - 2 * A;
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
        // two reciprocals per group instead of five divisions
        const double nd = (double)S[0], rn = 1.0 / nd;
        m1[ag] = div_rn((double)S[1], nd, rn);
        m2[ag] = div_rn((double)S[2], nd, rn);
        const double d2 = nd * (double)(S[0] - 1), r2 = 1.0 / d2;
        v1[ag] = sample_cov_r(S[0], S[1], S[1], S[3], d2, r2);
        v2[ag] = sample_cov_r(S[0], S[2], S[2], S[4], d2, r2);
        c12[ag] = sample_cov_r(S[0], S[1], S[2], S[5], d2, r2);
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

int64_t data_stats_max_cells(int n_ages, int n_conds) {
  const int64_t nsum = 6 * n_ages + 6 * n_conds * n_ages;
  return ((int64_t)data_stats_smem_limit() - (int64_t)sizeof(unsigned long long) * nsum * kWarps) /
         (int64_t)(sizeof(int2) + sizeof(unsigned short));
}

cudaError_t launch_data_stats(const DataStatsArgs& a, double* se, cudaStream_t s) {
  if (a.G <= 0) return cudaSuccess;
  const int A = a.cfg.n_ages, J = a.cfg.n_conds, K = 4 * A + 3 * J;
  const int64_t nsum = 6 * A + 6 * J * A;
  const size_t smem = sizeof(unsigned long long) * nsum * kWarps + (size_t)a.C * (sizeof(int2) + sizeof(unsigned short));
  if (smem > data_stats_smem_limit()) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(data_sums_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  // the sums of at most ~256 MB of (gene, resample) pairs at a time
  const int64_t per_gene = (int64_t)(a.n_boot + 1) * nsum * (int64_t)sizeof(unsigned long long);
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(a.G, ((int64_t)256 << 20) / per_gene));
  unsigned long long* S = nullptr;
  cudaError_t e = cudaMallocAsync(&S, (size_t)(chunk * per_gene), s);
  if (e != cudaSuccess) return e;
  for (int64_t g0 = 0; g0 < a.G && e == cudaSuccess; g0 += chunk) {
    const int64_t ng = std::min<int64_t>(chunk, a.G - g0);
    // enough CTAs to fill the GPU several times over, resamples split among them
    const int64_t want = (int64_t)4 * 152 * 5;
    const int groups = (int)std::max<int64_t>(1, std::min<int64_t>(a.n_boot + 1, (want + ng - 1) / ng));
    data_sums_kernel<<<dim3((unsigned)ng, (unsigned)groups), kThreads, smem, s>>>(a, g0, S);
    const int64_t items = ng * (a.n_boot + 1) * (2 * A + J);
    const int64_t blocks = std::min<int64_t>((items + 127) / 128, 65536);
    data_stats_kernel<<<(unsigned)blocks, 128, 0, s>>>(a, g0, ng, S);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(S, s);
  if (e != cudaSuccess) return e;
  if (ef != cudaSuccess) return ef;
  if (a.n_boot < 2 || !se) return cudaSuccess;
  const int64_t n = a.G * K;
  data_se_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.out, a.G, K, a.n_boot, se);
  return cudaGetLastError();
}

}  // namespace abc
