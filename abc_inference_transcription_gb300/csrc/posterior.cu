// posterior.cu — what the reference computes from the accepted particles:
// model probabilities with bootstrap intervals (scripts/model_probs.jl:1-28,
// driver :37-62) and per-gene posterior summaries (MAP, mean, quantile
// intervals and particle counts, scripts/posterior_kinetics.jl:1-33).
// FP64, built with -fmad=false: results are bit-identical to the C oracle.
#include <cuda_runtime.h>

#include "bitonic.cuh"
#include "common.cuh"
#include "kernels.h"

namespace abc {

// Julia's default quantile (Statistics.quantile, alpha = beta = 1) of a sorted
// vector: m = 1 - p, aleph = n p + m, j = clamp(trunc(aleph), 1, n - 1),
// gamma = clamp(aleph - j, 0, 1), v[j] + gamma (v[j+1] - v[j]) (1-based).
__device__ double quantile_sorted(const double* v, int64_t n, double p) {
  const double m = 1.0 + p * ((1.0 - 1.0) - 1.0);
  const double aleph = (double)n * p + m;
  int64_t j = (int64_t)aleph;
  if (j > n - 1) j = n - 1;
  if (j < 1 && n > 1) j = 1;
  double gmm = aleph - (double)j;
  gmm = gmm < 0.0 ? 0.0 : (gmm > 1.0 ? 1.0 : gmm);
  double a, b;
  if (n == 1) {
    a = v[0];
    b = v[0];
  } else {
    a = v[j - 1];
    b = v[j];
  }
  if (isfinite(a) && isfinite(b)) return a + gmm * (b - a);
  return (1.0 - gmm) * a + gmm * b;
}

// One thread per gene.  counts[g][m] = accepted particles of model group m.
// No acceptance: zeros; one group with acceptances: that group 1, 1, 1 (the
// `which` branch of model_probs.jl:41-48); otherwise l / sum(l) and n_boot
// bootstrap resamples of the sum(l) model labels (a multinomial draw, made
// as conditional binomials from the (bootstrap, gene) Philox stream), with
// quantiles 1 - alpha and alpha of the resampled proportions.
__global__ void model_probs_kernel(const int64_t* counts, int64_t G, int M, int n_boot, double alpha,
                                   uint64_t seed, double* prob, double* lb, double* ub, double* boot) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const int64_t* l = counts + g * M;
  double* P = prob + g * M;
  double* LB = lb + g * M;
  double* UB = ub + g * M;
  int64_t L = 0;
  int nz = 0, which = -1;
  for (int m = 0; m < M; ++m) {
    L += l[m];
    if (l[m] > 0) {
      nz++;
      which = m;
    }
    P[m] = 0.0;
    LB[m] = 0.0;
    UB[m] = 0.0;
  }
  if (L == 0) return;
  if (nz == 1) {
    P[which] = 1.0;
    LB[which] = 1.0;
    UB[which] = 1.0;
    return;
  }
  for (int m = 0; m < M; ++m) P[m] = (double)l[m] / (double)L;
  double* bv = boot + g * (int64_t)M * n_boot;
  for (int b = 0; b < n_boot; ++b) {
    Rng r;
    rng_init(r, seed, ST_AUX, (uint32_t)b, (uint32_t)g);
    int64_t nrem = L, lrem = L;
    for (int m = 0; m < M; ++m) {
      int64_t x;
      if (m == M - 1 || lrem == l[m]) x = nrem;
      else if (l[m] == 0 || nrem == 0) x = 0;
      else x = binomial(r, nrem, (double)l[m] / (double)lrem);
      nrem -= x;
      lrem -= l[m];
      bv[(int64_t)m * n_boot + b] = (double)x / (double)L;
    }
  }
  for (int m = 0; m < M; ++m) {
    double* v = bv + (int64_t)m * n_boot;
    for (int i = 1; i < n_boot; ++i) {  // insertion sort of n_boot values
      const double x = v[i];
      int j = i - 1;
      while (j >= 0 && v[j] > x) {
        v[j + 1] = v[j];
        --j;
      }
      v[j + 1] = x;
    }
    LB[m] = quantile_sorted(v, n_boot, 1.0 - alpha);
    UB[m] = quantile_sorted(v, n_boot, alpha);
  }
}

cudaError_t launch_model_probs(const int64_t* counts, int64_t G, int M, int n_boot, double alpha, uint64_t seed,
                               double* prob, double* lb, double* ub, double* boot, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  model_probs_kernel<<<(unsigned)((G + 127) / 128), 128, 0, s>>>(counts, G, M, n_boot, alpha, seed, prob, lb, ub,
                                                                 boot);
  return cudaGetLastError();
}

// scratch[c][aoff[g] + i] = theta[idx - 1][c] for the accepted particles of gene g
__global__ void post_gather_kernel(const int64_t* aoff, const int64_t* idx, const double* theta, int64_t ld,
                                   int npar, int64_t total, double* scratch) {
  const int64_t g = blockIdx.x;
  for (int64_t t = aoff[g] + threadIdx.x; t < aoff[g + 1]; t += blockDim.x) {
    const double* row = theta + (idx[t] - 1) * ld;
    for (int c = 0; c < npar; ++c) scratch[(int64_t)c * total + t] = row[c];
  }
}

constexpr int kPostSmem = 8192;  // segments up to this size sort in registers

// order-preserving 64-bit keys of doubles (negative values reversed)
__device__ __forceinline__ uint64_t dkey(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(uint64_t k) {
  const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

template <int EPT>
__device__ void post_sort_regs(double* v, int m, int n2, uint64_t* sK, int32_t* sP) {
  const int t = threadIdx.x;
  const int nt = n2 / EPT > 32 ? n2 / EPT : 32;
  const bool act = t < nt;
  uint64_t key[EPT];
  int32_t pp[EPT];
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const int i = t * EPT + e;
    const bool real = act && i < m;
    key[e] = real ? dkey(v[i]) : ~0ull;
    pp[e] = real ? 0 : 0x7fffffff;
  }
  bitonic_regs<EPT>(key, pp, n2, sK, sP);
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const int i = t * EPT + e;
    if (act && i < m) v[i] = dkey_inv(key[e]);
  }
}

// Ascending sort of each (parameter, gene) column of the gathered values.
__global__ void __launch_bounds__(1024, 1) post_sort_kernel(const int64_t* aoff, int64_t total, int64_t G,
                                                            double* scratch) {
  extern __shared__ uint64_t post_smem[];
  const int64_t g = blockIdx.x % G;
  const int c = (int)(blockIdx.x / G);
  double* v = scratch + (int64_t)c * total + aoff[g];
  const int64_t n = aoff[g + 1] - aoff[g];
  if (n <= 1) return;
  int64_t n2 = 1;
  while (n2 < n) n2 <<= 1;
  if (n2 <= kPostSmem) {
    uint64_t* sK = post_smem;
    int32_t* sP = reinterpret_cast<int32_t*>(post_smem + kPostSmem);
    const int m = (int)n, w = (int)n2;
    if (w <= 1024) post_sort_regs<1>(v, m, w, sK, sP);
    else if (w == 2048) post_sort_regs<2>(v, m, w, sK, sP);
    else if (w == 4096) post_sort_regs<4>(v, m, w, sK, sP);
    else post_sort_regs<8>(v, m, w, sK, sP);
    return;
  }
  for (int64_t k = 2; k <= n2; k <<= 1) {
    for (int64_t j = k >> 1; j > 0; j >>= 1) {
      for (int64_t i = threadIdx.x; i < n2; i += blockDim.x) {
        const int64_t partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
        if (partner > i && partner < n) {
          const double a = v[i], b = v[partner];
          if (b < a) {
            v[i] = b;
            v[partner] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void post_summary_kernel(const int64_t* aoff, const int64_t* idx, const double* theta, int64_t ld,
                                    int npar, int64_t G, int64_t total, const double* scratch, double q,
                                    double* map, double* mean, double* lb, double* ub, int64_t* n_out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= G * npar) return;
  const int64_t g = t / npar;
  const int c = (int)(t - g * npar);
  const int64_t o = aoff[g], n = aoff[g + 1] - o;
  if (c == 0 && n_out) n_out[g] = n;
  if (n == 0) {
    map[t] = NAN;
    mean[t] = NAN;
    lb[t] = NAN;
    ub[t] = NAN;
    return;
  }
  map[t] = theta[(idx[o] - 1) * ld + c];
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s = s + theta[(idx[o + i] - 1) * ld + c];
  mean[t] = s / (double)n;
  const double* v = scratch + (int64_t)c * total + o;
  lb[t] = quantile_sorted(v, n, 1.0 - q);
  ub[t] = quantile_sorted(v, n, q);
}

cudaError_t launch_posterior_summary(const int64_t* aoff, const int64_t* idx, int64_t G, int64_t total,
                                     const double* theta, int64_t ld, int npar, double q, double* scratch,
                                     double* map, double* mean, double* lb, double* ub, int64_t* n_out,
                                     cudaStream_t s) {
  if (G <= 0 || npar <= 0) return cudaSuccess;
  if (total > 0) {
    post_gather_kernel<<<(unsigned)G, 256, 0, s>>>(aoff, idx, theta, ld, npar, total, scratch);
    constexpr int smem = kPostSmem * (int)(sizeof(uint64_t) + sizeof(int32_t));
    static bool attr = false;
    if (!attr) {
      cudaError_t e = cudaFuncSetAttribute(post_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
      attr = true;
    }
    post_sort_kernel<<<(unsigned)(G * npar), 1024, smem, s>>>(aoff, total, G, scratch);
  }
  const int64_t n = G * npar;
  post_summary_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(aoff, idx, theta, ld, npar, G, total, scratch, q,
                                                                  map, mean, lb, ub, n_out);
  return cudaGetLastError();
}

}  // namespace abc
