// posterior.cu — what the reference computes from the accepted particles:
// model probabilities with bootstrap intervals (scripts/model_probs.jl:1-28,
// driver :37-62) and per-gene posterior summaries (MAP, mean, quantile
// intervals and particle counts, scripts/posterior_kinetics.jl:1-33).
// FP64, built with -fmad=false: results are bit-identical to the C oracle.
#include <cuda_runtime.h>

#include <atomic>

#include "common.cuh"
#include "smem_attr.h"
#include "kernels.h"

namespace abc {

// Julia's default quantile (Statistics.quantile, alpha = beta = 1) of a sorted
// vector: m = 1 - p, aleph = n p + m, j = clamp(trunc(aleph), 1, n - 1),
// gamma = clamp(aleph - j, 0, 1), v[j] + gamma (v[j+1] - v[j]) (1-based).
// position of Julia's default quantile (type 7: m = 1 - p, aleph = n p + m),
// j clamped to [1, n - 1], and its interpolation weight
__device__ __forceinline__ void quantile_pos(int64_t n, double p, int64_t& j, double& gmm) {
  const double m = 1.0 + p * ((1.0 - 1.0) - 1.0);
  const double aleph = (double)n * p + m;
  j = (int64_t)aleph;
  if (j > n - 1) j = n - 1;
  if (j < 1 && n > 1) j = 1;
  gmm = aleph - (double)j;
  gmm = gmm < 0.0 ? 0.0 : (gmm > 1.0 ? 1.0 : gmm);
}

// quantile from the order statistics a = v[j - 1], b = v[j] of the sorted
// values (v[0] twice for n = 1)
__device__ __forceinline__ double quantile_mix(double a, double b, double gmm) {
  if (isfinite(a) && isfinite(b)) return a + gmm * (b - a);
  return (1.0 - gmm) * a + gmm * b;
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

constexpr int kPostSmem = 8192;   // columns up to this size are staged in shared memory
constexpr int kSelThreads = 256;
constexpr int kSelSmall = 64;     // candidate sets this small are ranked by counting

// order-preserving 64-bit keys of doubles (negative values reversed)
__device__ __forceinline__ uint64_t dkey(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(uint64_t k) {
  const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

struct SelShared {
  unsigned hist[256];
  uint64_t cand[kSelSmall];
  uint64_t result;
  int bin, cnt, ncand;
  long long rr;
};

// The rank-th smallest (0-based) of the n keys K: radix select over 8-bit
// digits from the top, narrowing to the digit bucket that holds the rank;
// once the bucket has at most kSelSmall keys they are collected and the rank
// is found by counting.  Every thread of the block calls it.
__device__ uint64_t block_select(const uint64_t* K, int64_t n, int64_t rank, SelShared& sh) {
  uint64_t prefix = 0, mask = 0;
  long long rr = rank;
  const int lane = threadIdx.x & 31;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sh.hist[i] = 0u;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const uint64_t k = K[i];
      if ((k & mask) == prefix) atomicAdd(&sh.hist[(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      unsigned loc[8], sum = 0;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        loc[b] = sh.hist[lane * 8 + b];
        sum += loc[b];
      }
      unsigned incl = sum;
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      const long long excl = (long long)(incl - sum);
      if (rr >= excl && rr < (long long)incl) {
        long long c = excl;
        for (int b = 0; b < 8; ++b) {
          if (rr < c + (long long)loc[b]) {
            sh.bin = lane * 8 + b;
            sh.rr = rr - c;
            sh.cnt = (int)loc[b];
            break;
          }
          c += loc[b];
        }
      }
    }
    __syncthreads();
    prefix |= (uint64_t)sh.bin << shift;
    mask |= (uint64_t)255u << shift;
    rr = sh.rr;
    const int cnt = sh.cnt;
    __syncthreads();
    if (shift == 0) return prefix;  // every bit fixed
    if (cnt <= kSelSmall) {
      if (threadIdx.x == 0) sh.ncand = 0;
      __syncthreads();
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t k = K[i];
        if ((k & mask) == prefix) sh.cand[atomicAdd(&sh.ncand, 1)] = k;
      }
      __syncthreads();
      if (threadIdx.x < cnt) {
        const uint64_t x = sh.cand[threadIdx.x];
        int less = 0, eq = 0;
        for (int u = 0; u < cnt; ++u) {
          less += sh.cand[u] < x ? 1 : 0;
          eq += sh.cand[u] == x ? 1 : 0;
        }
        if (less <= rr && rr < less + eq) sh.result = x;  // equal keys write the same value
      }
      __syncthreads();
      const uint64_t res = sh.result;
      __syncthreads();
      return res;
    }
  }
  return prefix;
}

// Per (parameter, gene) column of the gathered values, the order statistics
// the two quantiles read: q4 = {v[j_lo - 1], v[j_lo], v[j_hi - 1], v[j_hi]} of
// the sorted column (quantile_pos with p = 1 - q and p = q).  Columns longer
// than kPostSmem are keyed in place in the scratch.
__global__ void __launch_bounds__(kSelThreads) post_select_kernel(const int64_t* aoff, int64_t total, int64_t G,
                                                                  double* scratch, double q, double* q4) {
  extern __shared__ uint64_t sel_keys[];
  __shared__ SelShared sh;
  const int64_t g = blockIdx.x % G;
  const int c = (int)(blockIdx.x / G);
  double* v = scratch + (int64_t)c * total + aoff[g];
  const int64_t n = aoff[g + 1] - aoff[g];
  double* out = q4 + ((int64_t)c * G + g) * 4;
  if (n == 0) return;
  if (n == 1) {
    if (threadIdx.x < 4) out[threadIdx.x] = v[0];
    return;
  }
  uint64_t* K;
  if (n <= kPostSmem) {
    K = sel_keys;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) K[i] = dkey(v[i]);
  } else {
    K = reinterpret_cast<uint64_t*>(v);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) K[i] = dkey(v[i]);
  }
  __syncthreads();
  int64_t jl, jh;
  double gl, gh;
  quantile_pos(n, 1.0 - q, jl, gl);
  quantile_pos(n, q, jh, gh);
  const int64_t ranks[4] = {jl - 1, jl, jh - 1, jh};
  for (int r = 0; r < 4; ++r) {
    const uint64_t k = block_select(K, n, ranks[r], sh);
    if (threadIdx.x == 0) out[r] = dkey_inv(k);
  }
}

// One block per gene.  counts[g][m] = accepted particles of model group m.
// No acceptance: zeros; one group with acceptances: that group 1, 1, 1 (the
// `which` branch of model_probs.jl:41-48); otherwise l / sum(l) and n_boot
// bootstrap resamples of the sum(l) model labels (a multinomial draw, made
// as conditional binomials from the (bootstrap, gene) Philox stream; the
// block's threads take the resamples), with quantiles 1 - alpha and alpha of
// the resampled proportions from the order statistics they read
// (block_select on order-preserving keys; keys: G x M x n_boot scratch).
__global__ void __launch_bounds__(kSelThreads) model_probs_kernel(const int64_t* counts, int64_t G, int M,
                                                                  int n_boot, double alpha, uint64_t seed,
                                                                  double* prob, double* lb, double* ub,
                                                                  uint64_t* keys) {
  __shared__ SelShared sh;
  __shared__ long long s_L;
  __shared__ int s_nz;
  const int64_t g = blockIdx.x;
  const int64_t* l = counts + g * M;
  double* P = prob + g * M;
  double* LB = lb + g * M;
  double* UB = ub + g * M;
  if (threadIdx.x == 0) {
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
    if (L > 0 && nz == 1) {
      P[which] = 1.0;
      LB[which] = 1.0;
      UB[which] = 1.0;
    }
    s_L = L;
    s_nz = nz;
  }
  __syncthreads();
  const int64_t L = s_L;
  if (L == 0 || s_nz == 1) return;
  for (int m = threadIdx.x; m < M; m += blockDim.x) P[m] = (double)l[m] / (double)L;
  uint64_t* kv = keys + g * (int64_t)M * n_boot;
  for (int b = threadIdx.x; b < n_boot; b += blockDim.x) {
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
      kv[(int64_t)m * n_boot + b] = dkey((double)x / (double)L);
    }
  }
  __syncthreads();
  int64_t jl, jh;
  double gl, gh;
  quantile_pos(n_boot, 1.0 - alpha, jl, gl);
  quantile_pos(n_boot, alpha, jh, gh);
  const int64_t ranks[4] = {n_boot == 1 ? 0 : jl - 1, n_boot == 1 ? 0 : jl, n_boot == 1 ? 0 : jh - 1,
                            n_boot == 1 ? 0 : jh};
  for (int m = 0; m < M; ++m) {
    double q[4];
    for (int r = 0; r < 4; ++r) q[r] = dkey_inv(block_select(kv + (int64_t)m * n_boot, n_boot, ranks[r], sh));
    if (threadIdx.x == 0) {
      LB[m] = quantile_mix(q[0], q[1], gl);
      UB[m] = quantile_mix(q[2], q[3], gh);
    }
  }
}

cudaError_t launch_model_probs(const int64_t* counts, int64_t G, int M, int n_boot, double alpha, uint64_t seed,
                               double* prob, double* lb, double* ub, double* boot, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  model_probs_kernel<<<(unsigned)G, kSelThreads, 0, s>>>(counts, G, M, n_boot, alpha, seed, prob, lb, ub,
                                                          reinterpret_cast<uint64_t*>(boot));
  return cudaGetLastError();
}

__global__ void post_summary_kernel(const int64_t* aoff, const int64_t* idx, const double* theta, int64_t ld,
                                    int npar, int64_t G, int64_t total, const double* q4, double q,
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
  const double* v4 = q4 + ((int64_t)c * G + g) * 4;
  int64_t j;
  double gl, gh;
  quantile_pos(n, 1.0 - q, j, gl);
  quantile_pos(n, q, j, gh);
  lb[t] = quantile_mix(v4[0], v4[1], gl);
  ub[t] = quantile_mix(v4[2], v4[3], gh);
}

cudaError_t launch_posterior_summary(const int64_t* aoff, const int64_t* idx, int64_t G, int64_t total,
                                     const double* theta, int64_t ld, int npar, double q, double* scratch,
                                     double* map, double* mean, double* lb, double* ub, int64_t* n_out,
                                     cudaStream_t s) {
  if (G <= 0 || npar <= 0) return cudaSuccess;
  // scratch: total x npar gathered values, then G x npar x 4 order statistics
  double* q4 = scratch + (size_t)total * npar;
  if (total > 0) {
    post_gather_kernel<<<(unsigned)G, 256, 0, s>>>(aoff, idx, theta, ld, npar, total, scratch);
    constexpr int smem = kPostSmem * (int)sizeof(uint64_t);
    static std::atomic<uint64_t> attr{0};  // devices where the limit is set, shared by all contexts
    cudaError_t e = set_smem_once(attr, post_select_kernel, smem);
    if (e != cudaSuccess) return e;
    post_select_kernel<<<(unsigned)(G * npar), kSelThreads, smem, s>>>(aoff, total, G, scratch, q, q4);
  }
  const int64_t n = G * npar;
  post_summary_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(aoff, idx, theta, ld, npar, G, total, q4, q,
                                                                  map, mean, lb, ub, n_out);
  return cudaGetLastError();
}

}  // namespace abc
