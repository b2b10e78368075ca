// distance_fp32.cu — FP32 particle x gene distance with a fused epilogue
// (candidate emission or subsample export) and the per-gene threshold pass.
// The P x G error matrix is never written in full.
#include "distance.cuh"
#include "kernels.h"

namespace abc {

// 256 threads = 16 x 16; thread (tx, ty) owns particles ty + 16 i and genes
// tx + 16 j (i, j < 8) of a 128 x 128 tile.  Statistics stream through shared
// memory kDistKc at a time, stored k-major so one row serves all threads.
__global__ void __launch_bounds__(256) dist_fast_kernel(const float* __restrict__ s32,
                                                        const float* __restrict__ sw,
                                                        const float* __restrict__ dw, int64_t P, int64_t G,
                                                        int K, const float* __restrict__ X, Cand* cand,
                                                        unsigned long long* n_cand, int64_t cap, float* esub,
                                                        int64_t stride, int64_t n_sub) {
  __shared__ float ss[kDistKc][kDistTile];
  __shared__ float sa[kDistKc][kDistTile];
  __shared__ float sd[kDistKc][kDistTile];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t g0 = (int64_t)blockIdx.x * kDistTile;
  const int64_t r0 = (int64_t)blockIdx.y * kDistTile;  // row = particle (emit) or subsample row
  const bool sample = esub != nullptr;
  const int64_t nrows = sample ? n_sub : P;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

  for (int k0 = 0; k0 < K; k0 += kDistKc) {
    // cooperative loads: 128 rows x kDistKc values for each of the three tiles
    for (int idx = threadIdx.x; idx < kDistKc * kDistTile; idx += 256) {
      const int r = idx / kDistKc, kk = idx - (idx / kDistKc) * kDistKc;
      const int k = k0 + kk;
      const int64_t row = r0 + r;
      float sv = 0.0f;
      if (row < nrows && k < K) {
        const int64_t p = sample ? row * stride : row;
        sv = s32[p * K + k];
      }
      ss[kk][r] = sv;
      const int64_t g = g0 + r;
      float av = 0.0f, dv = 0.0f;
      if (g < G && k < K) {
        av = sw[g * K + k];
        dv = dw[g * K + k];
      }
      sa[kk][r] = av;
      sd[kk][r] = dv;
    }
    __syncthreads();
    const int kc = (K - k0) < kDistKc ? (K - k0) : kDistKc;
#pragma unroll 4
    for (int kk = 0; kk < kc; ++kk) {
      float s[8], a[8], d[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) s[i] = ss[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        a[j] = sa[kk][tx + 16 * j];
        d[j] = sd[kk][tx + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float t = fmaf(-a[j], s[i], d[j]);
          acc[i][j] = fmaf(t, t, acc[i][j]);
        }
    }
    __syncthreads();
  }
  const float invK = 1.0f / (float)K;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t row = r0 + ty + 16 * i;
    if (row >= nrows) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t g = g0 + tx + 16 * j;
      if (g >= G) continue;
      float e = fminf(acc[i][j] * invK, 10.0f);
      if (acc[i][j] != acc[i][j]) e = acc[i][j];  // keep NaN (fminf would drop it)
      if (sample) {
        esub[row * G + g] = e;
      } else if (e <= X[g]) {
        unsigned long long slot = atomicAdd(n_cand, 1ull);
        if (slot < (unsigned long long)cap) {
          Cand c;
          c.p = (int32_t)row;
          c.g = (int32_t)g;
          cand[slot] = c;
        }
      }
    }
  }
}

cudaError_t launch_dist_fast(const float* s32, const float* sw, const float* dw, int64_t P, int64_t G, int K,
                             const float* X, Cand* cand, unsigned long long* n_cand, int64_t cap,
                             float* esub, int64_t stride, int64_t n_sub, cudaStream_t s) {
  const int64_t rows = esub ? n_sub : P;
  if (rows <= 0 || G <= 0) return cudaSuccess;
  dim3 grid((unsigned)((G + kDistTile - 1) / kDistTile), (unsigned)((rows + kDistTile - 1) / kDistTile));
  dist_fast_kernel<<<grid, 256, 0, s>>>(s32, sw, dw, P, G, K, X, cand, n_cand, cap, esub, stride, n_sub);
  return cudaGetLastError();
}

// One CTA per gene: histogram of the subsample errors on a sqrt scale, then
// the bin where the running count reaches k_sub gives X[g] (its upper edge
// widened by twice the FP32 error bound).
__global__ void __launch_bounds__(256) dist_threshold_kernel(const float* __restrict__ esub, int64_t n_sub,
                                                             int64_t G, int64_t k_sub, int K, float* X) {
  __shared__ unsigned int hist[kHistBins];
  __shared__ unsigned int csum[256];
  const int64_t g = blockIdx.x;
  for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) hist[b] = 0u;
  __syncthreads();
  for (int64_t r = threadIdx.x; r < n_sub; r += blockDim.x) {
    float e = esub[r * G + g];
    if (e == e) atomicAdd(&hist[hist_bin(e)], 1u);
  }
  __syncthreads();
  // per-thread chunk sums (16 bins each) and an exclusive scan by thread 0
  const int per = kHistBins / 256;
  unsigned int local = 0;
  for (int b = 0; b < per; ++b) local += hist[threadIdx.x * per + b];
  csum[threadIdx.x] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    int found = -1;
    for (int t = 0; t < 256 && found < 0; ++t) {
      if (run + csum[t] >= (unsigned long long)k_sub) {
        for (int b = 0; b < per; ++b) {
          run += hist[t * per + b];
          if (run >= (unsigned long long)k_sub) {
            found = t * per + b;
            break;
          }
        }
      } else {
        run += csum[t];
      }
    }
    float x;
    if (found < 0 || k_sub <= 0) {
      x = INFINITY;
    } else {
      float up = hist_upper(found);
      float xp = up + 1.01f * dist_bound_f(up, K);
      x = xp + 1.01f * dist_bound_f(xp, K);
    }
    X[g] = x;
  }
}

cudaError_t launch_dist_threshold(const float* esub, int64_t n_sub, int64_t G, int64_t k_sub, int K, float* X,
                                  cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  dist_threshold_kernel<<<(unsigned)G, 256, 0, s>>>(esub, n_sub, G, k_sub, K, X);
  return cudaGetLastError();
}

float dist_bound(float e, int K) { return dist_bound_f(e, K); }

// Surrogate screen: a lower confidence bound of the error of particle p for
// gene g under the predicted statistics (mean mu_pk, predictive std sd_pk):
//   L_pg = sum_k w_gk max(0, |d_gk - mu_pk| - z sd_pk)^2 / K,
// keep[p] = 1 when L_pg <= X[g] for some gene (X = calibrated threshold).
// A draw is dropped only when it is confidently far from every gene.  Same
// 128 x 128 tiling as dist_fast_kernel.
__global__ void __launch_bounds__(256) dist_screen_kernel(const float* __restrict__ mu,
                                                          const float* __restrict__ var,
                                                          const float* __restrict__ sw,
                                                          const float* __restrict__ dw, int64_t P, int64_t G,
                                                          int K, const float* __restrict__ X, float z,
                                                          uint8_t* keep, float* err_out) {
  __shared__ float sm[kDistKc][kDistTile];
  __shared__ float sv[kDistKc][kDistTile];
  __shared__ float sa[kDistKc][kDistTile];
  __shared__ float sd[kDistKc][kDistTile];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t g0 = (int64_t)blockIdx.x * kDistTile;
  const int64_t p0 = (int64_t)blockIdx.y * kDistTile;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  for (int k0 = 0; k0 < K; k0 += kDistKc) {
    for (int idx = threadIdx.x; idx < kDistKc * kDistTile; idx += 256) {
      const int r = idx / kDistKc, kk = idx - (idx / kDistKc) * kDistKc;
      const int k = k0 + kk;
      const int64_t p = p0 + r, g = g0 + r;
      float m = 0.0f, v = 0.0f, a = 0.0f, d = 0.0f;
      if (p < P && k < K) {
        m = mu[p * K + k];
        v = z * sqrtf(fmaxf(var[p * K + k], 0.0f));  // z x predictive std
      }
      if (g < G && k < K) {
        a = sw[g * K + k];
        d = dw[g * K + k];
      }
      sm[kk][r] = m;
      sv[kk][r] = v;
      sa[kk][r] = a;
      sd[kk][r] = d;
    }
    __syncthreads();
    const int kc = (K - k0) < kDistKc ? (K - k0) : kDistKc;
#pragma unroll 2
    for (int kk = 0; kk < kc; ++kk) {
      float m[8], v[8], a[8], d[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        m[i] = sm[kk][ty + 16 * i];
        v[i] = sv[kk][ty + 16 * i];
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        a[j] = sa[kk][tx + 16 * j];
        d[j] = sd[kk][tx + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float t = fmaxf(fabsf(fmaf(-a[j], m[i], d[j])) - a[j] * v[i], 0.0f);
          acc[i][j] = fmaf(t, t, acc[i][j]);
        }
    }
    __syncthreads();
  }
  const float invK = 1.0f / (float)K;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t p = p0 + ty + 16 * i;
    if (p >= P) continue;
    bool any = false;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t g = g0 + tx + 16 * j;
      if (g >= G) continue;
      const float e = acc[i][j] * invK;  // not clipped: far draws keep large expected errors
      if (err_out) err_out[p * G + g] = e;
      any = any || (e <= X[g]);
    }
    if (any) keep[p] = 1;
  }
}

cudaError_t launch_dist_screen(const float* mu, const float* var, const float* sw, const float* dw, int64_t P,
                               int64_t G, int K, const float* X, float z, uint8_t* keep, float* err_out,
                               cudaStream_t s) {
  if (P <= 0 || G <= 0) return cudaSuccess;
  dim3 grid((unsigned)((G + kDistTile - 1) / kDistTile), (unsigned)((P + kDistTile - 1) / kDistTile));
  dist_screen_kernel<<<grid, 256, 0, s>>>(mu, var, sw, dw, P, G, K, X, z, keep, err_out);
  return cudaGetLastError();
}

}  // namespace abc
