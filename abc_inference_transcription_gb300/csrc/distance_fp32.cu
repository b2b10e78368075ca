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
                                                        float* cand_e, unsigned long long* n_cand, int64_t cap,
                                                        float* esub, int64_t stride, int64_t n_sub) {
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
          if (cand_e) cand_e[slot] = e;
        }
      }
    }
  }
}

cudaError_t launch_dist_fast(const float* s32, const float* sw, const float* dw, int64_t P, int64_t G, int K,
                             const float* X, Cand* cand, float* cand_e, unsigned long long* n_cand, int64_t cap,
                             float* esub, int64_t stride, int64_t n_sub, cudaStream_t s) {
  const int64_t rows = esub ? n_sub : P;
  if (rows <= 0 || G <= 0) return cudaSuccess;
  dim3 grid((unsigned)((G + kDistTile - 1) / kDistTile), (unsigned)((rows + kDistTile - 1) / kDistTile));
  dist_fast_kernel<<<grid, 256, 0, s>>>(s32, sw, dw, P, G, K, X, cand, cand_e, n_cand, cap, esub, stride, n_sub);
  return cudaGetLastError();
}

// Cumulative histogram search shared by the threshold and refinement kernels:
// the first bin at which the running count of hist[0..kHistBins) reaches k
// (-1 if it never does).  One CTA of 256 threads; csum is 256 words of shared memory.
__device__ int hist_find(const unsigned int* hist, int64_t k, unsigned int* csum) {
  const int per = kHistBins / 256;
  unsigned int local = 0;
  for (int b = 0; b < per; ++b) local += hist[threadIdx.x * per + b];
  csum[threadIdx.x] = local;
  __syncthreads();
  int found = -1;
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    for (int t = 0; t < 256 && found < 0; ++t) {
      if (run + csum[t] >= (unsigned long long)k) {
        for (int b = 0; b < per; ++b) {
          run += hist[t * per + b];
          if (run >= (unsigned long long)k) {
            found = t * per + b;
            break;
          }
        }
      } else {
        run += csum[t];
      }
    }
  }
  return found;  // meaningful in thread 0
}

// One CTA per gene: histogram of the subsample errors on a sqrt scale, then
// the bin where the running count reaches k_sub gives X[g] (its upper edge
// widened by twice the error bound b0_g + b1 e of the candidate pass).
__global__ void __launch_bounds__(256) dist_threshold_kernel(const float* __restrict__ esub, int64_t n_sub,
                                                             int64_t G, int64_t k_sub, const float* b0, float b1,
                                                             float* X) {
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
  const int found = hist_find(hist, k_sub, csum);
  if (threadIdx.x == 0) {
    float x;
    if (found < 0 || k_sub <= 0) {
      x = INFINITY;
    } else {
      const float bg = b0[g];
      const float up = hist_upper(found);
      const float xp = up + 1.01f * (bg + b1 * up);
      x = xp + 1.01f * (bg + b1 * xp);
    }
    X[g] = x;
  }
}

cudaError_t launch_dist_threshold(const float* esub, int64_t n_sub, int64_t G, int64_t k_sub, const float* b0,
                                  float b1, float* X, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  dist_threshold_kernel<<<(unsigned)G, 256, 0, s>>>(esub, n_sub, G, k_sub, b0, b1, X);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// thresholds of the candidate pass and the refinement before the FP64 recheck
// ---------------------------------------------------------------------------

__global__ void fill_kernel(float* x, int64_t n, float v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

cudaError_t launch_fill(float* x, int64_t n, float v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, n, v);
  return cudaGetLastError();
}

// X_g for an error threshold e_g (eps, or thr[g]): every pair with err <= e_g
// has a candidate-pass error <= e_g + B_g(e_g) <= X_g = e_g + 2 B_g(e_g)
// (e_g rounded up to FP32 first).  e_g >= 10: every finite pair; e_g < 0: none.
__global__ void x_from_thr_kernel(const double* thr, double eps, int64_t G, const float* b0, float b1, float* X) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const double ev = thr ? thr[g] : eps;
  float x;
  if (ev >= 10.0) {
    x = INFINITY;
  } else if (ev < 0.0) {
    x = -1.0f;
  } else {
    const float e = __double2float_ru(ev);
    x = __fadd_ru(e, __fmul_ru(2.0f, __fmaf_ru(b1, e, b0[g])));
  }
  X[g] = x;
}

cudaError_t launch_x_from_thr(const double* thr, double eps, int64_t G, const float* b0, float b1, float* X,
                              cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  x_from_thr_kernel<<<(unsigned)((G + 255) / 256), 256, 0, s>>>(thr, eps, G, b0, b1, X);
  return cudaGetLastError();
}

// Histogram of the candidates' FP32 errors per gene (G x kHistBins counters).
__global__ void cand_hist_kernel(const Cand* cand, const float* e, int64_t n, unsigned int* hist) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = e[i];
    if (x == x) atomicAdd(&hist[(int64_t)cand[i].g * kHistBins + hist_bin(fmaxf(x, 0.0f))], 1u);
  }
}

// Per gene: when at least k candidates have an FP32 error <= a (the upper edge
// of the bin that completes k), k particles have err <= a' = (a + b0)/(1 - b1),
// so the k smallest errors are <= a', and every particle with err <= a' has an
// FP32 error <= a' + B(a').  Xt = a' + 2 B(a') keeps them all and passes the
// acceptance check (Xt - B(Xt) >= a' for b1 <= 1/2).  Xt never exceeds X.
// Only for a' < 10: at the clip value every particle beyond it ties at 10,
// whatever its unclipped error, so no tighter threshold is safe there.
__global__ void __launch_bounds__(256) refine_kernel(const unsigned int* hist, int64_t G, int64_t k, const float* X,
                                                     const float* b0, float b1, float* Xt) {
  __shared__ unsigned int csum[256];
  const int64_t g = blockIdx.x;
  const int found = hist_find(hist + g * kHistBins, k, csum);
  if (threadIdx.x == 0) {
    float x = X[g];
    if (found >= 0 && k > 0) {
      const float a = hist_upper(found);
      if (a < 10.0f) {
        const float bg = b0[g];
        const float a1 = __fdiv_ru(__fadd_ru(a, bg), __fsub_rd(1.0f, b1));
        const float xt = __fadd_ru(a1, __fmul_ru(2.0f, __fmaf_ru(b1, a1, bg)));
        if (a1 < 10.0f && xt < x) x = xt;
      }
    }
    Xt[g] = x;
  }
}

// Keep candidates with e <= Xt[g].  A block takes 4 x 256 candidates per
// iteration and appends its kept ones with one global atomic (positions from
// the warps' ballots), so the shared output counter sees one atomic per 1,024
// candidates instead of one per warp.
constexpr int kFilterItems = 4;
__global__ void __launch_bounds__(256) cand_filter_kernel(const Cand* cand, const float* e, int64_t n, const float* Xt,
                                                          Cand* out, unsigned long long* count) {
  __shared__ unsigned int wc[kFilterItems * 8];
  __shared__ unsigned long long base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t per = (int64_t)kFilterItems * blockDim.x;
  for (int64_t i0 = (int64_t)blockIdx.x * per; i0 < n; i0 += (int64_t)gridDim.x * per) {
    bool keep[kFilterItems];
    Cand cd[kFilterItems];
    unsigned m[kFilterItems];
#pragma unroll
    for (int j = 0; j < kFilterItems; ++j) {
      const int64_t i = i0 + (int64_t)j * blockDim.x + threadIdx.x;
      keep[j] = false;
      if (i < n) {
        cd[j] = cand[i];
        keep[j] = e[i] <= Xt[cd[j].g];
      }
      m[j] = __ballot_sync(0xffffffffu, keep[j]);
      if (lane == 0) wc[j * 8 + warp] = __popc(m[j]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // exclusive scan of the 32 warp counts, one reservation
      unsigned int run = 0;
      for (int q = 0; q < kFilterItems * 8; ++q) {
        const unsigned int v = wc[q];
        wc[q] = run;
        run += v;
      }
      base = run ? atomicAdd(count, (unsigned long long)run) : 0ull;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kFilterItems; ++j)
      if (keep[j]) out[base + wc[j * 8 + warp] + __popc(m[j] & ((1u << lane) - 1u))] = cd[j];
    __syncthreads();  // wc and base are rewritten by the next iteration
  }
}

__global__ void scatter_errors_kernel(const Cand* cand, const float* e, int64_t n, int64_t G, float* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[(int64_t)cand[i].p * G + cand[i].g] = e[i];
}

cudaError_t launch_scatter_errors(const Cand* cand, const float* e, int64_t n, int64_t G, float* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)((n + 255) / 256 < 16384 ? (n + 255) / 256 : 16384);
  scatter_errors_kernel<<<blocks, 256, 0, s>>>(cand, e, n, G, out);
  return cudaGetLastError();
}

cudaError_t launch_refine(const Cand* cand, const float* cand_e, int64_t n, int64_t G, int64_t k, const float* X,
                          const float* b0, float b1, unsigned int* hist, float* Xt, Cand* out,
                          unsigned long long* count, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(unsigned int) * (size_t)G * kHistBins, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (G <= 0) return cudaSuccess;
  const int blocks = (int)((n + 255) / 256 < 16384 ? (n + 255) / 256 : 16384);
  if (n > 0) cand_hist_kernel<<<blocks, 256, 0, s>>>(cand, cand_e, n, hist);
  refine_kernel<<<(unsigned)G, 256, 0, s>>>(hist, G, k, X, b0, b1, Xt);
  if (n > 0) cand_filter_kernel<<<blocks, 256, 0, s>>>(cand, cand_e, n, Xt, out, count);
  return cudaGetLastError();
}


// Surrogate screen of particle p against gene g under the predicted
// statistics (mean mu_pk, predictive std sd_pk), a = sqrt(w_gk):
//   mode 0, per-statistic lower bound
//     L_pg = sum_k max(0, |a (d_gk - mu_pk)| - z a sd_pk)^2 / K;
//   mode 1, lower quantile of the error's predictive distribution: with
//     s_pk ~ N(mu_pk, sd_pk^2) independent, err = sum_k a^2 (d - s)^2 / K has
//     mean m = sum_k (delta^2 + sig^2) / K and variance
//     v = sum_k (2 sig^4 + 4 sig^2 delta^2) / K^2 (delta = a (d - mu),
//     sig = a sd), and L_pg = m - z sqrt(v).
// keep[p] = 1 when L_pg <= X[g] for some gene (X = calibrated threshold).  A
// draw is dropped only when it is confidently far from every gene.  Same
// 128 x 128 tiling as dist_fast_kernel.
template <int MODE>
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
  constexpr int N2 = MODE ? 8 : 1;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t g0 = (int64_t)blockIdx.x * kDistTile;
  const int64_t p0 = (int64_t)blockIdx.y * kDistTile;
  float acc[8][8], acc2[N2][N2];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
#pragma unroll
  for (int i = 0; i < N2; ++i)
#pragma unroll
    for (int j = 0; j < N2; ++j) acc2[i][j] = 0.0f;
  for (int k0 = 0; k0 < K; k0 += kDistKc) {
    for (int idx = threadIdx.x; idx < kDistKc * kDistTile; idx += 256) {
      const int r = idx / kDistKc, kk = idx - (idx / kDistKc) * kDistKc;
      const int k = k0 + kk;
      const int64_t p = p0 + r, g = g0 + r;
      float m = 0.0f, v = 0.0f, a = 0.0f, d = 0.0f;
      if (p < P && k < K) {
        m = mu[p * K + k];
        v = sqrtf(fmaxf(var[p * K + k], 0.0f));  // predictive std
        if (MODE == 0) v *= z;
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
          if (MODE == 0) {
            const float t = fmaxf(fabsf(fmaf(-a[j], m[i], d[j])) - a[j] * v[i], 0.0f);
            acc[i][j] = fmaf(t, t, acc[i][j]);
          } else {
            const float dl = fmaf(-a[j], m[i], d[j]);
            const float sg = a[j] * v[i];
            const float s2 = sg * sg, d2 = dl * dl;
            acc[i][j] += d2 + s2;
            acc2[i & (N2 - 1)][j & (N2 - 1)] = fmaf(s2, fmaf(4.0f, d2, 2.0f * s2), acc2[i & (N2 - 1)][j & (N2 - 1)]);
          }
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
      // not clipped: far draws keep large predicted errors
      float e = acc[i][j] * invK;
      if (MODE == 1) e -= z * sqrtf(acc2[i & (N2 - 1)][j & (N2 - 1)]) * invK;
      if (err_out) err_out[p * G + g] = e;
      any = any || (e <= X[g]);
    }
    if (any) keep[p] = 1;
  }
}

cudaError_t launch_dist_screen(const float* mu, const float* var, const float* sw, const float* dw, int64_t P,
                               int64_t G, int K, const float* X, float z, int mode, uint8_t* keep, float* err_out,
                               cudaStream_t s) {
  if (P <= 0 || G <= 0) return cudaSuccess;
  dim3 grid((unsigned)((G + kDistTile - 1) / kDistTile), (unsigned)((P + kDistTile - 1) / kDistTile));
  if (mode == 1)
    dist_screen_kernel<1><<<grid, 256, 0, s>>>(mu, var, sw, dw, P, G, K, X, z, keep, err_out);
  else
    dist_screen_kernel<0><<<grid, 256, 0, s>>>(mu, var, sw, dw, P, G, K, X, z, keep, err_out);
  return cudaGetLastError();
}

}  // namespace abc
