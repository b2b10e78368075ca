// distance_fp64.cu — FP64 side of the distance step: weight preparation, the
// exact recheck in the reference's operation order (bit-identical to the
// oracle; built with -fmad=false), the full FP64 error matrix, and the
// per-gene grouping and (err, index) sort of accepted particles
// (scripts/accepted_particles.jl:20-26: findall + sortperm).
#include "distance.cuh"
#include "kernels.h"

namespace abc {

// sw, dw for every (g, k); s32[r][k] = stats[r * stride][k] for r < s32_rows.
__global__ void dist_prep_kernel(DistInputs in, float* sw, float* dw, float* s32, int64_t s32_rows,
                                 int64_t stride) {
  const int64_t n_gk = in.G * in.K;
  const int64_t n_pk = s32 ? s32_rows * in.K : 0;
  const double sig2 = 0.1 * 0.1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_gk + n_pk;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n_gk) {
      const double d = in.data[i], e = in.se[i];
      const double eps = (e + d != 0.0) ? 0.0 : 0.0001;
      const double w = 1.0 / ((e * e + sig2 * (d * d)) + eps);
      const double a = sqrt(w);
      sw[i] = (float)a;
      dw[i] = (float)(a * d);
    } else {
      const int64_t j = i - n_gk;
      const int64_t r = j / in.K, k = j - r * in.K;
      s32[j] = (float)in.stats[(r * stride) * in.K + k];
    }
  }
}

cudaError_t launch_dist_prep(const DistInputs& in, float* sw, float* dw, float* s32, int64_t s32_rows,
                             int64_t stride, cudaStream_t s) {
  const int64_t n = in.G * in.K + (s32 ? s32_rows * in.K : 0);
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
  dist_prep_kernel<<<blocks, 256, 0, s>>>(in, sw, dw, s32, s32_rows, stride);
  return cudaGetLastError();
}

__device__ __forceinline__ double den_term(double d, double e) {
  const double sig2 = 0.1 * 0.1;
  const double eps = (e + d != 0.0) ? 0.0 : 0.0001;
  return (e * e + sig2 * (d * d)) + eps;
}

__global__ void dist_den_kernel(DistInputs in, double* den, double* rden) {
  const int64_t n = in.G * in.K;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double b = den_term(in.data[i], in.se[i]);
    den[i] = b;
    rden[i] = 1.0 / b;
  }
}

cudaError_t launch_dist_den(const DistInputs& in, double* den, double* rden, cudaStream_t s) {
  const int64_t n = in.G * in.K;
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  dist_den_kernel<<<blocks, 256, 0, s>>>(in, den, rden);
  return cudaGetLastError();
}

// err of one (p, g) pair exactly as compute_trunc_errors / nlsqerror_part
// (scripts/compute_errors.jl:30-43): per family, sum of diff^2 / den in
// order, then part / K added to the total; clipped at 10.
__device__ __forceinline__ double err_exact(const DistInputs& in, int64_t p, int64_t g) {
  const double* s = in.stats + p * in.K;
  const double* d = in.data + g * in.K;
  const double* e = in.se + g * in.K;
  const double nK = (double)in.K;
  double tot = 0.0;
  int k = 0;
  if (in.den) {
    const double* dn = in.den + g * in.K;
    const double* ry = in.rden + g * in.K;
    const double rK = 1.0 / nK;
    for (int f = 0; f < in.n_fam; ++f) {
      double part = 0.0;
      for (int q = 0; q < in.fam[f]; ++q, ++k) {
        const double diff = d[k] - s[k];
        part = part + div_rn(diff * diff, dn[k], ry[k]);
      }
      tot = tot + div_rn(part, nK, rK);
    }
  } else {
    for (int f = 0; f < in.n_fam; ++f) {
      double part = 0.0;
      for (int q = 0; q < in.fam[f]; ++q, ++k) {
        const double diff = d[k] - s[k];
        part = part + (diff * diff) / den_term(d[k], e[k]);
      }
      tot = tot + part / nK;
    }
  }
  if (tot > 10.0) tot = 10.0;
  return tot;
}

__global__ void dist_recheck_kernel(DistInputs in, const Cand* cand, int64_t n, double* e64) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Cand c = cand[i];
    e64[i] = err_exact(in, c.p, c.g);
  }
}

cudaError_t launch_dist_recheck(const DistInputs& in, const Cand* cand, int64_t n, double* e64, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 127) / 128 < 65536 ? (n + 127) / 128 : 65536);
  dist_recheck_kernel<<<blocks, 128, 0, s>>>(in, cand, n, e64);
  return cudaGetLastError();
}

__global__ void dist_full_kernel(DistInputs in, double* err) {
  const int64_t n = in.P * in.G;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / in.G, g = i - (i / in.G) * in.G;
    err[i] = err_exact(in, p, g);
  }
}

cudaError_t launch_dist_full(const DistInputs& in, double* err, cudaStream_t s) {
  const int64_t n = in.P * in.G;
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
  dist_full_kernel<<<blocks, 256, 0, s>>>(in, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// grouping by gene: count, exclusive scan, scatter
// ---------------------------------------------------------------------------
__global__ void gene_count_kernel(const Cand* cand, int64_t n, int64_t* gcount) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd((unsigned long long*)&gcount[cand[i].g], 1ull);
}

__global__ void __launch_bounds__(1024) scan_kernel(const int64_t* cnt, int64_t G, int64_t* off) {
  __shared__ int64_t part[1024];
  const int64_t per = (G + 1023) / 1024;
  const int64_t b = threadIdx.x * per;
  int64_t s = 0;
  for (int64_t i = b; i < b + per && i < G; ++i) s += cnt[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int t = 0; t < 1024; ++t) {
      int64_t v = part[t];
      part[t] = run;
      run += v;
    }
  }
  __syncthreads();
  int64_t run = part[threadIdx.x];
  for (int64_t i = b; i < b + per && i < G; ++i) {
    off[i] = run;
    run += cnt[i];
  }
  if (b + per >= G && b < G) off[G] = run;
  if (G == 0 && threadIdx.x == 0) off[0] = 0;
}

__global__ void scatter_kernel(const Cand* cand, const double* e64, int64_t n, const int64_t* goff,
                               unsigned long long* cursor, int32_t* sp, double* se64) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Cand c = cand[i];
    unsigned long long pos = (unsigned long long)goff[c.g] + atomicAdd(&cursor[c.g], 1ull);
    sp[pos] = c.p;
    se64[pos] = e64[i];
  }
}

// Per-gene sort by (err, p): bitonic network in its all-ascending form, so
// that padding the segment to a power of two with +inf needs no storage (a
// real element is never exchanged with a padding slot).  NaN sorts last.
__device__ __forceinline__ bool key_less(double ea, int32_t pa, double eb, int32_t pb) {
  const bool na = ea != ea, nb = eb != eb;
  if (na != nb) return nb;
  if (na) return pa < pb;
  return ea < eb || (ea == eb && pa < pb);
}

constexpr int kSortSmem = 8192;  // segments up to this size sort in shared memory

__global__ void __launch_bounds__(1024) segsort_kernel(const int64_t* goff, int32_t* sp, double* se64) {
  extern __shared__ double sort_smem[];
  const int64_t g = blockIdx.x;
  const int64_t base = goff[g];
  const int64_t n = goff[g + 1] - base;
  if (n <= 1) return;
  int32_t* P = sp + base;
  double* E = se64 + base;
  int64_t n2 = 1;
  while (n2 < n) n2 <<= 1;
  if (n2 <= kSortSmem) {
    double* Es = sort_smem;
    int32_t* Ps = reinterpret_cast<int32_t*>(sort_smem + kSortSmem);
    const int m = (int)n;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      Es[i] = E[i];
      Ps[i] = P[i];
    }
    __syncthreads();
    for (int k = 2; k <= (int)n2; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < (int)n2; i += blockDim.x) {
          const int partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
          if (partner > i && partner < m) {
            const double ea = Es[i], eb = Es[partner];
            const int32_t pa = Ps[i], pb = Ps[partner];
            if (key_less(eb, pb, ea, pa)) {
              Es[i] = eb;
              Es[partner] = ea;
              Ps[i] = pb;
              Ps[partner] = pa;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      E[i] = Es[i];
      P[i] = Ps[i];
    }
    return;
  }
  for (int64_t k = 2; k <= n2; k <<= 1) {
    for (int64_t j = k >> 1; j > 0; j >>= 1) {
      for (int64_t i = threadIdx.x; i < n2; i += blockDim.x) {
        int64_t partner;
        if (j == (k >> 1))
          partner = i ^ (k - 1);  // flip step
        else
          partner = i ^ j;
        if (partner > i && partner < n) {
          double ea = E[i], eb = E[partner];
          int32_t pa = P[i], pb = P[partner];
          if (key_less(eb, pb, ea, pa)) {
            E[i] = eb;
            E[partner] = ea;
            P[i] = pb;
            P[partner] = pa;
          }
        }
      }
      __syncthreads();
    }
  }
}

cudaError_t launch_dist_group_sort(const Cand* cand, const double* e64, int64_t n, int64_t G, int64_t* gcount,
                                   int64_t* goff, int32_t* sp, double* se64, unsigned long long* gcursor,
                                   cudaStream_t s) {
  cudaError_t err = cudaMemsetAsync(gcount, 0, sizeof(int64_t) * (size_t)G, s);
  if (err) return err;
  err = cudaMemsetAsync(gcursor, 0, sizeof(unsigned long long) * (size_t)G, s);
  if (err) return err;
  if (n > 0) {
    int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
    gene_count_kernel<<<blocks, 256, 0, s>>>(cand, n, gcount);
  }
  scan_kernel<<<1, 1024, 0, s>>>(gcount, G, goff);
  if (n > 0) {
    int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
    scatter_kernel<<<blocks, 256, 0, s>>>(cand, e64, n, goff, gcursor, sp, se64);
    constexpr int smem = kSortSmem * (int)(sizeof(double) + sizeof(int32_t));
    static bool attr = false;
    if (!attr) {
      err = cudaFuncSetAttribute(segsort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (err) return err;
      attr = true;
    }
    segsort_kernel<<<(unsigned)G, 1024, smem, s>>>(goff, sp, se64);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// accepted prefixes
// ---------------------------------------------------------------------------
__global__ void accept_len_kernel(const int64_t* goff, const double* se64, int64_t G, int mode, double eps_all,
                                  const double* eps_g, int64_t k, const float* X, const float* b0, float b1,
                                  int64_t* alen, int* fail) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const double eps = eps_g ? eps_g[g] : eps_all;
  const double* E = se64 + goff[g];
  const int64_t n = goff[g + 1] - goff[g];
  // number of finite (non-NaN) entries: NaN sorts last
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (E[mid] == E[mid]) lo = mid + 1; else hi = mid;
  }
  const int64_t nn = lo;
  int64_t len;
  if (mode == 0) {
    lo = 0;
    hi = nn;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (E[mid] <= eps) lo = mid + 1; else hi = mid;
    }
    len = lo;
  } else {
    len = nn < k ? nn : k;
    const float x = X[g];
    bool ok;
    if (!(x < INFINITY)) {
      ok = true;  // every particle was a candidate
    } else if (len < k) {
      ok = false;
    } else {
      // every particle with err <= L had a candidate-pass error <= X
      const double L = (double)x - ((double)b0[g] + (double)b1 * (double)x);
      ok = E[k - 1] <= L;
    }
    if (!ok) fail[g] = 1;
  }
  alen[g] = len;
}

cudaError_t launch_dist_accept_len(const int64_t* goff, const double* se64, int64_t G, int mode, double eps,
                                   const double* eps_g, int64_t k, const float* X, const float* b0, float b1,
                                   int64_t* alen, int* fail, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  accept_len_kernel<<<(unsigned)((G + 127) / 128), 128, 0, s>>>(goff, se64, G, mode, eps, eps_g, k, X, b0, b1,
                                                                alen, fail);
  return cudaGetLastError();
}

__global__ void compact_kernel(const int64_t* goff, const int32_t* sp, const double* se64, const int64_t* aoff,
                               int64_t G, int64_t p_base, int64_t* idx, double* err) {
  const int64_t g = blockIdx.x;
  const int64_t src = goff[g], dst = aoff[g], n = aoff[g + 1] - aoff[g];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    idx[dst + i] = (int64_t)sp[src + i] + p_base + 1;
    if (err) err[dst + i] = se64[src + i];
  }
}

cudaError_t launch_dist_compact(const int64_t* goff, const int32_t* sp, const double* se64, const int64_t* aoff,
                                int64_t G, int64_t p_base, int64_t* idx, double* err, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  compact_kernel<<<(unsigned)G, 256, 0, s>>>(goff, sp, se64, aoff, G, p_base, idx, err);
  return cudaGetLastError();
}

cudaError_t launch_scan(const int64_t* cnt, int64_t G, int64_t* off, cudaStream_t s) {
  scan_kernel<<<1, 1024, 0, s>>>(cnt, G, off);
  return cudaGetLastError();
}

}  // namespace abc
