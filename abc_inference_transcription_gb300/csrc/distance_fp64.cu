// distance_fp64.cu — FP64 side of the distance step: weight preparation, the
// exact recheck in the reference's operation order (bit-identical to the
// oracle; built with -fmad=false), the full FP64 error matrix, and the
// per-gene grouping and (err, index) sort of accepted particles
// (scripts/accepted_particles.jl:20-26: findall + sortperm).
#include <algorithm>
#include <atomic>

#include "bitonic.cuh"
#include "smem_attr.h"
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

// FP64 errors of candidates already grouped by gene (sp, sg: particle and gene
// of each entry).  A warp takes 32 consecutive entries and walks the
// statistics in chunks of kRecheckCols columns: it copies the chunk of its 32
// rows into shared memory with coalesced loads (consecutive lanes read
// consecutive values, rows back to back), then each lane adds its pair's terms
// of that chunk from shared memory, carrying the family sums across chunks.
// The gene rows it reads (data, den, rden) are mostly the same for the whole
// warp and are broadcast.  Row stride kRecheckCols + 1 (odd) keeps the lanes'
// column reads on distinct banks; the small chunk keeps 32 warps resident per
// SM, enough to keep the FP64 pipe (the bound: six FP64 operations per term)
// busy.
constexpr int kRecheckWarps = 8;
constexpr int kRecheckCols = 24;
constexpr int kRecheckLd = kRecheckCols + 1;

__global__ void __launch_bounds__(kRecheckWarps * 32) recheck_grouped_kernel(DistInputs in, const int32_t* sp,
                                                                             const int32_t* sg, int64_t n,
                                                                             double* se64) {
  __shared__ double rs_smem[kRecheckWarps * 32 * kRecheckLd];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int K = in.K;
  double* S = rs_smem + warp * 32 * kRecheckLd;
  const double nK = (double)K;
  const double rK = 1.0 / nK;
  const int64_t n_chunks = (n + 31) >> 5;
  const int64_t wstride = (int64_t)gridDim.x * kRecheckWarps;
  for (int64_t ch = (int64_t)blockIdx.x * kRecheckWarps + warp; ch < n_chunks; ch += wstride) {
    const int64_t i = ch * 32 + lane;
    const bool mine = i < n;
    const int32_t p = mine ? sp[i] : 0;
    const int64_t g = mine ? sg[i] : 0;
    const int rows = (int)(n - ch * 32 < 32 ? n - ch * 32 : 32);
    const double* d = in.data + g * K;
    const double* dn = in.den + g * K;
    const double* ry = in.rden + g * K;
    double tot = 0.0, part = 0.0;
    // families: f is the open one, fend the column after its last term
    int f = 0, fend = in.fam[0];
    while (fend == 0 && f < in.n_fam) {  // leading empty families add 0 / K
      tot = tot + div_rn(part, nK, rK);
      ++f;
      fend = f < in.n_fam ? fend + in.fam[f] : -1;
    }
    for (int c0 = 0; c0 < K; c0 += kRecheckCols) {
      const int cw = K - c0 < kRecheckCols ? K - c0 : kRecheckCols;
      // flat copy of rows x cw values: lane takes e = lane + 32 t, (r, c) = divmod(e, cw)
      const int T = (rows * cw + 31) >> 5;
      int r = lane / cw, c = lane - (lane / cw) * cw;
      for (int t0 = 0; t0 < T; t0 += 8) {
        double v[8];
        int dst[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int32_t pr = __shfl_sync(0xffffffffu, p, r < 31 ? r : 31);
          const bool take = t0 + u < T && r < rows;
          dst[u] = take ? r * kRecheckLd + c : -1;
          v[u] = take ? __ldg(in.stats + (int64_t)pr * K + c0 + c) : 0.0;
          c += 32;
          while (c >= cw) {
            c -= cw;
            ++r;
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (dst[u] >= 0) S[dst[u]] = v[u];
      }
      __syncwarp();
      if (mine) {
        const double* s = S + lane * kRecheckLd - c0;
        for (int k = c0; k < c0 + cw; ++k) {
          const double diff = __ldg(d + k) - s[k];
          part = part + div_rn(diff * diff, __ldg(dn + k), __ldg(ry + k));
          while (k + 1 == fend) {  // close this family and any empty ones after it
            tot = tot + div_rn(part, nK, rK);
            part = 0.0;
            ++f;
            fend = f < in.n_fam ? fend + in.fam[f] : -1;
          }
        }
      }
      __syncwarp();
    }
    if (mine) {
      if (tot > 10.0) tot = 10.0;
      se64[i] = tot;
    }
  }
}

// ---------------------------------------------------------------------------
// Certified FP32 errors for selections that return indices only
// ---------------------------------------------------------------------------
// A candidate's error is evaluated in FP32 from two-float splits of its FP64
// inputs: x = h + l with |x - h - l| <= 2^-47 |x|, |l| <= 2^-23 |x| (data: h =
// RN32(x), l = RN32(x - h); statistics: h = the top 24 significand bits,
// exact integer bit manipulation, l = the remaining 29 bits rounded to float).
// With r = 1/den rounded to float, u = 2^-24:
//   delta = RN(RN(dh - sh) + RN(dl - sl))       (the hi parts cancel exactly)
//   T     = RN(delta RN(delta r))               per statistic
//   S     = Kahan sum of the T, e = RN(S RN(1/K))
// and, writing T* = (d - s)^2 / den for the exact term and a = den^-1/2 (so
// a |d| <= 10 because den >= 0.01 d^2): |delta - (d - s)| <= 2.0001 u |d - s| +
// 2^-45.4 (|d| + |s|), hence |T - T*| <= 7.03 u T* + 2^-44.4 (20 sqrt(T*) + T*)
// + 2^-90 (20 + sqrt(T*))^2; Kahan summation adds <= 2.1 u sum T, the final
// scaling 2.01 u, and the reference's FP64 evaluation differs from the exact
// value by < 1e-14 relative.  Altogether |e - err64| <= 11.2 u err +
// 2^-40 sqrt(err) + 2^-80; 1e-6 e + 1.5e-12 sqrt(e + 1e-12) covers that with a
// 1.5x margin, and approx_bound uses its linear majorant (1e-6 + 1e-12) e +
// 1e-12 (sqrt(x) <= (1 + x) / 2), one FMA instead of an FP64 square root;
// v - B(v) and v + B(v) are increasing in v.  The derivation
// needs every |d|, |s| in {0} u [2^-60, 2^60] (no underflow in the splits),
// den in [2^-120, 2^120] (1/den a normal float; an underflow in delta r then
// costs at most 2^-88 per term, far inside the bound's absolute part) and a
// finite result; other pairs are computed in FP64.
__device__ __forceinline__ bool key_less(double ea, int32_t pa, double eb, int32_t pb);
__device__ __forceinline__ double approx_bound(double v) { return fma(1.000001e-6, v, 1e-12); }

// x = h + l by truncation of the significand, on the two 32-bit halves of x
// (integer operations only): h keeps the sign, the exponent rebiased from 1023
// to 127 and the top 23 stored significand bits; l is the remaining 29 bits
// rounded to float and scaled by 2^(e - 1075).
__device__ __forceinline__ bool split_trunc(double x, float& h, float& l) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned mag = hi & 0x7fffffffu, sign = hi & 0x80000000u;
  const unsigned e = mag >> 20;
  const bool zero = (mag | lo) == 0u;
  const bool ok = zero || e - (1023u - 60u) <= 120u;  // exponent in [-60, 60]
  // ((e - 896) << 23) | (top 20 bits << 3) | (next 3 bits): the float's exponent and significand
  h = __uint_as_float(zero ? 0u : (sign | ((mag - (896u << 20)) << 3) | (lo >> 29)));
  const float r = __uint2float_rn(lo & 0x1fffffffu);
  const float scale = __uint_as_float(((e - 948u) & 0xffu) << 23);  // 2^(e - 1075); garbage when !ok
  l = zero ? 0.0f : __uint_as_float(__float_as_uint(__fmul_rn(r, scale)) | sign);
  return ok;
}

// per (gene, statistic): (h, l, 1/den, 0) with d = h + l
__global__ void ff_prep_genes_kernel(DistInputs in, float4* gt) {
  const int64_t n = in.G * in.K;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = in.data[i], den = in.den[i];
    const double ad = fabs(d);
    const bool ok = (d == 0.0 || (ad >= 0x1p-60 && ad <= 0x1p60)) && den >= 0x1p-120 && den <= 0x1p120;
    const float h = (float)d;
    gt[i] = make_float4(h, (float)(d - (double)h), ok ? (float)in.rden[i] : __int_as_float(0x7fc00000), 0.0f);
  }
}

// Candidates grouped by gene, statistics rows staged as in
// recheck_grouped_kernel.  v[i] = the certified FP32 error (10 exactly when
// it lies above 10 by more than its bound); pairs outside the derivation's
// range get their position appended to pos (FP64 later).
__global__ void __launch_bounds__(kRecheckWarps * 32) approx_grouped_kernel(DistInputs in, const int32_t* sp,
                                                                            const int32_t* sg, int64_t n,
                                                                            const float4* gt, float rK, double* v,
                                                                            int32_t* pos,
                                                                            unsigned long long* count) {
  __shared__ double rs_smem[kRecheckWarps * 32 * kRecheckLd];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int K = in.K;
  double* S = rs_smem + warp * 32 * kRecheckLd;
  const int64_t n_chunks = (n + 31) >> 5;
  const int64_t wstride = (int64_t)gridDim.x * kRecheckWarps;
  for (int64_t ch = (int64_t)blockIdx.x * kRecheckWarps + warp; ch < n_chunks; ch += wstride) {
    const int64_t i = ch * 32 + lane;
    const bool mine = i < n;
    const int32_t p = mine ? sp[i] : 0;
    const int64_t g = mine ? sg[i] : 0;
    const int rows = (int)(n - ch * 32 < 32 ? n - ch * 32 : 32);
    const float4* gk = gt + g * K;
    float acc = 0.0f, comp = 0.0f;
    bool ok = true;
    for (int c0 = 0; c0 < K; c0 += kRecheckCols) {
      const int cw = K - c0 < kRecheckCols ? K - c0 : kRecheckCols;
      const int T = (rows * cw + 31) >> 5;
      int r = lane / cw, c = lane - (lane / cw) * cw;
      for (int t0 = 0; t0 < T; t0 += 8) {
        double vv[8];
        int dst[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int32_t pr = __shfl_sync(0xffffffffu, p, r < 31 ? r : 31);
          const bool take = t0 + u < T && r < rows;
          dst[u] = take ? r * kRecheckLd + c : -1;
          vv[u] = take ? __ldg(in.stats + (int64_t)pr * K + c0 + c) : 0.0;
          c += 32;
          while (c >= cw) {
            c -= cw;
            ++r;
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (dst[u] >= 0) S[dst[u]] = vv[u];
      }
      __syncwarp();
      if (mine) {
        const double* s = S + lane * kRecheckLd - c0;
        for (int k = c0; k < c0 + cw; ++k) {
          float sh, sl;
          ok = split_trunc(s[k], sh, sl) && ok;
          const float4 q = __ldg(gk + k);
          const float x = __fsub_rn(q.x, sh);
          const float y = __fsub_rn(q.y, sl);
          const float dd = __fadd_rn(x, y);
          const float term = __fmul_rn(dd, __fmul_rn(dd, q.z));
          const float yk = __fsub_rn(term, comp);
          const float t = __fadd_rn(acc, yk);
          comp = __fsub_rn(__fsub_rn(t, acc), yk);
          acc = t;
        }
      }
      __syncwarp();
    }
    if (mine) {
      const float e = __fmul_rn(acc, rK);
      ok = ok && e == e && e < INFINITY;
      if (ok) {
        const double ed = (double)e;
        v[i] = ed - approx_bound(ed) >= 10.0 ? 10.0 : ed;
      } else {
        v[i] = 0.0;
        pos[atomicAdd(count, 1ull)] = (int32_t)i;
      }
    }
  }
}

// E[pos[j]] = the FP64 error of the pair at that position, j < *count
__global__ void recheck_list_kernel(DistInputs in, const int32_t* sp, const int32_t* sg, const int32_t* pos,
                                    const unsigned long long* count, double* E) {
  const int64_t m = (int64_t)*count;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = pos[j];
    E[i] = err_exact(in, sp[i], sg[i]);
  }
}

// After the sort by the certified values: a position whose interval
// [v - B(v), v + B(v)] overlaps a neighbour's in its gene's list, or holds
// the clip value 10 or the gene's threshold (modes 0 and 2), is appended to pos
// and its gene marked dirty.  Intervals have increasing ends along the sorted
// list, so an interval that overlaps no neighbour overlaps no other; every
// other pair is then in its exact place, and exact values for the listed
// pairs plus one more sort give the exact order.
__global__ void ambiguous_kernel(const int32_t* sg, const int64_t* goff, const double* E, int64_t n, int mode,
                                 double eps_all, const double* eps_g, int32_t* pos, unsigned long long* count,
                                 uint8_t* flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = E[i];
    if (v != v) continue;  // NaN: exact (FP64 path), sorts last
    const int64_t g = sg[i];
    const int64_t a = goff[g], b = goff[g + 1];
    const double B = approx_bound(v);
    bool amb = fabs(v - 10.0) <= B;
    if (i > a) {
      const double w = E[i - 1];
      if (w == w && w + approx_bound(w) >= v - B) amb = true;
    }
    if (i + 1 < b) {
      const double w = E[i + 1];
      if (w == w && v + B >= w - approx_bound(w)) amb = true;
    }
    if (mode != 1) {
      const double thr = eps_g ? eps_g[g] : eps_all;
      if (fabs(v - thr) <= B) amb = true;
    }
    flag[i] = amb ? 1 : 0;
    if (amb) pos[atomicAdd(count, 1ull)] = (int32_t)i;
  }
}

// After the FP64 values of the flagged positions are in: every maximal run
// of consecutive flagged positions in a gene's list is sorted in place by
// (err, p) (the neighbours of a run have intervals wholly below or above it,
// so nothing else moves); a run longer than kRunSort marks its gene for a
// full re-sort instead.
constexpr int kRunSort = 64;

__global__ void run_sort_kernel(const int32_t* sg, const int64_t* goff, const uint8_t* flag, int64_t n,
                                int32_t* sp, double* E, int* dirty) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[i]) continue;
    const int64_t g = sg[i];
    const int64_t a = goff[g], b = goff[g + 1];
    if (i > a && flag[i - 1]) continue;  // not the start of a run
    int64_t e = i + 1;
    while (e < b && flag[e] && e - i <= kRunSort) ++e;
    if (e - i > kRunSort) {
      dirty[g] = 1;
      continue;
    }
    for (int64_t j = i + 1; j < e; ++j) {  // insertion sort
      const double x = E[j];
      const int32_t px = sp[j];
      int64_t k = j - 1;
      while (k >= i && key_less(x, px, E[k], sp[k])) {
        E[k + 1] = E[k];
        sp[k + 1] = sp[k];
        --k;
      }
      E[k + 1] = x;
      sp[k + 1] = px;
    }
  }
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

// The same count with a per-block histogram in shared memory (G counters):
// one global atomic per (block, gene) instead of one per candidate, which
// all land on a few thousand addresses.
__global__ void __launch_bounds__(256) gene_count_smem_kernel(const Cand* cand, int64_t n, int G, int64_t chunk,
                                                              int64_t* gcount) {
  extern __shared__ unsigned int h[];
  for (int g = threadIdx.x; g < G; g += blockDim.x) h[g] = 0u;
  __syncthreads();
  const int64_t b0 = (int64_t)blockIdx.x * chunk, b1 = b0 + chunk < n ? b0 + chunk : n;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) atomicAdd(&h[cand[i].g], 1u);
  __syncthreads();
  for (int g = threadIdx.x; g < G; g += blockDim.x)
    if (h[g]) atomicAdd((unsigned long long*)&gcount[g], (unsigned long long)h[g]);
}

// Scatter of a contiguous chunk per block: local counts per gene, one global
// reservation per (block, gene), then positions from shared-memory atomics.
__global__ void __launch_bounds__(256) scatter_smem_kernel(const Cand* cand, int64_t n, int G, int64_t chunk,
                                                           const int64_t* goff, unsigned long long* cursor,
                                                           int32_t* sp, int32_t* sg) {
  extern __shared__ unsigned long long sb[];  // G reserved bases, then G local counters
  unsigned int* cnt = reinterpret_cast<unsigned int*>(sb + G);
  for (int g = threadIdx.x; g < G; g += blockDim.x) cnt[g] = 0u;
  __syncthreads();
  const int64_t b0 = (int64_t)blockIdx.x * chunk, b1 = b0 + chunk < n ? b0 + chunk : n;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) atomicAdd(&cnt[cand[i].g], 1u);
  __syncthreads();
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const unsigned int c = cnt[g];
    sb[g] = c ? (unsigned long long)goff[g] + atomicAdd(&cursor[g], (unsigned long long)c) : 0ull;
    cnt[g] = 0u;
  }
  __syncthreads();
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const Cand c = cand[i];
    const unsigned long long pos = sb[c.g] + atomicAdd(&cnt[c.g], 1u);
    sp[pos] = c.p;
    sg[pos] = c.g;
  }
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

__global__ void scatter_kernel(const Cand* cand, int64_t n, const int64_t* goff, unsigned long long* cursor,
                               int32_t* sp, int32_t* sg) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Cand c = cand[i];
    unsigned long long pos = (unsigned long long)goff[c.g] + atomicAdd(&cursor[c.g], 1ull);
    sp[pos] = c.p;
    sg[pos] = c.g;
  }
}

// Per-gene sort by (err, p), NaN last, ties by index.  Segments up to
// kSortSmem entries run the register-resident bitonic network of bitonic.cuh
// (EPT = n2 / 1024 entries per thread, n2 the padded power of two) on keys
// that are the bit patterns of the errors (monotone for the non-negative
// errors; NaN canonicalised to one pattern) with the index as tie-break;
// padding slots carry (all ones, INT32_MAX), above every real entry.  Longer
// segments run the same network on (err, p) in global memory.
__device__ __forceinline__ bool key_less(double ea, int32_t pa, double eb, int32_t pb) {
  const bool na = ea != ea, nb = eb != eb;
  if (na != nb) return nb;
  if (na) return pa < pb;
  return ea < eb || (ea == eb && pa < pb);
}

constexpr int kSortSmem = 8192;  // segments up to this size sort in registers
constexpr uint64_t kNanKey = 0x7ff8000000000000ull;

__device__ __forceinline__ uint64_t err_key(double e) {
  if (e != e) return kNanKey;
  if (e == 0.0) return 0ull;  // +0 and -0
  return (uint64_t)__double_as_longlong(e);
}

template <int EPT>
__device__ void sort_segment_regs(int32_t* P, double* E, int m, int n2, uint64_t* sK, int32_t* sP) {
  const int t = threadIdx.x;
  const int nt = n2 / EPT > 32 ? n2 / EPT : 32;  // threads holding entries
  const bool act = t < nt;
  uint64_t key[EPT];
  int32_t pp[EPT];
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const int i = t * EPT + e;
    const bool real = act && i < m;
    key[e] = real ? err_key(E[i]) : ~0ull;
    pp[e] = real ? P[i] : 0x7fffffff;
  }
  bitonic_regs<EPT>(key, pp, n2, sK, sP);
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const int i = t * EPT + e;
    if (act && i < m) {
      E[i] = __longlong_as_double((long long)key[e]);
      P[i] = pp[e];
    }
  }
}

__global__ void __launch_bounds__(1024, 1) segsort_kernel(const int64_t* goff, int32_t* sp, double* se64,
                                                          const int* dirty) {
  extern __shared__ uint64_t sort_smem[];
  const int64_t g = blockIdx.x;
  if (dirty && !dirty[g]) return;
  const int64_t base = goff[g];
  const int64_t n = goff[g + 1] - base;
  if (n <= 1) return;
  int32_t* P = sp + base;
  double* E = se64 + base;
  int64_t n2 = 1;
  while (n2 < n) n2 <<= 1;
  if (n2 <= kSortSmem) {
    uint64_t* sK = sort_smem;
    int32_t* sP = reinterpret_cast<int32_t*>(sort_smem + kSortSmem);
    const int m = (int)n, w = (int)n2;
    if (w <= 1024) sort_segment_regs<1>(P, E, m, w, sK, sP);
    else if (w == 2048) sort_segment_regs<2>(P, E, m, w, sK, sP);
    else if (w == 4096) sort_segment_regs<4>(P, E, m, w, sK, sP);
    else sort_segment_regs<8>(P, E, m, w, sK, sP);
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

cudaError_t launch_dist_group(const Cand* cand, int64_t n, int64_t G, int64_t* gcount, int64_t* goff,
                              unsigned long long* gcursor, int32_t* sp, int32_t* sg, cudaStream_t s) {
  cudaError_t err = cudaMemsetAsync(gcount, 0, sizeof(int64_t) * (size_t)G, s);
  if (err) return err;
  err = cudaMemsetAsync(gcursor, 0, sizeof(unsigned long long) * (size_t)G, s);
  if (err) return err;
  // shared-memory versions while G counters (and G reservations) fit in 48 KB
  const bool smem = G <= 4096;
  const int64_t chunk = 16384;  // candidates per block: ~2 G global atomics per 16,384 candidates at most
  const int64_t nb = (n + chunk - 1) / chunk;
  if (n > 0) {
    if (smem) {
      gene_count_smem_kernel<<<(unsigned)nb, 256, sizeof(unsigned int) * (size_t)G, s>>>(cand, n, (int)G, chunk,
                                                                                            gcount);
    } else {
      int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
      gene_count_kernel<<<blocks, 256, 0, s>>>(cand, n, gcount);
    }
  }
  scan_kernel<<<1, 1024, 0, s>>>(gcount, G, goff);
  if (n > 0) {
    if (smem) {
      scatter_smem_kernel<<<(unsigned)nb, 256, 12 * (size_t)G, s>>>(cand, n, (int)G, chunk, goff, gcursor, sp, sg);
    } else {
      int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
      scatter_kernel<<<blocks, 256, 0, s>>>(cand, n, goff, gcursor, sp, sg);
    }
  }
  return cudaGetLastError();
}

static cudaError_t launch_segsort(const int64_t* goff, int64_t G, int32_t* sp, double* se64, const int* dirty,
                                  cudaStream_t s) {
  constexpr int smem = kSortSmem * (int)(sizeof(uint64_t) + sizeof(int32_t));
  static std::atomic<uint64_t> attr{0};  // devices where the limit is set, shared by all contexts
  cudaError_t err = set_smem_once(attr, segsort_kernel, smem);
  if (err) return err;
  segsort_kernel<<<(unsigned)G, 1024, smem, s>>>(goff, sp, se64, dirty);
  return cudaGetLastError();
}

static int grouped_blocks(int64_t n) {
  const int64_t chunks = (n + 31) / 32;
  const int64_t want = (chunks + kRecheckWarps - 1) / kRecheckWarps;
  return (int)(want < 65536 ? want : 65536);
}

cudaError_t launch_dist_group_recheck_sort(const DistInputs& in, const Cand* cand, int64_t n, int64_t* gcount,
                                           int64_t* goff, unsigned long long* gcursor, int32_t* sp, int32_t* sg,
                                           double* se64, cudaStream_t s) {
  cudaError_t err = launch_dist_group(cand, n, in.G, gcount, goff, gcursor, sp, sg, s);
  if (err || n <= 0) return err;
  recheck_grouped_kernel<<<grouped_blocks(n), kRecheckWarps * 32, 0, s>>>(in, sp, sg, n, se64);
  err = cudaGetLastError();
  if (err) return err;
  return launch_segsort(goff, in.G, sp, se64, nullptr, s);
}

cudaError_t launch_dist_group_certify_sort(const DistInputs& in, const Cand* cand, int64_t n, int mode, double eps,
                                           const double* eps_g, int64_t* gcount, int64_t* goff,
                                           unsigned long long* gcursor, int32_t* sp, int32_t* sg, double* se64,
                                           float4* gt, int32_t* pos, uint8_t* flag,
                                           unsigned long long* counts, int* dirty, cudaStream_t s) {
  cudaError_t err = launch_dist_group(cand, n, in.G, gcount, goff, gcursor, sp, sg, s);
  if (err) return err;
  err = cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), s);
  if (err) return err;
  if (n <= 0) return cudaSuccess;
  const int64_t gk = in.G * in.K;
  ff_prep_genes_kernel<<<(unsigned)((gk + 255) / 256 < 4096 ? (gk + 255) / 256 : 4096), 256, 0, s>>>(in, gt);
  const float rK = (float)(1.0 / (double)in.K);
  approx_grouped_kernel<<<grouped_blocks(n), kRecheckWarps * 32, 0, s>>>(in, sp, sg, n, gt, rK, se64, pos,
                                                                         counts);
  const int list_blocks = 152 * 8;
  recheck_list_kernel<<<list_blocks, 128, 0, s>>>(in, sp, sg, pos, counts, se64);
  err = launch_segsort(goff, in.G, sp, se64, nullptr, s);
  if (err) return err;
  err = cudaMemsetAsync(dirty, 0, sizeof(int) * (size_t)in.G, s);
  if (err) return err;
  const int blocks = (int)((n + 255) / 256 < 65536 ? (n + 255) / 256 : 65536);
  ambiguous_kernel<<<blocks, 256, 0, s>>>(sg, goff, se64, n, mode, eps, eps_g, pos, counts + 1, flag);
  recheck_list_kernel<<<list_blocks, 128, 0, s>>>(in, sp, sg, pos, counts + 1, se64);
  run_sort_kernel<<<blocks, 256, 0, s>>>(sg, goff, flag, n, sp, se64, dirty);
  return launch_segsort(goff, in.G, sp, se64, dirty, s);
}

// ---------------------------------------------------------------------------
// accepted prefixes
// ---------------------------------------------------------------------------
__global__ void accept_len_kernel(const int64_t* goff, const double* se64, int64_t G, int mode, double eps_all,
                                  const double* eps_g, int64_t k, const float* X, const float* b0, float b1,
                                  int64_t* alen, int* fail, bool approx) {
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
      // certified values: the k-th error may be above its stored value by its bound
      ok = (approx ? E[k - 1] + approx_bound(E[k - 1]) : E[k - 1]) <= L;
    }
    if (!ok) fail[g] = 1;
  }
  alen[g] = len;
}

cudaError_t launch_dist_accept_len(const int64_t* goff, const double* se64, int64_t G, int mode, double eps,
                                   const double* eps_g, int64_t k, const float* X, const float* b0, float b1,
                                   int64_t* alen, int* fail, bool approx, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  accept_len_kernel<<<(unsigned)((G + 127) / 128), 128, 0, s>>>(goff, se64, G, mode, eps, eps_g, k, X, b0, b1,
                                                                alen, fail, approx);
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

// (particle, gene) of every accepted pair, in the lists' order (grouped by gene)
__global__ void accepted_pairs_kernel(const int64_t* aoff, const int64_t* idx, int64_t G, int64_t p_base, int32_t* sp,
                                      int32_t* sg) {
  const int64_t g = blockIdx.x;
  if (g >= G) return;
  for (int64_t i = aoff[g] + threadIdx.x; i < aoff[g + 1]; i += blockDim.x) {
    sp[i] = (int32_t)(idx[i] - 1 - p_base);
    sg[i] = (int32_t)g;
  }
}

cudaError_t launch_accepted_errors(const DistInputs& in, const int64_t* aoff, const int64_t* idx, int64_t G,
                                   int64_t p_base, int64_t n, int32_t* sp, int32_t* sg, double* err, cudaStream_t s) {
  if (G <= 0 || n <= 0) return cudaSuccess;
  accepted_pairs_kernel<<<(unsigned)G, 256, 0, s>>>(aoff, idx, G, p_base, sp, sg);
  recheck_grouped_kernel<<<grouped_blocks(n), kRecheckWarps * 32, 0, s>>>(in, sp, sg, n, err);
  return cudaGetLastError();
}

cudaError_t launch_scan(const int64_t* cnt, int64_t G, int64_t* off, cudaStream_t s) {
  scan_kernel<<<1, 1024, 0, s>>>(cnt, G, off);
  return cudaGetLastError();
}

}  // namespace abc
