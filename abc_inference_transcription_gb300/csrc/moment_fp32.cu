// moment_fp32.cu — production mode of the moment-ODE simulation (the FP64
// unit moment.cu is the oracle-exact mode): same exponential midpoint rule on
// the same substep grid, in FP32, with the augmented state ordered
//   [1, E G, Var G, E u, E l, Cov(G,u), Cov(G,l), Var u, Cov(u,l), Var l]
// in which the moment matrix of scripts/model.jl:74-86 is lower triangular:
// every moment depends only on itself and on moments listed before it.
// Products of lower-triangular matrices stay lower triangular, so an
// exponential product costs 220 FMA instead of 1000 and a substep 55 instead
// of 100.  Taylor order 8 after scaling to a column-sum norm <= 1/2
// (truncation < 6e-9, below FP32's 6e-8 resolution).  Substep and labelling indices are integers (the
// grid is aligned with every breakpoint), so the per-substep work has no FP64
// operation; rates, times and the statistics stay in FP64.  The transient
// phase applies the one-cycle propagator (the ordered product of the cycle's
// unlabelled substep propagators) once per cycle.  The default substep is
// cycle / 80 (every pulse, chase and age of the reference grid is a multiple
// of it): against the reference's recovered statistics it is as close as
// cycle / 400, and within 3e-3 of it.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "model.cuh"

namespace abc {
namespace {

constexpr int NA = 10;
constexpr int NT = NA * (NA + 1) / 2;  // 55 lower-triangular entries, row-major packed
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kTaylor = 8;

// packed index of (r, c), c <= r
__host__ __device__ constexpr int tri(int r, int c) { return r * (r + 1) / 2 + c; }

// the moment matrix times h in the permuted order (rows: 0 const, 1 EG, 2 VarG,
// 3 Eu, 4 El, 5 CovGu, 6 CovGl, 7 Varu, 8 Covul, 9 Varl); rates already times h
__device__ void build_tri(float* A, int lane, float kon, float koff, float al, float gam, float lam) {
  for (int i = lane; i < NT; i += 32) A[i] = 0.0f;
  __syncwarp();
  if (lane == 0) {
    const float ks = kon + koff, a1 = al * (1.0f - lam), a2 = al * lam;
    A[tri(1, 0)] = kon;
    A[tri(1, 1)] = -ks;
    A[tri(2, 0)] = kon;
    A[tri(2, 1)] = koff - kon;
    A[tri(2, 2)] = -2.0f * ks;
    A[tri(3, 1)] = a1;
    A[tri(3, 3)] = -gam;
    A[tri(4, 1)] = a2;
    A[tri(4, 4)] = -gam;
    A[tri(5, 2)] = a1;
    A[tri(5, 5)] = -(ks + gam);
    A[tri(6, 2)] = a2;
    A[tri(6, 6)] = -(ks + gam);
    A[tri(7, 1)] = a1;
    A[tri(7, 3)] = gam;
    A[tri(7, 5)] = 2.0f * a1;
    A[tri(7, 7)] = -2.0f * gam;
    A[tri(8, 5)] = a2;
    A[tri(8, 6)] = a1;
    A[tri(8, 8)] = -2.0f * gam;
    A[tri(9, 1)] = a2;
    A[tri(9, 4)] = gam;
    A[tri(9, 6)] = 2.0f * a2;
    A[tri(9, 9)] = -2.0f * gam;
  }
  __syncwarp();
}

// Output entries of a lane in a packed triangular product: o = lane and
// o = lane + 32 (when < 55), with their (row, column), kept in registers (a
// table in constant memory would serialise the lanes' distinct addresses).
struct LaneTri {
  int r0, c0, r1, c1;
  bool has1;
};

__device__ __forceinline__ void rc_of(int o, int& r, int& c) {
  r = 0;
  while ((r + 1) * (r + 2) / 2 <= o) ++r;
  c = o - r * (r + 1) / 2;
}

__device__ __forceinline__ LaneTri lane_tri(int lane) {
  LaneTri t;
  rc_of(lane, t.r0, t.c0);
  t.has1 = lane + 32 < NT;
  t.r1 = t.c1 = 0;
  if (t.has1) rc_of(lane + 32, t.r1, t.c1);
  return t;
}

__device__ __forceinline__ float tri_dot(const float* X, const float* Y, int r, int c) {
  float s = 0.0f;
  for (int k = c; k <= r; ++k) s = fmaf(X[tri(r, k)], Y[tri(k, c)], s);
  return s;
}

// Z = X Y, lower triangular, packed
__device__ __forceinline__ void tri_mul(const float* X, const float* Y, float* Z, const LaneTri& t, int lane) {
  const float z0 = tri_dot(X, Y, t.r0, t.c0);
  const float z1 = t.has1 ? tri_dot(X, Y, t.r1, t.c1) : 0.0f;
  Z[lane] = z0;
  if (t.has1) Z[lane + 32] = z1;
  __syncwarp();
}

__device__ void expm_tri(float* A, float* E, float* T, const LaneTri& t, int lane) {
  float norm = 0.0f;
  for (int c = 0; c < NA; ++c) {
    float s = 0.0f;
    for (int r = c; r < NA; ++r) s += fabsf(A[tri(r, c)]);
    norm = fmaxf(norm, s);
  }
  int sq = 0;
  while (norm > 0.5f) {
    norm *= 0.5f;
    sq++;
  }
  const float scale = ldexpf(1.0f, -sq);
  const float d0 = t.r0 == t.c0 ? 1.0f : 0.0f, d1 = t.r1 == t.c1 ? 1.0f : 0.0f;
  A[lane] *= scale;
  E[lane] = d0;
  if (t.has1) {
    A[lane + 32] *= scale;
    E[lane + 32] = d1;
  }
  __syncwarp();
  for (int n = kTaylor; n >= 1; --n) {
    tri_mul(A, E, T, t, lane);
    const float inv = 1.0f / (float)n;
    E[lane] = fmaf(T[lane], inv, d0);
    if (t.has1) E[lane + 32] = fmaf(T[lane + 32], inv, d1);
    __syncwarp();
  }
  for (int s = 0; s < sq; ++s) {
    tri_mul(E, E, T, t, lane);
    E[lane] = T[lane];
    if (t.has1) E[lane + 32] = T[lane + 32];
    __syncwarp();
  }
}

// division map (model.jl:98-111) in the permuted order
__device__ __forceinline__ void divide_p(float* v) {
  const float eu = v[3], el = v[4];
  v[5] *= 0.5f;
  v[6] *= 0.5f;
  v[7] = 0.25f * v[7] + 0.25f * eu;
  v[9] = 0.25f * v[9] + 0.25f * el;
  v[8] *= 0.25f;
  v[3] = 0.5f * eu;
  v[4] = 0.5f * el;
}

// y <- P y (P in shared or L1-resident global memory)
__device__ __forceinline__ void step_tri_s(const float* P, float* y) {
  float z[NA];
#pragma unroll
  for (int r = 0; r < NA; ++r) {
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c <= r; ++c) acc = fmaf(P[tri(r, c)], y[c], acc);
    z[r] = acc;
  }
#pragma unroll
  for (int r = 0; r < NA; ++r) y[r] = z[r];
}

// original moment index of each permuted position
__device__ __forceinline__ int orig_of(int r) {
  // 0 const, 1 EG(0), 2 VarG(3), 3 Eu(1), 4 El(2), 5 CovGu(4), 6 CovGl(5), 7 Varu(6), 8 Covul(7), 9 Varl(8)
  const int map[NA] = {-1, 0, 3, 1, 2, 4, 5, 6, 7, 8};
  return map[r];
}

__global__ void __launch_bounds__(kThreads) moment_kernel_f32(MomArgs a) {
  __shared__ float wsp[kWarps][3][NT];
  __shared__ float ss[NA];
  __shared__ double mom[kMaxConds * kMaxAges * 5];
  __shared__ double ds[kMaxConds * kMaxAges * 5];
  __shared__ PRec R;
  __shared__ int s_bad;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DevCfg& cfg = a.cfg;
  const int J = cfg.n_conds, A = cfg.n_ages;
  const int K = 4 * A + 3 * J;
  const int nsub = a.nsub;
  const double h = a.h, T = cfg.cycle;
  float* P0 = reinterpret_cast<float*>(a.scratch) + (size_t)blockIdx.x * 2 * nsub * NT;
  const LaneTri lt = lane_tri(lane);
  float* P1 = P0 + (size_t)nsub * NT;
  for (int64_t p = blockIdx.x; p < a.P; p += gridDim.x) {
    if (threadIdx.x == 0) s_bad = parse_theta(cfg, a.model, a.theta + p * a.ld, R, false) ? 1 : 0;
    __syncthreads();
    if (s_bad) {
      for (int k = threadIdx.x; k < K; k += blockDim.x) a.stats[p * K + k] = NAN;
      if (threadIdx.x == 0) atomicOr(a.status, 1);
      __syncthreads();
      continue;
    }
    // ---- propagators for every substep, without and with labelling
    float* Aw = wsp[warp][0];
    float* Ew = wsp[warp][1];
    float* Tw = wsp[warp][2];
    const float hf = (float)h, invT = (float)(1.0 / T), scal = (float)R.scal, lamf = (float)R.lam;
    const float koffh = (float)(R.koff * h);
    for (int task = warp; task < 2 * nsub; task += kWarps) {
      const int lab = task / nsub, idx = task - lab * nsub;
      const int k = idx / a.per_step;
      const float ph = ((float)idx + 0.5f) * hf;
      // alpha(t) = alpha_k size^s, size = 1 + phase / T (model.jl:25-27)
      const float al = (float)(R.alp[k] * h) * exp2f(scal * __log2f(fmaf(ph, invT, 1.0f)));
      build_tri(Aw, lane, (float)(R.kon[k] * h), koffh, al, (float)(R.gam[k] * h), lab ? lamf : 0.0f);
      expm_tri(Aw, Ew, Tw, lt, lane);
      float* dst = (lab ? P1 : P0) + (size_t)idx * NT;
      for (int i = lane; i < NT; i += 32) dst[i] = Ew[i];
      __syncwarp();
    }
    __syncthreads();
    // ---- one-cycle propagator without labelling, Phi = P[nsub-1] ... P[0]:
    // each warp multiplies a contiguous quarter in order, warp 0 joins them
    {
      const int q0 = warp * nsub / kWarps, q1 = (warp + 1) * nsub / kWarps;
      float* Q = wsp[warp][1];
      float* Pi = wsp[warp][0];
      Q[lane] = lt.r0 == lt.c0 ? 1.0f : 0.0f;
      if (lt.has1) Q[lane + 32] = lt.r1 == lt.c1 ? 1.0f : 0.0f;
      __syncwarp();
      for (int i = q0; i < q1; ++i) {
        const float* src = P0 + (size_t)i * NT;
        Pi[lane] = src[lane];
        if (lt.has1) Pi[lane + 32] = src[lane + 32];
        __syncwarp();
        tri_mul(Pi, Q, Tw, lt, lane);
        Q[lane] = Tw[lane];
        if (lt.has1) Q[lane + 32] = Tw[lane + 32];
        __syncwarp();
      }
    }
    __syncthreads();
    if (warp == 0) {
      float* Phi = wsp[0][1];
      for (int w = 1; w < kWarps; ++w) {
        tri_mul(wsp[w][1], Phi, wsp[0][2], lt, lane);
        Phi[lane] = wsp[0][2][lane];
        if (lt.has1) Phi[lane + 32] = wsp[0][2][lane + 32];
        __syncwarp();
      }
    }
    __syncthreads();
    // ---- transient phase (model.jl:114-142): one cycle from iv, then cycles
    // until the moments of E G, E u, Var G, Cov(G,u), Var u change by <= 1 %
    if (threadIdx.x == 0) {
      const float* Phi = wsp[0][1];
      float y[NA], e1[NA];
      y[0] = 1.0f;
      for (int r = 1; r < NA; ++r) y[r] = (float)a.iv[orig_of(r)];
      step_tri_s(Phi, y);
      for (int r = 0; r < NA; ++r) e1[r] = y[r];
      int it = 0;
      bool conv = false;
      while (!conv && it <= 100) {
        it++;
        divide_p(y);
        step_tri_s(Phi, y);
        const int chk[5] = {1, 3, 2, 5, 7};
        int nz = 0, ok = 0;
        for (int q = 0; q < 5; ++q) {
          const int r = chk[q];
          if (e1[r] > 0.0f) {
            nz++;
            if (fabsf((e1[r] - y[r]) / e1[r]) <= 0.01f) ok++;
          }
        }
        conv = ok == nz;
        for (int r = 0; r < NA; ++r) e1[r] = y[r];
      }
      divide_p(y);
      for (int r = 0; r < NA; ++r) ss[r] = y[r];
      if (a.iters) a.iters[p] = it;
    }
    __syncthreads();
    // ---- trajectories (model.jl:146-199), one (condition, age) per thread:
    // global substep s (midpoint t0 + (s + 1/2) h), divisions at multiples of
    // nsub, labelling iff s_lo <= s < s_hi, the end at s_end = (age - t0) / h
    const double t0 = cfg.t0;
    for (int t = threadIdx.x; t < J * A; t += blockDim.x) {
      const int j = t / A, ai = t - (t / A) * A;
      const double age = cfg.ages[ai];
      const double texp = (age - cfg.pulse[j]) - cfg.chase[j];
      const double tle = texp + cfg.pulse[j];
      const int s_lo = (int)lround((texp - t0) / h), s_hi = (int)lround((tle - t0) / h);
      const int s_end = (int)lround((age - t0) / h);
      float y[NA];
#pragma unroll
      for (int r = 0; r < NA; ++r) y[r] = ss[r];
      int idx = 0;
      for (int s = 0; s < s_end; ++s) {
        if (idx == nsub) {
          idx = 0;
          divide_p(y);
        }
        step_tri_s(((s >= s_lo && s < s_hi) ? P1 : P0) + (size_t)idx * NT, y);
        ++idx;
      }
      double* mo = mom + t * 5;
      mo[0] = y[3];
      mo[1] = y[4];
      mo[2] = y[7];
      mo[3] = y[8];
      mo[4] = y[9];
    }
    __syncthreads();
    if (a.moments)
      for (int i = threadIdx.x; i < J * A * 5; i += blockDim.x) a.moments[p * (J * A * 5) + i] = mom[i];
    // capture transform (model.jl:221-239) per (condition, age), then the
    // statistics per condition on the lanes of warp 0
    for (int t = threadIdx.x; t < J * A; t += blockDim.x) {
      const int j = t / A, ai = t - (t / A) * A;
      const double* bm = a.beta_mom + ((j < a.n_pulse_conds ? 0 : 1) * A + ai) * 3;
      const double mb = bm[0], m2 = bm[1], vb = bm[2];
      const double* sm = mom + (j * A + ai) * 5;
      double* d = ds + (j * A + ai) * 5;
      d[0] = sm[0] * mb;
      d[1] = sm[1] * mb;
      d[2] = ((mb - m2) * sm[0] + vb * (sm[0] * sm[0] + sm[2])) + mb * mb * sm[2];
      d[4] = ((mb - m2) * sm[1] + vb * (sm[1] * sm[1] + sm[4])) + mb * mb * sm[4];
      d[3] = vb * (sm[0] * sm[1] + sm[3]) + mb * mb * sm[3];
    }
    __syncthreads();
    if (threadIdx.x < 32)
      for (int j = threadIdx.x; j < J; j += 32) stats_from_moments_cond(cfg, ds, a.age_dist, a.stats + p * K, j);
    __syncthreads();
  }
}

}  // namespace

size_t moment_f32_scratch_per_cta(int nsub) { return (size_t)2 * nsub * NT * sizeof(float); }

cudaError_t launch_moment_f32(const MomArgs& a, int grid, cudaStream_t s) {
  if (a.P <= 0) return cudaSuccess;
  moment_kernel_f32<<<grid, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace abc
