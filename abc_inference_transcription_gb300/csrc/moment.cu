// moment.cu — the reference's deterministic simulation on the GPU: the
// 9-moment linear ODE of the telegraph model with labelling (scripts/model.jl:
// 67-96), its periodic steady state (transient_phase, :114-142), the
// multi-cycle trajectories with division (:98-111, :146-199), the capture
// moment transform (downsample, :221-239) and the 53 statistics
// (scripts/abc_simulation.jl:13-62).
//
// y' = A(t) y + b(t) is integrated by the exponential midpoint rule on a grid
// of step h aligned with every breakpoint: each substep applies
// expm(h A(t_mid)) to the state augmented with a constant 1.  The 10 x 10
// exponentials come from scaling and squaring with an 18-term Taylor
// polynomial in Horner form.  Same operations and order as the FP64 C oracle
// (built with -fmad=false here and -ffp-contract=off there): the results are
// bit-identical.
//
// One CTA of four warps per particle (grid-stride over particles):
//  A. the 2 x nsub substep propagators (without / with labelling), one
//     exponential per warp at a time, matrices in shared memory, each output
//     element summed by one lane in the oracle's order; cached per CTA in
//     global memory ([2][nsub][100] doubles);
//  B. the transient phase: lanes 0-9 of warp 0 hold the augmented state;
//  C. the J x A trajectories, one per thread, state in registers;
//  D. capture transform and statistics by thread 0.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "model.cuh"

namespace abc {
namespace {

constexpr int NA = 10;        // 9 moments + the constant 1
constexpr int NN = NA * NA;
constexpr int kMomThreads = 128;
constexpr int kMomWarps = kMomThreads / 32;

// rows of A(t) h, exactly as the oracle's build_A (model.jl:74-86 in the
// augmented form; index 9 carries the constant inputs)
__device__ void build_A(double* A, int lane, double kon, double koff, double al, double gam, double lam, double h) {
  for (int i = lane; i < NN; i += 32) A[i] = 0.0;
  __syncwarp();
  if (lane == 0) {
    const double ks = kon + koff;
    A[0 * NA + 0] = -ks; A[0 * NA + 9] = kon;
    A[1 * NA + 0] = (1.0 - lam) * al; A[1 * NA + 1] = -gam;
    A[2 * NA + 0] = lam * al; A[2 * NA + 2] = -gam;
    A[3 * NA + 0] = koff - kon; A[3 * NA + 3] = -2.0 * ks; A[3 * NA + 9] = kon;
    A[4 * NA + 3] = al * (1.0 - lam); A[4 * NA + 4] = -(ks + gam);
    A[5 * NA + 3] = al * lam; A[5 * NA + 5] = -(ks + gam);
    A[6 * NA + 0] = al * (1.0 - lam); A[6 * NA + 1] = gam; A[6 * NA + 4] = 2.0 * al * (1.0 - lam);
    A[6 * NA + 6] = -2.0 * gam;
    A[7 * NA + 4] = al * lam; A[7 * NA + 5] = al * (1.0 - lam); A[7 * NA + 7] = -2.0 * gam;
    A[8 * NA + 0] = al * lam; A[8 * NA + 2] = gam; A[8 * NA + 5] = 2.0 * al * lam; A[8 * NA + 8] = -2.0 * gam;
  }
  __syncwarp();
  for (int i = lane; i < NN; i += 32) A[i] *= h;
  __syncwarp();
}

// Z = X Y (10 x 10), each element summed over k in order by one lane
__device__ void mat_mul_warp(const double* X, const double* Y, double* Z, int lane) {
  for (int o = lane; o < NN; o += 32) {
    const int i = o / NA, j = o - (o / NA) * NA;
    double s = 0.0;
    for (int k = 0; k < NA; ++k) s += X[i * NA + k] * Y[k * NA + j];
    Z[o] = s;
  }
  __syncwarp();
}

// E = expm(A): scaling to a column-sum norm <= 1/2, Taylor to order 18 in
// Horner form, squaring back.  A is overwritten (scaled), T is scratch.
__device__ void expm_warp(double* A, double* E, double* T, int lane) {
  double norm = 0.0;
  for (int j = 0; j < NA; ++j) {
    double s = 0.0;
    for (int i = 0; i < NA; ++i) s += fabs(A[i * NA + j]);
    if (s > norm) norm = s;
  }
  int sq = 0;
  while (norm > 0.5) {
    norm *= 0.5;
    sq++;
  }
  const double scale = ldexp(1.0, -sq);
  for (int i = lane; i < NN; i += 32) {
    A[i] = A[i] * scale;
    E[i] = (i % (NA + 1) == 0) ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int n = 18; n >= 1; --n) {
    mat_mul_warp(A, E, T, lane);
    for (int i = lane; i < NN; i += 32) E[i] = T[i] / (double)n + ((i % (NA + 1) == 0) ? 1.0 : 0.0);
    __syncwarp();
  }
  for (int s = 0; s < sq; ++s) {
    mat_mul_warp(E, E, T, lane);
    for (int i = lane; i < NN; i += 32) E[i] = T[i];
    __syncwarp();
  }
}

// division map (periodic_boundary, model.jl:98-111) on a full state
__device__ __forceinline__ void divide(double* v) {
  const double e1 = v[1], e2 = v[2], e4 = v[4], e5 = v[5], e6 = v[6], e7 = v[7], e8 = v[8];
  v[4] = e4 / 2.0;
  v[5] = e5 / 2.0;
  v[6] = e6 / 4.0 + e1 / 4.0;
  v[8] = e8 / 4.0 + e2 / 4.0;
  v[7] = e7 / 4.0;
  v[1] = e1 / 2.0;
  v[2] = e2 / 2.0;
}

// the same map when lane i < 10 holds v[i]
__device__ __forceinline__ double divide_lane(double v, int lane) {
  const double e1 = __shfl_sync(0xffffffffu, v, 1), e2 = __shfl_sync(0xffffffffu, v, 2);
  switch (lane) {
    case 1: return e1 / 2.0;
    case 2: return e2 / 2.0;
    case 4: return v / 2.0;
    case 5: return v / 2.0;
    case 6: return v / 4.0 + e1 / 4.0;
    case 7: return v / 4.0;
    case 8: return v / 4.0 + e2 / 4.0;
    default: return v;
  }
}

struct Grid {
  double T, h;
  int nsub;
};

__device__ __forceinline__ int sub_index(const Grid& g, double tm) {
  const double md = tm - g.T * floor(tm / g.T);
  int idx = (int)floor(md / g.h);
  if (idx >= g.nsub) idx = g.nsub - 1;
  return idx;
}

// one substep on a state held by lanes 0-9: z_i = sum_j P_ij y_j
__device__ __forceinline__ double apply_lane(const double* P, double y, int lane) {
  double s = 0.0;
  const int i = lane < NA ? lane : 0;
  for (int j = 0; j < NA; ++j) s += P[i * NA + j] * __shfl_sync(0xffffffffu, y, j);
  return s;
}

__device__ void integrate_lane(const Grid& g, const double* P0, double& y, double ta, double tb, int lane) {
  const long n = lround((tb - ta) / g.h);
  for (long i = 0; i < n; ++i) {
    const double tm = ta + ((double)i + 0.5) * g.h;
    y = apply_lane(P0 + (size_t)sub_index(g, tm) * NN, y, lane);
  }
}

__device__ void integrate_thread(const Grid& g, const double* P0, const double* P1, double* y, double ta, double tb,
                                 double texp, double tle) {
  const long n = lround((tb - ta) / g.h);
  for (long i = 0; i < n; ++i) {
    const double tm = ta + ((double)i + 0.5) * g.h;
    const int idx = sub_index(g, tm);
    const double* P = ((tm >= texp && tm <= tle) ? P1 : P0) + (size_t)idx * NN;
    double z[NA];
#pragma unroll
    for (int r = 0; r < NA; ++r) {
      double s = 0.0;
#pragma unroll
      for (int c = 0; c < NA; ++c) s += P[r * NA + c] * y[c];
      z[r] = s;
    }
#pragma unroll
    for (int r = 0; r < NA; ++r) y[r] = z[r];
  }
}

__global__ void __launch_bounds__(kMomThreads) moment_kernel(MomArgs a) {
  __shared__ double wsp[kMomWarps][3][NN];
  __shared__ double ss[NA];
  __shared__ double mom[kMaxConds * kMaxAges * 5];
  __shared__ double ds[kMaxConds * kMaxAges * 5];
  __shared__ PRec R;
  __shared__ int s_bad;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DevCfg& cfg = a.cfg;
  const int J = cfg.n_conds, A = cfg.n_ages, S = cfg.n_steps;
  const int K = 4 * A + 3 * J;
  Grid g;
  g.T = cfg.cycle;
  g.h = a.h;
  g.nsub = a.nsub;
  double* P0 = a.scratch + (size_t)blockIdx.x * 2 * a.nsub * NN;
  double* P1 = P0 + (size_t)a.nsub * NN;
  for (int64_t p = blockIdx.x; p < a.P; p += gridDim.x) {
    if (threadIdx.x == 0) {
      DevCfg c1 = cfg;
      s_bad = parse_theta(c1, a.model, a.theta + p * a.ld, R, false) ? 1 : 0;
    }
    __syncthreads();
    if (s_bad) {
      for (int k = threadIdx.x; k < K; k += blockDim.x) a.stats[p * K + k] = NAN;
      if (threadIdx.x == 0) atomicOr(a.status, 1);
      __syncthreads();
      continue;
    }
    // ---- A: substep propagators
    double* Aw = wsp[warp][0];
    double* Ew = wsp[warp][1];
    double* Tw = wsp[warp][2];
    for (int task = warp; task < 2 * a.nsub; task += kMomWarps) {
      const int lab = task / a.nsub, idx = task - lab * a.nsub;
      const int k = idx / a.per_step;
      const double ph = ((double)idx + 0.5) * g.h;
      const double al = R.alp[k] * xpow(1.0 + ph / g.T, R.scal);
      build_A(Aw, lane, R.kon[k], R.koff, al, R.gam[k], lab ? R.lam : 0.0, g.h);
      expm_warp(Aw, Ew, Tw, lane);
      double* dst = (lab ? P1 : P0) + (size_t)idx * NN;
      for (int i = lane; i < NN; i += 32) dst[i] = Ew[i];
      __syncwarp();
    }
    __syncthreads();
    (void)S;
    // ---- B: transient phase (model.jl:114-142), lanes 0-9 of warp 0
    if (warp == 0) {
      double e1 = lane < 9 ? a.iv[lane] : (lane == 9 ? 1.0 : 0.0);
      integrate_lane(g, P0, e1, 0.0, g.T, lane);
      double e2 = e1;
      int it = 0;
      bool conv = false;
      while (!conv && it <= 100) {
        it++;
        double y = divide_lane(e1, lane);
        integrate_lane(g, P0, y, 0.0, g.T, lane);
        e2 = y;
        const bool chk = lane == 0 || lane == 1 || lane == 3 || lane == 4 || lane == 6;
        const bool nzl = chk && e1 > 0.0;
        const bool okl = nzl && fabs((e1 - e2) / e1) <= 0.01;
        conv = __popc(__ballot_sync(0xffffffffu, okl)) == __popc(__ballot_sync(0xffffffffu, nzl));
        e1 = e2;
      }
      const double sv = divide_lane(e2, lane);
      if (lane < NA) ss[lane] = sv;
      if (lane == 0 && a.iters) a.iters[p] = it;
    }
    __syncthreads();
    // ---- C: trajectories (model.jl:146-199), one (condition, age) per thread
    const double t0 = cfg.t0;
    for (int t = threadIdx.x; t < J * A; t += blockDim.x) {
      const int j = t / A, ai = t - (t / A) * A;
      const double age = cfg.ages[ai];
      const double texp = (age - cfg.pulse[j]) - cfg.chase[j];
      const double tle = texp + cfg.pulse[j];
      double y[NA];
#pragma unroll
      for (int i = 0; i < NA; ++i) y[i] = ss[i];
      double tau = t0;
      bool first = true;
      while (tau < age) {
        double tf = (tau < 0.0) ? tau + g.T : age;
        if (tf > age) tf = age;
        if (!first) divide(y);
        integrate_thread(g, P0, P1, y, tau, tf, texp, tle);
        first = false;
        tau = tf;
      }
      double* mo = mom + t * 5;
      mo[0] = y[1];
      mo[1] = y[2];
      mo[2] = y[6];
      mo[3] = y[7];
      mo[4] = y[8];
    }
    __syncthreads();
    if (a.moments)
      for (int i = threadIdx.x; i < J * A * 5; i += blockDim.x) a.moments[p * (J * A * 5) + i] = mom[i];
    // ---- D: capture moment transform (model.jl:221-239) and statistics
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

cudaError_t launch_moment(const MomArgs& a, int grid, cudaStream_t s) {
  if (a.P <= 0) return cudaSuccess;
  moment_kernel<<<grid, kMomThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace abc
