// kernels_fp64.cu — prior draw, particle setup, FP64 (oracle-mode) SSA and the
// fused capture + statistics kernel.  Built with -fmad=false: every FP64
// result here is bit-identical to the FP64 CPU oracle.
#include <type_traits>

#include "kernels.h"
#include "sampler32.cuh"

namespace abc {

// ---------------------------------------------------------------------------
// Prior draw (fix_params, scripts/abc_simulation.jl:3-11): one thread per
// particle, Philox stream ST_PRIOR, cell 0.  Column order of theta:
// kon(1|S), koff, alpha(1|S), gamma(1|S), lambda, [beta], [scaling].
// ---------------------------------------------------------------------------
__global__ void prior_kernel(PriorArgs A) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= A.n_particles) return;
  Rng r;
  rng_init(r, A.seed, ST_PRIOR, 0u, (uint32_t)(A.p_offset + p));
  double* th = A.theta + p * A.cfg.npar;
  const int S = A.cfg.n_steps;
  int i = 0;
  uint32_t a, b;
  for (int rate = 0; rate < 4; ++rate) {
    const double lo = A.lo[rate], hi = A.hi[rate];
    bool varies = (A.model == 3 && rate == 0) || (A.model == 4 && rate == 2) || (A.model == 5 && rate == 3);
    rng_pair(r, a, b);
    double base = lo + (hi - lo) * u52(a, b);
    if (!varies) {
      th[i++] = base;
    } else if (A.vary_mode == 0) {
      th[i++] = base;
      for (int k = 1; k < S; ++k) {
        rng_pair(r, a, b);
        th[i++] = lo + (hi - lo) * u52(a, b);
      }
    } else {
      for (int k = 0; k < S; ++k) {
        rng_pair(r, a, b);
        th[i++] = base + (A.lf0 + (A.lf1 - A.lf0) * u52(a, b));
      }
    }
  }
  rng_pair(r, a, b);
  th[i++] = A.lo[4] + (A.hi[4] - A.lo[4]) * u52(a, b);
  if (A.cfg.splicing) {
    rng_pair(r, a, b);
    th[i++] = A.lo[5] + (A.hi[5] - A.lo[5]) * u52(a, b);
  }
  if (A.cfg.scaling_column) {
    rng_pair(r, a, b);
    th[i++] = xexp10(A.lo[6] + (A.hi[6] - A.lo[6]) * u52(a, b));
  }
}

cudaError_t launch_prior(const PriorArgs& a, cudaStream_t s) {
  if (a.n_particles <= 0) return cudaSuccess;
  int blocks = (int)((a.n_particles + 127) / 128);
  prior_kernel<<<blocks, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// theta -> rates, thinning bounds and initial state; one thread per particle.
// ---------------------------------------------------------------------------
__global__ void setup_kernel(SetupArgs A) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= A.n_particles) return;
  PRec R;
  const int model = A.models ? A.models[p] : A.model;
  int st = (model >= 1 && model <= 5) ? parse_theta(A.cfg, model, A.theta + p * A.ld_theta, R) : -1;
  if (st) {
    atomicOr(A.status, STF_NONFINITE);
    // a harmless record: the trajectory sees no reactions
    for (int k = 0; k < kMaxSteps; ++k) R.kon[k] = R.alp[k] = R.gam[k] = R.amax[k] = 0.0;
    R.koff = R.lam = R.beta = R.scal = R.g0 = R.u0 = R.s0 = R.c0 = R.v0 = 0.0;
    R.cost = 1.0;
  }
  A.rec[p] = R;
  // rates in log2 units (times log2 e), so the production kernel's waiting
  // time is -log2(U) / a0 without a conversion per event
  constexpr double kL2E = 1.4426950408889634;
  PRecF F;
  for (int k = 0; k < kMaxSteps; ++k) {
    F.kon[k] = (float)(R.kon[k] * kL2E);
    F.alp[k] = (float)(R.alp[k] * kL2E);
    F.gam[k] = (float)(R.gam[k] * kL2E);
    F.amax[k] = (float)(R.amax[k] * kL2E);
  }
  F.koff = (float)(R.koff * kL2E);
  F.lam = (float)R.lam;
  F.beta = (float)(R.beta * kL2E);
  F.scal = (float)R.scal;
  if (A.fp32) {
    // rates beyond the FP32 range would stall the production kernel's clock
    bool ok = F.koff < 1e30f && F.beta < 1e30f;
    for (int k = 0; k < kMaxSteps; ++k) ok = ok && F.kon[k] < 1e30f && F.alp[k] < 1e30f && F.gam[k] < 1e30f;
    if (!ok) {
      atomicOr(A.status, STF_NONFINITE);
      memset(&F, 0, sizeof(F));
    }
  }
  A.recf[p] = F;
}

cudaError_t launch_setup(const SetupArgs& a, cudaStream_t s) {
  if (a.n_particles <= 0) return cudaSuccess;
  int blocks = (int)((a.n_particles + 63) / 64);
  setup_kernel<<<blocks, 64, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// SSA, FP64 oracle mode.
// ---------------------------------------------------------------------------
// Persistent: every lane owns one trajectory at a time and pulls the next
// (particle, cell) item from the global counter (warp-aggregated atomics).
__global__ void __launch_bounds__(128) ssa_kernel_fp64(SsaArgs A) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t cap = A.cfg.event_cap > 0 ? A.cfg.event_cap : kDefaultEventCap;
  Traj s;
  bool active = false, done = false;
  unsigned long long tot_ev = 0, tot_rej = 0;
  int err = 0;
  while (true) {
    const bool need = !active && !done;
    const unsigned mask = __ballot_sync(FULL, need);
    if (mask) {
      const int leader = __ffs(mask) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(A.counter, (unsigned long long)__popc(mask));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        const unsigned long long item = base + (unsigned long long)__popc(mask & ((1u << lane) - 1u));
        if (item >= (unsigned long long)A.n_items) {
          done = true;
        } else {
          traj_init(s, A, (int64_t)item);
          active = true;
        }
      }
    }
    if (__all_sync(FULL, done)) break;
    if (active) {
      const PRec& R = A.rec[s.plocal];
#pragma unroll 1
      for (int it = 0; it < kQuantum; ++it) {
        uint32_t ch;
        bool fin = step_fp64(s, R, A.cfg, ch);
        if (ch == CH_REJ) {
          tot_rej++;
        } else if (ch != CH_NULL) {
          s.ev++;
          if (s.ev > cap) {
            err |= STF_EVENT_CAP;
            fin = true;
          }
        }
        if (s.uu >= kOverflowCount || s.lu >= kOverflowCount || s.us >= kOverflowCount ||
            s.ls >= kOverflowCount) {
          err |= STF_OVERFLOW;
          fin = true;
        }
        if (s.stall > kMaxStall) {
          err |= STF_NONFINITE;
          fin = true;
        }
        if (fin) {
          A.counts[s.out] = make_int2(s.uu + s.us, s.lu + s.ls);
          if (A.events) A.events[s.out] = s.ev;
          if (A.hash) A.hash[s.out] = s.hash;
          tot_ev += (unsigned long long)s.ev;
          active = false;
          break;
        }
      }
    }
  }
  // warp totals -> one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    tot_ev += __shfl_xor_sync(FULL, tot_ev, o);
    tot_rej += __shfl_xor_sync(FULL, tot_rej, o);
    err |= __shfl_xor_sync(FULL, err, o);
  }
  if (lane == 0) {
    atomicAdd(&A.totals[0], tot_ev);
    atomicAdd(&A.totals[1], tot_rej);
    if (err) atomicOr(A.status, err);
  }
}

cudaError_t launch_ssa_fp64(const SsaArgs& a, int grid, cudaStream_t s) {
  ssa_kernel_fp64<<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// One thread per trajectory of the production mode: the gene state from the
// first word of the trajectory's main stream and the moment-matched first
// mRNA count (auxiliary stream), drawn from the distribution traj_init uses
// in the FP64 mode with FP32 samplers.  Runs at full occupancy instead of
// inside the production kernel's divergent refill path.
__global__ void __launch_bounds__(256) init_state_kernel(SsaArgs A) {
  const int64_t P = A.n_items / A.n_cells;
  const int C = (int)A.n_cells;
  __shared__ float mom[5];  // the particle's g0, u0, c0, v0 in FP32, and the rounded mean count
  for (int64_t pl = blockIdx.x; pl < P; pl += gridDim.x) {  // a block per particle, a thread per cell
    if (threadIdx.x == 0) {  // the FP64 -> FP32 conversions once per particle, not per cell
      const PRec& R = A.rec[pl];
      mom[0] = (float)R.g0;
      mom[1] = (float)R.u0;
      mom[2] = (float)R.c0;
      mom[3] = (float)R.v0;
      mom[4] = (float)fmin(floor(R.u0 + 0.5), 1.0e9);  // far above the count limit (2^23), reported there
    }
    __syncthreads();
    const float g0 = mom[0], u0 = mom[1], c0 = mom[2], v0 = mom[3], ur = mom[4];
    const uint32_t particle = (uint32_t)(A.p_offset + pl);
    for (int ci = threadIdx.x; ci < C; ci += blockDim.x) {
      const uint32_t cell = A.cell_id[ci];
      Rng r;
      rng_init(r, A.seed, ST_SSA, cell, particle);
      uint32_t w0, w1;
      rng_pair(r, w0, w1);
      const int G = u24(w0) < g0 ? 1 : 0;
      int u;
      if (A.cfg.splicing) {
        u = (int)ur;
      } else {
        Rng aux;
        rng_init(aux, A.seed, ST_AUX, cell, particle);
        u = initial_count32(g0, u0, c0, v0, G, w1, aux);
      }
      A.counts[pl * A.n_cells + ci] = make_int2(u, G);
    }
    __syncthreads();  // mom is rewritten for the next particle
  }
}

cudaError_t launch_init_states(const SsaArgs& a, int sms, cudaStream_t s) {
  if (a.n_items <= 0 || a.n_cells <= 0) return cudaSuccess;
  const int64_t P = a.n_items / a.n_cells, cap = (int64_t)sms * 16;
  init_state_kernel<<<(unsigned)(P < cap ? P : cap), 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Capture + statistics: one CTA (8 warps) per particle.  Warp w handles the
// (condition, age) groups w, w+8, ...: each lane thins its cells' counts
// binomially with the cell's capture efficiency (downsample,
// scripts/model.jl:221-239, realised per cell), accumulates exact integer
// moment sums, and the warp reduces them with shuffles.  One thread then
// forms the 4A + 3J statistics (abc_simulation.jl:23-46).
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long shfl_xor_ll(long long v, int o) {
  return __shfl_xor_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ __int128 shfl_xor_i128(__int128 v, int o) {
  unsigned long long lo = (unsigned long long)(unsigned __int128)v;
  long long hi = (long long)(v >> 64);
  lo = __shfl_xor_sync(0xffffffffu, lo, o);
  hi = __shfl_xor_sync(0xffffffffu, hi, o);
  return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | (unsigned __int128)lo);
}

// NARROW: 64-bit sums of the squared counts (production mode: counts at most
// 2^24, where FP32 increments stop, and at most 2^14 cells per group, so the
// sums stay below 2^62); 128-bit otherwise.
template <bool CAP32, bool NARROW>
__global__ void __launch_bounds__(256) stats_kernel(StatsArgs A) {
  __shared__ double mom[kMaxAges * kMaxConds * 5];
  __shared__ double wts[kMaxAges * kMaxConds];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ng = A.cfg.n_ages * A.cfg.n_conds;
  const int K = 4 * A.cfg.n_ages + 3 * A.cfg.n_conds;
  for (int i = threadIdx.x; i < ng; i += blockDim.x) wts[i] = A.age_dist[i];
  for (int64_t p = blockIdx.x; p < A.n_particles; p += gridDim.x) {
    const int2* cnt = A.counts + p * A.n_cells;
    const uint32_t pg = (uint32_t)(A.p_offset + p);
    for (int g = warp; g < ng; g += (blockDim.x >> 5)) {
      const int g0 = A.gstart[g], g1 = A.gstart[g + 1];
      using Sq = typename std::conditional<NARROW, long long, __int128>::type;
      long long su = 0, sl = 0;
      Sq suu = 0, sll = 0, sul = 0;
      for (int i = g0 + lane; i < g1; i += 32) {
        int2 c = cnt[i];
        Rng r;
        rng_init(r, A.seed, ST_CAPTURE, A.cell_id[i], pg);
        long long cu, cl;
        if (CAP32) {  // FP32 efficiencies: no FP64-pipe work per cell
          const float b32 = A.beta32[i];
          cu = binomial32(r, c.x, b32);
          cl = binomial32(r, c.y, b32);
        } else {
          cu = binomial(r, c.x, A.beta[i]);
          cl = binomial(r, c.y, A.beta[i]);
        }
        if (A.captured) A.captured[p * A.n_cells + i] = make_int2((int)cu, (int)cl);
        su += cu;
        sl += cl;
        suu += (Sq)(cu * cu);
        sll += (Sq)(cl * cl);
        sul += (Sq)(cu * cl);
      }
      for (int o = 16; o > 0; o >>= 1) {
        su += shfl_xor_ll(su, o);
        sl += shfl_xor_ll(sl, o);
        if (NARROW) {
          suu += (Sq)shfl_xor_ll((long long)suu, o);
          sll += (Sq)shfl_xor_ll((long long)sll, o);
          sul += (Sq)shfl_xor_ll((long long)sul, o);
        } else {
          suu += (Sq)shfl_xor_i128((__int128)suu, o);
          sll += (Sq)shfl_xor_i128((__int128)sll, o);
          sul += (Sq)shfl_xor_i128((__int128)sul, o);
        }
      }
      if (lane < 5) {  // lane j forms moment j: [E u, E l, Var u, Cov ul, Var l], one FP64 division each
        const long long n = g1 - g0;
        const double nd = (double)n;
        const double dn = nd * (double)(n - 1);
        __int128 x;
        if (lane == 0) x = su;
        else if (lane == 1) x = sl;
        else if (lane == 2) x = (__int128)n * suu - (__int128)su * su;
        else if (lane == 3) x = (__int128)n * sul - (__int128)su * sl;
        else x = (__int128)n * sll - (__int128)sl * sl;
        mom[g * 5 + lane] = i128_to_double(x) / (lane < 2 ? nd : dn);
      }
    }
    __syncthreads();
    if (warp == 0)  // one condition per lane
      for (int j = lane; j < A.cfg.n_conds; j += 32) stats_from_moments_cond(A.cfg, mom, wts, A.stats + p * K, j);
    __syncthreads();
  }
}

cudaError_t launch_stats(const StatsArgs& a, cudaStream_t s) {
  if (a.n_particles <= 0) return cudaSuccess;
  int blocks = (int)(a.n_particles < 1048576 ? a.n_particles : 1048576);
  if (a.fp32 && a.max_group_cells <= 16384)
    stats_kernel<true, true><<<blocks, 256, 0, s>>>(a);
  else if (a.fp32)
    stats_kernel<true, false><<<blocks, 256, 0, s>>>(a);
  else
    stats_kernel<false, false><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

int ssa_blocks_per_sm_fp64() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_kernel_fp64, 128, 0);
  return n;
}

}  // namespace abc
