// ssa.cuh — exact SSA of the telegraph gene with labelling, cell division and
// size-scaled transcription: one trajectory per (particle, cell).
//
// Reaction network (the network whose moment equations are f(y,p,lambda),
// scripts/model.jl:74-86):
//   G 0->1 @ kon(t);  G 1->0 @ koff;  G=1: transcription @ alpha(t), labelled
//   with probability lambda(t) (model.jl:58-64);  u -> u-1 @ gamma(t) u;
//   l -> l-1 @ gamma(t) l;  [splicing option: unspliced -> spliced @ beta,
//   decay acts on the spliced species].
//   alpha(t) = alpha_k size(t)^s, size = 1 + phase/T (model.jl:1-27), drawn by
//   thinning against alpha_k (1 + (k+1)/S)^s.  Rates are piecewise constant on
//   the S age steps of the cycle (model.jl:12-18).
//   Division at t = 0 mod T: every mRNA species -> Bin(n, 1/2) (the moment map
//   periodic_boundary, model.jl:98-111).  Start at t0 = -n_burn T
//   (abc_simulation.jl:73) from the periodic mean state, observe at the cell's
//   age (trajectories, model.jl:146-174).
//
// Random numbers: each iteration draws one pair of 32-bit words from the
// trajectory's Philox stream (waiting time, channel); division draws
// ceil(n/64) pairs per species.  Identical consumption in both precisions.
//
// Kernel shape: persistent; every lane owns one trajectory at a time and
// pulls the next (particle, cell) item from a global counter when it
// finishes (warp-aggregated atomics), so trajectories of very different
// lengths keep all lanes busy.
#pragma once
#include "model.cuh"

namespace abc {

constexpr uint64_t kFnvOff = 0xcbf29ce484222325ull;
constexpr uint64_t kFnvPrime = 0x100000001b3ull;
enum : uint32_t { CH_ON = 0, CH_OFF = 1, CH_TXU = 2, CH_TXL = 3, CH_DEGU = 4, CH_DEGL = 5, CH_REJ = 6,
                  CH_NULL = 7, CH_SPLU = 8, CH_SPLL = 9, CH_DIV = 10 };

// status word bits
enum : int { STF_EVENT_CAP = 1, STF_OVERFLOW = 2, STF_NONFINITE = 4 };

struct SsaArgs {
  DevCfg cfg;
  const PRec* rec;
  const PRecF* recf;
  const int32_t* cell_cond;  // internal (group-sorted) order
  const int32_t* cell_age;
  const uint32_t* cell_id;   // caller's cell index (random stream id)
  const uint32_t* order;     // optional particle order (work-size descending), NULL = identity
  int64_t n_cells;
  int64_t n_items;           // particles * cells
  int64_t p_offset;          // global index of local particle 0
  uint64_t seed;
  int2* counts;              // [P][C] (u, l) raw counts at observation
  int64_t* events;           // optional [P][C]
  uint64_t* hash;            // optional [P][C]
  unsigned long long* counter;
  unsigned long long* totals;  // [0] fired events, [1] thinning rejections
  int* status;
  int want_hash;
  uint32_t rk[20];           // Philox round keys (seed + r * Weyl), filled by the FP32 launcher
};

struct Traj {
  double t, t_end, step_edge, lab_edge, cycle_start, t_obs, tlab_end;
  int k, lab_state, G;
  int uu, us, lu, ls;
  Rng rng;
  uint64_t hash;
  int64_t ev;
  int64_t out;
  int plocal;
  int stall;  // consecutive events that did not advance the clock
};

// A clock that stops advancing (propensities so large that t + tau == t) is
// reported instead of looping: after this many consecutive such events the
// trajectory ends with STF_NONFINITE.
constexpr int kMaxStall = 1024;

ABC_HD double traj_tend(const Traj& s) {
  double te = s.step_edge;
  if (s.lab_state < 2 && s.lab_edge < te) te = s.lab_edge;
  if (s.t_obs < te) te = s.t_obs;
  return te;
}

__device__ __forceinline__ void traj_init(Traj& s, const SsaArgs& A, int64_t item) {
  const DevCfg& cfg = A.cfg;
  int64_t pl = item / A.n_cells;
  int64_t ci = item - pl * A.n_cells;
  if (A.order) pl = (int64_t)A.order[pl];
  s.plocal = (int)pl;
  s.out = pl * A.n_cells + ci;
  const PRec& R = A.rec[pl];
  int j = A.cell_cond[ci], a = A.cell_age[ci];
  s.t_obs = cfg.ages[a];
  double texp = (s.t_obs - cfg.pulse[j]) - cfg.chase[j];
  s.tlab_end = texp + cfg.pulse[j];
  s.cycle_start = cfg.t0;
  s.t = cfg.t0;
  s.k = 0;
  s.step_edge = (cfg.n_steps == 1) ? s.cycle_start + cfg.cycle : s.cycle_start + cfg.step_len;
  s.lab_state = 0;
  s.lab_edge = texp;
  rng_init(s.rng, A.seed, ST_SSA, A.cell_id[ci], (uint32_t)(A.p_offset + pl));
  uint32_t w0, w1;
  rng_pair(s.rng, w0, w1);
  s.G = ((double)w0 * ABC_TWO_M32 < R.g0) ? 1 : 0;
  s.uu = (int)floor(R.u0 + 0.5);
  s.us = cfg.splicing ? (int)floor(R.s0 + 0.5) : 0;
  s.lu = 0;
  s.ls = 0;
  s.hash = kFnvOff;
  s.ev = 0;
  s.stall = 0;
  s.t_end = traj_tend(s);
}

// Breakpoint at s.t_end (already reached).  Returns true when the observation
// time is reached.
__device__ __forceinline__ bool traj_breakpoint(Traj& s, const DevCfg& cfg) {
  s.t = s.t_end;
  if (s.t == s.t_obs) return true;
  while (s.lab_state < 2 && s.t == s.lab_edge) {
    s.lab_state++;
    if (s.lab_state == 1) s.lab_edge = s.tlab_end;
  }
  if (s.t == s.step_edge) {
    s.k++;
    if (s.k == cfg.n_steps) {
      s.k = 0;
      s.cycle_start = s.cycle_start + cfg.cycle;
      s.uu = (int)binom_half(s.rng, s.uu);
      if (cfg.splicing) s.us = (int)binom_half(s.rng, s.us);
      s.lu = (int)binom_half(s.rng, s.lu);
      if (cfg.splicing) s.ls = (int)binom_half(s.rng, s.ls);
      s.hash = (s.hash ^ (uint64_t)CH_DIV) * kFnvPrime;
    }
    s.step_edge = (s.k == cfg.n_steps - 1) ? s.cycle_start + cfg.cycle
                                           : s.cycle_start + (double)(s.k + 1) * cfg.step_len;
  }
  s.t_end = traj_tend(s);
  return false;
}

// One iteration in FP64 (bit-exact with the CPU oracle).  Returns true when
// the trajectory is complete; ch_out receives the channel (for counters).
__device__ __forceinline__ bool step_fp64(Traj& s, const PRec& R, const DevCfg& cfg, uint32_t& ch) {
  const int k = s.k;
  const double gam = R.gam[k];
  double a_on = s.G ? 0.0 : R.kon[k];
  double a_off = s.G ? R.koff : 0.0;
  double a_tx = s.G ? R.amax[k] : 0.0;
  double c1 = a_on;
  double c2 = c1 + a_off;
  double c3 = c2 + a_tx;
  double c4, c5, c6, a_last, a0;
  if (!cfg.splicing) {
    double a_du = gam * (double)s.uu;
    a_last = gam * (double)s.lu;
    c4 = c3 + a_du;
    c5 = c4;
    c6 = c4;
    a0 = c4 + a_last;
  } else {
    double a_su = R.beta * (double)s.uu;
    double a_sl = R.beta * (double)s.lu;
    double a_du = gam * (double)s.us;
    a_last = gam * (double)s.ls;
    c4 = c3 + a_su;
    c5 = c4 + a_sl;
    c6 = c5 + a_du;
    a0 = c6 + a_last;
  }
  uint32_t w0, w1;
  rng_pair(s.rng, w0, w1);
  ch = CH_NULL;
  if (!(a0 > 0.0)) return traj_breakpoint(s, cfg);
  double U1 = ((double)w0 + 0.5) * ABC_TWO_M32;
  double tau = -xlog(U1) / a0;
  double tn = s.t + tau;
  if (tn >= s.t_end) return traj_breakpoint(s, cfg);
  s.stall = (tn == s.t) ? s.stall + 1 : 0;
  s.t = tn;
  double r = ((double)w1 * ABC_TWO_M32) * a0;
  if (r < c1) {
    s.G = 1;
    ch = CH_ON;
  } else if (r < c2) {
    s.G = 0;
    ch = CH_OFF;
  } else if (r < c3) {
    double v = r - c2;
    double at = R.alp[k] * xpow(1.0 + (s.t - s.cycle_start) / cfg.cycle, R.scal);
    if (v < at) {
      double lam_cur = (s.lab_state == 1) ? R.lam : 0.0;
      if (v < at * lam_cur) {
        s.lu++;
        ch = CH_TXL;
      } else {
        s.uu++;
        ch = CH_TXU;
      }
    } else {
      ch = CH_REJ;
    }
  } else if (!cfg.splicing) {
    if (r < c4) {
      s.uu--;
      ch = CH_DEGU;
    } else if (a_last > 0.0) {
      s.lu--;
      ch = CH_DEGL;
    }
  } else {
    if (r < c4) {
      s.uu--;
      s.us++;
      ch = CH_SPLU;
    } else if (r < c5) {
      s.lu--;
      s.ls++;
      ch = CH_SPLL;
    } else if (r < c6) {
      s.us--;
      ch = CH_DEGU;
    } else if (a_last > 0.0) {
      s.ls--;
      ch = CH_DEGL;
    }
  }
  s.hash = (s.hash ^ (uint64_t)ch) * kFnvPrime;
  return false;
}

// One iteration in FP32 (propensities, waiting time and selection in FP32,
// clock in FP64).  Uniforms: 24-bit U1 in (0,1), 24-bit U2 in [0,1).
struct RatesF {
  float kon, gam, amax, alp;  // current age step
  float koff, lam, beta, scal;
};

__device__ __forceinline__ float powf_fast(float x, float s) {
  if (s == 1.0f) return x;
  if (s == 0.0f) return 1.0f;
  return exp2f(s * __log2f(x));
}

__device__ __forceinline__ bool step_fp32(Traj& s, const RatesF& q, const DevCfg& cfg, float invT,
                                          uint32_t& ch) {
  float a_on = s.G ? 0.0f : q.kon;
  float a_off = s.G ? q.koff : 0.0f;
  float a_tx = s.G ? q.amax : 0.0f;
  float c1 = a_on;
  float c2 = c1 + a_off;
  float c3 = c2 + a_tx;
  float c4, c5, c6, a_last, a0;
  if (!cfg.splicing) {
    float a_du = q.gam * (float)s.uu;
    a_last = q.gam * (float)s.lu;
    c4 = c3 + a_du;
    c5 = c4;
    c6 = c4;
    a0 = c4 + a_last;
  } else {
    float a_su = q.beta * (float)s.uu;
    float a_sl = q.beta * (float)s.lu;
    float a_du = q.gam * (float)s.us;
    a_last = q.gam * (float)s.ls;
    c4 = c3 + a_su;
    c5 = c4 + a_sl;
    c6 = c5 + a_du;
    a0 = c6 + a_last;
  }
  uint32_t w0, w1;
  rng_pair(s.rng, w0, w1);
  ch = CH_NULL;
  if (!(a0 > 0.0f)) return traj_breakpoint(s, cfg);
  float U1 = fmaf((float)(w0 >> 8), 5.9604644775390625e-08f, 2.98023223876953125e-08f);
  float tau = __fdividef(-__logf(U1), a0);
  double tn = s.t + (double)tau;
  if (tn >= s.t_end) return traj_breakpoint(s, cfg);
  s.stall = (tn == s.t) ? s.stall + 1 : 0;
  s.t = tn;
  float r = ((float)(w1 >> 8) * 5.9604644775390625e-08f) * a0;
  if (r < c1) {
    s.G = 1;
    ch = CH_ON;
  } else if (r < c2) {
    s.G = 0;
    ch = CH_OFF;
  } else if (r < c3) {
    float v = r - c2;
    float size = 1.0f + (float)(s.t - s.cycle_start) * invT;
    float at = q.alp * powf_fast(size, q.scal);
    if (v < at) {
      float lam_cur = (s.lab_state == 1) ? q.lam : 0.0f;
      if (v < at * lam_cur) {
        s.lu++;
        ch = CH_TXL;
      } else {
        s.uu++;
        ch = CH_TXU;
      }
    } else {
      ch = CH_REJ;
    }
  } else if (!cfg.splicing) {
    if (r < c4) {
      s.uu--;
      ch = CH_DEGU;
    } else if (a_last > 0.0f) {
      s.lu--;
      ch = CH_DEGL;
    }
  } else {
    if (r < c4) {
      s.uu--;
      s.us++;
      ch = CH_SPLU;
    } else if (r < c5) {
      s.lu--;
      s.ls++;
      ch = CH_SPLL;
    } else if (r < c6) {
      s.us--;
      ch = CH_DEGU;
    } else if (a_last > 0.0f) {
      s.ls--;
      ch = CH_DEGL;
    }
  }
  return false;
}

__device__ __forceinline__ void load_rates(RatesF& q, const PRecF& F, int k) {
  q.kon = F.kon[k];
  q.gam = F.gam[k];
  q.amax = F.amax[k];
  q.alp = F.alp[k];
}
__device__ __forceinline__ void load_particle(RatesF& q, const PRecF& F) {
  q.koff = F.koff;
  q.lam = F.lam;
  q.beta = F.beta;
  q.scal = F.scal;
}

// Persistent driver.  FP64 = true: oracle mode; false: production mode.
// Iterations between work refills are grouped in quanta of kQuantum so the
// warp votes are amortised.
constexpr int kQuantum = 16;
constexpr int64_t kDefaultEventCap = (int64_t)1 << 28;
constexpr int kOverflowCount = 1 << 30;

template <bool FP64>
__global__ void __launch_bounds__(128) ssa_kernel(SsaArgs A) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const float invT = (float)(1.0 / A.cfg.cycle);
  const int64_t cap = A.cfg.event_cap > 0 ? A.cfg.event_cap : kDefaultEventCap;
  Traj s;
  RatesF q;
  bool active = false, done = false;
  int kprev = -1;
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
          if (!FP64) load_particle(q, A.recf[s.plocal]);
          active = true;
          kprev = -1;
        }
      }
    }
    if (__all_sync(FULL, done)) break;
    if (active) {
      const PRec& R = A.rec[s.plocal];
#pragma unroll 1
      for (int it = 0; it < kQuantum; ++it) {
        uint32_t ch;
        bool fin;
        if (FP64) {
          fin = step_fp64(s, R, A.cfg, ch);
        } else {
          if (s.k != kprev) {
            load_rates(q, A.recf[s.plocal], s.k);
            kprev = s.k;
          }
          fin = step_fp32(s, q, A.cfg, invT, ch);
          if (A.want_hash) s.hash = (s.hash ^ (uint64_t)ch) * kFnvPrime;
        }
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

}  // namespace abc
