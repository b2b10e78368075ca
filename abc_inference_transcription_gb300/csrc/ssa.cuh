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
  int chunk = 1;             // production kernel: consecutive items a lane takes per pull
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
  if (cfg.splicing) {
    s.uu = (int)floor(R.u0 + 0.5);
    s.us = (int)floor(R.s0 + 0.5);
  } else {
    // moment-matched draw from the periodic state (initial_count), auxiliary stream blocks 0, 1, ...
    Rng aux;
    rng_init(aux, A.seed, ST_AUX, A.cell_id[ci], (uint32_t)(A.p_offset + pl));
    s.uu = (int)initial_count(R, s.G, w1, aux);
    s.us = 0;
  }
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

// Persistent driver of the FP64 oracle mode.  Iterations between work
// refills are grouped in quanta of kQuantum so the warp votes are amortised.
constexpr int kQuantum = 16;
constexpr int64_t kDefaultEventCap = (int64_t)1 << 28;
constexpr int kOverflowCount = 1 << 30;

}  // namespace abc
