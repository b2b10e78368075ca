// ssa_fp32.cuh — production SSA kernel (FP32 propensities, compensated FP32
// interval clock, FP64 only at breakpoints).
//
// Same reaction network, breakpoints and division as the FP64 oracle-mode
// kernel (ssa.cuh); what changes is how the work maps to the GB300:
//   * clock: within an interval (between two breakpoints, at most one age
//     step long) the elapsed time is an FP32 Kahan-compensated sum; the
//     interval start is kept in FP64 and every breakpoint re-anchors the
//     clock exactly, so no FP64 instruction runs per event (the FP64 pipe of
//     GB300 is narrow);
//   * random numbers: every iteration of every lane computes one Philox block
//     (U1 waiting time, U2 channel, U3 thinning/labelling), so all lanes run
//     Philox in lockstep; the round keys come precomputed in the kernel
//     parameters; uniforms are formed from mantissa bits (no int->float
//     conversion); division bits come from a disjoint counter range
//     (stream ST_AUX, block = cycle << 24 + i);
//   * molecule counts are FP32 integers (exact below 2^24; a count reaching
//     2^23 at a breakpoint is reported as ABC_ERR_NONFINITE), so propensities
//     need no conversion;
//   * channel update: predicated arithmetic, no divergent branches per event;
//   * lane state: a handful of registers, the breakpoint times are recomputed
//     from (cycle, step, labelling state, cell) when a breakpoint is reached.
// Results are a different (equally valid) realisation than the FP64 mode;
// they are reproducible for a given seed, independent of scheduling.
#pragma once
#include "ssa.cuh"

namespace abc {

constexpr float kCountLimitF = 8388608.0f;  // 2^23

struct LaneF {
  double t_bp;          // start of the current interval (FP64 breakpoints)
  int tq;               // the same in quanta of the breakpoint grid (integer breakpoints)
  float el, comp;       // elapsed time in the interval, Kahan compensation
  float len;            // interval length
  float ph0;            // cycle phase at the interval start
  float at0, at1;       // thinned transcription rate at0 + at1 x (elapsed time), scaling exponent 0 or 1
  float koff_amax;      // k_off + alpha_max of the current age step (the cumulative sum when G = 1)
  float lam_cur;        // labelling probability in this interval
  float uu, lu, us, ls; // molecule counts (exact integers in FP32)
  int k, cyc, lab, G;
  int j, a;
  int ev;               // fired events of this trajectory
  uint32_t block;       // next Philox block of the main stream
  uint32_t cell, particle;
  int plocal;
  int64_t out;
};

struct StepRates {
  float kon, gam, amax, alp;
};

__device__ __forceinline__ double f32_tend(const LaneF& s, const DevCfg& cfg) {
  const double cs = cfg.t0 + (double)s.cyc * cfg.cycle;
  double te = (s.k == cfg.n_steps - 1) ? cs + cfg.cycle : cs + (double)(s.k + 1) * cfg.step_len;
  const double tobs = cfg.ages[s.a];
  const double texp = (tobs - cfg.pulse[s.j]) - cfg.chase[s.j];
  if (s.lab == 0 && texp < te) te = texp;
  if (s.lab == 1 && texp + cfg.pulse[s.j] < te) te = texp + cfg.pulse[s.j];
  if (tobs < te) te = tobs;
  return te;
}

// the same on the integer breakpoint grid (DevCfg::grid_ok): every time is
// an exact integer number of quanta, so the interval end, its length and the
// cycle phase equal the FP64 ones bit for bit, without FP64 instructions
__device__ __forceinline__ int q_tend(const LaneF& s, const DevCfg& cfg) {
  const int cs = cfg.t0_q + s.cyc * cfg.cycle_q;
  int te = (s.k == cfg.n_steps - 1) ? cs + cfg.cycle_q : cs + (s.k + 1) * cfg.step_q;
  const int tobs = cfg.ages_q[s.a];
  const int texp = (tobs - cfg.pulse_q[s.j]) - cfg.chase_q[s.j];
  if (s.lab == 0 && texp < te) te = texp;
  if (s.lab == 1 && texp + cfg.pulse_q[s.j] < te) te = texp + cfg.pulse_q[s.j];
  if (tobs < te) te = tobs;
  return te;
}

template <bool GRID>
__device__ __forceinline__ void f32_interval(LaneF& s, const DevCfg& cfg, float lam, float alp, float scal,
                                             float invT) {
  if (GRID) {
    const int cs = cfg.t0_q + s.cyc * cfg.cycle_q;
    const int te = q_tend(s, cfg);
    s.len = (float)(te - s.tq) * cfg.quantum;
    s.ph0 = (float)(s.tq - cs) * cfg.quantum;
  } else {
    const double cs = cfg.t0 + (double)s.cyc * cfg.cycle;
    const double te = f32_tend(s, cfg);
    s.len = (float)(te - s.t_bp);
    s.ph0 = (float)(s.t_bp - cs);
  }
  s.el = 0.0f;
  s.comp = 0.0f;
  s.lam_cur = (s.lab == 1) ? lam : 0.0f;
  // alpha size^s with size = 1 + phase / T is linear in the elapsed time for s in {0, 1}
  s.at1 = alp * scal * invT;
  s.at0 = alp * fmaf(scal, s.ph0 * invT, 1.0f);
}

// Philox4x32-10 with precomputed round keys rk[2r], rk[2r+1].
__device__ __forceinline__ U4 philox_rk(U4 c, const uint32_t* rk) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c.z;
    U4 n;
    n.x = (uint32_t)(p1 >> 32) ^ c.y ^ rk[2 * r];
    n.y = (uint32_t)p1;
    n.z = (uint32_t)(p0 >> 32) ^ c.w ^ rk[2 * r + 1];
    n.w = (uint32_t)p0;
    c = n;
  }
  return c;
}

__device__ __forceinline__ U4 main_block(const LaneF& s, const uint32_t* rk) {
  U4 c;
  c.x = s.block;
  c.y = ST_SSA << 30;
  c.z = s.cell;
  c.w = s.particle;
  return philox_rk(c, rk);
}

// uniform in [0, 1) from the top 23 bits of a word (mantissa fill, no conversion)
__device__ __forceinline__ float u23(uint32_t w) { return __uint_as_float(0x3F800000u | (w >> 9)) - 1.0f; }

// Bin(n, 1/2) from the division stream of cycle `cyc`.
__device__ __forceinline__ float f32_halve(float nf, uint32_t& blk, const LaneF& s, const uint32_t* rk) {
  int n = (int)nf;
  int k = 0;
  while (n > 0) {
    U4 c;
    c.x = blk++;
    c.y = ST_AUX << 30;
    c.z = s.cell;
    c.w = s.particle;
    U4 o = philox_rk(c, rk);
    uint64_t lo = ((uint64_t)o.y << 32) | o.x;
    uint64_t hi = ((uint64_t)o.w << 32) | o.z;
    if (n < 64) lo &= (((uint64_t)1) << n) - 1;
    k += __popcll(lo);
    n -= 64;
    if (n > 0) {
      if (n < 64) hi &= (((uint64_t)1) << n) - 1;
      k += __popcll(hi);
      n -= 64;
    }
  }
  return (float)k;
}

// MINB: resident 128-thread blocks per SM the register allocation targets
// (8: no spills; 10: 48 registers with a few spills) -- chosen at run time by
// the autotuner (abc_autotune).
template <bool SPLICE, int MINB, bool GRID>
__global__ void __launch_bounds__(128, MINB) ssa_kernel_f32(SsaArgs A) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const DevCfg& cfg = A.cfg;
  const float invT = (float)(1.0 / cfg.cycle);
  const int cap = (int)(cfg.event_cap > 0 && cfg.event_cap < (int64_t)1 << 30 ? cfg.event_cap : kDefaultEventCap);
  LaneF s;
  StepRates q;
  float koff = 0.f, lam = 0.f, beta = 0.f, scal = 0.f;
  bool active = false, done = false;
  // Random words: each iteration consumes two words of the lane's stream
  // (blocks 1, 2, ... of its (cell, particle) counter, in order).  cur holds
  // the block being read (half: its z, w next), nxt the following one.  New
  // blocks are computed on even warp iterations only, by every lane whose nxt
  // is empty, so the Philox rounds run for the whole warp every other
  // iteration; two words per iteration and four per refill keep cur + nxt
  // from running dry whatever the iteration at which an item starts.
  U4 cur = {0u, 0u, 0u, 0u}, nxt = {0u, 0u, 0u, 0u};
  bool half = false, has_nxt = false;
  uint32_t it = 0;
  unsigned long long tot_ev = 0, tot_rej = 0;
  unsigned rej32 = 0;  // rejections since the lane's last item boundary (folded into tot_rej there)
  bool scal01 = true;
  int err = 0;
  s.plocal = 0;
  while (true) {
    ++it;
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
          int64_t pl = (int64_t)(item / (unsigned long long)A.n_cells);
          const int64_t ci = (int64_t)item - pl * A.n_cells;
          if (A.order) pl = (int64_t)A.order[pl];
          s.plocal = (int)pl;
          s.out = pl * A.n_cells + ci;
          s.j = A.cell_cond[ci];
          s.a = A.cell_age[ci];
          s.cell = A.cell_id[ci];
          s.particle = (uint32_t)(A.p_offset + pl);
          const PRecF& F = A.recf[pl];
          const PRec& R = A.rec[pl];
          koff = F.koff;
          lam = F.lam;
          beta = F.beta;
          scal = F.scal;
          scal01 = scal == 0.0f || scal == 1.0f;
          s.k = 0;
          s.cyc = 0;
          s.lab = 0;
          s.t_bp = cfg.t0;
          s.tq = cfg.t0_q;
          s.block = 0;
          const U4 w = main_block(s, A.rk);
          s.block = 1;
          cur = main_block(s, A.rk);
          s.block = 2;
          half = false;
          has_nxt = false;
          s.G = ((double)w.x * ABC_TWO_M32 < R.g0) ? 1 : 0;
          s.uu = floorf((float)R.u0 + 0.5f);
          s.us = SPLICE ? floorf((float)R.s0 + 0.5f) : 0.0f;
          s.lu = 0.0f;
          s.ls = 0.0f;
          s.ev = 0;
          q.kon = F.kon[0];
          q.gam = F.gam[0];
          q.amax = F.amax[0];
          q.alp = F.alp[0];
          s.koff_amax = koff + q.amax;
          f32_interval<GRID>(s, cfg, lam, q.alp, scal, invT);
          if (!(s.uu < kCountLimitF) || !(s.us < kCountLimitF)) err |= STF_OVERFLOW;
          active = true;
        }
      }
      // done only changes here, so the warp's exit test runs only after a refill
      if (__all_sync(FULL, done)) break;
    }
    if (!active) continue;

    // ---- one iteration: propensities, Philox block, waiting time
    // cumulative propensities: one of k_on, k_off is zero, so c2 and c3 are
    // selections (k_off + alpha_max is summed once per age step)
    float c4, c5 = 0.f, c6 = 0.f, a_last, a0;
    const float c1 = s.G ? 0.0f : q.kon, c2 = s.G ? koff : q.kon, c3 = s.G ? s.koff_amax : q.kon;
    if (!SPLICE) {
      a_last = q.gam * s.lu;
      c4 = fmaf(q.gam, s.uu, c3);
      a0 = c4 + a_last;
    } else {
      a_last = q.gam * s.ls;
      c4 = fmaf(beta, s.uu, c3);
      c5 = fmaf(beta, s.lu, c4);
      c6 = fmaf(q.gam, s.us, c5);
      a0 = c6 + a_last;
    }
    if ((it & 1u) == 0u && !has_nxt) {
      nxt = main_block(s, A.rk);
      s.block++;
      has_nxt = true;
    }
    const uint32_t wt = half ? cur.z : cur.x;  // waiting time (top 23 bits)
    const uint32_t wc = half ? cur.w : cur.y;  // channel (top 23 bits)
    if (half) {
      if (!has_nxt) {  // not reached by the refill schedule; keeps the stream order regardless
        nxt = main_block(s, A.rk);
        s.block++;
      }
      cur = nxt;
      has_nxt = false;
    }
    half = !half;
    const float U1 = 1.0f - u23(wt);  // (0, 1]
    const float tau = __fdividef(-__logf(U1), a0);
    const float y = tau - s.comp;
    const float tt = s.el + y;
    const float nc = (tt - s.el) - y;
    if (!((tt - nc) < s.len)) {
      // ---- breakpoint (interval end reached, or no reaction possible)
      bool fin, at_step;
      if (GRID) {
        s.tq = q_tend(s, cfg);
        fin = s.tq == cfg.ages_q[s.a];
        const int texp = (cfg.ages_q[s.a] - cfg.pulse_q[s.j]) - cfg.chase_q[s.j];
        while (!fin && s.lab < 2 && s.tq == (s.lab == 0 ? texp : texp + cfg.pulse_q[s.j])) s.lab++;
        const int cs = cfg.t0_q + s.cyc * cfg.cycle_q;
        at_step = s.tq == ((s.k == cfg.n_steps - 1) ? cs + cfg.cycle_q : cs + (s.k + 1) * cfg.step_q);
      } else {
        s.t_bp = f32_tend(s, cfg);
        fin = s.t_bp == cfg.ages[s.a];
        const double texp = (cfg.ages[s.a] - cfg.pulse[s.j]) - cfg.chase[s.j];
        while (!fin && s.lab < 2 && s.t_bp == (s.lab == 0 ? texp : texp + cfg.pulse[s.j])) s.lab++;
        const double cs = cfg.t0 + (double)s.cyc * cfg.cycle;
        at_step = s.t_bp == ((s.k == cfg.n_steps - 1) ? cs + cfg.cycle : cs + (double)(s.k + 1) * cfg.step_len);
      }
      if (!fin) {
        if (at_step) {
          s.k++;
          if (s.k == cfg.n_steps) {
            s.k = 0;
            s.cyc++;
            uint32_t blk = (uint32_t)s.cyc << 24;
            s.uu = f32_halve(s.uu, blk, s, A.rk);
            if (SPLICE) s.us = f32_halve(s.us, blk, s, A.rk);
            s.lu = f32_halve(s.lu, blk, s, A.rk);
            if (SPLICE) s.ls = f32_halve(s.ls, blk, s, A.rk);
          }
          const PRecF& F = A.recf[s.plocal];
          q.kon = F.kon[s.k];
          q.gam = F.gam[s.k];
          q.amax = F.amax[s.k];
          q.alp = F.alp[s.k];
          s.koff_amax = koff + q.amax;
        }
        f32_interval<GRID>(s, cfg, lam, q.alp, scal, invT);
        if (!(s.uu < kCountLimitF) || !(s.lu < kCountLimitF) || !(s.us < kCountLimitF) || !(s.ls < kCountLimitF)) {
          err |= STF_OVERFLOW;
          fin = true;
        }
      }
      if (fin) {
        A.counts[s.out] = make_int2((int)(s.uu + s.us), (int)(s.lu + s.ls));
        if (A.events) A.events[s.out] = s.ev;
        tot_ev += (unsigned long long)s.ev;
        tot_rej += rej32;
        rej32 = 0;
        active = false;
      }
      continue;
    }
    // ---- event: predicated channel update
    s.el = tt;
    s.comp = nc;
    const float r = u23(wc) * a0;
    const bool b1 = r >= c1, b2 = r >= c2, b3 = r >= c3, b4 = r >= c4;
    // alpha size^s: the per-interval linear form for s in {0, 1}, the general
    // power only for lanes with another exponent (a warp-uniform skip for the
    // reference's models)
    const float dt = s.el - s.comp;
    float at = fmaf(s.at1, dt, s.at0);
    if (!scal01) at = q.alp * exp2f(scal * __log2f(fmaf(s.ph0 + dt, invT, 1.0f)));
    // thinning uniform from the 9 low bits of both words (18 bits), x bound
    const uint32_t th = ((wt & 0x1FFu) << 9) | (wc & 0x1FFu);
    const float v = (__uint_as_float(0x3F800000u | (th << 5)) - 1.0f) * q.amax;
    const bool tx = b2 && !b3;
    const bool acc = tx && (v < at);
    const bool lab = acc && (v < at * s.lam_cur);
    s.G = !b1 ? 1 : (!b2 ? 0 : s.G);
    bool fired;
    if (!SPLICE) {
      const bool dl = b4 && (a_last > 0.0f);
      s.uu += ((acc && !lab) ? 1.0f : 0.0f) - ((b3 && !b4) ? 1.0f : 0.0f);
      s.lu += (lab ? 1.0f : 0.0f) - (dl ? 1.0f : 0.0f);
      fired = (!tx || acc) && (!b4 || dl);
    } else {
      const bool b5 = r >= c5, b6 = r >= c6;
      const bool su = b3 && !b4, sl = b4 && !b5, du = b5 && !b6, dl = b6 && (a_last > 0.0f);
      s.uu += ((acc && !lab) ? 1.0f : 0.0f) - (su ? 1.0f : 0.0f);
      s.us += (su ? 1.0f : 0.0f) - (du ? 1.0f : 0.0f);
      s.lu += (lab ? 1.0f : 0.0f) - (sl ? 1.0f : 0.0f);
      s.ls += (sl ? 1.0f : 0.0f) - (dl ? 1.0f : 0.0f);
      fired = (!tx || acc) && (!b6 || dl);
    }
    s.ev += fired ? 1 : 0;
    rej32 += (tx && !acc) ? 1u : 0u;
    if (s.ev > cap) {
      err |= STF_EVENT_CAP;
      A.counts[s.out] = make_int2((int)(s.uu + s.us), (int)(s.lu + s.ls));
      if (A.events) A.events[s.out] = s.ev;
      tot_ev += (unsigned long long)s.ev;
      tot_rej += rej32;
      rej32 = 0;
      active = false;
    }
  }
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
