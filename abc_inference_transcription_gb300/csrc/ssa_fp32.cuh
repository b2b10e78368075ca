// ssa_fp32.cuh — production SSA kernel (FP32 propensities, compensated FP32
// interval clock, breakpoints on an integer grid or in FP64).
//
// Same reaction network, breakpoints and division as the FP64 oracle-mode
// kernel (ssa.cuh); what changes is how the work maps to the GB300:
//   * trips: all lanes of a warp run in lockstep, two SSA iterations per
//     trip, both fed by one Philox4x32-10 block of the lane's stream (words
//     x, y for the first iteration, z, w for the second).  A lane that
//     reaches a breakpoint in the first iteration leaves the second one's
//     words unused, so the stream a trajectory consumes depends only on the
//     trajectory itself (reproducible, independent of scheduling).  The
//     counter words that are constant for a trajectory (stream, cell,
//     particle) are folded into the first Philox round once per trajectory;
//   * clock: within an interval (between two breakpoints, at most one age
//     step long) the elapsed time is an FP32 Kahan-compensated sum; the
//     interval start is an integer number of grid quanta (or FP64 when the
//     configuration's times are not on a power-of-two grid), so breakpoints
//     are exact and no FP64 instruction runs per event;
//   * waiting time from the low 23 bits of one word, the channel from a full
//     32-bit uniform of the other (rare channels keep their probability to
//     2^-32 of the total propensity);
//   * channels: [switch | decay u | decay l | transcription proposal], so
//     the switch toggles G and a proposal landing at the top by rounding is a
//     rejection.  Transcription alpha size(t)^s is thinned against its value
//     at the interval end (linear in time for s in {0, 1}: at0 + at1 t).
//     The channel is taken from 0/1 step values of the cumulative thresholds
//     and the counts and G are updated with FP32 arithmetic on them, which
//     runs on the full-rate FMA pipe instead of compare/select/predicate
//     instructions on the half-rate ALU pipe (the limit of this kernel);
//   * the hot loop (a trip) has no divergent control flow: breakpoints,
//     divisions, finished trajectories, refills and the event cap are handled
//     behind one warp-uniform test; events and rejections are counted in FP32
//     and flushed to integers at breakpoints;
//   * division: the lanes of the warp that divide in the same trip are
//     served one after another by the whole warp: each lane popcounts 1/32
//     of the Bin(n, 1/2) bits (stream ST_AUX, blocks cycle << 24 + i, the
//     bits of the FP64 mode's sampler layout in 128-bit blocks), summed with
//     a warp reduction;
//   * molecule counts are FP32 integers (exact below 2^24; a count reaching
//     2^23 at a breakpoint is reported as ABC_ERR_NONFINITE);
//   * work: each lane pulls `chunk` consecutive (particle, cell) items per
//     warp-aggregated atomic from the LPT-ordered particle list.
// Results are a different (equally valid) realisation than the FP64 mode.
#pragma once
#include <limits.h>

#include "ssa.cuh"

namespace abc {

constexpr float kCountLimitF = 8388608.0f;  // 2^23

// breakpoint times: integer quanta (GRID) or FP64
template <bool GRID>
struct BpTime {
  using T = double;
  __device__ static double never() { return INFINITY; }
};
template <>
struct BpTime<true> {
  using T = int32_t;
  __device__ static int32_t never() { return INT_MAX; }
};

template <bool GRID>
struct LaneF {
  using T = typename BpTime<GRID>::T;
  T te;                  // end of the current interval: the next breakpoint
  T step_edge;           // end of the current age step
  T lab_edge;            // next labelling edge (window start, then end, then never)
  T tlab_end;            // end of the labelling window
  T tobs;                // observation time (the cell's age)
  T cs;                  // start of the current cycle
  float el, comp;        // elapsed time in the interval, Kahan compensation
  float len;             // interval length
  float at0, at1;        // transcription rate at0 + at1 x (elapsed time), exponent s in {0, 1}
  float amax;            // its value at the interval end: the thinning bound
  float lamc;            // labelling probability in this interval
  float ph0;             // cycle phase at the interval start (general exponent only)
  float kon, gam;        // rates of the current age step
  float alp, scal;       // transcription rate of the step and size exponent (general exponent only)
  float uu, lu, us, ls;  // molecule counts (exact integers in FP32)
  float G;               // gene state, 0 or 1
  float evf, rejf;       // iterations that were not breakpoints, and rejections among them, since the last flush
  int k, lab, cyc;
  int ev;                // flushed iteration count of this trajectory
  int rej;               // flushed thinning rejections
  uint32_t block;        // next Philox block of the main stream
  uint32_t r1x, r1y, r1z;  // first Philox round: the trajectory's constant counter words folded in
  int plocal, ci;
};

// 0xCD9E8D57^-1 mod 2^32: the cell index back from the folded round-1 word r1y
constexpr uint32_t kPhiloxM1Inv = 0x6D7CAE67u;

// Philox4x32-10 with precomputed round keys rk[2r], rk[2r+1] (general counter).
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

// Block `block` of the main stream, counter (block, ST_SSA << 30, cell,
// particle): the first Philox round needs only the product of the block word, the rest of
// it (r1x, r1y, r1z) is fixed per trajectory.
__device__ __forceinline__ U4 main_block(uint32_t block, uint32_t r1x, uint32_t r1y, uint32_t r1z,
                                         const uint32_t* rk) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)block;
  U4 c;
  c.x = r1x;
  c.y = r1y;
  c.z = (uint32_t)(p0 >> 32) ^ r1z;
  c.w = (uint32_t)p0;
#pragma unroll
  for (int r = 1; r < 10; ++r) {
    const uint64_t q0 = (uint64_t)0xD2511F53u * (uint64_t)c.x;
    const uint64_t q1 = (uint64_t)0xCD9E8D57u * (uint64_t)c.z;
    U4 n;
    n.x = (uint32_t)(q1 >> 32) ^ c.y ^ rk[2 * r];
    n.y = (uint32_t)q1;
    n.z = (uint32_t)(q0 >> 32) ^ c.w ^ rk[2 * r + 1];
    n.w = (uint32_t)q0;
    c = n;
  }
  return c;
}

template <bool GRID>
__device__ __forceinline__ void fold_round1(LaneF<GRID>& s, uint32_t cell, uint32_t particle, const uint32_t* rk) {
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)cell;
  s.r1x = (uint32_t)(p1 >> 32) ^ (ST_SSA << 30) ^ rk[0];
  s.r1y = (uint32_t)p1;  // = cell * 0xCD9E8D57 mod 2^32
  s.r1z = particle ^ rk[1];
}

// Interval from t to the next breakpoint: its length, the thinning form of
// the transcription rate and its bound.  The particle's labelling
// probability, size exponent and the step's transcription rate are read from
// its record here (breakpoints only), so they hold no registers in the loop.
template <bool GRID, bool GENSCAL>
__device__ __forceinline__ void set_interval(LaneF<GRID>& s, typename LaneF<GRID>::T t, const DevCfg& cfg,
                                             const PRecF& F, float invT) {
  typename LaneF<GRID>::T te = s.step_edge;
  if (s.lab_edge < te) te = s.lab_edge;
  if (s.tobs < te) te = s.tobs;
  s.te = te;
  float ph0;
  if (GRID) {
    s.len = (float)(te - t) * cfg.quantum;
    ph0 = (float)(t - s.cs) * cfg.quantum;
  } else {
    s.len = (float)(te - t);
    ph0 = (float)(t - s.cs);
  }
  s.el = 0.0f;
  s.comp = 0.0f;
  s.lamc = (s.lab == 1) ? F.lam : 0.0f;
  const float alp = F.alp[s.k], scal = F.scal;
  if (!GENSCAL) {
    // alpha size^s with size = 1 + phase / T is linear in the elapsed time for
    // s in {0, 1}; fmaf is monotone in t, so its value at len bounds every
    // value the events of the interval compute
    s.at1 = alp * scal * invT;
    s.at0 = alp * fmaf(scal, ph0 * invT, 1.0f);
    s.amax = fmaf(s.at1, s.len, s.at0);
  } else {
    s.ph0 = ph0;
    s.alp = alp;
    s.scal = scal;
    // size^s is increasing in the phase (s >= 0): the value at the interval end, with margin
    s.amax = alp * exp2f(scal * __log2f(fmaf(ph0 + s.len, invT, 1.0f))) * 1.00001f;
  }
}

// 1 where the channel uniform r has passed threshold c, else 0
__device__ __forceinline__ float past(float r, float c) { return r >= c ? 1.0f : 0.0f; }

// One SSA iteration from two random words.  Returns true when the interval
// end (len) comes before the next reaction: a breakpoint, with the lane's
// state unchanged.  Otherwise applies the event or the thinning rejection.
// The channel is found from 0/1 step values of the cumulative thresholds and
// every update is FP32 arithmetic on them (FMA pipe), not selects: for
// thresholds h1 <= h2 <= ... each channel's indicator is a difference of
// neighbouring steps.  G is 0.0 or 1.0, so G x (rate) selects exactly.
template <bool SPLICE, bool GENSCAL, bool GRID>
__device__ __forceinline__ bool ev_step(LaneF<GRID>& s, float koff, float beta, float invT, float len, uint32_t wt,
                                        uint32_t wc) {
  const float G = s.G;
  const float sw = fmaf(G, koff, fmaf(-G, s.kon, s.kon));  // k_off if on, k_on if off (exact)
  float c2, c3 = 0.0f, c4 = 0.0f, top;
  if (!SPLICE) {
    c2 = fmaf(s.gam, s.uu, sw);   // decay of u
    top = fmaf(s.gam, s.lu, c2);  // decay of l
  } else {
    c2 = fmaf(beta, s.uu, sw);    // splicing of unlabelled
    c3 = fmaf(beta, s.lu, c2);    // splicing of labelled
    c4 = fmaf(s.gam, s.us, c3);   // decay of unlabelled spliced
    top = fmaf(s.gam, s.ls, c4);  // decay of labelled spliced
  }
  const float a0 = fmaf(G, s.amax, top);  // + transcription proposals (thinning bound) when on
  // waiting time: U1 in (0, 1] from the low 23 bits of wt (mantissa fill);
  // the rates are in log2 units, so -log2(U1) / a0 is the time
  const float U1 = 2.0f - __uint_as_float(0x3F800000u | (wt & 0x7FFFFFu));
  const float tau = __fdividef(-__log2f(U1), a0);  // a0 = 0 gives inf or NaN: a breakpoint
  const float y = tau - s.comp;
  const float tt = s.el + y;
  // no branch: at a breakpoint (ok = 0) every update of the counts, G and the
  // counters below is multiplied by zero, so the lane's state is unchanged;
  // the clock (el, comp) may advance past the interval, since the breakpoint
  // that follows starts a new interval at el = comp = 0
  const bool ok = tt < len;
  const float okf = ok ? 1.0f : 0.0f;
  s.comp = (tt - s.el) - y;
  s.el = tt;
  s.evf += okf;
  // channel: 32-bit uniform times a0
  const float r = __uint2float_rn(wc) * (a0 * 2.3283064365386963e-10f);
  float at;
  if (!GENSCAL)
    at = fmaf(s.at1, tt, s.at0);
  else
    at = s.alp * exp2f(s.scal * __log2f(fmaf(s.ph0 + tt, invT, 1.0f)));
  at = at * G;  // no transcription while off
  // [switch | ... | labelled tx | unlabelled tx | rejection] above top
  const float hs = past(r, sw), h2 = past(r, c2), ht = past(r, top);
  const float hl = past(r, fmaf(at, s.lamc, top)), ha = past(r, top + at);
  s.G = fmaf(okf - okf * hs, fmaf(-2.0f, G, 1.0f), G);  // r < sw: switch
  if (!SPLICE) {
    s.uu = fmaf(okf, (hl - ha) - (hs - h2), s.uu);  // unlabelled transcription - decay of u
    s.lu = fmaf(okf, (ht - hl) - (h2 - ht), s.lu);  // labelled transcription - decay of l
  } else {
    const float h3 = past(r, c3), h4 = past(r, c4);
    s.uu = fmaf(okf, (hl - ha) - (hs - h2), s.uu);  // transcription - splicing
    s.us = fmaf(okf, (hs - h2) - (h3 - h4), s.us);  // splicing - decay
    s.lu = fmaf(okf, (ht - hl) - (h2 - h3), s.lu);
    s.ls = fmaf(okf, (h2 - h3) - (h4 - ht), s.ls);
  }
  s.rejf = fmaf(okf, ha, s.rejf);  // thinning rejection (or a proposal that rounding put at the top)
  return !ok;
}

// Breakpoint at s.te (reached): labelling state, age step, cycle (division
// flagged in div; the counts are halved by the warp afterwards), next
// interval.  Returns true when the observation time is reached.
template <bool GRID, bool GENSCAL>
__device__ __forceinline__ bool on_breakpoint(LaneF<GRID>& s, const DevCfg& cfg, const PRecF* recf, float invT,
                                              bool& div) {
  using T = typename LaneF<GRID>::T;
  const T t = s.te;
  if (t == s.tobs) return true;
  while (s.lab < 2 && t == s.lab_edge) {
    s.lab++;
    s.lab_edge = (s.lab == 1) ? s.tlab_end : BpTime<GRID>::never();
  }
  const PRecF& F = recf[s.plocal];
  if (t == s.step_edge) {
    const T cyc_len = GRID ? (T)cfg.cycle_q : (T)cfg.cycle;
    const T step_len = GRID ? (T)cfg.step_q : (T)cfg.step_len;
    s.k++;
    if (s.k == cfg.n_steps) {
      s.k = 0;
      s.cs = s.cs + cyc_len;
      s.cyc++;
      div = true;
    }
    s.step_edge = (s.k == cfg.n_steps - 1) ? s.cs + cyc_len : s.cs + (T)(s.k + 1) * step_len;
    s.kon = F.kon[s.k];
    s.gam = F.gam[s.k];
  }
  set_interval<GRID, GENSCAL>(s, t, cfg, F, invT);
  return false;
}

// Bin(n, 1/2) of every species of lane L, computed by the whole warp.  The
// bits are those of the division sampler's layout: species in the order u,
// [spliced u], l, [spliced l], each from a fresh 128-bit block, blocks
// cycle << 24, +1, ... of stream ST_AUX; block i holds bits 128 i .. 128 i + 127
// (x, y low then z, w high).
__device__ __forceinline__ int warp_halve(int n, uint32_t& blk, uint32_t cell, uint32_t particle, int lane,
                                          const uint32_t* rk) {
  const int nb = (n + 127) >> 7;
  int k = 0;
  for (int i = lane; i < nb; i += 32) {
    U4 c;
    c.x = blk + (uint32_t)i;
    c.y = ST_AUX << 30;
    c.z = cell;
    c.w = particle;
    const U4 o = philox_rk(c, rk);
    uint64_t lo = ((uint64_t)o.y << 32) | o.x;
    uint64_t hi = ((uint64_t)o.w << 32) | o.z;
    const int m = n - (i << 7);
    if (m < 64) {
      lo &= (((uint64_t)1) << m) - 1;
      hi = 0;
    } else if (m < 128) {
      const int mh = m - 64;
      hi = (mh == 0) ? 0 : (hi & ((((uint64_t)1) << mh) - 1));
    }
    k += __popcll(lo) + __popcll(hi);
  }
  blk += (uint32_t)nb;
  return (int)__reduce_add_sync(0xffffffffu, (unsigned)k);
}

// Events and rejections counted in FP32 since the last flush: flushed to the
// integer counts at breakpoints and when the count reaches this (exact below 2^24)
constexpr float kFlushF = 4194304.0f;  // 2^22

template <bool GRID>
__device__ __forceinline__ void flush_counts(LaneF<GRID>& s) {
  s.ev += (int)s.evf;
  s.rej += (int)s.rejf;
  s.evf = 0.0f;
  s.rejf = 0.0f;
}

// MINB: resident 128-thread blocks per SM the register allocation targets
// (chosen at run time by the autotuner, abc_autotune).  GENSCAL: a general
// size exponent (the scaling column of theta) instead of s in {0, 1}.
//
// Loop shape: the hot part is one trip (a Philox block and two iterations)
// with no divergent control flow; everything rare -- breakpoints, divisions,
// finished trajectories, refills, the event cap -- is handled behind one
// warp-uniform test, for the lanes that need it.
template <bool SPLICE, int MINB, bool GRID, bool GENSCAL>
__global__ void __launch_bounds__(128, MINB) ssa_kernel_f32(SsaArgs A) {
  using T = typename LaneF<GRID>::T;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const DevCfg& cfg = A.cfg;
  const float invT = (float)(1.0 / cfg.cycle);
  const int cap = (int)(cfg.event_cap > 0 && cfg.event_cap < (int64_t)1 << 30 ? cfg.event_cap : kDefaultEventCap);
  const int chunk = A.chunk > 0 ? A.chunk : 1;
  __shared__ unsigned long long sh_tot[2];
  if (threadIdx.x < 2) sh_tot[threadIdx.x] = 0;
  __syncthreads();
  LaneF<GRID> s;
  s.block = 0;
  s.r1x = s.r1y = s.r1z = 0;
  s.len = -1.0f;  // no trajectory: every iteration is a breakpoint, which an inactive lane ignores
  s.el = s.comp = 0.0f;
  s.evf = s.rejf = 0.0f;
  float koff = 0.f, beta = 0.f;
  bool active = false, done = false;
  // work cursor: the launch keeps n_items below 2^31 (the host splits larger batches)
  uint32_t inext = 0;
  int left = 0;  // items left in this lane's pulled chunk
  int err = 0;
  bool bp = false, special = true;
  while (true) {
    if (__any_sync(FULL, special)) {
      // ---- breakpoints (divergent, short); divisions are flagged for the warp
      bool fin = false, div = false;
      if (active && bp) {
        flush_counts(s);
        fin = on_breakpoint<GRID, GENSCAL>(s, cfg, A.recf, invT, div);
      }
      // ---- divisions of this trip, one lane after another, by the whole warp
      unsigned dm = __ballot_sync(FULL, div);
      while (dm) {
        const int L = __ffs(dm) - 1;
        dm &= dm - 1u;
        const uint32_t cL = __shfl_sync(FULL, s.r1y, L) * kPhiloxM1Inv;
        const uint32_t pL = __shfl_sync(FULL, s.r1z, L) ^ A.rk[1];
        uint32_t blk = (uint32_t)__shfl_sync(FULL, s.cyc, L) << 24;
        const int nu = warp_halve((int)__shfl_sync(FULL, s.uu, L), blk, cL, pL, lane, A.rk);
        int ns = 0, nsl = 0;
        if (SPLICE) ns = warp_halve((int)__shfl_sync(FULL, s.us, L), blk, cL, pL, lane, A.rk);
        const int nl = warp_halve((int)__shfl_sync(FULL, s.lu, L), blk, cL, pL, lane, A.rk);
        if (SPLICE) nsl = warp_halve((int)__shfl_sync(FULL, s.ls, L), blk, cL, pL, lane, A.rk);
        if (lane == L) {
          s.uu = (float)nu;
          s.lu = (float)nl;
          if (SPLICE) {
            s.us = (float)ns;
            s.ls = (float)nsl;
          }
        }
      }
      if (active) {
        if (bp && !fin &&
            (!(s.uu < kCountLimitF) || !(s.lu < kCountLimitF) || !(s.us < kCountLimitF) || !(s.ls < kCountLimitF))) {
          err |= STF_OVERFLOW;
          fin = true;
        }
        if (!bp && s.evf >= kFlushF) flush_counts(s);
        if (s.ev - s.rej > cap) {
          err |= STF_EVENT_CAP;
          fin = true;
        }
        if (fin) {
          flush_counts(s);
          const int64_t out = (int64_t)s.plocal * A.n_cells + s.ci;
          A.counts[out] = make_int2((int)(s.uu + s.us), (int)(s.lu + s.ls));
          if (A.events) A.events[out] = s.ev - s.rej;
          atomicAdd(&sh_tot[0], (unsigned long long)(s.ev - s.rej));
          atomicAdd(&sh_tot[1], (unsigned long long)s.rej);
          active = false;
          s.len = -1.0f;
        }
      }
      // ---- lanes without a trajectory take the next item of their chunk, or pull a chunk
      const bool need = !active && !done;
      if (__any_sync(FULL, need)) {
        const bool pull = need && left == 0;
        const unsigned pm = __ballot_sync(FULL, pull);
        if (pm) {
          const int leader = __ffs(pm) - 1;
          unsigned long long base = 0;
          if (lane == leader)
            base = atomicAdd(A.counter, (unsigned long long)__popc(pm) * (unsigned long long)chunk);
          base = __shfl_sync(FULL, base, leader);
          if (pull) {
            const unsigned long long first = base + (unsigned long long)__popc(pm & ((1u << lane) - 1u)) * chunk;
            const long long rem = A.n_items - (long long)first;
            inext = (uint32_t)first;
            left = rem <= 0 ? 0 : (rem < chunk ? (int)rem : chunk);
          }
        }
        if (need) {
          if (left == 0) {
            done = true;
          } else {
            const uint32_t item = inext++;
            left--;
            uint32_t pl = item / (uint32_t)A.n_cells;
            const uint32_t ci = item - pl * (uint32_t)A.n_cells;
            if (A.order) pl = A.order[pl];
            s.plocal = (int)pl;
            s.ci = (int)ci;
            const int j = A.cell_cond[ci], a = A.cell_age[ci];
            fold_round1(s, A.cell_id[ci], (uint32_t)(A.p_offset + pl), A.rk);
            const PRecF& F = A.recf[pl];
            const PRec& R = A.rec[pl];
            koff = F.koff;
            beta = F.beta;
            s.kon = F.kon[0];
            s.gam = F.gam[0];
            s.k = 0;
            s.cyc = 0;
            s.lab = 0;
            T t0;
            if (GRID) {
              t0 = (T)cfg.t0_q;
              s.step_edge = (T)(cfg.n_steps == 1 ? cfg.t0_q + cfg.cycle_q : cfg.t0_q + cfg.step_q);
              s.tobs = (T)cfg.ages_q[a];
              const T texp = (s.tobs - (T)cfg.pulse_q[j]) - (T)cfg.chase_q[j];
              s.lab_edge = texp;
              s.tlab_end = texp + (T)cfg.pulse_q[j];
            } else {
              t0 = (T)cfg.t0;
              s.step_edge = (T)(cfg.n_steps == 1 ? cfg.t0 + cfg.cycle : cfg.t0 + cfg.step_len);
              s.tobs = (T)cfg.ages[a];
              const T texp = (s.tobs - (T)cfg.pulse[j]) - (T)cfg.chase[j];
              s.lab_edge = texp;
              s.tlab_end = texp + (T)cfg.pulse[j];
            }
            s.cs = t0;
            // initial state, drawn beforehand by init_state_kernel: (u, G)
            const int2 st0 = A.counts[(int64_t)pl * A.n_cells + ci];
            s.block = 1;
            s.G = st0.y ? 1.0f : 0.0f;
            s.uu = (float)st0.x;
            s.us = SPLICE ? floorf((float)R.s0 + 0.5f) : 0.0f;
            s.lu = 0.0f;
            s.ls = 0.0f;
            s.ev = 0;
            s.rej = 0;
            s.evf = 0.0f;
            s.rejf = 0.0f;
            set_interval<GRID, GENSCAL>(s, t0, cfg, F, invT);
            if (!(s.uu < kCountLimitF) || !(s.us < kCountLimitF)) err |= STF_OVERFLOW;
            active = true;
          }
        }
        if (__all_sync(FULL, done)) break;
      }
    }

    // ---- one trip: one Philox block, two iterations (the second sees a
    // negative interval, i.e. does nothing, once the first reached a breakpoint)
    const U4 w = main_block(s.block, s.r1x, s.r1y, s.r1z, A.rk);
    bp = ev_step<SPLICE, GENSCAL, GRID>(s, koff, beta, invT, s.len, w.x, w.y);
    bp = ev_step<SPLICE, GENSCAL, GRID>(s, koff, beta, invT, bp ? -1.0f : s.len, w.z, w.w) || bp;
    s.block++;
    special = active && (bp || s.evf >= kFlushF);
  }
  for (int o = 16; o > 0; o >>= 1) err |= __shfl_xor_sync(FULL, err, o);
  if (lane == 0 && err) atomicOr(A.status, err);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&A.totals[0], sh_tot[0]);
    atomicAdd(&A.totals[1], sh_tot[1]);
  }
}

}  // namespace abc
