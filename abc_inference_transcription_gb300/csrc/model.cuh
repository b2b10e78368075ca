// model.cuh — per-particle model records and the statistics aggregation.
//
// Reference (paths inside pthomaslab/abc_inference_transcription):
//   theta layout  hcat(kon, koff, alpha, gamma, lambda)  scripts/abc_simulation.jl:10
//   varying rate  get_vary_map / get_rate               scripts/model.jl:1-43
//   statistics    abc_sim                               scripts/abc_simulation.jl:23-46
//                 weighted_cov                          scripts/data_summary_statistics.jl:179-181
#pragma once
#include <cmath>
#include "common.cuh"

namespace abc {

constexpr int kMaxSteps = 8;
constexpr int kMaxAges = 8;
constexpr int kMaxConds = 16;

// Time grid and options, passed by value to every kernel.
struct DevCfg {
  double cycle, step_len, t0;
  double ages[kMaxAges];
  double pulse[kMaxConds];
  double chase[kMaxConds];
  int64_t event_cap;
  int n_steps, n_ages, n_conds, splicing, scaling_column, pulse_stat, chase_stat, npar;
  // Breakpoint grid (dcfg_set_grid): when every time above is an integer
  // multiple of quantum = 2^-e, the same times in quanta, so that the
  // production SSA places breakpoints with exact integer arithmetic.
  int grid_ok;
  float quantum;
  int32_t t0_q, cycle_q, step_q;
  int32_t ages_q[kMaxAges], pulse_q[kMaxConds], chase_q[kMaxConds];
};

// Host: find the coarsest quantum 2^-e (e = 0..20) of which t0, the cycle, the
// age step, every age, pulse and chase are exact integer multiples, with every
// breakpoint time (at most a few cycles) below 2^30 quanta; grid_ok = 0 if none.
inline void dcfg_set_grid(DevCfg& d) {
  d.grid_ok = 0;
  double horizon = std::fabs(d.t0) + 2.0 * d.cycle;
  for (int a = 0; a < d.n_ages; ++a) horizon = std::fmax(horizon, std::fabs(d.ages[a]) + std::fabs(d.t0));
  for (int e = 0; e <= 20; ++e) {
    const double sc = std::ldexp(1.0, e);
    auto ok = [&](double t) {
      const double x = t * sc;
      return x == std::floor(x) && std::fabs(x) < 1073741824.0;
    };
    bool all = ok(d.t0) && ok(d.cycle) && ok(d.step_len) && horizon * sc < 1073741824.0;
    for (int a = 0; a < d.n_ages && all; ++a) all = ok(d.ages[a]);
    for (int j = 0; j < d.n_conds && all; ++j) all = ok(d.pulse[j]) && ok(d.chase[j]);
    if (!all) continue;
    d.grid_ok = 1;
    d.quantum = (float)std::ldexp(1.0, -e);
    d.t0_q = (int32_t)(d.t0 * sc);
    d.cycle_q = (int32_t)(d.cycle * sc);
    d.step_q = (int32_t)(d.step_len * sc);
    for (int a = 0; a < kMaxAges; ++a) d.ages_q[a] = a < d.n_ages ? (int32_t)(d.ages[a] * sc) : 0;
    for (int j = 0; j < kMaxConds; ++j) {
      d.pulse_q[j] = j < d.n_conds ? (int32_t)(d.pulse[j] * sc) : 0;
      d.chase_q[j] = j < d.n_conds ? (int32_t)(d.chase[j] * sc) : 0;
    }
    return;
  }
}

// FP64 particle record (rates are 10^theta).
struct PRec {
  double kon[kMaxSteps], alp[kMaxSteps], gam[kMaxSteps], amax[kMaxSteps];
  double koff, lam, beta, scal;
  double g0, u0, s0;  // means at the start of a cycle (SSA initial state)
  double c0, v0;      // Cov(G, u) and Var u there (no splicing)
  double cost;        // expected fired events per trajectory (work estimate)
};

// FP32 copy of the rates for the production SSA, in log2 units: every rate
// (kon, alp, gam, amax, koff, beta) times log2 e; lam (a probability) and
// scal (an exponent) as they are.
struct PRecF {
  float kon[kMaxSteps], alp[kMaxSteps], gam[kMaxSteps], amax[kMaxSteps];
  float koff, lam, beta, scal;
};

// ---------------------------------------------------------------------------
// Initial state: periodic solution of the mean equations of (G, first mRNA
// species, spliced species) over one cycle with division, solved as the fixed
// point of the affine cycle map.  Exact exponential sub-steps with the
// substep-averaged source (16 per age step).
// ---------------------------------------------------------------------------
constexpr int kIcSub = 16;

ABC_HD void phi_pair(double z, double& e, double& ph) {
  e = xexp(-z);
  ph = (z > 1e-6) ? (1.0 - e) / z : 1.0 - 0.5 * z;
}

ABC_HD void mean_cycle(const DevCfg& cfg, const PRec& R, double& G, double& uu, double& us) {
  const int S = cfg.n_steps;
  const double T = cfg.cycle;
  const double h = (T / (double)S) / (double)kIcSub;
  for (int k = 0; k < S; ++k) {
    double kG = R.kon[k] + R.koff;
    double Ginf = R.kon[k] / kG;
    double eG, phG, eu, phu, es = 0.0, phs = 0.0;
    phi_pair(kG * h, eG, phG);
    double ku = cfg.splicing ? R.beta : R.gam[k];
    phi_pair(ku * h, eu, phu);
    if (cfg.splicing) phi_pair(R.gam[k] * h, es, phs);
    for (int i = 0; i < kIcSub; ++i) {
      double ph = ((double)(k * kIcSub + i) + 0.5) * h;
      double a = R.alp[k] * xpow(1.0 + ph / T, R.scal);
      double Gavg = Ginf + (G - Ginf) * phG;
      double Gn = Ginf + (G - Ginf) * eG;
      double uun = uu * eu + ((a * Gavg) * h) * phu;
      double usn = 0.0;
      if (cfg.splicing) usn = us * es + ((R.beta * (0.5 * (uu + uun))) * h) * phs;
      G = Gn;
      uu = uun;
      us = usn;
    }
  }
  uu = uu * 0.5;
  us = us * 0.5;
}

ABC_HD void initial_means(const DevCfg& cfg, PRec& R) {
  double b0 = 0.0, b1 = 0.0, b2 = 0.0;
  double c10 = 1.0, c11 = 0.0, c12 = 0.0;
  double c20 = 0.0, c21 = 1.0, c22 = 0.0;
  double c30 = 0.0, c31 = 0.0, c32 = 1.0;
  mean_cycle(cfg, R, b0, b1, b2);
  mean_cycle(cfg, R, c10, c11, c12);
  mean_cycle(cfg, R, c20, c21, c22);
  mean_cycle(cfg, R, c30, c31, c32);
  double mGG = c10 - b0;
  double muG = c11 - b1, muu = c21 - b1;
  double msG = c12 - b2, msu = c22 - b2, mss = c32 - b2;
  double g = b0 / (1.0 - mGG);
  double u = (b1 + muG * g) / (1.0 - muu);
  double s = cfg.splicing ? ((b2 + msG * g) + msu * u) / (1.0 - mss) : 0.0;
  if (!(g > 0.0)) g = 0.0;
  if (g > 1.0) g = 1.0;
  if (!(u > 0.0)) u = 0.0;
  if (!(s > 0.0)) s = 0.0;
  R.g0 = g;
  R.u0 = u;
  R.s0 = s;
}

// ---------------------------------------------------------------------------
// Initial state without splicing: the periodic solution, at the start of a
// cycle (after division), of the unlabelled moments x = (E G, E u, Cov(G,u),
// Var u) of the reaction network (model.jl:67-86 with lambda = 0) under the
// division map (model.jl:98-111: Cov/2, Var/4 + E/4, E/2), i.e. the state
// transient_phase converges to (model.jl:114-142).
//   E G' = kon - (kon + koff) E G
//   E u' = alpha(t) E G - gamma E u
//   C'   = alpha(t) E G (1 - E G) - (kon + koff + gamma) C
//   V'   = alpha(t) E G + gamma E u + 2 alpha(t) C - 2 gamma V
// Exponential sub-steps (16 per age step) with the sources averaged over the
// sub-step.  E G is periodic by itself; with it fixed, the cycle map of
// (E u, C, V) is affine with a lower-triangular matrix, solved directly.
// ---------------------------------------------------------------------------
ABC_HD void moment_cycle(const DevCfg& cfg, const PRec& R, double* x) {
  const int S = cfg.n_steps;
  const double T = cfg.cycle;
  const double h = (T / (double)S) / (double)kIcSub;
  double g = x[0], m = x[1], c = x[2], v = x[3];
  for (int k = 0; k < S; ++k) {
    const double kG = R.kon[k] + R.koff;
    const double Ginf = R.kon[k] / kG;
    const double gam = R.gam[k];
    double eG, phG, em, phm, ec, phc, ev, phv;
    phi_pair(kG * h, eG, phG);
    phi_pair(gam * h, em, phm);
    phi_pair((kG + gam) * h, ec, phc);
    phi_pair((2.0 * gam) * h, ev, phv);
    for (int i = 0; i < kIcSub; ++i) {
      const double ph = ((double)(k * kIcSub + i) + 0.5) * h;
      const double a = R.alp[k] * xpow(1.0 + ph / T, R.scal);
      const double Gavg = Ginf + (g - Ginf) * phG;
      const double gn = Ginf + (g - Ginf) * eG;
      const double mn = m * em + ((a * Gavg) * h) * phm;
      const double cn = c * ec + ((a * (Gavg * (1.0 - Gavg))) * h) * phc;
      const double src = (a * Gavg + gam * (0.5 * (m + mn))) + (2.0 * a) * (0.5 * (c + cn));
      const double vn = v * ev + (src * h) * phv;
      g = gn;
      m = mn;
      c = cn;
      v = vn;
    }
  }
  x[0] = g;
  x[1] = m * 0.5;
  x[2] = c * 0.5;
  x[3] = v * 0.25 + m * 0.25;
}

ABC_HD void initial_moments(const DevCfg& cfg, PRec& R) {
  double z[4] = {0.0, 0.0, 0.0, 0.0}, e[4] = {1.0, 0.0, 0.0, 0.0};
  moment_cycle(cfg, R, z);
  moment_cycle(cfg, R, e);
  double g = z[0] / (1.0 - (e[0] - z[0]));
  if (!(g > 0.0)) g = 0.0;
  if (g > 1.0) g = 1.0;
  double b[4] = {g, 0.0, 0.0, 0.0}, bm[4] = {g, 1.0, 0.0, 0.0};
  double bc[4] = {g, 0.0, 1.0, 0.0}, bv[4] = {g, 0.0, 0.0, 1.0};
  moment_cycle(cfg, R, b);
  moment_cycle(cfg, R, bm);
  moment_cycle(cfg, R, bc);
  moment_cycle(cfg, R, bv);
  const double mmm = bm[1] - b[1], mcc = bc[2] - b[2];
  const double mvm = bm[3] - b[3], mvc = bc[3] - b[3], mvv = bv[3] - b[3];
  double m = b[1] / (1.0 - mmm);
  double c = b[2] / (1.0 - mcc);
  double v = ((b[3] + mvm * m) + mvc * c) / (1.0 - mvv);
  if (!(m > 0.0)) m = 0.0;
  if (!(v > 0.0)) v = 0.0;
  if (!(c == c)) c = 0.0;
  R.g0 = g;
  R.u0 = m;
  R.s0 = 0.0;
  R.c0 = c;
  R.v0 = v;
}

// Unspliced count at the start of a trajectory, given the gene state G drawn
// with probability g0: conditional mean E[u | G] = u0 + c0 / g0 (G = 1) or
// u0 - c0 / (1 - g0) (G = 0), and within-state variance F E[u | G] with the
// Fano factor F = (v0 - c0^2 / (g0 (1 - g0))) / u0, so that E u, Var u and
// Cov(G, u) are those of the periodic solution.  Drawn as a zero-inflated
// Poisson (0 with probability 1 - w, else Poisson(mu / w), w = mu / (mu + F - 1))
// when F > 1, a Poisson(mu) otherwise.  wz: a 32-bit uniform word for the
// zero inflation; aux: the trajectory's auxiliary stream.
ABC_HD int64_t initial_count(const PRec& R, int G, uint32_t wz, Rng& aux) {
  const double g = R.g0, m = R.u0, c = R.c0, v = R.v0;
  double mu = m, vr = v;
  if (g > 0.0 && g < 1.0) {
    mu = G ? m + c / g : m - c / (1.0 - g);
    vr = v - (c * c) / (g * (1.0 - g));
  }
  if (!(mu > 0.0)) return 0;
  const double F = (m > 0.0 && vr > 0.0) ? vr / m : 0.0;
  double lam = mu;
  if (F > 1.0) {
    const double w = mu / (mu + (F - 1.0));
    if (!((double)wz * ABC_TWO_M32 < w)) return 0;
    lam = mu / w;
  }
  return poisson(aux, lam);
}

// theta -> record; returns 0 or a negative abc_status.
// with_ic: also the SSA initial state and work estimate (not needed by the moment ODE)
ABC_HD int parse_theta(const DevCfg& cfg, int model, const double* th, PRec& R, bool with_ic = true) {
  const int S = cfg.n_steps;
  int i = 0;
  double lk[kMaxSteps], la[kMaxSteps], lg[kMaxSteps];
  if (model == 3) {
    for (int k = 0; k < S; ++k) lk[k] = th[i++];
  } else {
    double v = th[i++];
    for (int k = 0; k < S; ++k) lk[k] = v;
  }
  double lkoff = th[i++];
  if (model == 4) {
    for (int k = 0; k < S; ++k) la[k] = th[i++];
  } else {
    double v = th[i++];
    for (int k = 0; k < S; ++k) la[k] = v;
  }
  if (model == 5) {
    for (int k = 0; k < S; ++k) lg[k] = th[i++];
  } else {
    double v = th[i++];
    for (int k = 0; k < S; ++k) lg[k] = v;
  }
  double llam = th[i++];
  R.beta = cfg.splicing ? xexp10(th[i++]) : 0.0;
  R.scal = cfg.scaling_column ? th[i++] : (model == 2 ? 0.0 : 1.0);
  R.koff = xexp10(lkoff);
  R.lam = xexp10(llam);
  for (int k = 0; k < S; ++k) {
    R.kon[k] = xexp10(lk[k]);
    R.alp[k] = xexp10(la[k]);
    R.gam[k] = xexp10(lg[k]);
    R.amax[k] = R.alp[k] * xpow(1.0 + (double)(k + 1) / (double)S, R.scal);
  }
  for (int k = S; k < kMaxSteps; ++k) R.kon[k] = R.alp[k] = R.gam[k] = R.amax[k] = 0.0;
  for (int k = 0; k < S; ++k)
    if (!(R.kon[k] < INFINITY) || !(R.alp[k] < INFINITY) || !(R.gam[k] < INFINITY)) return -5;
  if (!(R.koff < INFINITY) || R.lam != R.lam || R.scal != R.scal || R.scal < 0.0) return -5;
  if (!with_ic) return 0;
  R.c0 = R.v0 = 0.0;
  if (cfg.splicing)
    initial_means(cfg, R);
  else
    initial_moments(cfg, R);
  // work estimate: switching + transcription + decay events over the horizon
  double horizon = (double)(cfg.ages[0] - cfg.t0);
  double rate = 0.0;
  for (int k = 0; k < S; ++k) {
    double pon = R.kon[k] / (R.kon[k] + R.koff);
    rate = rate + (2.0 * pon * R.koff + 2.0 * pon * R.amax[k]);
  }
  R.cost = horizon * rate / (double)S + 1.0;
  return 0;
}

// ---------------------------------------------------------------------------
// Statistics from per-(condition, age) moments m[(j*A+a)*5 + {mu_u, mu_l,
// var_u, cov_ul, var_l}], in the reference layout
// [pulse_mean A | pulse_ff A | chase_mean A | chase_ff A | ratio J |
//  mean_corr J | corr_mean J].  Sums run left to right.
// ---------------------------------------------------------------------------
ABC_HD double wsum(const double* w, const double* x, int A) {
  double s = w[0] * x[0];
  for (int a = 1; a < A; ++a) s = s + w[a] * x[a];
  return s;
}
ABC_HD double wcov(const double* x, const double* y, const double* w, int A) {
  double mx = wsum(w, x, A), my = wsum(w, y, A);
  double s = w[0] * ((x[0] - mx) * (y[0] - my));
  for (int a = 1; a < A; ++a) s = s + w[a] * ((x[a] - mx) * (y[a] - my));
  return s;
}

// the statistics of condition j (its ratio, mean_corr and corr_mean, and the
// pulse or chase means and Fano factors when j is that condition); conditions
// write disjoint entries, so they may run in any order or in parallel
ABC_HD void stats_from_moments_cond(const DevCfg& cfg, const double* m, const double* age_dist, double* st, int j) {
  const int A = cfg.n_ages, J = cfg.n_conds;
  double w[kMaxAges], mu[kMaxAges], ml[kMaxAges], vu[kMaxAges], cv[kMaxAges], vl[kMaxAges];
  {
    for (int a = 0; a < A; ++a) {
      const double* g = m + (j * A + a) * 5;
      w[a] = age_dist[a * J + j];
      mu[a] = g[0];
      ml[a] = g[1];
      vu[a] = g[2];
      cv[a] = g[3];
      vl[a] = g[4];
    }
    double swu = wsum(w, mu, A), swl = wsum(w, ml, A);
    st[4 * A + j] = swl / (swu + swl);
    double tvu = wsum(w, vu, A) + wcov(mu, mu, w, A);
    double tvl = wsum(w, vl, A) + wcov(ml, ml, w, A);
    double stds = sqrt(fabs(tvu * tvl));
    st[4 * A + J + j] = wsum(w, cv, A) / stds;
    st[4 * A + 2 * J + j] = wcov(mu, ml, w, A) / stds;
    int off = (j == cfg.pulse_stat) ? 0 : (j == cfg.chase_stat) ? 2 * A : -1;
    if (off >= 0) {
      for (int a = 0; a < A; ++a) {
        double tot = mu[a] + ml[a];
        double eps = (tot == 0.0) ? 0.0001 : 0.0;
        st[off + a] = tot;
        st[off + A + a] = ((vu[a] + 2.0 * cv[a]) + vl[a]) / (tot + eps);
      }
    }
  }
}

ABC_HD void stats_from_moments(const DevCfg& cfg, const double* m, const double* age_dist, double* st) {
  for (int j = 0; j < cfg.n_conds; ++j) stats_from_moments_cond(cfg, m, age_dist, st, j);
}

// int128 -> double with the oracle's rounding (exact below 2^62).
ABC_HD double i128_to_double(__int128 x) {
  const __int128 lim = ((__int128)1) << 62;
  if (x >= -lim && x <= lim) return (double)(int64_t)x;
  bool neg = x < 0;
  unsigned __int128 ux = neg ? (unsigned __int128)(-x) : (unsigned __int128)x;
  double hi = (double)(uint64_t)(ux >> 64);
  double lo = (double)(uint64_t)ux;
  double v = hi * 18446744073709551616.0 + lo;
  return neg ? -v : v;
}

}  // namespace abc
