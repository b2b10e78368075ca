/*
 * abc_oracle.c — FP64 CPU oracle (TEST INFRASTRUCTURE ONLY; see abc_oracle.h).
 *
 * Compile with -ffp-contract=off: the SSA part must reproduce the GPU FP64
 * mode bit for bit, so no multiply-add may be fused.  Every expression below
 * is written in the same operation order as the CUDA kernels.
 *
 * Reference files cited (paths inside pthomaslab/abc_inference_transcription):
 *   scripts/model.jl, scripts/abc_simulation.jl, scripts/compute_errors.jl,
 *   scripts/accepted_particles.jl, scripts/data_summary_statistics.jl,
 *   scripts/recover_statistics.jl.
 */
#include "abc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as    */
/* easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies, key       */
/* bumped by the Weyl constants between rounds.                               */
/* ------------------------------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Random stream of one trajectory: counter = (block lo, block hi | stream<<30,
 * cell, particle), key = seed.  Words are consumed in pairs; one Philox block
 * gives two pairs. */
enum { ST_SSA = 0, ST_CAPTURE = 1, ST_PRIOR = 2, ST_AUX = 3 };
typedef struct {
  uint32_t k0, k1, cell, particle, tag;
  uint64_t block;
  uint32_t buf[4];
  int half;
} orc_rng;

static void rng_init(orc_rng* r, uint64_t seed, uint32_t stream, uint32_t cell, uint32_t particle) {
  r->k0 = (uint32_t)seed;
  r->k1 = (uint32_t)(seed >> 32);
  r->cell = cell;
  r->particle = particle;
  r->tag = stream << 30;
  r->block = 0;
  r->half = 0;
}

static void rng_pair(orc_rng* r, uint32_t* a, uint32_t* b) {
  if (r->half == 0) {
    uint32_t c[4] = {(uint32_t)r->block, ((uint32_t)(r->block >> 32) & 0x3fffffffu) | r->tag,
                     r->cell, r->particle};
    uint32_t k[2] = {r->k0, r->k1};
    orc_philox4x32_10(c, k, r->buf);
    r->block++;
    *a = r->buf[0];
    *b = r->buf[1];
    r->half = 1;
  } else {
    *a = r->buf[2];
    *b = r->buf[3];
    r->half = 0;
  }
}

#define TWO_M32 2.3283064365386963e-10 /* 2^-32 */
#define TWO_M52 2.220446049250313e-16  /* 2^-52 */

/* uniform in (0,1) from 52 bits of a pair */
static double u52open(uint32_t a, uint32_t b) {
  uint64_t x = ((uint64_t)a << 20) | (uint64_t)(b >> 12);
  return ((double)x + 0.5) * TWO_M52;
}
/* uniform in [0,1) from 52 bits of a pair */
static double u52(uint32_t a, uint32_t b) {
  uint64_t x = ((uint64_t)a << 20) | (uint64_t)(b >> 12);
  return (double)x * TWO_M52;
}

/* ------------------------------------------------------------------------- */
/* Deterministic log / exp written from their series (no libm): identical     */
/* bits on CPU and GPU when evaluated in the same order without contraction.  */
/* log: x = m 2^e, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s), s=(m-1)/(m+1), */
/* atanh series to s^25.  exp: x = k ln2 + r, |r| <= ln2/2, Taylor to r^14.   */
/* ln2 is split into a 32-bit head (exact k*LN2_HI) and its remainder.        */
/* ------------------------------------------------------------------------- */
static const double LN2_HI = 0.6931471803691238;
static const double LN2_LO = 1.9082149292705877e-10;
static const double INV_LN2 = 1.4426950408889634;
static const double LN10 = 2.302585092994046;
static const double SQRT2 = 1.4142135623730951;

double orc_xlog(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  uint64_t mb = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
  double m;
  memcpy(&m, &mb, 8);
  if (m > SQRT2) {
    m = m * 0.5;
    e = e + 1;
  }
  double s = (m - 1.0) / (m + 1.0);
  double z = s * s;
  double p = 0.04;
  p = p * z + 0.043478260869565216;
  p = p * z + 0.047619047619047616;
  p = p * z + 0.05263157894736842;
  p = p * z + 0.058823529411764705;
  p = p * z + 0.06666666666666667;
  p = p * z + 0.07692307692307693;
  p = p * z + 0.09090909090909091;
  p = p * z + 0.1111111111111111;
  p = p * z + 0.14285714285714285;
  p = p * z + 0.2;
  p = p * z + 0.3333333333333333;
  p = p * z + 1.0;
  double de = (double)e;
  return de * LN2_HI + (de * LN2_LO + (2.0 * s) * p);
}

double orc_xexp(double x) {
  if (x != x) return x;
  if (x > 709.0) return INFINITY;
  if (x < -745.0) return 0.0;
  double kd = floor(x * INV_LN2 + 0.5);
  double r = (x - kd * LN2_HI) - kd * LN2_LO;
  double p = 1.1470745597729725e-11;
  p = p * r + 1.6059043836821613e-10;
  p = p * r + 2.08767569878681e-09;
  p = p * r + 2.505210838544172e-08;
  p = p * r + 2.755731922398589e-07;
  p = p * r + 2.7557319223985893e-06;
  p = p * r + 2.48015873015873e-05;
  p = p * r + 0.0001984126984126984;
  p = p * r + 0.001388888888888889;
  p = p * r + 0.008333333333333333;
  p = p * r + 0.041666666666666664;
  p = p * r + 0.16666666666666666;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  int k = (int)kd;
  if (k >= -1021) {
    uint64_t eb = (uint64_t)(k + 1023) << 52;
    double sc;
    memcpy(&sc, &eb, 8);
    return p * sc;
  }
  uint64_t eb = (uint64_t)(k + 1023 + 60) << 52;
  double sc;
  memcpy(&sc, &eb, 8);
  return (p * sc) * 8.673617379884035e-19; /* 2^-60 */
}

static double xexp10(double x) { return orc_xexp(x * LN10); }
static double xpow(double x, double s) {
  if (s == 0.0) return 1.0;
  if (s == 1.0) return x;
  return orc_xexp(s * orc_xlog(x));
}

/* ------------------------------------------------------------------------- */
/* Binomial samplers                                                           */
/*   Bin(n, 1/2): popcount of n random bits (division, model.jl:98-111).        */
/*   Bin(n, p), n*min(p,1-p) < 10: inversion (Kachitvichyanukul & Schmeiser).  */
/*   otherwise: BTRD (Hormann 1993, "The generation of binomial random         */
/*   variates", J. Stat. Comput. Simul. 46:101-110).                           */
/* ------------------------------------------------------------------------- */
static int64_t binom_half(orc_rng* r, int64_t n) {
  int64_t k = 0;
  while (n > 0) {
    uint32_t a, b;
    rng_pair(r, &a, &b);
    uint64_t bits = ((uint64_t)b << 32) | (uint64_t)a;
    if (n < 64) bits &= (((uint64_t)1) << n) - 1;
    k += (int64_t)__builtin_popcountll(bits);
    n -= 64;
  }
  return k;
}

static int64_t binv(orc_rng* rr, int64_t n, double p) {
  double q = 1.0 - p;
  double s = p / q;
  double a = (double)(n + 1) * s;
  double r0 = orc_xexp((double)n * orc_xlog(q));
  for (;;) {
    uint32_t w0, w1;
    rng_pair(rr, &w0, &w1);
    double u = u52open(w0, w1);
    double f = r0;
    int64_t x = 0;
    for (;;) {
      if (u < f) return x;
      if (x >= n || x >= 110) break;
      u = u - f;
      x = x + 1;
      f = f * (a / (double)x - s);
    }
  }
}

/* Stirling series correction log(k!) - [(k+1/2)log(k+1) - (k+1) + log(2 pi)/2],
 * tabulated for k < 10 (values computed to 50 digits, rounded to double). */
static const double FC_TAB[10] = {0.08106146679532726, 0.0413406959554093, 0.02767792568499834,
                                  0.020790672103765093, 0.016644691189821193, 0.013876128823070748,
                                  0.01189670994589177, 0.010411265261972096, 0.009255462182712733,
                                  0.00833056343336287};
static double fc(double k) {
  if (k < 10.0) return FC_TAB[(int)k];
  double kp = k + 1.0;
  double r2 = 1.0 / (kp * kp);
  return (0.08333333333333333 - (0.002777777777777778 - 0.0007936507936507937 * r2) * r2) / kp;
}

static int64_t btrd(orc_rng* rr, int64_t n, double p) {
  double nd = (double)n;
  double m = floor((nd + 1.0) * p);
  double r = p / (1.0 - p);
  double nr = (nd + 1.0) * r;
  double npq = (nd * p) * (1.0 - p);
  double sq = sqrt(npq);
  double b = 1.15 + 2.53 * sq;
  double a = (-0.0873 + 0.0248 * b) + 0.01 * p;
  double c = nd * p + 0.5;
  double alpha = (2.83 + 5.1 / b) * sq;
  double vr = 0.92 - 4.2 / b;
  double urvr = 0.86 * vr;
  double nm = (nd - m) + 1.0;
  double h = ((m + 0.5) * orc_xlog((m + 1.0) / (r * nm)) + fc(m)) + fc(nd - m);
  for (;;) {
    uint32_t w0, w1;
    rng_pair(rr, &w0, &w1);
    double v = u52open(w0, w1);
    double u;
    if (v <= urvr) {
      u = v / vr - 0.43;
      return (int64_t)floor(((2.0 * a) / (0.5 - fabs(u)) + b) * u + c);
    }
    if (v >= vr) {
      rng_pair(rr, &w0, &w1);
      u = u52open(w0, w1) - 0.5;
    } else {
      u = v / vr - 0.93;
      u = (u < 0.0 ? -0.5 : 0.5) - u;
      rng_pair(rr, &w0, &w1);
      v = u52open(w0, w1) * vr;
    }
    double us = 0.5 - fabs(u);
    double kd = floor(((2.0 * a) / us + b) * u + c);
    if (kd < 0.0 || kd > nd) continue;
    v = (v * alpha) / (a / (us * us) + b);
    double km = fabs(kd - m);
    if (km <= 15.0) {
      double f = 1.0;
      if (m < kd) {
        for (double i = m + 1.0; i <= kd; i += 1.0) f = f * (nr / i - r);
      } else if (m > kd) {
        for (double i = kd + 1.0; i <= m; i += 1.0) v = v * (nr / i - r);
      }
      if (v <= f) return (int64_t)kd;
      continue;
    }
    v = orc_xlog(v);
    double rho = (km / npq) * (((km / 3.0 + 0.625) * km + 0.16666666666666666) / npq + 0.5);
    double t = (-km * km) / (2.0 * npq);
    if (v < t - rho) return (int64_t)kd;
    if (v > t + rho) continue;
    double nk = (nd - kd) + 1.0;
    double bound = (((h + (nd + 1.0) * orc_xlog(nm / nk)) + (kd + 0.5) * orc_xlog((nk * r) / (kd + 1.0))) -
                    fc(kd)) - fc(nd - kd);
    if (v <= bound) return (int64_t)kd;
  }
}

static int64_t binomial(orc_rng* r, int64_t n, double p) {
  if (n <= 0 || !(p > 0.0)) return 0;
  if (p >= 1.0) return n;
  int flip = p > 0.5;
  double pp = flip ? 1.0 - p : p;
  int64_t k = ((double)n * pp < 10.0) ? binv(r, n, pp) : btrd(r, n, pp);
  return flip ? n - k : k;
}

/* log(k!) from the Stirling series with the tabulated correction. */
static double logfact(double k) {
  return (((k + 0.5) * orc_xlog(k + 1.0) - (k + 1.0)) + 0.9189385332046728) + fc(k);
}

/* Poisson(lam): inversion below lam = 10, otherwise PTRS (W. Hormann, "The
 * transformed rejection method for generating Poisson random variables",
 * Insurance: Mathematics and Economics 12 (1993) 39-45).  Same operation
 * order as the GPU sampler. */
static int64_t poisson(orc_rng* r, double lam) {
  if (!(lam > 0.0)) return 0;
  uint32_t w0, w1;
  if (lam < 10.0) {
    rng_pair(r, &w0, &w1);
    double u = u52(w0, w1);
    double f = orc_xexp(-lam);
    int64_t k = 0;
    while (u >= f && k < 1000) {
      u = u - f;
      k = k + 1;
      f = f * (lam / (double)k);
    }
    return k;
  }
  const double slam = sqrt(lam);
  const double loglam = orc_xlog(lam);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < 1000; ++it) {
    rng_pair(r, &w0, &w1);
    const double U = u52(w0, w1) - 0.5;
    rng_pair(r, &w0, &w1);
    const double V = u52open(w0, w1);
    const double us = 0.5 - fabs(U);
    const double kd = floor((((2.0 * a) / us + b) * U + lam) + 0.43);
    if (us >= 0.07 && V <= vr) return (int64_t)kd;
    if (kd < 0.0 || (us < 0.013 && V > us)) continue;
    const double lhs = orc_xlog((V * inv_alpha) / (a / (us * us) + b));
    const double rhs = (kd * loglam - lam) - logfact(kd);
    if (lhs <= rhs) return (int64_t)kd;
  }
  return (int64_t)floor(lam + 0.5);
}

int64_t orc_poisson(double lam, uint64_t seed, uint32_t stream, uint32_t cell, uint32_t particle,
                    int64_t n_draws, int64_t* out) {
  orc_rng r;
  rng_init(&r, seed, stream, cell, particle);
  for (int64_t i = 0; i < n_draws; ++i) out[i] = poisson(&r, lam);
  return (int64_t)r.block;
}

int64_t orc_binomial(int64_t n, double p, uint64_t seed, uint32_t stream, uint32_t cell,
                     uint32_t particle, int64_t n_draws, int64_t* out) {
  orc_rng r;
  rng_init(&r, seed, stream, cell, particle);
  for (int64_t i = 0; i < n_draws; ++i) out[i] = (p == 0.5) ? binom_half(&r, n) : binomial(&r, n, p);
  return (int64_t)r.block;
}

/* ------------------------------------------------------------------------- */
/* Model parameters: theta layout hcat(kon, koff, alpha, gamma, lambda)        */
/* (abc_simulation.jl:10) with the varying rate expanded to n_steps columns    */
/* (get_vary_map, model.jl:30-43), then optional [beta_splice], [scaling].     */
/* ------------------------------------------------------------------------- */
int orc_num_params(const abc_config* cfg, int model) {
  if (model < 1 || model > 5) return ABC_ERR_INVALID;
  return 5 + (model >= 3 ? cfg->n_steps - 1 : 0) + (cfg->splicing ? 1 : 0) + (cfg->scaling_column ? 1 : 0);
}

typedef struct {
  int S;
  double kon[ABC_MAX_STEPS], alp[ABC_MAX_STEPS], gam[ABC_MAX_STEPS], amax[ABC_MAX_STEPS];
  double koff, lam, beta, scal, g0, u0, s0;
  double c0, v0; /* Cov(G, u) and Var u at the start of a cycle (no splicing) */
} rec_t;

/* One cycle of the mean equations (G, first mRNA species, spliced species)
 * followed by division; exact exponential sub-steps with the substep-averaged
 * source.  Used only to pick the SSA initial state. */
#define IC_SUB 16
static void phi_pair(double z, double* e, double* ph) {
  *e = orc_xexp(-z);
  *ph = (z > 1e-6) ? (1.0 - *e) / z : 1.0 - 0.5 * z;
}

static void mean_cycle(const abc_config* cfg, const rec_t* R, double x[3]) {
  const int S = R->S;
  const double T = cfg->cycle;
  const double h = (T / (double)S) / (double)IC_SUB;
  double G = x[0], uu = x[1], us = x[2];
  for (int k = 0; k < S; ++k) {
    double kG = R->kon[k] + R->koff;
    double Ginf = R->kon[k] / kG;
    double eG, phG, eu, phu, es = 0.0, phs = 0.0;
    phi_pair(kG * h, &eG, &phG);
    double ku = cfg->splicing ? R->beta : R->gam[k];
    phi_pair(ku * h, &eu, &phu);
    if (cfg->splicing) phi_pair(R->gam[k] * h, &es, &phs);
    for (int i = 0; i < IC_SUB; ++i) {
      double ph = ((double)(k * IC_SUB + i) + 0.5) * h;
      double a = R->alp[k] * xpow(1.0 + ph / T, R->scal);
      double Gavg = Ginf + (G - Ginf) * phG;
      double Gn = Ginf + (G - Ginf) * eG;
      double uun = uu * eu + ((a * Gavg) * h) * phu;
      double usn = 0.0;
      if (cfg->splicing) usn = us * es + ((R->beta * (0.5 * (uu + uun))) * h) * phs;
      G = Gn;
      uu = uun;
      us = usn;
    }
  }
  x[0] = G;
  x[1] = uu * 0.5;
  x[2] = us * 0.5;
}

static void initial_means(const abc_config* cfg, rec_t* R) {
  double b[3] = {0.0, 0.0, 0.0};
  double c1[3] = {1.0, 0.0, 0.0};
  double c2[3] = {0.0, 1.0, 0.0};
  double c3[3] = {0.0, 0.0, 1.0};
  mean_cycle(cfg, R, b);
  mean_cycle(cfg, R, c1);
  mean_cycle(cfg, R, c2);
  mean_cycle(cfg, R, c3);
  double mGG = c1[0] - b[0];
  double muG = c1[1] - b[1], muu = c2[1] - b[1];
  double msG = c1[2] - b[2], msu = c2[2] - b[2], mss = c3[2] - b[2];
  double g = b[0] / (1.0 - mGG);
  double u = (b[1] + muG * g) / (1.0 - muu);
  double s = cfg->splicing ? ((b[2] + msG * g) + msu * u) / (1.0 - mss) : 0.0;
  if (!(g > 0.0)) g = 0.0;
  if (g > 1.0) g = 1.0;
  if (!(u > 0.0)) u = 0.0;
  if (!(s > 0.0)) s = 0.0;
  R->g0 = g;
  R->u0 = u;
  R->s0 = s;
}

/* Periodic solution at the start of a cycle (after division) of the
 * unlabelled moments x = (E G, E u, Cov(G,u), Var u) of model.jl:67-86 with
 * lambda = 0, under the division map of model.jl:98-111 -- the state that
 * transient_phase (model.jl:114-142) converges to.  Exponential sub-steps
 * with sub-step-averaged sources; E G is periodic by itself, then the cycle
 * map of (E u, C, V) is affine with a lower-triangular matrix. */
static void moment_cycle(const abc_config* cfg, const rec_t* R, double x[4]) {
  const int S = R->S;
  const double T = cfg->cycle;
  const double h = (T / (double)S) / (double)IC_SUB;
  double g = x[0], m = x[1], c = x[2], v = x[3];
  for (int k = 0; k < S; ++k) {
    const double kG = R->kon[k] + R->koff;
    const double Ginf = R->kon[k] / kG;
    const double gam = R->gam[k];
    double eG, phG, em, phm, ec, phc, ev, phv;
    phi_pair(kG * h, &eG, &phG);
    phi_pair(gam * h, &em, &phm);
    phi_pair((kG + gam) * h, &ec, &phc);
    phi_pair((2.0 * gam) * h, &ev, &phv);
    for (int i = 0; i < IC_SUB; ++i) {
      const double ph = ((double)(k * IC_SUB + i) + 0.5) * h;
      const double a = R->alp[k] * xpow(1.0 + ph / T, R->scal);
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

static void initial_moments(const abc_config* cfg, rec_t* R) {
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
  R->g0 = g;
  R->u0 = m;
  R->s0 = 0.0;
  R->c0 = c;
  R->v0 = v;
}

/* Initial unspliced count given the gene state G: conditional mean
 * E[u | G] and within-state variance F E[u | G] of the periodic moments,
 * drawn as a zero-inflated Poisson when F > 1 (0 with probability 1 - w, else
 * Poisson(mu / w), w = mu / (mu + F - 1)), as a Poisson(mu) otherwise. */
static int64_t initial_count(const rec_t* R, int G, uint32_t wz, orc_rng* aux) {
  const double g = R->g0, m = R->u0, c = R->c0, v = R->v0;
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
    if (!((double)wz * TWO_M32 < w)) return 0;
    lam = mu / w;
  }
  return poisson(aux, lam);
}

static int parse_theta(const abc_config* cfg, int model, const double* th, rec_t* R) {
  const int S = cfg->n_steps;
  int i = 0;
  double lk[ABC_MAX_STEPS], la[ABC_MAX_STEPS], lg[ABC_MAX_STEPS];
  R->S = S;
  if (model == 3) for (int k = 0; k < S; ++k) lk[k] = th[i++];
  else { double v = th[i++]; for (int k = 0; k < S; ++k) lk[k] = v; }
  double lkoff = th[i++];
  if (model == 4) for (int k = 0; k < S; ++k) la[k] = th[i++];
  else { double v = th[i++]; for (int k = 0; k < S; ++k) la[k] = v; }
  if (model == 5) for (int k = 0; k < S; ++k) lg[k] = th[i++];
  else { double v = th[i++]; for (int k = 0; k < S; ++k) lg[k] = v; }
  double llam = th[i++];
  R->beta = cfg->splicing ? xexp10(th[i++]) : 0.0;
  R->scal = cfg->scaling_column ? th[i++] : (model == 2 ? 0.0 : 1.0);
  R->koff = xexp10(lkoff);
  R->lam = xexp10(llam);
  for (int k = 0; k < S; ++k) {
    R->kon[k] = xexp10(lk[k]);
    R->alp[k] = xexp10(la[k]);
    R->gam[k] = xexp10(lg[k]);
    R->amax[k] = R->alp[k] * xpow(1.0 + (double)(k + 1) / (double)S, R->scal);
  }
  for (int k = 0; k < S; ++k)
    if (!(R->kon[k] < INFINITY) || !(R->alp[k] < INFINITY) || !(R->gam[k] < INFINITY)) return ABC_ERR_NONFINITE;
  if (!(R->koff < INFINITY) || R->lam != R->lam || R->scal != R->scal || R->scal < 0.0) return ABC_ERR_NONFINITE;
  R->c0 = R->v0 = 0.0;
  if (cfg->splicing)
    initial_means(cfg, R);
  else
    initial_moments(cfg, R);
  return ABC_OK;
}

/* The SSA's initial state of n trajectories (cells 0..n-1 of one particle):
 * the gene state and the first mRNA count, as sim_traj draws them. */
int orc_initial_states(const abc_config* cfg, int model, const double* theta, uint64_t seed, uint32_t particle,
                       int64_t n, int32_t* G_out, int64_t* u_out) {
  rec_t R;
  int st = parse_theta(cfg, model, theta, &R);
  if (st) return st;
  for (int64_t c = 0; c < n; ++c) {
    orc_rng rng, aux;
    rng_init(&rng, seed, ST_SSA, (uint32_t)c, particle);
    rng_init(&aux, seed, ST_AUX, (uint32_t)c, particle);
    uint32_t w0, w1;
    rng_pair(&rng, &w0, &w1);
    const int G = ((double)w0 * TWO_M32 < R.g0) ? 1 : 0;
    G_out[c] = G;
    u_out[c] = cfg->splicing ? (int64_t)floor(R.u0 + 0.5) : initial_count(&R, G, w1, &aux);
  }
  return ABC_OK;
}

int orc_setup(const abc_config* cfg, int model, const double* theta, double* rec_out) {
  rec_t R;
  int st = parse_theta(cfg, model, theta, &R);
  if (st) return st;
  int S = R.S, i = 0;
  for (int k = 0; k < S; ++k) rec_out[i++] = R.kon[k];
  for (int k = 0; k < S; ++k) rec_out[i++] = R.alp[k];
  for (int k = 0; k < S; ++k) rec_out[i++] = R.gam[k];
  for (int k = 0; k < S; ++k) rec_out[i++] = R.amax[k];
  rec_out[i++] = R.koff; rec_out[i++] = R.lam; rec_out[i++] = R.beta; rec_out[i++] = R.scal;
  rec_out[i++] = R.g0; rec_out[i++] = R.u0; rec_out[i++] = R.s0;
  rec_out[i++] = R.c0; rec_out[i++] = R.v0;
  return ABC_OK;
}

/* ------------------------------------------------------------------------- */
/* Prior draw (fix_params, abc_simulation.jl:3-11), Philox stream 2, cell 0.   */
/* ------------------------------------------------------------------------- */
int orc_sample_prior(const abc_config* cfg, int model, int64_t P, uint64_t seed,
                     int64_t particle_offset, const abc_prior* pr, double* theta_out) {
  int npar = orc_num_params(cfg, model);
  if (npar < 0) return npar;
  const int S = cfg->n_steps;
  double lf0 = orc_xlog(pr->factor[0]) / LN10, lf1 = orc_xlog(pr->factor[1]) / LN10;
  double ls0 = cfg->scaling_column ? orc_xlog(pr->scaling[0]) / LN10 : 0.0;
  double ls1 = cfg->scaling_column ? orc_xlog(pr->scaling[1]) / LN10 : 0.0;
  for (int64_t p = 0; p < P; ++p) {
    orc_rng r;
    rng_init(&r, seed, ST_PRIOR, 0u, (uint32_t)(particle_offset + p));
    double* th = theta_out + p * npar;
    int i = 0;
    const double* rng_of[4] = {pr->kon, pr->koff, pr->alpha, pr->gamma};
    for (int rate = 0; rate < 4; ++rate) {
      const double* lohi = rng_of[rate];
      int varies = (model == 3 && rate == 0) || (model == 4 && rate == 2) || (model == 5 && rate == 3);
      uint32_t a, b;
      rng_pair(&r, &a, &b);
      double base = lohi[0] + (lohi[1] - lohi[0]) * u52(a, b);
      if (!varies) {
        th[i++] = base;
      } else if (pr->vary_mode == 0) {
        th[i++] = base;
        for (int k = 1; k < S; ++k) {
          rng_pair(&r, &a, &b);
          th[i++] = lohi[0] + (lohi[1] - lohi[0]) * u52(a, b);
        }
      } else {
        for (int k = 0; k < S; ++k) {
          rng_pair(&r, &a, &b);
          th[i++] = base + (lf0 + (lf1 - lf0) * u52(a, b));
        }
      }
    }
    uint32_t a, b;
    rng_pair(&r, &a, &b);
    th[i++] = pr->lambda[0] + (pr->lambda[1] - pr->lambda[0]) * u52(a, b);
    if (cfg->splicing) {
      rng_pair(&r, &a, &b);
      th[i++] = pr->beta[0] + (pr->beta[1] - pr->beta[0]) * u52(a, b);
    }
    if (cfg->scaling_column) {
      rng_pair(&r, &a, &b);
      th[i++] = xexp10(ls0 + (ls1 - ls0) * u52(a, b));
    }
  }
  return ABC_OK;
}

/* ------------------------------------------------------------------------- */
/* FP64 SSA of the reaction network equivalent to the moment equations         */
/* f(y,p,lambda) (model.jl:74-86):                                             */
/*   G 0->1 @ kon(t); G 1->0 @ koff; G=1: transcription @ alpha(t), labelled  */
/*   with probability lambda(t) (model.jl:58-64); u->u-1 @ gamma(t) u;        */
/*   l->l-1 @ gamma(t) l.  alpha(t) = alpha_k size(t)^s (model.jl:1-27) by     */
/*   thinning against alpha_k (1+(k+1)/S)^s.  Division at t = 0 mod T:          */
/*   u, l -> Bin(., 1/2) (model.jl:98-111).  Start t0 = -n_burn T               */
/*   (abc_simulation.jl:73), observed at the cell age (model.jl:146-174).      */
/* ------------------------------------------------------------------------- */
#define FNV_OFF 0xcbf29ce484222325ull
#define FNV_PRIME 0x100000001b3ull
enum { CH_ON = 0, CH_OFF = 1, CH_TXU = 2, CH_TXL = 3, CH_DEGU = 4, CH_DEGL = 5, CH_REJ = 6,
       CH_NULL = 7, CH_SPLU = 8, CH_SPLL = 9, CH_DIV = 10 };

typedef struct {
  int64_t ev, rej;
  uint64_t hash;
  int64_t u, l;
  int err;
} traj_out;

static void sim_traj(const abc_config* cfg, const rec_t* R, int j, int a, orc_rng* rng, orc_rng* aux,
                     traj_out* o) {
  const double T = cfg->cycle;
  const int S = cfg->n_steps;
  const double step_len = T / (double)S;
  const double t0 = -(double)cfg->n_burn_cycles * T;
  const double t_obs = cfg->ages[a];
  const double texp = (t_obs - cfg->pulse[j]) - cfg->chase[j];
  const double tlab_end = texp + cfg->pulse[j];
  const int64_t cap = cfg->event_cap > 0 ? cfg->event_cap : ((int64_t)1 << 28);
  const int sp = cfg->splicing;
  int stall = 0;
  double cycle_start = t0, t = t0;
  int k = 0;
  double step_edge = (S == 1) ? cycle_start + T : cycle_start + step_len;
  int lab_state = 0;
  double lab_edge = texp, lam_cur = 0.0;
  uint32_t w0, w1;
  rng_pair(rng, &w0, &w1);
  int G = ((double)w0 * TWO_M32 < R->g0) ? 1 : 0;
  /* splicing option: the means; reference model: the moment-matched draw */
  int64_t uu = sp ? (int64_t)floor(R->u0 + 0.5) : initial_count(R, G, w1, aux);
  int64_t us = sp ? (int64_t)floor(R->s0 + 0.5) : 0;
  int64_t lu = 0, ls = 0;
  uint64_t h = FNV_OFF;
  int64_t ev = 0, rej = 0;
  o->err = 0;
  for (;;) {
    double t_end = step_edge;
    if (lab_state < 2 && lab_edge < t_end) t_end = lab_edge;
    if (t_obs < t_end) t_end = t_obs;
    for (;;) {
      const double gam = R->gam[k];
      double a_on = G ? 0.0 : R->kon[k];
      double a_off = G ? R->koff : 0.0;
      double a_tx = G ? R->amax[k] : 0.0;
      double c1 = a_on;
      double c2 = c1 + a_off;
      double c3 = c2 + a_tx;
      double c4, c5, c6, a_last, a0;
      if (!sp) {
        double a_du = gam * (double)uu;
        a_last = gam * (double)lu;
        c4 = c3 + a_du;
        c5 = c4;
        c6 = c4;
        a0 = c4 + a_last;
      } else {
        double a_su = R->beta * (double)uu;
        double a_sl = R->beta * (double)lu;
        double a_du = gam * (double)us;
        a_last = gam * (double)ls;
        c4 = c3 + a_su;
        c5 = c4 + a_sl;
        c6 = c5 + a_du;
        a0 = c6 + a_last;
      }
      rng_pair(rng, &w0, &w1);
      if (!(a0 > 0.0)) break;
      double U1 = ((double)w0 + 0.5) * TWO_M32;
      double tau = -orc_xlog(U1) / a0;
      double tn = t + tau;
      if (tn >= t_end) break;
      stall = (tn == t) ? stall + 1 : 0;
      t = tn;
      double r = ((double)w1 * TWO_M32) * a0;
      uint32_t ch;
      if (r < c1) {
        G = 1;
        ch = CH_ON;
      } else if (r < c2) {
        G = 0;
        ch = CH_OFF;
      } else if (r < c3) {
        double v = r - c2;
        double at = R->alp[k] * xpow(1.0 + (t - cycle_start) / T, R->scal);
        if (v < at) {
          if (v < at * lam_cur) { lu++; ch = CH_TXL; }
          else { uu++; ch = CH_TXU; }
        } else {
          ch = CH_REJ;
        }
      } else if (!sp) {
        if (r < c4) { uu--; ch = CH_DEGU; }
        else if (a_last > 0.0) { lu--; ch = CH_DEGL; }
        else ch = CH_NULL;
      } else {
        if (r < c4) { uu--; us++; ch = CH_SPLU; }
        else if (r < c5) { lu--; ls++; ch = CH_SPLL; }
        else if (r < c6) { us--; ch = CH_DEGU; }
        else if (a_last > 0.0) { ls--; ch = CH_DEGL; }
        else ch = CH_NULL;
      }
      h = (h ^ (uint64_t)ch) * FNV_PRIME;
      if (ch == CH_REJ) {
        rej++;
      } else if (ch != CH_NULL) {
        ev++;
        if (ev > cap) { o->err = ABC_ERR_EVENT_CAP; goto done; }
      }
      if (stall > 1024) { o->err = ABC_ERR_NONFINITE; goto done; }
    }
    t = t_end;
    if (t == t_obs) break;
    while (lab_state < 2 && t == lab_edge) {
      lab_state++;
      if (lab_state == 1) { lam_cur = R->lam; lab_edge = tlab_end; }
      else lam_cur = 0.0;
    }
    if (t == step_edge) {
      k++;
      if (k == S) {
        k = 0;
        cycle_start = cycle_start + T;
        uu = binom_half(rng, uu);
        if (sp) us = binom_half(rng, us);
        lu = binom_half(rng, lu);
        if (sp) ls = binom_half(rng, ls);
        h = (h ^ (uint64_t)CH_DIV) * FNV_PRIME;
      }
      step_edge = (k == S - 1) ? cycle_start + T : cycle_start + (double)(k + 1) * step_len;
    }
  }
done:
  o->ev = ev;
  o->rej = rej;
  o->hash = h;
  o->u = uu + us;
  o->l = lu + ls;
}

/* ------------------------------------------------------------------------- */
/* Statistics (abc_simulation.jl:23-46 with weighted_cov,                      */
/* data_summary_statistics.jl:179-181).  Sums run left to right as Julia's     */
/* sum does for short vectors.                                                 */
/* ------------------------------------------------------------------------- */
static double wsum(const double* w, const double* x, int A) {
  double s = w[0] * x[0];
  for (int a = 1; a < A; ++a) s = s + w[a] * x[a];
  return s;
}
static double wcov(const double* x, const double* y, const double* w, int A) {
  double mx = wsum(w, x, A), my = wsum(w, y, A);
  double s = w[0] * ((x[0] - mx) * (y[0] - my));
  for (int a = 1; a < A; ++a) s = s + w[a] * ((x[a] - mx) * (y[a] - my));
  return s;
}

int orc_stats_from_moments(const abc_config* cfg, const double* m, const double* age_dist,
                           double* st) {
  const int A = cfg->n_ages, J = cfg->n_conds;
  double w[ABC_MAX_AGES], mu[ABC_MAX_AGES], ml[ABC_MAX_AGES], vu[ABC_MAX_AGES], cv[ABC_MAX_AGES],
      vl[ABC_MAX_AGES];
  for (int j = 0; j < J; ++j) {
    for (int a = 0; a < A; ++a) {
      const double* g = m + (j * A + a) * 5;
      w[a] = age_dist[a * J + j];
      mu[a] = g[0]; ml[a] = g[1]; vu[a] = g[2]; cv[a] = g[3]; vl[a] = g[4];
    }
    double swu = wsum(w, mu, A), swl = wsum(w, ml, A);
    st[4 * A + j] = swl / (swu + swl);
    double tvu = wsum(w, vu, A) + wcov(mu, mu, w, A);
    double tvl = wsum(w, vl, A) + wcov(ml, ml, w, A);
    double stds = sqrt(fabs(tvu * tvl));
    st[4 * A + J + j] = wsum(w, cv, A) / stds;
    st[4 * A + 2 * J + j] = wcov(mu, ml, w, A) / stds;
    int off = (j == cfg->pulse_stat_cond) ? 0 : (j == cfg->chase_stat_cond) ? 2 * A : -1;
    if (off >= 0) {
      for (int a = 0; a < A; ++a) {
        double tot = mu[a] + ml[a];
        double eps = (tot == 0.0) ? 0.0001 : 0.0;
        st[off + a] = tot;
        st[off + A + a] = ((vu[a] + 2.0 * cv[a]) + vl[a]) / (tot + eps);
      }
    }
  }
  return ABC_OK;
}

/* int128 -> double, the same two-step rounding as the GPU kernel */
static double i128_to_double(__int128 x) {
  if (x >= -(((__int128)1) << 62) && x <= (((__int128)1) << 62)) return (double)(int64_t)x;
  int neg = x < 0;
  unsigned __int128 ux = neg ? (unsigned __int128)(-x) : (unsigned __int128)x;
  double hi = (double)(uint64_t)(ux >> 64);
  double lo = (double)(uint64_t)ux;
  double v = hi * 18446744073709551616.0 + lo;
  return neg ? -v : v;
}

typedef struct {
  int64_t n, su, sl;
  __int128 suu, sll, sul;
} gsum_t;

static void group_moments(const gsum_t* g, double* out5) {
  double n = (double)g->n;
  double dn = n * (double)(g->n - 1);
  out5[0] = (double)g->su / n;
  out5[1] = (double)g->sl / n;
  __int128 nvu = (__int128)g->n * g->suu - (__int128)g->su * g->su;
  __int128 ncv = (__int128)g->n * g->sul - (__int128)g->su * g->sl;
  __int128 nvl = (__int128)g->n * g->sll - (__int128)g->sl * g->sl;
  out5[2] = i128_to_double(nvu) / dn;
  out5[3] = i128_to_double(ncv) / dn;
  out5[4] = i128_to_double(nvl) / dn;
}

int orc_simulate(const abc_config* cfg, int64_t C, const int32_t* cell_cond,
                 const int32_t* cell_age, const double* cell_beta, const double* age_dist,
                 int model, const double* theta, int64_t P, uint64_t seed,
                 int64_t particle_offset, int n_threads, int32_t* counts, int32_t* captured,
                 int64_t* events, uint64_t* hash, int64_t* rejections, double* stats) {
  int npar = orc_num_params(cfg, model);
  if (npar < 0) return npar;
  const int A = cfg->n_ages, J = cfg->n_conds, K = ABC_NSTATS(A, J);
  rec_t* R = (rec_t*)malloc(sizeof(rec_t) * (size_t)(P > 0 ? P : 1));
  int32_t* cap = (int32_t*)malloc(sizeof(int32_t) * 2 * (size_t)(P * C > 0 ? P * C : 1));
  int status = ABC_OK;
  int64_t rej_total = 0;
  for (int64_t p = 0; p < P; ++p) {
    int st = parse_theta(cfg, model, theta + p * npar, &R[p]);
    if (st) status = st;
  }
  if (status) goto out;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : rej_total)
#endif
  for (int64_t idx = 0; idx < P * C; ++idx) {
    int64_t p = idx / C, c = idx % C;
    orc_rng rng;
    traj_out o;
    rng_init(&rng, seed, ST_SSA, (uint32_t)c, (uint32_t)(particle_offset + p));
    orc_rng aux; /* initial state: auxiliary stream, blocks 0, 1, ... */
    rng_init(&aux, seed, ST_AUX, (uint32_t)c, (uint32_t)(particle_offset + p));
    sim_traj(cfg, &R[p], cell_cond[c], cell_age[c], &rng, &aux, &o);
    if (o.err) status = o.err;
    if (o.u > 2147483647 || o.l > 2147483647) status = ABC_ERR_NONFINITE;
    orc_rng rc;
    rng_init(&rc, seed, ST_CAPTURE, (uint32_t)c, (uint32_t)(particle_offset + p));
    int64_t cu = binomial(&rc, o.u, cell_beta[c]);
    int64_t cl = binomial(&rc, o.l, cell_beta[c]);
    cap[2 * idx] = (int32_t)cu;
    cap[2 * idx + 1] = (int32_t)cl;
    if (counts) { counts[2 * idx] = (int32_t)o.u; counts[2 * idx + 1] = (int32_t)o.l; }
    if (events) events[idx] = o.ev;
    if (hash) hash[idx] = o.hash;
    rej_total += o.rej;
  }
  if (rejections) *rejections = rej_total;
  if (status) goto out;
  if (captured) memcpy(captured, cap, sizeof(int32_t) * 2 * (size_t)(P * C));
  if (stats) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t p = 0; p < P; ++p) {
      gsum_t g[ABC_MAX_AGES * ABC_MAX_CONDS];
      double mom[ABC_MAX_AGES * ABC_MAX_CONDS * 5];
      memset(g, 0, sizeof(g));
      for (int64_t c = 0; c < C; ++c) {
        gsum_t* q = &g[cell_cond[c] * A + cell_age[c]];
        int64_t u = cap[2 * (p * C + c)], l = cap[2 * (p * C + c) + 1];
        q->n++;
        q->su += u;
        q->sl += l;
        q->suu += (__int128)(u * u);
        q->sll += (__int128)(l * l);
        q->sul += (__int128)(u * l);
      }
      for (int gi = 0; gi < A * J; ++gi) group_moments(&g[gi], mom + gi * 5);
      orc_stats_from_moments(cfg, mom, age_dist, stats + p * K);
    }
  }
out:
  free(R);
  free(cap);
  return status;
}

/* ------------------------------------------------------------------------- */
/* Moment ODE (the reference's own algorithm, model.jl:67-239,                 */
/* abc_simulation.jl:13-62).  Linear system y' = A(t) y + b(t) integrated by   */
/* the exponential midpoint rule on a grid aligned with every breakpoint      */
/* (age steps, labelling edges, ages, divisions); substep propagators are      */
/* cached per cycle position.                                                  */
/* ------------------------------------------------------------------------- */
#define NAUG 10
static void mat_mul(const double* X, const double* Y, double* Z) {
  double tmp[NAUG * NAUG];
  for (int i = 0; i < NAUG; ++i)
    for (int j = 0; j < NAUG; ++j) {
      double s = 0.0;
      for (int k = 0; k < NAUG; ++k) s += X[i * NAUG + k] * Y[k * NAUG + j];
      tmp[i * NAUG + j] = s;
    }
  memcpy(Z, tmp, sizeof(tmp));
}

static void expm(const double* A, double* E) {
  double norm = 0.0;
  for (int j = 0; j < NAUG; ++j) {
    double s = 0.0;
    for (int i = 0; i < NAUG; ++i) s += fabs(A[i * NAUG + j]);
    if (s > norm) norm = s;
  }
  int sq = 0;
  while (norm > 0.5) { norm *= 0.5; sq++; }
  double B[NAUG * NAUG], T[NAUG * NAUG];
  double scale = ldexp(1.0, -sq);
  for (int i = 0; i < NAUG * NAUG; ++i) B[i] = A[i] * scale;
  /* Horner: E = I + B(I + B/2 (I + B/3 (...))) */
  for (int i = 0; i < NAUG * NAUG; ++i) E[i] = (i % (NAUG + 1) == 0) ? 1.0 : 0.0;
  for (int n = 18; n >= 1; --n) {
    mat_mul(B, E, T);
    for (int i = 0; i < NAUG * NAUG; ++i) E[i] = T[i] / (double)n + ((i % (NAUG + 1) == 0) ? 1.0 : 0.0);
  }
  for (int s = 0; s < sq; ++s) mat_mul(E, E, E);
}

static void build_A(double* A, double kon, double koff, double al, double gam, double lam, double h) {
  memset(A, 0, sizeof(double) * NAUG * NAUG);
#define M_(i, j) A[(i) * NAUG + (j)]
  double ks = kon + koff;
  M_(0, 0) = -ks; M_(0, 9) = kon;
  M_(1, 0) = (1.0 - lam) * al; M_(1, 1) = -gam;
  M_(2, 0) = lam * al; M_(2, 2) = -gam;
  M_(3, 0) = koff - kon; M_(3, 3) = -2.0 * ks; M_(3, 9) = kon;
  M_(4, 3) = al * (1.0 - lam); M_(4, 4) = -(ks + gam);
  M_(5, 3) = al * lam; M_(5, 5) = -(ks + gam);
  M_(6, 0) = al * (1.0 - lam); M_(6, 1) = gam; M_(6, 4) = 2.0 * al * (1.0 - lam); M_(6, 6) = -2.0 * gam;
  M_(7, 4) = al * lam; M_(7, 5) = al * (1.0 - lam); M_(7, 7) = -2.0 * gam;
  M_(8, 0) = al * lam; M_(8, 2) = gam; M_(8, 5) = 2.0 * al * lam; M_(8, 8) = -2.0 * gam;
#undef M_
  for (int i = 0; i < NAUG * NAUG; ++i) A[i] *= h;
}

typedef struct {
  const abc_config* cfg;
  const rec_t* R;
  double h;
  int nsub;         /* substeps per cycle */
  int per_step;     /* substeps per age step */
  double* prop[2];  /* [lam][nsub][100] */
  unsigned char* have[2];
} mctx_t;

static const double* propagator(mctx_t* M, int idx, int lab) {
  double* P = M->prop[lab] + (size_t)idx * NAUG * NAUG;
  if (!M->have[lab][idx]) {
    const rec_t* R = M->R;
    int k = idx / M->per_step;
    double ph = ((double)idx + 0.5) * M->h;
    double al = R->alp[k] * xpow(1.0 + ph / M->cfg->cycle, R->scal);
    double A[NAUG * NAUG];
    build_A(A, R->kon[k], R->koff, al, R->gam[k], lab ? R->lam : 0.0, M->h);
    expm(A, P);
    M->have[lab][idx] = 1;
  }
  return P;
}

static void apply(const double* P, double* y) {
  double z[NAUG];
  for (int i = 0; i < NAUG; ++i) {
    double s = 0.0;
    for (int j = 0; j < NAUG; ++j) s += P[i * NAUG + j] * y[j];
    z[i] = s;
  }
  memcpy(y, z, sizeof(z));
}

/* integrate y over [ta, tb] (tb - ta <= one cycle, no division inside) */
static void integrate(mctx_t* M, double* y, double ta, double tb, double texp, double tlab_end) {
  const double T = M->cfg->cycle;
  long n = lround((tb - ta) / M->h);
  for (long i = 0; i < n; ++i) {
    double tm = ta + ((double)i + 0.5) * M->h;
    double md = tm - T * floor(tm / T);
    int idx = (int)floor(md / M->h);
    if (idx >= M->nsub) idx = M->nsub - 1;
    int lab = (tm >= texp && tm <= tlab_end) ? 1 : 0;
    apply(propagator(M, idx, lab), y);
  }
}

static void periodic_boundary(double* v) {
  /* model.jl:98-111 (0-based indices) */
  double e[NAUG];
  memcpy(e, v, sizeof(e));
  v[4] = e[4] / 2.0; v[5] = e[5] / 2.0;
  v[6] = e[6] / 4.0 + e[1] / 4.0; v[8] = e[8] / 4.0 + e[2] / 4.0;
  v[7] = e[7] / 4.0;
  v[1] = e[1] / 2.0; v[2] = e[2] / 2.0;
}

static int grid_ok(double x, double h) {
  double q = x / h;
  return fabs(q - nearbyint(q)) < 1e-7 * (1.0 + fabs(q));
}

int orc_moment_model(const abc_config* cfg, int model, const double* theta, const double* iv,
                     double h_max, double* moments_out, int* n_transient_iter,
                     const double* beta_mom, int n_pulse_conds, const double* age_dist,
                     int exact_capture, double* stats_out) {
  rec_t R;
  int st = parse_theta(cfg, model, theta, &R);
  if (st) return st;
  const double T = cfg->cycle;
  const int S = cfg->n_steps, A = cfg->n_ages, J = cfg->n_conds;
  const double t0 = -(double)cfg->n_burn_cycles * T;
  if (h_max <= 0.0) h_max = T / 400.0;
  int per_step = (int)ceil((T / (double)S) / h_max);
  double h = 0.0;
  for (; per_step < 200000; ++per_step) {
    h = T / (double)(S * per_step);
    int ok = grid_ok(t0, h);
    for (int a = 0; a < A && ok; ++a) ok = grid_ok(cfg->ages[a], h);
    for (int j = 0; j < J && ok; ++j) ok = grid_ok(cfg->pulse[j], h) && grid_ok(cfg->chase[j], h);
    if (ok) break;
  }
  if (per_step >= 200000) return ABC_ERR_INVALID;
  mctx_t M;
  M.cfg = cfg; M.R = &R; M.h = h; M.per_step = per_step; M.nsub = S * per_step;
  for (int l = 0; l < 2; ++l) {
    M.prop[l] = (double*)malloc(sizeof(double) * NAUG * NAUG * (size_t)M.nsub);
    M.have[l] = (unsigned char*)calloc((size_t)M.nsub, 1);
  }
  /* transient_phase, model.jl:114-142 */
  double e1[NAUG], e2[NAUG];
  for (int i = 0; i < 9; ++i) e1[i] = iv[i];
  e1[9] = 1.0;
  integrate(&M, e1, 0.0, T, -1.0, -0.9);
  memcpy(e2, e1, sizeof(e1));
  static const int chk[5] = {0, 1, 3, 4, 6};
  int k = 0, conv = 0;
  while (!conv && k <= 100) {
    k++;
    double y[NAUG];
    memcpy(y, e1, sizeof(y));
    periodic_boundary(y);
    integrate(&M, y, 0.0, T, -1.0, -0.9);
    memcpy(e2, y, sizeof(y));
    int nz = 0, okc = 0;
    for (int q = 0; q < 5; ++q) {
      int i = chk[q];
      if (e1[i] > 0.0) {
        nz++;
        if (fabs((e1[i] - e2[i]) / e1[i]) <= 0.01) okc++;
      }
    }
    if (okc == nz) conv = 1;
    memcpy(e1, e2, sizeof(e1));
  }
  if (n_transient_iter) *n_transient_iter = k;
  double ss[NAUG];
  memcpy(ss, e2, sizeof(ss));
  periodic_boundary(ss);
  /* trajectories / syntheticdata, model.jl:146-199 */
  for (int j = 0; j < J; ++j) {
    for (int a = 0; a < A; ++a) {
      double age = cfg->ages[a];
      double texp = (age - cfg->pulse[j]) - cfg->chase[j];
      double tle = texp + cfg->pulse[j];
      double y[NAUG];
      memcpy(y, ss, sizeof(y));
      double tau = t0;
      int first = 1;
      while (tau < age) {
        double tf = (tau < 0.0) ? tau + T : age;
        if (tf > age) tf = age;
        if (!first) periodic_boundary(y);
        integrate(&M, y, tau, tf, texp, tle);
        first = 0;
        tau = tf;
      }
      double* mo = moments_out + (j * A + a) * 5;
      mo[0] = y[1]; mo[1] = y[2]; mo[2] = y[6]; mo[3] = y[7]; mo[4] = y[8];
    }
  }
  for (int l = 0; l < 2; ++l) { free(M.prop[l]); free(M.have[l]); }
  if (stats_out && beta_mom && age_dist) {
    /* downsample, model.jl:221-239, per age cluster of the pulse or chase cells */
    double ds[ABC_MAX_AGES * ABC_MAX_CONDS * 5];
    for (int j = 0; j < J; ++j)
      for (int a = 0; a < A; ++a) {
        const double* bm = beta_mom + ((j < n_pulse_conds ? 0 : 1) * A + a) * 3;
        double mb = bm[0], m2 = bm[1], vb = bm[2];
        const double* s = moments_out + (j * A + a) * 5;
        double* d = ds + (j * A + a) * 5;
        d[0] = s[0] * mb;
        d[1] = s[1] * mb;
        if (!exact_capture) {
          d[2] = ((mb - m2) * s[0] + vb * (s[0] * s[0] + s[2])) + mb * mb * s[2];
          d[4] = ((mb - m2) * s[1] + vb * (s[1] * s[1] + s[4])) + mb * mb * s[4];
          d[3] = vb * (s[0] * s[1] + s[3]) + mb * mb * s[3];
        } else {
          d[2] = ((mb - m2) * s[0] + vb * (s[0] * s[0])) + m2 * s[2];
          d[4] = ((mb - m2) * s[1] + vb * (s[1] * s[1])) + m2 * s[4];
          d[3] = vb * (s[0] * s[1]) + m2 * s[3];
        }
      }
    orc_stats_from_moments(cfg, ds, age_dist, stats_out);
  }
  return ABC_OK;
}

int orc_moment_batch(const abc_config* cfg, int model, const double* theta, int64_t P,
                     const double* iv, double h_max, const double* beta_mom, int n_pulse_conds,
                     const double* age_dist, int n_threads, double* stats_out) {
  int npar = orc_num_params(cfg, model);
  if (npar < 0) return npar;
  const int A = cfg->n_ages, J = cfg->n_conds, K = ABC_NSTATS(A, J);
  int status = ABC_OK;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t p = 0; p < P; ++p) {
    double mom[ABC_MAX_AGES * ABC_MAX_CONDS * 5];
    int st = orc_moment_model(cfg, model, theta + p * npar, iv, h_max, mom, NULL, beta_mom,
                              n_pulse_conds, age_dist, 0, stats_out + p * K);
    if (st) status = st;
  }
  return status;
}

/* ------------------------------------------------------------------------- */
/* Errors (compute_errors.jl:30-70) and acceptance (accepted_particles.jl).    */
/* ------------------------------------------------------------------------- */
int orc_errors(const double* data, const double* se, int64_t G, int K, int n_fam,
               const int32_t* fam, const double* stats, int64_t P, int n_threads, double* err) {
  int one = K;
  if (n_fam <= 0 || !fam) { n_fam = 1; fam = &one; }
  const double sig2 = 0.1 * 0.1;
  const double nK = (double)K;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(static)
#endif
  for (int64_t p = 0; p < P; ++p) {
    const double* s = stats + p * K;
    for (int64_t g = 0; g < G; ++g) {
      const double* d = data + g * K;
      const double* e = se + g * K;
      double tot = 0.0;
      int k = 0;
      for (int f = 0; f < n_fam; ++f) {
        double part = 0.0;
        for (int q = 0; q < fam[f]; ++q, ++k) {
          double eps = (e[k] + d[k] != 0.0) ? 0.0 : 0.0001;
          double diff = d[k] - s[k];
          part = part + (diff * diff) / ((e[k] * e[k] + sig2 * (d[k] * d[k])) + eps);
        }
        tot = tot + part / nK;
      }
      if (tot > 10.0) tot = 10.0;
      err[p * G + g] = tot;
    }
  }
  return ABC_OK;
}

typedef struct { double e; int64_t i; } pair_t;
static int cmp_pair(const void* x, const void* y) {
  const pair_t* a = (const pair_t*)x;
  const pair_t* b = (const pair_t*)y;
  if (a->e < b->e) return -1;
  if (a->e > b->e) return 1;
  return (a->i < b->i) ? -1 : (a->i > b->i);
}

/* Per gene (accepted_particles.jl:20-29): the particles with err <= eps (mode
 * 0) or the ceil(q P) smallest finite errors (mode 1), sorted by (err, index),
 * 1-based.  The list lengths need no sort, so offsets are counted first; the
 * lists are then filled one gene per thread (idx == NULL: offsets only). */
int64_t orc_accept(const double* err, int64_t P, int64_t G, int mode, double eps_or_q,
                   int64_t* offsets, int64_t* idx, int64_t cap) {
  const int64_t kq = (int64_t)ceil(eps_or_q * (double)P);
  offsets[0] = 0;
  for (int64_t g = 0; g < G; ++g) {
    int64_t n = 0;
    for (int64_t p = 0; p < P; ++p) {
      const double e = err[p * G + g];
      if (e != e) continue;
      if (mode == 0 && !(e <= eps_or_q)) continue;
      n++;
    }
    if (mode == 1 && n > kq) n = kq;
    offsets[g + 1] = offsets[g] + n;
  }
  const int64_t total = offsets[G];
  if (!idx) return total;
#pragma omp parallel
  {
    pair_t* buf = (pair_t*)malloc(sizeof(pair_t) * (size_t)(P > 0 ? P : 1));
#pragma omp for schedule(dynamic, 1)
    for (int64_t g = 0; g < G; ++g) {
      int64_t n = 0;
      for (int64_t p = 0; p < P; ++p) {
        const double e = err[p * G + g];
        if (e != e) continue;
        if (mode == 0 && !(e <= eps_or_q)) continue;
        buf[n].e = e;
        buf[n].i = p;
        n++;
      }
      qsort(buf, (size_t)n, sizeof(pair_t), cmp_pair);
      const int64_t len = offsets[g + 1] - offsets[g];
      for (int64_t q = 0; q < len; ++q)
        if (offsets[g] + q < cap) idx[offsets[g] + q] = buf[q].i + 1;
    }
    free(buf);
  }
  return total;
}

/* ------------------------------------------------------------------------- */
/* Downstream of the acceptance: model probabilities with bootstrap bounds    */
/* (model_probs.jl:1-28, per-gene cases :41-48) and posterior summaries       */
/* (posterior_kinetics.jl:1-33).  Julia's default quantile (alpha = beta = 1).*/
/* ------------------------------------------------------------------------- */
static double quantile_sorted(const double* v, int64_t n, double p) {
  double m = 1.0 + p * ((1.0 - 1.0) - 1.0);
  double aleph = (double)n * p + m;
  int64_t j = (int64_t)aleph;
  if (j > n - 1) j = n - 1;
  if (j < 1 && n > 1) j = 1;
  double g = aleph - (double)j;
  g = g < 0.0 ? 0.0 : (g > 1.0 ? 1.0 : g);
  double a = n == 1 ? v[0] : v[j - 1], b = n == 1 ? v[0] : v[j];
  if (isfinite(a) && isfinite(b)) return a + g * (b - a);
  return (1.0 - g) * a + g * b;
}

static int cmp_dbl(const void* x, const void* y) {
  double a = *(const double*)x, b = *(const double*)y;
  return (a > b) - (a < b);
}

int orc_model_probs(const int64_t* counts, int64_t G, int M, int n_boot, double alpha, uint64_t seed,
                    double* prob, double* lb, double* ub) {
  double* bv = (double*)malloc(sizeof(double) * (size_t)M * n_boot);
  if (!bv) return ABC_ERR_NOMEM;
  for (int64_t g = 0; g < G; ++g) {
    const int64_t* l = counts + g * M;
    double *P = prob + g * M, *LB = lb + g * M, *UB = ub + g * M;
    int64_t L = 0;
    int nz = 0, which = -1;
    for (int m = 0; m < M; ++m) {
      L += l[m];
      if (l[m] > 0) { nz++; which = m; }
      P[m] = LB[m] = UB[m] = 0.0;
    }
    if (L == 0) continue;
    if (nz == 1) { P[which] = LB[which] = UB[which] = 1.0; continue; }
    for (int m = 0; m < M; ++m) P[m] = (double)l[m] / (double)L;
    for (int b = 0; b < n_boot; ++b) {
      orc_rng r;
      rng_init(&r, seed, 3u, (uint32_t)b, (uint32_t)g);
      int64_t nrem = L, lrem = L;
      for (int m = 0; m < M; ++m) {
        int64_t x;
        if (m == M - 1 || lrem == l[m]) x = nrem;
        else if (l[m] == 0 || nrem == 0) x = 0;
        else x = binomial(&r, nrem, (double)l[m] / (double)lrem);
        nrem -= x;
        lrem -= l[m];
        bv[(int64_t)m * n_boot + b] = (double)x / (double)L;
      }
    }
    for (int m = 0; m < M; ++m) {
      qsort(bv + (int64_t)m * n_boot, (size_t)n_boot, sizeof(double), cmp_dbl);
      LB[m] = quantile_sorted(bv + (int64_t)m * n_boot, n_boot, 1.0 - alpha);
      UB[m] = quantile_sorted(bv + (int64_t)m * n_boot, n_boot, alpha);
    }
  }
  free(bv);
  return ABC_OK;
}

int orc_posterior_summary(const double* theta, int64_t ld, int npar, const int64_t* off, const int64_t* idx,
                          int64_t G, double q, double* map, double* mean, double* lb, double* ub,
                          int64_t* n_out) {
  int64_t maxn = 1;
  for (int64_t g = 0; g < G; ++g)
    if (off[g + 1] - off[g] > maxn) maxn = off[g + 1] - off[g];
  double* v = (double*)malloc(sizeof(double) * (size_t)maxn);
  if (!v) return ABC_ERR_NOMEM;
  for (int64_t g = 0; g < G; ++g) {
    const int64_t o = off[g], n = off[g + 1] - off[g];
    if (n_out) n_out[g] = n;
    for (int c = 0; c < npar; ++c) {
      const int64_t t = g * npar + c;
      if (n == 0) { map[t] = mean[t] = lb[t] = ub[t] = NAN; continue; }
      map[t] = theta[(idx[o] - 1) * ld + c];
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i) {
        v[i] = theta[(idx[o + i] - 1) * ld + c];
        s = s + v[i];
      }
      mean[t] = s / (double)n;
      qsort(v, (size_t)n, sizeof(double), cmp_dbl);
      lb[t] = quantile_sorted(v, n, 1.0 - q);
      ub[t] = quantile_sorted(v, n, q);
    }
  }
  free(v);
  return ABC_OK;
}

/* ------------------------------------------------------------------------- */
/* Data-side statistics and bootstrap standard errors                         */
/* (data_summary_statistics.jl:1-216).  Cells in the stable (condition, age)  */
/* order; draw i of (seed, family, resample, gene) from its own Philox        */
/* counter; statistics from exact integer sums.                              */
/* ------------------------------------------------------------------------- */
static int64_t draw_pos(uint64_t seed, int fam, int b, int64_t g, int64_t i, int64_t n) {
  uint32_t c[4] = {(uint32_t)(i >> 1), ((uint32_t)((uint64_t)i >> 33) & 0x3fffffffu) | (3u << 30),
                   (uint32_t)b | ((uint32_t)(fam + 1) << 24), (uint32_t)g};
  uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)}, o[4];
  orc_philox4x32_10(c, k, o);
  /* floor(x n / 2^52) of a 52-bit uniform integer x, exact */
  uint32_t hi = (i & 1) ? o[2] : o[0], lo = (i & 1) ? o[3] : o[1];
  uint64_t x = ((uint64_t)hi << 20) | (uint64_t)(lo >> 12);
  return (int64_t)(((unsigned __int128)x * (unsigned __int128)(uint64_t)n) >> 52);
}

static double sample_cov(unsigned long long n, unsigned long long sx, unsigned long long sy, unsigned long long sxy) {
  __int128 num = (__int128)n * (__int128)sxy - (__int128)sx * (__int128)sy;
  return i128_to_double(num) / ((double)n * (double)(n - 1));
}

static void data_one(const abc_config* cfg, int64_t C, const int32_t* cond_s, const int32_t* age_s,
                     const int64_t* id_s, const int64_t* gs, const double* age_dist, const int32_t* u,
                     const int32_t* l, int64_t g, int b, uint64_t seed, double* st) {
  const int A = cfg->n_ages, J = cfg->n_conds;
  unsigned long long Sp[2][ABC_MAX_AGES][3];
  unsigned long long Sg[ABC_MAX_CONDS * ABC_MAX_AGES][6];
  memset(Sp, 0, sizeof(Sp));
  memset(Sg, 0, sizeof(Sg));
  for (int f = 0; f < 2; ++f) {
    int cond = f == 0 ? cfg->pulse_stat_cond : cfg->chase_stat_cond;
    int64_t base = gs[cond * A], n = gs[(cond + 1) * A] - base;
    for (int64_t i = 0; i < n; ++i) {
      int64_t cell = base + (b == 0 ? i : draw_pos(seed, f, b, g, i, n));
      int64_t id = id_s[cell];
      unsigned long long x = (unsigned long long)u[id] + (unsigned long long)l[id];
      int ag = age_s[cell];
      Sp[f][ag][0] += 1ull;
      Sp[f][ag][1] += x;
      Sp[f][ag][2] += x * x;
    }
  }
  for (int64_t i = 0; i < C; ++i) {
    int64_t cell = b == 0 ? i : draw_pos(seed, 2, b, g, i, C);
    int64_t id = id_s[cell];
    unsigned long long uu = (unsigned long long)u[id], ll = (unsigned long long)l[id];
    unsigned long long* S = Sg[cond_s[cell] * A + age_s[cell]];
    S[0] += 1ull; S[1] += uu; S[2] += ll; S[3] += uu * uu; S[4] += ll * ll; S[5] += uu * ll;
  }
  for (int f = 0; f < 2; ++f) {
    int off = f == 0 ? 0 : 2 * A;
    for (int ag = 0; ag < A; ++ag) {
      unsigned long long n = Sp[f][ag][0];
      double m = 0.0, ff = 0.0;
      if (n > 0) {
        m = (double)Sp[f][ag][1] / (double)n;
        double v = sample_cov(n, Sp[f][ag][1], Sp[f][ag][1], Sp[f][ag][2]);
        double eps = (m == 0.0) ? 0.0001 : 0.0;
        ff = v / (m + eps);
      }
      st[off + ag] = m;
      st[off + A + ag] = ff;
    }
  }
  for (int j = 0; j < J; ++j) {
    double m1[ABC_MAX_AGES] = {0}, m2[ABC_MAX_AGES] = {0}, v1[ABC_MAX_AGES] = {0}, v2[ABC_MAX_AGES] = {0};
    double c12[ABC_MAX_AGES] = {0}, w[ABC_MAX_AGES] = {0};
    unsigned long long nj = 0, suj = 0, slj = 0;
    for (int ag = 0; ag < A; ++ag) {
      unsigned long long* S = Sg[j * A + ag];
      nj += S[0]; suj += S[1]; slj += S[2];
      if (S[0] == 0) {
        m1[ag] = m2[ag] = v1[ag] = v2[ag] = c12[ag] = 0.0;
      } else {
        m1[ag] = (double)S[1] / (double)S[0];
        m2[ag] = (double)S[2] / (double)S[0];
        v1[ag] = sample_cov(S[0], S[1], S[1], S[3]);
        v2[ag] = sample_cov(S[0], S[2], S[2], S[4]);
        c12[ag] = sample_cov(S[0], S[1], S[2], S[5]);
      }
    }
    double mu = (double)suj / (double)nj, ml = (double)slj / (double)nj;
    st[4 * A + j] = (mu + ml > 0.0) ? ml / (mu + ml) : 0.0;
    for (int ag = 0; ag < A; ++ag) {
      if (b == 0) {
        w[ag] = age_dist[ag * J + j];
      } else {
        double x = (double)Sg[j * A + ag][0] / (double)nj;
        w[ag] = x == x ? x : 0.0;
      }
    }
    double tv1 = wsum(w, v1, A) + wcov(m1, m1, w, A);
    double tv2 = wsum(w, v2, A) + wcov(m2, m2, w, A);
    int any_cov = 0;
    for (int ag = 0; ag < A; ++ag) any_cov = any_cov || (c12[ag] != 0.0);
    int tv_ok = tv1 != 0.0 && tv2 != 0.0;
    st[4 * A + J + j] = (any_cov && tv_ok) ? wsum(w, c12, A) / sqrt(fabs(tv1 * tv2)) : 0.0;
    st[4 * A + 2 * J + j] = tv_ok ? wcov(m1, m2, w, A) / sqrt(fabs(tv1 * tv2)) : 0.0;
  }
}

int orc_data_stats(const abc_config* cfg, int64_t C, const int32_t* cell_cond, const int32_t* cell_age,
                   const double* age_dist, const int32_t* u, const int32_t* l, int64_t G, int n_boot,
                   uint64_t seed, double* stats, double* se) {
  const int A = cfg->n_ages, J = cfg->n_conds, K = 4 * A + 3 * J, NG = A * J;
  int32_t* cond_s = (int32_t*)malloc(sizeof(int32_t) * (size_t)C);
  int32_t* age_s = (int32_t*)malloc(sizeof(int32_t) * (size_t)C);
  int64_t* id_s = (int64_t*)malloc(sizeof(int64_t) * (size_t)C);
  int64_t gs[ABC_MAX_CONDS * ABC_MAX_AGES + 1];
  double* boot = (double*)malloc(sizeof(double) * (size_t)(n_boot + 1) * K);
  if (!cond_s || !age_s || !id_s || !boot) return ABC_ERR_NOMEM;
  /* stable counting sort by group = condition * A + age */
  memset(gs, 0, sizeof(gs));
  for (int64_t i = 0; i < C; ++i) gs[cell_cond[i] * A + cell_age[i] + 1]++;
  for (int q = 0; q < NG; ++q) gs[q + 1] += gs[q];
  int64_t cur[ABC_MAX_CONDS * ABC_MAX_AGES];
  for (int q = 0; q < NG; ++q) cur[q] = gs[q];
  for (int64_t i = 0; i < C; ++i) {
    int q = cell_cond[i] * A + cell_age[i];
    int64_t pos = cur[q]++;
    cond_s[pos] = cell_cond[i];
    age_s[pos] = cell_age[i];
    id_s[pos] = i;
  }
  for (int64_t g = 0; g < G; ++g) {
    for (int b = 0; b <= n_boot; ++b)
      data_one(cfg, C, cond_s, age_s, id_s, gs, age_dist, u + g * C, l + g * C, g, b, seed, boot + (size_t)b * K);
    memcpy(stats + g * K, boot, sizeof(double) * K);
    if (se && n_boot >= 2) {
      for (int k = 0; k < K; ++k) {
        double s = 0.0;
        for (int b = 1; b <= n_boot; ++b) s = s + boot[(size_t)b * K + k];
        double m = s / (double)n_boot, q = 0.0;
        for (int b = 1; b <= n_boot; ++b) {
          double d = boot[(size_t)b * K + k] - m;
          q = q + d * d;
        }
        se[g * K + k] = sqrt((1.0 / (double)(n_boot - 1)) * q);
      }
    }
  }
  free(cond_s); free(age_s); free(id_s); free(boot);
  return ABC_OK;
}
