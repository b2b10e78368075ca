// common.cuh — primitives shared by the kernels (and their host-side helpers):
// Philox4x32-10 streams, deterministic FP64 log/exp, binomial samplers.
//
// FP64 arithmetic here must give the same bits on the GPU as the FP64 CPU
// oracle: translation units that include this header for FP64 work are built
// with -fmad=false (device) and -ffp-contract=off (host), and every
// expression keeps the oracle's operation order.
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define ABC_HD __host__ __device__ __forceinline__
#else
#define ABC_HD inline
#endif

namespace abc {

// ---------------------------------------------------------------------------
// bit casts
// ---------------------------------------------------------------------------
ABC_HD uint64_t d2u(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
ABC_HD double u2d(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
ABC_HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers:
// as easy as 1, 2, 3").
// ---------------------------------------------------------------------------
struct U4 {
  uint32_t x, y, z, w;
};

ABC_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c.x;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c.z;
    U4 n;
    n.x = (uint32_t)(p1 >> 32) ^ c.y ^ k0;
    n.y = (uint32_t)p1;
    n.z = (uint32_t)(p0 >> 32) ^ c.w ^ k1;
    n.w = (uint32_t)p0;
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Stream ids (top two bits of counter word 1).
enum : uint32_t { ST_SSA = 0, ST_CAPTURE = 1, ST_PRIOR = 2, ST_AUX = 3 };

// Random stream of one (particle, cell, purpose): counter = (block lo,
// block hi | stream<<30, cell, particle), key = seed.  Words are consumed in
// pairs; one Philox block yields two pairs.
struct Rng {
  uint32_t k0, k1, cell, particle, tag;
  uint32_t b2, b3;
  int half;
  uint64_t block;
};

ABC_HD void rng_init(Rng& r, uint64_t seed, uint32_t stream, uint32_t cell, uint32_t particle) {
  r.k0 = (uint32_t)seed;
  r.k1 = (uint32_t)(seed >> 32);
  r.cell = cell;
  r.particle = particle;
  r.tag = stream << 30;
  r.block = 0;
  r.half = 0;
  r.b2 = r.b3 = 0;
}

ABC_HD void rng_pair(Rng& r, uint32_t& a, uint32_t& b) {
  if (r.half == 0) {
    U4 c;
    c.x = (uint32_t)r.block;
    c.y = ((uint32_t)(r.block >> 32) & 0x3fffffffu) | r.tag;
    c.z = r.cell;
    c.w = r.particle;
    U4 o = philox4x32_10(c, r.k0, r.k1);
    r.block++;
    a = o.x;
    b = o.y;
    r.b2 = o.z;
    r.b3 = o.w;
    r.half = 1;
  } else {
    a = r.b2;
    b = r.b3;
    r.half = 0;
  }
}

#define ABC_TWO_M32 2.3283064365386963e-10
#define ABC_TWO_M52 2.220446049250313e-16

ABC_HD double u52open(uint32_t a, uint32_t b) {
  uint64_t x = ((uint64_t)a << 20) | (uint64_t)(b >> 12);
  return ((double)x + 0.5) * ABC_TWO_M52;
}
ABC_HD double u52(uint32_t a, uint32_t b) {
  uint64_t x = ((uint64_t)a << 20) | (uint64_t)(b >> 12);
  return (double)x * ABC_TWO_M52;
}

// ---------------------------------------------------------------------------
// Deterministic log / exp from their series (no library math): log via
// x = m 2^e, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)) summed to
// s^25; exp via x = k ln2 + r, |r| <= ln2/2, Taylor to r^14.  ln2 is split in
// a 32-significant-bit head (k * head exact) and the remainder.
// Positive normal arguments only (log); results within ~2 ulp.
// ---------------------------------------------------------------------------
#define ABC_LN2_HI 0.6931471803691238
#define ABC_LN2_LO 1.9082149292705877e-10
#define ABC_INV_LN2 1.4426950408889634
#define ABC_LN10 2.302585092994046
#define ABC_SQRT2 1.4142135623730951

ABC_HD double xlog(double x) {
  uint64_t b = d2u(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = u2d((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
  if (m > ABC_SQRT2) {
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
  return de * ABC_LN2_HI + (de * ABC_LN2_LO + (2.0 * s) * p);
}

ABC_HD double xexp(double x) {
  if (x != x) return x;
  if (x > 709.0) return INFINITY;
  if (x < -745.0) return 0.0;
  double kd = floor(x * ABC_INV_LN2 + 0.5);
  double r = (x - kd * ABC_LN2_HI) - kd * ABC_LN2_LO;
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
  if (k >= -1021) return p * u2d((uint64_t)(k + 1023) << 52);
  return (p * u2d((uint64_t)(k + 1023 + 60) << 52)) * 8.673617379884035e-19;
}

ABC_HD double xexp10(double x) { return xexp(x * ABC_LN10); }
ABC_HD double xpow(double x, double s) {
  if (s == 0.0) return 1.0;
  if (s == 1.0) return x;
  return xexp(s * xlog(x));
}

// ---------------------------------------------------------------------------
// Binomial samplers.  Bin(n, 1/2): popcount of n random bits.  Bin(n, p):
// inversion when n min(p,1-p) < 10 (Kachitvichyanukul & Schmeiser 1988),
// BTRD otherwise (Hormann 1993, "The generation of binomial random
// variates", J. Stat. Comput. Simul. 46:101-110).
// ---------------------------------------------------------------------------
ABC_HD int64_t binom_half(Rng& r, int64_t n) {
  int64_t k = 0;
  while (n > 0) {
    uint32_t a, b;
    rng_pair(r, a, b);
    uint64_t bits = ((uint64_t)b << 32) | (uint64_t)a;
    if (n < 64) bits &= (((uint64_t)1) << n) - 1;
    k += (int64_t)popc64(bits);
    n -= 64;
  }
  return k;
}

ABC_HD int64_t binv(Rng& rr, int64_t n, double p) {
  double q = 1.0 - p;
  double s = p / q;
  double a = (double)(n + 1) * s;
  double r0 = xexp((double)n * xlog(q));
  for (;;) {
    uint32_t w0, w1;
    rng_pair(rr, w0, w1);
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

// Stirling-series correction log(k!) - [(k+1/2) log(k+1) - (k+1) + log(2 pi)/2],
// tabulated below 10 (50-digit values rounded to double).
ABC_HD double stirling_fc(double k) {
  if (k < 10.0) {
    switch ((int)k) {
      case 0: return 0.08106146679532726;
      case 1: return 0.0413406959554093;
      case 2: return 0.02767792568499834;
      case 3: return 0.020790672103765093;
      case 4: return 0.016644691189821193;
      case 5: return 0.013876128823070748;
      case 6: return 0.01189670994589177;
      case 7: return 0.010411265261972096;
      case 8: return 0.009255462182712733;
      default: return 0.00833056343336287;
    }
  }
  double kp = k + 1.0;
  double r2 = 1.0 / (kp * kp);
  return (0.08333333333333333 - (0.002777777777777778 - 0.0007936507936507937 * r2) * r2) / kp;
}

ABC_HD int64_t btrd(Rng& rr, int64_t n, double p) {
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
  double h = ((m + 0.5) * xlog((m + 1.0) / (r * nm)) + stirling_fc(m)) + stirling_fc(nd - m);
  for (;;) {
    uint32_t w0, w1;
    rng_pair(rr, w0, w1);
    double v = u52open(w0, w1);
    double u;
    if (v <= urvr) {
      u = v / vr - 0.43;
      return (int64_t)floor(((2.0 * a) / (0.5 - fabs(u)) + b) * u + c);
    }
    if (v >= vr) {
      rng_pair(rr, w0, w1);
      u = u52open(w0, w1) - 0.5;
    } else {
      u = v / vr - 0.93;
      u = (u < 0.0 ? -0.5 : 0.5) - u;
      rng_pair(rr, w0, w1);
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
    v = xlog(v);
    double rho = (km / npq) * (((km / 3.0 + 0.625) * km + 0.16666666666666666) / npq + 0.5);
    double t = (-km * km) / (2.0 * npq);
    if (v < t - rho) return (int64_t)kd;
    if (v > t + rho) continue;
    double nk = (nd - kd) + 1.0;
    double bound = (((h + (nd + 1.0) * xlog(nm / nk)) + (kd + 0.5) * xlog((nk * r) / (kd + 1.0))) -
                    stirling_fc(kd)) - stirling_fc(nd - kd);
    if (v <= bound) return (int64_t)kd;
  }
}

// log(k!) from the Stirling series with the tabulated correction above.
ABC_HD double logfact(double k) {
  return (((k + 0.5) * xlog(k + 1.0) - (k + 1.0)) + 0.9189385332046728) + stirling_fc(k);
}

// Poisson(lam): inversion by sequential search below lam = 10, otherwise
// PTRS, the transformed rejection with squeeze of W. Hormann, "The
// transformed rejection method for generating Poisson random variables",
// Insurance: Mathematics and Economics 12 (1993) 39-45.  Both loops are
// bounded (the acceptance rate of PTRS is about 0.9 per try).
ABC_HD int64_t poisson(Rng& r, double lam) {
  if (!(lam > 0.0)) return 0;
  uint32_t w0, w1;
  if (lam < 10.0) {
    rng_pair(r, w0, w1);
    double u = u52(w0, w1);
    double f = xexp(-lam);
    int64_t k = 0;
    while (u >= f && k < 1000) {
      u = u - f;
      k = k + 1;
      f = f * (lam / (double)k);
    }
    return k;
  }
  const double slam = sqrt(lam);
  const double loglam = xlog(lam);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < 1000; ++it) {
    rng_pair(r, w0, w1);
    const double U = u52(w0, w1) - 0.5;
    rng_pair(r, w0, w1);
    const double V = u52open(w0, w1);
    const double us = 0.5 - fabs(U);
    const double kd = floor((((2.0 * a) / us + b) * U + lam) + 0.43);
    if (us >= 0.07 && V <= vr) return (int64_t)kd;
    if (kd < 0.0 || (us < 0.013 && V > us)) continue;
    const double lhs = xlog((V * inv_alpha) / (a / (us * us) + b));
    const double rhs = (kd * loglam - lam) - logfact(kd);
    if (lhs <= rhs) return (int64_t)kd;
  }
  return (int64_t)floor(lam + 0.5);
}

ABC_HD int64_t binomial(Rng& r, int64_t n, double p) {
  if (n <= 0 || !(p > 0.0)) return 0;
  if (p >= 1.0) return n;
  bool flip = p > 0.5;
  double pp = flip ? 1.0 - p : p;
  int64_t k = ((double)n * pp < 10.0) ? binv(r, n, pp) : btrd(r, n, pp);
  return flip ? n - k : k;
}

}  // namespace abc
