// sampler32.cuh — FP32 samplers of the production mode: Poisson (initial
// states), binomial (capture) and the moment-matched initial count.  The
// same methods as the FP64 samplers of common.cuh, with all arithmetic in
// FP32, the final exact log-density tests included (each rewritten in log1p
// form so that its terms stay of the order of the deviation, not of n).
// Device code only; tested directly against the exact distributions
// (tests/test_samplers32.py).
#pragma once
#include "common.cuh"
#include "model.cuh"

namespace abc {

// Stirling-series remainder log k! - [(k + 1/2) log(k + 1) - (k + 1) + log(2 pi)/2]
// in FP32 (stirling_fc of common.cuh: the table below 10, the series above).
__device__ __forceinline__ float stirling_fc32(float k) {
  if (k < 10.0f) {
    switch ((int)k) {
      case 0: return 0.08106146679532726f;
      case 1: return 0.0413406959554093f;
      case 2: return 0.02767792568499834f;
      case 3: return 0.020790672103765093f;
      case 4: return 0.016644691189821193f;
      case 5: return 0.013876128823070748f;
      case 6: return 0.01189670994589177f;
      case 7: return 0.010411265261972096f;
      case 8: return 0.009255462182712733f;
      default: return 0.00833056343336287f;
    }
  }
  const float kp = k + 1.0f;
  const float r2 = 1.0f / (kp * kp);
  return (0.08333333333333333f - (0.002777777777777778f - 0.0007936507936507937f * r2) * r2) / kp;
}

// 24-bit uniforms in [0, 1) and (0, 1) for the FP32 samplers of the production mode
__device__ __forceinline__ float u24open(uint32_t w) { return ((float)(w >> 8) + 0.5f) * 5.9604644775390625e-8f; }
__device__ __forceinline__ float u24(uint32_t w) { return (float)(w >> 8) * 5.9604644775390625e-8f; }

// Poisson(lam) for the production mode: the FP64 sampler's two methods
// (inversion below lam = 10; Hormann's PTRS transformed rejection above) in
// FP32.  PTRS's final log-density test, k log lam - lam - log k!, cancels to a
// few units from terms of order lam log lam; it is evaluated in the form
// (d - k log1p(d / lam)) - log(k + 1)/2 - log(2 pi)/2 - fc(k), d = k + 1 - lam,
// whose terms are of order d, so FP32 keeps it to ~1e-7 |d| (GB300 runs FP64
// and its conversions at 1/64 of the FP32 rate).  Both loops are bounded.
__device__ inline int poisson32(Rng& r, float lam) {
  if (!(lam > 0.0f)) return 0;
  if (lam > 1.0e9f) return 1000000000;  // far above the production mode's count limit (2^23), reported there
  uint32_t w0, w1;
  if (lam < 10.0f) {
    rng_pair(r, w0, w1);
    float u = u24(w0);
    float f = expf(-lam);
    int k = 0;
    while (u >= f && k < 1000) {
      u = u - f;
      k = k + 1;
      f = f * (lam / (float)k);
    }
    return k;
  }
  const float slam = sqrtf(lam);
  const float b = 0.931f + 2.53f * slam;
  const float a = -0.059f + 0.02483f * b;
  const float inv_alpha = 1.1239f + 1.1328f / (b - 3.4f);
  const float vr = 0.9277f - 3.6224f / (b - 2.0f);
  for (int it = 0; it < 1000; ++it) {
    rng_pair(r, w0, w1);
    const float U = u24(w0) - 0.5f;
    const float V = u24open(w1);
    const float us = 0.5f - fabsf(U);
    const float kd = floorf((((2.0f * a) / us + b) * U + lam) + 0.43f);
    if (us >= 0.07f && V <= vr) return (int)kd;
    if (kd < 0.0f || (us < 0.013f && V > us)) continue;
    const float lhs = logf((V * inv_alpha) / (a / (us * us) + b));
    const float d = (kd + 1.0f) - lam;
    const float rhs = ((d - kd * log1pf(d / lam)) - 0.5f * logf(kd + 1.0f)) - 0.91893853320467274f - stirling_fc32(kd);
    if (lhs <= rhs) return (int)kd;
  }
  return (int)floorf(lam + 0.5f);
}

// initial_count (model.cuh) with FP32 arithmetic and the FP32 Poisson sampler:
// the same moment-matched zero-inflated Poisson given G, from the periodic
// moments (g0, u0, c0, v0) in FP32.
__device__ inline int initial_count32(float g, float m, float c, float v, int G, uint32_t wz, Rng& aux) {
  float mu = m, vr = v;
  if (g > 0.0f && g < 1.0f) {
    mu = G ? m + c / g : m - c / (1.0f - g);
    vr = v - (c * c) / (g * (1.0f - g));
  }
  if (!(mu > 0.0f)) return 0;
  const float F = (m > 0.0f && vr > 0.0f) ? vr / m : 0.0f;
  float lam = mu;
  if (F > 1.0f) {
    const float w = mu / (mu + (F - 1.0f));
    if (!((float)(wz >> 8) * 5.9604644775390625e-8f < w)) return 0;
    lam = mu / w;
  }
  return poisson32(aux, lam);
}

// ---------------------------------------------------------------------------
// Binomial capture for the FP32 production mode: the same two methods as the
// FP64 samplers of common.cuh (inversion below n p = 10, Kachitvichyanukul &
// Schmeiser 1988; BTRD above, Hormann 1993) in FP32, which runs at the full
// rate where the FP64 samplers are bound by GB300's narrow FP64 pipe.  BTRD's
// final exact test (the log-density comparison between its two squeezes)
// has terms (n + 1) log(...) of order n; it is evaluated with log1p of the
// ratios' distances from 1, (n + 2) p - (j + 1) formed by one FMA, so each
// term is of order |k - m| and FP32 keeps the sum to ~1e-7 of that.  Counts
// are below 2^23 in this mode.  A different realisation than the FP64 mode's,
// drawn from the same distribution.
// ---------------------------------------------------------------------------
__device__ inline int binv32(Rng& rr, int n, float p) {
  const float q = 1.0f - p;
  const float s = p / q;
  const float a = (float)(n + 1) * s;
  const float r0 = expf((float)n * log1pf(-p));
  uint32_t w[2] = {0u, 0u};
  for (int it = 0; it < 64; ++it) {
    if ((it & 1) == 0) rng_pair(rr, w[0], w[1]);
    float u = u24(w[it & 1]);
    float f = r0;
    int x = 0;
    for (;;) {
      if (u < f) return x;
      if (x >= n || x >= 110) break;
      u = u - f;
      x = x + 1;
      f = f * (a / (float)x - s);
    }
  }
  return (int)floorf((float)n * p + 0.5f);
}

__device__ inline int btrd32(Rng& rr, int n, float p) {
  const float nd = (float)n;
  const float q = 1.0f - p;
  const float m = floorf((nd + 1.0f) * p);
  const float r = p / q;
  const float nr = (nd + 1.0f) * r;
  const float npq = (nd * p) * q;
  const float sq = sqrtf(npq);
  const float b = 1.15f + 2.53f * sq;
  const float a = (-0.0873f + 0.0248f * b) + 0.01f * p;
  const float c = nd * p + 0.5f;
  const float alpha = (2.83f + 5.1f / b) * sq;
  const float vr = 0.92f - 4.2f / b;
  const float urvr = 0.86f * vr;
  for (int it = 0; it < 1000; ++it) {
    uint32_t w0, w1;
    rng_pair(rr, w0, w1);
    float v = u24open(w0);
    float u;
    if (v <= urvr) {
      u = v / vr - 0.43f;
      return (int)floorf(((2.0f * a) / (0.5f - fabsf(u)) + b) * u + c);
    }
    if (v >= vr) {
      u = u24open(w1) - 0.5f;
    } else {
      u = v / vr - 0.93f;
      u = (u < 0.0f ? -0.5f : 0.5f) - u;
      v = u24open(w1) * vr;
    }
    const float us = 0.5f - fabsf(u);
    const float kd = floorf(((2.0f * a) / us + b) * u + c);
    if (kd < 0.0f || kd > nd) continue;
    v = (v * alpha) / (a / (us * us) + b);
    const float km = fabsf(kd - m);
    if (km <= 15.0f) {
      float f = 1.0f;
      if (m < kd) {
        for (float i = m + 1.0f; i <= kd; i += 1.0f) f = f * (nr / i - r);
      } else if (m > kd) {
        for (float i = kd + 1.0f; i <= m; i += 1.0f) v = v * (nr / i - r);
      }
      if (v <= f) return (int)kd;
      continue;
    }
    const float lv = logf(v);
    const float rho = (km / npq) * (((km / 3.0f + 0.625f) * km + 0.16666667f) / npq + 0.5f);
    const float t = (-km * km) / (2.0f * npq);
    if (lv < t - rho) return (int)kd;
    if (lv > t + rho) continue;
    // exact test: log f(k) - log f(m) against log v, with
    //   log((m + 1) / (r nm)) = -log1p(em),  em = ((n + 2) p - (m + 1)) / ((m + 1) q),
    //   log(nm / nk) = log1p((k - m) / nk),  log(nk r / (k + 1)) = log1p(ek), likewise
    const float nk = (nd - kd) + 1.0f;
    const float em = fmaf(nd + 2.0f, p, -(m + 1.0f)) / ((m + 1.0f) * q);
    const float ek = fmaf(nd + 2.0f, p, -(kd + 1.0f)) / ((kd + 1.0f) * q);
    const float h = ((m + 0.5f) * -log1pf(em) + stirling_fc32(m)) + stirling_fc32(nd - m);
    const float bound = (((h + (nd + 1.0f) * log1pf((kd - m) / nk)) + (kd + 0.5f) * log1pf(ek)) -
                         stirling_fc32(kd)) - stirling_fc32(nd - kd);
    if (lv <= bound) return (int)kd;
  }
  return (int)floorf(nd * p + 0.5f);
}

// Bin(n, p) for a capture efficiency p given in FP32 (1 - p is exact for p > 1/2)
__device__ __forceinline__ int binomial32(Rng& r, int n, float p) {
  if (n <= 0 || !(p > 0.0f)) return 0;
  if (p >= 1.0f) return n;
  const bool flip = p > 0.5f;
  const float pp = flip ? 1.0f - p : p;
  const int k = ((float)n * pp < 10.0f) ? binv32(r, n, pp) : btrd32(r, n, pp);
  return flip ? n - k : k;
}

}  // namespace abc
