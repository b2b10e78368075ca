// sampler32.cuh — FP32 samplers of the production mode: Poisson (initial
// states), binomial (capture) and the moment-matched initial count.  The
// same methods as the FP64 samplers of common.cuh, with the per-draw
// arithmetic in FP32; each algorithm's final exact log-density test, a small
// fraction of the draws, stays in FP64.  Device code only; tested directly
// against the exact distributions (tests/test_samplers32.py).
#pragma once
#include "common.cuh"
#include "model.cuh"

namespace abc {

// 24-bit uniforms in [0, 1) and (0, 1) for the FP32 samplers of the production mode
__device__ __forceinline__ float u24open(uint32_t w) { return ((float)(w >> 8) + 0.5f) * 5.9604644775390625e-8f; }
__device__ __forceinline__ float u24(uint32_t w) { return (float)(w >> 8) * 5.9604644775390625e-8f; }

// Poisson(lam) for the production mode: the FP64 sampler's two methods
// (inversion below lam = 10; Hormann's PTRS transformed rejection above) with
// the per-draw arithmetic in FP32; PTRS's final log-density test, between its
// squeezes, stays in FP64 (k log lam - lam - log k! cancels to a few units
// from terms of order lam log lam).  Both loops are bounded.
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
    const double ld = (double)lam, kk = (double)kd;
    const double lhs = xlog(((double)V * (double)inv_alpha) / ((double)a / ((double)us * (double)us) + (double)b));
    const double rhs = (kk * xlog(ld) - ld) - logfact(kk);
    if (lhs <= rhs) return (int)kd;
  }
  return (int)floorf(lam + 0.5f);
}

// initial_count (model.cuh) with FP32 arithmetic and the FP32 Poisson sampler:
// the same moment-matched zero-inflated Poisson given G.
__device__ inline int initial_count32(const PRec& R, int G, uint32_t wz, Rng& aux) {
  const float g = (float)R.g0, m = (float)R.u0, c = (float)R.c0, v = (float)R.v0;
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
// Schmeiser 1988; BTRD above, Hormann 1993) with the per-draw arithmetic in
// FP32, which runs at the full rate where the FP64 samplers are bound by
// GB300's narrow FP64 pipe.  Only BTRD's final exact test (the log-density
// comparison between its two squeezes, a small fraction of the draws) stays
// in FP64, where (n + 1) log(...) needs the precision.  Counts are below 2^23
// in this mode.  A different realisation than the FP64 mode's, drawn from the
// same distribution.
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
    // exact test in FP64 (log f(k) - log f(m) against log v)
    const double ndd = (double)n, pdd = (double)p, rd = pdd / (1.0 - pdd), md = (double)m, kdd = (double)kd;
    const double nm = (ndd - md) + 1.0, nk = (ndd - kdd) + 1.0;
    const double h = ((md + 0.5) * xlog((md + 1.0) / (rd * nm)) + stirling_fc(md)) + stirling_fc(ndd - md);
    const double bound = (((h + (ndd + 1.0) * xlog(nm / nk)) + (kdd + 0.5) * xlog((nk * rd) / (kdd + 1.0))) -
                          stirling_fc(kdd)) - stirling_fc(ndd - kdd);
    if ((double)lv <= bound) return (int)kd;
  }
  return (int)floorf(nd * p + 0.5f);
}

__device__ __forceinline__ int64_t binomial32(Rng& r, int64_t n, double p) {
  if (n <= 0 || !(p > 0.0)) return 0;
  if (p >= 1.0) return n;
  const bool flip = p > 0.5;
  const float pp = (float)(flip ? 1.0 - p : p);
  const int ni = (int)n;
  const int k = ((float)ni * pp < 10.0f) ? binv32(r, ni, pp) : btrd32(r, ni, pp);
  return flip ? n - k : k;
}

}  // namespace abc
