// distance.cuh — shared pieces of the particle x gene distance kernels.
//
// err_pg = min(10, sum_f sum_{k in f} (d_gk - s_pk)^2 / (se_gk^2 + 0.01 d_gk^2 + eps_gk) / K)
// with eps_gk = 1e-4 iff se_gk + d_gk == 0 (scripts/compute_errors.jl:30-43,
// clipped at 10 by :159-161).
//
// Fast path (FP32 CUDA cores): with a = sqrt(w_gk) the term is
// (a d - a s)^2; a and a*d are formed in FP64 and rounded once, so
// t = fma(-a, s, a d) and acc = fma(t, t, acc): two FMAs per (p, g, k).
// Because w d^2 <= 1/0.01 = 100 for every gene, |a d| <= 10, and a forward
// error analysis of the FP32 evaluation gives
//   |err32 - err64| <= B(err) = 1.5 u (64 sqrt(err) + (K + 8) err),  u = 2^-24,
// B increasing in err.  Pairs whose FP32 error lies within B of the threshold
// are rechecked in FP64 in the reference's operation order.
#pragma once
#include <math.h>

namespace abc {

#if defined(__CUDACC__)
#define ABC_HDF __host__ __device__ __forceinline__
#else
#define ABC_HDF inline
#endif

ABC_HDF float dist_bound_f(float e, int K) {
  if (!(e >= 0.0f)) e = 0.0f;
  const float u = 5.9604644775390625e-08f;
  return 1.5f * u * (64.0f * sqrtf(e) + (float)(K + 8) * e) + 1e-30f;
}

#if defined(__CUDACC__)
// Correctly rounded a / b (round to nearest) from y = RN(1/b), in three FP64
// operations instead of a full division: q0 = RN(a y) is within one ulp of
// a / b, the remainder r = a - b q0 is exact (one FMA), and RN(q0 + r y) =
// RN(a / b) (Markstein's theorem: P. Markstein, IBM J. Res. Dev. 34(1), 1990;
// J.-M. Muller et al., Handbook of Floating-Point Arithmetic, ch. 4).  The
// theorem needs a, b and the quotient away from underflow and overflow; outside
// [2^-900, 2^900) x [2^-400, 2^400) (and for zero, NaN, infinity) the IEEE
// division is used.  The ranges are tested on the biased exponent fields with
// integer instructions: FP64 comparisons would share the FP64 pipe, the
// recheck's bottleneck, with the six arithmetic operations of a term.
__device__ __forceinline__ double div_rn(double a, double b, double y) {
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;  // 2^-900 = 2^(123 - 1023)
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;  // 2^-400 = 2^(623 - 1023)
  if (ea - 123u < 1800u && eb - 623u < 800u) {
    const double q0 = a * y;
    const double r = fma(-q0, b, a);
    return fma(r, y, q0);
  }
  return a / b;
}

// RN32(x) from the bit fields of x (integer operations; GB300 runs FP64 -> FP32
// conversions on its narrow FP64 pipe): the top 23 stored significand bits,
// rounded to nearest even on bit 28 and the sticky bits 0-27, with the carry
// rippling into the exponent (and to infinity above the float range); the
// conversion instruction only for results below the normal float range and
// for zero, infinity and NaN.  Identical to (float)x.
__device__ __forceinline__ float rn32_bits(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned mag = hi & 0x7fffffffu;
  const unsigned e = mag >> 20;
  if (e - 897u > 253u) return (float)x;  // e outside [897, 1150]
  unsigned f = (hi & 0x80000000u) | ((mag - (896u << 20)) << 3) | (lo >> 29);
  const unsigned rb = (lo >> 28) & 1u, sticky = lo & 0x0fffffffu;
  f += rb & ((sticky != 0u) | (f & 1u));
  return __uint_as_float(f);
}
#endif

constexpr int kDistTile = 128;  // particles and genes per CTA tile
constexpr int kDistKc = 16;     // statistics per shared-memory stage
constexpr int kHistBins = 4096; // threshold histogram bins (sqrt scale on [0, 10])

ABC_HDF int hist_bin(float e) {
  float x = sqrtf(e * 0.1f) * (float)kHistBins;
  int b = (int)x;
  return b < 0 ? 0 : (b >= kHistBins ? kHistBins - 1 : b);
}
ABC_HDF float hist_upper(int b) {
  float q = (float)(b + 1) / (float)kHistBins;
  return 10.0f * q * q * 1.0000005f;
}

}  // namespace abc
