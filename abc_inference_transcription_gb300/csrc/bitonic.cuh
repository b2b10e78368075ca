// bitonic.cuh — register-resident bitonic sort of one segment per block.
//
// All-ascending form of the bitonic network (the first step of every merge
// of size k pairs i with i ^ (k - 1), the others i with i ^ j), over n2 (a
// power of two) entries of (64-bit key, 32-bit index) compared
// lexicographically.  Thread t holds the EPT consecutive entries
// t * EPT ... t * EPT + EPT - 1 in registers (nt = max(32, n2 / EPT) threads
// hold entries; the block may be larger).  Steps whose partner lies in the
// same thread run on registers, steps whose partner lies in the same warp on
// shuffles, and only the steps across warps (partner distance >= 32 EPT)
// exchange through shared memory (sK, sP: n2 entries each).  Every thread of
// the block must call it (it contains block barriers).
#pragma once
#include <stdint.h>

namespace abc {

// (ka, pa) receives the smaller entry
__device__ __forceinline__ void bs_cas_lo(uint64_t& ka, int32_t& pa, uint64_t& kb, int32_t& pb) {
  const bool sw = kb < ka || (kb == ka && pb < pa);
  const uint64_t tk = sw ? kb : ka;
  const int32_t tp = sw ? pb : pa;
  kb = sw ? ka : kb;
  pb = sw ? pa : pb;
  ka = tk;
  pa = tp;
}

// own entry becomes min (lower) or max of (own, other)
__device__ __forceinline__ void bs_keep(uint64_t& k, int32_t& p, uint64_t ok, int32_t op, bool lower) {
  const bool other_less = ok < k || (ok == k && op < p);
  const bool take = lower ? other_less : !other_less;
  k = take ? ok : k;
  p = take ? op : p;
}

template <int EPT, int J, bool FLIP>
__device__ __forceinline__ void bs_step_in_thread(uint64_t* key, int32_t* pp) {
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const int f = FLIP ? (e ^ (2 * J - 1)) : (e ^ J);
    if (f > e) bs_cas_lo(key[e], pp[e], key[f], pp[f]);
  }
}

template <int EPT>
__device__ __forceinline__ void bs_in_thread(uint64_t* key, int32_t* pp, int j, bool flip) {
  if (EPT >= 2 && j == 1) {
    if (flip) bs_step_in_thread<EPT, 1, true>(key, pp); else bs_step_in_thread<EPT, 1, false>(key, pp);
  } else if (EPT >= 4 && j == 2) {
    if (flip) bs_step_in_thread<EPT, 2, true>(key, pp); else bs_step_in_thread<EPT, 2, false>(key, pp);
  } else if (EPT >= 8 && j == 4) {
    if (flip) bs_step_in_thread<EPT, 4, true>(key, pp); else bs_step_in_thread<EPT, 4, false>(key, pp);
  }
}

__device__ __forceinline__ void bs_shfl_entry(uint64_t k, int32_t p, int mask, uint64_t& ok, int32_t& op) {
  const unsigned lo = __shfl_xor_sync(0xffffffffu, (unsigned)k, mask);
  const unsigned hi = __shfl_xor_sync(0xffffffffu, (unsigned)(k >> 32), mask);
  op = __shfl_xor_sync(0xffffffffu, p, mask);
  ok = ((uint64_t)hi << 32) | lo;
}

template <int EPT>
__device__ __forceinline__ void bitonic_regs(uint64_t* key, int32_t* pp, int n2, uint64_t* sK, int32_t* sP) {
  const int t = threadIdx.x;
  const int nt = n2 / EPT > 32 ? n2 / EPT : 32;
  const bool act = t < nt;
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const bool flip = j == (k >> 1);
      if (j < EPT) {
        bs_in_thread<EPT>(key, pp, j, flip);
      } else if (j < 32 * EPT) {
        if (act) {
          if (!flip) {
            const int mask = j / EPT;
            const bool lower = (t & mask) == 0;
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
              uint64_t ok;
              int32_t op;
              bs_shfl_entry(key[e], pp[e], mask, ok, op);
              bs_keep(key[e], pp[e], ok, op, lower);
            }
          } else {
            // entry e pairs with the partner's entry EPT - 1 - e
            const int mask = k / EPT - 1;
            const bool lower = (t & ((mask + 1) >> 1)) == 0;
#pragma unroll
            for (int e = 0; e < (EPT + 1) / 2; ++e) {
              const int f = EPT - 1 - e;
              uint64_t o1, o2;
              int32_t q1, q2;
              bs_shfl_entry(key[f], pp[f], mask, o1, q1);
              if (f != e) bs_shfl_entry(key[e], pp[e], mask, o2, q2);
              bs_keep(key[e], pp[e], o1, q1, lower);
              if (f != e) bs_keep(key[f], pp[f], o2, q2, lower);
            }
          }
        }
      } else {
        // across warps: entry (t, e) in slot e * nt + t
        if (act) {
#pragma unroll
          for (int e = 0; e < EPT; ++e) {
            sK[e * nt + t] = key[e];
            sP[e * nt + t] = pp[e];
          }
        }
        __syncthreads();
        if (act) {
          const int mask = flip ? k / EPT - 1 : j / EPT;
          const bool lower = (t & (flip ? (mask + 1) >> 1 : mask)) == 0;
          const int tp = t ^ mask;
#pragma unroll
          for (int e = 0; e < EPT; ++e) {
            const int f = flip ? EPT - 1 - e : e;
            bs_keep(key[e], pp[e], sK[f * nt + tp], sP[f * nt + tp], lower);
          }
        }
        __syncthreads();
      }
    }
  }
}

}  // namespace abc
