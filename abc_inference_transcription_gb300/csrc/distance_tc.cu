// distance_tc.cu — the particle x gene candidate pass as a tensor-core GEMM
// (tcgen05 MMA with TF32 or BF16 operands, accumulators in tensor memory,
// operands staged by TMA) with a fused candidate epilogue.
//
// The reference error (scripts/compute_errors.jl:30-43) of particle p for gene g
// is (1/K) sum_k w_gk (d_gk - s_pk)^2, w_gk = 1/((se_gk^2 + 0.01 d_gk^2) + eps_gk).
// Expanded:
//   K err_pg = c_g + sum_k [ (-2 w_gk d_gk) s_pk + w_gk s_pk^2 ],   c_g = sum_k w_gk d_gk^2,
// i.e. one GEMM of A = [s | s^2] (particles, K-major rows) against
// B = [-2 w d | w] (genes, K-major rows) of depth 2K, FP32 accumulation.
// Three-term modes split each operand into hi + lo parts and accumulate
// hi*hi + hi*lo + lo*hi: TF32 parts leave every product exact to ~2^-21,
// BF16 parts (MMAs at twice the TF32 rate, half the operand bytes) to ~2^-17.
//
// CTA: 18 warps, one persistent CTA per SM.  Warp 0 issues TMA loads of
// 128 x 128-byte (A) and 256 x 128-byte (B) boxes with the 128-byte swizzle
// into a ring of shared-memory stages; warp 1 owns 512 tensor-memory columns
// (two 128 x 256 FP32 accumulators) and issues the MMAs; warps 2-17 read the
// finished accumulator (four warps per TMEM lane quarter, a quarter of the
// columns each), compare acc <= Y_g (Y_g = K X_g - c_g rounded up) and append
// candidates with their raw accumulator to this CTA's own output segment
// through a shared-memory counter; the gather that concatenates the segments
// turns the accumulator into the FP32 error, clipped at 10 like the
// reference's.  The epilogue of one tile
// overlaps the MMAs of the next.  Every wait on an mbarrier is bounded by a
// clock limit; a wait that runs out sets an error bit, the CTA stops issuing
// work, waits (bounded) for its copies and MMAs in flight, frees its tensor
// memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstring>

#include "distance.cuh"
#include "smem_attr.h"
#include "kernels.h"
#include "tcgen05.cuh"

namespace abc {
namespace {

using namespace tc;

constexpr int BM = 128;          // particles per tile = TMEM lanes
constexpr int BN = 256;          // genes per tile = TMEM columns per accumulator
constexpr int BK = 32;           // FP32 values per 128-byte swizzled row (one TMA box width)
constexpr int kEpiWarps = 16;                // four per TMEM lane quarter, each a quarter of the columns
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kEpiGroups = BN / 32 / (kEpiWarps / 4);  // 32-column groups per epilogue warp
constexpr int kThreads = 64 + kEpiThreads;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kABytes = BM * BK * 4;    // 16 KB
constexpr uint32_t kBBytes = BN * BK * 4;    // 32 KB
static_assert(kABytes >> 4 == 1024 && kBBytes >> 4 == 2048, "descriptor offsets in 16-byte units");

template <int NH>
struct Cfg {
  static constexpr int kStages = NH == 1 ? 4 : 2;
  static constexpr uint32_t kStageBytes = NH * (kABytes + kBBytes);
  static constexpr uint32_t kTileBytes = kStages * kStageBytes;
  // tiles + barriers (2 S + 5) + tmem slot + counters + per-gene Y and column masks of a tile
  static constexpr uint32_t kSmem = 1024 + kTileBytes + 256 + BN * 4 + BN / 8;
};

// Instruction descriptor: D = F32, A = B = TF32, both K-major, M = 128, N = 256.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

// The same tile shape with BF16 operands (D = F32, A = B = BF16, K-major, K = 16 per MMA).
constexpr uint32_t kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdescBf16), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory"); }

// v[j] for a lane-dependent j, by a 5-level select tree on the bits of j
// (a dynamically indexed register array would go to local memory).
__device__ __forceinline__ float pick32(const uint32_t (&v)[32], uint32_t j) {
  uint32_t a16[16], a8[8], a4[4], a2[2];
#pragma unroll
  for (int i = 0; i < 16; ++i) a16[i] = (j & 1u) ? v[2 * i + 1] : v[2 * i];
#pragma unroll
  for (int i = 0; i < 8; ++i) a8[i] = (j & 2u) ? a16[2 * i + 1] : a16[2 * i];
#pragma unroll
  for (int i = 0; i < 4; ++i) a4[i] = (j & 4u) ? a8[2 * i + 1] : a8[2 * i];
#pragma unroll
  for (int i = 0; i < 2; ++i) a2[i] = (j & 8u) ? a4[2 * i + 1] : a4[2 * i];
  return __uint_as_float((j & 16u) ? a2[1] : a2[0]);
}

// Smallest float above y (y itself for +inf and NaN).
__device__ __forceinline__ float next_up(float y) {
  if (y != y || y == INFINITY) return y;
  if (y == 0.0f) return __uint_as_float(1u);
  const uint32_t u = __float_as_uint(y);
  return __uint_as_float(y > 0.0f ? u + 1u : u - 1u);
}

// Per-tile inputs of the epilogue, written by epilogue threads et < BN:
// Yn[j] = next_up(Y_g) and bit j of CM[w] set when column 32 w + j is a gene
// g < G with Y_g and c_g not NaN (its accumulators are finite in every row
// without a NaN statistic).
__device__ __forceinline__ void epi_fill(int et, int64_t g0, const TcArgs& a, float* Yn, uint32_t* CM) {
  static_assert(kEpiThreads >= BN && BN % 32 == 0, "one epilogue thread per column, whole warps");
  if (et < BN) {
    const int64_t g = g0 + et;
    bool ok = false;
    float y = -INFINITY;
    if (g < a.G) {
      y = a.Y[g];
      const float c = a.cg[g];
      ok = y == y && c == c;
    }
    Yn[et] = ok ? next_up(y) : -INFINITY;
    const uint32_t b = __ballot_sync(0xffffffffu, ok);
    if ((et & 31) == 0) CM[et >> 5] = b;
  }
}

// Epilogue of one warp: its 32 accumulator rows (one TMEM lane quarter, lane =
// particle row) x NG groups of 32 columns starting at TMEM address taddr.
// For finite acc and Y, acc <= Y iff acc < next_up(Y) iff the sign bit of
// the rounded difference acc - next_up(Y) is set (a nonzero difference keeps
// its sign under rounding; acc == next_up(Y) gives +0): one subtraction (FMA
// pipe) and one funnel shift per element build the lane's candidate mask,
// which the column mask CM (genes with finite accumulators) and the row mask
// rm (0 for a particle with a NaN statistic or beyond P) then restrict.  A
// warp with any candidate takes its positions in the CTA segment with one
// shared-memory atomic plus the lanes' exclusive prefix (a ballot when no lane
// holds more than one candidate, the common case); each candidate stores
// (p, g) and the raw accumulator, which tc_gather_kernel turns into the
// clipped FP32 error.
template <int NG>
__device__ __forceinline__ void epi_warp(uint32_t taddr, const float* Yn, const uint32_t* CM, int64_t row,
                                         uint32_t rm, int64_t g0, uint32_t* s_count, const TcArgs& a, int lane) {
#pragma unroll 1
  for (int gi = 0; gi < NG; ++gi) {
    __syncwarp();
    uint32_t v[32];
    tmem_ld32(taddr + (uint32_t)(gi * 32), v);
    const float4* Y4 = reinterpret_cast<const float4*>(Yn + gi * 32);
    uint32_t m[4] = {0u, 0u, 0u, 0u};  // four independent chains, columns 8c .. 8c + 7
#pragma unroll
    for (int j4 = 7; j4 >= 0; --j4) {
      const float4 y = Y4[j4];
      uint32_t& mc = m[j4 >> 1];
      mc = __funnelshift_l(__float_as_uint(__fsub_rn(__uint_as_float(v[4 * j4 + 3]), y.w)), mc, 1);
      mc = __funnelshift_l(__float_as_uint(__fsub_rn(__uint_as_float(v[4 * j4 + 2]), y.z)), mc, 1);
      mc = __funnelshift_l(__float_as_uint(__fsub_rn(__uint_as_float(v[4 * j4 + 1]), y.y)), mc, 1);
      mc = __funnelshift_l(__float_as_uint(__fsub_rn(__uint_as_float(v[4 * j4 + 0]), y.x)), mc, 1);
    }
    uint32_t msk = (m[0] | (m[1] << 8) | (m[2] << 16) | (m[3] << 24)) & CM[gi] & rm;
    const uint32_t has = __ballot_sync(0xffffffffu, msk != 0u);
    if (has == 0u) continue;
    const uint32_t cnt = __popc(msk);
    uint32_t excl, total;
    if (__all_sync(0xffffffffu, cnt <= 1u)) {
      excl = __popc(has & ((1u << lane) - 1u));
      total = __popc(has);
    } else {
      uint32_t incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      excl = incl - cnt;
      total = __shfl_sync(0xffffffffu, incl, 31);
    }
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(s_count, total);
    uint32_t pos = __shfl_sync(0xffffffffu, base, 0) + excl;
    while (msk) {
      const uint32_t j = (uint32_t)__ffs(msk) - 1u;
      msk &= msk - 1u;
      if ((int64_t)pos < a.seg_cap) {
        const int64_t slot = (int64_t)blockIdx.x * a.seg_cap + pos;
        Cand cd;
        cd.p = (int32_t)row;
        cd.g = (int32_t)(g0 + gi * 32 + (int)j);
        a.cand[slot] = cd;
        a.cand_e[slot] = pick32(v, j);
      }
      ++pos;
    }
  }
}

enum : int { kErrProducer = 1, kErrMma = 2, kErrEpilogue = 4, kErrDrain = 8 };

// TF32 operands streamed for both A and B (modes 1 and 2).  K-steps that lie
// wholly in the zero padding beyond the 2K real columns are skipped.
template <int NH>
__global__ void __launch_bounds__(kThreads, 1)
    dist_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a) {
  const int twoK = 2 * a.K;
  using C = Cfg<NH>;
  constexpr int S = C::kStages;
  extern __shared__ uint8_t smem_raw[];
  // 128-byte swizzle atoms repeat every 1024 bytes of shared-space address
  uint8_t* smem = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = (uint64_t*)(smem + C::kTileBytes);
  uint64_t* empty = full + S;
  uint64_t* tfull = empty + S;
  uint64_t* tempty = tfull + 2;
  uint64_t* drain = tempty + 2;
  uint32_t* tslot = (uint32_t*)(drain + 1);
  uint32_t* s_count = tslot + 1;
  uint32_t* s_abort = tslot + 2;
  float* Ys = (float*)(smem + C::kTileBytes + 256);
  uint32_t* CM = (uint32_t*)(Ys + BN);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiThreads);
    }
    mbar_init(drain, 1);
    *s_count = 0;
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const int n_tiles = a.nM * a.nN;
  const uint32_t smem_base = su32(smem);

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer
      int stage = 0;
      uint32_t phase = 0;
      uint32_t issued = 0;       // bit s: stage s has a load in flight or consumed
      uint32_t issued_par = 0;   // bit s: parity of the last phase issued on full[s]
      bool ok = true;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        const int m = t / a.nN, n = t - (t / a.nN) * a.nN;
        for (int c = 0; c < a.n_chunks; ++c) {
          if (!mbar_wait(&empty[stage], phase ^ 1)) {
            atomicOr(a.err, kErrProducer);
            ok = false;
            break;
          }
          mbar_expect_tx(&full[stage], C::kStageBytes);
          const uint32_t st = smem_base + stage * C::kStageBytes;
#pragma unroll
          for (int h = 0; h < NH; ++h)
            tma_load(st + h * kABytes, &tmA, &full[stage], h * a.KA + c * BK, m * BM);
#pragma unroll
          for (int h = 0; h < NH; ++h)
            tma_load(st + NH * kABytes + h * kBBytes, &tmB, &full[stage], h * a.KA + c * BK, n * BN);
          issued |= 1u << stage;
          issued_par = (issued_par & ~(1u << stage)) | (phase << stage);
          if (++stage == S) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // loads still in flight land before the CTA leaves
      for (int s = 0; s < S; ++s)
        if ((issued >> s) & 1u)
          if (!mbar_wait(&full[s], (issued_par >> s) & 1u)) atomicOr(a.err, kErrDrain);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      int stage = 0;
      uint32_t phase = 0;
      int acc = 0;
      uint32_t acc_phase = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        if (!mbar_wait(&tempty[acc], acc_phase ^ 1)) {
          atomicOr(a.err, kErrMma);
          break;
        }
        tc_fence_after();
        const uint32_t d_tmem = tbase + (uint32_t)(acc * BN);
        for (int c = 0; c < a.n_chunks; ++c) {
          if (!mbar_wait(&full[stage], phase)) {
            atomicOr(a.err, kErrMma);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t st = smem_base + stage * C::kStageBytes;
          const uint64_t a0 = sw128_desc(st), b0 = sw128_desc(st + NH * kABytes);
#pragma unroll
          for (int kk = 0; kk < BK / 8; ++kk) {
            if (c * BK + kk * 8 >= twoK) break;  // zero padding: nothing to add
            const uint64_t adv = (uint64_t)(kk * 32) >> 4;  // 8 TF32 = 32 bytes along K
            mma_tf32(d_tmem, a0 + adv, b0 + adv, (c | kk) != 0);
            if (NH == 2) {
              const uint64_t a1 = sw128_desc(st + kABytes), b1 = sw128_desc(st + NH * kABytes + kBBytes);
              mma_tf32(d_tmem, a0 + adv, b1 + adv, 1u);  // hi x lo
              mma_tf32(d_tmem, a1 + adv, b0 + adv, 1u);  // lo x hi
            }
          }
          mma_commit(&empty[stage]);  // stage reusable once these MMAs have read it
          if (++stage == S) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (!ok) break;
        mma_commit(&tfull[acc]);
        if (++acc == 2) {
          acc = 0;
          acc_phase ^= 1;
        }
      }
      mma_commit(drain);
      if (!mbar_wait(drain, 0)) atomicOr(a.err, kErrDrain);
    }
  } else {
    // ---------------- epilogue: warps 2.. ; TMEM lane quarter = warp % 4,
    // kEpiGroups 32-column groups from column 32 kEpiGroups part
    const int et = threadIdx.x - 64;
    const int q = warp & 3;
    const int part = (warp - 2) >> 2;
    int acc = 0;
    uint32_t acc_phase = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
      const int m = t / a.nN, n = t - (t / a.nN) * a.nN;
      const int64_t row = (int64_t)m * BM + q * 32 + lane;
      const uint32_t rm = (row < a.P && !a.rowbad[row]) ? 0xffffffffu : 0u;
      epi_bar();  // readers of the previous tile's Y are done
      epi_fill(et, (int64_t)n * BN, a, Ys, CM);
      const bool got = mbar_wait(&tfull[acc], acc_phase);
      if (!got) atomicOr(s_abort, 1u);
      epi_bar();
      if (*(volatile uint32_t*)s_abort) {
        atomicOr(a.err, kErrEpilogue);
        break;
      }
      tc_fence_after();
      const int col0 = part * kEpiGroups * 32;
      epi_warp<kEpiGroups>(tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + col0), Ys + col0,
                           CM + col0 / 32, row, rm, (int64_t)n * BN + col0, s_count, a, lane);
      tc_fence_before();
      mbar_arrive(&tempty[acc]);
      if (++acc == 2) {
        acc = 0;
        acc_phase ^= 1;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTmemCols));
  if (threadIdx.x == 0) a.seg_count[blockIdx.x] = *s_count;
}

// ---------------------------------------------------------------------------
// Candidate pass with the gene operand resident in shared memory: TF32 one
// term (mode 1) or BF16 hi/lo three terms (mode 3, BF3).
//
// A 128 x 256 tile of the streaming kernel above loads particle and gene rows
// for every tile (240 KB at depth 160 in one-term mode, 480 KB in three-term
// mode) through L2, which makes L2-to-SM bandwidth the limit.  Here each CTA
// keeps the gene rows of one 256-gene tile (n_chunks x 32 KB) in shared memory
// for all of its particle tiles and streams only the particle rows through a
// ring of 16 KB stages.  Work: nN gene tiles x cpt = max(1, grid / nN)
// particle-tile sequences (m = j, j + cpt, ...), handed to the CTAs
// round-robin; the CTAs that hold different gene tiles walk the same particle
// sequence in the same order, so each particle tile comes from DRAM about once
// and from L2 after that.  Roles, barriers, bounded waits and the epilogue are
// those of dist_tc_kernel; two more barriers (bfull, bempty) order the
// gene-row loads of successive assignments against the MMAs that read them.
//
// BF3 rows hold hi at [0, 2K) and lo at [H, H + 2K) with H a multiple of 16
// (one BF16 K-step), so K-step s < H/16 of a particle row is a hi step, paired
// with gene K-steps s (hi x hi) and s + H/16 (hi x lo), and K-step
// H/16 <= s < 2H/16 a lo step, paired with gene K-step s - H/16 (lo x hi):
// the whole gene row is resident, so any gene K-step is at hand.
// ---------------------------------------------------------------------------
constexpr int kResMaxStages = 4;
constexpr uint32_t kResSmemMax = 227u * 1024u;  // dynamic shared memory of one CTA

__host__ __device__ constexpr uint32_t res_smem(int n_chunks, int stages) {
  return 1024u + (uint32_t)n_chunks * kBBytes + (uint32_t)stages * kABytes + 256u + BN * 4u + BN / 8u;
}

template <bool BF3>
__global__ void __launch_bounds__(kThreads, 1)
    dist_tc_res_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a,
                       int S) {
  constexpr int kEl = BF3 ? 64 : 32;  // values per 128-byte chunk
  constexpr int kStepEl = kEl / 4;    // values per K-step (32 bytes)
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
  const int NC = a.n_chunks;
  uint8_t* ring = smem + (uint32_t)NC * kBBytes;
  uint64_t* full = (uint64_t*)(ring + (uint32_t)S * kABytes);
  uint64_t* empty = full + kResMaxStages;
  uint64_t* tfull = empty + kResMaxStages;
  uint64_t* tempty = tfull + 2;
  uint64_t* bfull = tempty + 2;
  uint64_t* bempty = bfull + 1;
  uint64_t* drain = bempty + 1;
  uint32_t* tslot = (uint32_t*)(drain + 1);
  uint32_t* s_count = tslot + 1;
  uint32_t* s_abort = tslot + 2;
  float* Ys = (float*)((uint8_t*)full + 256);
  uint32_t* CM = (uint32_t*)(Ys + BN);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int st = 0; st < S; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiThreads);
    }
    mbar_init(bfull, 1);
    mbar_init(bempty, 1);
    mbar_init(drain, 1);
    *s_count = 0;
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t b_base = su32(smem), ring_base = su32(ring);
  const int cpt = max(1, (int)gridDim.x / a.nN);
  const int n_assign = a.nN * cpt;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer: gene rows once per assignment, particle rows per tile
      int stage = 0;
      uint32_t phase = 0, issued = 0, issued_par = 0;
      bool ok = true;
      uint32_t b_issued = 0;  // gene-row loads issued (one per assignment)
      for (int as = blockIdx.x; as < n_assign && ok; as += gridDim.x) {
        const int n = as % a.nN, j = as / a.nN;
        if (b_issued > 0 && !mbar_wait(bempty, (b_issued - 1) & 1u)) {  // the previous gene rows are no longer read
          atomicOr(a.err, kErrProducer);
          break;
        }
        mbar_expect_tx(bfull, (uint32_t)NC * kBBytes);
        for (int c = 0; c < NC; ++c) tma_load(b_base + (uint32_t)c * kBBytes, &tmB, bfull, c * kEl, n * BN);
        ++b_issued;
        for (int m = j; m < a.nM && ok; m += cpt) {
          for (int c = 0; c < NC; ++c) {
            if (!mbar_wait(&empty[stage], phase ^ 1)) {
              atomicOr(a.err, kErrProducer);
              ok = false;
              break;
            }
            mbar_expect_tx(&full[stage], kABytes);
            tma_load(ring_base + (uint32_t)stage * kABytes, &tmA, &full[stage], c * kEl, m * BM);
            issued |= 1u << stage;
            issued_par = (issued_par & ~(1u << stage)) | (phase << stage);
            if (++stage == S) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      // loads still in flight land before the CTA leaves
      for (int st = 0; st < S; ++st)
        if ((issued >> st) & 1u)
          if (!mbar_wait(&full[st], (issued_par >> st) & 1u)) atomicOr(a.err, kErrDrain);
      if (b_issued > 0 && !mbar_wait(bfull, (b_issued - 1) & 1u)) atomicOr(a.err, kErrDrain);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      int stage = 0;
      uint32_t phase = 0;
      int acc = 0;
      uint32_t acc_phase = 0;
      bool ok = true;
      uint32_t k_as = 0;
      const int hs = a.KA / kStepEl;                    // K-steps per half (BF3)
      const int n_steps = BF3 ? 2 * hs : (2 * a.K + kStepEl - 1) / kStepEl;  // K-steps holding real values
      // descriptors by offset: chunk c of the gene rows and stage s of the ring are kBBytes / kABytes
      // apart, K-step kk of a chunk 32 bytes in (the start-address field counts 16-byte units)
      const uint64_t bd0 = sw128_desc(b_base), ad0 = sw128_desc(ring_base);
      for (int as = blockIdx.x; as < n_assign && ok; as += gridDim.x, ++k_as) {
        const int j = as / a.nN;
        if (!mbar_wait(bfull, k_as & 1u)) {
          atomicOr(a.err, kErrMma);
          break;
        }
        for (int m = j; m < a.nM && ok; m += cpt) {
          if (!mbar_wait(&tempty[acc], acc_phase ^ 1)) {
            atomicOr(a.err, kErrMma);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d_tmem = tbase + (uint32_t)(acc * BN);
          for (int c = 0; c < NC; ++c) {
            if (!mbar_wait(&full[stage], phase)) {
              atomicOr(a.err, kErrMma);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t a0 = ad0 + (uint64_t)(stage * (int)(kABytes >> 4));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const int st_a = c * 4 + kk;  // K-step of the particle row
              if (st_a >= n_steps) break;   // zero padding: nothing to add
              const uint64_t adv = (uint64_t)(kk * 2);  // 32 bytes along K
              if (BF3) {
                // gene K-step t: resident chunk t / 4, 32 (t % 4) bytes in
                const int t0 = st_a < hs ? st_a : st_a - hs;
                mma_bf16(d_tmem, a0 + adv, bd0 + (uint64_t)(((t0 >> 2) << 11) + ((t0 & 3) << 1)),
                         st_a != 0);  // hi x hi, or lo x hi
                if (st_a < hs) {
                  const int t1 = st_a + hs;
                  mma_bf16(d_tmem, a0 + adv, bd0 + (uint64_t)(((t1 >> 2) << 11) + ((t1 & 3) << 1)), 1u);  // hi x lo
                }
              } else {
                mma_tf32(d_tmem, a0 + adv, bd0 + (uint64_t)((c << 11) + kk * 2), st_a != 0);
              }
            }
            mma_commit(&empty[stage]);
            if (++stage == S) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          mma_commit(&tfull[acc]);
          if (++acc == 2) {
            acc = 0;
            acc_phase ^= 1;
          }
        }
        mma_commit(bempty);  // the gene rows may be replaced once these MMAs are done
      }
      mma_commit(drain);
      if (!mbar_wait(drain, 0)) atomicOr(a.err, kErrDrain);
    }
  } else {
    // ---------------- epilogue (as in dist_tc_kernel)
    const int et = threadIdx.x - 64;
    const int q = warp & 3;
    const int part = (warp - 2) >> 2;
    int acc = 0;
    uint32_t acc_phase = 0;
    bool stop = false;
    for (int as = blockIdx.x; as < n_assign && !stop; as += gridDim.x) {
      const int n = as % a.nN, j = as / a.nN;
      for (int m = j; m < a.nM; m += cpt) {
        const int64_t row = (int64_t)m * BM + q * 32 + lane;
        const uint32_t rm = (row < a.P && !a.rowbad[row]) ? 0xffffffffu : 0u;
        epi_bar();  // readers of the previous tile's Y are done
        epi_fill(et, (int64_t)n * BN, a, Ys, CM);
        const bool got = mbar_wait(&tfull[acc], acc_phase);
        if (!got) atomicOr(s_abort, 1u);
        epi_bar();
        if (*(volatile uint32_t*)s_abort) {
          atomicOr(a.err, kErrEpilogue);
          stop = true;
          break;
        }
        tc_fence_after();
        const int col0 = part * kEpiGroups * 32;
        epi_warp<kEpiGroups>(tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + col0), Ys + col0,
                             CM + col0 / 32, row, rm, (int64_t)n * BN + col0, s_count, a, lane);
        tc_fence_before();
        mbar_arrive(&tempty[acc]);
        if (++acc == 2) {
          acc = 0;
          acc_phase ^= 1;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTmemCols));
  if (threadIdx.x == 0) a.seg_count[blockIdx.x] = *s_count;
}

// ---------------------------------------------------------------------------
// operand preparation
// ---------------------------------------------------------------------------

// FP32 -> TF32 with round-to-nearest (ties away from zero on the magnitude),
// NaN and infinities passed through.
__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7F800000u) == 0x7F800000u) return x;
  u = (u + 0x1000u) & 0xFFFFE000u;
  return __uint_as_float(u);
}

// hi/lo TF32 parts of an FP64 value: hi = tf32(x), lo = tf32(x - hi)
__device__ __forceinline__ void split_tf32(double x, float& hi, float& lo) {
  hi = tf32_rn((float)x);
  const double r = x - (double)hi;
  lo = (hi == hi && fabs(hi) < INFINITY) ? tf32_rn((float)r) : 0.0f;
}



// flags[0]: bit 0 = an operand is infinite in FP32; flags[1] / flags[2] = the
// largest w and the largest s^2 (FP32 bit patterns of non-negative values,
// ordered like unsigned integers), so the host can check that no w s^2 product
// leaves the FP32 range.
__device__ __forceinline__ void note_max(unsigned* slot, float v) {
  if (v == v) atomicMax(slot, __float_as_uint(fabsf(v)));
}

// hi/lo TF32 parts of an FP32 value: hi = tf32(x), lo = tf32(x - hi) (x - hi is exact)
__device__ __forceinline__ void split_tf32f(float x, float& hi, float& lo) {
  hi = tf32_rn(x);
  lo = fabsf(hi) < INFINITY ? tf32_rn(x - hi) : 0.0f;
}

// hi/lo BF16 parts (as the FP32 values they represent exactly)
__device__ __forceinline__ float bf16_rn(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ void split_bf16(double x, float& hi, float& lo) {
  hi = bf16_rn((float)x);
  const double r = x - (double)hi;
  lo = (hi == hi && fabs(hi) < INFINITY) ? bf16_rn((float)r) : 0.0f;
}
__device__ __forceinline__ void split_bf16f(float x, float& hi, float& lo) {
  hi = bf16_rn(x);
  lo = (hi == hi && fabsf(hi) < INFINITY) ? bf16_rn(x - hi) : 0.0f;  // x - hi is exact in FP32
}

// operand element i of the pass's type: TF32 values as FP32, or BF16
template <bool BF>
__device__ __forceinline__ void put_op(void* base, int64_t i, float v) {
  if (BF)
    ((__nv_bfloat16*)base)[i] = __float2bfloat16_rn(v);  // v is a BF16 value: exact
  else
    ((float*)base)[i] = v;
}
template <bool BF>
__device__ __forceinline__ void split_opf(float x, float& hi, float& lo) {
  if (BF)
    split_bf16f(x, hi, lo);
  else
    split_tf32f(x, hi, lo);
}

// A rows: [s (K) | s^2 (K) | 0 ...] per half, in FP32 (s rounded once from FP64,
// s^2 = fl(s s): both within 2^-23 relative, inside the bound's rounding terms).
// One warp per row, rows strided over the grid; the overflow monitors are
// reduced per warp before one atomic each.
// One warp per batch of R consecutive rows (R x K <= 32 kPrepLoads values): all
// of the batch's loads are issued before any conversion, so each warp keeps
// up to kPrepLoads 256-byte requests in flight (HBM needs that many bytes in
// flight per SM to stream at full rate).
constexpr int kPrepLoads = 16;

template <bool BF>
__global__ void tc_prep_rows_kernel(const double* stats, int64_t P, int K, int H, int ld_, int NH, void* A,
                                    uint8_t* rowbad, unsigned* flags) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t ld = ld_;
  const int R = K <= 32 * kPrepLoads ? (32 * kPrepLoads) / K < 4 ? (32 * kPrepLoads) / K : 4 : 1;
  unsigned inf = 0, mx = 0;
  // pairs of statistics per lane: BF16, K even (rows and the lo / s^2 offsets
  // stay 4-byte aligned in A), and 16-byte aligned statistics rows
  const bool pairs = BF && (K & 1) == 0 && ((reinterpret_cast<uintptr_t>(stats) & 15) == 0);
  for (int64_t p0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * R; p0 < P; p0 += warps * R) {
    const int rows = P - p0 < R ? (int)(P - p0) : R;
    uint32_t nanr = 0;  // bit r: row p0 + r holds a NaN statistic
    if (K > 32 * kPrepLoads) {  // very wide rows: one row at a time
      const double* srow = stats + p0 * K;
      const int64_t arow = p0 * ld;
      for (int k = lane; k < K; k += 32) {
        const float sv = rn32_bits(srow[k]);
        const float s2 = sv * sv;
        float h1, l1, h2, l2;
        split_opf<BF>(sv, h1, l1);
        split_opf<BF>(s2, h2, l2);
        put_op<BF>(A, arow + k, h1);
        put_op<BF>(A, arow + K + k, h2);
        if (NH == 2) {
          put_op<BF>(A, arow + H + k, l1);
          put_op<BF>(A, arow + H + K + k, l2);
        }
        if (fabsf(sv) == INFINITY || fabsf(s2) == INFINITY) inf = 1u;
        if (s2 == s2) mx = max(mx, __float_as_uint(s2));
        if (sv != sv) nanr = 1u;
      }
    } else if (BF && pairs) {
      // BF16 with K even and 16-byte aligned rows: a lane takes two adjacent
      // statistics of one row (flat index f = 2 (lane + 32 t)) with one 16-byte
      // load and stores each operand pair as one 4-byte bf16x2
      const int n = rows * K;
      double2 v[kPrepLoads / 2];
      {
        const double2* src = reinterpret_cast<const double2*>(stats + p0 * K);
#pragma unroll
        for (int t = 0; t < kPrepLoads / 2; ++t) {
          const int f = 2 * (lane + 32 * t);
          v[t] = f < n ? __ldg(src + (f >> 1)) : make_double2(0.0, 0.0);
        }
      }
      int r = (2 * lane) / K, k = 2 * lane - ((2 * lane) / K) * K;
#pragma unroll
      for (int t = 0; t < kPrepLoads / 2; ++t) {
        if (2 * (lane + 32 * t) < n) {
          const float s0 = rn32_bits(v[t].x), s1 = rn32_bits(v[t].y);
          const float q0 = s0 * s0, q1 = s1 * s1;
          float h1a, l1a, h2a, l2a, h1b, l1b, h2b, l2b;
          split_bf16f(s0, h1a, l1a);
          split_bf16f(q0, h2a, l2a);
          split_bf16f(s1, h1b, l1b);
          split_bf16f(q1, h2b, l2b);
          __nv_bfloat162* row = reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<__nv_bfloat16*>(A) + (p0 + r) * ld);
          row[k >> 1] = __floats2bfloat162_rn(h1a, h1b);  // the values are BF16: exact
          row[(K + k) >> 1] = __floats2bfloat162_rn(h2a, h2b);
          if (NH == 2) {
            row[(H + k) >> 1] = __floats2bfloat162_rn(l1a, l1b);
            row[(H + K + k) >> 1] = __floats2bfloat162_rn(l2a, l2b);
          }
          if (fabsf(s0) == INFINITY || fabsf(q0) == INFINITY || fabsf(s1) == INFINITY || fabsf(q1) == INFINITY)
            inf = 1u;
          if (q0 == q0) mx = max(mx, __float_as_uint(q0));
          if (q1 == q1) mx = max(mx, __float_as_uint(q1));
          if (s0 != s0 || s1 != s1) nanr |= 1u << r;
        }
        k += 64;
        while (k >= K) {
          k -= K;
          ++r;
        }
      }
    } else {
      // flat index f = lane + 32 t over rows x K, (r, k) = divmod(f, K)
      const int n = rows * K;
      double v[kPrepLoads];
      {
        const double* src = stats + p0 * K;  // rows are contiguous
#pragma unroll
        for (int t = 0; t < kPrepLoads; ++t) {
          const int f = lane + 32 * t;
          v[t] = f < n ? __ldg(src + f) : 0.0;
        }
      }
      int r = lane / K, k = lane - (lane / K) * K;
#pragma unroll
      for (int t = 0; t < kPrepLoads; ++t) {
        if (lane + 32 * t < n) {
          const float sv = rn32_bits(v[t]);
          const float s2 = sv * sv;
          float h1, l1, h2, l2;
          split_opf<BF>(sv, h1, l1);
          split_opf<BF>(s2, h2, l2);
          const int64_t arow = (p0 + r) * ld;
          put_op<BF>(A, arow + k, h1);
          put_op<BF>(A, arow + K + k, h2);
          if (NH == 2) {
            put_op<BF>(A, arow + H + k, l1);
            put_op<BF>(A, arow + H + K + k, l2);
          }
          if (fabsf(sv) == INFINITY || fabsf(s2) == INFINITY) inf = 1u;
          if (s2 == s2) mx = max(mx, __float_as_uint(s2));
          if (sv != sv) nanr |= 1u << r;
        }
        k += 32;
        while (k >= K) {
          k -= K;
          ++r;
        }
      }
    }
    nanr = __reduce_or_sync(0xffffffffu, nanr);
    if (lane < rows) rowbad[p0 + lane] = (uint8_t)((nanr >> lane) & 1u);
    for (int rr = 0; rr < rows; ++rr) {
      const int64_t arow = (p0 + rr) * ld;
      for (int k = 2 * K + lane; k < H; k += 32) {
        put_op<BF>(A, arow + k, 0.0f);
        if (NH == 2) put_op<BF>(A, arow + H + k, 0.0f);
      }
      for (int k = NH * H + lane; k < ld_; k += 32) put_op<BF>(A, arow + k, 0.0f);
    }
  }
  inf = __reduce_or_sync(0xffffffffu, inf);
  mx = __reduce_max_sync(0xffffffffu, mx);
  if (lane == 0) {
    if (inf) atomicOr(&flags[0], 1u);
    if (mx) atomicMax(&flags[2], mx);
  }
}

// B rows: [-2 w d (K) | w (K) | 0 ...] per half; c_g = sum_k w d^2 in FP64; the
// per-gene term of the error bound b0_g = 5 beta c_g / K.
template <bool BF>
__global__ void tc_prep_genes_kernel(const double* data, const double* se, int64_t G, int K, int H, int ld_, int NH,
                                     double beta, void* B, double* cg64, float* cg32, float* b0, unsigned* flags) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const int64_t ld = ld_;
  const double sig2 = 0.1 * 0.1;
  double c = 0.0;
  bool bad = false;
  for (int k = NH * H; k < ld_; ++k) put_op<BF>(B, g * ld + k, 0.0f);
  for (int k = 0; k < H; ++k) {
    double v = 0.0;
    if (k < 2 * K) {
      const int kk = k < K ? k : k - K;
      const double d = data[g * K + kk], e = se[g * K + kk];
      const double eps = (e + d != 0.0) ? 0.0 : 0.0001;
      const double w = 1.0 / ((e * e + sig2 * (d * d)) + eps);
      v = k < K ? -2.0 * w * d : w;
      if (fabsf((float)v) == INFINITY) bad = true;
      if (k >= K) note_max(&flags[1], (float)w);
      else c += w * d * d;
    }
    float hi, lo;
    if (BF)
      split_bf16(v, hi, lo);
    else
      split_tf32(v, hi, lo);
    put_op<BF>(B, g * ld + k, hi);
    if (NH == 2) put_op<BF>(B, g * ld + H + k, lo);
  }
  if (bad) atomicOr(&flags[0], 1u);
  cg64[g] = c;
  cg32[g] = (float)c;
  b0[g] = (float)(5.0 * beta * c / (double)K);
}

// Y_g = K X_g - c_g rounded up; X < 0 accepts no pair.  Errors are clipped at
// 10 (scripts/compute_errors.jl:62-64), so X >= 10 accepts every finite pair,
// however large its unclipped error.
__global__ void tc_y_kernel(const float* X, const double* cg64, int64_t G, int K, float* Y) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const float x = X[g];
  float y;
  if (x != x) y = x;
  else if (x >= 10.0f) y = INFINITY;
  else if (x < 0.0f) y = -INFINITY;
  else y = __double2float_ru((double)x * (double)K - cg64[g]);
  Y[g] = y;
}

// Concatenate the per-CTA segments: out[off_b + i] = seg_b[i], segment b in
// blockIdx.y, its entries spread over the gridDim.x blocks of that row.
__global__ void tc_gather_kernel(const Cand* seg, const float* seg_e, const unsigned* count, int n_seg,
                                 int64_t seg_cap, const float* cg, float invK, Cand* out, float* out_e) {
  __shared__ int64_t off;
  const int b = blockIdx.y;
  if (threadIdx.x < 32) {  // off_b = sum of the earlier segments' counts, one warp
    unsigned long long o = 0;
    for (int i = threadIdx.x; i < b; i += 32) o += count[i];
    for (int d = 16; d > 0; d >>= 1) o += __shfl_xor_sync(0xffffffffu, o, d);
    if (threadIdx.x == 0) off = (int64_t)o;
  }
  __syncthreads();
  const int64_t n = count[b];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const Cand cd = seg[(int64_t)b * seg_cap + i];
    out[off + i] = cd;
    out_e[off + i] = fminf((seg_e[(int64_t)b * seg_cap + i] + cg[cd.g]) * invK, 10.0f);
  }
}

// rows x cols row-major operand, 128-byte swizzled boxes of box_rows x (one
// 128-byte row: 32 FP32 / TF32 values, or 64 BF16 values when bf16)
bool make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int box_rows, bool bf16 = false) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  memset(map, 0, sizeof(*map));
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const int es = bf16 ? 2 : 4;
  cuuint64_t strides[1] = {(cuuint64_t)cols * es};
  cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return encode(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base,
                dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NH>
cudaError_t launch_nh(const void* A, const void* B, const TcArgs& args, int grid, cudaStream_t s) {
  static std::atomic<uint64_t> attr{0};  // devices where the limit is set, shared by all contexts
  cudaError_t e = set_smem_once(attr, dist_tc_kernel<NH>, (int)Cfg<NH>::kSmem);
  if (e != cudaSuccess) return e;
  CUtensorMap ma, mb;
  const int64_t ld = (int64_t)NH * args.KA;
  if (!make_map(&ma, A, args.P, ld, BM) || !make_map(&mb, B, args.G, ld, BN)) return cudaErrorInvalidValue;
  dist_tc_kernel<NH><<<grid, kThreads, Cfg<NH>::kSmem, s>>>(ma, mb, args);
  return cudaGetLastError();
}

constexpr int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

TcLayout tc_layout(int K, int mode) {
  TcLayout L;
  if (mode == 3) {
    L.H = round_up(2 * K, 16);
    L.ld = round_up(2 * L.H, 64);
    L.n_chunks = L.ld / 64;
    L.es = 2;
  } else {
    L.H = round_up(2 * K, BK);
    L.ld = mode == 1 ? L.H : 2 * L.H;
    L.n_chunks = L.H / BK;
    L.es = 4;
  }
  return L;
}

double tc_beta(int K, int nh) {
  // |K e32 - K e| <= beta * sum_k |term_k| with sum_k |term_k| <= 5 c_g + 4 K e:
  //   one term: products of two round-to-nearest TF32 values, relative error
  //     (1 + 2^-11)^2 - 1 (plus 2^-24 from the FP64 -> FP32 step), exact FP32 products,
  //     2K accumulations at <= 2^-23 each (truncating adder);
  //   three terms: representation error of hi + lo <= 2^-21 per operand, the
  //     dropped lo*lo <= 2^-22, 6K accumulations.
  // Plus the final FP32 rounding of Y / e, with a 10 % safety factor.
  //   BF16 three terms (nh = 3): hi = RN_bf16(x), lo = RN_bf16(x - hi) leave
  //     |x - hi - lo| <= 2^-9 |x - hi| <= 2^-18 |x|, plus <= 2^-22 from the
  //     FP64 -> FP32 steps, per operand; the dropped lo*lo <= 2^-18; BF16 x BF16
  //     products are exact in FP32; 6K accumulations.
  const double u23 = 1.1920928955078125e-07;
  double b;
  if (nh == 1)
    b = (std::pow(1.0 + 4.8828125e-04 + 5.960464477539063e-08, 2) - 1.0) + (2.0 * K + 4) * u23;
  else if (nh == 3)
    b = 2.0 * (3.814697265625e-06 + 2.384185791015625e-07) + 3.814697265625e-06 + (6.0 * K + 4) * u23;
  else
    b = 2.0 * 4.76837158203125e-07 + 2.384185791015625e-07 + (6.0 * K + 4) * u23;
  return 1.1 * b;
}

cudaError_t launch_tc_prep(const DistInputs& in, int mode, double beta, void* A, void* B, uint8_t* rowbad,
                           double* cg64, float* cg32, float* b0, unsigned* flags, cudaStream_t s) {
  const TcLayout L = tc_layout(in.K, mode);
  const int NH = mode == 1 ? 1 : 2;
  const bool bf = mode == 3;
  if (in.P > 0) {
    const int64_t blocks = (in.P + 31) / 32 < 8192 ? (in.P + 31) / 32 : 8192;
    if (bf)
      tc_prep_rows_kernel<true><<<(unsigned)blocks, 256, 0, s>>>(in.stats, in.P, in.K, L.H, L.ld, NH, A, rowbad,
                                                                 flags);
    else
      tc_prep_rows_kernel<false><<<(unsigned)blocks, 256, 0, s>>>(in.stats, in.P, in.K, L.H, L.ld, NH, A, rowbad,
                                                                  flags);
  }
  if (in.G > 0) {
    const unsigned gb = (unsigned)((in.G + 127) / 128);
    if (bf)
      tc_prep_genes_kernel<true><<<gb, 128, 0, s>>>(in.data, in.se, in.G, in.K, L.H, L.ld, NH, beta, B, cg64, cg32,
                                                    b0, flags);
    else
      tc_prep_genes_kernel<false><<<gb, 128, 0, s>>>(in.data, in.se, in.G, in.K, L.H, L.ld, NH, beta, B, cg64, cg32,
                                                     b0, flags);
  }
  return cudaGetLastError();
}

cudaError_t launch_tc_y(const float* X, const double* cg64, int64_t G, int K, float* Y, cudaStream_t s) {
  if (G <= 0) return cudaSuccess;
  tc_y_kernel<<<(unsigned)((G + 255) / 256), 256, 0, s>>>(X, cg64, G, K, Y);
  return cudaGetLastError();
}

int tc_grid(int64_t P, int64_t G, int sms) {
  const int64_t tiles = ((P + BM - 1) / BM) * ((G + BN - 1) / BN);
  return (int)(tiles < sms ? tiles : sms);
}

template <bool BF3>
static cudaError_t launch_res(const void* A, const void* B, const TcArgs& args, int grid, int stages,
                              cudaStream_t s) {
  const uint32_t smem = res_smem(args.n_chunks, stages);
  static std::atomic<uint64_t> attr{0};
  // the largest configuration sets the limit once per device; smaller ones fit under it
  cudaError_t e = set_smem_once(attr, dist_tc_res_kernel<BF3>, (int)kResSmemMax);
  if (e != cudaSuccess) return e;
  CUtensorMap ma, mb;
  const int64_t ld = (int64_t)args.n_chunks * (BF3 ? 64 : 32);  // row length in values
  if (!make_map(&ma, A, args.P, ld, BM, BF3) || !make_map(&mb, B, args.G, ld, BN, BF3)) return cudaErrorInvalidValue;
  dist_tc_res_kernel<BF3><<<grid, kThreads, smem, s>>>(ma, mb, args, stages);
  return cudaGetLastError();
}

int tc_res_stages(int n_chunks) {
  for (int st = kResMaxStages; st >= 2; --st)
    if (res_smem(n_chunks, st) <= kResSmemMax) return st;
  return 0;
}

bool tc_mode3_fits(int K) { return tc_res_stages(tc_layout(K, 3).n_chunks) != 0; }

cudaError_t launch_dist_tc(int mode, const void* A, const void* B, const TcArgs& args, int grid, cudaStream_t s) {
  if (args.P <= 0 || args.G <= 0) return cudaSuccess;
  const int stages = mode == 2 ? 0 : tc_res_stages(args.n_chunks);
  if (mode == 3) return stages ? launch_res<true>(A, B, args, grid, stages, s) : cudaErrorInvalidValue;
  if (mode == 2) return launch_nh<2>(A, B, args, grid, s);
  return stages ? launch_res<false>(A, B, args, grid, stages, s) : launch_nh<1>(A, B, args, grid, s);
}

cudaError_t launch_tc_gather(const Cand* seg, const float* seg_e, const unsigned* count, int n_seg, int64_t seg_cap,
                             const float* cg, int K, Cand* out, float* out_e, cudaStream_t s) {
  if (n_seg <= 0) return cudaSuccess;
  tc_gather_kernel<<<dim3(32, (unsigned)n_seg), 256, 0, s>>>(seg, seg_e, count, n_seg, seg_cap, cg, 1.0f / (float)K,
                                                              out, out_e);
  return cudaGetLastError();
}

}  // namespace abc
