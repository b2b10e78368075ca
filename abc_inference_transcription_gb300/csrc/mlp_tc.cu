// mlp_tc.cu — the surrogate's GEMMs on the tcgen05 tensor cores:
//   C[M][N] = sum_k A[m][k] B[n][k]   (both operands K-major, BF16, FP32
//   accumulation in tensor memory), one output tile of 128 x 128 per CTA,
//   ensemble member = blockIdx.z, optional split of the reduction
//   (blockIdx.y = m tile + split * m tiles) for the weight gradients.
// Warp 0 issues TMA loads (3D maps: reduction, rows, member; 64-wide BF16 boxes
// with the 128-byte swizzle) into a 3-stage ring; one lane of warp 1 issues
// tcgen05.mma.kind::f16 (M = N = 128, K = 16); all four warps then read their
// 32 accumulator rows with tcgen05.ld and apply the fused epilogue (bias +
// SiLU, bias, one partial sum per reduction split, or the SiLU derivative), writing the
// row-major result and, where the backward pass needs it, the transposed
// BF16 copy.  Waits are bounded (about one second); a wait that runs out sets
// the error word, and the CTA drains its copies and MMAs before it frees its
// tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>

#include "kernels.h"
#include "smem_attr.h"
#include "mlp.cuh"
#include "tcgen05.cuh"

namespace abc {
namespace {

using namespace tc;

constexpr int BM = 128, BN = 128, BK = 64;  // BK BF16 values = one 128-byte swizzled row
constexpr int kStages = 3;
constexpr uint32_t kTileBytes = BM * BK * 2;  // A and B tiles alike (BN = BM)
constexpr uint32_t kStageBytes = 2 * kTileBytes;
constexpr uint32_t kTmemCols = 128;
constexpr int kSmem = 1024 + kStages * kStageBytes + 128;

// D = F32, A = B = BF16, both K-major, M = 128, N = 128
constexpr uint32_t kIdescBf16 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdescBf16), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }

template <int EPI>
__global__ void __launch_bounds__(128, 1)
    mlp_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcGemm g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = (uint64_t*)(smem + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* done = empty + kStages;
  uint32_t* tslot = (uint32_t*)(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int z = blockIdx.z;
  const int n_mt = (g.M + BM - 1) / BM;
  const int mt = blockIdx.y % n_mt, split = blockIdx.y / n_mt;
  const int m0 = mt * BM, n0 = blockIdx.x * BN;
  const int nk = (g.K + BK - 1) / BK;
  const int per = (nk + g.k_split - 1) / g.k_split;
  const int c0 = split * per, c1 = min(nk, c0 + per);
  if (threadIdx.x == 0) {
    for (int st = 0; st < kStages; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t sbase = su32(smem);
  const bool work = c1 > c0;
  if (work && warp == 0 && lane == 0) {
    // ---- TMA producer
    int last_par[kStages] = {-1, -1, -1};
    for (int c = c0; c < c1; ++c) {
      const int i = c - c0, st = i % kStages;
      const uint32_t ph = (uint32_t)(i / kStages) & 1u;
      if (!mbar_wait(&empty[st], ph ^ 1u)) {
        atomicOr(g.err, 1);
        break;
      }
      mbar_expect_tx(&full[st], kStageBytes);
      const uint32_t sa = sbase + st * kStageBytes;
      tma_load3(sa, &tmA, &full[st], c * BK, m0, g.a_shared ? 0 : z);
      tma_load3(sa + kTileBytes, &tmB, &full[st], c * BK, n0, z);
      last_par[st] = (int)ph;
    }
    for (int st = 0; st < kStages; ++st)  // copies in flight land before the CTA leaves
      if (last_par[st] >= 0 && !mbar_wait(&full[st], (uint32_t)last_par[st])) atomicOr(g.err, 8);
  } else if (work && warp == 1 && lane == 0) {
    // ---- MMA issuer
    for (int c = c0; c < c1; ++c) {
      const int i = c - c0, st = i % kStages;
      const uint32_t ph = (uint32_t)(i / kStages) & 1u;
      if (!mbar_wait(&full[st], ph)) {
        atomicOr(g.err, 2);
        break;
      }
      tc_fence_after();
      const uint32_t sa = sbase + st * kStageBytes;
      const uint64_t da = sw128_desc(sa), db = sw128_desc(sa + kTileBytes);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;  // 16 BF16 = 32 bytes along K
        mma_bf16(tbase, da + adv, db + adv, (c > c0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&empty[st]);
    }
    mma_commit(done);  // arrives once every MMA above has completed
  }
  // ---- epilogue: warp w holds accumulator rows 32 w .. 32 w + 31
  bool have = work && mbar_wait(done, 0);
  have = __all_sync(0xffffffffu, have);
  if (work && !have && lane == 0) atomicOr(g.err, 4);
  tc_fence_after();
  const int m = m0 + warp * 32 + lane;
  const uint32_t lane_addr = tbase + ((uint32_t)(warp * 32) << 16);
  if (have) {
    const float* bias = g.bias ? g.bias + z * g.sBias : nullptr;
#pragma unroll 1
    for (int cc = 0; cc < BN / 32; ++cc) {
      __syncwarp();
      uint32_t v[32];
      tmem_ld32(lane_addr + (uint32_t)(cc * 32), v);
      if (m >= g.M) continue;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int n = n0 + cc * 32 + j;
        if (n >= g.N) continue;
        const float a = __uint_as_float(v[j]);
        if (EPI == EPI_HIDDEN) {
          const float zz = a + (bias ? bias[n] : 0.0f);
          if (g.outf) g.outf[z * g.sOutf + (int64_t)m * g.ldf + n] = zz;
          const __nv_bfloat16 h = __float2bfloat16(zz * sigm(zz));
          g.outh[z * g.sOuth + (int64_t)m * g.ldh + n] = h;
          if (g.outhT) g.outhT[z * g.sOuthT + (int64_t)n * g.ldhT + m] = h;
        } else if (EPI == EPI_LINEAR) {
          g.outf[z * g.sOutf + (int64_t)m * g.ldf + n] = a + (bias ? bias[n] : 0.0f);
        } else if (EPI == EPI_PARTIAL) {
          g.outf[split * g.sSplit + z * g.sOutf + (int64_t)m * g.ldf + n] = a;
        } else {
          const float zp = g.zprev[z * g.sZ + (int64_t)m * g.ldz + n];
          const float sg = sigm(zp);
          const __nv_bfloat16 d = __float2bfloat16(a * (sg * (1.0f + zp * (1.0f - sg))));
          g.outh[z * g.sOuth + (int64_t)m * g.ldh + n] = d;
          if (g.outhT) g.outhT[z * g.sOuthT + (int64_t)n * g.ldhT + m] = d;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTmemCols));
}

// 3D map over [members][rows][K] BF16 (K contiguous): box 64 x 128 x 1, 128-byte swizzle
bool make_map3(CUtensorMap* map, const __nv_bfloat16* base, int64_t K, int64_t ld, int64_t rows, int64_t members,
               int64_t member_stride) {
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
  const int64_t row_bytes = ld * 2;
  int64_t mstride = member_stride * 2;
  if (members <= 1) mstride = ((rows * row_bytes + 15) / 16) * 16;
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)(members < 1 ? 1 : members)};
  cuuint64_t strides[2] = {(cuuint64_t)row_bytes, (cuuint64_t)mstride};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)BM, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)base, dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int EPI>
cudaError_t launch_epi(const CUtensorMap& ma, const CUtensorMap& mb, const TcGemm& g, int members, cudaStream_t s) {
  static std::atomic<uint64_t> attr{0};  // devices where the limit is set, shared by all contexts
  cudaError_t e = set_smem_once(attr, mlp_tc_kernel<EPI>, kSmem);
  if (e != cudaSuccess) return e;
  const int n_mt = (g.M + BM - 1) / BM;
  dim3 grid((unsigned)((g.N + BN - 1) / BN), (unsigned)(n_mt * g.k_split), (unsigned)members);
  mlp_tc_kernel<EPI><<<grid, 128, kSmem, s>>>(ma, mb, g);
  return cudaGetLastError();
}

}  // namespace

cudaError_t mlp_tc_gemm(int epi, const TcOperand& A, const TcOperand& B, const TcGemm& g, int members,
                        cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
  if ((A.ld * 2) % 16 || (B.ld * 2) % 16 || (A.member_stride * 2) % 16 || (B.member_stride * 2) % 16)
    return cudaErrorInvalidValue;
  CUtensorMap ma, mb;
  if (!make_map3(&ma, A.ptr, g.K, A.ld, A.rows, g.a_shared ? 1 : members, A.member_stride) ||
      !make_map3(&mb, B.ptr, g.K, B.ld, B.rows, members, B.member_stride))
    return cudaErrorInvalidValue;
  switch (epi) {
    case EPI_HIDDEN: return launch_epi<EPI_HIDDEN>(ma, mb, g, members, s);
    case EPI_LINEAR: return launch_epi<EPI_LINEAR>(ma, mb, g, members, s);
    case EPI_PARTIAL: return launch_epi<EPI_PARTIAL>(ma, mb, g, members, s);
    default: return launch_epi<EPI_DSILU>(ma, mb, g, members, s);
  }
}

}  // namespace abc
