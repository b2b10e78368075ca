// mlp.cuh — the surrogate network: an ensemble of MLPs mapping normalised
// log-parameters to the means and log-variances of the summary statistics.
//
// Per member: IN_PAD -> H -> H -> H -> O_PAD, SiLU on the hidden layers,
// FP32 master weights with BF16 copies for the GEMMs (FP32 accumulation).
// Flat parameter layout per member (row-major, "x W" convention):
//   W1[IN_PAD][H] b1[H] W2[H][H] b2[H] W3[H][H] b3[H] W4[H][O_PAD] b4[O_PAD]
// Output columns: [0, K) means, [K, 2K) log-variances, the rest zero padding.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace abc {

constexpr int kMlpInPad = 16;
constexpr int kMlpHidden = 256;

struct MlpDims {
  int in_dim, K, in_pad, H, out_pad;
  int64_t off_w1, off_b1, off_w2, off_b2, off_w3, off_b3, off_w4, off_b4, n_params;
};

inline MlpDims mlp_dims(int in_dim, int K) {
  MlpDims d;
  d.in_dim = in_dim;
  d.K = K;
  d.in_pad = kMlpInPad;
  d.H = kMlpHidden;
  d.out_pad = ((2 * K + 15) / 16) * 16;
  int64_t o = 0;
  d.off_w1 = o; o += (int64_t)d.in_pad * d.H;
  d.off_b1 = o; o += d.H;
  d.off_w2 = o; o += (int64_t)d.H * d.H;
  d.off_b2 = o; o += d.H;
  d.off_w3 = o; o += (int64_t)d.H * d.H;
  d.off_b3 = o; o += d.H;
  d.off_w4 = o; o += (int64_t)d.H * d.out_pad;
  d.off_b4 = o; o += d.out_pad;
  d.n_params = o;
  return d;
}

// GEMM epilogues.
enum MlpEpi : int {
  EPI_HIDDEN = 0,    // z = C + bias -> Zf32 (optional), act = silu(z) -> bf16 out
  EPI_LINEAR = 1,    // C + bias -> fp32 out
  EPI_PARTIAL = 2,   // C into fp32 out + split * sSplit: one slice per reduction split (split-K over
                     // the batch), summed in split order afterwards, so the result does not depend on timing
  EPI_DSILU = 3      // bf16 out = C * silu'(Zprev)
};

// Tensor-core GEMM C[M][N] = sum_k A[m][k] B[n][k] (mlp_tc.cu): both operands
// K-major BF16 ([rows][ld], K contiguous; ld * 2 bytes a multiple of 16), one
// operand set per ensemble member.
struct TcOperand {
  const __nv_bfloat16* ptr;
  int64_t ld;             // elements between rows
  int64_t rows;           // M for A, N for B
  int64_t member_stride;  // elements between members
};

struct TcGemm {
  int M, N, K;
  int k_split;   // reduction split over blockIdx.y (EPI_PARTIAL)
  int a_shared;  // one A for every member
  const float* bias;
  int64_t sBias;
  const float* zprev;  // EPI_DSILU: pre-activation [M][ldz]
  int64_t sZ;
  int ldz;
  float* outf;         // EPI_HIDDEN (optional), EPI_LINEAR, EPI_PARTIAL: [M][ldf]
  int64_t sSplit;      // EPI_PARTIAL: stride between the slices of the reduction splits
  int64_t sOutf;
  int ldf;
  __nv_bfloat16* outh;   // EPI_HIDDEN, EPI_DSILU: [M][ldh]
  int64_t sOuth;
  int ldh;
  __nv_bfloat16* outhT;  // optional transposed copy [N][ldhT]
  int64_t sOuthT;
  int ldhT;
  int* err;              // nonzero: a bounded wait ran out
};

// reduction splits of the weight-gradient GEMMs for a batch of B rows, and
// blocks of the loss kernel (sizes of the partial-sum buffers)
inline int mlp_wgrad_splits(int B) { return B / 128 < 1 ? 1 : (B / 128 > 16 ? 16 : B / 128); }
inline int mlp_loss_blocks(int B, int out_pad) {
  const int n = (B * out_pad + 255) / 256;
  return n < 1024 ? n : 1024;
}

cudaError_t mlp_tc_gemm(int epi, const TcOperand& A, const TcOperand& B, const TcGemm& g, int members,
                        cudaStream_t s);

}  // namespace abc
