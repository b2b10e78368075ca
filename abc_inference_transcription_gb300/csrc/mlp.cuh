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

// C[M][N] = op(A) op(B) (+ bias), BF16 operands, FP32 accumulation.
// TA: A is stored K x M (use A^T); TB: B is stored N x K (use B^T).
// Epilogues.
enum MlpEpi : int {
  EPI_HIDDEN = 0,    // z = C + bias -> Zf32 (optional), act = silu(z) -> bf16 out
  EPI_LINEAR = 1,    // C + bias -> fp32 out
  EPI_ATOMIC = 2,    // atomicAdd C into fp32 out (split-K over the batch)
  EPI_DSILU = 3      // bf16 out = C * silu'(Zprev)
};

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  const float* bias;
  const float* zprev;   // EPI_DSILU: pre-activation of the layer
  float* outf;
  __nv_bfloat16* outh;
  int M, N, K;
  int lda, ldb, ldo;
  int64_t sA, sB, sBias, sZ, sOut;  // per-member strides (blockIdx.z)
  int k_split;                       // EPI_ATOMIC: K range per blockIdx.y slice... (split count)
};

}  // namespace abc
