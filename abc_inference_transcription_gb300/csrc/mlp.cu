// mlp.cu — forward, backward and Adam of the surrogate ensemble.  Every GEMM
// runs on the tcgen05 tensor cores (mlp_tc.cu) with both operands K-major, so
// the passes keep transposed BF16 copies where the backward pass reduces over
// the batch: W^T for the forward GEMMs, and X0^T, A_l^T, dY^T, dZ_l^T
// ([features][batch]) for the weight gradients.  See mlp.cuh for the layout.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "mlp.cuh"

namespace abc {

// ---------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------
// Glorot-uniform weights, zero biases and zero padding; Philox stream ST_AUX,
// cell = parameter block, particle = member.
__global__ void mlp_init_kernel(MlpDims d, int members, uint64_t seed, float* P) {
  const int64_t n = d.n_params * members;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(i / d.n_params);
    const int64_t q = i - (int64_t)e * d.n_params;
    float bound = 0.0f;
    bool valid = false;
    if (q >= d.off_w1 && q < d.off_b1) {
      const int64_t r = (q - d.off_w1) / d.H;
      valid = r < d.in_dim;
      bound = sqrtf(6.0f / (float)(d.in_dim + d.H));
    } else if ((q >= d.off_w2 && q < d.off_b2) || (q >= d.off_w3 && q < d.off_b3)) {
      valid = true;
      bound = sqrtf(6.0f / (float)(2 * d.H));
    } else if (q >= d.off_w4 && q < d.off_b4) {
      const int64_t c = (q - d.off_w4) % d.out_pad;
      valid = c < 2 * d.K;
      bound = 0.5f * sqrtf(6.0f / (float)(d.H + 2 * d.K));
    }
    float v = 0.0f;
    if (valid) {
      U4 c;
      c.x = (uint32_t)(q >> 2);
      c.y = (ST_AUX << 30) | 0x1000000u;
      c.z = (uint32_t)e;
      c.w = 0x4d4c5021u;
      U4 o = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
      const uint32_t w = (q & 3) == 0 ? o.x : (q & 3) == 1 ? o.y : (q & 3) == 2 ? o.z : o.w;
      v = bound * (2.0f * ((float)(w >> 8) * 5.9604644775390625e-08f) - 1.0f);
    }
    P[i] = v;
  }
}

__global__ void mlp_to_bf16_kernel(const float* src, __nv_bfloat16* dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16(src[i]);
}

// BF16 transposed weights: W_l [R][C] at off_w -> W_l^T [C][R] at the same
// offset (biases copied), for the K-major forward GEMMs.
__global__ void mlp_weights_t_kernel(const float* P, MlpDims d, int members, __nv_bfloat16* PT) {
  const int64_t n = d.n_params * members;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / d.n_params, q = i - e * d.n_params;
    int64_t off = -1, R = 0, Cc = 0;
    if (q >= d.off_w1 && q < d.off_b1) { off = d.off_w1; R = d.in_pad; Cc = d.H; }
    else if (q >= d.off_w2 && q < d.off_b2) { off = d.off_w2; R = d.H; Cc = d.H; }
    else if (q >= d.off_w3 && q < d.off_b3) { off = d.off_w3; R = d.H; Cc = d.H; }
    else if (q >= d.off_w4 && q < d.off_b4) { off = d.off_w4; R = d.H; Cc = d.out_pad; }
    if (off < 0) {
      PT[i] = __float2bfloat16(P[i]);
    } else {
      const int64_t t = q - off, r = t / Cc, c = t - r * Cc;   // source element (r, c)
      PT[e * d.n_params + off + c * R + r] = __float2bfloat16(P[i]);
    }
  }
}

// rows of the batch for member e: idx = (a_e * (base + i) + b_e) mod N
__global__ void mlp_gather_kernel(const float* xn, const float* yn, int64_t N, int in_pad, int K, int B, int64_t base,
                                  const uint64_t* perm_ab, __nv_bfloat16* X0, __nv_bfloat16* X0T, int ldT, float* T,
                                  int64_t sX, int64_t sT) {
  const int e = blockIdx.y;
  const uint64_t a = perm_ab[2 * e], b = perm_ab[2 * e + 1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
    const int64_t pos = base + i;
    const bool ok = pos < N;
    const int64_t r = ok ? (int64_t)((a * (uint64_t)pos + b) % (uint64_t)N) : 0;
    for (int c = 0; c < in_pad; ++c) {
      const __nv_bfloat16 x = __float2bfloat16(ok ? xn[r * in_pad + c] : 0.0f);
      X0[e * sX + (int64_t)i * in_pad + c] = x;
      if (X0T) X0T[(int64_t)e * in_pad * ldT + (int64_t)c * ldT + i] = x;
    }
    for (int k = 0; k < K; ++k) T[e * sT + (int64_t)i * K + k] = ok ? yn[r * K + k] : __int_as_float(0x7fc00000);
  }
}

// Gaussian negative log-likelihood on standardised targets; dY = dL/dY / count.
constexpr float kLvMin = -9.0f, kLvMax = 9.0f;

__global__ void __launch_bounds__(256) mlp_loss_kernel(const float* Y, const float* T, int B, int K, int out_pad,
                                                       float inv_count, __nv_bfloat16* dY, __nv_bfloat16* dYT, int ldT,
                                                       float* loss_part, int64_t sY, int64_t sT) {
  const int e = blockIdx.y;
  float local = 0.0f;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < B * out_pad; idx += gridDim.x * blockDim.x) {
    const int i = idx / out_pad, c = idx - (idx / out_pad) * out_pad;
    float grad = 0.0f;
    if (c < K) {
      const float t = T[e * sT + (int64_t)i * K + c];
      if (t == t) {
        const float mu = Y[e * sY + (int64_t)i * out_pad + c];
        const float lv_raw = Y[e * sY + (int64_t)i * out_pad + K + c];
        const float lv = fminf(fmaxf(lv_raw, kLvMin), kLvMax);
        const float r = t - mu;
        const float ei = __expf(-lv);
        local += 0.5f * (lv + r * r * ei);
        grad = -r * ei * inv_count;
      }
    } else if (c < 2 * K) {
      const float t = T[e * sT + (int64_t)i * K + (c - K)];
      if (t == t) {
        const float mu = Y[e * sY + (int64_t)i * out_pad + (c - K)];
        const float lv_raw = Y[e * sY + (int64_t)i * out_pad + c];
        const bool inside = lv_raw > kLvMin && lv_raw < kLvMax;
        const float lv = fminf(fmaxf(lv_raw, kLvMin), kLvMax);
        const float r = t - mu;
        grad = inside ? 0.5f * (1.0f - r * r * __expf(-lv)) * inv_count : 0.0f;
      }
    }
    const __nv_bfloat16 gb = __float2bfloat16(grad);
    dY[e * sY + idx] = gb;
    dYT[(int64_t)e * out_pad * ldT + (int64_t)c * ldT + i] = gb;
  }
  // block sum in a fixed order: warps by shuffles, then warp 0 over the warp sums
  __shared__ float wsum[8];
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    loss_part[e * gridDim.x + blockIdx.x] = t * inv_count;
  }
}

// loss[e] += sum of the member's block partials, in block order (the epoch
// loss accumulates over the batches in stream order)
__global__ void mlp_loss_sum_kernel(const float* loss_part, int n_blocks, float* loss) {
  const int e = blockIdx.x;
  if (threadIdx.x != 0) return;
  float t = 0.0f;
  for (int b = 0; b < n_blocks; ++b) t += loss_part[e * n_blocks + b];
  loss[e] += t;
}

// out[z][off + i] = sum over the used reduction splits of part[split][z][off + i], in split order
__global__ void mlp_split_sum_kernel(const float* part, int used, int64_t sSplit, int64_t sMember, int64_t off,
                                     int64_t n, float* out) {
  const int z = blockIdx.y;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float acc = 0.0f;
    for (int sp = 0; sp < used; ++sp) acc += part[sp * sSplit + z * sMember + off + i];
    out[z * sMember + off + i] = acc;
  }
}

// db[n] = sum_i dZ[i][n] for every member
__global__ void mlp_colsum_kernel(const __nv_bfloat16* dZ, int B, int N, int64_t sZ, float* db, int64_t sDb) {
  const int e = blockIdx.y;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.0f;
  for (int i = 0; i < B; ++i) s += __bfloat162float(dZ[e * sZ + (int64_t)i * N + n]);
  db[e * sDb + n] = s;
}

__global__ void mlp_adam_kernel(float* P, const float* G, float* m, float* v, __nv_bfloat16* Ph, int64_t n, float lr,
                                float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = G[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float p = P[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    P[i] = p;
    Ph[i] = __float2bfloat16(p);
  }
}

// ensemble combination in standardised units -> caller units
// Targets are learnt as z = (asinh(y / c) - m) / s (c = 0: z = (y - m) / s);
// the predictive mean and variance map back through y = c sinh(m + s z)
// (delta method for the variance).
__global__ void mlp_combine_kernel(const float* Y, int N, int K, int out_pad, int members, int64_t sY,
                                   const float* ymean, const float* ystd, const float* yscale, double* mean_out,
                                   double* var_out, double* disagree, int aleatoric_only) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float worst = 0.0f;
  for (int k = 0; k < K; ++k) {
    float mu = 0.0f, mu2 = 0.0f, ale = 0.0f;
    for (int e = 0; e < members; ++e) {
      const float a = Y[e * sY + (int64_t)i * out_pad + k];
      const float lv = fminf(fmaxf(Y[e * sY + (int64_t)i * out_pad + K + k], kLvMin), kLvMax);
      mu += a;
      mu2 += a * a;
      ale += __expf(lv);
    }
    const float inv = 1.0f / (float)members;
    mu *= inv;
    const float epi = fmaxf(mu2 * inv - mu * mu, 0.0f);
    ale *= inv;
    const float var = aleatoric_only ? ale : ale + epi;
    worst = fmaxf(worst, sqrtf(epi / fmaxf(ale, 1e-12f)));
    const double u = (double)mu * (double)ystd[k] + (double)ymean[k];
    const double vu = (double)var * (double)ystd[k] * (double)ystd[k];
    const double c = yscale ? (double)yscale[k] : 0.0;
    if (c > 0.0) {
      const double ch = c * cosh(u);
      if (mean_out) mean_out[(int64_t)i * K + k] = c * sinh(u);
      if (var_out) var_out[(int64_t)i * K + k] = ch * ch * vu;
    } else {
      if (mean_out) mean_out[(int64_t)i * K + k] = u;
      if (var_out) var_out[(int64_t)i * K + k] = vu;
    }
  }
  if (disagree) disagree[i] = worst;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int blocks_for(int64_t n, int t) { return (int)std::min<int64_t>((n + t - 1) / t, 65536); }

// BF16 copies of the parameters: as stored (for dX = dZ W^T) and transposed
// (for the forward GEMMs)
cudaError_t mlp_refresh_bf16(const MlpDims& d, int members, const float* P, __nv_bfloat16* Ph, __nv_bfloat16* PhT,
                             cudaStream_t s) {
  const int64_t n = d.n_params * members;
  mlp_to_bf16_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, Ph, n);
  mlp_weights_t_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, d, members, PhT);
  return cudaGetLastError();
}

cudaError_t mlp_init(const MlpDims& d, int members, uint64_t seed, float* P, __nv_bfloat16* Ph, __nv_bfloat16* PhT,
                     cudaStream_t s) {
  const int64_t n = d.n_params * members;
  mlp_init_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d, members, seed, P);
  return mlp_refresh_bf16(d, members, P, Ph, PhT, s);
}

cudaError_t mlp_gather(const float* xn, const float* yn, int64_t N, const MlpDims& d, int B, int64_t base,
                       const uint64_t* perm_ab, int members, __nv_bfloat16* X0, __nv_bfloat16* X0T, int ldT, float* T,
                       cudaStream_t s) {
  dim3 grid((B + 255) / 256, members);
  mlp_gather_kernel<<<grid, 256, 0, s>>>(xn, yn, N, d.in_pad, d.K, B, base, perm_ab, X0, X0T, ldT, T,
                                          (int64_t)B * d.in_pad, (int64_t)B * d.K);
  return cudaGetLastError();
}

// Forward pass of all members for B rows.  X0: [members or 1][B][in_pad] (sX = 0:
// one input for every member).  Z: [members][3][B][H] fp32 (may be null), Ah:
// [members][3][B][H] bf16, AhT: [members][3][H][ldT] (transposed activations
// for the weight gradients; null for inference), Y: [members][B][out_pad].
cudaError_t mlp_forward(const MlpDims& d, int members, int B, const __nv_bfloat16* X0, int64_t sX,
                        const __nv_bfloat16* WhT, const float* Pf, float* Z, __nv_bfloat16* Ah, __nv_bfloat16* AhT,
                        int ldT, float* Y, int* err, cudaStream_t s) {
  const int H = d.H;
  const int64_t sZ = 3 * (int64_t)B * H, sL = (int64_t)B * H, sLT = (int64_t)H * ldT;
  const int64_t w_off[4] = {d.off_w1, d.off_w2, d.off_w3, d.off_w4};
  const int64_t b_off[4] = {d.off_b1, d.off_b2, d.off_b3, d.off_b4};
  cudaError_t e;
  for (int layer = 0; layer < 4; ++layer) {
    const int K = layer == 0 ? d.in_pad : H;
    const int N = layer == 3 ? d.out_pad : H;
    TcOperand A, Bw;
    A.ptr = layer == 0 ? X0 : Ah + (layer - 1) * sL;
    A.ld = K;
    A.rows = B;
    A.member_stride = layer == 0 ? sX : sZ;
    Bw.ptr = WhT + w_off[layer];   // W^T [N][K]
    Bw.ld = K;
    Bw.rows = N;
    Bw.member_stride = d.n_params;
    TcGemm g{};
    g.M = B;
    g.N = N;
    g.K = K;
    g.k_split = 1;
    g.a_shared = (layer == 0 && sX == 0) ? 1 : 0;
    g.bias = Pf + b_off[layer];
    g.sBias = d.n_params;
    g.err = err;
    if (layer < 3) {
      g.outf = Z ? Z + layer * sL : nullptr;
      g.sOutf = sZ;
      g.ldf = H;
      g.outh = Ah + layer * sL;
      g.sOuth = sZ;
      g.ldh = H;
      g.outhT = AhT ? AhT + layer * sLT : nullptr;
      g.sOuthT = 3 * sLT;
      g.ldhT = ldT;
      e = mlp_tc_gemm(EPI_HIDDEN, A, Bw, g, members, s);
    } else {
      g.outf = Y;
      g.sOutf = (int64_t)B * d.out_pad;
      g.ldf = d.out_pad;
      e = mlp_tc_gemm(EPI_LINEAR, A, Bw, g, members, s);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Backward pass: dY (bf16 [members][B][out_pad]) and dY^T ([members][out_pad][ldT])
// -> parameter gradients Gf (fp32, zeroed here).  dW_l = A_{l-1}^T dZ_l from the
// transposed copies (reduction over the batch split across CTAs, each split
// writing its own slice of Gpart, the slices summed in split order so that a
// training run is reproducible bit for bit); dZ_l = (dZ_{l+1} W_{l+1}^T)
// silu'(Z_l) with its transposed copy.
cudaError_t mlp_backward(const MlpDims& d, int members, int B, const __nv_bfloat16* X0T, const __nv_bfloat16* Wh,
                         const float* Z, const __nv_bfloat16* AhT, const __nv_bfloat16* dY, const __nv_bfloat16* dYT,
                         __nv_bfloat16* dZa, __nv_bfloat16* dZb, __nv_bfloat16* dZTa, __nv_bfloat16* dZTb, int ldT,
                         float* Gf, float* Gpart, int* err, cudaStream_t s) {
  const int H = d.H;
  const int64_t sZ = 3 * (int64_t)B * H, sL = (int64_t)B * H, sLT = (int64_t)H * ldT, sP = d.n_params;
  const int splits = mlp_wgrad_splits(B);
  const int nk = (B + 63) / 64, per = (nk + splits - 1) / splits;
  const int used = (nk + per - 1) / per;  // splits that receive reduction chunks
  cudaError_t e = cudaMemsetAsync(Gf, 0, sizeof(float) * d.n_params * members, s);
  if (e) return e;
  auto wgrad = [&](const TcOperand& A, const TcOperand& Bg, int M, int N, int64_t off) {
    TcGemm g{};
    g.M = M;
    g.N = N;
    g.K = B;
    g.k_split = splits;
    g.outf = Gpart + off;
    g.sOutf = sP;
    g.sSplit = sP * members;
    g.ldf = N;
    g.err = err;
    cudaError_t r = mlp_tc_gemm(EPI_PARTIAL, A, Bg, g, members, s);
    if (r != cudaSuccess) return r;
    const int64_t n = (int64_t)M * N;
    mlp_split_sum_kernel<<<dim3((unsigned)std::min<int64_t>((n + 255) / 256, 1024), members), 256, 0, s>>>(
        Gpart, used, sP * members, sP, off, n, Gf);
    return cudaGetLastError();
  };
  // layer 4: dW4 = A3^T dY (M = H, N = out_pad), db4 = colsum(dY)
  {
    TcOperand A{AhT + 2 * sLT, ldT, H, 3 * sLT};
    TcOperand Bg{dYT, ldT, d.out_pad, (int64_t)d.out_pad * ldT};
    if ((e = wgrad(A, Bg, H, d.out_pad, d.off_w4))) return e;
    mlp_colsum_kernel<<<dim3((d.out_pad + 127) / 128, members), 128, 0, s>>>(dY, B, d.out_pad, (int64_t)B * d.out_pad,
                                                                             Gf + d.off_b4, sP);
  }
  const __nv_bfloat16* grad_in = dY;
  int64_t s_gin = (int64_t)B * d.out_pad;
  int ld_gin = d.out_pad;
  const int64_t w_next[3] = {d.off_w2, d.off_w3, d.off_w4};
  const int64_t b_off[3] = {d.off_b1, d.off_b2, d.off_b3};
  const int64_t w_off[3] = {d.off_w1, d.off_w2, d.off_w3};
  __nv_bfloat16* bufs[2] = {dZa, dZb};
  __nv_bfloat16* bufsT[2] = {dZTa, dZTb};
  for (int layer = 2; layer >= 0; --layer) {
    __nv_bfloat16* dZ = bufs[layer & 1];
    __nv_bfloat16* dZT = bufsT[layer & 1];
    {
      // dZ_l = (grad_in W_{l+1}^T) silu'(Z_l): W_{l+1} stored [H][out] is the K-major [N = H][K = out] operand
      const int Kn = layer == 2 ? d.out_pad : H;
      TcOperand A{grad_in, ld_gin, B, s_gin};
      TcOperand Bw{Wh + w_next[layer], Kn, H, sP};
      TcGemm g{};
      g.M = B;
      g.N = H;
      g.K = Kn;
      g.k_split = 1;
      g.zprev = Z + layer * sL;
      g.sZ = sZ;
      g.ldz = H;
      g.outh = dZ;
      g.sOuth = sL;
      g.ldh = H;
      g.outhT = dZT;
      g.sOuthT = sLT;
      g.ldhT = ldT;
      g.err = err;
      if ((e = mlp_tc_gemm(EPI_DSILU, A, Bw, g, members, s))) return e;
    }
    {
      // dW_l = A_{l-1}^T dZ_l (M = in_l, N = H), db_l = colsum(dZ_l)
      const int Min = layer == 0 ? d.in_pad : H;
      TcOperand A = layer == 0 ? TcOperand{X0T, ldT, d.in_pad, (int64_t)d.in_pad * ldT}
                               : TcOperand{AhT + (layer - 1) * sLT, ldT, H, 3 * sLT};
      TcOperand Bg{dZT, ldT, H, sLT};
      if ((e = wgrad(A, Bg, Min, H, w_off[layer]))) return e;
      mlp_colsum_kernel<<<dim3((H + 127) / 128, members), 128, 0, s>>>(dZ, B, H, sL, Gf + b_off[layer], sP);
    }
    grad_in = dZ;
    s_gin = sL;
    ld_gin = H;
  }
  return cudaGetLastError();
}

cudaError_t mlp_loss(const MlpDims& d, int members, int B, int valid_rows, const float* Y, const float* T,
                     __nv_bfloat16* dY, __nv_bfloat16* dYT, int ldT, float* loss, float* loss_part, cudaStream_t s) {
  const float inv = 1.0f / (float)(std::max(1, valid_rows) * d.K);
  const int nb = mlp_loss_blocks(B, d.out_pad);
  mlp_loss_kernel<<<dim3(nb, members), 256, 0, s>>>(Y, T, B, d.K, d.out_pad, inv, dY, dYT, ldT, loss_part,
                                                    (int64_t)B * d.out_pad, (int64_t)B * d.K);
  mlp_loss_sum_kernel<<<members, 32, 0, s>>>(loss_part, nb, loss);
  return cudaGetLastError();
}

cudaError_t mlp_adam(const MlpDims& d, int members, float* P, const float* G, float* m, float* v,
                     __nv_bfloat16* Ph, __nv_bfloat16* PhT, float lr, int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
  const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
  const int64_t n = d.n_params * members;
  mlp_adam_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, G, m, v, Ph, n, lr, b1, b2, eps, c1, c2);
  mlp_weights_t_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, d, members, PhT);
  return cudaGetLastError();
}

cudaError_t mlp_combine(const MlpDims& d, int members, int N, const float* Y, const float* ymean, const float* ystd,
                        const float* yscale, double* mean_out, double* var_out, double* disagree, int aleatoric_only,
                        cudaStream_t s) {
  mlp_combine_kernel<<<(N + 127) / 128, 128, 0, s>>>(Y, N, d.K, d.out_pad, members, (int64_t)N * d.out_pad, ymean,
                                                     ystd, yscale, mean_out, var_out, disagree, aleatoric_only);
  return cudaGetLastError();
}

}  // namespace abc
