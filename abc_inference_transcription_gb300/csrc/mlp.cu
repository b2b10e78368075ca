// mlp.cu — forward, backward and Adam kernels of the surrogate ensemble.
// GEMMs use BF16 tensor-core tiles (16x16x16 fragments, FP32 accumulation);
// the ensemble member is blockIdx.z.  See mlp.cuh for the layout.
#include <cuda_bf16.h>
#include <mma.h>

#include "common.cuh"
#include "kernels.h"
#include "mlp.cuh"

namespace abc {

using namespace nvcuda;

constexpr int GBM = 64, GBN = 64, GBK = 32;

__device__ __forceinline__ float sigmoidf_fast(float z) { return 1.0f / (1.0f + __expf(-z)); }

template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(128) mlp_gemm_kernel(GemmArgs g) {
  __shared__ __align__(128) __nv_bfloat16 As[GBM][GBK + 8];
  __shared__ __align__(128) __nv_bfloat16 Bs[GBK][GBN + 8];
  __shared__ __align__(128) float Cs[GBM][GBN + 4];
  const int z = blockIdx.z;
  const __nv_bfloat16* A = g.A + z * g.sA;
  const __nv_bfloat16* B = g.B + z * g.sB;
  const int n_mt = (g.M + GBM - 1) / GBM;
  const int mt = blockIdx.y % n_mt;
  const int split = blockIdx.y / n_mt;
  const int m0 = mt * GBM, n0 = blockIdx.x * GBN;
  int kbeg = 0, kend = g.K;
  if (EPI == EPI_ATOMIC) {
    const int per = (((g.K + g.k_split - 1) / g.k_split) + GBK - 1) / GBK * GBK;
    kbeg = split * per;
    kend = min(g.K, kbeg + per);
  }
  const int warp = threadIdx.x >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) wmma::fill_fragment(acc[i][j], 0.0f);
  const __nv_bfloat16 zero = __float2bfloat16(0.0f);
  for (int k0 = kbeg; k0 < kend; k0 += GBK) {
    for (int idx = threadIdx.x; idx < GBM * GBK; idx += 128) {
      int r, c;
      if (TA) { c = idx / GBM; r = idx - c * GBM; }  // consecutive threads along m (contiguous in A)
      else { r = idx / GBK; c = idx - r * GBK; }     // consecutive threads along k
      const int m = m0 + r, k = k0 + c;
      __nv_bfloat16 v = zero;
      if (m < g.M && k < kend) v = TA ? A[(int64_t)k * g.lda + m] : A[(int64_t)m * g.lda + k];
      As[r][c] = v;
    }
    for (int idx = threadIdx.x; idx < GBK * GBN; idx += 128) {
      int r, c;
      if (TB) { r = idx % GBK; c = idx / GBK; }      // consecutive threads along k (contiguous in B)
      else { r = idx / GBN; c = idx - r * GBN; }     // consecutive threads along n
      const int k = k0 + r, n = n0 + c;
      __nv_bfloat16 v = zero;
      if (n < g.N && k < kend) v = TB ? B[(int64_t)n * g.ldb + k] : B[(int64_t)k * g.ldb + n];
      Bs[r][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 16) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, __nv_bfloat16, wmma::row_major> fa[2];
      wmma::fragment<wmma::matrix_b, 16, 16, 16, __nv_bfloat16, wmma::row_major> fb[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) wmma::load_matrix_sync(fa[i], &As[wm * 32 + i * 16][kk], GBK + 8);
#pragma unroll
      for (int j = 0; j < 2; ++j) wmma::load_matrix_sync(fb[j], &Bs[kk][wn * 32 + j * 16], GBN + 8);
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) wmma::mma_sync(acc[i][j], fa[i], fb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
      wmma::store_matrix_sync(&Cs[wm * 32 + i * 16][wn * 32 + j * 16], acc[i][j], GBN + 4, wmma::mem_row_major);
  __syncthreads();
  const float* bias = g.bias ? g.bias + z * g.sBias : nullptr;
  for (int idx = threadIdx.x; idx < GBM * GBN; idx += 128) {
    const int r = idx / GBN, c = idx - r * GBN;
    const int m = m0 + r, n = n0 + c;
    if (m >= g.M || n >= g.N) continue;
    const float v = Cs[r][c];
    const int64_t o = (int64_t)m * g.ldo + n;
    if (EPI == EPI_HIDDEN) {
      const float zz = v + (bias ? bias[n] : 0.0f);
      if (g.outf) g.outf[z * g.sOut + o] = zz;
      g.outh[z * g.sOut + o] = __float2bfloat16(zz * sigmoidf_fast(zz));
    } else if (EPI == EPI_LINEAR) {
      g.outf[z * g.sOut + o] = v + (bias ? bias[n] : 0.0f);
    } else if (EPI == EPI_ATOMIC) {
      atomicAdd(&g.outf[z * g.sOut + o], v);
    } else {
      const float zp = g.zprev[z * g.sZ + o];
      const float s = sigmoidf_fast(zp);
      g.outh[z * g.sOut + o] = __float2bfloat16(v * (s * (1.0f + zp * (1.0f - s))));
    }
  }
}

template <bool TA, bool TB, int EPI>
static cudaError_t gemm(const GemmArgs& g, int members, int splits, cudaStream_t s) {
  const int n_mt = (g.M + GBM - 1) / GBM;
  dim3 grid((g.N + GBN - 1) / GBN, n_mt * splits, members);
  GemmArgs a = g;
  a.k_split = splits;
  mlp_gemm_kernel<TA, TB, EPI><<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

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

// rows of the batch for member e: idx = (a_e * (base + i) + b_e) mod N
__global__ void mlp_gather_kernel(const float* xn, const float* yn, int64_t N, int in_pad, int K, int B, int64_t base,
                                  const uint64_t* perm_ab, __nv_bfloat16* X0, float* T, int64_t sX, int64_t sT) {
  const int e = blockIdx.y;
  const uint64_t a = perm_ab[2 * e], b = perm_ab[2 * e + 1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
    const int64_t pos = base + i;
    const bool ok = pos < N;
    const int64_t r = ok ? (int64_t)((a * (uint64_t)pos + b) % (uint64_t)N) : 0;
    for (int c = 0; c < in_pad; ++c)
      X0[e * sX + (int64_t)i * in_pad + c] = __float2bfloat16(ok ? xn[r * in_pad + c] : 0.0f);
    for (int k = 0; k < K; ++k) T[e * sT + (int64_t)i * K + k] = ok ? yn[r * K + k] : __int_as_float(0x7fc00000);
  }
}

// Gaussian negative log-likelihood on standardised targets; dY = dL/dY / count.
constexpr float kLvMin = -9.0f, kLvMax = 9.0f;

__global__ void mlp_loss_kernel(const float* Y, const float* T, int B, int K, int out_pad, float inv_count,
                                __nv_bfloat16* dY, float* loss, int64_t sY, int64_t sT) {
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
    dY[e * sY + idx] = __float2bfloat16(grad);
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&loss[e], local * inv_count);
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

cudaError_t mlp_init(const MlpDims& d, int members, uint64_t seed, float* P, __nv_bfloat16* Ph, cudaStream_t s) {
  const int64_t n = d.n_params * members;
  mlp_init_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d, members, seed, P);
  mlp_to_bf16_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, Ph, n);
  return cudaGetLastError();
}

cudaError_t mlp_to_bf16(const float* src, __nv_bfloat16* dst, int64_t n, cudaStream_t s) {
  mlp_to_bf16_kernel<<<blocks_for(n, 256), 256, 0, s>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t mlp_gather(const float* xn, const float* yn, int64_t N, const MlpDims& d, int B, int64_t base,
                       const uint64_t* perm_ab, int members, __nv_bfloat16* X0, float* T, cudaStream_t s) {
  dim3 grid((B + 255) / 256, members);
  mlp_gather_kernel<<<grid, 256, 0, s>>>(xn, yn, N, d.in_pad, d.K, B, base, perm_ab, X0, T, (int64_t)B * d.in_pad,
                                          (int64_t)B * d.K);
  return cudaGetLastError();
}

// Forward pass of all members for a batch of B rows.  X0: [members or 1][B][in_pad]
// (sX = 0 shares one input).  Z: [members][3][B][H] fp32 (may be null),
// Ah: [members][3][B][H] bf16, Y: [members][B][out_pad].
cudaError_t mlp_forward(const MlpDims& d, int members, int B, const __nv_bfloat16* X0, int64_t sX,
                        const __nv_bfloat16* Wh, const float* Pf, float* Z, __nv_bfloat16* Ah, float* Y,
                        cudaStream_t s) {
  const int H = d.H;
  const int64_t sZ = 3 * (int64_t)B * H, sL = (int64_t)B * H;
  cudaError_t err;
  for (int layer = 0; layer < 3; ++layer) {
    GemmArgs g{};
    g.A = layer == 0 ? X0 : Ah + (layer - 1) * sL;
    g.sA = layer == 0 ? sX : sZ;
    g.B = Wh + (layer == 0 ? d.off_w1 : layer == 1 ? d.off_w2 : d.off_w3);
    g.sB = d.n_params;
    g.bias = Pf + (layer == 0 ? d.off_b1 : layer == 1 ? d.off_b2 : d.off_b3);
    g.sBias = d.n_params;
    g.outf = Z ? Z + layer * sL : nullptr;
    g.outh = Ah + layer * sL;
    g.sOut = sZ;
    g.M = B;
    g.N = H;
    g.K = layer == 0 ? d.in_pad : H;
    g.lda = g.K;
    g.ldb = H;
    g.ldo = H;
    err = gemm<false, false, EPI_HIDDEN>(g, members, 1, s);
    if (err) return err;
  }
  GemmArgs g{};
  g.A = Ah + 2 * sL;
  g.sA = sZ;
  g.B = Wh + d.off_w4;
  g.sB = d.n_params;
  g.bias = Pf + d.off_b4;
  g.sBias = d.n_params;
  g.outf = Y;
  g.sOut = (int64_t)B * d.out_pad;
  g.M = B;
  g.N = d.out_pad;
  g.K = H;
  g.lda = H;
  g.ldb = d.out_pad;
  g.ldo = d.out_pad;
  return gemm<false, false, EPI_LINEAR>(g, members, 1, s);
}

// Backward pass: loss gradient dY (bf16 [members][B][out_pad]) -> parameter
// gradients Gf (fp32, zeroed here).  dA, dZ: [members][B][H] bf16 scratch.
cudaError_t mlp_backward(const MlpDims& d, int members, int B, const __nv_bfloat16* X0, int64_t sX,
                         const __nv_bfloat16* Wh, const float* Z, const __nv_bfloat16* Ah, const __nv_bfloat16* dY,
                         __nv_bfloat16* dZa, __nv_bfloat16* dZb, float* Gf, cudaStream_t s) {
  const int H = d.H;
  const int64_t sZ = 3 * (int64_t)B * H, sL = (int64_t)B * H, sP = d.n_params;
  const int splits = std::max(1, std::min(32, B / 256));
  cudaError_t err = cudaMemsetAsync(Gf, 0, sizeof(float) * d.n_params * members, s);
  if (err) return err;
  // layer 4: dW4 = A3^T dY, db4 = colsum(dY)
  {
    GemmArgs g{};
    g.A = Ah + 2 * sL; g.sA = sZ; g.lda = H;                 // A3 stored [B][H] -> op = A3^T (M=H, K=B)
    g.B = dY; g.sB = (int64_t)B * d.out_pad; g.ldb = d.out_pad;
    g.outf = Gf + d.off_w4; g.sOut = sP; g.ldo = d.out_pad;
    g.M = H; g.N = d.out_pad; g.K = B;
    if ((err = gemm<true, false, EPI_ATOMIC>(g, members, splits, s))) return err;
    mlp_colsum_kernel<<<dim3((d.out_pad + 127) / 128, members), 128, 0, s>>>(dY, B, d.out_pad, (int64_t)B * d.out_pad,
                                                                             Gf + d.off_b4, sP);
  }
  // dZ3 = (dY W4^T) * silu'(Z3)
  const __nv_bfloat16* grad_in = dY;
  int64_t s_gin = (int64_t)B * d.out_pad;
  int ld_gin = d.out_pad;
  int64_t w_off[3] = {d.off_w2, d.off_w3, d.off_w4};
  int64_t b_off[3] = {d.off_b1, d.off_b2, d.off_b3};
  int64_t wgrad_off[3] = {d.off_w1, d.off_w2, d.off_w3};
  __nv_bfloat16* bufs[2] = {dZa, dZb};
  for (int layer = 2; layer >= 0; --layer) {
    __nv_bfloat16* dZ = bufs[layer & 1];
    {
      GemmArgs g{};
      g.A = grad_in; g.sA = s_gin; g.lda = ld_gin;
      g.B = Wh + w_off[layer]; g.sB = sP; g.ldb = (layer == 2) ? d.out_pad : H;   // W_{l+1} stored [H][out]
      g.zprev = Z + layer * sL; g.sZ = sZ;
      g.outh = dZ; g.sOut = sL; g.ldo = H;
      g.M = B; g.N = H; g.K = (layer == 2) ? d.out_pad : H;
      if ((err = gemm<false, true, EPI_DSILU>(g, members, 1, s))) return err;
    }
    {
      GemmArgs g{};
      const __nv_bfloat16* in = layer == 0 ? X0 : Ah + (layer - 1) * sL;
      g.A = in; g.sA = layer == 0 ? sX : sZ; g.lda = layer == 0 ? d.in_pad : H;
      g.B = dZ; g.sB = sL; g.ldb = H;
      g.outf = Gf + wgrad_off[layer]; g.sOut = sP; g.ldo = H;
      g.M = layer == 0 ? d.in_pad : H; g.N = H; g.K = B;
      if ((err = gemm<true, false, EPI_ATOMIC>(g, members, splits, s))) return err;
      mlp_colsum_kernel<<<dim3((H + 127) / 128, members), 128, 0, s>>>(dZ, B, H, sL, Gf + b_off[layer], sP);
    }
    grad_in = dZ;
    s_gin = sL;
    ld_gin = H;
  }
  return cudaGetLastError();
}

cudaError_t mlp_loss(const MlpDims& d, int members, int B, int valid_rows, const float* Y, const float* T,
                     __nv_bfloat16* dY, float* loss, cudaStream_t s) {
  const float inv = 1.0f / (float)(std::max(1, valid_rows) * d.K);
  dim3 grid(std::min(1024, (B * d.out_pad + 255) / 256), members);
  mlp_loss_kernel<<<grid, 256, 0, s>>>(Y, T, B, d.K, d.out_pad, inv, dY, loss, (int64_t)B * d.out_pad,
                                       (int64_t)B * d.K);
  return cudaGetLastError();
}

cudaError_t mlp_adam(const MlpDims& d, int members, float* P, const float* G, float* m, float* v,
                     __nv_bfloat16* Ph, float lr, int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
  const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
  const int64_t n = d.n_params * members;
  mlp_adam_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, G, m, v, Ph, n, lr, b1, b2, eps, c1, c2);
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
