// surrogate.cu — C ABI of the learned pre-screen: an ensemble of MLPs from
// log-parameters to the means and log-variances of the summary statistics,
// trained on the pipeline's own SSA output by the kernels of mlp.cu, and the
// screen that sends to the exact SSA only the prior draws whose predicted
// error lies under a gene's threshold plus a calibrated margin, or whose
// ensemble disagrees.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/abcgpu.h"
#include "kernels.h"
#include "mlp.cuh"

namespace abc {
cudaError_t mlp_init(const MlpDims& d, int members, uint64_t seed, float* P, __nv_bfloat16* Ph, __nv_bfloat16* PhT,
                     cudaStream_t s);
cudaError_t mlp_refresh_bf16(const MlpDims& d, int members, const float* P, __nv_bfloat16* Ph, __nv_bfloat16* PhT,
                             cudaStream_t s);
cudaError_t mlp_gather(const float* xn, const float* yn, int64_t N, const MlpDims& d, int B, int64_t base,
                       const uint64_t* perm_ab, int members, __nv_bfloat16* X0, __nv_bfloat16* X0T, int ldT, float* T,
                       cudaStream_t s);
cudaError_t mlp_forward(const MlpDims& d, int members, int B, const __nv_bfloat16* X0, int64_t sX,
                        const __nv_bfloat16* WhT, const float* Pf, float* Z, __nv_bfloat16* Ah, __nv_bfloat16* AhT,
                        int ldT, float* Y, int* err, cudaStream_t s);
cudaError_t mlp_backward(const MlpDims& d, int members, int B, const __nv_bfloat16* X0T, const __nv_bfloat16* Wh,
                         const float* Z, const __nv_bfloat16* AhT, const __nv_bfloat16* dY, const __nv_bfloat16* dYT,
                         __nv_bfloat16* dZa, __nv_bfloat16* dZb, __nv_bfloat16* dZTa, __nv_bfloat16* dZTb, int ldT,
                         float* Gf, float* Gpart, int* err, cudaStream_t s);
cudaError_t mlp_loss(const MlpDims& d, int members, int B, int valid_rows, const float* Y, const float* T,
                     __nv_bfloat16* dY, __nv_bfloat16* dYT, int ldT, float* loss, float* loss_part, cudaStream_t s);
cudaError_t mlp_adam(const MlpDims& d, int members, float* P, const float* G, float* m, float* v,
                     __nv_bfloat16* Ph, __nv_bfloat16* PhT, float lr, int step, cudaStream_t s);
cudaError_t mlp_combine(const MlpDims& d, int members, int N, const float* Y, const float* ymean, const float* ystd,
                        const float* yscale, double* mean_out, double* var_out, double* disagree, int aleatoric_only,
                        cudaStream_t s);
}  // namespace abc

using namespace abc;

namespace {

template <typename T>
struct Buf {
  T* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t n) {
    if (p && n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) cap = std::max<size_t>(n, 1);
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// column mean / standard deviation over finite values (two passes)
__global__ void col_norm_kernel(const double* X, int64_t N, int ld, int cols, double* mean, double* sd) {
  __shared__ double red[256];
  __shared__ double cnt[256];
  const int c = blockIdx.x;
  if (c >= cols) return;
  double s = 0.0, n = 0.0;
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
    const double v = X[i * ld + c];
    if (isfinite(v)) { s += v; n += 1.0; }
  }
  red[threadIdx.x] = s;
  cnt[threadIdx.x] = n;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) { red[threadIdx.x] += red[threadIdx.x + o]; cnt[threadIdx.x] += cnt[threadIdx.x + o]; }
    __syncthreads();
  }
  const double mu = cnt[0] > 0.0 ? red[0] / cnt[0] : 0.0;
  const double nn = cnt[0];
  __syncthreads();
  double q = 0.0;
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
    const double v = X[i * ld + c];
    if (isfinite(v)) q += (v - mu) * (v - mu);
  }
  red[threadIdx.x] = q;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    mean[c] = mu;
    const double v = nn > 1.0 ? red[0] / (nn - 1.0) : 1.0;
    sd[c] = v > 1e-24 ? sqrt(v) : 1.0;
  }
}

// theta (FP64, row stride ld) -> standardised FP32 [N][in_pad] (zero padding)
__global__ void norm_x_kernel(const double* th, int64_t N, int in_dim, int ld, const double* mean, const double* sd,
                              int in_pad, float* xf, __nv_bfloat16* xh) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N * in_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / in_pad;
    const int c = (int)(i - r * in_pad);
    float v = 0.0f;
    if (c < in_dim) v = (float)((th[r * ld + c] - mean[c]) / sd[c]);
    if (xf) xf[i] = v;
    if (xh) xh[i] = __float2bfloat16(v);
  }
}

// statistics -> standardised FP32 targets, NaN where not finite
__global__ void norm_y_kernel(const double* st, int64_t N, int K, const double* mean, const double* sd, float* yf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N * K; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % K);
    const double v = st[i];
    yf[i] = isfinite(v) ? (float)((v - mean[c]) / sd[c]) : __int_as_float(0x7fc00000);
  }
}

// per statistic: scale c = mean |y| over finite values (1 if none), then y <- asinh(y / c) in place
__global__ void asinh_scale_kernel(double* st, int64_t N, int K, float* scale) {
  __shared__ double red[256];
  __shared__ double cnt[256];
  const int c = blockIdx.x;
  double s = 0.0, n = 0.0;
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
    const double v = st[i * K + c];
    if (isfinite(v)) { s += fabs(v); n += 1.0; }
  }
  red[threadIdx.x] = s;
  cnt[threadIdx.x] = n;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) { red[threadIdx.x] += red[threadIdx.x + o]; cnt[threadIdx.x] += cnt[threadIdx.x + o]; }
    __syncthreads();
  }
  double sc = cnt[0] > 0.0 ? red[0] / cnt[0] : 1.0;
  if (!(sc > 1e-12)) sc = 1.0;
  __syncthreads();
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
    const double v = st[i * K + c];
    if (isfinite(v)) st[i * K + c] = asinh(v / sc);
  }
  if (threadIdx.x == 0) scale[c] = (float)sc;
}

__global__ void asinh_apply_kernel(double* st, int64_t N, int K, const float* scale) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N * K; i += (int64_t)gridDim.x * blockDim.x) {
    const float c = scale[i % K];
    const double v = st[i];
    if (c > 0.0f && isfinite(v)) st[i] = asinh(v / (double)c);
  }
}

__global__ void d2f_kernel(const double* a, float* b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void disagree_keep_kernel(const double* dis, int64_t N, double dmax, uint8_t* keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    if (!(dis[i] <= dmax)) keep[i] = 1;
}

__global__ void count_keep_kernel(const uint8_t* keep, int64_t N, unsigned long long* n) {
  unsigned long long c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    c += keep[i] ? 1ull : 0ull;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(n, c);
}

int blocks(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 65536); }

// Survivor compaction in ascending row order: per-1024-row counts, one scan,
// then a scatter with warp-ballot ranks inside each block.
constexpr int kCompactRows = 1024;

__global__ void compact_count_kernel(const uint8_t* keep, int64_t N, unsigned int* counts) {
  __shared__ unsigned int warp_n[32];
  const int64_t i = (int64_t)blockIdx.x * kCompactRows + threadIdx.x;
  const bool k = i < N && keep[i];
  const unsigned b = __ballot_sync(0xffffffffu, k);
  if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = 0;
    for (int w = 0; w < kCompactRows / 32; ++w) t += warp_n[w];
    counts[blockIdx.x] = t;
  }
}

__global__ void compact_scan_kernel(unsigned int* counts, int64_t nb, unsigned long long* total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long run = 0;
  for (int64_t b = 0; b < nb; ++b) {
    const unsigned int c = counts[b];
    counts[b] = (unsigned int)run;
    run += c;
  }
  *total = run;
}

__global__ void compact_scatter_kernel(const uint8_t* keep, int64_t N, const unsigned int* start, const double* th,
                                       int ld, double* th_out, int64_t* idx_out) {
  __shared__ unsigned int warp_base[32];
  const int64_t i = (int64_t)blockIdx.x * kCompactRows + threadIdx.x;
  const bool k = i < N && keep[i];
  const unsigned b = __ballot_sync(0xffffffffu, k);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_base[warp] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int run = 0;
    for (int w = 0; w < kCompactRows / 32; ++w) {
      const unsigned int c = warp_base[w];
      warp_base[w] = run;
      run += c;
    }
  }
  __syncthreads();
  if (!k) return;
  const int64_t pos = (int64_t)start[blockIdx.x] + warp_base[warp] + __popc(b & ((1u << lane) - 1u));
  if (idx_out) idx_out[pos] = i;
  if (th_out)
    for (int c = 0; c < ld; ++c) th_out[pos * ld + c] = th[i * ld + c];
}

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t gcd_u64(uint64_t a, uint64_t b) {
  while (b) { uint64_t t = a % b; a = b; b = t; }
  return a;
}

constexpr int kPredChunk = 65536;

}  // namespace

struct abc_surrogate {
  MlpDims d;
  int members = 4;
  uint64_t seed = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int step = 0;
  bool normed = false;
  int screen_mode = 0;           // 0: per-statistic lower bound, 1: error-distribution lower quantile
  Buf<float> P, G, Am, Av, ymf, ysf, yscf;  // yscf: asinh scale per statistic (0: identity)
  Buf<__nv_bfloat16> Ph, PhT;   // BF16 weights as stored and transposed
  Buf<int> tcerr;                // tensor-core GEMM error word
  Buf<double> xm, xs, ym, ys;
  // training / batch scratch
  Buf<double> th64, st64;
  Buf<float> xn, yn, T, Z, Y;
  Buf<__nv_bfloat16> X0, Ah, dY, dZa, dZb;
  Buf<__nv_bfloat16> X0T, AhT, dYT, dZTa, dZTb;  // [features][ldT] copies for the weight gradients
  int ldT = 0;
  Buf<float> loss, loss_part;  // per-member loss; per-block partial sums of the loss kernel
  Buf<float> Gpart;            // weight-gradient partial sums, one slice per reduction split
  Buf<uint64_t> perm;
  // prediction scratch
  Buf<double> pm, pv, pd;
  Buf<float> pmf, pvf, sw, dw, X;
  Buf<double> gd, gs;
  Buf<uint8_t> keep;
  Buf<unsigned long long> cnt;
};

static int sfail(abc_surrogate* s, int st, const std::string& m) {
  if (s) s->err = m;
  return st;
}
#define SK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      return sfail(s, e_ == cudaErrorMemoryAllocation ? ABC_ERR_NOMEM : ABC_ERR_CUDA,                \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                              \
  } while (0)

static int ensure_batch(abc_surrogate* s, int B) {
  const MlpDims& d = s->d;
  const size_t E = s->members;
  SK(s->X0.ensure(E * B * d.in_pad));
  SK(s->T.ensure(E * B * d.K));
  SK(s->Z.ensure(E * 3 * B * d.H));
  SK(s->Ah.ensure(E * 3 * B * d.H));
  SK(s->Y.ensure(E * B * d.out_pad));
  SK(s->dY.ensure(E * B * d.out_pad));
  SK(s->dZa.ensure(E * B * d.H));
  SK(s->dZb.ensure(E * B * d.H));
  s->ldT = (B + 7) / 8 * 8;   // 16-byte rows for the tensor maps
  const size_t lt = (size_t)s->ldT;
  SK(s->X0T.ensure(E * d.in_pad * lt));
  SK(s->AhT.ensure(E * 3 * d.H * lt));
  SK(s->dYT.ensure(E * d.out_pad * lt));
  SK(s->dZTa.ensure(E * d.H * lt));
  SK(s->dZTb.ensure(E * d.H * lt));
  SK(s->loss.ensure(E));
  SK(s->loss_part.ensure(E * (size_t)mlp_loss_blocks(B, d.out_pad)));
  SK(s->Gpart.ensure((size_t)mlp_wgrad_splits(B) * E * (size_t)d.n_params));
  SK(s->perm.ensure(2 * E));
  return ABC_OK;
}

// the tensor-core GEMMs report a bounded wait that ran out in tcerr
static int check_tc(abc_surrogate* s) {
  int h = 0;
  SK(cudaMemcpy(&h, s->tcerr.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    SK(cudaMemset(s->tcerr.p, 0, sizeof(int)));
    return sfail(s, ABC_ERR_CUDA, "tensor-core GEMM: a bounded wait ran out (code " + std::to_string(h) + ")");
  }
  return ABC_OK;
}

// gather a batch, forward, loss and backward (gradients in s->G)
static int train_step(abc_surrogate* s, int B, int64_t base, int valid, int64_t N) {
  const MlpDims& d = s->d;
  const int E = s->members;
  SK(mlp_gather(s->xn.p, s->yn.p, N, d, B, base, s->perm.p, E, s->X0.p, s->X0T.p, s->ldT, s->T.p, s->stream));
  SK(mlp_forward(d, E, B, s->X0.p, (int64_t)B * d.in_pad, s->PhT.p, s->P.p, s->Z.p, s->Ah.p, s->AhT.p, s->ldT,
                 s->Y.p, s->tcerr.p, s->stream));
  SK(mlp_loss(d, E, B, valid, s->Y.p, s->T.p, s->dY.p, s->dYT.p, s->ldT, s->loss.p, s->loss_part.p, s->stream));
  SK(mlp_backward(d, E, B, s->X0T.p, s->Ph.p, s->Z.p, s->AhT.p, s->dY.p, s->dYT.p, s->dZa.p, s->dZb.p, s->dZTa.p,
                  s->dZTb.p, s->ldT, s->G.p, s->Gpart.p, s->tcerr.p, s->stream));
  return ABC_OK;
}

extern "C" {

int abc_surrogate_create(abc_surrogate** out, int in_dim, int n_stats, int ensemble, uint64_t seed) {
  if (!out || in_dim < 1 || in_dim > kMlpInPad || n_stats < 1 || n_stats > 256 || ensemble < 1 || ensemble > 16)
    return ABC_ERR_INVALID;
  *out = nullptr;
  abc_surrogate* s = new (std::nothrow) abc_surrogate();
  if (!s) return ABC_ERR_NOMEM;
  s->d = mlp_dims(in_dim, n_stats);
  s->members = ensemble;
  s->seed = seed;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return ABC_ERR_CUDA;
  }
  const size_t n = (size_t)s->d.n_params * ensemble;
  if (s->P.ensure(n) || s->G.ensure(n) || s->Am.ensure(n) || s->Av.ensure(n) || s->Ph.ensure(n) ||
      s->PhT.ensure(n) || s->tcerr.ensure(1) || cudaMemset(s->tcerr.p, 0, sizeof(int)) != cudaSuccess ||
      s->xm.ensure(kMlpInPad) || s->xs.ensure(kMlpInPad) || s->ym.ensure(n_stats) || s->ys.ensure(n_stats) ||
      s->ymf.ensure(n_stats) || s->ysf.ensure(n_stats) || s->yscf.ensure(n_stats) || s->cnt.ensure(1) ||
      cudaMemset(s->yscf.p, 0, sizeof(float) * n_stats) != cudaSuccess) {
    cudaStreamDestroy(s->stream);
    delete s;
    return ABC_ERR_NOMEM;
  }
  if (mlp_init(s->d, ensemble, seed, s->P.p, s->Ph.p, s->PhT.p, s->stream) != cudaSuccess ||
      cudaMemsetAsync(s->Am.p, 0, n * sizeof(float), s->stream) != cudaSuccess ||
      cudaMemsetAsync(s->Av.p, 0, n * sizeof(float), s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess) {
    cudaStreamDestroy(s->stream);
    delete s;
    return ABC_ERR_CUDA;
  }
  *out = s;
  return ABC_OK;
}

int abc_surrogate_destroy(abc_surrogate* s) {
  if (!s) return ABC_OK;
  cudaStreamSynchronize(s->stream);
  s->yscf.release();
  s->P.release(); s->G.release(); s->Am.release(); s->Av.release(); s->Ph.release(); s->ymf.release();
  s->PhT.release(); s->tcerr.release(); s->X0T.release(); s->AhT.release(); s->dYT.release(); s->dZTa.release();
  s->dZTb.release();
  s->ysf.release(); s->xm.release(); s->xs.release(); s->ym.release(); s->ys.release(); s->th64.release();
  s->st64.release(); s->xn.release(); s->yn.release(); s->T.release(); s->Z.release(); s->Y.release();
  s->X0.release(); s->Ah.release(); s->dY.release(); s->dZa.release(); s->dZb.release(); s->loss.release();
  s->loss_part.release(); s->Gpart.release();
  s->perm.release(); s->pm.release(); s->pv.release(); s->pd.release(); s->pmf.release(); s->pvf.release();
  s->sw.release(); s->dw.release(); s->X.release(); s->gd.release(); s->gs.release(); s->keep.release();
  s->cnt.release();
  cudaStreamDestroy(s->stream);
  delete s;
  return ABC_OK;
}

const char* abc_surrogate_last_error(const abc_surrogate* s) { return s ? s->err.c_str() : "null surrogate"; }

int abc_surrogate_num_params(const abc_surrogate* s) { return s ? (int)s->d.n_params : ABC_ERR_INVALID; }

int abc_surrogate_set_screen_mode(abc_surrogate* s, int mode) {
  if (!s) return ABC_ERR_INVALID;
  if (mode != 0 && mode != 1) return sfail(s, ABC_ERR_INVALID, "screen mode must be 0 or 1");
  s->screen_mode = mode;
  return ABC_OK;
}

// load host data and standardise it (normalisation constants from this data
// when `fit_norm`, else the stored ones)
static int load_training(abc_surrogate* s, const double* theta, const double* stats, int64_t N, bool fit_norm) {
  const MlpDims& d = s->d;
  SK(s->th64.ensure((size_t)N * d.in_dim));
  SK(s->st64.ensure((size_t)N * d.K));
  SK(s->xn.ensure((size_t)N * d.in_pad));
  SK(s->yn.ensure((size_t)N * d.K));
  SK(cudaMemcpyAsync(s->th64.p, theta, sizeof(double) * N * d.in_dim, cudaMemcpyHostToDevice, s->stream));
  SK(cudaMemcpyAsync(s->st64.p, stats, sizeof(double) * N * d.K, cudaMemcpyHostToDevice, s->stream));
  if (fit_norm) {
    asinh_scale_kernel<<<d.K, 256, 0, s->stream>>>(s->st64.p, N, d.K, s->yscf.p);
    col_norm_kernel<<<d.in_dim, 256, 0, s->stream>>>(s->th64.p, N, d.in_dim, d.in_dim, s->xm.p, s->xs.p);
    col_norm_kernel<<<d.K, 256, 0, s->stream>>>(s->st64.p, N, d.K, d.K, s->ym.p, s->ys.p);
    SK(cudaGetLastError());
    d2f_kernel<<<1, 256, 0, s->stream>>>(s->ym.p, s->ymf.p, d.K);
    d2f_kernel<<<1, 256, 0, s->stream>>>(s->ys.p, s->ysf.p, d.K);
    s->normed = true;
  } else {
    asinh_apply_kernel<<<blocks(N * d.K), 256, 0, s->stream>>>(s->st64.p, N, d.K, s->yscf.p);
  }
  norm_x_kernel<<<blocks(N * d.in_pad), 256, 0, s->stream>>>(s->th64.p, N, d.in_dim, d.in_dim, s->xm.p, s->xs.p,
                                                              d.in_pad, s->xn.p, nullptr);
  norm_y_kernel<<<blocks(N * d.K), 256, 0, s->stream>>>(s->st64.p, N, d.K, s->ym.p, s->ys.p, s->yn.p);
  SK(cudaGetLastError());
  return ABC_OK;
}

int abc_surrogate_train(abc_surrogate* s, const double* theta, const double* stats, int64_t N, int epochs, int batch,
                        double lr, double* epoch_loss) {
  if (!s) return ABC_ERR_INVALID;
  if (!theta || !stats || N < 2 || epochs < 1 || batch < 16 || batch > 65536 || !(lr > 0.0))
    return sfail(s, ABC_ERR_INVALID, "abc_surrogate_train: bad arguments");
  int st = load_training(s, theta, stats, N, true);
  if (st) return st;
  const int B = batch;
  st = ensure_batch(s, B);
  if (st) return st;
  const MlpDims& d = s->d;
  const int E = s->members;
  uint64_t rs = s->seed ^ 0x5ab5ull ^ ((uint64_t)s->step << 20);
  std::vector<uint64_t> ab(2 * E);
  for (int ep = 0; ep < epochs; ++ep) {
    for (int e = 0; e < E; ++e) {
      uint64_t a;
      do { a = (splitmix(rs) % (uint64_t)N) | 1ull; } while (gcd_u64(a, (uint64_t)N) != 1ull);
      ab[2 * e] = a;
      ab[2 * e + 1] = splitmix(rs) % (uint64_t)N;
    }
    SK(cudaMemcpyAsync(s->perm.p, ab.data(), sizeof(uint64_t) * 2 * E, cudaMemcpyHostToDevice, s->stream));
    SK(cudaMemsetAsync(s->loss.p, 0, sizeof(float) * E, s->stream));
    int nb = 0;
    for (int64_t base = 0; base < N; base += B, ++nb) {
      const int valid = (int)std::min<int64_t>(B, N - base);
      st = train_step(s, B, base, valid, N);
      if (st) return st;
      s->step++;
      SK(mlp_adam(d, E, s->P.p, s->G.p, s->Am.p, s->Av.p, s->Ph.p, s->PhT.p, (float)lr, s->step, s->stream));
    }
    if (epoch_loss) {
      std::vector<float> hl(E);
      SK(cudaMemcpyAsync(hl.data(), s->loss.p, sizeof(float) * E, cudaMemcpyDeviceToHost, s->stream));
      SK(cudaStreamSynchronize(s->stream));
      double m = 0.0;
      for (int e = 0; e < E; ++e) m += hl[e];
      epoch_loss[ep] = m / (double)E / (double)nb;
    }
  }
  SK(cudaStreamSynchronize(s->stream));
  return check_tc(s);
}

// one forward/backward pass without update: per-member loss and gradients
// (gradient check against the CPU reference network)
int abc_surrogate_gradients(abc_surrogate* s, const double* theta, const double* stats, int64_t N, double* loss,
                            float* grads) {
  if (!s) return ABC_ERR_INVALID;
  if (!s->normed) return sfail(s, ABC_ERR_STATE, "normalisation not set (train or set_norm first)");
  if (!theta || !stats || N < 1 || N > 65536) return sfail(s, ABC_ERR_INVALID, "abc_surrogate_gradients: 1 <= N <= 65536");
  int st = load_training(s, theta, stats, N, false);
  if (st) return st;
  const int B = (int)N;
  st = ensure_batch(s, B);
  if (st) return st;
  const MlpDims& d = s->d;
  const int E = s->members;
  std::vector<uint64_t> ab(2 * E);
  for (int e = 0; e < E; ++e) { ab[2 * e] = 1; ab[2 * e + 1] = 0; }
  SK(cudaMemcpyAsync(s->perm.p, ab.data(), sizeof(uint64_t) * 2 * E, cudaMemcpyHostToDevice, s->stream));
  SK(cudaMemsetAsync(s->loss.p, 0, sizeof(float) * E, s->stream));
  st = train_step(s, B, 0, B, N);
  if (st) return st;
  std::vector<float> hl(E);
  SK(cudaMemcpyAsync(hl.data(), s->loss.p, sizeof(float) * E, cudaMemcpyDeviceToHost, s->stream));
  if (grads)
    SK(cudaMemcpyAsync(grads, s->G.p, sizeof(float) * d.n_params * E, cudaMemcpyDeviceToHost, s->stream));
  SK(cudaStreamSynchronize(s->stream));
  if (loss)
    for (int e = 0; e < E; ++e) loss[e] = hl[e];
  return check_tc(s);
}

int abc_surrogate_get_params(abc_surrogate* s, float* params) {
  if (!s || !params) return ABC_ERR_INVALID;
  SK(cudaMemcpyAsync(params, s->P.p, sizeof(float) * s->d.n_params * s->members, cudaMemcpyDeviceToHost, s->stream));
  SK(cudaStreamSynchronize(s->stream));
  return ABC_OK;
}

int abc_surrogate_set_params(abc_surrogate* s, const float* params) {
  if (!s || !params) return ABC_ERR_INVALID;
  const int64_t n = s->d.n_params * s->members;
  SK(cudaMemcpyAsync(s->P.p, params, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
  SK(mlp_refresh_bf16(s->d, s->members, s->P.p, s->Ph.p, s->PhT.p, s->stream));
  SK(cudaStreamSynchronize(s->stream));
  return ABC_OK;
}

int abc_surrogate_get_norm(abc_surrogate* s, double* xmean, double* xstd, double* ymean, double* ystd) {
  if (!s) return ABC_ERR_INVALID;
  if (xmean) SK(cudaMemcpy(xmean, s->xm.p, sizeof(double) * s->d.in_dim, cudaMemcpyDeviceToHost));
  if (xstd) SK(cudaMemcpy(xstd, s->xs.p, sizeof(double) * s->d.in_dim, cudaMemcpyDeviceToHost));
  if (ymean) SK(cudaMemcpy(ymean, s->ym.p, sizeof(double) * s->d.K, cudaMemcpyDeviceToHost));
  if (ystd) SK(cudaMemcpy(ystd, s->ys.p, sizeof(double) * s->d.K, cudaMemcpyDeviceToHost));
  return ABC_OK;
}

int abc_surrogate_set_norm(abc_surrogate* s, const double* xmean, const double* xstd, const double* ymean,
                           const double* ystd) {
  if (!s || !xmean || !xstd || !ymean || !ystd) return ABC_ERR_INVALID;
  for (int i = 0; i < s->d.in_dim; ++i)
    if (!(xstd[i] > 0.0)) return sfail(s, ABC_ERR_INVALID, "xstd must be > 0");
  for (int k = 0; k < s->d.K; ++k)
    if (!(ystd[k] > 0.0)) return sfail(s, ABC_ERR_INVALID, "ystd must be > 0");
  SK(cudaMemcpy(s->xm.p, xmean, sizeof(double) * s->d.in_dim, cudaMemcpyHostToDevice));
  SK(cudaMemcpy(s->xs.p, xstd, sizeof(double) * s->d.in_dim, cudaMemcpyHostToDevice));
  SK(cudaMemcpy(s->ym.p, ymean, sizeof(double) * s->d.K, cudaMemcpyHostToDevice));
  SK(cudaMemcpy(s->ys.p, ystd, sizeof(double) * s->d.K, cudaMemcpyHostToDevice));
  d2f_kernel<<<1, 256, 0, s->stream>>>(s->ym.p, s->ymf.p, s->d.K);
  d2f_kernel<<<1, 256, 0, s->stream>>>(s->ys.p, s->ysf.p, s->d.K);
  SK(cudaMemsetAsync(s->yscf.p, 0, sizeof(float) * s->d.K, s->stream));  // identity target transform
  SK(cudaStreamSynchronize(s->stream));
  s->normed = true;
  return ABC_OK;
}

// predictions for device theta rows [0, N): mean, total variance (aleatoric +
// ensemble), disagreement = max_k sqrt(ensemble var / aleatoric var)
static int predict_chunk(abc_surrogate* s, const double* d_theta, int ld, int64_t n, double* d_mean, double* d_var,
                         double* d_dis, int aleatoric_only = 0) {
  const MlpDims& d = s->d;
  const int E = s->members;
  SK(s->X0.ensure((size_t)n * d.in_pad));
  SK(s->Ah.ensure((size_t)E * 3 * n * d.H));
  SK(s->Y.ensure((size_t)E * n * d.out_pad));
  norm_x_kernel<<<blocks(n * d.in_pad), 256, 0, s->stream>>>(d_theta, n, d.in_dim, ld, s->xm.p, s->xs.p, d.in_pad,
                                                              nullptr, s->X0.p);
  SK(cudaGetLastError());
  SK(mlp_forward(d, E, (int)n, s->X0.p, 0, s->PhT.p, s->P.p, nullptr, s->Ah.p, nullptr, 0, s->Y.p, s->tcerr.p,
                 s->stream));
  SK(mlp_combine(d, E, (int)n, s->Y.p, s->ymf.p, s->ysf.p, s->yscf.p, d_mean, d_var, d_dis, aleatoric_only,
                 s->stream));
  return ABC_OK;
}

int abc_surrogate_predict_device(abc_surrogate* s, const double* d_theta, int ld_theta, int64_t N, double* d_mean,
                                 double* d_var, double* d_disagree) {
  if (!s) return ABC_ERR_INVALID;
  if (!s->normed) return sfail(s, ABC_ERR_STATE, "surrogate not trained");
  if (!d_theta || N < 0 || ld_theta < s->d.in_dim) return sfail(s, ABC_ERR_INVALID, "bad arguments");
  for (int64_t p0 = 0; p0 < N; p0 += kPredChunk) {
    const int64_t n = std::min<int64_t>(kPredChunk, N - p0);
    int st = predict_chunk(s, d_theta + p0 * ld_theta, ld_theta, n, d_mean ? d_mean + p0 * s->d.K : nullptr,
                           d_var ? d_var + p0 * s->d.K : nullptr, d_disagree ? d_disagree + p0 : nullptr);
    if (st) return st;
  }
  SK(cudaStreamSynchronize(s->stream));
  return check_tc(s);
}

int abc_surrogate_predict(abc_surrogate* s, const double* theta, int64_t N, double* mean, double* var,
                          double* disagree) {
  if (!s) return ABC_ERR_INVALID;
  if (!theta || N < 1) return sfail(s, ABC_ERR_INVALID, "bad arguments");
  const int K = s->d.K;
  SK(s->th64.ensure((size_t)N * s->d.in_dim));
  SK(s->pm.ensure((size_t)N * K));
  SK(s->pv.ensure((size_t)N * K));
  SK(s->pd.ensure((size_t)N));
  SK(cudaMemcpyAsync(s->th64.p, theta, sizeof(double) * N * s->d.in_dim, cudaMemcpyHostToDevice, s->stream));
  int st = abc_surrogate_predict_device(s, s->th64.p, s->d.in_dim, N, s->pm.p, s->pv.p, s->pd.p);
  if (st) return st;
  if (mean) SK(cudaMemcpy(mean, s->pm.p, sizeof(double) * N * K, cudaMemcpyDeviceToHost));
  if (var) SK(cudaMemcpy(var, s->pv.p, sizeof(double) * N * K, cudaMemcpyDeviceToHost));
  if (disagree) SK(cudaMemcpy(disagree, s->pd.p, sizeof(double) * N, cudaMemcpyDeviceToHost));
  return ABC_OK;
}

// screen device theta rows; keep[p] = 1 for particles to simulate exactly.
// thr: per-gene error threshold; X = thr + margin.  err_out (optional, host,
// N x G): the predicted expected errors (for calibration on small sets).
int abc_surrogate_screen_device(abc_surrogate* s, const double* d_theta, int ld_theta, int64_t N, const double* data,
                                const double* se, int64_t G, const double* thr, double margin, double z,
                                double disagree_max, uint8_t* d_keep, int64_t* n_keep, double* err_out) {
  if (!s) return ABC_ERR_INVALID;
  if (!s->normed) return sfail(s, ABC_ERR_STATE, "surrogate not trained");
  const int K = s->d.K;
  if (!d_theta || !data || !se || !thr || !d_keep || N < 0 || G < 1 || ld_theta < s->d.in_dim)
    return sfail(s, ABC_ERR_INVALID, "abc_surrogate_screen: bad arguments");
  if (err_out && (double)N * (double)G > 2.5e8) return sfail(s, ABC_ERR_INVALID, "err_out only for N x G <= 2.5e8");
  SK(s->gd.ensure((size_t)G * K));
  SK(s->gs.ensure((size_t)G * K));
  SK(s->sw.ensure((size_t)G * K));
  SK(s->dw.ensure((size_t)G * K));
  SK(s->X.ensure((size_t)G));
  SK(cudaMemcpyAsync(s->gd.p, data, sizeof(double) * G * K, cudaMemcpyHostToDevice, s->stream));
  SK(cudaMemcpyAsync(s->gs.p, se, sizeof(double) * G * K, cudaMemcpyHostToDevice, s->stream));
  DistInputs in{};
  in.data = s->gd.p;
  in.se = s->gs.p;
  in.stats = nullptr;
  in.G = G;
  in.P = 0;
  in.K = K;
  in.n_fam = 1;
  in.fam[0] = K;
  SK(launch_dist_prep(in, s->sw.p, s->dw.p, nullptr, 0, 1, s->stream));
  std::vector<float> hx((size_t)G);
  for (int64_t g = 0; g < G; ++g) hx[g] = (float)(thr[g] + margin);
  SK(cudaMemcpyAsync(s->X.p, hx.data(), sizeof(float) * G, cudaMemcpyHostToDevice, s->stream));
  SK(cudaMemsetAsync(d_keep, 0, (size_t)N, s->stream));
  SK(s->pm.ensure((size_t)kPredChunk * K));
  SK(s->pv.ensure((size_t)kPredChunk * K));
  SK(s->pd.ensure((size_t)kPredChunk));
  SK(s->pmf.ensure((size_t)kPredChunk * K));
  SK(s->pvf.ensure((size_t)kPredChunk * K));
  Buf<float> eo;
  if (err_out) SK(eo.ensure((size_t)N * G));
  for (int64_t p0 = 0; p0 < N; p0 += kPredChunk) {
    const int64_t n = std::min<int64_t>(kPredChunk, N - p0);
    int st = predict_chunk(s, d_theta + p0 * ld_theta, ld_theta, n, s->pm.p, s->pv.p, s->pd.p, 0);
    if (st) return st;
    d2f_kernel<<<blocks(n * K), 256, 0, s->stream>>>(s->pm.p, s->pmf.p, n * K);
    d2f_kernel<<<blocks(n * K), 256, 0, s->stream>>>(s->pv.p, s->pvf.p, n * K);
    SK(launch_dist_screen(s->pmf.p, s->pvf.p, s->sw.p, s->dw.p, n, G, K, s->X.p, (float)z, s->screen_mode, d_keep + p0,
                          err_out ? eo.p + p0 * G : nullptr, s->stream));
    disagree_keep_kernel<<<blocks(n), 256, 0, s->stream>>>(s->pd.p, n, disagree_max, d_keep + p0);
    SK(cudaGetLastError());
  }
  SK(cudaMemsetAsync(s->cnt.p, 0, sizeof(unsigned long long), s->stream));
  count_keep_kernel<<<blocks(N), 256, 0, s->stream>>>(d_keep, N, s->cnt.p);
  unsigned long long hk = 0;
  SK(cudaMemcpyAsync(&hk, s->cnt.p, sizeof(hk), cudaMemcpyDeviceToHost, s->stream));
  if (err_out) {
    std::vector<float> tmp((size_t)N * G);
    SK(cudaMemcpyAsync(tmp.data(), eo.p, sizeof(float) * N * G, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    for (size_t i = 0; i < tmp.size(); ++i) err_out[i] = tmp[i];
  }
  SK(cudaStreamSynchronize(s->stream));
  eo.release();
  if (n_keep) *n_keep = (int64_t)hk;
  return check_tc(s);
}

// Rows with keep[p] != 0, in ascending order: theta rows copied to d_theta_out
// (row stride ld), their indices to d_idx_out (either may be NULL).  Uses the
// surrogate's stream and a scratch array of N/1024 counters.
int abc_surrogate_compact_device(abc_surrogate* s, const uint8_t* d_keep, const double* d_theta, int ld_theta,
                                 int64_t N, double* d_theta_out, int64_t* d_idx_out, int64_t* n_out) {
  if (!s) return ABC_ERR_INVALID;
  if (!d_keep || N < 0 || (d_theta_out && (!d_theta || ld_theta < 1)))
    return sfail(s, ABC_ERR_INVALID, "abc_surrogate_compact_device: bad arguments");
  if (N == 0) {
    if (n_out) *n_out = 0;
    return ABC_OK;
  }
  const int64_t nb = (N + kCompactRows - 1) / kCompactRows;
  Buf<unsigned int> counts;
  SK(counts.ensure((size_t)nb));
  compact_count_kernel<<<(unsigned)nb, kCompactRows, 0, s->stream>>>(d_keep, N, counts.p);
  compact_scan_kernel<<<1, 32, 0, s->stream>>>(counts.p, nb, s->cnt.p);
  compact_scatter_kernel<<<(unsigned)nb, kCompactRows, 0, s->stream>>>(d_keep, N, counts.p, d_theta, ld_theta,
                                                                       d_theta_out, d_idx_out);
  SK(cudaGetLastError());
  unsigned long long total = 0;
  SK(cudaMemcpyAsync(&total, s->cnt.p, sizeof(total), cudaMemcpyDeviceToHost, s->stream));
  SK(cudaStreamSynchronize(s->stream));
  counts.release();
  if (n_out) *n_out = (int64_t)total;
  return ABC_OK;
}

}  // extern "C"
