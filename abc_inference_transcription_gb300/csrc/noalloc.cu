// noalloc.cu — abc_simulate_noalloc: the simulate -> capture -> statistics
// chain without any device allocation by the library.
//
// Who needs it: callers that may not call cudaMalloc while they run, e.g. a
// host runtime that reserves all device memory up front in its own pool and
// forbids allocations afterwards, or code that must not trigger the implicit
// device synchronisation of cudaMalloc/cudaFree in a latency-critical loop.
// Such a caller cannot use abc_create (which allocates the context's
// buffers), so this entry point takes everything it needs as arguments and
// keeps its scratch -- particle records, per-cell counts, the work counter,
// the status word and the sorted cell table -- in one file-scope device array
// of fixed size (kNoAllocScratchBytes).  Every GPU that loads the library
// holds that array until the process exits.
//
// Host code must not use the array's name as a device address: it is only a
// host-side stand-in.  The first call on each device (with that device
// current) looks up the device address with cudaGetSymbolAddress.  The
// address is kept for the rest of the process: calls after a cudaDeviceReset of that device are not supported
// (the module, and with it the array, is reloaded at a new address).  All calls share the one array and
// it keeps the last call's contents: the counter, event totals and status
// word are cleared on every call, everything else is overwritten.  Calls that
// overlap on the GPU (other streams, other host threads) race on the array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/abcgpu.h"
#include "kernels.h"

using namespace abc;

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ABC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return ABC_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return ABC_OK;
}

int check_config(const abc_config* cfg) {
  if (!(cfg->cycle > 0.0) || !std::isfinite(cfg->cycle)) return ABC_ERR_INVALID;
  if (cfg->n_steps < 1 || cfg->n_steps > ABC_MAX_STEPS) return ABC_ERR_INVALID;
  if (cfg->n_ages < 1 || cfg->n_ages > ABC_MAX_AGES) return ABC_ERR_INVALID;
  if (cfg->n_conds < 1 || cfg->n_conds > ABC_MAX_CONDS) return ABC_ERR_INVALID;
  if (cfg->n_burn_cycles < 1) return ABC_ERR_INVALID;
  if (cfg->pulse_stat_cond < 0 || cfg->pulse_stat_cond >= cfg->n_conds || cfg->chase_stat_cond < 0 ||
      cfg->chase_stat_cond >= cfg->n_conds)
    return ABC_ERR_INVALID;
  if (cfg->precision != ABC_FP64 && cfg->precision != ABC_FP32) return ABC_ERR_INVALID;
  const double t0 = -(double)cfg->n_burn_cycles * cfg->cycle;
  for (int a = 0; a < cfg->n_ages; ++a)
    if (!(cfg->ages[a] > 0.0 && cfg->ages[a] < cfg->cycle)) return ABC_ERR_INVALID;
  for (int j = 0; j < cfg->n_conds; ++j) {
    if (!(cfg->pulse[j] > 0.0) || !(cfg->chase[j] >= 0.0)) return ABC_ERR_INVALID;
    for (int a = 0; a < cfg->n_ages; ++a)
      if (!((cfg->ages[a] - cfg->pulse[j]) - cfg->chase[j] > t0)) return ABC_ERR_INVALID;
  }
  return ABC_OK;
}

}  // namespace

extern "C" int abc_simulate_noalloc(const abc_config* cfg, int model, int64_t n_cells, const int32_t* cell_cond,
                                    const int32_t* cell_age, const double* cell_beta, const double* age_dist,
                                    const double* d_theta, int64_t P, uint64_t seed, int64_t particle_offset,
                                    double* d_stats, void* stream_ptr) {
  if (!cfg || check_config(cfg)) return ABC_ERR_INVALID;
  if (model < 1 || model > 5 || P < 0) return ABC_ERR_INVALID;
  if (particle_offset < 0 || particle_offset + P > (int64_t(1) << 32)) return ABC_ERR_INVALID;
  if (n_cells < 2 || n_cells > (int64_t(1) << 31) || !cell_cond || !cell_age || !cell_beta || !age_dist)
    return ABC_ERR_INVALID;
  if (P == 0) return ABC_OK;
  if (!d_theta || !d_stats) return ABC_ERR_INVALID;
  const int A = cfg->n_ages, J = cfg->n_conds, NG = A * J;
  const int64_t C = n_cells;

  // scratch layout (256-byte aligned parts); reject what does not fit
  size_t off = 0;
  const size_t o_misc = off;   off = align256(off + 4 * sizeof(unsigned long long) + sizeof(int));
  const size_t o_cond = off;   off = align256(off + sizeof(int32_t) * C);
  const size_t o_age = off;    off = align256(off + sizeof(int32_t) * C);
  const size_t o_id = off;     off = align256(off + sizeof(uint32_t) * C);
  const size_t o_beta = off;   off = align256(off + sizeof(double) * C);
  const size_t o_beta32 = off; off = align256(off + sizeof(float) * C);
  const size_t o_gs = off;     off = align256(off + sizeof(int32_t) * (NG + 1));
  const size_t o_w = off;      off = align256(off + sizeof(double) * NG);
  const size_t o_rec = off;    off = align256(off + sizeof(PRec) * (size_t)P);
  const size_t o_recf = off;   off = align256(off + sizeof(PRecF) * (size_t)P);
  const size_t o_cnt = off;
  if ((double)P * (double)C * (double)sizeof(int2) > (double)kNoAllocScratchBytes) return ABC_ERR_INVALID;
  off = align256(off + sizeof(int2) * (size_t)P * (size_t)C);
  if (off > kNoAllocScratchBytes) return ABC_ERR_INVALID;

  // cell table in group order (condition * A + age), as abc_set_cells keeps it
  std::vector<int64_t> count(NG, 0);
  for (int64_t i = 0; i < C; ++i) {
    if (cell_cond[i] < 0 || cell_cond[i] >= J || cell_age[i] < 0 || cell_age[i] >= A) return ABC_ERR_INVALID;
    if (!(cell_beta[i] >= 0.0 && cell_beta[i] <= 1.0)) return ABC_ERR_INVALID;
    count[cell_cond[i] * A + cell_age[i]]++;
  }
  for (int g = 0; g < NG; ++g)
    if (count[g] < 2 || !std::isfinite(age_dist[g])) return ABC_ERR_INVALID;
  std::vector<int64_t> perm(C);
  for (int64_t i = 0; i < C; ++i) perm[i] = i;
  std::stable_sort(perm.begin(), perm.end(), [&](int64_t x, int64_t y) {
    return cell_cond[x] * A + cell_age[x] < cell_cond[y] * A + cell_age[y];
  });
  std::vector<int32_t> hc(C), ha(C), gs(NG + 1, 0);
  std::vector<uint32_t> hid(C);
  std::vector<double> hb(C);
  for (int64_t i = 0; i < C; ++i) {
    const int64_t s = perm[i];
    hc[i] = cell_cond[s];
    ha[i] = cell_age[s];
    hid[i] = (uint32_t)s;
    hb[i] = cell_beta[s];
  }
  for (int g = 0; g < NG; ++g) gs[g + 1] = gs[g] + (int32_t)count[g];

  void* base = nullptr;
  int st = scratch_for_current_device(&base);
  if (st) return st;
  unsigned char* S = (unsigned char*)base;
  cudaStream_t stream = (cudaStream_t)stream_ptr;
  unsigned long long* misc = (unsigned long long*)(S + o_misc);
  int* status = (int*)(S + o_misc + 4 * sizeof(unsigned long long));
  int32_t* d_cond = (int32_t*)(S + o_cond);
  int32_t* d_age = (int32_t*)(S + o_age);
  uint32_t* d_id = (uint32_t*)(S + o_id);
  double* d_beta = (double*)(S + o_beta);
  float* d_beta32 = (float*)(S + o_beta32);
  int32_t* d_gs = (int32_t*)(S + o_gs);
  double* d_w = (double*)(S + o_w);
  PRec* d_rec = (PRec*)(S + o_rec);
  PRecF* d_recf = (PRecF*)(S + o_recf);
  int2* d_cnt = (int2*)(S + o_cnt);

#define NA_CK(call)                              \
  do {                                           \
    if ((call) != cudaSuccess) return ABC_ERR_CUDA; \
  } while (0)
  NA_CK(cudaMemcpyAsync(d_cond, hc.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice, stream));
  NA_CK(cudaMemcpyAsync(d_age, ha.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice, stream));
  NA_CK(cudaMemcpyAsync(d_id, hid.data(), sizeof(uint32_t) * C, cudaMemcpyHostToDevice, stream));
  NA_CK(cudaMemcpyAsync(d_beta, hb.data(), sizeof(double) * C, cudaMemcpyHostToDevice, stream));
  std::vector<float> hb32(hb.begin(), hb.end());
  NA_CK(cudaMemcpyAsync(d_beta32, hb32.data(), sizeof(float) * C, cudaMemcpyHostToDevice, stream));
  NA_CK(cudaMemcpyAsync(d_gs, gs.data(), sizeof(int32_t) * (NG + 1), cudaMemcpyHostToDevice, stream));
  NA_CK(cudaMemcpyAsync(d_w, age_dist, sizeof(double) * NG, cudaMemcpyHostToDevice, stream));
  // what must start at zero: work counter, event totals, status word
  NA_CK(cudaMemsetAsync(misc, 0, 4 * sizeof(unsigned long long) + sizeof(int), stream));

  DevCfg d;
  memset(&d, 0, sizeof(d));
  d.cycle = cfg->cycle;
  d.step_len = cfg->cycle / (double)cfg->n_steps;
  d.t0 = -(double)cfg->n_burn_cycles * cfg->cycle;
  for (int a = 0; a < ABC_MAX_AGES; ++a) d.ages[a] = cfg->ages[a];
  for (int j = 0; j < ABC_MAX_CONDS; ++j) {
    d.pulse[j] = cfg->pulse[j];
    d.chase[j] = cfg->chase[j];
  }
  d.event_cap = cfg->event_cap;
  d.n_steps = cfg->n_steps;
  d.n_ages = A;
  d.n_conds = J;
  d.splicing = cfg->splicing ? 1 : 0;
  d.scaling_column = cfg->scaling_column ? 1 : 0;
  d.pulse_stat = cfg->pulse_stat_cond;
  d.chase_stat = cfg->chase_stat_cond;
  d.npar = 5 + (model >= 3 ? cfg->n_steps - 1 : 0) + d.splicing + d.scaling_column;
  dcfg_set_grid(d);

  SetupArgs sa;
  sa.cfg = d;
  sa.model = model;
  sa.models = nullptr;
  sa.ld_theta = d.npar;
  sa.theta = d_theta;
  sa.n_particles = P;
  sa.rec = d_rec;
  sa.recf = d_recf;
  sa.status = status;
  sa.fp32 = cfg->precision == ABC_FP32 ? 1 : 0;
  NA_CK(launch_setup(sa, stream));

  int dev = 0, sms = 0;
  NA_CK(cudaGetDevice(&dev));
  NA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const bool fp64 = cfg->precision == ABC_FP64;
  const int bps = std::max(1, fp64 ? ssa_blocks_per_sm_fp64() : ssa_blocks_per_sm_fp32());
  SsaArgs ss;
  ss.cfg = d;
  ss.rec = d_rec;
  ss.recf = d_recf;
  ss.cell_cond = d_cond;
  ss.cell_age = d_age;
  ss.cell_id = d_id;
  ss.order = nullptr;
  ss.n_cells = C;
  ss.n_items = P * C;
  ss.p_offset = particle_offset;
  ss.seed = seed;
  ss.counts = d_cnt;
  ss.events = nullptr;
  ss.hash = nullptr;
  ss.counter = misc;
  ss.totals = misc + 1;
  ss.status = status;
  ss.want_hash = 0;
  int64_t grid = std::min<int64_t>((int64_t)bps * sms, (ss.n_items + 127) / 128);
  grid = std::max<int64_t>(grid, 1);
  // the production kernel takes each trajectory's initial state from the count array
  if (!fp64) NA_CK(launch_init_states(ss, sms, stream));
  NA_CK(fp64 ? launch_ssa_fp64(ss, (int)grid, stream) : launch_ssa_fp32(ss, (int)grid, stream));

  StatsArgs sta;
  sta.cfg = d;
  sta.counts = d_cnt;
  sta.beta = d_beta;
  sta.cell_id = d_id;
  sta.gstart = d_gs;
  sta.age_dist = d_w;
  sta.n_cells = C;
  sta.n_particles = P;
  sta.p_offset = particle_offset;
  sta.seed = seed;
  sta.stats = d_stats;
  sta.captured = nullptr;
  sta.fp32 = fp64 ? 0 : 1;
  sta.beta32 = d_beta32;
  sta.max_group_cells = *std::max_element(count.begin(), count.end());
  NA_CK(launch_stats(sta, stream));

  int hs = 0;
  NA_CK(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  NA_CK(cudaStreamSynchronize(stream));
#undef NA_CK
  if (hs & STF_EVENT_CAP) return ABC_ERR_EVENT_CAP;
  if (hs & (STF_OVERFLOW | STF_NONFINITE)) return ABC_ERR_NONFINITE;
  return ABC_OK;
}
