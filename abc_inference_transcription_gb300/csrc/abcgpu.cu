// abcgpu.cu — the C ABI (include/abcgpu.h): context, device memory, stream,
// and the host-side orchestration of the kernels.  No compute happens on the
// host; without a CUDA device every call fails with ABC_ERR_CUDA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/abcgpu.h"
#include "distance.cuh"
#include "kernels.h"

using namespace abc;

namespace {

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;  // elements
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// counts buffer budget per simulate chunk: 10^6 particles x 2,000 cells run as
// one persistent launch (16 GB of the GB300's HBM), so the heaviest
// trajectories of the whole batch start first
constexpr size_t kChunkBytes = size_t(16) << 30;
// the production kernel's work cursor is 32-bit: items (particles x cells) per launch below 2^31
constexpr int64_t kMaxItemsPerLaunch = (int64_t(1) << 31) - 1;
// work chunks (consecutive items per lane per pull) the batch autotuner times
constexpr int kTuneChunks[] = {1, 4, 16};
constexpr int kNumTuneChunks = 3;

}  // namespace

struct abc_ctx {
  abc_config cfg;
  DevCfg dcfg;
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // cells, internal order = sorted by group (cond*A + age)
  bool cells_set = false;
  int64_t C = 0;
  std::vector<int64_t> perm;  // internal -> caller index
  DBuf<int32_t> d_cond, d_age, d_gstart;
  DBuf<uint32_t> d_id;
  DBuf<double> d_beta, d_age_dist;
  DBuf<float> d_beta32;  // capture efficiencies in FP32 for the production mode's capture
  int64_t max_group_cells = INT64_MAX;  // cells of the largest (condition, age) group
  // simulation workspace
  DBuf<double> d_theta, d_stats;
  DBuf<int32_t> d_models;
  DBuf<uint32_t> d_order, d_ohist;  // work order (heaviest particles first) and its counting-sort scratch
  DBuf<PRec> d_rec;
  DBuf<PRecF> d_recf;
  DBuf<int2> d_counts, d_captured;
  DBuf<int64_t> d_events;
  DBuf<uint64_t> d_hash;
  DBuf<unsigned long long> d_misc;  // [0] work counter, [1] events, [2] rejections
  DBuf<int> d_status;
  int64_t last_events = 0, last_rej = 0;
  int variant = 0;  // production SSA kernel variant chosen by abc_autotune
  int work_chunk = 1;  // items a lane takes per pull of the production kernel (abc_set_work_chunk)
  bool graph_mode = false;           // simulate chain as a CUDA graph (abc_set_graph)
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_instantiations = 0, graph_updates = 0;
  // per-phase device timing (abc_profile): 4 events per chunk
  bool prof = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double phase_ms[3] = {0, 0, 0};
  // selection workspace and results
  DBuf<double> d_data, d_se, d_sel_stats, d_se64, d_out_err, d_den, d_rden;
  DBuf<float> d_sw, d_dw, d_s32, d_X, d_esub;
  DBuf<Cand> d_cand;
  DBuf<float> d_cande;  // FP32 error of each candidate
  // tensor-core candidate pass: operands, per-gene terms, per-CTA output segments
  int dist_mode = 3;       // 0 FP32 CUDA cores, 1 TF32 one-term, 2 TF32 three-term, 3 BF16 three-term
  int dist_mode_used = -1;
  DBuf<float> d_tcA, d_tcB, d_cg32, d_b0, d_Y, d_Xt, d_seg_e;
  DBuf<uint8_t> d_rowbad;  // per particle of the candidate pass: a statistic is NaN
  DBuf<double> d_cg64;
  DBuf<unsigned> d_tcflags, d_segcount, d_hist;
  DBuf<int> d_tcerr;
  DBuf<Cand> d_seg, d_cand2;
  int64_t seg_cap = int64_t(1) << 16;
  DBuf<int32_t> d_sp, d_sg;
  DBuf<int64_t> d_gcount, d_goff, d_alen, d_aoff, d_out_idx;
  DBuf<unsigned long long> d_gcursor, d_ncand;
  DBuf<int> d_fail;
  DBuf<double> d_thr;
  cudaEvent_t sel_ev[2] = {nullptr, nullptr};
  double sel_fast_ms = 0.0;  // candidate-pass kernel time of the last selection (abc_profile)
  int sel_fast_passes = 0;
  int64_t cand_cap = int64_t(1) << 22;
  int64_t sel_G = 0, sel_P = 0, sel_total = 0, sel_cands = 0, sel_rechecked = 0, sel_cands_emitted = 0;
  bool sel_ready = false;
  bool sel_errors = true;        // selections keep the FP64 error of every accepted pair
  bool sel_errors_exact = true;  // the last selection's stored errors are FP64
  DistInputs sel_in;             // inputs of the last selection (device buffers; stats as given)
  DBuf<int32_t> d_asp, d_asg;    // accepted pairs for abc_accept_errors
  DBuf<double> d_aerr;
  DBuf<float4> d_ffg;
  DBuf<int32_t> d_pos;
  DBuf<uint8_t> d_flag;
  DBuf<unsigned long long> d_cnt2;
  DBuf<int> d_dirty;
};

static int fail(abc_ctx* c, int status, const std::string& msg) {
  if (c) c->err = msg;
  return status;
}

static int cuda_fail(abc_ctx* c, cudaError_t e, const char* where) {
  return fail(c, e == cudaErrorMemoryAllocation ? ABC_ERR_NOMEM : ABC_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
  } while (0)

static int validate_config(const abc_config* cfg, std::string& msg) {
  if (!(cfg->cycle > 0.0) || !std::isfinite(cfg->cycle)) return msg = "cycle must be > 0", ABC_ERR_INVALID;
  if (cfg->n_steps < 1 || cfg->n_steps > ABC_MAX_STEPS) return msg = "n_steps out of range", ABC_ERR_INVALID;
  if (cfg->n_ages < 1 || cfg->n_ages > ABC_MAX_AGES) return msg = "n_ages out of range", ABC_ERR_INVALID;
  if (cfg->n_conds < 1 || cfg->n_conds > ABC_MAX_CONDS) return msg = "n_conds out of range", ABC_ERR_INVALID;
  if (cfg->n_burn_cycles < 1) return msg = "n_burn_cycles must be >= 1", ABC_ERR_INVALID;
  if (cfg->pulse_stat_cond < 0 || cfg->pulse_stat_cond >= cfg->n_conds || cfg->chase_stat_cond < 0 ||
      cfg->chase_stat_cond >= cfg->n_conds)
    return msg = "pulse/chase statistic condition out of range", ABC_ERR_INVALID;
  if (cfg->precision != ABC_FP64 && cfg->precision != ABC_FP32) return msg = "bad precision", ABC_ERR_INVALID;
  const double t0 = -(double)cfg->n_burn_cycles * cfg->cycle;
  for (int a = 0; a < cfg->n_ages; ++a)
    if (!(cfg->ages[a] > 0.0 && cfg->ages[a] < cfg->cycle)) return msg = "ages must lie in (0, cycle)", ABC_ERR_INVALID;
  for (int j = 0; j < cfg->n_conds; ++j) {
    if (!(cfg->pulse[j] > 0.0) || !(cfg->chase[j] >= 0.0)) return msg = "pulse must be > 0, chase >= 0", ABC_ERR_INVALID;
    for (int a = 0; a < cfg->n_ages; ++a) {
      double texp = (cfg->ages[a] - cfg->pulse[j]) - cfg->chase[j];
      if (!(texp > t0)) return msg = "labelling starts before the simulated horizon", ABC_ERR_INVALID;
    }
  }
  return ABC_OK;
}

static DevCfg make_dcfg(const abc_config* cfg) {
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
  d.n_ages = cfg->n_ages;
  d.n_conds = cfg->n_conds;
  d.splicing = cfg->splicing ? 1 : 0;
  d.scaling_column = cfg->scaling_column ? 1 : 0;
  d.pulse_stat = cfg->pulse_stat_cond;
  d.chase_stat = cfg->chase_stat_cond;
  d.npar = 0;
  dcfg_set_grid(d);
  return d;
}

static int npar_of(const abc_config* cfg, int model) {
  if (model < 1 || model > 5) return ABC_ERR_INVALID;
  return 5 + (model >= 3 ? cfg->n_steps - 1 : 0) + (cfg->splicing ? 1 : 0) + (cfg->scaling_column ? 1 : 0);
}

extern "C" {

int abc_create(abc_ctx** out, const abc_config* cfg) {
  if (!out || !cfg) return ABC_ERR_INVALID;
  *out = nullptr;
  std::string msg;
  int st = validate_config(cfg, msg);
  if (st) {
    fprintf(stderr, "abc_create: %s\n", msg.c_str());
    return st;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ABC_ERR_CUDA;
  abc_ctx* c = new (std::nothrow) abc_ctx();
  if (!c) return ABC_ERR_NOMEM;
  c->cfg = *cfg;
  c->dcfg = make_dcfg(cfg);
  c->device = dev;
  if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return ABC_ERR_CUDA;
  }
  if (c->d_misc.ensure(4) || c->d_status.ensure(1)) {
    cudaStreamDestroy(c->stream);
    delete c;
    return ABC_ERR_NOMEM;
  }
  *out = c;
  return ABC_OK;
}

int abc_destroy(abc_ctx* c) {
  if (!c) return ABC_OK;
  cudaStreamSynchronize(c->stream);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->d_cond.release(); c->d_age.release(); c->d_gstart.release(); c->d_id.release();
  c->d_beta.release(); c->d_beta32.release(); c->d_age_dist.release(); c->d_theta.release(); c->d_stats.release();
  c->d_models.release(); c->d_order.release(); c->d_ohist.release(); c->d_rec.release(); c->d_recf.release(); c->d_counts.release(); c->d_captured.release();
  c->d_events.release(); c->d_hash.release(); c->d_misc.release(); c->d_status.release();
  c->d_data.release(); c->d_se.release(); c->d_sel_stats.release(); c->d_se64.release(); c->d_sg.release();
  c->d_ffg.release(); c->d_pos.release(); c->d_flag.release(); c->d_cnt2.release();
  c->d_dirty.release();
  c->d_out_err.release(); c->d_sw.release(); c->d_dw.release(); c->d_s32.release(); c->d_X.release();
  c->d_esub.release(); c->d_cand.release(); c->d_sp.release(); c->d_gcount.release(); c->d_goff.release();
  c->d_cande.release(); c->d_den.release(); c->d_rden.release(); c->d_tcA.release(); c->d_tcB.release(); c->d_rowbad.release(); c->d_cg32.release(); c->d_b0.release();
  c->d_Y.release(); c->d_Xt.release(); c->d_seg_e.release(); c->d_cg64.release(); c->d_tcflags.release();
  c->d_segcount.release(); c->d_hist.release(); c->d_tcerr.release(); c->d_seg.release(); c->d_cand2.release();
  c->d_alen.release(); c->d_aoff.release(); c->d_out_idx.release(); c->d_gcursor.release();
  c->d_ncand.release(); c->d_fail.release(); c->d_thr.release();
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : c->sel_ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
  return ABC_OK;
}

const char* abc_last_error(const abc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int abc_breakpoint_grid(const abc_config* cfg, double* quantum) {
  if (!cfg) return ABC_ERR_INVALID;
  std::string msg;
  const int st = validate_config(cfg, msg);
  if (st) return st;
  const DevCfg d = make_dcfg(cfg);
  if (quantum) *quantum = d.grid_ok ? (double)d.quantum : 0.0;
  return d.grid_ok ? 1 : 0;
}

int abc_num_params(const abc_ctx* c, int model) {
  if (!c) return ABC_ERR_INVALID;
  return npar_of(&c->cfg, model);
}

int abc_num_stats(const abc_ctx* c) {
  if (!c) return ABC_ERR_INVALID;
  return ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
}

void* abc_stream(abc_ctx* c) { return c ? (void*)c->stream : nullptr; }

int abc_set_cells(abc_ctx* c, int64_t n_cells, const int32_t* cell_cond, const int32_t* cell_age,
                  const double* cell_beta, const double* age_dist) {
  if (!c) return ABC_ERR_INVALID;
  if (n_cells < 2 || n_cells > (int64_t(1) << 31) || !cell_cond || !cell_age || !cell_beta || !age_dist)
    return fail(c, ABC_ERR_INVALID, "abc_set_cells: bad arguments");
  const int A = c->cfg.n_ages, J = c->cfg.n_conds, NG = A * J;
  std::vector<int64_t> count(NG, 0);
  for (int64_t i = 0; i < n_cells; ++i) {
    if (cell_cond[i] < 0 || cell_cond[i] >= J || cell_age[i] < 0 || cell_age[i] >= A)
      return fail(c, ABC_ERR_INVALID, "abc_set_cells: condition or age group out of range");
    if (!(cell_beta[i] >= 0.0 && cell_beta[i] <= 1.0))
      return fail(c, ABC_ERR_INVALID, "abc_set_cells: capture efficiency outside [0, 1]");
    count[cell_cond[i] * A + cell_age[i]]++;
  }
  for (int g = 0; g < NG; ++g)
    if (count[g] < 2) return fail(c, ABC_ERR_INVALID, "abc_set_cells: every (condition, age) group needs >= 2 cells");
  for (int i = 0; i < NG; ++i)
    if (!std::isfinite(age_dist[i])) return fail(c, ABC_ERR_INVALID, "abc_set_cells: non-finite weight");
  std::vector<int64_t> perm(n_cells);
  for (int64_t i = 0; i < n_cells; ++i) perm[i] = i;
  std::stable_sort(perm.begin(), perm.end(), [&](int64_t x, int64_t y) {
    return cell_cond[x] * A + cell_age[x] < cell_cond[y] * A + cell_age[y];
  });
  std::vector<int32_t> hc(n_cells), ha(n_cells), gs(NG + 1, 0);
  std::vector<uint32_t> hid(n_cells);
  std::vector<double> hb(n_cells);
  for (int64_t i = 0; i < n_cells; ++i) {
    int64_t s = perm[i];
    hc[i] = cell_cond[s];
    ha[i] = cell_age[s];
    hid[i] = (uint32_t)s;
    hb[i] = cell_beta[s];
  }
  for (int g = 0; g < NG; ++g) gs[g + 1] = gs[g] + (int32_t)count[g];
  CK(cudaStreamSynchronize(c->stream));
  CK(c->d_cond.ensure(n_cells));
  CK(c->d_age.ensure(n_cells));
  CK(c->d_id.ensure(n_cells));
  CK(c->d_beta.ensure(n_cells));
  CK(c->d_beta32.ensure(n_cells));
  CK(c->d_gstart.ensure(NG + 1));
  CK(c->d_age_dist.ensure(NG));
  CK(cudaMemcpy(c->d_cond.p, hc.data(), sizeof(int32_t) * n_cells, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_age.p, ha.data(), sizeof(int32_t) * n_cells, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_id.p, hid.data(), sizeof(uint32_t) * n_cells, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_beta.p, hb.data(), sizeof(double) * n_cells, cudaMemcpyHostToDevice));
  std::vector<float> hb32(hb.begin(), hb.end());
  CK(cudaMemcpy(c->d_beta32.p, hb32.data(), sizeof(float) * n_cells, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_gstart.p, gs.data(), sizeof(int32_t) * (NG + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_age_dist.p, age_dist, sizeof(double) * NG, cudaMemcpyHostToDevice));
  c->perm = perm;
  c->C = n_cells;
  c->max_group_cells = 0;
  for (int g = 0; g < NG; ++g) c->max_group_cells = std::max<int64_t>(c->max_group_cells, gs[g + 1] - gs[g]);
  c->cells_set = true;
  return ABC_OK;
}

static int sample_prior_impl(abc_ctx* c, int model, int64_t P, uint64_t seed, int64_t particle_offset,
                             const abc_prior* prior, double* theta_out, bool device_out) {
  if (!c) return ABC_ERR_INVALID;
  const int npar = npar_of(&c->cfg, model);
  if (npar < 0 || P < 0 || !prior || (!theta_out && P > 0)) return fail(c, ABC_ERR_INVALID, "abc_sample_prior: bad arguments");
  if (particle_offset < 0 || particle_offset + P > (int64_t(1) << 32))
    return fail(c, ABC_ERR_INVALID, "abc_sample_prior: particle index beyond 2^32");
  if (P == 0) return ABC_OK;
  if (prior->vary_mode == 1 && !(prior->factor[0] > 0.0 && prior->factor[1] > 0.0))
    return fail(c, ABC_ERR_INVALID, "abc_sample_prior: factor bounds must be > 0");
  if (c->cfg.scaling_column && !(prior->scaling[0] > 0.0 && prior->scaling[1] > 0.0))
    return fail(c, ABC_ERR_INVALID, "abc_sample_prior: scaling bounds must be > 0");
  PriorArgs a;
  a.cfg = c->dcfg;
  a.cfg.npar = npar;
  a.model = model;
  a.n_particles = P;
  a.p_offset = particle_offset;
  a.seed = seed;
  const double* src[6] = {prior->kon, prior->koff, prior->alpha, prior->gamma, prior->lambda, prior->beta};
  for (int i = 0; i < 6; ++i) {
    a.lo[i] = src[i][0];
    a.hi[i] = src[i][1];
  }
  a.lo[6] = c->cfg.scaling_column ? xlog(prior->scaling[0]) / ABC_LN10 : 0.0;
  a.hi[6] = c->cfg.scaling_column ? xlog(prior->scaling[1]) / ABC_LN10 : 0.0;
  a.vary_mode = prior->vary_mode;
  a.lf0 = prior->vary_mode == 1 ? xlog(prior->factor[0]) / ABC_LN10 : 0.0;
  a.lf1 = prior->vary_mode == 1 ? xlog(prior->factor[1]) / ABC_LN10 : 0.0;
  if (device_out) {
    a.theta = theta_out;
    CK(launch_prior(a, c->stream));
    return ABC_OK;
  }
  CK(c->d_theta.ensure((size_t)P * npar));
  a.theta = c->d_theta.p;
  CK(launch_prior(a, c->stream));
  CK(cudaMemcpyAsync(theta_out, c->d_theta.p, sizeof(double) * P * npar, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ABC_OK;
}

int abc_sample_prior(abc_ctx* c, int model, int64_t P, uint64_t seed, int64_t particle_offset,
                     const abc_prior* prior, double* theta_out) {
  return sample_prior_impl(c, model, P, seed, particle_offset, prior, theta_out, false);
}

int abc_sample_prior_device(abc_ctx* c, int model, int64_t P, uint64_t seed, int64_t particle_offset,
                            const abc_prior* prior, double* d_theta_out) {
  return sample_prior_impl(c, model, P, seed, particle_offset, prior, d_theta_out, true);
}

// Enqueue setup -> SSA -> capture/statistics for particles [0, P) of
// d_theta (device), writing d_stats (device).  Chunked so that the per-cell
// counts stay within kChunkBytes.
static int npar_max(const abc_config* cfg) { return npar_of(cfg, 3); }

static cudaError_t prof_mark(abc_ctx* c) {
  if (!c->prof) return cudaSuccess;
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    c->ev_pool.push_back(e);
  }
  return cudaEventRecord(c->ev_pool[c->ev_used++], c->stream);
}

// device workspace of a simulation of P particles, processed in chunks that
// keep the per-cell count buffer under kChunkBytes
static int prepare_simulate(abc_ctx* c, int64_t P, bool want_cells, int64_t* chunk_out) {
  const int64_t C = c->C;
  int64_t chunk = std::max<int64_t>(1, (int64_t)(kChunkBytes / (sizeof(int2) * (size_t)C)));
  chunk = std::min<int64_t>(chunk, std::max<int64_t>(1, kMaxItemsPerLaunch / std::max<int64_t>(C, 1)));
  if (want_cells) chunk = P;  // per-cell outputs are requested for small P only
  chunk = std::min<int64_t>(chunk, std::max<int64_t>(P, 1));
  CK(c->d_rec.ensure(chunk));
  CK(c->d_recf.ensure(chunk));
  CK(c->d_order.ensure(chunk));
  CK(c->d_ohist.ensure(128));
  CK(c->d_counts.ensure((size_t)chunk * C));
  if (want_cells) {
    CK(c->d_captured.ensure((size_t)chunk * C));
    CK(c->d_events.ensure((size_t)chunk * C));
    CK(c->d_hash.ensure((size_t)chunk * C));
  }
  *chunk_out = chunk;
  return ABC_OK;
}

static int enqueue_simulate(abc_ctx* c, int model, const int32_t* d_models, const double* d_theta, int64_t ld,
                            int64_t P, uint64_t seed, int64_t p_offset, double* d_stats, bool want_cells) {
  const int npar = d_models ? npar_max(&c->cfg) : npar_of(&c->cfg, model);
  const int K = ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
  const int64_t C = c->C;
  int64_t chunk = 0;
  int pst = prepare_simulate(c, P, want_cells, &chunk);
  if (pst) return pst;
  CK(cudaMemsetAsync(c->d_misc.p, 0, sizeof(unsigned long long) * 4, c->stream));
  CK(cudaMemsetAsync(c->d_status.p, 0, sizeof(int), c->stream));
  c->ev_used = 0;
  const bool fp64 = c->cfg.precision == ABC_FP64;
  const int bps = fp64 ? ssa_blocks_per_sm_fp64() : ssa_blocks_per_sm_fp32(c->variant);
  for (int64_t p0 = 0; p0 < P; p0 += chunk) {
    const int64_t n = std::min(chunk, P - p0);
    SetupArgs sa;
    sa.cfg = c->dcfg;
    sa.cfg.npar = npar;
    sa.model = model;
    sa.models = d_models ? d_models + p0 : nullptr;
    sa.ld_theta = ld;
    sa.theta = d_theta + p0 * ld;
    sa.n_particles = n;
    sa.rec = c->d_rec.p;
    sa.recf = c->d_recf.p;
    sa.status = c->d_status.p;
    sa.fp32 = fp64 ? 0 : 1;
    CK(prof_mark(c));
    CK(launch_setup(sa, c->stream));
    CK(launch_work_order(c->d_rec.p, n, c->d_ohist.p, c->d_order.p, c->stream));
    SsaArgs ss;
    ss.cfg = sa.cfg;
    ss.rec = c->d_rec.p;
    ss.recf = c->d_recf.p;
    ss.cell_cond = c->d_cond.p;
    ss.cell_age = c->d_age.p;
    ss.cell_id = c->d_id.p;
    ss.order = c->d_order.p;
    ss.n_cells = C;
    ss.n_items = n * C;
    ss.p_offset = p_offset + p0;
    ss.seed = seed;
    ss.counts = c->d_counts.p;
    ss.events = want_cells ? c->d_events.p : nullptr;
    ss.hash = want_cells ? c->d_hash.p : nullptr;
    ss.counter = c->d_misc.p;
    ss.totals = c->d_misc.p + 1;
    ss.status = c->d_status.p;
    ss.want_hash = want_cells ? 1 : 0;
    ss.chunk = c->work_chunk;
    // production mode: the trajectories' initial states, drawn in FP64 before the SSA
    if (!fp64) CK(launch_init_states(ss, c->sms, c->stream));
    CK(prof_mark(c));
    CK(cudaMemsetAsync(c->d_misc.p, 0, sizeof(unsigned long long), c->stream));
    const int64_t warps_needed = (ss.n_items + 31) / 32;
    int64_t grid = (int64_t)std::max(1, bps) * c->sms;
    grid = std::min<int64_t>(grid, (warps_needed + 3) / 4);
    grid = std::max<int64_t>(grid, 1);
    CK(fp64 ? launch_ssa_fp64(ss, (int)grid, c->stream) : launch_ssa_fp32(ss, (int)grid, c->stream, c->variant));
    CK(prof_mark(c));
    StatsArgs st;
    st.cfg = sa.cfg;
    st.counts = c->d_counts.p;
    st.beta = c->d_beta.p;
    st.cell_id = c->d_id.p;
    st.gstart = c->d_gstart.p;
    st.age_dist = c->d_age_dist.p;
    st.n_cells = C;
    st.n_particles = n;
    st.p_offset = p_offset + p0;
    st.seed = seed;
    st.stats = d_stats + p0 * K;
    st.captured = want_cells ? c->d_captured.p : nullptr;
    st.fp32 = fp64 ? 0 : 1;
    st.beta32 = c->d_beta32.p;
    st.max_group_cells = c->max_group_cells;
    CK(launch_stats(st, c->stream));
    CK(prof_mark(c));
  }
  return ABC_OK;
}

static int check_sim_args(abc_ctx* c, int model, int64_t P, int64_t particle_offset) {
  if (!c->cells_set) return fail(c, ABC_ERR_STATE, "abc_set_cells must be called before simulating");
  if (npar_of(&c->cfg, model) < 0) return fail(c, ABC_ERR_INVALID, "model must be 1..5");
  if (P < 0) return fail(c, ABC_ERR_INVALID, "negative particle count");
  if (particle_offset < 0 || particle_offset + P > (int64_t(1) << 32))
    return fail(c, ABC_ERR_INVALID, "particle index beyond 2^32");
  return ABC_OK;
}

static int finish_status(abc_ctx* c) {
  int hs = 0;
  unsigned long long tot[3] = {0, 0, 0};
  CK(cudaMemcpyAsync(&hs, c->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(tot, c->d_misc.p, sizeof(tot), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->last_events = (int64_t)tot[1];
  c->last_rej = (int64_t)tot[2];
  if (c->prof) {
    c->phase_ms[0] = c->phase_ms[1] = c->phase_ms[2] = 0.0;
    for (size_t i = 0; i + 3 < c->ev_used; i += 4) {
      for (int ph = 0; ph < 3; ++ph) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c->ev_pool[i + ph], c->ev_pool[i + ph + 1]));
        c->phase_ms[ph] += ms;
      }
    }
  }
  c->ev_used = 0;
  if (hs & STF_EVENT_CAP) return fail(c, ABC_ERR_EVENT_CAP, "a trajectory exceeded the event cap");
  if (hs & (STF_OVERFLOW | STF_NONFINITE))
    return fail(c, ABC_ERR_NONFINITE, "non-finite rate or molecule count overflow");
  return ABC_OK;
}

// The simulate -> capture -> statistics chain, as one CUDA graph when graph
// mode is on: the chain is captured on the context's stream, the instantiated
// graph is updated in place (new seed, pointers) when its topology is
// unchanged, re-instantiated otherwise, and launched once.  Workspace is
// grown before the capture (no allocation inside it); profiling events are
// not recorded inside the graph.
static int enqueue_chain(abc_ctx* c, int model, const int32_t* d_models, const double* d_theta, int64_t ld, int64_t P,
                         uint64_t seed, int64_t p_offset, double* d_stats) {
  if (!c->graph_mode) return enqueue_simulate(c, model, d_models, d_theta, ld, P, seed, p_offset, d_stats, false);
  int64_t chunk = 0;
  int st = prepare_simulate(c, P, false, &chunk);
  if (st) return st;
  const bool prof = c->prof;
  c->prof = false;
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    c->prof = prof;
    return cuda_fail(c, e, "cudaStreamBeginCapture");
  }
  st = enqueue_simulate(c, model, d_models, d_theta, ld, P, seed, p_offset, d_stats, false);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
  c->prof = prof;
  if (st || ec != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return st ? st : cuda_fail(c, ec, "cudaStreamEndCapture");
  }
  if (c->gexec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(c->gexec, g, &info) != cudaSuccess) {
      (void)cudaGetLastError();
      cudaGraphExecDestroy(c->gexec);
      c->gexec = nullptr;
    } else {
      c->graph_updates++;
    }
  }
  if (!c->gexec) {
    e = cudaGraphInstantiate(&c->gexec, g, 0);
    if (e != cudaSuccess) {
      c->gexec = nullptr;
      cudaGraphDestroy(g);
      return cuda_fail(c, e, "cudaGraphInstantiate");
    }
    c->graph_instantiations++;
  }
  e = cudaGraphLaunch(c->gexec, c->stream);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphLaunch");
  return ABC_OK;
}

int abc_set_graph(abc_ctx* c, int enable) {
  if (!c) return ABC_ERR_INVALID;
  c->graph_mode = enable != 0;
  return ABC_OK;
}

int abc_graph_counters(const abc_ctx* c, int64_t* instantiations, int64_t* updates) {
  if (!c) return ABC_ERR_INVALID;
  if (instantiations) *instantiations = c->graph_instantiations;
  if (updates) *updates = c->graph_updates;
  return ABC_OK;
}

int abc_simulate_device(abc_ctx* c, int model, const double* d_theta, int64_t P, uint64_t seed,
                        int64_t particle_offset, double* d_stats) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, model, P, particle_offset);
  if (st) return st;
  if (P == 0) return ABC_OK;
  if (!d_theta || !d_stats) return fail(c, ABC_ERR_INVALID, "null device pointer");
  return enqueue_chain(c, model, nullptr, d_theta, npar_of(&c->cfg, model), P, seed, particle_offset, d_stats);
}

int abc_simulate_batch_device(abc_ctx* c, const int32_t* d_models, const double* d_theta, int64_t ld_theta,
                              int64_t P, uint64_t seed, int64_t particle_offset, double* d_stats) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, 1, P, particle_offset);
  if (st) return st;
  if (P == 0) return ABC_OK;
  if (!d_models || !d_theta || !d_stats) return fail(c, ABC_ERR_INVALID, "null device pointer");
  if (ld_theta < npar_max(&c->cfg)) return fail(c, ABC_ERR_INVALID, "ld_theta below the largest npar");
  return enqueue_chain(c, 0, d_models, d_theta, ld_theta, P, seed, particle_offset, d_stats);
}

int abc_simulate_batch(abc_ctx* c, const int32_t* models, const double* theta, int64_t ld_theta, int64_t P,
                       uint64_t seed, int64_t particle_offset, double* stats_out) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, 1, P, particle_offset);
  if (st) return st;
  if (P == 0) return ABC_OK;
  if (!models || !theta || !stats_out) return fail(c, ABC_ERR_INVALID, "null host pointer");
  if (ld_theta < npar_max(&c->cfg)) return fail(c, ABC_ERR_INVALID, "ld_theta below the largest npar");
  for (int64_t p = 0; p < P; ++p)
    if (models[p] < 1 || models[p] > 5) return fail(c, ABC_ERR_INVALID, "model ids must be 1..5");
  const int K = ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
  CK(c->d_models.ensure((size_t)P));
  CK(c->d_theta.ensure((size_t)P * ld_theta));
  CK(c->d_stats.ensure((size_t)P * K));
  CK(cudaMemcpyAsync(c->d_models.p, models, sizeof(int32_t) * P, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_theta.p, theta, sizeof(double) * P * ld_theta, cudaMemcpyHostToDevice, c->stream));
  st = enqueue_chain(c, 0, c->d_models.p, c->d_theta.p, ld_theta, P, seed, particle_offset, c->d_stats.p);
  if (st) return st;
  CK(cudaMemcpyAsync(stats_out, c->d_stats.p, sizeof(double) * P * K, cudaMemcpyDeviceToHost, c->stream));
  return finish_status(c);
}

int abc_synchronize(abc_ctx* c) {
  if (!c) return ABC_ERR_INVALID;
  return finish_status(c);
}

int abc_simulate(abc_ctx* c, int model, const double* theta, int64_t P, uint64_t seed, int64_t particle_offset,
                 double* stats_out) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, model, P, particle_offset);
  if (st) return st;
  if (P == 0) return ABC_OK;
  if (!theta || !stats_out) return fail(c, ABC_ERR_INVALID, "null host pointer");
  const int npar = npar_of(&c->cfg, model);
  const int K = ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
  CK(c->d_theta.ensure((size_t)P * npar));
  CK(c->d_stats.ensure((size_t)P * K));
  CK(cudaMemcpyAsync(c->d_theta.p, theta, sizeof(double) * P * npar, cudaMemcpyHostToDevice, c->stream));
  st = enqueue_simulate(c, model, nullptr, c->d_theta.p, npar, P, seed, particle_offset, c->d_stats.p, false);
  if (st) return st;
  CK(cudaMemcpyAsync(stats_out, c->d_stats.p, sizeof(double) * P * K, cudaMemcpyDeviceToHost, c->stream));
  return finish_status(c);
}

int abc_simulate_cells(abc_ctx* c, int model, const double* theta, int64_t P, uint64_t seed,
                       int64_t particle_offset, int32_t* counts_out, int32_t* captured_out, int64_t* events_out,
                       uint64_t* hash_out, double* stats_out) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, model, P, particle_offset);
  if (st) return st;
  if (P == 0) return ABC_OK;
  if (!theta) return fail(c, ABC_ERR_INVALID, "null theta");
  const int64_t C = c->C;
  if ((double)P * (double)C * 24.0 > (double)(size_t(8) << 30))
    return fail(c, ABC_ERR_INVALID, "abc_simulate_cells: P x C too large for per-cell output");
  const int npar = npar_of(&c->cfg, model);
  const int K = ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
  CK(c->d_theta.ensure((size_t)P * npar));
  CK(c->d_stats.ensure((size_t)P * K));
  CK(cudaMemcpyAsync(c->d_theta.p, theta, sizeof(double) * P * npar, cudaMemcpyHostToDevice, c->stream));
  st = enqueue_simulate(c, model, nullptr, c->d_theta.p, npar, P, seed, particle_offset, c->d_stats.p, true);
  if (st) return st;
  std::vector<int2> cnt((size_t)P * C), cap((size_t)P * C);
  std::vector<int64_t> ev((size_t)P * C);
  std::vector<uint64_t> hs((size_t)P * C);
  CK(cudaMemcpyAsync(cnt.data(), c->d_counts.p, sizeof(int2) * P * C, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(cap.data(), c->d_captured.p, sizeof(int2) * P * C, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(ev.data(), c->d_events.p, sizeof(int64_t) * P * C, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(hs.data(), c->d_hash.p, sizeof(uint64_t) * P * C, cudaMemcpyDeviceToHost, c->stream));
  if (stats_out)
    CK(cudaMemcpyAsync(stats_out, c->d_stats.p, sizeof(double) * P * K, cudaMemcpyDeviceToHost, c->stream));
  st = finish_status(c);
  // internal (group-sorted) order -> caller's cell order
  for (int64_t p = 0; p < P; ++p)
    for (int64_t i = 0; i < C; ++i) {
      const int64_t src = p * C + i, dst = p * C + c->perm[i];
      if (counts_out) { counts_out[2 * dst] = cnt[src].x; counts_out[2 * dst + 1] = cnt[src].y; }
      if (captured_out) { captured_out[2 * dst] = cap[src].x; captured_out[2 * dst + 1] = cap[src].y; }
      if (events_out) events_out[dst] = ev[src];
      if (hash_out) hash_out[dst] = hs[src];
    }
  return st;
}

// Times the production kernel for every (register variant, work chunk) pair
// on a sample already on the device (d_models NULL: one model), twice each in
// alternating order, keeping each pair's faster SSA-kernel time; the context
// keeps the fastest pair, unless it is within 2 % of the first pair (variant
// 0, the spill-free allocation, with the first chunk).  ms_out[v * n_chunks + i].
static int tune_impl(abc_ctx* c, int model, const int32_t* d_models, const double* d_theta, int64_t ld, int64_t P,
                     uint64_t seed, const int* chunks, int n_chunks, double* ms_out, int* chosen_v, int* chosen_c) {
  const bool prof = c->prof;
  c->prof = true;
  const int n_cfg = kSsaVariants * n_chunks;
  std::vector<double> t((size_t)n_cfg, 1e300);
  for (int rep = 0; rep < 2; ++rep) {
    for (int i = 0; i < n_cfg; ++i) {
      const int k = rep == 0 ? i : n_cfg - 1 - i;
      c->variant = k / n_chunks;
      c->work_chunk = chunks[k % n_chunks];
      int st = enqueue_simulate(c, model, d_models, d_theta, ld, P, seed, 0, c->d_stats.p, false);
      if (!st) st = finish_status(c);
      if (st) {
        c->prof = prof;
        c->variant = 0;
        c->work_chunk = chunks[0];
        return st;
      }
      t[k] = std::min(t[k], (double)c->phase_ms[1]);
    }
  }
  int best = 0;
  for (int k = 1; k < n_cfg; ++k)
    if (t[k] < t[best]) best = k;
  if (t[best] > 0.98 * t[0]) best = 0;
  if (ms_out)
    for (int k = 0; k < n_cfg; ++k) ms_out[k] = t[k];
  c->prof = prof;
  c->variant = best / n_chunks;
  c->work_chunk = chunks[best % n_chunks];
  if (chosen_v) *chosen_v = c->variant;
  if (chosen_c) *chosen_c = c->work_chunk;
  return ABC_OK;
}

int abc_autotune(abc_ctx* c, int model, const double* theta, int64_t P, uint64_t seed, double* ms_out,
                 int* chosen) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, model, P, 0);
  if (st) return st;
  if (P < 1 || !theta) return fail(c, ABC_ERR_INVALID, "abc_autotune: needs a theta sample");
  if (c->cfg.precision != ABC_FP32) {
    if (chosen) *chosen = 0;
    return ABC_OK;  // the FP64 oracle mode has a single kernel
  }
  const int npar = npar_of(&c->cfg, model);
  const int K = ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
  CK(c->d_theta.ensure((size_t)P * npar));
  CK(c->d_stats.ensure((size_t)P * K));
  CK(cudaMemcpyAsync(c->d_theta.p, theta, sizeof(double) * P * npar, cudaMemcpyHostToDevice, c->stream));
  const int keep_chunk = c->work_chunk;
  return tune_impl(c, model, nullptr, c->d_theta.p, npar, P, seed, &keep_chunk, 1, ms_out, chosen, nullptr);
}

int abc_autotune_batch(abc_ctx* c, const int32_t* models, const double* theta, int64_t ld_theta, int64_t P,
                       uint64_t seed, double* ms_out, int* chosen_variant, int* chosen_chunk) {
  if (!c) return ABC_ERR_INVALID;
  int st = check_sim_args(c, 1, P, 0);
  if (st) return st;
  if (P < 1 || !theta || !models) return fail(c, ABC_ERR_INVALID, "abc_autotune_batch: needs a sample");
  if (ld_theta < npar_max(&c->cfg)) return fail(c, ABC_ERR_INVALID, "ld_theta below the largest npar");
  for (int64_t p = 0; p < P; ++p)
    if (models[p] < 1 || models[p] > 5) return fail(c, ABC_ERR_INVALID, "model ids must be 1..5");
  if (c->cfg.precision != ABC_FP32) {
    if (chosen_variant) *chosen_variant = 0;
    if (chosen_chunk) *chosen_chunk = c->work_chunk;
    return ABC_OK;
  }
  const int K = ABC_NSTATS(c->cfg.n_ages, c->cfg.n_conds);
  CK(c->d_models.ensure((size_t)P));
  CK(c->d_theta.ensure((size_t)P * ld_theta));
  CK(c->d_stats.ensure((size_t)P * K));
  CK(cudaMemcpyAsync(c->d_models.p, models, sizeof(int32_t) * P, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_theta.p, theta, sizeof(double) * P * ld_theta, cudaMemcpyHostToDevice, c->stream));
  return tune_impl(c, 0, c->d_models.p, c->d_theta.p, ld_theta, P, seed, kTuneChunks, kNumTuneChunks, ms_out,
                   chosen_variant, chosen_chunk);
}

int abc_set_work_chunk(abc_ctx* c, int chunk) {
  if (!c || chunk < 1 || chunk > 1024) return ABC_ERR_INVALID;
  c->work_chunk = chunk;
  return ABC_OK;
}

int abc_set_variant(abc_ctx* c, int variant) {
  if (!c || variant < 0 || variant >= kSsaVariants) return ABC_ERR_INVALID;
  c->variant = variant;
  return ABC_OK;
}

int abc_profile(abc_ctx* c, int enable) {
  if (!c) return ABC_ERR_INVALID;
  c->prof = enable != 0;
  c->ev_used = 0;
  return ABC_OK;
}

int abc_profile_read(const abc_ctx* c, double* ms_out) {
  if (!c || !ms_out) return ABC_ERR_INVALID;
  for (int i = 0; i < 3; ++i) ms_out[i] = c->phase_ms[i];
  return ABC_OK;
}

int abc_last_counters(const abc_ctx* c, int64_t* events, int64_t* rejections) {
  if (!c) return ABC_ERR_INVALID;
  if (events) *events = c->last_events;
  if (rejections) *rejections = c->last_rej;
  return ABC_OK;
}

// ---------------------------------------------------------------------------
// distance + acceptance
// ---------------------------------------------------------------------------
static int load_dist_inputs(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
                            const int32_t* fam, const double* stats, int64_t P, DistInputs& in,
                            bool stats_on_device = false) {
  if (!data || !se || !stats || G <= 0 || P <= 0 || K <= 0)
    return fail(c, ABC_ERR_INVALID, "distance: bad arguments");
  if (P > (int64_t(1) << 31) - 1 || G > (int64_t(1) << 31) - 1)
    return fail(c, ABC_ERR_INVALID, "distance: P and G must be < 2^31");
  in.G = G;
  in.P = P;
  in.K = K;
  if (n_fam <= 0 || !fam) {
    in.n_fam = 1;
    in.fam[0] = K;
  } else {
    if (n_fam > 16) return fail(c, ABC_ERR_INVALID, "distance: at most 16 families");
    int sum = 0;
    for (int f = 0; f < n_fam; ++f) {
      if (fam[f] < 0) return fail(c, ABC_ERR_INVALID, "distance: negative family size");
      in.fam[f] = fam[f];
      sum += fam[f];
    }
    if (sum != K) return fail(c, ABC_ERR_INVALID, "distance: family sizes must sum to K");
    in.n_fam = n_fam;
  }
  CK(c->d_data.ensure((size_t)G * K));
  CK(c->d_se.ensure((size_t)G * K));
  CK(cudaMemcpyAsync(c->d_data.p, data, sizeof(double) * G * K, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_se.p, se, sizeof(double) * G * K, cudaMemcpyHostToDevice, c->stream));
  in.data = c->d_data.p;
  in.se = c->d_se.p;
  CK(c->d_den.ensure((size_t)G * K));
  CK(c->d_rden.ensure((size_t)G * K));
  CK(launch_dist_den(in, c->d_den.p, c->d_rden.p, c->stream));
  in.den = c->d_den.p;
  in.rden = c->d_rden.p;
  if (stats_on_device) {
    in.stats = stats;
  } else {
    CK(c->d_sel_stats.ensure((size_t)P * K));
    CK(cudaMemcpyAsync(c->d_sel_stats.p, stats, sizeof(double) * P * K, cudaMemcpyHostToDevice, c->stream));
    in.stats = c->d_sel_stats.p;
  }
  return ABC_OK;
}

int abc_errors(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
               const int32_t* fam, const double* stats, int64_t P, double* err_out) {
  if (!c) return ABC_ERR_INVALID;
  if (!err_out) return fail(c, ABC_ERR_INVALID, "abc_errors: null output");
  DistInputs in;
  int st = load_dist_inputs(c, data, se, G, K, n_fam, fam, stats, P, in);
  if (st) return st;
  DBuf<double> out;
  CK(out.ensure((size_t)P * G));
  cudaError_t e = launch_dist_full(in, out.p, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(err_out, out.p, sizeof(double) * P * G, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  out.release();
  if (e != cudaSuccess) return cuda_fail(c, e, "abc_errors");
  return ABC_OK;
}

static const int64_t kCandLimit = int64_t(1) << 28;  // candidates carry 12 B plus 20 B in the recheck and sort

static int prof_begin(abc_ctx* c) {
  if (c->prof && !c->sel_ev[0]) {
    CK(cudaEventCreate(&c->sel_ev[0]));
    CK(cudaEventCreate(&c->sel_ev[1]));
  }
  if (c->prof) CK(cudaEventRecord(c->sel_ev[0], c->stream));
  return ABC_OK;
}

static int prof_end(abc_ctx* c) {
  if (!c->prof) return ABC_OK;
  CK(cudaEventRecord(c->sel_ev[1], c->stream));
  CK(cudaEventSynchronize(c->sel_ev[1]));
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, c->sel_ev[0], c->sel_ev[1]));
  c->sel_fast_ms += ms;
  c->sel_fast_passes += 1;
  return ABC_OK;
}

// FP32 candidate pass on the CUDA cores; candidates and their FP32 errors in
// d_cand / d_cande, count in *n.
static int candidate_pass_simt(abc_ctx* c, const DistInputs& in, int64_t* n) {
  for (int attempt = 0; attempt < 2; ++attempt) {
    CK(c->d_cand.ensure((size_t)c->cand_cap));
    CK(c->d_cande.ensure((size_t)c->cand_cap));
    CK(cudaMemsetAsync(c->d_ncand.p, 0, sizeof(unsigned long long), c->stream));
    int st = prof_begin(c);
    if (st) return st;
    CK(launch_dist_fast(c->d_s32.p, c->d_sw.p, c->d_dw.p, in.P, in.G, in.K, c->d_X.p, c->d_cand.p, c->d_cande.p,
                        c->d_ncand.p, c->cand_cap, nullptr, 0, 0, c->stream));
    st = prof_end(c);
    if (st) return st;
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, c->d_ncand.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if ((int64_t)h <= c->cand_cap) {
      *n = (int64_t)h;
      return ABC_OK;
    }
    if ((int64_t)h > kCandLimit)
      return fail(c, ABC_ERR_CAPACITY,
                  "more than 2^28 candidates (a threshold at the clip value 10 ties too many particles)");
    c->cand_cap = (int64_t)h + (int64_t)h / 8 + 1024;
  }
  return fail(c, ABC_ERR_CAPACITY, "candidate buffer overflow");
}

// Tensor-core candidate pass: each CTA appends to its own segment; the
// segments are concatenated into d_cand / d_cande.
static int candidate_pass_tc(abc_ctx* c, const DistInputs& in, int nh, int64_t* n) {
  const int grid = tc_grid(in.P, in.G, c->sms);
  const TcLayout L = tc_layout(in.K, nh);
  CK(launch_tc_y(c->d_X.p, c->d_cg64.p, in.G, in.K, c->d_Y.p, c->stream));
  CK(c->d_segcount.ensure((size_t)grid));
  CK(c->d_tcerr.ensure(1));
  std::vector<unsigned> cnt((size_t)grid);
  for (int attempt = 0; attempt < 2; ++attempt) {
    CK(c->d_seg.ensure((size_t)grid * (size_t)c->seg_cap));
    CK(c->d_seg_e.ensure((size_t)grid * (size_t)c->seg_cap));
    CK(cudaMemsetAsync(c->d_segcount.p, 0, sizeof(unsigned) * grid, c->stream));
    CK(cudaMemsetAsync(c->d_tcerr.p, 0, sizeof(int), c->stream));
    TcArgs a;
    a.P = in.P;
    a.G = in.G;
    a.K = in.K;
    a.KA = L.H;
    a.n_chunks = L.n_chunks;
    a.cg = c->d_cg32.p;
    a.rowbad = c->d_rowbad.p;
    a.nM = (int)((in.P + 127) / 128);
    a.nN = (int)((in.G + 255) / 256);
    a.Y = c->d_Y.p;
    a.cand = c->d_seg.p;
    a.cand_e = c->d_seg_e.p;
    a.seg_cap = c->seg_cap;
    a.seg_count = c->d_segcount.p;
    a.err = c->d_tcerr.p;
    int st = prof_begin(c);
    if (st) return st;
    CK(launch_dist_tc(nh, c->d_tcA.p, c->d_tcB.p, a, grid, c->stream));
    st = prof_end(c);
    if (st) return st;
    int herr = 0;
    CK(cudaMemcpyAsync(cnt.data(), c->d_segcount.p, sizeof(unsigned) * grid, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&herr, c->d_tcerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (herr)
      return fail(c, ABC_ERR_CUDA,
                  "tensor-core distance pass: a bounded wait ran out (code " + std::to_string(herr) + ")");
    int64_t total = 0, mx = 0;
    for (int b = 0; b < grid; ++b) {
      total += cnt[b];
      mx = std::max<int64_t>(mx, cnt[b]);
    }
    if (total > kCandLimit)
      return fail(c, ABC_ERR_CAPACITY,
                  "more than 2^28 candidates (a threshold at the clip value 10 ties too many particles)");
    if (mx <= c->seg_cap) {
      CK(c->d_cand.ensure((size_t)std::max<int64_t>(total, 1)));
      CK(c->d_cande.ensure((size_t)std::max<int64_t>(total, 1)));
      CK(launch_tc_gather(c->d_seg.p, c->d_seg_e.p, c->d_segcount.p, grid, c->seg_cap, c->d_cg32.p, in.K, c->d_cand.p,
                          c->d_cande.p, c->stream));
      *n = total;
      return ABC_OK;
    }
    c->seg_cap = mx + mx / 4 + 1024;
  }
  return fail(c, ABC_ERR_CAPACITY, "candidate segment overflow");
}

// Operands of the candidate pass and its error bound |e32 - e| <= b0[g] + b1 e.
// Tensor cores (the requested mode) unless an operand is infinite or w s^2
// could leave the FP32 range; then the FP32 CUDA-core pass.
static int prepare_candidate_pass(abc_ctx* c, const DistInputs& in, int* dmode_out, float* b1_out) {
  const int64_t G = in.G, P = in.P;
  const int K = in.K;
  CK(c->d_sw.ensure((size_t)G * K));
  CK(c->d_dw.ensure((size_t)G * K));
  CK(c->d_b0.ensure((size_t)G));
  int dmode = c->dist_mode;
  float b1 = 0.0f;
  if (dmode == 3 && !tc_mode3_fits(K)) dmode = 2;  // gene rows too long to stay in shared memory
  if (dmode) {
    const size_t words = tc_layout(K, dmode).words();
    CK(c->d_tcA.ensure((size_t)P * words));
    CK(c->d_tcB.ensure((size_t)G * words));
    CK(c->d_rowbad.ensure((size_t)std::max<int64_t>(P, 1)));
    CK(c->d_cg64.ensure((size_t)G));
    CK(c->d_cg32.ensure((size_t)G));
    CK(c->d_Y.ensure((size_t)G));
    CK(c->d_tcflags.ensure(3));
    CK(cudaMemsetAsync(c->d_tcflags.p, 0, sizeof(unsigned) * 3, c->stream));
    const double beta = tc_beta(K, dmode);
    CK(launch_tc_prep(in, dmode, beta, c->d_tcA.p, c->d_tcB.p, c->d_rowbad.p, c->d_cg64.p, c->d_cg32.p, c->d_b0.p,
                      c->d_tcflags.p, c->stream));
    unsigned fl[3];
    CK(cudaMemcpyAsync(fl, c->d_tcflags.p, sizeof(fl), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float maxw, maxs2;
    memcpy(&maxw, &fl[1], 4);
    memcpy(&maxs2, &fl[2], 4);
    if (fl[0] || (double)maxw * (double)maxs2 * (4.0 * K) > 1e37) dmode = 0;
    else b1 = (float)(4.0 * beta);
  }
  // FP32 statistics of every particle for the CUDA-core pass; the tensor-core
  // pass needs them only for the threshold subsample (converted there)
  if (dmode == 0) CK(c->d_s32.ensure((size_t)P * K));
  CK(launch_dist_prep(in, c->d_sw.p, c->d_dw.p, dmode == 0 ? c->d_s32.p : nullptr, P, 1, c->stream));
  if (dmode == 0) {
    // 1.5 u (64 sqrt(e) + (K + 8) e) <= 48 u + 1.5 u (K + 40) e, u = 2^-24
    const double u = 5.9604644775390625e-08;
    b1 = (float)(1.5 * u * (K + 40));
    CK(launch_fill(c->d_b0.p, G, (float)(48.0 * u), c->stream));
  }
  c->dist_mode_used = dmode;
  *dmode_out = dmode;
  *b1_out = b1;
  return ABC_OK;
}

// mode 0: err <= eps; mode 1: top ceil(q P) per gene; mode 2: err <= thr[g] per gene
static int select_impl(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
                       const int32_t* fam, const double* stats, bool stats_on_device, int64_t P, int mode,
                       double eps_or_q, const double* thr, int64_t* n_accepted_total) {
  if (!c) return ABC_ERR_INVALID;
  c->sel_ready = false;
  if (mode < 0 || mode > 2) return fail(c, ABC_ERR_INVALID, "mode must be 0 (eps), 1 (top-q) or 2 (per-gene thr)");
  if (mode == 1 && !(eps_or_q > 0.0 && eps_or_q <= 1.0)) return fail(c, ABC_ERR_INVALID, "q must be in (0, 1]");
  if (mode == 0 && eps_or_q != eps_or_q) return fail(c, ABC_ERR_INVALID, "eps is NaN");
  if (mode == 2) {
    if (!thr) return fail(c, ABC_ERR_INVALID, "mode 2 needs per-gene thresholds");
    for (int64_t g = 0; g < G; ++g)
      if (thr[g] != thr[g]) return fail(c, ABC_ERR_INVALID, "threshold is NaN");
  }
  DistInputs in;
  int st = load_dist_inputs(c, data, se, G, K, n_fam, fam, stats, P, in, stats_on_device);
  if (st) return st;
  c->sel_in = in;
  CK(c->d_thr.ensure((size_t)G));
  if (mode == 2) CK(cudaMemcpyAsync(c->d_thr.p, thr, sizeof(double) * G, cudaMemcpyHostToDevice, c->stream));
  CK(c->d_X.ensure((size_t)G));
  CK(c->d_ncand.ensure(1));
  CK(c->d_gcount.ensure((size_t)G));
  CK(c->d_goff.ensure((size_t)G + 1));
  CK(c->d_gcursor.ensure((size_t)G));
  CK(c->d_alen.ensure((size_t)G));
  CK(c->d_aoff.ensure((size_t)G + 1));
  CK(c->d_fail.ensure((size_t)G));
  c->sel_fast_ms = 0.0;
  c->sel_fast_passes = 0;
  int dmode = 0;
  float b1 = 0.0f;
  st = prepare_candidate_pass(c, in, &dmode, &b1);
  if (st) return st;
  const int64_t kq = mode == 1 ? (int64_t)std::ceil(eps_or_q * (double)P) : 0;
  std::vector<float> hX((size_t)G);
  if (mode == 0 || mode == 2) {
    CK(launch_x_from_thr(mode == 2 ? c->d_thr.p : nullptr, eps_or_q, G, c->d_b0.p, b1, c->d_X.p, c->stream));
  } else {
    // thresholds from a strided subsample
    const int64_t n_sub = std::min<int64_t>(P, 32768);
    const int64_t stride = std::max<int64_t>(1, P / n_sub);
    const int64_t k_sub = (int64_t)std::ceil(2.0 * eps_or_q * (double)n_sub) + 16;
    if (k_sub >= n_sub) {
      std::fill(hX.begin(), hX.end(), INFINITY);
      CK(cudaMemcpyAsync(c->d_X.p, hX.data(), sizeof(float) * G, cudaMemcpyHostToDevice, c->stream));
    } else {
      CK(c->d_esub.ensure((size_t)n_sub * G));
      int64_t sub_stride = stride;
      if (dmode) {
        // the subsample rows, compacted
        CK(c->d_s32.ensure((size_t)n_sub * K));
        CK(launch_dist_prep(in, c->d_sw.p, c->d_dw.p, c->d_s32.p, n_sub, stride, c->stream));
        sub_stride = 1;
      }
      CK(launch_dist_fast(c->d_s32.p, c->d_sw.p, c->d_dw.p, P, G, K, nullptr, nullptr, nullptr, nullptr, 0,
                          c->d_esub.p, sub_stride, n_sub, c->stream));
      CK(launch_dist_threshold(c->d_esub.p, n_sub, G, k_sub, c->d_b0.p, b1, c->d_X.p, c->stream));
      if (dmode) {
        // about k_sub of every n_sub particles per gene pass X: size the per-CTA
        // segments for that (with room for imbalance) so one pass suffices
        const int grid = tc_grid(P, G, c->sms);
        const double est = (double)G * (double)k_sub * ((double)P / (double)n_sub);
        const int64_t want = (int64_t)(1.5 * est / grid) + 4096;
        c->seg_cap = std::max(c->seg_cap, std::min<int64_t>(want, kCandLimit / grid + 1));
      }
      CK(cudaMemcpyAsync(hX.data(), c->d_X.p, sizeof(float) * G, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  int64_t ncand = 0;
  c->sel_rechecked = 0;
  c->sel_cands_emitted = 0;
  for (int round = 0; round < 4; ++round) {
    st = dmode ? candidate_pass_tc(c, in, dmode, &ncand) : candidate_pass_simt(c, in, &ncand);
    if (st) return st;
    const Cand* rc = c->d_cand.p;
    const float* Xacc = c->d_X.p;
    int64_t nre = ncand;
    if (mode == 1) {
      // only candidates that can still be among the k smallest go to the FP64 recheck
      CK(c->d_hist.ensure((size_t)G * kHistBins));
      CK(c->d_Xt.ensure((size_t)G));
      CK(c->d_cand2.ensure((size_t)std::max<int64_t>(ncand, 1)));
      CK(launch_refine(c->d_cand.p, c->d_cande.p, ncand, G, kq, c->d_X.p, c->d_b0.p, b1, c->d_hist.p, c->d_Xt.p,
                       c->d_cand2.p, c->d_ncand.p, c->stream));
      unsigned long long h = 0;
      CK(cudaMemcpyAsync(&h, c->d_ncand.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      nre = (int64_t)h;
      rc = c->d_cand2.p;
      Xacc = c->d_Xt.p;
    }
    CK(c->d_se64.ensure((size_t)std::max<int64_t>(nre, 1)));
    CK(c->d_sp.ensure((size_t)std::max<int64_t>(nre, 1)));
    CK(c->d_sg.ensure((size_t)std::max<int64_t>(nre, 1)));
    if (c->sel_errors) {
      CK(launch_dist_group_recheck_sort(in, rc, nre, c->d_gcount.p, c->d_goff.p, c->d_gcursor.p, c->d_sp.p,
                                        c->d_sg.p, c->d_se64.p, c->stream));
    } else {
      // indices only: certified FP32 errors, FP64 where they cannot decide
      CK(c->d_ffg.ensure((size_t)G * K));
      CK(c->d_pos.ensure((size_t)std::max<int64_t>(nre, 1)));
      CK(c->d_flag.ensure((size_t)std::max<int64_t>(nre, 1)));
      CK(c->d_cnt2.ensure(2));
      CK(c->d_dirty.ensure((size_t)G));
      CK(launch_dist_group_certify_sort(in, rc, nre, mode, eps_or_q, mode == 2 ? c->d_thr.p : nullptr,
                                        c->d_gcount.p, c->d_goff.p, c->d_gcursor.p, c->d_sp.p, c->d_sg.p,
                                        c->d_se64.p, c->d_ffg.p, c->d_pos.p, c->d_flag.p,
                                        c->d_cnt2.p,
                                        c->d_dirty.p, c->stream));
    }
    CK(cudaMemsetAsync(c->d_fail.p, 0, sizeof(int) * G, c->stream));
    CK(launch_dist_accept_len(c->d_goff.p, c->d_se64.p, G, mode == 2 ? 0 : mode, eps_or_q,
                              mode == 2 ? c->d_thr.p : nullptr, kq, Xacc, c->d_b0.p, b1, c->d_alen.p, c->d_fail.p,
                              !c->sel_errors, c->stream));
    c->sel_cands_emitted += ncand;
    if (c->sel_errors) {
      c->sel_rechecked += nre;
    } else {
      unsigned long long hc[2] = {0ull, 0ull};
      CK(cudaMemcpyAsync(hc, c->d_cnt2.p, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      c->sel_rechecked += (int64_t)(hc[0] + hc[1]);
    }
    if (mode != 1) break;
    std::vector<int> hf((size_t)G);
    CK(cudaMemcpyAsync(hf.data(), c->d_fail.p, sizeof(int) * G, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    bool any = false;
    for (int64_t g = 0; g < G; ++g) {
      if (hf[g]) {
        any = true;
        hX[g] = (round >= 1 || !(hX[g] < INFINITY)) ? INFINITY : 4.0f * hX[g] + 0.1f;
      }
    }
    if (!any) break;
    if (round == 3) return fail(c, ABC_ERR_CAPACITY, "top-q selection did not converge");
    CK(cudaMemcpyAsync(c->d_X.p, hX.data(), sizeof(float) * G, cudaMemcpyHostToDevice, c->stream));
  }
  CK(launch_scan(c->d_alen.p, G, c->d_aoff.p, c->stream));
  int64_t total = 0;
  CK(cudaMemcpyAsync(&total, c->d_aoff.p + G, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  CK(c->d_out_idx.ensure((size_t)std::max<int64_t>(total, 1)));
  CK(c->d_out_err.ensure((size_t)std::max<int64_t>(total, 1)));
  CK(launch_dist_compact(c->d_goff.p, c->d_sp.p, c->d_se64.p, c->d_aoff.p, G, 0, c->d_out_idx.p, c->d_out_err.p,
                         c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->sel_G = G;
  c->sel_P = P;
  c->sel_total = total;
  c->sel_errors_exact = c->sel_errors;
  c->sel_cands = c->sel_cands_emitted;
  c->sel_ready = true;
  if (n_accepted_total) *n_accepted_total = total;
  return ABC_OK;
}

int abc_errors_select(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
                      const int32_t* fam, const double* stats, int64_t P, int mode, double eps_or_q,
                      int64_t* n_accepted_total) {
  if (mode == 2) return fail(c, ABC_ERR_INVALID, "per-gene thresholds: use abc_errors_select_thr");
  return select_impl(c, data, se, G, K, n_fam, fam, stats, false, P, mode, eps_or_q, nullptr, n_accepted_total);
}

int abc_errors_select_thr(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
                          const int32_t* fam, const double* stats, int64_t P, const double* thr,
                          int64_t* n_accepted_total) {
  return select_impl(c, data, se, G, K, n_fam, fam, stats, false, P, 2, 0.0, thr, n_accepted_total);
}

int abc_errors_select_device(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
                             const int32_t* fam, const double* d_stats, int64_t P, int mode, double eps_or_q,
                             const double* thr, int64_t* n_accepted_total) {
  return select_impl(c, data, se, G, K, n_fam, fam, d_stats, true, P, mode, eps_or_q, thr, n_accepted_total);
}

int abc_errors_candidate(abc_ctx* c, const double* data, const double* se, int64_t G, int K, int n_fam,
                         const int32_t* fam, const double* stats, int64_t P, float* err_out, double* b0_out,
                         double* b1_out, int* mode_used) {
  if (!c) return ABC_ERR_INVALID;
  if (!err_out) return fail(c, ABC_ERR_INVALID, "abc_errors_candidate: null output");
  if (P * G > kCandLimit) return fail(c, ABC_ERR_INVALID, "abc_errors_candidate: P G must be <= 2^28");
  DistInputs in;
  int st = load_dist_inputs(c, data, se, G, K, n_fam, fam, stats, P, in);
  if (st) return st;
  int dmode = 0;
  float b1 = 0.0f;
  st = prepare_candidate_pass(c, in, &dmode, &b1);
  if (st) return st;
  CK(c->d_X.ensure((size_t)G));
  CK(c->d_ncand.ensure(1));
  CK(launch_fill(c->d_X.p, G, INFINITY, c->stream));
  int64_t n = 0;
  c->cand_cap = std::max<int64_t>(c->cand_cap, P * G);
  st = dmode ? candidate_pass_tc(c, in, dmode, &n) : candidate_pass_simt(c, in, &n);
  if (st) return st;
  DBuf<float> out;
  CK(out.ensure((size_t)P * G));
  CK(launch_fill(out.p, P * G, NAN, c->stream));
  CK(launch_scatter_errors(c->d_cand.p, c->d_cande.p, n, G, out.p, c->stream));
  cudaError_t e = cudaMemcpyAsync(err_out, out.p, sizeof(float) * P * G, cudaMemcpyDeviceToHost, c->stream);
  std::vector<float> hb0((size_t)G);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hb0.data(), c->d_b0.p, sizeof(float) * G, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  out.release();
  if (e != cudaSuccess) return cuda_fail(c, e, "abc_errors_candidate");
  if (b0_out)
    for (int64_t g = 0; g < G; ++g) b0_out[g] = hb0[g];
  if (b1_out) *b1_out = b1;
  if (mode_used) *mode_used = dmode;
  return ABC_OK;
}

int abc_accept_fetch(abc_ctx* c, int64_t* gene_offsets, int64_t* particle_idx, double* err) {
  if (!c) return ABC_ERR_INVALID;
  if (!c->sel_ready) return fail(c, ABC_ERR_STATE, "no selection result: call abc_errors_select first");
  if (!gene_offsets || (!particle_idx && c->sel_total > 0)) return fail(c, ABC_ERR_INVALID, "null output");
  CK(cudaMemcpyAsync(gene_offsets, c->d_aoff.p, sizeof(int64_t) * (c->sel_G + 1), cudaMemcpyDeviceToHost, c->stream));
  if (c->sel_total > 0) {
    CK(cudaMemcpyAsync(particle_idx, c->d_out_idx.p, sizeof(int64_t) * c->sel_total, cudaMemcpyDeviceToHost,
                       c->stream));
    if (err) {
      if (!c->sel_errors_exact)
        return fail(c, ABC_ERR_STATE, "the selection kept no FP64 errors (abc_set_select_errors(ctx, 0)); pass err = NULL");
      CK(cudaMemcpyAsync(err, c->d_out_err.p, sizeof(double) * c->sel_total, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  CK(cudaStreamSynchronize(c->stream));
  return ABC_OK;
}

int abc_accept_errors(abc_ctx* c, double* err) {
  if (!c) return ABC_ERR_INVALID;
  if (!c->sel_ready) return fail(c, ABC_ERR_STATE, "no selection result: call abc_errors_select first");
  if (c->sel_total <= 0) return ABC_OK;
  if (!err) return fail(c, ABC_ERR_INVALID, "null output");
  if (c->sel_errors_exact) {
    CK(cudaMemcpyAsync(err, c->d_out_err.p, sizeof(double) * c->sel_total, cudaMemcpyDeviceToHost, c->stream));
  } else {
    const size_t n = (size_t)c->sel_total;
    CK(c->d_asp.ensure(n));
    CK(c->d_asg.ensure(n));
    CK(c->d_aerr.ensure(n));
    CK(launch_accepted_errors(c->sel_in, c->d_aoff.p, c->d_out_idx.p, c->sel_G, 0, c->sel_total, c->d_asp.p,
                              c->d_asg.p, c->d_aerr.p, c->stream));
    CK(cudaMemcpyAsync(err, c->d_aerr.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return ABC_OK;
}

int abc_set_select_errors(abc_ctx* c, int keep_errors) {
  if (!c) return ABC_ERR_INVALID;
  c->sel_errors = keep_errors != 0;
  return ABC_OK;
}

int abc_select_profile_read(const abc_ctx* c, double* fast_ms, int* fast_passes) {
  if (!c) return ABC_ERR_INVALID;
  if (fast_ms) *fast_ms = c->sel_fast_ms;
  if (fast_passes) *fast_passes = c->sel_fast_passes;
  return ABC_OK;
}

static bool grid_ok(double x, double h) {
  const double q = x / h;
  return std::fabs(q - std::nearbyint(q)) < 1e-7 * (1.0 + std::fabs(q));
}

int abc_moment_simulate(abc_ctx* c, int model, const double* theta, int64_t P, const double* iv, double h_max,
                        const double* beta_mom, int n_pulse_conds, const double* age_dist, double* stats_out,
                        double* moments_out, int32_t* iters_out) {
  if (!c) return ABC_ERR_INVALID;
  const int npar = npar_of(&c->cfg, model);
  if (npar < 0) return fail(c, ABC_ERR_INVALID, "model must be 1..5");
  if (c->cfg.splicing) return fail(c, ABC_ERR_INVALID, "the moment model has no splicing");
  if (!theta || !iv || !beta_mom || !age_dist || !stats_out || P < 0)
    return fail(c, ABC_ERR_INVALID, "abc_moment_simulate: bad arguments");
  if (P == 0) return ABC_OK;
  const abc_config& cf = c->cfg;
  const double T = cf.cycle;
  const int S = cf.n_steps, A = cf.n_ages, J = cf.n_conds, K = 4 * A + 3 * J;
  const double t0 = -(double)cf.n_burn_cycles * T;
  // substep grid: the coarsest h <= h_max dividing every breakpoint (oracle's rule);
  // default cycle / 400 (FP64, the oracle's) or cycle / 80 (FP32 production mode)
  if (!(h_max > 0.0)) h_max = cf.precision == ABC_FP32 ? T / 80.0 : T / 400.0;
  int per_step = (int)std::ceil((T / (double)S) / h_max);
  double h = 0.0;
  for (; per_step < 200000; ++per_step) {
    h = T / (double)(S * per_step);
    bool ok = grid_ok(t0, h);
    for (int a = 0; a < A && ok; ++a) ok = grid_ok(cf.ages[a], h);
    for (int j = 0; j < J && ok; ++j) ok = grid_ok(cf.pulse[j], h) && grid_ok(cf.chase[j], h);
    if (ok) break;
  }
  if (per_step >= 200000 || (int64_t)S * per_step > 20000)
    return fail(c, ABC_ERR_INVALID, "no substep grid aligned with the breakpoints");
  MomArgs a;
  memset(&a, 0, sizeof(a));
  a.cfg = c->dcfg;
  a.ld = npar;
  a.P = P;
  a.model = model;
  for (int i = 0; i < 9; ++i) a.iv[i] = iv[i];
  a.h = h;
  a.per_step = per_step;
  a.nsub = S * per_step;
  a.n_pulse_conds = n_pulse_conds;
  const bool f32 = cf.precision == ABC_FP32;
  const int grid = (int)std::min<int64_t>(P, (int64_t)c->sms * (f32 ? 16 : 8));
  const size_t scr_doubles = f32 ? (moment_f32_scratch_per_cta(a.nsub) + 7) / 8 : (size_t)2 * a.nsub * 100;
  DBuf<double> d_theta, d_bm, d_ad, d_stats, d_mom, d_scr;
  DBuf<int> d_it;
  CK(d_theta.ensure((size_t)P * npar));
  CK(d_bm.ensure((size_t)2 * A * 3));
  CK(d_ad.ensure((size_t)A * J));
  CK(d_stats.ensure((size_t)P * K));
  CK(d_scr.ensure((size_t)grid * scr_doubles));
  if (moments_out) CK(d_mom.ensure((size_t)P * J * A * 5));
  if (iters_out) CK(d_it.ensure((size_t)P));
  CK(cudaMemcpyAsync(d_theta.p, theta, sizeof(double) * P * npar, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_bm.p, beta_mom, sizeof(double) * 2 * A * 3, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_ad.p, age_dist, sizeof(double) * A * J, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d_status.p, 0, sizeof(int), c->stream));
  a.theta = d_theta.p;
  a.beta_mom = d_bm.p;
  a.age_dist = d_ad.p;
  a.stats = d_stats.p;
  a.moments = moments_out ? d_mom.p : nullptr;
  a.iters = iters_out ? d_it.p : nullptr;
  a.scratch = d_scr.p;
  a.status = c->d_status.p;
  if (c->prof && !c->sel_ev[0]) {
    CK(cudaEventCreate(&c->sel_ev[0]));
    CK(cudaEventCreate(&c->sel_ev[1]));
  }
  if (c->prof) CK(cudaEventRecord(c->sel_ev[0], c->stream));
  CK(f32 ? launch_moment_f32(a, grid, c->stream) : launch_moment(a, grid, c->stream));
  if (c->prof) CK(cudaEventRecord(c->sel_ev[1], c->stream));
  CK(cudaMemcpyAsync(stats_out, d_stats.p, sizeof(double) * P * K, cudaMemcpyDeviceToHost, c->stream));
  if (moments_out)
    CK(cudaMemcpyAsync(moments_out, d_mom.p, sizeof(double) * P * J * A * 5, cudaMemcpyDeviceToHost, c->stream));
  if (iters_out) CK(cudaMemcpyAsync(iters_out, d_it.p, sizeof(int) * P, cudaMemcpyDeviceToHost, c->stream));
  int hst = 0;
  CK(cudaMemcpyAsync(&hst, c->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->prof) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, c->sel_ev[0], c->sel_ev[1]));
    c->sel_fast_ms = ms;
    c->sel_fast_passes = 1;
  }
  if (hst) return fail(c, ABC_ERR_NONFINITE, "abc_moment_simulate: non-finite rates for some particles (NaN rows)");
  return ABC_OK;
}

int abc_data_stats(abc_ctx* c, const int32_t* u, const int32_t* l, int64_t G, int n_boot, uint64_t seed,
                   double* stats_out, double* se_out) {
  if (!c) return ABC_ERR_INVALID;
  if (!c->cells_set) return fail(c, ABC_ERR_STATE, "abc_data_stats: call abc_set_cells first");
  if (!u || !l || !stats_out || G < 0 || n_boot < 0 || n_boot > 10000 || (se_out && n_boot < 2))
    return fail(c, ABC_ERR_INVALID, "abc_data_stats: bad arguments (standard errors need n_boot >= 2)");
  if (c->C > data_stats_max_cells(c->cfg.n_ages, c->cfg.n_conds))
    return fail(c, ABC_ERR_INVALID, "abc_data_stats: too many cells for the per-gene shared-memory table");
  const int64_t C = c->C;
  for (int64_t i = 0; i < G * C; ++i)
    if (u[i] < 0 || l[i] < 0 || u[i] > (1 << 20) || l[i] > (1 << 20))
      return fail(c, ABC_ERR_INVALID, "abc_data_stats: counts must lie in [0, 2^20]");
  if (G == 0) return ABC_OK;
  const int K = 4 * c->cfg.n_ages + 3 * c->cfg.n_conds;
  DBuf<int32_t> du, dl;
  DBuf<double> dout, dse;
  CK(du.ensure((size_t)G * C));
  CK(dl.ensure((size_t)G * C));
  CK(dout.ensure((size_t)G * (n_boot + 1) * K));
  if (se_out) CK(dse.ensure((size_t)G * K));
  CK(cudaMemcpyAsync(du.p, u, sizeof(int32_t) * G * C, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(dl.p, l, sizeof(int32_t) * G * C, cudaMemcpyHostToDevice, c->stream));
  DataStatsArgs a;
  a.cfg = c->dcfg;
  a.u = du.p;
  a.l = dl.p;
  a.G = G;
  a.C = C;
  a.cell_cond = c->d_cond.p;
  a.cell_age = c->d_age.p;
  a.cell_id = c->d_id.p;
  a.gstart = c->d_gstart.p;
  a.age_dist = c->d_age_dist.p;
  a.n_boot = n_boot;
  a.seed = seed;
  a.out = dout.p;
  if (c->prof && !c->sel_ev[0]) {
    CK(cudaEventCreate(&c->sel_ev[0]));
    CK(cudaEventCreate(&c->sel_ev[1]));
  }
  if (c->prof) CK(cudaEventRecord(c->sel_ev[0], c->stream));
  CK(launch_data_stats(a, se_out ? dse.p : nullptr, c->stream));
  if (c->prof) CK(cudaEventRecord(c->sel_ev[1], c->stream));
  // the estimate is resample 0 of each gene
  CK(cudaMemcpy2DAsync(stats_out, sizeof(double) * K, dout.p, sizeof(double) * K * (n_boot + 1), sizeof(double) * K,
                       (size_t)G, cudaMemcpyDeviceToHost, c->stream));
  if (se_out) CK(cudaMemcpyAsync(se_out, dse.p, sizeof(double) * G * K, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->prof) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, c->sel_ev[0], c->sel_ev[1]));
    c->sel_fast_ms = ms;
    c->sel_fast_passes = 1;
  }
  return ABC_OK;
}

int abc_model_probs(abc_ctx* c, const int64_t* counts, int64_t G, int M, int n_boot, double alpha, uint64_t seed,
                    double* prob, double* lb, double* ub) {
  if (!c) return ABC_ERR_INVALID;
  if (!counts || !prob || !lb || !ub || G < 0 || M < 1 || M > 64 || n_boot < 1 || n_boot > 100000 ||
      !(alpha > 0.0 && alpha < 1.0))
    return fail(c, ABC_ERR_INVALID, "abc_model_probs: bad arguments");
  for (int64_t i = 0; i < G * M; ++i)
    if (counts[i] < 0) return fail(c, ABC_ERR_INVALID, "abc_model_probs: negative count");
  if (G == 0) return ABC_OK;
  DBuf<int64_t> d_counts;
  DBuf<double> d_out, d_boot;
  cudaError_t e = d_counts.ensure((size_t)G * M);
  if (e == cudaSuccess) e = d_out.ensure((size_t)3 * G * M);
  if (e == cudaSuccess) e = d_boot.ensure((size_t)G * M * n_boot);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_counts.p, counts, sizeof(int64_t) * G * M, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = launch_model_probs(d_counts.p, G, M, n_boot, alpha, seed, d_out.p, d_out.p + G * M, d_out.p + 2 * G * M,
                           d_boot.p, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(prob, d_out.p, sizeof(double) * G * M, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(lb, d_out.p + G * M, sizeof(double) * G * M, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ub, d_out.p + 2 * G * M, sizeof(double) * G * M, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  d_counts.release();
  d_out.release();
  d_boot.release();
  if (e != cudaSuccess) return cuda_fail(c, e, "abc_model_probs");
  return ABC_OK;
}

int abc_posterior_summary(abc_ctx* c, const double* theta, int64_t ld, int npar, int theta_on_device, double q,
                          double* map, double* mean, double* lb, double* ub, int64_t* n_particles) {
  if (!c) return ABC_ERR_INVALID;
  if (!c->sel_ready) return fail(c, ABC_ERR_STATE, "no selection result: call abc_errors_select first");
  if (!theta || !map || !mean || !lb || !ub || npar < 1 || ld < npar || !(q > 0.0 && q < 1.0))
    return fail(c, ABC_ERR_INVALID, "abc_posterior_summary: bad arguments");
  const int64_t G = c->sel_G, P = c->sel_P, total = c->sel_total;
  DBuf<double> d_theta, d_scr, d_out;
  DBuf<int64_t> d_n;
  const double* th = theta;
  cudaError_t e = cudaSuccess;
  if (!theta_on_device) {
    e = d_theta.ensure((size_t)P * ld);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_theta.p, theta, sizeof(double) * P * ld, cudaMemcpyHostToDevice, c->stream);
    th = d_theta.p;
  }
  if (e == cudaSuccess) e = d_scr.ensure((size_t)total * npar + (size_t)4 * G * npar);
  if (e == cudaSuccess) e = d_out.ensure((size_t)4 * G * npar);
  if (e == cudaSuccess) e = d_n.ensure((size_t)G);
  if (e == cudaSuccess)
    e = launch_posterior_summary(c->d_aoff.p, c->d_out_idx.p, G, total, th, ld, npar, q, d_scr.p, d_out.p,
                                 d_out.p + G * npar, d_out.p + 2 * G * npar, d_out.p + 3 * G * npar, d_n.p,
                                 c->stream);
  double* outs[4] = {map, mean, lb, ub};
  for (int i = 0; i < 4 && e == cudaSuccess; ++i)
    e = cudaMemcpyAsync(outs[i], d_out.p + (size_t)i * G * npar, sizeof(double) * G * npar, cudaMemcpyDeviceToHost,
                        c->stream);
  if (e == cudaSuccess && n_particles)
    e = cudaMemcpyAsync(n_particles, d_n.p, sizeof(int64_t) * G, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  d_theta.release();
  d_scr.release();
  d_out.release();
  d_n.release();
  if (e != cudaSuccess) return cuda_fail(c, e, "abc_posterior_summary");
  return ABC_OK;
}

int abc_set_distance_mode(abc_ctx* c, int mode) {
  if (!c) return ABC_ERR_INVALID;
  if (mode < 0 || mode > 3) return fail(c, ABC_ERR_INVALID, "distance mode must be 0, 1, 2 or 3");
  c->dist_mode = mode;
  return ABC_OK;
}

int abc_get_distance_mode(const abc_ctx* c, int* requested, int* used) {
  if (!c) return ABC_ERR_INVALID;
  if (requested) *requested = c->dist_mode;
  if (used) *used = c->dist_mode_used;
  return ABC_OK;
}

int abc_select_counters(const abc_ctx* c, int64_t* candidates, int64_t* rechecked) {
  if (!c) return ABC_ERR_INVALID;
  if (candidates) *candidates = c->sel_cands;
  if (rechecked) *rechecked = c->sel_rechecked;
  return ABC_OK;
}

}  // extern "C"
