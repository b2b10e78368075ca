// kernels.h — internal launchers shared by the C-ABI translation unit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ssa.cuh"

namespace abc {

struct StatsArgs {
  DevCfg cfg;
  const int2* counts;        // [P][C] internal cell order
  const double* beta;        // [C] internal order
  const uint32_t* cell_id;   // [C] caller's cell index
  const int32_t* gstart;     // [A*J + 1] group starts, group = cond*A + age
  const double* age_dist;    // [A*J] row-major (a*J + j)
  int64_t n_cells;
  int64_t n_particles;
  int64_t p_offset;
  uint64_t seed;
  double* stats;             // [P][K]
  int2* captured;            // optional [P][C]
  int fp32 = 0;              // production mode: FP32 binomial capture (a different realisation)
  const float* beta32 = nullptr;  // [C] the capture efficiencies in FP32 (production mode)
  int64_t max_group_cells = INT64_MAX;  // cells of the largest (condition, age) group
};

struct SetupArgs {
  DevCfg cfg;
  int model;
  const int32_t* models;     // optional per-particle model (overrides model)
  int64_t ld_theta;          // theta row stride (>= npar of the particle's model)
  const double* theta;       // [P][ld_theta]
  int64_t n_particles;
  PRec* rec;
  PRecF* recf;
  int* status;
  int fp32 = 0;              // production mode: FP32 rates beyond its range are an error
};

struct PriorArgs {
  DevCfg cfg;
  int model;
  int64_t n_particles;
  int64_t p_offset;
  uint64_t seed;
  double lo[7], hi[7];       // kon, koff, alpha, gamma, lambda, beta, log10 scaling
  double lf0, lf1;           // log10 factor bounds
  int vary_mode;
  double* theta;             // [P][npar]
};

// ---------------------------------------------------------------------------
// distance + acceptance (scripts/compute_errors.jl:30-70, accepted_particles.jl)
// ---------------------------------------------------------------------------
struct DistInputs {
  const double* data;   // [G][K]
  const double* se;     // [G][K]
  const double* stats;  // [P][K]
  const double* den = nullptr;   // [G][K] (se^2 + 0.01 d^2) + eps, or null (computed per term)
  const double* rden = nullptr;  // [G][K] RN(1 / den) (with den)
  int64_t G, P;
  int K;
  int n_fam;
  int fam[16];          // family sizes (sum K)
};

struct Cand {
  int32_t p, g;
};

// Tensor-core candidate pass (distance_tc.cu).  A = [s | s^2] per particle and
// B = [-2 w d | w] per gene; K err = c_g + A.B accumulated in FP32.  Operand
// rows hold the hi part at [0, 2K) and, in the three-term modes, the lo part at
// [H, H + 2K), zero elsewhere up to the row length ld:
//   mode 1  TF32 hi only,   H = 2K rounded up to 32, ld = H;
//   mode 2  TF32 hi and lo, H = 2K rounded up to 32, ld = 2H;
//   mode 3  BF16 hi and lo, H = 2K rounded up to 16, ld = 2H rounded up to 64.
struct TcLayout {
  int H;         // offset of the lo part (values)
  int ld;        // row length (values)
  int n_chunks;  // 128-byte chunks the MMA loop walks: per half (mode 2) or per row (modes 1, 3)
  int es;        // bytes per value (4 TF32, 2 BF16)
  size_t words() const { return (size_t)ld * es / 4; }  // row length in 4-byte words
};
TcLayout tc_layout(int K, int mode);
struct TcArgs {
  int64_t P, G;
  int K, KA, n_chunks, nM, nN;  // KA = TcLayout::H
  const float* Y;       // per gene: K X_g - c_g rounded up (candidate iff acc <= Y_g)
  const float* cg;      // per gene c_g in FP32 (NaN: the gene's operand row holds a NaN)
  const uint8_t* rowbad;  // per particle: 1 if a statistic is NaN (its accumulators are NaN)
  Cand* cand;           // per-CTA segments of seg_cap entries
  float* cand_e;        // raw accumulator of each candidate (K err - c_g)
  int64_t seg_cap;
  unsigned* seg_count;  // per CTA: candidates found (may exceed seg_cap)
  int* err;             // nonzero: a bounded wait ran out
};
// mode 3 needs the gene tile resident in shared memory; false: K too large, use mode 2
bool tc_mode3_fits(int K);
// relative error factor beta: |e32 - e| <= beta (5 c_g / K + 4 e)
double tc_beta(int K, int nh);
int tc_grid(int64_t P, int64_t G, int sms);
// flags[0] bit 0: an operand is infinite in FP32; flags[1], flags[2]: max w, max s^2 (FP32 bits)
cudaError_t launch_tc_prep(const DistInputs& in, int mode, double beta, void* A, void* B, uint8_t* rowbad,
                           double* cg64, float* cg32, float* b0, unsigned* flags, cudaStream_t s);
cudaError_t launch_tc_y(const float* X, const double* cg64, int64_t G, int K, float* Y, cudaStream_t s);
// mode 1: TF32 one term, 2: TF32 hi/lo three terms, 3: BF16 hi/lo three terms
cudaError_t launch_dist_tc(int mode, const void* A, const void* B, const TcArgs& args, int grid, cudaStream_t s);
// concatenates the per-CTA segments; seg_e holds raw accumulators, out_e the
// clipped FP32 errors min((acc + c_g) / K, 10)
cudaError_t launch_tc_gather(const Cand* seg, const float* seg_e, const unsigned* count, int n_seg, int64_t seg_cap,
                             const float* cg, int K, Cand* out, float* out_e, cudaStream_t s);

// per (g,k): sw = sqrt(w), dw = sqrt(w) d in FP32, w = 1/((se^2 + 0.01 d^2) + eps)
// and s32[r][k] = stats[r stride][k] in FP32 for r < s32_rows (s32 may be null)
cudaError_t launch_dist_prep(const DistInputs& in, float* sw, float* dw, float* s32, int64_t s32_rows,
                             int64_t stride, cudaStream_t s);
// FP32 direct distance: emit (p, g) with min(10, err32) <= X[g] (mode emit), or
// write err32 of the particles p = row*stride into esub[row][g] (mode sample).
cudaError_t launch_dist_fast(const float* s32, const float* sw, const float* dw, int64_t P, int64_t G, int K,
                             const float* X, Cand* cand, float* cand_e, unsigned long long* n_cand, int64_t cap,
                             float* esub, int64_t stride, int64_t n_sub, cudaStream_t s);
// Error bound of a candidate pass, linear per gene: |e32 - e| <= b0[g] + b1 e.
// per gene: X[g] = upper edge of the histogram bin where the count of esub
// reaches k_sub, plus the bound (+inf when fewer than k_sub finite values).
cudaError_t launch_dist_threshold(const float* esub, int64_t n_sub, int64_t G, int64_t k_sub, const float* b0,
                                  float b1, float* X, cudaStream_t s);
cudaError_t launch_fill(float* x, int64_t n, float v, cudaStream_t s);
// dense[p G + g] = e of candidate (p, g)
cudaError_t launch_scatter_errors(const Cand* cand, const float* e, int64_t n, int64_t G, float* out, cudaStream_t s);
// X[g] = e_g + 2 B_g(e_g) for e_g = thr[g] (or eps when thr is null); +inf for e_g >= 10, -1 for e_g < 0.
cudaError_t launch_x_from_thr(const double* thr, double eps, int64_t G, const float* b0, float b1, float* X,
                              cudaStream_t s);
// top-k refinement before the FP64 recheck: per-gene histogram of the
// candidates' FP32 errors, a tighter Xt <= X from the bin completing k, and
// the candidates with e <= Xt appended to out (count in *count).
cudaError_t launch_refine(const Cand* cand, const float* cand_e, int64_t n, int64_t G, int64_t k, const float* X,
                          const float* b0, float b1, unsigned int* hist, float* Xt, Cand* out,
                          unsigned long long* count, cudaStream_t s);
// den[g][k] = (se^2 + 0.01 d^2) + eps_gk, the denominators of the error terms,
// evaluated as in the per-term FP64 expression (bit-identical), and rden = 1/den.
cudaError_t launch_dist_den(const DistInputs& in, double* den, double* rden, cudaStream_t s);
// Group candidates by gene (goff: G + 1 offsets; sp, sg: particle and gene per
// entry), evaluate their FP64 errors in the reference's operation order (se64;
// needs in.den and in.rden) and sort each gene's list by (err, p).
cudaError_t launch_dist_group_recheck_sort(const DistInputs& in, const Cand* cand, int64_t n, int64_t* gcount,
                                           int64_t* goff, unsigned long long* gcursor, int32_t* sp, int32_t* sg,
                                           double* se64, cudaStream_t s);
// The same grouping and order with certified FP32 errors instead of FP64 ones
// (selections that return indices only): se64 holds each pair's certified
// value or, where that cannot decide the order or the threshold (mode 0/2:
// eps or eps_g), its FP64 error.  Scratch: gt (G x K float4), pos and flag
// (n), counts (2: pairs computed in FP64 before / after the sort), dirty (G).
cudaError_t launch_dist_group_certify_sort(const DistInputs& in, const Cand* cand, int64_t n, int mode, double eps,
                                           const double* eps_g, int64_t* gcount, int64_t* goff,
                                           unsigned long long* gcursor, int32_t* sp, int32_t* sg, double* se64,
                                           float4* gt, int32_t* pos, uint8_t* flag,
                                           unsigned long long* counts, int* dirty, cudaStream_t s);
// accepted prefix length per gene (mode 0: err <= eps; mode 1: the k smallest
// finite errors) and, in mode 1, a failure flag when the candidate threshold
// X[g] could have excluded a member of the top k.
cudaError_t launch_dist_accept_len(const int64_t* goff, const double* se64, int64_t G, int mode, double eps,
                                   const double* eps_g, int64_t k, const float* X, const float* b0, float b1,
                                   int64_t* alen, int* fail, bool approx, cudaStream_t s);
// compact the accepted prefixes: idx (1-based particle index + p_base) and err.
cudaError_t launch_dist_compact(const int64_t* goff, const int32_t* sp, const double* se64, const int64_t* aoff,
                                int64_t G, int64_t p_base, int64_t* idx, double* err, cudaStream_t s);
cudaError_t launch_scan(const int64_t* cnt, int64_t G, int64_t* off, cudaStream_t s);
// FP64 errors, in the reference's operation order, of accepted pairs given as
// per-gene lists (offsets aoff, 1-based indices idx - p_base); needs in.den,
// in.rden.  sp, sg: n scratch entries each.
cudaError_t launch_accepted_errors(const DistInputs& in, const int64_t* aoff, const int64_t* idx, int64_t G,
                                   int64_t p_base, int64_t n, int32_t* sp, int32_t* sg, double* err, cudaStream_t s);
// full FP64 error matrix [P][G]
cudaError_t launch_dist_full(const DistInputs& in, double* err, cudaStream_t s);

// moment ODE (moment.cu)
struct MomArgs {
  DevCfg cfg;
  const double* theta;  // [P][ld]
  int64_t ld, P;
  int model;
  double iv[9];
  double h;             // substep (T / (n_steps per_step)), aligned with every breakpoint
  int per_step, nsub;   // substeps per age step and per cycle
  const double* beta_mom;  // [2][A][3]: capture mean, mean of squares, sample variance (pulse, chase cells)
  int n_pulse_conds;
  const double* age_dist;  // [A][J]
  double* stats;           // [P][K]
  double* moments;         // [P][J][A][5] or null
  int* iters;              // [P] transient cycles or null
  double* scratch;         // [grid][2][nsub][100]
  int* status;
};
cudaError_t launch_moment(const MomArgs& a, int grid, cudaStream_t s);
// FP32 production mode (moment_fp32.cu); scratch: moment_f32_scratch_per_cta(nsub) bytes per CTA
size_t moment_f32_scratch_per_cta(int nsub);
cudaError_t launch_moment_f32(const MomArgs& a, int grid, cudaStream_t s);

// data-side statistics and bootstrap standard errors (datastats.cu)
struct DataStatsArgs {
  DevCfg cfg;
  const int32_t* u;  // [G][C] counts, caller's cell order
  const int32_t* l;
  int64_t G, C;
  const int32_t* cell_cond;   // group-sorted cell table (abc_set_cells)
  const int32_t* cell_age;
  const uint32_t* cell_id;    // caller's index of each sorted cell
  const int32_t* gstart;      // [J A + 1] group starts
  const double* age_dist;     // [A][J]
  int n_boot;
  uint64_t seed;
  double* out;                // [G][n_boot + 1][K]
};
cudaError_t launch_data_stats(const DataStatsArgs& a, double* se, cudaStream_t s);
// cells that fit the per-gene shared-memory table of launch_data_stats
int64_t data_stats_max_cells(int n_ages, int n_conds);

// model probabilities with bootstrap intervals and per-gene posterior summaries (posterior.cu)
cudaError_t launch_model_probs(const int64_t* counts, int64_t G, int M, int n_boot, double alpha, uint64_t seed,
                               double* prob, double* lb, double* ub, double* boot, cudaStream_t s);
// scratch: total * npar + 4 * G * npar doubles
cudaError_t launch_posterior_summary(const int64_t* aoff, const int64_t* idx, int64_t G, int64_t total,
                                     const double* theta, int64_t ld, int npar, double q, double* scratch,
                                     double* map, double* mean, double* lb, double* ub, int64_t* n_out,
                                     cudaStream_t s);

cudaError_t launch_prior(const PriorArgs& a, cudaStream_t s);
cudaError_t launch_setup(const SetupArgs& a, cudaStream_t s);
cudaError_t launch_ssa_fp64(const SsaArgs& a, int grid, cudaStream_t s);
// Initial state of every (particle, cell) trajectory of a production-SSA
// launch, in FP64 exactly as the oracle mode draws it: counts[item] =
// (first mRNA count, gene state).  The production kernel reads it at the
// trajectory start and overwrites it with the final counts.
cudaError_t launch_init_states(const SsaArgs& a, int sms, cudaStream_t s);
constexpr int kSsaVariants = 2;
cudaError_t launch_ssa_fp32(const SsaArgs& a, int grid, cudaStream_t s, int variant = 0);
cudaError_t launch_stats(const StatsArgs& a, cudaStream_t s);
// surrogate screen: keep[p] = 1 if L_pg <= X[g] for some g; mode 0:
// L = sum_k w max(0, |d - mu| - z sqrt(var))^2 / K, mode 1: L = m - z sqrt(v)
// with m, v the mean and variance of the error under s ~ N(mu, var)
cudaError_t launch_dist_screen(const float* mu, const float* var, const float* sw, const float* dw, int64_t P,
                               int64_t G, int K, const float* X, float z, int mode, uint8_t* keep, float* err_out,
                               cudaStream_t s);

// particles ordered by expected trajectory cost, descending (hist128: 128 scratch words)
cudaError_t launch_work_order(const PRec* rec, int64_t P, unsigned int* hist128, uint32_t* order, cudaStream_t s);
int ssa_blocks_per_sm_fp64();
int ssa_blocks_per_sm_fp32(int variant = 0);

}  // namespace abc
