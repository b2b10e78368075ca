/*
 * abcgpu.h — C ABI of libabcgpu.so, the GB300 (sm_103a) implementation of the
 * ABC simulation + rejection hot path of pthomaslab/abc_inference_transcription.
 *
 * The reference has no FFI layer: its "API" is a set of Julia functions that
 * are `include`d by wrapper.jl.  Every entry point below names the reference
 * function (file:line, paths inside the reference project) whose role it takes.
 *
 * Conventions
 *   - Status: 0 on success, a negative abc_status on failure.  Nothing aborts
 *     or traps; abc_last_error() returns a message for the last failure.
 *   - Matrices are ROW-MAJOR with the row index first ("P x npar" means row p
 *     holds particle p).  A Julia caller passes the transpose of its
 *     column-major matrix (identical memory).
 *   - Particle indices returned by the acceptance step are 1-based (reference
 *     convention, scripts/accepted_particles.jl:20-26).
 *   - Host pointers unless the function name ends in _device.
 *   - One context = one CUDA stream = one host thread.  Independent contexts
 *     are safe to use from different threads.
 *   - No CPU fallback: without a usable CUDA device abc_create fails.
 */
#ifndef ABCGPU_H
#define ABCGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ABC_MAX_AGES   8
#define ABC_MAX_CONDS 16
#define ABC_MAX_STEPS  8
#define ABC_MAX_PARAMS 32
#define ABC_MAX_FAMILIES 16

/* Statistics per particle in the reference layout (scripts/compute_errors.jl:51,55-57):
 * pulse_mean[A], pulse_ff[A], chase_mean[A], chase_ff[A], ratio[J], mean_corr[J], corr_mean[J]. */
#define ABC_NSTATS(A, J) (4 * (A) + 3 * (J))

typedef enum abc_status {
  ABC_OK = 0,
  ABC_ERR_INVALID = -1,   /* bad argument or configuration */
  ABC_ERR_CUDA = -2,      /* a CUDA runtime call failed */
  ABC_ERR_NOMEM = -3,     /* device allocation failed */
  ABC_ERR_EVENT_CAP = -4, /* a trajectory exceeded abc_config.event_cap fired events */
  ABC_ERR_NONFINITE = -5, /* non-finite rate or count overflow inside a kernel */
  ABC_ERR_CAPACITY = -6,  /* candidate buffer could not be grown or top-q did not converge */
  ABC_ERR_STATE = -7,     /* call order violated (e.g. simulate before set_cells) */
  ABC_ERR_IO = -8         /* a file could not be opened, written or parsed */
} abc_status;

/* Model index m, as in wrapper.jl:47-51 and scripts/abc_simulation.jl:82-85. */
typedef enum abc_model {
  ABC_MODEL_CONST = 1,       /* constant rates, transcription scales with size */
  ABC_MODEL_CONST_CONST = 2, /* constant rates, no size scaling */
  ABC_MODEL_KON = 3,         /* burst frequency k_on varies over the age steps */
  ABC_MODEL_ALPHA = 4,       /* burst size (synthesis rate) varies */
  ABC_MODEL_GAMMA = 5        /* decay rate varies */
} abc_model;

typedef enum abc_precision {
  ABC_FP64 = 0, /* oracle mode: bit-exact with the FP64 CPU oracle */
  ABC_FP32 = 1  /* production mode: FP32 propensities and interval clock, exact breakpoints */
} abc_precision;

/* Time grid, labelling conditions and model options (all times in the unit of
 * the rates; the reference uses hours with cycle = 20, scripts/abc_simulation.jl:65-79). */
typedef struct abc_config {
  double  cycle;                  /* cell-cycle length T */
  int32_t n_burn_cycles;          /* trajectories start at t0 = -n_burn_cycles*T (reference 3, abc_simulation.jl:73) */
  int32_t n_steps;                /* age steps of a varying rate (reference 5, model.jl:181) */
  int32_t n_ages;                 /* A: observation ages (reference 5, abc_simulation.jl:74) */
  int32_t n_conds;                /* J: labelling conditions (reference 11, abc_simulation.jl:65) */
  double  ages[ABC_MAX_AGES];     /* observation ages, each in (0, T) */
  double  pulse[ABC_MAX_CONDS];   /* pulse length per condition */
  double  chase[ABC_MAX_CONDS];   /* chase length per condition */
  int32_t pulse_stat_cond;        /* 0-based condition giving pulse mean/FF (reference j==6 -> 5) */
  int32_t chase_stat_cond;        /* 0-based condition giving chase mean/FF (reference j==7 -> 6) */
  int32_t splicing;               /* 0: reference model (G,u,l); 1: unspliced->spliced, extra theta column */
  int32_t scaling_column;         /* 0: size-scaling exponent fixed by the model; 1: last theta column */
  int32_t precision;              /* abc_precision */
  int32_t reserved0;
  int64_t event_cap;              /* fired events allowed per trajectory (<= 0: 2^28) */
} abc_config;

/* Prior of the log10 rates (scripts/abc_simulation.jl:3-11).  Ranges are log10
 * bounds except scaling, whose bounds are linear (drawn log-uniformly). */
typedef struct abc_prior {
  double kon[2], koff[2], alpha[2], gamma[2], lambda[2], beta[2], scaling[2];
  int32_t vary_mode;   /* 0: the varying rate gets n_steps independent draws (reference);
                          1: base draw times a log-uniform factor per step */
  int32_t reserved0;
  double factor[2];    /* linear factor bounds for vary_mode 1, e.g. {0.2, 5} */
} abc_prior;

typedef struct abc_ctx abc_ctx;

/* Create a context on the current CUDA device.  Replaces the global model
 * configuration of scripts/abc_simulation.jl:64-85. */
int abc_create(abc_ctx** out, const abc_config* cfg);
int abc_destroy(abc_ctx* ctx);
const char* abc_last_error(const abc_ctx* ctx);
/* Number of theta columns for a model under this context's configuration
 * (get_vary_map, scripts/model.jl:30-43, plus the optional extensions). */
int abc_num_params(const abc_ctx* ctx, int model);
/* Number of statistics per particle, 4A + 3J (scripts/compute_errors.jl:51). */
int abc_num_stats(const abc_ctx* ctx);
/* cudaStream_t used by the context, as void*. */
void* abc_stream(abc_ctx* ctx);

/* Synthetic cell table: labelling condition (0-based), age group (0-based) and
 * capture efficiency of each cell, and the A x J age/condition weights
 * (row-major, weights[a*J + j]).  Replaces betas / age / pulse_idx / chase_idx /
 * age_id_distribution (scripts/abc_simulation.jl:14, scripts/load_process_data.jl:68-81).
 * Every (condition, age) group must hold at least 2 cells. */
int abc_set_cells(abc_ctx* ctx, int64_t n_cells, const int32_t* cell_cond,
                  const int32_t* cell_age, const double* cell_beta,
                  const double* age_dist);

/* Prior draw, fix_params (scripts/abc_simulation.jl:3-11).  theta_out: P x npar. */
int abc_sample_prior(abc_ctx* ctx, int model, int64_t n_particles, uint64_t seed,
                     int64_t particle_offset, const abc_prior* prior, double* theta_out);

/* Same draw written to device memory (d_theta_out: P x npar), stream-ordered
 * on abc_stream(ctx). */
int abc_sample_prior_device(abc_ctx* ctx, int model, int64_t n_particles, uint64_t seed,
                            int64_t particle_offset, const abc_prior* prior, double* d_theta_out);

/* Simulate particles and return their statistics, abc_sim
 * (scripts/abc_simulation.jl:13-62; the per-particle loop at :88-97).
 * theta: P x npar (log10 rates), stats_out: P x nstats.  Particle p uses the
 * random streams of global particle index particle_offset + p. */
int abc_simulate(abc_ctx* ctx, int model, const double* theta, int64_t n_particles,
                 uint64_t seed, int64_t particle_offset, double* stats_out);
/* Same with device pointers, stream-ordered on abc_stream(ctx); returns after
 * enqueueing.  abc_synchronize() reports kernel status words. */
int abc_simulate_device(abc_ctx* ctx, int model, const double* d_theta, int64_t n_particles,
                        uint64_t seed, int64_t particle_offset, double* d_stats);
int abc_synchronize(abc_ctx* ctx);

/* Several models in one launch (the five-model ABC batch): particle p is
 * simulated with model models[p] (1..5) from theta row p; the row stride
 * ld_theta must be at least the largest npar of any model (9 for the reference
 * configuration).  Same output as abc_simulate. */
int abc_simulate_batch(abc_ctx* ctx, const int32_t* models, const double* theta, int64_t ld_theta,
                       int64_t n_particles, uint64_t seed, int64_t particle_offset, double* stats_out);
int abc_simulate_batch_device(abc_ctx* ctx, const int32_t* d_models, const double* d_theta, int64_t ld_theta,
                              int64_t n_particles, uint64_t seed, int64_t particle_offset, double* d_stats);

/* abc_simulate_device without any device allocation by the library.  It has
 * no counterpart in the reference.  For callers that may not call cudaMalloc
 * while they run (a runtime that reserved all device memory in its own pool,
 * or a latency-critical loop that must avoid the implicit synchronisation of
 * cudaMalloc/cudaFree) and therefore cannot use abc_create.  Context-free:
 * the cell table comes as host arrays (as for abc_set_cells), theta and the
 * statistics are DEVICE pointers, and the work runs on the caller's stream
 * (cudaStream_t as void*); the call waits for it to finish.  All scratch
 * (particle records, per-cell counts, work counter, status word, sorted cell
 * table) lives in one fixed 64 MiB device array owned by the library and held
 * by every GPU that loads it until exit; particles x cells x 8 bytes plus
 * about 500 bytes per particle must fit, else ABC_ERR_INVALID (e.g. up to
 * ~4,000 particles with 2,000 cells).  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress); the address is kept for
 * the rest of the process, so calls after a cudaDeviceReset of that device
 * are not supported.  Calls
 * share the array: calls that overlap on the GPU race, so serialise them. */
int abc_simulate_noalloc(const abc_config* cfg, int model, int64_t n_cells, const int32_t* cell_cond,
                         const int32_t* cell_age, const double* cell_beta, const double* age_dist,
                         const double* d_theta, int64_t n_particles, uint64_t seed, int64_t particle_offset,
                         double* d_stats, void* stream);

/* Per-cell view of abc_simulate for parity tests: raw counts (u, l) at the
 * observation time, captured counts, fired-event counts and event-sequence
 * hashes, each P x C in the caller's cell order (any pointer may be NULL). */
int abc_simulate_cells(abc_ctx* ctx, int model, const double* theta, int64_t n_particles,
                       uint64_t seed, int64_t particle_offset, int32_t* counts_out,
                       int32_t* captured_out, int64_t* events_out, uint64_t* hash_out,
                       double* stats_out);

/* Counters of the last simulate call: fired events and thinning rejections. */
int abc_last_counters(const abc_ctx* ctx, int64_t* events, int64_t* rejections);
/* Per-kernel device timing (CUDA events on the context stream), the tracing
 * counterpart of the reference's @time (scripts/abc_simulation.jl:88).
 * abc_profile_read returns, for the last synchronized simulate call, the
 * milliseconds spent in [setup, SSA, capture+statistics] kernels. */
int abc_profile(abc_ctx* ctx, int enable);
/* Whether the configuration's times (t0, cycle, age step, ages, pulses,
 * chases) are all integer multiples of a power-of-two quantum, in which case
 * the production SSA places breakpoints with integer arithmetic instead of
 * FP64: returns 1 (and *quantum, may be NULL) or 0; ABC_ERR_INVALID for an
 * invalid configuration.  Host only.  No reference counterpart. */
int abc_breakpoint_grid(const abc_config* cfg, double* quantum);
/* Autotuner (no reference counterpart; the reference tunes nothing): times the
 * production SSA kernel variants (register allocation for 8 or 10 resident
 * blocks per SM) on a sample of particles, twice each in alternating order,
 * and keeps the fastest for this context (variant 0, the one without register
 * spills, unless another is more than 2 % faster).  ms_out: the faster kernel
 * milliseconds of each variant (2 entries, may be NULL). */
int abc_autotune(abc_ctx* ctx, int model, const double* theta, int64_t n_particles, uint64_t seed,
                 double* ms_out, int* chosen);
/* Autotuner over the kernel's two tunable axes, on a mixed-model sample
 * (rows padded to ld_theta, as abc_simulate_batch; no reference
 * counterpart): register variant (8 or 10 resident blocks per SM) x work
 * chunk (1, 4 or 16 consecutive (particle, cell) items per lane and pull),
 * each pair timed twice in alternating order; the context keeps the fastest
 * pair unless it is within 2 % of (variant 0, chunk 1).  ms_out: 6 entries,
 * ms_out[variant * 3 + chunk index] (may be NULL). */
int abc_autotune_batch(abc_ctx* ctx, const int32_t* models, const double* theta, int64_t ld_theta,
                       int64_t n_particles, uint64_t seed, double* ms_out, int* chosen_variant,
                       int* chosen_chunk);
int abc_set_variant(abc_ctx* ctx, int variant);
/* Work items (consecutive cells of a particle) a lane of the production
 * kernel takes per pull from the work counter, 1..1024 (default 1). */
int abc_set_work_chunk(abc_ctx* ctx, int chunk);
int abc_profile_read(const abc_ctx* ctx, double* ms_out);

/* Error matrix, compute_trunc_errors / nlsqerror_part (scripts/compute_errors.jl:30-70):
 * err[p*G+g] = min(10, sum_f sum_{k in f} (d-s)^2/(se^2+0.01 d^2+eps)/K).
 * data, se: G x K; stats: P x K; family sizes sum to K (NULL: one family). */
int abc_errors(abc_ctx* ctx, const double* data, const double* se, int64_t n_genes, int K,
               int n_families, const int32_t* family_sizes, const double* stats,
               int64_t n_particles, double* err_out);

/* Acceptance, scripts/accepted_particles.jl:12-32.  mode 0: accept err <= eps
 * (reference eps = 4.8); mode 1: accept the ceil(q*P) smallest errors per gene.
 * Accepted sets equal the FP64 oracle's; lists are sorted by (err, index).
 * Results stay in the context; fetch them with abc_accept_fetch. */
int abc_errors_select(abc_ctx* ctx, const double* data, const double* se, int64_t n_genes,
                      int K, int n_families, const int32_t* family_sizes,
                      const double* stats, int64_t n_particles, int mode, double eps_or_q,
                      int64_t* n_accepted_total);
/* Acceptance with a threshold per gene (thr: G entries, host), e.g. the
 * thresholds a top-q selection produced; same output as abc_errors_select. */
int abc_errors_select_thr(abc_ctx* ctx, const double* data, const double* se, int64_t n_genes, int K,
                          int n_families, const int32_t* family_sizes, const double* stats,
                          int64_t n_particles, const double* thr, int64_t* n_accepted_total);
/* abc_errors_select with the statistics in device memory (e.g. the d_stats of
 * abc_simulate_device); mode 2 takes per-gene thresholds thr (host). */
int abc_errors_select_device(abc_ctx* ctx, const double* data, const double* se, int64_t n_genes, int K,
                             int n_families, const int32_t* family_sizes, const double* d_stats,
                             int64_t n_particles, int mode, double eps_or_q, const double* thr,
                             int64_t* n_accepted_total);
/* Whether selections keep the FP64 error of every accepted pair (1, the
 * default) or return indices only (0).  With 0 the accepted sets and their
 * order are the same, but the order is decided from certified FP32 errors
 * (|e32 - err64| <= (1e-6 + 1e-12) e32 + 1e-12, derived in distance_fp64.cu)
 * and FP64 is computed only for pairs those cannot place;
 * abc_accept_fetch then requires err = NULL.  The reference's acceptance
 * writes indices only (scripts/accepted_particles.jl:21-29). */
int abc_set_select_errors(abc_ctx* ctx, int keep_errors);
/* FP64 errors (compute_errors.jl:30-43, 62-64, the reference's operation
 * order) of the last selection's accepted pairs, in the order of
 * abc_accept_fetch's indices; for selections made with
 * abc_set_select_errors(ctx, 0), computed now for the accepted pairs only --
 * e.g. a particle shard's local top-k, which a host merge of several shards'
 * lists needs.  The statistics of the selection must still be in place (a
 * d_stats pointer given to abc_errors_select_device). */
int abc_accept_errors(abc_ctx* ctx, double* err);
/* gene_offsets: G+1 entries; particle_idx: 1-based, n_accepted_total entries;
 * err: FP64 errors of the accepted pairs (may be NULL; must be NULL after a
 * selection with abc_set_select_errors(ctx, 0)). */
int abc_accept_fetch(abc_ctx* ctx, int64_t* gene_offsets, int64_t* particle_idx, double* err);
/* CUDA graph mode for the simulation chain (setup -> work order -> SSA ->
 * capture + statistics) of abc_simulate_device, abc_simulate_batch_device
 * and abc_simulate_batch: each call captures the chain on the context's
 * stream and updates one instantiated graph in place (re-instantiating only
 * when the chain's shape changes), then launches it.  Results are identical
 * to the plain launches.  No reference counterpart. */
int abc_set_graph(abc_ctx* ctx, int enable);
/* graph instantiations and in-place updates so far */
int abc_graph_counters(const abc_ctx* ctx, int64_t* instantiations, int64_t* updates);
/* Counters of the last selection: pairs emitted by the FP32 candidate
 * pass(es), and pairs rechecked in FP64 (after the top-k refinement). */
int abc_select_counters(const abc_ctx* ctx, int64_t* candidates, int64_t* rechecked);
/* With abc_profile on: device milliseconds of the candidate-pass kernel of
 * the last selection, summed over its passes, and the number of passes. */
int abc_select_profile_read(const abc_ctx* ctx, double* fast_ms, int* fast_passes);
/* Candidate pass of the selections (the FP32 screen in front of the FP64
 * recheck of scripts/compute_errors.jl:30-43; no reference counterpart, the
 * reference evaluates every pair in FP64):
 *   0  FP32 on the CUDA cores, 2 FMA per (particle, gene, statistic);
 *   1  TF32 tensor cores, K err = c_g + [s | s^2] . [-2 w d | w], one term;
 *   2  as 1 with hi/lo TF32 splits (three terms, ~FP32 products);
 *   3  as 2 with hi/lo BF16 splits (products to ~2^-17 relative; BF16 MMAs
 *      with the gene rows resident in shared memory; default).  Rows longer
 *      than 4K = 384 values (K > 96) do not fit; such a selection runs mode 2.
 * Modes 1-3 fall back to 0 for a selection whose inputs hold an infinite
 * value or could overflow FP32 in w s^2.  Accepted sets do not depend on the
 * mode: every mode is followed by the same FP64 recheck. */
int abc_set_distance_mode(abc_ctx* ctx, int mode);
/* requested mode, and the mode the last selection used (-1 before any). */
int abc_get_distance_mode(const abc_ctx* ctx, int* requested, int* used);
/* Diagnostic: the candidate pass's FP32 error of every pair (row-major
 * [P][G], P G <= 2^28; NaN where the pass yields NaN) with its error bound
 * |err_out - err| <= b0_out[g] + b1_out err against the exact error of
 * abc_errors (both clipped at 10), and the mode used.  b0_out, b1_out and
 * mode_used may be NULL. */
int abc_errors_candidate(abc_ctx* ctx, const double* data, const double* se, int64_t n_genes, int n_stats,
                         int n_fam, const int32_t* fam, const double* stats, int64_t n_particles, float* err_out,
                         double* b0_out, double* b1_out, int* mode_used);

/* ------------------------------------------------------------------------
 * Deterministic simulation (the reference's own): the 9-moment ODE of the
 * model (scripts/model.jl:67-96), its periodic steady state by the 1 %
 * transient rule from iv (:114-142, iv as in abc_simulation.jl:70-71), the
 * multi-cycle trajectories with division for every (condition, age)
 * (:98-111, :146-199), the capture moment transform with the per-cluster
 * capture moments beta_mom[2][A][3] = {mean, mean of squares, sample
 * variance} of the pulse and the chase cells (:221-239), and the statistics
 * of abc_simulation.jl:13-62 with age_dist[A][J].  Exponential midpoint rule
 * on a substep grid h <= h_max aligned with every breakpoint (h_max <= 0:
 * cycle / 400 in FP64, cycle / 80 in FP32).  stats_out [P][K]; moments_out [P][J][A][5] (E u, E l, Var u,
 * Cov ul, Var l before capture) and iters_out [P] (transient cycles) may be
 * NULL.  No splicing.  Replaces the CVODE-based abc_sim path.  Precision of
 * the context: ABC_FP64 = the oracle's arithmetic, bit for bit; ABC_FP32 =
 * production mode (FP32 propagators and states on the triangular form of the
 * moment matrix, FP64 rates and statistics). */
int abc_moment_simulate(abc_ctx* ctx, int model, const double* theta, int64_t n_particles, const double* iv,
                        double h_max, const double* beta_mom, int n_pulse_conds, const double* age_dist,
                        double* stats_out, double* moments_out, int32_t* iters_out);

/* Data side (scripts/data_summary_statistics.jl:1-216): the statistics of
 * observed counts, u[g][c] and l[g][c] (non-negative integers <= 2^20, cells
 * in the order given to abc_set_cells), per gene in the simulated layout
 * (pulse mean and FF of u + l per age over the pulse-statistic cells, chase
 * likewise, per-condition ratio of means, mean_corr and corr_mean with the
 * context's age weights), and, if se_out is not NULL, their bootstrap
 * standard errors over n_boot >= 2 resamples of the cells (per family, as the
 * reference's get_*_se; the correlation resamples re-weight the ages by their
 * resampled fractions within each condition).  Resamples come from a Philox
 * stream keyed by (seed, family, resample, gene).  stats_out, se_out [G][K]. */
int abc_data_stats(abc_ctx* ctx, const int32_t* u_counts, const int32_t* l_counts, int64_t n_genes, int n_boot,
                   uint64_t seed, double* stats_out, double* se_out);

/* ------------------------------------------------------------------------
 * Downstream of the acceptance.
 *
 * Model probabilities (scripts/model_probs.jl:1-28, per-gene driver :37-62):
 * counts[g][m] = accepted particles of model group m for gene g.  No
 * acceptance: zeros; one group: that group's probability and bounds 1;
 * otherwise counts / sum and the quantiles 1 - alpha and alpha (Julia's
 * default quantile) of n_boot bootstrap resamples of the accepted model
 * labels (the reference uses n_boot = 100, alpha = 0.95).  The resamples come
 * from a Philox stream keyed by (seed, bootstrap, gene), not from Julia's RNG.
 * Outputs [G][M]. */
int abc_model_probs(abc_ctx* ctx, const int64_t* counts, int64_t n_genes, int n_groups, int n_boot, double alpha,
                    uint64_t seed, double* prob, double* lower, double* upper);
/* Posterior summaries of the last selection (scripts/posterior_kinetics.jl:
 * 1-33, get_n_particles, get_posterior_estimate "map"/"mean",
 * get_posterior_ci): per gene and parameter column the parameters of the
 * first accepted particle (lowest error), the mean over the accepted
 * particles (summed in list order), and the quantiles 1 - q and q; NaN for a
 * gene without acceptance.  theta: [P][ld] with the selection's particle
 * order, on the host or (theta_on_device) the device.  Outputs [G][npar],
 * n_particles[G] (may be NULL). */
int abc_posterior_summary(abc_ctx* ctx, const double* theta, int64_t ld, int npar, int theta_on_device, double q,
                          double* map, double* mean, double* lower, double* upper, int64_t* n_particles);

/* ------------------------------------------------------------------------
 * Learned pre-screen.  No reference counterpart: the reference simulates
 * every prior draw.  An ensemble of MLPs (log-parameters -> means and
 * log-variances of the statistics; 3 x 256 SiLU hidden layers; FP32 master
 * weights, BF16 tensor-core GEMMs) is trained on the pipeline's own SSA output;
 * the screen keeps a prior draw when its predicted expected error
 * sum_k w (d - mu)^2 + w var, / K, is within a gene's threshold plus a
 * calibrated margin for some gene, or when the ensemble disagrees.
 * ------------------------------------------------------------------------ */
typedef struct abc_surrogate abc_surrogate;
int abc_surrogate_create(abc_surrogate** out, int in_dim, int n_stats, int ensemble, uint64_t seed);
int abc_surrogate_destroy(abc_surrogate* s);
const char* abc_surrogate_last_error(const abc_surrogate* s);
int abc_surrogate_num_params(const abc_surrogate* s);
/* theta: N x in_dim (log10 rates), stats: N x n_stats (non-finite entries are
 * masked).  Fits the input/output standardisation on this data, then runs
 * `epochs` passes of Adam (batch rows per step).  epoch_loss: mean Gaussian NLL. */
int abc_surrogate_train(abc_surrogate* s, const double* theta, const double* stats, int64_t n, int epochs,
                        int batch, double lr, double* epoch_loss);
/* Loss per member and gradients (members x num_params floats) of one batch, no update. */
int abc_surrogate_gradients(abc_surrogate* s, const double* theta, const double* stats, int64_t n,
                            double* loss, float* grads);
int abc_surrogate_get_params(abc_surrogate* s, float* params);
int abc_surrogate_set_params(abc_surrogate* s, const float* params);
int abc_surrogate_get_norm(abc_surrogate* s, double* xmean, double* xstd, double* ymean, double* ystd);
int abc_surrogate_set_norm(abc_surrogate* s, const double* xmean, const double* xstd, const double* ymean,
                           const double* ystd);
/* Ensemble mean, total predictive variance and disagreement
 * (max_k sqrt(ensemble variance / mean aleatoric variance)) per row. */
int abc_surrogate_predict(abc_surrogate* s, const double* theta, int64_t n, double* mean, double* var,
                          double* disagree);
int abc_surrogate_predict_device(abc_surrogate* s, const double* d_theta, int ld_theta, int64_t n,
                                 double* d_mean, double* d_var, double* d_disagree);
/* d_keep[p] = 1 for the draws to simulate exactly: the lower confidence
 * bound sum_k w max(0, |d - mu| - z sd)^2 / K of the error (mu, sd: predicted
 * mean and total predictive std of each statistic) is <= thr[g] + margin for
 * some gene, or the disagreement exceeds disagree_max.  data, se: G x n_stats
 * (host), thr: per-gene error threshold (host).  err_out (host, n x G,
 * optional, small n only): the bounds, for calibration. */
int abc_surrogate_screen_device(abc_surrogate* s, const double* d_theta, int ld_theta, int64_t n,
                                const double* data, const double* se, int64_t n_genes, const double* thr,
                                double margin, double z, double disagree_max, uint8_t* d_keep, int64_t* n_keep,
                                double* err_out);
/* Statistic of abc_surrogate_screen_device.  0 (default): per-statistic lower
 * bound L = sum_k w_k max(0, |d_k - mu_k| - z sd_k)^2 / K.  1: lower quantile of
 * the error's predictive distribution, L = m - z sqrt(v), where m and v are
 * the mean and variance of sum_k w_k (d_k - s_k)^2 / K for independent
 * s_k ~ N(mu_k, sd_k^2).  No reference counterpart. */
int abc_surrogate_set_screen_mode(abc_surrogate* s, int mode);
/* Survivors of a screen in ascending order: rows with d_keep != 0 copied from
 * d_theta (row stride ld_theta) to d_theta_out and their indices to d_idx_out
 * (either output may be NULL); *n_out = number of survivors. */
int abc_surrogate_compact_device(abc_surrogate* s, const uint8_t* d_keep, const double* d_theta, int ld_theta,
                                 int64_t n, double* d_theta_out, int64_t* d_idx_out, int64_t* n_out);

/* ---- on-disk text formats (host only, no context) ----------------------
 * Tab-delimited rows as the reference's DelimitedFiles.writedlm writes them;
 * floats in the shortest form that reads back to the same double (Julia's
 * spelling: "1.0", "2.5e-5", NaN, Inf).  append != 0 appends, as the
 * reference's scripts do.  Return ABC_OK, ABC_ERR_INVALID or ABC_ERR_IO. */
/* particles_<model>.txt (scripts/accepted_particles.jl:21-29): one line per
 * gene with its accepted 1-based indices, or "0" when none; gene_offsets has
 * n_genes + 1 entries (the layout abc_accept_fetch returns). */
int abc_write_particles(const char* path, int append, int64_t n_genes, const int64_t* gene_offsets,
                        const int64_t* particle_idx);
/* rows x cols row-major matrix with leading dimension ld: sets_<model>.txt
 * (scripts/abc_simulation.jl:93-94), the s_pulse / s_chase / s_ratios /
 * s_mean_corr / s_corr_mean files (:47-60), error_<model>.txt
 * (scripts/compute_errors.jl:66-67), model_prob / l_bound / u_bound
 * (scripts/model_probs.jl:54-61), posterior estimates
 * (scripts/posterior_kinetics.jl:72-75). */
int abc_write_matrix(const char* path, int append, int64_t rows, int64_t cols, const double* m, int64_t ld);
/* one float as abc_write_matrix writes it (buf_len >= 32); returns its length */
int abc_format_double(double x, char* buf, int buf_len);
/* particles file -> offsets (n_genes + 1) and 1-based indices, as
 * scripts/posterior_kinetics.jl:56-60 reads it ("0" = no particle).  First
 * call with gene_offsets = particle_idx = NULL for the sizes. */
int abc_read_particles(const char* path, int64_t* n_genes, int64_t* n_total, int64_t* gene_offsets,
                       int64_t* particle_idx);

#ifdef __cplusplus
}
#endif
#endif /* ABCGPU_H */
