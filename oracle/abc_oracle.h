/*
 * abc_oracle.h — FP64 CPU oracle of the ABC simulation + rejection hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libabcgpu.so, the
 * abc_inference_transcription_gb300 package) links, imports or calls this
 * code.  It is used by tests/, by __graft_entry__.smoke() as the checker, and
 * by bench.py's CPU baseline / reference arm.
 *
 * Three oracles, each restating the reference's algorithm in plain C:
 *   (i)   moment ODE  (scripts/model.jl:1-239, scripts/abc_simulation.jl:13-62)
 *   (ii)  FP64 SSA of the same reaction network, project specification,
 *         bit-exact partner of the GPU FP64 mode
 *   (iii) distance + acceptance (scripts/compute_errors.jl:30-70,
 *         scripts/accepted_particles.jl:9-32)
 *
 * How each is pinned: (i) against the reference's golden outputs
 * data/recovered_statistics (fixtures in tests/golden/); the Philox stream
 * against the Random123 known-answer vectors; (ii) statistically against (i);
 * (iii) parity unpinned -- the reference ships no error matrix, accepted list
 * or raw data to recompute them from, so (iii) is checked only against an
 * independent numpy restatement of the same formulas.
 */
#ifndef ABC_ORACLE_H
#define ABC_ORACLE_H
#include <stdint.h>
#include "../include/abcgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* primitives */
void    orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double  orc_xlog(double x);
double  orc_xexp(double x);
/* n draws of Poisson(lam) from one stream (inversion below 10, PTRS above). */
int64_t orc_poisson(double lam, uint64_t seed, uint32_t stream, uint32_t cell, uint32_t particle,
                    int64_t n_draws, int64_t* out);
int64_t orc_binomial(int64_t n, double p, uint64_t seed, uint32_t stream, uint32_t cell,
                     uint32_t particle, int64_t n_draws, int64_t* out);

int orc_num_params(const abc_config* cfg, int model);

/* prior draw (fix_params, abc_simulation.jl:3-11) */
int orc_sample_prior(const abc_config* cfg, int model, int64_t P, uint64_t seed,
                     int64_t particle_offset, const abc_prior* prior, double* theta_out);

/* per-particle setup: rates and the initial means at the start of a cycle.
 * rec_out: 4*S + 7 doubles: kon[S], alp[S], gam[S], amax[S], koff, lam, beta, scal, g0, u0, s0 */
int orc_setup(const abc_config* cfg, int model, const double* theta, double* rec_out);
/* Initial (G, u) of trajectories of cells 0..n-1 of one particle, as the SSA draws them. */
int orc_initial_states(const abc_config* cfg, int model, const double* theta, uint64_t seed, uint32_t particle,
                       int64_t n, int32_t* G_out, int64_t* u_out);

/* FP64 SSA + capture + statistics over P particles x C cells (OpenMP over
 * trajectories when n_threads > 1).  Any output may be NULL.
 * counts/captured: P x C x 2 (u, l); events, hash: P x C; stats: P x nstats. */
int orc_simulate(const abc_config* cfg, int64_t C, const int32_t* cell_cond,
                 const int32_t* cell_age, const double* cell_beta, const double* age_dist,
                 int model, const double* theta, int64_t P, uint64_t seed,
                 int64_t particle_offset, int n_threads, int32_t* counts, int32_t* captured,
                 int64_t* events, uint64_t* hash, int64_t* rejections, double* stats);

/* statistics from per-(condition, age) group moments: m[(j*A + a)*5 + {mu_u, mu_l, var_u, cov_ul, var_l}] */
int orc_stats_from_moments(const abc_config* cfg, const double* m, const double* age_dist,
                           double* stats);

/* moment ODE (reference algorithm).
 * iv: 9 initial moments for the transient phase (abc_simulation.jl:70-71 or recover_statistics.jl:33-34).
 * moments_out: J x A x 5 (mu_u, mu_l, var_u, cov_ul, var_l) before capture.
 * If stats_out != NULL and beta_mom != NULL, also the downsampled statistics:
 *   beta_mom[(set*A + a)*3 + {mean, mean of squares, sample var}] with set 0 = pulse cells
 *   (conditions j < n_pulse_conds), set 1 = chase cells; exact_capture selects the exact
 *   expectation of the empirical moments instead of the reference formula (model.jl:221-239). */
int orc_moment_model(const abc_config* cfg, int model, const double* theta, const double* iv,
                     double h_max, double* moments_out, int* n_transient_iter,
                     const double* beta_mom, int n_pulse_conds, const double* age_dist,
                     int exact_capture, double* stats_out);
int orc_moment_batch(const abc_config* cfg, int model, const double* theta, int64_t P,
                     const double* iv, double h_max, const double* beta_mom, int n_pulse_conds,
                     const double* age_dist, int n_threads, double* stats_out);

/* errors (compute_trunc_errors), err: P x G */
int orc_errors(const double* data, const double* se, int64_t G, int K, int n_fam,
               const int32_t* fam, const double* stats, int64_t P, int n_threads, double* err);
/* acceptance from an error matrix: mode 0 eps, mode 1 top ceil(q*P).
 * offsets: G+1; idx: 1-based particle indices sorted by (err, index). Returns total or <0. */
int64_t orc_accept(const double* err, int64_t P, int64_t G, int mode, double eps_or_q,
                   int64_t* offsets, int64_t* idx, int64_t cap);

int orc_model_probs(const int64_t* counts, int64_t G, int M, int n_boot, double alpha, uint64_t seed,
                    double* prob, double* lb, double* ub);
int orc_posterior_summary(const double* theta, int64_t ld, int npar, const int64_t* off, const int64_t* idx,
                          int64_t G, double q, double* map, double* mean, double* lb, double* ub,
                          int64_t* n_out);
int orc_data_stats(const abc_config* cfg, int64_t C, const int32_t* cell_cond, const int32_t* cell_age,
                   const double* age_dist, const int32_t* u, const int32_t* l, int64_t G, int n_boot,
                   uint64_t seed, double* stats, double* se);
#ifdef __cplusplus
}
#endif
#endif
