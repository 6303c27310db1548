/*
 * busseq_gb300.h -- C ABI of the GB300-native BUSseq Gibbs sampler.
 *
 * The reference (Anguscgm/BUSseq_gpu, a single CUDA C program) exposes no
 * library: its boundary is the executable's command line and its text files.
 * This header is the drop-in boundary of that path as a shared library
 * (libbusseq_gb300.so); the `busseq` executable built on top of it keeps the
 * reference's command line and output files.  Each entry point names the
 * reference code it replaces (BUSseq_gpu.cu:line).
 *
 * Conventions: plain C types, caller-owned host buffers, an opaque handle per
 * chain, one GPU, not thread-safe per handle.  Every function returns 0
 * (BUSSEQ_OK) or a negative error code; busseq_last_error() then describes the
 * failure.  Arrays use the reference's layouts: counts row-major [cell][gene]
 * with cells grouped batch by batch; beta/L [k*G+g]; nu/phi [b*G+g];
 * gamma [0/1*B+b]; pi [b*K+k].
 */
#ifndef BUSSEQ_GB300_H
#define BUSSEQ_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BUSSEQ_OK 0
#define BUSSEQ_ERR_ARG (-1)      /* invalid argument or input data            */
#define BUSSEQ_ERR_CUDA (-2)     /* CUDA runtime error                        */
#define BUSSEQ_ERR_NOMEM (-3)    /* device or host allocation failed          */
#define BUSSEQ_ERR_STATE (-4)    /* call out of order (e.g. no run begun)     */
#define BUSSEQ_ERR_SAMPLER (-5)  /* a device sampler cap or copy wait bound   */
#define BUSSEQ_ERR_IO (-6)       /* file could not be read or written         */

#define BUSSEQ_MAX_BATCHES 128   /* BUSseq_gpu.cu:9-10 (__constant__ d_n_b[128]) */
#define BUSSEQ_MAX_TYPES 64

/* W update: the reference's Metropolis move with a uniform proposal
 * (BUSseq_gpu.cu:820-854), or a K-way categorical draw from the same full
 * conditional. */
#define BUSSEQ_W_MH 0
#define BUSSEQ_W_GIBBS 1

/* Stage ids for busseq_run_stage: contiguous groups of the reference's sweep
 * order (BUSseq_gpu.cu:1267-1398). */
#define BUSSEQ_STAGE_ZX_GAMMA_ALPHA_L 0 /* Z/X, gamma0, gamma1, alpha, L, p/tau0 */
#define BUSSEQ_STAGE_BETA_NU 1          /* beta, nu                            */
#define BUSSEQ_STAGE_DELTA 2
#define BUSSEQ_STAGE_PHI 3
#define BUSSEQ_STAGE_W 4
#define BUSSEQ_STAGE_PI 5               /* pi, then the new cell order         */

typedef struct busseq_handle busseq_handle;

typedef struct busseq_dims {
  int32_t B;            /* batches (2..128), reference -B                      */
  int32_t K;            /* cell types (1..64), reference -K                    */
  int64_t G;            /* genes, reference -G                                 */
  const int32_t* n_b;   /* [B] cells per batch, reference -N file               */
} busseq_dims;

typedef struct busseq_options {
  uint64_t seed;        /* key of every random draw (reference -s)             */
  double p0;            /* initial p; the reference uses rand()*0.5/RAND_MAX    */
  int32_t w_update;     /* BUSSEQ_W_MH (default) or BUSSEQ_W_GIBBS             */
  int32_t keep_draws;   /* store every kept draw (needed for reference -p)      */
  int32_t device;       /* CUDA device ordinal                                 */
  int32_t chunk_cells;  /* cells per gene-pass chunk; 0 = default (128 for the
                           random-walk sampler when a (batch, type) segment
                           averages under 512 cells, else 256)                 */
  int32_t hmc_leapfrog; /* 0: random-walk MH for alpha, beta, nu, delta, phi (the
                           reference's sampler); L > 0: one Hamiltonian Monte Carlo
                           transition of that block per sweep with L leapfrog
                           steps (not in the reference)                         */
  int32_t zx_summaries; /* 1: over the kept sweeps, count Z = 1 and sum X at every
                           Y == 0 entry (busseq_get_zx_summaries; not in the
                           reference, which writes the last sweep's Z and X)    */
  int32_t hmc_gene_accept; /* with hmc_leapfrog > 0: 1 moves every gene's block
                           (alpha, beta, nu, log phi) along one shared trajectory
                           and accepts or rejects each gene on its own energy
                           change (the block posterior factorises over genes
                           given delta); delta then takes the random-walk step.
                           0: one decision for the whole block, delta included */
  int32_t test_nb_inv_cap; /* tests of the failure path only: > 0 lowers the search
                           cap of the Z/X update's NB inversion (default and
                           maximum 1024), so that the cap is reached and the run
                           reports BUSSEQ_ERR_SAMPLER; 0 for every real run      */
  int32_t zx_unit;      /* Y == 0 entries per Z/X work unit (a warp's claim),
                           16..512; 0 = default (512).  Launch shape only: the
                           draws do not depend on it                          */
  int32_t zx_ctas_per_sm; /* resident Z/X CTAs per SM, 1..4; 0 = default (4).
                           Launch shape only                                   */
  int32_t reserved[2];
} busseq_options;

/* Posterior estimates (BUSseq_gpu.cu:1557-1813).  Every pointer is a
 * caller-owned host buffer of the stated length, or NULL to skip it. */
typedef struct busseq_estimates {
  int32_t* Z;       /* [N*G] last sweep's dropout indicators (_post_Z)       */
  int32_t* X;       /* [N*G] last sweep's underlying counts (_post_X)        */
  double* gamma;    /* [2B]  posterior means (_post_gamma)                  */
  double* alpha;    /* [G]                                                  */
  double* L;        /* [(K-1)*G] posterior P(L=1), k >= 1 (_post_L)          */
  double* beta;     /* [K*G] posterior means, row k=0 is 0 (_post_beta)     */
  double* p_tau0;   /* [2]  posterior means of p and tau0 (_post_p)         */
  double* nu;       /* [B*G] row b=0 is 0 (_post_nu)                         */
  double* delta;    /* [N]                                                  */
  double* phi;      /* [B*G]                                                */
  int32_t* W;       /* [N]  posterior mode, 0-based (_post_W)               */
  double* pi;       /* [B*K]                                                */
} busseq_estimates;

/* Kept draws in the reference's file layout: one row per scalar, one column
 * per kept sweep (BUSseq_gpu.cu:1845-2018).  NULL pointers are skipped. */
typedef struct busseq_preserved {
  double* gamma;    /* [2B][n_kept]        */
  double* alpha;    /* [G][n_kept]         */
  int32_t* L;       /* [(K-1)G][n_kept]    */
  double* beta;     /* [(K-1)G][n_kept]    */
  double* p_tau0;   /* [2][n_kept]         */
  double* nu;       /* [(B-1)G][n_kept]    */
  double* delta;    /* [N][n_kept]         */
  double* phi;      /* [BG][n_kept]        */
  int32_t* W;       /* [N][n_kept]         */
  double* pi;       /* [BK][n_kept]        */
} busseq_preserved;

/* Full sampler state in single precision (the kernels' working precision).
 * Used by tests and by callers that checkpoint a chain. */
typedef struct busseq_state {
  int32_t* X;       /* [N*G] */
  uint8_t* Z;       /* [N*G] */
  int32_t* W;       /* [N]   */
  int8_t* L;        /* [K*G] */
  float* alpha;     /* [G]   */
  float* mu_alpha;  /* [G]   */
  float* beta;      /* [K*G] */
  float* nu;        /* [B*G] */
  float* mu_nu;     /* [B]   */
  float* delta;     /* [N]   */
  float* mu_delta;  /* [N]   */
  float* phi;       /* [B*G] */
  float* gamma;     /* [2B]  */
  float* pi;        /* [B*K] */
  float* p_tau0;    /* [2]   */
} busseq_state;

/* Log acceptance ratios (likelihood + prior) computed by the last sweep or
 * stage, for diagnostics and parity tests.  NULL pointers are skipped. */
typedef struct busseq_log_ratios {
  double* gamma;    /* [2B]  */
  double* alpha;    /* [G]   */
  double* beta;     /* [K*G] (k >= 1) */
  double* nu;       /* [B*G] (b >= 1) */
  double* delta;    /* [N]   */
  double* phi;      /* [B*G] */
  double* W;        /* [N]   MH: the log ratio of the proposal; K-way draw: the
                       log weight of the drawn type minus that of the current one */
} busseq_log_ratios;

/* ---- lifecycle ------------------------------------------------------------ */

/* Uploads the N x G counts (host or device pointer, row-major, rows of G
 * int32) and initialises the chain.  Replaces reading the count file's
 * contents into device memory and the initialisation of BUSseq_gpu.cu:1143-1244. */
int busseq_create(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, const busseq_options* opt,
                  busseq_handle** out);

/* Releases all device memory of the chain.  Safe with NULL. */
void busseq_destroy(busseq_handle* h);

/* Runs n_iter sweeps (n_burnin of burn-in), with p and tau0 held for the
 * first n_unchanged sweeps, then computes the posterior summaries.
 * Replaces BUSseq_gpu.cu:1246-1608. */
int busseq_run(busseq_handle* h, int32_t n_iter, int32_t n_burnin, int32_t n_unchanged);

/* Incremental form of busseq_run: busseq_begin fixes the run's lengths and
 * resets the sweep counter; busseq_sweeps enqueues `count` sweeps (CUDA graphs,
 * asynchronous); busseq_finish waits and computes the posterior summaries. */
int busseq_begin(busseq_handle* h, int32_t n_iter, int32_t n_burnin, int32_t n_unchanged);
int busseq_sweeps(busseq_handle* h, int32_t count);
int busseq_finish(busseq_handle* h);
int busseq_synchronize(busseq_handle* h);

/* Copies the posterior estimates into host buffers (BUSseq_gpu.cu:1557-1813). */
int busseq_get_estimates(busseq_handle* h, busseq_estimates* out);

/* Copies the kept draws (requires keep_draws; BUSseq_gpu.cu:1845-2018). */
int busseq_get_preserved(busseq_handle* h, busseq_preserved* out);

/* BIC of the posterior estimates, marginalising dropouts and cell types
 * (BUSseq_gpu.cu:967-1024 and :1815-1843). */
int busseq_bic(busseq_handle* h, double* bic);

/* BIC without any device allocation.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc -- code whose device memory is all
 * owned by a framework's pool or arena, or that must not grow its footprint
 * after start-up.  The caller passes device pointers: Y [N*G] int32 (row
 * stride G), the estimates in busseq_estimates' layouts (double), and out_dev
 * [2] = {BIC, log-likelihood}.  Work is enqueued on cuda_stream (NULL = the
 * default stream); synchronise it before reading out_dev.
 * Scratch: a fixed static __device__ array of BUSSEQ_NOALLOC_BIC_MAX_TYPES_X_CELLS
 * doubles (8 MB) plus BUSSEQ_NOALLOC_BIC_MAX_CELLS ints (1 MB), held by every
 * GPU that loads the library until the process exits.  Larger problems are
 * rejected (BUSSEQ_ERR_ARG).  All calls share that array: calls that overlap
 * on the GPU (other streams, other host threads) race.  The kernels run on the
 * calling thread's current device, which must own every pointer passed in
 * (checked; BUSSEQ_ERR_ARG otherwise).  Each call made outside stream capture
 * looks up the array's device address again (so a device reset, after which
 * the library's module is loaded afresh, is followed); a call made during
 * capture reuses the address found by the last call outside capture on that
 * device, so make the first call on a device before any stream capture. */
#define BUSSEQ_NOALLOC_BIC_MAX_TYPES_X_CELLS (1 << 20)
#define BUSSEQ_NOALLOC_BIC_MAX_CELLS (1 << 18)
int busseq_bic_noalloc(const busseq_dims* dims, const int32_t* Y_dev, const double* alpha_dev,
                       const double* beta_dev, const double* nu_dev, const double* delta_dev,
                       const double* phi_dev, const double* gamma_dev, const double* pi_dev, double* out_dev,
                       void* cuda_stream);

/* ---- state access, single stages, diagnostics ----------------------------- */

/* n draws from one of the device samplers that the sweep kernels use, into
 * host memory, for distribution tests.  Draw j uses the Philox stream (seed,
 * 40 + family, j, 0), the streams of the FP64 oracle's sample functions.
 *   kind 0: Gamma(shape a, scale 1), Marsaglia-Tsang         out: float[n]
 *   kind 1: Poisson(a), inversion / PTRS                      out: int32[n]
 *   kind 2: NB(mean a, size b) as the Z/X update draws it     out: int32[n]
 *   kind 3: NB(mean a, size b), Gamma-Poisson always          out: int32[n]
 *   kind 4: NB(mean a, size b), inversion always (b >= 1)     out: int32[n]
 * No counterpart in the reference, whose samplers (BUSseq_gpu.cu:34-218) are
 * only called inside its update kernels.  Returns BUSSEQ_ERR_SAMPLER when a
 * sampler cap was reached. */
int busseq_sample_draws(int32_t kind, double a, double b, uint64_t seed, int64_t n, void* out);

/* Batch-corrected counts [N*G] (cells x genes, the layout of Y): each imputed
 * count of the last sweep (_post_X) mapped by randomised quantile matching
 * from NB(exp(alpha_g + beta_gw + nu_bg + delta_i), phi_bg) to the batch-free
 * NB(exp(alpha_g + beta_gw), phi_1g), with the posterior means and the
 * posterior-mode type w = W_i.  Not in BUSseq_gpu.cu: the BUSseq method's
 * corrected read counts, computed from the outputs that BUSseq_gpu.cu writes
 * (:1557-1813).  The uniforms are keyed by the handle's seed, so a call is
 * reproducible.  out is a host buffer, or device memory when out_is_device. */
int busseq_corrected_counts(busseq_handle* h, int32_t* out, int32_t out_is_device);

/* Posterior summaries of the imputation [N*G] (cells x genes), over the kept
 * sweeps of a finished run made with opt.zx_summaries: x_mean = E[X] (= Y
 * where Y > 0) and z_prob = P(Z = 1) (0 where Y > 0).  NULL pointers are
 * skipped. */
int busseq_get_zx_summaries(busseq_handle* h, float* x_mean, float* z_prob);

int busseq_get_state(busseq_handle* h, busseq_state* out);
/* Replaces the whole state; derived data (exp(delta), exp(alpha+beta+nu), the
 * cell order) is recomputed on the device. */
int busseq_set_state(busseq_handle* h, const busseq_state* in);

/* Checkpoint and resume (no reference equivalent: the reference program can
 * neither stop nor continue a run).  busseq_checkpoint_save writes the chain
 * state (X and Z of the Y == 0 entries, W, L and every parameter), and, when a
 * run has begun, its lengths, sweep counters, posterior accumulators and kept
 * draws, to `path` (through `path`.tmp and a rename).  busseq_checkpoint_load
 * restores them into a handle created from the same counts (checked by a
 * fingerprint), dimensions, seed, W move and keep_draws setting; the run then
 * continues with busseq_sweeps / busseq_finish.  Draws are keyed by the sweep
 * index, so a resumed run reproduces an uninterrupted one bit for bit. */
int busseq_checkpoint_save(busseq_handle* h, const char* path);
int busseq_checkpoint_load(busseq_handle* h, const char* path);

/* Gradient-based block update (opt.hmc_leapfrog > 0).
 * busseq_hmc_stats: out[0] step size, out[1] acceptance rate over the kept
 * sweeps so far, out[2] acceptance probability of the last transition, out[3]
 * its change of the Hamiltonian.
 * busseq_hmc_gradient: the gradient of the block's log posterior at the
 * current state, and (when `metric` is not NULL) the diagonal metric the
 * transitions would adapt to there, in the flat layout
 *   alpha [G] | beta [K*G] | nu [B*G] | log phi [B*G] | delta [N]
 * (fixed coordinates: gradient 0, metric 1; with hmc_gene_accept delta is
 * fixed).
 * busseq_hmc_logpost_diff: log posterior of the current state minus that of
 * `from` (same conditioning: X, W, L, p, tau0 of the current state).
 * busseq_hmc_gene_logpost_diff (hmc_gene_accept chains): the same change per
 * gene, out[G]: gene g's block (alpha_g, beta_g., nu_g., phi_.g) with delta
 * held at the current state's (`from` must carry the same delta).
 * With hmc_gene_accept, out[1] of busseq_hmc_stats is the mean fraction of
 * genes accepted and out[2] their mean acceptance probability.  */
int busseq_hmc_stats(busseq_handle* h, double out[4]);
int busseq_hmc_gradient(busseq_handle* h, double* grad, double* metric);
int busseq_hmc_logpost_diff(busseq_handle* h, const busseq_state* from, double* out);
int busseq_hmc_gene_logpost_diff(busseq_handle* h, const busseq_state* from, double* out);

/* Position of the current run: sweeps launched so far, run length and burn-in
 * length (all 0 before busseq_begin).  NULL pointers are skipped. */
int busseq_get_progress(busseq_handle* h, int32_t* n_done, int32_t* n_iter, int32_t* n_burnin);

/* Runs one stage of the sweep at sweep index `iter` (p and tau0 are redrawn in
 * stage 0 when iter >= n_unchanged). */
int busseq_run_stage(busseq_handle* h, int32_t stage, int32_t iter, int32_t n_unchanged);

int busseq_get_log_ratios(busseq_handle* h, busseq_log_ratios* out);

/* Makes the chain launch its work on `cuda_stream` (a cudaStream_t) instead of
 * its own stream.  Pass NULL to go back to the chain's own stream. */
int busseq_set_stream(busseq_handle* h, void* cuda_stream);

/* Times each kernel of `n_sweeps` sweeps with CUDA events on the chain's
 * stream (sweeps launched one kernel at a time, outside graphs).  Writes up to
 * `cap` average durations in milliseconds and returns the number of kernels
 * through *n_out; busseq_kernel_name(i) names kernel i. */
int busseq_profile(busseq_handle* h, int32_t n_sweeps, double* ms_avg, int32_t cap, int32_t* n_out);
const char* busseq_kernel_name(int32_t i);

/* Algorithmic HBM bytes of one launch of kernel i at this chain's size. */
double busseq_kernel_bytes(busseq_handle* h, int32_t i);

/* Number of kernel launches one sweep makes (burn-in and kept sweeps). */
int busseq_launches_per_sweep(busseq_handle* h, int32_t kept);

/* ---- batches of chains (not in the reference) ----------------------------- */

/* A set of chains on one device -- for instance one per K of a BIC sweep --
 * whose sweeps are launched together: one CUDA graph holds one sweep of every
 * chain as independent branches, so a launch advances all of them and their
 * kernels overlap.  Every handle must have begun a run with the same n_iter and
 * n_burnin and have made the same number of sweeps; the draws of each chain
 * are those it makes alone.  Restarting a chain (busseq_begin) invalidates the
 * batch.  Handles stay owned by the caller. */
typedef struct busseq_batch busseq_batch;
int busseq_batch_create(busseq_handle* const* handles, int32_t n, busseq_batch** out);
int busseq_batch_sweeps(busseq_batch* b, int32_t count);
int busseq_batch_synchronize(busseq_batch* b);
void* busseq_batch_stream(busseq_batch* b);  /* the cudaStream_t the batch launches on */
void busseq_batch_destroy(busseq_batch* b);

/* Autotuner of the launch shapes: by coordinate descent over the gene-pass
 * chunk length (64, 128, 192, 256 cells), the Z/X work-unit length (128, 256,
 * 384, 512 entries) and the resident Z/X CTAs per SM (2, 3, 4), each candidate
 * timed over `sweeps` burn-in sweeps (after 3 untimed ones) of a scratch
 * handle on the same counts, from the starting values in *opt (0 = default).
 * Writes the fastest shape into opt->chunk_cells, opt->zx_unit and
 * opt->zx_ctas_per_sm and its time per sweep into *ms_per_sweep (may be NULL).
 * None of the three changes a draw: a chain run with the tuned options draws
 * what it draws with the defaults (up to the order of floating-point partial
 * sums). */
int busseq_autotune(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, busseq_options* opt,
                    int32_t sweeps, double* ms_per_sweep);

/* Autotuner of the gene-pass chunk length (cells of one (batch, type) segment
 * per CTA): times `sweeps` burn-in sweeps of a scratch handle for each of the
 * n_cand candidates (1..256) and returns the fastest in *best, with the
 * per-sweep times in ms_per_sweep[n_cand] (may be NULL). */
int busseq_autotune_chunk(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, const busseq_options* opt,
                          const int32_t* candidates, int32_t n_cand, int32_t sweeps, int32_t* best,
                          double* ms_per_sweep);

/* ---- files (the reference's formats) -------------------------------------- */

/* Parses a whitespace-separated N x G integer count file (BUSseq_gpu.cu:1143-1161)
 * with all host threads.  A file that starts with "BUSSEQY1" is read as binary
 * counts instead (see busseq_write_counts_binary). */
int busseq_read_counts(const char* path, int64_t N, int64_t G, int32_t* out);

/* Writes Y [N*G] as a binary count file: the 8 bytes "BUSSEQY1", int64 N,
 * int64 G, then the N*G int32 counts row-major, little-endian (not in the
 * reference; a text count file converted once loads without parsing). */
int busseq_write_counts_binary(const char* path, int64_t N, int64_t G, const int32_t* Y);

/* Writes the _post_*, _BIC and (print_preserved) _preserved_* files with the
 * reference's names and formats (BUSseq_gpu.cu:1610-2018). */
int busseq_write_outputs(busseq_handle* h, const char* prefix, int32_t print_preserved);

/* Writes <prefix>_post_X_mean.txt and <prefix>_post_Z_prob.txt, the tables of
 * busseq_get_zx_summaries in the format of _post_X (%lf values). */
int busseq_write_zx_summaries(busseq_handle* h, const char* prefix);

/* Writes <prefix>_corrected_X.txt: the batch-corrected counts of
 * busseq_corrected_counts as an N x G table in the format of _post_X. */
int busseq_write_corrected(busseq_handle* h, const char* prefix);

/* ---- synthetic data (the BUSseq generative model) ------------------------- */

typedef struct busseq_sim_params {
  double alpha_lo, alpha_hi;      /* alpha_g ~ U(lo, hi)                       */
  double de_frac;                 /* fraction of genes with beta_gk != 0, k>=1 */
  double beta_lo, beta_hi;        /* |beta_gk| ~ U(lo, hi), random sign        */
  double nu_step, nu_sd;          /* nu_bg ~ N(nu_step*(b-1), nu_sd^2), b>=1   */
  double delta_sd;                /* delta_bi ~ N(0, sd^2), first cell 0       */
  double phi_lo, phi_hi;          /* phi_bg ~ U(lo, hi)                        */
  double pi_conc;                 /* pi_b ~ Dirichlet(conc * 1_K)              */
  double gamma0, gamma1;          /* Z ~ Bernoulli(logistic(g0 + g1 X))        */
} busseq_sim_params;

/* Draws Y [N*G] and the true W [N] (and optionally the true X) from the
 * model, deterministically from `seed`, with all host threads. */
int busseq_simulate(const busseq_dims* dims, const busseq_sim_params* prm, uint64_t seed, int32_t* Y,
                    int32_t* W_true, int32_t* X_true);

const char* busseq_last_error(void);
const char* busseq_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BUSSEQ_GB300_H */
