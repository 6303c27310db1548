// Device-side state of one BUSseq chain and the constants of the model.
//
// Layout in HBM (N cells in batch-contiguous order, G genes, Gp = G rounded up
// to GENE_TILE so every row starts on a 512-byte boundary):
//   Y, X        int32  [N][Gp]   observed counts / imputed underlying counts
//   y0m, zm     uint32 [N][Gp/32] bit masks: Y == 0, dropout indicator Z
//   beta, L     [K][Gp]          (reference layout k*G+g)
//   nu, phi     [B][Gp]          (reference layout b*G+g)
//   E           [B][K][Gp]       exp(alpha_g + beta_kg + nu_bg), kept current
//   W, delta, Dexp = exp(delta)  [N]
//   perm        [N]              cells sorted by (batch, cell type), rebuilt
//                                after every W update
//   gchunk      int4 [cap_g]     gene-pass work list: {b, k, first, count} runs
//                                of <= CG cells of one (batch, type) segment
//   ctile       int4 [cap_c]     cell-pass work list: runs of <= CELL_TILE cells
//   part        f64 [cap_g][4][Gp] per-chunk partial sums of the gene passes
//   zij, zval   int2 / uint8 [nz0]   the entries with Y == 0 ({cell, gene},
//                                row-major order; Y never changes) and their Z
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace bq {

// ---- hyper-parameters of the model (BUSseq_gpu.cu:12-32) ------------------
constexpr float P_INIT_BOUND = 0.5f;
constexpr float TAU0_INIT = 0.005f;
constexpr float GAMMA0_INIT = 0.0f;
constexpr float GAMMA1_INIT = -0.3f;
constexpr float PHI_INIT = 5.0f;
constexpr double XI_PI = 2.0;
constexpr double SIGMA2_ALPHA = 5.0;
constexpr double SIGMA2_NU = 5.0;
constexpr double SIGMA2_DELTA = 5.0;
constexpr double SIGMA2_GAMMA0 = 3.0;
constexpr double KAPPA_GAMMA1 = 0.001;
constexpr double TAU_GAMMA1 = 0.01;
constexpr double KAPPA_PHI = 1.0;
constexpr double TAU_PHI = 0.1;
constexpr double A_P = 1.0;
constexpr double B_P = 3.0;
constexpr double A_TAU0 = 2.0;
constexpr double B_TAU0 = 0.01;
constexpr double TAU1 = 100.0;
constexpr float RW_STEP = 0.1f;  // random-walk proposal s.d. of alpha, beta, nu, delta, gamma0

// ---- launch geometry -------------------------------------------------------
constexpr int GENE_TILE = 128;     // genes per gene-pass CTA (one per thread)
constexpr int MAX_CG = 256;        // largest gene-pass chunk (cells staged in shared memory)
constexpr int CELL_TILE = 8;       // cells per cell-pass CTA
constexpr int CELL_THREADS = 256;  // threads of a cell-pass CTA (4 genes each per step)
// Cell passes stream the tile's X rows through shared memory in X_STAGES
// stages of DELTA_WIDTH (delta) or W_WIDTH (W) genes.
constexpr int X_STAGES = 3;
constexpr int DELTA_WIDTH = 2 * CELL_THREADS;
constexpr int W_WIDTH = 2 * CELL_THREADS;
constexpr int DELTA_SMEM = X_STAGES * CELL_TILE * DELTA_WIDTH * (int)sizeof(int);
constexpr int W_SMEM = X_STAGES * CELL_TILE * W_WIDTH * (int)sizeof(int);
constexpr int MAX_B = 128;
constexpr int MAX_K = 64;
constexpr int NSLOT = 4;           // partial-sum slots per (chunk, gene)
constexpr int GSLOT = 8;           // slots of a Z/X partial of the gamma statistics (6 used)
constexpr int PHI_HIST_SLICES = 8;  // slices of a batch's cells in the initial count tables of phi
constexpr int PHI_TAB = 64;        // counts below this read lgamma differences from a table
constexpr int ZX_THREADS = 256;    // threads of a Z/X CTA
constexpr int ZX_UNIT = 512;       // most zero entries per Z/X work unit (one warp, one partial)
constexpr int ZX_HIST = 128;       // counts below this read the gamma terms from a per-batch table
constexpr int ZX_CTAS_PER_SM = 4;  // resident Z/X CTAs per SM (the kernel's launch bound)
constexpr int ZGP_UNITS = 4;       // Z/X work units per chunk of the Gamma-Poisson pass
constexpr int ZGP_CTAS_PER_SM = 3;  // resident k_zx_gp CTAs per SM (its launch bound)
constexpr int DECIDE_GAMMA_THREADS = 256;  // threads of a gamma-decision CTA (one per batch)
constexpr int DEC_THREADS = 256;   // per-gene decision CTAs: 32 genes x 8 warps splitting their segments

// ---- stages (groups of the reference's sweep order, BUSseq_gpu.cu:1267-1398)
enum Stage : int {
  STAGE_ZX_GAMMA_ALPHA_L = 0,  // Z/X, gamma0, gamma1, alpha, L (and p, tau0 at the tail)
  STAGE_PTAU_BETA_NU = 1,      // (p, tau0 already drawn) beta, nu
  STAGE_DELTA = 2,
  STAGE_PHI = 3,
  STAGE_W = 4,
  STAGE_PI = 5,                // pi, then the new cell order
  N_STAGES = 6
};

// Proposal families (bit mask for the proposal kernel).
enum PropMask : int {
  PROP_GAMMA = 1, PROP_ALPHA = 2, PROP_BETA = 4, PROP_NU = 8, PROP_DELTA = 16, PROP_PHI = 32,
  PROP_ALL = 63
};

// Unevaluated sum hi + lo of two floats (a "float-float" value, ~48 bits).
struct FF {
  float hi, lo;
};

// Device scalars of the HMC block update (double [HS_COUNT]).
enum HmcScalar : int {
  HS_EPS = 0,         // step size (adapted during burn-in)
  HS_HBAR = 1,        // dual-averaging statistic
  HS_MU = 2,          // dual-averaging shrinkage point, log(10 eps0)
  HS_M = 3,           // dual-averaging iteration count
  HS_LOG_EPS_BAR = 4, // averaged log step size
  HS_EPS_USED = 5,    // jittered step size of the current transition
  HS_LAST_DH = 6,     // H(end) - H(start) of the last transition
  HS_LAST_ACC = 7,    // min(1, exp(-dH)) of the last transition
  HS_ACCEPTED = 8,    // 1 if the last transition was accepted
  HS_N_KEPT = 9,      // transitions in kept sweeps
  HS_ACC_KEPT = 10,   // accepted transitions in kept sweeps
  HS_COUNT = 16
};
constexpr double HMC_TARGET_ACCEPT = 0.7;
constexpr int HMC_BLOCK_MAX = 24;  // largest K + B - 1 with a per-gene block metric
constexpr double HMC_EPS0 = 0.05;

struct DevState {
  // dimensions and run configuration
  int B, K;
  int64_t G, N, Gp, Gw;
  int n_tiles;      // ceil(G / GENE_TILE)
  int cap_g, CG;    // gene-pass chunk capacity and chunk length
  int cap_c;        // cell-pass tile capacity
  int n_static;     // CTAs evaluating the static (Y > 0) gamma terms
  int ymax;         // largest observed count
  int w_update;     // 0: MH with uniform proposal (reference), 1: K-way Gibbs
  int nb_inv_cap;   // search cap of the NB inversion in k_zx (NB_INV_MAX_K unless a test lowers it)
  int n_burnin, n_unchanged, keep_draws, n_kept;
  uint64_t seed;

  // data
  const int32_t* Y;
  int32_t* X;
  const uint32_t* y0m;
  uint32_t* zm;
  const int32_t* batch_of;   // [N]
  const int32_t* batch_off;  // [B+1]
  const int32_t* yhist;      // [B][ymax+1] counts of Y values (Y > 0 entries only)

  // parameters (float) and indicators
  int32_t* W;
  int8_t* L;
  float* alpha;
  float* mu_alpha;
  float* beta;
  float* nu;
  float* mu_nu;    // [B]
  float* delta;
  float* mu_delta;
  float* Dexp;
  float* phi;
  float* gamma;    // [2][B]
  float* pi;       // [B][K]
  float* p_tau0;   // [2]
  float* E;        // [B][K][Gp]

  // proposals of the current sweep
  float* alpha_p;
  float* beta_p;   // [K][Gp]
  float* nu_p;     // [B][Gp]
  float* delta_p;  // [N]
  float* phi_p;    // [B][Gp]

  // gradient-based block update (hmc_L > 0 selects it); flat layout
  // alpha [Gp] | beta [K][Gp] | nu [B][Gp] | psi [B][Gp] | delta [N]
  int hmc_L;
  int hmc_gene;     // 1: per-gene decisions, delta fixed in the transition
  int64_t hmc_D;
  float* psi;       // [B][Gp] log phi: the position of the phi block
  float* hmc_mom;   // [D] momentum
  float* hmc_mom0;  // [D] momentum at the start of the transition
  float* hmc_grad;  // [D] gradient of the log posterior
  float* hmc_mass;  // [D] diagonal metric
  float* hmc_th0;   // [D] coordinates at the start of the transition
  float* hmc_part;  // [cap_g][NSLOT][Gp] per-chunk gradient (and information) sums
  float* hmc_cpart; // [n_tiles][N] per-tile sums of d ll / d delta
  float* hmc_cpartw;// [n_tiles][N] per-tile observed information of delta
  FF* hmc_hpart;    // [n_tiles * cap_g] per-CTA log-likelihood change
  FF* hmc_epart;    // [ceil(D / 256)] per-CTA kinetic minus prior change
  double* hmc_sc;   // [HS_COUNT]
  // per-gene block metric over (alpha_g, beta_g1..g(K-1), nu_g1..g(B-1)):
  // hmc_nb = K + B - 1 coordinates, Cholesky factor packed [nb (nb + 1) / 2][G]
  // (0: diagonal metric everywhere)
  int hmc_nb;
  float* hmc_chol;
  float* hmc_minv;  // [nb * nb][G] inverse of each gene's block metric (velocity and kinetic energy)
  // frozen data of the metric: the information part of every diagonal mass
  // (without the priors, which follow the current L and tau0) and the
  // per-segment information sums W_bkg of the blocks [B*K][G]
  float* hmc_fis;
  float* hmc_wbk;
  FF* hmc_epart_b;  // [ceil(G / 256)] per-CTA kinetic minus prior change of the gene blocks
  // per-gene decisions (hmc_gene): kinetic minus prior change per diagonal
  // coordinate [D] and per gene block [Gp], and each gene's outcome [Gp]
  float* hmc_e;
  float* hmc_eb;
  uint8_t* hmc_gacc;
  float* phi_tab;  // [B][PHI_TAB][Gp]: sum_{j<x} log((phi_p + j) / (phi + j)) for the current proposal
  float* phi_lgd0; // [B][Gp]: lgamma(phi_p) - lgamma(phi)
  // The lgamma part of the phi ratio depends on an entry only through x, and
  // the entries with Y > 0 keep x = Y: their part comes from these static
  // tables once per (batch, gene) instead of once per entry (k_propose for
  // Y < PHI_TAB, k_phi_static for the rest).
  int32_t* phi_cnt;      // [B][PHI_TAB][Gp] number of cells with Y = y, 0 < y < PHI_TAB
  int64_t* phi_big_off;  // [B*G + 1] start of each (batch, gene) run in phi_big_y
  int32_t* phi_big_y;    // the Y values >= PHI_TAB of each (batch, gene), in cell order
  double* phi_static;    // [B][Gp] the static part of the current proposal's phi sum
  float* gamma_p;  // [2][B]

  // cell order and work lists
  int32_t* perm;
  int4* gchunk;
  int4* ctile;
  int32_t* seg_cnt;  // [B][K]
  int2* seg_chunk;   // [B][K] {first chunk, number of chunks} of each (batch, type) segment

  // the entries with Y == 0 and their Z/X work units
  const int2* zij;          // [nz0] {cell, gene}
  uint8_t* zval;            // [nz0] Z
  int64_t nz0;
  const int2* zcta;         // [n_zcta] Z/X work units {first entry, count}, each inside one batch
  const int32_t* zcta_batch;
  const int32_t* zfirst;    // [B+1] first unit of each batch
  int n_zcta;
  uint8_t* beta_acc;        // [K][Gp] accepted beta of the current sweep

  // scratch (partial sums and completion counters)
  double* part;    // [cap_g][NSLOT][Gp]
  double* gpart;   // [n_zcta][GSLOT] each Z/X unit's gamma statistics (k_zx)
  double* gstat;   // [n_static][4]
  float4* zx_gtab;    // [B][ZX_HIST] per count x < ZX_HIST: softplus(-g0 - g1 x) and the three gamma
                      // terms of the sweep's proposals (built by k_propose)
  unsigned* zx_ctr;   // [4] work counter and finished-warp counter of k_zx, then of k_zx_gp
                      // (zero between launches)
  int zx_ctas;        // Z/X CTAs per launch (resident on every SM)
  // The NB proposals drawn as Gamma-Poisson mixtures, left by k_zx to k_zx_gp:
  int4* zgp_rec;            // [nz0] each unit's, in unit order from the unit's first list entry on:
                            // {list entry, cell, gene, X}
  float2* zgp_mp;           // [nz0] and their {mu, phi}
  int32_t* zgp_cnt;         // [n_zcta] how many each unit has
  const int4* zgchunk;      // [n_gchunk] {first unit, units, batch, 0}: ZGP_UNITS units of one batch
  const int32_t* gfirst;    // [B+1] first chunk of each batch
  double* gpart_gp;         // [n_gchunk][GSLOT] each chunk's gamma statistics: its units' partials
                            // plus its Gamma-Poisson draws (what k_decide_gamma reads)
  int n_gchunk;
  int zgp_ctas;             // k_zx_gp CTAs per launch
  double* tpart;   // per-CTA sums: [n_tiles][MAX_B] at initialisation, [ceil(G / 32)][2] in k_decide_alpha
  unsigned* cnt_tile;  // [n_tiles]
  unsigned* cnt_glob;  // [4]

  int* iter;       // sweep index, advanced on the device at the end of a sweep
  int* err;        // sampler / numerical error bits

  // log acceptance ratios of the last sweep (likelihood + prior), double
  double* lr_gamma;  // [2][B]
  double* lr_alpha;  // [G]
  double* lr_beta;   // [K][G]
  double* lr_nu;     // [B][G]
  double* lr_delta;  // [N]
  double* lr_phi;    // [B][G]
  double* lr_W;      // [N]

  // posterior accumulators (kept sweeps)
  double* acc_alpha;
  double* acc_beta;   // [K][G]
  double* acc_L;      // [K][G]
  double* acc_nu;     // [B][G]
  double* acc_delta;  // [N]
  double* acc_phi;    // [B][G]
  double* acc_gamma;  // [2B]
  double* acc_pi;     // [B*K]
  double* acc_ptau;   // [2]
  int32_t* acc_wcnt;  // [N][K]
  int32_t* acc_zn;    // [nz0] kept sweeps with Z = 1 at each Y == 0 entry (zx_summaries, else null)
  int64_t* acc_xs;    // [nz0] sum of X there over the kept sweeps

  // preserved draws, [kept sweep][scalar] (only when keep_draws)
  float* keep_gamma;
  float* keep_alpha;
  float* keep_beta;   // (K-1)*G per sweep
  int8_t* keep_L;     // (K-1)*G per sweep
  float* keep_ptau;
  float* keep_nu;     // (B-1)*G per sweep
  float* keep_delta;
  float* keep_phi;    // B*G per sweep
  int16_t* keep_W;
  float* keep_pi;
};

// Posterior estimates on the device (double precision).
struct Estimates {
  double *gamma, *alpha, *L, *beta, *ptau, *nu, *delta, *phi, *pi;
  int32_t* W;
};

// Tables of the BIC (all null: every entry computes its own values).
struct alignas(16) BicGene {  // per (batch, gene)
  double ean, phi, lphi, lgphi;  // exp(alpha + nu), phi, log phi, lgamma phi
};
struct BicTabs {
  double* eb;   // [K][G] exp(beta)
  BicGene* bg;  // [B][G]
  double* ty;   // [B][ny] -softplus(g0 + g1 y) - lgamma(1 + y)
  int ny;
};

// eta = alpha + beta + nu, always summed in this order so that every kernel
// rounds it identically.
__device__ __forceinline__ float eta3(float a, float b, float n) { return (a + b) + n; }

// exp(a + b + c) with the sum carried as a float pair (TwoSum), so the result
// has the error of one expf and one product instead of that of a rounded eta
// (about 1e-6 relative for eta near 8, systematic across the cells of a gene).
__device__ __forceinline__ float exp_sum3(float a, float b, float c) {
  const float s1 = a + b;
  const float bb = s1 - a;
  const float e1 = (a - (s1 - bb)) + (b - bb);
  const float s2 = s1 + c;
  const float cc = s2 - s1;
  const float e2 = (s1 - (s2 - cc)) + (c - cc);
  const float lo = e1 + e2;
  const float hi = expf(s2);
  return fmaf(hi, lo, hi);
}

}  // namespace bq
