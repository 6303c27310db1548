// Kernel entry points (defined in gene_kernels.cu, cell_kernels.cu and
// init_kernels.cu).
#pragma once
#include "busseq_dev.h"

namespace bq {

namespace corr {
struct NbDist;
}

// Per-call tables of the batch-corrected counts (k_correct_prep).
struct CorrTables {
  corr::NbDist* target;  // [K][G] NB(exp(alpha_g + beta_gk), phi_1g)
  double* target_sd;     // [K][G]
  double* nu_exp;        // [B][G] exp(nu_bg)
};


__global__ void k_propose(DevState s, int mask, int64_t t0);
__global__ void k_zx(DevState s, int kept);
__global__ void k_zx_gp(DevState s, int kept);
__global__ void k_decide_gamma(DevState s);
__global__ void k_zx_summary(DevState s, int n_kept, float* x_mean, float* z_prob);
__global__ void k_zx_summary_zeros(DevState s, int n_kept, float* x_mean, float* z_prob);
__global__ void k_alpha(DevState s);
__global__ void k_decide_alpha(DevState s);
__global__ void k_beta_nu(DevState s);
__global__ void k_decide_beta(DevState s);
__global__ void k_decide_nu_E(DevState s);
__global__ void k_phi(DevState s);
__global__ void k_phi_static(DevState s);
__global__ void k_phi_hist(DevState s, int64_t* n_big, const int64_t* off, int fill);
__global__ void k_decide_phi(DevState s);
__global__ void k_delta(DevState s);
__global__ void k_w_mh(DevState s);
__global__ void k_w_gibbs(DevState s);
__global__ void k_sort_pi(DevState s, int do_pi, int advance);
__global__ void k_posterior(DevState s, int advance);
int64_t propose_count(const DevState& s);
int64_t propose_phi_offset(const DevState& s);  // the first phi proposal of k_propose

__global__ void k_init_scan(DevState s, int64_t* libsize, int* ymax, int32_t* rowcnt);
__global__ void k_init_hist(DevState s, int32_t* hist);
__global__ void k_zlist_fill(DevState s, const int64_t* rowoff, int2* zij);
__global__ void k_zval_from_mask(DevState s);
__global__ void k_zmask_from_zval(DevState s);
__global__ void k_zlist_gather_x(DevState s, int32_t* out);
__global__ void k_hmc_grad(DevState s);
__global__ void k_hmc_grad_metric(DevState s, int metric_mode);
__global__ void k_hmc_assemble(DevState s, int metric_mode);
__global__ void k_hmc_start(DevState s);
__global__ void k_hmc_leap(DevState s, int first);
__global__ void k_hmc_refresh_E(DevState s);
__global__ void k_hmc_dll(DevState s, int per_gene);
__global__ void k_hmc_dll_prep(DevState s);
__global__ void k_hmc_dll_static(DevState s, int base, int per_gene);
__global__ void k_hmc_energy(DevState s, int kick, int per_gene);
__global__ void k_hmc_accept(DevState s, int n_hpart, int n_epart, int n_epart_b, int mode);
__global__ void k_hmc_accept_genes(DevState s, double* dlp);
__global__ void k_hmc_metric_blocks(DevState s, int metric_mode);
__global__ void k_hmc_mass(DevState s);
__global__ void k_hmc_start_blocks(DevState s);
__global__ void k_hmc_leap_blocks(DevState s, int first);
__global__ void k_hmc_energy_blocks(DevState s, int kick, int per_gene);
__global__ void k_hmc_finish(DevState s);
__global__ void k_hmc_set_th0(DevState s, const float* src);
__global__ void k_hmc_unit_mass(DevState s);
__global__ void k_zlist_scatter_x(DevState s, const int32_t* in);
__global__ void k_y_fingerprint(DevState s, unsigned long long* out);
__global__ void k_init_w_delta(DevState s, const int64_t* libsize, int* bad_cell);
__global__ void k_init_raw(DevState s);
__global__ void k_init_finish(DevState s, int fresh);
__global__ void k_finalize(DevState s, Estimates e, int n_kept);
// A table to format as text (format_kernels.cu): entry (r, c) at p[r sr + c sc].
enum FmtKind : int { FMT_I32 = 0, FMT_F32 = 1, FMT_I8 = 2, FMT_I16 = 3 };
struct FmtSrc {
  const void* p;
  int kind;  // FmtKind
  int64_t sr, sc;
};
__global__ void k_fmt_row_len(FmtSrc src, int64_t cols, int64_t* row_len, int* bad);
__global__ void k_fmt_rows(FmtSrc src, int64_t cols, const int64_t* row_off, char* out);
__global__ void k_z_dense_i32(DevState s, int32_t* out, int64_t ld);
__global__ void k_z_dense_u8(DevState s, uint8_t* out, int64_t ld);
__global__ void k_bic_cell(DevState s, Estimates e, double* ll_ik, BicTabs tb);
__global__ void k_bic_tables(DevState s, Estimates e, BicTabs tb);
// k_bic_tables (when tb has tables), k_bic_cell and k_bic_total on st; out
// receives {BIC, log-likelihood}
void launch_bic(const DevState& s, const Estimates& e, double* ll_ik, const BicTabs& tb, double* out,
                cudaStream_t st);
// bytes of the BIC tables: BicGene [B][G] first, then exp(beta) [K][G] and the
// count terms [B][ny] as doubles
int64_t bic_table_bytes(const DevState& s, int ny);
int bic_table_counts(const DevState& s);  // ny: the counts 0 .. ny-1 that the count table covers
__global__ void k_correct_prep(DevState s, Estimates e, CorrTables tb);
__global__ void k_correct(DevState s, Estimates e, CorrTables tb, int32_t* out, int64_t ld);
__global__ void k_bic_total(DevState s, Estimates e, const double* ll_ik, double* out);

}  // namespace bq
