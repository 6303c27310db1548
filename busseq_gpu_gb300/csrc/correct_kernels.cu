// Batch-corrected counts by randomised quantile matching.
//
// Not part of BUSseq_gpu.cu: its outputs -- the imputed underlying counts of
// the last sweep (_post_X, BUSseq_gpu.cu:1628-1645) and the posterior means
// (:1557-1813) -- are the inputs of this step, which the BUSseq method
// (Song, Chan and Wei, Nat. Commun. 11:3274, 2020) applies downstream.
//
// The imputed count x of gene g in cell i (batch b, posterior-mode type
// w = W_i) is read as a draw of NB(mu, phi) with
//   mu = exp(alpha_g + beta_gw + nu_bg + delta_i),  phi = phi_bg.
// Its randomised probability integral transform
//   u = F(x - 1) + v (F(x) - F(x - 1)),  v ~ U(0, 1),
// is uniform on (0, 1), and the corrected count is its quantile under the
// batch-free distribution NB(mu*, phi*) with mu* = exp(alpha_g + beta_gw),
// phi* = phi_1g:
//   x* = min {k >= 0 : F*(k) >= u}.
// That removes the batch (nu_bg, phi_bg) and cell-size (delta_i) effects and
// keeps the cell type's.
//
// The arithmetic (FP64, two regimes) is in correct_math.h.
#include "busseq_dev.h"
#include "correct_math.h"
#include "kernels.h"
#include "rng.h"

namespace bq {

// One thread per (cell, gene): blockIdx.x over gene tiles, cells strided over
// blockIdx.y.  out has row stride ld.
__global__ void __launch_bounds__(256) k_correct(DevState s, Estimates e, int32_t* out, int64_t ld) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= s.G) return;
  const double alpha = e.alpha[g];
  const double phi1 = e.phi[g];
  for (int64_t i = blockIdx.y; i < s.N; i += gridDim.y) {
    const int b = s.batch_of[i];
    const int w = e.W[i];
    const int x = s.X[i * s.Gp + g];
    const double ab = alpha + e.beta[(int64_t)w * s.G + g];
    const double mu = exp((ab + e.nu[(int64_t)b * s.G + g]) + e.delta[i]);
    Stream st(s.seed, SID_CORRECT, (uint64_t)(i * s.G + g), 0u);
    const uint32_t w0 = st.next_u32();
    const uint32_t w1 = st.next_u32();
    out[i * ld + g] = corr::corrected_count(mu, e.phi[(int64_t)b * s.G + g], exp(ab), phi1, x, u64_to_unit_d(w0, w1));
  }
}

}  // namespace bq
