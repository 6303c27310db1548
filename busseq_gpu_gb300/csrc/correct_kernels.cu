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

namespace {

constexpr int CORR_THREADS = 256;
constexpr int CORR_CHUNK = 1024;  // genes of one row per CTA pass (4 per thread)

struct CorrEntry {
  double mu, phi, mu_t, phi_t, v;
  int x;
};

__device__ __forceinline__ CorrEntry corr_entry(const DevState& s, const Estimates& e, int64_t i, int64_t g, int b,
                                                int w) {
  CorrEntry c;
  c.x = s.X[i * s.Gp + g];
  const double ab = e.alpha[g] + e.beta[(int64_t)w * s.G + g];
  c.mu = exp((ab + e.nu[(int64_t)b * s.G + g]) + e.delta[i]);
  c.mu_t = exp(ab);
  c.phi = e.phi[(int64_t)b * s.G + g];
  c.phi_t = e.phi[g];
  Stream st(s.seed, SID_CORRECT, (uint64_t)(i * s.G + g), 0u);
  const uint32_t w0 = st.next_u32();
  const uint32_t w1 = st.next_u32();
  c.v = u64_to_unit_d(w0, w1);
  return c;
}

}  // namespace

// Each CTA takes CORR_CHUNK genes of one row at a time (rows strided over
// blockIdx.y).  Pass 1 finishes every entry that the forward sums settle
// (most of them) and queues the rest in shared memory; pass 2 hands the queue
// to consecutive threads, so the continued-fraction work runs in full warps
// instead of stalling the warps of the cheap entries.  out has row stride ld.
__global__ void __launch_bounds__(CORR_THREADS) k_correct(DevState s, Estimates e, int32_t* out, int64_t ld) {
  __shared__ int queue[CORR_CHUNK];
  __shared__ int n_queue;
  const int64_t g0 = (int64_t)blockIdx.x * CORR_CHUNK;
  const int n_g = (int)(s.G - g0 < CORR_CHUNK ? s.G - g0 : CORR_CHUNK);
  for (int64_t i = blockIdx.y; i < s.N; i += gridDim.y) {
    if (threadIdx.x == 0) n_queue = 0;
    __syncthreads();
    const int b = s.batch_of[i];
    const int w = e.W[i];
    for (int j = threadIdx.x; j < n_g; j += CORR_THREADS) {
      const int64_t g = g0 + j;
      const CorrEntry c = corr_entry(s, e, i, g, b, w);
      const int r = corr::corrected_count_t<true>(c.mu, c.phi, c.mu_t, c.phi_t, c.x, c.v);
      if (r >= 0) out[i * ld + g] = r;
      else queue[atomicAdd(&n_queue, 1)] = j;
    }
    __syncthreads();
    const int nq = n_queue;
    for (int q = threadIdx.x; q < nq; q += CORR_THREADS) {
      const int64_t g = g0 + queue[q];
      const CorrEntry c = corr_entry(s, e, i, g, b, w);
      out[i * ld + g] = corr::corrected_count(c.mu, c.phi, c.mu_t, c.phi_t, c.x, c.v);
    }
    __syncthreads();
  }
}

}  // namespace bq
