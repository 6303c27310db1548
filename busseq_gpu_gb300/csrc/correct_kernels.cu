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
// The arithmetic (FP64, two regimes) is in correct_math.h.  The source mean is
// formed as exp(alpha_g + beta_gw) exp(nu_bg) exp(delta_i) from per-call
// tables (a few ulps from exp of the sum).
#include "busseq_dev.h"
#include "correct_math.h"
#include "kernels.h"
#include "rng.h"

namespace bq {

namespace {

constexpr int CORR_THREADS = 256;
constexpr int CORR_CHUNK = 1024;  // genes of one row per CTA pass (4 per thread)

// Source distribution of entry (i, g): mu = mu_t * exp(nu_bg) * exp(delta_i).
__device__ __forceinline__ void corr_source(const CorrTables& tb, const Estimates& e, int64_t G, int64_t g, int b,
                                            double mu_t, double dexp, corr::NbDist& src, double& sd) {
  const double mu = mu_t * tb.nu_exp[(int64_t)b * G + g] * dexp;
  const double ph = e.phi[(int64_t)b * G + g];
  src.set(mu, ph);
  sd = corr::nb_sd(mu, ph);
}

__device__ __forceinline__ double corr_uniform(const DevState& s, int64_t i, int64_t g) {
  Stream st(s.seed, SID_CORRECT, (uint64_t)(i * s.G + g), 0u);
  const uint32_t w0 = st.next_u32();
  const uint32_t w1 = st.next_u32();
  return u64_to_unit_d(w0, w1);
}

}  // namespace

// Per-call tables: the target distribution NB(exp(alpha_g + beta_gk), phi_1g)
// of every (type, gene) with its standard deviation, and exp(nu_bg).
__global__ void k_correct_prep(DevState s, Estimates e, CorrTables tb) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)s.K * s.G; t += stride) {
    const int64_t g = t % s.G;
    const double mu_t = exp(e.alpha[g] + e.beta[t]);
    corr::NbDist d;
    d.set(mu_t, e.phi[g]);
    tb.target[t] = d;
    tb.target_sd[t] = corr::nb_sd(mu_t, e.phi[g]);
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)s.B * s.G; t += stride)
    tb.nu_exp[t] = exp(e.nu[t]);
}

// Each CTA takes CORR_CHUNK genes of one row at a time (rows strided over
// blockIdx.y).  The entries are first ordered by count with a counting sort in
// shared memory, so that the lanes of a warp run forward sums of about the
// same length (the source sum runs to x, the target's to about x again).
// Pass 1 finishes every entry that the forward sums settle (most of them) and
// queues the rest; pass 2 hands the queue to consecutive threads, so the
// continued-fraction work runs in full warps instead of stalling the warps of
// the cheap entries.  Each entry's result depends only on the entry, so the
// order of work does not change the output.  out has row stride ld.
constexpr int CORR_BINS = corr::CORR_SMALL + 2;  // counts 0 .. CORR_SMALL, and larger

__global__ void __launch_bounds__(CORR_THREADS) k_correct(DevState s, Estimates e, CorrTables tb, int32_t* out,
                                                          int64_t ld) {
  __shared__ int queue[CORR_CHUNK];
  __shared__ uint16_t order[CORR_CHUNK];
  __shared__ int bin_base[CORR_BINS];
  __shared__ int n_queue;
  const int64_t g0 = (int64_t)blockIdx.x * CORR_CHUNK;
  const int n_g = (int)(s.G - g0 < CORR_CHUNK ? s.G - g0 : CORR_CHUNK);
  constexpr int PER = CORR_CHUNK / CORR_THREADS;
  for (int64_t i = blockIdx.y; i < s.N; i += gridDim.y) {
    if (threadIdx.x == 0) n_queue = 0;
    for (int q = threadIdx.x; q < CORR_BINS; q += CORR_THREADS) bin_base[q] = 0;
    __syncthreads();
    const int b = s.batch_of[i];
    const int64_t w = e.W[i];
    const double dexp = exp(e.delta[i]);
    int key[PER];
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int j = threadIdx.x + r * CORR_THREADS;
      const int x = j < n_g ? s.X[i * s.Gp + g0 + j] : 0;
      key[r] = j < n_g ? (x > corr::CORR_SMALL ? CORR_BINS - 1 : x) : -1;
      if (key[r] >= 0) atomicAdd(&bin_base[key[r]], 1);
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive scan of the bin counts, then each bin's cursor
      int carry = 0;
      for (int q0 = 0; q0 < CORR_BINS; q0 += 32) {
        const int q = q0 + (int)threadIdx.x;
        const int v = q < CORR_BINS ? bin_base[q] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if ((int)threadIdx.x >= o) incl += t;
        }
        if (q < CORR_BINS) bin_base[q] = carry + incl - v;
        carry += __shfl_sync(0xffffffffu, incl, 31);
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PER; ++r)
      if (key[r] >= 0) order[atomicAdd(&bin_base[key[r]], 1)] = (uint16_t)(threadIdx.x + r * CORR_THREADS);
    __syncthreads();
    for (int q = threadIdx.x; q < n_g; q += CORR_THREADS) {
      const int j = order[q];
      const int64_t g = g0 + j;
      corr::NbDist dst = tb.target[w * s.G + g];
      corr::NbDist src;
      double sd;
      corr_source(tb, e, s.G, g, b, dst.mu, dexp, src, sd);
      const int r = corr::corrected_count_t<true>(src, dst, sd, tb.target_sd[w * s.G + g], s.X[i * s.Gp + g],
                                                  corr_uniform(s, i, g));
      if (r >= 0) out[i * ld + g] = r;
      else queue[atomicAdd(&n_queue, 1)] = j;
    }
    __syncthreads();
    const int nq = n_queue;
    for (int q = threadIdx.x; q < nq; q += CORR_THREADS) {
      const int64_t g = g0 + queue[q];
      corr::NbDist dst = tb.target[w * s.G + g];
      corr::NbDist src;
      double sd;
      corr_source(tb, e, s.G, g, b, dst.mu, dexp, src, sd);
      out[i * ld + g] = corr::corrected_count_t<false>(src, dst, sd, tb.target_sd[w * s.G + g], s.X[i * s.Gp + g],
                                                       corr_uniform(s, i, g));
    }
    __syncthreads();
  }
}

}  // namespace bq
