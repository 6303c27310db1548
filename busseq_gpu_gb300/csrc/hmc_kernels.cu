// Gradient-based block update (Hamiltonian Monte Carlo) of
//   theta = (alpha_g, beta_gk (k >= 1), nu_bg (b >= 1), delta_i (not the first
//            cell of a batch), psi_bg = log phi_bg)
// given X, W, L, p and tau0.  This replaces the reference's five random-walk
// Metropolis steps (BUSseq_gpu.cu:602-632, :670-818) with one transition that
// leaves the same conditional density invariant:
//   log p = sum_{i,g} [lgamma(x + phi) - lgamma(phi) + phi log phi
//                      - (phi + x) log(phi + mu) + x eta]
//         - (alpha - mu_alpha)^2 / (2 sigma2_alpha) - beta^2 / (2 v(L))
//         - (nu - mu_nu)^2 / (2 sigma2_nu) - (delta - mu_delta)^2 / (2 sigma2_delta)
//         + kappa psi - tau_phi e^psi,
// the priors of the reference's MH steps, with v(L) = tau1 or tau0.
//
// Coordinates live in the parameter arrays themselves; momentum, gradient,
// metric and the start of the trajectory use one flat layout of length
//   D = Gp (1 + K + 2B) + N:  alpha [Gp] | beta [K][Gp] | nu [B][Gp] | psi [B][Gp] | delta [N]
// (padding genes, beta_0, nu_0 and the first cell of each batch are fixed).
//
// One transition: gradient at theta0 (with the metric during its adaptation),
// momentum p ~ N(0, M), L leapfrog steps (kick, drift, gradient; the gradient
// pass forms exp(alpha + beta + nu) itself), a final half kick, the change of
// the Hamiltonian (likelihood part from a cancellation-free per-entry pass,
// prior and kinetic parts per coordinate), the Metropolis decision and, if
// rejected, a restore; the E table is refreshed once, after the transition.
// Step size: dual averaging (Hoffman and Gelman, JMLR 15, 2014, algorithm 5)
// during burn-in with a random jitter of +-10 %; metric: a block per gene over
// (alpha, beta, nu) from the sums of the observed information, the diagonal
// observed information of delta and of psi, adapted at the transition starts
// of the first half of burn-in, then frozen.  The observed information
// phi mu (phi + x) / (phi + mu)^2 of an entry's eta is positive and is the
// actual curvature where the chain is; the expected (Fisher) information
// phi mu / (phi + mu) equals it only on average over x ~ NB(mu, phi) and
// understates it wherever the counts run above the current means (a chain
// still far from equilibrium), which shrinks the adapted step size.
#include "kernels_common.cuh"

namespace bq {

// ---------------------------------------------------------------------------
// Layout helpers
// ---------------------------------------------------------------------------
enum HmcKind : int { HK_ALPHA = 0, HK_BETA = 1, HK_NU = 2, HK_PSI = 3, HK_DELTA = 4 };

struct HmcCoord {
  int kind;     // HmcKind
  int seg;      // k for beta, b for nu / psi, batch for delta
  int64_t idx;  // gene g, or cell i
  bool free;    // updated by the transition
  float* pos;   // the parameter it lives in
};

__device__ __forceinline__ HmcCoord hmc_coord(const DevState& s, int64_t d) {
  const int64_t Gp = s.Gp;
  HmcCoord c{};
  const int64_t nb = Gp, nk = Gp * s.K, nn = Gp * s.B;
  if (d < nb) {
    c.kind = HK_ALPHA;
    c.idx = d;
    c.free = d < s.G;
    c.pos = s.alpha + d;
    return c;
  }
  d -= nb;
  if (d < nk) {
    c.kind = HK_BETA;
    c.seg = (int)(d / Gp);
    c.idx = d % Gp;
    c.free = c.seg > 0 && c.idx < s.G;
    c.pos = s.beta + d;
    return c;
  }
  d -= nk;
  if (d < nn) {
    c.kind = HK_NU;
    c.seg = (int)(d / Gp);
    c.idx = d % Gp;
    c.free = c.seg > 0 && c.idx < s.G;
    c.pos = s.nu + d;
    return c;
  }
  d -= nn;
  if (d < nn) {
    c.kind = HK_PSI;
    c.seg = (int)(d / Gp);
    c.idx = d % Gp;
    c.free = c.idx < s.G;
    c.pos = s.psi + d;
    return c;
  }
  d -= nn;
  c.kind = HK_DELTA;
  c.idx = d;
  c.seg = s.batch_of[d];
  c.free = d != s.batch_off[c.seg] && !s.hmc_gene;  // per-gene decisions: delta is held
  c.pos = s.delta + d;
  return c;
}

// Coordinates of the per-gene blocks (alpha, beta, nu) are moved by the block
// kernels when the block metric is on.
__device__ __forceinline__ bool hmc_in_block(const DevState& s, const HmcCoord& c) {
  return s.hmc_nb > 0 && c.kind <= HK_NU;
}

// Leapfrog step of gene g's coordinates.  With per-gene decisions every gene
// scales the transition's step by its own factor in [0.5, 1.5), drawn per
// transition: the genes' trajectories then differ in length, and none stays at
// a period of its (nearly Gaussian) conditional, where a fixed length would
// return it to its start or reflect it (the factor does not depend on the
// state, so each gene's transition stays reversible).
__device__ __forceinline__ float hmc_eps_gene(const DevState& s, int64_t g) {
  const float eps = (float)s.hmc_sc[HS_EPS_USED];
  if (!s.hmc_gene) return eps;
  return eps * (0.5f + uniform_at(s.seed, SID_HMC_ACC, 1 + (uint64_t)g, (uint32_t)*s.iter, 1));
}

__device__ __forceinline__ bool hmc_adapt_metric(const DevState& s, int iter) {
  return iter == 0 || iter < s.n_burnin / 2;
}

// metric_mode 0: never (the gradients inside a trajectory: the metric must not
// change along it), 1: while it adapts (the gradient at the start of a
// transition), 2: always (the test entry point).
__device__ __forceinline__ bool hmc_metric_now(const DevState& s, int metric_mode) {
  return metric_mode == 2 || (metric_mode == 1 && hmc_adapt_metric(s, *s.iter));
}

// psi(z0 + x) - psi(z0 + 32)... differences of the digamma / trigamma
// functions for arguments >= 32 from their asymptotic series
//   psi(z)  = log z - 1/(2z) - 1/(12 z^2) + 1/(120 z^4) - 1/(252 z^6)
//   psi'(z) = 1/z + 1/(2 z^2) + 1/(6 z^3) - 1/(30 z^5) + 1/(42 z^7)
// (the first omitted terms are below 1e-12 at z = 32).
__device__ __forceinline__ float digamma_tail(float z) {
  const float r = fast_rcp(z), r2 = r * r;
  return -0.5f * r - r2 * (1.0f / 12.0f - r2 * (1.0f / 120.0f - r2 * (1.0f / 252.0f)));
}
__device__ __forceinline__ float trigamma_asym(float z) {
  const float r = fast_rcp(z), r2 = r * r;
  return r * (1.0f + r * (0.5f + r * (1.0f / 6.0f - r2 * (1.0f / 30.0f - r2 * (1.0f / 42.0f)))));
}

constexpr int HMC_TAB = 32;  // digamma / trigamma differences tabulated for counts below this

// log x from the hardware base-2 logarithm (lg2.approx.f32, absolute error
// about 2^-22).  Used only for gradients: their errors cost acceptance rate,
// never correctness, since the decision uses the accurate change of the log
// likelihood from k_hmc_dll.
__device__ __forceinline__ float log_hw(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r * 0.6931471805599453f;
}

// Sums 8 per-lane values (v[u], one per chunk cell j0+u) over the warp: after
// the exchange, lanes with lane % 4 == 0 hold the warp total of value
// ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1).
__device__ __forceinline__ float transpose_sum8(float (&v)[8], int lane) {
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
  float a[4], b2[2];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float send = h16 ? v[q] : v[q + 4];
    const float recv = __shfl_xor_sync(0xffffffffu, send, 16);
    a[q] = (h16 ? v[q + 4] : v[q]) + recv;
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float send = h8 ? a[q] : a[q + 2];
    const float recv = __shfl_xor_sync(0xffffffffu, send, 8);
    b2[q] = (h8 ? a[q + 2] : a[q]) + recv;
  }
  float c = h4 ? b2[1] : b2[0];
  c += __shfl_xor_sync(0xffffffffu, h4 ? b2[0] : b2[1], 4);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  return c;
}

__device__ __forceinline__ int transpose_slot(int lane) {
  return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// ---------------------------------------------------------------------------
// Gradient pass (gene-pass layout: CTA = 128 genes x one chunk of cells of one
// (batch, type)).  Per-gene partial sums go to part slots 0 (sum d ll / d eta),
// 1 (sum d ll / d psi), and, while the metric adapts, 2 (observed information
// of eta) and 3 (observed information of psi); per-cell sums over the CTA's
// genes go to hmc_cpart[tile][cell] (and hmc_cpartw for the information).
// ---------------------------------------------------------------------------
// Sum of HMC partial slot `slot` of gene g over the chunks of segment (b, k),
// in float (gradients need no more).
__device__ __forceinline__ float hmc_seg_sum(const DevState& s, int b, int k, int slot, int64_t g) {
  const int2 r = s.seg_chunk[b * s.K + k];
  float acc = 0.0f;
  for (int c = r.x; c < r.x + r.y; ++c) acc += __ldg(&s.hmc_part[((int64_t)c * NSLOT + slot) * s.Gp + g]);
  return acc;
}

// METRIC: the variant run at the start of a transition, which (while the
// metric adapts, or always for metric_mode 2) also sums the information terms;
// the leapfrog passes run the lean variant (less shared memory, more CTAs).
template <bool METRIC>
__device__ __forceinline__ void hmc_grad_body(const DevState& s, int metric_mode) {
  __shared__ float tdg[HMC_TAB][GENE_TILE];
  __shared__ float ttg[METRIC ? HMC_TAB : 1][GENE_TILE];
  __shared__ __align__(16) int s_i[MAX_CG];
  __shared__ __align__(16) float s_D[MAX_CG];
  __shared__ float s_cell[GENE_TILE / 32][MAX_CG];
  __shared__ float s_cellw[METRIC ? GENE_TILE / 32 : 1][METRIC ? MAX_CG : 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  if (len == 0) return;
  const bool adapt = METRIC && hmc_metric_now(s, metric_mode);
  // per-cell (delta) sums of the gradient: not with per-gene decisions (delta is
  // held); of the information: while the metric adapts (with per-gene
  // decisions it scales delta's random-walk step)
  const bool cells = !s.hmc_gene;
  const bool cellw = METRIC && adapt;
  const int len8 = (len + 7) & ~7;
  for (int j = tid; j < len8; j += GENE_TILE) {
    const bool in = j < len;
    const int i = in ? s.perm[start + j] : (int)s.N;
    s_i[j] = i;
    s_D[j] = in ? s.Dexp[i] : 0.0f;
  }
  const bool gv = g < s.G;
  const float ph = gv ? s.phi[(int64_t)b * Gp + g] : 1.0f;
  // exp(alpha + beta + nu) at the current position, as k_hmc_refresh_E forms it
  const float M = gv ? exp_sum3(s.alpha[g], s.beta[(int64_t)k * Gp + g], s.nu[(int64_t)b * Gp + g]) : 0.0f;
  const float iph = fast_rcp(ph);
  // sum_{j<x} 1/(ph + j) (and 1/(ph + j)^2) for x < HMC_TAB
  {
    float dg = 0.0f, tg = 0.0f;
    for (int x = 0; x < HMC_TAB; ++x) {
      tdg[x][tid] = dg;
      if (METRIC) ttg[x][tid] = tg;
      const float r = fast_rcp(ph + (float)x);
      dg += r;
      tg = fmaf(r, r, tg);
    }
  }
  const float z32 = ph + (float)HMC_TAB;
  const float dg32 = tdg[HMC_TAB - 1][tid] + fast_rcp(z32 - 1.0f);
  const float iz32h = fast_rcp(z32 - 0.5f);
  float tg32 = 0.0f, tasym32 = 0.0f;
  if (METRIC) {
    tg32 = ttg[HMC_TAB - 1][tid] + fast_rcp((z32 - 1.0f) * (z32 - 1.0f));
    tasym32 = trigamma_asym(z32);
  }
  __syncthreads();
  const char* Xg = reinterpret_cast<const char*>(s.X + g);
  const uint32_t row_bytes = (uint32_t)(Gp * sizeof(int));
  KahanF ar, ap, aw, ai;
  for (int j0 = 0; j0 < len8; j0 += 8) {
    int xr[8];
    float dv[8], rv[8], wv[8];
    load8(Xg, row_bytes, s_i, s_D, j0, xr, dv);
    float fr = 0.0f, fp = 0.0f, fw = 0.0f, fi = 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int x = xr[u];
      const float xf = (float)x;
      const float mu = M * dv[u];
      const float rc = fast_rcp(ph + mu);
      const float r = ph * (xf - mu) * rc;
      // psi(ph + x) - psi(ph): table, or for x >= 32 the asymptotic series
      // psi(z) = log(z - 1/2) + 1/(24 (z - 1/2)^2) + O((z - 1/2)^-4)
      float dg;
      if (x < HMC_TAB) {
        dg = tdg[x][tid];
      } else {
        const float iz = fast_rcp(ph + xf - 0.5f);
        dg = dg32 + log_hw((ph + xf - 0.5f) * iz32h) + (iz * iz - iz32h * iz32h) * (1.0f / 24.0f);
      }
      const float d1 = dg + log_hw(ph * rc) + (mu - xf) * rc;  // d ll / d phi
      fr += r;
      fp = fmaf(ph, d1, fp);
      rv[u] = gv ? r : 0.0f;
      if (METRIC && adapt) {
        const float w = ph * mu * (ph + xf) * (rc * rc);  // -d2 ll / d eta2
        const float tg = x < HMC_TAB ? ttg[x][tid] : tg32 + (tasym32 - trigamma_asym(ph + xf));
        const float d2 = -tg + iph - 2.0f * rc + (ph + xf) * rc * rc;  // d2 ll / d phi2
        fw += w;
        fi -= ph * (d1 + ph * d2);
        wv[u] = gv ? w : 0.0f;
      }
    }
    ar.add(fr);
    ap.add(fp);
    if (cells) {
      const float cs = transpose_sum8(rv, lane);
      if ((lane & 3) == 0) s_cell[warp][j0 + transpose_slot(lane)] = cs;
    }
    if (METRIC && adapt) {
      aw.add(fw);
      ai.add(fi);
      const float cw = transpose_sum8(wv, lane);
      if ((lane & 3) == 0) s_cellw[warp][j0 + transpose_slot(lane)] = cw;
    }
  }
  float* pr = s.hmc_part + (int64_t)row * NSLOT * Gp + g;
  pr[0] = gv ? ar.s - ar.c : 0.0f;
  pr[Gp] = gv ? ap.s - ap.c : 0.0f;
  if (METRIC && adapt) {
    pr[2 * Gp] = gv ? aw.s - aw.c : 0.0f;
    pr[3 * Gp] = gv ? ai.s - ai.c : 0.0f;
  }
  if (!cells && !cellw) return;  // uniform over the grid
  __syncthreads();
  for (int j = tid; j < len; j += GENE_TILE) {
    float t = 0.0f, tw = 0.0f;
#pragma unroll
    for (int w = 0; w < GENE_TILE / 32; ++w) {
      if (cells) t += s_cell[w][j];
      if (cellw) tw += s_cellw[w][j];
    }
    if (cells) s.hmc_cpart[(int64_t)tile * s.N + s_i[j]] = t;
    if (cellw) s.hmc_cpartw[(int64_t)tile * s.N + s_i[j]] = tw;
  }
}

__global__ void __launch_bounds__(GENE_TILE) k_hmc_grad(DevState s) { hmc_grad_body<false>(s, 0); }
__global__ void __launch_bounds__(GENE_TILE) k_hmc_grad_metric(DevState s, int metric_mode) {
  hmc_grad_body<true>(s, metric_mode);
}

// Precision of a free coordinate's prior; psi's (tau_phi phi) stays in the
// frozen part.
__device__ __forceinline__ double hmc_prior_precision(const DevState& s, const HmcCoord& c) {
  switch (c.kind) {
    case HK_ALPHA: return 1.0 / SIGMA2_ALPHA;
    case HK_BETA: return 1.0 / (s.L[(int64_t)c.seg * s.Gp + c.idx] == 1 ? TAU1 : (double)s.p_tau0[1]);
    case HK_NU: return 1.0 / SIGMA2_NU;
    case HK_PSI: return 0.0;
    default: return 1.0 / SIGMA2_DELTA;
  }
}

// Gradient (and metric) of every coordinate from the partial sums, plus the
// priors (thread per coordinate).
constexpr float HMC_MASS_FLOOR = 1e-2f;

__global__ void k_hmc_assemble(DevState s, int metric_mode) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= s.hmc_D) return;
  const bool adapt = hmc_metric_now(s, metric_mode);
  const HmcCoord c = hmc_coord(s, d);
  double gr = 0.0, m = 1.0;
  if (c.free) {
    const int64_t g = c.idx;
    const int B = s.B, K = s.K;
    switch (c.kind) {
      case HK_ALPHA: {
        float sr = 0.0f, sw = 0.0f;
        for (int b = 0; b < B; ++b)
          for (int k = 0; k < K; ++k) {
            sr += hmc_seg_sum(s, b, k, 0, g);
            if (adapt) sw += hmc_seg_sum(s, b, k, 2, g);
          }
        gr = sr - ((double)s.alpha[g] - (double)s.mu_alpha[g]) / SIGMA2_ALPHA;
        m = sw + 1.0 / SIGMA2_ALPHA;
        break;
      }
      case HK_BETA: {
        float sr = 0.0f, sw = 0.0f;
        for (int b = 0; b < B; ++b) {
          sr += hmc_seg_sum(s, b, c.seg, 0, g);
          if (adapt) sw += hmc_seg_sum(s, b, c.seg, 2, g);
        }
        const double v = s.L[(int64_t)c.seg * s.Gp + g] == 1 ? TAU1 : (double)s.p_tau0[1];
        gr = sr - (double)*c.pos / v;
        m = sw + 1.0 / v;
        break;
      }
      case HK_NU: {
        float sr = 0.0f, sw = 0.0f;
        for (int k = 0; k < K; ++k) {
          sr += hmc_seg_sum(s, c.seg, k, 0, g);
          if (adapt) sw += hmc_seg_sum(s, c.seg, k, 2, g);
        }
        gr = sr - ((double)*c.pos - (double)s.mu_nu[c.seg]) / SIGMA2_NU;
        m = sw + 1.0 / SIGMA2_NU;
        break;
      }
      case HK_PSI: {
        float sp = 0.0f, si = 0.0f;
        for (int k = 0; k < K; ++k) {
          sp += hmc_seg_sum(s, c.seg, k, 1, g);
          if (adapt) si += hmc_seg_sum(s, c.seg, k, 3, g);
        }
        const double ph = s.phi[(int64_t)c.seg * s.Gp + g];
        gr = sp + KAPPA_PHI - TAU_PHI * ph;
        m = si + TAU_PHI * ph;
        break;
      }
      default: {  // delta
        float sr = 0.0f, sw = 0.0f;
        for (int t = 0; t < s.n_tiles; ++t) {
          sr += s.hmc_cpart[(int64_t)t * s.N + c.idx];
          if (adapt) sw += s.hmc_cpartw[(int64_t)t * s.N + c.idx];
        }
        gr = sr - ((double)*c.pos - (double)s.mu_delta[c.idx]) / SIGMA2_DELTA;
        m = sw + 1.0 / SIGMA2_DELTA;
        break;
      }
    }
  }
  s.hmc_grad[d] = c.free ? (float)gr : 0.0f;
  if (adapt) {
    s.hmc_mass[d] = c.free ? fmaxf((float)m, HMC_MASS_FLOOR) : 1.0f;
    s.hmc_fis[d] = c.free ? (float)(m - hmc_prior_precision(s, c)) : 0.0f;
    if (s.hmc_gene && c.kind == HK_DELTA && c.idx != s.batch_off[c.seg]) {
      // held in the transition; its information scales its random-walk step
      float sw = 0.0f;
      for (int t = 0; t < s.n_tiles; ++t) sw += s.hmc_cpartw[(int64_t)t * s.N + c.idx];
      s.hmc_fis[d] = sw;
    }
  }
}

// The diagonal metric of the transition: the frozen information part plus the
// priors' precisions under the current L and tau0 (L and tau0 are held fixed
// within a transition, so the metric may follow them).
__global__ void k_hmc_mass(DevState s) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= s.hmc_D) return;
  const HmcCoord c = hmc_coord(s, d);
  s.hmc_mass[d] = c.free ? fmaxf(s.hmc_fis[d] + (float)hmc_prior_precision(s, c), HMC_MASS_FLOOR) : 1.0f;
}

// Momentum p ~ N(0, M) and the start of the trajectory; thread 0 draws the
// transition's jittered step size.
__global__ void k_hmc_start(DevState s) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  if (d == 0) {
    const float u = uniform_at(s.seed, SID_HMC_ACC, 0, iter, 1);
    s.hmc_sc[HS_EPS_USED] = s.hmc_sc[HS_EPS] * (0.9 + 0.2 * (double)u);
  }
  if (d >= s.hmc_D) return;
  const HmcCoord c = hmc_coord(s, d);
  if (c.free && hmc_in_block(s, c)) return;  // k_hmc_start_blocks draws these
  float p = 0.0f;
  if (c.free) {
    Stream st(s.seed, SID_HMC_MOM, (uint64_t)d, iter);
    p = sqrtf(s.hmc_mass[d]) * normal(st);
  }
  s.hmc_mom[d] = p;
  s.hmc_mom0[d] = p;
  s.hmc_th0[d] = *c.pos;
}

// exp(.) of the coordinates that feed the per-entry means.
__device__ __forceinline__ void hmc_derived(const DevState& s, const HmcCoord& c, float v) {
  if (c.kind == HK_PSI) s.phi[(int64_t)c.seg * s.Gp + c.idx] = expf(v);
  else if (c.kind == HK_DELTA) s.Dexp[c.idx] = expf(v);
}

// One leapfrog step: kick (half at the first step, full afterwards: the
// previous step's closing half kick merged in), then drift.
__global__ void k_hmc_leap(DevState s, int first) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= s.hmc_D) return;
  const HmcCoord c = hmc_coord(s, d);
  if (!c.free || hmc_in_block(s, c)) return;
  const float eps = c.kind == HK_DELTA ? (float)s.hmc_sc[HS_EPS_USED] : hmc_eps_gene(s, c.idx);
  const float p = s.hmc_mom[d] + (first ? 0.5f : 1.0f) * eps * s.hmc_grad[d];
  s.hmc_mom[d] = p;
  const float v = *c.pos + eps * p / s.hmc_mass[d];
  *c.pos = v;
  hmc_derived(s, c, v);
}

// E = exp(alpha + beta + nu) after the transition (for the W move).
__global__ void k_hmc_refresh_E(DevState s) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t Gp = s.Gp;
  if (t >= (int64_t)s.B * s.K * Gp) return;
  const int64_t g = t % Gp;
  const int64_t bk = t / Gp;
  const int k = (int)(bk % s.K), b = (int)(bk / s.K);
  s.E[t] = g < s.G ? exp_sum3(s.alpha[g], s.beta[(int64_t)k * Gp + g], s.nu[(int64_t)b * Gp + g]) : 1.0f;
}

// ---------------------------------------------------------------------------
// The lgamma part H(x) of the log-likelihood change depends on an entry only
// through x, and the entries with Y > 0 keep x = Y: their part comes from the
// static count tables once per (batch, gene).
// ---------------------------------------------------------------------------
// phi at the start of the transition and now, as k_hmc_dll forms them.
__device__ __forceinline__ void hmc_phi_pair(const DevState& s, int b, int64_t g, float& ph0, float& ph1,
                                             float& dph) {
  const int64_t Gp = s.Gp, o_psi = Gp * (1 + s.K + s.B);
  const float p0 = s.hmc_th0[o_psi + (int64_t)b * Gp + g], p1 = s.psi[(int64_t)b * Gp + g];
  ph0 = expf(p0);
  dph = ph0 * expm1f(p1 - p0);
  ph1 = ph0 + dph;
}

// One thread per (batch, gene): H(x) for x < PHI_TAB into phi_tab,
// lgamma(phi1) - lgamma(phi0) into phi_lgd0, and sum_y count(y) H(y) over the
// Y values 1 .. PHI_TAB-1 into phi_static (counts loaded ahead of the serial sum).
__global__ void k_hmc_dll_prep(DevState s) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)s.B * s.G) return;
  const int b = (int)(t / s.G);
  const int64_t g = t % s.G, Gp = s.Gp;
  float ph0, ph1, dph;
  hmc_phi_pair(s, b, g, ph0, ph1, dph);
  float* tab = s.phi_tab + (int64_t)b * PHI_TAB * Gp + g;
  const int32_t* cnt = s.phi_cnt + (int64_t)b * PHI_TAB * Gp + g;
  KahanF stat;
  float h = 0.0f;
  for (int x0 = 0; x0 < PHI_TAB; x0 += 16) {
    int c[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) c[u] = __ldg(cnt + (int64_t)(x0 + u) * Gp);
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int x = x0 + u;
      tab[(int64_t)x * Gp] = h;
      if (c[u]) stat.add((float)c[u] * h);
      h += log_ratio(ph1 + (float)x, ph0 + (float)x, dph);
    }
  }
  s.phi_lgd0[(int64_t)b * Gp + g] = lgamma_diff(ph0, ph1, dph);
  s.phi_static[(int64_t)b * Gp + g] = stat.value();
}

// One warp per (batch, gene) (warps striding over the pairs): the Stirling
// differences of its Y >= PHI_TAB values plus the part k_hmc_dll_prep left,
// summed per CTA (fixed order) into hmc_hpart[base + blockIdx.x], next to
// k_hmc_dll's per-CTA partials; with per_gene, each pair's total goes to
// phi_static[b][g] instead.
__global__ void __launch_bounds__(256) k_hmc_dll_static(DevState s, int base, int per_gene) {
  __shared__ FF sw[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nbg = (int64_t)s.B * s.G, nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  FF v{0.0f, 0.0f};  // this warp's (batch, gene) pairs, in order
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nbg; w += nw) {  // uniform per warp
    const int b = (int)(w / s.G);
    const int64_t g = w % s.G, pos = (int64_t)b * s.Gp + g;
    KahanF acc;
    const int64_t o0 = s.phi_big_off[w], o1 = s.phi_big_off[w + 1];
    if (o1 > o0) {
      float ph0, ph1, dph;
      hmc_phi_pair(s, b, g, ph0, ph1, dph);
      const float lgd0 = s.phi_lgd0[pos];
      for (int64_t q0 = o0; q0 < o1; q0 += 32 * 8) {  // eight values per lane in flight
        int yv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int64_t q = q0 + u * 32 + lane;
          yv[u] = q < o1 ? __ldg(s.phi_big_y + q) : -1;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (yv[u] >= 0) {
            const float y = (float)yv[u];
            acc.add(lgamma_diff_large(ph0 + y, ph1 + y, dph) - lgd0);
          }
      }
    }
    FF f = acc.ff();
    if (per_gene) {  // uniform over the grid
      f = ff_warp_sum(f);
      if (lane == 0) s.phi_static[pos] += ff_value(f);
      continue;
    }
    if (lane == 0) {
      const double d = s.phi_static[pos];
      const float hi = (float)d;
      f = ff_add(f, FF{hi, (float)(d - (double)hi)});
    }
    v = ff_add(v, f);
  }
  v = ff_warp_sum(v);
  if (lane == 0) sw[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    FF t = sw[0];
    for (int i = 1; i < 8; ++i) t = ff_add(t, sw[i]);
    s.hmc_hpart[base + blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------------------
// Change of the log likelihood between the start of the trajectory (th0) and
// the current coordinates, per entry without cancellation:
//   dl = H(x) + phi1 log(phi1/phi0) - (phi1 + x) log((phi1 + mu1) / (phi0 + mu0))
//        - dphi log1p(mu0 / phi0) + x deta,
//   H(x) = [lgamma(phi1 + x) - lgamma(phi1)] - [lgamma(phi0 + x) - lgamma(phi0)],
//   mu1 - mu0 = mu0 expm1(deta), phi1 - phi0 = phi0 expm1(psi1 - psi0).
// One float-float partial per CTA in hmc_hpart; with per_gene, each gene's
// chunk sum in part slot 0 instead (the decisions sum them per gene).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(GENE_TILE) k_hmc_dll(DevState s, int per_gene) {
  __shared__ float tab[PHI_TAB][GENE_TILE];
  __shared__ __align__(16) int s_i[MAX_CG];
  __shared__ __align__(16) float s_D[MAX_CG];
  __shared__ float s_dd[MAX_CG];
  __shared__ FF shf[GENE_TILE / 32];
  __shared__ long long shn[GENE_TILE / 32];
  const int tid = threadIdx.x;
  const int tile = blockIdx.x, row = blockIdx.y;
  const int cta = row * gridDim.x + tile;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  if (len == 0) {
    if (tid == 0) s.hmc_hpart[cta] = FF{0.0f, 0.0f};
    return;
  }
  const float* th0 = s.hmc_th0;
  const int64_t o_beta = Gp, o_nu = Gp * (1 + s.K), o_psi = Gp * (1 + s.K + s.B), o_delta = Gp * (1 + s.K + 2 * s.B);
  const int len8 = (len + 7) & ~7;
  for (int j = tid; j < len8; j += GENE_TILE) {
    const bool in = j < len;
    const int i = in ? s.perm[start + j] : (int)s.N;
    s_i[j] = i;
    const float d0 = in ? th0[o_delta + i] : 0.0f;
    s_D[j] = in ? expf(d0) : 0.0f;  // exp(delta0)
    s_dd[j] = in ? s.delta[i] - d0 : 0.0f;
  }
  const bool gv = g < s.G;
  float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f, n0 = 0.f, n1 = 0.f, p0 = 0.f, p1 = 0.f;
  if (gv) {
    a0 = th0[g];
    a1 = s.alpha[g];
    b0 = th0[o_beta + (int64_t)k * Gp + g];
    b1 = s.beta[(int64_t)k * Gp + g];
    n0 = th0[o_nu + (int64_t)b * Gp + g];
    n1 = s.nu[(int64_t)b * Gp + g];
    p0 = th0[o_psi + (int64_t)b * Gp + g];
    p1 = s.psi[(int64_t)b * Gp + g];
  }
  const float M0 = gv ? exp_sum3(a0, b0, n0) : 0.0f;
  const float dA = (a1 - a0) + (b1 - b0) + (n1 - n0);
  const float ph0 = expf(p0);
  const float dph = ph0 * expm1f(p1 - p0);
  const float ph1 = ph0 + dph;
  const float c1 = ph1 * log_ratio(ph1, ph0, dph);
  // H(x) for x < PHI_TAB and lgamma(phi1) - lgamma(phi0), from k_hmc_dll_prep
  const float lgd0 = gv ? s.phi_lgd0[(int64_t)b * Gp + g] : 0.0f;
  {
    const float* tg = s.phi_tab + (int64_t)b * PHI_TAB * Gp + g;
#pragma unroll 8
    for (int x = 0; x < PHI_TAB; ++x) tab[x][tid] = gv ? tg[(int64_t)x * Gp] : 0.0f;
  }
  __syncthreads();
  // Y == 0 bit of the entry (row N, the padding row, is all zero); the H(x) of
  // the entries with Y > 0 is k_hmc_dll_static's
  const uint32_t* ym = s.y0m + (g >> 5);
  const int64_t Gw = s.Gw;
  const int bit = (int)(g & 31);
  const float iph0 = fast_rcp(ph0);
  const char* Xg = reinterpret_cast<const char*>(s.X + g);
  const uint32_t row_bytes = (uint32_t)(Gp * sizeof(int));
  KahanF acc;
  for (int j0 = 0; j0 < len8; j0 += 8) {
    int xr[8];
    float dv[8];
    load8(Xg, row_bytes, s_i, s_D, j0, xr, dv);
    uint32_t zw[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) zw[u] = ym[(int64_t)s_i[j0 + u] * Gw];
    float f = 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int x = xr[u];
      const float xf = (float)x;
      const float mu0 = M0 * dv[u];
      const float de = dA + s_dd[j0 + u];
      const float dmu = mu0 * expm1f(de);
      const bool y0 = (zw[u] >> bit) & 1u;
      float hx = y0 && x < PHI_TAB ? tab[x][tid] : 0.0f;
      if (y0 && x >= PHI_TAB) hx = lgamma_diff_large(ph0 + xf, ph1 + xf, dph) - lgd0;  // rare
      const float t = hx + c1 - (ph1 + xf) * log_ratio(ph1 + mu0 + dmu, ph0 + mu0, dph + dmu) -
                      dph * log1p_fast(mu0 * iph0) + xf * de;
      f += dv[u] > 0.0f ? t : 0.0f;  // padding cells contribute nothing
    }
    acc.add(f);
  }
  if (per_gene) {  // uniform over the grid
    if (gv) s.part[(int64_t)row * NSLOT * Gp + g] = acc.value();
    return;
  }
  FF fsum[1] = {gv ? acc.ff() : FF{0.0f, 0.0f}};
  long long nn[1] = {0};
  block_sum_ff<1, 1>(fsum, nn, shf, shn);
  if (tid == 0) s.hmc_hpart[cta] = fsum[0];
}

// Closing half kick, then per coordinate the kinetic change minus the prior
// change (cancellation-free), summed per CTA into hmc_epart.
__global__ void __launch_bounds__(256) k_hmc_energy(DevState s, int kick, int per_gene) {
  __shared__ FF shf[8];
  __shared__ long long shn[8];
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.0f;
  if (d < s.hmc_D) {
    const HmcCoord c = hmc_coord(s, d);
    if (c.free && !hmc_in_block(s, c)) {
      float p = s.hmc_mom[d];
      if (kick) {
        const float eps = c.kind == HK_DELTA ? (float)s.hmc_sc[HS_EPS_USED] : hmc_eps_gene(s, c.idx);
        p += 0.5f * eps * s.hmc_grad[d];
        s.hmc_mom[d] = p;
      }
      const float p0 = s.hmc_mom0[d];
      const float dK = p == p0 ? 0.0f : (p - p0) * (p + p0) * 0.5f / s.hmc_mass[d];
      const float v1 = *c.pos, v0 = s.hmc_th0[d];
      const float dv = v1 - v0;
      float dprior;
      switch (c.kind) {
        case HK_ALPHA: {
          const float m = s.mu_alpha[c.idx];
          dprior = -dv * ((v1 - m) + (v0 - m)) * (float)(0.5 / SIGMA2_ALPHA);
          break;
        }
        case HK_BETA: {
          const double v = s.L[(int64_t)c.seg * s.Gp + c.idx] == 1 ? TAU1 : (double)s.p_tau0[1];
          dprior = (float)(-(double)dv * ((double)v1 + (double)v0) * 0.5 / v);
          break;
        }
        case HK_NU: {
          const float m = s.mu_nu[c.seg];
          dprior = -dv * ((v1 - m) + (v0 - m)) * (float)(0.5 / SIGMA2_NU);
          break;
        }
        case HK_PSI:
          dprior = (float)KAPPA_PHI * dv - (float)TAU_PHI * expf(v0) * expm1f(dv);
          break;
        default: {
          const float m = s.mu_delta[c.idx];
          dprior = -dv * ((v1 - m) + (v0 - m)) * (float)(0.5 / SIGMA2_DELTA);
          break;
        }
      }
      e = dK - dprior;
    }
    if (per_gene) s.hmc_e[d] = e;
  }
  if (per_gene) return;  // uniform over the grid
  FF f[1] = {FF{e, 0.0f}};
  long long n[1] = {0};
  block_sum_ff<1, 1>(f, n, shf, shn);
  if (threadIdx.x == 0) s.hmc_epart[blockIdx.x] = f[0];
}

// Per-gene decisions (hmc_gene): gene g's change of H = -log p + K is
//   dH_g = -(its log-likelihood change: the chunk sums in part slot 0 over its
//           (batch, type) segments, plus phi_static[b][g] over the batches)
//          + (kinetic minus prior change of its coordinates: hmc_e over
//             alpha_g, beta_gk, nu_bg, psi_bg, and hmc_eb[g] for its block),
// decided on its own uniform (stream SID_HMC_ACC, entity 1 + g).  Per CTA: the
// sum of the acceptance probabilities into hmc_hpart and the number accepted
// into hmc_epart, for k_hmc_accept (mode 2).  With dlp, only the change of
// each gene's log posterior (-dH_g, zero momenta) is written there.
__global__ void __launch_bounds__(256) k_hmc_accept_genes(DevState s, double* dlp) {
  __shared__ FF shf[8 * 2];
  __shared__ long long shn[8];
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t Gp = s.Gp;
  const int B = s.B, K = s.K;
  const uint32_t iter = (uint32_t)*s.iter;
  double a = 0.0;
  long long nacc = 0;
  if (g < s.G) {
    double dll = 0.0, e = 0.0;
    for (int b = 0; b < B; ++b) {
      for (int k = 0; k < K; ++k) dll += seg_sum(s, b, k, 0, g);
      dll += s.phi_static[(int64_t)b * Gp + g];
    }
    e += s.hmc_e[g];
    for (int k = 1; k < K; ++k) e += s.hmc_e[Gp + (int64_t)k * Gp + g];
    for (int b = 1; b < B; ++b) e += s.hmc_e[Gp * (1 + K) + (int64_t)b * Gp + g];
    for (int b = 0; b < B; ++b) e += s.hmc_e[Gp * (1 + K + B) + (int64_t)b * Gp + g];
    if (s.hmc_nb > 0) e += s.hmc_eb[g];
    const double dH = -dll + e;
    if (dlp) {
      dlp[g] = -dH;
    } else {
      a = dH == dH ? fmin(1.0, exp(-dH)) : 0.0;
      const float u = uniform_at(s.seed, SID_HMC_ACC, 1 + (uint64_t)g, iter, 0);
      const bool accept = dH == dH && (double)logf(u) < -dH;
      s.hmc_gacc[g] = accept ? 1 : 0;
      nacc = accept ? 1 : 0;
    }
  }
  if (dlp) return;  // uniform over the grid
  const float ah = (float)a;
  FF f[1] = {FF{ah, (float)(a - (double)ah)}};
  long long n[1] = {nacc};
  block_sum_ff<1, 1>(f, n, shf, shn);
  if (threadIdx.x == 0) {
    s.hmc_hpart[blockIdx.x] = f[0];
    s.hmc_epart[blockIdx.x] = FF{(float)n[0], 0.0f};
  }
}

// The Metropolis decision on H = -log p + K (one CTA), and the step-size
// adaptation.  mode 1 only reports the change of the log posterior
// (-(H1 - H0) with zero momenta) in HS_LAST_DH; mode 2 takes the per-gene
// decisions of k_hmc_accept_genes (n_hpart = n_epart = its CTAs) and adapts the
// step size to their mean acceptance probability.
__global__ void __launch_bounds__(256) k_hmc_accept(DevState s, int n_hpart, int n_epart, int n_epart_b, int mode) {
  __shared__ FF shf[8 * 2];
  __shared__ long long shn[8];
  FF acc{0.0f, 0.0f}, ace{0.0f, 0.0f};
  for (int t = threadIdx.x; t < n_hpart; t += blockDim.x) acc = ff_add(acc, s.hmc_hpart[t]);
  for (int t = threadIdx.x; t < n_epart; t += blockDim.x) ace = ff_add(ace, s.hmc_epart[t]);
  if (s.hmc_nb > 0 && mode != 2)
    for (int t = threadIdx.x; t < n_epart_b; t += blockDim.x) ace = ff_add(ace, s.hmc_epart_b[t]);
  FF f[2] = {acc, ace};
  long long n[1] = {0};
  block_sum_ff<2, 1>(f, n, shf, shn);
  if (threadIdx.x != 0) return;
  double* sc = s.hmc_sc;
  const int iter = *s.iter;
  double a, acc_frac;
  if (mode == 2) {
    a = ff_value(f[0]) / (double)s.G;         // mean acceptance probability over the genes
    acc_frac = ff_value(f[1]) / (double)s.G;  // fraction of genes accepted
    sc[HS_LAST_DH] = 0.0;
  } else {
    const double dll = ff_value(f[0]);
    const double dH = -dll + ff_value(f[1]);
    sc[HS_LAST_DH] = dH;
    if (mode == 1) {
      sc[HS_LAST_DH] = -dH;
      return;
    }
    a = dH == dH ? fmin(1.0, exp(-dH)) : 0.0;
    const float u = uniform_at(s.seed, SID_HMC_ACC, 0, (uint32_t)iter, 0);
    const bool accept = dH == dH && (double)logf(u) < -dH;
    sc[HS_ACCEPTED] = accept ? 1.0 : 0.0;
    acc_frac = accept ? 1.0 : 0.0;
  }
  sc[HS_LAST_ACC] = a;
  if (iter >= s.n_burnin) {
    sc[HS_N_KEPT] += 1.0;
    sc[HS_ACC_KEPT] += acc_frac;
  }
  // dual averaging during burn-in, restarted when the metric freezes
  if (iter < s.n_burnin) {
    const int restart = s.n_burnin / 2;
    if (iter == restart) {
      sc[HS_HBAR] = 0.0;
      sc[HS_M] = 0.0;
      sc[HS_MU] = log(10.0 * sc[HS_EPS]);
      sc[HS_LOG_EPS_BAR] = 0.0;
    }
    const double gam = 0.05, t0 = 10.0, kap = 0.75, target = HMC_TARGET_ACCEPT;
    const double m = sc[HS_M] + 1.0;
    sc[HS_M] = m;
    sc[HS_HBAR] = (1.0 - 1.0 / (m + t0)) * sc[HS_HBAR] + (target - a) / (m + t0);
    const double log_eps = sc[HS_MU] - sqrt(m) / gam * sc[HS_HBAR];
    const double w = pow(m, -kap);
    sc[HS_LOG_EPS_BAR] = w * log_eps + (1.0 - w) * sc[HS_LOG_EPS_BAR];
    sc[HS_EPS] = exp(fmin(fmax(log_eps, -12.0), 2.0));
    if (iter == s.n_burnin - 1) sc[HS_EPS] = exp(fmin(fmax(sc[HS_LOG_EPS_BAR], -12.0), 2.0));
  }
}

// Restores the start of the trajectory when the transition was rejected (with
// per-gene decisions: the coordinates of each rejected gene).
__global__ void k_hmc_finish(DevState s) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= s.hmc_D) return;
  if (!s.hmc_gene && s.hmc_sc[HS_ACCEPTED] != 0.0) return;
  const HmcCoord c = hmc_coord(s, d);
  if (!c.free) return;
  if (s.hmc_gene && s.hmc_gacc[c.idx]) return;  // c.idx is the gene of every free coordinate there
  const float v = s.hmc_th0[d];
  *c.pos = v;
  hmc_derived(s, c, v);
}

// ---------------------------------------------------------------------------
// Per-gene block metric.  Within gene g the coordinates
//   u = (alpha_g, beta_g1 .. beta_g(K-1), nu_g1 .. nu_g(B-1))
// enter every entry's eta through a_bk . u (a_bk: 1 for alpha, 1 for beta_k if
// k >= 1, 1 for nu_b if b >= 1), so the observed information of u is
//   F_g = sum_{b,k} W_bkg a_bk a_bk^T,   W_bkg = sum over the cells of (b, k) of
//   phi mu (phi + x) / (phi + mu)^2  (part slot 2, per segment),
// plus the priors' precisions on the diagonal.  Its Cholesky factor turns the
// strong alpha-beta and alpha-nu correlations (alpha is informed only by
// type-0 cells once the betas are free) into unit scale.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t hmc_block_pos(const DevState& s, int j, int64_t g) {
  const int K = s.K;
  if (j == 0) return g;                                              // alpha
  if (j < K) return s.Gp + (int64_t)j * s.Gp + g;                    // beta_j
  return s.Gp * (1 + K) + (int64_t)(j - K + 1) * s.Gp + g;           // nu_(j-K+1)
}

__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }  // j <= i

// per-gene storage of the factor and the inverse (gene-major)
constexpr int HMC_TRI = HMC_BLOCK_MAX * (HMC_BLOCK_MAX + 1) / 2;
constexpr int HMC_SQ = HMC_BLOCK_MAX * HMC_BLOCK_MAX;

__global__ void k_hmc_metric_blocks(DevState s, int metric_mode) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= s.G || s.hmc_nb == 0) return;
  const bool adapt = hmc_metric_now(s, metric_mode);
  const int K = s.K, B = s.B, nb = s.hmc_nb;
  float F[HMC_TRI];
  for (int t = 0; t < nb * (nb + 1) / 2; ++t) F[t] = 0.0f;
  for (int b = 0; b < B; ++b)
    for (int k = 0; k < K; ++k) {
      float* wp = s.hmc_wbk + ((int64_t)b * K + k) * s.G + g;
      if (adapt) *wp = hmc_seg_sum(s, b, k, 2, g);
      const float w = *wp;
      // a_bk has ones at 0, k (k >= 1) and K - 1 + b (b >= 1)
      int idx[3], n = 0;
      idx[n++] = 0;
      if (k >= 1) idx[n++] = k;
      if (b >= 1) idx[n++] = K - 1 + b;
      for (int p = 0; p < n; ++p)
        for (int q = 0; q <= p; ++q) F[tri(idx[p], idx[q])] += w;
    }
  // the priors' precisions under the current L and tau0
  F[tri(0, 0)] += (float)(1.0 / SIGMA2_ALPHA);
  for (int k = 1; k < K; ++k)
    F[tri(k, k)] += (float)(1.0 / (s.L[(int64_t)k * s.Gp + g] == 1 ? TAU1 : (double)s.p_tau0[1]));
  for (int b = 1; b < B; ++b) F[tri(K - 1 + b, K - 1 + b)] += (float)(1.0 / SIGMA2_NU);
  // in-place Cholesky F = L L^T (lower); a non-positive pivot falls back to
  // the diagonal
  bool ok = true;
  for (int i = 0; i < nb && ok; ++i) {
    for (int j = 0; j <= i; ++j) {
      float v = F[tri(i, j)];
      for (int q = 0; q < j; ++q) v -= F[tri(i, q)] * F[tri(j, q)];
      if (i == j) {
        if (!(v > 0.0f)) {
          ok = false;
          break;
        }
        F[tri(i, i)] = sqrtf(v);
      } else {
        F[tri(i, j)] = v / F[tri(j, j)];
      }
    }
  }
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j <= i; ++j) {
      float v;
      if (ok) v = F[tri(i, j)];
      else v = i == j ? sqrtf(fmaxf(s.hmc_mass[hmc_block_pos(s, i, g)], HMC_MASS_FLOOR)) : 0.0f;
      F[tri(i, j)] = v;
      s.hmc_chol[g * HMC_TRI + tri(i, j)] = v;
    }
  // M^{-1} = L^{-T} L^{-1}: invert L in place (lower), then the product
  for (int i = 0; i < nb; ++i) {
    F[tri(i, i)] = 1.0f / F[tri(i, i)];
    for (int j = 0; j < i; ++j) {
      float v = 0.0f;
      for (int q = j; q < i; ++q) v += F[tri(i, q)] * F[tri(q, j)];
      F[tri(i, j)] = -v * F[tri(i, i)];
    }
  }
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j <= i; ++j) {
      float v = 0.0f;
      for (int q = i; q < nb; ++q) v += F[tri(q, i)] * F[tri(q, j)];
      s.hmc_minv[g * HMC_SQ + i * nb + j] = v;
      s.hmc_minv[g * HMC_SQ + j * nb + i] = v;
    }
}


// The gene-block kernels run one warp per gene: lane i < nb holds block
// coordinate i, and the products with the factor or the inverse gather the
// other coordinates by shuffles.
__device__ __forceinline__ float* hmc_block_ptr(const DevState& s, int i, int64_t g) {
  if (i == 0) return s.alpha + g;
  if (i < s.K) return s.beta + (int64_t)i * s.Gp + g;
  return s.nu + (int64_t)(i - s.K + 1) * s.Gp + g;
}

// sum_j A[i][j] x_j over the warp's block (A row-major, nb x nb, at `a`).
__device__ __forceinline__ float hmc_row_dot(const float* a, int nb, int lane, float x) {
  float acc = 0.0f;
  for (int j = 0; j < nb; ++j) {
    const float xj = __shfl_sync(0xffffffffu, x, j);
    if (lane < nb) acc = fmaf(a[lane * nb + j], xj, acc);
  }
  return acc;
}

// Momentum of the gene blocks: p = L z, z ~ N(0, I).
__global__ void __launch_bounds__(128) k_hmc_start_blocks(DevState s) {
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= s.G || s.hmc_nb == 0) return;  // whole warps leave together
  const int nb = s.hmc_nb;
  const uint32_t iter = (uint32_t)*s.iter;
  float z = 0.0f;
  if (lane < nb) {
    Stream st(s.seed, SID_HMC_MOM, (uint64_t)s.hmc_D + (uint64_t)g * HMC_BLOCK_MAX + lane, iter);
    z = normal(st);
  }
  const float* L = s.hmc_chol + g * HMC_TRI;
  float p = 0.0f;
  for (int q = 0; q < nb; ++q) {
    const float zq = __shfl_sync(0xffffffffu, z, q);
    if (lane < nb && q <= lane) p = fmaf(L[tri(lane, q)], zq, p);
  }
  if (lane < nb) {
    const int64_t d = hmc_block_pos(s, lane, g);
    s.hmc_mom[d] = p;
    s.hmc_mom0[d] = p;
    s.hmc_th0[d] = *hmc_block_ptr(s, lane, g);
  }
}

// Kick and drift of the gene blocks: p += c eps grad, u += eps M^{-1} p.
__global__ void __launch_bounds__(128) k_hmc_leap_blocks(DevState s, int first) {
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= s.G || s.hmc_nb == 0) return;
  const int nb = s.hmc_nb;
  const float eps = hmc_eps_gene(s, g);
  float p = 0.0f;
  int64_t d = 0;
  if (lane < nb) {
    d = hmc_block_pos(s, lane, g);
    p = s.hmc_mom[d] + (first ? 0.5f : 1.0f) * eps * s.hmc_grad[d];
    s.hmc_mom[d] = p;
  }
  const float v = hmc_row_dot(s.hmc_minv + g * HMC_SQ, nb, lane, p);
  if (lane < nb) *hmc_block_ptr(s, lane, g) += eps * v;
}

// Closing half kick of the gene blocks, then their kinetic change
// (p^T M^{-1} p - p0^T M^{-1} p0) / 2 minus the prior change, per CTA.
__global__ void __launch_bounds__(256) k_hmc_energy_blocks(DevState s, int kick, int per_gene) {
  __shared__ FF shf[8];
  __shared__ long long shn[8];
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  float e = 0.0f;
  if (g < s.G && s.hmc_nb > 0) {
    const int nb = s.hmc_nb, K = s.K;
    const float eps = hmc_eps_gene(s, g);
    float p = 0.0f, p0 = 0.0f, dprior = 0.0f;
    if (lane < nb) {
      const int64_t d = hmc_block_pos(s, lane, g);
      p = s.hmc_mom[d];
      if (kick) {
        p += 0.5f * eps * s.hmc_grad[d];
        s.hmc_mom[d] = p;
      }
      p0 = s.hmc_mom0[d];
      // prior change of this coordinate (cancellation-free)
      const float v1 = *hmc_block_ptr(s, lane, g), v0 = s.hmc_th0[d];
      if (lane == 0) {
        const float m = s.mu_alpha[g];
        dprior = -(v1 - v0) * ((v1 - m) + (v0 - m)) * (float)(0.5 / SIGMA2_ALPHA);
      } else if (lane < K) {
        const double v = s.L[(int64_t)lane * s.Gp + g] == 1 ? TAU1 : (double)s.p_tau0[1];
        dprior = (float)(-(double)(v1 - v0) * ((double)v1 + (double)v0) * 0.5 / v);
      } else {
        const float m = s.mu_nu[lane - K + 1];
        dprior = -(v1 - v0) * ((v1 - m) + (v0 - m)) * (float)(0.5 / SIGMA2_NU);
      }
    }
    const bool same = __all_sync(0xffffffffu, p == p0);
    float dk = 0.0f;
    if (!same) {
      const float* a = s.hmc_minv + g * HMC_SQ;
      const float v = hmc_row_dot(a, nb, lane, p);
      const float v0 = hmc_row_dot(a, nb, lane, p0);
      dk = 0.5f * (p * v - p0 * v0);
    }
    e = dk - dprior;
  }
  if (per_gene) {  // uniform over the grid; warps are whole genes
    const double eg = warp_sum((double)e);
    if (g < s.G && s.hmc_nb > 0 && lane == 0) s.hmc_eb[g] = (float)eg;
    return;
  }
  FF f[1] = {FF{e, 0.0f}};
  long long n[1] = {0};
  block_sum_ff<1, 1>(f, n, shf, shn);
  if (threadIdx.x == 0) s.hmc_epart_b[blockIdx.x] = f[0];
}

// Unit metric before the first adaptation.
__global__ void k_hmc_unit_mass(DevState s) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d < s.hmc_D) s.hmc_mass[d] = 1.0f;
}

// Loads `src` (flat layout) into th0 for the log-posterior difference.
__global__ void k_hmc_set_th0(DevState s, const float* src) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= s.hmc_D) return;
  s.hmc_th0[d] = src[d];
  s.hmc_mom[d] = 0.0f;
  s.hmc_mom0[d] = 0.0f;
}

}  // namespace bq
