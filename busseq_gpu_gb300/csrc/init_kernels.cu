// Initialisation, posterior summaries and BIC.
//
// Initialisation restates BUSseq_gpu.cu:1163-1244 (kernels :369-482) as a
// handful of passes instead of the reference's B*K*G*3 single-block launches:
//   k_init_scan    Y == 0 bit masks, library sizes, largest count
//   k_init_hist    histogram of the positive counts per batch (gamma statistics)
//   k_init_w_delta W ~ Cat(pi_init), delta = log(lib_i) - log(lib_first of batch)
//   k_sort_pi      cell order (no pi draw)
//   k_init_raw     raw means of log(1 + Y e^-delta) per (batch, type, gene) and
//                  alpha, beta, nu, L from them; mu_nu from the batch means
//   k_init_finish  phi, gamma, pi, mu_delta, exp(delta), exp(alpha+beta+nu)
// Summaries: k_finalize (posterior means, P(L=1), W mode; :1557-1608) and
// k_bic_cell + k_bic_total (:967-1024, :1815-1843).
#include "kernels_common.cuh"
#include "bic_series.h"

namespace bq {

__global__ void k_init_scan(DevState s, int64_t* libsize, int* ymax, int32_t* rowcnt) {
  const int64_t i = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __shared__ long long sh_sum[32];
  __shared__ int sh_max[32];
  __shared__ int sh_cnt[32];
  long long sum = 0;
  int mx = 0, nzero = 0;
  for (int64_t w = warp; w < s.Gw; w += nw) {
    const int64_t g = w * 32 + lane;
    const int y = g < s.G ? s.Y[i * s.Gp + g] : 1;
    const unsigned m = __ballot_sync(0xffffffffu, y == 0);
    if (lane == 0) {
      const_cast<uint32_t*>(s.y0m)[i * s.Gw + w] = m;
      nzero += __popc(m);
    }
    if (g < s.G) {
      sum += y;
      mx = max(mx, y);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  if (lane == 0) { sh_sum[warp] = sum; sh_max[warp] = mx; sh_cnt[warp] = nzero; }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    int m = 0, c = 0;
    for (int w = 0; w < nw; ++w) { t += sh_sum[w]; m = max(m, sh_max[w]); c += sh_cnt[w]; }
    libsize[i] = t;
    rowcnt[i] = c;
    atomicMax(ymax, m);
  }
}

// The list of entries with Y == 0, row by row: one warp per cell, 32 mask
// words at a time, positions from a warp prefix sum of the words' popcounts.
__global__ void k_zlist_fill(DevState s, const int64_t* rowoff, int2* zij) {
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= s.N) return;
  const int lane = threadIdx.x & 31;
  int64_t base = rowoff[i];
  for (int64_t w0 = 0; w0 < s.Gw; w0 += 32) {
    const int64_t w = w0 + lane;
    const uint32_t m = w < s.Gw ? s.y0m[i * s.Gw + w] : 0u;
    const int c = __popc(m);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int64_t pos = base + incl - c;
    uint32_t mm = m;
    while (mm) {
      const int bit = __ffs(mm) - 1;
      mm &= mm - 1u;
      zij[pos++] = make_int2((int)i, (int)(w * 32 + bit));
    }
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// zval[j] = Z bit of entry j from the bit mask (after a state upload).
__global__ void k_zval_from_mask(DevState s) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= s.nz0) return;
  const int2 ig = s.zij[j];
  s.zval[j] = (uint8_t)((s.zm[(int64_t)ig.x * s.Gw + (ig.y >> 5)] >> (ig.y & 31)) & 1u);
}

// Bit mask from zval (the mask must be cleared first).
__global__ void k_zmask_from_zval(DevState s) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= s.nz0) return;
  if (!s.zval[j]) return;
  const int2 ig = s.zij[j];
  atomicOr(&s.zm[(int64_t)ig.x * s.Gw + (ig.y >> 5)], 1u << (ig.y & 31));
}

// X at the Y == 0 entries, in list order (checkpoint files store only these:
// X equals Y everywhere else).
__global__ void k_zlist_gather_x(DevState s, int32_t* out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= s.nz0) return;
  const int2 ig = s.zij[j];
  out[j] = s.X[(int64_t)ig.x * s.Gp + ig.y];
}

__global__ void k_zlist_scatter_x(DevState s, const int32_t* in) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= s.nz0) return;
  const int2 ig = s.zij[j];
  s.X[(int64_t)ig.x * s.Gp + ig.y] = in[j];
}

// Order-independent 64-bit fingerprint of Y: sum over entries of
// (Y + 1) * mix(entry index + 0x9E3779B97F4A7C15) mod 2^64, mix = the
// SplitMix64 finaliser (the offset keeps every entry's weight nonzero: the
// finaliser maps 0 to 0).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_y_fingerprint(DevState s, unsigned long long* out) {
  const int64_t total = s.N * s.G;
  uint64_t acc = 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / s.G, g = e - i * s.G;
    acc += (uint64_t)(s.Y[i * s.Gp + g] + 1) * mix64((uint64_t)e + 0x9E3779B97F4A7C15ull);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, (unsigned long long)acc);
}

// Histogram of Y > 0 per batch; warp-aggregated so that repeated small values
// cost one atomic per distinct value per warp.
// One CTA per cell: counts below HIST_SMEM_BINS go to a shared-memory
// histogram (one shared atomic per distinct value of a warp's 32 counts) and
// the CTA adds its non-zero bins to the batch's histogram; larger counts go
// to the global histogram directly.  Counts are integers, so the result does
// not depend on the order of the additions.
constexpr int HIST_SMEM_BINS = 4096;
__global__ void __launch_bounds__(256) k_init_hist(DevState s, int32_t* hist) {
  __shared__ int sh[HIST_SMEM_BINS];
  const int64_t i = blockIdx.x;
  const int b = s.batch_of[i];
  const int lane = threadIdx.x & 31;
  int32_t* h = hist + (int64_t)b * (s.ymax + 1);
  const int nbins = min(HIST_SMEM_BINS, s.ymax + 1);
  for (int t = threadIdx.x; t < nbins; t += blockDim.x) sh[t] = 0;
  __syncthreads();
  for (int64_t g0 = (int64_t)(threadIdx.x & ~31); g0 < s.Gp; g0 += blockDim.x) {
    const int64_t g = g0 + lane;
    const int y = g < s.G ? s.Y[i * s.Gp + g] : 0;
    const unsigned same = __match_any_sync(0xffffffffu, y);
    if (y > 0 && __ffs(same) - 1 == lane) {
      if (y < nbins) atomicAdd(&sh[y], __popc(same));
      else atomicAdd(&h[y], __popc(same));
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nbins; t += blockDim.x)
    if (sh[t]) atomicAdd(&h[t], sh[t]);
}

__global__ void k_init_w_delta(DevState s, const int64_t* libsize, int* bad_cell) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.N) return;
  const int b = s.batch_of[i];
  const int K = s.K;
  Stream st(s.seed, SID_INIT_W, (uint64_t)i, 0u);
  const float u = st.uniform();
  // pi_init[k] = (k+1) / (K(K+1)/2), first_pi (BUSseq_gpu.cu:392-397)
  const double den = K * (K + 1) / 2.0;
  int k = 0;
  double acc = 1.0 / den;
  while ((double)u > acc && k < K - 1) { ++k; acc += (k + 1) / den; }
  s.W[i] = k;
  const int64_t l = libsize[i], l0 = libsize[s.batch_off[b]];
  if (l <= 0) atomicMin(bad_cell, (int)i);
  s.delta[i] = (float)(log((double)l) - log((double)l0));
}

// Raw means and the parameters derived from them.  Gene-pass layout: CTA =
// (gene tile, chunk of one (batch, type) segment).  Tile tails compute, per
// gene, raw[b][k] = mean over the segment of log(1 + Y e^-delta), then
//   alpha = mu_alpha = raw[0][0], beta_k = raw[0][k] - raw[0][0],
//   nu_b = (sum_k raw[b][k] - sum_k raw[0][k]) / K, L_k ~ prior odds;
// the last tile turns the batch sums into mu_nu (BUSseq_gpu.cu:1232-1241).
__global__ void __launch_bounds__(GENE_TILE) k_init_raw(DevState s) {
  __shared__ double sh[(GENE_TILE / 32) * MAX_B];
  __shared__ int sh_flag;
  __shared__ int s_i[MAX_CG];
  __shared__ float s_e[MAX_CG];  // exp(-delta) of the chunk's cells
  const int tid = threadIdx.x;
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  const bool valid = g < s.G;
  if (len > 0) {  // uniform over the CTA
    for (int j = tid; j < len; j += blockDim.x) {
      const int i = s.perm[start + j];
      s_i[j] = i;
      s_e[j] = expf(-s.delta[i]);
    }
    __syncthreads();
  }
  if (len > 0 && valid) {
    double acc = 0.0;
    for (int j0 = 0; j0 < len; j0 += 32) {
      const int jn = min(32, len - j0);
      float f = 0.0f;
      for (int jj = 0; jj < jn; jj += 8) {  // eight rows' loads in flight, summed in cell order
        float yv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          yv[u] = jj + u < jn ? (float)__ldg(&s.Y[(int64_t)s_i[j0 + jj + u] * Gp + g]) : 0.0f;
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (jj + u < jn) f += log1pf(yv[u] * s_e[j0 + jj + u]);
      }
      acc += f;
    }
    s.part[(int64_t)row * NSLOT * Gp + g] = acc;
  }
  if (!arrive_last(&s.cnt_tile[tile], (unsigned)s.cap_g, &sh_flag)) return;
  const int B = s.B, K = s.K;
  double bsum[MAX_B];
  for (int b = 0; b < B; ++b) bsum[b] = 0.0;
  if (valid) {
    const double p0 = s.p_tau0[0];
    const double log_rat_base = log(p0 / (1.0 - p0)) + (log((double)TAU0_INIT) - log(TAU1)) / 2.0;
    double raw0[MAX_K];
    double nusum0 = 0.0;
    for (int b = 0; b < B; ++b) {
      double rsum = 0.0;
      for (int k = 0; k < K; ++k) {
        double sumbk = 0.0;
        const int2 sc = s.seg_chunk[b * K + k];  // the segment's chunks, in chunk order
        for (int c = sc.x; c < sc.x + sc.y; ++c) {
          if (s.gchunk[c].w == 0) continue;
          sumbk += __ldcg(&s.part[(int64_t)c * NSLOT * Gp + g]);
        }
        const int n = s.seg_cnt[b * K + k];
        const double raw = n == 0 ? 0.0 : sumbk / n;
        bsum[b] += sumbk;
        rsum += raw;
        if (b == 0) raw0[k] = raw;
      }
      if (b == 0) {
        nusum0 = rsum;
        s.nu[g] = 0.0f;
      } else {
        s.nu[(int64_t)b * Gp + g] = (float)((rsum - nusum0) / K);
      }
    }
    s.alpha[g] = (float)raw0[0];
    s.mu_alpha[g] = (float)raw0[0];
    s.beta[g] = 0.0f;
    s.L[g] = 0;
    for (int k = 1; k < K; ++k) {
      const double bt = raw0[k] - raw0[0];
      s.beta[(int64_t)k * Gp + g] = (float)bt;
      const double lr = log_rat_base + bt * bt * (1.0 / TAU0_INIT - 1.0 / TAU1) / 2.0;
      const float u = uniform_at(s.seed, SID_INIT_L, (uint64_t)k * (uint64_t)s.G + (uint64_t)g, 0u, 0);
      s.L[(int64_t)k * Gp + g] = (double)u > 1.0 / (1.0 + exp(lr)) ? 1 : 0;
    }
  }
  // per-tile batch sums -> tpart[tile][b]
  const int lane = tid & 31, warp = tid >> 5;
  for (int b = 0; b < B; ++b) {
    const double v = warp_sum(bsum[b]);
    if (lane == 0) sh[warp * MAX_B + b] = v;
  }
  __syncthreads();
  if (tid < B) {
    double t = 0.0;
    for (int w = 0; w < GENE_TILE / 32; ++w) t += sh[w * MAX_B + tid];
    s.tpart[(int64_t)tile * MAX_B + tid] = t;
  }
  if (!arrive_last(&s.cnt_glob[3], (unsigned)s.n_tiles, &sh_flag)) return;
  if (tid < B) {
    double t = 0.0;
    for (int tt = 0; tt < s.n_tiles; ++tt) t += __ldcg(&s.tpart[(int64_t)tt * MAX_B + tid]);
    sh[tid] = t / ((double)(s.batch_off[tid + 1] - s.batch_off[tid]) * (double)s.G);
  }
  __syncthreads();
  if (tid < B) s.mu_nu[tid] = tid == 0 ? 0.0f : (float)(sh[tid] - sh[0]);
}

// Parameters that do not come from the data, and the derived tables.
// Padded genes get harmless values (beta = nu = 0, phi = 1, E = 1).
__global__ void k_init_finish(DevState s, int fresh) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t Gp = s.Gp, G = s.G;
  const int B = s.B, K = s.K;
  if (fresh) {
    if (t < B) { s.gamma[t] = GAMMA0_INIT; s.gamma[B + t] = GAMMA1_INIT; }
    if (t < (int64_t)B * K) s.pi[t] = (float)(((t % K) + 1) / (K * (K + 1) / 2.0));
    if (t < (int64_t)B * Gp) s.phi[t] = (t % Gp) < G ? PHI_INIT : 1.0f;
    if (t < s.N) s.mu_delta[t] = s.delta[t];
    if (t == 0) s.p_tau0[1] = TAU0_INIT;
  }
  if (t < s.N) s.Dexp[t] = expf(s.delta[t]);
  if (s.psi && t < (int64_t)B * Gp) s.psi[t] = logf(s.phi[t]);
  if (t < Gp && t >= G) {
    s.alpha[t] = 0.0f;
    for (int k = 0; k < K; ++k) s.beta[(int64_t)k * Gp + t] = 0.0f;
    for (int b = 0; b < B; ++b) {
      s.nu[(int64_t)b * Gp + t] = 0.0f;
      s.phi[(int64_t)b * Gp + t] = 1.0f;
    }
  }
  if (t < Gp) {
    const float a = t < G ? s.alpha[t] : 0.0f;
    for (int b = 0; b < B; ++b) {
      const float nv = s.nu[(int64_t)b * Gp + t];
      for (int k = 0; k < K; ++k)
        s.E[((int64_t)b * K + k) * Gp + t] = t < G ? exp_sum3(a, s.beta[(int64_t)k * Gp + t], nv) : 1.0f;
    }
  }
}

// ---------------------------------------------------------------------------
// Posterior summaries: means over kept sweeps, P(L = 1), W mode.
// est layout: gamma[2B] alpha[G] L[(K-1)G] beta[K G] ptau[2] nu[B G] delta[N] phi[B G] pi[B K]
// ---------------------------------------------------------------------------
// Static tables of the phi update: one thread per (batch, gene) walks the
// batch's cells in order.  fill = 0: counts of Y = 1 .. PHI_TAB-1 into phi_cnt
// and the number of larger values into n_big; fill = 1: the larger values
// into phi_big_y from phi_big_off, in cell order (so every sum over them has a
// fixed order).
// fill = 0: per (batch, gene), the counts of Y = 1 .. PHI_TAB - 1 (added
// into phi_cnt) and, per slice of the batch's cells, how many Y >= PHI_TAB
// there are (n_big[slice][batch * G + gene]); fill = 1: those larger Y in cell
// order, each slice from the offset `off` the host summed from the first
// pass.  One CTA per (tile of GENE_TILE genes, batch, slice of the cells), a
// thread per gene walking its slice; the first pass counts in shared memory
// (each thread its own column) and adds the table to phi_cnt once (integer
// additions: the order does not matter).
__global__ void __launch_bounds__(GENE_TILE) k_phi_hist(DevState s, int64_t* n_big, const int64_t* off, int fill) {
  __shared__ int sc[PHI_TAB][GENE_TILE];
  const int b = blockIdx.y, sl = blockIdx.z, tid = threadIdx.x;
  const int64_t g = (int64_t)blockIdx.x * GENE_TILE + tid, Gp = s.Gp;
  const bool live = g < s.G;
  const int64_t t = (int64_t)b * s.G + g, slot = (int64_t)sl * s.B * s.G + t;
  if (fill) {
    // only the slices that hold large values walk their cells again (a
    // warp-uniform exit: the first pass's counts are in n_big)
    if (!__any_sync(0xffffffffu, live && n_big[slot] > 0)) return;
  } else {
    for (int y = 0; y < PHI_TAB; ++y) sc[y][tid] = 0;
  }
  int64_t pos = fill && live ? off[slot] : 0;
  int64_t nb = 0;
  const int c0 = s.batch_off[b], nc = s.batch_off[b + 1] - c0;
  const int i0 = c0 + (int)((int64_t)nc * sl / PHI_HIST_SLICES);
  const int i1 = c0 + (int)((int64_t)nc * (sl + 1) / PHI_HIST_SLICES);
  if (live) {
#pragma unroll 8
    for (int i = i0; i < i1; ++i) {
      const int y = __ldg(s.Y + (int64_t)i * Gp + g);  // read-only: the loads may pass the stores below
      if (y >= PHI_TAB) {
        if (fill) s.phi_big_y[pos++] = y;
        ++nb;
      } else if (y > 0 && !fill) {
        ++sc[y][tid];
      }
    }
  }
  if (fill || !live) return;
  int32_t* cnt = s.phi_cnt + (int64_t)b * PHI_TAB * Gp + g;
  for (int y = 1; y < PHI_TAB; ++y)
    if (sc[y][tid]) atomicAdd(cnt + (int64_t)y * Gp, sc[y][tid]);
  n_big[slot] = nb;
}

// Posterior summaries of the imputation as dense [N][G] tables: E[X] and
// P(Z = 1), from Y where Y > 0 and from the kept-sweep sums at the Y == 0
// entries (one thread per entry of the dense table, then of the zero list).
__global__ void k_zx_summary(DevState s, int n_kept, float* x_mean, float* z_prob) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t NG = s.N * s.G;
  for (int64_t t = t0; t < NG; t += stride) {
    const int64_t i = t / s.G, g = t - i * s.G;
    if (x_mean) x_mean[t] = (float)s.Y[i * s.Gp + g];
    if (z_prob) z_prob[t] = 0.0f;
  }
}

__global__ void k_zx_summary_zeros(DevState s, int n_kept, float* x_mean, float* z_prob) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const double inv = 1.0 / (double)n_kept;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < s.nz0; e += stride) {
    const int2 ig = s.zij[e];
    const int64_t t = (int64_t)ig.x * s.G + ig.y;
    if (x_mean) x_mean[t] = (float)((double)s.acc_xs[e] * inv);
    if (z_prob) z_prob[t] = (float)((double)s.acc_zn[e] * inv);
  }
}

// Z as a dense [N][ld] table from the bit mask [N][Gw]: one thread per mask
// word, 32 outputs each (int32 for the estimates, uint8 for the state).
__global__ void k_z_dense_i32(DevState s, int32_t* out, int64_t ld) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < s.N * s.Gw; t += stride) {
    const int64_t i = t / s.Gw, w = t - i * s.Gw;
    const uint32_t m = s.zm[t];
    const int64_t g0 = w * 32;
    const int n = (int)(s.G - g0 < 32 ? s.G - g0 : 32);
    for (int j = 0; j < n; ++j) out[i * ld + g0 + j] = (int32_t)((m >> j) & 1u);
  }
}

__global__ void k_z_dense_u8(DevState s, uint8_t* out, int64_t ld) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < s.N * s.Gw; t += stride) {
    const int64_t i = t / s.Gw, w = t - i * s.Gw;
    const uint32_t m = s.zm[t];
    const int64_t g0 = w * 32;
    const int n = (int)(s.G - g0 < 32 ? s.G - g0 : 32);
    for (int j = 0; j < n; ++j) out[i * ld + g0 + j] = (uint8_t)((m >> j) & 1u);
  }
}

__global__ void k_finalize(DevState s, Estimates e, int n_kept) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t G = s.G, Gp = s.Gp, N = s.N;
  const int B = s.B, K = s.K;
  const bool have = n_kept > 0;
  const double inv = have ? 1.0 / n_kept : 0.0;
  for (int64_t t = t0; t < (int64_t)K * G; t += stride) {
    const int k = (int)(t / G);
    const int64_t g = t % G;
    if (k == 0) {
      e.alpha[g] = have ? s.acc_alpha[g] * inv : s.alpha[g];
      e.beta[g] = 0.0;
    } else {
      e.beta[t] = have ? s.acc_beta[t] * inv : s.beta[(int64_t)k * Gp + g];
      e.L[t - G] = have ? s.acc_L[t] * inv : s.L[(int64_t)k * Gp + g];
    }
  }
  for (int64_t t = t0; t < (int64_t)B * G; t += stride) {
    const int b = (int)(t / G);
    const int64_t g = t % G;
    e.phi[t] = have ? s.acc_phi[t] * inv : s.phi[(int64_t)b * Gp + g];
    e.nu[t] = b == 0 ? 0.0 : (have ? s.acc_nu[t] * inv : s.nu[(int64_t)b * Gp + g]);
  }
  for (int64_t i = t0; i < N; i += stride) {
    e.delta[i] = have ? s.acc_delta[i] * inv : s.delta[i];
    if (have) {
      int best = 0, bc = s.acc_wcnt[i * K];
      for (int k = 1; k < K; ++k) {
        const int c = s.acc_wcnt[i * K + k];
        if (c > bc) { bc = c; best = k; }
      }
      e.W[i] = best;
    } else {
      e.W[i] = s.W[i];
    }
  }
  for (int64_t t = t0; t < 2 * B; t += stride) e.gamma[t] = have ? s.acc_gamma[t] * inv : s.gamma[t];
  for (int64_t t = t0; t < (int64_t)B * K; t += stride) e.pi[t] = have ? s.acc_pi[t] * inv : s.pi[t];
  for (int64_t t = t0; t < 2; t += stride) e.ptau[t] = have ? s.acc_ptau[t] * inv : s.p_tau0[t];
}

// ---------------------------------------------------------------------------
// BIC.  Per cell i and type k: sum over genes of the dropout-marginal
// log-likelihood of Y (BUSseq_gpu.cu:967-1007), with the estimates, in double
// precision.  FP64 runs at a small fraction of the FP32 rate here, so the
// per-entry work is kept to one logarithm, log(mu + phi), by Tang's table
// method (bic_series.h), two products for mu and a few sums:
//   k_bic_tables  exp(beta) per (type, gene); exp(alpha + nu), phi, log phi
//                 and lgamma(phi) per (batch, gene); -softplus(g0 + g1 y) -
//                 lgamma(1 + y) per (batch, count)
//   k_bic_cell    one CTA per cell: mu = exp(alpha + nu) e^delta e^beta, the
//                 clamped log p and log(1 - p) (:977-986), the Y > 0 term and,
//                 for Y = 0, the reference's series over x = 0 .. floor(3 mu)-1
//                 (bic_zero_term: float-float recurrence, stopped once the
//                 rest is provably below 2^-60 of the sum)
// Without tables (the allocation-free entry point) each entry computes them.
// ---------------------------------------------------------------------------
__global__ void k_bic_tables(DevState s, Estimates e, BicTabs tb) {
  const int64_t G = s.G, KG = (int64_t)s.K * G, BG = (int64_t)s.B * G, BY = (int64_t)s.B * tb.ny;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < KG + BG + BY; t += stride) {
    if (t < KG) {
      tb.eb[t] = exp(e.beta[t]);
    } else if (t < KG + BG) {
      const int64_t u = t - KG, g = u % G;
      const double phi = e.phi[u];
      tb.bg[u] = BicGene{exp(e.alpha[g] + e.nu[u]), phi, log(phi), lgamma(phi)};
    } else {
      const int64_t u = t - KG - BG;
      const int b = (int)(u / tb.ny), y = (int)(u % tb.ny);
      const double tt = e.gamma[b] + e.gamma[s.B + b] * y;
      const double sp = tt > 0 ? tt + log1p(exp(-tt)) : log1p(exp(tt));
      tb.ty[u] = -sp - lgamma(1.0 + y);
    }
  }
}

// Shared memory of k_bic_cell beyond its static arrays: K running sums per
// thread, then per job slot (K per thread) mu, phi, the result, the sorted
// order and the length class.
size_t bic_cell_smem(int K, int bd) {
  const size_t slots = (size_t)K * bd;
  return slots * sizeof(double) + slots * (3 * sizeof(double) + sizeof(uint16_t) + sizeof(uint8_t));
}

// One CTA per cell, the genes in passes of blockDim.x (one gene per thread,
// all K types).  A pass first forms every term but the zero counts' series
// (those entries add NB(0) and queue a job of mu and phi), then sorts the
// pass's jobs by series length class (floor(log2 floor(3 mu)), longest
// first) and hands them out in that order, so a warp's lanes run series of
// similar length instead of waiting on one gene's long series; each result
// returns to its job's slot and the owning thread adds its jobs in type order,
// so the sums do not depend on the order the jobs ran in.
__global__ void __launch_bounds__(256) k_bic_cell(DevState s, Estimates e, double* ll_ik, BicTabs tb) {
  extern __shared__ double s_acc[];  // [K][blockDim.x] running sums, then the job arrays
  __shared__ double s_log[2 * BIC_LOG_TAB];
  __shared__ int s_ccnt[BIC_CLASSES], s_cfill[BIC_CLASSES], s_njobs;
  const int64_t i = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, bd = blockDim.x;
  const int b = s.batch_of[i];
  const int B = s.B, K = s.K;
  const int64_t G = s.G, Gp = s.Gp;
  const int slots = K * bd;
  double* s_mu = s_acc + slots;
  double* s_ph = s_mu + slots;
  double* s_res = s_ph + slots;
  uint16_t* s_perm = reinterpret_cast<uint16_t*>(s_res + slots);
  uint8_t* s_cls = reinterpret_cast<uint8_t*>(s_perm + slots);
  for (int j = tid; j < BIC_LOG_TAB; j += bd) bic_log_entry(s_log, j);
  for (int k = 0; k < K; ++k) s_acc[k * bd + tid] = 0.0;
  if (tid < BIC_CLASSES) s_ccnt[tid] = 0;
  const BicCell cc = bic_cell(e.gamma[b], e.gamma[B + b]);
  const double g0 = cc.g0, g1 = cc.g1;
  const double di = e.delta[i], edi = exp(di);
  __syncthreads();
  for (int64_t gbase = 0; gbase < G; gbase += bd) {
    const int64_t g = gbase + tid;
    uint64_t jmask = 0;  // types whose series this thread queued, in its slots tid * K + 0, 1, ...
    if (g < G) {
      const int y = s.Y[i * Gp + g];
      const int64_t bgi = (int64_t)b * G + g;
      double phi, lphi, lgphi, ean;
      if (tb.bg) {
        const BicGene v = tb.bg[bgi];
        ean = v.ean * edi;  // exp(alpha + nu + delta)
        phi = v.phi;
        lphi = v.lphi;
        lgphi = v.lgphi;
      } else {
        phi = e.phi[bgi];
        lphi = log(phi);
        lgphi = lgamma(phi);
        ean = 0.0;
      }
      const double an = e.alpha[g] + e.nu[bgi] + di;
      double base = 0.0;
      if (y) {
        if (tb.ty && y < tb.ny) {
          base = tb.ty[(int64_t)b * tb.ny + y] + lgamma(phi + y) - lgphi;
        } else {
          const double t = g0 + g1 * y;
          const double sp = t > 0 ? t + log1p(exp(-t)) : log1p(exp(t));
          base = -sp + lgamma(phi + y) - lgamma(1.0 + y) - lgphi;
        }
      }
      int nj = 0;
      for (int k = 0; k < K; ++k) {
        const double eta = an + e.beta[(int64_t)k * G + g];
        const double mu = tb.eb ? ean * tb.eb[(int64_t)k * G + g] : exp(eta);
        const double lq = bic_log(s_log, mu + phi);
        double logp = eta - lq, log1mp = lphi - lq;
        if (logp < -250.0) logp = -250.0;
        if (log1mp < -250.0) log1mp = -250.0;
        double v;
        if (y) {
          v = base + y * logp + phi * log1mp;
        } else {
          v = phi * log1mp;  // log NB(0)
          const double xm = 3.0 * mu;
          const int x_max = xm > (double)BIC_SERIES_MAX_TERMS ? BIC_SERIES_MAX_TERMS : (int)xm;
          if (x_max > 1) {
            if (cc.ff && phi <= 1.0e6) {
              const int slot = tid * K + nj++;
              s_mu[slot] = mu;
              s_ph[slot] = phi;
              const int cls = BIC_CLASSES - 1 - (31 - __clz(x_max));  // longest first
              s_cls[slot] = (uint8_t)cls;
              atomicAdd(&s_ccnt[cls], 1);
              jmask |= 1ull << k;
            } else {
              v = bic_zero_series(mu, logp, log1mp, phi, g0, g1);
            }
          }
        }
        s_acc[k * bd + tid] += v;
      }
    }
    __syncthreads();
    if (warp == 0) {  // class offsets; the counts are cleared for the next pass
      const int c0 = lane < BIC_CLASSES ? s_ccnt[lane] : 0;
      int incl = c0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane < BIC_CLASSES) {
        s_cfill[lane] = incl - c0;
        s_ccnt[lane] = 0;
      }
      if (lane == 31) s_njobs = incl;
    }
    __syncthreads();
    {
      int m = 0;
      for (uint64_t jm = jmask; jm; jm &= jm - 1, ++m) {
        const int slot = tid * K + m;
        s_perm[atomicAdd(&s_cfill[s_cls[slot]], 1)] = (uint16_t)slot;
      }
    }
    __syncthreads();
    const int nj_all = s_njobs;
    for (int j = tid; j < nj_all; j += bd) {
      const int slot = s_perm[j];
      s_res[slot] = bic_zero_close(cc, s_log, s_mu[slot], s_ph[slot]);
    }
    __syncthreads();
    {
      int m = 0;
      for (uint64_t jm = jmask; jm; jm &= jm - 1, ++m) {
        const int k = __ffsll((long long)jm) - 1;
        s_acc[k * bd + tid] += s_res[tid * K + m];
      }
    }
  }
  __syncthreads();
  // per type, a fixed-order sum over the CTA's threads
  for (int k = warp; k < K; k += bd >> 5) {
    double v = 0.0;
    for (int t = lane; t < bd; t += 32) v += s_acc[k * bd + t];
    v = warp_sum(v);
    if (lane == 0) ll_ik[(int64_t)k * s.N + i] = v;
  }
}

__global__ void k_bic_total(DevState s, Estimates e, const double* ll_ik, double* out) {
  __shared__ double sh[32];
  const int K = s.K;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < s.N; i += blockDim.x) {
    const int b = s.batch_of[i];
    double mx = ll_ik[i];
    for (int k = 1; k < K; ++k) mx = fmax(mx, ll_ik[(int64_t)k * s.N + i]);
    double sum = 0.0;
    for (int k = 0; k < K; ++k) sum += e.pi[b * K + k] * exp(ll_ik[(int64_t)k * s.N + i] - mx);
    acc += mx + log(sum);
  }
  double v[1] = {acc};
  block_sum<1>(v, sh);
  if (threadIdx.x == 0) {
    const double B = s.B, G = (double)s.G, N = (double)s.N;
    const double nparam = (B + G) * K + 2 * B + G * (B * 2 - 1) + N - B;
    out[0] = -2.0 * v[0] + log(G * N) * nparam;
    out[1] = v[0];
  }
}

int bic_table_counts(const DevState& s) { return s.ymax + 1 < (1 << 16) ? s.ymax + 1 : (1 << 16); }

int64_t bic_table_bytes(const DevState& s, int ny) {
  return ((int64_t)s.K * s.G + (int64_t)s.B * ny) * (int64_t)sizeof(double) +
         (int64_t)s.B * s.G * (int64_t)sizeof(BicGene);
}

// threads of a k_bic_cell CTA: at most 2048 job slots (K per thread), a
// multiple of 32
int bic_cell_threads(int K) {
  const int bd = (2048 / K) & ~31;
  return bd < 32 ? 32 : (bd > 256 ? 256 : bd);
}

void launch_bic(const DevState& s, const Estimates& e, double* ll_ik, const BicTabs& tb, double* out,
                cudaStream_t st) {
  const int64_t n_tab = tb.eb ? (int64_t)s.K * s.G + (int64_t)s.B * s.G + (int64_t)s.B * tb.ny : 0;
  if (n_tab > 0) {
    const int64_t nb = (n_tab + 255) / 256;
    k_bic_tables<<<(unsigned)(nb < 152 * 16 ? nb : 152 * 16), 256, 0, st>>>(s, e, tb);
  }
  const int bd = bic_cell_threads(s.K);
  // every K's shape stays within 2048 job slots; the limit is raised to that
  // size on calls made outside stream capture (the allocation-free entry point
  // makes its first call on a device outside capture), so it holds for any K
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone)
    cudaFuncSetAttribute(k_bic_cell, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bic_cell_smem(1, 2048));
  k_bic_cell<<<(unsigned)s.N, bd, bic_cell_smem(s.K, bd), st>>>(s, e, ll_ik, tb);
  k_bic_total<<<1, 1024, 0, st>>>(s, e, ll_ik, out);
}

}  // namespace bq
