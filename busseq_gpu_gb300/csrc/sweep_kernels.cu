// The per-sweep kernels of the BUSseq Gibbs sampler.
//
// One sweep is seven launches (captured in a CUDA graph by the host):
//   k_propose     all random-walk / Gamma proposals of the sweep
//   k_zx_alpha    Z/X update (BUSseq_gpu.cu:484-512) fused with the gamma
//                 sufficient statistics (:514-600) and the alpha sums
//                 (:602-632); the last CTA of each gene tile decides alpha and
//                 redraws L (:634-648); the very last CTA decides gamma0,
//                 gamma1 and draws p, tau0 (:650-668)
//   k_beta_nu     beta sums (:670-707) and, speculatively on both outcomes of
//                 beta, the nu sums (:709-737); tile tails decide both
//   k_delta       per-cell delta update (:739-778), decided in the CTA
//   k_phi         phi sums (:780-818); tile tails decide
//   k_w_mh / k_w_gibbs  per-cell W update (:820-854), decided in the CTA
//   k_sort_pi     pi Dirichlet draw (:856-890) and the (batch, type) cell order
//
// Gene passes: a CTA owns GENE_TILE consecutive genes (one per thread) and one
// chunk of <= CG cells that share batch b and type k, so every per-gene
// parameter of the chunk lives in registers and X is read as one coalesced
// 512-byte row segment per cell.  Sums are accumulated in float over at most
// 32 cells, then in double; per-chunk partials are reduced in a fixed order by
// the last CTA of the tile, so the sweep is bit-reproducible.
#include "kernels_common.cuh"

namespace bq {

// ---------------------------------------------------------------------------
// Proposals (all families of one sweep; `mask` selects families)
// ---------------------------------------------------------------------------
__global__ void k_propose(DevState s, int mask) {
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t G = s.G, Gp = s.Gp;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // [0,B) gamma | [.., +G) alpha | (K-1)G beta | (B-1)G nu | N delta | B G phi
  if (t < s.B) {
    if (mask & PROP_GAMMA) {
      const int b = (int)t;
      Stream st(s.seed, SID_GAMMA, (uint64_t)b, iter);
      const float z = normal(st);
      s.gamma_p[b] = __fmaf_rn(RW_STEP, z, s.gamma[b]);
      Stream sg(s.seed, SID_GAMMA1_PROP, (uint64_t)b, iter);
      int err = 0;
      const float g1 = s.gamma[s.B + b];
      float gn = -(gamma_mt(sg, -10.0f * g1, &err) * 0.1f);
      if (!(gn < 0.0f)) gn = -1.0e-30f;  // a Gamma draw that underflowed to 0
      s.gamma_p[s.B + b] = gn;
      if (err) atomicOr(s.err, err);
    }
    return;
  }
  t -= s.B;
  if (t < G) {
    if (mask & PROP_ALPHA) {
      Stream st(s.seed, SID_ALPHA, (uint64_t)t, iter);
      s.alpha_p[t] = __fmaf_rn(RW_STEP, normal(st), s.alpha[t]);
    }
    return;
  }
  t -= G;
  if (t < (int64_t)(s.K - 1) * G) {
    if (mask & PROP_BETA) {
      const int k = 1 + (int)(t / G);
      const int64_t g = t % G;
      Stream st(s.seed, SID_BETA, (uint64_t)t, iter);
      s.beta_p[k * Gp + g] = __fmaf_rn(RW_STEP, normal(st), s.beta[k * Gp + g]);
    }
    return;
  }
  t -= (int64_t)(s.K - 1) * G;
  if (t < (int64_t)(s.B - 1) * G) {
    if (mask & PROP_NU) {
      const int b = 1 + (int)(t / G);
      const int64_t g = t % G;
      Stream st(s.seed, SID_NU, (uint64_t)t, iter);
      s.nu_p[b * Gp + g] = __fmaf_rn(RW_STEP, normal(st), s.nu[b * Gp + g]);
    }
    return;
  }
  t -= (int64_t)(s.B - 1) * G;
  if (t < s.N) {
    if (mask & PROP_DELTA) {
      Stream st(s.seed, SID_DELTA, (uint64_t)t, iter);
      s.delta_p[t] = __fmaf_rn(RW_STEP, normal(st), s.delta[t]);
    }
    return;
  }
  t -= s.N;
  if (t < (int64_t)s.B * G) {
    if (mask & PROP_PHI) {
      const int b = (int)(t / G);
      const int64_t g = t % G;
      Stream st(s.seed, SID_PHI_PROP, (uint64_t)t, iter);
      int err = 0;
      float pn = gamma_mt(st, s.phi[b * Gp + g], &err);
      if (!(pn > 0.0f)) pn = 1.0e-30f;
      s.phi_p[b * Gp + g] = pn;
      if (err) atomicOr(s.err, err);
    }
  }
}

int64_t propose_count(const DevState& s) {
  return (int64_t)s.B + s.G + (int64_t)(s.K - 1) * s.G + (int64_t)(s.B - 1) * s.G + s.N + (int64_t)s.B * s.G;
}

// ---------------------------------------------------------------------------
// Z/X update of one entry with Y == 0 (BUSseq_gpu.cu:484-512).
// x (current X) is replaced by the new X; z receives the new Z.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void zx_entry(uint64_t seed, uint64_t ent, uint32_t iter, float mu, float phi, float g0,
                                         float g1, int& x, int& z, int* errp) {
  Stream st(seed, SID_ZX, ent, iter);
  if (x == 0) {
    const float u = st.uniform();
    z = u > 1.0f / (1.0f + expf(g0));
  } else {
    z = 1;
  }
  if (z) {
    int err = 0;
    const int xn = negbin(st, mu, phi, &err);
    const float u = st.uniform();
    // log[(1 + e^{-g0 - g1 x_old}) / (1 + e^{-g0 - g1 x_new})]
    const float lr = softplusf(-g0 - g1 * (float)x) - softplusf(-g0 - g1 * (float)xn);
    if (logf(u) <= lr) x = xn;
    if (err) atomicOr(errp, err);
  } else {
    x = 0;
  }
}

// Static part of the gamma statistics: entries with Y > 0 keep X = Y and
// Z = 0, so their terms only depend on the histogram of Y per batch.
__device__ void gamma_static_cta(const DevState& s, int sidx, double* sh) {
  const int slices = (s.ymax + GENE_TILE - 1) / GENE_TILE;
  double v[3] = {0.0, 0.0, 0.0};
  int b = -1;
  if (sidx < s.n_static) {
    b = sidx / slices;
    const int y = (sidx % slices) * GENE_TILE + (int)threadIdx.x + 1;
    if (y <= s.ymax) {
      const int cnt = s.yhist[(int64_t)b * (s.ymax + 1) + y];
      if (cnt) {
        const float g0 = s.gamma[b], g1 = s.gamma[s.B + b];
        const float g0p = s.gamma_p[b], g1p = s.gamma_p[s.B + b];
        const float yf = (float)y;
        const float t = fmaf(g1, yf, g0);
        const float d1 = (g1p - g1) * yf;
        v[0] = (double)cnt * (double)softplus_diff(t, g0p - g0);
        v[1] = (double)cnt * (double)softplus_diff(t, d1);
        v[2] = (double)cnt * (double)softplus_diff(fmaf(g1, yf, g0p), d1);
      }
    }
  }
  block_sum<3>(v, sh);
  if (threadIdx.x == 0 && sidx < s.n_static) {
    s.gstat[(int64_t)sidx * 4 + 0] = v[0];
    s.gstat[(int64_t)sidx * 4 + 1] = v[1];
    s.gstat[(int64_t)sidx * 4 + 2] = v[2];
    s.gstat[(int64_t)sidx * 4 + 3] = (double)b;
  }
}

// gamma0 / gamma1 decisions and the p, tau0 draw: run by the last CTA of
// k_zx_alpha, after every tile tail and every static CTA has finished.
__device__ void zx_global_tail(const DevState& s, uint32_t iter, double* sh) {
  const int tid = threadIdx.x;
  const int64_t nct = (int64_t)s.cap_g * s.n_tiles;
  // ---- p and tau0 (only once iter >= n_unchanged) -------------------------
  if ((int)iter >= s.n_unchanged) {
    double v[2] = {0.0, 0.0};
    for (int t = tid; t < s.n_tiles; t += blockDim.x) {
      v[0] += __ldcg(&s.tpart[2 * t]);
      v[1] += __ldcg(&s.tpart[2 * t + 1]);
    }
    block_sum<2>(v, sh);
    if (tid == 0) {
      const double cnt = v[0], bsq = v[1];
      const double tot = (double)s.G * (double)(s.K - 1);
      int err = 0;
      Stream sp(s.seed, SID_P, 0, iter);
      const float ga = gamma_mt(sp, (float)(cnt + A_P), &err);
      const float gb = gamma_mt(sp, (float)(tot - cnt + B_P), &err);
      s.p_tau0[0] = ga / (ga + gb);
      Stream stt(s.seed, SID_TAU0, 0, iter);
      const double shape = A_TAU0 + (tot - cnt) / 2.0;
      const double rate = B_TAU0 + bsq / 2.0;
      const float gt = gamma_mt(stt, (float)shape, &err);
      s.p_tau0[1] = (float)(1.0 / ((double)gt * (1.0 / rate)));
      if (err) atomicOr(s.err, err);
    }
  }
  // ---- gamma0 then gamma1, per batch --------------------------------------
  for (int b = 0; b < s.B; ++b) {
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t c = tid; c < nct; c += blockDim.x) {
      const int4 ch = s.gchunk[c / s.n_tiles];
      if (ch.w == 0 || ch.x != b) continue;
#pragma unroll
      for (int j = 0; j < 6; ++j) v[j] += __ldcg(&s.gpart[c * GSLOT + j]);
    }
    for (int c = tid; c < s.n_static; c += blockDim.x) {
      if ((int)__ldcg(&s.gstat[(int64_t)c * 4 + 3]) != b) continue;
      v[6] += __ldcg(&s.gstat[(int64_t)c * 4 + 0]);
      v[7] += __ldcg(&s.gstat[(int64_t)c * 4 + 1]);
      v[8] += __ldcg(&s.gstat[(int64_t)c * 4 + 2]);
    }
    block_sum<9>(v, sh);
    if (tid == 0) {
      const float g0 = s.gamma[b], g1 = s.gamma[s.B + b];
      const float g0p = s.gamma_p[b], g1p = s.gamma_p[s.B + b];
      const double nZ = v[0], XZ = v[1], n0 = v[2];
      const double c0 = (double)softplus_diff(g0, g0p - g0);
      const double lr0 = (double)(g0p - g0) * nZ - (v[3] + n0 * c0 + v[6]);
      const double prior0 = ((double)g0 * g0 - (double)g0p * g0p) / (2.0 * SIGMA2_GAMMA0);
      const float u0 = uniform_at(s.seed, SID_GAMMA, (uint64_t)b, iter, 2);
      const bool acc0 = (double)logf(u0) <= lr0 + prior0;
      s.lr_gamma[b] = lr0 + prior0;
      if (acc0) s.gamma[b] = g0p;
      const double lr1 = (double)(g1p - g1) * XZ - (acc0 ? (v[5] + v[8]) : (v[4] + v[7]));
      const double pv = -(double)g1, nv = -(double)g1p;
      const double prior1 = (KAPPA_GAMMA1 - 1.0) * (log(nv) - log(pv)) + TAU_GAMMA1 * (pv - nv) -
                            lgamma(10.0 * nv) + (10.0 * nv - 1.0) * log(pv) + 10.0 * nv * (log(10.0) + 1.0) +
                            lgamma(10.0 * pv) - (10.0 * pv - 1.0) * log(nv) - 10.0 * pv * (log(10.0) + 1.0);
      const float u1 = uniform_at(s.seed, SID_GAMMA, (uint64_t)b, iter, 3);
      s.lr_gamma[s.B + b] = lr1 + prior1;
      if ((double)logf(u1) <= lr1 + prior1) s.gamma[s.B + b] = g1p;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Pass 1: Z/X + gamma statistics + alpha sums; tails: alpha, L, gamma, p, tau0
//
// The CTA walks its chunk ZX_ROWS cells at a time.  Entries with Y == 0 (the
// only ones whose Z/X change) are first gathered into a shared-memory queue,
// so the expensive negative-binomial draws run on all lanes instead of on the
// scattered ~1/6 of lanes that hold a zero; the per-entry alpha terms then run
// densely over the whole tile.
// ---------------------------------------------------------------------------
constexpr int ZX_ROWS = 8;

// Copies the chunk's cell indices and exp(delta) into shared memory.
__device__ __forceinline__ void stage_chunk(const DevState& s, int start, int len, int* s_i, float* s_D) {
  for (int j = threadIdx.x; j < len; j += blockDim.x) {
    const int i = s.perm[start + j];
    s_i[j] = i;
    s_D[j] = s.Dexp[i];
  }
}

__global__ void __launch_bounds__(GENE_TILE) k_zx_alpha(DevState s) {
  __shared__ double sh[(GENE_TILE / 32) * 9];
  __shared__ int sh_flag;
  __shared__ int s_i[MAX_CG];
  __shared__ float s_D[MAX_CG];
  __shared__ int xs[ZX_ROWS][GENE_TILE];             // X of the current cells, updated in place
  __shared__ unsigned char zs[ZX_ROWS][GENE_TILE];   // bit 0: Z, bit 1: X changed
  __shared__ unsigned short q1[ZX_ROWS * GENE_TILE], q2[ZX_ROWS * GENE_TILE];
  __shared__ int q1n, q2n;
  __shared__ float sM[GENE_TILE], sPh[GENE_TILE];
  const int tid = threadIdx.x, lane = tid & 31;
  const uint32_t iter = (uint32_t)*s.iter;
  const int tile = blockIdx.x;
  const int row = blockIdx.y;
  const unsigned glob_total = (unsigned)s.n_tiles * (gridDim.y - (unsigned)s.cap_g) + (unsigned)s.n_tiles;

  if (row >= s.cap_g) {  // static gamma CTAs
    gamma_static_cta(s, (row - s.cap_g) * s.n_tiles + tile, sh);
    if (arrive_last(&s.cnt_glob[0], glob_total, &sh_flag)) zx_global_tail(s, iter, sh);
    return;
  }

  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp, Gw = s.Gw;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  const bool valid = g < s.G;

  if (len > 0) {
    const float M = valid ? s.E[((int64_t)b * s.K + k) * Gp + g] : 0.0f;
    const float ph = valid ? s.phi[(int64_t)b * Gp + g] : 1.0f;
    const float ca = valid ? expm1f(s.alpha_p[g] - s.alpha[g]) : 0.0f;
    sM[tid] = M;
    sPh[tid] = ph;
    stage_chunk(s, start, len, s_i, s_D);
    if (tid == 0) { q1n = 0; q2n = 0; }
    const float g0 = s.gamma[b], g1 = s.gamma[s.B + b];
    const float g0p = s.gamma_p[b], dg0 = g0p - g0, dg1 = s.gamma_p[s.B + b] - g1;
    const float zthr = 1.0f / (1.0f + expf(g0));
    const uint64_t G64 = (uint64_t)s.G;
    const uint64_t gbase = (uint64_t)tile * GENE_TILE;
    int64_t sx = 0, xz = 0;
    int nz = 0, n0 = 0;
    KahanF la, d0, d1a, d1b;
    __syncthreads();
    for (int j0 = 0; j0 < len; j0 += ZX_ROWS) {
      const int rn = min(ZX_ROWS, len - j0);
      // gather X and the Y == 0 bits of the group (independent loads first)
      int xr[ZX_ROWS];
      uint32_t mw[ZX_ROWS];
#pragma unroll
      for (int r = 0; r < ZX_ROWS; ++r) {
        xr[r] = 0;
        mw[r] = 0u;
        if (r < rn) {
          const int64_t i = s_i[j0 + r];
          if (valid) xr[r] = s.X[i * Gp + g];
          mw[r] = s.y0m[i * Gw + (g >> 5)];
        }
      }
#pragma unroll
      for (int r = 0; r < ZX_ROWS; ++r) {
        if (r < rn) {
          xs[r][tid] = xr[r];
          zs[r][tid] = 0;
          const bool y0 = valid && ((mw[r] >> lane) & 1u);
          const unsigned m = __ballot_sync(0xffffffffu, y0);
          if (m) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&q1n, __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (y0) q1[base + __popc(m & ((1u << lane) - 1u))] = (unsigned short)((r << 8) | tid);
          }
        }
      }
      __syncthreads();
      // Z for the Y == 0 entries; those with Z = 1 go on to the NB queue
      const int Q1 = q1n;
      for (int q = tid; q < Q1; q += GENE_TILE) {
        const int item = q1[q];
        const int r = item >> 8, t = item & 0xFF;
        int z = 1;
        if (xs[r][t] == 0) {
          const uint64_t ent = (uint64_t)s_i[j0 + r] * G64 + gbase + (uint64_t)t;
          z = uniform_at(s.seed, SID_ZX, ent, iter, 0) > zthr;
        }
        if (z) {
          q2[atomicAdd(&q2n, 1)] = (unsigned short)item;
        } else {
          ++n0;  // Z = 0 and X stays 0
        }
      }
      __syncthreads();
      // imputation X ~ NB independence MH for the entries with Z = 1 (BUSseq_gpu.cu:497-506)
      const int Q2 = q2n;
      float d0f = 0.0f, d1af = 0.0f, d1bf = 0.0f;
      for (int q = tid; q < Q2; q += GENE_TILE) {
        const int item = q2[q];
        const int r = item >> 8, t = item & 0xFF;
        const int xo = xs[r][t];
        const uint64_t ent = (uint64_t)s_i[j0 + r] * G64 + gbase + (uint64_t)t;
        Stream st(s.seed, SID_ZX, ent, iter);
        if (xo == 0) st.next_u32();  // the uniform of the Z draw
        int err = 0;
        const int xn = negbin(st, sM[t] * s_D[j0 + r], sPh[t], &err);
        const float u = st.uniform();
        const float lr = softplusf(-g0 - g1 * (float)xo) - softplusf(-g0 - g1 * (float)xn);
        const int x = logf(u) <= lr ? xn : xo;
        if (err) atomicOr(s.err, err);
        xs[r][t] = x;
        zs[r][t] = (unsigned char)(1 | (x != xo ? 2 : 0));
        ++nz;
        xz += x;
        if (x == 0) {
          ++n0;
        } else {
          const float xf = (float)x;
          const float tt = fmaf(g1, xf, g0);
          const float d1 = dg1 * xf;
          d0f += softplus_diff(tt, dg0);
          d1af += softplus_diff(tt, d1);
          d1bf += softplus_diff(fmaf(g1, xf, g0p), d1);
        }
      }
      d0.add(d0f);
      d1a.add(d1af);
      d1b.add(d1bf);
      __syncthreads();
      // write back X and the Z bits; alpha terms over the whole tile
      float laf = 0.0f;
#pragma unroll
      for (int r = 0; r < ZX_ROWS; ++r) {
        if (r < rn) {
          const int64_t i = s_i[j0 + r];
          const int x = xs[r][tid];
          const int zz = zs[r][tid];
          const unsigned zb = __ballot_sync(0xffffffffu, zz & 1);
          if (lane == 0) s.zm[i * Gw + (g >> 5)] = zb;
          if (__any_sync(0xffffffffu, zz & 2) && valid) s.X[i * Gp + g] = x;
          if (valid) {
            const float mu = M * s_D[j0 + r];
            sx += x;
            laf += (ph + (float)x) * log1p_fast(ca * fast_div(mu, ph + mu));
          }
        }
      }
      la.add(laf);
      if (tid == 0) { q1n = 0; q2n = 0; }
      __syncthreads();
    }
    if (valid) {
      s.part[((int64_t)row * NSLOT + 0) * Gp + g] = (double)sx;
      s.part[((int64_t)row * NSLOT + 1) * Gp + g] = la.value();
    }
    double v[6] = {(double)nz, (double)xz, (double)n0, d0.value(), d1a.value(), d1b.value()};
    block_sum<6>(v, sh);
    if (tid == 0) {
      double* gp = s.gpart + ((int64_t)row * s.n_tiles + tile) * GSLOT;
#pragma unroll
      for (int j = 0; j < 6; ++j) gp[j] = v[j];
    }
  }

  if (!arrive_last(&s.cnt_tile[tile], (unsigned)s.cap_g, &sh_flag)) return;

  // ---- tile tail: alpha decision, then L (old beta, old p and tau0) -------
  double lv[2] = {0.0, 0.0};
  if (valid) {
    double Sx = 0.0, La = 0.0;
    for (int c = 0; c < s.cap_g; ++c) {
      if (s.gchunk[c].w == 0) continue;
      Sx += __ldcg(&s.part[((int64_t)c * NSLOT + 0) * Gp + g]);
      La += __ldcg(&s.part[((int64_t)c * NSLOT + 1) * Gp + g]);
    }
    const float a = s.alpha[g], ap = s.alpha_p[g];
    const double ma = s.mu_alpha[g];
    const double lr = (double)(ap - a) * Sx - La;
    const double prior = (((double)a - ma) * ((double)a - ma) - ((double)ap - ma) * ((double)ap - ma)) /
                         (2.0 * SIGMA2_ALPHA);
    const float ua = uniform_at(s.seed, SID_ALPHA, (uint64_t)g, iter, 2);
    s.lr_alpha[g] = lr + prior;
    if ((double)logf(ua) <= lr + prior) s.alpha[g] = ap;

    const float p = s.p_tau0[0], tau0 = s.p_tau0[1];
    const float base = logf(p) - logf(1.0f - p) - (logf((float)TAU1) - logf(tau0)) * 0.5f;
    const float qd = 1.0f / (2.0f * tau0) - 1.0f / (2.0f * (float)TAU1);
    for (int kk = 1; kk < s.K; ++kk) {
      const float bt = s.beta[(int64_t)kk * Gp + g];
      const float lo = base + bt * bt * qd;
      const float u = uniform_at(s.seed, SID_L, (uint64_t)(kk - 1) * (uint64_t)s.G + (uint64_t)g, iter, 0);
      const int Lk = u > 1.0f / (1.0f + expf(lo)) ? 1 : 0;
      s.L[(int64_t)kk * Gp + g] = (int8_t)Lk;
      lv[0] += Lk;
      if (!Lk) lv[1] += (double)bt * (double)bt;
    }
  }
  block_sum<2>(lv, sh);
  if (tid == 0) {
    s.tpart[2 * tile] = lv[0];
    s.tpart[2 * tile + 1] = lv[1];
  }
  if (arrive_last(&s.cnt_glob[0], glob_total, &sh_flag)) zx_global_tail(s, iter, sh);
}

// ---------------------------------------------------------------------------
// Pass 2: beta sums and nu sums under both beta outcomes; tails decide
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(GENE_TILE) k_beta_nu(DevState s) {
  __shared__ int sh_flag;
  __shared__ int s_i[MAX_CG];
  __shared__ float s_D[MAX_CG];
  const int tid = threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  const bool valid = g < s.G;
  const bool work = len > 0 && (k > 0 || b > 0);

  if (work) stage_chunk(s, start, len, s_i, s_D);
  __syncthreads();
  if (work && valid) {
    const float bt = s.beta[(int64_t)k * Gp + g];
    const float M = exp_sum3(s.alpha[g], bt, s.nu[(int64_t)b * Gp + g]);
    const float ph = s.phi[(int64_t)b * Gp + g];
    const float eb = k > 0 ? s.beta_p[(int64_t)k * Gp + g] - bt : 0.0f;
    const float cb = expm1f(eb), fb = expf(eb);
    const float en = b > 0 ? s.nu_p[(int64_t)b * Gp + g] - s.nu[(int64_t)b * Gp + g] : 0.0f;
    const float cn = expm1f(en);
    int64_t sx = 0;
    KahanF lb, ln0, ln1;
    for (int j0 = 0; j0 < len; j0 += 8) {
      int xr[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) xr[u] = j0 + u < len ? s.X[(int64_t)s_i[j0 + u] * Gp + g] : 0;
      float lbf = 0.0f, ln0f = 0.0f, ln1f = 0.0f;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (j0 + u < len) {
          const int x = xr[u];
          const float mu = M * s_D[j0 + u];
          const float w = ph + (float)x;
          const float p = fast_div(mu, ph + mu);
          sx += x;
          if (k > 0) lbf += w * log1p_fast(cb * p);
          if (b > 0) {
            ln0f += w * log1p_fast(cn * p);
            if (k > 0) {
              const float mu1 = mu * fb;
              ln1f += w * log1p_fast(cn * fast_div(mu1, ph + mu1));
            }
          }
        }
      }
      lb.add(lbf);
      ln0.add(ln0f);
      ln1.add(ln1f);
    }
    double* pr = s.part + (int64_t)row * NSLOT * Gp + g;
    pr[0] = (double)sx;
    pr[Gp] = lb.value();
    pr[2 * Gp] = ln0.value();
    pr[3 * Gp] = ln1.value();
  }

  if (!arrive_last(&s.cnt_tile[tile], (unsigned)s.cap_g, &sh_flag)) return;
  if (!valid) return;

  // ---- tile tail: beta (k >= 1), then nu (b >= 1) -------------------------
  const double tau0 = s.p_tau0[1];
  uint64_t accmask = 0;
  for (int kk = 1; kk < s.K; ++kk) {
    double Sx = 0.0, Lb = 0.0;
    for (int c = 0; c < s.cap_g; ++c) {
      const int4 cc = s.gchunk[c];
      if (cc.w == 0 || cc.y != kk) continue;
      const double* pr = s.part + (int64_t)c * NSLOT * Gp + g;
      Sx += __ldcg(pr);
      Lb += __ldcg(pr + Gp);
    }
    const int64_t pos = (int64_t)kk * Gp + g;
    const float bo = s.beta[pos], bn = s.beta_p[pos];
    const double var = s.L[pos] == 1 ? TAU1 : tau0;
    const double lr = (double)(bn - bo) * Sx - Lb;
    const double prior = ((double)bo * bo - (double)bn * bn) / (2.0 * var);
    const float u = uniform_at(s.seed, SID_BETA, (uint64_t)(kk - 1) * (uint64_t)s.G + (uint64_t)g, iter, 2);
    s.lr_beta[(int64_t)kk * s.G + g] = lr + prior;
    if ((double)logf(u) <= lr + prior) {
      s.beta[pos] = bn;
      accmask |= (1ull << kk);
    }
  }
  for (int bb = 1; bb < s.B; ++bb) {
    double Sx = 0.0, Ln = 0.0;
    for (int c = 0; c < s.cap_g; ++c) {
      const int4 cc = s.gchunk[c];
      if (cc.w == 0 || cc.x != bb) continue;
      const double* pr = s.part + (int64_t)c * NSLOT * Gp + g;
      Sx += __ldcg(pr);
      Ln += __ldcg(pr + ((cc.y > 0 && ((accmask >> cc.y) & 1ull)) ? 3 : 2) * Gp);
    }
    const int64_t pos = (int64_t)bb * Gp + g;
    const float vo = s.nu[pos], vn = s.nu_p[pos];
    const double mn = s.mu_nu[bb];
    const double lr = (double)(vn - vo) * Sx - Ln;
    const double prior = (((double)vo - mn) * ((double)vo - mn) - ((double)vn - mn) * ((double)vn - mn)) /
                         (2.0 * SIGMA2_NU);
    const float u = uniform_at(s.seed, SID_NU, (uint64_t)(bb - 1) * (uint64_t)s.G + (uint64_t)g, iter, 2);
    s.lr_nu[(int64_t)bb * s.G + g] = lr + prior;
    if ((double)logf(u) <= lr + prior) s.nu[pos] = vn;
  }
  // E = exp(alpha + beta + nu) for the new parameters of this gene
  const float a = s.alpha[g];
  for (int bb = 0; bb < s.B; ++bb) {
    const float nv = s.nu[(int64_t)bb * Gp + g];
    for (int kk = 0; kk < s.K; ++kk)
      s.E[((int64_t)bb * s.K + kk) * Gp + g] = exp_sum3(a, s.beta[(int64_t)kk * Gp + g], nv);
  }
}

// ---------------------------------------------------------------------------
// Pass 4: phi sums; tails decide phi per (batch, gene)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(GENE_TILE) k_phi(DevState s) {
  __shared__ float tab[PHI_TAB][GENE_TILE];
  __shared__ int sh_flag;
  __shared__ int s_i[MAX_CG];
  __shared__ float s_D[MAX_CG];
  const int tid = threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  const bool valid = g < s.G;

  if (len > 0) stage_chunk(s, start, len, s_i, s_D);
  __syncthreads();
  if (len > 0 && valid) {
    const float ph = s.phi[(int64_t)b * Gp + g];
    const float pp = s.phi_p[(int64_t)b * Gp + g];
    const float dl = pp - ph;
    const float M = s.E[((int64_t)b * s.K + k) * Gp + g];
    const float iph = 1.0f / ph;
    // Per entry (BUSseq_gpu.cu:799-802, regrouped so that no large terms cancel):
    //   t = [lgamma(pp+x) - lgamma(pp)] - [lgamma(ph+x) - lgamma(ph)]
    //       - (pp + x) log((pp + mu) / (ph + mu)) + pp log(pp / ph) - dl log(1 + mu / ph)
    const float lgd0 = lgamma_diff(ph, pp, dl);
    const float c1 = pp * log_ratio(pp, ph, dl);
    float h = 0.0f;
    tab[0][tid] = 0.0f;
    for (int x = 1; x < PHI_TAB; ++x) {
      const float j = (float)(x - 1);
      h += log_ratio(pp + j, ph + j, dl);
      tab[x][tid] = h;
    }
    KahanF acc;
    for (int j0 = 0; j0 < len; j0 += 8) {
      int xr[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) xr[u] = j0 + u < len ? s.X[(int64_t)s_i[j0 + u] * Gp + g] : 0;
      float f = 0.0f;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (j0 + u < len) {
          const int x = xr[u];
          const float mu = M * s_D[j0 + u];
          const float xf = (float)x;
          const float hx = (unsigned)x < (unsigned)PHI_TAB ? tab[x][tid] : lgamma_diff(ph + xf, pp + xf, dl) - lgd0;
          f += hx - (pp + xf) * log_ratio(pp + mu, ph + mu, dl) + c1 - dl * log1p_fast(mu * iph);
        }
      }
      acc.add(f);
    }
    s.part[(int64_t)row * NSLOT * Gp + g] = acc.value();
  }

  if (!arrive_last(&s.cnt_tile[tile], (unsigned)s.cap_g, &sh_flag)) return;
  if (!valid) return;

  for (int bb = 0; bb < s.B; ++bb) {
    double S = 0.0;
    for (int c = 0; c < s.cap_g; ++c) {
      const int4 cc = s.gchunk[c];
      if (cc.w == 0 || cc.x != bb) continue;
      S += __ldcg(s.part + (int64_t)c * NSLOT * Gp + g);
    }
    const int64_t pos = (int64_t)bb * Gp + g;
    const float ph = s.phi[pos], pp = s.phi_p[pos];
    const float dl = pp - ph;
    const double lgd0 = (double)lgamma_diff(ph, pp, dl);    // lgamma(pp) - lgamma(ph)
    const double l1 = (double)log_ratio(pp, ph, dl);        // log(pp / ph)
    const double lph = (double)logf(ph);
    // Gamma(1, rate 0.1) prior and Gamma(phi, 1) proposal (BUSseq_gpu.cu:811-814)
    const double prior = (1.0 - (double)ph) * l1 + (double)dl * lph + (1.0 - TAU_PHI) * (double)dl - lgd0;
    const float u = uniform_at(s.seed, SID_PHI_ACC, (uint64_t)bb * (uint64_t)s.G + (uint64_t)g, iter, 0);
    s.lr_phi[(int64_t)bb * s.G + g] = S + prior;
    if ((double)logf(u) <= S + prior) s.phi[pos] = pp;
  }
}

// ---------------------------------------------------------------------------
// Cell passes: one CTA per tile of <= CELL_TILE cells of one (batch, type)
// ---------------------------------------------------------------------------
// Sums over the CTA of CELL_TILE per-thread doubles; results in sh_out[r].
__device__ __forceinline__ void cell_reduce(double (&acc)[CELL_TILE], double* sh, double* sh_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) {
    const double v = warp_sum(acc[r]);
    if (lane == 0) sh[warp * CELL_TILE + r] = v;
  }
  __syncthreads();
  if (threadIdx.x < CELL_TILE) {
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += sh[w * CELL_TILE + threadIdx.x];
    sh_out[threadIdx.x] = t;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(CELL_THREADS) k_delta(DevState s) {
  __shared__ double sh[(CELL_THREADS / 32) * CELL_TILE];
  __shared__ double sh_l[CELL_TILE], sh_x[CELL_TILE];
  __shared__ int sh_i[CELL_TILE];
  __shared__ float sh_D[CELL_TILE], sh_c[CELL_TILE];
  const int4 t = s.ctile[blockIdx.x];
  const int b = t.x, k = t.y, start = t.z, len = t.w;
  if (len == 0) return;
  const int tid = threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp, G = s.G;
  if (tid < CELL_TILE) {
    const int i = s.perm[start + (tid < len ? tid : 0)];
    sh_i[tid] = i;
    sh_D[tid] = s.Dexp[i];
    sh_c[tid] = tid < len ? expm1f(s.delta_p[i] - s.delta[i]) : 0.0f;
  }
  __syncthreads();
  KahanF acc[CELL_TILE];
  int sxi[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) sxi[r] = 0;
  const float* Er = s.E + ((int64_t)b * s.K + k) * Gp;
  const float* Pr = s.phi + (int64_t)b * Gp;
  for (int64_t g4 = (int64_t)tid * 4; g4 < Gp; g4 += (int64_t)CELL_THREADS * 4) {
    const float4 e = *reinterpret_cast<const float4*>(Er + g4);
    const float4 ph = *reinterpret_cast<const float4*>(Pr + g4);
    const float ev[4] = {e.x, e.y, e.z, e.w}, pv[4] = {ph.x, ph.y, ph.z, ph.w};
#pragma unroll
    for (int r = 0; r < CELL_TILE; ++r) {
      if (r < len) {
        const int4 xv = *reinterpret_cast<const int4*>(s.X + (int64_t)sh_i[r] * Gp + g4);
        const int xs[4] = {xv.x, xv.y, xv.z, xv.w};
        float a = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (g4 + q < G) {
            const float mu = ev[q] * sh_D[r];
            a += (pv[q] + (float)xs[q]) * log1p_fast(sh_c[r] * fast_div(mu, pv[q] + mu));
            sxi[r] += xs[q];
          }
        }
        acc[r].add(a);
      }
    }
  }
  double al[CELL_TILE], ax[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) { al[r] = acc[r].value(); ax[r] = (double)sxi[r]; }
  cell_reduce(al, sh, sh_l);
  cell_reduce(ax, sh, sh_x);
  if (tid < len) {
    const int i = sh_i[tid];
    if (i != s.batch_off[b]) {  // the first cell of each batch keeps delta = 0
      const float d = s.delta[i], dp = s.delta_p[i];
      const double md = s.mu_delta[i];
      const double lr = (double)(dp - d) * sh_x[tid] - sh_l[tid];
      const double prior = (((double)d - md) * ((double)d - md) - ((double)dp - md) * ((double)dp - md)) /
                           (2.0 * SIGMA2_DELTA);
      const float u = uniform_at(s.seed, SID_DELTA, (uint64_t)i, iter, 2);
      s.lr_delta[i] = lr + prior;
      if ((double)logf(u) <= lr + prior) {
        s.delta[i] = dp;
        s.Dexp[i] = expf(dp);
      }
    }
  }
}

// Log-likelihood change of one entry when its type moves and beta changes by
// eps:  eps x - (phi + x) log[(phi + mu e^eps) / (phi + mu)].
__device__ __forceinline__ float type_shift_term(float eps, float mu, float ph, int x) {
  float lg;
  if (fabsf(eps) < 0.5f) lg = log1p_fast(expm1f(eps) * fast_div(mu, ph + mu));
  else lg = logf(ph + mu * expf(eps)) - logf(ph + mu);
  return eps * (float)x - (ph + (float)x) * lg;
}

// W by Metropolis-Hastings with a uniform proposal (the reference's move).
__global__ void __launch_bounds__(CELL_THREADS) k_w_mh(DevState s) {
  __shared__ double sh[(CELL_THREADS / 32) * CELL_TILE];
  __shared__ double sh_l[CELL_TILE];
  __shared__ int sh_i[CELL_TILE], sh_kp[CELL_TILE];
  __shared__ float sh_D[CELL_TILE], sh_u[CELL_TILE];
  const int4 t = s.ctile[blockIdx.x];
  const int b = t.x, k = t.y, start = t.z, len = t.w;
  if (len == 0) return;
  const int tid = threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp, G = s.G;
  if (tid < CELL_TILE) {
    const int i = s.perm[start + (tid < len ? tid : 0)];
    sh_i[tid] = i;
    sh_D[tid] = s.Dexp[i];
    Stream st(s.seed, SID_W, (uint64_t)i, iter);
    const uint32_t r0 = st.next_u32();
    sh_kp[tid] = tid < len ? (int)(((uint64_t)r0 * (uint64_t)s.K) >> 32) : k;
    sh_u[tid] = st.uniform();
  }
  __syncthreads();
  KahanF acc[CELL_TILE];
  const float* Er = s.E + ((int64_t)b * s.K + k) * Gp;
  const float* Pr = s.phi + (int64_t)b * Gp;
  const float* Bk = s.beta + (int64_t)k * Gp;
  for (int64_t g4 = (int64_t)tid * 4; g4 < Gp; g4 += (int64_t)CELL_THREADS * 4) {
    const float4 e = *reinterpret_cast<const float4*>(Er + g4);
    const float4 ph = *reinterpret_cast<const float4*>(Pr + g4);
    const float4 bk = *reinterpret_cast<const float4*>(Bk + g4);
    const float ev[4] = {e.x, e.y, e.z, e.w}, pv[4] = {ph.x, ph.y, ph.z, ph.w}, bv[4] = {bk.x, bk.y, bk.z, bk.w};
#pragma unroll
    for (int r = 0; r < CELL_TILE; ++r) {
      if (r < len && sh_kp[r] != k) {
        const float4 bp = *reinterpret_cast<const float4*>(s.beta + (int64_t)sh_kp[r] * Gp + g4);
        const int4 xv = *reinterpret_cast<const int4*>(s.X + (int64_t)sh_i[r] * Gp + g4);
        const float bpv[4] = {bp.x, bp.y, bp.z, bp.w};
        const int xs[4] = {xv.x, xv.y, xv.z, xv.w};
        float a = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (g4 + q < G) a += type_shift_term(bpv[q] - bv[q], ev[q] * sh_D[r], pv[q], xs[q]);
        acc[r].add(a);
      }
    }
  }
  double al[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) al[r] = acc[r].value();
  cell_reduce(al, sh, sh_l);
  if (tid < len) {
    const int i = sh_i[tid], kp = sh_kp[tid];
    const double rhs = (double)logf(s.pi[b * s.K + kp]) - (double)logf(s.pi[b * s.K + k]) + sh_l[tid];
    s.lr_W[i] = rhs;
    if ((double)logf(sh_u[tid]) <= rhs) s.W[i] = kp;
  }
}

// W by a K-way categorical draw from its full conditional (Gibbs).  Targets
// the same conditional as the reference's MH move.  One CTA handles the tile's
// cells two at a time and the types eight at a time.
constexpr int GIBBS_CELLS = 2;
constexpr int GIBBS_TYPES = 8;
__global__ void __launch_bounds__(CELL_THREADS) k_w_gibbs(DevState s) {
  __shared__ double sh_red[(CELL_THREADS / 32) * GIBBS_CELLS * GIBBS_TYPES];
  __shared__ double sh_lp[CELL_TILE][MAX_K];
  __shared__ int sh_i[CELL_TILE];
  __shared__ float sh_D[CELL_TILE];
  const int4 t = s.ctile[blockIdx.x];
  const int b = t.x, k = t.y, start = t.z, len = t.w;
  if (len == 0) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = CELL_THREADS / 32;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp, G = s.G;
  const int K = s.K;
  if (tid < CELL_TILE) {
    const int i = s.perm[start + (tid < len ? tid : 0)];
    sh_i[tid] = i;
    sh_D[tid] = s.Dexp[i];
  }
  __syncthreads();
  const float* Er = s.E + ((int64_t)b * K + k) * Gp;
  const float* Pr = s.phi + (int64_t)b * Gp;
  const float* Bk = s.beta + (int64_t)k * Gp;
  for (int r0 = 0; r0 < len; r0 += GIBBS_CELLS) {
    for (int k0 = 0; k0 < K; k0 += GIBBS_TYPES) {
      KahanF acc[GIBBS_CELLS][GIBBS_TYPES];
      for (int64_t g = tid; g < G; g += CELL_THREADS) {
        const float e = Er[g], ph = Pr[g], bk = Bk[g];
        float bt[GIBBS_TYPES];
#pragma unroll
        for (int kk = 0; kk < GIBBS_TYPES; ++kk) bt[kk] = (k0 + kk < K) ? s.beta[(int64_t)(k0 + kk) * Gp + g] : bk;
#pragma unroll
        for (int r = 0; r < GIBBS_CELLS; ++r) {
          if (r0 + r < len) {
            const int x = s.X[(int64_t)sh_i[r0 + r] * Gp + g];
            const float mu = e * sh_D[r0 + r];
#pragma unroll
            for (int kk = 0; kk < GIBBS_TYPES; ++kk)
              if (k0 + kk < K && k0 + kk != k) acc[r][kk].add(type_shift_term(bt[kk] - bk, mu, ph, x));
          }
        }
      }
#pragma unroll
      for (int r = 0; r < GIBBS_CELLS; ++r)
#pragma unroll
        for (int kk = 0; kk < GIBBS_TYPES; ++kk) {
          const double v = warp_sum(acc[r][kk].value());
          if (lane == 0) sh_red[(warp * GIBBS_CELLS + r) * GIBBS_TYPES + kk] = v;
        }
      __syncthreads();
      if (tid < GIBBS_CELLS * GIBBS_TYPES) {
        const int r = tid / GIBBS_TYPES, kk = tid % GIBBS_TYPES;
        double tsum = 0.0;
        for (int w = 0; w < nw; ++w) tsum += sh_red[(w * GIBBS_CELLS + r) * GIBBS_TYPES + kk];
        if (r0 + r < len && k0 + kk < K) sh_lp[r0 + r][k0 + kk] = tsum;
      }
      __syncthreads();
    }
  }
  if (tid < len) {
    const int i = sh_i[tid];
    double mx = -1e300;
    for (int kk = 0; kk < K; ++kk) {
      const double lp = sh_lp[tid][kk] + (double)logf(s.pi[b * K + kk]);
      sh_lp[tid][kk] = lp;
      mx = fmax(mx, lp);
    }
    double tot = 0.0;
    for (int kk = 0; kk < K; ++kk) tot += exp(sh_lp[tid][kk] - mx);
    const float u = uniform_at(s.seed, SID_W, (uint64_t)i, iter, 0);
    const double target = (double)u * tot;
    double cum = 0.0;
    int pick = K - 1;
    for (int kk = 0; kk < K; ++kk) {
      cum += exp(sh_lp[tid][kk] - mx);
      if (target < cum) { pick = kk; break; }
    }
    s.W[i] = pick;
    s.lr_W[i] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// pi (Dirichlet) and the (batch, type) cell order; one CTA per batch.
// do_pi = 0 at initialisation.  The last CTA advances the sweep index when
// `advance` is set.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_sort_pi(DevState s, int do_pi, int advance) {
  __shared__ int cnt[MAX_K], base[MAX_K], run[MAX_K], rtot[MAX_K], gb[MAX_K + 1], cb[MAX_K + 1];
  __shared__ int wcnt[32][MAX_K];
  __shared__ float gk[MAX_K];
  __shared__ int sh_flag;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int K = s.K;
  const uint32_t iter = (uint32_t)*s.iter;
  const int off = s.batch_off[b], nb = s.batch_off[b + 1] - off;
  if (tid < K) { cnt[tid] = 0; run[tid] = 0; }
  __syncthreads();
  for (int j = tid; j < nb; j += blockDim.x) atomicAdd(&cnt[s.W[off + j]], 1);
  __syncthreads();
  if (tid == 0) {
    int acc = 0, ga = 0, ca = 0;
    for (int kk = 0; kk < K; ++kk) {
      base[kk] = acc;
      gb[kk] = ga;
      cb[kk] = ca;
      acc += cnt[kk];
      ga += (cnt[kk] + s.CG - 1) / s.CG;
      ca += (cnt[kk] + CELL_TILE - 1) / CELL_TILE;
    }
    gb[K] = ga;
    cb[K] = ca;
  }
  if (tid < K) s.seg_cnt[b * K + tid] = cnt[tid];
  if (do_pi && tid < K) {
    Stream st(s.seed, SID_PI, (uint64_t)(b * K + tid), iter);
    int err = 0;
    gk[tid] = gamma_mt(st, (float)((double)cnt[tid] + XI_PI), &err);
    if (err) atomicOr(s.err, err);
  }
  __syncthreads();
  if (do_pi && tid == 0) {
    float tot = 0.0f;
    for (int kk = 0; kk < K; ++kk) tot += gk[kk];
    for (int kk = 0; kk < K; ++kk) s.pi[b * K + kk] = gk[kk] / tot;
  }
  // stable counting sort of the batch's cells by type
  for (int r0 = 0; r0 < nb; r0 += blockDim.x) {
    const int j = r0 + tid;
    const bool act = j < nb;
    const int kk = act ? s.W[off + j] : MAX_K + 1;
    const unsigned same = __match_any_sync(0xffffffffu, kk);
    const int rank = __popc(same & ((1u << lane) - 1u));
    for (int q = tid; q < 32 * MAX_K; q += blockDim.x) wcnt[q / MAX_K][q % MAX_K] = 0;
    __syncthreads();
    if (act && rank == 0) wcnt[warp][kk] = __popc(same);
    __syncthreads();
    if (tid < K) {  // exclusive prefix over warps, per type
      int acc = 0;
      for (int w = 0; w < 32; ++w) {
        const int c = wcnt[w][tid];
        wcnt[w][tid] = acc;
        acc += c;
      }
      rtot[tid] = acc;
    }
    __syncthreads();
    if (act) s.perm[off + base[kk] + run[kk] + wcnt[warp][kk] + rank] = off + j;
    __syncthreads();
    if (tid < K) run[tid] += rtot[tid];
    __syncthreads();
  }
  // work lists of this batch: gene-pass chunks (CG cells) and cell tiles
  int gofs = 0, cofs = 0;
  for (int bb = 0; bb < b; ++bb) {
    const int n = s.batch_off[bb + 1] - s.batch_off[bb];
    gofs += n / s.CG + K;
    cofs += n / CELL_TILE + K;
  }
  const int gcap = nb / s.CG + K, ccap = nb / CELL_TILE + K;
  for (int q = tid; q < gcap; q += blockDim.x) {
    int4 v = make_int4(b, 0, off, 0);
    if (q < gb[K]) {
      int kk = 0;
      while (q >= gb[kk + 1]) ++kk;
      // split the segment into equal-length chunks of at most CG cells
      const int n = cnt[kk], nc = (n + s.CG - 1) / s.CG, c = q - gb[kk];
      const int c0 = (int)((int64_t)c * n / nc), c1 = (int)((int64_t)(c + 1) * n / nc);
      v = make_int4(b, kk, off + base[kk] + c0, c1 - c0);
    }
    s.gchunk[gofs + q] = v;
  }
  for (int q = tid; q < ccap; q += blockDim.x) {
    int4 v = make_int4(b, 0, off, 0);
    if (q < cb[K]) {
      int kk = 0;
      while (q >= cb[kk + 1]) ++kk;
      const int n = cnt[kk], nc = (n + CELL_TILE - 1) / CELL_TILE, c = q - cb[kk];
      const int c0 = (int)((int64_t)c * n / nc), c1 = (int)((int64_t)(c + 1) * n / nc);
      v = make_int4(b, kk, off + base[kk] + c0, c1 - c0);
    }
    s.ctile[cofs + q] = v;
  }
  if (advance && arrive_last(&s.cnt_glob[1], (unsigned)s.B, &sh_flag) && tid == 0) *s.iter += 1;
}

// ---------------------------------------------------------------------------
// Posterior accumulation of one kept sweep (and optional draw storage).
// ---------------------------------------------------------------------------
__global__ void k_posterior(DevState s, int advance) {
  __shared__ int sh_flag;
  const int it = *s.iter;
  const int kept = it - s.n_burnin;
  const bool store = s.keep_draws && kept >= 0 && kept < s.n_kept;  // draw slot inside the run
  const int64_t G = s.G, Gp = s.Gp, N = s.N;
  const int B = s.B, K = s.K;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)K * G; t += stride) {
    const int k = (int)(t / G);
    const int64_t g = t % G;
    if (k == 0) {
      s.acc_alpha[g] += s.alpha[g];
      if (store) s.keep_alpha[(int64_t)kept * G + g] = s.alpha[g];
      continue;
    }
    const float bt = s.beta[(int64_t)k * Gp + g];
    const int8_t l = s.L[(int64_t)k * Gp + g];
    s.acc_beta[t] += bt;
    s.acc_L[t] += l;
    if (store) {
      s.keep_beta[(int64_t)kept * (K - 1) * G + t - G] = bt;
      s.keep_L[(int64_t)kept * (K - 1) * G + t - G] = l;
    }
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)B * G; t += stride) {
    const int b = (int)(t / G);
    const int64_t g = t % G;
    const float ph = s.phi[(int64_t)b * Gp + g];
    s.acc_phi[t] += ph;
    if (store) s.keep_phi[(int64_t)kept * B * G + t] = ph;
    if (b > 0) {
      const float nv = s.nu[(int64_t)b * Gp + g];
      s.acc_nu[t] += nv;
      if (store) s.keep_nu[(int64_t)kept * (B - 1) * G + t - G] = nv;
    }
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    s.acc_delta[i] += s.delta[i];
    s.acc_wcnt[i * K + s.W[i]] += 1;
    if (store) {
      s.keep_delta[(int64_t)kept * N + i] = s.delta[i];
      s.keep_W[(int64_t)kept * N + i] = (int16_t)s.W[i];
    }
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 2 * B + B * K + 2; t += stride) {
    if (t < 2 * B) {
      s.acc_gamma[t] += s.gamma[t];
      if (store) s.keep_gamma[(int64_t)kept * 2 * B + t] = s.gamma[t];
    } else if (t < 2 * B + B * K) {
      const int64_t q = t - 2 * B;
      s.acc_pi[q] += s.pi[q];
      if (store) s.keep_pi[(int64_t)kept * B * K + q] = s.pi[q];
    } else {
      const int64_t q = t - 2 * B - B * K;
      s.acc_ptau[q] += s.p_tau0[q];
      if (store) s.keep_ptau[(int64_t)kept * 2 + q] = s.p_tau0[q];
    }
  }
  if (advance && arrive_last(&s.cnt_glob[2], gridDim.x, &sh_flag) && threadIdx.x == 0) *s.iter += 1;
}

}  // namespace bq
