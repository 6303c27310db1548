// Gene-side kernels of a sweep: proposals, the Z/X imputation, and the
// per-gene Metropolis updates alpha, beta, nu, phi with their decisions.
//
//   k_propose       every random-walk / Gamma proposal of the sweep
//   k_zx            Z/X update (BUSseq_gpu.cu:484-512) over the static list of
//                   Y == 0 entries, warps taking work units of 512 entries,
//                   with the per-batch sufficient statistics of the gamma
//                   updates (:514-600); its first CTAs also evaluate the gamma
//                   terms of the Y > 0 entries from the histogram of Y
//   k_zx_gp         the NB proposals of k_zx drawn as Gamma-Poisson mixtures
//   k_alpha         alpha sums (:602-623)
//   k_decide_gamma  gamma0 / gamma1 decisions, one CTA per batch (a branch of
//                   the sweep's graph beside the alpha and beta passes)
//   k_decide_alpha  alpha decisions, L redraw (:634-648), p and tau0 (:650-668)
//                   in the last gene CTA
//   k_beta_nu       beta sums (:676-694) and the nu sums (:715-728) under both
//                   outcomes of the beta of the cell's type
//   k_decide_beta   beta decisions (:696-707)
//   k_decide_nu_E   nu decisions (:730-737) and the table E = exp(alpha+beta+nu)
//   k_phi_static    phi sums, the lgamma part of the entries with Y >= 64 (k_propose
//                   sums that of the smaller Y > 0 with the lgamma table)
//   k_phi           phi sums (:789-804), the rest
//   k_decide_phi    phi decisions (:806-818)
//
// Gene passes: a CTA owns GENE_TILE consecutive genes (one per thread) and one
// chunk of <= CG cells that share batch b and type k (the cell order is
// rebuilt after every W update), so every per-gene parameter of the chunk
// lives in registers and X is read as coalesced 512-byte row segments.  The
// chunk's cell indices and exp(delta) are staged in shared memory and eight
// rows are loaded at a time.  Per-chunk partial sums (Kahan-compensated float
// per thread, then double) go to `part`; the decision kernels reduce them in a
// fixed order, so a sweep is bit-reproducible.
#include "kernels_common.cuh"

namespace bq {

// ---------------------------------------------------------------------------
// Proposals (all families of one sweep; `mask` selects families)
// ---------------------------------------------------------------------------
// t0: the first proposal of the launch (a launch of the phi proposals alone
// starts at propose_phi_offset).
__global__ void k_propose(DevState s, int mask, int64_t t0) {
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t G = s.G, Gp = s.Gp;
  int64_t t = t0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
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
      // the reference's step; with the per-gene HMC decisions, 2.4 conditional
      // standard deviations from the cell's adapted observed information (the
      // optimal scale of a one-dimensional random walk)
      const float step = s.hmc_gene ? 2.4f / sqrtf(s.hmc_fis[s.hmc_D - s.N + t] + (float)(1.0 / SIGMA2_DELTA))
                                    : RW_STEP;
      s.delta_p[t] = __fmaf_rn(step, normal(st), s.delta[t]);
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
      const float ph = s.phi[b * Gp + g];
      float pn = gamma_mt(st, ph, &err);
      if (!(pn > 0.0f)) pn = 1.0e-30f;
      s.phi_p[b * Gp + g] = pn;
      if (err) atomicOr(s.err, err);
      // lgamma differences of the phi update: h(x) = sum_{j<x} log((pn + j) / (ph + j))
      // for x < PHI_TAB, and lgamma(pn) - lgamma(ph)
      const float dl = pn - ph;
      float* tab = s.phi_tab + (int64_t)b * PHI_TAB * Gp + g;
      // with the static counts of Y = x (entries with Y > 0), their share of the
      // phi sum below the table's end; k_phi_static adds the larger Y
      const int32_t* cnt = s.phi_cnt ? s.phi_cnt + (int64_t)b * PHI_TAB * Gp + g : nullptr;
      KahanF stat;
      float h = 0.0f;
      tab[0] = 0.0f;
      for (int x0 = 0; x0 < PHI_TAB; x0 += 16) {
        int c[16];  // the block's counts, loaded ahead of the serial sum
#pragma unroll
        for (int u = 0; u < 16; ++u) c[u] = (cnt && x0 + u > 0) ? __ldg(cnt + (int64_t)(x0 + u) * Gp) : 0;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int x = x0 + u;
          if (x == 0) continue;
          const float j = (float)(x - 1);
          h += log_ratio(pn + j, ph + j, dl);
          tab[(int64_t)x * Gp] = h;
          if (c[u]) stat.add((float)c[u] * h);
        }
      }
      if (cnt) s.phi_static[b * Gp + g] = stat.value();
      s.phi_lgd0[b * Gp + g] = lgamma_diff(ph, pn, dl);
    }
    return;
  }
  t -= (int64_t)s.B * G;
  if (t < (int64_t)s.B * ZX_HIST) {
    // The Z/X update's table for count x of batch b: softplus(-g0 - g1 x) (its
    // MH ratio) and the three gamma terms of the sweep's proposals
    // (BUSseq_gpu.cu:524-576).  The proposals are drawn again from their own
    // streams, exactly as the batch's thread above draws them.
    if (mask & PROP_GAMMA) {
      const int b = (int)(t / ZX_HIST), x = (int)(t % ZX_HIST);
      Stream st(s.seed, SID_GAMMA, (uint64_t)b, iter);
      const float g0 = s.gamma[b], g1 = s.gamma[s.B + b];
      const float g0p = __fmaf_rn(RW_STEP, normal(st), g0);
      Stream sg(s.seed, SID_GAMMA1_PROP, (uint64_t)b, iter);
      int err = 0;
      float g1p = -(gamma_mt(sg, -10.0f * g1, &err) * 0.1f);
      if (!(g1p < 0.0f)) g1p = -1.0e-30f;
      const float xf = (float)x;
      const float tt = fmaf(g1, xf, g0), d1 = (g1p - g1) * xf;
      s.zx_gtab[(int64_t)b * ZX_HIST + x] =
          make_float4(softplusf(-g0 - g1 * xf), softplus_diff(tt, g0p - g0), softplus_diff(tt, d1),
                      softplus_diff(fmaf(g1, xf, g0p), d1));
    }
  }
}

int64_t propose_phi_offset(const DevState& s) {
  return (int64_t)s.B + s.G + (int64_t)(s.K - 1) * s.G + (int64_t)(s.B - 1) * s.G + s.N;
}

int64_t propose_count(const DevState& s) {
  return (int64_t)s.B + s.G + (int64_t)(s.K - 1) * s.G + (int64_t)(s.B - 1) * s.G + s.N + (int64_t)s.B * s.G +
         (int64_t)s.B * ZX_HIST;
}

// ---------------------------------------------------------------------------
// Z / X of the entries with Y == 0 (BUSseq_gpu.cu:484-512)
// ---------------------------------------------------------------------------
// Static part of the gamma statistics: entries with Y > 0 keep X = Y and
// Z = 0, so their terms only depend on the histogram of Y per batch.
__device__ void gamma_static_cta(const DevState& s, int sidx, double* sh) {
  const int slices = (s.ymax + ZX_THREADS - 1) / ZX_THREADS;
  double v[3] = {0.0, 0.0, 0.0};
  int b = -1;
  if (sidx < s.n_static) {
    b = sidx / slices;
    const int y = (sidx % slices) * ZX_THREADS + (int)threadIdx.x + 1;
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

// The three gamma-statistic terms of one entry with X = x > 0 (BUSseq_gpu.cu:
// 514-600): softplus(t + dg0) - softplus(t), softplus(t + d1) - softplus(t)
// and softplus(tp + d1) - softplus(tp), t = g0 + g1 x, tp = g0' + g1 x,
// d1 = (g1' - g1) x.
struct GammaTerms {
  float g0, g1, g0p, dg0, dg1;
  __device__ __forceinline__ void add(int x, float w, float& d0, float& d1a, float& d1b) const {
    const float xf = (float)x;
    const float tt = fmaf(g1, xf, g0);
    const float d1 = dg1 * xf;
    d0 = fmaf(w, softplus_diff(tt, dg0), d0);
    d1a = fmaf(w, softplus_diff(tt, d1), d1a);
    d1b = fmaf(w, softplus_diff(fmaf(g1, xf, g0p), d1), d1b);
  }
};

// Work units: runs of <= ZX_UNIT list entries of one batch (built at
// initialisation).  The launch holds ZX_CTAS_PER_SM CTAs on every SM; each
// warp takes units from a counter until none are left, so no warp ever waits
// for another (a unit rich in slow draws only delays its own warp, which then
// takes fewer units).  The first n_static CTAs first evaluate the static gamma
// terms of the Y > 0 entries.  The counter resets itself: the last warp to
// finish zeroes it for the next launch.
//
// A unit is read in parts of 128 entries (4 per lane):
// Phase 1 (all lanes busy): the entry's loads, block 0 of its Philox stream
// (an entry with X = 0 reads its Z uniform there, and every NB proposal starts
// there) and the Z draw.  An entry that needs an NB proposal by inversion of
// the distribution function is staged in the warp's queue with the two words
// it will use and a cost class, 0..30 by the expected length of the search,
// mu (-log(1 - u)) with u the inversion's uniform, longest first.  An entry
// that needs a Gamma-Poisson draw is listed for k_zx_gp with its cell, gene,
// X, mu and phi.
// Phase 2: a counting sort over (class, rank) - counts from ballots and match
// masks, so the order is deterministic - lays the queue out in class order.
// Phase 3: the lanes take the sorted queue 32 entries at a time, so lanes of
// one warp run searches of similar length.  Only full rounds of 32 run before
// the unit's last part: the shortest searches wait for the next part, so a
// round leaves lanes idle only at the end of a unit.  Each entry's draws come
// from its own stream, so neither the order nor the round changes them.  The
// gamma statistics of the drawn values are summed per lane (counts below
// ZX_HIST read their terms from the per-batch table that k_propose built; the
// MH ratio reads softplus(-g0 - g1 x) there too) and reduced over the warp
// into the unit's partial, in a fixed order.
constexpr int ZX_WARPS = ZX_THREADS / 32;
constexpr int ZX_PART = 128;
constexpr int ZX_PER_LANE = ZX_PART / 32;
constexpr int ZX_NCLS = 32;
constexpr int ZX_Q = ZX_PART + 32;  // fewer than 32 entries carried over plus one part
static_assert(ZX_UNIT % ZX_PART == 0 && ZX_UNIT <= 65536 && ZX_NCLS == 32 && ZX_Q <= 256,
              "unit and queue layout");

__device__ __forceinline__ int zx_class(float mu, float u_nb) {
  // a sort key only (the draws do not depend on it): the hardware logarithm
  const float key = mu * -__log2f(1.0f - u_nb) * 0.6931471805599453f;  // 1 - u is exact for u = (2m+1) 2^-24
  const int bin = key < 60.0f ? (int)(key * 0.5f) : 30;
  return 30 - bin;
}

// One warp's staging area: the inversion queue.
struct ZxQueue {
  float mu[ZX_Q], ph[ZX_Q];
  int xo[ZX_Q], kr[ZX_Q];
  uint32_t wu[ZX_Q], wa[ZX_Q];  // the inversion's uniform and the MH uniform
  uint16_t e[ZX_Q];             // position in the unit
  uint8_t perm[ZX_Q];
  int cnt[ZX_NCLS];
};

// Per-lane sums of one unit.
struct ZxAcc {
  long long nz = 0, xz = 0, n0 = 0;
  float d0 = 0.0f, d1a = 0.0f, d1b = 0.0f;
};

// The MH decision of an NB proposal (BUSseq_gpu.cu:497-506), the entry's
// writes and its gamma statistics.
__device__ __forceinline__ void zx_finish(const DevState& s, int kept, const float4* gtab, const GammaTerms& gt,
                                          int64_t jj, int2 ig, int xo, int xn, float ua, int err, ZxAcc& a) {
  // log[(1 + e^{-g0 - g1 x_old}) / (1 + e^{-g0 - g1 x_new})]
  const float spo = (unsigned)xo < (unsigned)ZX_HIST ? __ldg(&gtab[xo].x) : softplusf(-gt.g0 - gt.g1 * (float)xo);
  const float spn = (unsigned)xn < (unsigned)ZX_HIST ? __ldg(&gtab[xn].x) : softplusf(-gt.g0 - gt.g1 * (float)xn);
  const int x = log_fast(ua) <= spo - spn ? xn : xo;
  if (err) atomicOr(s.err, err);
  if (x != xo) s.X[(int64_t)ig.x * s.Gp + ig.y] = x;
  s.zval[jj] = 1;
  if (kept && s.acc_zn) {  // posterior summaries (entries with Z = 0 keep X = 0 and add nothing)
    s.acc_zn[jj] += 1;
    s.acc_xs[jj] += x;
  }
  ++a.nz;
  a.xz += x;
  if (x == 0) {
    ++a.n0;
  } else if (x < ZX_HIST) {
    const float4 t = __ldg(&gtab[x]);
    a.d0 += t.y;
    a.d1a += t.z;
    a.d1b += t.w;
  } else {
    gt.add(x, 1.0f, a.d0, a.d1a, a.d1b);
  }
}

__global__ void __launch_bounds__(ZX_THREADS, ZX_CTAS_PER_SM) k_zx(DevState s, int kept) {
  __shared__ double sh[ZX_WARPS * 3];
  __shared__ ZxQueue qs[ZX_WARPS];
  if ((int)blockIdx.x < s.n_static) gamma_static_cta(s, blockIdx.x, sh);  // the whole CTA, before any unit
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ZxQueue& q = qs[warp];
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp;
  const uint64_t G64 = (uint64_t)s.G;
  const uint32_t k0 = (uint32_t)s.seed, k1 = (uint32_t)(s.seed >> 32);
  const unsigned lt = (1u << lane) - 1u;
  for (;;) {
    int unit = 0;
    if (lane == 0) unit = (int)atomicAdd(&s.zx_ctr[0], 1u);
    unit = __shfl_sync(0xffffffffu, unit, 0);  // warp-uniform: the whole warp leaves together
    if (unit >= s.n_zcta) break;
    const int2 run = s.zcta[unit];
    const int b = s.zcta_batch[unit];
    const float4* gtab = s.zx_gtab + (int64_t)b * ZX_HIST;
    const int64_t eoff = (int64_t)b * s.K;
    GammaTerms gt;
    gt.g0 = s.gamma[b];
    gt.g1 = s.gamma[s.B + b];
    gt.g0p = s.gamma_p[b];
    gt.dg0 = gt.g0p - gt.g0;
    gt.dg1 = s.gamma_p[s.B + b] - gt.g1;
    const float zthr = 1.0f / (1.0f + expf(gt.g0));
    ZxAcc acc;
    int n_iq = 0, n_gq = 0;  // warp-uniform: the queue's length, the Gamma-Poisson entries listed
    const int64_t gpo = run.x;  // the unit's record slots: one per entry of the unit
    q.cnt[lane] = 0;
    __syncwarp();
    for (int part = 0; part * ZX_PART < run.y; ++part) {
      const int hb = part * ZX_PART;
      const bool last = hb + ZX_PART >= run.y;
      // ---- phase 1: loads hoisted over the lane's four entries ------------
      int ei[ZX_PER_LANE], eg[ZX_PER_LANE], exo[ZX_PER_LANE];
      float emu[ZX_PER_LANE], eph[ZX_PER_LANE];
#pragma unroll
      for (int u = 0; u < ZX_PER_LANE; ++u) {
        const int e = hb + u * 32 + lane;
        const int2 ig = e < run.y ? s.zij[(int64_t)run.x + e] : make_int2(-1, 0);
        ei[u] = ig.x;
        eg[u] = ig.y;
      }
      int ew[ZX_PER_LANE];
      float eD[ZX_PER_LANE];
#pragma unroll
      for (int u = 0; u < ZX_PER_LANE; ++u) {
        if (ei[u] >= 0) {
          const int64_t i = ei[u], g = eg[u];
          ew[u] = s.W[i];
          eD[u] = s.Dexp[i];
          eph[u] = s.phi[(int64_t)b * Gp + g];
          exo[u] = s.X[i * Gp + g];
        } else {
          ew[u] = 0;
          eD[u] = 0.0f;
          eph[u] = 1.0f;
          exo[u] = 0;
        }
      }
#pragma unroll
      for (int u = 0; u < ZX_PER_LANE; ++u)
        emu[u] = ei[u] >= 0 ? s.E[(eoff + ew[u]) * Gp + eg[u]] * eD[u] : 0.0f;
#pragma unroll
      for (int u = 0; u < ZX_PER_LANE; ++u) {
        const int e = hb + u * 32 + lane;
        bool inv = false, gpn = false;
        int cls = -1;
        const float mu = emu[u], ph = eph[u];
        const int xo = exo[u];
        U32x4 r{0u, 0u, 0u, 0u};
        if (ei[u] >= 0) {
          const uint64_t ent = (uint64_t)ei[u] * G64 + (uint64_t)eg[u];
          r = philox4x32_10(U32x4{(uint32_t)ent, ((uint32_t)(ent >> 32) & 0xFFFFu) | (SID_ZX << 16), 0u, iter}, k0,
                            k1);
          const bool z = xo != 0 || u32_to_unit(r.x) > zthr;
          if (z) {
            if (negbin_use_inversion(mu, ph)) {
              inv = true;
              cls = zx_class(mu, u32_to_unit(xo == 0 ? r.y : r.x));
            } else {
              gpn = true;
            }
          } else {
            s.zval[(int64_t)run.x + e] = 0;  // Z = 0 and X stays 0
            ++acc.n0;
          }
        }
        const unsigned im = __ballot_sync(0xffffffffu, inv);
        const unsigned gm = __ballot_sync(0xffffffffu, gpn);
        const unsigned grp = __match_any_sync(0xffffffffu, cls);
        if (inv) {
          const int slot = n_iq + __popc(im & lt);
          q.mu[slot] = mu;
          q.ph[slot] = ph;
          q.xo[slot] = xo;
          q.e[slot] = (uint16_t)e;
          q.kr[slot] = (cls << 16) | (q.cnt[cls] + __popc(grp & lt));
          q.wu[slot] = xo == 0 ? r.y : r.x;
          q.wa[slot] = xo == 0 ? r.z : r.y;
        }
        if (gpn) {  // the record k_zx_gp draws from, with what was loaded for it here
          const int64_t o = gpo + n_gq + __popc(gm & lt);
          s.zgp_rec[o] = make_int4(run.x + e, ei[u], eg[u], xo);
          s.zgp_mp[o] = make_float2(mu, ph);
        }
        __syncwarp();
        if (inv && (grp & lt) == 0) q.cnt[cls] += __popc(grp);  // the class group's first lane
        __syncwarp();
        n_iq += __popc(im);
        n_gq += __popc(gm);
      }
      // ---- phase 2: class offsets (lane = class), then the queue order ----
      {
        const int tot = q.cnt[lane];
        int incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        __syncwarp();
        q.cnt[lane] = incl - tot;
        __syncwarp();
        for (int j = lane; j < n_iq; j += 32) {
          const int kr = q.kr[j];
          q.perm[q.cnt[kr >> 16] + (kr & 0xFFFF)] = (uint8_t)j;
        }
        __syncwarp();
      }
      // ---- phase 3a: the inversions, X ~ NB independence MH
      //      (BUSseq_gpu.cu:497-506), 32 queue positions at a time -----------
      const int n_run = last ? n_iq : (n_iq & ~31);
      for (int p0 = 0; p0 < n_run; p0 += 32) {
        const int p = p0 + lane;
        if (p >= n_run) continue;
        const int j = q.perm[p];
        const int64_t jj = (int64_t)run.x + q.e[j];
        const int2 ig = s.zij[jj];  // for the write of X, loaded ahead of the search
        const int xo = q.xo[j];
        int err = 0;
        const int xn = negbin_invert_u(u32_to_unit(q.wu[j]), q.mu[j], q.ph[j], &err, s.nb_inv_cap);
        zx_finish(s, kept, gtab, gt, jj, ig, xo, xn, u32_to_unit(q.wa[j]), err, acc);
      }
      __syncwarp();
      // ---- carry the shortest searches (fewer than 32) to the next part ----
      if (!last) {
        const int left = n_iq - n_run;
        const bool has = lane < left;
        float cmu = 0.0f, cph = 0.0f;
        int cxo = 0, ckr = 0;
        uint32_t cwu = 0u, cwa = 0u;
        uint16_t ce = 0;
        if (has) {
          const int j = q.perm[n_run + lane];
          cmu = q.mu[j];
          cph = q.ph[j];
          cxo = q.xo[j];
          ckr = q.kr[j];
          cwu = q.wu[j];
          cwa = q.wa[j];
          ce = q.e[j];
        }
        const int cc = has ? (ckr >> 16) : 64 + lane;
        const unsigned grp = __match_any_sync(0xffffffffu, cc);
        __syncwarp();
        q.cnt[lane] = 0;
        __syncwarp();
        if (has) {
          q.mu[lane] = cmu;
          q.ph[lane] = cph;
          q.xo[lane] = cxo;
          q.kr[lane] = (cc << 16) | __popc(grp & lt);
          q.wu[lane] = cwu;
          q.wa[lane] = cwa;
          q.e[lane] = ce;
          if ((grp & lt) == 0) q.cnt[cc] = __popc(grp);
        }
        __syncwarp();
        n_iq = left;
      }
    }
    if (lane == 0) s.zgp_cnt[unit] = n_gq;
    // ---- the unit's partial: a fixed-order warp reduction -----------------
    const FF f0 = ff_warp_sum(FF{acc.d0, 0.0f}), f1 = ff_warp_sum(FF{acc.d1a, 0.0f}),
             f2 = ff_warp_sum(FF{acc.d1b, 0.0f});
    const long long nz = i64_warp_sum(acc.nz), xz = i64_warp_sum(acc.xz), n0 = i64_warp_sum(acc.n0);
    if (lane == 0) {
      double* gp = s.gpart + (int64_t)unit * GSLOT;
      gp[0] = (double)nz;
      gp[1] = (double)xz;
      gp[2] = (double)n0;
      gp[3] = ff_value(f0);
      gp[4] = ff_value(f1);
      gp[5] = ff_value(f2);
    }
    __syncwarp();  // the queue's counts are reset by the next unit
  }
  // the last warp to finish zeroes both counters for the next launch
  if (lane == 0) {
    __threadfence();
    const unsigned total = gridDim.x * (unsigned)ZX_WARPS;
    if (atomicAdd(&s.zx_ctr[1], 1u) == total - 1u) {
      s.zx_ctr[0] = 0u;
      s.zx_ctr[1] = 0u;
      __threadfence();
    }
  }
}

// The NB proposals that k_zx listed for Gamma-Poisson draws (phi < 1 or
// mu >= NB_INV_MU: BUSseq_gpu.cu:199-210's method), in a pass of their own so
// that every lane of a round runs the same sampler and k_zx carries none of
// its code.  Warps take chunks of ZGP_UNITS units of one batch from a counter
// and draw the chunk's listed entries 32 at a time in unit order; each lane
// reads its entry's record, generates blocks 0 and 1 of the entry's stream
// with the other lanes, draws the Gamma-Poisson proposal and decides it as
// k_zx decides an inversion's.  The chunk's partial is its units' partials from
// k_zx plus the gamma statistics of these draws, summed in a fixed order, so
// the sums do not depend on which warp took the chunk; the gamma decisions
// then read one partial per chunk.
__global__ void __launch_bounds__(ZX_THREADS, ZGP_CTAS_PER_SM) k_zx_gp(DevState s, int kept) {
  const int lane = threadIdx.x & 31;
  const uint32_t iter = (uint32_t)*s.iter;
  const uint64_t G64 = (uint64_t)s.G;
  const uint32_t k0 = (uint32_t)s.seed, k1 = (uint32_t)(s.seed >> 32);
  for (;;) {
    int c = 0;
    if (lane == 0) c = (int)atomicAdd(&s.zx_ctr[2], 1u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= s.n_gchunk) break;
    const int4 ch = s.zgchunk[c];  // {first unit, units (<= 32), batch}
    const int b = ch.z;
    // the units' list lengths and their exclusive prefix (lane = unit of the chunk)
    const int cnt = lane < ch.y ? s.zgp_cnt[ch.x + lane] : 0;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - cnt;
    const float4* gtab = s.zx_gtab + (int64_t)b * ZX_HIST;
    GammaTerms gt;
    gt.g0 = s.gamma[b];
    gt.g1 = s.gamma[s.B + b];
    gt.g0p = s.gamma_p[b];
    gt.dg0 = gt.g0p - gt.g0;
    gt.dg1 = s.gamma_p[s.B + b] - gt.g1;
    ZxAcc acc;
    for (int p0 = 0; p0 < total; p0 += 32) {
      const int p = p0 + lane;
      // the unit holding list position p: the last one whose prefix is <= p
      // (an empty unit shares its prefix with the next one)
      int uu = 0;
      for (int t = 1; t < ch.y; ++t)
        if (p >= __shfl_sync(0xffffffffu, excl, t)) uu = t;
      const int base = __shfl_sync(0xffffffffu, excl, uu);
      if (p < total) {
        const int64_t o = (int64_t)s.zcta[ch.x + uu].x + (p - base);
        const int4 ra = s.zgp_rec[o];
        const float2 rb = s.zgp_mp[o];
        const int64_t jj = ra.x;
        const int2 ig = make_int2(ra.y, ra.z);
        const int xo = ra.w;
        const float mu = rb.x, ph = rb.y;
        const uint64_t ent = (uint64_t)ra.y * G64 + (uint64_t)ra.z;
        const U32x4 r = philox4x32_10(
            U32x4{(uint32_t)ent, ((uint32_t)(ent >> 32) & 0xFFFFu) | (SID_ZX << 16), 0u, iter}, k0, k1);
        StreamAhead st(Stream::resume(s.seed, SID_ZX, ent, iter, r.x, r.y, r.z, r.w, xo == 0));
        int err = 0;
        const int xn = negbin_gamma_poisson(st, mu, ph, &err);
        zx_finish(s, kept, gtab, gt, jj, ig, xo, xn, st.uniform(), err, acc);
      }
    }
    const FF f0 = ff_warp_sum(FF{acc.d0, 0.0f}), f1 = ff_warp_sum(FF{acc.d1a, 0.0f}),
             f2 = ff_warp_sum(FF{acc.d1b, 0.0f});
    const long long nz = i64_warp_sum(acc.nz), xz = i64_warp_sum(acc.xz), n0 = i64_warp_sum(acc.n0);
    // (the warp sums are lane 0's) the chunk's unit partials first, in unit order
    if (lane == 0) {
      double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int t = 0; t < ch.y; ++t)
#pragma unroll
        for (int q = 0; q < 6; ++q) v[q] += s.gpart[(int64_t)(ch.x + t) * GSLOT + q];
      double* gp = s.gpart_gp + (int64_t)c * GSLOT;
      gp[0] = v[0] + (double)nz;
      gp[1] = v[1] + (double)xz;
      gp[2] = v[2] + (double)n0;
      gp[3] = v[3] + ff_value(f0);
      gp[4] = v[4] + ff_value(f1);
      gp[5] = v[5] + ff_value(f2);
    }
  }
  // the last warp to finish zeroes both counters for the next launch
  if (lane == 0) {
    __threadfence();
    const unsigned total = gridDim.x * (unsigned)ZX_WARPS;
    if (atomicAdd(&s.zx_ctr[3], 1u) == total - 1u) {
      s.zx_ctr[2] = 0u;
      s.zx_ctr[3] = 0u;
      __threadfence();
    }
  }
}

// ---------------------------------------------------------------------------
// Gene passes
// ---------------------------------------------------------------------------
// Copies the chunk's cell indices and exp(delta) into shared memory and pads
// the chunk to a multiple of 8 cells with the all-zero row N of X and
// exp(delta) = 0: a padding entry has x = 0 and mu = 0, and every per-entry
// term below is then exactly zero, so the inner loops need no bounds tests.
// Returns the padded length.
__device__ __forceinline__ int stage_chunk(const DevState& s, int start, int len, int* s_i, float* s_D) {
  const int len8 = (len + 7) & ~7;
  for (int j = threadIdx.x; j < len8; j += blockDim.x) {
    const bool in = j < len;
    const int i = in ? s.perm[start + j] : (int)s.N;
    s_i[j] = i;
    s_D[j] = in ? s.Dexp[i] : 0.0f;
  }
  return len8;
}

// alpha: sum of x and of (phi + x) log1p(expm1(alpha' - alpha) p) over the chunk.
// FAST: |c| <= 1/2, the term by log1p_shift (one reciprocal); otherwise the
// general form (a random-walk step beyond 0.405, about four of its sd).
template <bool FAST>
__device__ __forceinline__ void alpha_sums(const char* Xg, uint32_t row_bytes, const int* s_i, const float* s_D,
                                           int len8, float M, float ph, float ca, int64_t& sx, KahanF& la) {
  const float c2 = 2.0f + ca, ph2 = 2.0f * ph;
  for (int j0 = 0; j0 < len8; j0 += 8) {
    int xr[8];
    float dv[8];
    load8(Xg, row_bytes, s_i, s_D, j0, xr, dv);
    float f = 0.0f;
    int s8 = 0;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const float mu = M * dv[u];
      s8 += xr[u];
      const float l = FAST ? log1p_shift(ca * mu, fmaf(c2, mu, ph2)) : log1p_near0(ca * fast_div(mu, ph + mu));
      f = fmaf(ph + (float)xr[u], l, f);
    }
    sx += s8;
    la.add(f);
  }
}

__global__ void __launch_bounds__(GENE_TILE) k_alpha(DevState s) {
  __shared__ __align__(16) int s_i[MAX_CG];
  __shared__ __align__(16) float s_D[MAX_CG];
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + threadIdx.x;
  if (len == 0) return;
  const int len8 = stage_chunk(s, start, len, s_i, s_D);
  __syncthreads();
  if (g >= s.G) return;
  const char* Xg = reinterpret_cast<const char*>(s.X + g);
  const uint32_t row_bytes = (uint32_t)(Gp * sizeof(int));
  const float M = s.E[((int64_t)b * s.K + k) * Gp + g];
  const float ph = s.phi[(int64_t)b * Gp + g];
  const float ca = expm1f(s.alpha_p[g] - s.alpha[g]);
  int64_t sx = 0;
  KahanF la;
  if (fabsf(ca) <= 0.5f) alpha_sums<true>(Xg, row_bytes, s_i, s_D, len8, M, ph, ca, sx, la);
  else alpha_sums<false>(Xg, row_bytes, s_i, s_D, len8, M, ph, ca, sx, la);
  double* pr = s.part + (int64_t)row * NSLOT * Gp + g;
  pr[0] = (double)sx;
  pr[Gp] = la.value();
}

// Chunk sums of k_beta_nu for one CTA-uniform case: HB = the chunk's type
// has a beta (k > 0), HN = its batch has a nu (b > 0).  FAST: both shifts'
// |expm1(step)| <= 1/2, every term by log1p_shift.
template <bool HB, bool HN, bool FAST>
__device__ __forceinline__ void beta_nu_sums(const char* Xg, uint32_t row_bytes, const int* s_i, const float* s_D,
                                             int len8, float M, float ph, float cb, float fb, float cn, int64_t& sx,
                                             KahanF& lb, KahanF& ln0, KahanF& ln1) {
  const float cb2 = 2.0f + cb, cn2 = 2.0f + cn, ph2 = 2.0f * ph;
  for (int j0 = 0; j0 < len8; j0 += 8) {
    int xr[8];
    float dv[8];
    load8(Xg, row_bytes, s_i, s_D, j0, xr, dv);
    float lbf = 0.0f, ln0f = 0.0f, ln1f = 0.0f;
    int s8 = 0;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int x = xr[u];
      const float mu = M * dv[u];
      const float w = ph + (float)x;
      s8 += x;
      if (FAST) {
        if (HB) lbf = fmaf(w, log1p_shift(cb * mu, fmaf(cb2, mu, ph2)), lbf);
        if (HN) {
          ln0f = fmaf(w, log1p_shift(cn * mu, fmaf(cn2, mu, ph2)), ln0f);
          if (HB) {
            const float mu1 = mu * fb;
            ln1f = fmaf(w, log1p_shift(cn * mu1, fmaf(cn2, mu1, ph2)), ln1f);
          }
        }
      } else {
        const float p = fast_div(mu, ph + mu);
        if (HB) lbf += w * log1p_near0(cb * p);
        if (HN) {
          ln0f += w * log1p_near0(cn * p);
          if (HB) {
            const float mu1 = mu * fb;
            ln1f += w * log1p_near0(cn * fast_div(mu1, ph + mu1));
          }
        }
      }
    }
    sx += s8;
    if (HB) lb.add(lbf);
    if (HN) ln0.add(ln0f);
    if (HB && HN) ln1.add(ln1f);
  }
}

template <bool FAST>
__device__ __forceinline__ void beta_nu_case(int b, int k, const char* Xg, uint32_t row_bytes, const int* s_i,
                                             const float* s_D, int len8, float M, float ph, float cb, float fb,
                                             float cn, int64_t& sx, KahanF& lb, KahanF& ln0, KahanF& ln1) {
  if (k > 0 && b > 0)
    beta_nu_sums<true, true, FAST>(Xg, row_bytes, s_i, s_D, len8, M, ph, cb, fb, cn, sx, lb, ln0, ln1);
  else if (k > 0)
    beta_nu_sums<true, false, FAST>(Xg, row_bytes, s_i, s_D, len8, M, ph, cb, fb, cn, sx, lb, ln0, ln1);
  else
    beta_nu_sums<false, true, FAST>(Xg, row_bytes, s_i, s_D, len8, M, ph, cb, fb, cn, sx, lb, ln0, ln1);
}

__global__ void __launch_bounds__(GENE_TILE) k_beta_nu(DevState s) {
  __shared__ __align__(16) int s_i[MAX_CG];
  __shared__ __align__(16) float s_D[MAX_CG];
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + threadIdx.x;
  if (len == 0 || (k == 0 && b == 0)) return;
  const int len8 = stage_chunk(s, start, len, s_i, s_D);
  __syncthreads();
  if (g >= s.G) return;
  const char* Xg = reinterpret_cast<const char*>(s.X + g);
  const uint32_t row_bytes = (uint32_t)(Gp * sizeof(int));
  const float bt = s.beta[(int64_t)k * Gp + g];
  const float M = exp_sum3(s.alpha[g], bt, s.nu[(int64_t)b * Gp + g]);
  const float ph = s.phi[(int64_t)b * Gp + g];
  const float eb = k > 0 ? s.beta_p[(int64_t)k * Gp + g] - bt : 0.0f;
  const float cb = expm1f(eb), fb = expf(eb);
  const float en = b > 0 ? s.nu_p[(int64_t)b * Gp + g] - s.nu[(int64_t)b * Gp + g] : 0.0f;
  const float cn = expm1f(en);
  int64_t sx = 0;
  KahanF lb, ln0, ln1;
  if (fabsf(cb) <= 0.5f && fabsf(cn) <= 0.5f)
    beta_nu_case<true>(b, k, Xg, row_bytes, s_i, s_D, len8, M, ph, cb, fb, cn, sx, lb, ln0, ln1);
  else
    beta_nu_case<false>(b, k, Xg, row_bytes, s_i, s_D, len8, M, ph, cb, fb, cn, sx, lb, ln0, ln1);
  double* pr = s.part + (int64_t)row * NSLOT * Gp + g;
  pr[0] = (double)sx;
  pr[Gp] = lb.value();
  pr[2 * Gp] = ln0.value();
  pr[3 * Gp] = ln1.value();
}

__global__ void __launch_bounds__(GENE_TILE) k_phi(DevState s) {
  __shared__ float tab[PHI_TAB][GENE_TILE];
  __shared__ __align__(16) int s_i[MAX_CG];
  __shared__ __align__(16) float s_D[MAX_CG];
  const int tid = threadIdx.x;
  const int tile = blockIdx.x, row = blockIdx.y;
  const int4 ch = s.gchunk[row];
  const int b = ch.x, k = ch.y, start = ch.z, len = ch.w;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * GENE_TILE + tid;
  if (len == 0) return;
  const int len8 = stage_chunk(s, start, len, s_i, s_D);
  // the proposal's table of lgamma differences, built by k_propose
  const float* tg = s.phi_tab + (int64_t)b * PHI_TAB * Gp + g;
#pragma unroll 8
  for (int x = 0; x < PHI_TAB; ++x) tab[x][tid] = tg[(int64_t)x * Gp];
  __syncthreads();
  if (g >= s.G) return;
  const float ph = s.phi[(int64_t)b * Gp + g];
  const float pp = s.phi_p[(int64_t)b * Gp + g];
  const float dl = pp - ph;
  const float M = s.E[((int64_t)b * s.K + k) * Gp + g];
  const float iph = 1.0f / ph;
  // Per entry (BUSseq_gpu.cu:799-802, regrouped so that no large terms cancel):
  //   t = [lgamma(pp+x) - lgamma(pp)] - [lgamma(ph+x) - lgamma(ph)]
  //       - (pp + x) log((pp + mu) / (ph + mu)) + pp log(pp / ph) - dl log(1 + mu / ph)
  const float lgd0 = s.phi_lgd0[(int64_t)b * Gp + g];
  const float c1 = pp * log_ratio(pp, ph, dl);
  const char* Xg = reinterpret_cast<const char*>(s.X + g);
  const uint32_t row_bytes = (uint32_t)(Gp * sizeof(int));
  // Y == 0 bit of the entry (row N, the padding row, is all zero); the lgamma
  // part of the entries with Y > 0 is k_phi_static's
  const uint32_t* ym = s.y0m + (g >> 5);
  const int64_t Gw = s.Gw;
  const int bit = (int)(g & 31);
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
      const float mu = M * dv[u];
      const float xf = (float)x;
      const bool y0 = (zw[u] >> bit) & 1u;
      float hx = y0 && (unsigned)x < (unsigned)PHI_TAB ? tab[x][tid] : 0.0f;
      // an imputed count past the table (rare): both arguments are past the shift range
      if (y0 && x >= PHI_TAB) hx = lgamma_diff_large(ph + xf, pp + xf, dl) - lgd0;
      f += hx - (pp + xf) * log_ratio(pp + mu, ph + mu, dl) + c1 - dl * log1p_fast(mu * iph);
    }
    acc.add(f);
  }
  s.part[(int64_t)row * NSLOT * Gp + g] = acc.value();
}

// The lgamma part of the phi sums of the entries with Y >= PHI_TAB, one warp
// per (batch, gene) (warps striding over the pairs), lanes taking the gene's
// values in turn, added to the part
// below the table that k_propose left in phi_static.  Fixed-order float-float
// sums, so the result is reproducible.
__global__ void __launch_bounds__(256) k_phi_static(DevState s) {
  const int lane = threadIdx.x & 31;
  const int64_t nbg = (int64_t)s.B * s.G, nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nbg; w += nw) {  // uniform per warp
    const int64_t o0 = s.phi_big_off[w], o1 = s.phi_big_off[w + 1];
    if (o1 == o0) continue;
    const int b = (int)(w / s.G);
    const int64_t g = w % s.G;
    const int64_t pos = (int64_t)b * s.Gp + g;
    const float ph = s.phi[pos], pp = s.phi_p[pos];
    const float dl = pp - ph, lgd0 = s.phi_lgd0[pos];
    KahanF acc;
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
          acc.add(lgamma_diff_large(ph + y, pp + y, dl) - lgd0);
        }
    }
    const FF tot = ff_warp_sum(acc.ff());
    if (lane == 0) s.phi_static[pos] += ff_value(tot);
  }
}

// ---------------------------------------------------------------------------
// Decisions
// ---------------------------------------------------------------------------
// gamma0 then gamma1 of batch b, one CTA (BUSseq_gpu.cu:514-600).
__device__ void gamma_decide_cta(const DevState& s, int b, uint32_t iter, double* sh) {
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  // the batch's Z/X chunk partials (k_zx_gp folds the units' partials into
  // them), four chunks' loads in flight per thread
  const int c_end = s.gfirst[b + 1], stride = (int)blockDim.x;
  int c = s.gfirst[b] + (int)threadIdx.x;
  for (; c + 3 * stride < c_end; c += 4 * stride) {
    double t[4][6];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int q = 0; q < 6; ++q) t[u][q] = __ldg(&s.gpart_gp[(int64_t)(c + u * stride) * GSLOT + q]);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int q = 0; q < 6; ++q) v[q] += t[u][q];
  }
  for (; c < c_end; c += stride) {
#pragma unroll
    for (int q = 0; q < 6; ++q) v[q] += __ldg(&s.gpart_gp[(int64_t)c * GSLOT + q]);
  }
  const int slices = (s.ymax + ZX_THREADS - 1) / ZX_THREADS;
  for (int c = b * slices + threadIdx.x; c < (b + 1) * slices && c < s.n_static; c += blockDim.x) {
    v[6] += s.gstat[(int64_t)c * 4 + 0];
    v[7] += s.gstat[(int64_t)c * 4 + 1];
    v[8] += s.gstat[(int64_t)c * 4 + 2];
  }
  block_sum<9>(v, sh);
  if (threadIdx.x != 0) return;
  const float g0 = s.gamma[b], g1 = s.gamma[s.B + b];
  const float g0p = s.gamma_p[b], g1p = s.gamma_p[s.B + b];
  const double nZ = v[0], XZ = v[1], n0 = v[2];
  // entries with Y == 0 and X == 0 all contribute softplus(g0p) - softplus(g0)
  const double c0 = (double)softplus_diff(g0, g0p - g0);
  const double lr0 = (double)(g0p - g0) * nZ - (v[3] + n0 * c0 + v[6]);
  const double prior0 = ((double)g0 * g0 - (double)g0p * g0p) / (2.0 * SIGMA2_GAMMA0);
  const float u0 = uniform_at(s.seed, SID_GAMMA, (uint64_t)b, iter, 2);
  const bool acc0 = (double)logf(u0) <= lr0 + prior0;
  s.lr_gamma[b] = lr0 + prior0;
  if (acc0) s.gamma[b] = g0p;
  const double lr1 = (double)(g1p - g1) * XZ - (acc0 ? (v[5] + v[8]) : (v[4] + v[7]));
  // -gamma1 ~ Gamma(kappa, rate tau) prior, -10 gamma1 Gamma proposal (BUSseq_gpu.cu:588-600)
  const double pv = -(double)g1, nv = -(double)g1p;
  const double prior1 = (KAPPA_GAMMA1 - 1.0) * (log(nv) - log(pv)) + TAU_GAMMA1 * (pv - nv) - lgamma(10.0 * nv) +
                        (10.0 * nv - 1.0) * log(pv) + 10.0 * nv * (log(10.0) + 1.0) + lgamma(10.0 * pv) -
                        (10.0 * pv - 1.0) * log(nv) - 10.0 * pv * (log(10.0) + 1.0);
  const float u1 = uniform_at(s.seed, SID_GAMMA, (uint64_t)b, iter, 3);
  s.lr_gamma[s.B + b] = lr1 + prior1;
  if ((double)logf(u1) <= lr1 + prior1) s.gamma[s.B + b] = g1p;
}

// gamma0 and gamma1 of batch blockIdx.x.
__global__ void __launch_bounds__(DECIDE_GAMMA_THREADS) k_decide_gamma(DevState s) {
  __shared__ double sh[(DECIDE_GAMMA_THREADS / 32) * 9];
  gamma_decide_cta(s, blockIdx.x, (uint32_t)*s.iter, sh);
}

// One CTA per 32 genes: alpha decisions and L; the last CTA draws p and tau0.
// The CTA's four warps split each gene's chunk partials (chunks c = w, w + 4,
// ...) so that more loads are in flight, and add the four slices in a fixed
// order; they split the types of the L redraw the same way.
constexpr int DA_SLICES = GENE_TILE / 32;
__global__ void __launch_bounds__(GENE_TILE) k_decide_alpha(DevState s) {
  __shared__ double sh[(GENE_TILE / 32) * 2];
  __shared__ double s_sum[DA_SLICES][2][32];
  __shared__ int sh_flag;
  const uint32_t iter = (uint32_t)*s.iter;
  const int tid = threadIdx.x, lane = tid & 31, sl = tid >> 5;
  const int tile = blockIdx.x;
  const int64_t Gp = s.Gp;
  const int64_t g = (int64_t)tile * 32 + lane;
  if (s.hmc_L == 0) {  // alpha: random-walk MH (the HMC block updates it otherwise)
    double Sx = 0.0, La = 0.0;
    if (g < s.G) {
#pragma unroll 4
      for (int c = sl; c < s.cap_g; c += DA_SLICES) {
        const bool used = s.gchunk[c].w > 0;
        const double a0 = __ldg(&s.part[((int64_t)c * NSLOT + 0) * Gp + g]);
        const double a1 = __ldg(&s.part[((int64_t)c * NSLOT + 1) * Gp + g]);
        Sx += used ? a0 : 0.0;
        La += used ? a1 : 0.0;
      }
    }
    s_sum[sl][0][lane] = Sx;
    s_sum[sl][1][lane] = La;
    __syncthreads();
    if (sl == 0 && g < s.G) {
      Sx = s_sum[0][0][lane];
      La = s_sum[0][1][lane];
#pragma unroll
      for (int w = 1; w < DA_SLICES; ++w) {
        Sx += s_sum[w][0][lane];
        La += s_sum[w][1][lane];
      }
      const float a = s.alpha[g], ap = s.alpha_p[g];
      const double ma = s.mu_alpha[g];
      const double lr = (double)(ap - a) * Sx - La;
      const double prior = (((double)a - ma) * ((double)a - ma) - ((double)ap - ma) * ((double)ap - ma)) /
                           (2.0 * SIGMA2_ALPHA);
      const float ua = uniform_at(s.seed, SID_ALPHA, (uint64_t)g, iter, 2);
      s.lr_alpha[g] = lr + prior;
      if ((double)logf(ua) <= lr + prior) s.alpha[g] = ap;
    }
  }
  double lv[2] = {0.0, 0.0};
  if (g < s.G) {
    // L from the current beta, p and tau0 (BUSseq_gpu.cu:634-648)
    const float p = s.p_tau0[0], tau0 = s.p_tau0[1];
    const float base = logf(p) - logf(1.0f - p) - (logf((float)TAU1) - logf(tau0)) * 0.5f;
    const float qd = 1.0f / (2.0f * tau0) - 1.0f / (2.0f * (float)TAU1);
    for (int kk = 1 + sl; kk < s.K; kk += DA_SLICES) {
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
  if (!arrive_last(&s.cnt_glob[0], gridDim.x, &sh_flag)) return;
  if ((int)iter < s.n_unchanged) return;
  // p ~ Beta(sum L + 1, G(K-1) - sum L + 3), tau0 = 1 / Gamma(...) (BUSseq_gpu.cu:650-668)
  double v[2] = {0.0, 0.0};
  for (int t = tid; t < (int)gridDim.x; t += blockDim.x) {
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

// beta_gk for k >= 1: one thread per (k, g) (BUSseq_gpu.cu:696-707).
// The per-gene decisions below take 32 genes per CTA, each gene split over
// DEC_SLICES warps: warp w sums the chunk partials of the segments w, w +
// DEC_SLICES, ... (batches for beta, types for nu and phi) with both slots'
// loads in flight, and warp 0 adds the slices in a fixed order and decides.
// A thread per gene with one segment after the other would wait for every
// segment's loads in turn.
constexpr int DEC_SLICES = DEC_THREADS / 32;

// Both slots' sums over the chunks c of range r of gene g.
__device__ __forceinline__ void chunk_sums2(const DevState& s, int2 r, int slot_a, int slot_b, int64_t g, double& a,
                                            double& b) {
  const int64_t Gp = s.Gp;
#pragma unroll 2
  for (int c = r.x; c < r.x + r.y; ++c) {
    a += __ldg(&s.part[((int64_t)c * NSLOT + slot_a) * Gp + g]);
    b += __ldg(&s.part[((int64_t)c * NSLOT + slot_b) * Gp + g]);
  }
}

// One slot's sum over the chunks c of range r of gene g.
__device__ __forceinline__ void chunk_sums1(const DevState& s, int2 r, int slot, int64_t g, double& a) {
  const int64_t Gp = s.Gp;
#pragma unroll 4
  for (int c = r.x; c < r.x + r.y; ++c) a += __ldg(&s.part[((int64_t)c * NSLOT + slot) * Gp + g]);
}

// The slices' two sums of gene lane, added in slice order (valid in warp 0).
__device__ __forceinline__ void dec_combine(double (&sm)[DEC_SLICES][2][32], int sl, int lane, double& a, double& b) {
  sm[sl][0][lane] = a;
  sm[sl][1][lane] = b;
  __syncthreads();
  if (sl == 0) {
    a = sm[0][0][lane];
    b = sm[0][1][lane];
#pragma unroll
    for (int w = 1; w < DEC_SLICES; ++w) {
      a += sm[w][0][lane];
      b += sm[w][1][lane];
    }
  }
}

// beta_k,g for k >= 1 (BUSseq_gpu.cu:696-707); slices over batches.
__global__ void __launch_bounds__(DEC_THREADS) k_decide_beta(DevState s) {
  __shared__ double sm[DEC_SLICES][2][32];
  const int lane = threadIdx.x & 31, sl = threadIdx.x >> 5;
  const int64_t t = (int64_t)blockIdx.x * 32 + lane;
  const int64_t G = s.G, Gp = s.Gp;
  const bool live = t < (int64_t)(s.K - 1) * G;
  const int k = live ? 1 + (int)(t / G) : 1;
  const int64_t g = live ? t % G : 0;
  double Sx = 0.0, Lb = 0.0;
  if (live)
    for (int b = sl; b < s.B; b += DEC_SLICES) chunk_sums2(s, s.seg_chunk[b * s.K + k], 0, 1, g, Sx, Lb);
  dec_combine(sm, sl, lane, Sx, Lb);
  if (sl != 0 || !live) return;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t pos = (int64_t)k * Gp + g;
  const float bo = s.beta[pos], bn = s.beta_p[pos];
  const double var = s.L[pos] == 1 ? TAU1 : (double)s.p_tau0[1];
  const double lr = (double)(bn - bo) * Sx - Lb;
  const double prior = ((double)bo * bo - (double)bn * bn) / (2.0 * var);
  const float u = uniform_at(s.seed, SID_BETA, (uint64_t)t, iter, 2);
  s.lr_beta[(int64_t)k * G + g] = lr + prior;
  const bool acc = (double)logf(u) <= lr + prior;
  if (acc) s.beta[pos] = bn;
  s.beta_acc[pos] = acc ? 1 : 0;
}

// nu_b,g for b >= 1 (BUSseq_gpu.cu:730-737), then the table
// E = exp(alpha + beta + nu) of every type for the new nu; slices over types.
__global__ void __launch_bounds__(DEC_THREADS) k_decide_nu_E(DevState s) {
  __shared__ double sm[DEC_SLICES][2][32];
  __shared__ float s_nu[32];
  const int lane = threadIdx.x & 31, sl = threadIdx.x >> 5;
  const int64_t t = (int64_t)blockIdx.x * 32 + lane;
  const int64_t G = s.G, Gp = s.Gp;
  const bool live = t < (int64_t)s.B * G;
  const int b = live ? (int)(t / G) : 0;
  const int64_t g = live ? t % G : 0;
  const int64_t pos = (int64_t)b * Gp + g;
  double Sx = 0.0, Ln = 0.0;
  if (live && b > 0)
    for (int k = sl; k < s.K; k += DEC_SLICES) {
      const bool bacc = k > 0 && s.beta_acc[(int64_t)k * Gp + g];
      chunk_sums2(s, s.seg_chunk[b * s.K + k], 0, bacc ? 3 : 2, g, Sx, Ln);
    }
  dec_combine(sm, sl, lane, Sx, Ln);
  if (sl == 0 && live) {
    float nv = s.nu[pos];
    if (b > 0) {
      const uint32_t iter = (uint32_t)*s.iter;
      const float vn = s.nu_p[pos];
      const double mn = s.mu_nu[b];
      const double lr = (double)(vn - nv) * Sx - Ln;
      const double prior = (((double)nv - mn) * ((double)nv - mn) - ((double)vn - mn) * ((double)vn - mn)) /
                           (2.0 * SIGMA2_NU);
      const float u = uniform_at(s.seed, SID_NU, (uint64_t)(b - 1) * (uint64_t)G + (uint64_t)g, iter, 2);
      s.lr_nu[(int64_t)b * G + g] = lr + prior;
      if ((double)logf(u) <= lr + prior) {
        s.nu[pos] = vn;
        nv = vn;
      }
    }
    s_nu[lane] = nv;
  }
  __syncthreads();
  if (!live) return;
  const float a = s.alpha[g], nv = s_nu[lane];
  for (int k = sl; k < s.K; k += DEC_SLICES)
    s.E[((int64_t)b * s.K + k) * Gp + g] = exp_sum3(a, s.beta[(int64_t)k * Gp + g], nv);
}

// phi_b,g (BUSseq_gpu.cu:806-818); slices over types.
__global__ void __launch_bounds__(DEC_THREADS) k_decide_phi(DevState s) {
  __shared__ double sm[DEC_SLICES][2][32];
  const int lane = threadIdx.x & 31, sl = threadIdx.x >> 5;
  const int64_t t = (int64_t)blockIdx.x * 32 + lane;
  const int64_t G = s.G, Gp = s.Gp;
  const bool live = t < (int64_t)s.B * G;
  const int b = live ? (int)(t / G) : 0;
  const int64_t g = live ? t % G : 0;
  double S = 0.0, unused = 0.0;
  if (live)
    for (int k = sl; k < s.K; k += DEC_SLICES) chunk_sums1(s, s.seg_chunk[b * s.K + k], 0, g, S);
  dec_combine(sm, sl, lane, S, unused);
  if (sl != 0 || !live) return;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t pos = (int64_t)b * Gp + g;
  S += s.phi_static[pos];
  const float ph = s.phi[pos], pp = s.phi_p[pos];
  const float dl = pp - ph;
  const double lgd0 = (double)lgamma_diff(ph, pp, dl);  // lgamma(pp) - lgamma(ph)
  const double l1 = (double)log_ratio(pp, ph, dl);      // log(pp / ph)
  const double lph = (double)logf(ph);
  // Gamma(1, rate 0.1) prior and Gamma(phi, 1) proposal (BUSseq_gpu.cu:811-814)
  const double prior = (1.0 - (double)ph) * l1 + (double)dl * lph + (1.0 - TAU_PHI) * (double)dl - lgd0;
  const float u = uniform_at(s.seed, SID_PHI_ACC, (uint64_t)t, iter, 0);
  s.lr_phi[(int64_t)b * G + g] = S + prior;
  if ((double)logf(u) <= S + prior) s.phi[pos] = pp;
}

}  // namespace bq
