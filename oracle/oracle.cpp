// ===========================================================================
// FP64 CPU oracle of the BUSseq Gibbs sweep -- TEST INFRASTRUCTURE ONLY.
//
// This file is the checker.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference arm of bench.py load it; the product library never
// links, loads or calls it.
//
// It restates, in double precision and in plain C++, the conditional updates
// of the reference BUSseq_gpu.cu (Anguscgm/BUSseq_gpu):
//   Z/X            BUSseq_gpu.cu:484-512
//   gamma0/gamma1  BUSseq_gpu.cu:514-600   (driver :1274-1297)
//   alpha          BUSseq_gpu.cu:602-632   (driver :1299-1307)
//   L, p, tau0     BUSseq_gpu.cu:634-668   (driver :1309-1321)
//   beta           BUSseq_gpu.cu:670-707   (driver :1323-1332)
//   nu             BUSseq_gpu.cu:709-737   (driver :1334-1345)
//   delta          BUSseq_gpu.cu:739-778   (driver :1347-1359)
//   phi            BUSseq_gpu.cu:780-818   (driver :1361-1375)
//   W (MH)         BUSseq_gpu.cu:820-854   (driver :1377-1385), plus the K-way
//                  categorical (Gibbs) draw of the same conditional
//   pi             BUSseq_gpu.cu:856-890   (driver :1387-1398)
//   init           BUSseq_gpu.cu:369-482, :1163-1244
//   posterior      BUSseq_gpu.cu:1557-1608, :938-959
//   BIC            BUSseq_gpu.cu:967-1024, :1815-1843
//
// Randomness: the reference uses cuRAND XORWOW and R's rgamma; neither is
// reproduced.  The oracle instead consumes the SAME counter-based uniforms as
// the CUDA kernels (Philox4x32-10 keyed by seed, stream id, entity, sweep),
// restated here independently of the product header, and runs double
// precision versions of the same published samplers (Box-Muller,
// Marsaglia-Tsang gamma, inversion / Hormann PTRS Poisson) in the same
// consumption order.  Every comparison that decides a discrete outcome
// records a normalised margin, so a test can tell a genuine disagreement from
// a near-tie that single-precision kernels may legitimately decide the other
// way.
//
// Parity of the likelihood formulas with the reference itself is pinned by
// golden vectors produced by the reference's own kernels
// (tests/golden/make_ref_golden.py, oracle/ref_harness.cpp).
// ===========================================================================
#include <stdint.h>
#include <math.h>
#include <string.h>
#include <stdlib.h>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---- hyper-parameters: BUSseq_gpu.cu:12-32 --------------------------------
constexpr double TAU0_INIT = 0.005;
constexpr double GAMMA0_INIT = 0.0;
constexpr double GAMMA1_INIT = -0.3;
constexpr double PHI_INIT = 5.0;
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

// ---- stream ids (must agree with the kernels' counter layout) -------------
enum : uint32_t {
  SID_ZX = 1, SID_GAMMA = 2, SID_GAMMA1_PROP = 3, SID_ALPHA = 4, SID_L = 5,
  SID_P = 6, SID_TAU0 = 7, SID_BETA = 8, SID_NU = 9, SID_DELTA = 10,
  SID_PHI_PROP = 11, SID_PHI_ACC = 12, SID_W = 13, SID_PI = 14,
  SID_INIT_W = 20, SID_INIT_L = 21
};

// ---- Philox4x32-10 (Salmon et al., SC'11), restated -----------------------
static inline void philox(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ ctr[1] ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ ctr[3] ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    ctr[0] = n0; ctr[1] = n1; ctr[2] = n2; ctr[3] = n3;
  }
}

struct Stream {
  uint32_t key0, key1, cx, cy, block, iter;
  uint32_t buf[4];
  int used;
  Stream(uint64_t seed, uint32_t sid, uint64_t ent, uint32_t it)
      : key0((uint32_t)(seed & 0xFFFFFFFFu)), key1((uint32_t)(seed >> 32)),
        cx((uint32_t)(ent & 0xFFFFFFFFu)),
        cy((uint32_t)((ent >> 32) & 0xFFFFu) | (sid << 16)), block(0), iter(it), used(4) {}
  uint32_t u32() {
    if (used == 4) {
      uint32_t c[4] = {cx, cy, block, iter};
      philox(c, key0, key1);
      ++block;
      memcpy(buf, c, sizeof(buf));
      used = 0;
    }
    return buf[used++];
  }
  // (2m+1) 2^-24, m = top 23 bits: the same value the kernels use in float.
  double unif() { return ((double)(u32() >> 9) + 0.5) / 8388608.0; }
};

// ---- margins ---------------------------------------------------------------
static inline void mark(double* mg, double diff, double scale) {
  if (!mg) return;
  const double m = fabs(diff) / scale;
  if (m < *mg) *mg = m;
}

// ---- samplers (double precision, same consumption order as the kernels) ---
static double normal(Stream& s) {
  const double u1 = s.unif();
  const double u2 = s.unif();
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925 * u2);
}

static double gamma_mt(Stream& s, double a, double* mg) {
  if (!(a > 0.0)) return 0.0;
  const bool boost = a < 1.0;
  mark(mg, a - 1.0, 1.0);
  const double aa = boost ? a + 1.0 : a;
  const double d = aa - 1.0 / 3.0;
  const double c = 1.0 / sqrt(9.0 * d);
  double x = d;
  for (int it = 0; it < 64; ++it) {
    const double z = normal(s);
    double v = 1.0 + c * z;
    mark(mg, v, 1.0 + fabs(c * z));
    if (v <= 0.0) continue;
    v = v * v * v;
    const double u = s.unif();
    const double z2 = z * z;
    const double sq = 1.0 - 0.0331 * (z2 * z2);
    mark(mg, u - sq, 1.0 + 0.0331 * z2 * z2);
    if (u < sq) { x = d * v; break; }
    const double lhs = log(u);
    const double rhs = 0.5 * z2 + d * (1.0 - v + log(v));
    mark(mg, lhs - rhs, 1.0 + fabs(lhs) + 0.5 * z2 + d * (1.0 + v + fabs(log(v))));
    if (lhs < rhs) { x = d * v; break; }
  }
  if (boost) {
    const double u = s.unif();
    x = x * exp(log(u) / a);
  }
  return x;
}

static int poisson(Stream& s, double lam, double* mg) {
  if (!(lam > 0.0)) return 0;
  if (lam > 1.0e9) lam = 1.0e9;
  mark(mg, lam - 10.0, 10.0);
  if (lam < 10.0) {
    const double u = s.unif();
    double p = exp(-lam);
    double F = p;
    int k = 0;
    for (;;) {
      mark(mg, u - F, 1.0);
      if (!(u > F) || k >= 256) break;
      ++k;
      p = p * (lam / (double)k);
      const double Fn = F + p;
      if (Fn == F) break;
      F = Fn;
    }
    return k;
  }
  const double slam = sqrt(lam);
  const double loglam = log(lam);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < 64; ++it) {
    const double U = s.unif() - 0.5;
    const double V = s.unif();
    const double us = 0.5 - fabs(U);
    const double arg = (2.0 * a / us + b) * U + lam + 0.43;
    const double kf = floor(arg);
    mark(mg, std::min(arg - kf, kf + 1.0 - arg), 1.0 + lam);
    mark(mg, us - 0.07, 1.0);
    mark(mg, V - vr, 1.0);
    if (us >= 0.07 && V <= vr) return (int)kf;
    mark(mg, us - 0.013, 1.0);
    mark(mg, V - us, 1.0);
    if (kf < 0.0 || (us < 0.013 && V > us)) continue;
    const double lhs = log(V) + log(invalpha) - log(a / (us * us) + b);
    const double rhs = -lam + kf * loglam - lgamma(kf + 1.0);
    mark(mg, lhs - rhs, 1.0 + fabs(lhs) + lam + fabs(kf * loglam));
    if (lhs <= rhs) return (int)kf;
  }
  return (int)lam;
}

// NB(mu, phi): inversion of the distribution function when mu < 32 and
// phi >= 1 (one uniform), Gamma-Poisson otherwise; the same method switch as
// the kernels, so both consume the same uniforms.
static int negbin(Stream& s, double mu, double phi, double* mg) {
  mark(mg, mu - 32.0, 32.0);
  mark(mg, phi - 1.0, 1.0);
  if (mu < 32.0 && phi >= 1.0) {
    const double q = mu / (phi + mu);
    double p = exp(phi * log1p(-q));
    double F = p;
    const double u = s.unif();
    int k = 0;
    for (;;) {
      mark(mg, u - F, 1.0);
      if (!(u > F) || k >= 1024) break;
      p = p * (q * ((phi + (double)k) / (double)(k + 1)));
      ++k;
      const double Fn = F + p;
      if (Fn == F) break;
      F = Fn;
    }
    return k;
  }
  const double g = gamma_mt(s, phi, mg);
  return poisson(s, g * (mu / phi), mg);
}

static inline double softplus(double t) {
  return t > 0.0 ? t + log1p(exp(-t)) : log1p(exp(t));
}

// (phi + X) * [log(phi + e^{m + new}) - log(phi + e^{m + old})] - (new - old) X
// is minus the reference's fill_prop_* term; this returns the term itself:
//   (new - old) X + (phi + X) (log(phi + e^{m+old}) - log(phi + e^{m+new}))
static inline double nb_shift_term(double xold, double xnew, double m, double phi, int X) {
  return (xnew - xold) * X + (phi + X) * (log(phi + exp(m + xold)) - log(phi + exp(m + xnew)));
}

// The absolute sizes of nb_shift_term's two pieces.
static inline double nb_shift_scale(double xold, double xnew, double m, double phi, int X) {
  return fabs((xnew - xold) * X) + fabs((phi + X) * (log(phi + exp(m + xold)) - log(phi + exp(m + xnew))));
}

}  // namespace orc

using namespace orc;

extern "C" {

// Full sampler state in double precision.  Layouts follow the reference:
// beta/L [k*G+g], nu/phi [b*G+g], gamma [0/1*B+b], pi [b*K+k], X/Y/Z [i*G+g].
typedef struct orc_state {
  int32_t B, K;
  int64_t G, N;
  const int32_t* n_b;
  const int32_t* Y;
  int32_t* X;
  uint8_t* Z;
  int32_t* W;
  int8_t* L;
  double* alpha;
  double* mu_alpha;
  double* beta;
  double* nu;
  double* mu_nu;      // [B], entry 0 unused (0)
  double* delta;
  double* mu_delta;
  double* phi;
  double* gamma;
  double* pi;
  double* p_tau0;     // [2] = {p, tau0}
  uint64_t seed;
} orc_state;

// Diagnostics of the last stage run.  Any pointer may be NULL.
typedef struct orc_debug {
  double* lr_gamma;   // [2B]  log acceptance ratio (likelihood + prior) of gamma0, gamma1
  double* lr_alpha;   // [G]
  double* lr_beta;    // [K*G] (k >= 1 used)
  double* lr_nu;      // [B*G] (b >= 1 used)
  double* lr_delta;   // [N]
  double* lr_phi;     // [B*G]
  double* lr_W;       // [N]  MH: log ratio; Gibbs: unused
  double* mg_zx;      // [N*G] min normalised margin of the entry's discrete decisions
  double* mg_gamma;   // [2B]  |log u - log r|
  double* mg_alpha;   // [G]
  double* mg_L;       // [K*G]
  double* mg_beta;    // [K*G]
  double* mg_nu;      // [B*G]
  double* mg_delta;   // [N]
  double* mg_phi;     // [B*G]
  double* mg_W;       // [N]
  double* mg_ptau;    // [2]
  double* mg_pi;      // [B*K]
  // Size of the single-precision pieces behind each log ratio: the sum over
  // its entries of the absolute values of the parts a float kernel evaluates
  // term by term (for the eta shifts |(new - old) X| + |(phi + X) log ratio|;
  // for gamma the softplus differences; for phi the lgamma difference, the two
  // log ratios and pn log(pn / po)).  A float evaluation errs by a few units in
  // the last place of each piece, so this bounds the error a correct kernel
  // can make.
  double* sc_gamma;   // [2B]
  double* sc_alpha;   // [G]
  double* sc_beta;    // [K*G]
  double* sc_nu;      // [B*G]
  double* sc_delta;   // [N]
  double* sc_phi;     // [B*G]
  double* sc_W;       // [N]
} orc_debug;

// Stages group the reference's sweep order (BUSseq_gpu.cu:1267-1398) the way
// the kernels do: [Z/X, gamma0, gamma1, alpha, L, p+tau0], [beta, nu], [delta],
// [phi], [W], [pi].
enum { ORC_STAGE_ZX_GAMMA_ALPHA_L = 0, ORC_STAGE_BETA_NU = 1, ORC_STAGE_DELTA = 2,
       ORC_STAGE_PHI = 3, ORC_STAGE_W = 4, ORC_STAGE_PI = 5 };

static inline std::vector<int64_t> batch_offsets(const orc_state* st) {
  std::vector<int64_t> off(st->B + 1, 0);
  for (int b = 0; b < st->B; ++b) off[b + 1] = off[b] + st->n_b[b];
  return off;
}

static inline int batch_of(const std::vector<int64_t>& off, int64_t i) {
  int b = 0;
  while (i >= off[b + 1]) ++b;
  return b;
}

static inline double mu_of(const orc_state* st, int b, int64_t i, int64_t g) {
  const int64_t G = st->G;
  return exp(st->alpha[g] + st->beta[(int64_t)st->W[i] * G + g] + st->nu[b * G + g] + st->delta[i]);
}

// --- Z / X : BUSseq_gpu.cu:484-512 -----------------------------------------
static void stage_zx(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t N = st->N, G = st->G;
  const int B = st->B;
  auto off = batch_offsets(st);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    const double g0 = st->gamma[b], g1 = st->gamma[B + b];
    for (int64_t g = 0; g < G; ++g) {
      const int64_t pos = i * G + g;
      double mg = INFINITY;
      if (st->Y[pos] == 0) {
        Stream s(st->seed, SID_ZX, (uint64_t)pos, (uint32_t)iter);
        int z;
        if (st->X[pos] == 0) {
          const double u = s.unif();
          const double thr = 1.0 / (1.0 + exp(g0));
          mark(&mg, u - thr, 1.0);
          z = u > thr;
        } else {
          z = 1;
        }
        st->Z[pos] = (uint8_t)z;
        if (z) {
          const double mu = mu_of(st, b, i, g);
          const int xn = negbin(s, mu, st->phi[b * G + g], &mg);
          const double u = s.unif();
          // log[(1 + e^{-g0-g1 Xold}) / (1 + e^{-g0-g1 Xnew})]
          const double lr = softplus(-g0 - g1 * st->X[pos]) - softplus(-g0 - g1 * xn);
          const double lu = log(u);
          mark(&mg, lu - lr, 1.0 + fabs(lu) + fabs(lr));
          if (lu <= lr) st->X[pos] = xn;
        } else {
          st->X[pos] = 0;
        }
      }
      if (dbg && dbg->mg_zx) dbg->mg_zx[pos] = mg;
    }
  }
}

// --- gamma0 then gamma1 : BUSseq_gpu.cu:514-600 -----------------------------
static void stage_gamma(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t G = st->G;
  const int B = st->B;
  auto off = batch_offsets(st);
  for (int b = 0; b < B; ++b) {
    Stream s(st->seed, SID_GAMMA, (uint64_t)b, (uint32_t)iter);
    const double u0 = s.unif(), u1 = s.unif();
    const double z = sqrt(-2.0 * log(u0)) * cos(6.283185307179586476925 * u1);
    const double ua0 = s.unif(), ua1 = s.unif();
    double g0 = st->gamma[b];
    const double g1 = st->gamma[B + b];
    const double g0n = g0 + 0.1 * z;
    Stream sg(st->seed, SID_GAMMA1_PROP, (uint64_t)b, (uint32_t)iter);
    const double g1n = -gamma_mt(sg, -10.0 * g1, nullptr) * 0.1;
    const int64_t lo = off[b] * G, hi = off[b + 1] * G;
    // gamma0: sum of (g0n - g0) Z - [sp(g0n + g1 X) - sp(g0 + g1 X)]
    double lr0 = 0.0, sc0 = 0.0;
#pragma omp parallel for reduction(+ : lr0, sc0)
    for (int64_t pos = lo; pos < hi; ++pos) {
      const int X = st->X[pos], Z = st->Z[pos];
      double prop, prev, t;
      t = g0n + g1 * X;
      prop = g0n * Z - softplus(t);
      const double spn = softplus(t);
      t = g0 + g1 * X;
      prev = g0 * Z - softplus(t);
      lr0 += prop - prev;
      sc0 += fabs(spn - softplus(t));
    }
    if (dbg && dbg->sc_gamma) dbg->sc_gamma[b] = sc0;
    const double prior0 = (g0 * g0 - g0n * g0n) / (2.0 * SIGMA2_GAMMA0);
    const double l0 = log(ua0);
    if (dbg && dbg->lr_gamma) dbg->lr_gamma[b] = lr0 + prior0;
    if (dbg && dbg->mg_gamma) dbg->mg_gamma[b] = fabs(l0 - (prior0 + lr0));
    if (l0 <= prior0 + lr0) { g0 = g0n; st->gamma[b] = g0n; }
    // gamma1 with the updated gamma0
    double lr1 = 0.0, sc1 = 0.0;
#pragma omp parallel for reduction(+ : lr1, sc1)
    for (int64_t pos = lo; pos < hi; ++pos) {
      const int X = st->X[pos], Z = st->Z[pos];
      const double prop = g1n * X * Z - softplus(g0 + g1n * X);
      const double prev = g1 * X * Z - softplus(g0 + g1 * X);
      lr1 += prop - prev;
      sc1 += fabs(softplus(g0 + g1n * X) - softplus(g0 + g1 * X));
    }
    if (dbg && dbg->sc_gamma) dbg->sc_gamma[B + b] = sc1;
    const double pv = -g1, nv = -g1n;
    const double prior1 = (KAPPA_GAMMA1 - 1.0) * (log(nv) - log(pv)) + TAU_GAMMA1 * (pv - nv) -
                          lgamma(10.0 * nv) + (10.0 * nv - 1.0) * log(pv) + 10.0 * nv * (log(10.0) + 1.0) +
                          lgamma(10.0 * pv) - (10.0 * pv - 1.0) * log(nv) - 10.0 * pv * (log(10.0) + 1.0);
    const double l1 = log(ua1);
    if (dbg && dbg->lr_gamma) dbg->lr_gamma[B + b] = lr1 + prior1;
    if (dbg && dbg->mg_gamma) dbg->mg_gamma[B + b] = fabs(l1 - (prior1 + lr1));
    if (l1 <= prior1 + lr1) st->gamma[B + b] = g1n;
  }
}

// --- alpha : BUSseq_gpu.cu:602-632 ------------------------------------------
static void stage_alpha(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t N = st->N, G = st->G;
  auto off = batch_offsets(st);
  std::vector<int> bat(N);
  for (int64_t i = 0; i < N; ++i) bat[i] = batch_of(off, i);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    Stream s(st->seed, SID_ALPHA, (uint64_t)g, (uint32_t)iter);
    const double u0 = s.unif(), u1 = s.unif();
    const double z = sqrt(-2.0 * log(u0)) * cos(6.283185307179586476925 * u1);
    const double ua = s.unif();
    const double a = st->alpha[g], an = a + 0.1 * z;
    double lr = 0.0, sc = 0.0;
    for (int64_t i = 0; i < N; ++i) {
      const int b = bat[i];
      const double phi = st->phi[b * G + g];
      const double m = st->beta[(int64_t)st->W[i] * G + g] + st->nu[b * G + g] + st->delta[i];
      lr += nb_shift_term(a, an, m, phi, st->X[i * G + g]);
      sc += nb_shift_scale(a, an, m, phi, st->X[i * G + g]);
    }
    if (dbg && dbg->sc_alpha) dbg->sc_alpha[g] = sc;
    const double ma = st->mu_alpha[g];
    const double prior = ((a - ma) * (a - ma) - (an - ma) * (an - ma)) / (2.0 * SIGMA2_ALPHA);
    const double lu = log(ua);
    if (dbg && dbg->lr_alpha) dbg->lr_alpha[g] = lr + prior;
    if (dbg && dbg->mg_alpha) dbg->mg_alpha[g] = fabs(lu - (lr + prior));
    if (lu <= lr + prior) st->alpha[g] = an;
  }
}

// --- L : BUSseq_gpu.cu:634-648 ----------------------------------------------
static void stage_L(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t G = st->G;
  const int K = st->K;
  const double p = st->p_tau0[0], tau0 = st->p_tau0[1];
#pragma omp parallel for schedule(static)
  for (int64_t pos = G; pos < (int64_t)K * G; ++pos) {
    const double bt = st->beta[pos];
    const double lo = log(p) - log(1.0 - p) - (log(TAU1) - log(tau0)) / 2.0 +
                      bt * bt * (1.0 / (2.0 * tau0) - 1.0 / (2.0 * TAU1));
    Stream s(st->seed, SID_L, (uint64_t)(pos - G), (uint32_t)iter);
    const double u = s.unif();
    const double thr = 1.0 / (1.0 + exp(lo));
    if (dbg && dbg->mg_L) dbg->mg_L[pos] = fabs(u - thr);
    st->L[pos] = (int8_t)(u > thr ? 1 : 0);
  }
}

// --- p, tau0 : BUSseq_gpu.cu:650-668, driver :1313-1321 ---------------------
static void stage_ptau(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t G = st->G;
  const int K = st->K;
  int64_t cnt = 0;
  double bsq = 0.0;
  for (int64_t pos = G; pos < (int64_t)K * G; ++pos) {
    cnt += st->L[pos];
    if (st->L[pos] == 0) bsq += st->beta[pos] * st->beta[pos];
  }
  const double tot = (double)G * (double)(K - 1);
  double mgp = INFINITY, mgt = INFINITY;
  Stream sp(st->seed, SID_P, 0, (uint32_t)iter);
  const double ga = gamma_mt(sp, (double)cnt + A_P, &mgp);
  const double gb = gamma_mt(sp, tot - (double)cnt + B_P, &mgp);
  st->p_tau0[0] = ga / (ga + gb);
  Stream stt(st->seed, SID_TAU0, 0, (uint32_t)iter);
  const double shape = A_TAU0 + (tot - (double)cnt) / 2.0;
  const double rate = B_TAU0 + bsq / 2.0;
  st->p_tau0[1] = 1.0 / (gamma_mt(stt, shape, &mgt) * (1.0 / rate));
  if (dbg && dbg->mg_ptau) { dbg->mg_ptau[0] = mgp; dbg->mg_ptau[1] = mgt; }
}

// --- beta : BUSseq_gpu.cu:670-707 -------------------------------------------
static void stage_beta(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t N = st->N, G = st->G;
  const int K = st->K;
  auto off = batch_offsets(st);
  std::vector<int> bat(N);
  for (int64_t i = 0; i < N; ++i) bat[i] = batch_of(off, i);
  const double tau0 = st->p_tau0[1];
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    std::vector<double> lr(K, 0.0), bn(K, 0.0), ua(K, 0.0);
    for (int k = 1; k < K; ++k) {
      Stream s(st->seed, SID_BETA, (uint64_t)((k - 1) * G + g), (uint32_t)iter);
      const double u0 = s.unif(), u1 = s.unif();
      const double z = sqrt(-2.0 * log(u0)) * cos(6.283185307179586476925 * u1);
      ua[k] = s.unif();
      bn[k] = st->beta[k * G + g] + 0.1 * z;
    }
    std::vector<double> sc(K, 0.0);
    for (int64_t i = 0; i < N; ++i) {
      const int k = st->W[i];
      if (k == 0) continue;
      const int b = bat[i];
      const double m = st->alpha[g] + st->nu[b * G + g] + st->delta[i];
      lr[k] += nb_shift_term(st->beta[k * G + g], bn[k], m, st->phi[b * G + g], st->X[i * G + g]);
      sc[k] += nb_shift_scale(st->beta[k * G + g], bn[k], m, st->phi[b * G + g], st->X[i * G + g]);
    }
    if (dbg && dbg->sc_beta)
      for (int k = 1; k < K; ++k) dbg->sc_beta[k * G + g] = sc[k];
    for (int k = 1; k < K; ++k) {
      const int64_t pos = k * G + g;
      const double bo = st->beta[pos];
      const double var = st->L[pos] == 1 ? TAU1 : tau0;
      const double prior = (bo * bo - bn[k] * bn[k]) / (2.0 * var);
      const double lu = log(ua[k]);
      if (dbg && dbg->lr_beta) dbg->lr_beta[pos] = lr[k] + prior;
      if (dbg && dbg->mg_beta) dbg->mg_beta[pos] = fabs(lu - (lr[k] + prior));
      if (lu <= lr[k] + prior) st->beta[pos] = bn[k];
    }
  }
}

// --- nu : BUSseq_gpu.cu:709-737 ---------------------------------------------
static void stage_nu(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t G = st->G;
  const int B = st->B;
  auto off = batch_offsets(st);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    for (int b = 1; b < B; ++b) {
      const int64_t pos = b * G + g;
      Stream s(st->seed, SID_NU, (uint64_t)((b - 1) * G + g), (uint32_t)iter);
      const double u0 = s.unif(), u1 = s.unif();
      const double z = sqrt(-2.0 * log(u0)) * cos(6.283185307179586476925 * u1);
      const double ua = s.unif();
      const double vo = st->nu[pos], vn = vo + 0.1 * z;
      double lr = 0.0, sc = 0.0;
      for (int64_t i = off[b]; i < off[b + 1]; ++i) {
        const double m = st->alpha[g] + st->beta[(int64_t)st->W[i] * G + g] + st->delta[i];
        lr += nb_shift_term(vo, vn, m, st->phi[pos], st->X[i * G + g]);
        sc += nb_shift_scale(vo, vn, m, st->phi[pos], st->X[i * G + g]);
      }
      if (dbg && dbg->sc_nu) dbg->sc_nu[pos] = sc;
      const double mn = st->mu_nu[b];
      const double prior = ((vo - mn) * (vo - mn) - (vn - mn) * (vn - mn)) / (2.0 * SIGMA2_NU);
      const double lu = log(ua);
      if (dbg && dbg->lr_nu) dbg->lr_nu[pos] = lr + prior;
      if (dbg && dbg->mg_nu) dbg->mg_nu[pos] = fabs(lu - (lr + prior));
      if (lu <= lr + prior) st->nu[pos] = vn;
    }
  }
}

// --- delta : BUSseq_gpu.cu:739-778 ------------------------------------------
static void stage_delta(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t N = st->N, G = st->G;
  auto off = batch_offsets(st);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    if (i == off[b]) continue;  // first cell of each batch stays at 0
    Stream s(st->seed, SID_DELTA, (uint64_t)i, (uint32_t)iter);
    const double u0 = s.unif(), u1 = s.unif();
    const double z = sqrt(-2.0 * log(u0)) * cos(6.283185307179586476925 * u1);
    const double ua = s.unif();
    const double dn = st->delta[i] + 0.1 * z, d = st->delta[i];
    const int k = st->W[i];
    double lr = 0.0, sc = 0.0;
    for (int64_t g = 0; g < G; ++g) {
      const double m = st->alpha[g] + st->beta[(int64_t)k * G + g] + st->nu[b * G + g];
      lr += nb_shift_term(d, dn, m, st->phi[b * G + g], st->X[i * G + g]);
      sc += nb_shift_scale(d, dn, m, st->phi[b * G + g], st->X[i * G + g]);
    }
    if (dbg && dbg->sc_delta) dbg->sc_delta[i] = sc;
    const double md = st->mu_delta[i];
    const double prior = ((d - md) * (d - md) - (dn - md) * (dn - md)) / (2.0 * SIGMA2_DELTA);
    const double lu = log(ua);
    if (dbg && dbg->lr_delta) dbg->lr_delta[i] = lr + prior;
    if (dbg && dbg->mg_delta) dbg->mg_delta[i] = fabs(lu - (lr + prior));
    if (lu <= lr + prior) st->delta[i] = dn;
  }
}

// --- phi : BUSseq_gpu.cu:780-818 --------------------------------------------
static void stage_phi(orc_state* st, int iter, orc_debug* dbg) {
  const int64_t G = st->G;
  const int B = st->B;
  auto off = batch_offsets(st);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    for (int b = 0; b < B; ++b) {
      const int64_t pos = b * G + g;
      Stream sp(st->seed, SID_PHI_PROP, (uint64_t)pos, (uint32_t)iter);
      const double po = st->phi[pos];
      const double pn = gamma_mt(sp, po, nullptr);
      Stream sa(st->seed, SID_PHI_ACC, (uint64_t)pos, (uint32_t)iter);
      const double ua = sa.unif();
      double lr = 0.0, sc = 0.0;
      const double dl = pn - po, c1 = pn * log(pn / po);
      for (int64_t i = off[b]; i < off[b + 1]; ++i) {
        const int X = st->X[i * G + g];
        const double eta = exp(st->alpha[g] + st->beta[(int64_t)st->W[i] * G + g] + st->nu[pos] + st->delta[i]);
        lr += lgamma(pn + X) + pn * log(pn) - lgamma(pn) - (pn + X) * log(pn + eta) + lgamma(po) +
              (po + X) * log(po + eta) - lgamma(po + X) - po * log(po);
        // the same term as a float kernel forms it: h - (pn + X) l1 + c1 - dl l2
        const double h = (lgamma(pn + X) - lgamma(pn)) - (lgamma(po + X) - lgamma(po));
        sc += fabs(h) + fabs((pn + X) * log((pn + eta) / (po + eta))) + fabs(c1) + fabs(dl * log1p(eta / po));
      }
      if (dbg && dbg->sc_phi) dbg->sc_phi[pos] = sc;
      const double prior = (KAPPA_PHI - po) * log(pn) - (KAPPA_PHI - pn) * log(po) + (1.0 - TAU_PHI) * (pn - po) +
                           lgamma(po) - lgamma(pn);
      const double lu = log(ua);
      if (dbg && dbg->lr_phi) dbg->lr_phi[pos] = lr + prior;
      if (dbg && dbg->mg_phi) dbg->mg_phi[pos] = fabs(lu - (lr + prior));
      if (lu <= lr + prior) st->phi[pos] = pn;
    }
  }
}

// --- W : BUSseq_gpu.cu:820-854 (MH) and the K-way categorical --------------
static void stage_W(orc_state* st, int iter, int w_update, orc_debug* dbg) {
  const int64_t N = st->N, G = st->G;
  const int K = st->K;
  auto off = batch_offsets(st);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    const int k = st->W[i];
    Stream s(st->seed, SID_W, (uint64_t)i, (uint32_t)iter);
    if (w_update == 0) {
      const uint32_t r0 = s.u32();
      const int kn = (int)(((uint64_t)r0 * (uint64_t)K) >> 32);
      const double ua = s.unif();
      double lr = 0.0, sc = 0.0;
      for (int64_t g = 0; g < G; ++g) {
        const double m = st->alpha[g] + st->nu[b * G + g] + st->delta[i];
        lr += nb_shift_term(st->beta[(int64_t)k * G + g], st->beta[(int64_t)kn * G + g], m, st->phi[b * G + g],
                            st->X[i * G + g]);
        sc += nb_shift_scale(st->beta[(int64_t)k * G + g], st->beta[(int64_t)kn * G + g], m, st->phi[b * G + g],
                             st->X[i * G + g]);
      }
      if (dbg && dbg->sc_W) dbg->sc_W[i] = sc;
      const double rhs = log(st->pi[b * K + kn] / st->pi[b * K + k]) + lr;
      const double lu = log(ua);
      if (dbg && dbg->lr_W) dbg->lr_W[i] = rhs;
      if (dbg && dbg->mg_W) dbg->mg_W[i] = (kn == k) ? INFINITY : fabs(lu - rhs);
      if (lu <= rhs) st->W[i] = kn;
    } else {
      const double u = s.unif();
      std::vector<double> lp(K, 0.0);
      for (int kk = 0; kk < K; ++kk) {
        if (kk == k) continue;
        double lr = 0.0;
        for (int64_t g = 0; g < G; ++g) {
          const double m = st->alpha[g] + st->nu[b * G + g] + st->delta[i];
          lr += nb_shift_term(st->beta[(int64_t)k * G + g], st->beta[(int64_t)kk * G + g], m, st->phi[b * G + g],
                              st->X[i * G + g]);
        }
        lp[kk] = lr;
      }
      double mx = -INFINITY;
      for (int kk = 0; kk < K; ++kk) {
        lp[kk] += log(st->pi[b * K + kk]);
        mx = std::max(mx, lp[kk]);
      }
      double tot = 0.0;
      for (int kk = 0; kk < K; ++kk) tot += exp(lp[kk] - mx);
      const double target = u * tot;
      double cum = 0.0, mg = INFINITY;
      int pick = K - 1;
      bool done = false;
      for (int kk = 0; kk < K; ++kk) {
        cum += exp(lp[kk] - mx);
        mg = std::min(mg, fabs(cum - target) / tot);
        if (!done && target < cum) { pick = kk; done = true; }
      }
      if (dbg && dbg->mg_W) dbg->mg_W[i] = mg;
      if (dbg && dbg->lr_W) dbg->lr_W[i] = lp[pick] - lp[k];  // log weight of the draw relative to the current type
      if (dbg && dbg->sc_W) {  // size of that log weight's float pieces
        double sc = 0.0;
        for (int64_t g = 0; g < G && pick != k; ++g) {
          const double m = st->alpha[g] + st->nu[b * G + g] + st->delta[i];
          sc += nb_shift_scale(st->beta[(int64_t)k * G + g], st->beta[(int64_t)pick * G + g], m, st->phi[b * G + g],
                               st->X[i * G + g]);
        }
        dbg->sc_W[i] = sc;
      }
      st->W[i] = pick;
    }
  }
}

// --- pi : BUSseq_gpu.cu:856-890 (a correct Dirichlet draw) ------------------
static void stage_pi(orc_state* st, int iter, orc_debug* dbg) {
  const int B = st->B, K = st->K;
  auto off = batch_offsets(st);
  for (int b = 0; b < B; ++b) {
    std::vector<int64_t> cnt(K, 0);
    for (int64_t i = off[b]; i < off[b + 1]; ++i) cnt[st->W[i]]++;
    std::vector<double> gk(K);
    double tot = 0.0;
    for (int k = 0; k < K; ++k) {
      Stream s(st->seed, SID_PI, (uint64_t)(b * K + k), (uint32_t)iter);
      double mg = INFINITY;
      gk[k] = gamma_mt(s, (double)cnt[k] + XI_PI, &mg);
      if (dbg && dbg->mg_pi) dbg->mg_pi[b * K + k] = mg;
      tot += gk[k];
    }
    for (int k = 0; k < K; ++k) st->pi[b * K + k] = gk[k] / tot;
  }
}

int orc_stage(orc_state* st, int stage, int iter, int n_unchanged, int w_update, orc_debug* dbg) {
  switch (stage) {
    case ORC_STAGE_ZX_GAMMA_ALPHA_L:
      stage_zx(st, iter, dbg);
      stage_gamma(st, iter, dbg);
      stage_alpha(st, iter, dbg);
      stage_L(st, iter, dbg);
      if (iter >= n_unchanged) stage_ptau(st, iter, dbg);
      return 0;
    case ORC_STAGE_BETA_NU:
      stage_beta(st, iter, dbg);
      stage_nu(st, iter, dbg);
      return 0;
    case ORC_STAGE_DELTA: stage_delta(st, iter, dbg); return 0;
    case ORC_STAGE_PHI: stage_phi(st, iter, dbg); return 0;
    case ORC_STAGE_W: stage_W(st, iter, w_update, dbg); return 0;
    case ORC_STAGE_PI: stage_pi(st, iter, dbg); return 0;
    default: return -1;
  }
}

// Fine-grained entry points (one reference block each), for unit tests.
int orc_step(orc_state* st, const char* which, int iter, int w_update, orc_debug* dbg) {
  if (!strcmp(which, "zx")) stage_zx(st, iter, dbg);
  else if (!strcmp(which, "gamma")) stage_gamma(st, iter, dbg);
  else if (!strcmp(which, "alpha")) stage_alpha(st, iter, dbg);
  else if (!strcmp(which, "L")) stage_L(st, iter, dbg);
  else if (!strcmp(which, "ptau")) stage_ptau(st, iter, dbg);
  else if (!strcmp(which, "beta")) stage_beta(st, iter, dbg);
  else if (!strcmp(which, "nu")) stage_nu(st, iter, dbg);
  else if (!strcmp(which, "delta")) stage_delta(st, iter, dbg);
  else if (!strcmp(which, "phi")) stage_phi(st, iter, dbg);
  else if (!strcmp(which, "W")) stage_W(st, iter, w_update, dbg);
  else if (!strcmp(which, "pi")) stage_pi(st, iter, dbg);
  else return -1;
  return 0;
}

// One whole sweep in the reference's order (BUSseq_gpu.cu:1267-1398).
int orc_sweep(orc_state* st, int iter, int n_unchanged, int w_update) {
  for (int s = 0; s <= ORC_STAGE_PI; ++s) orc_stage(st, s, iter, n_unchanged, w_update, nullptr);
  return 0;
}

// --- initialisation : BUSseq_gpu.cu:369-482, :1163-1244 ---------------------
// orc_init_given_W: everything of the reference's initialisation that does
// not draw random numbers, for a given W.  delta from library sizes
// (first_delta_W, :419-443), raw means (fill_raw_means + selective_mean,
// :369-382 / :1210-1221), gamma/phi/nu (first_gamma, first_nu_phi), beta
// (first_beta_L without L), alpha = mu_alpha, X = Y, Z = 0, mu_nu (fill_mu_nu +
// mean_on_gpu + first_mu_nu, :1232-1241), mu_delta, pi (first_pi).  Optional
// outputs: raw means [b][k][g] and batch means [b].
int orc_init_given_W(orc_state* st, double* raw_out, double* batch_means_out) {
  const int64_t N = st->N, G = st->G;
  const int B = st->B, K = st->K;
  auto off = batch_offsets(st);
  std::vector<int64_t> lib(N, 0);
#pragma omp parallel for
  for (int64_t i = 0; i < N; ++i) {
    int64_t s = 0;
    for (int64_t g = 0; g < G; ++g) s += st->Y[i * G + g];
    lib[i] = s;
  }
  for (int b = 0; b < B; ++b)
    for (int k = 0; k < K; ++k) st->pi[b * K + k] = (k + 1) / (K * (K + 1) / 2.0);
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    st->delta[i] = log((double)lib[i]) - log((double)lib[off[b]]);
  }
  std::vector<double> raw((size_t)B * K * G, 0.0);
  std::vector<int64_t> cnt((size_t)B * K, 0);
  std::vector<int> bat(N);
  for (int64_t i = 0; i < N; ++i) { bat[i] = batch_of(off, i); cnt[bat[i] * K + st->W[i]]++; }
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    for (int64_t i = 0; i < N; ++i)
      raw[((size_t)bat[i] * K + st->W[i]) * G + g] += log(1.0 + st->Y[i * G + g] / exp(st->delta[i]));
    for (int b = 0; b < B; ++b)
      for (int k = 0; k < K; ++k) {
        const int64_t c = cnt[b * K + k];
        double& r = raw[((size_t)b * K + k) * G + g];
        r = c == 0 ? 0.0 : r / (double)c;
      }
  }
  for (int b = 0; b < B; ++b) { st->gamma[b] = GAMMA0_INIT; st->gamma[B + b] = GAMMA1_INIT; }
  for (int64_t pos = 0; pos < (int64_t)B * G; ++pos) {
    st->phi[pos] = PHI_INIT;
    const int b = (int)(pos / G);
    const int64_t g = pos % G;
    if (b == 0) { st->nu[pos] = 0.0; continue; }
    double t1 = 0.0, t2 = 0.0;
    for (int k = 0; k < K; ++k) {
      t1 += raw[((size_t)b * K + k) * G + g];
      t2 += raw[(size_t)k * G + g];
    }
    st->nu[pos] = (t1 - t2) / K;
  }
  for (int64_t pos = 0; pos < (int64_t)K * G; ++pos)
    st->beta[pos] = pos < G ? 0.0 : raw[pos] - raw[pos % G];
  for (int64_t pos = 0; pos < N * G; ++pos) { st->X[pos] = st->Y[pos]; st->Z[pos] = 0; }
  for (int64_t g = 0; g < G; ++g) { st->alpha[g] = raw[g]; st->mu_alpha[g] = raw[g]; }
  std::vector<double> mb(B, 0.0);
  for (int b = 0; b < B; ++b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s)
    for (int64_t i = off[b]; i < off[b + 1]; ++i)
      for (int64_t g = 0; g < G; ++g) s += log(1.0 + st->Y[i * G + g] / exp(st->delta[i]));
    mb[b] = s / ((double)st->n_b[b] * (double)G);
  }
  st->mu_nu[0] = 0.0;
  for (int b = 1; b < B; ++b) st->mu_nu[b] = mb[b] - mb[0];
  for (int64_t i = 0; i < N; ++i) st->mu_delta[i] = st->delta[i];
  if (raw_out) memcpy(raw_out, raw.data(), sizeof(double) * raw.size());
  if (batch_means_out) memcpy(batch_means_out, mb.data(), sizeof(double) * B);
  return 0;
}

// Full initialisation: W ~ Cat(pi_init) per cell (first_delta_W), the
// deterministic part above, L ~ its prior odds (first_beta_L), p = p0 (the
// caller's value; the reference draws it with srand(seed); rand()), tau0.
int orc_init(orc_state* st, double p0) {
  const int64_t N = st->N, G = st->G;
  const int K = st->K;
  auto off = batch_offsets(st);
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    Stream s(st->seed, SID_INIT_W, (uint64_t)i, 0u);
    const double u = s.unif();
    int k = 0;
    double acc = (0 + 1) / (K * (K + 1) / 2.0);
    while (u > acc && k < K - 1) { ++k; acc += (k + 1) / (K * (K + 1) / 2.0); }
    st->W[i] = k;
    (void)b;
  }
  orc_init_given_W(st, nullptr, nullptr);
  const double log_rat_base = log(p0 / (1.0 - p0)) + (log(TAU0_INIT) - log(TAU1)) / 2.0;
  for (int64_t pos = 0; pos < (int64_t)K * G; ++pos) {
    if (pos < G) { st->L[pos] = 0; continue; }
    const double lr = log_rat_base + st->beta[pos] * st->beta[pos] * (1.0 / TAU0_INIT - 1.0 / TAU1) / 2.0;
    Stream s(st->seed, SID_INIT_L, (uint64_t)pos, 0u);
    st->L[pos] = (int8_t)(s.unif() > 1.0 / (1.0 + exp(lr)) ? 1 : 0);
  }
  st->p_tau0[0] = p0;
  st->p_tau0[1] = TAU0_INIT;
  return 0;
}

// --- BIC : BUSseq_gpu.cu:967-1024 and :1833 ---------------------------------
// Uses the posterior estimates stored in the state's parameter arrays.
// Per-(i,k) partials are returned in ll_ik [k*N+i] when non-NULL.
double orc_bic(const orc_state* st, double* ll_ik) {
  const int64_t N = st->N, G = st->G;
  const int B = st->B, K = st->K;
  auto off = batch_offsets(st);
  std::vector<double> part((size_t)K * N, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t ik = 0; ik < (int64_t)K * N; ++ik) {
    const int k = (int)(ik / N);
    const int64_t i = ik % N;
    const int b = batch_of(off, i);
    const double g0 = st->gamma[b], g1 = st->gamma[B + b];
    double acc = 0.0;
    for (int64_t g = 0; g < G; ++g) {
      const double mu = exp(st->alpha[g] + st->beta[(int64_t)k * G + g] + st->nu[b * G + g] + st->delta[i]);
      const double phi = st->phi[b * G + g];
      const int Y = st->Y[i * G + g];
      const double pbgk = mu / (mu + phi);
      double logp, log1mp;
      if (pbgk < exp(-250.0)) { logp = -250.0; log1mp = log(1.0 - pbgk); }
      else if (1.0 - pbgk < exp(-250.0)) { logp = log(pbgk); log1mp = -250.0; }
      else { logp = log(pbgk); log1mp = log(1.0 - pbgk); }
      if (Y) {
        acc += -log(1.0 + exp(g0 + g1 * Y)) + lgamma(phi + Y) - lgamma(1.0 + Y) - lgamma(phi) + Y * logp +
               phi * log1mp;
      } else {
        const int x_max = (int)(3.0 * mu);
        double s = phi * log1mp;
        for (int x = 1; x < x_max; ++x) {
          const double t = g0 + g1 * x - log(1.0 + exp(g0 + g1 * x)) + lgamma(phi + x) - lgamma(1.0 + x) -
                           lgamma(phi) + x * logp + phi * log1mp;
          if (t > s) s = t + log(1.0 + exp(s - t));
          else s += log(1.0 + exp(t - s));
        }
        acc += s;
      }
    }
    part[(size_t)k * N + i] = acc;
  }
  double ll = 0.0;
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    double mx = part[i];
    for (int k = 1; k < K; ++k) mx = std::max(mx, part[(size_t)k * N + i]);
    double s = 0.0;
    for (int k = 0; k < K; ++k) s += st->pi[b * K + k] * exp(part[(size_t)k * N + i] - mx);
    ll += mx + log(s);
  }
  if (ll_ik) memcpy(ll_ik, part.data(), sizeof(double) * part.size());
  const double nparam = (double)((B + G) * K + 2 * B + G * (B * 2 - 1) + N - B);
  return -2.0 * ll + log((double)G * (double)N) * nparam;
}

// Raw uniforms of one stream, for cross-checking the kernels' generator.
void orc_uniforms(uint64_t seed, uint32_t sid, uint64_t ent, uint32_t iter, int n, double* out) {
  Stream s(seed, sid, ent, iter);
  for (int j = 0; j < n; ++j) out[j] = s.unif();
}

void orc_philox(const uint32_t ctr_in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c[4] = {ctr_in[0], ctr_in[1], ctr_in[2], ctr_in[3]};
  philox(c, k0, k1);
  memcpy(out, c, sizeof(c));
}

// Samplers, exposed for distribution tests of the oracle itself.
void orc_sample_gamma(uint64_t seed, double a, int n, double* out) {
  for (int j = 0; j < n; ++j) {
    Stream s(seed, 40u, (uint64_t)j, 0u);
    out[j] = gamma_mt(s, a, nullptr);
  }
}
void orc_sample_poisson(uint64_t seed, double lam, int n, int32_t* out) {
  for (int j = 0; j < n; ++j) {
    Stream s(seed, 41u, (uint64_t)j, 0u);
    out[j] = poisson(s, lam, nullptr);
  }
}
void orc_sample_negbin(uint64_t seed, double mu, double phi, int n, int32_t* out) {
  for (int j = 0; j < n; ++j) {
    Stream s(seed, 42u, (uint64_t)j, 0u);
    out[j] = negbin(s, mu, phi, nullptr);
  }
}

// Per-term likelihood differences exactly as the reference's fill_prop_*
// kernels write them, for pinning against the reference's own outputs.
double orc_term_shift(double xold, double xnew, double m, double phi, int X) {
  return nb_shift_term(xold, xnew, m, phi, X);
}
double orc_term_phi(double po, double pn, double eta, int X) {
  return lgamma(pn + X) + pn * log(pn) - lgamma(pn) - (pn + X) * log(pn + eta) + lgamma(po) +
         (po + X) * log(po + eta) - lgamma(po + X) - po * log(po);
}
double orc_term_gamma0(double g0o, double g0n, double g1, int X, int Z) {
  return (g0n * Z - softplus(g0n + g1 * X)) - (g0o * Z - softplus(g0o + g1 * X));
}
double orc_term_gamma1(double g0, double g1o, double g1n, int X, int Z) {
  return (g1n * X * Z - softplus(g0 + g1n * X)) - (g1o * X * Z - softplus(g0 + g1o * X));
}

// ---------------------------------------------------------------------------
// Gradient-based block update (Hamiltonian Monte Carlo).  Not in the
// reference: its alpha, beta, nu, delta and phi steps are random-walk
// Metropolis (BUSseq_gpu.cu:602-818).  The target is the same conditional
// density those steps leave invariant, taken jointly over
//   theta = (alpha_g, beta_gk (k >= 1), nu_bg (b >= 1), delta_i (not the first
//            cell of a batch), psi_bg = log phi_bg)
// given X, W, L, p and tau0:
//   log p = sum_{i,g} [lgamma(x + phi) - lgamma(phi) + phi log phi
//                      - (phi + x) log(phi + mu) + x eta]      (eta = log mu)
//         - (alpha - mu_alpha)^2 / (2 sigma2_alpha) - beta^2 / (2 v(L))
//         - (nu - mu_nu)^2 / (2 sigma2_nu) - (delta - mu_delta)^2 / (2 sigma2_delta)
//         + kappa psi - tau_phi e^psi          (Gamma(kappa, rate tau) prior on phi
//                                               and the Jacobian of psi = log phi)
// with v(L) = tau1 if L = 1 else tau0, exactly the priors of the MH steps
// (:625-632, :696-707, :730-737, :763-778, :806-818).  Terms constant in theta
// (lgamma(x + 1)) are dropped.
// ---------------------------------------------------------------------------
double orc_hmc_logpost(const orc_state* st) {
  const int64_t G = st->G, N = st->N;
  const int B = st->B, K = st->K;
  auto off = batch_offsets(st);
  double ll = 0.0;
#pragma omp parallel for reduction(+ : ll) schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    double acc = 0.0;
    for (int64_t g = 0; g < G; ++g) {
      const double x = st->X[i * G + g];
      const double ph = st->phi[b * G + g];
      const double eta = st->alpha[g] + st->beta[(int64_t)st->W[i] * G + g] + st->nu[b * G + g] + st->delta[i];
      const double mu = exp(eta);
      acc += lgamma(x + ph) - lgamma(ph) + ph * log(ph) - (ph + x) * log(ph + mu) + x * eta;
    }
    ll += acc;
  }
  double pr = 0.0;
  const double tau0 = st->p_tau0[1];
  for (int64_t g = 0; g < G; ++g) {
    const double da = st->alpha[g] - st->mu_alpha[g];
    pr -= da * da / (2.0 * SIGMA2_ALPHA);
    for (int k = 1; k < K; ++k) {
      const double bt = st->beta[k * G + g];
      pr -= bt * bt / (2.0 * (st->L[k * G + g] == 1 ? TAU1 : tau0));
    }
    for (int b = 1; b < B; ++b) {
      const double dn = st->nu[b * G + g] - st->mu_nu[b];
      pr -= dn * dn / (2.0 * SIGMA2_NU);
    }
    for (int b = 0; b < B; ++b) {
      const double ph = st->phi[b * G + g];
      pr += KAPPA_PHI * log(ph) - TAU_PHI * ph;
    }
  }
  for (int b = 0; b < B; ++b)
    for (int64_t i = off[b] + 1; i < off[b + 1]; ++i) {
      const double dd = st->delta[i] - st->mu_delta[i];
      pr -= dd * dd / (2.0 * SIGMA2_DELTA);
    }
  return ll + pr;
}

// Gradient of orc_hmc_logpost with respect to theta (psi = log phi), and the
// diagonal metric used by the kernels: the observed information of the
// eta-coordinates, sum phi mu (phi + x) / (phi + mu)^2 over the coordinate's
// entries, and of psi, each plus the prior's curvature.  Fixed
// coordinates (beta_0, nu_0, the first cell of each batch) get gradient 0 and
// metric 1.  Any output pointer may be NULL.
int orc_hmc_grad(const orc_state* st, double* ga, double* gb, double* gn, double* gd, double* gp, double* ma,
                 double* mb, double* mn, double* md, double* mp) {
  const int64_t G = st->G, N = st->N;
  const int B = st->B, K = st->K;
  auto off = batch_offsets(st);
  std::vector<double> sa(G, 0.0), sb((size_t)K * G, 0.0), sn((size_t)B * G, 0.0), sp((size_t)B * G, 0.0);
  std::vector<double> wa(G, 0.0), wb((size_t)K * G, 0.0), wn((size_t)B * G, 0.0), ip((size_t)B * G, 0.0);
  std::vector<double> sd(N, 0.0), wd(N, 0.0);
  // per cell: delta sums; per gene: the rest (cells of a batch in order)
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < G; ++g) {
    for (int b = 0; b < B; ++b) {
      const double ph = st->phi[b * G + g];
      for (int64_t i = off[b]; i < off[b + 1]; ++i) {
        const int k = st->W[i];
        const double x = st->X[i * G + g];
        const double mu = exp(st->alpha[g] + st->beta[(int64_t)k * G + g] + st->nu[b * G + g] + st->delta[i]);
        const double r = ph * (x - mu) / (ph + mu);
        const double w = ph * mu * (ph + x) / ((ph + mu) * (ph + mu));
        sa[g] += r;
        wa[g] += w;
        sb[(size_t)k * G + g] += r;
        wb[(size_t)k * G + g] += w;
        sn[(size_t)b * G + g] += r;
        wn[(size_t)b * G + g] += w;
        double dg = 0.0, tg = 0.0;  // psi(x + phi) - psi(phi), psi'(phi) - psi'(x + phi)
        for (int j = 0; j < (int)x; ++j) {
          dg += 1.0 / (ph + j);
          tg += 1.0 / ((ph + j) * (ph + j));
        }
        const double d1 = dg + log(ph) - log(ph + mu) + (mu - x) / (ph + mu);           // d ll / d phi
        const double d2 = -tg + 1.0 / ph - 2.0 / (ph + mu) + (ph + x) / ((ph + mu) * (ph + mu));  // d2 ll / d phi2
        sp[(size_t)b * G + g] += ph * d1;
        ip[(size_t)b * G + g] -= ph * d1 + ph * ph * d2;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    const int k = st->W[i];
    double s = 0.0, w = 0.0;
    for (int64_t g = 0; g < G; ++g) {
      const double ph = st->phi[b * G + g];
      const double x = st->X[i * G + g];
      const double mu = exp(st->alpha[g] + st->beta[(int64_t)k * G + g] + st->nu[b * G + g] + st->delta[i]);
      s += ph * (x - mu) / (ph + mu);
      w += ph * mu * (ph + x) / ((ph + mu) * (ph + mu));
    }
    sd[i] = s;
    wd[i] = w;
  }
  const double tau0 = st->p_tau0[1];
  for (int64_t g = 0; g < G; ++g) {
    if (ga) ga[g] = sa[g] - (st->alpha[g] - st->mu_alpha[g]) / SIGMA2_ALPHA;
    if (ma) ma[g] = wa[g] + 1.0 / SIGMA2_ALPHA;
    for (int k = 0; k < K; ++k) {
      const int64_t pos = (int64_t)k * G + g;
      const double v = st->L[pos] == 1 ? TAU1 : tau0;
      if (gb) gb[pos] = k == 0 ? 0.0 : sb[pos] - st->beta[pos] / v;
      if (mb) mb[pos] = k == 0 ? 1.0 : wb[pos] + 1.0 / v;
    }
    for (int b = 0; b < B; ++b) {
      const int64_t pos = (int64_t)b * G + g;
      if (gn) gn[pos] = b == 0 ? 0.0 : sn[pos] - (st->nu[pos] - st->mu_nu[b]) / SIGMA2_NU;
      if (mn) mn[pos] = b == 0 ? 1.0 : wn[pos] + 1.0 / SIGMA2_NU;
      const double ph = st->phi[pos];
      if (gp) gp[pos] = sp[pos] + KAPPA_PHI - TAU_PHI * ph;
      if (mp) mp[pos] = ip[pos] + TAU_PHI * ph;
    }
  }
  for (int b = 0; b < B; ++b)
    for (int64_t i = off[b]; i < off[b + 1]; ++i) {
      const bool first = i == off[b];
      if (gd) gd[i] = first ? 0.0 : sd[i] - (st->delta[i] - st->mu_delta[i]) / SIGMA2_DELTA;
      if (md) md[i] = first ? 1.0 : wd[i] + 1.0 / SIGMA2_DELTA;
    }
  return 0;
}

// ---------------------------------------------------------------------------
// Batch-corrected counts.  Not in the reference: the BUSseq method's corrected
// read counts, computed from what the reference writes (_post_X, the
// posterior means, the posterior-mode W; BUSseq_gpu.cu:1557-1813).  Each
// imputed count x of cell i (batch b, type w) and gene g is mapped by
// randomised quantile matching from NB(mu, phi_bg), mu = exp(alpha_g + beta_gw
// + nu_bg + delta_i), to NB(mu*, phi_1g), mu* = exp(alpha_g + beta_gw):
//   u  = F(x - 1) + v P(x),  v from stream 17 (entity i*G+g, sweep 0): the two
//        words w0, w1 give v = (2m + 1) 2^-53, m = the top 52 bits of w0:w1;
//   x* = min {k : F*(k) >= u}.
// Restated by direct summation: every pmf term comes from its own logarithm,
//   log P(k) = lgamma(k + phi) - lgamma(phi) - lgamma(k + 1) + phi log p + k log q,
// p = phi / (phi + mu), q = mu / (phi + mu), and each tail is summed on the side
// of the mode where it is small (lower tails from 0, upper tails outwards), so
// both are accurate to a few ulps per term.  margin[e] is the relative distance
// of the entry's position from the nearer of the two tail values bracketing x*,
// negated where the position lies below 1e-280 and is floored there (as the
// kernel does).
// ---------------------------------------------------------------------------
namespace {
struct NbTerms {
  double phi, lp, lq, lgphi, mode;
  NbTerms(double mu, double ph)
      : phi(ph), lp(-log1p(mu / ph)), lq(-log1p(ph / mu)), lgphi(lgamma(ph)),
        mode(ph > 1.0 ? floor((ph - 1.0) * mu / ph) : 0.0) {}
  double lpmf(double k) const { return lgamma(k + phi) - lgphi - lgamma(k + 1.0) + phi * lp + k * lq; }
  double pmf(double k) const { return exp(lpmf(k)); }
  double lower(int64_t k) const {  // F(k)
    double s = 0.0;
    for (int64_t j = 0; j <= k; ++j) s += pmf((double)j);
    return s;
  }
  double upper(int64_t k) const {  // S(k)
    double s = 0.0;
    for (int64_t j = k + 1;; ++j) {
      const double p = pmf((double)j);
      s += p;
      if ((double)j > mode && (p <= 1e-18 * s || p == 0.0)) break;
    }
    return s;
  }
};
}  // namespace

void orc_corrected_counts(const orc_state* st, int32_t* out, double* margin) {
  const int64_t G = st->G, N = st->N;
  auto off = batch_offsets(st);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < N; ++i) {
    const int b = batch_of(off, i);
    const int w = st->W[i];
    for (int64_t g = 0; g < G; ++g) {
      const int64_t e = i * G + g;
      const int64_t x = st->X[e];
      const double ab = st->alpha[g] + st->beta[(int64_t)w * G + g];
      const double mu = exp((ab + st->nu[b * G + g]) + st->delta[i]);
      Stream s(st->seed, 17u, (uint64_t)e, 0u);
      const uint32_t w0 = s.u32(), w1 = s.u32();
      const uint64_t m = ((((uint64_t)w0) << 32) | (uint64_t)w1) >> 12;
      const double v = (double)(2 * m + 1) * 1.1102230246251565404236316680908203125e-16;
      // position of u: the smaller of F(x-1) + v P(x) and S(x) + (1 - v) P(x)
      const NbTerms src(mu, st->phi[b * G + g]);
      const double px = src.pmf((double)x);
      double Fm, Sx;
      if ((double)x <= src.mode) {
        Fm = x > 0 ? src.lower(x - 1) : 0.0;
        Sx = 1.0 - Fm - px;
      } else {
        Sx = src.upper(x);
        Fm = 1.0 - Sx - px;
      }
      const double ulo = Fm + v * px;
      const bool up = ulo > 0.5;
      const double t_raw = up ? Sx + (1.0 - v) * px : ulo;
      const bool saturated = !(t_raw >= 1e-280);
      const double t = saturated ? 1e-280 : t_raw;
      // quantile under NB(exp(alpha + beta_w), phi_1g)
      const NbTerms dst(exp(ab), st->phi[g]);
      int64_t k;
      double mg;
      if (!up) {
        double F = 0.0, p = 0.0;
        for (k = 0;; ++k) {
          p = dst.pmf((double)k);
          F += p;
          if (F >= t) break;
        }
        mg = std::min(t - (F - p), F - t) / t;
      } else {
        // a point beyond the answer: past the mode with P(k) below 1e-22 t
        const double lthr = log(t) - 50.0;
        int64_t hi = (int64_t)dst.mode + 1, step = 1;
        while (dst.lpmf((double)hi) > lthr) { hi += step; step *= 2; }
        double S = dst.upper(hi);
        k = hi;
        for (;;) {  // S(k - 1) = S(k) + P(k)
          const double p = dst.pmf((double)k);
          if (k == 0 || S + p > t) { mg = k == 0 ? 1.0 : std::min(t - S, S + p - t) / t; break; }
          S += p;
          --k;
        }
      }
      out[e] = (int32_t)k;
      if (margin) margin[e] = saturated ? -mg : mg;
    }
  }
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // extern "C"
