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
// Arithmetic: FP64 throughout (a one-off pass after the chain; tails down to
// 1e-300 stay resolvable).  Each position on the probability scale is kept as
// the tail that carries it accurately: (upper = false, t = F) or
// (upper = true, t = S = 1 - F).  Two regimes:
//  * small counts (x <= 64, p^phi representable): F is summed from k = 0 by the
//    pmf recurrence P(k+1) = P(k) (k + phi) q / (k + 1) with a table of 1/(k+1);
//    absolute error a few ulps per term;
//  * otherwise the tail at a point comes from the continued fraction of the
//    regularised incomplete beta function, F(k) = I_p(phi, k + 1) and
//    S(k) = I_q(k + 1, phi) (p = phi / (phi + mu), q = 1 - p), relative error
//    ~1e-12, and the quantile is bracketed with it (exponential steps from a
//    standardised-score guess, then bisection) and finished by the pmf
//    recurrence in the direction in which the kept tail grows (F upwards,
//    S downwards), so no step subtracts.
#include "busseq_dev.h"
#include "kernels.h"
#include "rng.h"

namespace bq {

namespace {

constexpr int CORR_SMALL = 64;        // counts whose F is summed from 0
constexpr int CORR_GUESS_SMALL = 40;  // guesses below this start the target walk at 0
constexpr int CORR_WALK = 16;         // brackets at most this wide are finished by the recurrence
constexpr int CORR_CF_MAX = 4096;     // continued-fraction terms; convergence takes O(sqrt(max(a, b)))
constexpr int CORR_KMAX = 1 << 30;    // largest corrected count
constexpr double CORR_LOG_TINY = -700.0;  // log P(0) above which the recurrence from 0 starts
constexpr double CORR_T_MIN = 1e-300;     // floor of a tail probability

struct InvTab {
  double v[CORR_SMALL + 1];
};
constexpr InvTab make_inv_tab() {
  InvTab t{};
  for (int j = 0; j <= CORR_SMALL; ++j) t.v[j] = 1.0 / (double)(j + 1);
  return t;
}
__constant__ InvTab c_inv = make_inv_tab();  // 1 / (j + 1)

// NB(mu, phi) in the size parametrisation, P(k) = C(k + phi - 1, k) p^phi q^k.
struct NbDist {
  double phi, p, q, lp, lq, lg_phi;
  bool have_lg;
  __device__ void set(double mu, double ph) {
    phi = ph;
    p = ph / (ph + mu);
    q = mu / (ph + mu);
    lp = -log1p(mu / ph);
    lq = -log1p(ph / mu);
    have_lg = false;
  }
  __device__ double log_p0() const { return phi * lp; }
  __device__ double lgamma_phi() {  // only the continued-fraction regime needs it
    if (!have_lg) { lg_phi = lgamma(phi); have_lg = true; }
    return lg_phi;
  }
};

struct Tail {
  double t;    // F(k) (upper false) or S(k) = 1 - F(k) (upper true)
  double pmf;  // P(k)
  bool upper;
  __device__ double F() const { return upper ? 1.0 - t : t; }
  __device__ double S() const { return upper ? t : 1.0 - t; }
};

// Continued fraction 26.5.8 of Abramowitz and Stegun for the regularised
// incomplete beta function:
//   I_x(a, b) = x^a (1 - x)^b / (a B(a, b)) / K,  K = 1 + d1 / (1 + d2 / (1 + ...)),
//   d_{2m+1} = -(a + m)(a + b + m) x / ((a + 2m)(a + 2m + 1)),
//   d_{2m}   = m (b - m) x / ((a + 2m - 1)(a + 2m)),
// converging fast for x < (a + 1) / (a + b + 2).  K is evaluated forwards by
// the modified Lentz method (Thompson and Barnett, J. Comput. Phys. 64, 1986).
__device__ double inc_beta_cf(double a, double b, double x) {
  constexpr double TINY = 1e-300, EPS = 1e-15;
  double f = 1.0, C = 1.0, D = 0.0;
  for (int m = 0; m < CORR_CF_MAX; ++m) {
    const double a2m = a + 2.0 * m;
    double d = -(a + m) * (a + b + m) * x / (a2m * (a2m + 1.0));
    D = 1.0 + d * D;
    if (fabs(D) < TINY) D = TINY;
    C = 1.0 + d / C;
    if (fabs(C) < TINY) C = TINY;
    D = 1.0 / D;
    const double del1 = C * D;
    f *= del1;
    const double m1 = m + 1.0;
    d = m1 * (b - m1) * x / ((a2m + 1.0) * (a2m + 2.0));
    D = 1.0 + d * D;
    if (fabs(D) < TINY) D = TINY;
    C = 1.0 + d / C;
    if (fabs(C) < TINY) C = TINY;
    D = 1.0 / D;
    const double del2 = C * D;
    f *= del2;
    if (fabs(del1 - 1.0) < EPS && fabs(del2 - 1.0) < EPS) break;
  }
  return f;
}

// The tail of NB at k that the continued fraction resolves, with P(k).
// c = p^phi q^(k+1) / B(phi, k + 1) is the common prefactor: F(k) = c / (phi K),
// S(k) = c / ((k + 1) K'), and P(k) = c / (q (phi + k)).
__device__ Tail nb_tail(NbDist& d, int k) {
  const double kk = (double)k;
  const double lbeta = d.lgamma_phi() + lgamma(kk + 1.0) - lgamma(d.phi + kk + 1.0);
  const double c = exp(d.phi * d.lp + (kk + 1.0) * d.lq - lbeta);
  Tail r;
  r.pmf = c / (d.q * (d.phi + kk));
  r.upper = !(d.p < (d.phi + 1.0) / (d.phi + kk + 3.0));
  if (!r.upper) r.t = c / (d.phi * inc_beta_cf(d.phi, kk + 1.0, d.p));
  else r.t = c / ((kk + 1.0) * inc_beta_cf(kk + 1.0, d.phi, d.q));
  return r;
}

// Position of the randomised PIT of x under d, as the smaller tail.
__device__ void source_position(NbDist& d, int x, double v, bool& upper, double& t) {
  if (x <= CORR_SMALL && d.log_p0() > CORR_LOG_TINY) {
    double pm = exp(d.log_p0()), F = 0.0;
    for (int j = 0; j < x; ++j) {
      F += pm;
      pm *= (j + d.phi) * d.q * c_inv.v[j];
    }
    const double u = F + v * pm;
    upper = u > 0.5;
    t = upper ? 1.0 - u : u;
  } else {
    const Tail T = nb_tail(d, x);
    const double w = 1.0 - v;  // exact
    if (!T.upper) {
      const double ulo = T.t - w * T.pmf;  // F(x - 1) + v P(x)
      upper = ulo > 0.5;
      t = upper ? 1.0 - ulo : ulo;
    } else {
      const double shi = T.t + w * T.pmf;  // S(x - 1) - v P(x)
      upper = shi <= 0.5;
      t = upper ? shi : 1.0 - shi;
    }
  }
  t = fmax(t, CORR_T_MIN);
}

// min {k : F(k) >= u} for the position (upper, t) of u, starting from guess k0.
__device__ int target_quantile(NbDist& d, bool upper, double t, int k0) {
  if (k0 < CORR_GUESS_SMALL && d.log_p0() > CORR_LOG_TINY) {
    const double u = upper ? 1.0 - t : t;
    double pm = exp(d.log_p0()), F = pm;
    int j = 0;
    while (F < u && j < CORR_SMALL) {
      pm *= (j + d.phi) * d.q * c_inv.v[j];
      ++j;
      F += pm;
    }
    if (F >= u) return j;
    k0 = CORR_SMALL;
  }
  // predicate of the answer: k >= x*  <=>  F(k) >= u  <=>  S(k) <= t (upper)
  auto pred = [&](const Tail& T) { return upper ? T.S() <= t : T.F() >= t; };
  int lo, hi;  // pred(lo) false (lo = -1: F = 0), pred(hi) true
  Tail Tlo{}, Thi{};
  Tail T0 = nb_tail(d, k0);
  int step = CORR_WALK / 2;
  if (pred(T0)) {
    hi = k0;
    Thi = T0;
    for (;;) {
      lo = hi - step;
      if (lo < 0) { lo = -1; break; }
      Tlo = nb_tail(d, lo);
      if (!pred(Tlo)) break;
      hi = lo;
      Thi = Tlo;
      step *= 2;
    }
  } else {
    lo = k0;
    Tlo = T0;
    for (;;) {
      hi = (lo > CORR_KMAX - step) ? CORR_KMAX : lo + step;
      Thi = nb_tail(d, hi);
      if (pred(Thi)) break;
      if (hi == CORR_KMAX) return CORR_KMAX;
      lo = hi;
      Tlo = Thi;
      step = step < CORR_KMAX / 4 ? step * 2 : step;
    }
  }
  while (hi - lo > CORR_WALK) {
    const int mid = lo + (hi - lo) / 2;
    const Tail Tm = nb_tail(d, mid);
    if (pred(Tm)) { hi = mid; Thi = Tm; } else { lo = mid; Tlo = Tm; }
  }
  if (!upper) {
    // F upwards from lo
    double F, pm;
    int j;
    if (lo < 0) { j = 0; pm = exp(d.log_p0()); F = pm; }
    else { j = lo + 1; pm = Tlo.pmf * (lo + d.phi) * d.q / (double)(lo + 1); F = Tlo.F() + pm; }
    for (; j < hi; ++j) {
      if (F >= t) return j;
      pm *= (j + d.phi) * d.q / (double)(j + 1);
      F += pm;
    }
    return hi;
  }
  // S downwards from hi: S(j - 1) = S(j) + P(j)
  double S = Thi.S(), pm = Thi.pmf;
  for (int j = hi; j > lo + 1; --j) {
    S += pm;
    if (S > t) return j;
    pm *= (double)j / ((j - 1 + d.phi) * d.q);
  }
  return lo + 1;
}

}  // namespace

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
    const double mus = exp(ab);
    Stream st(s.seed, SID_CORRECT, (uint64_t)(i * s.G + g), 0u);
    const uint32_t w0 = st.next_u32();
    const uint32_t w1 = st.next_u32();
    const double v = u64_to_unit_d(w0, w1);
    NbDist src;
    src.set(mu, e.phi[(int64_t)b * s.G + g]);
    bool upper;
    double t;
    source_position(src, x, v, upper, t);
    NbDist dst;
    dst.set(mus, phi1);
    // standardised-score guess: mu* + sd* (x + 1/2 - mu) / sd
    const double sd = sqrt(mu + mu * mu / src.phi), sds = sqrt(mus + mus * mus / phi1);
    const double guess = mus + sds * (((double)x + 0.5 - mu) / sd);
    const int k0 = !(guess > 0.0) ? 0 : (guess >= (double)CORR_KMAX ? CORR_KMAX : (int)guess);
    out[i * ld + g] = target_quantile(dst, upper, t, k0);
  }
}

}  // namespace bq
