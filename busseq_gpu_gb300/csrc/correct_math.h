// Randomised quantile matching between two negative binomial distributions,
// the arithmetic of the batch-corrected counts (k_correct).  Host + device so
// that the same code compiles for both; FP64 throughout.
//
// NB(mu, phi) in the size parametrisation: P(k) = C(k + phi - 1, k) p^phi q^k,
// p = phi / (phi + mu), q = mu / (phi + mu), F(k) = P(X <= k), S(k) = 1 - F(k).
//
// The count x under the source distribution has the randomised probability
// integral transform u = F(x - 1) + v P(x), v ~ U(0, 1); the corrected count
// is x* = min {k : F*(k) >= u} under the target distribution.  A position u
// is carried as the tail that holds it accurately: (upper = false, t = u) or
// (upper = true, t = 1 - u).  Two regimes:
//  * small counts (at most CORR_SMALL, p^phi representable, the position not
//    in the far upper tail): F summed from k = 0 by the pmf recurrence
//    P(k+1) = P(k) (k + phi) q / (k + 1), absolute error a few ulps per term,
//    so positions in the upper tail are used only down to t = 2^-10 (relative
//    error ~1e-11 there);
//  * otherwise the tail at a point comes from the continued fraction of the
//    regularised incomplete beta function, F(k) = I_p(phi, k + 1),
//    S(k) = I_q(k + 1, phi) (relative error ~1e-12), and the quantile is
//    bracketed with it (exponential steps from a guess, then bisection) and
//    finished by the pmf recurrence in the direction in which the kept tail
//    grows (F upwards, S downwards), so that no step subtracts.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define CQ_HD __host__ __device__
#define CQ_HDI __host__ __device__ __forceinline__
#else
#define CQ_HD inline
#define CQ_HDI inline
#endif

namespace bq {
namespace corr {

constexpr int CORR_SMALL = 64;             // counts whose F is summed from 0
constexpr int CORR_GUESS_SMALL = 40;       // guesses below this start the target walk at 0
constexpr int CORR_WALK = 16;              // brackets at most this wide are finished by the recurrence
constexpr int CORR_CF_MAX = 4096;          // continued-fraction term pairs; convergence takes O(sqrt(max(a, b)))
constexpr int CORR_KMAX = 1 << 30;         // largest corrected count
constexpr double CORR_LOG_TINY = -700.0;   // log P(0) above which the recurrence from 0 starts
constexpr double CORR_T_MIN = 1e-280;      // floor of a tail probability (well inside the normal range)
constexpr double CORR_UPPER_MIN = 1.0 / 1024.0;  // smallest upper tail taken from a forward sum

struct InvTab {
  double v[CORR_SMALL + 1];
};
constexpr InvTab make_inv_tab() {
  InvTab t{};
  for (int j = 0; j <= CORR_SMALL; ++j) t.v[j] = 1.0 / (double)(j + 1);
  return t;
}
#if defined(__CUDACC__)
__constant__ InvTab c_inv_dev = make_inv_tab();  // 1 / (j + 1)
#endif
constexpr InvTab c_inv_host = make_inv_tab();

CQ_HDI double inv_int1(int j) {  // 1 / (j + 1), 0 <= j <= CORR_SMALL
#if defined(__CUDA_ARCH__)
  return c_inv_dev.v[j];
#else
  return c_inv_host.v[j];
#endif
}

struct NbDist {
  double phi, p, q, lp, lq, lg_phi;
  bool have_lg;
  CQ_HDI void set(double mu, double ph) {
    phi = ph;
    p = ph / (ph + mu);
    q = mu / (ph + mu);
    lp = -log1p(mu / ph);
    lq = -log1p(ph / mu);
    have_lg = false;
  }
  CQ_HDI double log_p0() const { return phi * lp; }
  CQ_HDI double lgamma_phi() {  // only the continued-fraction regime needs it
    if (!have_lg) {
      lg_phi = lgamma(phi);
      have_lg = true;
    }
    return lg_phi;
  }
};

struct Tail {
  double t;    // F(k) (upper false) or S(k) (upper true)
  double pmf;  // P(k)
  bool upper;
  CQ_HDI double F() const { return upper ? 1.0 - t : t; }
  CQ_HDI double S() const { return upper ? t : 1.0 - t; }
};

// Continued fraction 26.5.8 of Abramowitz and Stegun for the regularised
// incomplete beta function:
//   I_x(a, b) = x^a (1 - x)^b / (a B(a, b)) / K,  K = 1 + d1 / (1 + d2 / (1 + ...)),
//   d_{2m+1} = -(a + m)(a + b + m) x / ((a + 2m)(a + 2m + 1)),
//   d_{2m}   = m (b - m) x / ((a + 2m - 1)(a + 2m)),
// converging fast for x < (a + 1) / (a + b + 2).  K is evaluated forwards by
// the modified Lentz method (Thompson and Barnett, J. Comput. Phys. 64, 1986).
CQ_HD double inc_beta_cf(double a, double b, double x) {
  const double TINY = 1e-300, EPS = 1e-15;
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

// The tail at k that the continued fraction resolves, with P(k).
// c = p^phi q^(k+1) / B(phi, k + 1) is the common prefactor: F(k) = c / (phi K),
// S(k) = c / ((k + 1) K'), and P(k) = c / (q (phi + k)).
CQ_HD Tail nb_tail(NbDist& d, int k) {
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

// Position of the randomised PIT of x under d.
CQ_HD void source_position(NbDist& d, int x, double v, bool& upper, double& t) {
  if (x <= CORR_SMALL && d.log_p0() > CORR_LOG_TINY) {
    double pm = exp(d.log_p0()), F = 0.0;
    for (int j = 0; j < x; ++j) {
      F += pm;
      pm *= (j + d.phi) * d.q * inv_int1(j);
    }
    const double u = F + v * pm;
    if (u <= 1.0 - CORR_UPPER_MIN) {
      upper = u > 0.5;
      t = fmax(upper ? 1.0 - u : u, CORR_T_MIN);
      return;
    }
  }
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
  t = fmax(t, CORR_T_MIN);
}

// min {k : F(k) >= u} for the position (upper, t) of u, starting from guess k0.
CQ_HD int target_quantile(NbDist& d, bool upper, double t, int k0) {
  if (k0 < CORR_GUESS_SMALL && d.log_p0() > CORR_LOG_TINY && (!upper || t >= CORR_UPPER_MIN)) {
    const double u = upper ? 1.0 - t : t;
    double pm = exp(d.log_p0()), F = pm;
    int j = 0;
    while (F < u && j < CORR_SMALL) {
      pm *= (j + d.phi) * d.q * inv_int1(j);
      ++j;
      F += pm;
    }
    if (F >= u) return j;
    k0 = CORR_SMALL;
  }
  // the answer is the least k with pred(k): F(k) >= t (lower) or S(k) <= t (upper)
  auto pred = [&](const Tail& T) { return upper ? T.S() <= t : T.F() >= t; };
  int lo, hi;  // pred(lo) false (lo = -1: F = 0), pred(hi) true
  Tail Tlo{0.0, 0.0, false}, Thi{0.0, 0.0, false};
  const Tail T0 = nb_tail(d, k0);
  int step = CORR_WALK / 2;
  if (pred(T0)) {
    hi = k0;
    Thi = T0;
    for (;;) {
      lo = hi - step;
      if (lo < 0) {
        lo = -1;
        break;
      }
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
    if (pred(Tm)) {
      hi = mid;
      Thi = Tm;
    } else {
      lo = mid;
      Tlo = Tm;
    }
  }
  if (!upper) {  // F upwards from lo
    double F, pm;
    int j;
    if (lo < 0) {
      j = 0;
      pm = exp(d.log_p0());
      F = pm;
    } else {
      j = lo + 1;
      pm = Tlo.pmf * (lo + d.phi) * d.q / (double)(lo + 1);
      F = Tlo.F() + pm;
    }
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

// The corrected count of x ~ NB(mu, phi) onto NB(mu_t, phi_t) for the uniform v.
CQ_HD int corrected_count(double mu, double phi, double mu_t, double phi_t, int x, double v) {
  NbDist src;
  src.set(mu, phi);
  bool upper;
  double t;
  source_position(src, x, v, upper, t);
  NbDist dst;
  dst.set(mu_t, phi_t);
  // standardised-score guess: mu_t + sd_t (x + 1/2 - mu) / sd
  const double sd = sqrt(mu + mu * mu / phi), sdt = sqrt(mu_t + mu_t * mu_t / phi_t);
  const double guess = mu_t + sdt * (((double)x + 0.5 - mu) / sd);
  const int k0 = !(guess > 0.0) ? 0 : (guess >= (double)CORR_KMAX ? CORR_KMAX : (int)guess);
  return target_quantile(dst, upper, t, k0);
}

}  // namespace corr
}  // namespace bq
