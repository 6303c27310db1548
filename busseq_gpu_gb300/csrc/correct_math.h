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
//    P(k+1) = P(k) (q + (phi - 1) q / (k + 1)) (one fused multiply-add with a
//    table of 1 / (k + 1)), absolute error a few ulps per term,
//    so positions in the upper tail are used only down to t = 2^-10 (relative
//    error ~1e-11 there);
//  * otherwise the tail at a point comes from the continued fraction of the
//    regularised incomplete beta function, F(k) = I_p(phi, k + 1),
//    S(k) = I_q(k + 1, phi) (relative error ~1e-12); the quantile search
//    evaluates it once at a standardised-score guess and walks from there by
//    the pmf recurrence (target_walk), with bracketing and bisection as the
//    fallback for a guess that is far off (target_bracket).
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define CQ_HD __host__ __device__ inline
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
constexpr int CORR_WALK_MAX = 64;          // pmf steps per walk from one continued fraction
constexpr int CORR_ROUNDS = 8;             // walks before falling back to bracketing

struct InvTab {
  double v[CORR_SMALL + 1];
};
constexpr InvTab make_inv_tab() {
  InvTab t{};
  for (int j = 0; j <= CORR_SMALL; ++j) t.v[j] = 1.0 / (double)(j + 1);
  return t;
}
#if defined(__CUDACC__)
static __constant__ InvTab c_inv_dev = make_inv_tab();  // 1 / (j + 1)
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
  double mu, phi, q, lp, p0;  // p0 = P(0) = p^phi
  double cq;                  // (phi - 1) q: P(j+1) / P(j) = q + cq / (j + 1)
  double p, lq, lg_phi;       // continued-fraction regime only (cf_prepare)
  bool cf_ready;
  CQ_HDI void set(double m, double ph) {
    mu = m;
    phi = ph;
    q = m / (ph + m);
    lp = -log1p(m / ph);
    p0 = exp(ph * lp);
    cq = (ph - 1.0) * q;
    cf_ready = false;
  }
  CQ_HDI double log_p0() const { return phi * lp; }
  CQ_HDI void cf_prepare() {
    if (!cf_ready) {
      p = phi / (phi + mu);
      lq = -log1p(phi / mu);
      lg_phi = lgamma(phi);
      cf_ready = true;
    }
  }
};

// Standard deviation of NB(mu, phi): the scale of the quantile guess.
CQ_HDI double nb_sd(double mu, double phi) { return sqrt(mu + mu * mu / phi); }

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
// converging fast for x < (a + 1) / (a + b + 2).  K is the limit of the
// convergents A_j / B_j of the fundamental recurrences
//   A_j = A_{j-1} + d_j A_{j-2},  B_j = B_{j-1} + d_j B_{j-2}
//   (A_{-1} = 1, A_0 = 1, B_{-1} = 0, B_0 = 1),
// carried scaled by the product of the denominators m_1 .. m_j of the
// d_j = n_j / m_j, which turns each step into multiplications only:
//   A'_j = m_j A'_{j-1} + n_j m_{j-1} A'_{j-2}  (likewise B').
// After each pair of terms the four values are divided by B'_j (one division
// per pair), which leaves B'_j = 1 and A'_j = the current convergent.
CQ_HD double inc_beta_cf(double a, double b, double x) {
  const double EPS = 1e-15;
  double Am = 1.0, A = 1.0, Bm = 0.0, B = 1.0, mprev = 1.0, f = 1.0;
  for (int m = 0; m < CORR_CF_MAX; ++m) {
    const double a2m = a + 2.0 * m;
    const double n1 = -(a + m) * (a + b + m) * x, m1 = a2m * (a2m + 1.0);
    double An = m1 * A + (n1 * mprev) * Am, Bn = m1 * B + (n1 * mprev) * Bm;
    Am = A; A = An; Bm = B; B = Bn;
    const double mm = m + 1.0;
    const double n2 = mm * (b - mm) * x, m2 = (a2m + 1.0) * (a2m + 2.0);
    An = m2 * A + (n2 * m1) * Am;
    Bn = m2 * B + (n2 * m1) * Bm;
    Am = A; A = An; Bm = B; B = Bn;
    mprev = m2;
    const double den = fabs(B) > 1e-250 ? B : (B < 0.0 ? -1e-250 : 1e-250);
    const double r = 1.0 / den;
    A *= r; Am *= r; Bm *= r; B *= r;
    const double fn = A;
    const bool done = fabs(fn - f) <= EPS * fabs(fn);
    f = fn;
    if (done) break;
  }
  return f;
}

// The tail at k that the continued fraction resolves, with P(k).
// c = p^phi q^(k+1) / B(phi, k + 1) is the common prefactor: F(k) = c / (phi K),
// S(k) = c / ((k + 1) K'), and P(k) = c / (q (phi + k)).
CQ_HD Tail nb_tail(NbDist& d, int k) {
  d.cf_prepare();
  const double kk = (double)k;
  const double lbeta = d.lg_phi + lgamma(kk + 1.0) - lgamma(d.phi + kk + 1.0);
  const double c = exp(d.phi * d.lp + (kk + 1.0) * d.lq - lbeta);
  Tail r;
  r.pmf = c / (d.q * (d.phi + kk));
  r.upper = !(d.p < (d.phi + 1.0) / (d.phi + kk + 3.0));
  if (!r.upper) r.t = c / (d.phi * inc_beta_cf(d.phi, kk + 1.0, d.p));
  else r.t = c / ((kk + 1.0) * inc_beta_cf(kk + 1.0, d.phi, d.q));
  return r;
}

// Position of the randomised PIT of x under d from the forward sum; false if
// x is out of its range or the position lies in the far upper tail.
CQ_HDI bool source_small(const NbDist& d, int x, double v, bool& upper, double& t) {
  if (x > CORR_SMALL || !(d.log_p0() > CORR_LOG_TINY)) return false;
  double pm = d.p0, F = 0.0;
  for (int j = 0; j < x; ++j) {
    F += pm;
    pm *= fma(d.cq, inv_int1(j), d.q);
  }
  const double u = F + v * pm;
  if (!(u <= 1.0 - CORR_UPPER_MIN)) return false;
  upper = u > 0.5;
  t = fmax(upper ? 1.0 - u : u, CORR_T_MIN);
  return true;
}

// Position of the randomised PIT of x under d from the continued fraction at x.
CQ_HD void source_cf(NbDist& d, int x, double v, bool& upper, double& t) {
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

// min {k : F(k) >= u} by the forward sum from 0, for small guesses; false if
// out of its range (the answer is then above CORR_SMALL or needs the tails).
CQ_HDI bool target_small(const NbDist& d, bool upper, double t, int k0, int& out) {
  if (k0 >= CORR_GUESS_SMALL || !(d.log_p0() > CORR_LOG_TINY) || (upper && t < CORR_UPPER_MIN)) return false;
  const double u = upper ? 1.0 - t : t;
  double pm = d.p0, F = pm;
  int j = 0;
  while (F < u && j < CORR_SMALL) {
    pm *= fma(d.cq, inv_int1(j), d.q);
    ++j;
    F += pm;
  }
  out = j;
  return F >= u;
}

// min {k : F(k) >= u} for the position (upper, t) of u: bracket from k0 by
// exponential steps, bisect with the continued fraction, finish by the pmf
// recurrence in the direction in which the kept tail grows.
CQ_HD int target_bracket(NbDist& d, bool upper, double t, int k0) {
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
      step = step < CORR_KMAX / 4 ? step * 2 : step;
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
      pm = d.p0;
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

// min {k : F(k) >= u}: one continued fraction at the guess k0, then pmf walks
// towards the answer.  A walk in which the kept tail shrinks (F downwards, S
// upwards) subtracts, so it stops once that tail has fallen below 1/1024 of
// the value it started from (relative error then below ~1e-12) and restarts
// from a new continued fraction; a guess that is far off ends in bracketing.
CQ_HD int target_walk(NbDist& d, bool upper, double t, int k0) {
  int k = k0;
  for (int round = 0; round < CORR_ROUNDS; ++round) {
    const Tail T = nb_tail(d, k);
    double pm = T.pmf;
    if (!upper) {
      double F = T.F();
      if (F >= t) {
        const double floor = F * (1.0 / 1024.0);
        for (int n = 0; n < CORR_WALK_MAX; ++n) {  // F(k - 1) = F(k) - P(k)
          if (k == 0) return 0;
          const double Fm = F - pm;
          if (Fm < t) return k;
          pm *= (double)k / ((k - 1 + d.phi) * d.q);
          F = Fm;
          --k;
          if (F < floor) break;
        }
      } else {
        for (int n = 0; n < CORR_WALK_MAX; ++n) {  // F(k + 1) = F(k) + P(k + 1)
          if (k >= CORR_KMAX) return CORR_KMAX;
          pm *= (k + d.phi) * d.q / (double)(k + 1);
          F += pm;
          ++k;
          if (F >= t) return k;
        }
      }
    } else {
      double S = T.S();
      if (S <= t) {
        for (int n = 0; n < CORR_WALK_MAX; ++n) {  // S(k - 1) = S(k) + P(k)
          if (k == 0) return 0;
          S += pm;
          if (S > t) return k;
          pm *= (double)k / ((k - 1 + d.phi) * d.q);
          --k;
        }
      } else {
        const double floor = S * (1.0 / 1024.0);
        for (int n = 0; n < CORR_WALK_MAX; ++n) {  // S(k + 1) = S(k) - P(k + 1)
          if (k >= CORR_KMAX) return CORR_KMAX;
          pm *= (k + d.phi) * d.q / (double)(k + 1);
          S -= pm;
          ++k;
          if (S <= t) return k;
          if (S < floor) break;
        }
      }
    }
  }
  return target_bracket(d, upper, t, k);
}

// The corrected count of x under src onto dst for the uniform v; sd and sd_t
// are the two standard deviations.  FAST_ONLY: return -1 instead of
// evaluating any continued fraction (the caller then repeats the call with
// FAST_ONLY false); a result it does return is the one the full call gives.
template <bool FAST_ONLY>
CQ_HD int corrected_count_t(NbDist& src, NbDist& dst, double sd, double sd_t, int x, double v) {
  bool upper;
  double t;
  if (!source_small(src, x, v, upper, t)) {
    if (FAST_ONLY) return -1;
    source_cf(src, x, v, upper, t);
  }
  // standardised-score guess: mu_t + sd_t (x + 1/2 - mu) / sd
  const double guess = dst.mu + sd_t * (((double)x + 0.5 - src.mu) / sd);
  int k0 = !(guess > 0.0) ? 0 : (guess >= (double)CORR_KMAX ? CORR_KMAX : (int)guess);
  int r;
  if (target_small(dst, upper, t, k0, r)) return r;
  if (FAST_ONLY) return -1;
  if (k0 < CORR_GUESS_SMALL && dst.log_p0() > CORR_LOG_TINY && (!upper || t >= CORR_UPPER_MIN)) k0 = CORR_SMALL;
  return target_walk(dst, upper, t, k0);
}

// The corrected count of x ~ NB(mu, phi) onto NB(mu_t, phi_t) for the uniform v.
CQ_HD int corrected_count(double mu, double phi, double mu_t, double phi_t, int x, double v) {
  NbDist src, dst;
  src.set(mu, phi);
  dst.set(mu_t, phi_t);
  return corrected_count_t<false>(src, dst, nb_sd(mu, phi), nb_sd(mu_t, phi_t), x, v);
}

}  // namespace corr
}  // namespace bq
