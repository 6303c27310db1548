// The dropout-marginal likelihood of a zero count, in double precision.
//
// For Y = 0 the reference (BUSseq_gpu.cu:990-1003) sums, in log space,
//   S = NB(0) + sum_{x=1}^{x_max-1} NB(x) sigmoid(g0 + g1 x),   x_max = floor(3 mu),
// with NB(x) = Gamma(phi + x) / (Gamma(phi) x!) p^x (1-p)^phi, p = mu / (mu + phi),
// one lgamma-based term and one log-add per x, and the clamps log p >= -250,
// log(1-p) >= -250 (:977-986).  Here the same sum is formed without any
// logarithm inside the loop: with r_x = NB(x) sigmoid(s_x) / NB(0),
// s_x = g0 + g1 x and F_x = exp(s_x),
//   r_x = r_{x-1} a_x b_x,  a_x = (phi + x - 1) / x * p,
//   b_x = e^{g1} (1 + F_{x-1}) / (1 + F_x)     (= sigmoid(s_x) / sigmoid(s_{x-1})),
// kept as R * exp(off) with R rescaled by 2^+-930 whenever it leaves
// [2^-930, 2^930], so neither the NB mode (r can reach e^700) nor a vanishing
// sigmoid under- or overflows.  log S = phi log(1-p) + log(1 + exp(off) sum R).
//
// Early exit, without changing the sum beyond double rounding: for g1 < 0,
// b_y = e^{g1} (1 + F_{y-1}) / (1 + e^{g1} F_{y-1}) grows with F_{y-1}, and F
// decreases, so b_y <= b_{x+1} for every y > x; a_y decreases in y when
// phi > 1 and is at most p when phi <= 1.  So with rho = a_{x+1} b_{x+1} (p
// b_{x+1} when phi <= 1) below 1, every later term is at most r_x rho^k and
// the rest of the series at most r_x rho / (1 - rho).  The loop stops when
// that bound falls below 2^-60 of the running sum (a quarter of double
// precision's rounding unit), or when r has underflowed to exactly 0.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define BQ_BIC_HD __host__ __device__ __forceinline__
#else
#define BQ_BIC_HD inline
#endif

namespace bq {

constexpr int BIC_SERIES_MAX_TERMS = 1 << 24;  // x_max is capped there (mu beyond 5.6e6)
constexpr int BIC_CLASSES = 32;                // series length classes: floor(log2 x_max) < 32

// The same sum term by term in log space (the reference's form, with the NB
// term by its recurrence): used only where the recurrence above does not
// apply, g1 >= 0 (the model's gamma1 is negative) or exp(g0 + g1) beyond 1e300.
BQ_BIC_HD double bic_zero_series_logspace(int x_max, double logp, double lw0, double phi, double g0, double g1) {
  double sacc = lw0, lnb = lw0;
  for (int x = 1; x < x_max; ++x) {
    lnb += log((phi + (double)(x - 1)) / (double)x) + logp;
    const double sx = g0 + g1 * (double)x;
    const double t = (sx > 0.0 ? -log1p(exp(-sx)) : sx - log1p(exp(sx))) + lnb;
    sacc = t > sacc ? t + log1p(exp(sacc - t)) : sacc + log1p(exp(t - sacc));
  }
  return sacc;
}

// log S for a zero count; logp and log1mp already clamped as the reference does.
BQ_BIC_HD double bic_zero_series(double mu, double logp, double log1mp, double phi, double g0, double g1) {
  const double lw0 = phi * log1mp;  // log NB(0)
  const double xm = 3.0 * mu;
  const int x_max = xm > (double)BIC_SERIES_MAX_TERMS ? BIC_SERIES_MAX_TERMS : (int)xm;
  if (x_max <= 1) return lw0;
  if (!(g1 < 0.0) || g0 + g1 > 690.0) return bic_zero_series_logspace(x_max, logp, lw0, phi, g0, g1);
  const double p = exp(logp);
  const double c = exp(g1);                 // e^{g1}
  const double big = 8.7e279, small = 1.0 / 8.7e279;  // 2^930, 2^-930
  const double ln_big = 930.0 * 0.69314718055994530942;
  // x = 1: r_1 = phi p sigmoid(s_1), in log form (the only logarithms of the series)
  const double s1 = g0 + g1;
  const double lsig1 = s1 > 0.0 ? -log1p(exp(-s1)) : s1 - log1p(exp(s1));
  double off = log(phi) + logp + lsig1;
  double R = 1.0, acc = 1.0;
  double F = exp(s1);  // F_1; it only decreases (g1 < 0), and once it underflows b_x is e^{g1}
  for (int x = 1; x + 1 < x_max; ++x) {
    // the factors of step x + 1
    const double xd = (double)x;
    const double a = (phi + xd) / (xd + 1.0) * p;
    const double Fn = F * c;
    const double b = c * (1.0 + F) / (1.0 + Fn);
    const double rho = (phi > 1.0 ? a : p) * b;
    if (R == 0.0 || (rho < 1.0 && R * rho < 8.673617379884035e-19 * acc * (1.0 - rho))) break;  // 2^-60
    F = Fn;
    R *= a * b;
    acc += R;
    if (acc > big) {                        // rescale the frame
      R *= small;
      acc *= small;
      off += ln_big;
    }
  }
  // log(1 + exp(off) acc), the x = 0 term being 1 in this frame
  const double l1 = off + log(acc);
  return lw0 + (l1 > 0.0 ? l1 + log1p(exp(-l1)) : log1p(exp(l1)));
}

// ---------------------------------------------------------------------------
// The same recurrence in float-float arithmetic (an unevaluated sum hi + lo of
// two floats, 48 bits of significand): products exact by fmaf, sums exact by
// TwoSum (Knuth), each result renormalised.  GB300 runs FP64 at a small
// fraction of its FP32 rate, and the double loop above does two divisions per
// term; here a term is about sixty FP32 operations.  Each operation errs by a
// few units of 2^-48 relative, so over the few hundred terms a series takes
// the sum S errs by below 1e-12 relative and log S by below 1e-12 absolute
// (tests/test_bic_series.py checks it against the reference's log-space form).
// The frame is rescaled by 2^+-100 (float range); the loop, its early exit and
// the x = 1 logarithms are the double version's.  Where the float range does
// not hold (exp(g0 + g1) above 2^110, phi above 1e6) it defers to the double
// version.
struct BicFF {
  float hi, lo;
};

BQ_BIC_HD BicFF bff(double v) {
  const float h = (float)v;
  return BicFF{h, (float)(v - (double)h)};
}

BQ_BIC_HD BicFF bff_norm(float s, float e) {  // FastTwoSum, |s| >= |e|
  const float h = s + e;
  return BicFF{h, e - (h - s)};
}

BQ_BIC_HD BicFF bff_add(BicFF a, BicFF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);  // TwoSum error
  return bff_norm(s, e + (a.lo + b.lo));
}

BQ_BIC_HD BicFF bff_add1(BicFF a) {  // a + 1
  return bff_add(a, BicFF{1.0f, 0.0f});
}

BQ_BIC_HD BicFF bff_mul(BicFF a, BicFF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);  // the product's rounding error, exactly
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return bff_norm(p, e);
}

BQ_BIC_HD BicFF bff_rcp(BicFF d) {  // 1 / d: the float reciprocal and one correction step
  const float r = 1.0f / d.hi;
  const float e = fmaf(-d.hi, r, 1.0f) - d.lo * r;  // 1 - d r
  return bff_norm(r, r * e);
}

BQ_BIC_HD BicFF bff_scale(BicFF a, float f) { return BicFF{a.hi * f, a.lo * f}; }  // f a power of two

// The float-float recurrence from x = 1 (r_1 = 1 in the frame): returns the
// frame's sum (the x = 0 term included, as 1) and the number of 2^100
// rescales.  F is e^{s_1}, cf e^{g1}.
struct BicSum {
  BicFF acc;
  int nres;
};

BQ_BIC_HD BicSum bic_ff_loop(int x_max, BicFF pf, BicFF phif, BicFF cf, BicFF F, bool big_phi) {
  const float big = 1.2676506e30f, small = 7.888609e-31f;  // 2^100, 2^-100
  BicFF R{1.0f, 0.0f}, acc{1.0f, 0.0f};
  int nres = 0;
  for (int x = 1; x + 1 < x_max; ++x) {
    const float xf = (float)x;  // exact: x < 2^24
    const BicFF a = bff_mul(bff_mul(bff_add(phif, BicFF{xf, 0.0f}), bff_rcp(BicFF{xf + 1.0f, 0.0f})), pf);
    const BicFF Fn = bff_mul(F, cf);
    const BicFF b = bff_mul(bff_mul(cf, bff_add1(F)), bff_rcp(bff_add1(Fn)));
    const float rho = (big_phi ? a.hi : pf.hi) * b.hi;
    if (R.hi == 0.0f || (rho < 1.0f && R.hi * rho < 8.6736174e-19f * acc.hi * (1.0f - rho))) break;  // 2^-60
    F = Fn;
    R = bff_mul(R, bff_mul(a, b));
    acc = bff_add(acc, R);
    if (acc.hi > big) {  // rescale the frame
      R = bff_scale(R, small);
      acc = bff_scale(acc, small);
      ++nres;
    }
  }
  return BicSum{acc, nres};
}

BQ_BIC_HD double bic_zero_series_ff(double mu, double logp, double log1mp, double phi, double g0, double g1) {
  const double lw0 = phi * log1mp;  // log NB(0)
  const double xm = 3.0 * mu;
  const int x_max = xm > (double)BIC_SERIES_MAX_TERMS ? BIC_SERIES_MAX_TERMS : (int)xm;
  if (x_max <= 1) return lw0;
  if (!(g1 < 0.0) || g0 + g1 > 76.0 || phi > 1.0e6) return bic_zero_series(mu, logp, log1mp, phi, g0, g1);
  const double s1 = g0 + g1;
  const double lsig1 = s1 > 0.0 ? -log1p(exp(-s1)) : s1 - log1p(exp(s1));
  const BicSum r = bic_ff_loop(x_max, bff(exp(logp)), bff(phi), bff(exp(g1)), bff(exp(s1)), phi > 1.0);
  const double off = log(phi) + logp + lsig1 + r.nres * (100.0 * 0.69314718055994530942);
  const double l1 = off + log((double)r.acc.hi + (double)r.acc.lo);
  return lw0 + (l1 > 0.0 ? l1 + log1p(exp(-l1)) : log1p(exp(l1)));
}

// ---------------------------------------------------------------------------
// Double-precision logarithm by table lookup (P. T. P. Tang, "Table-driven
// implementation of the logarithm function in IEEE floating-point
// arithmetic", ACM TOMS 16(4), 1990).  For a positive normal x = 2^e m,
// m in [1, 2), with j the top seven bits of m's fraction, c_j = 1 + (j + 1/2)
// / 128 the centre of m's interval and t_j = fl(1 / c_j):
//   log x = e log 2 - log t_j + log(1 + r),   r = m t_j - 1 (one fma),
// |r| <= 2^-8 (1 + 2^-52), and log(1 + r) = r - r^2/2 + r^3/3 - ... - r^6/6
// leaves out less than |r|^7 / 7 < 2^-58.  log 2 is split as a 42-bit head
// (so that e log 2_head is exact for |e| < 2^11) and its remainder.  The
// result errs by a few units of 2^-53 times max(1, |log x|); it is summed into
// the BIC's double sums, where the library logarithm errs alike.
// The table (t_j, -log t_j) is built once per CTA in shared memory on the
// device, once per process on the host.
constexpr int BIC_LOG_TAB = 128;
constexpr double BIC_LN2_HI = 0x1.62e42fefa38p-1;     // ln 2 rounded to 42 bits
constexpr double BIC_LN2_LO = 5.497923018708371e-14;  // ln 2 - BIC_LN2_HI

BQ_BIC_HD uint64_t bic_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

BQ_BIC_HD double bic_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

// entry j of the table: tab[j] = t_j, tab[BIC_LOG_TAB + j] = -log t_j
BQ_BIC_HD void bic_log_entry(double* tab, int j) {
  const double t = 1.0 / (1.0 + ((double)j + 0.5) / (double)BIC_LOG_TAB);
  tab[j] = t;
  tab[BIC_LOG_TAB + j] = -log(t);
}

BQ_BIC_HD double bic_log(const double* tab, double x) {
  if (!(x >= 2.2250738585072014e-308 && x <= 1.7976931348623157e308)) return log(x);  // not positive normal
  const uint64_t u = bic_bits(x);
  const int e = (int)(u >> 52) - 1023;
  const int j = (int)((u >> 45) & (uint64_t)(BIC_LOG_TAB - 1));
  const double m = bic_from_bits((u & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
  const double r = fma(m, tab[j], -1.0);
  double q = -1.0 / 6.0;
  q = fma(q, r, 1.0 / 5.0);
  q = fma(q, r, -1.0 / 4.0);
  q = fma(q, r, 1.0 / 3.0);
  q = fma(q, r, -1.0 / 2.0);
  const double lp = fma(q * r, r, r);  // log(1 + r)
  const double ed = (double)e;
  return fma(ed, BIC_LN2_HI, tab[BIC_LOG_TAB + j]) + fma(ed, BIC_LN2_LO, lp);
}

// log(1 + s) for s >= 0, to a few units of 2^-53 times max(1, log(1 + s))
// absolute: with w = fl(1 + s), log(1 + s) = log w + log(1 + c / w),
// c = s - (w - 1) (exact while w <= 2; below half an ulp of w beyond), and
// |c / w| <= 2^-53, so log(1 + c / w) = c / w to 2^-106 and a float
// reciprocal of w suffices for it.
BQ_BIC_HD double bic_log1p(const double* tab, double s) {
  const double w = 1.0 + s;
  if (w == 1.0) return s;
  const double c = s - (w - 1.0);
  return bic_log(tab, w) + c * (double)(1.0f / (float)w);
}

// ---------------------------------------------------------------------------
// The zero-count term with its per-cell constants hoisted (the device BIC).
// Per batch: s_1 = g0 + g1, log sigmoid(s_1), sigmoid(s_1), e^{g1} and
// e^{s_1}; per entry mu and phi (and the clamped logs for NB(0)).  The series
// is bic_ff_loop; its closing log(1 + exp(off) acc) is formed as one log1p of
// S = phi p sigmoid(s_1) acc (exp(off) itself is that product), with p = mu /
// (mu + phi) from a reciprocal refined twice by Newton's step (2^-52
// relative), unless the frame was rescaled, when it takes the log form of
// bic_zero_series_ff.  A tiny or subnormal S is absorbed by log1p(S) = S, so
// its relative rounding never matters.
struct BicCell {
  double g0, g1, lsig1, sig1;
  BicFF cf, F1;
  bool ff;  // the float-float recurrence applies (g1 < 0, g0 + g1 <= 76)
};

BQ_BIC_HD BicCell bic_cell(double g0, double g1) {
  BicCell c;
  c.g0 = g0;
  c.g1 = g1;
  const double s1 = g0 + g1;
  c.lsig1 = s1 > 0.0 ? -log1p(exp(-s1)) : s1 - log1p(exp(s1));
  c.sig1 = exp(c.lsig1);
  c.ff = g1 < 0.0 && s1 <= 76.0;
  c.cf = bff(exp(g1));
  c.F1 = bff(c.ff ? exp(s1) : 0.0);
  return c;
}

// mu / q to 2^-52 relative, for 0 < q < 1e30 (the float reciprocal's range)
BQ_BIC_HD double bic_quot(double mu, double q) {
  if (!(q < 1.0e30)) return mu / q;
  double r = (double)(1.0f / (float)q);
  r = fma(r, fma(-q, r, 1.0), r);
  r = fma(r, fma(-q, r, 1.0), r);
  return mu * r;
}

// The series part of a zero count's term, log(1 + exp(off) acc), for an entry
// on the float-float path (c.ff, phi <= 1e6, floor(3 mu) >= 2).  Only a
// rescaled frame (rare) takes logarithms of mu, phi and mu + phi.
BQ_BIC_HD double bic_zero_close(const BicCell& c, const double* tab, double mu, double phi) {
  const double q = mu + phi;
  const double xm = 3.0 * mu;
  const int x_max = xm > (double)BIC_SERIES_MAX_TERMS ? BIC_SERIES_MAX_TERMS : (int)xm;
  const double p = bic_quot(mu, q);
  const BicSum r = bic_ff_loop(x_max, bff(p), bff(phi), c.cf, c.F1, phi > 1.0);
  const double acc = (double)r.acc.hi + (double)r.acc.lo;
  if (r.nres == 0) return bic_log1p(tab, phi * p * c.sig1 * acc);
  const double lq = bic_log(tab, q);
  const double off = (bic_log(tab, phi) - lq) + bic_log(tab, mu) + c.lsig1;  // log(phi p sigmoid(s_1))
  const double l1 = off + r.nres * (100.0 * 0.69314718055994530942) + bic_log(tab, acc);
  return l1 > 0.0 ? l1 + log1p(exp(-l1)) : log1p(exp(l1));
}

// The whole zero-count term: NB(0) and the series (the reference's form where
// the float-float recurrence does not apply).
BQ_BIC_HD double bic_zero_term(const BicCell& c, const double* tab, double mu, double logp, double log1mp,
                               double phi) {
  const double lw0 = phi * log1mp;  // log NB(0)
  const double xm = 3.0 * mu;
  const int x_max = xm > (double)BIC_SERIES_MAX_TERMS ? BIC_SERIES_MAX_TERMS : (int)xm;
  if (x_max <= 1) return lw0;
  if (!c.ff || phi > 1.0e6) return bic_zero_series(mu, logp, log1mp, phi, c.g0, c.g1);
  return lw0 + bic_zero_close(c, tab, mu, phi);
}

}  // namespace bq
