// Counter-based random numbers and the distribution samplers behind every
// conditional update of the BUSseq Gibbs sweep.
//
// The reference draws from one stored cuRAND XORWOW state per (cell, gene)
// entry (BUSseq_gpu.cu:220-224, 48 bytes each, 4.8 GB at N = G = 10^4) and
// from R's rgamma (BUSseq_gpu.cu:34-197).  This build stores no generator
// state at all: every draw is a pure function of
//     (seed, stream id, entity index, sweep index, block number)
// through Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11).  A conditional update keys its
// stream by the entity it updates (entry i*G+g, gene g, cell i, ...), so the
// draws do not depend on launch shape, thread mapping or processing order,
// and a CPU restatement can consume exactly the same uniforms.
//
// Samplers (all written from the published methods named beside them):
//   normal   : Box-Muller, cosine branch only (Box and Muller 1958)
//   gamma    : Marsaglia and Tsang (2000), with the U^(1/a) boost for a < 1
//   poisson  : sequential inversion for lambda < 10, PTRS transformed
//              rejection with squeeze (Hormann 1993) for lambda >= 10
//   NB       : gamma-Poisson mixture, as the reference's rnbinom
//              (BUSseq_gpu.cu:199-210)
//
// Everything here is single precision on the device; every rejection loop
// has an iteration cap that raises a flag instead of spinning forever.
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define BQ_HD __host__ __device__ __forceinline__
#else
#define BQ_HD inline
#endif

namespace bq {

// ---------------------------------------------------------------------------
// Stream ids: one per kind of random decision in a sweep.
// ---------------------------------------------------------------------------
enum StreamId : uint32_t {
  SID_ZX = 1,            // entry i*G+g : Z Bernoulli, NB proposal, MH accept
  SID_GAMMA = 2,         // batch b     : gamma0 proposal (u0,u1), gamma0 accept (u2), gamma1 accept (u3)
  SID_GAMMA1_PROP = 3,   // batch b     : gamma1 proposal (Gamma draw)
  SID_ALPHA = 4,         // gene g      : proposal (u0,u1), accept (u2)
  SID_L = 5,             // (k-1)*G+g   : indicator L
  SID_P = 6,             // 0           : p ~ Beta (two Gamma draws)
  SID_TAU0 = 7,          // 0           : tau0 (one Gamma draw)
  SID_BETA = 8,          // (k-1)*G+g   : proposal (u0,u1), accept (u2)
  SID_NU = 9,            // (b-1)*G+g   : proposal (u0,u1), accept (u2)
  SID_DELTA = 10,        // cell i      : proposal (u0,u1), accept (u2)
  SID_PHI_PROP = 11,     // b*G+g       : proposal (Gamma draw)
  SID_PHI_ACC = 12,      // b*G+g       : accept (u0)
  SID_W = 13,            // cell i      : proposal / categorical (u0), accept (u1)
  SID_PI = 14,           // b*K+k       : Dirichlet component (Gamma draw)
  SID_HMC_MOM = 15,      // coordinate d: momentum of the HMC block update
  SID_HMC_ACC = 16,      // 0           : HMC accept (u0), step-size jitter (u1);
                         // 1 + gene g  : per-gene accept (u0), the gene's step factor (u1)
  SID_CORRECT = 17,      // entry i*G+g : randomised PIT of the batch-corrected count (two words)
  SID_INIT_W = 20,       // cell i      : initial cell type
  SID_INIT_L = 21,       // k*G+g       : initial indicator L
  SID_SIM = 30,          // synthetic-data generator (not used by the sampler)
  SID_TEST_GAMMA = 40,   // draw j      : busseq_sample_draws (distribution tests), the
  SID_TEST_POISSON = 41, //               same streams as the oracle's sample functions
  SID_TEST_NEGBIN = 42
};

// Iteration caps of the rejection samplers.  Hitting one sets an error bit.
constexpr int GAMMA_MAX_ITER = 64;
constexpr int POISSON_MAX_ITER = 64;
constexpr int POISSON_INV_MAX_K = 256;
constexpr float POISSON_MAX_LAMBDA = 1.0e9f;
enum SamplerErr : int { ERR_GAMMA_CAP = 1, ERR_POISSON_CAP = 2 };

// ---------------------------------------------------------------------------
// Philox4x32-10
// ---------------------------------------------------------------------------
struct U32x4 { uint32_t x, y, z, w; };

BQ_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  hi = __umulhi(a, b);
  lo = a * b;
#else
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
#endif
}

BQ_HD U32x4 philox4x32_10(U32x4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c.x, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
    c = U32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

// Uniform on the open interval (0,1): (2m+1) * 2^-24 with m the top 23 bits.
// Every value is exact in float and in double, so a double-precision
// restatement sees the very same numbers.
BQ_HD float u32_to_unit(uint32_t r) {
  return ((float)(r >> 9) + 0.5f) * 1.1920928955078125e-07f;
}

// Uniform on (0,1) with 53-bit resolution: (2m+1) 2^-53, m = the top 52 bits
// of the 64-bit word (w0, w1).  Exact in double, and so is 1 - v.
BQ_HD double u64_to_unit_d(uint32_t w0, uint32_t w1) {
  const uint64_t m = ((((uint64_t)w0) << 32) | (uint64_t)w1) >> 12;
  return (double)(2 * m + 1) * 1.1102230246251565404236316680908203125e-16;
}

// Counter layout: x = entity bits 0..31, y = entity bits 32..47 | stream<<16,
// z = block number within the stream, w = sweep index.  Key = seed.
struct Stream {
  uint32_t k0, k1, c0, c1, blk, it;
  uint32_t b0, b1, b2, b3;
  int n;
  BQ_HD Stream(uint64_t seed, uint32_t sid, uint64_t entity, uint32_t iter)
      : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), c0((uint32_t)entity),
        c1(((uint32_t)(entity >> 32) & 0xFFFFu) | (sid << 16)), blk(0), it(iter),
        b0(0), b1(0), b2(0), b3(0), n(0) {}
  BQ_HD uint32_t next_u32() {
    if (n == 0) {
      const U32x4 r = philox4x32_10(U32x4{c0, c1, blk, it}, k0, k1);
      ++blk;
      b0 = r.x; b1 = r.y; b2 = r.z; b3 = r.w;
      n = 4;
    }
    const uint32_t v = b0;
    b0 = b1; b1 = b2; b2 = b3;
    --n;
    return v;
  }
  BQ_HD float uniform() { return u32_to_unit(next_u32()); }
  // The stream with block 0 = (w0, w1, w2, w3) already generated; when
  // `skip_first` is set the first word counts as consumed.
  BQ_HD static Stream resume(uint64_t seed, uint32_t sid, uint64_t entity, uint32_t iter, uint32_t w0, uint32_t w1,
                             uint32_t w2, uint32_t w3, bool skip_first) {
    Stream s(seed, sid, entity, iter);
    s.blk = 1;
    s.b0 = skip_first ? w1 : w0;
    s.b1 = skip_first ? w2 : w1;
    s.b2 = skip_first ? w3 : w2;
    s.b3 = w3;
    s.n = skip_first ? 3 : 4;
    return s;
  }
};

// A Stream whose next block is generated ahead of need, at the point of
// construction.  A sampler that runs past the buffered words at different
// draws in different lanes of a warp (a rejection, the U^(1/a) boost, a second
// Poisson try) then takes those words from registers instead of running
// Philox in a divergent branch.  The words and their order are Stream's.
struct StreamAhead {
  Stream s;
  uint32_t a0, a1, a2, a3;
  bool ahead;
  BQ_HD explicit StreamAhead(const Stream& base) : s(base), ahead(true) {
    const U32x4 r = philox4x32_10(U32x4{s.c0, s.c1, s.blk, s.it}, s.k0, s.k1);
    a0 = r.x; a1 = r.y; a2 = r.z; a3 = r.w;
  }
  BQ_HD uint32_t next_u32() {
    if (s.n == 0 && ahead) {
      s.b0 = a0; s.b1 = a1; s.b2 = a2; s.b3 = a3;
      s.n = 4;
      ++s.blk;
      ahead = false;
    }
    return s.next_u32();
  }
  BQ_HD float uniform() { return u32_to_unit(next_u32()); }
};

// ---------------------------------------------------------------------------
// Single-precision math shims (device intrinsics vs. host libm)
// ---------------------------------------------------------------------------
BQ_HD float cospi2f(float u) {  // cos(2*pi*u)
#if defined(__CUDA_ARCH__)
  return cospif(2.0f * u);
#else
  return (float)cos(6.283185307179586 * (double)u);
#endif
}

BQ_HD float bq_lgammaf(float x) {
#if defined(__CUDA_ARCH__)
  return lgammaf(x);
#else
  return (float)lgamma((double)x);
#endif
}

// 1 / b from the hardware reciprocal approximation (rcp.approx.ftz.f32, about
// 1 ulp) and a / b as a times that; b is a positive normal number wherever
// these are used.
BQ_HD float fast_rcp(float b) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return r;
#else
  return 1.0f / b;
#endif
}

BQ_HD float fast_div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return a * fast_rcp(b);
#else
  return a / b;
#endif
}

BQ_HD int float_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_int(x);
#else
  int i;
  memcpy(&i, &x, sizeof i);
  return i;
#endif
}

BQ_HD float bits_float(int i) {
#if defined(__CUDA_ARCH__)
  return __int_as_float(i);
#else
  float x;
  memcpy(&x, &i, sizeof x);
  return x;
#endif
}

// Logarithms without branches or library calls.  A positive normal float is
// split as x = 2^e m with m in [sqrt(1/2), sqrt(2)) by integer arithmetic on
// its bits (0x3F3504F3 is sqrt(1/2)); then
//   log x = e log 2 + log m,   log m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...),
//   s = (m - 1) / (m + 1),  |s| <= 0.1716,
// summed to s^9 (the first omitted term is below 3e-9 relative), with log 2
// split into a 16-bit head and a tail so that e log 2 carries no rounding.
// log_mant takes f = m - 1, which callers may supply exactly.
constexpr float LN2_HI = 0.693145751953125f;
constexpr float LN2_LO = 1.42860682030941723212e-06f;
constexpr int SQRT_HALF_BITS = 0x3F3504F3;

BQ_HD float log_mant(float f, int e) {
  const float s = fast_div(f, 2.0f + f);
  const float t = s * s;
  float p = 2.0f / 9.0f;
  p = fmaf(p, t, 2.0f / 7.0f);
  p = fmaf(p, t, 2.0f / 5.0f);
  p = fmaf(p, t, 2.0f / 3.0f);
  const float lm = fmaf(s * t, p, 2.0f * s);
  const float ef = (float)e;
  return fmaf(ef, LN2_HI, fmaf(ef, LN2_LO, lm));
}

BQ_HD int log_exponent(int bits) { return (bits - SQRT_HALF_BITS) >> 23; }

// log x for a positive normal float x.
BQ_HD float log_fast(float x) {
  const int bits = float_bits(x);
  const int e = log_exponent(bits);
  return log_mant(bits_float(bits - (e << 23)) - 1.0f, e);
}

// log(1 + y) for y > -1.  While 1 + y lies in [sqrt(1/2), sqrt(2)) the
// exponent is 0 and f = y is used as given, so small y loses nothing to the
// rounding of 1 + y; outside that range |log(1 + y)| > 0.34 and the rounding
// of 1 + y (2^-24 relative) is immaterial.
BQ_HD float log1p_fast(float y) {
  const int bits = float_bits(1.0f + y);
  const int e = log_exponent(bits);
  const float f = e == 0 ? y : bits_float(bits - (e << 23)) - 1.0f;
  return log_mant(f, e);
}

// log1p for arguments that are nearly always inside (-0.29, 0.29), where the
// exponent is 0 and log_mant applies directly; others take log1p_fast.  The
// branch is taken uniformly by a warp in the Metropolis sums, whose arguments
// are expm1(step) * p with p in (0, 1).
BQ_HD float log1p_near0(float y) {
  if (fabsf(y) < 0.29f) return log_mant(y, 0);
  return log1p_fast(y);
}

// log(a / b) for a, b > 0 given d = a - b.  With r = a / b: while r lies in
// [sqrt(1/2), sqrt(2)) the mantissa argument is d / b (no cancellation for
// a close to b); otherwise |log r| > 0.34 and r itself is relatively
// accurate, including a << b.  One reciprocal serves both quotients.
BQ_HD float log_ratio(float a, float b, float d) {
  const float rb = fast_rcp(b);
  const int bits = float_bits(a * rb);
  const int e = log_exponent(bits);
  const float f = e == 0 ? d * rb : bits_float(bits - (e << 23)) - 1.0f;
  return log_mant(f, e);
}

// log(1 + c mu / (phi + mu)) for |c| <= 1/2, the per-entry term of every
// random-walk shift of eta (alpha, beta, nu, delta) with c = expm1(step).
// With r = c mu / (phi + mu), log(1 + r) = 2 atanh(s), s = r / (2 + r)
// = c mu / (2 phi + (2 + c) mu): the caller passes cmu = c mu and
// den = 2 phi + (2 + c) mu (one fma), so the term costs one reciprocal.  |s| is
// below 1/3, and the series 2 (s + s^3/3 + ... + s^11/11) leaves out less
// than 1.5e-7 of the value.
BQ_HD float two_atanh_small(float s);
BQ_HD float log1p_shift(float cmu, float den) { return two_atanh_small(fast_div(cmu, den)); }

// 2 atanh(s) for |s| <= 1/3 (the series of log1p_shift): log(a / b) with
// s = (a - b) / (a + b), to 1.5e-7 relative.
BQ_HD float two_atanh_small(float s) {
  const float t = s * s;
  float p = 2.0f / 11.0f;
  p = fmaf(p, t, 2.0f / 9.0f);
  p = fmaf(p, t, 2.0f / 7.0f);
  p = fmaf(p, t, 2.0f / 5.0f);
  p = fmaf(p, t, 2.0f / 3.0f);
  return fmaf(s * t, p, 2.0f * s);
}

// log(k!) for integer-valued k >= 0: exact values below 16, Stirling's series
// (x - 1/2) log x - x + log(2 pi)/2 + 1/(12x) - 1/(360x^3), x = k + 1 >= 17,
// above (truncation error below 1e-9).
BQ_HD float log_factorial(float k) {
  if (k < 16.0f) {
    // log(k!) for k = 0..15, chosen by a branch-free binary select
    const int i = (int)k;
    const float t0[8] = {0.000000000e+00f, 0.000000000e+00f, 6.931471806e-01f, 1.791759469e+00f,
                         3.178053830e+00f, 4.787491743e+00f, 6.579251212e+00f, 8.525161361e+00f};
    const float t1[8] = {1.060460290e+01f, 1.280182748e+01f, 1.510441257e+01f, 1.750230785e+01f,
                         1.998721450e+01f, 2.255216385e+01f, 2.519122118e+01f, 2.789927138e+01f};
    float v = 0.0f;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int j = 0; j < 8; ++j) {
      v = (i == j) ? t0[j] : v;
      v = (i == j + 8) ? t1[j] : v;
    }
    return v;
  }
  const float x = k + 1.0f;
  const float r = fast_rcp(x);
  return (x - 0.5f) * log_fast(x) - x + 0.918938533204672742f + r * (1.0f / 12.0f - (r * r) * (1.0f / 360.0f));
}

// ---------------------------------------------------------------------------
// Samplers
// ---------------------------------------------------------------------------
// Standard normal: z = sqrt(-2 log u1) cos(2 pi u2).  Consumes 2 uniforms.
template <class S>
BQ_HD float normal(S& s) {
  const float u1 = s.uniform();
  const float u2 = s.uniform();
  return sqrtf(-2.0f * log_fast(u1)) * cospi2f(u2);
}

// Gamma(shape a, scale 1), Marsaglia and Tsang (2000).  Each try consumes a
// normal (2 uniforms) and, unless 1 + c z <= 0, one more uniform.  Shapes
// below one draw Gamma(a+1) and multiply by U^(1/a) (one more uniform).
template <class S>
BQ_HD float gamma_mt(S& s, float a, int* err) {
  if (!(a > 0.0f)) return 0.0f;
  const bool boost = a < 1.0f;
  const float aa = boost ? a + 1.0f : a;
  const float d = aa - (1.0f / 3.0f);
  const float c = 1.0f / sqrtf(9.0f * d);
  float x = d;
  int it = 0;
  for (; it < GAMMA_MAX_ITER; ++it) {
    const float z = normal(s);
    float v = 1.0f + c * z;
    if (v <= 0.0f) continue;
    v = v * v * v;
    const float u = s.uniform();
    const float z2 = z * z;
    if (u < 1.0f - 0.0331f * (z2 * z2)) { x = d * v; break; }
    if (log_fast(u) < 0.5f * z2 + d * (1.0f - v + log_fast(v))) { x = d * v; break; }
  }
  if (it == GAMMA_MAX_ITER) *err |= ERR_GAMMA_CAP;
  if (boost) {
    const float u = s.uniform();
    x = x * expf(fast_div(log_fast(u), a));
  }
  return x;
}

// Poisson(lambda).  Inversion below 10 (one uniform), PTRS above (two
// uniforms per try).
template <class S>
BQ_HD int poisson(S& s, float lam, int* err) {
  if (!(lam > 0.0f)) return 0;
  if (lam > POISSON_MAX_LAMBDA) lam = POISSON_MAX_LAMBDA;
  if (lam < 10.0f) {
    const float u = s.uniform();
    float p = expf(-lam);
    float F = p;
    int k = 0;
    while (u > F && k < POISSON_INV_MAX_K) {
      ++k;
      p = p * fast_div(lam, (float)k);
      const float Fn = F + p;
      if (Fn == F) break;  // the cumulative sum stopped growing
      F = Fn;
    }
    return k;
  }
  const float slam = sqrtf(lam);
  const float loglam = log_fast(lam);
  const float b = 0.931f + 2.53f * slam;
  const float a = -0.059f + 0.02483f * b;
  const float invalpha = 1.1239f + 1.1328f / (b - 3.4f);
  const float vr = 0.9277f - 3.6224f / (b - 2.0f);
  for (int it = 0; it < POISSON_MAX_ITER; ++it) {
    const float U = s.uniform() - 0.5f;
    const float V = s.uniform();
    const float us = 0.5f - fabsf(U);
    const float kf = floorf((fast_div(2.0f * a, us) + b) * U + lam + 0.43f);
    if (us >= 0.07f && V <= vr) return (int)kf;
    if (kf < 0.0f || (us < 0.013f && V > us)) continue;
    const float lhs = log_fast(fast_div(V * invalpha, fast_div(a, us * us) + b));
    const float rhs = -lam + kf * loglam - log_factorial(kf);
    if (lhs <= rhs) return (int)kf;
  }
  *err |= ERR_POISSON_CAP;
  return (int)lam;
}

// Negative binomial with mean mu and size phi.
//  * mu < NB_INV_MU and phi >= 1: inversion of the NB distribution function
//    with one uniform, P(0) = (phi / (phi + mu))^phi and
//    P(x+1) = P(x) (phi + x) / (x + 1) * mu / (phi + mu);
//  * otherwise Gamma(phi, mu/phi) then Poisson, as the reference's rnbinom
//    (BUSseq_gpu.cu:199-210).
// Both draw exactly from NB(mu, phi); the switch keeps the common small-mean
// draws to one uniform and a short loop.
constexpr float NB_INV_MU = 32.0f;
constexpr int NB_INV_MAX_K = 1024;
enum : int { ERR_NB_INV_CAP = 4 };

BQ_HD bool negbin_use_inversion(float mu, float phi) { return mu < NB_INV_MU && phi >= 1.0f; }

// e^x from the hardware base-2 exponential (a few ulp, plus the rounding of
// x log2(e): below 1e-5 relative for |x| < 100).
BQ_HD float exp_fast(float x) {
#if defined(__CUDA_ARCH__)
  return __expf(x);
#else
  return expf(x);
#endif
}

// The search of the inversion for a given uniform u: the smallest k with
// u <= F(k), F summed from P(0) = (1 - q)^phi by P(k+1) = P(k) q (phi + k) /
// (k + 1), q = mu / (phi + mu).  The counter is kept in float (exact below
// 2^24).  The search also stops where F no longer grows in single precision
// (u within 2^-24 of 1 past the last representable step); max_k caps it and
// raises ERR_NB_INV_CAP (a test of the failure path passes a small cap).
BQ_HD int negbin_invert_u(float u, float mu, float phi, int* err, int max_k = NB_INV_MAX_K) {
  const float q = fast_div(mu, phi + mu);
  const float qphi = q * phi;
  const float cap = (float)max_k;
  float p = exp_fast(phi * log1p_fast(-q));
  float F = p, k = 0.0f;
  bool grow = true, go = u > F;
  while (go) {
    const float k1 = k + 1.0f;
    p = p * (fmaf(q, k, qphi) * fast_rcp(k1));
    k = k1;
    const float Fn = F + p;
    grow = Fn != F;
    go = u > Fn && grow && k < cap;
    F = Fn;
  }
  if (grow && u > F) *err |= ERR_NB_INV_CAP;  // stopped by the cap
  return (int)k;
}

BQ_HD int negbin_inversion(Stream& s, float mu, float phi, int* err, int max_k = NB_INV_MAX_K) {
  return negbin_invert_u(s.uniform(), mu, phi, err, max_k);
}

template <class S>
BQ_HD int negbin_gamma_poisson(S& s, float mu, float phi, int* err) {
  const float g = gamma_mt(s, phi, err);
  return poisson(s, g * (mu / phi), err);
}

BQ_HD int negbin(Stream& s, float mu, float phi, int* err) {
  return negbin_use_inversion(mu, phi) ? negbin_inversion(s, mu, phi, err) : negbin_gamma_poisson(s, mu, phi, err);
}

// ---------------------------------------------------------------------------
// Numerically stable differences used by every Metropolis ratio
// ---------------------------------------------------------------------------
BQ_HD float softplusf(float t) {
  return t > 0.0f ? t + log1p_fast(expf(-t)) : log1p_fast(expf(t));
}

// softplus(t + dlt) - softplus(t) without cancellation.
BQ_HD float softplus_diff(float t, float dlt) {
  if (fabsf(dlt) < 0.5f) {
    const float sig = 1.0f / (1.0f + expf(-t));
    return log1p_fast(sig * expm1f(dlt));
  }
  return softplusf(t + dlt) - softplusf(t);
}

// log(a / b) as log_ratio, given rb = 1 / b.
BQ_HD float log_ratio_rcp(float a, float rb, float d) {
  const int bits = float_bits(a * rb);
  const int e = log_exponent(bits);
  const float f = e == 0 ? d * rb : bits_float(bits - (e << 23)) - 1.0f;
  return log_mant(f, e);
}

// lgamma(zq) - lgamma(zz) for zz, zq >= 8, dlt = zq - zz, from the
// difference of Stirling's series
//   lgamma(z) = (z - 1/2) log z - z + log(2 pi)/2 + S(z),
//   S(z) = 1/(12z) - 1/(360z^3) + 1/(1260z^5) - ...   (next term < 1e-9 at z = 8)
// rearranged as (zq - 1/2) log(zq / zz) + dlt (log zz - 1) + S(zq) - S(zz).
// With w = 1/(zq zz): 1/zq - 1/zz = -dlt w, and S(zq) - S(zz) factors as
// -dlt w [1/12 - (q + w)/360 + (q^2 + w q - w^2)/1260], q = 1/zq^2 + 1/zz^2,
// so no difference of nearly equal numbers is formed.
BQ_HD float lgamma_diff_large(float zz, float zq, float dlt) {
  const float w = fast_rcp(zz * zq);
  const float rz = zq * w, rq = zz * w;
  const float q = fmaf(rq, rq, rz * rz);
  const float poly = (1.0f / 12.0f) - (q + w) * (1.0f / 360.0f) + fmaf(q, q, w * (q - w)) * (1.0f / 1260.0f);
  const float tail = -dlt * w * poly;
  return fmaf(zq - 0.5f, log_ratio_rcp(zq, rz, dlt), fmaf(dlt, log_fast(zz) - 1.0f, tail));
}

// lgamma(zp) - lgamma(z) for z, zp > 0, dlt = zp - z, without cancellation:
// arguments below 8 are shifted up with lgamma(x+1) = lgamma(x) + log x.
BQ_HD float lgamma_diff(float z, float zp, float dlt) {
  float acc = 0.0f;
  float zz = z, zq = zp;
  for (int j = 0; j < 8 && (zz < 8.0f || zq < 8.0f); ++j) {
    acc -= log_ratio(zq, zz, dlt);
    zz += 1.0f;
    zq += 1.0f;
  }
  return acc + lgamma_diff_large(zz, zq, dlt);
}

}  // namespace bq
