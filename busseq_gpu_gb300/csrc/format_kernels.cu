// Text formatting of large tables on the device, for the output files whose
// size scales with N x G or with the kept sweeps (_post_X.txt, _post_Z.txt,
// _corrected_X.txt, _preserved_*.txt).  The layout is the host writer's (and
// the reference's, BUSseq_gpu.cu:1610-2018): a tab between the columns of a
// row and a newline at its end; integers in decimal, floating-point values as
// printf("%f") prints them.
//
// Two passes, one CTA per row: k_fmt_row_len measures each row's text, the host
// turns the lengths into offsets, and k_fmt_rows writes every row at its
// offset -- each thread takes a contiguous run of the row's entries, a CTA-wide
// scan of the runs' lengths places them, and the thread writes its run.
//
// "%f" of a float value v = m 2^e (m < 2^24): printf rounds the exact value to
// six decimals, ties to even; here R = v 10^6 is formed exactly in 64-bit
// integers (m 10^6 < 2^44) and rounded the same way, which covers |v| < 2^43.
// Larger magnitudes raise a flag and the host writer formats that file.
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace bq {

namespace {

constexpr int FMT_THREADS = 256;

__device__ __forceinline__ int dec_len_u(uint64_t u) {
  int n = 1;
  while (u >= 10u) {
    u /= 10u;
    ++n;
  }
  return n;
}

// Writes the last len decimal digits of u (zero-padded) at [p, p + len).
__device__ __forceinline__ void dec_put_u(uint64_t u, char* p, int len) {
  for (int i = len - 1; i >= 0; --i) {
    p[i] = (char)('0' + (int)(u % 10u));
    u /= 10u;
  }
}

// One entry of a float table in "%f": sign, integer part, six decimals, or
// the special forms; *bad set for magnitudes this path does not cover.
struct F6 {
  bool neg, special;
  uint64_t ipart;
  uint32_t frac;
  int special_kind;  // 0 nan, 1 inf
};

__device__ __forceinline__ F6 f6_split(float v, int* bad) {
  F6 f{};
  const uint32_t bits = __float_as_uint(v);
  f.neg = (bits >> 31) != 0;
  const int E = (int)((bits >> 23) & 0xFF);
  const uint32_t frac23 = bits & 0x7FFFFFu;
  if (E == 0xFF) {
    f.special = true;
    f.special_kind = frac23 ? 0 : 1;
    return f;
  }
  const uint64_t m = E ? (uint64_t)(frac23 | 0x800000u) : (uint64_t)frac23;
  const int e = E ? E - 150 : -149;
  const uint64_t t = m * 1000000ull;  // < 2^44
  uint64_t R;
  if (e >= 0) {
    if (e > 19) {
      *bad = 1;
      return f;
    }
    R = t << e;
  } else {
    const int sh = -e;
    if (sh >= 64) {
      R = 0;  // t < 2^44 is below half a unit
    } else {
      const uint64_t q = t >> sh, rem = t & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
      R = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
    }
  }
  f.ipart = R / 1000000ull;
  f.frac = (uint32_t)(R % 1000000ull);
  return f;
}

__device__ __forceinline__ int f6_len(const F6& f) {
  if (f.special) return (f.neg ? 1 : 0) + 3;
  return (f.neg ? 1 : 0) + dec_len_u(f.ipart) + 7;
}

__device__ __forceinline__ void f6_put(const F6& f, char* p, int len) {
  if (f.neg) *p++ = '-';
  if (f.special) {
    const char* w = f.special_kind ? "inf" : "nan";
    p[0] = w[0];
    p[1] = w[1];
    p[2] = w[2];
    return;
  }
  const int il = len - (f.neg ? 1 : 0) - 7;
  dec_put_u(f.ipart, p, il);
  p[il] = '.';
  dec_put_u(f.frac, p + il + 1, 6);
}

// Value of entry (r, c) as text: its length (and, with out, the characters).
__device__ __forceinline__ int fmt_entry(const FmtSrc& src, int64_t r, int64_t c, char* out, int* bad) {
  const int64_t k = r * src.sr + c * src.sc;
  int64_t iv;
  switch (src.kind) {
    case FMT_F32: {
      const F6 f = f6_split(static_cast<const float*>(src.p)[k], bad);
      const int len = f6_len(f);
      if (out) f6_put(f, out, len);
      return len;
    }
    case FMT_I8: iv = static_cast<const int8_t*>(src.p)[k]; break;
    case FMT_I16: iv = static_cast<const int16_t*>(src.p)[k]; break;
    default: iv = static_cast<const int32_t*>(src.p)[k]; break;
  }
  const uint64_t u = iv < 0 ? (uint64_t)(-iv) : (uint64_t)iv;
  const int dl = dec_len_u(u), len = dl + (iv < 0 ? 1 : 0);
  if (out) {
    if (iv < 0) out[0] = '-';
    dec_put_u(u, out + (iv < 0 ? 1 : 0), dl);
  }
  return len;
}

// The run of columns [c0, c1) of thread t in a row of `cols` entries.
__device__ __forceinline__ void run_of(int64_t cols, int t, int64_t& c0, int64_t& c1) {
  const int64_t per = (cols + FMT_THREADS - 1) / FMT_THREADS;
  c0 = (int64_t)t * per;
  c1 = c0 + per < cols ? c0 + per : cols;
  if (c0 > cols) c0 = cols;
}

// Exclusive CTA-wide scan of one int64 per thread; returns the thread's prefix
// and writes the total to *total.
__device__ int64_t cta_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sum[FMT_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  int64_t before = 0, all = 0;
  for (int w = 0; w < FMT_THREADS / 32; ++w) {
    if (w < warp) before += warp_sum[w];
    all += warp_sum[w];
  }
  __syncthreads();
  *total = all;
  return before + incl - v;
}

}  // namespace

// row_len[r] = length of row r's text, separators and newline included; *bad
// set if an entry is outside what the device formatter covers.
__global__ void __launch_bounds__(FMT_THREADS) k_fmt_row_len(FmtSrc src, int64_t cols, int64_t* row_len, int* bad) {
  const int64_t r = blockIdx.x;
  int64_t c0, c1;
  run_of(cols, threadIdx.x, c0, c1);
  int64_t n = 0;
  int b = 0;
  for (int64_t c = c0; c < c1; ++c) n += fmt_entry(src, r, c, nullptr, &b) + 1;
  if (b) atomicOr(bad, 1);
  int64_t total;
  cta_exclusive_scan(n, &total);
  if (threadIdx.x == 0) row_len[r] = total;
}

// Writes row r at out + row_off[r].
__global__ void __launch_bounds__(FMT_THREADS) k_fmt_rows(FmtSrc src, int64_t cols, const int64_t* row_off,
                                                          char* out) {
  const int64_t r = blockIdx.x;
  int64_t c0, c1;
  run_of(cols, threadIdx.x, c0, c1);
  int64_t n = 0;
  int b = 0;
  for (int64_t c = c0; c < c1; ++c) n += fmt_entry(src, r, c, nullptr, &b) + 1;
  int64_t total;
  const int64_t pos = cta_exclusive_scan(n, &total);
  char* p = out + row_off[r] + pos;
  for (int64_t c = c0; c < c1; ++c) {
    const int len = fmt_entry(src, r, c, p, &b);
    p[len] = c + 1 < cols ? '\t' : '\n';
    p += len + 1;
  }
}

}  // namespace bq
