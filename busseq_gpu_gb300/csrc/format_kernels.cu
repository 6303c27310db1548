// Text formatting of large integer tables on the device, for the output files
// whose size scales with N x G (_post_X.txt, _corrected_X.txt).  The layout is
// the host writer's: decimal integers ("-" for negatives), a tab between the
// columns of a row and a newline at its end (BUSseq_gpu.cu:1628-1645 writes the
// same "%d\t" / "%d\n" sequence).
//
// Two passes, one CTA per row: k_fmt_row_len measures each row's text, the host
// turns the lengths into offsets, and k_fmt_rows writes every row at its
// offset -- each thread takes a contiguous run of the row's entries, a CTA-wide
// scan of the runs' lengths places them, and the thread writes its run.
#include <cuda_runtime.h>
#include <stdint.h>

namespace bq {

namespace {

constexpr int FMT_THREADS = 256;

__device__ __forceinline__ int dec_len(int32_t v) {
  uint32_t u = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
  int n = 1;
  while (u >= 10u) {
    u /= 10u;
    ++n;
  }
  return n + (v < 0 ? 1 : 0);
}

// Writes v at p (dec_len(v) characters).
__device__ __forceinline__ void dec_put(int32_t v, char* p, int len) {
  uint32_t u = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
  if (v < 0) p[0] = '-';
  char* q = p + len - 1;
  do {
    *q-- = (char)('0' + u % 10u);
    u /= 10u;
  } while (u);
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

// row_len[r] = length of row r's text, separators and newline included.
__global__ void __launch_bounds__(FMT_THREADS) k_fmt_row_len(const int32_t* M, int64_t ld, int64_t cols,
                                                             int64_t* row_len) {
  const int64_t r = blockIdx.x;
  int64_t c0, c1;
  run_of(cols, threadIdx.x, c0, c1);
  int64_t n = 0;
  for (int64_t c = c0; c < c1; ++c) n += dec_len(M[r * ld + c]) + 1;
  int64_t total;
  cta_exclusive_scan(n, &total);
  if (threadIdx.x == 0) row_len[r] = total;
}

// Writes row r at out + row_off[r].
__global__ void __launch_bounds__(FMT_THREADS) k_fmt_rows(const int32_t* M, int64_t ld, int64_t cols,
                                                          const int64_t* row_off, char* out) {
  const int64_t r = blockIdx.x;
  int64_t c0, c1;
  run_of(cols, threadIdx.x, c0, c1);
  int64_t n = 0;
  for (int64_t c = c0; c < c1; ++c) n += dec_len(M[r * ld + c]) + 1;
  int64_t total;
  const int64_t pos = cta_exclusive_scan(n, &total);
  char* p = out + row_off[r] + pos;
  for (int64_t c = c0; c < c1; ++c) {
    const int32_t v = M[r * ld + c];
    const int len = dec_len(v);
    dec_put(v, p, len);
    p[len] = c + 1 < cols ? '\t' : '\n';
    p += len + 1;
  }
}

}  // namespace bq
