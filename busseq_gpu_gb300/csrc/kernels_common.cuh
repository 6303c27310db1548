// Device helpers shared by the sweep, initialisation and summary kernels.
#pragma once
#include "busseq_dev.h"
#include "rng.h"

namespace bq {

// The idx-th uniform (idx < 4) of stream (sid, entity) at sweep `iter`.
// Matches the idx-th call of Stream::uniform() on a fresh stream.
__device__ __forceinline__ float uniform_at(uint64_t seed, uint32_t sid, uint64_t ent, uint32_t iter, int idx) {
  const U32x4 r = philox4x32_10(
      U32x4{(uint32_t)ent, ((uint32_t)(ent >> 32) & 0xFFFFu) | (sid << 16), 0u, iter}, (uint32_t)seed,
      (uint32_t)(seed >> 32));
  const uint32_t v = idx == 0 ? r.x : idx == 1 ? r.y : idx == 2 ? r.z : r.w;
  return u32_to_unit(v);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum of NV doubles per thread; result valid in thread 0.
// `sh` must hold (blockDim.x / 32) * NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = warp_sum(v[j]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) sh[warp * NV + j] = v[j];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += sh[w * NV + j];
      v[j] = t;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Float-float sums.  GB300 runs FP64 at a small fraction of the FP32 rate, so
// the sweep kernels reduce in unevaluated pairs hi + lo of floats (about 48
// significant bits): Knuth's TwoSum gives the exact rounding error of hi + hi',
// which is folded into lo, and a final Fast2Sum renormalises the pair.  The
// reduction trees have a fixed shape, so the sums are bit-reproducible.
// ---------------------------------------------------------------------------
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  const float e = (a.hi - (s - v)) + (b.hi - v);
  const float t = e + (a.lo + b.lo);
  const float hi = s + t;
  return FF{hi, t - (hi - s)};
}

__device__ __forceinline__ double ff_value(FF v) { return (double)v.hi + (double)v.lo; }

__device__ __forceinline__ FF ff_warp_sum(FF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const FF w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
    v = ff_add(v, w);
  }
  return v;
}

__device__ __forceinline__ long long i64_warp_sum(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// CTA sums of NF float-float and NI integer values per thread; results valid
// in thread 0.  `shf` holds (blockDim.x / 32) * NF pairs, `shn`
// (blockDim.x / 32) * NI integers.
template <int NF, int NI>
__device__ __forceinline__ void block_sum_ff(FF (&f)[NF], long long (&n)[NI], FF* shf, long long* shn) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < NF; ++j) f[j] = ff_warp_sum(f[j]);
#pragma unroll
  for (int j = 0; j < NI; ++j) n[j] = i64_warp_sum(n[j]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < NF; ++j) shf[warp * NF + j] = f[j];
#pragma unroll
    for (int j = 0; j < NI; ++j) shn[warp * NI + j] = n[j];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NF; ++j) {
      FF t = shf[j];
      for (int w = 1; w < nw; ++w) t = ff_add(t, shf[w * NF + j]);
      f[j] = t;
    }
#pragma unroll
    for (int j = 0; j < NI; ++j) {
      long long t = shn[j];
      for (int w = 1; w < nw; ++w) t += shn[w * NI + j];
      n[j] = t;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies global -> shared (cp.async.bulk), completed on an
// mbarrier that counts the bytes.  One thread arms the barrier with the
// stage's byte count and issues the row copies; every thread waits on the
// barrier's phase parity.  Waits give up after WAIT_CYCLES SM clocks (about
// one second) so that a copy that never lands cannot hang the GPU: the caller
// then raises ERR_COPY_TIMEOUT and leaves without using the stage.
// ---------------------------------------------------------------------------
enum : int { ERR_COPY_TIMEOUT = 8 };
constexpr long long WAIT_CYCLES = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the asynchronous copy engine.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with parity `parity`; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > WAIT_CYCLES) return false;
  return true;
}

// Orders this thread's earlier shared-memory accesses before later
// asynchronous-proxy accesses (a stage buffer is refilled after it was read).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Completion counter: every CTA of a group calls this once after its global
// writes; it returns true in exactly one CTA (the last to arrive), which then
// sees every other CTA's writes.  The last CTA resets the counter.
__device__ __forceinline__ bool arrive_last(unsigned* counter, unsigned total, int* sh_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(counter, 1u);
    *sh_flag = (prev == total - 1u);
    if (*sh_flag) *counter = 0u;
  }
  __syncthreads();
  const bool last = *sh_flag != 0;
  if (last) __threadfence();
  return last;
}

// Compensated (Kahan) float accumulator: float-pipe throughput with an error
// that does not grow with the number of terms.
struct KahanF {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  __device__ __forceinline__ FF ff() const { return FF{s, -c}; }
};

// log-likelihood shift of one NB entry when eta moves by eps, without the
// linear eps * X part:   (phi + X) * log1p(c * p),  c = expm1(eps), p = mu / (phi + mu)
__device__ __forceinline__ float nb_shift_log(float w, float c, float p) { return w * log1pf(c * p); }

// X and exp(delta) of chunk cells j0..j0+7 for the gene whose column starts
// at Xg (128-bit shared loads; row offsets by one 32x32->64-bit multiply-add).
__device__ __forceinline__ void load8(const char* Xg, uint32_t row_bytes, const int* s_i, const float* s_D, int j0,
                                      int (&xr)[8], float (&dv)[8]) {
  const int4 ia = *reinterpret_cast<const int4*>(s_i + j0);
  const int4 ib = *reinterpret_cast<const int4*>(s_i + j0 + 4);
  const float4 da = *reinterpret_cast<const float4*>(s_D + j0);
  const float4 db = *reinterpret_cast<const float4*>(s_D + j0 + 4);
  const int iv[8] = {ia.x, ia.y, ia.z, ia.w, ib.x, ib.y, ib.z, ib.w};
#pragma unroll
  for (int u = 0; u < 8; ++u) xr[u] = *reinterpret_cast<const int*>(Xg + (uint64_t)(uint32_t)iv[u] * row_bytes);
  dv[0] = da.x; dv[1] = da.y; dv[2] = da.z; dv[3] = da.w;
  dv[4] = db.x; dv[5] = db.y; dv[6] = db.z; dv[7] = db.w;
}

// Sum of part slot `slot` of gene g over the chunks of segment (b, k).
__device__ __forceinline__ double seg_sum(const DevState& s, int b, int k, int slot, int64_t g) {
  const int2 r = s.seg_chunk[b * s.K + k];
  double acc = 0.0;
  for (int c = r.x; c < r.x + r.y; ++c) acc += __ldg(&s.part[((int64_t)c * NSLOT + slot) * s.Gp + g]);
  return acc;
}

}  // namespace bq
