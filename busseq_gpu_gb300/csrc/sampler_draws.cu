// Draws from the device samplers, for distribution tests.
//
// The sweep kernels call the samplers of rng.h inline (gamma in the phi and
// gamma1 proposals, p, tau0 and pi; NB in the Z/X update).  This entry point
// runs the very same device functions in a plain kernel, one draw per thread,
// so a test can compare many draws with closed-form distributions (KS and
// chi-square) and with the FP64 oracle's samplers on the same Philox streams
// (stream 40 + family, entity = draw index, sweep 0).
#include "busseq_gb300.h"
#include "kernels_common.cuh"

#include <cuda_runtime.h>

extern "C" int busseq_internal_set_error(int code, const char* msg);

namespace bq {

__global__ void k_sample_draws(int kind, float a, float b, uint64_t seed, int64_t n, float* out_f, int32_t* out_i,
                               int* err_out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int err = 0;
  switch (kind) {
    case 0: {
      Stream st(seed, SID_TEST_GAMMA, (uint64_t)j, 0u);
      out_f[j] = gamma_mt(st, a, &err);
      break;
    }
    case 1: {
      Stream st(seed, SID_TEST_POISSON, (uint64_t)j, 0u);
      out_i[j] = poisson(st, a, &err);
      break;
    }
    default: {
      Stream st(seed, SID_TEST_NEGBIN, (uint64_t)j, 0u);
      out_i[j] = kind == 2 ? negbin(st, a, b, &err)
               : kind == 3 ? negbin_gamma_poisson(st, a, b, &err)
                           : negbin_inversion(st, a, b, &err);
      break;
    }
  }
  if (err) atomicOr(err_out, err);
}

}  // namespace bq

extern "C" int busseq_sample_draws(int32_t kind, double a, double b, uint64_t seed, int64_t n, void* out) {
  if (!out || n < 1 || kind < 0 || kind > 4)
    return busseq_internal_set_error(BUSSEQ_ERR_ARG, "busseq_sample_draws: bad kind, count or output");
  if (!(a > 0.0) || (kind >= 2 && !(b > 0.0)) || (kind == 4 && b < 1.0))
    return busseq_internal_set_error(BUSSEQ_ERR_ARG, "busseq_sample_draws: parameters out of range");
  void* d_out = nullptr;
  int* d_err = nullptr;
  cudaError_t e = cudaMalloc(&d_out, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d_err, 0, sizeof(int));
  if (e == cudaSuccess) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    bq::k_sample_draws<<<blocks, 256>>>(kind, (float)a, (float)b, seed, n, static_cast<float*>(d_out),
                                        static_cast<int32_t*>(d_out), d_err);
    e = cudaGetLastError();
  }
  int err = 0;
  if (e == cudaSuccess) e = cudaMemcpy(out, d_out, (size_t)n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d_out);
  cudaFree(d_err);
  if (e != cudaSuccess) return busseq_internal_set_error(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
  if (err) return busseq_internal_set_error(BUSSEQ_ERR_SAMPLER, "busseq_sample_draws: a sampler cap was reached");
  return BUSSEQ_OK;
}
