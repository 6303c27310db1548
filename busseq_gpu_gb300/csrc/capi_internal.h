// Internals shared by the C-ABI translation units (capi.cu, checkpoint.cu,
// batch.cu): the handle, error reporting and the sweep launchers.
#pragma once
#include "busseq_gb300.h"
#include "busseq_dev.h"

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

namespace bqc {

// Records a formatted message for busseq_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);

inline int64_t round_up(int64_t a, int64_t m) { return (a + m - 1) / m * m; }
inline unsigned blocks_for(int64_t n, int t) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

}  // namespace bqc

#define CUDA_TRY(x)                                                                            \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) return bqc::fail(BUSSEQ_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)

#define LAUNCH_CHECK(name)                                                                     \
  do {                                                                                         \
    cudaError_t e_ = cudaGetLastError();                                                       \
    if (e_ != cudaSuccess)                                                                     \
      return bqc::fail(BUSSEQ_ERR_CUDA, "launch of %s: %s", name, cudaGetErrorString(e_));     \
  } while (0)

#define TRY(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != BUSSEQ_OK) return r_; \
  } while (0)

struct busseq_handle {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // a captured sweep's side branch (k_phi_static, the gamma decisions) and
  // its fork and join events
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork[2] = {nullptr, nullptr}, ev_join = nullptr;
  bq::DevState s{};
  busseq_options opt{};
  std::vector<int32_t> n_b, off;
  std::vector<void*> allocs;
  // run
  bool begun = false, finished = false;
  int n_iter = 0, n_burnin = 0, n_unchanged = 0, iter_host = 0, n_kept = 0;
  cudaGraphExec_t g_burn = nullptr, g_keep = nullptr;
  std::vector<void*> run_allocs;  // accumulators and kept draws of the current run
  // summaries
  bq::Estimates est{};
  double* ll_ik = nullptr;
  double* bic_out = nullptr;
  bool est_valid = false;

  ~busseq_handle() {
    if (g_burn) cudaGraphExecDestroy(g_burn);
    if (g_keep) cudaGraphExecDestroy(g_keep);
    for (void* p : run_allocs) cudaFree(p);
    for (void* p : allocs) cudaFree(p);
    for (cudaEvent_t e : ev_fork)
      if (e) cudaEventDestroy(e);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side_stream) cudaStreamDestroy(side_stream);
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  template <class T>
  int alloc(T** p, size_t count, bool run_scoped = false) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return bqc::fail(BUSSEQ_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    e = cudaMemsetAsync(q, 0, bytes, stream);
    if (e != cudaSuccess) return bqc::fail(BUSSEQ_ERR_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
    (run_scoped ? run_allocs : allocs).push_back(q);
    *p = static_cast<T*>(q);
    return BUSSEQ_OK;
  }
};

namespace bqc {

int check_device_error(busseq_handle* h);
int launch_sweep(busseq_handle* h, cudaStream_t st, int kept);
std::vector<int> sweep_sequence(const busseq_handle* h, int kept);
int zmask_from_zval(busseq_handle* h);
int z_dense_async(busseq_handle* h, int esize, void** out);
int z_to_host(busseq_handle* h, void* dst, int esize);
int capture(busseq_handle* h, int kept, cudaGraphExec_t* out);
int ensure_estimates(busseq_handle* h);

}  // namespace bqc
