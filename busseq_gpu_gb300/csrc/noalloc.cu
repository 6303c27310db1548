// BIC of a set of estimates without allocating any device memory.
//
// Some callers cannot call cudaMalloc: code that runs under a framework which
// owns every device allocation (a fixed memory pool or arena), code that must
// not grow the device footprint after start-up, and plugins embedded in a host
// process that forbids allocation on its hot path.  This entry point serves
// them: the caller passes device pointers to the counts, the estimates and a
// two-double result buffer, and the per-(cell, type) log-likelihood scratch
// lives in a file-scope __device__ array of fixed size instead of memory from
// cudaMalloc.
//
// The array is static device memory: every GPU that loads this library holds
// it (8 MB of doubles + 1 MB of ints) until the process exits.
#include "busseq_gb300.h"
#include "busseq_dev.h"
#include "kernels.h"

#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

extern "C" int busseq_internal_set_error(int code, const char* msg);

namespace {

constexpr int64_t kMaxDoubles = BUSSEQ_NOALLOC_BIC_MAX_TYPES_X_CELLS;
constexpr int64_t kMaxCells = BUSSEQ_NOALLOC_BIC_MAX_CELLS;
constexpr int kMaxDevices = 64;

// Shared by every call on a device: [K][N] log-likelihoods.
static __device__ __align__(256) double g_bic_ll[kMaxDoubles];
// [0, N): batch of each cell; [kMaxCells, kMaxCells + B + 1): batch offsets.
static __device__ __align__(256) int32_t g_bic_batch[kMaxCells + bq::MAX_B + 1];

struct DeviceScratch {
  bool ready = false;
  double* ll = nullptr;
  int32_t* batch = nullptr;
};
DeviceScratch g_scratch[kMaxDevices];
std::mutex g_mu;

struct BatchOffsets {
  int32_t off[bq::MAX_B + 1];
};

__global__ void k_noalloc_batches(int32_t* batch, BatchOffsets o, int B, int64_t N, int64_t off_slot) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    int b = 0;
    while (b + 1 < B && i >= o.off[b + 1]) ++b;
    batch[i] = b;
  }
  if (i <= B) batch[off_slot + i] = o.off[i];
}

int err(int code, const char* msg) { return busseq_internal_set_error(code, msg); }

}  // namespace

extern "C" int busseq_bic_noalloc(const busseq_dims* dims, const int32_t* Y_dev, const double* alpha_dev,
                                  const double* beta_dev, const double* nu_dev, const double* delta_dev,
                                  const double* phi_dev, const double* gamma_dev, const double* pi_dev,
                                  double* out_dev, void* cuda_stream) {
  if (!dims || !dims->n_b || !Y_dev || !alpha_dev || !beta_dev || !nu_dev || !delta_dev || !phi_dev || !gamma_dev ||
      !pi_dev || !out_dev)
    return err(BUSSEQ_ERR_ARG, "busseq_bic_noalloc: NULL argument");
  const int B = dims->B, K = dims->K;
  const int64_t G = dims->G;
  if (B < 1 || B > bq::MAX_B || K < 1 || K > bq::MAX_K || G < 1)
    return err(BUSSEQ_ERR_ARG, "busseq_bic_noalloc: B must be in 1..128, K in 1..64 and G positive");
  // The true total first (64-bit), so that the message below reports it.
  int64_t N = 0;
  for (int b = 0; b < B; ++b) {
    if (dims->n_b[b] < 1) return err(BUSSEQ_ERR_ARG, "busseq_bic_noalloc: every batch needs at least one cell");
    N += dims->n_b[b];
  }
  if (N > kMaxCells || N * (int64_t)K > kMaxDoubles) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "busseq_bic_noalloc: N = %lld cells and K = %d types exceed the fixed scratch "
             "(at most %lld cells and N*K <= %lld); use busseq_bic instead",
             (long long)N, K, (long long)kMaxCells, (long long)kMaxDoubles);
    return err(BUSSEQ_ERR_ARG, msg);
  }
  BatchOffsets o{};
  o.off[0] = 0;
  for (int b = 0; b < B; ++b) o.off[b + 1] = o.off[b] + dims->n_b[b];

  // The scratch's device addresses, taken with the caller's device current.
  // Host code may not use the arrays' names as addresses.  The lookup is
  // repeated on every call made outside stream capture, so that a module
  // loaded again (after cudaDeviceReset, or in another context on the same
  // device) is found at its new address; a call made during capture uses the
  // address of the last call made outside capture on this device.
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return err(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return err(BUSSEQ_ERR_ARG, "busseq_bic_noalloc: device ordinal out of range");
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return err(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
  DeviceScratch sc;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (cap == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_bic_ll);
      if (e != cudaSuccess) return err(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
      g_scratch[dev].ll = static_cast<double*>(p);
      e = cudaGetSymbolAddress(&p, g_bic_batch);
      if (e != cudaSuccess) return err(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
      g_scratch[dev].batch = static_cast<int32_t*>(p);
      g_scratch[dev].ready = true;
    } else if (!g_scratch[dev].ready) {
      return err(BUSSEQ_ERR_STATE,
                 "busseq_bic_noalloc: the first call on a device must come before any stream capture");
    }
    sc = g_scratch[dev];
  }

  // Every pointer must be device (or managed) memory that the current device
  // can address: the kernels run on the current device.
  const void* ptrs[] = {Y_dev, alpha_dev, beta_dev, nu_dev, delta_dev, phi_dev, gamma_dev, pi_dev, out_dev};
  for (const void* q : ptrs) {
    cudaPointerAttributes a{};
    e = cudaPointerGetAttributes(&a, q);
    if (e != cudaSuccess) return err(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
    if (!((a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged))
      return err(BUSSEQ_ERR_ARG,
                 "busseq_bic_noalloc: every array must be device memory of the current device");
  }

  // A view of the caller's arrays in the layout the BIC kernels read
  // (row stride G, estimates in the reference's layouts).  k_bic_cell and
  // k_bic_total read only B, K, G, N, Gp, Y, batch_of and batch_off of the
  // state, so every other field of this view stays zero.
  bq::DevState s{};
  s.B = B;
  s.K = K;
  s.G = G;
  s.N = N;
  s.Gp = G;
  s.Gw = (G + 31) / 32;
  s.Y = Y_dev;
  s.batch_of = sc.batch;
  s.batch_off = sc.batch + kMaxCells;
  bq::Estimates est{};
  est.alpha = const_cast<double*>(alpha_dev);
  est.beta = const_cast<double*>(beta_dev);
  est.nu = const_cast<double*>(nu_dev);
  est.delta = const_cast<double*>(delta_dev);
  est.phi = const_cast<double*>(phi_dev);
  est.gamma = const_cast<double*>(gamma_dev);
  est.pi = const_cast<double*>(pi_dev);

  const int64_t nfill = N > B + 1 ? N : B + 1;
  k_noalloc_batches<<<(unsigned)((nfill + 255) / 256), 256, 0, st>>>(sc.batch, o, B, N, kMaxCells);
  // Every [k][i] entry of the scratch is written by k_bic_cell before
  // k_bic_total reads it, so nothing has to be cleared between calls.
  // no tables: each entry computes exp(beta), lgamma(phi) and the rest itself
  bq::launch_bic(s, est, sc.ll, bq::BicTabs{}, out_dev, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return err(BUSSEQ_ERR_CUDA, cudaGetErrorString(e));
  return BUSSEQ_OK;
}
