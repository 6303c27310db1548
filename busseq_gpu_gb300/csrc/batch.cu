// Batches of chains launched as one CUDA graph per sweep, and the autotuners
// of the launch shapes (neither in the reference).
#include "capi_internal.h"

#include <vector>

using namespace bqc;

// ---------------------------------------------------------------------------
// Batches of chains: one CUDA graph holds one sweep of every chain as
// independent branches (forked from and joined to the batch's stream), so a
// single launch advances all chains and the kernels of different chains run
// concurrently, filling the SMs that one chain's small or tail-heavy kernels
// leave idle.  Each chain keeps its own state, streams of random numbers and
// device sweep counter, so its draws are those of the chain run alone.
// ---------------------------------------------------------------------------
struct busseq_batch {
  int device = 0;
  std::vector<busseq_handle*> hs;
  cudaStream_t root = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t g_burn = nullptr, g_keep = nullptr;
  ~busseq_batch() {
    if (g_burn) cudaGraphExecDestroy(g_burn);
    if (g_keep) cudaGraphExecDestroy(g_keep);
    for (cudaEvent_t e : join) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (done) cudaEventDestroy(done);
    if (root) cudaStreamDestroy(root);
  }
};

namespace {

int capture_batch(busseq_batch* b, int kept, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal));
  int r = BUSSEQ_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->root);
  for (size_t c = 0; c < b->hs.size() && r == BUSSEQ_OK && e == cudaSuccess; ++c) {
    busseq_handle* h = b->hs[c];
    e = cudaStreamWaitEvent(h->own_stream, b->fork, 0);
    if (e == cudaSuccess) r = launch_sweep(h, h->own_stream, kept);
    if (r == BUSSEQ_OK && e == cudaSuccess) e = cudaEventRecord(b->join[c], h->own_stream);
    if (r == BUSSEQ_OK && e == cudaSuccess) e = cudaStreamWaitEvent(b->root, b->join[c], 0);
  }
  const cudaError_t e_end = cudaStreamEndCapture(b->root, &g);
  if (r != BUSSEQ_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e == cudaSuccess) e = e_end;
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(BUSSEQ_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
  return BUSSEQ_OK;
}

}  // namespace

extern "C" {

int busseq_batch_create(busseq_handle* const* hs, int32_t n, busseq_batch** out) {
  if (!hs || !out || n <= 0) return fail(BUSSEQ_ERR_ARG, "a batch needs at least one handle");
  *out = nullptr;
  for (int c = 0; c < n; ++c) {
    busseq_handle* h = hs[c];
    if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle %d", c);
    if (!h->begun) return fail(BUSSEQ_ERR_STATE, "handle %d: busseq_begin has not been called", c);
    if (h->device != hs[0]->device) return fail(BUSSEQ_ERR_ARG, "handle %d is on another device", c);
    if (h->n_iter != hs[0]->n_iter || h->n_burnin != hs[0]->n_burnin || h->iter_host != hs[0]->iter_host)
      return fail(BUSSEQ_ERR_ARG, "handle %d: the chains of a batch need the same run length, burn-in and "
                  "progress", c);
    for (int d = 0; d < c; ++d)
      if (hs[d] == h) return fail(BUSSEQ_ERR_ARG, "handle %d appears twice", c);
  }
  CUDA_TRY(cudaSetDevice(hs[0]->device));
  for (int c = 0; c < n; ++c) CUDA_TRY(cudaStreamSynchronize(hs[c]->stream));
  auto* b = new busseq_batch();
  b->device = hs[0]->device;
  b->hs.assign(hs, hs + n);
  int r = BUSSEQ_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  b->join.assign(n, nullptr);
  for (int c = 0; c < n && e == cudaSuccess; ++c) e = cudaEventCreateWithFlags(&b->join[c], cudaEventDisableTiming);
  if (e != cudaSuccess) r = fail(BUSSEQ_ERR_CUDA, "batch streams: %s", cudaGetErrorString(e));
  if (r == BUSSEQ_OK) r = capture_batch(b, 0, &b->g_burn);
  if (r == BUSSEQ_OK) r = capture_batch(b, 1, &b->g_keep);
  if (r != BUSSEQ_OK) {
    delete b;
    return r;
  }
  *out = b;
  return BUSSEQ_OK;
}

int busseq_batch_sweeps(busseq_batch* b, int32_t count) {
  if (!b) return fail(BUSSEQ_ERR_ARG, "NULL batch");
  busseq_handle* h0 = b->hs[0];
  for (busseq_handle* h : b->hs)
    if (!h->begun || h->iter_host != h0->iter_host || h->n_iter != h0->n_iter || h->n_burnin != h0->n_burnin)
      return fail(BUSSEQ_ERR_STATE, "a chain of the batch was restarted or advanced on its own");
  if (count < 0 || h0->iter_host + count > h0->n_iter)
    return fail(BUSSEQ_ERR_ARG, "requested sweeps exceed the run length (%d of %d done)", h0->iter_host, h0->n_iter);
  CUDA_TRY(cudaSetDevice(b->device));
  // order the batch after whatever the chains' own streams hold
  for (busseq_handle* h : b->hs) {
    CUDA_TRY(cudaEventRecord(b->done, h->stream));
    CUDA_TRY(cudaStreamWaitEvent(b->root, b->done, 0));
  }
  for (int c = 0; c < count; ++c) {
    CUDA_TRY(cudaGraphLaunch(h0->iter_host < h0->n_burnin ? b->g_burn : b->g_keep, b->root));
    for (busseq_handle* h : b->hs) ++h->iter_host;
  }
  // and the chains' later work after the batch
  CUDA_TRY(cudaEventRecord(b->done, b->root));
  for (busseq_handle* h : b->hs) CUDA_TRY(cudaStreamWaitEvent(h->stream, b->done, 0));
  return BUSSEQ_OK;
}

int busseq_batch_synchronize(busseq_batch* b) {
  if (!b) return fail(BUSSEQ_ERR_ARG, "NULL batch");
  CUDA_TRY(cudaSetDevice(b->device));
  CUDA_TRY(cudaStreamSynchronize(b->root));
  for (busseq_handle* h : b->hs) TRY(check_device_error(h));
  return BUSSEQ_OK;
}

void* busseq_batch_stream(busseq_batch* b) { return b ? (void*)b->root : nullptr; }

void busseq_batch_destroy(busseq_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->root) cudaStreamSynchronize(b->root);
  delete b;
}

// Milliseconds per sweep of `sweeps` timed burn-in sweeps (after `warm`
// untimed ones) of a scratch handle with options `o` on the given counts.
static int time_sweeps(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, busseq_options o,
                       int32_t sweeps, double* ms_per_sweep) {
  const int warm = 3;
  o.keep_draws = 0;
  busseq_handle* h = nullptr;
  TRY(busseq_create(dims, Y, Y_is_device, &o, &h));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = busseq_begin(h, warm + sweeps, warm + sweeps, 0);
  if (r == BUSSEQ_OK) r = busseq_sweeps(h, warm);
  if (r == BUSSEQ_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
    r = fail(BUSSEQ_ERR_CUDA, "cudaEventCreate failed");
  float ms = 0.0f;
  if (r == BUSSEQ_OK && cudaEventRecord(e0, h->stream) != cudaSuccess) r = fail(BUSSEQ_ERR_CUDA, "event record");
  if (r == BUSSEQ_OK) r = busseq_sweeps(h, sweeps);
  if (r == BUSSEQ_OK && cudaEventRecord(e1, h->stream) != cudaSuccess) r = fail(BUSSEQ_ERR_CUDA, "event record");
  if (r == BUSSEQ_OK) r = check_device_error(h);
  if (r == BUSSEQ_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) r = fail(BUSSEQ_ERR_CUDA, "event time");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  busseq_destroy(h);
  if (r == BUSSEQ_OK) *ms_per_sweep = (double)ms / sweeps;
  return r;
}

// Gene-pass chunk length by measurement: for every candidate, a scratch
// handle on the same counts (a device copy when Y is on the host) runs three
// untimed and `sweeps` timed burn-in sweeps; the fastest candidate wins.  The
// scratch handles use the options' seed, so the caller's chains are untouched.
int busseq_autotune_chunk(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, const busseq_options* opt,
                          const int32_t* candidates, int32_t n_cand, int32_t sweeps, int32_t* best,
                          double* ms_per_sweep) {
  if (!dims || !Y || !opt || !candidates || n_cand <= 0 || sweeps <= 0 || !best)
    return fail(BUSSEQ_ERR_ARG, "bad autotune arguments");
  double best_ms = 0.0;
  *best = 0;
  for (int c = 0; c < n_cand; ++c) {
    if (candidates[c] <= 0 || candidates[c] > bq::MAX_CG)
      return fail(BUSSEQ_ERR_ARG, "chunk candidate %d outside 1..%d", candidates[c], bq::MAX_CG);
    busseq_options o = *opt;
    o.chunk_cells = candidates[c];
    double per = 0.0;
    TRY(time_sweeps(dims, Y, Y_is_device, o, sweeps, &per));
    if (ms_per_sweep) ms_per_sweep[c] = per;
    if (*best == 0 || per < best_ms) {
      best_ms = per;
      *best = candidates[c];
    }
  }
  return BUSSEQ_OK;
}

// Launch shapes by coordinate descent: the chunk length, then the Z/X unit
// length, then the Z/X CTAs per SM, each set to its fastest candidate with the
// others held; the pass is repeated once if it moved any of them.
int busseq_autotune(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, busseq_options* opt,
                    int32_t sweeps, double* ms_per_sweep) {
  if (!dims || !dims->n_b || dims->B < 1 || !Y || !opt || sweeps <= 0)
    return fail(BUSSEQ_ERR_ARG, "bad autotune arguments");
  static const int32_t chunk_c[] = {64, 128, 192, 256};
  static const int32_t unit_c[] = {128, 256, 384, 512};
  static const int32_t ctas_c[] = {2, 3, 4};
  busseq_options cur = *opt;
  if (cur.chunk_cells <= 0) {  // the handle's default (busseq_create)
    int64_t n = 0;
    for (int b = 0; b < dims->B; ++b) n += dims->n_b[b];
    cur.chunk_cells =
        cur.hmc_leapfrog <= 0 && n / std::max<int64_t>(1, (int64_t)dims->B * dims->K) < 512 ? 128 : bq::MAX_CG;
  }
  if (cur.zx_unit <= 0) cur.zx_unit = bq::ZX_UNIT;
  if (cur.zx_ctas_per_sm <= 0) cur.zx_ctas_per_sm = bq::ZX_CTAS_PER_SM;
  double best_ms = 0.0;
  TRY(time_sweeps(dims, Y, Y_is_device, cur, sweeps, &best_ms));
  for (int pass = 0; pass < 2; ++pass) {
    bool moved = false;
    for (int knob = 0; knob < 3; ++knob) {
      const int32_t* cand = knob == 0 ? chunk_c : knob == 1 ? unit_c : ctas_c;
      const int n = knob == 2 ? 3 : 4;
      for (int c = 0; c < n; ++c) {
        busseq_options o = cur;
        int32_t* field = knob == 0 ? &o.chunk_cells : knob == 1 ? &o.zx_unit : &o.zx_ctas_per_sm;
        if (*field == cand[c]) continue;
        *field = cand[c];
        double per = 0.0;
        TRY(time_sweeps(dims, Y, Y_is_device, o, sweeps, &per));
        if (per < best_ms) {
          best_ms = per;
          cur = o;
          moved = true;
        }
      }
    }
    if (!moved) break;
  }
  opt->chunk_cells = cur.chunk_cells;
  opt->zx_unit = cur.zx_unit;
  opt->zx_ctas_per_sm = cur.zx_ctas_per_sm;
  if (ms_per_sweep) *ms_per_sweep = best_ms;
  return BUSSEQ_OK;
}

}  // extern "C"
