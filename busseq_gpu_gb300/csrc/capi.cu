// C ABI of the GB300 BUSseq sampler: memory, initialisation, CUDA-graph
// sweeps, stages, summaries.  See include/busseq_gb300.h for the contract.
#include "capi_internal.h"
#include "rng.h"
#include "correct_math.h"
#include "kernels.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <string>
#include <vector>

namespace bqc {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

}  // namespace bqc

using namespace bqc;

namespace {

const char* const kKernelNames[] = {"k_propose",      "k_zx",           "k_alpha",      "k_decide_alpha",
                                    "k_beta_nu",      "k_decide_beta",  "k_decide_nu_E", "k_delta",
                                    "k_phi",          "k_decide_phi",   "k_w",          "k_sort_pi",
                                    "k_posterior",    "k_hmc_grad",     "k_hmc_assemble", "k_hmc_start",
                                    "k_hmc_leap0",    "k_hmc_leap",     "k_hmc_refresh_E", "k_hmc_dll",
                                    "k_hmc_energy",   "k_hmc_accept",   "k_hmc_finish", "k_hmc_metric_blocks",
                                    "k_hmc_start_blocks", "k_hmc_leap_blocks0", "k_hmc_leap_blocks",
                                    "k_hmc_energy_blocks", "k_hmc_mass", "k_hmc_grad_start",
                                    "k_hmc_assemble_start", "k_phi_static", "k_hmc_dll_static",
                                    "k_hmc_accept_genes", "k_zx_gp", "k_decide_gamma",
                                    "k_propose_phi"};
constexpr int kNumKernels = 37;
enum : int {
  KID_PROPOSE = 0, KID_ZX = 1, KID_ALPHA = 2, KID_DECIDE_ALPHA = 3, KID_BETA_NU = 4, KID_DECIDE_BETA = 5,
  KID_DECIDE_NU_E = 6, KID_DELTA = 7, KID_PHI = 8, KID_DECIDE_PHI = 9, KID_W = 10, KID_SORT_PI = 11,
  KID_POSTERIOR = 12, KID_HMC_GRAD = 13, KID_HMC_ASSEMBLE = 14, KID_HMC_START = 15, KID_HMC_LEAP0 = 16,
  KID_HMC_LEAP = 17, KID_HMC_E = 18, KID_HMC_DLL = 19, KID_HMC_ENERGY = 20, KID_HMC_ACCEPT = 21,
  KID_HMC_FINISH = 22, KID_HMC_METRIC_BLOCKS = 23, KID_HMC_START_BLOCKS = 24, KID_HMC_LEAP_BLOCKS0 = 25,
  KID_HMC_LEAP_BLOCKS = 26, KID_HMC_ENERGY_BLOCKS = 27, KID_HMC_MASS = 28, KID_HMC_GRAD_START = 29,
  KID_HMC_ASSEMBLE_START = 30, KID_PHI_STATIC = 31, KID_HMC_DLL_STATIC = 32, KID_HMC_ACCEPT_GENES = 33,
  KID_ZX_GP = 34, KID_DECIDE_GAMMA = 35, KID_PROPOSE_PHI = 36
};

}  // namespace

namespace bqc {

int check_device_error(busseq_handle* h) {
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  int err = 0;
  CUDA_TRY(cudaMemcpy(&err, h->s.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    return fail(BUSSEQ_ERR_SAMPLER,
                "a device-side bound was reached (flags 0x%x: 1 Gamma, 2 Poisson and 4 NB sampler caps, "
                "8 shared-memory copy wait)",
                err);
  }
  return BUSSEQ_OK;
}

// CTAs of the per-(batch, gene) static kernels: one wave, warps striding over
// the (batch, gene) pairs.
constexpr unsigned STATIC_CTAS = 152 * 8;

// Enqueue kernel `which` of a sweep on `st` (used for graph capture, for
// profiling and for single stages).
int launch_kernel(busseq_handle* h, int which, cudaStream_t st, int kept, const bq::DevState& s) {
  using namespace bq;
  const dim3 gene_grid(s.n_tiles, s.cap_g);
  switch (which) {
    case 0:
      // the random-walk sweep's phi proposals are KID_PROPOSE_PHI's
      k_propose<<<blocks_for(propose_count(s), 256), 256, 0, st>>>(
          s, s.hmc_L > 0 ? (int)(s.hmc_gene ? PROP_GAMMA | PROP_DELTA : PROP_GAMMA) : (int)(PROP_ALL & ~PROP_PHI),
          0);
      LAUNCH_CHECK("k_propose");
      break;
    case KID_PROPOSE_PHI:
      k_propose<<<blocks_for((int64_t)s.B * s.G, 256), 256, 0, st>>>(s, PROP_PHI, propose_phi_offset(s));
      LAUNCH_CHECK("k_propose_phi");
      break;
    case 1:
      k_zx<<<(unsigned)s.zx_ctas, ZX_THREADS, 0, st>>>(s, kept);
      LAUNCH_CHECK("k_zx");
      break;
    case KID_ZX_GP:
      k_zx_gp<<<(unsigned)s.zgp_ctas, ZX_THREADS, 0, st>>>(s, kept);
      LAUNCH_CHECK("k_zx_gp");
      break;
    case KID_DECIDE_GAMMA:
      k_decide_gamma<<<s.B, DECIDE_GAMMA_THREADS, 0, st>>>(s);
      LAUNCH_CHECK("k_decide_gamma");
      break;
    case 2:
      k_alpha<<<gene_grid, GENE_TILE, 0, st>>>(s);
      LAUNCH_CHECK("k_alpha");
      break;
    case 3:
      k_decide_alpha<<<blocks_for(s.G, 32), GENE_TILE, 0, st>>>(s);
      LAUNCH_CHECK("k_decide_alpha");
      break;
    case 4:
      k_beta_nu<<<gene_grid, GENE_TILE, 0, st>>>(s);
      LAUNCH_CHECK("k_beta_nu");
      break;
    case 5:
      k_decide_beta<<<blocks_for((int64_t)std::max(1, s.K - 1) * s.G, 32), DEC_THREADS, 0, st>>>(s);
      LAUNCH_CHECK("k_decide_beta");
      break;
    case 6:
      k_decide_nu_E<<<blocks_for((int64_t)s.B * s.G, 32), DEC_THREADS, 0, st>>>(s);
      LAUNCH_CHECK("k_decide_nu_E");
      break;
    case 7:
      k_delta<<<s.cap_c, CELL_THREADS, DELTA_SMEM, st>>>(s);
      LAUNCH_CHECK("k_delta");
      break;
    case 8:
      k_phi<<<gene_grid, GENE_TILE, 0, st>>>(s);
      LAUNCH_CHECK("k_phi");
      break;
    case KID_PHI_STATIC:
      k_phi_static<<<STATIC_CTAS, 256, 0, st>>>(s);
      LAUNCH_CHECK("k_phi_static");
      break;
    case KID_HMC_DLL_STATIC:
      k_hmc_dll_prep<<<blocks_for((int64_t)s.B * s.G, 256), 256, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_dll_prep");
      k_hmc_dll_static<<<STATIC_CTAS, 256, 0, st>>>(s, s.n_tiles * s.cap_g, s.hmc_gene);
      LAUNCH_CHECK("k_hmc_dll_static");
      break;
    case 9:
      k_decide_phi<<<blocks_for((int64_t)s.B * s.G, 32), DEC_THREADS, 0, st>>>(s);
      LAUNCH_CHECK("k_decide_phi");
      break;
    case 10:
      if (s.w_update == BUSSEQ_W_GIBBS) k_w_gibbs<<<s.cap_c, CELL_THREADS, 0, st>>>(s);
      else k_w_mh<<<s.cap_c, CELL_THREADS, W_SMEM, st>>>(s);
      LAUNCH_CHECK("k_w");
      break;
    case 11:
      k_sort_pi<<<s.B, 1024, 0, st>>>(s, 1, kept ? 0 : 1);
      LAUNCH_CHECK("k_sort_pi");
      break;
    case 12: {
      const unsigned nb = (unsigned)std::min<int64_t>(blocks_for((int64_t)s.K * s.G, 256), 152 * 8);
      k_posterior<<<nb, 256, 0, st>>>(s, 1);
      LAUNCH_CHECK("k_posterior");
      break;
    }
    case KID_HMC_GRAD:
    case KID_HMC_GRAD_START:
      if (which == KID_HMC_GRAD_START) k_hmc_grad_metric<<<gene_grid, GENE_TILE, 0, st>>>(s, 1);
      else k_hmc_grad<<<gene_grid, GENE_TILE, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_grad");
      break;
    case KID_HMC_ASSEMBLE:
    case KID_HMC_ASSEMBLE_START:
      k_hmc_assemble<<<blocks_for(s.hmc_D, 256), 256, 0, st>>>(s, which == KID_HMC_ASSEMBLE_START ? 1 : 0);
      LAUNCH_CHECK("k_hmc_assemble");
      break;
    case KID_HMC_START:
      k_hmc_start<<<blocks_for(s.hmc_D, 256), 256, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_start");
      break;
    case KID_HMC_LEAP0:
    case KID_HMC_LEAP:
      k_hmc_leap<<<blocks_for(s.hmc_D, 256), 256, 0, st>>>(s, which == KID_HMC_LEAP0 ? 1 : 0);
      LAUNCH_CHECK("k_hmc_leap");
      break;
    case KID_HMC_E:
      k_hmc_refresh_E<<<blocks_for((int64_t)s.B * s.K * s.Gp, 256), 256, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_refresh_E");
      break;
    case KID_HMC_DLL:
      k_hmc_dll<<<gene_grid, GENE_TILE, 0, st>>>(s, s.hmc_gene);
      LAUNCH_CHECK("k_hmc_dll");
      break;
    case KID_HMC_ENERGY:
      k_hmc_energy<<<blocks_for(s.hmc_D, 256), 256, 0, st>>>(s, 1, s.hmc_gene);
      LAUNCH_CHECK("k_hmc_energy");
      break;
    case KID_HMC_ACCEPT_GENES:
      k_hmc_accept_genes<<<blocks_for(s.G, 256), 256, 0, st>>>(s, nullptr);
      LAUNCH_CHECK("k_hmc_accept_genes");
      break;
    case KID_HMC_ACCEPT:
      if (s.hmc_gene) {
        const int ng = (int)blocks_for(s.G, 256);
        k_hmc_accept<<<1, 256, 0, st>>>(s, ng, ng, 0, 2);
        LAUNCH_CHECK("k_hmc_accept");
        break;
      }
      k_hmc_accept<<<1, 256, 0, st>>>(s, s.n_tiles * s.cap_g + STATIC_CTAS, (int)blocks_for(s.hmc_D, 256),
                                      (int)blocks_for(s.G * 32, 256), 0);
      LAUNCH_CHECK("k_hmc_accept");
      break;
    case KID_HMC_METRIC_BLOCKS:
      k_hmc_metric_blocks<<<blocks_for(s.G, 128), 128, 0, st>>>(s, 1);
      LAUNCH_CHECK("k_hmc_metric_blocks");
      break;
    case KID_HMC_START_BLOCKS:
      k_hmc_start_blocks<<<blocks_for(s.G * 32, 128), 128, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_start_blocks");
      break;
    case KID_HMC_LEAP_BLOCKS0:
    case KID_HMC_LEAP_BLOCKS:
      k_hmc_leap_blocks<<<blocks_for(s.G * 32, 128), 128, 0, st>>>(s, which == KID_HMC_LEAP_BLOCKS0 ? 1 : 0);
      LAUNCH_CHECK("k_hmc_leap_blocks");
      break;
    case KID_HMC_MASS:
      k_hmc_mass<<<blocks_for(s.hmc_D, 256), 256, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_mass");
      break;
    case KID_HMC_ENERGY_BLOCKS:
      k_hmc_energy_blocks<<<blocks_for(s.G * 32, 256), 256, 0, st>>>(s, 1, s.hmc_gene);
      LAUNCH_CHECK("k_hmc_energy_blocks");
      break;
    case KID_HMC_FINISH:
      k_hmc_finish<<<blocks_for(s.hmc_D, 256), 256, 0, st>>>(s);
      LAUNCH_CHECK("k_hmc_finish");
      break;
    default:
      return fail(BUSSEQ_ERR_ARG, "no kernel %d", which);
  }
  return BUSSEQ_OK;
}

// The kernels of one sweep, in order.  Random-walk MH (the reference's sweep):
// proposals, Z/X, alpha, L, p/tau0, gamma, beta, nu, delta, phi, W, pi.  HMC:
// proposals of gamma, Z/X, L, p/tau0, gamma, one HMC transition of
// (alpha, beta, nu, delta, log phi), W, pi; with per-gene decisions the
// transition moves (alpha, beta, nu, log phi) gene by gene and delta follows by
// the random-walk step.
std::vector<int> sweep_sequence(const busseq_handle* h, int kept) {
  std::vector<int> q;
  if (h->s.hmc_L > 0) {
    const bool blocks = h->s.hmc_nb > 0;
    q = {KID_PROPOSE, KID_ZX, KID_ZX_GP, KID_DECIDE_GAMMA, KID_DECIDE_ALPHA, KID_HMC_GRAD_START,
         KID_HMC_ASSEMBLE_START, KID_HMC_MASS};
    if (blocks) q.push_back(KID_HMC_METRIC_BLOCKS);
    q.push_back(KID_HMC_START);
    if (blocks) q.push_back(KID_HMC_START_BLOCKS);
    for (int l = 0; l < h->s.hmc_L; ++l) {
      q.push_back(l == 0 ? KID_HMC_LEAP0 : KID_HMC_LEAP);
      if (blocks) q.push_back(l == 0 ? KID_HMC_LEAP_BLOCKS0 : KID_HMC_LEAP_BLOCKS);
      q.push_back(KID_HMC_GRAD);
      q.push_back(KID_HMC_ASSEMBLE);
    }
    q.push_back(KID_HMC_DLL_STATIC);
    q.push_back(KID_HMC_DLL);
    q.push_back(KID_HMC_ENERGY);
    if (blocks) q.push_back(KID_HMC_ENERGY_BLOCKS);
    if (h->s.hmc_gene) q.push_back(KID_HMC_ACCEPT_GENES);
    q.push_back(KID_HMC_ACCEPT);
    q.push_back(KID_HMC_FINISH);
    q.push_back(KID_HMC_E);
    if (h->s.hmc_gene) q.push_back(KID_DELTA);  // delta by the random-walk step, given the new genes
    q.push_back(KID_W);
    q.push_back(KID_SORT_PI);
  } else {
    for (int k = 0; k <= KID_SORT_PI; ++k) {
      if (k == KID_PHI) q.push_back(KID_PHI_STATIC);
      q.push_back(k);
      if (k == KID_PROPOSE) q.push_back(KID_PROPOSE_PHI);
      if (k == KID_ZX) {
        q.push_back(KID_ZX_GP);
        q.push_back(KID_DECIDE_GAMMA);
      }
    }
  }
  if (kept) q.push_back(KID_POSTERIOR);
  return q;
}

// One sweep, enqueued while `st` is being captured into a graph.  Three
// kernels leave the main line on the handle's side stream: the phi proposals
// with their lgamma tables and k_phi_static read only phi and the static
// counts and are first read by k_phi; the gamma decisions need the Z/X
// partials of k_zx_gp and are read only by the next sweep (and the posterior
// accumulation).  They run beside the main line, filling the SMs that Z/X's
// tail and the small decision kernels leave idle; the branch joins before
// k_phi, or at the end of the sweep.
int launch_sweep(busseq_handle* h, cudaStream_t st, int kept) {
  const std::vector<int> seq = sweep_sequence(h, kept);
  cudaStream_t side = h->side_stream;
  bool open = false;  // the side branch has work that the main line has not joined
  auto fork = [&](int which, int ev) -> int {
    CUDA_TRY(cudaEventRecord(h->ev_fork[ev], st));
    CUDA_TRY(cudaStreamWaitEvent(side, h->ev_fork[ev], 0));
    TRY(launch_kernel(h, which, side, kept, h->s));
    open = true;
    return BUSSEQ_OK;
  };
  auto join = [&]() -> int {
    if (!open) return BUSSEQ_OK;
    CUDA_TRY(cudaEventRecord(h->ev_join, side));
    CUDA_TRY(cudaStreamWaitEvent(st, h->ev_join, 0));
    open = false;
    return BUSSEQ_OK;
  };
  const bool has_phi = std::find(seq.begin(), seq.end(), (int)KID_PROPOSE_PHI) != seq.end();
  for (int k : seq) {
    if (k == KID_PROPOSE_PHI || k == KID_PHI_STATIC || k == KID_DECIDE_GAMMA) continue;
    if (k == KID_PHI || k == KID_POSTERIOR) TRY(join());
    TRY(launch_kernel(h, k, st, kept, h->s));
    if (k == KID_PROPOSE && has_phi) {
      TRY(fork(KID_PROPOSE_PHI, 0));
      TRY(launch_kernel(h, KID_PHI_STATIC, side, kept, h->s));
    }
    if (k == KID_ZX_GP) TRY(fork(KID_DECIDE_GAMMA, 1));
  }
  return join();
}

// Z as a bit mask [N][Gw] in s.zm, from the per-entry zval (for transfers).
int zmask_from_zval(busseq_handle* h) {
  const bq::DevState& s = h->s;
  CUDA_TRY(cudaMemsetAsync(s.zm, 0, (size_t)s.N * s.Gw * sizeof(uint32_t), h->stream));
  if (s.nz0 > 0) {
    bq::k_zmask_from_zval<<<blocks_for(s.nz0, 256), 256, 0, h->stream>>>(s);
    LAUNCH_CHECK("k_zmask_from_zval");
  }
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return BUSSEQ_OK;
}

// Z as a dense [N][G] table of int32 (esize 4) or uint8 (esize 1) in a
// stream-ordered device allocation, enqueued on the handle's stream (the
// caller copies it and frees it there).
int z_dense_async(busseq_handle* h, int esize, void** out) {
  const bq::DevState& s = h->s;
  *out = nullptr;
  CUDA_TRY(cudaMemsetAsync(s.zm, 0, (size_t)s.N * s.Gw * sizeof(uint32_t), h->stream));
  if (s.nz0 > 0) {
    bq::k_zmask_from_zval<<<blocks_for(s.nz0, 256), 256, 0, h->stream>>>(s);
    LAUNCH_CHECK("k_zmask_from_zval");
  }
  void* d = nullptr;
  CUDA_TRY(cudaMallocAsync(&d, (size_t)s.N * s.G * esize, h->stream));
  const unsigned grid = std::min<unsigned>(blocks_for(s.N * s.Gw, 256), 152 * 16);
  if (esize == 4) bq::k_z_dense_i32<<<grid, 256, 0, h->stream>>>(s, static_cast<int32_t*>(d), s.G);
  else bq::k_z_dense_u8<<<grid, 256, 0, h->stream>>>(s, static_cast<uint8_t*>(d), s.G);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFreeAsync(d, h->stream);
    return fail(BUSSEQ_ERR_CUDA, "Z table: %s", cudaGetErrorString(e));
  }
  *out = d;
  return BUSSEQ_OK;
}

int z_to_host(busseq_handle* h, void* dst, int esize) {
  const bq::DevState& s = h->s;
  const size_t bytes = (size_t)s.N * s.G * esize;
  void* d = nullptr;
  TRY(z_dense_async(h, esize, &d));
  cudaError_t e = cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, h->stream);
  const cudaError_t e2 = cudaFreeAsync(d, h->stream);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "Z table: %s", cudaGetErrorString(e));
  return BUSSEQ_OK;
}

int capture(busseq_handle* h, int kept, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(h->own_stream, cudaStreamCaptureModeThreadLocal));
  const int r = launch_sweep(h, h->own_stream, kept);
  cudaError_t e = cudaStreamEndCapture(h->own_stream, &g);
  if (r != BUSSEQ_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return BUSSEQ_OK;
}

int ensure_estimates(busseq_handle* h) {
  bq::Estimates& e = h->est;
  const int64_t G = h->s.G, N = h->s.N;
  const int B = h->s.B, K = h->s.K;
  if (!e.alpha) {
    TRY(h->alloc(&e.gamma, 2 * B));
    TRY(h->alloc(&e.alpha, G));
    TRY(h->alloc(&e.L, std::max<int64_t>(1, (K - 1) * G)));
    TRY(h->alloc(&e.beta, K * G));
    TRY(h->alloc(&e.ptau, 2));
    TRY(h->alloc(&e.nu, B * G));
    TRY(h->alloc(&e.delta, N));
    TRY(h->alloc(&e.phi, B * G));
    TRY(h->alloc(&e.pi, B * K));
    TRY(h->alloc(&e.W, N));
  }
  if (!h->est_valid) {
    bq::k_finalize<<<std::min<unsigned>(blocks_for((int64_t)K * G, 256), 152 * 8), 256, 0, h->stream>>>(
        h->s, e, h->finished ? h->n_kept : 0);
    LAUNCH_CHECK("k_finalize");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->est_valid = true;
  }
  return BUSSEQ_OK;
}

}  // namespace bqc

extern "C" {

const char* busseq_last_error(void) { return g_err.c_str(); }

int busseq_internal_set_error(int code, const char* msg) { return fail(code, "%s", msg); }

}  // extern "C"

namespace {

// Formats the device table `src` (rows x cols) as text on the device into a
// malloc'ed host buffer.  Returns 1 (nothing allocated) when an entry lies
// outside what the device formatter covers.
int format_table(busseq_handle* h, const bq::FmtSrc& src, int64_t rows, int64_t cols, char** buf, int64_t* len) {
  *buf = nullptr;
  *len = 0;
  if (rows == 0 || cols == 0) return BUSSEQ_OK;
  if (rows > INT_MAX) return fail(BUSSEQ_ERR_ARG, "table of %lld rows", (long long)rows);
  int64_t* d_len = nullptr;
  int* d_bad = nullptr;
  char* d_txt = nullptr;
  char* host = nullptr;
  int bad = 0;
  std::vector<int64_t> off((size_t)rows + 1, 0);
  cudaError_t e = cudaMallocAsync((void**)&d_len, (size_t)(rows + 1) * sizeof(int64_t), h->stream);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_bad, sizeof(int), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int), h->stream);
  if (e == cudaSuccess) {
    bq::k_fmt_row_len<<<(unsigned)rows, 256, 0, h->stream>>>(src, cols, d_len, d_bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(off.data() + 1, d_len, (size_t)rows * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  int64_t total = 0;
  if (e == cudaSuccess && !bad) {
    for (int64_t i = 0; i < rows; ++i) off[i + 1] += off[i];
    total = off[rows];
    host = static_cast<char*>(malloc((size_t)std::max<int64_t>(total, 1)));
    if (!host) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_len, off.data(), (size_t)rows * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_txt, (size_t)std::max<int64_t>(total, 1), h->stream);
    if (e == cudaSuccess) {
      bq::k_fmt_rows<<<(unsigned)rows, 256, 0, h->stream>>>(src, cols, d_len, d_txt);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, d_txt, (size_t)total, cudaMemcpyDeviceToHost, h->stream);
  }
  if (d_txt) cudaFreeAsync(d_txt, h->stream);
  if (d_bad) cudaFreeAsync(d_bad, h->stream);
  if (d_len) cudaFreeAsync(d_len, h->stream);
  const cudaError_t e2 = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) {
    free(host);
    return fail(e == cudaErrorMemoryAllocation ? BUSSEQ_ERR_NOMEM : BUSSEQ_ERR_CUDA, "formatting a table: %s",
                cudaGetErrorString(e));
  }
  if (bad) return 1;
  *buf = host;
  *len = total;
  return BUSSEQ_OK;
}

}  // namespace

extern "C" {

// X (which = 0) or Z (which = 1) of the last sweep, or the batch-corrected
// counts (which = 2), as the text of _post_X.txt / _post_Z.txt /
// _corrected_X.txt (the host writer's layout), formatted on the device; *buf
// is malloc'ed, the caller frees it.
int busseq_internal_format_xz(busseq_handle* h, int which, char** buf, int64_t* len) {
  if (!h || !buf || !len) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  const bq::DevState& s = h->s;
  const int64_t N = s.N;
  bq::FmtSrc src{s.X, bq::FMT_I32, s.Gp, 1};
  int32_t* d_tab = nullptr;
  if (which == 1) {  // Z unpacked from its bit mask into a temporary int table
    TRY(zmask_from_zval(h));
    CUDA_TRY(cudaMalloc((void**)&d_tab, std::max<size_t>((size_t)N * s.G * sizeof(int32_t), 4)));
    bq::k_z_dense_i32<<<std::min<unsigned>(blocks_for(N * s.Gw, 256), 152 * 16), 256, 0, h->stream>>>(s, d_tab, s.G);
    src = bq::FmtSrc{d_tab, bq::FMT_I32, s.G, 1};
  } else if (which == 2) {  // the corrected counts into a temporary int table
    CUDA_TRY(cudaMalloc((void**)&d_tab, std::max<size_t>((size_t)N * s.G * sizeof(int32_t), 4)));
    const int r = busseq_corrected_counts(h, d_tab, 1);
    if (r != BUSSEQ_OK) {
      cudaFree(d_tab);
      return r;
    }
    src = bq::FmtSrc{d_tab, bq::FMT_I32, s.G, 1};
  }
  const int r = format_table(h, src, N, s.G, buf, len);
  if (d_tab) cudaFree(d_tab);
  if (r == 1) return fail(BUSSEQ_ERR_STATE, "table outside the device formatter");  // integers never are
  return r;
}

// The posterior summaries of the imputation as text (which: 0 E[X] for
// _post_X_mean.txt, 1 P(Z = 1) for _post_Z_prob.txt), formatted on the device.
// Returns 1 when a value lies outside the device formatter.
int busseq_internal_format_zx_summary(busseq_handle* h, int which, char** buf, int64_t* len) {
  if (!h || !buf || !len) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  if (!h->opt.zx_summaries) return fail(BUSSEQ_ERR_STATE, "the chain was created without zx_summaries");
  if (!h->finished || h->n_kept <= 0 || !h->s.acc_zn)
    return fail(BUSSEQ_ERR_STATE, "no finished run with kept sweeps");
  CUDA_TRY(cudaSetDevice(h->device));
  const bq::DevState& s = h->s;
  float* d = nullptr;
  CUDA_TRY(cudaMallocAsync((void**)&d, std::max<size_t>((size_t)s.N * s.G * sizeof(float), 4), h->stream));
  float* xm = which == 0 ? d : nullptr;
  float* zp = which == 0 ? nullptr : d;
  bq::k_zx_summary<<<152 * 8, 256, 0, h->stream>>>(s, h->n_kept, xm, zp);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && s.nz0 > 0) {
    bq::k_zx_summary_zeros<<<152 * 8, 256, 0, h->stream>>>(s, h->n_kept, xm, zp);
    e = cudaGetLastError();
  }
  int r = BUSSEQ_OK;
  if (e == cudaSuccess) r = format_table(h, bq::FmtSrc{d, bq::FMT_F32, s.G, 1}, s.N, s.G, buf, len);
  cudaFreeAsync(d, h->stream);
  const cudaError_t e2 = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess && r == BUSSEQ_OK) e = e2;
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "zx summaries: %s", cudaGetErrorString(e));
  return r;
}

// One _preserved_*.txt table (which: 0 gamma, 1 alpha, 2 L, 3 beta, 4 p, 5 nu,
// 6 delta, 7 phi, 8 W, 9 pi; rows = scalars, columns = kept sweeps, as
// busseq_get_preserved lays them out), formatted on the device.  Returns 1 when
// a value lies outside the device formatter (the caller then formats on the
// host).
int busseq_internal_format_preserved(busseq_handle* h, int which, char** buf, int64_t* len) {
  if (!h || !buf || !len) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  const bq::DevState& s = h->s;
  if (!h->finished || !s.keep_draws) return fail(BUSSEQ_ERR_STATE, "no finished run with kept draws");
  CUDA_TRY(cudaSetDevice(h->device));
  const int64_t nk = h->n_kept, G = s.G, N = s.N;
  const int B = s.B, K = s.K;
  const void* p = nullptr;
  int kind = bq::FMT_F32;
  int64_t nscal = 0;
  switch (which) {
    case 0: p = s.keep_gamma; nscal = 2 * B; break;
    case 1: p = s.keep_alpha; nscal = G; break;
    case 2: p = s.keep_L; nscal = (K - 1) * G; kind = bq::FMT_I8; break;
    case 3: p = s.keep_beta; nscal = (K - 1) * G; break;
    case 4: p = s.keep_ptau; nscal = 2; break;
    case 5: p = s.keep_nu; nscal = (B - 1) * G; break;
    case 6: p = s.keep_delta; nscal = N; break;
    case 7: p = s.keep_phi; nscal = (int64_t)B * G; break;
    case 8: p = s.keep_W; nscal = N; kind = bq::FMT_I16; break;
    case 9: p = s.keep_pi; nscal = (int64_t)B * K; break;
    default: return fail(BUSSEQ_ERR_ARG, "no preserved table %d", which);
  }
  return format_table(h, bq::FmtSrc{p, kind, 1, nscal}, nscal, nk, buf, len);
}

int busseq_internal_dims(busseq_handle* h, int32_t* B, int32_t* K, int64_t* G, int64_t* N, int32_t* n_kept,
                         int32_t* kept_draws) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  *B = h->s.B;
  *K = h->s.K;
  *G = h->s.G;
  *N = h->s.N;
  *n_kept = h->finished ? h->n_kept : 0;
  *kept_draws = h->s.keep_draws;
  return BUSSEQ_OK;
}
const char* busseq_version(void) { return "busseq_gb300 0.1 (sm_103a)"; }

int busseq_create(const busseq_dims* dims, const int32_t* Y, int32_t Y_is_device, const busseq_options* optp,
                  busseq_handle** out) {
  if (!dims || !Y || !out) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  *out = nullptr;
  const int B = dims->B, K = dims->K;
  const int64_t G = dims->G;
  if (B < 2) return fail(BUSSEQ_ERR_ARG, "The batch number must be greater than one.");
  if (B > BUSSEQ_MAX_BATCHES) return fail(BUSSEQ_ERR_ARG, "at most %d batches are supported", BUSSEQ_MAX_BATCHES);
  if (K < 1 || K > BUSSEQ_MAX_TYPES) return fail(BUSSEQ_ERR_ARG, "K must be in 1..%d", BUSSEQ_MAX_TYPES);
  if (G < 1) return fail(BUSSEQ_ERR_ARG, "G must be positive");
  if (!dims->n_b) return fail(BUSSEQ_ERR_ARG, "n_b is NULL");
  int64_t N = 0;
  for (int b = 0; b < B; ++b) {
    if (dims->n_b[b] < K)
      return fail(BUSSEQ_ERR_ARG, "The sample size in any batch must be greater than the assumed cell type number.");
    N += dims->n_b[b];
  }
  if (N >= INT_MAX) return fail(BUSSEQ_ERR_ARG, "too many cells");
  busseq_options opt{};
  if (optp) opt = *optp;
  else opt.p0 = 0.25;
  if (!(opt.p0 > 0.0 && opt.p0 < 1.0)) return fail(BUSSEQ_ERR_ARG, "p0 must be in (0, 1)");
  CUDA_TRY(cudaSetDevice(opt.device));
  // the cell passes stage 48 KB of X rows per CTA (with their static shared
  // memory, above the 48 KB default)
  CUDA_TRY(cudaFuncSetAttribute(bq::k_delta, cudaFuncAttributeMaxDynamicSharedMemorySize, bq::DELTA_SMEM));
  CUDA_TRY(cudaFuncSetAttribute(bq::k_w_mh, cudaFuncAttributeMaxDynamicSharedMemorySize, bq::W_SMEM));

  busseq_handle* h = new busseq_handle();
  h->device = opt.device;
  h->opt = opt;
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    delete h;
    return fail(BUSSEQ_ERR_CUDA, "cudaStreamCreate / cudaEventCreate failed");
  }
  h->stream = h->own_stream;
  h->n_b.assign(dims->n_b, dims->n_b + B);
  h->off.assign(B + 1, 0);
  for (int b = 0; b < B; ++b) h->off[b + 1] = h->off[b] + h->n_b[b];
  const int r = [&]() -> int {
    bq::DevState& s = h->s;
    s.B = B;
    s.K = K;
    s.G = G;
    s.N = N;
    s.Gp = round_up(G, bq::GENE_TILE);
    s.Gw = s.Gp / 32;
    s.n_tiles = (int)((G + bq::GENE_TILE - 1) / bq::GENE_TILE);
    // default chunk length: 128 cells for the random-walk sampler when a
    // (batch, type) segment averages under 512 cells (config 1: 1.8 % faster
    // per sweep than 256), else 256 (config 4: 2 % faster than 128; with the
    // gradient-based update, whose passes build per-chunk digamma tables,
    // config 2: 0.8 % faster); busseq_autotune tunes it
    const int64_t mean_seg = N / std::max<int64_t>(1, (int64_t)B * K);
    s.CG = opt.chunk_cells > 0 ? std::min(opt.chunk_cells, bq::MAX_CG)
                               : (opt.hmc_leapfrog <= 0 && mean_seg < 512 ? 128 : bq::MAX_CG);
    s.cap_g = 0;
    s.cap_c = 0;
    for (int b = 0; b < B; ++b) {
      s.cap_g += h->n_b[b] / s.CG + K;
      s.cap_c += h->n_b[b] / bq::CELL_TILE + K;
    }
    s.w_update = opt.w_update == BUSSEQ_W_GIBBS ? BUSSEQ_W_GIBBS : BUSSEQ_W_MH;
    s.nb_inv_cap = opt.test_nb_inv_cap > 0 ? std::min(opt.test_nb_inv_cap, bq::NB_INV_MAX_K) : bq::NB_INV_MAX_K;
    s.seed = opt.seed;
    s.n_burnin = 0;
    s.n_unchanged = INT_MAX;
    const int64_t Gp = s.Gp;
    int32_t* Yd = nullptr;
    TRY(h->alloc(&Yd, N * Gp));
    s.Y = Yd;
    // one extra all-zero row: the gene passes pad their cell chunks with it
    TRY(h->alloc(&s.X, (N + 1) * Gp));
    uint32_t* y0m = nullptr;  // one extra all-zero row, read for the padding row of a chunk
    TRY(h->alloc(&y0m, (N + 1) * s.Gw));
    s.y0m = y0m;
    TRY(h->alloc(&s.zm, N * s.Gw));
    int32_t *bo = nullptr, *boff = nullptr;
    TRY(h->alloc(&bo, N));
    TRY(h->alloc(&boff, B + 1));
    s.batch_of = bo;
    s.batch_off = boff;
    TRY(h->alloc(&s.W, N));
    TRY(h->alloc(&s.L, K * Gp));
    TRY(h->alloc(&s.alpha, Gp));
    TRY(h->alloc(&s.mu_alpha, Gp));
    TRY(h->alloc(&s.beta, K * Gp));
    TRY(h->alloc(&s.nu, B * Gp));
    TRY(h->alloc(&s.mu_nu, B));
    TRY(h->alloc(&s.delta, N));
    TRY(h->alloc(&s.mu_delta, N));
    TRY(h->alloc(&s.Dexp, N));
    TRY(h->alloc(&s.phi, B * Gp));
    TRY(h->alloc(&s.gamma, 2 * B));
    TRY(h->alloc(&s.pi, B * K));
    TRY(h->alloc(&s.p_tau0, 2));
    TRY(h->alloc(&s.E, (int64_t)B * K * Gp));
    TRY(h->alloc(&s.alpha_p, Gp));
    TRY(h->alloc(&s.beta_p, K * Gp));
    TRY(h->alloc(&s.nu_p, B * Gp));
    TRY(h->alloc(&s.delta_p, N));
    TRY(h->alloc(&s.phi_p, B * Gp));
    TRY(h->alloc(&s.phi_tab, (int64_t)B * bq::PHI_TAB * Gp));
    TRY(h->alloc(&s.phi_lgd0, B * Gp));
    TRY(h->alloc(&s.gamma_p, 2 * B));
    TRY(h->alloc(&s.perm, N));
    TRY(h->alloc(&s.gchunk, s.cap_g));
    TRY(h->alloc(&s.ctile, s.cap_c));
    TRY(h->alloc(&s.seg_cnt, B * K));
    TRY(h->alloc(&s.part, (int64_t)s.cap_g * bq::NSLOT * Gp));
    // the gradient-based block update
    s.hmc_L = std::max(0, opt.hmc_leapfrog);
    s.hmc_gene = s.hmc_L > 0 && opt.hmc_gene_accept ? 1 : 0;
    s.hmc_D = Gp * (1 + K + 2 * B) + N;
    if (s.hmc_L > 0) {
      TRY(h->alloc(&s.psi, B * Gp));
      TRY(h->alloc(&s.hmc_mom, s.hmc_D));
      TRY(h->alloc(&s.hmc_mom0, s.hmc_D));
      TRY(h->alloc(&s.hmc_grad, s.hmc_D));
      TRY(h->alloc(&s.hmc_mass, s.hmc_D));
      TRY(h->alloc(&s.hmc_th0, s.hmc_D));
      TRY(h->alloc(&s.hmc_part, (int64_t)s.cap_g * bq::NSLOT * Gp));
      TRY(h->alloc(&s.hmc_cpart, (int64_t)s.n_tiles * N));
      TRY(h->alloc(&s.hmc_cpartw, (int64_t)s.n_tiles * N));
      TRY(h->alloc(&s.hmc_hpart, (int64_t)s.n_tiles * s.cap_g + STATIC_CTAS));
      TRY(h->alloc(&s.hmc_epart, (int64_t)blocks_for(s.hmc_D, 256)));
      TRY(h->alloc(&s.hmc_sc, (int64_t)bq::HS_COUNT));
      TRY(h->alloc(&s.hmc_fis, s.hmc_D));
      CUDA_TRY(cudaMemsetAsync(s.hmc_fis, 0, (size_t)s.hmc_D * sizeof(float), h->stream));
      if (s.hmc_gene) {
        TRY(h->alloc(&s.hmc_e, s.hmc_D));
        TRY(h->alloc(&s.hmc_eb, Gp));
        TRY(h->alloc(&s.hmc_gacc, Gp));
      }
      s.hmc_nb = (K + B - 1 <= bq::HMC_BLOCK_MAX) ? K + B - 1 : 0;
      if (s.hmc_nb > 0) {
        TRY(h->alloc(&s.hmc_chol, (int64_t)bq::HMC_BLOCK_MAX * (bq::HMC_BLOCK_MAX + 1) / 2 * G));
        TRY(h->alloc(&s.hmc_wbk, (int64_t)B * K * G));
        TRY(h->alloc(&s.hmc_minv, (int64_t)bq::HMC_BLOCK_MAX * bq::HMC_BLOCK_MAX * G));
        TRY(h->alloc(&s.hmc_epart_b, (int64_t)blocks_for(G * 32, 256)));
      }
      bq::k_hmc_unit_mass<<<blocks_for(s.hmc_D, 256), 256, 0, h->stream>>>(s);
      LAUNCH_CHECK("k_hmc_unit_mass");
    }
    TRY(h->alloc(&s.tpart, std::max<int64_t>((int64_t)s.n_tiles * bq::MAX_B, 2 * (int64_t)blocks_for(G, 32))));
    TRY(h->alloc(&s.cnt_tile, s.n_tiles));
    TRY(h->alloc(&s.cnt_glob, 8));
    TRY(h->alloc(&s.iter, 1));
    TRY(h->alloc(&s.err, 1));
    TRY(h->alloc(&s.lr_gamma, 2 * B));
    TRY(h->alloc(&s.lr_alpha, G));
    TRY(h->alloc(&s.lr_beta, K * G));
    TRY(h->alloc(&s.lr_nu, B * G));
    TRY(h->alloc(&s.lr_delta, N));
    TRY(h->alloc(&s.lr_phi, B * G));
    TRY(h->alloc(&s.lr_W, N));
    TRY(h->alloc(&h->ll_ik, (int64_t)K * N));
    TRY(h->alloc(&h->bic_out, 2));
    int64_t* libsize;
    int *ymax_d, *bad;
    int32_t* rowcnt;
    TRY(h->alloc(&libsize, N));
    TRY(h->alloc(&ymax_d, 1));
    TRY(h->alloc(&bad, 1));
    TRY(h->alloc(&rowcnt, N));
    TRY(h->alloc(&s.seg_chunk, (int64_t)B * K));
    TRY(h->alloc(&s.beta_acc, (int64_t)K * Gp));

    // ---- upload ----------------------------------------------------------
    CUDA_TRY(cudaMemcpy2DAsync(Yd, Gp * sizeof(int32_t), Y, G * sizeof(int32_t), G * sizeof(int32_t), N,
                               Y_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    std::vector<int32_t> bo_h(N);
    for (int b = 0; b < B; ++b)
      for (int64_t i = h->off[b]; i < h->off[b + 1]; ++i) bo_h[i] = b;
    CUDA_TRY(cudaMemcpyAsync(bo, bo_h.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(boff, h->off.data(), (B + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    const float ptau0[2] = {(float)opt.p0, bq::TAU0_INIT};
    CUDA_TRY(cudaMemcpyAsync(s.p_tau0, ptau0, sizeof(ptau0), cudaMemcpyHostToDevice, h->stream));
    const int big = INT_MAX;
    CUDA_TRY(cudaMemcpyAsync(bad, &big, sizeof(int), cudaMemcpyHostToDevice, h->stream));

    // ---- initialisation (BUSseq_gpu.cu:1163-1244) --------------------------
    bq::k_init_scan<<<(unsigned)N, 256, 0, h->stream>>>(s, libsize, ymax_d, rowcnt);
    LAUNCH_CHECK("k_init_scan");
    int ymax = 0;
    std::vector<int32_t> rowcnt_h(N);
    CUDA_TRY(cudaMemcpyAsync(&ymax, ymax_d, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaMemcpyAsync(rowcnt_h.data(), rowcnt, N * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (ymax < 0) return fail(BUSSEQ_ERR_ARG, "counts must be non-negative");
    if (ymax > (1 << 26)) return fail(BUSSEQ_ERR_ARG, "counts above 2^26 are not supported");
    s.ymax = std::max(ymax, 1);
    s.n_static = B * ((s.ymax + bq::ZX_THREADS - 1) / bq::ZX_THREADS);
    int32_t* hist;
    TRY(h->alloc(&hist, (int64_t)B * (s.ymax + 1)));
    s.yhist = hist;
    TRY(h->alloc(&s.gstat, (int64_t)s.n_static * 4));
    // the entries with Y == 0 (row-major) and their Z/X work units, one batch per unit
    std::vector<int64_t> rowoff_h(N + 1, 0);
    for (int64_t i = 0; i < N; ++i) rowoff_h[i + 1] = rowoff_h[i] + rowcnt_h[i];
    s.nz0 = rowoff_h[N];
    // work units of zx_unit entries (the options' launch shape, at most ZX_UNIT)
    const int64_t zx_unit = opt.zx_unit > 0 ? std::max(16, std::min(opt.zx_unit, bq::ZX_UNIT)) : bq::ZX_UNIT;
    std::vector<int2> zcta_h;
    std::vector<int32_t> zbatch_h, zfirst_h(B + 1, 0);
    for (int b = 0; b < B; ++b) {
      zfirst_h[b] = (int32_t)zcta_h.size();
      const int64_t lo = rowoff_h[h->off[b]], hi = rowoff_h[h->off[b + 1]];
      for (int64_t e = lo; e < hi; e += zx_unit) {
        if (e > INT_MAX) return fail(BUSSEQ_ERR_ARG, "too many zero counts (more than 2^31)");
        zcta_h.push_back(make_int2((int)e, (int)std::min<int64_t>(zx_unit, hi - e)));
        zbatch_h.push_back(b);
      }
    }
    zfirst_h[B] = (int32_t)zcta_h.size();
    s.n_zcta = (int)zcta_h.size();
    int64_t* rowoff;
    int2 *zij, *zcta;
    int32_t *zbatch, *zfirst;
    TRY(h->alloc(&rowoff, N + 1));
    TRY(h->alloc(&zij, std::max<int64_t>(1, s.nz0)));
    TRY(h->alloc(&s.zval, std::max<int64_t>(1, s.nz0)));
    TRY(h->alloc(&zcta, std::max(1, s.n_zcta)));
    TRY(h->alloc(&zbatch, std::max(1, s.n_zcta)));
    TRY(h->alloc(&zfirst, B + 1));
    TRY(h->alloc(&s.gpart, (int64_t)std::max(1, s.n_zcta) * bq::GSLOT));
    TRY(h->alloc(&s.zx_gtab, (int64_t)B * bq::ZX_HIST));
    TRY(h->alloc(&s.zx_ctr, 4));
    // the Gamma-Poisson lists of the units and the chunks of k_zx_gp (ZGP_UNITS units of one batch)
    std::vector<int4> zgchunk_h;
    std::vector<int32_t> gfirst_h(B + 1, 0);
    for (int b = 0; b < B; ++b) {
      gfirst_h[b] = (int32_t)zgchunk_h.size();
      for (int u = zfirst_h[b]; u < zfirst_h[b + 1]; u += bq::ZGP_UNITS)
        zgchunk_h.push_back(make_int4(u, std::min(bq::ZGP_UNITS, zfirst_h[b + 1] - u), b, 0));
    }
    gfirst_h[B] = (int32_t)zgchunk_h.size();
    s.n_gchunk = (int)zgchunk_h.size();
    int4* zgchunk;
    int32_t* gfirst;
    TRY(h->alloc(&s.zgp_rec, std::max<int64_t>(1, s.nz0)));
    TRY(h->alloc(&s.zgp_mp, std::max<int64_t>(1, s.nz0)));
    TRY(h->alloc(&s.zgp_cnt, std::max(1, s.n_zcta)));
    TRY(h->alloc(&zgchunk, std::max(1, s.n_gchunk)));
    TRY(h->alloc(&gfirst, B + 1));
    TRY(h->alloc(&s.gpart_gp, (int64_t)std::max(1, s.n_gchunk) * bq::GSLOT));
    {  // the Z/X launches: ZX_CTAS_PER_SM CTAs on every SM (and at least one per static-term slice)
      int nsm = 0;
      CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, opt.device));
      const int64_t want = (s.n_zcta + bq::ZX_THREADS / 32 - 1) / (bq::ZX_THREADS / 32);
      const int per_sm = opt.zx_ctas_per_sm > 0 ? std::min(opt.zx_ctas_per_sm, bq::ZX_CTAS_PER_SM) : bq::ZX_CTAS_PER_SM;
      s.zx_ctas = (int)std::max<int64_t>({(int64_t)s.n_static, std::min<int64_t>(want, (int64_t)nsm * per_sm),
                                          (int64_t)1});
      const int64_t want_gp = (s.n_gchunk + bq::ZX_THREADS / 32 - 1) / (bq::ZX_THREADS / 32);
      s.zgp_ctas = (int)std::max<int64_t>(std::min<int64_t>(want_gp, (int64_t)nsm * bq::ZGP_CTAS_PER_SM), 1);
    }
    if (s.n_gchunk) {
      CUDA_TRY(cudaMemcpyAsync(zgchunk, zgchunk_h.data(), zgchunk_h.size() * sizeof(int4), cudaMemcpyHostToDevice,
                               h->stream));
    }
    CUDA_TRY(cudaMemcpyAsync(gfirst, gfirst_h.data(), (B + 1) * 4, cudaMemcpyHostToDevice, h->stream));
    s.zgchunk = zgchunk;
    s.gfirst = gfirst;
    CUDA_TRY(cudaMemcpyAsync(rowoff, rowoff_h.data(), (N + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    if (s.n_zcta) {
      CUDA_TRY(cudaMemcpyAsync(zcta, zcta_h.data(), zcta_h.size() * sizeof(int2), cudaMemcpyHostToDevice, h->stream));
      CUDA_TRY(cudaMemcpyAsync(zbatch, zbatch_h.data(), zbatch_h.size() * 4, cudaMemcpyHostToDevice, h->stream));
    }
    CUDA_TRY(cudaMemcpyAsync(zfirst, zfirst_h.data(), (B + 1) * 4, cudaMemcpyHostToDevice, h->stream));
    s.zij = zij;
    s.zcta = zcta;
    s.zcta_batch = zbatch;
    s.zfirst = zfirst;
    bq::k_zlist_fill<<<blocks_for(N, 8), 256, 0, h->stream>>>(s, rowoff, zij);
    LAUNCH_CHECK("k_zlist_fill");
    bq::k_init_hist<<<(unsigned)N, 256, 0, h->stream>>>(s, hist);
    LAUNCH_CHECK("k_init_hist");
    bq::k_init_w_delta<<<blocks_for(N, 256), 256, 0, h->stream>>>(s, libsize, bad);
    LAUNCH_CHECK("k_init_w_delta");
    int bad_h = 0;
    CUDA_TRY(cudaMemcpyAsync(&bad_h, bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (bad_h != INT_MAX) return fail(BUSSEQ_ERR_ARG, "cell %d has no counts (library size 0)", bad_h);
    bq::k_sort_pi<<<B, 1024, 0, h->stream>>>(s, 0, 0);
    LAUNCH_CHECK("k_sort_pi");
    bq::k_init_raw<<<dim3(s.n_tiles, s.cap_g), bq::GENE_TILE, 0, h->stream>>>(s);
    LAUNCH_CHECK("k_init_raw");
    const int64_t nfin = std::max<int64_t>(std::max<int64_t>(N, (int64_t)B * Gp), (int64_t)B * K);
    bq::k_init_finish<<<blocks_for(nfin, 256), 256, 0, h->stream>>>(s, 1);
    LAUNCH_CHECK("k_init_finish");
    CUDA_TRY(cudaMemcpyAsync(s.X, s.Y, (size_t)N * Gp * sizeof(int32_t), cudaMemcpyDeviceToDevice, h->stream));
    {
      // static tables of the phi update and of the HMC log-likelihood change:
      // counts of small Y, the larger Y in cell order
      const int64_t nbg = (int64_t)B * G;
      TRY(h->alloc(&s.phi_cnt, (int64_t)B * bq::PHI_TAB * Gp));
      TRY(h->alloc(&s.phi_static, B * Gp));
      const int nsl = bq::PHI_HIST_SLICES;
      int64_t *nbig, *soff;
      TRY(h->alloc(&nbig, nsl * nbg, true));
      TRY(h->alloc(&soff, nsl * nbg, true));
      const dim3 hist_grid((unsigned)s.n_tiles, (unsigned)B, (unsigned)nsl);
      bq::k_phi_hist<<<hist_grid, bq::GENE_TILE, 0, h->stream>>>(s, nbig, nullptr, 0);
      LAUNCH_CHECK("k_phi_hist");
      std::vector<int64_t> n_h((size_t)nsl * nbg), off_h(nbg + 1, 0), soff_h((size_t)nsl * nbg);
      CUDA_TRY(cudaMemcpyAsync(n_h.data(), nbig, n_h.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
      CUDA_TRY(cudaStreamSynchronize(h->stream));
      // the large values of (batch, gene) t in cell order: slice after slice
      for (int64_t t = 0; t < nbg; ++t) {
        int64_t p = off_h[t];
        for (int q = 0; q < nsl; ++q) {
          soff_h[(size_t)q * nbg + t] = p;
          p += n_h[(size_t)q * nbg + t];
        }
        off_h[t + 1] = p;
      }
      TRY(h->alloc(&s.phi_big_off, nbg + 1));
      TRY(h->alloc(&s.phi_big_y, std::max<int64_t>(1, off_h[nbg])));
      CUDA_TRY(cudaMemcpyAsync(s.phi_big_off, off_h.data(), (nbg + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                               h->stream));
      CUDA_TRY(cudaMemcpyAsync(soff, soff_h.data(), soff_h.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                               h->stream));
      bq::k_phi_hist<<<hist_grid, bq::GENE_TILE, 0, h->stream>>>(s, nbig, soff, 1);
      LAUNCH_CHECK("k_phi_hist");
      CUDA_TRY(cudaStreamSynchronize(h->stream));  // off_h leaves scope
    }
    CUDA_TRY(cudaMemsetAsync(s.zm, 0, (size_t)N * s.Gw * sizeof(uint32_t), h->stream));
    CUDA_TRY(cudaMemsetAsync(s.zval, 0, (size_t)std::max<int64_t>(1, s.nz0), h->stream));
    CUDA_TRY(cudaMemsetAsync(s.iter, 0, sizeof(int), h->stream));
    return check_device_error(h);
  }();
  if (r != BUSSEQ_OK) {
    delete h;
    return r;
  }
  *out = h;
  return BUSSEQ_OK;
}

void busseq_destroy(busseq_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
}

int busseq_begin(busseq_handle* h, int32_t n_iter, int32_t n_burnin, int32_t n_unchanged) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (n_iter < 0 || n_burnin < 0) return fail(BUSSEQ_ERR_ARG, "iteration counts must be non-negative");
  if (n_burnin > n_iter) return fail(BUSSEQ_ERR_ARG, "Burn-in iterations must be less than total number of iterations.");
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (h->g_burn) { cudaGraphExecDestroy(h->g_burn); h->g_burn = nullptr; }
  if (h->g_keep) { cudaGraphExecDestroy(h->g_keep); h->g_keep = nullptr; }
  for (void* p : h->run_allocs) cudaFree(p);
  h->run_allocs.clear();
  bq::DevState& s = h->s;
  const int64_t G = s.G, N = s.N;
  const int B = s.B, K = s.K;
  h->n_iter = n_iter;
  h->n_burnin = n_burnin;
  h->n_unchanged = n_unchanged;
  h->n_kept = n_iter - n_burnin;
  h->iter_host = 0;
  h->finished = false;
  h->est_valid = false;
  s.n_burnin = n_burnin;
  s.n_unchanged = n_unchanged;
  s.n_kept = h->n_kept;
  s.keep_draws = (h->opt.keep_draws && h->n_kept > 0) ? 1 : 0;
  TRY(h->alloc(&s.acc_alpha, G, true));
  TRY(h->alloc(&s.acc_beta, K * G, true));
  TRY(h->alloc(&s.acc_L, K * G, true));
  TRY(h->alloc(&s.acc_nu, B * G, true));
  TRY(h->alloc(&s.acc_delta, N, true));
  TRY(h->alloc(&s.acc_phi, B * G, true));
  TRY(h->alloc(&s.acc_gamma, 2 * B, true));
  TRY(h->alloc(&s.acc_pi, B * K, true));
  TRY(h->alloc(&s.acc_ptau, 2, true));
  TRY(h->alloc(&s.acc_wcnt, N * K, true));
  s.acc_zn = nullptr;
  s.acc_xs = nullptr;
  if (h->opt.zx_summaries && h->n_kept > 0) {
    TRY(h->alloc(&s.acc_zn, std::max<int64_t>(1, s.nz0), true));
    TRY(h->alloc(&s.acc_xs, std::max<int64_t>(1, s.nz0), true));
  }
  s.keep_gamma = s.keep_alpha = s.keep_beta = s.keep_ptau = s.keep_nu = s.keep_delta = s.keep_phi = s.keep_pi =
      nullptr;
  s.keep_L = nullptr;
  s.keep_W = nullptr;
  if (s.keep_draws) {
    const int64_t nk = h->n_kept;
    TRY(h->alloc(&s.keep_gamma, nk * 2 * B, true));
    TRY(h->alloc(&s.keep_alpha, nk * G, true));
    TRY(h->alloc(&s.keep_beta, nk * std::max(1, K - 1) * G, true));
    TRY(h->alloc(&s.keep_L, nk * std::max(1, K - 1) * G, true));
    TRY(h->alloc(&s.keep_ptau, nk * 2, true));
    TRY(h->alloc(&s.keep_nu, nk * (B - 1) * G, true));
    TRY(h->alloc(&s.keep_delta, nk * N, true));
    TRY(h->alloc(&s.keep_phi, nk * B * G, true));
    TRY(h->alloc(&s.keep_W, nk * N, true));
    TRY(h->alloc(&s.keep_pi, nk * B * K, true));
  }
  if (s.hmc_L > 0) {  // step size and its adaptation start afresh with every run
    double sc[bq::HS_COUNT] = {0.0};
    sc[bq::HS_EPS] = bq::HMC_EPS0;
    sc[bq::HS_MU] = log(10.0 * bq::HMC_EPS0);
    CUDA_TRY(cudaMemcpyAsync(s.hmc_sc, sc, sizeof sc, cudaMemcpyHostToDevice, h->stream));
  }
  CUDA_TRY(cudaMemsetAsync(s.iter, 0, sizeof(int), h->stream));
  CUDA_TRY(cudaMemsetAsync(s.cnt_tile, 0, s.n_tiles * sizeof(unsigned), h->stream));
  CUDA_TRY(cudaMemsetAsync(s.cnt_glob, 0, 8 * sizeof(unsigned), h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  TRY(capture(h, 0, &h->g_burn));
  TRY(capture(h, 1, &h->g_keep));
  h->begun = true;
  return BUSSEQ_OK;
}

int busseq_sweeps(busseq_handle* h, int32_t count) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (!h->begun) return fail(BUSSEQ_ERR_STATE, "busseq_begin has not been called");
  if (count < 0 || h->iter_host + count > h->n_iter)
    return fail(BUSSEQ_ERR_ARG, "requested sweeps exceed the run length (%d of %d done)", h->iter_host, h->n_iter);
  for (int c = 0; c < count; ++c) {
    cudaGraphExec_t g = h->iter_host < h->n_burnin ? h->g_burn : h->g_keep;
    CUDA_TRY(cudaGraphLaunch(g, h->stream));
    ++h->iter_host;
  }
  return BUSSEQ_OK;
}

int busseq_synchronize(busseq_handle* h) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  return check_device_error(h);
}

int busseq_finish(busseq_handle* h) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (!h->begun || h->iter_host != h->n_iter)
    return fail(BUSSEQ_ERR_STATE, "the run is not complete (%d of %d sweeps)", h->iter_host, h->n_iter);
  TRY(check_device_error(h));
  h->finished = true;
  h->est_valid = false;
  return ensure_estimates(h);
}

int busseq_run(busseq_handle* h, int32_t n_iter, int32_t n_burnin, int32_t n_unchanged) {
  TRY(busseq_begin(h, n_iter, n_burnin, n_unchanged));
  TRY(busseq_sweeps(h, n_iter));
  return busseq_finish(h);
}

int busseq_get_estimates(busseq_handle* h, busseq_estimates* o) {
  if (!h || !o) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  TRY(ensure_estimates(h));
  const bq::DevState& s = h->s;
  const int64_t G = s.G, N = s.N;
  const int B = s.B, K = s.K;
  const bq::Estimates& e = h->est;
  // Z is unpacked on the handle's stream while the estimates and X go to the
  // host on the side stream, so the two large reads overlap the unpacking.
  cudaStream_t side = h->side_stream;
  CUDA_TRY(cudaEventRecord(h->ev_fork[0], h->stream));
  CUDA_TRY(cudaStreamWaitEvent(side, h->ev_fork[0], 0));
  void* zdev = nullptr;
  if (o->Z) TRY(z_dense_async(h, 4, &zdev));
  auto cp = [&](void* dst, const void* src, size_t bytes) -> int {
    if (dst) CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, side));
    return BUSSEQ_OK;
  };
  TRY(cp(o->gamma, e.gamma, 2 * B * sizeof(double)));
  TRY(cp(o->alpha, e.alpha, G * sizeof(double)));
  if (K > 1) TRY(cp(o->L, e.L, (K - 1) * G * sizeof(double)));
  TRY(cp(o->beta, e.beta, K * G * sizeof(double)));
  TRY(cp(o->p_tau0, e.ptau, 2 * sizeof(double)));
  TRY(cp(o->nu, e.nu, B * G * sizeof(double)));
  TRY(cp(o->delta, e.delta, N * sizeof(double)));
  TRY(cp(o->phi, e.phi, B * G * sizeof(double)));
  TRY(cp(o->W, e.W, N * sizeof(int32_t)));
  TRY(cp(o->pi, e.pi, B * K * sizeof(double)));
  if (o->X) CUDA_TRY(cudaMemcpy2DAsync(o->X, G * 4, s.X, s.Gp * 4, G * 4, N, cudaMemcpyDeviceToHost, side));
  cudaError_t ez = cudaSuccess;
  if (zdev) {
    ez = cudaMemcpyAsync(o->Z, zdev, (size_t)N * G * 4, cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t ef = cudaFreeAsync(zdev, h->stream);
    if (ez == cudaSuccess) ez = ef;
  }
  const cudaError_t e1 = cudaStreamSynchronize(side);
  const cudaError_t e2 = cudaStreamSynchronize(h->stream);
  if (ez != cudaSuccess || e1 != cudaSuccess || e2 != cudaSuccess)
    return fail(BUSSEQ_ERR_CUDA, "estimates to the host: %s",
                cudaGetErrorString(ez != cudaSuccess ? ez : e1 != cudaSuccess ? e1 : e2));
  return BUSSEQ_OK;
}

int busseq_get_preserved(busseq_handle* h, busseq_preserved* o) {
  if (!h || !o) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  const bq::DevState& s = h->s;
  if (!h->finished) return fail(BUSSEQ_ERR_STATE, "no finished run");
  if (!s.keep_draws) return fail(BUSSEQ_ERR_STATE, "draws were not kept (set keep_draws)");
  const int64_t nk = h->n_kept, G = s.G, N = s.N;
  const int B = s.B, K = s.K;
  // device layout [kept][scalar] -> reference layout [scalar][kept]
  auto tr_f = [&](double* dst, const float* src, int64_t nscal) -> int {
    if (!dst || nscal <= 0) return BUSSEQ_OK;
    std::vector<float> buf((size_t)nk * nscal);
    CUDA_TRY(cudaMemcpy(buf.data(), src, buf.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int64_t it = 0; it < nk; ++it)
      for (int64_t j = 0; j < nscal; ++j) dst[j * nk + it] = buf[it * nscal + j];
    return BUSSEQ_OK;
  };
  TRY(tr_f(o->gamma, s.keep_gamma, 2 * B));
  TRY(tr_f(o->alpha, s.keep_alpha, G));
  TRY(tr_f(o->beta, s.keep_beta, (K - 1) * G));
  TRY(tr_f(o->p_tau0, s.keep_ptau, 2));
  TRY(tr_f(o->nu, s.keep_nu, (B - 1) * G));
  TRY(tr_f(o->delta, s.keep_delta, N));
  TRY(tr_f(o->phi, s.keep_phi, B * G));
  TRY(tr_f(o->pi, s.keep_pi, B * K));
  if (o->L && K > 1) {
    const int64_t ns = (K - 1) * G;
    std::vector<int8_t> buf((size_t)nk * ns);
    CUDA_TRY(cudaMemcpy(buf.data(), s.keep_L, buf.size(), cudaMemcpyDeviceToHost));
    for (int64_t it = 0; it < nk; ++it)
      for (int64_t j = 0; j < ns; ++j) o->L[j * nk + it] = buf[it * ns + j];
  }
  if (o->W) {
    std::vector<int16_t> buf((size_t)nk * N);
    CUDA_TRY(cudaMemcpy(buf.data(), s.keep_W, buf.size() * 2, cudaMemcpyDeviceToHost));
    for (int64_t it = 0; it < nk; ++it)
      for (int64_t j = 0; j < N; ++j) o->W[j * nk + it] = buf[it * N + j];
  }
  return BUSSEQ_OK;
}

int busseq_bic(busseq_handle* h, double* bic) {
  if (!h || !bic) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  TRY(ensure_estimates(h));
  const bq::DevState& s = h->s;
  const int ny = bq::bic_table_counts(s);
  char* scratch = nullptr;
  CUDA_TRY(cudaMallocAsync((void**)&scratch, (size_t)bq::bic_table_bytes(s, ny), h->stream));
  bq::BicTabs tb;
  tb.bg = reinterpret_cast<bq::BicGene*>(scratch);
  tb.eb = reinterpret_cast<double*>(scratch + (size_t)s.B * s.G * sizeof(bq::BicGene));
  tb.ty = tb.eb + (size_t)s.K * s.G;
  tb.ny = ny;
  bq::launch_bic(s, h->est, h->ll_ik, tb, h->bic_out, h->stream);
  cudaError_t e = cudaGetLastError();
  const cudaError_t e2 = cudaFreeAsync(scratch, h->stream);  // also when a launch failed
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "BIC kernels: %s", cudaGetErrorString(e));
  double out[2];
  CUDA_TRY(cudaMemcpyAsync(out, h->bic_out, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  *bic = out[0];
  return BUSSEQ_OK;
}

int busseq_corrected_counts(busseq_handle* h, int32_t* out, int32_t out_is_device) {
  if (!h || !out) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  TRY(ensure_estimates(h));
  const bq::DevState& s = h->s;
  if (s.N == 0 || s.G == 0) return BUSSEQ_OK;
  const size_t n_tab = (size_t)s.K * s.G, out_bytes = out_is_device ? 0 : (size_t)s.N * s.G * 4;
  const size_t off_sd = n_tab * sizeof(bq::corr::NbDist), off_nu = off_sd + n_tab * 8,
               off_out = off_nu + (size_t)s.B * s.G * 8, bytes = off_out + out_bytes;
  char* scratch = nullptr;
  CUDA_TRY(cudaMallocAsync((void**)&scratch, bytes, h->stream));
  bq::CorrTables tb{reinterpret_cast<bq::corr::NbDist*>(scratch), reinterpret_cast<double*>(scratch + off_sd),
                    reinterpret_cast<double*>(scratch + off_nu)};
  int32_t* dst = out_is_device ? out : reinterpret_cast<int32_t*>(scratch + off_out);
  bq::k_correct_prep<<<std::min<unsigned>(blocks_for((int64_t)n_tab, 256), 152 * 8), 256, 0, h->stream>>>(
      s, h->est, tb);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    const dim3 grid((unsigned)((s.G + 1023) / 1024), (unsigned)std::min<int64_t>(s.N, 65535));
    bq::k_correct<<<grid, 256, 0, h->stream>>>(s, h->est, tb, dst, s.G);  // 1024 genes of a row per CTA
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !out_is_device)
    e = cudaMemcpyAsync(out, dst, out_bytes, cudaMemcpyDeviceToHost, h->stream);
  const cudaError_t e2 = cudaFreeAsync(scratch, h->stream);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "k_correct: %s", cudaGetErrorString(e));
  return BUSSEQ_OK;
}

int busseq_get_zx_summaries(busseq_handle* h, float* x_mean, float* z_prob) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (!h->opt.zx_summaries) return fail(BUSSEQ_ERR_STATE, "the chain was created without zx_summaries");
  if (!h->finished || h->n_kept <= 0 || !h->s.acc_zn)
    return fail(BUSSEQ_ERR_STATE, "no finished run with kept sweeps");
  if (!x_mean && !z_prob) return BUSSEQ_OK;
  CUDA_TRY(cudaSetDevice(h->device));
  const bq::DevState& s = h->s;
  const size_t bytes = (size_t)s.N * s.G * sizeof(float);
  float* d = nullptr;
  CUDA_TRY(cudaMallocAsync((void**)&d, 2 * bytes, h->stream));
  float* dx = x_mean ? d : nullptr;
  float* dz = z_prob ? d + (size_t)s.N * s.G : nullptr;
  const unsigned grid = 152 * 8;
  bq::k_zx_summary<<<grid, 256, 0, h->stream>>>(s, h->n_kept, dx, dz);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && s.nz0 > 0) {
    bq::k_zx_summary_zeros<<<grid, 256, 0, h->stream>>>(s, h->n_kept, dx, dz);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && x_mean) e = cudaMemcpyAsync(x_mean, dx, bytes, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && z_prob) e = cudaMemcpyAsync(z_prob, dz, bytes, cudaMemcpyDeviceToHost, h->stream);
  const cudaError_t e2 = cudaFreeAsync(d, h->stream);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "zx summaries: %s", cudaGetErrorString(e));
  return BUSSEQ_OK;
}

int busseq_get_state(busseq_handle* h, busseq_state* o) {
  if (!h || !o) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const bq::DevState& s = h->s;
  const int64_t G = s.G, N = s.N, Gp = s.Gp;
  const int B = s.B, K = s.K;
  auto rows = [&](void* dst, const void* src, size_t esz, int64_t nrows) -> int {
    if (dst) CUDA_TRY(cudaMemcpy2D(dst, G * esz, src, Gp * esz, G * esz, nrows, cudaMemcpyDeviceToHost));
    return BUSSEQ_OK;
  };
  auto flat = [&](void* dst, const void* src, size_t bytes) -> int {
    if (dst) CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return BUSSEQ_OK;
  };
  TRY(rows(o->X, s.X, 4, N));
  if (o->Z) TRY(z_to_host(h, o->Z, 1));
  TRY(flat(o->W, s.W, N * 4));
  TRY(rows(o->L, s.L, 1, K));
  TRY(flat(o->alpha, s.alpha, G * 4));
  TRY(flat(o->mu_alpha, s.mu_alpha, G * 4));
  TRY(rows(o->beta, s.beta, 4, K));
  TRY(rows(o->nu, s.nu, 4, B));
  TRY(flat(o->mu_nu, s.mu_nu, B * 4));
  TRY(flat(o->delta, s.delta, N * 4));
  TRY(flat(o->mu_delta, s.mu_delta, N * 4));
  TRY(rows(o->phi, s.phi, 4, B));
  TRY(flat(o->gamma, s.gamma, 2 * B * 4));
  TRY(flat(o->pi, s.pi, B * K * 4));
  TRY(flat(o->p_tau0, s.p_tau0, 2 * 4));
  return BUSSEQ_OK;
}

int busseq_set_state(busseq_handle* h, const busseq_state* in) {
  if (!h || !in) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  bq::DevState& s = h->s;
  const int64_t G = s.G, N = s.N, Gp = s.Gp;
  const int B = s.B, K = s.K;
  auto rows = [&](void* dst, const void* src, size_t esz, int64_t nrows) -> int {
    if (src) CUDA_TRY(cudaMemcpy2D(dst, Gp * esz, src, G * esz, G * esz, nrows, cudaMemcpyHostToDevice));
    return BUSSEQ_OK;
  };
  auto flat = [&](void* dst, const void* src, size_t bytes) -> int {
    if (src) CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return BUSSEQ_OK;
  };
  if (in->W) {
    for (int64_t i = 0; i < N; ++i)
      if (in->W[i] < 0 || in->W[i] >= K) return fail(BUSSEQ_ERR_ARG, "W[%lld] out of range", (long long)i);
  }
  TRY(rows(s.X, in->X, 4, N));
  if (in->Z) {
    std::vector<uint32_t> zm((size_t)N * s.Gw, 0u);
    for (int64_t i = 0; i < N; ++i)
      for (int64_t g = 0; g < G; ++g)
        if (in->Z[i * G + g]) zm[i * s.Gw + (g >> 5)] |= 1u << (g & 31);
    CUDA_TRY(cudaMemcpy(s.zm, zm.data(), zm.size() * 4, cudaMemcpyHostToDevice));
    if (s.nz0 > 0) {
      bq::k_zval_from_mask<<<blocks_for(s.nz0, 256), 256, 0, h->stream>>>(s);
      LAUNCH_CHECK("k_zval_from_mask");
    }
  }
  TRY(flat(s.W, in->W, N * 4));
  TRY(rows(s.L, in->L, 1, K));
  TRY(flat(s.alpha, in->alpha, G * 4));
  TRY(flat(s.mu_alpha, in->mu_alpha, G * 4));
  TRY(rows(s.beta, in->beta, 4, K));
  TRY(rows(s.nu, in->nu, 4, B));
  TRY(flat(s.mu_nu, in->mu_nu, B * 4));
  TRY(flat(s.delta, in->delta, N * 4));
  TRY(flat(s.mu_delta, in->mu_delta, N * 4));
  TRY(rows(s.phi, in->phi, 4, B));
  TRY(flat(s.gamma, in->gamma, 2 * B * 4));
  TRY(flat(s.pi, in->pi, B * K * 4));
  TRY(flat(s.p_tau0, in->p_tau0, 2 * 4));
  const int64_t nfin = std::max<int64_t>(std::max<int64_t>(N, (int64_t)B * Gp), (int64_t)B * K);
  bq::k_init_finish<<<blocks_for(nfin, 256), 256, 0, h->stream>>>(s, 0);
  LAUNCH_CHECK("k_init_finish");
  bq::k_sort_pi<<<B, 1024, 0, h->stream>>>(s, 0, 0);
  LAUNCH_CHECK("k_sort_pi");
  h->est_valid = false;
  return check_device_error(h);
}

int busseq_run_stage(busseq_handle* h, int32_t stage, int32_t iter, int32_t n_unchanged) {
  using namespace bq;
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (iter < 0) return fail(BUSSEQ_ERR_ARG, "iter must be non-negative");
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaMemcpyAsync(h->s.iter, &iter, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  DevState s = h->s;
  s.n_unchanged = n_unchanged;
  cudaStream_t st = h->stream;
  const unsigned pb = blocks_for(propose_count(s), 256);
  auto run = [&](std::initializer_list<int> ks) -> int {
    for (int k : ks) TRY(launch_kernel(h, k, st, 0, s));
    return BUSSEQ_OK;
  };
  switch (stage) {
    case BUSSEQ_STAGE_ZX_GAMMA_ALPHA_L:
      k_propose<<<pb, 256, 0, st>>>(s, PROP_GAMMA | PROP_ALPHA, 0);
      LAUNCH_CHECK("k_propose");
      TRY(run({KID_ZX, KID_ZX_GP, KID_DECIDE_GAMMA, 2, 3}));
      break;
    case BUSSEQ_STAGE_BETA_NU:
      k_propose<<<pb, 256, 0, st>>>(s, PROP_BETA | PROP_NU, 0);
      LAUNCH_CHECK("k_propose");
      TRY(run({4, 5, 6}));
      break;
    case BUSSEQ_STAGE_DELTA:
      k_propose<<<pb, 256, 0, st>>>(s, PROP_DELTA, 0);
      LAUNCH_CHECK("k_propose");
      TRY(run({7}));
      break;
    case BUSSEQ_STAGE_PHI:
      k_propose<<<pb, 256, 0, st>>>(s, PROP_PHI, 0);
      LAUNCH_CHECK("k_propose");
      TRY(run({KID_PHI_STATIC, 8, 9}));
      break;
    case BUSSEQ_STAGE_W:
      TRY(run({10}));
      break;
    case BUSSEQ_STAGE_PI:
      k_sort_pi<<<s.B, 1024, 0, st>>>(s, 1, 0);
      LAUNCH_CHECK("k_sort_pi");
      break;
    default:
      return fail(BUSSEQ_ERR_ARG, "unknown stage %d", stage);
  }
  h->est_valid = false;
  return check_device_error(h);
}

// ---------------------------------------------------------------------------
// Checkpoint and resume (no reference equivalent: the reference cannot stop
// and continue a run).  Draws are counter-based, keyed by (seed, sweep index),
// so the chain state, the run's accumulators and the sweep counters are all a
// run needs to continue exactly where it stopped.
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

// Flat padded layout (alpha [Gp] | beta [K][Gp] | nu [B][Gp] | psi [B][Gp] |
// delta [N]) <-> the unpadded one of the ABI (alpha [G] | beta [K*G] |
// nu [B*G] | psi [B*G] | delta [N]).
template <typename S, typename D>
void hmc_unpad(const bq::DevState& s, const S* src, D* dst) {
  const int64_t G = s.G, Gp = s.Gp;
  const int64_t rows = 1 + s.K + 2 * s.B;
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t g = 0; g < G; ++g) dst[r * G + g] = (D)src[r * Gp + g];
  for (int64_t i = 0; i < s.N; ++i) dst[rows * G + i] = (D)src[rows * Gp + i];
}

int need_hmc(busseq_handle* h) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (h->s.hmc_L <= 0) return fail(BUSSEQ_ERR_STATE, "the chain was created without hmc_leapfrog");
  return BUSSEQ_OK;
}

// The change of the block's log posterior from `from` to the current state:
// in total (per_gene 0, out[0]) or per gene (per_gene 1, out[G]; delta is
// held, so the two states must share it).
int logpost_diff(busseq_handle* h, const busseq_state* from, int per_gene, double* out) {
  TRY(need_hmc(h));
  if (!from || !out || !from->alpha || !from->beta || !from->nu || !from->phi || !from->delta)
    return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  const bq::DevState& s = h->s;
  const int64_t G = s.G, Gp = s.Gp, N = s.N;
  const int B = s.B, K = s.K;
  std::vector<float> th((size_t)s.hmc_D, 0.0f);
  for (int64_t g = 0; g < G; ++g) {
    th[g] = from->alpha[g];
    for (int k = 0; k < K; ++k) th[Gp + k * Gp + g] = from->beta[k * G + g];
    for (int b = 0; b < B; ++b) {
      th[Gp * (1 + K) + b * Gp + g] = from->nu[b * G + g];
      th[Gp * (1 + K + B) + b * Gp + g] = logf(from->phi[b * G + g]);
    }
  }
  for (int64_t i = 0; i < N; ++i) th[Gp * (1 + K + 2 * B) + i] = from->delta[i];
  float* d = nullptr;
  double* dg = nullptr;
  CUDA_TRY(cudaMalloc(&d, s.hmc_D * 4));
  if (per_gene && cudaMalloc(&dg, std::max<int64_t>(G, 1) * sizeof(double)) != cudaSuccess) {
    cudaFree(d);
    return fail(BUSSEQ_ERR_NOMEM, "log posterior difference: no device memory");
  }
  cudaError_t e = cudaMemcpyAsync(d, th.data(), s.hmc_D * 4, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) {
    const dim3 gene_grid(s.n_tiles, s.cap_g);
    bq::k_hmc_set_th0<<<blocks_for(s.hmc_D, 256), 256, 0, h->stream>>>(s, d);
    bq::k_hmc_dll_prep<<<blocks_for((int64_t)s.B * s.G, 256), 256, 0, h->stream>>>(s);
    bq::k_hmc_dll_static<<<STATIC_CTAS, 256, 0, h->stream>>>(s, s.n_tiles * s.cap_g, per_gene);
    bq::k_hmc_dll<<<gene_grid, bq::GENE_TILE, 0, h->stream>>>(s, per_gene);
    bq::k_hmc_energy<<<blocks_for(s.hmc_D, 256), 256, 0, h->stream>>>(s, 0, per_gene);
    if (s.hmc_nb > 0) bq::k_hmc_energy_blocks<<<blocks_for(s.G * 32, 256), 256, 0, h->stream>>>(s, 0, per_gene);
    if (per_gene) {
      bq::k_hmc_accept_genes<<<blocks_for(s.G, 256), 256, 0, h->stream>>>(s, dg);
    } else {
      bq::k_hmc_accept<<<1, 256, 0, h->stream>>>(s, s.n_tiles * s.cap_g + STATIC_CTAS,
                                                 (int)blocks_for(s.hmc_D, 256),
                                                 (int)blocks_for(s.G * 32, 256), 1);
    }
    e = cudaGetLastError();
  }
  double sc[bq::HS_COUNT];
  if (e == cudaSuccess && !per_gene) e = cudaMemcpyAsync(sc, s.hmc_sc, sizeof sc, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && per_gene) e = cudaMemcpyAsync(out, dg, G * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  cudaFree(dg);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "log posterior difference: %s", cudaGetErrorString(e));
  if (!per_gene) *out = sc[bq::HS_LAST_DH];
  return check_device_error(h);
}

}  // namespace

extern "C" {

int busseq_hmc_stats(busseq_handle* h, double out[4]) {
  TRY(need_hmc(h));
  if (!out) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  double sc[bq::HS_COUNT];
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  CUDA_TRY(cudaMemcpy(sc, h->s.hmc_sc, sizeof sc, cudaMemcpyDeviceToHost));
  out[0] = sc[bq::HS_EPS];
  out[1] = sc[bq::HS_N_KEPT] > 0 ? sc[bq::HS_ACC_KEPT] / sc[bq::HS_N_KEPT] : 0.0;
  out[2] = sc[bq::HS_LAST_ACC];
  out[3] = sc[bq::HS_LAST_DH];
  return BUSSEQ_OK;
}

int busseq_hmc_gradient(busseq_handle* h, double* grad, double* metric) {
  TRY(need_hmc(h));
  if (!grad) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  const bq::DevState& s = h->s;
  const dim3 gene_grid(s.n_tiles, s.cap_g);
  // the adapted metric of the chain (the mass and its frozen information
  // part) is kept: the call works on copies
  std::vector<float> mass_keep(s.hmc_D), fis_keep(s.hmc_D);
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  CUDA_TRY(cudaMemcpy(mass_keep.data(), s.hmc_mass, s.hmc_D * 4, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(fis_keep.data(), s.hmc_fis, s.hmc_D * 4, cudaMemcpyDeviceToHost));
  bq::k_hmc_grad_metric<<<gene_grid, bq::GENE_TILE, 0, h->stream>>>(s, 2);
  LAUNCH_CHECK("k_hmc_grad");
  bq::k_hmc_assemble<<<blocks_for(s.hmc_D, 256), 256, 0, h->stream>>>(s, 2);
  LAUNCH_CHECK("k_hmc_assemble");
  TRY(check_device_error(h));
  std::vector<float> gf(s.hmc_D), mf(s.hmc_D);
  CUDA_TRY(cudaMemcpy(gf.data(), s.hmc_grad, s.hmc_D * 4, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(mf.data(), s.hmc_mass, s.hmc_D * 4, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(s.hmc_mass, mass_keep.data(), s.hmc_D * 4, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(s.hmc_fis, fis_keep.data(), s.hmc_D * 4, cudaMemcpyHostToDevice));
  hmc_unpad(s, gf.data(), grad);
  if (metric) hmc_unpad(s, mf.data(), metric);
  return BUSSEQ_OK;
}

int busseq_hmc_logpost_diff(busseq_handle* h, const busseq_state* from, double* out) {
  return logpost_diff(h, from, 0, out);
}

int busseq_hmc_gene_logpost_diff(busseq_handle* h, const busseq_state* from, double* out) {
  TRY(need_hmc(h));
  if (!h->s.hmc_gene) return fail(BUSSEQ_ERR_STATE, "the chain was created without hmc_gene_accept");
  return logpost_diff(h, from, 1, out);
}

int busseq_get_progress(busseq_handle* h, int32_t* n_done, int32_t* n_iter, int32_t* n_burnin) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (n_done) *n_done = h->begun ? h->iter_host : 0;
  if (n_iter) *n_iter = h->begun ? h->n_iter : 0;
  if (n_burnin) *n_burnin = h->begun ? h->n_burnin : 0;
  return BUSSEQ_OK;
}

int busseq_get_log_ratios(busseq_handle* h, busseq_log_ratios* o) {
  if (!h || !o) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const bq::DevState& s = h->s;
  auto cp = [&](double* dst, const double* src, int64_t n) -> int {
    if (dst) CUDA_TRY(cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost));
    return BUSSEQ_OK;
  };
  TRY(cp(o->gamma, s.lr_gamma, 2 * s.B));
  TRY(cp(o->alpha, s.lr_alpha, s.G));
  TRY(cp(o->beta, s.lr_beta, (int64_t)s.K * s.G));
  TRY(cp(o->nu, s.lr_nu, (int64_t)s.B * s.G));
  TRY(cp(o->delta, s.lr_delta, s.N));
  TRY(cp(o->phi, s.lr_phi, (int64_t)s.B * s.G));
  TRY(cp(o->W, s.lr_W, s.N));
  return BUSSEQ_OK;
}

int busseq_set_stream(busseq_handle* h, void* cuda_stream) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
  return BUSSEQ_OK;
}

const char* busseq_kernel_name(int32_t i) { return (i >= 0 && i < kNumKernels) ? kKernelNames[i] : ""; }

int busseq_profile(busseq_handle* h, int32_t n_sweeps, double* ms_avg, int32_t cap, int32_t* n_out) {
  if (!h) return fail(BUSSEQ_ERR_ARG, "NULL handle");
  if (n_sweeps <= 0) return fail(BUSSEQ_ERR_ARG, "n_sweeps must be positive");
  CUDA_TRY(cudaSetDevice(h->device));
  // burn-in sweeps (every kernel but the posterior accumulation); time per
  // kernel id, summed over its launches in a sweep
  const std::vector<int> seq = sweep_sequence(h, 0);
  const size_t nl = seq.size();
  std::vector<cudaEvent_t> ev(nl * 2 * n_sweeps);
  for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
  int r = BUSSEQ_OK;
  for (int sw = 0; sw < n_sweeps && r == BUSSEQ_OK; ++sw)
    for (size_t k = 0; k < nl && r == BUSSEQ_OK; ++k) {
      cudaEventRecord(ev[((size_t)sw * nl + k) * 2], h->stream);
      r = launch_kernel(h, seq[k], h->stream, 0, h->s);
      cudaEventRecord(ev[((size_t)sw * nl + k) * 2 + 1], h->stream);
    }
  if (r == BUSSEQ_OK) r = check_device_error(h);
  std::vector<double> tot(kNumKernels, 0.0);
  if (r == BUSSEQ_OK)
    for (int sw = 0; sw < n_sweeps; ++sw)
      for (size_t k = 0; k < nl; ++k) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev[((size_t)sw * nl + k) * 2], ev[((size_t)sw * nl + k) * 2 + 1]);
        tot[seq[k]] += ms;
      }
  for (auto& e : ev) cudaEventDestroy(e);
  if (r != BUSSEQ_OK) return r;
  for (int k = 0; k < kNumKernels && k < cap; ++k) ms_avg[k] = tot[k] / n_sweeps;
  if (n_out) *n_out = std::min<int>(kNumKernels, cap);
  h->est_valid = false;
  return BUSSEQ_OK;
}

double busseq_kernel_bytes(busseq_handle* h, int32_t i) {
  if (!h) return 0.0;
  const bq::DevState& s = h->s;
  const double E = (double)s.N * (double)s.G;
  const double params = 8.0 * ((double)s.K * s.G + 2.0 * s.B * s.G + s.N);
  const double part = 8.0 * (double)s.cap_g * s.Gp;  // one slot of the per-chunk partials
  switch (i) {
    case 0: return params;                          // proposals
    case 1: return 17.0 * (double)s.nz0;            // per zero entry: {cell, gene}, X in + out, Z out
    case 2: return 4.0 * E;                         // read X
    case 3: return 2.0 * part + params;             // alpha partials
    case 4: return 4.0 * E;
    case 5: return 2.0 * part + params;
    case 6: return 2.0 * part + 4.0 * s.B * s.K * s.G;  // nu partials, E table out
    case 7: return 4.0 * E;
    case 8: return 4.0 * E;
    case 9: return part + params;
    case 10: return 4.0 * E;
    case 11: return 8.0 * s.N;                      // W in, cell order out
    case 12: return params;
    case 13: return 4.0 * E;                        // HMC gradient pass: read X
    case 19: return 4.0 * E;                        // HMC log-likelihood change: read X
    case 29: return 4.0 * E;                        // HMC gradient at the start of a transition
    default: return 0.0;
  }
}

int busseq_launches_per_sweep(busseq_handle* h, int32_t kept) {
  if (!h) return 0;
  int n = 0;
  for (int k : sweep_sequence(h, kept)) n += k == KID_HMC_DLL_STATIC ? 2 : 1;  // prep + static
  return n;
}


}  // extern "C"

