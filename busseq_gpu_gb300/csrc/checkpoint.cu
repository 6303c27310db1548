// Checkpoint and resume of a chain (not in the reference): the state, the run's
// accumulators and kept draws, the sweep counters and a fingerprint of Y, so
// that a resumed run makes exactly the draws of the uninterrupted one.
#include "capi_internal.h"
#include "kernels.h"

#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

using namespace bqc;

namespace {

struct CkHeader {
  char magic[8];
  uint32_t version;
  int32_t B, K;
  int32_t w_update, keep_draws;
  int32_t begun, finished, n_iter, n_burnin, n_unchanged, iter_host, iter_dev;
  int64_t G, N, nz0;
  uint64_t seed, y_fingerprint;
  int32_t hmc_leapfrog, zx_summaries, hmc_gene_accept, pad;
};
constexpr char kCkMagic[8] = {'B', 'U', 'S', 'S', 'E', 'Q', 'C', 'K'};
constexpr uint32_t kCkVersion = 3;

struct DevBlock {
  void* p;
  size_t bytes;
};

// The run's accumulators and kept draws, in file order (sizes as allocated by
// busseq_begin).
std::vector<DevBlock> run_blocks(const busseq_handle* h) {
  const bq::DevState& s = h->s;
  const size_t G = (size_t)s.G, N = (size_t)s.N, nk = (size_t)h->n_kept;
  const size_t B = (size_t)s.B, K = (size_t)s.K;  // B >= 2, K >= 1
  std::vector<DevBlock> v = {
      {s.acc_alpha, G * 8},     {s.acc_beta, K * G * 8},  {s.acc_L, K * G * 8},   {s.acc_nu, B * G * 8},
      {s.acc_delta, N * 8},     {s.acc_phi, B * G * 8},   {s.acc_gamma, 2 * B * 8}, {s.acc_pi, B * K * 8},
      {s.acc_ptau, 2 * 8},      {s.acc_wcnt, N * K * 4}};
  if (s.keep_draws) {
    const size_t km = K > 1 ? K - 1 : 1;
    const std::vector<DevBlock> k = {
        {s.keep_gamma, nk * 2 * B * 4}, {s.keep_alpha, nk * G * 4},      {s.keep_beta, nk * km * G * 4},
        {s.keep_L, nk * km * G},        {s.keep_ptau, nk * 2 * 4},       {s.keep_nu, nk * (B - 1) * G * 4},
        {s.keep_delta, nk * N * 4},     {s.keep_phi, nk * B * G * 4},    {s.keep_W, nk * N * 2},
        {s.keep_pi, nk * B * K * 4}};
    v.insert(v.end(), k.begin(), k.end());
  }
  if (s.acc_zn) {
    v.push_back({s.acc_zn, (size_t)std::max<int64_t>(1, s.nz0) * 4});
    v.push_back({s.acc_xs, (size_t)std::max<int64_t>(1, s.nz0) * 8});
  }
  if (s.hmc_L > 0) {  // log phi as the chain holds it, the adapted metric and the step size
    v.push_back({s.psi, (size_t)s.B * s.Gp * 4});
    v.push_back({s.hmc_mass, (size_t)s.hmc_D * 4});
    v.push_back({s.hmc_sc, (size_t)bq::HS_COUNT * 8});
    v.push_back({s.hmc_fis, (size_t)s.hmc_D * 4});
    if (s.hmc_nb > 0) {
      v.push_back({s.hmc_chol, (size_t)bq::HMC_BLOCK_MAX * (bq::HMC_BLOCK_MAX + 1) / 2 * s.G * 4});
      v.push_back({s.hmc_wbk, (size_t)s.B * s.K * s.G * 4});
      v.push_back({s.hmc_minv, (size_t)bq::HMC_BLOCK_MAX * bq::HMC_BLOCK_MAX * s.G * 4});
    }
  }
  return v;
}

int y_fingerprint(busseq_handle* h, uint64_t* out) {
  unsigned long long* d = nullptr;
  CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned long long), h->stream);
  if (e == cudaSuccess) {
    bq::k_y_fingerprint<<<152 * 8, 256, 0, h->stream>>>(h->s, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "Y fingerprint: %s", cudaGetErrorString(e));
  return BUSSEQ_OK;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

int write_block(FILE* f, const void* host, uint64_t bytes, const char* path) {
  if (fwrite(&bytes, 8, 1, f) != 1 || (bytes && fwrite(host, 1, bytes, f) != bytes))
    return fail(BUSSEQ_ERR_IO, "cannot write %s", path);
  return BUSSEQ_OK;
}

int read_block(FILE* f, void* host, uint64_t bytes, const char* path, const char* what) {
  uint64_t n = 0;
  if (fread(&n, 8, 1, f) != 1) return fail(BUSSEQ_ERR_IO, "%s: truncated before %s", path, what);
  if (n != bytes) return fail(BUSSEQ_ERR_IO, "%s: %s holds %llu bytes, expected %llu", path, what,
                              (unsigned long long)n, (unsigned long long)bytes);
  if (bytes && fread(host, 1, bytes, f) != bytes) return fail(BUSSEQ_ERR_IO, "%s: truncated in %s", path, what);
  return BUSSEQ_OK;
}

}  // namespace

extern "C" {

int busseq_checkpoint_save(busseq_handle* h, const char* path) {
  if (!h || !path) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  TRY(check_device_error(h));
  const bq::DevState& s = h->s;
  const int64_t G = s.G, N = s.N;
  const int B = s.B, K = s.K;
  CkHeader hd{};
  memcpy(hd.magic, kCkMagic, 8);
  hd.version = kCkVersion;
  hd.B = B;
  hd.K = K;
  hd.G = G;
  hd.N = N;
  hd.nz0 = s.nz0;
  hd.seed = h->opt.seed;
  hd.w_update = h->opt.w_update;
  hd.keep_draws = h->opt.keep_draws;
  hd.hmc_leapfrog = h->s.hmc_L;
  hd.zx_summaries = h->opt.zx_summaries ? 1 : 0;
  hd.hmc_gene_accept = h->s.hmc_gene;
  hd.begun = h->begun ? 1 : 0;
  hd.finished = h->finished ? 1 : 0;
  hd.n_iter = h->n_iter;
  hd.n_burnin = h->n_burnin;
  hd.n_unchanged = h->n_unchanged;
  hd.iter_host = h->iter_host;
  CUDA_TRY(cudaMemcpy(&hd.iter_dev, s.iter, sizeof(int), cudaMemcpyDeviceToHost));
  TRY(y_fingerprint(h, &hd.y_fingerprint));

  // chain state: parameters through busseq_get_state, X and Z at the Y == 0 entries
  std::vector<int32_t> W(N), zx(std::max<int64_t>(s.nz0, 1));
  std::vector<int8_t> L((size_t)K * G);
  std::vector<float> alpha(G), mu_alpha(G), beta((size_t)K * G), nu((size_t)B * G), mu_nu(B), delta(N),
      mu_delta(N), phi((size_t)B * G), gamma(2 * B), pi((size_t)B * K), ptau(2);
  std::vector<uint8_t> zval(std::max<int64_t>(s.nz0, 1));
  busseq_state st{};
  st.W = W.data();
  st.L = L.data();
  st.alpha = alpha.data();
  st.mu_alpha = mu_alpha.data();
  st.beta = beta.data();
  st.nu = nu.data();
  st.mu_nu = mu_nu.data();
  st.delta = delta.data();
  st.mu_delta = mu_delta.data();
  st.phi = phi.data();
  st.gamma = gamma.data();
  st.pi = pi.data();
  st.p_tau0 = ptau.data();
  TRY(busseq_get_state(h, &st));
  if (s.nz0 > 0) {
    int32_t* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, s.nz0 * 4));
    bq::k_zlist_gather_x<<<blocks_for(s.nz0, 256), 256, 0, h->stream>>>(s, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(zx.data(), d, s.nz0 * 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(zval.data(), s.zval, s.nz0, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "checkpoint gather: %s", cudaGetErrorString(e));
  }

  File out;
  const std::string tmp = std::string(path) + ".tmp";
  out.f = fopen(tmp.c_str(), "wb");
  if (!out.f) return fail(BUSSEQ_ERR_IO, "cannot open %s for writing", tmp.c_str());
  if (fwrite(&hd, sizeof hd, 1, out.f) != 1) return fail(BUSSEQ_ERR_IO, "cannot write %s", tmp.c_str());
  TRY(write_block(out.f, h->n_b.data(), 4ull * B, path));
  TRY(write_block(out.f, zx.data(), 4ull * s.nz0, path));
  TRY(write_block(out.f, zval.data(), (uint64_t)s.nz0, path));
  TRY(write_block(out.f, W.data(), 4ull * N, path));
  TRY(write_block(out.f, L.data(), (uint64_t)K * G, path));
  for (const std::vector<float>* v : {&alpha, &mu_alpha, &beta, &nu, &mu_nu, &delta, &mu_delta, &phi, &gamma, &pi,
                                      &ptau})
    TRY(write_block(out.f, v->data(), 4ull * v->size(), path));
  if (h->begun) {
    for (const DevBlock& blk : run_blocks(h)) {
      std::vector<uint8_t> buf(blk.bytes);
      CUDA_TRY(cudaMemcpy(buf.data(), blk.p, blk.bytes, cudaMemcpyDeviceToHost));
      TRY(write_block(out.f, buf.data(), blk.bytes, path));
    }
  }
  if (fclose(out.f) != 0) {
    out.f = nullptr;
    return fail(BUSSEQ_ERR_IO, "cannot write %s", tmp.c_str());
  }
  out.f = nullptr;
  if (rename(tmp.c_str(), path) != 0) return fail(BUSSEQ_ERR_IO, "cannot rename %s to %s", tmp.c_str(), path);
  return BUSSEQ_OK;
}

int busseq_checkpoint_load(busseq_handle* h, const char* path) {
  if (!h || !path) return fail(BUSSEQ_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  bq::DevState& s = h->s;
  const int64_t G = s.G, N = s.N;
  const int B = s.B, K = s.K;
  File in;
  in.f = fopen(path, "rb");
  if (!in.f) return fail(BUSSEQ_ERR_IO, "cannot open %s", path);
  CkHeader hd{};
  if (fread(&hd, sizeof hd, 1, in.f) != 1) return fail(BUSSEQ_ERR_IO, "%s: truncated header", path);
  if (memcmp(hd.magic, kCkMagic, 8) != 0 || hd.version != kCkVersion)
    return fail(BUSSEQ_ERR_IO, "%s is not a busseq checkpoint (version %u)", path, kCkVersion);
  if (hd.B != B || hd.K != K || hd.G != G || hd.N != N || hd.nz0 != s.nz0)
    return fail(BUSSEQ_ERR_ARG, "%s was written for B=%d K=%d G=%lld N=%lld, this chain has B=%d K=%d G=%lld N=%lld",
                path, hd.B, hd.K, (long long)hd.G, (long long)hd.N, B, K, (long long)G, (long long)N);
  if (hd.seed != h->opt.seed || hd.w_update != h->opt.w_update || hd.keep_draws != h->opt.keep_draws ||
      hd.hmc_leapfrog != h->s.hmc_L || hd.zx_summaries != (h->opt.zx_summaries ? 1 : 0) ||
      hd.hmc_gene_accept != h->s.hmc_gene)
    return fail(BUSSEQ_ERR_ARG, "%s was written with another seed, W move, keep_draws, HMC or zx_summaries setting",
                path);
  uint64_t fp = 0;
  TRY(y_fingerprint(h, &fp));
  if (fp != hd.y_fingerprint) return fail(BUSSEQ_ERR_ARG, "%s was written for different counts", path);
  std::vector<int32_t> nb(B), W(N), zx(std::max<int64_t>(s.nz0, 1));
  TRY(read_block(in.f, nb.data(), 4ull * B, path, "n_b"));
  if (nb != h->n_b) return fail(BUSSEQ_ERR_ARG, "%s was written for other batch sizes", path);
  std::vector<uint8_t> zval(std::max<int64_t>(s.nz0, 1));
  std::vector<int8_t> L((size_t)K * G);
  std::vector<float> alpha(G), mu_alpha(G), beta((size_t)K * G), nu((size_t)B * G), mu_nu(B), delta(N),
      mu_delta(N), phi((size_t)B * G), gamma(2 * B), pi((size_t)B * K), ptau(2);
  TRY(read_block(in.f, zx.data(), 4ull * s.nz0, path, "X"));
  TRY(read_block(in.f, zval.data(), (uint64_t)s.nz0, path, "Z"));
  TRY(read_block(in.f, W.data(), 4ull * N, path, "W"));
  TRY(read_block(in.f, L.data(), (uint64_t)K * G, path, "L"));
  const char* names[] = {"alpha", "mu_alpha", "beta", "nu", "mu_nu", "delta", "mu_delta", "phi", "gamma", "pi",
                         "p_tau0"};
  int ni = 0;
  for (std::vector<float>* v : {&alpha, &mu_alpha, &beta, &nu, &mu_nu, &delta, &mu_delta, &phi, &gamma, &pi, &ptau})
    TRY(read_block(in.f, v->data(), 4ull * v->size(), path, names[ni++]));
  for (int64_t j = 0; j < s.nz0; ++j)
    if (zx[j] < 0 || zval[j] > 1) return fail(BUSSEQ_ERR_IO, "%s: invalid X or Z value at entry %lld", path, (long long)j);

  // the state first (busseq_set_state recomputes the derived arrays), then
  // the run (busseq_begin resets its counters; the saved ones replace them)
  busseq_state st{};
  st.W = W.data();
  st.L = L.data();
  st.alpha = alpha.data();
  st.mu_alpha = mu_alpha.data();
  st.beta = beta.data();
  st.nu = nu.data();
  st.mu_nu = mu_nu.data();
  st.delta = delta.data();
  st.mu_delta = mu_delta.data();
  st.phi = phi.data();
  st.gamma = gamma.data();
  st.pi = pi.data();
  st.p_tau0 = ptau.data();
  TRY(busseq_set_state(h, &st));
  if (s.nz0 > 0) {
    int32_t* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, s.nz0 * 4));
    cudaError_t e = cudaMemcpyAsync(d, zx.data(), s.nz0 * 4, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
      bq::k_zlist_scatter_x<<<blocks_for(s.nz0, 256), 256, 0, h->stream>>>(s, d);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.zval, zval.data(), s.nz0, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(BUSSEQ_ERR_CUDA, "checkpoint scatter: %s", cudaGetErrorString(e));
  }
  if (hd.begun) {
    if (hd.iter_host < 0 || hd.iter_host > hd.n_iter || hd.iter_dev != hd.iter_host)
      return fail(BUSSEQ_ERR_IO, "%s: inconsistent sweep counters", path);
    TRY(busseq_begin(h, hd.n_iter, hd.n_burnin, hd.n_unchanged));
    for (const DevBlock& blk : run_blocks(h)) {
      std::vector<uint8_t> buf(blk.bytes);
      TRY(read_block(in.f, buf.data(), blk.bytes, path, "run accumulators"));
      CUDA_TRY(cudaMemcpy(blk.p, buf.data(), blk.bytes, cudaMemcpyHostToDevice));
    }
    CUDA_TRY(cudaMemcpy(s.iter, &hd.iter_dev, sizeof(int), cudaMemcpyHostToDevice));
    h->iter_host = hd.iter_host;
  }
  h->est_valid = false;
  if (hd.begun && hd.finished) TRY(busseq_finish(h));
  return check_device_error(h);
}

// ---- gradient-based block update: statistics and test entry points --------
}  // extern "C"
