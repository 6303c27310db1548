// ===========================================================================
// Reference chain runner -- TEST INFRASTRUCTURE ONLY.
//
// Runs a whole BUSseq chain with the reference implementation's own kernels,
// so that a chain of this project's sampler can be compared with it on the
// same data (posterior means, ARI of the cell types).  It loads
// oracle/_ref/busseq_ref.cubin (the reference's device code, compiled by
// oracle/build.py from BUSseq_gpu.cu where it lies; nothing of it is copied
// here) and replays, through the CUDA driver API, the launch sequence of the
// reference's host program:
//   initialisation  BUSseq_gpu.cu:1163-1244 (curand states, p0 from
//                   srand(seed)/rand(), library sizes, first_* kernels, raw
//                   means, mu_nu into the __constant__ d_mu_nu, mu_delta)
//   burn-in sweeps  BUSseq_gpu.cu:1267-1398, p and tau0 from iter >= -u
//   kept sweeps     BUSseq_gpu.cu:1413-1555, with the store_* kernels and the
//                   device copies of p and tau0 (:1546-1554)
// with the same kernels, grids, block sizes, dynamic shared memory and
// arguments.  Two deliberate differences, neither of which touches a
// reference kernel's arithmetic:
//   * pi (update_pi, :866-890) is NOT launched: its __syncthreads (:887) sits
//     inside `if (tid < K)` of a 1024-thread block (a divergent barrier), and
//     thread 0 sums d_pi without waiting for the other threads' draws.  The
//     per-(batch, type) counts are computed by the reference's own fill_I_W /
//     sum_on_gpu launches (stored per batch instead of overwriting one row),
//     read back, and pi_b ~ Dirichlet(count + xi_pi) is drawn on the host
//     (std::gamma_distribution, seeded from the chain's seed).
//   * every sweep's launches (up to the pi counts) are captured once into a
//     CUDA graph (one with the p / tau0 block, one without) and replayed; the
//     kernels and their order are unchanged.
// Between sweeps the host checks that every parameter is finite and that no
// mean exp(alpha + beta + nu + delta) can overflow, and stops the chain with
// an error instead of launching the reference's unbounded rejection loops on
// such a state.
//
// The posterior means are not computed here: the kept draws, in the
// reference's [scalar][kept sweep] layout, are written to <out_dir> as raw
// little-endian files (preserved_<name>.bin) and summarised by
// oracle/ref_chain.py.  The state right after initialisation is written too
// (init_<name>.bin), so that the other chain can start from it.  With
// REF_CHAIN_INIT_ONLY set the program stops after writing it; with
// REF_CHAIN_START_DIR=<dir> the chain starts instead from the state in <dir>
// (start_<name>.bin), keeping the priors of its own initialisation.
//
// usage: ref_chain <cubin> <Y.i32> <G> <K> <seed> <n_iter> <n_burnin>
//                  <n_unchanged> <out_dir> <n_1> ... <n_B>
// Prints one JSON line (p0, timings, launches).
// ===========================================================================
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <random>
#include <string>
#include <vector>

namespace {

void die(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  fprintf(stderr, "ref_chain: %s failed: %s\n", what, s ? s : "?");
  exit(2);
}
#define CK(x)                            \
  do {                                   \
    CUresult r_ = (x);                   \
    if (r_ != CUDA_SUCCESS) die(#x, r_); \
  } while (0)

CUmodule g_mod;
CUstream g_stream;
long long g_launches = 0;

CUfunction fn(const char* mangled) {
  CUfunction f;
  CK(cuModuleGetFunction(&f, g_mod, mangled));
  return f;
}

template <typename... A>
void go(CUfunction f, unsigned grid, unsigned block, unsigned smem, A... a) {
  void* args[] = {(void*)&a...};
  CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, g_stream, args, nullptr));
  ++g_launches;
}

// Every buffer gets 4 KB of zeroed slack past its end: a categorical search
// that meets a rounding-short sum may read one element past its row.
CUdeviceptr dalloc(size_t bytes) {
  CUdeviceptr p;
  CK(cuMemAlloc(&p, bytes + 4096));
  CK(cuMemsetD8(p, 0, bytes + 4096));
  return p;
}

template <typename T>
std::vector<T> down(CUdeviceptr p, size_t n) {
  std::vector<T> v(n);
  if (n) CK(cuMemcpyDtoH(v.data(), p, n * sizeof(T)));
  return v;
}

bool write_file(const std::string& path, const void* data, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = fwrite(data, 1, bytes, f) == bytes;
  return fclose(f) == 0 && ok;
}

// hyper-parameters of the reference (BUSseq_gpu.cu:12-32) that the host side uses
constexpr double XI_PI = 2.0;
constexpr double TAU0_INIT = 0.005;
constexpr double TAU1 = 100.0;
constexpr double P_INIT_BOUND = 0.5;

}  // namespace

int main(int argc, char** argv) {
  if (argc < 12) {
    fprintf(stderr,
            "usage: ref_chain <cubin> <Y.i32> <G> <K> <seed> <n_iter> <n_burnin> <n_unchanged> <out_dir> "
            "<n_1> ... <n_B>\n");
    return 1;
  }
  const int G = atoi(argv[3]), K = atoi(argv[4]), seed = atoi(argv[5]);
  const int n_iter = atoi(argv[6]), n_burnin = atoi(argv[7]), n_unchanged = atoi(argv[8]);
  const std::string out_dir = argv[9];
  const int B = argc - 10;
  std::vector<int> n_b(B);
  long long Nll = 0;
  for (int b = 0; b < B; ++b) {
    n_b[b] = atoi(argv[10 + b]);
    Nll += n_b[b];
  }
  const int n_pres = n_iter - n_burnin;
  if (B < 2 || B > 128 || K < 2 || G < 1 || n_iter < 1 || n_burnin < 0 || n_pres < 1 || Nll * G >= (1ll << 31)) {
    fprintf(stderr, "ref_chain: bad dimensions or run lengths\n");
    return 1;
  }
  for (int b = 0; b < B; ++b)
    if (n_b[b] < K) {
      fprintf(stderr, "ref_chain: every batch needs at least K cells\n");
      return 1;
    }
  const int N = (int)Nll;
  const long long NG = (long long)N * G;
  std::vector<int32_t> Y((size_t)NG);
  {
    FILE* f = fopen(argv[2], "rb");
    if (!f || fread(Y.data(), 4, Y.size(), f) != Y.size()) {
      fprintf(stderr, "ref_chain: cannot read %zu counts from %s\n", Y.size(), argv[2]);
      return 1;
    }
    fclose(f);
  }

  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxSetCurrent(ctx));
  CK(cuModuleLoad(&g_mod, argv[1]));
  CK(cuStreamCreate(&g_stream, CU_STREAM_NON_BLOCKING));
  CUdeviceptr sym_n_b, sym_mu_nu;
  {
    size_t sz;
    CK(cuModuleGetGlobal(&sym_n_b, &sz, g_mod, "d_n_b"));
    CK(cuMemcpyHtoD(sym_n_b, n_b.data(), 4 * B));  // :1139
    CK(cuModuleGetGlobal(&sym_mu_nu, &sz, g_mod, "d_mu_nu"));
  }

  // ---- kernels (reference file:line) ---------------------------------------
  CUfunction k_init_rand = fn("_Z17initialize_curandiP17curandStateXORWOWi");                   // :220
  CUfunction k_sum_d = fn("_Z10sum_on_gpuIdEvPT_S1_i");                                          // :236
  CUfunction k_sum_i = fn("_Z10sum_on_gpuIiEvPT_S1_i");                                          // :236
  CUfunction k_sel_mean = fn("_Z21selective_mean_on_gpuPdS_Pii");                                // :267
  CUfunction k_mean_d = fn("_Z11mean_on_gpuPdS_i");                                              // :300
  CUfunction k_raw_means = fn("_Z14fill_raw_meansPiPdS_S0_S_iiii");                              // :369
  CUfunction k_first_gamma = fn("_Z11first_gammaPdi");                                           // :384
  CUfunction k_first_pi = fn("_Z8first_piPdii");                                                 // :392
  CUfunction k_first_nu_phi = fn("_Z12first_nu_phiPdS_S_iii");                                   // :399
  CUfunction k_first_delta_W = fn("_Z13first_delta_WP17curandStateXORWOWPdPiS1_S2_ii");          // :419
  CUfunction k_first_beta_L = fn("_Z12first_beta_LP17curandStateXORWOWPddS1_Piii");              // :445
  CUfunction k_first_Z = fn("_Z7first_ZPii");                                                    // :464
  CUfunction k_fill_mu_nu = fn("_Z10fill_mu_nuPiPdS0_ii");                                       // :470
  CUfunction k_first_mu_nu = fn("_Z11first_mu_nuPdi");                                           // :478
  CUfunction k_zx = fn("_Z10update_Z_XP17curandStateXORWOWPiS1_PdS2_S2_S2_S2_S2_S1_S1_iii");     // :484
  CUfunction k_prop_gamma = fn("_Z13propose_gammaP17curandStateXORWOWPdS1_i");                   // :514
  CUfunction k_fill_g0 = fn("_Z16fill_prop_gamma0PdS_PiS0_S_iii");                               // :524
  CUfunction k_fill_g1 = fn("_Z16fill_prop_gamma1PdS_PiS0_S_iii");                               // :551
  CUfunction k_upd_g0 = fn("_Z13update_gamma0P17curandStateXORWOWPdS1_S1_i");                    // :578
  CUfunction k_upd_g1 = fn("_Z13update_gamma1P17curandStateXORWOWPdS1_S1_i");                    // :588
  CUfunction k_prop_alpha = fn("_Z13propose_alphaP17curandStateXORWOWPdS1_i");                   // :602
  CUfunction k_fill_alpha = fn("_Z15fill_prop_alphaPdS_S_S_S_S_PiS0_S_iiii");                    // :608
  CUfunction k_upd_alpha = fn("_Z12update_alphaP17curandStateXORWOWPdS1_S1_S1_i");               // :625
  CUfunction k_upd_L = fn("_Z8update_LP17curandStateXORWOWPdS1_Pii");                            // :634
  CUfunction k_upd_p = fn("_Z8update_pP17curandStateXORWOWPiPdii");                              // :650
  CUfunction k_fill_Lb = fn("_Z16fill_I_L_beta_sqPiPdS0_i");                                     // :654
  CUfunction k_upd_tau0 = fn("_Z11update_tau0P17curandStateXORWOWPiPdii");                       // :664
  CUfunction k_prop_beta = fn("_Z12propose_betaP17curandStateXORWOWPdS1_i");                     // :670
  CUfunction k_fill_beta = fn("_Z14fill_prop_betaPdS_S_S_S_S_PiS0_S_iiii");                      // :676
  CUfunction k_upd_beta = fn("_Z11update_betaP17curandStateXORWOWPdS1_PiS1_S1_i");               // :696
  CUfunction k_prop_nu = fn("_Z10propose_nuP17curandStateXORWOWPdS1_i");                         // :709
  CUfunction k_fill_nu = fn("_Z12fill_prop_nuPdS_S_S_S_S_PiS0_S_iiii");                          // :715
  CUfunction k_upd_nu = fn("_Z9update_nuP17curandStateXORWOWPdS1_S1_ii");                        // :730
  CUfunction k_prop_delta = fn("_Z13propose_deltaP17curandStateXORWOWPdS1_i");                   // :739
  CUfunction k_fill_delta = fn("_Z15fill_prop_deltaPdS_S_S_S_S_PiS0_S_ii");                      // :746
  CUfunction k_upd_delta = fn("_Z12update_deltaP17curandStateXORWOWPdS1_S1_S1_i");               // :763
  CUfunction k_prop_phi = fn("_Z11propose_phiP17curandStateXORWOWPdS1_i");                       // :780
  CUfunction k_fill_phi = fn("_Z13fill_prop_phiPdS_S_S_S_S_PiS0_S_ii");                          // :789
  CUfunction k_upd_phi = fn("_Z10update_phiP17curandStateXORWOWPdS1_S1_i");                      // :806
  CUfunction k_prop_W = fn("_Z9propose_WP17curandStateXORWOWPiii");                              // :820
  CUfunction k_fill_W = fn("_Z11fill_prop_WPiS_PdS0_S0_S0_S0_S_S0_ii");                          // :831
  CUfunction k_upd_W = fn("_Z8update_WP17curandStateXORWOWPiPdS2_S1_ii");                        // :846
  CUfunction k_fill_IW = fn("_Z8fill_I_WPiS_ii");                                                // :856
  CUfunction k_st_gamma = fn("_Z11store_gammaPdS_iii");                                          // :892
  CUfunction k_st_alpha = fn("_Z11store_alphaPdS_iii");                                          // :898
  CUfunction k_st_Lbeta = fn("_Z12store_L_betaPiS_PdS0_iii");                                    // :904
  CUfunction k_st_nuphi = fn("_Z12store_nu_phiPdS_S_S_iiii");                                    // :914
  CUfunction k_st_deltaW = fn("_Z13store_delta_WPdS_PiS0_iii");                                  // :923
  CUfunction k_st_pi = fn("_Z8store_piPdS_iii");                                                 // :932

  const unsigned T = 1024;  // threads_per_block (:1141)
  auto grid = [&](long long n) { return (unsigned)((n - 1) / T + 1); };
  const unsigned S_D = T * sizeof(double), S_I = T * sizeof(int);
  auto I = [](CUdeviceptr base, long long elems) { return base + 4ull * elems; };  // int* + offset
  auto D = [](CUdeviceptr base, long long elems) { return base + 8ull * elems; };  // double* + offset

  // ---- allocations (:1166-1202, :1252-1273, :1401-1411) ---------------------
  CUdeviceptr d_Y = dalloc(4 * NG);
  CK(cuMemcpyHtoD(d_Y, Y.data(), 4 * NG));
  CUdeviceptr d_states = dalloc(48 * NG);  // sizeof(curandStateXORWOW)
  CUdeviceptr d_p = dalloc(16), d_gamma = dalloc(16ull * B), d_pi = dalloc(8ull * B * K);
  CUdeviceptr d_phi = dalloc(8ull * B * G), d_W = dalloc(4ull * N), d_sum_per_cell = dalloc(4ull * N);
  CUdeviceptr d_delta = dalloc(8ull * N), d_alpha = dalloc(8ull * G), d_beta = dalloc(8ull * G * K);
  CUdeviceptr d_L = dalloc(4ull * G * K), d_nu = dalloc(8ull * B * G), d_Z = dalloc(4 * NG), d_X = dalloc(4 * NG);
  CUdeviceptr d_mu_alpha = dalloc(8ull * G), d_mu_delta = dalloc(8ull * N), d_raw_means = dalloc(8ull * B * K * G);
  CUdeviceptr d_temp_int = dalloc(4ull * (N > n_pres ? N : n_pres)), d_temp_double = dalloc(8 * NG);
  CUdeviceptr d_count = dalloc(4ull * K * N), d_mean = dalloc(8ull * B);
  const long long log_rho_len = (long long)(N > G ? N : G) * (B > K ? B : K);
  CUdeviceptr d_log_rho = dalloc(8 * log_rho_len);
  CUdeviceptr d_pgamma = dalloc(16ull * B), d_palpha = dalloc(8ull * G), d_pbeta = dalloc(8ull * G * (K - 1));
  CUdeviceptr d_pnu = dalloc(8ull * G * (B - 1)), d_pdelta = dalloc(8ull * N), d_pphi = dalloc(8ull * B * G);
  CUdeviceptr d_pW = dalloc(4ull * N);
  CUdeviceptr d_pres_gamma = dalloc(16ull * B * n_pres), d_pres_alpha = dalloc(8ull * G * n_pres);
  CUdeviceptr d_pres_L = dalloc(4ull * G * (K - 1) * n_pres), d_pres_p = dalloc(16ull * n_pres);
  CUdeviceptr d_pres_beta = dalloc(8ull * G * (K - 1) * n_pres), d_pres_nu = dalloc(8ull * G * (B - 1) * n_pres);
  CUdeviceptr d_pres_delta = dalloc(8ull * N * n_pres), d_pres_phi = dalloc(8ull * B * G * n_pres);
  CUdeviceptr d_pres_W = dalloc(4ull * N * n_pres), d_pres_pi = dalloc(8ull * B * K * n_pres);

  // ---- initialisation, in the order of :1163-1244 --------------------------
  const auto t_init0 = std::chrono::steady_clock::now();
  go(k_init_rand, grid(NG), T, 0, seed, d_states, (int)NG);
  srand((unsigned)seed);
  const double p0 = ((double)rand() * P_INIT_BOUND) / RAND_MAX;
  {
    const double p[2] = {p0, TAU0_INIT};
    CK(cuMemcpyHtoD(d_p, p, sizeof p));
  }
  for (int i = 0; i < N; ++i) go(k_sum_i, 1u, T, S_I, I(d_Y, (long long)i * G), I(d_sum_per_cell, i), G);
  go(k_first_pi, grid((long long)B * K), T, 0, d_pi, K, B * K);
  go(k_first_delta_W, grid(N), T, 0, d_states, d_pi, d_sum_per_cell, d_delta, d_W, N, K);
  {
    long long si = 0;
    for (int b = 0; b < B; ++b) {
      if (b > 0) si += n_b[b - 1];
      for (int k = 0; k < K; ++k)
        for (int g = 0; g < G; ++g) {
          go(k_raw_means, grid(n_b[b]), T, 0, I(d_Y, si * G), D(d_delta, si), I(d_W, si), d_temp_double, d_temp_int,
             k, g, G, n_b[b]);
          go(k_sum_i, 1u, T, S_I, d_temp_int, d_count, n_b[b]);
          go(k_sel_mean, 1u, T, S_D, d_temp_double, D(d_raw_means, (long long)b * K * G + (long long)k * G + g),
             d_count, n_b[b]);
        }
    }
  }
  const double log_rat_base = log(p0 / (1 - p0)) + (log(TAU0_INIT) - log(TAU1)) / 2;
  go(k_first_gamma, grid(B), T, 0, d_gamma, B);
  go(k_first_nu_phi, grid((long long)B * G), T, 0, d_raw_means, d_nu, d_phi, G, K, B * G);
  go(k_first_beta_L, grid((long long)G * K), T, 0, d_states, d_raw_means, log_rat_base, d_beta, d_L, G, G * K);
  go(k_first_Z, grid(NG), T, 0, d_Z, (int)NG);
  CK(cuMemcpyDtoDAsync(d_alpha, d_raw_means, 8ull * G, g_stream));
  CK(cuMemcpyDtoDAsync(d_X, d_Y, 4 * NG, g_stream));
  CK(cuMemcpyDtoDAsync(d_mu_alpha, d_raw_means, 8ull * G, g_stream));
  {
    long long si = 0;
    for (int b = 0; b < B; ++b) {
      go(k_fill_mu_nu, grid((long long)n_b[b] * G), T, 0, I(d_Y, si * G), D(d_delta, si), d_temp_double, G,
         n_b[b] * G);
      go(k_mean_d, 1u, T, S_D, d_temp_double, D(d_mean, b), n_b[b] * G);
      si += n_b[b];
    }
  }
  go(k_first_mu_nu, 1u, T, 0, d_mean, B - 1);
  CK(cuStreamSynchronize(g_stream));
  {
    std::vector<double> mu_nu = down<double>(D(d_mean, 1), B - 1);
    CK(cuMemcpyHtoD(sym_mu_nu, mu_nu.data(), 8ull * (B - 1)));
  }
  CK(cuMemcpyDtoDAsync(d_mu_delta, d_delta, 8ull * N, g_stream));
  CK(cuStreamSynchronize(g_stream));
  const double init_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_init0).count();

  // The initial state (X = Y and Z = 0 are implied), so that another sampler
  // can start its chain from exactly this state.
  bool wrote = true;
  {
    struct Out { const char* name; CUdeviceptr p; size_t bytes; };
    const Out outs[] = {
        {"W", d_W, 4ull * N}, {"delta", d_delta, 8ull * N}, {"mu_delta", d_mu_delta, 8ull * N},
        {"alpha", d_alpha, 8ull * G}, {"mu_alpha", d_mu_alpha, 8ull * G}, {"beta", d_beta, 8ull * K * G},
        {"L", d_L, 4ull * K * G}, {"nu", d_nu, 8ull * B * G}, {"phi", d_phi, 8ull * B * G},
        {"gamma", d_gamma, 16ull * B}, {"pi", d_pi, 8ull * B * K}, {"p", d_p, 16}, {"mu_nu", D(d_mean, 1), 8ull * (B - 1)},
    };
    for (const Out& o : outs) {
      std::vector<char> h = down<char>(o.p, o.bytes);
      wrote &= write_file(out_dir + "/init_" + o.name + ".bin", h.data(), h.size());
    }
  }

  // Only the initial state wanted (REF_CHAIN_INIT_ONLY): stop here.
  if (getenv("REF_CHAIN_INIT_ONLY")) {
    printf("{\"impl\": \"reference .cu kernels, BUSseq_gpu.cu:1163-1244\", \"init_only\": true, \"p0\": %.17g, "
           "\"init_s\": %.3f, \"files_written\": %s}\n", p0, init_s, wrote ? "true" : "false");
    return wrote ? 0 : 3;
  }
  // A given starting state (REF_CHAIN_START_DIR): after the reference's own
  // initialisation (which fixes the priors mu_alpha, mu_nu and mu_delta), the
  // chain state is replaced by the one in that directory (start_<name>.bin:
  // X, Z [N*G] int32; W [N] int32; L [K*G] int32; alpha [G], beta [K*G],
  // nu [B*G], delta [N], phi [B*G], gamma [2B], pi [B*K], p [2] double).
  if (const char* sd = getenv("REF_CHAIN_START_DIR")) {
    struct In { const char* name; CUdeviceptr p; size_t bytes; };
    const In ins[] = {
        {"X", d_X, 4ull * NG}, {"Z", d_Z, 4ull * NG}, {"W", d_W, 4ull * N}, {"L", d_L, 4ull * K * G},
        {"alpha", d_alpha, 8ull * G}, {"beta", d_beta, 8ull * K * G}, {"nu", d_nu, 8ull * B * G},
        {"delta", d_delta, 8ull * N}, {"phi", d_phi, 8ull * B * G}, {"gamma", d_gamma, 16ull * B},
        {"pi", d_pi, 8ull * B * K}, {"p", d_p, 16},
    };
    for (const In& in : ins) {
      std::vector<char> h(in.bytes);
      const std::string path = std::string(sd) + "/start_" + in.name + ".bin";
      FILE* f = fopen(path.c_str(), "rb");
      if (!f || fread(h.data(), 1, h.size(), f) != h.size()) {
        fprintf(stderr, "ref_chain: cannot read %zu bytes from %s\n", h.size(), path.c_str());
        return 1;
      }
      fclose(f);
      CK(cuMemcpyHtoD(in.p, h.data(), h.size()));
    }
  }

  // ---- one sweep up to the pi counts, in the order of :1267-1398 -----------
  // The pi counts of batch b go to d_count[b*K + k] (the reference reuses
  // d_count[k] for every batch and consumes it in update_pi right away).
  auto sweep_body = [&](bool update_p_tau0) {
    go(k_zx, grid(NG), T, 0, d_states, d_Y, d_W, d_alpha, d_beta, d_nu, d_delta, d_gamma, d_phi, d_Z, d_X, B, N, G);
    go(k_prop_gamma, grid(B), T, 0, d_states, d_pgamma, d_gamma, B);
    long long si = 0;
    for (int b = 0; b < B; ++b) {
      if (b > 0) si += n_b[b - 1];
      go(k_fill_g0, grid((long long)n_b[b] * G), T, 0, d_pgamma, d_gamma, I(d_Z, si * G), I(d_X, si * G),
         d_temp_double, b, B, n_b[b] * G);
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, b), n_b[b] * G);
    }
    go(k_upd_g0, grid(B), T, 0, d_states, d_pgamma, d_log_rho, d_gamma, B);
    si = 0;
    for (int b = 0; b < B; ++b) {
      if (b > 0) si += n_b[b - 1];
      go(k_fill_g1, grid((long long)n_b[b] * G), T, 0, d_pgamma, d_gamma, I(d_Z, si * G), I(d_X, si * G),
         d_temp_double, b, B, n_b[b] * G);
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, b), n_b[b] * G);
    }
    go(k_upd_g1, grid(B), T, 0, d_states, d_pgamma, d_log_rho, d_gamma, B);
    go(k_prop_alpha, grid(G), T, 0, d_states, d_palpha, d_alpha, G);
    for (int g = 0; g < G; ++g) {
      go(k_fill_alpha, grid(N), T, 0, d_palpha, d_alpha, d_beta, d_nu, d_delta, d_phi, d_W, d_X, d_temp_double, g, B, N,
         G);
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, g), N);
    }
    go(k_upd_alpha, grid(G), T, 0, d_states, d_palpha, d_log_rho, d_mu_alpha, d_alpha, G);
    go(k_upd_L, grid((long long)G * (K - 1)), T, 0, d_states, d_p, D(d_beta, G), I(d_L, G), G * (K - 1));
    if (update_p_tau0) {
      go(k_sum_i, 1u, T, S_I, I(d_L, G), d_count, G * (K - 1));
      go(k_fill_Lb, grid((long long)G * (K - 1)), T, 0, I(d_L, G), D(d_beta, G), d_temp_double, G * (K - 1));
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_p, 1), G * (K - 1));
      go(k_upd_p, 1u, 1u, 0, d_states, d_count, d_p, G, K);
      go(k_upd_tau0, 1u, 1u, 0, d_states, d_count, d_p, G, K);
    }
    go(k_prop_beta, grid((long long)G * (K - 1)), T, 0, d_states, d_pbeta, D(d_beta, G), G * (K - 1));
    for (int k = 1; k < K; ++k)
      for (int g = 0; g < G; ++g) {
        go(k_fill_beta, grid(N), T, 0, d_pbeta, d_beta, d_alpha, d_nu, d_delta, d_phi, d_W, d_X, d_temp_double, g, k, N,
           G);
        go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, (long long)(k - 1) * G + g), N);
      }
    go(k_upd_beta, grid((long long)G * (K - 1)), T, 0, d_states, d_pbeta, d_log_rho, I(d_L, G), D(d_beta, G), d_p,
       G * (K - 1));
    go(k_prop_nu, grid((long long)G * (B - 1)), T, 0, d_states, d_pnu, D(d_nu, G), G * (B - 1));
    si = 0;
    for (int b = 1; b < B; ++b) {
      si += n_b[b - 1];
      for (int g = 0; g < G; ++g) {
        go(k_fill_nu, grid(n_b[b]), T, 0, d_pnu, d_nu, d_alpha, d_beta, D(d_delta, si), d_phi, I(d_W, si),
           I(d_X, si * G), d_temp_double, b, g, G, n_b[b]);
        go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, (long long)(b - 1) * G + g), n_b[b]);
      }
    }
    go(k_upd_nu, grid((long long)G * (B - 1)), T, 0, d_states, d_pnu, d_log_rho, D(d_nu, G), G, G * (B - 1));
    go(k_prop_delta, grid(N), T, 0, d_states, d_pdelta, d_delta, N);
    si = 0;
    for (int b = 0; b < B; ++b) {
      for (int i = 1; i < n_b[b]; ++i) {
        go(k_fill_delta, grid(G), T, 0, d_pdelta, d_delta, d_alpha, d_beta, d_nu, d_phi, d_W, d_X, d_temp_double,
           (int)(si + i), G);
        go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, si + i), G);
      }
      si += n_b[b];
    }
    go(k_upd_delta, grid(N), T, 0, d_states, d_pdelta, d_log_rho, d_mu_delta, d_delta, N);
    go(k_prop_phi, grid((long long)B * G), T, 0, d_states, d_pphi, d_phi, B * G);
    si = 0;
    long long bg = 0;
    for (int b = 0; b < B; ++b) {
      if (b > 0) si += n_b[b - 1];
      for (int g = 0; g < G; ++g) {
        go(k_fill_phi, grid(n_b[b]), T, 0, D(d_pphi, bg), D(d_phi, bg), D(d_alpha, g), D(d_beta, g), D(d_nu, bg),
           D(d_delta, si), I(d_W, si), I(d_X, si * G + g), d_temp_double, b, G);
        go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, bg), n_b[b]);
        ++bg;
      }
    }
    go(k_upd_phi, grid((long long)B * G), T, 0, d_states, d_pphi, d_log_rho, d_phi, B * G);
    go(k_prop_W, grid(N), T, 0, d_states, d_pW, N, K);
    for (int i = 0; i < N; ++i) {
      go(k_fill_W, grid(G), T, 0, d_pW, d_W, d_alpha, d_beta, d_nu, d_delta, d_phi, d_X, d_temp_double, i, G);
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, i), G);
    }
    go(k_upd_W, grid(N), T, 0, d_states, d_pW, d_log_rho, d_pi, d_W, N, K);
    si = 0;
    for (int b = 0; b < B; ++b) {
      if (b > 0) si += n_b[b - 1];
      for (int k = 0; k < K; ++k) {
        go(k_fill_IW, grid(n_b[b]), T, 0, I(d_W, si), d_temp_int, k, n_b[b]);
        go(k_sum_i, 1u, T, S_I, d_temp_int, I(d_count, (long long)b * K + k), n_b[b]);
      }
    }
  };

  // Both sweep variants captured once as graphs; direct launches if capture fails.
  CUgraphExec exec[2] = {nullptr, nullptr};
  long long launches_per_graph[2] = {0, 0};
  bool graphs = getenv("REF_CHAIN_NO_GRAPH") == nullptr;
  for (int v = 0; v < 2 && graphs; ++v) {
    const long long l0 = g_launches;
    if (cuStreamBeginCapture(g_stream, CU_STREAM_CAPTURE_MODE_THREAD_LOCAL) != CUDA_SUCCESS) {
      graphs = false;
      break;
    }
    sweep_body(v == 1);
    CUgraph graph;
    CK(cuStreamEndCapture(g_stream, &graph));
    CK(cuGraphInstantiate(&exec[v], graph, 0));
    CK(cuGraphDestroy(graph));
    launches_per_graph[v] = g_launches - l0;
    g_launches = l0;
  }

  std::mt19937_64 pi_rng((uint64_t)seed * 0x9E3779B97F4A7C15ull + 0x5851F42D4C957F2Dull);
  std::vector<int32_t> h_count((size_t)B * K);
  std::vector<double> h_pi((size_t)B * K);
  auto draw_pi = [&]() {
    CK(cuMemcpyDtoHAsync(h_count.data(), d_count, 4ull * B * K, g_stream));
    CK(cuStreamSynchronize(g_stream));
    for (int b = 0; b < B; ++b) {
      double tot = 0.0;
      for (int k = 0; k < K; ++k) {
        std::gamma_distribution<double> gam(h_count[(size_t)b * K + k] + XI_PI, 1.0);
        h_pi[(size_t)b * K + k] = gam(pi_rng);
        tot += h_pi[(size_t)b * K + k];
      }
      for (int k = 0; k < K; ++k) h_pi[(size_t)b * K + k] /= tot;
    }
    CK(cuMemcpyHtoDAsync(d_pi, h_pi.data(), 8ull * B * K, g_stream));
  };
  // false when a parameter is not finite or a mean could overflow
  auto state_ok = [&](std::string* why) {
    CK(cuStreamSynchronize(g_stream));
    auto alpha = down<double>(d_alpha, G), beta = down<double>(d_beta, (size_t)K * G);
    auto nu = down<double>(d_nu, (size_t)B * G), phi = down<double>(d_phi, (size_t)B * G);
    auto delta = down<double>(d_delta, N), gam = down<double>(d_gamma, 2 * B), p = down<double>(d_p, 2);
    double amax = -1e300, bmax = -1e300, nmax = -1e300, dmax = -1e300;
    bool fin = true;
    for (double v : alpha) { fin &= std::isfinite(v); amax = fmax(amax, v); }
    for (double v : beta) { fin &= std::isfinite(v); bmax = fmax(bmax, v); }
    for (double v : nu) { fin &= std::isfinite(v); nmax = fmax(nmax, v); }
    for (double v : delta) { fin &= std::isfinite(v); dmax = fmax(dmax, v); }
    for (double v : phi) fin &= std::isfinite(v) && v > 0.0 && v < 1e200;
    for (double v : gam) fin &= std::isfinite(v);
    for (double v : p) fin &= std::isfinite(v);
    if (!fin) { *why = "a parameter is not finite (or phi left (0, 1e200))"; return false; }
    if (amax + bmax + nmax + dmax > 650.0) { *why = "a mean exp(alpha+beta+nu+delta) could overflow"; return false; }
    return true;
  };

  // ---- burn-in and kept sweeps ---------------------------------------------
  const auto t0 = std::chrono::steady_clock::now();
  long long sweep_launches = 0;
  std::string why;
  int done = 0;
  for (int it = 0; it < n_iter; ++it) {
    if (!state_ok(&why)) break;
    const int v = it >= n_unchanged ? 1 : 0;  // :1312 (burn-in) and :1459 (kept, iter >= u - b)
    if (graphs) {
      CK(cuGraphLaunch(exec[v], g_stream));
      sweep_launches += launches_per_graph[v];
    } else {
      const long long l0 = g_launches;
      sweep_body(v == 1);
      sweep_launches += g_launches - l0;
    }
    draw_pi();
    if (it >= n_burnin) {  // :1546-1554
      const int k_it = it - n_burnin;
      const long long l0 = g_launches;
      go(k_st_gamma, grid(2ll * B), T, 0, d_gamma, d_pres_gamma, k_it, n_pres, 2 * B);
      go(k_st_alpha, grid(G), T, 0, d_alpha, d_pres_alpha, k_it, n_pres, G);
      go(k_st_Lbeta, grid((long long)G * (K - 1)), T, 0, I(d_L, G), d_pres_L, D(d_beta, G), d_pres_beta, k_it, n_pres,
         G * (K - 1));
      CK(cuMemcpyDtoDAsync(D(d_pres_p, k_it), d_p, 8, g_stream));
      CK(cuMemcpyDtoDAsync(D(d_pres_p, (long long)n_pres + k_it), D(d_p, 1), 8, g_stream));
      go(k_st_nuphi, grid((long long)B * G), T, 0, d_nu, d_pres_nu, d_phi, d_pres_phi, k_it, n_pres, G, B * G);
      go(k_st_deltaW, grid(N), T, 0, d_delta, d_pres_delta, d_W, d_pres_W, k_it, n_pres, N);
      go(k_st_pi, grid((long long)B * K), T, 0, d_pi, d_pres_pi, k_it, n_pres, B * K);
      sweep_launches += g_launches - l0;
    }
    ++done;
  }
  CK(cuStreamSynchronize(g_stream));
  const double mcmc_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

  if (done == n_iter) {
    struct Out { const char* name; CUdeviceptr p; size_t bytes; };
    const Out outs[] = {
        {"gamma", d_pres_gamma, 16ull * B * n_pres},
        {"alpha", d_pres_alpha, 8ull * G * n_pres},
        {"L", d_pres_L, 4ull * G * (K - 1) * n_pres},
        {"beta", d_pres_beta, 8ull * G * (K - 1) * n_pres},
        {"p", d_pres_p, 16ull * n_pres},
        {"nu", d_pres_nu, 8ull * G * (B - 1) * n_pres},
        {"delta", d_pres_delta, 8ull * N * n_pres},
        {"phi", d_pres_phi, 8ull * B * G * n_pres},
        {"W", d_pres_W, 4ull * N * n_pres},
        {"pi", d_pres_pi, 8ull * B * K * n_pres},
    };
    for (const Out& o : outs) {
      std::vector<char> h = down<char>(o.p, o.bytes);
      wrote &= write_file(out_dir + "/preserved_" + o.name + ".bin", h.data(), h.size());
    }
  }
  printf("{\"impl\": \"reference .cu kernels, BUSseq_gpu.cu:1163-1555\", \"N\": %d, \"G\": %d, \"K\": %d, \"B\": %d, "
         "\"seed\": %d, \"n_iter\": %d, \"n_burnin\": %d, \"n_unchanged\": %d, \"p0\": %.17g, \"sweeps_done\": %d, "
         "\"ok\": %s, \"error\": \"%s\", \"init_s\": %.3f, \"mcmc_s\": %.3f, \"seconds_per_sweep\": %.6f, "
         "\"launches_per_sweep\": %.1f, \"graphs\": %s, \"files_written\": %s, "
         "\"pi\": \"host Dirichlet(count + 2) draws; update_pi not launched\"}\n",
         N, G, K, B, seed, n_iter, n_burnin, n_unchanged, p0, done, done == n_iter ? "true" : "false", why.c_str(),
         init_s, mcmc_s, done ? mcmc_s / done : 0.0, done ? (double)sweep_launches / done : 0.0,
         graphs ? "true" : "false", wrote ? "true" : "false");
  return done == n_iter && wrote ? 0 : 3;
}
