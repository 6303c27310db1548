// ===========================================================================
// Reference sweep timer -- MEASUREMENT INFRASTRUCTURE ONLY.
//
// Times the reference implementation's Gibbs sweep on this GPU.  It loads
// oracle/_ref/busseq_ref.cubin (the reference's device code, compiled by
// oracle/build.py from BUSseq_gpu.cu where it lies; nothing of it is copied
// into this repository) and replays, through the CUDA driver API, the launch
// sequence of one burn-in sweep of the reference's host loop
// (BUSseq_gpu.cu:1267-1398): the same kernels, grids, block sizes, dynamic
// shared memory and argument values, one launch after another on the default
// stream.  The initial state is simple (X = Y, Z = 0, random W, alpha from the
// gene means, beta = nu = delta = 0, phi = 5, gamma = (0, -0.3), uniform pi,
// p = 0.25, tau0 = 0.005); the reference is launch-bound, so its time per
// sweep does not depend on the state.  p and tau0 are updated in every timed
// sweep (iter >= n_unchanged), as in the later part of a run.  The pi draw
// update_pi (:866-890) is left out: its barrier at :886 is inside a branch
// that only K of the block's 1024 threads take, which is not run here.
//
// usage: ref_sweep_timer <cubin> <Y.i32> <G> <K> <seed> <sweeps> <n_1> ... <n_B>
//   Y.i32: N*G int32 counts, cell-major, cells batch-contiguous.
// Prints one JSON line: sweeps, seconds per sweep, launches per sweep.
// ===========================================================================
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

namespace {

void die(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  fprintf(stderr, "ref_sweep_timer: %s failed: %s\n", what, s ? s : "?");
  exit(2);
}
#define CK(x)                                  \
  do {                                         \
    CUresult r_ = (x);                         \
    if (r_ != CUDA_SUCCESS) die(#x, r_);       \
  } while (0)

CUmodule g_mod;
long long g_launches = 0;

CUfunction fn(const char* mangled) {
  CUfunction f;
  CK(cuModuleGetFunction(&f, g_mod, mangled));
  return f;
}

// One launch with the argument values given in order (each passed by address).
template <typename... A>
void go(CUfunction f, unsigned grid, unsigned block, unsigned smem, A... a) {
  void* args[] = {(void*)&a...};
  CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, 0, args, nullptr));
  ++g_launches;
}

CUdeviceptr dalloc(size_t bytes) {
  CUdeviceptr p;
  CK(cuMemAlloc(&p, bytes ? bytes : 8));
  CK(cuMemsetD8(p, 0, bytes ? bytes : 8));
  return p;
}

template <typename T>
CUdeviceptr up(const std::vector<T>& v) {
  CUdeviceptr p = dalloc(v.size() * sizeof(T));
  CK(cuMemcpyHtoD(p, v.data(), v.size() * sizeof(T)));
  return p;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 9) {
    fprintf(stderr, "usage: ref_sweep_timer <cubin> <Y.i32> <G> <K> <seed> <sweeps> <n_1> ... <n_B>\n");
    return 1;
  }
  const int G = atoi(argv[3]), K = atoi(argv[4]), seed = atoi(argv[5]), sweeps = atoi(argv[6]);
  const int B = argc - 7;
  std::vector<int> n_b(B);
  for (int b = 0; b < B; ++b) n_b[b] = atoi(argv[7 + b]);
  int N = 0;
  for (int b = 0; b < B; ++b) N += n_b[b];
  if (B < 2 || B > 128 || K < 2 || G < 1 || sweeps < 1) {
    fprintf(stderr, "bad dimensions\n");
    return 1;
  }
  std::vector<int32_t> Y((size_t)N * G);
  {
    FILE* f = fopen(argv[2], "rb");
    if (!f || fread(Y.data(), 4, Y.size(), f) != Y.size()) {
      fprintf(stderr, "cannot read %zu counts from %s\n", Y.size(), argv[2]);
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
  {
    CUdeviceptr sym;
    size_t sz;
    CK(cuModuleGetGlobal(&sym, &sz, g_mod, "d_n_b"));
    CK(cuMemcpyHtoD(sym, n_b.data(), 4 * B));
    std::vector<double> mu_nu(B, 0.0);
    CK(cuModuleGetGlobal(&sym, &sz, g_mod, "d_mu_nu"));
    CK(cuMemcpyHtoD(sym, mu_nu.data(), 8 * B));
  }

  // ---- kernels (reference file:line) ---------------------------------------
  CUfunction k_init_rand = fn("_Z17initialize_curandiP17curandStateXORWOWi");                  // :220
  CUfunction k_zx = fn("_Z10update_Z_XP17curandStateXORWOWPiS1_PdS2_S2_S2_S2_S2_S1_S1_iii");    // :484
  CUfunction k_prop_gamma = fn("_Z13propose_gammaP17curandStateXORWOWPdS1_i");                  // :514
  CUfunction k_fill_g0 = fn("_Z16fill_prop_gamma0PdS_PiS0_S_iii");                              // :524
  CUfunction k_fill_g1 = fn("_Z16fill_prop_gamma1PdS_PiS0_S_iii");                              // :551
  CUfunction k_upd_g0 = fn("_Z13update_gamma0P17curandStateXORWOWPdS1_S1_i");                   // :578
  CUfunction k_upd_g1 = fn("_Z13update_gamma1P17curandStateXORWOWPdS1_S1_i");                   // :588
  CUfunction k_prop_alpha = fn("_Z13propose_alphaP17curandStateXORWOWPdS1_i");                  // :602
  CUfunction k_fill_alpha = fn("_Z15fill_prop_alphaPdS_S_S_S_S_PiS0_S_iiii");                   // :608
  CUfunction k_upd_alpha = fn("_Z12update_alphaP17curandStateXORWOWPdS1_S1_S1_i");              // :625
  CUfunction k_upd_L = fn("_Z8update_LP17curandStateXORWOWPdS1_Pii");                           // :634
  CUfunction k_upd_p = fn("_Z8update_pP17curandStateXORWOWPiPdii");                             // :650
  CUfunction k_fill_Lb = fn("_Z16fill_I_L_beta_sqPiPdS0_i");                                    // :654
  CUfunction k_upd_tau0 = fn("_Z11update_tau0P17curandStateXORWOWPiPdii");                      // :664
  CUfunction k_prop_beta = fn("_Z12propose_betaP17curandStateXORWOWPdS1_i");                    // :670
  CUfunction k_fill_beta = fn("_Z14fill_prop_betaPdS_S_S_S_S_PiS0_S_iiii");                     // :676
  CUfunction k_upd_beta = fn("_Z11update_betaP17curandStateXORWOWPdS1_PiS1_S1_i");              // :696
  CUfunction k_prop_nu = fn("_Z10propose_nuP17curandStateXORWOWPdS1_i");                        // :709
  CUfunction k_fill_nu = fn("_Z12fill_prop_nuPdS_S_S_S_S_PiS0_S_iiii");                         // :715
  CUfunction k_upd_nu = fn("_Z9update_nuP17curandStateXORWOWPdS1_S1_ii");                       // :730
  CUfunction k_prop_delta = fn("_Z13propose_deltaP17curandStateXORWOWPdS1_i");                  // :739
  CUfunction k_fill_delta = fn("_Z15fill_prop_deltaPdS_S_S_S_S_PiS0_S_ii");                     // :746
  CUfunction k_upd_delta = fn("_Z12update_deltaP17curandStateXORWOWPdS1_S1_S1_i");              // :763
  CUfunction k_prop_phi = fn("_Z11propose_phiP17curandStateXORWOWPdS1_i");                      // :780
  CUfunction k_fill_phi = fn("_Z13fill_prop_phiPdS_S_S_S_S_PiS0_S_ii");                         // :789
  CUfunction k_upd_phi = fn("_Z10update_phiP17curandStateXORWOWPdS1_S1_i");                     // :806
  CUfunction k_prop_W = fn("_Z9propose_WP17curandStateXORWOWPiii");                             // :820
  CUfunction k_fill_W = fn("_Z11fill_prop_WPiS_PdS0_S0_S0_S0_S_S0_ii");                         // :831
  CUfunction k_upd_W = fn("_Z8update_WP17curandStateXORWOWPiPdS2_S1_ii");                       // :846
  CUfunction k_fill_IW = fn("_Z8fill_I_WPiS_ii");                                               // :856
  CUfunction k_sum_d = fn("_Z10sum_on_gpuIdEvPT_S1_i");                                         // :236
  CUfunction k_sum_i = fn("_Z10sum_on_gpuIiEvPT_S1_i");                                         // :236

  const unsigned T = 1024;  // threads_per_block of the reference (:1141)
  auto grid = [&](long long n) { return (unsigned)((n - 1) / T + 1); };

  // ---- state ----------------------------------------------------------------
  const size_t NG = (size_t)N * G;
  CUdeviceptr d_states = dalloc(NG * 48);  // sizeof(curandStateXORWOW) = 48
  go(k_init_rand, grid((long long)NG), T, 0, seed, d_states, (int)NG);

  std::vector<double> alpha(G), beta((size_t)K * G, 0.0), nu((size_t)B * G, 0.0), delta(N, 0.0),
      phi((size_t)B * G, 5.0), gamma(2 * B), pi((size_t)B * K, 1.0 / K), p = {0.25, 0.005};
  for (int g = 0; g < G; ++g) {
    double s = 0;
    for (int i = 0; i < N; ++i) s += Y[(size_t)i * G + g];
    alpha[g] = log(s / N + 1.0);
  }
  for (int b = 0; b < B; ++b) {
    gamma[b] = 0.0;
    gamma[B + b] = -0.3;
  }
  std::vector<int32_t> W(N), L((size_t)K * G, 0), Z(NG, 0);
  uint64_t lcg = (uint64_t)seed * 6364136223846793005ull + 1442695040888963407ull;
  for (int i = 0; i < N; ++i) {
    lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
    W[i] = (int)((lcg >> 33) % (uint64_t)K);
  }
  CUdeviceptr d_Y = up(Y), d_X = up(Y), d_Z = up(Z), d_W = up(W), d_L = up(L);
  CUdeviceptr d_alpha = up(alpha), d_mu_alpha = up(alpha), d_beta = up(beta), d_nu = up(nu);
  CUdeviceptr d_delta = up(delta), d_mu_delta = up(delta), d_phi = up(phi), d_gamma = up(gamma);
  CUdeviceptr d_pi = up(pi), d_p = up(p);
  const long long log_rho_len = (long long)(N > G ? N : G) * (B > K ? B : K);
  CUdeviceptr d_log_rho = dalloc(8 * log_rho_len);
  CUdeviceptr d_temp_double = dalloc(8 * NG);
  CUdeviceptr d_temp_int = dalloc(4 * (size_t)(N > 4096 ? N : 4096));
  CUdeviceptr d_count = dalloc(4 * (size_t)K * N);
  CUdeviceptr d_pgamma = dalloc(8 * 2 * B), d_palpha = dalloc(8 * (size_t)G), d_pbeta = dalloc(8 * (size_t)G * (K - 1));
  CUdeviceptr d_pnu = dalloc(8 * (size_t)G * (B - 1)), d_pdelta = dalloc(8 * (size_t)N), d_pphi = dalloc(8 * (size_t)B * G);
  CUdeviceptr d_pW = dalloc(4 * (size_t)N);
  CK(cuCtxSynchronize());

  auto I = [](CUdeviceptr base, long long elems) { return base + 4ull * elems; };  // int* + offset
  auto D = [](CUdeviceptr base, long long elems) { return base + 8ull * elems; };  // double* + offset
  const unsigned S_D = T * sizeof(double), S_I = T * sizeof(int);

  // ---- one burn-in sweep, in the order of BUSseq_gpu.cu:1267-1398 ----------
  auto sweep = [&]() {
    go(k_zx, grid((long long)NG), T, 0, d_states, d_Y, d_W, d_alpha, d_beta, d_nu, d_delta, d_gamma, d_phi, d_Z, d_X, B,
       N, G);
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
    // alpha
    go(k_prop_alpha, grid(G), T, 0, d_states, d_palpha, d_alpha, G);
    for (int g = 0; g < G; ++g) {
      go(k_fill_alpha, grid(N), T, 0, d_palpha, d_alpha, d_beta, d_nu, d_delta, d_phi, d_W, d_X, d_temp_double, g, B, N,
         G);
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, g), N);
    }
    go(k_upd_alpha, grid(G), T, 0, d_states, d_palpha, d_log_rho, d_mu_alpha, d_alpha, G);
    // L, then p and tau0 (iter >= n_unchanged)
    go(k_upd_L, grid((long long)G * (K - 1)), T, 0, d_states, d_p, D(d_beta, G), I(d_L, G), G * (K - 1));
    go(k_sum_i, 1u, T, S_I, I(d_L, G), d_count, G * (K - 1));
    go(k_fill_Lb, grid((long long)G * (K - 1)), T, 0, I(d_L, G), D(d_beta, G), d_temp_double, G * (K - 1));
    go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_p, 1), G * (K - 1));
    go(k_upd_p, 1u, 1u, 0, d_states, d_count, d_p, G, K);
    go(k_upd_tau0, 1u, 1u, 0, d_states, d_count, d_p, G, K);
    // beta
    go(k_prop_beta, grid((long long)G * (K - 1)), T, 0, d_states, d_pbeta, D(d_beta, G), G * (K - 1));
    for (int k = 1; k < K; ++k)
      for (int g = 0; g < G; ++g) {
        go(k_fill_beta, grid(N), T, 0, d_pbeta, d_beta, d_alpha, d_nu, d_delta, d_phi, d_W, d_X, d_temp_double, g, k, N,
           G);
        go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, (long long)(k - 1) * G + g), N);
      }
    go(k_upd_beta, grid((long long)G * (K - 1)), T, 0, d_states, d_pbeta, d_log_rho, I(d_L, G), D(d_beta, G), d_p,
       G * (K - 1));
    // nu
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
    // delta
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
    // phi
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
    // W
    go(k_prop_W, grid(N), T, 0, d_states, d_pW, N, K);
    for (int i = 0; i < N; ++i) {
      go(k_fill_W, grid(G), T, 0, d_pW, d_W, d_alpha, d_beta, d_nu, d_delta, d_phi, d_X, d_temp_double, i, G);
      go(k_sum_d, 1u, T, S_D, d_temp_double, D(d_log_rho, i), G);
    }
    go(k_upd_W, grid(N), T, 0, d_states, d_pW, d_log_rho, d_pi, d_W, N, K);
    // pi
    si = 0;
    for (int b = 0; b < B; ++b) {
      if (b > 0) si += n_b[b - 1];
      for (int k = 0; k < K; ++k) {
        go(k_fill_IW, grid(n_b[b]), T, 0, I(d_W, si), d_temp_int, k, n_b[b]);
        go(k_sum_i, 1u, T, S_I, d_temp_int, I(d_count, k), n_b[b]);
      }
      // update_pi (BUSseq_gpu.cu:866-890) is NOT launched: its __syncthreads at
      // :886 sits inside `if (tid < K)` of a 1024-thread block, a divergent
      // barrier; B single-block launches of ~3.4e5 per sweep are left out.
    }
  };

  sweep();  // warm-up
  CK(cuCtxSynchronize());
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  const long long l0 = g_launches;
  CK(cuEventRecord(e0, 0));
  for (int s = 0; s < sweeps; ++s) sweep();
  CK(cuEventRecord(e1, 0));
  CK(cuEventSynchronize(e1));
  float ms = 0.f;
  CK(cuEventElapsedTime(&ms, e0, e1));
  const double sps = ms / 1000.0 / sweeps;
  printf("{\"impl\": \"reference .cu kernels, launch sequence of BUSseq_gpu.cu:1267-1398\", \"N\": %d, \"G\": %d, "
         "\"K\": %d, \"B\": %d, \"sweeps\": %d, \"seconds_per_sweep\": %.6f, \"sweeps_per_s\": %.6f, "
         "\"launches_per_sweep\": %lld}\n",
         N, G, K, B, sweeps, sps, 1.0 / sps, (g_launches - l0) / sweeps);
  return 0;
}
