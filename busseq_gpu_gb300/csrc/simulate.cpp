// Synthetic data from the BUSseq generative model (host, all threads).
//
//   alpha_g ~ U(alpha_lo, alpha_hi)
//   beta_g0 = 0; for k >= 1, beta_gk = 0 with probability 1 - de_frac, else
//              +/- U(beta_lo, beta_hi) with a random sign
//   nu_0g = 0; nu_bg ~ N(nu_step * b, nu_sd^2) for b >= 1
//   delta_bi ~ N(0, delta_sd^2), 0 for the first cell of each batch
//   phi_bg ~ U(phi_lo, phi_hi);  pi_b ~ Dirichlet(pi_conc 1_K);  W_i ~ Cat(pi_b)
//   X_ig ~ NB(mean exp(alpha_g + beta_g,W_i + nu_bg + delta_i), size phi_bg)
//   Z_ig ~ Bernoulli(logistic(gamma0 + gamma1 X_ig));  Y = X (1 - Z)
// Every draw comes from its own counter-based stream, so the data depend only
// on the seed, not on the number of threads.
#include "busseq_gb300.h"
#include "rng.h"

#include <math.h>

#include <algorithm>
#include <thread>
#include <vector>

extern "C" int busseq_internal_set_error(int code, const char* msg);

namespace {
enum : uint32_t { SUB_ALPHA = 1, SUB_BETA = 2, SUB_NU = 3, SUB_DELTA = 4, SUB_PHI = 5, SUB_PI = 6, SUB_W = 7, SUB_X = 8 };

inline double unif(bq::Stream& s) { return (double)s.uniform(); }
inline double norm(bq::Stream& s) { return (double)bq::normal(s); }
}  // namespace

extern "C" int busseq_simulate(const busseq_dims* dims, const busseq_sim_params* prm, uint64_t seed, int32_t* Y,
                               int32_t* W_true, int32_t* X_true) {
  if (!dims || !prm || !Y || !dims->n_b) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "NULL argument");
  const int B = dims->B, K = dims->K;
  const int64_t G = dims->G;
  if (B < 1 || K < 1 || G < 1) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "bad dimensions");
  std::vector<int64_t> off(B + 1, 0);
  for (int b = 0; b < B; ++b) off[b + 1] = off[b] + dims->n_b[b];
  const int64_t N = off[B];
  using bq::Stream;
  const uint32_t sid = bq::SID_SIM;
  std::vector<double> alpha(G), beta((size_t)K * G, 0.0), nu((size_t)B * G, 0.0), phi((size_t)B * G), delta(N),
      pi((size_t)B * K);
  std::vector<int32_t> W(N);
  for (int64_t g = 0; g < G; ++g) {
    Stream s(seed, sid, (uint64_t)g, SUB_ALPHA);
    alpha[g] = prm->alpha_lo + (prm->alpha_hi - prm->alpha_lo) * unif(s);
    for (int k = 1; k < K; ++k) {
      Stream sb(seed, sid, (uint64_t)k * G + g, SUB_BETA);
      if (unif(sb) < prm->de_frac) {
        const double mag = prm->beta_lo + (prm->beta_hi - prm->beta_lo) * unif(sb);
        beta[(size_t)k * G + g] = unif(sb) < 0.5 ? -mag : mag;
      }
    }
    for (int b = 0; b < B; ++b) {
      Stream sn(seed, sid, (uint64_t)b * G + g, SUB_NU);
      if (b > 0) nu[(size_t)b * G + g] = prm->nu_step * b + prm->nu_sd * norm(sn);
      Stream sp(seed, sid, (uint64_t)b * G + g, SUB_PHI);
      phi[(size_t)b * G + g] = prm->phi_lo + (prm->phi_hi - prm->phi_lo) * unif(sp);
    }
  }
  for (int b = 0; b < B; ++b) {
    double tot = 0.0;
    for (int k = 0; k < K; ++k) {
      Stream s(seed, sid, (uint64_t)b * K + k, SUB_PI);
      int err = 0;
      pi[(size_t)b * K + k] = bq::gamma_mt(s, (float)prm->pi_conc, &err);
      tot += pi[(size_t)b * K + k];
    }
    for (int k = 0; k < K; ++k) pi[(size_t)b * K + k] /= tot;
  }
  for (int b = 0; b < B; ++b)
    for (int64_t i = off[b]; i < off[b + 1]; ++i) {
      Stream sd(seed, sid, (uint64_t)i, SUB_DELTA);
      delta[i] = i == off[b] ? 0.0 : prm->delta_sd * norm(sd);
      Stream sw(seed, sid, (uint64_t)i, SUB_W);
      const double u = unif(sw);
      int k = 0;
      double acc = pi[(size_t)b * K];
      while (u > acc && k < K - 1) acc += pi[(size_t)b * K + ++k];
      W[i] = k;
    }
  const int nt = std::max(1, (int)std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) {
    th.emplace_back([&, t]() {
      for (int64_t i = t; i < N; i += nt) {
        int b = 0;
        while (i >= off[b + 1]) ++b;
        int64_t lib = 0;
        int64_t gmax = 0;
        double mumax = -1.0;
        for (int64_t g = 0; g < G; ++g) {
          const double mu = exp(alpha[g] + beta[(size_t)W[i] * G + g] + nu[(size_t)b * G + g] + delta[i]);
          Stream s(seed, sid, (uint64_t)i * (uint64_t)G + (uint64_t)g, SUB_X);
          int err = 0;
          const int x = bq::negbin(s, (float)mu, (float)phi[(size_t)b * G + g], &err);
          const double pz = 1.0 / (1.0 + exp(-(prm->gamma0 + prm->gamma1 * x)));
          const int y = unif(s) < pz ? 0 : x;
          Y[i * G + g] = y;
          if (X_true) X_true[i * G + g] = x;
          lib += y;
          if (mu > mumax) { mumax = mu; gmax = g; }
        }
        if (lib == 0) Y[i * G + gmax] = 1;  // the model needs a positive library size
      }
    });
  }
  for (auto& x : th) x.join();
  if (W_true)
    for (int64_t i = 0; i < N; ++i) W_true[i] = W[i];
  return BUSSEQ_OK;
}
