// busseq -- drop-in replacement of the reference BUSseq_gpu executable.
//
// Same command line (getopt "B:N:G:K:s:c:i:b:u:po:", BUSseq_gpu.cu:1048),
// same defaults and derived defaults (:1028-1111), same checks and messages
// (:1120-1134), same stdout phase lines and output files (:1118-2018).
// Options the reference does not have are long options only:
//   --w-update=mh|gibbs   W move (default mh, the reference's)
//   --device=D            CUDA device ordinal
//   --stats               print per-phase wall times to stderr
//   --corrected           also write <prefix>_corrected_X.txt, the batch-corrected
//                         counts (randomised quantile matching of _post_X)
//   --posterior-zx        also write <prefix>_post_X_mean.txt and _post_Z_prob.txt,
//                         E[X] and P(Z = 1) over the kept sweeps
//   --hmc=L               replace the random-walk steps of alpha, beta, nu, delta and
//                         phi by one Hamiltonian Monte Carlo transition with L
//                         leapfrog steps per sweep
//   --hmc-gene            with --hmc: accept or reject each gene's block on its own
//                         (delta by an adapted random-walk step)
#include "busseq_gb300.h"

#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <chrono>
#include <string>
#include <vector>

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

[[noreturn]] void die_lib(const char* what) {
  fprintf(stderr, "busseq: %s: %s\n", what, busseq_last_error());
  exit(1);
}

}  // namespace

int main(int argc, char** argv) {
  int B = 4;
  std::vector<int32_t> n_b = {300, 300, 200, 200};
  n_b.resize(200, 0);
  long G = 3000;
  int K = 5;
  int seed = 0;
  char count_data[4096] = "count_data/demo_count.txt";
  int n_iter = 4000, n_burnin = 2000, n_unchanged = 500;
  int print_preserved = 0;
  char output_file[4096] = "demo_output";
  char n_file[4096] = "";
  int n_file_flag = 0, burnin_flag = 1, unchanged_flag = 1, seed_flag = 1;
  int w_update = BUSSEQ_W_MH, device = 0, stats = 0, ck_every = 0, stop_after = 0, corrected = 0, posterior_zx = 0;
  int hmc_leapfrog = 0, hmc_gene = 0;
  std::string ck_path, resume_path;

  static struct option longopts[] = {{"w-update", required_argument, nullptr, 1000},
                                     {"device", required_argument, nullptr, 1001},
                                     {"stats", no_argument, nullptr, 1002},
                                     {"checkpoint", required_argument, nullptr, 1003},
                                     {"checkpoint-every", required_argument, nullptr, 1004},
                                     {"resume", required_argument, nullptr, 1005},
                                     {"stop-after", required_argument, nullptr, 1006},
                                     {"corrected", no_argument, nullptr, 1007},
                                     {"posterior-zx", no_argument, nullptr, 1008},
                                     {"hmc", required_argument, nullptr, 1009},
                                     {"hmc-gene", no_argument, nullptr, 1010},
                                     {nullptr, 0, nullptr, 0}};
  int opt;
  while ((opt = getopt_long(argc, argv, "B:N:G:K:s:c:i:b:u:po:", longopts, nullptr)) != -1) {
    switch (opt) {
      case 'B': B = atoi(optarg); break;
      case 'N': n_file_flag = 1; snprintf(n_file, sizeof(n_file), "%s", optarg); break;
      case 'G': G = atol(optarg); break;
      case 'K': K = atoi(optarg); break;
      case 's': seed_flag = 0; seed = atoi(optarg); break;
      case 'c': snprintf(count_data, sizeof(count_data), "%s", optarg); break;
      case 'i': n_iter = atoi(optarg); break;
      case 'b': burnin_flag = 0; n_burnin = atoi(optarg); break;
      case 'u': unchanged_flag = 0; n_unchanged = atoi(optarg); break;
      case 'p': print_preserved = 1; break;
      case 'o': snprintf(output_file, sizeof(output_file), "%s", optarg); break;
      case 1000:
        if (!strcmp(optarg, "gibbs")) w_update = BUSSEQ_W_GIBBS;
        else if (!strcmp(optarg, "mh")) w_update = BUSSEQ_W_MH;
        else { fprintf(stderr, "--w-update must be mh or gibbs\n"); return 1; }
        break;
      case 1001: device = atoi(optarg); break;
      case 1002: stats = 1; break;
      case 1003: ck_path = optarg; break;
      case 1004: ck_every = atoi(optarg); break;
      case 1005: resume_path = optarg; break;
      case 1006: stop_after = atoi(optarg); break;
      case 1007: corrected = 1; break;
      case 1008: posterior_zx = 1; break;
      case 1009: {
        char* end = nullptr;
        const long L = strtol(optarg, &end, 10);
        if (!end || *end || L < 1 || L > 1000) {
          fprintf(stderr, "--hmc takes a number of leapfrog steps from 1 to 1000\n");
          return 1;
        }
        hmc_leapfrog = (int)L;
        break;
      }
      case 1010: hmc_gene = 1; break;
      default:
        // The reference's usage line byte for byte (BUSseq_gpu.cu:1088), lower-case
        // flag names and stray parenthesis included: its stdout is part of the
        // drop-in contract.
        printf("Error Usage: %s [-b batch] [-n sample_size_file] [-g gene] [-k celltype] "
               "[-c count_data_file)] [-i iterations] [-b burnin] [-u unchanged_iterations] "
               "[-p print_preserved] [-o output_prefix] \n",
               argv[0]);
        exit(1);
    }
  }
  if (hmc_gene && !hmc_leapfrog) {
    fprintf(stderr, "--hmc-gene needs --hmc=L\n");
    return 1;
  }
  if (B > BUSSEQ_MAX_BATCHES || B > (int)n_b.size()) {
    printf("At most %d batches are supported.\n", BUSSEQ_MAX_BATCHES);
    return -1;
  }
  if (argc > 1) {
    if (n_file_flag) {
      FILE* f = fopen(n_file, "r");
      if (!f) { printf("Cannot open the batch-size file %s.\n", n_file); return -1; }
      for (int b = 0; b < B; ++b)
        if (fscanf(f, "%d", &n_b[b]) != 1) { printf("Cannot read %d batch sizes from %s.\n", B, n_file); return -1; }
      fclose(f);
    }
    if (burnin_flag) n_burnin = n_iter / 2;
    if (unchanged_flag) n_unchanged = (0.3 * n_iter > 500) ? (int)(0.3 * n_iter) : 500;
  }
  if (seed_flag) {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    seed = (int)tv.tv_usec;
  }
  printf("Seed is %d\n", seed);
  if (n_burnin > n_iter) {
    printf("Burn-in iterations must be less than total number of iterations.\n");
    return -1;
  }
  if (B < 2) {
    printf("The batch number must be greater than one.\n");
    return -1;
  }
  for (int b = 0; b < B; ++b)
    if (n_b[b] < K) {
      printf("The sample size in any batch must be greater than the assumed cell type number.\n");
      return -1;
    }
  int64_t N = 0;
  for (int b = 0; b < B; ++b) N += n_b[b];
  fflush(stdout);

  double t0 = now_s();
  printf("Start reading file.\n");
  fflush(stdout);
  std::vector<int32_t> Y((size_t)N * G);
  if (busseq_read_counts(count_data, N, G, Y.data()) != BUSSEQ_OK) die_lib("reading the count file");
  double t1 = now_s();

  printf("Start initialization.\n");
  fflush(stdout);
  srand((unsigned)seed);
  const double p0 = ((double)rand() * 0.5) / RAND_MAX;  // p_init_bound = 0.5 (BUSseq_gpu.cu:1172-1173)
  busseq_dims dims{B, K, G, n_b.data()};
  busseq_options o{};
  o.seed = (uint64_t)(uint32_t)seed;
  o.p0 = p0 > 0.0 ? p0 : 1e-9;
  o.w_update = w_update;
  o.keep_draws = print_preserved;
  o.zx_summaries = posterior_zx;
  o.hmc_leapfrog = hmc_leapfrog;
  o.hmc_gene_accept = hmc_gene;
  o.device = device;
  busseq_handle* h = nullptr;
  if (busseq_create(&dims, Y.data(), 0, &o, &h) != BUSSEQ_OK) die_lib("initialisation");
  std::vector<int32_t>().swap(Y);
  double t2 = now_s();

  printf("Start MCMC.\n");
  fflush(stdout);
  int done = 0;
  if (!resume_path.empty()) {
    // --resume: the run's lengths come from the checkpoint
    if (busseq_checkpoint_load(h, resume_path.c_str()) != BUSSEQ_OK) die_lib("resuming");
    if (busseq_get_progress(h, &done, &n_iter, &n_burnin) != BUSSEQ_OK) die_lib("resuming");
    if (n_iter == 0) {
      fprintf(stderr, "%s holds no run in progress\n", resume_path.c_str());
      return 1;
    }
    fprintf(stderr, "resumed from %s at sweep %d of %d\n", resume_path.c_str(), done, n_iter);
  } else if (busseq_begin(h, n_iter, n_burnin, n_unchanged) != BUSSEQ_OK) {
    die_lib("starting the run");
  }
  // sweeps up to `target`, with a checkpoint every ck_every sweeps and at the
  // end of each phase when --checkpoint is given
  if (stop_after > 0 && ck_path.empty()) {
    fprintf(stderr, "--stop-after needs --checkpoint\n");
    return 1;
  }
  auto advance_to = [&](int target, const char* what) {
    if (stop_after > 0 && target > stop_after) target = stop_after;
    while (done < target) {
      int step = target - done;
      if (ck_every > 0 && step > ck_every - done % ck_every) step = ck_every - done % ck_every;
      if (busseq_sweeps(h, step) != BUSSEQ_OK) die_lib(what);
      done += step;
      if (!ck_path.empty() && (done == target || (ck_every > 0 && done % ck_every == 0)))
        if (busseq_synchronize(h) != BUSSEQ_OK || busseq_checkpoint_save(h, ck_path.c_str()) != BUSSEQ_OK)
          die_lib("writing the checkpoint");
    }
    if (busseq_synchronize(h) != BUSSEQ_OK) die_lib(what);
  };
  auto stop_here = [&]() {
    if (stop_after > 0 && done >= stop_after && done < n_iter) {
      fprintf(stderr, "stopped after sweep %d of %d; checkpoint in %s\n", done, n_iter, ck_path.c_str());
      busseq_destroy(h);
      exit(0);
    }
  };
  advance_to(n_burnin, "burn-in");
  stop_here();
  printf("Burnin completed. Start recording iterations.\n");
  fflush(stdout);
  advance_to(n_iter, "sampling");
  stop_here();
  double t3 = now_s();

  printf("Start posterior inference.\n");
  fflush(stdout);
  if (busseq_finish(h) != BUSSEQ_OK) die_lib("posterior inference");
  printf("Start writing output files.\n");
  if (print_preserved) printf("Start writing preserved iterations.\n");
  fflush(stdout);
  if (busseq_write_outputs(h, output_file, print_preserved) != BUSSEQ_OK) die_lib("writing outputs");
  if (corrected && busseq_write_corrected(h, output_file) != BUSSEQ_OK) die_lib("writing corrected counts");
  if (posterior_zx && busseq_write_zx_summaries(h, output_file) != BUSSEQ_OK) die_lib("writing Z/X summaries");
  double t4 = now_s();
  if (stats) {
    fprintf(stderr,
            "{\"read_s\": %.3f, \"init_s\": %.3f, \"mcmc_s\": %.3f, \"iters_per_s\": %.2f, \"post_write_s\": %.3f}\n",
            t1 - t0, t2 - t1, t3 - t2, n_iter / (t3 - t2 > 0 ? t3 - t2 : 1e-9), t4 - t3);
  }
  busseq_destroy(h);
  return 0;
}
