// ===========================================================================
// Reference-kernel harness -- TEST INFRASTRUCTURE ONLY (golden-vector maker).
//
// Loads oracle/_ref/busseq_ref.cubin, which oracle/build_ref.py compiles from
// the reference source BUSseq_gpu.cu where it lies (nothing of it is copied
// into this repository), and launches the reference's DETERMINISTIC kernels
// (the per-element log-ratio fills, the BIC fills, the initialisation means)
// on inputs read from a file, through the CUDA driver API.  The outputs are
// written back so that tests/golden/make_ref_golden.py can store them as
// fixtures; tests then check the FP64 oracle against them on the CPU.
//
// Kernels used (reference file:line):
//   fill_prop_gamma0/1     BUSseq_gpu.cu:524-576
//   fill_prop_alpha        BUSseq_gpu.cu:608-623
//   fill_prop_beta         BUSseq_gpu.cu:676-694
//   fill_prop_nu           BUSseq_gpu.cu:715-728
//   fill_prop_delta        BUSseq_gpu.cu:746-761
//   fill_prop_phi          BUSseq_gpu.cu:789-804
//   fill_prop_W            BUSseq_gpu.cu:831-844
//   fill_log_likelihood_1  BUSseq_gpu.cu:967-1007
//   fill_log_likelihood_2  BUSseq_gpu.cu:1009-1024
//   first_delta_W          BUSseq_gpu.cu:419-443
//   fill_raw_means + sum_on_gpu<int> + selective_mean_on_gpu  (:369-382, :236-298)
//   first_nu_phi, first_pi BUSseq_gpu.cu:392-417
//   fill_mu_nu + mean_on_gpu BUSseq_gpu.cu:470-476, :300-327
//   mode_on_gpu            BUSseq_gpu.cu:944-959
//   initialize_curand      BUSseq_gpu.cu:220-224 (only to give first_delta_W a state)
//
// File format (input and output): a sequence of records
//   u32 name_len | name bytes | u8 dtype (0=f64, 1=i32) | u64 count | data
// ===========================================================================
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <map>
#include <string>
#include <vector>

namespace {

struct Arr {
  uint8_t dtype = 0;
  std::vector<double> f;
  std::vector<int32_t> i;
};

std::map<std::string, Arr> g_in, g_out;

void die(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  fprintf(stderr, "ref_harness: %s failed: %s\n", what, s ? s : "?");
  exit(2);
}
#define CK(x) do { CUresult r_ = (x); if (r_ != CUDA_SUCCESS) die(#x, r_); } while (0)

bool read_file(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  for (;;) {
    uint32_t nl;
    if (fread(&nl, 4, 1, f) != 1) break;
    std::string name(nl, '\0');
    if (fread(&name[0], 1, nl, f) != nl) return false;
    uint8_t dt;
    uint64_t cnt;
    if (fread(&dt, 1, 1, f) != 1 || fread(&cnt, 8, 1, f) != 1) return false;
    Arr a;
    a.dtype = dt;
    if (dt == 0) { a.f.resize(cnt); if (fread(a.f.data(), 8, cnt, f) != cnt) return false; }
    else { a.i.resize(cnt); if (fread(a.i.data(), 4, cnt, f) != cnt) return false; }
    g_in[name] = std::move(a);
  }
  fclose(f);
  return true;
}

bool write_file(const char* path) {
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  for (auto& kv : g_out) {
    const uint32_t nl = (uint32_t)kv.first.size();
    fwrite(&nl, 4, 1, f);
    fwrite(kv.first.data(), 1, nl, f);
    fwrite(&kv.second.dtype, 1, 1, f);
    const uint64_t cnt = kv.second.dtype == 0 ? kv.second.f.size() : kv.second.i.size();
    fwrite(&cnt, 8, 1, f);
    if (kv.second.dtype == 0) fwrite(kv.second.f.data(), 8, cnt, f);
    else fwrite(kv.second.i.data(), 4, cnt, f);
  }
  fclose(f);
  return true;
}

const std::vector<double>& F(const char* n) {
  auto it = g_in.find(n);
  if (it == g_in.end() || it->second.dtype != 0) { fprintf(stderr, "missing f64 input %s\n", n); exit(3); }
  return it->second.f;
}
const std::vector<int32_t>& I(const char* n) {
  auto it = g_in.find(n);
  if (it == g_in.end() || it->second.dtype != 1) { fprintf(stderr, "missing i32 input %s\n", n); exit(3); }
  return it->second.i;
}

struct Dev {
  CUdeviceptr p = 0;
  size_t bytes = 0;
};

Dev up_f(const std::vector<double>& v) {
  Dev d; d.bytes = v.size() * 8;
  CK(cuMemAlloc(&d.p, d.bytes ? d.bytes : 8));
  if (d.bytes) CK(cuMemcpyHtoD(d.p, v.data(), d.bytes));
  return d;
}
Dev up_i(const std::vector<int32_t>& v) {
  Dev d; d.bytes = v.size() * 4;
  CK(cuMemAlloc(&d.p, d.bytes ? d.bytes : 8));
  if (d.bytes) CK(cuMemcpyHtoD(d.p, v.data(), d.bytes));
  return d;
}
Dev alloc(size_t bytes) {
  Dev d; d.bytes = bytes;
  CK(cuMemAlloc(&d.p, bytes ? bytes : 8));
  CK(cuMemsetD8(d.p, 0, bytes ? bytes : 8));
  return d;
}
std::vector<double> down_f(CUdeviceptr p, size_t n) {
  std::vector<double> v(n);
  if (n) CK(cuMemcpyDtoH(v.data(), p, n * 8));
  return v;
}
std::vector<int32_t> down_i(CUdeviceptr p, size_t n) {
  std::vector<int32_t> v(n);
  if (n) CK(cuMemcpyDtoH(v.data(), p, n * 4));
  return v;
}

CUmodule g_mod;
CUfunction fn(const char* mangled) {
  CUfunction f;
  CK(cuModuleGetFunction(&f, g_mod, mangled));
  return f;
}
void launch(CUfunction f, unsigned grid, unsigned block, unsigned smem, void** args) {
  CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, 0, args, nullptr));
}
unsigned blocks(long n) { return (unsigned)((n + 1023) / 1024 > 0 ? (n + 1023) / 1024 : 1); }

void put_f(const char* n, const std::vector<double>& v) { Arr a; a.dtype = 0; a.f = v; g_out[n] = a; }
void put_i(const char* n, const std::vector<int32_t>& v) { Arr a; a.dtype = 1; a.i = v; g_out[n] = a; }

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) { fprintf(stderr, "usage: ref_harness <cubin> <in.bin> <out.bin>\n"); return 1; }
  if (!read_file(argv[2])) { fprintf(stderr, "cannot read %s\n", argv[2]); return 1; }
  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxSetCurrent(ctx));
  CK(cuModuleLoad(&g_mod, argv[1]));

  const auto& dims = I("dims");  // B, K, G, N
  const int B = dims[0], K = dims[1], G = dims[2], N = dims[3];
  const auto& nb = I("n_b");
  {
    CUdeviceptr sym; size_t sz;
    CK(cuModuleGetGlobal(&sym, &sz, g_mod, "d_n_b"));
    CK(cuMemcpyHtoD(sym, nb.data(), 4 * B));
  }
  std::vector<int> off(B + 1, 0);
  for (int b = 0; b < B; ++b) off[b + 1] = off[b] + nb[b];

  Dev dY = up_i(I("Y")), dX = up_i(I("X")), dZ = up_i(I("Z")), dW = up_i(I("W")), dWp = up_i(I("W_prop"));
  Dev da = up_f(F("alpha")), dap = up_f(F("alpha_prop")), db = up_f(F("beta")), dbp = up_f(F("beta_prop"));
  Dev dn = up_f(F("nu")), dnp = up_f(F("nu_prop")), dd = up_f(F("delta")), ddp = up_f(F("delta_prop"));
  Dev dp = up_f(F("phi")), dpp = up_f(F("phi_prop")), dg = up_f(F("gamma")), dgp = up_f(F("gamma_prop"));
  Dev dpi = up_f(F("pi"));
  Dev tmp = alloc((size_t)N * G * 8);
  Dev tmpi = alloc((size_t)(N > 4096 ? N : 4096) * 4);

  // ---- alpha: temp[i] for every gene g ------------------------------------
  {
    CUfunction f = fn("_Z15fill_prop_alphaPdS_S_S_S_S_PiS0_S_iiii");
    std::vector<double> out;
    for (int g = 0; g < G; ++g) {
      int gg = g, BB = B, NN = N, GG = G;
      void* args[] = {&dap.p, &da.p, &db.p, &dn.p, &dd.p, &dp.p, &dW.p, &dX.p, &tmp.p, &gg, &BB, &NN, &GG};
      launch(f, blocks(N), 1024, 0, args);
      auto v = down_f(tmp.p, N);
      out.insert(out.end(), v.begin(), v.end());
    }
    put_f("alpha_terms", out);  // [g][i]
  }
  // ---- beta: temp[i] for every (k >= 1, g) --------------------------------
  {
    CUfunction f = fn("_Z14fill_prop_betaPdS_S_S_S_S_PiS0_S_iiii");
    std::vector<double> out;
    for (int k = 1; k < K; ++k)
      for (int g = 0; g < G; ++g) {
        int gg = g, kk = k, NN = N, GG = G;
        void* args[] = {&dbp.p, &db.p, &da.p, &dn.p, &dd.p, &dp.p, &dW.p, &dX.p, &tmp.p, &gg, &kk, &NN, &GG};
        launch(f, blocks(N), 1024, 0, args);
        auto v = down_f(tmp.p, N);
        out.insert(out.end(), v.begin(), v.end());
      }
    put_f("beta_terms", out);  // [k-1][g][i]
  }
  // ---- nu: temp[i within batch] for every (b >= 1, g) ---------------------
  {
    CUfunction f = fn("_Z12fill_prop_nuPdS_S_S_S_S_PiS0_S_iiii");
    std::vector<double> out;
    for (int b = 1; b < B; ++b)
      for (int g = 0; g < G; ++g) {
        CUdeviceptr d_delta = dd.p + 8ull * off[b], d_W = dW.p + 4ull * off[b], d_X = dX.p + 4ull * off[b] * G;
        int bb = b, gg = g, GG = G, n = nb[b];
        void* args[] = {&dnp.p, &dn.p, &da.p, &db.p, &d_delta, &dp.p, &d_W, &d_X, &tmp.p, &bb, &gg, &GG, &n};
        launch(f, blocks(n), 1024, 0, args);
        auto v = down_f(tmp.p, n);
        out.insert(out.end(), v.begin(), v.end());
      }
    put_f("nu_terms", out);  // [b-1][g][i - off_b]
  }
  // ---- delta: temp[g] for every cell i ------------------------------------
  {
    CUfunction f = fn("_Z15fill_prop_deltaPdS_S_S_S_S_PiS0_S_ii");
    std::vector<double> out;
    for (int i = 0; i < N; ++i) {
      int ii = i, GG = G;
      void* args[] = {&ddp.p, &dd.p, &da.p, &db.p, &dn.p, &dp.p, &dW.p, &dX.p, &tmp.p, &ii, &GG};
      launch(f, blocks(G), 1024, 0, args);
      auto v = down_f(tmp.p, G);
      out.insert(out.end(), v.begin(), v.end());
    }
    put_f("delta_terms", out);  // [i][g]
  }
  // ---- phi: temp[i within batch] for every (b, g) -------------------------
  {
    CUfunction f = fn("_Z13fill_prop_phiPdS_S_S_S_S_PiS0_S_ii");
    std::vector<double> out;
    for (int b = 0; b < B; ++b)
      for (int g = 0; g < G; ++g) {
        const int bg = b * G + g;
        CUdeviceptr pp = dpp.p + 8ull * bg, po = dp.p + 8ull * bg, a = da.p + 8ull * g, bt = db.p + 8ull * g;
        CUdeviceptr nu = dn.p + 8ull * bg, de = dd.p + 8ull * off[b], w = dW.p + 4ull * off[b];
        CUdeviceptr x = dX.p + 4ull * ((size_t)off[b] * G + g);
        int bb = b, GG = G;
        void* args[] = {&pp, &po, &a, &bt, &nu, &de, &w, &x, &tmp.p, &bb, &GG};
        launch(f, blocks(nb[b]), 1024, 0, args);
        auto v = down_f(tmp.p, nb[b]);
        out.insert(out.end(), v.begin(), v.end());
      }
    put_f("phi_terms", out);  // [b][g][i - off_b]
  }
  // ---- W: temp[g] for every cell i (proposal W_prop) ----------------------
  {
    CUfunction f = fn("_Z11fill_prop_WPiS_PdS0_S0_S0_S0_S_S0_ii");
    std::vector<double> out;
    for (int i = 0; i < N; ++i) {
      int ii = i, GG = G;
      void* args[] = {&dWp.p, &dW.p, &da.p, &db.p, &dn.p, &dd.p, &dp.p, &dX.p, &tmp.p, &ii, &GG};
      launch(f, blocks(G), 1024, 0, args);
      auto v = down_f(tmp.p, G);
      out.insert(out.end(), v.begin(), v.end());
    }
    put_f("W_terms", out);  // [i][g]
  }
  // ---- gamma0 / gamma1: temp[pos within batch] for every b ----------------
  {
    CUfunction f0 = fn("_Z16fill_prop_gamma0PdS_PiS0_S_iii");
    CUfunction f1 = fn("_Z16fill_prop_gamma1PdS_PiS0_S_iii");
    std::vector<double> o0, o1;
    for (int b = 0; b < B; ++b) {
      CUdeviceptr z = dZ.p + 4ull * off[b] * G, x = dX.p + 4ull * off[b] * G;
      int bb = b, BB = B, bound = nb[b] * G;
      void* args[] = {&dgp.p, &dg.p, &z, &x, &tmp.p, &bb, &BB, &bound};
      launch(f0, blocks(bound), 1024, 0, args);
      auto v = down_f(tmp.p, bound);
      o0.insert(o0.end(), v.begin(), v.end());
      launch(f1, blocks(bound), 1024, 0, args);
      v = down_f(tmp.p, bound);
      o1.insert(o1.end(), v.begin(), v.end());
    }
    put_f("gamma0_terms", o0);
    put_f("gamma1_terms", o1);
  }
  // ---- BIC fills ----------------------------------------------------------
  {
    CUfunction f1 = fn("_Z21fill_log_likelihood_1PdS_S_S_S_S_S_PiS_i");
    CUfunction f2 = fn("_Z21fill_log_likelihood_2PdS_S_ii");
    std::vector<double> ll1;          // [i][k][g]
    std::vector<double> part((size_t)K * N, 0.0);  // [k][i]
    for (int b = 0; b < B; ++b)
      for (int i = off[b]; i < off[b + 1]; ++i)
        for (int k = 0; k < K; ++k) {
          CUdeviceptr bt = db.p + 8ull * k * G, nu = dn.p + 8ull * b * G, de = dd.p + 8ull * i;
          CUdeviceptr g0 = dg.p + 8ull * b, g1 = dg.p + 8ull * (B + b), ph = dp.p + 8ull * b * G;
          CUdeviceptr y = dY.p + 4ull * i * G;
          int GG = G;
          void* args[] = {&da.p, &bt, &nu, &de, &g0, &g1, &ph, &y, &tmp.p, &GG};
          launch(f1, blocks(G), 1024, 0, args);
          auto v = down_f(tmp.p, G);
          double s = 0.0;
          for (double t : v) s += t;
          part[(size_t)k * N + i] = s;
          ll1.insert(ll1.end(), v.begin(), v.end());
        }
    put_f("ll1_terms", ll1);
    Dev dpart = up_f(part);
    int NN = N, KK = K;
    void* args[] = {&dpi.p, &dpart.p, &tmp.p, &NN, &KK};
    launch(f2, blocks(N), 1024, 0, args);
    put_f("ll2_terms", down_f(tmp.p, N));
    put_f("ll_partial", part);
  }
  // ---- initialisation: delta from library sizes, raw means, nu/phi, pi ----
  {
    // library sizes with the reference's own block sum
    CUfunction fsum = fn("_Z10sum_on_gpuIiEvPT_S1_i");
    Dev lib = alloc((size_t)N * 4);
    for (int i = 0; i < N; ++i) {
      CUdeviceptr y = dY.p + 4ull * i * G, o = lib.p + 4ull * i;
      int GG = G;
      void* args[] = {&y, &o, &GG};
      launch(fsum, 1, 1024, 1024 * 4, args);
    }
    put_i("libsize", down_i(lib.p, N));
    CUfunction fpi = fn("_Z8first_piPdii");
    Dev pi0 = alloc((size_t)B * K * 8);
    {
      int KK = K, bound = B * K;
      void* args[] = {&pi0.p, &KK, &bound};
      launch(fpi, 1, 1024, 0, args);
    }
    put_f("init_pi", down_f(pi0.p, (size_t)B * K));
    // first_delta_W needs curand states; seed them with the reference kernel
    const size_t state_bytes = 64;  // >= sizeof(curandStateXORWOW) (48 bytes)
    Dev states = alloc((size_t)N * state_bytes);
    {
      CUfunction fini = fn("_Z17initialize_curandiP17curandStateXORWOWi");
      int seed = 13579, len = N;
      void* args[] = {&seed, &states.p, &len};
      launch(fini, blocks(N), 1024, 0, args);
    }
    Dev dW0 = alloc((size_t)N * 4), dd0 = alloc((size_t)N * 8);
    {
      CUfunction fdw = fn("_Z13first_delta_WP17curandStateXORWOWPdPiS1_S2_ii");
      int NN = N, KK = K;
      void* args[] = {&states.p, &pi0.p, &lib.p, &dd0.p, &dW0.p, &NN, &KK};
      launch(fdw, blocks(N), 1024, 0, args);
    }
    put_i("init_W", down_i(dW0.p, N));
    put_f("init_delta", down_f(dd0.p, N));
    CUfunction fraw = fn("_Z14fill_raw_meansPiPdS_S0_S_iiii");
    CUfunction fsel = fn("_Z21selective_mean_on_gpuPdS_Pii");
    Dev raw = alloc((size_t)B * K * G * 8), cnt = alloc(8);
    for (int b = 0; b < B; ++b)
      for (int k = 0; k < K; ++k)
        for (int g = 0; g < G; ++g) {
          CUdeviceptr y = dY.p + 4ull * off[b] * G, de = dd0.p + 8ull * off[b], w = dW0.p + 4ull * off[b];
          int kk = k, gg = g, GG = G, n = nb[b];
          void* a1[] = {&y, &de, &w, &tmp.p, &tmpi.p, &kk, &gg, &GG, &n};
          launch(fraw, blocks(n), 1024, 0, a1);
          void* a2[] = {&tmpi.p, &cnt.p, &n};
          launch(fsum, 1, 1024, 1024 * 4, a2);
          CUdeviceptr o = raw.p + 8ull * ((size_t)(b * K + k) * G + g);
          void* a3[] = {&tmp.p, &o, &cnt.p, &n};
          launch(fsel, 1, 1024, 1024 * 8, a3);
        }
    put_f("init_raw_means", down_f(raw.p, (size_t)B * K * G));
    CUfunction fnp = fn("_Z12first_nu_phiPdS_S_iii");
    Dev nu0 = alloc((size_t)B * G * 8), phi0 = alloc((size_t)B * G * 8);
    {
      int GG = G, KK = K, bound = B * G;
      void* args[] = {&raw.p, &nu0.p, &phi0.p, &GG, &KK, &bound};
      launch(fnp, blocks(B * G), 1024, 0, args);
    }
    put_f("init_nu", down_f(nu0.p, (size_t)B * G));
    put_f("init_phi", down_f(phi0.p, (size_t)B * G));
    CUfunction fmn = fn("_Z10fill_mu_nuPiPdS0_ii");
    CUfunction fmean = fn("_Z11mean_on_gpuPdS_i");
    Dev mean = alloc((size_t)B * 8);
    for (int b = 0; b < B; ++b) {
      CUdeviceptr y = dY.p + 4ull * off[b] * G, de = dd0.p + 8ull * off[b];
      int GG = G, bound = nb[b] * G;
      void* a1[] = {&y, &de, &tmp.p, &GG, &bound};
      launch(fmn, blocks(bound), 1024, 0, a1);
      CUdeviceptr o = mean.p + 8ull * b;
      void* a2[] = {&tmp.p, &o, &bound};
      launch(fmean, 1, 1024, 1024 * 8, a2);
    }
    put_f("init_batch_means", down_f(mean.p, B));
  }
  // ---- posterior mode of W from per-(k, i) counts -------------------------
  {
    CUfunction fmode = fn("_Z11mode_on_gpuPiS_ii");
    Dev counts = up_i(I("mode_counts"));  // [k][i]
    Dev post = alloc((size_t)N * 4);
    int NN = N, KK = K;
    void* args[] = {&counts.p, &post.p, &NN, &KK};
    launch(fmode, blocks(N), 1024, 0, args);
    put_i("mode_W", down_i(post.p, N));
  }
  CK(cuCtxSynchronize());
  if (!write_file(argv[3])) { fprintf(stderr, "cannot write %s\n", argv[3]); return 1; }
  printf("ref_harness: wrote %zu arrays\n", g_out.size());
  return 0;
}
