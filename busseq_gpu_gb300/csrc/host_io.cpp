// Count-file parser and output writers with the reference's formats.
//
// Reading: BUSseq_gpu.cu:1143-1161 reads N*G integers with fscanf("%d"); here
// the whole file is read once and parsed by every host thread (two passes:
// count the tokens of each slice, then parse each slice into its place).
// Writing: BUSseq_gpu.cu:1610-2018 -- tab-separated rows, "%lf" for floating
// point, "%d" for integers; rows are formatted in parallel and written in order.
//
// Binary counts (not in the reference): a file that starts with the 8 bytes
// "BUSSEQY1" holds int64 N, int64 G and then N*G int32 counts, row-major,
// little-endian.  busseq_read_counts recognises it by that magic and reads it
// with one pread per host thread; busseq_write_counts_binary writes it (a text
// count file converted once loads without parsing afterwards).
//
// Compressed counts (not in the reference): a gzip file (magic 1f 8b) of either
// format is inflated into memory and then parsed as above.  zlib is loaded at
// run time (libz.so.1), so the build does not depend on its headers.
#include "busseq_gb300.h"

#include <dlfcn.h>
#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <functional>
#include <string>
#include <thread>
#include <vector>

extern "C" int busseq_internal_set_error(int code, const char* msg);

namespace {

int nthreads() {
  const unsigned n = std::thread::hardware_concurrency();
  return n == 0 ? 1 : (int)std::min(n, 64u);
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Parses [b, e): counts tokens (out == NULL) or stores them.  Returns the
// number of tokens, or -1 (and *bad = position) on a malformed token.
int64_t parse_slice(const char* b, const char* e, int32_t* out, int64_t cap, const char** bad) {
  int64_t n = 0;
  const char* p = b;
  while (p < e) {
    while (p < e && is_space(*p)) ++p;
    if (p >= e) break;
    bool neg = false;
    if (*p == '-' || *p == '+') { neg = *p == '-'; ++p; }
    if (p >= e || *p < '0' || *p > '9') { *bad = p; return -1; }
    int64_t v = 0;
    while (p < e && *p >= '0' && *p <= '9') {
      v = v * 10 + (*p - '0');
      if (v > 2147483647LL) { *bad = p; return -1; }
      ++p;
    }
    if (p < e && !is_space(*p)) { *bad = p; return -1; }
    if (out) {
      if (n >= cap) { *bad = p; return -1; }
      out[n] = (int32_t)(neg ? -v : v);
    }
    ++n;
  }
  return n;
}

struct Table {
  int64_t rows = 0, cols = 0;
  // formats cell (r, c) into buf, returns length
  std::function<int(int64_t, int64_t, char*)> cell;
  bool trailing_tab_no_newline = false;  // the _post_p.txt layout
};

int fmt_int(int64_t v, char* buf) {
  char tmp[24];
  int n = 0;
  const bool neg = v < 0;
  uint64_t u = neg ? (uint64_t)(-v) : (uint64_t)v;
  do { tmp[n++] = (char)('0' + u % 10); u /= 10; } while (u);
  int k = 0;
  if (neg) buf[k++] = '-';
  while (n) buf[k++] = tmp[--n];
  return k;
}

int fmt_lf(double v, char* buf) { return snprintf(buf, 64, "%f", v); }

int write_table(const std::string& path, const Table& t) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return busseq_internal_set_error(BUSSEQ_ERR_IO, ("cannot open " + path + " for writing").c_str());
  const int nt = nthreads();
  const int64_t rows_per_task = std::max<int64_t>(1, (int64_t)(1 << 20) / std::max<int64_t>(1, t.cols));
  std::vector<std::string> bufs(nt);
  int64_t r0 = 0;
  bool ok = true;
  while (r0 < t.rows && ok) {
    std::vector<std::thread> th;
    for (int w = 0; w < nt; ++w) {
      const int64_t a = r0 + w * rows_per_task, b = std::min(t.rows, a + rows_per_task);
      bufs[w].clear();
      if (a >= b) continue;
      th.emplace_back([&, w, a, b]() {
        std::string& s = bufs[w];
        s.reserve((size_t)((b - a) * t.cols * 10));
        char cell[80];
        for (int64_t r = a; r < b; ++r) {
          for (int64_t c = 0; c < t.cols; ++c) {
            const int n = t.cell(r, c, cell);
            s.append(cell, (size_t)n);
            if (t.trailing_tab_no_newline) s.push_back('\t');
            else s.push_back(c + 1 < t.cols ? '\t' : '\n');
          }
        }
      });
    }
    for (auto& x : th) x.join();
    for (int w = 0; w < nt; ++w)
      if (!bufs[w].empty() && fwrite(bufs[w].data(), 1, bufs[w].size(), f) != bufs[w].size()) ok = false;
    r0 += (int64_t)nt * rows_per_task;
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) return busseq_internal_set_error(BUSSEQ_ERR_IO, ("write failed: " + path).c_str());
  return BUSSEQ_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

constexpr char kBinMagic[8] = {'B', 'U', 'S', 'S', 'E', 'Q', 'Y', '1'};
constexpr int64_t kBinHeader = 24;

bool host_little_endian() {
  const uint32_t one = 1;
  unsigned char c;
  memcpy(&c, &one, 1);
  return c == 1;
}

// Reads the N*G int32 payload of a binary count file, one pread per thread.
int read_counts_binary(int fd, const char* path, int64_t N, int64_t G, int64_t file_size, int32_t* out) {
  int64_t hdr[2];
  if (pread(fd, hdr, sizeof hdr, 8) != (ssize_t)sizeof hdr)
    return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("short header in ") + path).c_str());
  if (hdr[0] != N || hdr[1] != G) {
    char msg[240];
    snprintf(msg, sizeof(msg), "binary count file %s holds N=%lld G=%lld, expected N=%lld G=%lld", path,
             (long long)hdr[0], (long long)hdr[1], (long long)N, (long long)G);
    return busseq_internal_set_error(BUSSEQ_ERR_IO, msg);
  }
  const int64_t bytes = N * G * 4;
  if (file_size != kBinHeader + bytes)
    return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("binary count file of the wrong size: ") + path).c_str());
  const int nt = std::max(1, std::min(nthreads(), (int)(bytes >> 24) + 1));
  std::vector<int> ok(nt, 1);
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) {
    th.emplace_back([&, t]() {
      int64_t a = (bytes / nt) * t, b = t + 1 == nt ? bytes : (bytes / nt) * (t + 1);
      a &= ~int64_t(3);
      if (t + 1 != nt) b &= ~int64_t(3);
      char* dst = reinterpret_cast<char*>(out);
      while (a < b) {
        const ssize_t r = pread(fd, dst + a, (size_t)std::min<int64_t>(b - a, 1 << 30), kBinHeader + a);
        if (r <= 0) { ok[t] = 0; return; }
        a += r;
      }
    });
  }
  for (auto& x : th) x.join();
  for (int t = 0; t < nt; ++t)
    if (!ok[t]) return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("short read of ") + path).c_str());
  return BUSSEQ_OK;
}

// The same payload from a buffer holding the whole (inflated) file.
int binary_from_buffer(const char* buf, int64_t size, const char* path, int64_t N, int64_t G, int32_t* out) {
  int64_t hdr[2];
  memcpy(hdr, buf + 8, sizeof hdr);
  if (hdr[0] != N || hdr[1] != G) {
    char msg[240];
    snprintf(msg, sizeof(msg), "binary count file %s holds N=%lld G=%lld, expected N=%lld G=%lld", path,
             (long long)hdr[0], (long long)hdr[1], (long long)N, (long long)G);
    return busseq_internal_set_error(BUSSEQ_ERR_IO, msg);
  }
  if (size != kBinHeader + N * G * 4)
    return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("binary count file of the wrong size: ") + path).c_str());
  memcpy(out, buf + kBinHeader, (size_t)(N * G * 4));
  return BUSSEQ_OK;
}

// N*G whitespace-separated integers from a buffer, parsed by every host thread
// (two passes: count the tokens of each slice, then parse each into place).
int text_from_buffer(const char* base, int64_t sz, const char* path, int64_t N, int64_t G, int32_t* out) {
  const int nt = std::max(1, std::min(nthreads(), (int)(sz / (1 << 16)) + 1));
  std::vector<const char*> starts(nt + 1);
  const char* end = base + sz;
  starts[0] = base;
  starts[nt] = end;
  for (int t = 1; t < nt; ++t) {
    const char* p = base + (size_t)sz * t / nt;
    if (p < starts[t - 1]) p = starts[t - 1];
    while (p < end && !is_space(*p)) ++p;  // never split a token
    starts[t] = p;
  }
  std::vector<int64_t> cnt(nt, 0);
  std::vector<const char*> bad(nt, nullptr);
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t]() { cnt[t] = parse_slice(starts[t], starts[t + 1], nullptr, 0, &bad[t]); });
    for (auto& x : th) x.join();
  }
  int64_t total = 0;
  for (int t = 0; t < nt; ++t) {
    if (cnt[t] < 0) {
      char msg[160];
      snprintf(msg, sizeof(msg), "malformed count at byte %lld of %s", (long long)(bad[t] - base), path);
      return busseq_internal_set_error(BUSSEQ_ERR_IO, msg);
    }
    total += cnt[t];
  }
  if (total != N * G) {
    char msg[200];
    snprintf(msg, sizeof(msg), "count file %s holds %lld numbers, expected N*G = %lld", path, (long long)total,
             (long long)(N * G));
    return busseq_internal_set_error(BUSSEQ_ERR_IO, msg);
  }
  std::vector<int64_t> pre(nt + 1, 0);
  for (int t = 0; t < nt; ++t) pre[t + 1] = pre[t] + cnt[t];
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t]() { parse_slice(starts[t], starts[t + 1], out + pre[t], cnt[t], &bad[t]); });
    for (auto& x : th) x.join();
  }
  return BUSSEQ_OK;
}

// A whole gzip file inflated into `buf` through zlib's gz interface, loaded
// from libz.so.1 at run time.
int inflate_gzip(const char* path, std::vector<char>& buf) {
  using gz_open_t = void* (*)(const char*, const char*);
  using gz_buffer_t = int (*)(void*, unsigned);
  using gz_read_t = int (*)(void*, void*, unsigned);
  using gz_close_t = int (*)(void*);
  void* lib = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!lib) return busseq_internal_set_error(BUSSEQ_ERR_IO, "compressed count files need zlib (libz.so.1)");
  const auto gz_open = reinterpret_cast<gz_open_t>(dlsym(lib, "gzopen"));
  const auto gz_buffer = reinterpret_cast<gz_buffer_t>(dlsym(lib, "gzbuffer"));
  const auto gz_read = reinterpret_cast<gz_read_t>(dlsym(lib, "gzread"));
  const auto gz_close = reinterpret_cast<gz_close_t>(dlsym(lib, "gzclose"));
  int r = BUSSEQ_OK;
  if (!gz_open || !gz_read || !gz_close) {
    r = busseq_internal_set_error(BUSSEQ_ERR_IO, "libz.so.1 lacks the gz interface");
  } else if (void* gz = gz_open(path, "rb")) {
    if (gz_buffer) gz_buffer(gz, 1u << 20);
    constexpr size_t kChunk = size_t(1) << 26;
    size_t have = 0;
    for (;;) {
      buf.resize(have + kChunk);
      const int got = gz_read(gz, buf.data() + have, (unsigned)kChunk);
      if (got < 0) {
        r = busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("corrupt compressed count file ") + path).c_str());
        break;
      }
      have += (size_t)got;
      if (got == 0) break;
    }
    buf.resize(r == BUSSEQ_OK ? have : 0);
    gz_close(gz);
  } else {
    r = busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("cannot open count file ") + path).c_str());
  }
  dlclose(lib);
  return r;
}

}  // namespace

extern "C" {

int busseq_write_counts_binary(const char* path, int64_t N, int64_t G, const int32_t* Y) {
  if (!path || !Y || N <= 0 || G <= 0) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "bad arguments");
  if (!host_little_endian()) return busseq_internal_set_error(BUSSEQ_ERR_IO, "binary counts need a little-endian host");
  FILE* f = fopen(path, "wb");
  if (!f) return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("cannot open ") + path + " for writing").c_str());
  const int64_t hdr[2] = {N, G};
  bool ok = fwrite(kBinMagic, 1, 8, f) == 8 && fwrite(hdr, 8, 2, f) == 2;
  const size_t n = (size_t)(N * G);
  for (size_t o = 0; ok && o < n;) {
    const size_t c = std::min<size_t>(n - o, (size_t)1 << 26);
    ok = fwrite(Y + o, 4, c, f) == c;
    o += c;
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("write failed: ") + path).c_str());
  return BUSSEQ_OK;
}

int busseq_read_counts(const char* path, int64_t N, int64_t G, int32_t* out) {
  if (!path || !out || N <= 0 || G <= 0) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "bad arguments");
  auto no_negative = [&]() {
    for (int64_t i = 0; i < N * G; ++i)
      if (out[i] < 0) return busseq_internal_set_error(BUSSEQ_ERR_IO, "negative count in the count file");
    return (int)BUSSEQ_OK;
  };
  {
    const int fd = open(path, O_RDONLY);
    if (fd >= 0) {
      char magic[8];
      const off_t size = lseek(fd, 0, SEEK_END);
      const bool head = size >= 2 && pread(fd, magic, 8, 0) >= 2;
      const bool gz = head && (unsigned char)magic[0] == 0x1f && (unsigned char)magic[1] == 0x8b;
      if (gz) {
        close(fd);
        std::vector<char> buf;
        int r = inflate_gzip(path, buf);
        if (r != BUSSEQ_OK) return r;
        const int64_t n = (int64_t)buf.size();
        if (n >= kBinHeader && memcmp(buf.data(), kBinMagic, 8) == 0) {
          r = host_little_endian() ? binary_from_buffer(buf.data(), n, path, N, G, out)
                                   : busseq_internal_set_error(BUSSEQ_ERR_IO, "binary counts need a little-endian host");
        } else {
          r = text_from_buffer(buf.data(), n, path, N, G, out);
        }
        return r != BUSSEQ_OK ? r : no_negative();
      }
      const bool bin = size >= kBinHeader && head && memcmp(magic, kBinMagic, 8) == 0;
      int r = BUSSEQ_OK;
      if (bin) {
        r = host_little_endian() ? read_counts_binary(fd, path, N, G, (int64_t)size, out)
                                 : busseq_internal_set_error(BUSSEQ_ERR_IO, "binary counts need a little-endian host");
      }
      close(fd);
      if (bin) return r != BUSSEQ_OK ? r : no_negative();
    }
  }
  FILE* f = fopen(path, "rb");
  if (!f) return busseq_internal_set_error(BUSSEQ_ERR_IO, (std::string("cannot open count file ") + path).c_str());
  fseek(f, 0, SEEK_END);
  const long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::vector<char> buf((size_t)std::max(0L, sz));
  const size_t got = sz > 0 ? fread(buf.data(), 1, (size_t)sz, f) : 0;
  fclose(f);
  if ((long)got != sz) return busseq_internal_set_error(BUSSEQ_ERR_IO, "short read of the count file");
  const int r = text_from_buffer(buf.data(), (int64_t)sz, path, N, G, out);
  return r != BUSSEQ_OK ? r : no_negative();
}

int busseq_internal_dims(busseq_handle* h, int32_t* B, int32_t* K, int64_t* G, int64_t* N, int32_t* n_kept,
                         int32_t* kept_draws);
int busseq_internal_format_xz(busseq_handle* h, int which, char** buf, int64_t* len);
int busseq_internal_format_preserved(busseq_handle* h, int which, char** buf, int64_t* len);
int busseq_internal_format_zx_summary(busseq_handle* h, int which, char** buf, int64_t* len);

int busseq_write_outputs(busseq_handle* h, const char* prefix, int32_t print_preserved) {
  if (!h || !prefix) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "NULL argument");
  int32_t B, K, nk, kd;
  int64_t G, N;
  int r = busseq_internal_dims(h, &B, &K, &G, &N, &nk, &kd);
  if (r) return r;
  std::vector<int32_t> W(N);
  std::vector<double> gamma(2 * B), alpha(G), L((size_t)std::max(1, K - 1) * G), beta((size_t)K * G), ptau(2),
      nu((size_t)B * G), delta(N), phi((size_t)B * G), pi((size_t)B * K);
  busseq_estimates e{};
  e.gamma = gamma.data(); e.alpha = alpha.data(); e.L = L.data();
  e.beta = beta.data(); e.p_tau0 = ptau.data(); e.nu = nu.data(); e.delta = delta.data();
  e.phi = phi.data(); e.W = W.data(); e.pi = pi.data();
  if ((r = busseq_get_estimates(h, &e))) return r;
  const std::string pre(prefix);
  auto ints = [](const std::vector<int32_t>& v, int64_t cols) {
    Table t;
    t.rows = (int64_t)v.size() / cols;
    t.cols = cols;
    t.cell = [&v, cols](int64_t r, int64_t c, char* b) { return fmt_int(v[r * cols + c], b); };
    return t;
  };
  auto dbls = [](const double* v, int64_t rows, int64_t cols) {
    Table t;
    t.rows = rows;
    t.cols = cols;
    t.cell = [v, cols](int64_t r, int64_t c, char* b) { return fmt_lf(v[r * cols + c], b); };
    return t;
  };
  // _post_Z, _post_X: last sweep's state (BUSseq_gpu.cu:1613-1645)
  // the N x G tables of Z and X are formatted on the device
  for (int which = 1; which >= 0; --which) {
    const std::string path = pre + (which ? "_post_Z.txt" : "_post_X.txt");
    char* txt = nullptr;
    int64_t len = 0;
    if ((r = busseq_internal_format_xz(h, which, &txt, &len))) return r;
    FILE* f = fopen(path.c_str(), "wb");
    const bool ok = f && (len == 0 || fwrite(txt, 1, (size_t)len, f) == (size_t)len);
    const bool closed = f && fclose(f) == 0;
    free(txt);
    if (!ok || !closed) return busseq_internal_set_error(BUSSEQ_ERR_IO, ("write failed: " + path).c_str());
  }
  if ((r = write_table(pre + "_post_gamma.txt", dbls(gamma.data(), 2, B)))) return r;
  if ((r = write_table(pre + "_post_alpha.txt", dbls(alpha.data(), G, 1)))) return r;
  if ((r = write_table(pre + "_post_L.txt", dbls(L.data(), K - 1, G)))) return r;
  for (int64_t g = 0; g < G; ++g) beta[g] = 0.0;  // the first row is printed as literal zeros
  if ((r = write_table(pre + "_post_beta.txt", dbls(beta.data(), K, G)))) return r;
  {
    Table t = dbls(ptau.data(), 1, 2);
    t.trailing_tab_no_newline = true;  // "p\ttau0\t" without a newline (BUSseq_gpu.cu:1725-1727)
    if ((r = write_table(pre + "_post_p.txt", t))) return r;
  }
  for (int64_t g = 0; g < G; ++g) nu[g] = 0.0;
  if ((r = write_table(pre + "_post_nu.txt", dbls(nu.data(), B, G)))) return r;
  if ((r = write_table(pre + "_post_delta.txt", dbls(delta.data(), N, 1)))) return r;
  if ((r = write_table(pre + "_post_phi.txt", dbls(phi.data(), B, G)))) return r;
  if ((r = write_table(pre + "_post_W.txt", ints(W, 1)))) return r;
  if ((r = write_table(pre + "_post_pi.txt", dbls(pi.data(), B, K)))) return r;
  double bic = 0.0;
  if ((r = busseq_bic(h, &bic))) return r;
  if ((r = write_table(pre + "_BIC.txt", dbls(&bic, 1, 1)))) return r;
  if (!print_preserved) return BUSSEQ_OK;
  if (!kd || nk <= 0) return busseq_internal_set_error(BUSSEQ_ERR_STATE, "no kept draws to print (keep_draws off)");
  // the kept-draw tables are formatted on the device ("%f" exactly for the float
  // draws); a table holding a value outside the device formatter (|v| >= 2^43,
  // never expected) sends all of them to the host writer below
  {
    static const char* const names[10] = {"_preserved_gamma.txt", "_preserved_alpha.txt", "_preserved_L.txt",
                                          "_preserved_beta.txt",  "_preserved_p.txt",     "_preserved_nu.txt",
                                          "_preserved_delta.txt", "_preserved_phi.txt",   "_preserved_W.txt",
                                          "_preserved_pi.txt"};
    bool device_ok = true;
    for (int which = 0; which < 10 && device_ok; ++which) {
      char* txt = nullptr;
      int64_t len = 0;
      r = busseq_internal_format_preserved(h, which, &txt, &len);
      if (r == 1) {
        device_ok = false;
        break;
      }
      if (r) return r;
      const std::string path = pre + names[which];
      FILE* f = fopen(path.c_str(), "wb");
      const bool ok = f && (len == 0 || fwrite(txt, 1, (size_t)len, f) == (size_t)len);
      const bool closed = f && fclose(f) == 0;
      free(txt);
      if (!ok || !closed) return busseq_internal_set_error(BUSSEQ_ERR_IO, ("write failed: " + path).c_str());
    }
    if (device_ok) return BUSSEQ_OK;
  }
  const int64_t n = nk;
  std::vector<double> pg((size_t)2 * B * n), pa((size_t)G * n), pb((size_t)(K - 1) * G * n), pp((size_t)2 * n),
      pn((size_t)(B - 1) * G * n), pd((size_t)N * n), pf((size_t)B * G * n), ppi((size_t)B * K * n);
  std::vector<int32_t> pL((size_t)(K - 1) * G * n), pW((size_t)N * n);
  busseq_preserved p{};
  p.gamma = pg.data(); p.alpha = pa.data(); p.L = pL.data(); p.beta = pb.data(); p.p_tau0 = pp.data();
  p.nu = pn.data(); p.delta = pd.data(); p.phi = pf.data(); p.W = pW.data(); p.pi = ppi.data();
  if ((r = busseq_get_preserved(h, &p))) return r;
  if ((r = write_table(pre + "_preserved_gamma.txt", dbls(pg.data(), 2 * B, n)))) return r;
  if ((r = write_table(pre + "_preserved_alpha.txt", dbls(pa.data(), G, n)))) return r;
  if ((r = write_table(pre + "_preserved_L.txt", ints(pL, n)))) return r;
  if ((r = write_table(pre + "_preserved_beta.txt", dbls(pb.data(), (K - 1) * G, n)))) return r;
  if ((r = write_table(pre + "_preserved_p.txt", dbls(pp.data(), 2, n)))) return r;
  if ((r = write_table(pre + "_preserved_nu.txt", dbls(pn.data(), (B - 1) * G, n)))) return r;
  if ((r = write_table(pre + "_preserved_delta.txt", dbls(pd.data(), N, n)))) return r;
  if ((r = write_table(pre + "_preserved_phi.txt", dbls(pf.data(), B * G, n)))) return r;
  if ((r = write_table(pre + "_preserved_W.txt", ints(pW, n)))) return r;
  if ((r = write_table(pre + "_preserved_pi.txt", dbls(ppi.data(), B * K, n)))) return r;
  return BUSSEQ_OK;
}

int busseq_write_zx_summaries(busseq_handle* h, const char* prefix) {
  if (!h || !prefix) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "NULL argument");
  const std::string pre(prefix);
  for (int which = 0; which < 2; ++which) {
    const std::string path = pre + (which ? "_post_Z_prob.txt" : "_post_X_mean.txt");
    char* txt = nullptr;
    int64_t len = 0;
    int r = busseq_internal_format_zx_summary(h, which, &txt, &len);  // tables and text on the device
    if (r == 1) {  // a value outside the device formatter: format on the host
      int32_t B, K, nk, kd;
      int64_t G, N;
      if ((r = busseq_internal_dims(h, &B, &K, &G, &N, &nk, &kd))) return r;
      std::vector<float> xm((size_t)N * G), zp((size_t)N * G);
      if ((r = busseq_get_zx_summaries(h, xm.data(), zp.data()))) return r;
      const std::vector<float>& v = which ? zp : xm;
      Table t;
      t.rows = N;
      t.cols = G;
      t.cell = [&v, G](int64_t i, int64_t g, char* b) { return fmt_lf((double)v[i * G + g], b); };
      if ((r = write_table(path, t))) return r;
      continue;
    }
    if (r) return r;
    FILE* f = fopen(path.c_str(), "wb");
    const bool ok = f && (len == 0 || fwrite(txt, 1, (size_t)len, f) == (size_t)len);
    const bool closed = f && fclose(f) == 0;
    free(txt);
    if (!ok || !closed) return busseq_internal_set_error(BUSSEQ_ERR_IO, ("write failed: " + path).c_str());
  }
  return BUSSEQ_OK;
}

int busseq_write_corrected(busseq_handle* h, const char* prefix) {
  if (!h || !prefix) return busseq_internal_set_error(BUSSEQ_ERR_ARG, "NULL argument");
  const std::string path = std::string(prefix) + "_corrected_X.txt";
  char* txt = nullptr;
  int64_t len = 0;
  int r = busseq_internal_format_xz(h, 2, &txt, &len);  // counts and text on the device
  if (r) return r;
  FILE* f = fopen(path.c_str(), "wb");
  const bool ok = f && (len == 0 || fwrite(txt, 1, (size_t)len, f) == (size_t)len);
  const bool closed = f && fclose(f) == 0;
  free(txt);
  if (!ok || !closed) return busseq_internal_set_error(BUSSEQ_ERR_IO, ("write failed: " + path).c_str());
  return BUSSEQ_OK;
}

}  // extern "C"
