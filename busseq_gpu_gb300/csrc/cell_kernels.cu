// Cell passes (delta, W), the pi draw with the cell order, and the posterior
// accumulation of kept sweeps.
//
// Cell passes: one CTA per tile of <= CELL_TILE cells that share batch b and
// type k, 256 threads striding over genes with 128-bit loads; every decision
// is taken in the CTA (BUSseq_gpu.cu:739-778 for delta, :820-854 for W).
#include "kernels_common.cuh"

namespace bq {

// ---------------------------------------------------------------------------
// Cell passes: one CTA per tile of <= CELL_TILE cells of one (batch, type)
// ---------------------------------------------------------------------------
// Sums over the CTA of CELL_TILE per-thread float-float values; results in
// sh_out[r].  `sh` holds (blockDim.x / 32) * CELL_TILE pairs.
__device__ __forceinline__ void cell_reduce(FF (&acc)[CELL_TILE], FF* sh, FF* sh_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) {
    const FF v = ff_warp_sum(acc[r]);
    if (lane == 0) sh[warp * CELL_TILE + r] = v;
  }
  __syncthreads();
  if (threadIdx.x < CELL_TILE) {
    FF t = sh[threadIdx.x];
    for (int w = 1; w < nw; ++w) t = ff_add(t, sh[w * CELL_TILE + threadIdx.x]);
    sh_out[threadIdx.x] = t;
  }
  __syncthreads();
}

// Integer version of cell_reduce.
__device__ __forceinline__ void cell_reduce_i(long long (&acc)[CELL_TILE], long long* sh, long long* sh_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) {
    const long long v = i64_warp_sum(acc[r]);
    if (lane == 0) sh[warp * CELL_TILE + r] = v;
  }
  __syncthreads();
  if (threadIdx.x < CELL_TILE) {
    long long t = 0;
    for (int w = 0; w < nw; ++w) t += sh[w * CELL_TILE + threadIdx.x];
    sh_out[threadIdx.x] = t;
  }
  __syncthreads();
}

// X rows of a cell tile, streamed through shared memory: a ring of NST stages,
// each holding the tile's rows over WIDTH consecutive genes, filled by bulk
// asynchronous copies that warp 0 issues NST stages ahead of the compute (lane
// 0 arms the stage's barrier, lane r copies row r, so the warp that also
// computes spends little time on the copies).  Row starts are 16-byte aligned
// (Gp is a multiple of GENE_TILE) and every copy is a multiple of 16 bytes.
static_assert(CELL_TILE <= 32, "one lane of warp 0 per row of a tile");
template <int WIDTH, int NST>
struct XRowRing {
  int* buf;       // [NST][CELL_TILE][WIDTH]
  uint64_t* bar;  // [NST]
  const int* X;
  const int* rows;  // the tile's cell indices (shared memory)
  int64_t Gp;
  int len, n_steps;

  static constexpr int bytes() { return NST * CELL_TILE * WIDTH * (int)sizeof(int); }

  __device__ void init(int tid) {
    if (tid == 0) {
      for (int q = 0; q < NST; ++q) mbar_init(&bar[q], 1);
      mbar_init_fence();
    }
  }
  // Called by all of warp 0 (lane = its lane).
  __device__ void issue(int step, int lane) const {
    const int st = step % NST;
    const int64_t g0 = (int64_t)step * WIDTH;
    const uint32_t nb = (uint32_t)((Gp - g0 < WIDTH ? Gp - g0 : WIDTH) * (int64_t)sizeof(int));
    if (lane == 0) mbar_arrive_expect_tx(&bar[st], nb * (uint32_t)len);
    __syncwarp();
    if (lane < len)
      bulk_copy_g2s(buf + (st * CELL_TILE + lane) * WIDTH, X + (int64_t)rows[lane] * Gp + g0, nb, &bar[st]);
  }
  __device__ void prologue(int tid) const {
    if (tid < 32)
      for (int q = 0; q < NST && q < n_steps; ++q) issue(q, tid);
  }
  __device__ bool wait(int step) { return mbar_wait(&bar[step % NST], (uint32_t)((step / NST) & 1)); }
  __device__ const int* row(int step, int r) const { return buf + ((step % NST) * CELL_TILE + r) * WIDTH; }
  // After every thread finished reading stage `step`: refill it.
  __device__ void advance(int tid, int step) const {
    if (tid < 32 && step + NST < n_steps) {
      fence_proxy_async_smem();
      issue(step + NST, tid);
    }
  }
  // Failure at `step`: flag it and let the copies in flight land before the
  // CTA exits (bounded waits).
  __device__ void abandon(int tid, int step, int* err) {
    if (tid == 0) {
      atomicOr(err, ERR_COPY_TIMEOUT);
      const int issued = step + NST < n_steps ? step + NST : n_steps;
      for (int q = step; q < issued; ++q) wait(q);
    }
    __syncthreads();
  }
};

using DeltaRing = XRowRing<DELTA_WIDTH, X_STAGES>;
using WRing = XRowRing<W_WIDTH, X_STAGES>;
static_assert(DeltaRing::bytes() == DELTA_SMEM && WRing::bytes() == W_SMEM, "ring sizes");

__global__ void __launch_bounds__(CELL_THREADS, 4) k_delta(DevState s) {
  extern __shared__ __align__(128) int xbuf[];
  __shared__ __align__(8) uint64_t bar[X_STAGES];
  __shared__ FF sh[(CELL_THREADS / 32) * CELL_TILE];
  __shared__ long long shi[(CELL_THREADS / 32) * CELL_TILE];
  __shared__ FF sh_l[CELL_TILE];
  __shared__ long long sh_x[CELL_TILE];
  __shared__ int sh_i[CELL_TILE];
  __shared__ float sh_D[CELL_TILE], sh_c[CELL_TILE];
  const int4 t = s.ctile[blockIdx.x];
  const int b = t.x, k = t.y, start = t.z, len = t.w;
  if (len == 0) return;
  const int tid = threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp, G = s.G;
  DeltaRing ring{xbuf, bar, s.X, sh_i, Gp, len, (int)((Gp + DELTA_WIDTH - 1) / DELTA_WIDTH)};
  ring.init(tid);
  float cd = 0.0f;
  if (tid < CELL_TILE) {
    const int i = s.perm[start + (tid < len ? tid : 0)];
    sh_i[tid] = i;
    sh_D[tid] = s.Dexp[i];
    cd = tid < len ? expm1f(s.delta_p[i] - s.delta[i]) : 0.0f;
    sh_c[tid] = cd;
  }
  // every cell's |expm1(step)| <= 1/2: the terms by log1p_shift (one reciprocal)
  const bool fast = __syncthreads_and(fabsf(cd) <= 0.5f) != 0;
  ring.prologue(tid);
  float acc[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) acc[r] = 0.0f;
  int sxi[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) sxi[r] = 0;
  const float* Er = s.E + ((int64_t)b * s.K + k) * Gp;
  const float* Pr = s.phi + (int64_t)b * Gp;
  for (int step = 0; step < ring.n_steps; ++step) {
    const int64_t g2 = (int64_t)step * DELTA_WIDTH + tid * 2;
    const bool in = g2 < G;
    float2 e = make_float2(0.f, 0.f), ph = e;
    if (in) {
      e = *reinterpret_cast<const float2*>(Er + g2);
      ph = *reinterpret_cast<const float2*>(Pr + g2);
    }
    const bool two = g2 + 1 < G;
    const bool ok = ring.wait(step);
    if (in) {
#pragma unroll
      for (int r = 0; r < CELL_TILE; ++r) {
        if (r < len) {
          const int2 xv = *reinterpret_cast<const int2*>(ring.row(step, r) + tid * 2);
          const float D = sh_D[r], c = sh_c[r];
          const float mu0 = e.x * D, mu1 = e.y * D;
          const float l0 = fast ? log1p_shift(c * mu0, fmaf(2.0f + c, mu0, 2.0f * ph.x))
                                : log1p_near0(c * fast_div(mu0, ph.x + mu0));
          float a = (ph.x + (float)xv.x) * l0;
          int sxv = xv.x;
          if (two) {
            const float l1 = fast ? log1p_shift(c * mu1, fmaf(2.0f + c, mu1, 2.0f * ph.y))
                                  : log1p_near0(c * fast_div(mu1, ph.y + mu1));
            a = fmaf(ph.y + (float)xv.y, l1, a);
            sxv += xv.y;
          }
          sxi[r] += sxv;
          acc[r] += a;
        }
      }
    }
    if (!__syncthreads_and(ok)) {
      ring.abandon(tid, step, s.err);
      return;
    }
    ring.advance(tid, step);
  }
  FF al[CELL_TILE];
  long long ax[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) { al[r] = FF{acc[r], 0.0f}; ax[r] = sxi[r]; }
  cell_reduce(al, sh, sh_l);
  cell_reduce_i(ax, shi, sh_x);
  if (tid < len) {
    const int i = sh_i[tid];
    if (i != s.batch_off[b]) {  // the first cell of each batch keeps delta = 0
      const float d = s.delta[i], dp = s.delta_p[i];
      const double md = s.mu_delta[i];
      const double lr = (double)(dp - d) * (double)sh_x[tid] - ff_value(sh_l[tid]);
      const double prior = (((double)d - md) * ((double)d - md) - ((double)dp - md) * ((double)dp - md)) /
                           (2.0 * SIGMA2_DELTA);
      const float u = uniform_at(s.seed, SID_DELTA, (uint64_t)i, iter, 2);
      s.lr_delta[i] = lr + prior;
      if ((double)logf(u) <= lr + prior) {
        s.delta[i] = dp;
        s.Dexp[i] = expf(dp);
      }
    }
  }
}

// Log-likelihood change of one entry when its type moves and beta changes by
// eps = beta' - beta:  eps x - (phi + x) log[(phi + mu') / (phi + mu)], with
// mu' = mu e^eps read from the table exp(alpha + beta + nu) of the new type.
__device__ __forceinline__ float type_shift_term(float eps, float mu, float mup, float ph, int x) {
  const float xf = (float)x;
  return fmaf(eps, xf, -(ph + xf) * log_ratio(ph + mup, ph + mu, mup - mu));
}

// W by Metropolis-Hastings with a uniform proposal (the reference's move).
__global__ void __launch_bounds__(CELL_THREADS, 4) k_w_mh(DevState s) {
  extern __shared__ __align__(128) int xbuf[];
  __shared__ __align__(8) uint64_t bar[X_STAGES];
  __shared__ FF sh[(CELL_THREADS / 32) * CELL_TILE];
  __shared__ FF sh_l[CELL_TILE];
  __shared__ int sh_i[CELL_TILE], sh_kp[CELL_TILE], sh_ai[CELL_TILE], sh_ar[CELL_TILE], sh_na;
  __shared__ float sh_D[CELL_TILE], sh_u[CELL_TILE];
  const int4 t = s.ctile[blockIdx.x];
  const int b = t.x, k = t.y, start = t.z, len = t.w;
  if (len == 0) return;
  const int tid = threadIdx.x;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp, G = s.G;
  if (tid < CELL_TILE) {
    const int i = s.perm[start + (tid < len ? tid : 0)];
    sh_i[tid] = i;
    sh_D[tid] = s.Dexp[i];
    Stream st(s.seed, SID_W, (uint64_t)i, iter);
    const uint32_t r0 = st.next_u32();
    sh_kp[tid] = tid < len ? (int)(((uint64_t)r0 * (uint64_t)s.K) >> 32) : k;
    sh_u[tid] = st.uniform();
  }
  __syncthreads();
  // cells whose proposed type differs from the current one; only their X rows
  // are read
  if (tid == 0) {
    int na = 0;
    for (int r = 0; r < len; ++r)
      if (sh_kp[r] != k) {
        sh_ai[na] = sh_i[r];
        sh_ar[na] = r;
        ++na;
      }
    sh_na = na;
  }
  WRing ring{xbuf, bar, s.X, sh_ai, Gp, 0, (int)((Gp + W_WIDTH - 1) / W_WIDTH)};
  ring.init(tid);
  __syncthreads();
  const int na = sh_na;
  ring.len = na;
  if (na > 0) ring.prologue(tid);
  float acc[CELL_TILE];
#pragma unroll
  for (int r = 0; r < CELL_TILE; ++r) acc[r] = 0.0f;
  const float* Eb = s.E + (int64_t)b * s.K * Gp;
  const float* Er = Eb + (int64_t)k * Gp;
  const float* Pr = s.phi + (int64_t)b * Gp;
  const float* Bk = s.beta + (int64_t)k * Gp;
  for (int step = 0; na > 0 && step < ring.n_steps; ++step) {
    const int64_t g2 = (int64_t)step * W_WIDTH + tid * 2;
    const bool in = g2 < G;
    float2 e = make_float2(0.f, 0.f), ph = e, bk = e;
    if (in) {
      e = *reinterpret_cast<const float2*>(Er + g2);
      ph = *reinterpret_cast<const float2*>(Pr + g2);
      bk = *reinterpret_cast<const float2*>(Bk + g2);
    }
    const bool two = g2 + 1 < G;
    const bool ok = ring.wait(step);
    if (in) {
#pragma unroll
      for (int a = 0; a < CELL_TILE; ++a) {
        if (a < na) {
          const int r = sh_ar[a];
          const int64_t kp_off = (int64_t)sh_kp[r] * Gp + g2;
          const float2 bp = *reinterpret_cast<const float2*>(s.beta + kp_off);
          const float2 ep = *reinterpret_cast<const float2*>(Eb + kp_off);
          const int2 xv = *reinterpret_cast<const int2*>(ring.row(step, a) + tid * 2);
          const float D = sh_D[r];
          float v = type_shift_term(bp.x - bk.x, e.x * D, ep.x * D, ph.x, xv.x);
          if (two) v += type_shift_term(bp.y - bk.y, e.y * D, ep.y * D, ph.y, xv.y);
          acc[a] += v;
        }
      }
    }
    if (!__syncthreads_and(ok)) {
      ring.abandon(tid, step, s.err);
      return;
    }
    ring.advance(tid, step);
  }
  FF al[CELL_TILE];
#pragma unroll
  for (int a = 0; a < CELL_TILE; ++a) al[a] = FF{acc[a], 0.0f};
  cell_reduce(al, sh, sh_l);  // sh_l[a]: active slot a
  if (tid < len) {
    const int i = sh_i[tid], kp = sh_kp[tid];
    int a = -1;
    for (int q = 0; q < na; ++q)
      if (sh_ar[q] == tid) a = q;
    const double ll = a >= 0 ? ff_value(sh_l[a]) : 0.0;
    const double rhs = (double)logf(s.pi[b * s.K + kp]) - (double)logf(s.pi[b * s.K + k]) + ll;
    s.lr_W[i] = rhs;
    if ((double)logf(sh_u[tid]) <= rhs) s.W[i] = kp;
  }
}

// W by a K-way categorical draw from its full conditional (Gibbs).  Targets
// the same conditional as the reference's MH move.  One CTA handles the tile's
// cells two at a time and the types eight at a time.
constexpr int GIBBS_CELLS = 2;
constexpr int GIBBS_TYPES = 8;
__global__ void __launch_bounds__(CELL_THREADS) k_w_gibbs(DevState s) {
  __shared__ FF sh_red[(CELL_THREADS / 32) * GIBBS_CELLS * GIBBS_TYPES];
  __shared__ double sh_lp[CELL_TILE][MAX_K];
  __shared__ int sh_i[CELL_TILE];
  __shared__ float sh_D[CELL_TILE];
  const int4 t = s.ctile[blockIdx.x];
  const int b = t.x, k = t.y, start = t.z, len = t.w;
  if (len == 0) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = CELL_THREADS / 32;
  const uint32_t iter = (uint32_t)*s.iter;
  const int64_t Gp = s.Gp, G = s.G;
  const int K = s.K;
  if (tid < CELL_TILE) {
    const int i = s.perm[start + (tid < len ? tid : 0)];
    sh_i[tid] = i;
    sh_D[tid] = s.Dexp[i];
  }
  __syncthreads();
  const float* Eb = s.E + (int64_t)b * K * Gp;
  const float* Er = Eb + (int64_t)k * Gp;
  const float* Pr = s.phi + (int64_t)b * Gp;
  const float* Bk = s.beta + (int64_t)k * Gp;
  for (int r0 = 0; r0 < len; r0 += GIBBS_CELLS) {
    for (int k0 = 0; k0 < K; k0 += GIBBS_TYPES) {
      KahanF acc[GIBBS_CELLS][GIBBS_TYPES];
      for (int64_t g = tid; g < G; g += CELL_THREADS) {
        const float e = Er[g], ph = Pr[g], bk = Bk[g];
        float bt[GIBBS_TYPES], et[GIBBS_TYPES];
#pragma unroll
        for (int kk = 0; kk < GIBBS_TYPES; ++kk) {
          bt[kk] = (k0 + kk < K) ? s.beta[(int64_t)(k0 + kk) * Gp + g] : bk;
          et[kk] = (k0 + kk < K) ? Eb[(int64_t)(k0 + kk) * Gp + g] : e;
        }
#pragma unroll
        for (int r = 0; r < GIBBS_CELLS; ++r) {
          if (r0 + r < len) {
            const int x = s.X[(int64_t)sh_i[r0 + r] * Gp + g];
            const float D = sh_D[r0 + r];
            const float mu = e * D;
#pragma unroll
            for (int kk = 0; kk < GIBBS_TYPES; ++kk)
              if (k0 + kk < K && k0 + kk != k) acc[r][kk].add(type_shift_term(bt[kk] - bk, mu, et[kk] * D, ph, x));
          }
        }
      }
#pragma unroll
      for (int r = 0; r < GIBBS_CELLS; ++r)
#pragma unroll
        for (int kk = 0; kk < GIBBS_TYPES; ++kk) {
          const FF v = ff_warp_sum(acc[r][kk].ff());
          if (lane == 0) sh_red[(warp * GIBBS_CELLS + r) * GIBBS_TYPES + kk] = v;
        }
      __syncthreads();
      if (tid < GIBBS_CELLS * GIBBS_TYPES) {
        const int r = tid / GIBBS_TYPES, kk = tid % GIBBS_TYPES;
        FF tsum = sh_red[r * GIBBS_TYPES + kk];
        for (int w = 1; w < nw; ++w) tsum = ff_add(tsum, sh_red[(w * GIBBS_CELLS + r) * GIBBS_TYPES + kk]);
        if (r0 + r < len && k0 + kk < K) sh_lp[r0 + r][k0 + kk] = ff_value(tsum);
      }
      __syncthreads();
    }
  }
  if (tid < len) {
    const int i = sh_i[tid];
    double mx = -1e300;
    for (int kk = 0; kk < K; ++kk) {
      const double lp = sh_lp[tid][kk] + (double)logf(s.pi[b * K + kk]);
      sh_lp[tid][kk] = lp;
      mx = fmax(mx, lp);
    }
    double tot = 0.0;
    for (int kk = 0; kk < K; ++kk) tot += exp(sh_lp[tid][kk] - mx);
    const float u = uniform_at(s.seed, SID_W, (uint64_t)i, iter, 0);
    const double target = (double)u * tot;
    double cum = 0.0;
    int pick = K - 1;
    for (int kk = 0; kk < K; ++kk) {
      cum += exp(sh_lp[tid][kk] - mx);
      if (target < cum) { pick = kk; break; }
    }
    s.W[i] = pick;
    // diagnostic: log weight of the drawn type relative to the current one
    s.lr_W[i] = sh_lp[tid][pick] - sh_lp[tid][k];
  }
}

// ---------------------------------------------------------------------------
// pi (Dirichlet) and the (batch, type) cell order; one CTA per batch.
// do_pi = 0 at initialisation.  The last CTA advances the sweep index when
// `advance` is set.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_sort_pi(DevState s, int do_pi, int advance) {
  __shared__ int cnt[MAX_K], base[MAX_K], run[MAX_K], rtot[MAX_K], gb[MAX_K + 1], cb[MAX_K + 1];
  __shared__ int wcnt[32][MAX_K];
  __shared__ float gk[MAX_K];
  __shared__ int sh_flag;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int K = s.K;
  const uint32_t iter = (uint32_t)*s.iter;
  const int off = s.batch_off[b], nb = s.batch_off[b + 1] - off;
  if (tid < K) { cnt[tid] = 0; run[tid] = 0; }
  __syncthreads();
  for (int j = tid; j < nb; j += blockDim.x) atomicAdd(&cnt[s.W[off + j]], 1);
  __syncthreads();
  if (tid == 0) {
    int acc = 0, ga = 0, ca = 0;
    for (int kk = 0; kk < K; ++kk) {
      base[kk] = acc;
      gb[kk] = ga;
      cb[kk] = ca;
      acc += cnt[kk];
      ga += (cnt[kk] + s.CG - 1) / s.CG;
      ca += (cnt[kk] + CELL_TILE - 1) / CELL_TILE;
    }
    gb[K] = ga;
    cb[K] = ca;
  }
  if (tid < K) s.seg_cnt[b * K + tid] = cnt[tid];
  if (do_pi && tid < K) {
    Stream st(s.seed, SID_PI, (uint64_t)(b * K + tid), iter);
    int err = 0;
    gk[tid] = gamma_mt(st, (float)((double)cnt[tid] + XI_PI), &err);
    if (err) atomicOr(s.err, err);
  }
  __syncthreads();
  if (do_pi && tid == 0) {
    float tot = 0.0f;
    for (int kk = 0; kk < K; ++kk) tot += gk[kk];
    for (int kk = 0; kk < K; ++kk) s.pi[b * K + kk] = gk[kk] / tot;
  }
  // stable counting sort of the batch's cells by type
  for (int r0 = 0; r0 < nb; r0 += blockDim.x) {
    const int j = r0 + tid;
    const bool act = j < nb;
    const int kk = act ? s.W[off + j] : MAX_K + 1;
    const unsigned same = __match_any_sync(0xffffffffu, kk);
    const int rank = __popc(same & ((1u << lane) - 1u));
    for (int q = tid; q < 32 * MAX_K; q += blockDim.x) wcnt[q / MAX_K][q % MAX_K] = 0;
    __syncthreads();
    if (act && rank == 0) wcnt[warp][kk] = __popc(same);
    __syncthreads();
    if (tid < K) {  // exclusive prefix over warps, per type
      int acc = 0;
      for (int w = 0; w < 32; ++w) {
        const int c = wcnt[w][tid];
        wcnt[w][tid] = acc;
        acc += c;
      }
      rtot[tid] = acc;
    }
    __syncthreads();
    if (act) s.perm[off + base[kk] + run[kk] + wcnt[warp][kk] + rank] = off + j;
    __syncthreads();
    if (tid < K) run[tid] += rtot[tid];
    __syncthreads();
  }
  // work lists of this batch: gene-pass chunks (CG cells) and cell tiles
  int gofs = 0, cofs = 0;
  for (int bb = 0; bb < b; ++bb) {
    const int n = s.batch_off[bb + 1] - s.batch_off[bb];
    gofs += n / s.CG + K;
    cofs += n / CELL_TILE + K;
  }
  const int gcap = nb / s.CG + K, ccap = nb / CELL_TILE + K;
  // (batch, type) segment -> its run of gene-pass chunks, for the decision kernels
  if (tid < K) s.seg_chunk[b * K + tid] = make_int2(gofs + gb[tid], gb[tid + 1] - gb[tid]);
  for (int q = tid; q < gcap; q += blockDim.x) {
    int4 v = make_int4(b, 0, off, 0);
    if (q < gb[K]) {
      int kk = 0;
      while (q >= gb[kk + 1]) ++kk;
      // split the segment into equal-length chunks of at most CG cells
      const int n = cnt[kk], nc = (n + s.CG - 1) / s.CG, c = q - gb[kk];
      const int c0 = (int)((int64_t)c * n / nc), c1 = (int)((int64_t)(c + 1) * n / nc);
      v = make_int4(b, kk, off + base[kk] + c0, c1 - c0);
    }
    s.gchunk[gofs + q] = v;
  }
  for (int q = tid; q < ccap; q += blockDim.x) {
    int4 v = make_int4(b, 0, off, 0);
    if (q < cb[K]) {
      int kk = 0;
      while (q >= cb[kk + 1]) ++kk;
      const int n = cnt[kk], nc = (n + CELL_TILE - 1) / CELL_TILE, c = q - cb[kk];
      const int c0 = (int)((int64_t)c * n / nc), c1 = (int)((int64_t)(c + 1) * n / nc);
      v = make_int4(b, kk, off + base[kk] + c0, c1 - c0);
    }
    s.ctile[cofs + q] = v;
  }
  if (advance && arrive_last(&s.cnt_glob[1], (unsigned)s.B, &sh_flag) && tid == 0) *s.iter += 1;
}

// ---------------------------------------------------------------------------
// Posterior accumulation of one kept sweep (and optional draw storage).
// ---------------------------------------------------------------------------
__global__ void k_posterior(DevState s, int advance) {
  __shared__ int sh_flag;
  const int it = *s.iter;
  const int kept = it - s.n_burnin;
  const bool store = s.keep_draws && kept >= 0 && kept < s.n_kept;  // draw slot inside the run
  const int64_t G = s.G, Gp = s.Gp, N = s.N;
  const int B = s.B, K = s.K;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)K * G; t += stride) {
    const int k = (int)(t / G);
    const int64_t g = t % G;
    if (k == 0) {
      s.acc_alpha[g] += s.alpha[g];
      if (store) s.keep_alpha[(int64_t)kept * G + g] = s.alpha[g];
      continue;
    }
    const float bt = s.beta[(int64_t)k * Gp + g];
    const int8_t l = s.L[(int64_t)k * Gp + g];
    s.acc_beta[t] += bt;
    s.acc_L[t] += l;
    if (store) {
      s.keep_beta[(int64_t)kept * (K - 1) * G + t - G] = bt;
      s.keep_L[(int64_t)kept * (K - 1) * G + t - G] = l;
    }
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)B * G; t += stride) {
    const int b = (int)(t / G);
    const int64_t g = t % G;
    const float ph = s.phi[(int64_t)b * Gp + g];
    s.acc_phi[t] += ph;
    if (store) s.keep_phi[(int64_t)kept * B * G + t] = ph;
    if (b > 0) {
      const float nv = s.nu[(int64_t)b * Gp + g];
      s.acc_nu[t] += nv;
      if (store) s.keep_nu[(int64_t)kept * (B - 1) * G + t - G] = nv;
    }
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    s.acc_delta[i] += s.delta[i];
    s.acc_wcnt[i * K + s.W[i]] += 1;
    if (store) {
      s.keep_delta[(int64_t)kept * N + i] = s.delta[i];
      s.keep_W[(int64_t)kept * N + i] = (int16_t)s.W[i];
    }
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 2 * B + B * K + 2; t += stride) {
    if (t < 2 * B) {
      s.acc_gamma[t] += s.gamma[t];
      if (store) s.keep_gamma[(int64_t)kept * 2 * B + t] = s.gamma[t];
    } else if (t < 2 * B + B * K) {
      const int64_t q = t - 2 * B;
      s.acc_pi[q] += s.pi[q];
      if (store) s.keep_pi[(int64_t)kept * B * K + q] = s.pi[q];
    } else {
      const int64_t q = t - 2 * B - B * K;
      s.acc_ptau[q] += s.p_tau0[q];
      if (store) s.keep_ptau[(int64_t)kept * 2 + q] = s.p_tau0[q];
    }
  }
  if (advance && arrive_last(&s.cnt_glob[2], gridDim.x, &sh_flag) && threadIdx.x == 0) *s.iter += 1;
}

}  // namespace bq
