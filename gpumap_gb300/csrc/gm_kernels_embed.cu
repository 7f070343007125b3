// Embedding phase: fuzzy simplicial set over the published k-NN (self
// prepended), edge scheduling and negative-sampling SGD.  Restates the
// reference's embedding_kernel.cuh and Impl::embed (impl.cuh:335-500) with
// every count and threshold kept on the device (no host round trips).
#include <algorithm>

#include <mutex>

#include "gm_common.cuh"
#include "gm_kernels.h"

namespace gm {

// Scalar slots in EmbedScratch.
//   fscal: 0 mean_dist, 1 max_w, 2 rounding, 3 x_min, 4 x_max
//   iscal: 0 nnz (directed + extras), 1 extras, 2 nnz after trim, 3 max degree,
//          4 rows n (read by the SGD epochs so a captured graph stays valid)
enum { FS_MEAN = 0, FS_MAXW = 1, FS_ROUND = 2, FS_XMIN = 3, FS_XMAX = 4 };
enum { IS_NNZ = 0, IS_EXTRA = 1, IS_NNZ2 = 2, IS_MAXDEG = 3, IS_N = 4 };

namespace {

constexpr float kSmoothTol = 1e-5f;  // SMOOTH_K_TOLERANCE
constexpr float kMinKDistScale = 1e-3f;

// Embed-time k-NN (reference prepend_self_knn_kernel, embedding_kernel.cuh:599-631):
// column 0 is the row itself at distance 0; column c >= 1 is published
// neighbour c-1 (the k-th is dropped); euclidean distances are square-rooted.
GM_D uint32_t eidx(const uint32_t *pub_idx, int k, int row, int c) {
  return c == 0 ? (uint32_t)row : pub_idx[(size_t)row * (k + 1) + (c - 1)];
}
GM_D float edist(const float *pub_dist, int k, int row, int c, int euclid) {
  if (c == 0) return 0.0f;
  const float v = pub_dist[(size_t)row * (k + 1) + (c - 1)];
  return euclid ? __fsqrt_rn(v > 0.0f ? v : 0.0f) : v;
}
GM_D bool valid_d(float v) { return isfinite(v) && v >= 0.0f && v < FLT_MAX / 2.0f; }

GM_D float membership(float dist, float rho, float sigma) {
  const float dr = __fsub_rn(dist, rho);
  if (dr <= 0.0f || sigma == 0.0f) return 1.0f;
  const float v = gm_expf(-__fdiv_rn(dr, sigma));
  return v < FLT_MIN ? FLT_MIN : v;
}

// Block sums of the embed-time distances (256 per block, FP32 tree).
__global__ void k_mean_partial(const float *pub_dist, int n, int k, int euclid,
                               float *part, int *ipart) {
  __shared__ float ss[256];
  __shared__ float sc[256];
  const int t = threadIdx.x;
  const long g = (long)blockIdx.x * 256 + t;
  float v = 0.0f, c = 0.0f;
  if (g < (long)n * k) {
    const int row = (int)(g / k), ki = (int)(g % k);
    const float raw = edist(pub_dist, k, row, ki, euclid);
    if (raw >= 0.0f && raw < FLT_MAX / 2.0f) {
      v = raw;
      c = 1.0f;
    }
  }
  ss[t] = v;
  sc[t] = c;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (t < s) {
      ss[t] = __fadd_rn(ss[t], ss[t + s]);
      sc[t] = __fadd_rn(sc[t], sc[t + s]);
    }
    __syncthreads();
  }
  if (t == 0) {
    part[blockIdx.x] = ss[0];
    ipart[blockIdx.x] = (int)sc[0];
  }
}

// Ordered sum of the partials: a block stages them in shared memory by
// coalesced loads, then thread 0 adds them in index order.
constexpr int kMeanStage = 4096;
__global__ void k_mean_final(const float *part, const int *ipart, int nb, float *fscal) {
  __shared__ float sp[kMeanStage];
  __shared__ int si[kMeanStage];
  float s = 0.0f;
  long c = 0;
  for (int i0 = 0; i0 < nb; i0 += kMeanStage) {
    const int m = min(kMeanStage, nb - i0);
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      sp[i] = part[i0 + i];
      si[i] = ipart[i0 + i];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int i = 0; i < m; ++i) {
        s = __fadd_rn(s, sp[i]);
        c += si[i];
      }
  }
  if (threadIdx.x == 0)
    fscal[FS_MEAN] = (c > 0 && isfinite(s) && s > 0.0f) ? __fdiv_rn(s, (float)c) : 1.0f;
}

// sigma / rho per row, one warp per row; the bisection's target sum is
// accumulated in FP64 by a fixed butterfly (reference smooth_knn_dist_kernel,
// embedding_kernel.cuh:135-207).
// sigma / rho by bisection (reference smooth_knn_dist, one warp per row for
// k > 16).  The bisection's target sum is accumulated in FP64 by the fixed
// xor-butterfly order of 32 lanes, term c on lane c (the terms of lanes >= k
// are +0, adding them is exact).
__global__ void k_smooth_knn(const float *pub_dist, int n, int k, int euclid,
                             const float *fscal, double target, float *sigma,
                             float *rho) {
  const int lane = threadIdx.x & 31;
  const long gid = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gid >= n) return;
  const int row = (int)gid;
  const float raw = lane < k ? edist(pub_dist, k, row, lane, euclid) : 0.0f;
  const float san = (lane < k && valid_d(raw)) ? raw : 0.0f;
  float sum = 0.0f;
  for (int c = 0; c < k; ++c) sum = __fadd_rn(sum, __shfl_sync(0xffffffffu, san, c));
  const unsigned nz = __ballot_sync(0xffffffffu, lane < k && san > 0.0f);
  const float mean_dist = fscal[FS_MEAN];
  if (nz == 0u) {
    if (lane == 0) {
      rho[row] = 0.0f;
      sigma[row] = __fmul_rn(kMinKDistScale, mean_dist);
    }
    return;
  }
  const float r = __shfl_sync(0xffffffffu, raw, __ffs(nz) - 1);
  const float row_mean = __fdiv_rn(sum, (float)k);
  float lo = 0.0f, hi = FLT_MAX, mid = 1.0f;
  const bool contrib = lane >= 2 && lane < k;
  const float dj = __fsub_rn(san, r);
  for (int it = 0; it < 64; ++it) {
    double term = 0.0;
    if (contrib) term = (dj > 0.0f) ? (double)gm_expf(__fdiv_rn(-dj, mid)) : 1.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
    if (fabs(term - target) < (double)kSmoothTol) break;
    if (term > target) {
      hi = mid;
      mid = __fmul_rn(__fadd_rn(lo, hi), 0.5f);
    } else {
      lo = mid;
      mid = (hi == FLT_MAX) ? __fmul_rn(mid, 2.0f) : __fmul_rn(__fadd_rn(lo, hi), 0.5f);
    }
  }
  if (lane != 0) return;
  if (!isfinite(mid) || mid <= 0.0f) mid = 1.0f;
  const float min_scale = __fmul_rn(kMinKDistScale, (r > 0.0f) ? row_mean : mean_dist);
  rho[row] = r;
  sigma[row] = mid < min_scale ? min_scale : mid;
}

// The same for k <= 16 with four lanes per row (eight rows per warp).  Lane
// q of a row holds terms c = q, q+4, q+8, q+12 and forms
// (t[q] + t[q+8]) + (t[q+4] + t[q+12]); two more xor steps over the four
// lanes finish the sum.  For k <= 16 this is exactly the 32-lane butterfly's
// tree (its first step only adds the exact zeros of lanes 16-31, the next two
// are these per-lane additions), so every bit agrees with the warp-per-row
// form, with a quarter of the FP64 additions (FP64 is slow on this part).
__global__ void k_smooth_knn4(const float *pub_dist, int n, int k, int euclid,
                              const float *fscal, double target, float *sigma,
                              float *rho) {
  const int lane = threadIdx.x & 31;
  const int q = lane & 3, base = lane - q;
  const long gid = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const bool live = gid < n;
  const int row = live ? (int)gid : 0;
  float raw[4], san[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = q + 4 * j;
    raw[j] = (live && c < k) ? edist(pub_dist, k, row, c, euclid) : 0.0f;
    san[j] = (live && c < k && valid_d(raw[j])) ? raw[j] : 0.0f;
  }
  // row sum in column order, first nonzero column
  float sum = 0.0f;
  int first = 64;
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const float v = __shfl_sync(0xffffffffu, san[c >> 2], base + (c & 3));
    if (c < k) {
      sum = __fadd_rn(sum, v);
      if (first == 64 && v > 0.0f) first = c;
    }
  }
  const float mean_dist = fscal[FS_MEAN];
  float r = 0.0f;
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const float v = __shfl_sync(0xffffffffu, raw[c >> 2], base + (c & 3));
    if (c == first) r = v;
  }
  const float row_mean = __fdiv_rn(sum, (float)k);
  float lo = 0.0f, hi = FLT_MAX, mid = 1.0f;
  float dj[4];
  bool contrib[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = q + 4 * j;
    contrib[j] = c >= 2 && c < k;
    dj[j] = __fsub_rn(san[j], r);
  }
  bool done = !live || first == 64;
  for (int it = 0; it < 64; ++it) {
    if (__all_sync(0xffffffffu, done)) break;
    double t[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      t[j] = 0.0;
      if (contrib[j] && !done) t[j] = (dj[j] > 0.0f) ? (double)gm_expf(__fdiv_rn(-dj[j], mid)) : 1.0;
    }
    double term = (t[0] + t[2]) + (t[1] + t[3]);
    term += __shfl_xor_sync(0xffffffffu, term, 2);
    term += __shfl_xor_sync(0xffffffffu, term, 1);
    if (done) continue;
    if (fabs(term - target) < (double)kSmoothTol) {
      done = true;
      continue;
    }
    if (term > target) {
      hi = mid;
      mid = __fmul_rn(__fadd_rn(lo, hi), 0.5f);
    } else {
      lo = mid;
      mid = (hi == FLT_MAX) ? __fmul_rn(mid, 2.0f) : __fmul_rn(__fadd_rn(lo, hi), 0.5f);
    }
  }
  if (!live || q != 0) return;
  if (first == 64) {
    rho[row] = 0.0f;
    sigma[row] = __fmul_rn(kMinKDistScale, mean_dist);
    return;
  }
  if (!isfinite(mid) || mid <= 0.0f) mid = 1.0f;
  const float min_scale = __fmul_rn(kMinKDistScale, (r > 0.0f) ? row_mean : mean_dist);
  rho[row] = r;
  sigma[row] = mid < min_scale ? min_scale : mid;
}

// Directed membership p_ij for batch rows and the fuzzy union
// w = p_ij + p_ji - p_ij p_ji; flag marks edges whose reverse is absent
// (reference: embedding_kernel.cuh:214-320).
__global__ void k_memb_sym(const uint32_t *pub_idx, const float *pub_dist, int n, int k,
                           int euclid, const float *sigma, const float *rho,
                           const int *batch, int nb, int *coo_row, int *coo_col,
                           float *coo_val, int *flag) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nb * k) return;
  const int bi = tid / k, ki = tid - bi * k;
  const int row = batch[bi];
  const uint32_t raw_col = eidx(pub_idx, k, row, ki);
  const bool valid_col = raw_col < (uint32_t)n;
  const int col = valid_col ? (int)raw_col : row;
  const float dist = edist(pub_dist, k, row, ki, euclid);
  float pij = 0.0f;
  if (valid_col && col != row && valid_d(dist)) pij = membership(dist, rho[row], sigma[row]);
  const int i = row, j = col;
  float pji = 0.0f;
  for (int kj = 0; kj < k; ++kj) {
    if ((int)eidx(pub_idx, k, j, kj) == i) {
      const float dji = edist(pub_dist, k, j, kj, euclid);
      if (!valid_d(dji)) break;
      pji = membership(dji, rho[j], sigma[j]);
      break;
    }
  }
  const float w = __fmaf_rn(-pij, pji, __fadd_rn(pij, pji));
  coo_row[tid] = i;
  coo_col[tid] = j;
  coo_val[tid] = w;
  flag[tid] = (pji == 0.0f) ? 1 : 0;
}

__global__ void k_write_extras(const int *idx, const int *cnt, int ndir, int *coo_row,
                               int *coo_col, float *coo_val, int *iscal) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = *cnt;
  if (q == 0) {
    iscal[IS_NNZ] = ndir + c;
    iscal[IS_EXTRA] = c;
  }
  if (q >= c) return;
  const int src = idx[q];
  coo_row[ndir + q] = coo_col[src];
  coo_col[ndir + q] = coo_row[src];
  coo_val[ndir + q] = coo_val[src];
}

// max_w over non-negative weights via the int ordering of their bits.
__global__ void k_max_w(const float *vals, const int *iscal, float *fscal) {
  const int nnz = iscal[IS_NNZ];
  float m = 0.0f;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += gridDim.x * blockDim.x)
    m = fmaxf(m, vals[q]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f)
    atomicMax(reinterpret_cast<int *>(&fscal[FS_MAXW]), __float_as_int(m));
}

// Trim flag: keep w >= max_w / n_epochs (reference trim_graph, :348-400).
__global__ void k_trim_flags(const float *vals, const int *iscal, const float *fscal,
                             int n_epochs, int *flag, int nmax) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nmax) return;
  const int nnz = iscal[IS_NNZ];
  const float mw = fscal[FS_MAXW];
  int keep = 0;
  if (q < nnz && mw > 0.0f) keep = vals[q] >= __fdiv_rn(mw, (float)n_epochs) ? 1 : 0;
  flag[q] = keep;
}

// Gather survivors; epochs_per_sample; head degrees; epoch state
// (reference: :469-495, :405-460).
__global__ void k_gather_sched(const int *idx, const int *iscal, const int *crow,
                               const int *ccol, const float *cval, const float *fscal,
                               int n_epochs, float nsr_inv, int *trow, int *tcol,
                               float *eps, float *next_s, float *next_n, int *deg) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= iscal[IS_NNZ2]) return;
  const int src = idx[q];
  const float mw = fscal[FS_MAXW];
  const float w = cval[src];
  const float ns = __fmul_rn((float)n_epochs, __fdiv_rn(w, mw));
  const float e = (ns > 0.0f) ? __fdiv_rn((float)n_epochs, ns) : -1.0f;
  trow[q] = crow[src];
  tcol[q] = ccol[src];
  eps[q] = e;
  next_s[q] = e;
  next_n[q] = __fmul_rn(e, nsr_inv);
  atomicAdd(&deg[crow[src]], 1);
}

__global__ void k_max_deg(const int *deg, int n, int *iscal) {
  int m = 0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    m = max(m, deg[q]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(&iscal[IS_MAXDEG], m);
}

// Gradient rounding factor 2^ceil-ish via frexp (reference :433-460).
__global__ void k_rounding(int *iscal, float *fscal, float alpha) {
  const int nnz = iscal[IS_NNZ2];
  const int md = iscal[IS_MAXDEG];
  float r = 1.0f;
  if (nnz > 0 && md > 0) {
    const float max_abs = __fmul_rn(__fmul_rn((float)md, 4.0f), fabsf(alpha));
    const float denom = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, (float)md), FLT_EPSILON));
    const float delta = __fdiv_rn(max_abs, denom);
    int ex;
    frexpf(delta, &ex);
    r = ldexpf(1.0f, ex);
  }
  fscal[FS_ROUND] = r;
}

GM_D float fclip(float v) {
  if (!isfinite(v)) return 0.0f;
  return fmaxf(fminf(v, 4.0f), -4.0f);
}
GM_D float trunc_grad(float rounding, float x) {
  return __fsub_rn(__fadd_rn(rounding, x), rounding);
}

// One edge of one SGD epoch (reference optimize_batch_kernel, :509-589;
// Hogwild updates, tail moved by rounded atomics, head accumulated then
// added).  Embedding positions are read through L2 (ld.global.cg): in the
// persistent kernel other SMs update them between epochs.  The positions of
// the head, the tail and the first kNegAhead negative samples (rows drawn in
// the same Philox order) are fetched together; a sample that is this edge's
// own tail is advanced by this thread's tail update, which in sequential
// order precedes the read.  powf(d2, b - 1) and powf(d2, b) share one log.
constexpr int kNegAhead = 8;

// 8-byte embedding row read through L2, issued where it stands (volatile, a
// memory clobber): the sample positions are fetched ahead of their use.
GM_D float2 ld_pos(const float *p) {
  float2 v;
  asm volatile("ld.global.cg.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p) : "memory");
  return v;
}

// x mod n by a precomputed 64-bit reciprocal, exact for every 32-bit x and
// n >= 1 (Lemire, Kaser and Kurz, "Faster remainder by direct computation",
// 2019): M = floor((2^64 - 1) / n) + 1, x mod n = high64((M * x mod 2^64) * n).
GM_D uint32_t fastmod(uint32_t x, uint64_t M, uint32_t n) {
  return (uint32_t)__umul64hi(M * (uint64_t)x, (uint64_t)n);
}

// Number of negative samples of an active edge at epoch fe.
GM_D int sgd_n_neg(float fe, float nn, float ep_neg) {
  return (int)__fdiv_rn(__fsub_rn(fe, nn), ep_neg);
}

// One edge of one epoch.  The head and tail positions are read first; the
// first kNegAhead negative samples (rows from this edge's Philox stream,
// blocks 0 and 1, words in order, computed directly into registers) are
// fetched together after the attraction and the tail update, ahead of the
// sequential repulsions.  powf(d2, b - 1) and powf(d2, b) share one log.
GM_D void sgd_edge(float *emb, int row, int j, int kk, float ep, float &ns, float &nn, int n,
                   uint64_t M, float rounding, float alpha, float fe, float gamma, float a,
                   float b, float nsr_inv, uint64_t seed, unsigned &my_edges, unsigned &my_negs) {
  ++my_edges;
  float *cp = emb + (size_t)j * 2;
  float *op = emb + (size_t)kk * 2;
  const float2 cpv = ld_pos(cp), opv = ld_pos(op);
  float cur0 = cpv.x, cur1 = cpv.y;
  const float ep_neg = __fmul_rn(ep, nsr_inv);
  const int n_neg = sgd_n_neg(fe, nn, ep_neg);
  int rr[kNegAhead];
  float2 qq[kNegAhead];
  if (n_neg > 0) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    uint32_t w[8];
    philox_block((uint32_t)row, 0u, kTagNegSample, 0u, k0, k1, w);
    if (n_neg > 4) philox_block((uint32_t)row, 1u, kTagNegSample, 0u, k0, k1, w + 4);
#pragma unroll
    for (int p = 0; p < kNegAhead; ++p) {
      if (p < n_neg) {
        rr[p] = (int)fastmod(w[p], M, (uint32_t)n);
      }
    }
  }
  const float dx = __fsub_rn(cur0, opv.x), dy = __fsub_rn(cur1, opv.y);
  const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
  float attr = 0.0f;
  if (d2 > 0.0f) {
    const float lg = gm_logf(d2);
    const float bm1 = __fsub_rn(b, 1.0f);
    const float p_bm1 = bm1 == 0.0f ? 1.0f : gm_expf(__fmul_rn(bm1, lg));
    const float p_b = b == 0.0f ? 1.0f : gm_expf(__fmul_rn(b, lg));
    attr = __fdiv_rn(__fmul_rn(__fmul_rn(-2.0f, __fmul_rn(a, b)), p_bm1),
                     __fadd_rn(__fmul_rn(a, p_b), 1.0f));
  }
  float g0 = __fmul_rn(fclip(__fmul_rn(attr, dx)), alpha);
  float g1 = __fmul_rn(fclip(__fmul_rn(attr, dy)), alpha);
  cur0 = __fadd_rn(cur0, g0);
  cur1 = __fadd_rn(cur1, g1);
  const float t0 = trunc_grad(rounding, -g0), t1 = trunc_grad(rounding, -g1);
  // both coordinates in one vector reduction (each element added
  // atomically, exactly as two scalar adds; rows are 8-byte aligned)
  atomicAdd(reinterpret_cast<float2 *>(op), make_float2(t0, t1));
  ns = __fadd_rn(ns, ep);
  // the samples' positions are read after the attraction, where the
  // reference reads them: by then the epoch's attraction updates are landing,
  // and the repulsion must see them (read at the start of the edge, they
  // give a measurably different layout); fetched together, one round trip
#pragma unroll
  for (int p = 0; p < kNegAhead; ++p)
    if (p < n_neg) qq[p] = ld_pos(emb + (size_t)rr[p] * 2);
  if (n_neg > 0) {
    const float two_gb = __fmul_rn(__fmul_rn(2.0f, gamma), b);
    const float a4 = __fmul_rn(4.0f, alpha);
    // one negative sample: repulsion from q, head moved in sequence
    auto negative = [&](int r, float q0, float q1) {
      if (r == j) return;
      const float ex = __fsub_rn(cur0, q0), ey = __fsub_rn(cur1, q1);
      const float d2n = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
      float rep = 0.0f;
      // repulsion: d2n^b by the hardware exp2 / log2 (__powf); these sampled
      // Hogwild updates are compared statistically, and the attraction
      // above keeps the series pow
      if (d2n > 0.0f)
        rep = __fdiv_rn(two_gb, __fmul_rn(__fadd_rn(0.001f, d2n),
                                          __fadd_rn(__fmul_rn(a, __powf(d2n, b)), 1.0f)));
      const float h0 = (rep > 0.0f) ? __fmul_rn(fclip(__fmul_rn(rep, ex)), alpha) : a4;
      const float h1 = (rep > 0.0f) ? __fmul_rn(fclip(__fmul_rn(rep, ey)), alpha) : a4;
      cur0 = __fadd_rn(cur0, h0);
      cur1 = __fadd_rn(cur1, h1);
      g0 = __fadd_rn(g0, h0);
      g1 = __fadd_rn(g1, h1);
    };
#pragma unroll
    for (int p = 0; p < kNegAhead; ++p) {
      if (p < n_neg) negative(rr[p], qq[p].x, qq[p].y);
    }
    if (n_neg > kNegAhead) {
      // draws past kNegAhead: the same stream from block 2 on
      Philox g;
      philox_init(g, seed, (uint32_t)row, kTagNegSample);
      g.block = kNegAhead / 4;
      for (int p = kNegAhead; p < n_neg; ++p) {
        const int r = (int)fastmod(philox_next(g), M, (uint32_t)n);
        const float2 q = ld_pos(emb + (size_t)r * 2);
        negative(r, q.x, q.y);
      }
    }
    nn = __fadd_rn(nn, __fmul_rn((float)n_neg, ep_neg));
    my_negs += (unsigned)n_neg;
  }
  atomicAdd(reinterpret_cast<float2 *>(cp),
            make_float2(trunc_grad(rounding, g0), trunc_grad(rounding, g1)));
}

// Edges [first, nnz) step stride of one epoch, state in global memory.
GM_D void sgd_epoch_edges(float *emb, const int *head, const int *tail, const float *eps,
                          float *next_s, float *next_n, int nnz, int n, uint64_t M,
                          float rounding, float alpha, int epoch, float gamma, float a, float b,
                          float nsr_inv, uint64_t seed, int first, int stride,
                          unsigned &my_edges, unsigned &my_negs) {
  const float fe = (float)epoch;
  for (int row = first; row < nnz; row += stride) {
    float ns = next_s[row];
    if (ns > fe) continue;
    float nn = next_n[row];
    sgd_edge(emb, row, head[row], tail[row], eps[row], ns, nn, n, M, rounding, alpha, fe, gamma, a,
             b, nsr_inv, seed, my_edges, my_negs);
    next_s[row] = ns;
    next_n[row] = nn;
  }
}

GM_D void sgd_stats(unsigned my_edges, unsigned my_negs, unsigned long long *stat) {
  if (!stat) return;
  for (int o = 16; o > 0; o >>= 1) {
    my_edges += __shfl_xor_sync(0xffffffffu, my_edges, o);
    my_negs += __shfl_xor_sync(0xffffffffu, my_negs, o);
  }
  if ((threadIdx.x & 31) == 0 && my_edges) {
    atomicAdd(&stat[7], (unsigned long long)my_edges);
    atomicAdd(&stat[8], (unsigned long long)my_negs);
  }
}

// One SGD epoch per launch.
__global__ void k_sgd_epoch(float *emb, const int *head, const int *tail,
                            const int *iscal, const float *eps, float *next_s,
                            float *next_n, float alpha, int epoch, float gamma, float a,
                            float b, float nsr_inv, uint64_t seed, const float *fscal,
                            unsigned long long *stat) {
  unsigned my_edges = 0, my_negs = 0;
  const int n = iscal[IS_N];
  const uint64_t M = ~0ull / (uint64_t)max(n, 1) + 1ull;
  sgd_epoch_edges(emb, head, tail, eps, next_s, next_n, iscal[IS_NNZ2], n, M,
                  fscal[FS_ROUND], alpha, epoch, gamma, a, b, nsr_inv, seed,
                  blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, my_edges,
                  my_negs);
  sgd_stats(my_edges, my_negs, stat);
}

// Grid-wide barrier of a co-resident (cooperative) grid on a monotonic
// arrival counter: the barrier after epoch e completes when the counter
// reaches (e + 1) * gridDim.x.  The wait is bounded; on timeout it records
// kDevErrSpin and returns false, and every block then leaves its epoch loop.
constexpr unsigned kBarrierSpinLimit = 1u << 24;
GM_D unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// Arrival: the CTA's work for this epoch is done (bar.sync), made visible
// (fence) and counted.
GM_D void grid_arrive(unsigned *count) {
  __syncthreads();
  if (threadIdx.x == 0)
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
}
// Wait until every CTA has arrived (count >= target); bounded.
GM_D bool grid_wait(unsigned *count, unsigned target, unsigned *err) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned it = 0;
    while (ld_acquire(count) < target) {
      if (++it > kBarrierSpinLimit) {
        ok = 0;
        atomicOr(err, kDevErrSpin);
        break;
      }
      __nanosleep(16);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// All epochs in one cooperative launch, a grid barrier between epochs (the
// reference's kernel boundary): learning rate and seed advance exactly as the
// host loop of the per-epoch form.  A thread's first kRegEdges edges keep
// their indices and sampling clocks in registers for the whole call.
constexpr int kRegEdges = 2;
constexpr int kSgdThreads = 512;
__global__ void __launch_bounds__(kSgdThreads)
    k_sgd_persistent(float *emb, const int *head, const int *tail, const int *iscal,
                     const float *eps, float *next_s, float *next_n, float alpha0, int n_epochs,
                     float gamma, float a, float b, float nsr_inv, uint64_t seed,
                     const float *fscal, unsigned *bar, unsigned *err,
                     unsigned long long *stat) {
  const int nnz = iscal[IS_NNZ2], n = iscal[IS_N];
  const uint64_t M = ~0ull / (uint64_t)max(n, 1) + 1ull;
  const float rounding = fscal[FS_ROUND];
  unsigned my_edges = 0, my_negs = 0;
  // slot i of the grid handles edge i, in the schedule's order (a head's
  // edges in adjacent lanes, as in the reference's one-thread-per-edge
  // epochs).  Warp-sized runs of slots are dealt round-robin over the CTAs
  // (run w to CTA w mod gridDim.x), so the active edges spread over every SM
  // instead of filling the first few; the map from (CTA, thread) to slot is
  // a bijection on [0, gridDim.x * blockDim.x).
  const int first = (((int)threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x) * 32 + ((int)threadIdx.x & 31);
  const int stride = gridDim.x * blockDim.x;
  int rrow[kRegEdges], rj[kRegEdges], rk[kRegEdges];
  float rep[kRegEdges], rns[kRegEdges], rnn[kRegEdges];
#pragma unroll
  for (int t = 0; t < kRegEdges; ++t) {
    const int slot = first + t * stride;
    if (slot < nnz) {
      const int row = slot;
      rrow[t] = row;
      rj[t] = head[row], rk[t] = tail[row], rep[t] = eps[row];
      rns[t] = next_s[row], rnn[t] = next_n[row];
    }
  }
  float alpha = alpha0;
  for (int ep = 0; ep < n_epochs; ++ep) {
    const float fe = (float)ep;
    const uint64_t sd = seed + (uint64_t)ep;
#pragma unroll
    for (int t = 0; t < kRegEdges; ++t) {
      if (first + t * stride < nnz && rns[t] <= fe)
        sgd_edge(emb, rrow[t], rj[t], rk[t], rep[t], rns[t], rnn[t], n, M, rounding, alpha, fe,
                 gamma, a, b, nsr_inv, sd, my_edges, my_negs);
    }
    for (int row = first + kRegEdges * stride; row < nnz; row += stride) {
      float ns = next_s[row];
      if (ns > fe) continue;
      float nn = next_n[row];
      sgd_edge(emb, row, head[row], tail[row], eps[row], ns, nn, n, M, rounding, alpha, fe, gamma,
               a, b, nsr_inv, sd, my_edges, my_negs);
      next_s[row] = ns;
      next_n[row] = nn;
    }
    alpha = __fmul_rn(alpha0, __fsub_rn(1.0f, __fdiv_rn((float)ep, (float)n_epochs)));
    if (ep + 1 < n_epochs) {
      grid_arrive(bar);
      if (!grid_wait(bar, (unsigned)(ep + 1) * gridDim.x, err)) break;
    }
  }
#pragma unroll
  for (int t = 0; t < kRegEdges; ++t)
    if (first + t * stride < nnz) next_s[rrow[t]] = rns[t], next_n[rrow[t]] = rnn[t];
  sgd_stats(my_edges, my_negs, stat);
}

__global__ void k_set_int(int *p, int v) { *p = v; }

__global__ void k_epoch_init(const float *eps, int nnz, float nsr_inv, float *next_s,
                             float *next_n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nnz) return;
  next_s[q] = eps[q];
  next_n[q] = __fmul_rn(eps[q], nsr_inv);
}

// x-range of the embedding (first component) for the noise scale.
__global__ void k_xrange_partial(const float *emb, int n, float *part) {
  __shared__ float smin[256], smax[256];
  const int t = threadIdx.x;
  float mn = FLT_MAX, mx = -FLT_MAX;
  for (int i = blockIdx.x * 256 + t; i < n; i += gridDim.x * 256) {
    const float v = emb[(size_t)i * 2];
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  smin[t] = mn;
  smax[t] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (t < s) {
      smin[t] = fminf(smin[t], smin[t + s]);
      smax[t] = fmaxf(smax[t], smax[t + s]);
    }
    __syncthreads();
  }
  if (t == 0) {
    part[2 * blockIdx.x] = smin[0];
    part[2 * blockIdx.x + 1] = smax[0];
  }
}

__global__ void k_add_noise(float *emb, const int *batch, int nb, const float *part,
                            int nparts, float noise_scale, uint64_t seed) {
  __shared__ float s_scale;
  if (threadIdx.x == 0) {
    float mn = FLT_MAX, mx = -FLT_MAX;
    for (int i = 0; i < nparts; ++i) {
      mn = fminf(mn, part[2 * i]);
      mx = fmaxf(mx, part[2 * i + 1]);
    }
    s_scale = __fmul_rn(noise_scale, __fsub_rn(mx, mn));
  }
  __syncthreads();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nb * 2) return;
  const int node = batch[tid >> 1], comp = tid & 1;
  Philox g;
  philox_init(g, seed, (uint32_t)tid, kTagNoise);
  const float z = gm_normal(g);
  float *p = emb + (size_t)node * 2 + comp;
  *p = __fadd_rn(*p, __fmul_rn(z, s_scale));
}

// Rows not selected this round move to the membership-weighted mean of their
// neighbours' positions, read from a snapshot (reference :811-894).  Ids
// outside [0, n) are skipped.
__global__ void k_heuristic(const uint32_t *pub_idx, const float *pub_dist, int n, int k,
                            int euclid, const float *sigma, const float *rho,
                            const int *unsel, int nu, const float *snap, float *emb) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nu) return;
  const int row = unsel[q];
  const float sg = sigma[row], rh = rho[row];
  float wsum = 0.0f, a0 = 0.0f, a1 = 0.0f;
  for (int ki = 0; ki < k; ++ki) {
    const int col = (int)eidx(pub_idx, k, row, ki);
    if (col == row) continue;
    const float dist = edist(pub_dist, k, row, ki, euclid);
    if (!valid_d(dist)) continue;
    if (col < 0 || col >= n) continue;
    const float w = membership(dist, rh, sg);
    wsum = __fadd_rn(wsum, w);
    a0 = __fmaf_rn(w, snap[(size_t)col * 2], a0);
    a1 = __fmaf_rn(w, snap[(size_t)col * 2 + 1], a1);
  }
  if (wsum > 0.0f) {
    emb[(size_t)row * 2] = __fdiv_rn(a0, wsum);
    emb[(size_t)row * 2 + 1] = __fdiv_rn(a1, wsum);
  }
}

__global__ void k_mark_rows(const int *rows, int nr, int *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nr) flag[rows[i]] = 1;
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

void launch_mark_rows(const int *rows, int nr, int *flag, cudaStream_t s) {
  if (nr <= 0) return;
  k_mark_rows<<<cdiv(nr, 256), 256, 0, s>>>(rows, nr, flag);
  note_launch();
}

void launch_fuzzy_graph(const uint32_t *pub_idx, const float *pub_dist, int n, int k,
                        int euclidean, const int *batch, int nb, double log2_target,
                        EmbedScratch &e, cudaStream_t s) {
  const long total = (long)n * k;
  const int nbl = cdiv(total, 256);
  k_mean_partial<<<nbl, 256, 0, s>>>(pub_dist, n, k, euclidean, e.partial, e.ipartial);
  note_launch();
  k_mean_final<<<1, 256, 0, s>>>(e.partial, e.ipartial, nbl, e.fscal);
  note_launch();
  if (k <= 16)
    k_smooth_knn4<<<cdiv((long)n * 4, 256), 256, 0, s>>>(pub_dist, n, k, euclidean, e.fscal,
                                                         log2_target, e.sigma, e.rho);
  else
    k_smooth_knn<<<cdiv((long)n * 32, 256), 256, 0, s>>>(pub_dist, n, k, euclidean, e.fscal,
                                                         log2_target, e.sigma, e.rho);
  note_launch();
  const int ndir = nb * k;
  if (ndir > 0)
    k_memb_sym<<<cdiv(ndir, 256), 256, 0, s>>>(pub_idx, pub_dist, n, k, euclidean, e.sigma,
                                               e.rho, batch, nb, e.coo_row, e.coo_col,
                                               e.coo_val, e.t_row);
    note_launch();
  compact_flags(e.t_row, ndir, -1, e.t_col, e.iscal + IS_EXTRA, e.tmp2, s);
  k_write_extras<<<cdiv(ndir > 0 ? ndir : 1, 256), 256, 0, s>>>(
      e.t_col, e.iscal + IS_EXTRA, ndir, e.coo_row, e.coo_col, e.coo_val, e.iscal);
  note_launch();
}

void launch_schedule(int n, int nb, int k, float alpha0, int n_epochs, int neg_rate,
                     EmbedScratch &e, cudaStream_t s) {
  if (n <= 0 || n_epochs <= 0 || nb <= 0) {
    cudaMemsetAsync(e.iscal + IS_NNZ2, 0, sizeof(int), s);
    return;
  }
  const int nmax = 2 * nb * k;
  cudaMemsetAsync(e.fscal + FS_MAXW, 0, sizeof(float), s);
  cudaMemsetAsync(e.iscal + IS_MAXDEG, 0, sizeof(int), s);
  cudaMemsetAsync(e.deg, 0, sizeof(int) * (size_t)n, s);
  k_max_w<<<min(cdiv(nmax, 256), 1024), 256, 0, s>>>(e.coo_val, e.iscal, e.fscal);
  note_launch();
  k_trim_flags<<<cdiv(nmax, 256), 256, 0, s>>>(e.coo_val, e.iscal, e.fscal, n_epochs,
                                               e.t_row, nmax);
  note_launch();
  compact_flags_dev(e.t_row, e.iscal + IS_NNZ, nmax, e.t_col, e.iscal + IS_NNZ2, e.tmp2, s);
  // t_col holds survivor indices; gather into (t_row, flag_tail, t_val)
  const float nsr_inv = 1.0f / (float)neg_rate;  // inf when 0: no negatives
  k_gather_sched<<<cdiv(nmax, 256), 256, 0, s>>>(e.t_col, e.iscal, e.coo_row, e.coo_col,
                                                 e.coo_val, e.fscal, n_epochs, nsr_inv,
                                                 e.t_row, e.flag_tail, e.t_val, e.next_s,
                                                 e.next_n, e.deg);
  note_launch();
  k_max_deg<<<min(cdiv(n, 256), 1024), 256, 0, s>>>(e.deg, n, e.iscal);
  note_launch();
  k_rounding<<<1, 1, 0, s>>>(e.iscal, e.fscal, alpha0);
  note_launch();
}

void launch_optimize_layout(float *emb, int n, int nb, int k, float alpha0, float gamma,
                            float a, float b, int n_epochs, int neg_rate, uint64_t seed,
                            EmbedScratch &e, cudaStream_t s) {
  launch_schedule(n, nb, k, alpha0, n_epochs, neg_rate, e, s);
  if (n <= 0 || n_epochs <= 0 || nb <= 0) return;
  launch_set_int(e.iscal + IS_N, n, s);
  launch_sgd(emb, e.t_row, e.flag_tail, e.t_val, e.next_s, e.next_n, e.iscal, e.fscal,
             cdiv(2 * nb * k, 256), alpha0, gamma, a, b, n_epochs, neg_rate, seed, s, nullptr);
}

void launch_set_int(int *p, int v, cudaStream_t s) {
  k_set_int<<<1, 1, 0, s>>>(p, v);
  note_launch();
}

void launch_epoch_init(const float *eps, int nnz, int neg_rate, float *next_s,
                       float *next_n, cudaStream_t s) {
  if (nnz <= 0) return;
  k_epoch_init<<<cdiv(nnz, 256), 256, 0, s>>>(eps, nnz, 1.0f / (float)neg_rate, next_s,
                                              next_n);
  note_launch();
}

void launch_sgd(float *emb, const int *head, const int *tail, const float *eps,
                float *next_s, float *next_n, const int *iscal, const float *fscal,
                int grid, float alpha0, float gamma, float a, float b, int n_epochs,
                int neg_rate, uint64_t seed, cudaStream_t s, unsigned long long *stat) {
  if (n_epochs <= 0 || grid <= 0) return;
  const float nsr_inv = 1.0f / (float)neg_rate;
  float alpha = alpha0;
  uint64_t cur_seed = seed;
  for (int ep = 0; ep < n_epochs; ++ep) {
    k_sgd_epoch<<<grid, 256, 0, s>>>(emb, head, tail, iscal, eps, next_s, next_n, alpha, ep,
                                     gamma, a, b, nsr_inv, cur_seed, fscal, stat);
    note_launch();
    // alpha and seed for the next epoch (reference embedding_kernel.cuh:790-792)
    alpha = alpha0 * (1.0f - (float)ep / (float)n_epochs);
    cur_seed += 1;
  }
}

int sgd_persistent_grid(int device) {
  // per device, once (sessions on several host threads may launch at once)
  static std::mutex mu;
  static int grid[64] = {0};
  if (device < 0 || device >= 64) return 0;
  std::lock_guard<std::mutex> g(mu);
  if (!grid[device]) {
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sgd_persistent, kSgdThreads, 0);
    grid[device] = std::max(1, sms) * std::max(1, std::min(occ, 1));
  }
  return grid[device];
}

cudaError_t launch_sgd_persistent(float *emb, const int *head, const int *tail,
                                  const float *eps, float *next_s, float *next_n,
                                  const int *iscal, const float *fscal, float alpha0,
                                  float gamma, float a, float b, int n_epochs, int neg_rate,
                                  uint64_t seed, unsigned *bar, unsigned *err, int device,
                                  cudaStream_t s, unsigned long long *stat, int max_ctas) {
  if (n_epochs <= 0) return cudaSuccess;
  int grid = sgd_persistent_grid(device);
  if (max_ctas > 0) grid = std::min(grid, max_ctas);
  if (grid <= 0) return cudaErrorInvalidDevice;
  cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  float nsr_inv = 1.0f / (float)neg_rate;
  void *args[] = {&emb, &head, &tail, &iscal, &eps, &next_s, &next_n, &alpha0, &n_epochs,
                  &gamma, &a, &b, &nsr_inv, &seed, &fscal, &bar, &err, &stat};
  e = cudaLaunchCooperativeKernel((const void *)k_sgd_persistent, dim3(grid), dim3(kSgdThreads),
                                  args, 0, s);
  note_launch();
  return e;
}

cudaError_t launch_sgd_call(float *emb, const int *head, const int *tail, const float *eps,
                            float *next_s, float *next_n, const int *iscal, const float *fscal,
                            float alpha0, float gamma, float a, float b, int n_epochs, int neg_rate,
                            uint64_t seed, unsigned *bar, unsigned *err, int device, cudaStream_t s,
                            unsigned long long *stat, int max_ctas) {
  return launch_sgd_persistent(emb, head, tail, eps, next_s, next_n, iscal, fscal, alpha0, gamma,
                               a, b, n_epochs, neg_rate, seed, bar, err, device, s, stat, max_ctas);
}

void launch_add_noise(float *emb, int n, const int *batch, int nb, float noise_scale,
                      uint64_t seed, EmbedScratch &e, cudaStream_t s) {
  if (nb <= 0 || noise_scale == 0.0f || n <= 0) return;
  const int nparts = min(cdiv(n, 256), 256);
  k_xrange_partial<<<nparts, 256, 0, s>>>(emb, n, e.partial);
  note_launch();
  k_add_noise<<<cdiv(nb * 2, 256), 256, 0, s>>>(emb, batch, nb, e.partial, nparts,
                                                noise_scale, seed);
  note_launch();
}

void launch_heuristic(const uint32_t *pub_idx, const float *pub_dist, int n, int k,
                      int euclidean, const int *unsel, int nu, float *emb,
                      EmbedScratch &e, cudaStream_t s) {
  if (nu <= 0 || n <= 0 || k <= 0) return;
  cudaMemcpyAsync(e.snap, emb, sizeof(float) * 2 * (size_t)n, cudaMemcpyDeviceToDevice, s);
  k_heuristic<<<cdiv(nu, 128), 128, 0, s>>>(pub_idx, pub_dist, n, k, euclidean, e.sigma,
                                            e.rho, unsel, nu, e.snap, emb);
  note_launch();
}

}  // namespace gm
