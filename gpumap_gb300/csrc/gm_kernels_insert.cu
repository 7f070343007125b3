// Insertion phase: NN-Descent insertion of a contiguous batch of new rows.
// Restates the reference's insertion_kernel.cuh (run_insertion, :926-1095)
// with a deterministic reverse step and a canonical FP32 distance.
#include <algorithm>

#include "gm_common.cuh"
#include "gm_kernels.h"

namespace gm {

namespace {

// ||x||^2 for each batch row by a sequential fma chain over the features.
// Cosine: normalises the row in place first and stores 1.0
// (reference: preprocess_l2_norms_kernel, insertion_kernel.cuh:31-81).
// Squared norms of kNormRows rows per CTA: the rows are staged in shared
// memory a chunk of up to kNormChunk features at a time by float4 loads of
// all threads (rows are 16-byte aligned, ld a multiple of 4), then lanes
// 0..kNormRows-1 of warp 0 run the sequential fma chains.  Cosine rows are
// normalised in place, and snorms gets sqrt(norm) rounded up.
constexpr int kNormRows = 8, kNormChunk = 1024;
__global__ void __launch_bounds__(256)
    k_row_norms(float *X, float *norms, float *snorms, int ld, int d, int row0, int nrows,
                int cosine) {
  __shared__ __align__(16) float tile[kNormRows][kNormChunk + 4];
  __shared__ float s_scale[kNormRows];
  const int r0 = blockIdx.x * kNormRows;
  const int rows = min(kNormRows, nrows - r0);
  const int tid = threadIdx.x, lane = tid & 31;
  float acc = 0.0f;
  for (int c0 = 0; c0 < d; c0 += kNormChunk) {
    const int w = min(kNormChunk, d - c0);
    const int w4 = (w + 3) >> 2;  // float4 columns (the row padding is zero)
    for (int r = 0; r < rows; ++r) {
      const float4 *src = reinterpret_cast<const float4 *>(X + (size_t)(row0 + r0 + r) * ld + c0);
      for (int c = tid; c < w4; c += blockDim.x)
        *reinterpret_cast<float4 *>(&tile[r][4 * c]) = src[c];
    }
    __syncthreads();
    if (tid < rows)
      for (int c = 0; c < w; ++c) {
        const float v = tile[lane][c];
        acc = __fmaf_rn(v, v, acc);
      }
    __syncthreads();
  }
  if (tid < rows) {
    const size_t row = (size_t)(row0 + r0 + lane);
    float nv = acc;
    s_scale[lane] = 0.0f;
    if (cosine) {
      s_scale[lane] = __fsqrt_rn(acc);
      nv = 1.0f;
    }
    norms[row] = nv;
    snorms[row] = __fsqrt_ru(nv);
  }
  __syncthreads();
  if (cosine) {
    for (int r = 0; r < rows; ++r) {
      const float nrm = s_scale[r];
      if (!(nrm > 0.0f)) continue;
      float *x = X + (size_t)(row0 + r0 + r) * ld;
      for (int c = tid; c < d; c += blockDim.x) x[c] = __fdiv_rn(x[c], nrm);
    }
  }
}

__device__ __forceinline__ bool contains(const int *a, int m, int v) {
  for (int i = 0; i < m; ++i)
    if (a[i] == v) return true;
  return false;
}

// Random unique initial neighbours: up to 16 from the recent window
// [window_start, n), the rest from [0, n); distances FLT_MAX
// (reference: initialize_random_neighbors_kernel, insertion_kernel.cuh:170-248).
__global__ void k_random_init(Key *g_key, int row0, int nrows, int n, int window_start,
                              uint64_t seed) {
  const int rl = blockIdx.x * blockDim.x + threadIdx.x;
  if (rl >= nrows) return;
  const int gid = row0 + rl;
  Key *row = g_key + (size_t)gid * kListW;
  if (n <= 1) {
    for (int i = 0; i < kListW; ++i) row[i] = kEmptyKey;
    return;
  }
  Philox g;
  philox_init(g, seed, (uint32_t)gid, kTagInitNeighbors);
  const int max_fill = min(kListW, n - 1);
  const int wsize = n - window_start;
  const int wquota = min(kListW / 2, max(0, wsize - 1));
  int filled[kListW];
  int f = 0;
  int att = 0;
  const int max_att = wquota * 16;
  while (f < wquota && att < max_att) {
    ++att;
    const int c = window_start + (int)(philox_next(g) % (uint32_t)wsize);
    if (c == gid || contains(filled, f, c)) continue;
    filled[f++] = c;
  }
  // Full-range phase; bounded, then a deterministic sweep as a fallback.
  for (uint32_t a = 0; f < max_fill && a < (1u << 20); ++a) {
    const int c = (int)(philox_next(g) % (uint32_t)n);
    if (c == gid || contains(filled, f, c)) continue;
    filled[f++] = c;
  }
  for (int c = 0; f < max_fill && c < n; ++c) {
    if (c == gid || contains(filled, f, c)) continue;
    filled[f++] = c;
  }
  for (int i = 0; i < f; ++i) row[i] = make_key(FLT_MAX, filled[i]);
  for (int i = f; i < kListW; ++i) row[i] = kEmptyKey;
}

// Two-hop candidates, one warp per batch row.  Position p = kk*k + j visits
// slot kk of neighbour j (round robin); a position is kept if its id is in
// range, not self, not a current neighbour and its first occurrence; the
// first 256 kept positions in order are the candidates
// (reference: sample_forward_candidates_kernel, insertion_kernel.cuh:250-321).
constexpr int kSampWarps = 4;
__global__ void k_sample_candidates(const Key *g_key, int row0, int nrows, int n,
                                    int k, int *cand, int *cand_cnt) {
  extern __shared__ int smem_sc[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = blockIdx.x * kSampWarps + warp;
  if (rl >= nrows) return;
  const int P = k * k;
  int *cv = smem_sc + warp * (kListW + P);
  int *nb = cv + P;
  const int gid = row0 + rl;
  if (lane < k) {
    const int e = key_id(g_key[(size_t)gid * kListW + lane]);
    nb[lane] = (e >= 0 && e < n) ? e : kIdSentinel;
  }
  __syncwarp();
  for (int p = lane; p < P; p += 32) {
    const int kk = p / k, j = p - kk * k;
    const int nbr = nb[j];
    int c = -1;
    if (nbr != kIdSentinel) {
      const int e = key_id(g_key[(size_t)nbr * kListW + kk]);
      if ((uint32_t)e < (uint32_t)n && e != gid) {
        bool isnb = false;
        for (int q = 0; q < k; ++q) isnb |= (nb[q] == e);
        if (!isnb) c = e;
      }
    }
    cv[p] = c;
  }
  __syncwarp();
  int *out = cand + (size_t)rl * kMaxCand;
  int base = 0;
  for (int p0 = 0; p0 < P && base < kMaxCand; p0 += 32) {
    const int p = p0 + lane;
    bool keep = false;
    if (p < P) {
      const int c = cv[p];
      if (c >= 0) {
        keep = true;
        for (int q = 0; q < p; ++q)
          if (cv[q] == c) {
            keep = false;
            break;
          }
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    const int idx = base + __popc(bal & ((1u << lane) - 1u));
    if (keep && idx < kMaxCand) out[idx] = cv[p];
    base += __popc(bal);
  }
  const int cnt = min(base, kMaxCand);
  for (int i = cnt + lane; i < kMaxCand; i += 32) out[i] = -1;
  if (lane == 0) cand_cnt[rl] = cnt;
}

// Candidate distances, one CTA per batch row and one thread per candidate.
// Feature chunks of 32 are staged in shared memory; each thread runs the
// sequential fma chain over the features (canonical distance)
// (reference: compute_candidate_distances_kernel, insertion_kernel.cuh:337-405).
constexpr int kDistChunk = 32;
__global__ void __launch_bounds__(256) k_candidate_dists(
    const float *X, const float *norms, int ld, int d, int row0,
    const int *cand, const int *cand_cnt, float *cand_dist, unsigned long long *stat) {
  __shared__ float As[kDistChunk];
  __shared__ float Bs[kMaxCand][kDistChunk + 1];
  const int rl = blockIdx.x, t = threadIdx.x;
  const int gid = row0 + rl;
  const int cnt = cand_cnt[rl];
  if (cnt == 0) {
    cand_dist[(size_t)rl * kMaxCand + t] = -1.0f;
    return;
  }
  const int *cl = cand + (size_t)rl * kMaxCand;
  const int mycand = (t < cnt) ? cl[t] : -1;
  if (t == 0 && stat) atomicAdd(&stat[4], (unsigned long long)(cnt + 1));
  float acc = 0.0f;
  const int q = t & 7;
  for (int k0 = 0; k0 < d; k0 += kDistChunk) {
    const int col = k0 + 4 * q;
    if (t < 8) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (col < ld) v = *reinterpret_cast<const float4 *>(X + (size_t)gid * ld + col);
      As[4 * q] = v.x; As[4 * q + 1] = v.y; As[4 * q + 2] = v.z; As[4 * q + 3] = v.w;
    }
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int r = (t >> 3) + 32 * p;
      if (r < cnt) {
        const int c = cl[r];
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (col < ld) v = __ldg(reinterpret_cast<const float4 *>(X + (size_t)c * ld + col));
        Bs[r][4 * q] = v.x; Bs[r][4 * q + 1] = v.y; Bs[r][4 * q + 2] = v.z; Bs[r][4 * q + 3] = v.w;
      }
    }
    __syncthreads();
    if (t < cnt) {
      const int kend = min(kDistChunk, d - k0);
      for (int kk = 0; kk < kend; ++kk) acc = __fmaf_rn(As[kk], Bs[t][kk], acc);
    }
    __syncthreads();
  }
  float out = -1.0f;
  if (t < cnt) out = canon_dist(norms[gid], norms[mycand], acc);
  cand_dist[(size_t)rl * kMaxCand + t] = out;
}

// Forward merge of a batch row's candidates into its own list.  The
// reference sorts all 256 slots with -1 sentinels first and stops at the
// first sentinel (insertion_kernel.cuh:407-534), so the merge only takes
// effect when all 256 slots hold valid candidates; that rule is kept.
__global__ void k_forward_merge(Key *g_key, int row0, int nrows,
                                const int *cand, const int *cand_cnt,
                                const float *cand_dist) {
  const int rl = blockIdx.x * blockDim.x + threadIdx.x;
  if (rl >= nrows) return;
  if (cand_cnt[rl] < kMaxCand) return;
  const int gid = row0 + rl;
  const int *ci = cand + (size_t)rl * kMaxCand;
  const float *cd = cand_dist + (size_t)rl * kMaxCand;
  int sid[kListW];
  float sd[kListW];
  for (int i = 0; i < kListW; ++i) {
    sid[i] = -1;
    sd[i] = -1.0f;
  }
  // sort_candidates: insertion sort keeping 32, skipping ties with the tail.
  int filled = 0;
  for (int i = 0; i < kMaxCand; ++i) {
    const int id = ci[i];
    const float dv = cd[i];
    if (filled >= kListW && dv >= sd[kListW - 1]) continue;
    int pos = filled < kListW ? filled : kListW - 1;
    while (pos > 0) {
      const bool shift = (dv < sd[pos - 1]) || (dv == sd[pos - 1] && id < sid[pos - 1]);
      if (!shift) break;
      sid[pos] = sid[pos - 1];
      sd[pos] = sd[pos - 1];
      --pos;
    }
    sid[pos] = id;
    sd[pos] = dv;
    if (filled < kListW) ++filled;
  }
  int lid[kListW];
  float ldv[kListW];
  Key *gk = g_key + (size_t)gid * kListW;
  for (int i = 0; i < kListW; ++i) {
    lid[i] = key_id(gk[i]);
    ldv[i] = key_dist(gk[i]);
  }
  bool updated = false;
  for (int i = 0; i < kListW; ++i) {
    const int id = sid[i];
    const float dv = sd[i];
    if (contains(lid, kListW, id)) continue;
    const int tail = kListW - 1;
    if (dv > ldv[tail] || dv < 0.0f || (dv == ldv[tail] && id >= lid[tail])) break;
    int pos = tail;
    while (pos > 0) {
      const bool shift = (dv < ldv[pos - 1]) || (dv == ldv[pos - 1] && id < lid[pos - 1]);
      if (!shift) break;
      lid[pos] = lid[pos - 1];
      ldv[pos] = ldv[pos - 1];
      --pos;
    }
    lid[pos] = id;
    ldv[pos] = dv;
    updated = true;
  }
  if (updated)
    for (int i = 0; i < kListW; ++i) gk[i] = make_key(ldv[i], lid[i]);
}

// Reverse step: each (batch row i, existing candidate j, dist) is offered to
// j's list.  The reference scatters up to 32 arrivals per j and merges them
// (insertion_kernel.cuh:548-640); merging every offer gives the same final
// list as merging the best 32, which is one of the reference's outcomes.
// Offers that cannot change j's list (dist above j's last entry, or i
// already listed) are dropped without taking the lock.
constexpr int kRevWarps = 8;
__global__ void k_reverse_insert(Key *g_key, int *locks, int *dirty, unsigned *err, int row0,
                                 int nrows, const int *cand, const int *cand_cnt,
                                 const float *cand_dist) {
  __shared__ Key s_key[kRevWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = blockIdx.x * kRevWarps + warp;
  if (rl >= nrows) return;
  const int gid = row0 + rl;
  const int cnt = cand_cnt[rl];
  for (int s0 = 0; s0 < cnt; s0 += 32) {
    const int s = s0 + lane;
    int j = -1;
    Key ck = 0;
    bool want = false;
    if (s < cnt) {
      j = cand[(size_t)rl * kMaxCand + s];
      const float dv = cand_dist[(size_t)rl * kMaxCand + s];
      if (j >= 0 && j < row0 && dv >= 0.0f) {
        ck = make_key(dv, gid);
        const Key *row = g_key + (size_t)j * kListW;
        if (ck < __ldcg(&row[kListW - 1])) {
          want = true;
          for (int w = 0; w < kListW; ++w)
            if (__ldcg(&row[w]) == ck) want = false;
        }
      }
    }
    unsigned bal = __ballot_sync(0xffffffffu, want);
    while (bal) {
      const int src = __ffs(bal) - 1;
      bal &= bal - 1u;
      const int tj = __shfl_sync(0xffffffffu, j, src);
      const Key tk = __shfl_sync(0xffffffffu, ck, src);
      if (lane == 0) s_key[warp] = tk;
      __syncwarp();
      const int pos = warp_locked_merge(tj, &s_key[warp], 1, g_key, locks, err);
      if (lane == 0 && pos >= 0 && pos < kListW) dirty[tj] = 1;
      __syncwarp();
    }
  }
}

// Copies the first k working entries into the authoritative list (the
// reference's CPU diff, insertion_kernel.cuh:1034-1089) and publishes the row
// with sentinels for invalid or self ids plus the validity flag in column k
// (impl.cuh:103-144, matrix_utils.cuh:128-174).
__global__ void k_adopt_publish(const Key *g_key, int *knn_ids, float *knn_dists, uint32_t *pub_idx,
                                float *pub_dist, int k, int row0, int nrows,
                                const int *rows, const int *n_rows_dev, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nl = n_rows_dev ? *n_rows_dev : 0;
  if (i >= nrows + nl) return;
  const int row = (i < nrows) ? row0 + i : rows[i - nrows];
  bool valid_row = false;
  for (int j = 0; j < k; ++j) {
    const Key key = g_key[(size_t)row * kListW + j];
    const int e = key_id(key);
    const float dv = key_dist(key);
    knn_ids[(size_t)row * k + j] = e;
    knn_dists[(size_t)row * k + j] = dv;
    const int id = e >= 0 ? e : -e - 1;
    const bool valid = id >= 0 && id < n && id != row;
    valid_row |= valid;
    pub_idx[(size_t)row * (k + 1) + j] = valid ? (uint32_t)id : kPubIdxSentinel;
    pub_dist[(size_t)row * (k + 1) + j] = valid ? dv : FLT_MAX;
  }
  pub_idx[(size_t)row * (k + 1) + k] = valid_row ? 1u : 0u;
}

// New rows' embedding: N(0,1), then (if a pre-batch neighbour has a finite
// distance) the exp(-(d - d_min))-weighted mean of the pre-batch neighbours
// (reference: insertion_kernel.cuh:790-907).
__global__ void k_embed_init(const Key *g_key, float *emb,
                             int k, int row0, int nrows, int n) {
  const int rl = blockIdx.x * blockDim.x + threadIdx.x;
  if (rl >= nrows) return;
  const int row = row0 + rl;
  Philox g;
  philox_init(g, 42ull, (uint32_t)row, kTagInitEmbedding);
  float e0 = gm_normal(g);
  float e1 = gm_normal(g);
  const Key *keys = g_key + (size_t)row * kListW;
  int ids[kListW];
  float ds[kListW];
  float dmin = FLT_MAX;
  for (int j = 0; j < k; ++j) {
    ids[j] = key_id(keys[j]);
    ds[j] = key_dist(keys[j]);
    const int id = ids[j];
    if (id < 0 || id >= n || id >= row0) continue;
    if (ds[j] < dmin) dmin = ds[j];
  }
  if (dmin != FLT_MAX) {
    float wsum = 0.0f, a0 = 0.0f, a1 = 0.0f;
    for (int j = 0; j < k; ++j) {
      const int id = ids[j];
      if (id < 0 || id >= n || id >= row0) continue;
      const float w = gm_expf(-__fsub_rn(ds[j], dmin));
      wsum = __fadd_rn(wsum, w);
      a0 = __fmaf_rn(w, emb[(size_t)id * 2], a0);
      a1 = __fmaf_rn(w, emb[(size_t)id * 2 + 1], a1);
    }
    if (wsum > 0.0f) {
      e0 = __fdiv_rn(a0, wsum);
      e1 = __fdiv_rn(a1, wsum);
    }
  }
  emb[(size_t)row * 2] = e0;
  emb[(size_t)row * 2 + 1] = e1;
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

void launch_row_norms(const DevState &st, int row0, int nrows, cudaStream_t s) {
  if (nrows <= 0) return;
  k_row_norms<<<cdiv(nrows, kNormRows), 256, 0, s>>>(st.X, st.norms, st.snorms, st.ld, st.d,
                                                      row0, nrows, st.cosine);
  note_launch();
}

void launch_random_init(const DevState &st, int row0, int nrows, int n,
                        int window_start, uint64_t seed, cudaStream_t s) {
  if (nrows <= 0) return;
  k_random_init<<<cdiv(nrows, 128), 128, 0, s>>>(st.g_key, row0, nrows, n, window_start,
                                                 seed);
  note_launch();
}

void launch_sample_candidates(const DevState &st, int row0, int nrows, int n,
                              int *cand, int *cand_cnt, cudaStream_t s) {
  if (nrows <= 0) return;
  const size_t smem = (size_t)kSampWarps * (kListW + st.k * st.k) * sizeof(int);
  k_sample_candidates<<<cdiv(nrows, kSampWarps), kSampWarps * 32, smem, s>>>(
      st.g_key, row0, nrows, n, st.k, cand, cand_cnt);
  note_launch();
}

void launch_candidate_dists(const DevState &st, int row0, int nrows,
                            const int *cand, const int *cand_cnt,
                            float *cand_dist, cudaStream_t s) {
  if (nrows <= 0) return;
  k_candidate_dists<<<nrows, 256, 0, s>>>(st.X, st.norms, st.ld, st.d, row0, cand,
                                          cand_cnt, cand_dist, st.stat);
  note_launch();
}

void launch_forward_merge(const DevState &st, int row0, int nrows,
                          const int *cand, const int *cand_cnt,
                          const float *cand_dist, cudaStream_t s) {
  if (nrows <= 0) return;
  k_forward_merge<<<cdiv(nrows, 64), 64, 0, s>>>(st.g_key, row0, nrows, cand, cand_cnt,
                                                 cand_dist);
  note_launch();
}

void launch_reverse_insert(const DevState &st, int row0, int nrows,
                           const int *cand, const int *cand_cnt,
                           const float *cand_dist, cudaStream_t s) {
  if (nrows <= 0 || row0 <= 0) return;
  k_reverse_insert<<<cdiv(nrows, kRevWarps), kRevWarps * 32, 0, s>>>(
      st.g_key, st.locks, st.dirty, st.err, row0, nrows, cand, cand_cnt, cand_dist);
  note_launch();
}

void launch_adopt_and_publish(const DevState &st, int row0, int nrows,
                              const int *rows, const int *n_rows_dev, int n_rows_max,
                              int n, cudaStream_t s) {
  const int total = nrows + n_rows_max;
  if (total <= 0) return;
  k_adopt_publish<<<cdiv(total, 128), 128, 0, s>>>(
      st.g_key, st.knn_ids, st.knn_dists, st.pub_idx, st.pub_dist, st.k, row0, nrows,
      rows, n_rows_dev, n);
  note_launch();
}

void launch_embed_init(const DevState &st, int row0, int nrows, int n,
                       cudaStream_t s) {
  if (nrows <= 0) return;
  k_embed_init<<<cdiv(nrows, 128), 128, 0, s>>>(st.g_key, st.emb, st.k, row0, nrows, n);
  note_launch();
}

}  // namespace gm
