// Update phase: one NN-Descent local-join round over a batch of rows.
// Restates the reference's UpdateAlgo (update_kernel.cuh:689-1054) with the
// sampling, reverse lists, merge and publish all on the device.
#include <mutex>

#include "gm_common.cuh"
#include "gm_kernels.h"

#include <algorithm>

namespace gm {

namespace {

// Per-row Bloom filter: 4 sets of 512 bits, 4 hashes (reference
// buffers.cuh:35-137).  Row r owns words [r*64, r*64+64).
GM_D uint32_t bloom_h0(uint32_t v) {
  v *= 1103515245u;
  v += 12345u;
  v ^= v << 13;
  v ^= v >> 17;
  v ^= v << 5;
  return v;
}
GM_D uint32_t bloom_h1(uint32_t v) {
  v *= 1664525u;
  v += 1013904223u;
  v ^= v << 13;
  v ^= v >> 17;
  v ^= v << 5;
  return v;
}
GM_D bool bloom_check(const uint32_t *bits, uint32_t key) {
  const uint32_t base = (key % 4u) * 512u;
  uint32_t h = bloom_h0(key);
  const uint32_t h1 = bloom_h1(key);
  for (int i = 0; i < 4; ++i) {
    if (i > 0) h += h1;
    const uint32_t b = base + h % 512u;
    if (!((bits[b >> 5] >> (b & 31u)) & 1u)) return false;
  }
  return true;
}
GM_D void bloom_add(uint32_t *bits, uint32_t key) {
  const uint32_t base = (key % 4u) * 512u;
  uint32_t h = bloom_h0(key);
  const uint32_t h1 = bloom_h1(key);
  for (int i = 0; i < 4; ++i) {
    if (i > 0) h += h1;
    const uint32_t b = base + h % 512u;
    bits[b >> 5] |= (1u << (b & 31u));
  }
}

// New/old samples of each batch row from its authoritative k-list: new
// entries (up to 32) are sampled, marked old and recorded in the Bloom
// filter; old entries the filter has not seen are sampled (up to 32)
// (reference: UpdateAlgo::sample_graph, update_kernel.cuh:750-807).
__global__ void k_sample_graph(int *knn_ids, uint32_t *bloom, const int *batch,
                               int nb, int n, int k, int *fwd_new, int *fwd_old,
                               int4 *sizes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int row = batch[i];
  int *list = knn_ids + (size_t)row * k;
  uint32_t *bits = bloom + (size_t)row * 64;
  int xn = 0, xo = 0;
  for (int j = 0; j < k; ++j) {
    const int e = list[j];
    const bool isnew = e >= 0;
    const int id = isnew ? e : -e - 1;
    if ((uint32_t)id >= (uint32_t)n) continue;
    if (!isnew) {
      if (bloom_check(bits, (uint32_t)id)) continue;
      if (xo < kSamples) fwd_old[(size_t)row * kSamples + xo++] = id;
    } else if (xn < kSamples) {
      list[j] = -id - 1;
      fwd_new[(size_t)row * kSamples + xn++] = id;
      bloom_add(bits, (uint32_t)id);
    }
    if (xo == kSamples && xn == kSamples) break;
  }
  int4 sz = sizes[row];
  sz.x = xn;
  sz.z = xo;
  sizes[row] = sz;
}

GM_D int fwd_count(int4 s, int which) { return which ? s.z : s.x; }

__global__ void k_rev_count(const int *batch, int nb, int n, const int *fwd,
                            const int4 *sizes, int which, int *cnt) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nb * kSamples) return;
  const int i = tid / kSamples, s = tid - i * kSamples;
  const int row = batch[i];
  if (s >= fwd_count(sizes[row], which)) return;
  const int j = fwd[(size_t)row * kSamples + s];
  if (j < 0 || j >= n) return;
  atomicAdd(&cnt[j], 1);
}

__global__ void k_rev_fill(const int *batch, int nb, int n, const int *fwd,
                           const int4 *sizes, int which, const int *off, int *fill,
                           int *csr) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nb * kSamples) return;
  const int i = tid / kSamples, s = tid - i * kSamples;
  const int row = batch[i];
  if (s >= fwd_count(sizes[row], which)) return;
  const int j = fwd[(size_t)row * kSamples + s];
  if (j < 0 || j >= n) return;
  const int pos = off[j] + atomicAdd(&fill[j], 1);
  csr[pos] = row;
}

// Reverse list of j: its sources in ascending id order, capped at the 32
// smallest.  The reference keeps the first 32 atomic arrivals
// (add_rev_edges_kernel, update_kernel.cuh:122-146); ascending-id is one of
// its possible outcomes and makes the round deterministic.
__global__ void k_rev_finalize(int n, const int *cnt, const int *off, const int *csr,
                               int *rev, int4 *sizes, int which) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int c = cnt[j];
  if (c == 0) return;
  int v[kSamples];
  int m = 0;
  const int *src = csr + off[j];
  for (int q = 0; q < c; ++q) {
    const int x = src[q];
    if (m == kSamples && x >= v[kSamples - 1]) continue;
    int pos = (m < kSamples) ? m : kSamples - 1;
    while (pos > 0 && v[pos - 1] > x) {
      v[pos] = v[pos - 1];
      --pos;
    }
    v[pos] = x;
    if (m < kSamples) ++m;
  }
  int *out = rev + (size_t)j * kSamples;
  for (int q = 0; q < m; ++q) out[q] = v[q];
  int4 sz = sizes[j];
  if (which) sz.w = m; else sz.y = m;
  sizes[j] = sz;
}

__global__ void k_join_flags(const int4 *sizes, int n, int *flag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int4 s = sizes[j];
  flag[j] = (s.x + s.y) > 0 ? 1 : 0;
}

// Local join of one node per CTA.  New list N = forward-new + unseen
// reverse-new, old list O = forward-old + unseen reverse-old.  Distances of
// N x (N ++ O) are formed as an FP32 tile with a sequential fma chain per
// pair; every pair is then offered to both endpoints' lists: N members get
// all other N and O members, O members get the N members
// (reference: local_join_kernel, update_kernel.cuh:377-687).
constexpr int kLJThreads = 256;
constexpr int kLJWarps = kLJThreads / 32;
constexpr int kLJKC = 32;
constexpr int kLJR = kJoinMax;      // 64 tile rows (N)
constexpr int kLJC = 2 * kJoinMax;  // 128 tile cols (N ++ O)

// One feature chunk of the node's rows: N (A) and N ++ O (B), feature-major.
struct LJStage {
  float As[kLJKC][kLJR + 4];
  float Bs[kLJKC][kLJC + 4];
};
struct LJSmem {
  int cid[kLJC];
  float nrm[kLJC];
  // two chunk stages (chunk i in stage i & 1: one barrier per chunk), and
  // over them, once the products are done, the node's distance tile
  union {
    LJStage st[2];
    float D[kLJR][kLJC + 1];
  } u;
  Key lst[kLJWarps][kListW];
  Key cb[kLJWarps][kLJC];
  int nN, nC;
};

__global__ void __launch_bounds__(kLJThreads, 3) k_local_join(
    const int *join_nodes, const int *n_join_dev, const int *fwd_new,
    const int *fwd_old, const int *rev_new, const int *rev_old, const int4 *sizes,
    const float *X, const float *norms, int ld, int d, int n, int k, Key *g_key,
    int *locks, int *dirty, unsigned *err, unsigned long long *stat) {
  extern __shared__ __align__(16) unsigned char lj_raw[];
  LJSmem &S = *reinterpret_cast<LJSmem *>(lj_raw);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int n_join = *n_join_dev;
  // Persistent CTAs: each walks the join list with a grid stride.
  for (int bi = blockIdx.x; bi < n_join; bi += gridDim.x) {
    __syncthreads();  // previous node's shared data is no longer read
    const int u = join_nodes[bi];
    if (warp == 0) {
      // join lists built by warp 0, entries in sample order (ballot
      // compaction): N = forward-new ++ reverse-new not already in
      // forward-new, then forward-old ++ reverse-old not in forward-old
      const int4 sz = sizes[u];
      const unsigned lt = (1u << lane) - 1u;
      const int *fn = fwd_new + (size_t)u * kSamples;
      const int *rn = rev_new + (size_t)u * kSamples;
      const int *fo = fwd_old + (size_t)u * kSamples;
      const int *ro = rev_old + (size_t)u * kSamples;
      int v = lane < sz.x ? fn[lane] : -1;
      bool ok = v >= 0 && v < n;
      unsigned bal = __ballot_sync(0xffffffffu, ok);
      if (ok) S.cid[__popc(bal & lt)] = v;
      const int nfn = __popc(bal);
      __syncwarp();
      v = lane < sz.y ? rn[lane] : -1;
      ok = v >= 0 && v < n;
      for (int q = 0; q < nfn && ok; ++q) ok = S.cid[q] != v;
      bal = __ballot_sync(0xffffffffu, ok);
      if (ok) S.cid[nfn + __popc(bal & lt)] = v;
      const int nN = nfn + __popc(bal);
      __syncwarp();
      v = lane < sz.z ? fo[lane] : -1;
      ok = v >= 0 && v < n;
      bal = __ballot_sync(0xffffffffu, ok);
      if (ok) S.cid[nN + __popc(bal & lt)] = v;
      const int nfo = nN + __popc(bal);
      __syncwarp();
      v = lane < sz.w ? ro[lane] : -1;
      ok = v >= 0 && v < n;
      for (int q = nN; q < nfo && ok; ++q) ok = S.cid[q] != v;
      bal = __ballot_sync(0xffffffffu, ok);
      if (ok) S.cid[nfo + __popc(bal & lt)] = v;
      const int nC = nfo + __popc(bal);
      if (lane == 0) {
        S.nN = nN;
        S.nC = nC;
        if (stat && nN > 0) {
          atomicAdd(&stat[0], 1ull);
          atomicAdd(&stat[1], (unsigned long long)nC);
          atomicAdd(&stat[2], (unsigned long long)nN * (unsigned long long)nC);
        }
      }
    }
    __syncthreads();
    const int nN = S.nN, nC = S.nC;
    if (nN == 0) continue;
    for (int c = t; c < nC; c += kLJThreads) S.nrm[c] = norms[S.cid[c]];

    // ---- FP32 distance tile over the node's real extent (rows N, columns
    // N ++ O): one 4 x 4 micro-tile per thread when the tile has at most
    // kLJThreads of them (every node at k <= 16: about 30 x 90), else 4 x 8
    // (at most 16 x 16); the threads past the last micro-tile only stage
    const bool narrow = ((nN + 3) >> 2) * ((nC + 3) >> 2) <= kLJThreads;
    const int mw = narrow ? 4 : 8;
    const int mtc = (nC + mw - 1) / mw;
    const bool active = t < ((nN + 3) >> 2) * mtc;
    const int r0 = active ? (t / mtc) * 4 : 0, c0 = active ? (t % mtc) * mw : 0;
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    // feature chunks: the next chunk's loads are issued before this chunk's
    // products, so their latency overlaps the arithmetic
    float4 pa[2], pb[4];
    auto fetch = [&](int k0) {
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const int f = t + p * kLJThreads;
        const int r = f >> 3, q = f & 7;
        const int col = k0 + 4 * q;
        pa[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < nN && col < ld)
          pa[p] = __ldg(reinterpret_cast<const float4 *>(X + (size_t)S.cid[r] * ld + col));
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int f = t + p * kLJThreads;
        const int r = f >> 3, q = f & 7;
        const int col = k0 + 4 * q;
        pb[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < nC && col < ld)
          pb[p] = __ldg(reinterpret_cast<const float4 *>(X + (size_t)S.cid[r] * ld + col));
      }
    };
    // chunk i is stored in stage i & 1, whose last readers (the products of
    // chunk i - 2) every thread has finished before the barrier of chunk
    // i - 1, so one barrier per chunk orders both uses
    fetch(0);
    int sb = 0;
    for (int k0 = 0; k0 < d; k0 += kLJKC, sb ^= 1) {
      LJStage &G = S.u.st[sb];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const int f = t + p * kLJThreads;
        const int r = f >> 3, q = f & 7;
        G.As[4 * q][r] = pa[p].x; G.As[4 * q + 1][r] = pa[p].y;
        G.As[4 * q + 2][r] = pa[p].z; G.As[4 * q + 3][r] = pa[p].w;
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int f = t + p * kLJThreads;
        const int r = f >> 3, q = f & 7;
        G.Bs[4 * q][r] = pb[p].x; G.Bs[4 * q + 1][r] = pb[p].y;
        G.Bs[4 * q + 2][r] = pb[p].z; G.Bs[4 * q + 3][r] = pb[p].w;
      }
      __syncthreads();
      if (k0 + kLJKC < d) fetch(k0 + kLJKC);
      if (active) {
        const int kend = min(kLJKC, d - k0);
        for (int kk = 0; kk < kend; ++kk) {
          const float4 a = *reinterpret_cast<const float4 *>(&G.As[kk][r0]);
          const float4 b0 = *reinterpret_cast<const float4 *>(&G.Bs[kk][c0]);
          const float av[4] = {a.x, a.y, a.z, a.w};
          const float bv[4] = {b0.x, b0.y, b0.z, b0.w};
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
          if (!narrow) {
            const float4 b1 = *reinterpret_cast<const float4 *>(&G.Bs[kk][c0 + 4]);
            const float bw[4] = {b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][4 + j] = __fmaf_rn(av[i], bw[j], acc[i][4 + j]);
          }
        }
      }
    }
    __syncthreads();  // every product is done before the tile overwrites the stages
    if (active) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int r = r0 + i, c = c0 + j;
          if (j < mw && r < nN && c < nC) S.u.D[r][c] = canon_dist(S.nrm[r], S.nrm[c], acc[i][j]);
        }
    }
    __syncthreads();

    // ---- offer pairs to both endpoints, one target per warp at a time.
    // An offer can only act if it is below the target's last entry and not
    // already listed with this distance; the snapshot (8-byte slots, never
    // torn) filters the rest without taking the lock.
    for (int tt = warp; tt < nC; tt += kLJWarps) {
      const int idt = S.cid[tt];
      S.lst[warp][lane] = __ldcg(&g_key[(size_t)idt * kListW + lane]);
      __syncwarp();
      const Key worst = S.lst[warp][kListW - 1];
      const int ncand = (tt < nN) ? nC : nN;
      int m = 0;
      for (int c0b = 0; c0b < ncand; c0b += 32) {
        const int c = c0b + lane;
        bool pass = false;
        Key ck = 0;
        if (c < ncand && c != tt) {
          const int cidv = S.cid[c];
          const float dv = (tt < nN) ? S.u.D[tt][c] : S.u.D[c][tt];
          ck = make_key(dv, cidv);
          if (cidv != idt && ck < worst) {
            pass = true;
            for (int q = 0; q < kListW; ++q)
              if (S.lst[warp][q] == ck) {
                pass = false;
                break;
              }
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, pass);
        if (pass) S.cb[warp][m + __popc(bal & ((1u << lane) - 1u))] = ck;
        m += __popc(bal);
      }
      __syncwarp();
      if (m > 0) {
        const int pos = warp_locked_merge(idt, S.cb[warp], m, g_key, locks, err);
        if (lane == 0) {
          if (pos >= 0 && pos < kListW) atomicMax(&dirty[idt], pos < k ? 2 : 1);
          if (stat) atomicAdd(&stat[3], 1ull);
        }
      }
      __syncwarp();
    }
  }
}

// update_graph + sort_lists + publish (reference: update_kernel.cuh:810-878,
// 986-1050) for every row, as the reference does: a row whose working list
// did not change this round can still gain an entry, when an id that was a
// placeholder in its k-list (and so skipped as a duplicate) has since been
// pushed out of the k-list.  rows == nullptr means rows 0..n-1.
__global__ void k_merge_publish(const int *rows, const int *n_rows_dev,
                                const Key *g_key, int *knn_ids,
                                float *knn_dists, const int *dirty,
                                uint32_t *pub_idx, float *pub_dist, int k, int n,
                                int *edge_counter, int *report_flag) {
  const int nr = rows ? *n_rows_dev : n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nr; i += gridDim.x * blockDim.x) {
  const int row = rows ? rows[i] : i;
  int lid[kListW];
  float ldv[kListW];
  int *kl = knn_ids + (size_t)row * k;
  float *kd = knn_dists + (size_t)row * k;
  for (int j = 0; j < k; ++j) {
    lid[j] = kl[j];
    ldv[j] = kd[j];
  }
  int h = 0, edges = 0;
  for (int j = 0; j < kListW; ++j) {
    const Key key = g_key[(size_t)row * kListW + j];
    const float nd = key_dist(key);
    if (nd == FLT_MAX) break;
    const int nid = key_id(key);
    if (nid < 0 || nid >= n || nid == row) continue;
    // insert_to_ordered_list (update_kernel.cuh:87-120)
    if (nd > ldv[k - 1]) continue;
    int idx = k;
    bool dup = false;
    for (int q = 0; q < k; ++q) {
      const int e = lid[q];
      if ((e >= 0 ? e : -e - 1) == nid) {
        dup = true;
        break;
      }
      if (idx == k && ldv[q] > nd) idx = q;
    }
    if (dup || idx == k) continue;
    for (int q = k - 1; q > idx; --q) {
      lid[q] = lid[q - 1];
      ldv[q] = ldv[q - 1];
    }
    lid[idx] = nid;
    ldv[idx] = nd;
    h = 2;
    ++edges;
  }
  const int dd = dirty[row];
  if (dd > h) h = dd;
  int report = 0;
  if (h >= 1) {
    // sort_lists: ascending (dist, id_with_flag)
    for (int a = 1; a < k; ++a) {
      const int e = lid[a];
      const float dv = ldv[a];
      int b = a;
      while (b > 0 && (ldv[b - 1] > dv || (ldv[b - 1] == dv && lid[b - 1] > e))) {
        lid[b] = lid[b - 1];
        ldv[b] = ldv[b - 1];
        --b;
      }
      lid[b] = e;
      ldv[b] = dv;
    }
    for (int j = 0; j < k; ++j) {
      kl[j] = lid[j];
      kd[j] = ldv[j];
    }
    if (h == 2) {
      bool valid_row = false;
      for (int j = 0; j < k; ++j) {
        const int e = lid[j];
        const int id = e >= 0 ? e : -e - 1;
        const bool valid = id >= 0 && id < n && id != row;
        valid_row |= valid;
        pub_idx[(size_t)row * (k + 1) + j] = valid ? (uint32_t)id : kPubIdxSentinel;
        pub_dist[(size_t)row * (k + 1) + j] = valid ? ldv[j] : FLT_MAX;
      }
      if (valid_row) {
        pub_idx[(size_t)row * (k + 1) + k] = 1u;
        report = 1;
      }
    }
  }
  report_flag[row] = report;
  if (edges) atomicAdd(edge_counter, edges);
  }
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

void launch_sample_graph(const DevState &st, const UpdScratch &u, const int *batch,
                         int nb, int n, cudaStream_t s) {
  if (nb <= 0) return;
  k_sample_graph<<<cdiv(nb, 128), 128, 0, s>>>(st.knn_ids, st.bloom, batch, nb, n,
                                                st.k, u.fwd_new, u.fwd_old, u.sizes);
  note_launch();
}

void build_reverse(const DevState &st, const UpdScratch &u, const int *batch, int nb,
                   int n, int which, int *tmp, cudaStream_t s) {
  if (nb <= 0 || n <= 0) return;
  const int *fwd = which ? u.fwd_old : u.fwd_new;
  int *rev = which ? u.rev_old : u.rev_new;
  cudaMemsetAsync(u.cnt, 0, sizeof(int) * (size_t)n, s);
  cudaMemsetAsync(u.fill, 0, sizeof(int) * (size_t)n, s);
  const int work = nb * kSamples;
  k_rev_count<<<cdiv(work, 256), 256, 0, s>>>(batch, nb, n, fwd, u.sizes, which, u.cnt);
  note_launch();
  exclusive_scan(u.cnt, u.off, n, tmp, s);
  k_rev_fill<<<cdiv(work, 256), 256, 0, s>>>(batch, nb, n, fwd, u.sizes, which, u.off,
                                            u.fill, u.csr);
  note_launch();
  k_rev_finalize<<<cdiv(n, 128), 128, 0, s>>>(n, u.cnt, u.off, u.csr, rev, u.sizes,
                                              which);
  note_launch();
  (void)st;
}

void launch_local_join(const DevState &st, const UpdScratch &u, const int *join_nodes,
                       const int *n_join_dev, int n_join_max, int n, cudaStream_t s) {
  if (n_join_max <= 0) return;
  const size_t smem = sizeof(LJSmem);
  // per device, once (sessions on several host threads may launch at once)
  static std::mutex mu;
  static int ctas[32] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int grid_ctas = 0;
  if (dev < 32) {
    std::lock_guard<std::mutex> g(mu);
    if (!ctas[dev]) {
      cudaFuncSetAttribute(k_local_join, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      int sms = 0, per_sm = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_local_join, kLJThreads, smem);
      ctas[dev] = std::max(1, sms * std::max(per_sm, 1));
    }
    grid_ctas = ctas[dev];
  }

  const int grid = std::min(n_join_max, grid_ctas > 0 ? grid_ctas : 1024);
  k_local_join<<<grid, kLJThreads, smem, s>>>(
      join_nodes, n_join_dev, u.fwd_new, u.fwd_old, u.rev_new, u.rev_old, u.sizes, st.X,
      st.norms, st.ld, st.d, n, st.k, st.g_key, st.locks, st.dirty, st.err, st.stat);
  note_launch();
}

void launch_join_flags(const UpdScratch &u, int n, int *flag, cudaStream_t s) {
  if (n <= 0) return;
  k_join_flags<<<cdiv(n, 256), 256, 0, s>>>(u.sizes, n, flag);
  note_launch();
}

void launch_merge_publish(const DevState &st, const UpdScratch &u, const int *rows,
                          const int *n_rows_dev, int n_rows_max, int n,
                          int *edge_counter, int *report_flag, cudaStream_t s) {
  if (n_rows_max <= 0) return;
  k_merge_publish<<<std::min(cdiv(n_rows_max, 128), 2048), 128, 0, s>>>(
      rows, n_rows_dev, st.g_key, st.knn_ids, st.knn_dists, st.dirty,
      st.pub_idx, st.pub_dist, st.k, n, edge_counter, report_flag);
  note_launch();
  (void)u;
}

}  // namespace gm
