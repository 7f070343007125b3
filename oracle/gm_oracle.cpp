// ORACLE -- test infrastructure only.  A sequential CPU restatement of the
// reference's progressive UMAP cycle (jjmmwon/gpumap: cpp/src/impl.cuh,
// cpp/src/kernels/{insertion,update,embedding}_kernel.cuh, buffers.cuh,
// queue.cuh).  Only the tests, the smoke check and the benchmark's CPU
// baseline load it; the product never does.
//
// Parity pins (the reference has no tests or golden vectors for its CUDA
// path and cannot be built here -- it needs RAFT/RMM and CUDA 12.6 -- so its
// CUDA path is "parity unpinned"; what this file does pin):
//  * The reference draws randomness from cuRAND Philox streams, which are not
//    reproduced.  This restatement and the GPU engine both use
//    Philox4x32-10 (Salmon et al., SC'11) keyed (seed, stream id, purpose).
//  * Distances use one canonical FP32 formula: dot = sequential fma over the
//    features, dist = max(0, (|a|^2 + |b|^2) - 2 dot).
//  * Where the reference keeps an arbitrary subset chosen by atomic arrival
//    order (reverse sample lists capped at 32, reverse insertion candidates
//    capped at 32), the subset is pinned: the 32 smallest source ids for
//    reverse samples; all offers (equivalent to the best 32) for reverse
//    insertion candidates.
//  * exp/log are the Cody-Waite + Taylor / atanh-series float32 functions
//    shared with the GPU, so weights and sigmas are bit-reproducible.
// Compile with -ffp-contract=off (and -mfma on x86_64 so fmaf is inline).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <deque>
#include <numeric>
#include <random>
#include <vector>

namespace {

constexpr int W = 32;      // MAX_NEIGHBORS (buffers.cuh:17)
constexpr int MAXC = 256;  // MAX_CANDIDATES (buffers.cuh:18)
constexpr int NS = 32;     // NUM_SAMPLES (buffers.cuh:19)
constexpr int SENT = 0x7fffffff;

// ---- Philox4x32-10 ------------------------------------------------------
struct Rng {
  uint32_t k0, k1, stream, tag, block, pos, buf[4];
};
void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
void rng_init(Rng &g, uint64_t seed, uint32_t stream, uint32_t tag) {
  g.k0 = (uint32_t)seed;
  g.k1 = (uint32_t)(seed >> 32);
  g.stream = stream;
  g.tag = tag;
  g.block = 0;
  g.pos = 4;
}
uint32_t rng_next(Rng &g) {
  if (g.pos == 4) {
    uint32_t c[4] = {g.stream, g.block, g.tag, 0u};
    philox(c, g.k0, g.k1);
    std::memcpy(g.buf, c, sizeof(c));
    ++g.block;
    g.pos = 0;
  }
  return g.buf[g.pos++];
}
constexpr uint32_t TAG_INIT_NB = 0x11u, TAG_INIT_EMB = 0x22u, TAG_NEG = 0x33u, TAG_NOISE = 0x44u;

// ---- float32 exp / log / pow (same steps as the GPU) ----------------------
float o_expf(float x) {
  if (x != x) return x;
  if (x > 88.72283f) return INFINITY;
  if (x < -87.33654f) return 0.0f;
  const float n = rintf(x * 1.44269504088896341f);
  float r = fmaf(-n, 0.693145751953125f, x);
  r = fmaf(-n, 1.428606765330187e-06f, r);
  float p = 1.0f / 5040.0f;
  p = fmaf(p, r, 1.0f / 720.0f);
  p = fmaf(p, r, 1.0f / 120.0f);
  p = fmaf(p, r, 1.0f / 24.0f);
  p = fmaf(p, r, 1.0f / 6.0f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  return ldexpf(p, (int)n);
}
float o_logf(float x) {
  if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
  if (std::isinf(x)) return x;
  int e;
  float m = frexpf(x, &e);
  if (m < 0.70710678f) {
    m = m * 2.0f;
    e -= 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 1.0f / 9.0f;
  p = fmaf(p, s2, 1.0f / 7.0f);
  p = fmaf(p, s2, 1.0f / 5.0f);
  p = fmaf(p, s2, 1.0f / 3.0f);
  p = fmaf(p, s2, 1.0f);
  const float lm = (2.0f * s) * p;
  const float fe = (float)e;
  return fmaf(fe, 0.693145751953125f, fmaf(fe, 1.428606765330187e-06f, lm));
}
float o_powf(float x, float y) {
  if (y == 0.0f) return 1.0f;
  if (x == 0.0f) return y > 0.0f ? 0.0f : INFINITY;
  return o_expf(y * o_logf(x));
}
float o_normal(Rng &g) {
  for (int a = 0; a < 16; ++a) {
    const float u1 = fmaf((float)(rng_next(g) >> 8), 1.0f / 16777216.0f, 0.5f / 16777216.0f);
    const float u2 = fmaf((float)(rng_next(g) >> 8), 1.0f / 16777216.0f, 0.5f / 16777216.0f);
    const float v1 = 2.0f * u1 - 1.0f, v2 = 2.0f * u2 - 1.0f;
    const float s = v1 * v1 + v2 * v2;
    if (s > 0.0f && s < 1.0f) return v1 * sqrtf((-2.0f * o_logf(s)) / s);
  }
  return 0.0f;
}

bool less_item(float da, int ia, float db, int ib) { return da < db || (da == db && ia < ib); }
int strip(int e) { return e >= 0 ? e : -e - 1; }

// ---- Bloom filter (buffers.cuh:35-137): 4 sets x 512 bits, 4 hashes ------
uint32_t bh0(uint32_t v) { v *= 1103515245u; v += 12345u; v ^= v << 13; v ^= v >> 17; v ^= v << 5; return v; }
uint32_t bh1(uint32_t v) { v *= 1664525u; v += 1013904223u; v ^= v << 13; v ^= v >> 17; v ^= v << 5; return v; }

struct Session {
  size_t N, d, ld;
  int k, metric, neg_rate, max_epoch;
  int precision = 0;  // 1: exact insertion (brute force under the canonical distance)
  float a, b, alpha;
  std::vector<float> X, norms;
  std::vector<int> gid;      // N x 32 working lists
  std::vector<float> gd;
  std::vector<int> dirty;
  std::vector<int> kid;      // N x k authoritative lists (old flag = sign)
  std::vector<float> kd;
  std::vector<uint32_t> pidx;  // N x (k+1)
  std::vector<float> pdist;
  std::vector<float> emb;     // N x 2
  std::vector<uint32_t> bloom;  // N x 64
  bool bloom_clean = true;
  size_t n_ins = 0, ins_head = 0, emb_head = 0, cursor = SIZE_MAX, sweeps = 0;
  std::deque<uint32_t> uq;
  std::vector<char> uq_in;
  std::deque<uint32_t> hist;
  std::mt19937 rng{42};
  bool ins_done = false, upd_done = false, emb_done = false;
  // last embedding call
  std::vector<float> sigma, rho;
  std::vector<int> coo_r, coo_c, t_r, t_c;
  std::vector<float> coo_v, t_e;
  int last_extra = 0, last_maxdeg = 0;
};

// ---- working-list offer (update_kernel.cuh:310-375 semantics) ------------
// An id already listed with a finite distance is skipped (the reference's
// rule).  An id listed as a placeholder -- a random initial neighbour at
// FLT_MAX -- is replaced: the placeholder is removed and the offer inserted.
// The reference skips those too, which makes its result depend on whether
// the placeholder was evicted before the offer arrived (lock order); the
// replacement rule gives the same list for any order of offers.
int list_offer(int *ids, float *ds, int cid, float cd) {
  for (int i = 0; i < W; ++i)
    if (ids[i] == cid) {
      if (ds[i] != FLT_MAX) return W;
      for (int q = i; q < W - 1; ++q) {
        ids[q] = ids[q + 1];
        ds[q] = ds[q + 1];
      }
      ids[W - 1] = SENT;
      ds[W - 1] = FLT_MAX;
      break;
    }
  int pos = W;
  for (int i = 0; i < W; ++i)
    if (less_item(cd, cid, ds[i], ids[i])) {
      pos = i;
      break;
    }
  if (pos == W) return W;
  for (int i = W - 1; i > pos; --i) {
    ids[i] = ids[i - 1];
    ds[i] = ds[i - 1];
  }
  ids[pos] = cid;
  ds[pos] = cd;
  return pos;
}

float dist_of(const Session &S, size_t a, size_t b) {
  const float *xa = &S.X[a * S.ld], *xb = &S.X[b * S.ld];
  float dot = 0.0f;
  for (size_t i = 0; i < S.d; ++i) dot = fmaf(xa[i], xb[i], dot);
  const float v = (S.norms[a] + S.norms[b]) - 2.0f * dot;
  return v <= 0.0f ? 0.0f : v;
}

void publish_row(Session &S, size_t row, size_t n, bool always_flag) {
  const int k = S.k;
  bool valid_row = false;
  for (int j = 0; j < k; ++j) {
    const int id = strip(S.kid[row * k + j]);
    const bool valid = id >= 0 && (size_t)id < n && (size_t)id != row;
    valid_row |= valid;
    S.pidx[row * (k + 1) + j] = valid ? (uint32_t)id : 0xffffffffu;
    S.pdist[row * (k + 1) + j] = valid ? S.kd[row * k + j] : FLT_MAX;
  }
  if (always_flag) S.pidx[row * (k + 1) + k] = valid_row ? 1u : 0u;
  else if (valid_row) S.pidx[row * (k + 1) + k] = 1u;
}

void uq_push(Session &S, uint32_t v) {
  if (v < S.uq_in.size() && !S.uq_in[v]) {
    S.uq_in[v] = 1;
    S.uq.push_back(v);
  }
}
std::vector<uint32_t> uq_pop(Session &S, size_t m) {
  m = std::min(m, S.uq.size());
  std::vector<uint32_t> out;
  for (size_t i = 0; i < m; ++i) {
    out.push_back(S.uq.front());
    S.uq_in[S.uq.front()] = 0;
    S.uq.pop_front();
  }
  return out;
}

// ---- insertion (impl.cuh:220-253; insertion_kernel.cuh:926-1095) ----------
uint32_t insert(Session &S, uint32_t n_ops) {
  const size_t q = S.n_ins - S.ins_head;
  if (q == 0 || n_ops == 0) return 0;
  const size_t B = std::min<size_t>(n_ops, q);
  const size_t row0 = S.ins_head;
  S.ins_head += B;
  S.hist.push_back((uint32_t)row0);
  if (S.hist.size() > 3) S.hist.pop_front();
  const int wstart = (int)S.hist.front();
  const int seed_i = (int)(n_ops * 9973u + (uint32_t)S.n_ins * 7919u);
  const uint64_t seed = (uint64_t)(int64_t)seed_i;
  const int n = (int)S.n_ins;
  const int k = S.k;
  if (!S.bloom_clean) {
    std::fill(S.bloom.begin(), S.bloom.end(), 0u);
    S.bloom_clean = true;
  }
  std::fill(S.dirty.begin(), S.dirty.begin() + n, 0);
  // K1: norms (cosine: normalise, norm column = 1)
  for (size_t r = row0; r < row0 + B; ++r) {
    float *x = &S.X[r * S.ld];
    float acc = 0.0f;
    for (size_t i = 0; i < S.d; ++i) acc = fmaf(x[i], x[i], acc);
    if (S.metric == 1) {
      const float nrm = sqrtf(acc);
      if (nrm > 0.0f)
        for (size_t i = 0; i < S.d; ++i) x[i] = x[i] / nrm;
      S.norms[r] = 1.0f;
    } else {
      S.norms[r] = acc;
    }
  }
  if (S.precision == 1) {
    // exact lists: the 32 smallest (dist, id) keys over the inserted rows
    const size_t n_eff = row0 + B;
    for (size_t r = row0; r < row0 + B; ++r) {
      std::vector<std::pair<float, int>> all;
      for (size_t j = 0; j < n_eff; ++j)
        if (j != r) all.push_back({dist_of(S, r, j), (int)j});
      const size_t m = std::min<size_t>(W, all.size());
      std::partial_sort(all.begin(), all.begin() + (long)m, all.end());
      for (int i = 0; i < W; ++i) {
        S.gid[r * W + i] = i < (int)m ? all[i].second : SENT;
        S.gd[r * W + i] = i < (int)m ? all[i].first : FLT_MAX;
      }
    }
    for (size_t j = 0; j < row0; ++j)
      for (size_t r = row0; r < row0 + B; ++r)
        if (list_offer(&S.gid[j * W], &S.gd[j * W], (int)r, dist_of(S, j, r)) < W) S.dirty[j] = 1;
  } else {
    // K3: random initial neighbours (insertion_kernel.cuh:170-248)
    for (size_t r = row0; r < row0 + B; ++r) {
      int *ids = &S.gid[r * W];
      float *ds = &S.gd[r * W];
      for (int i = 0; i < W; ++i) {
        ids[i] = SENT;
        ds[i] = FLT_MAX;
      }
      if (n <= 1) continue;
      Rng g;
      rng_init(g, seed, (uint32_t)r, TAG_INIT_NB);
      const int max_fill = std::min(W, n - 1);
      const int wsize = n - wstart;
      const int quota = std::min(W / 2, std::max(0, wsize - 1));
      std::vector<int> f;
      auto has = [&](int c) { return std::find(f.begin(), f.end(), c) != f.end(); };
      int att = 0;
      while ((int)f.size() < quota && att < quota * 16) {
        ++att;
        const int c = wstart + (int)(rng_next(g) % (uint32_t)wsize);
        if (c == (int)r || has(c)) continue;
        f.push_back(c);
      }
      for (uint32_t t = 0; (int)f.size() < max_fill && t < (1u << 20); ++t) {
        const int c = (int)(rng_next(g) % (uint32_t)n);
        if (c == (int)r || has(c)) continue;
        f.push_back(c);
      }
      for (int c = 0; (int)f.size() < max_fill && c < n; ++c)
        if (c != (int)r && !has(c)) f.push_back(c);
      for (size_t i = 0; i < f.size(); ++i) ids[i] = f[i];
    }
    std::vector<int> cand(B * MAXC), ccnt(B);
    std::vector<float> cdist(B * MAXC);
    for (int it = 0; it < 10; ++it) {
      // K4: two-hop candidates (insertion_kernel.cuh:250-321)
      for (size_t rl = 0; rl < B; ++rl) {
        const int g = (int)(row0 + rl);
        int nb[W];
        for (int j = 0; j < k; ++j) {
          const int e = S.gid[(size_t)g * W + j];
          nb[j] = (e >= 0 && e < n) ? e : SENT;
        }
        int *out = &cand[rl * MAXC];
        int cnt = 0;
        for (int kk = 0; kk < k && cnt < MAXC; ++kk)
          for (int j = 0; j < k && cnt < MAXC; ++j) {
            if (nb[j] == SENT) continue;
            const int c = S.gid[(size_t)nb[j] * W + kk];
            if ((uint32_t)c >= (uint32_t)n || c == g) continue;
            bool skip = false;
            for (int q2 = 0; q2 < k; ++q2) skip |= (nb[q2] == c);
            for (int q2 = 0; q2 < cnt && !skip; ++q2) skip |= (out[q2] == c);
            if (skip) continue;
            out[cnt++] = c;
          }
        for (int i = cnt; i < MAXC; ++i) out[i] = -1;
        ccnt[rl] = cnt;
      }
      // K5: distances (-1 for empty slots)
      for (size_t rl = 0; rl < B; ++rl)
        for (int s = 0; s < MAXC; ++s)
          cdist[rl * MAXC + s] =
              s < ccnt[rl] ? dist_of(S, row0 + rl, (size_t)cand[rl * MAXC + s]) : -1.0f;
      // K6: forward merge; -1 sentinels sort first and stop the merge, so only
      // rows with all 256 slots valid change (insertion_kernel.cuh:407-534)
      for (size_t rl = 0; rl < B; ++rl) {
        const int *ci = &cand[rl * MAXC];
        const float *cd = &cdist[rl * MAXC];
        int sid[W];
        float sd[W];
        for (int i = 0; i < W; ++i) {
          sid[i] = -1;
          sd[i] = -1.0f;
        }
        int filled = 0;
        for (int i = 0; i < MAXC; ++i) {
          const int id = ci[i];
          const float dv = cd[i];
          if (filled >= W && dv >= sd[W - 1]) continue;
          int pos = filled < W ? filled : W - 1;
          while (pos > 0 && (dv < sd[pos - 1] || (dv == sd[pos - 1] && id < sid[pos - 1]))) {
            sid[pos] = sid[pos - 1];
            sd[pos] = sd[pos - 1];
            --pos;
          }
          sid[pos] = id;
          sd[pos] = dv;
          if (filled < W) ++filled;
        }
        int *li = &S.gid[(row0 + rl) * W];
        float *lf = &S.gd[(row0 + rl) * W];
        int nl[W];
        float nd[W];
        std::memcpy(nl, li, sizeof(nl));
        std::memcpy(nd, lf, sizeof(nd));
        bool upd = false;
        for (int i = 0; i < W; ++i) {
          const int id = sid[i];
          const float dv = sd[i];
          bool in = false;
          for (int q2 = 0; q2 < W; ++q2) in |= (nl[q2] == id);
          if (in) continue;
          if (dv > nd[W - 1] || dv < 0.0f || (dv == nd[W - 1] && id >= nl[W - 1])) break;
          int pos = W - 1;
          while (pos > 0 && (dv < nd[pos - 1] || (dv == nd[pos - 1] && id < nl[pos - 1]))) {
            nl[pos] = nl[pos - 1];
            nd[pos] = nd[pos - 1];
            --pos;
          }
          nl[pos] = id;
          nd[pos] = dv;
          upd = true;
        }
        if (upd) {
          std::memcpy(li, nl, sizeof(nl));
          std::memcpy(lf, nd, sizeof(nd));
        }
      }
      // K7/K8: reverse offers into existing rows (< row0)
      if (row0 > 0)
        for (size_t rl = 0; rl < B; ++rl)
          for (int s = 0; s < ccnt[rl]; ++s) {
            const int j = cand[rl * MAXC + s];
            const float dv = cdist[rl * MAXC + s];
            if (j < 0 || (size_t)j >= row0 || dv < 0.0f) continue;
            if (list_offer(&S.gid[(size_t)j * W], &S.gd[(size_t)j * W], (int)(row0 + rl), dv) < W)
              S.dirty[j] = 1;
          }
    }
  }
  // CPU diff + publish (insertion_kernel.cuh:1034-1089; impl.cuh:103-144)
  std::vector<uint32_t> affected;
  for (size_t r = row0; r < row0 + B; ++r) affected.push_back((uint32_t)r);
  for (size_t r = 0; r < row0; ++r)
    if (S.dirty[r]) affected.push_back((uint32_t)r);
  for (uint32_t r : affected) {
    for (int j = 0; j < k; ++j) {
      S.kid[(size_t)r * k + j] = S.gid[(size_t)r * W + j];
      S.kd[(size_t)r * k + j] = S.gd[(size_t)r * W + j];
    }
    publish_row(S, r, (size_t)n, true);
  }
  // K9/K10 embedding init (insertion_kernel.cuh:790-907)
  for (size_t r = row0; r < row0 + B; ++r) {
    Rng g;
    rng_init(g, 42ull, (uint32_t)r, TAG_INIT_EMB);
    float e0 = o_normal(g), e1 = o_normal(g);
    const int *ids = &S.gid[r * W];
    const float *ds = &S.gd[r * W];
    float dmin = FLT_MAX;
    for (int j = 0; j < k; ++j) {
      const int id = ids[j];
      if (id < 0 || id >= n || (size_t)id >= row0) continue;
      if (ds[j] < dmin) dmin = ds[j];
    }
    if (dmin != FLT_MAX) {
      float ws = 0.0f, a0 = 0.0f, a1 = 0.0f;
      for (int j = 0; j < k; ++j) {
        const int id = ids[j];
        if (id < 0 || id >= n || (size_t)id >= row0) continue;
        const float w = o_expf(-(ds[j] - dmin));
        ws = ws + w;
        a0 = fmaf(w, S.emb[(size_t)id * 2], a0);
        a1 = fmaf(w, S.emb[(size_t)id * 2 + 1], a1);
      }
      if (ws > 0.0f) {
        e0 = a0 / ws;
        e1 = a1 / ws;
      }
    }
    S.emb[r * 2] = e0;
    S.emb[r * 2 + 1] = e1;
  }
  for (uint32_t v : affected) uq_push(S, v);
  return (uint32_t)B;
}

// ---- one local-join round (update_kernel.cuh:689-1054) ---------------------
size_t update_round(Session &S, std::vector<uint32_t> batch, std::vector<uint32_t> &affected) {
  std::sort(batch.begin(), batch.end());
  batch.erase(std::unique(batch.begin(), batch.end()), batch.end());
  const int n = (int)S.n_ins, k = S.k;
  std::vector<int> fn((size_t)n * NS), fo((size_t)n * NS), rn((size_t)n * NS), ro((size_t)n * NS);
  std::vector<int> xn(n, 0), xo(n, 0), yn(n, 0), yo(n, 0);
  std::fill(S.dirty.begin(), S.dirty.begin() + n, 0);
  // sample_graph (update_kernel.cuh:750-807)
  for (uint32_t row : batch) {
    int *list = &S.kid[(size_t)row * k];
    uint32_t *bits = &S.bloom[(size_t)row * 64];
    for (int j = 0; j < k; ++j) {
      const int e = list[j];
      const int id = strip(e);
      if ((uint32_t)id >= (uint32_t)n) continue;
      if (e < 0) {
        const uint32_t key = (uint32_t)id, base = (key % 4u) * 512u;
        uint32_t h = bh0(key);
        bool present = true;
        for (int t = 0; t < 4 && present; ++t) {
          if (t) h += bh1(key);
          const uint32_t bit = base + h % 512u;
          present = (bits[bit >> 5] >> (bit & 31u)) & 1u;
        }
        if (present) continue;
        if (xo[row] < NS) fo[(size_t)row * NS + xo[row]++] = id;
      } else if (xn[row] < NS) {
        list[j] = -id - 1;
        fn[(size_t)row * NS + xn[row]++] = id;
        const uint32_t key = (uint32_t)id, base = (key % 4u) * 512u;
        uint32_t h = bh0(key);
        for (int t = 0; t < 4; ++t) {
          if (t) h += bh1(key);
          const uint32_t bit = base + h % 512u;
          bits[bit >> 5] |= 1u << (bit & 31u);
        }
      }
      if (xo[row] == NS && xn[row] == NS) break;
    }
  }
  S.bloom_clean = false;
  // reverse samples, the 32 smallest source ids (add_rev_edges_kernel, :122-146)
  for (int which = 0; which < 2; ++which) {
    const std::vector<int> &f = which ? fo : fn;
    const std::vector<int> &x = which ? xo : xn;
    std::vector<int> &rv = which ? ro : rn;
    std::vector<int> &y = which ? yo : yn;
    for (uint32_t row : batch)  // ascending source order
      for (int s = 0; s < x[row]; ++s) {
        const int j = f[(size_t)row * NS + s];
        if (j < 0 || j >= n) continue;
        if (y[j] < NS) rv[(size_t)j * NS + y[j]++] = (int)row;
      }
  }
  // local join (update_kernel.cuh:377-687)
  for (int u = 0; u < n; ++u) {
    if (xn[u] + yn[u] == 0) continue;
    std::vector<int> N, O;
    for (int s = 0; s < xn[u]; ++s) N.push_back(fn[(size_t)u * NS + s]);
    const size_t nf = N.size();
    for (int s = 0; s < yn[u]; ++s) {
      const int v = rn[(size_t)u * NS + s];
      if (std::find(N.begin(), N.begin() + (long)nf, v) == N.begin() + (long)nf) N.push_back(v);
    }
    for (int s = 0; s < xo[u]; ++s) O.push_back(fo[(size_t)u * NS + s]);
    const size_t of = O.size();
    for (int s = 0; s < yo[u]; ++s) {
      const int v = ro[(size_t)u * NS + s];
      if (std::find(O.begin(), O.begin() + (long)of, v) == O.begin() + (long)of) O.push_back(v);
    }
    auto offer = [&](int t, int c, float dv) {
      if (t == c) return;
      const int pos = list_offer(&S.gid[(size_t)t * W], &S.gd[(size_t)t * W], c, dv);
      if (pos < W) S.dirty[t] = std::max(S.dirty[t], pos < k ? 2 : 1);
    };
    for (size_t r = 0; r < N.size(); ++r)
      for (size_t c = 0; c < N.size(); ++c)
        if (r != c) offer(N[r], N[c], dist_of(S, (size_t)N[r], (size_t)N[c]));
    for (size_t r = 0; r < N.size(); ++r)
      for (size_t c = 0; c < O.size(); ++c) {
        const float dv = dist_of(S, (size_t)N[r], (size_t)O[c]);
        offer(N[r], O[c], dv);
        offer(O[c], N[r], dv);
      }
  }
  // update_graph + dirty scan + sort_lists + publish (:810-878, :986-1050)
  size_t edges = 0;
  for (int i = 0; i < n; ++i) {
    int h = 0;
    int *li = &S.kid[(size_t)i * k];
    float *lf = &S.kd[(size_t)i * k];
    for (int j = 0; j < W; ++j) {
      const float nd = S.gd[(size_t)i * W + j];
      if (nd == FLT_MAX) break;
      const int nid = S.gid[(size_t)i * W + j];
      if (nid >= n || nid == i) continue;
      if (nd > lf[k - 1]) continue;
      int idx = k;
      bool dup = false;
      for (int q = 0; q < k; ++q) {
        if (strip(li[q]) == nid) {
          dup = true;
          break;
        }
        if (idx == k && lf[q] > nd) idx = q;
      }
      if (dup || idx == k) continue;
      for (int q = k - 1; q > idx; --q) {
        li[q] = li[q - 1];
        lf[q] = lf[q - 1];
      }
      li[idx] = nid;
      lf[idx] = nd;
      h = 2;
      ++edges;
    }
    h = std::max(h, S.dirty[i]);
    if (h == 0) continue;
    std::vector<std::pair<float, int>> v;
    for (int j = 0; j < k; ++j) v.push_back({lf[j], li[j]});
    std::sort(v.begin(), v.end());
    for (int j = 0; j < k; ++j) {
      lf[j] = v[j].first;
      li[j] = v[j].second;
    }
    if (h == 2) {
      publish_row(S, (size_t)i, (size_t)n, false);
      bool valid_row = false;
      for (int j = 0; j < k; ++j) {
        const int id = strip(li[j]);
        valid_row |= (id >= 0 && id < n && id != i);
      }
      if (valid_row) affected.push_back((uint32_t)i);
    }
  }
  return edges;
}

uint32_t update(Session &S, uint32_t n_ops, size_t &changed) {
  changed = 0;
  const size_t n = S.n_ins;
  if (n_ops == 0 || S.upd_done || n == 0) return 0;
  const size_t thr = (size_t)(0.0001f * (float)n);
  uint32_t left = n_ops;
  while (left > 0) {
    std::vector<uint32_t> batch;
    if ((size_t)left >= n) {
      uq_pop(S, S.uq.size());
      batch.resize(n);
      std::iota(batch.begin(), batch.end(), 0u);
    } else if ((size_t)left >= S.uq.size()) {
      batch = uq_pop(S, S.uq.size());
      std::vector<char> seen(n, 0);
      for (uint32_t v : batch) seen[v] = 1;
      std::uniform_int_distribution<uint32_t> dist(0, (uint32_t)(n - 1));
      uint32_t st = dist(S.rng);
      while (batch.size() < (size_t)left) {
        const uint32_t c = (st++) % (uint32_t)n;
        if (!seen[c]) {
          seen[c] = 1;
          batch.push_back(c);
        }
      }
    } else {
      batch = uq_pop(S, left);
    }
    if (batch.empty()) break;
    const size_t raw = batch.size();
    std::vector<uint32_t> aff;
    changed += update_round(S, batch, aff);
    left -= (uint32_t)raw;
    for (uint32_t v : aff) uq_push(S, v);
    if (S.uq.size() < thr) {
      S.upd_done = (n == S.N);
      break;
    }
  }
  return n_ops - left;
}

// ---- fuzzy simplicial set + scheduling (embedding_kernel.cuh) -------------
struct Embed {
  const uint32_t *pidx;
  const float *pdist;
  int n, k;
  bool euclid;
  uint32_t idx(int row, int c) const { return c == 0 ? (uint32_t)row : pidx[(size_t)row * (k + 1) + c - 1]; }
  float dist(int row, int c) const {
    if (c == 0) return 0.0f;
    const float v = pdist[(size_t)row * (k + 1) + c - 1];
    return euclid ? sqrtf(v > 0.0f ? v : 0.0f) : v;
  }
};
bool valid_d(float v) { return std::isfinite(v) && v >= 0.0f && v < FLT_MAX / 2.0f; }
float memb(float dist, float rho, float sigma) {
  const float dr = dist - rho;
  if (dr <= 0.0f || sigma == 0.0f) return 1.0f;
  const float v = o_expf(-(dr / sigma));
  return v < FLT_MIN ? FLT_MIN : v;
}

// Returns nnz; fills COO, sigma/rho, extras count.
void fuzzy_graph(const Embed &E, const std::vector<int> &batch, std::vector<float> &sigma,
                 std::vector<float> &rho, std::vector<int> &cr, std::vector<int> &cc,
                 std::vector<float> &cv, int &extras, float &mean_out) {
  const int n = E.n, k = E.k;
  // K15 global mean: per 256-item block FP32 tree, blocks summed in order
  const long total = (long)n * k;
  float sum = 0.0f;
  long cnt = 0;
  for (long b0 = 0; b0 < total || (b0 == 0 && total == 0); b0 += 256) {
    float ss[256], sc[256];
    for (int t = 0; t < 256; ++t) {
      ss[t] = 0.0f;
      sc[t] = 0.0f;
      const long g = b0 + t;
      if (g < total) {
        const float raw = E.dist((int)(g / k), (int)(g % k));
        if (raw >= 0.0f && raw < FLT_MAX / 2.0f) {
          ss[t] = raw;
          sc[t] = 1.0f;
        }
      }
    }
    for (int s = 128; s > 0; s >>= 1)
      for (int t = 0; t < s; ++t) {
        ss[t] = ss[t] + ss[t + s];
        sc[t] = sc[t] + sc[t + s];
      }
    sum = sum + ss[0];
    cnt += (long)sc[0];
    if (total == 0) break;
  }
  const float mean = (cnt > 0 && std::isfinite(sum) && sum > 0.0f) ? sum / (float)cnt : 1.0f;
  mean_out = mean;
  // K16 smooth_knn_dist (:135-207), FP64 butterfly sum of the terms
  const double target = std::log2((double)(k - 1));
  sigma.assign(n, 0.0f);
  rho.assign(n, 0.0f);
  for (int row = 0; row < n; ++row) {
    float raw[32], san[32];
    for (int c = 0; c < 32; ++c) {
      raw[c] = c < k ? E.dist(row, c) : 0.0f;
      san[c] = (c < k && valid_d(raw[c])) ? raw[c] : 0.0f;
    }
    float s = 0.0f;
    int start = -1;
    for (int c = 0; c < k; ++c) {
      s = s + san[c];
      if (start < 0 && san[c] > 0.0f) start = c;
    }
    if (start < 0) {
      rho[row] = 0.0f;
      sigma[row] = 1e-3f * mean;
      continue;
    }
    const float row_mean = s / (float)k;
    const float r = raw[start];
    float lo = 0.0f, hi = FLT_MAX, mid = 1.0f;
    for (int it = 0; it < 64; ++it) {
      double v[32];
      for (int l = 0; l < 32; ++l) {
        v[l] = 0.0;
        if (l >= 2 && l < k) {
          const float dj = san[l] - r;
          v[l] = dj > 0.0f ? (double)o_expf(-dj / mid) : 1.0;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        double nv[32];
        for (int l = 0; l < 32; ++l) nv[l] = v[l] + v[l ^ o];
        std::memcpy(v, nv, sizeof(v));
      }
      const double psum = v[0];
      if (std::fabs(psum - target) < (double)1e-5f) break;
      if (psum > target) {
        hi = mid;
        mid = (lo + hi) * 0.5f;
      } else {
        lo = mid;
        mid = (hi == FLT_MAX) ? mid * 2.0f : (lo + hi) * 0.5f;
      }
    }
    if (!std::isfinite(mid) || mid <= 0.0f) mid = 1.0f;
    const float ms = 1e-3f * (r > 0.0f ? row_mean : mean);
    rho[row] = r;
    sigma[row] = mid < ms ? ms : mid;
  }
  // K17 + K18 (:214-320): directed part in batch order, extras in that order
  const int nb = (int)batch.size();
  cr.assign((size_t)nb * k, 0);
  cc.assign((size_t)nb * k, 0);
  cv.assign((size_t)nb * k, 0.0f);
  std::vector<int> er, ec;
  std::vector<float> ev;
  for (int t = 0; t < nb * k; ++t) {
    const int row = batch[t / k], ki = t % k;
    const uint32_t rc = E.idx(row, ki);
    const bool vcol = rc < (uint32_t)n;
    const int col = vcol ? (int)rc : row;
    const float dist = E.dist(row, ki);
    float pij = 0.0f;
    if (vcol && col != row && valid_d(dist)) pij = memb(dist, rho[row], sigma[row]);
    float pji = 0.0f;
    for (int kj = 0; kj < k; ++kj)
      if ((int)E.idx(col, kj) == row) {
        const float dji = E.dist(col, kj);
        if (!valid_d(dji)) break;
        pji = memb(dji, rho[col], sigma[col]);
        break;
      }
    const float w = fmaf(-pij, pji, pij + pji);
    cr[t] = row;
    cc[t] = col;
    cv[t] = w;
    if (pji == 0.0f) {
      er.push_back(col);
      ec.push_back(row);
      ev.push_back(w);
    }
  }
  extras = (int)er.size();
  cr.insert(cr.end(), er.begin(), er.end());
  cc.insert(cc.end(), ec.begin(), ec.end());
  cv.insert(cv.end(), ev.begin(), ev.end());
}

// Edge scheduling (run_optimize_layout, :726-778); returns max degree.
int schedule(int n, const std::vector<int> &cr, const std::vector<int> &cc,
             const std::vector<float> &cv, int n_epochs, float alpha, std::vector<int> &tr,
             std::vector<int> &tc, std::vector<float> &te, float &max_w, float &rounding) {
  max_w = 0.0f;
  for (float v : cv) max_w = std::max(max_w, v);
  tr.clear();
  tc.clear();
  te.clear();
  rounding = 1.0f;
  if (!(max_w > 0.0f)) return 0;
  const float thr = max_w / (float)n_epochs;
  std::vector<int> deg(n, 0);
  for (size_t q = 0; q < cv.size(); ++q) {
    if (!(cv[q] >= thr)) continue;
    const float ns = (float)n_epochs * (cv[q] / max_w);
    tr.push_back(cr[q]);
    tc.push_back(cc[q]);
    te.push_back(ns > 0.0f ? (float)n_epochs / ns : -1.0f);
    deg[cr[q]] += 1;
  }
  int md = 0;
  for (int v : deg) md = std::max(md, v);
  if (!tr.empty() && md > 0) {
    const float max_abs = ((float)md * 4.0f) * std::fabs(alpha);
    const float delta = max_abs / (1.0f - (2.0f * (float)md) * FLT_EPSILON);
    int ex;
    frexpf(delta, &ex);
    rounding = ldexpf(1.0f, ex);
  }
  return md;
}

float fclip(float v) {
  if (!std::isfinite(v)) return 0.0f;
  return std::max(std::min(v, 4.0f), -4.0f);
}
float tgrad(float r, float x) { return (r + x) - r; }

// SGD epochs, edges in order within an epoch (optimize_batch_kernel, :509-589).
void sgd(float *emb, int n, const int *head, const int *tail, const float *eps, int nnz,
         float rounding, float alpha0, float gamma, float a, float b, int n_epochs,
         int neg_rate, uint64_t seed) {
  const float nsr_inv = 1.0f / (float)neg_rate;
  std::vector<float> ns(eps, eps + nnz), nn(nnz);
  for (int q = 0; q < nnz; ++q) nn[q] = eps[q] * nsr_inv;
  float alpha = alpha0;
  for (int ep = 0; ep < n_epochs; ++ep) {
    const float fe = (float)ep;
    const uint64_t sd = seed + (uint64_t)ep;
    for (int row = 0; row < nnz; ++row) {
      if (ns[row] > fe) continue;
      const float e = eps[row], en = e * nsr_inv;
      const int j = head[row], kk = tail[row];
      float c0 = emb[(size_t)j * 2], c1 = emb[(size_t)j * 2 + 1];
      const float o0 = emb[(size_t)kk * 2], o1 = emb[(size_t)kk * 2 + 1];
      const float dx = c0 - o0, dy = c1 - o1;
      const float d2 = dx * dx + dy * dy;
      float attr = 0.0f;
      if (d2 > 0.0f) attr = ((-2.0f * (a * b)) * o_powf(d2, b - 1.0f)) / (a * o_powf(d2, b) + 1.0f);
      float g0 = fclip(attr * dx) * alpha, g1 = fclip(attr * dy) * alpha;
      c0 = c0 + g0;
      c1 = c1 + g1;
      emb[(size_t)kk * 2] += tgrad(rounding, -g0);
      emb[(size_t)kk * 2 + 1] += tgrad(rounding, -g1);
      ns[row] = ns[row] + e;
      const float nv = nn[row];
      const float ratio = (fe - nv) / en;
      const int n_neg = (ratio > 0.0f && ratio < 2147483520.0f) ? (int)ratio : 0;
      if (n_neg > 0) {
        Rng g;
        rng_init(g, sd, (uint32_t)row, TAG_NEG);
        for (int p = 0; p < n_neg; ++p) {
          const int r = (int)(rng_next(g) % (uint32_t)n);
          if (r == j) continue;
          const float q0 = emb[(size_t)r * 2], q1 = emb[(size_t)r * 2 + 1];
          const float ex = c0 - q0, ey = c1 - q1;
          const float d2n = ex * ex + ey * ey;
          float rep = 0.0f;
          if (d2n > 0.0f) rep = ((2.0f * gamma) * b) / ((0.001f + d2n) * (a * o_powf(d2n, b) + 1.0f));
          const float h0 = rep > 0.0f ? fclip(rep * ex) * alpha : 4.0f * alpha;
          const float h1 = rep > 0.0f ? fclip(rep * ey) * alpha : 4.0f * alpha;
          c0 = c0 + h0;
          c1 = c1 + h1;
          g0 = g0 + h0;
          g1 = g1 + h1;
        }
        nn[row] = nv + (float)n_neg * en;
      }
      emb[(size_t)j * 2] += tgrad(rounding, g0);
      emb[(size_t)j * 2 + 1] += tgrad(rounding, g1);
    }
    alpha = alpha0 * (1.0f - (float)ep / (float)n_epochs);
  }
}

// ---- embedding phase (impl.cuh:335-500) ------------------------------------
uint32_t embed(Session &S, uint32_t n_ops) {
  const size_t n = S.n_ins;
  if (n_ops == 0 || n == 0) return 0;
  const size_t total_n = S.N;
  std::vector<int> batch;
  if ((size_t)n_ops >= n) {
    S.emb_head = S.n_ins;
    batch.resize(n);
    std::iota(batch.begin(), batch.end(), 0);
    S.cursor = n - 1;
    if (S.cursor == total_n - 1 && S.upd_done) ++S.sweeps;
  } else {
    for (size_t v = S.emb_head; v < S.n_ins; ++v) batch.push_back((int)v);
    S.emb_head = S.n_ins;
    size_t left = batch.size() >= (size_t)n_ops ? 0 : (size_t)n_ops - batch.size();
    if (left > 0) {
      std::vector<char> seen(n, 0);
      for (int v : batch) seen[v] = 1;
      size_t cur = (S.cursor == SIZE_MAX) ? 0 : (S.cursor + 1) % n;
      for (size_t checked = 0; left > 0 && checked < n; ++checked) {
        if (!seen[cur]) {
          seen[cur] = 1;
          batch.push_back((int)cur);
          S.cursor = cur;
          if (S.cursor == total_n - 1 && S.upd_done) ++S.sweeps;
          --left;
        }
        cur = (cur + 1) % n;
      }
    }
  }
  const int ni = (int)n, k = S.k;
  Embed E{S.pidx.data(), S.pdist.data(), ni, k, S.metric == 0};
  float mean = 0.0f;
  fuzzy_graph(E, batch, S.sigma, S.rho, S.coo_r, S.coo_c, S.coo_v, S.last_extra, mean);
  if (S.sweeps > 2) S.emb_done = S.upd_done;
  // noise (add_embedding_noise, :953-1007)
  {
    float mn = FLT_MAX, mx = -FLT_MAX;
    for (int i = 0; i < ni; ++i) {
      mn = std::min(mn, S.emb[(size_t)i * 2]);
      mx = std::max(mx, S.emb[(size_t)i * 2]);
    }
    const float scale = 0.001f * (mx - mn);
    const uint64_t seed = 42ull ^ (uint64_t)S.sweeps;
    for (int t = 0; t < (int)batch.size() * 2; ++t) {
      Rng g;
      rng_init(g, seed, (uint32_t)t, TAG_NOISE);
      const float z = o_normal(g);
      float &p = S.emb[(size_t)batch[t >> 1] * 2 + (t & 1)];
      p = p + z * scale;
    }
  }
  float max_w = 0.0f, rounding = 1.0f;
  S.last_maxdeg = schedule(ni, S.coo_r, S.coo_c, S.coo_v, S.max_epoch, S.alpha, S.t_r, S.t_c,
                           S.t_e, max_w, rounding);
  if (!S.t_r.empty())
    sgd(S.emb.data(), ni, S.t_r.data(), S.t_c.data(), S.t_e.data(), (int)S.t_r.size(), rounding,
        S.alpha, 1.0f, S.a, S.b, S.max_epoch, S.neg_rate, 42ull);
  // heuristic reposition of unselected rows (:811-894)
  std::vector<char> inb(n, 0);
  for (int v : batch) inb[v] = 1;
  std::vector<float> snap(S.emb.begin(), S.emb.begin() + (long)n * 2);
  for (int row = 0; row < ni; ++row) {
    if (inb[row]) continue;
    float ws = 0.0f, a0 = 0.0f, a1 = 0.0f;
    for (int ki = 0; ki < k; ++ki) {
      const int col = (int)E.idx(row, ki);
      if (col == row) continue;
      const float dist = E.dist(row, ki);
      if (!valid_d(dist)) continue;
      if (col < 0 || col >= ni) continue;
      const float w = memb(dist, S.rho[row], S.sigma[row]);
      ws = ws + w;
      a0 = fmaf(w, snap[(size_t)col * 2], a0);
      a1 = fmaf(w, snap[(size_t)col * 2 + 1], a1);
    }
    if (ws > 0.0f) {
      S.emb[(size_t)row * 2] = a0 / ws;
      S.emb[(size_t)row * 2 + 1] = a1 / ws;
    }
  }
  return (uint32_t)batch.size();
}

}  // namespace

extern "C" {

struct gmo_session {
  Session s;
};

gmo_session *gmo_create(uint64_t n_instances, uint64_t n_features, int k, int metric, float a,
                        float b, float alpha, int neg_rate, int max_epoch, int precision) {
  if (k < 1 || k > 32 || n_features < 1) return nullptr;
  auto *o = new gmo_session();
  Session &S = o->s;
  S.N = n_instances;
  S.d = n_features;
  S.ld = (n_features + 3) / 4 * 4;
  S.k = k;
  S.metric = metric;
  S.a = a;
  S.b = b;
  S.alpha = alpha;
  S.neg_rate = neg_rate;
  S.max_epoch = max_epoch;
  S.precision = precision;
  const size_t N = std::max<size_t>(n_instances, 1);
  S.X.assign(N * S.ld, 0.0f);
  S.norms.assign(N, 0.0f);
  S.gid.assign(N * W, SENT);
  S.gd.assign(N * W, FLT_MAX);
  S.dirty.assign(N, 0);
  S.kid.assign(N * k, SENT);
  S.kd.assign(N * k, FLT_MAX);
  S.pidx.assign(N * (k + 1), 0xffffffffu);
  S.pdist.assign(N * (k + 1), FLT_MAX);
  S.emb.assign(N * 2, 0.0f);
  S.bloom.assign(N * 64, 0u);
  S.uq_in.assign(N, 0);
  return o;
}

void gmo_destroy(gmo_session *o) { delete o; }

int gmo_append(gmo_session *o, const float *rows, uint64_t n_rows, uint64_t n_cols) {
  Session &S = o->s;
  if (n_rows == 0) return 0;
  if (n_cols != S.d) return -2;
  if (S.n_ins + n_rows > S.N) return -3;
  for (uint64_t r = 0; r < n_rows; ++r)
    std::memcpy(&S.X[(S.n_ins + r) * S.ld], rows + r * n_cols, n_cols * sizeof(float));
  S.n_ins += n_rows;
  return 0;
}

// result_out (15): ops x3, completed x3, n_inserted, changed edges,
// pending, ins queue, upd queue, emb queue, (unused) x3
int gmo_run(gmo_session *o, uint32_t ni, uint32_t nu, uint32_t ne, int64_t *res) {
  Session &S = o->s;
  int64_t r[15] = {0};
  if (!S.ins_done) {
    r[0] = insert(S, ni);
    S.ins_done = (S.ins_head == S.n_ins) && S.n_ins == S.N;
  }
  if (nu != 0 && !S.upd_done) {
    size_t ch = 0;
    r[1] = update(S, nu, ch);
    r[7] = (int64_t)ch;
  }
  if (ne != 0 && S.n_ins != 0 && !S.emb_done) r[2] = embed(S, ne);
  r[3] = S.ins_done;
  r[4] = S.upd_done;
  r[5] = S.emb_done;
  r[6] = (int64_t)S.n_ins;
  r[8] = (int64_t)S.n_ins;
  r[9] = (int64_t)(S.n_ins - S.ins_head);
  r[10] = (int64_t)S.uq.size();
  r[11] = (int64_t)S.n_ins;
  if (res) std::memcpy(res, r, sizeof(r));
  return 0;
}

// Buffer ids as in include/gpumap_gb300_ops.h (GM_BUF_*).
int gmo_copy(gmo_session *o, int which, void *out, uint64_t bytes) {
  Session &S = o->s;
  const void *src = nullptr;
  size_t cap = 0;
  switch (which) {
    case 0: src = S.gid.data(); cap = S.gid.size() * 4; break;
    case 1: src = S.gd.data(); cap = S.gd.size() * 4; break;
    case 2: src = S.kid.data(); cap = S.kid.size() * 4; break;
    case 3: src = S.kd.data(); cap = S.kd.size() * 4; break;
    case 4: src = S.norms.data(); cap = S.norms.size() * 4; break;
    case 5: src = S.bloom.data(); cap = S.bloom.size() * 4; break;
    case 6: src = S.sigma.data(); cap = S.sigma.size() * 4; break;
    case 7: src = S.rho.data(); cap = S.rho.size() * 4; break;
    case 8: src = S.coo_r.data(); cap = S.coo_r.size() * 4; break;
    case 9: src = S.coo_c.data(); cap = S.coo_c.size() * 4; break;
    case 10: src = S.coo_v.data(); cap = S.coo_v.size() * 4; break;
    case 11: src = S.t_r.data(); cap = S.t_r.size() * 4; break;
    case 12: src = S.t_c.data(); cap = S.t_c.size() * 4; break;
    case 13: src = S.t_e.data(); cap = S.t_e.size() * 4; break;
    case 14: src = S.X.data(); cap = S.X.size() * 4; break;
    case 15: src = S.pidx.data(); cap = S.pidx.size() * 4; break;
    case 16: src = S.pdist.data(); cap = S.pdist.size() * 4; break;
    case 17: src = S.emb.data(); cap = S.emb.size() * 4; break;
    default: return -1;
  }
  if (bytes > cap) return -1;
  if (bytes) std::memcpy(out, src, bytes);
  return 0;
}

uint64_t gmo_size(gmo_session *o, int which) {
  Session &S = o->s;
  switch (which) {
    case 6: case 7: return S.sigma.size() * 4;
    case 8: case 9: case 10: return S.coo_r.size() * 4;
    case 11: case 12: case 13: return S.t_r.size() * 4;
    default: return 0;
  }
}

int gmo_scalars(gmo_session *o, int64_t *out, int n) {
  Session &S = o->s;
  const int64_t v[11] = {(int64_t)S.n_ins, (int64_t)S.ins_head, (int64_t)S.emb_head,
                         S.cursor == SIZE_MAX ? -1 : (int64_t)S.cursor, (int64_t)S.sweeps,
                         (int64_t)S.coo_r.size(), S.last_extra, (int64_t)S.t_r.size(),
                         S.last_maxdeg, (int64_t)S.uq.size(), 0};
  for (int i = 0; i < n && i < 11; ++i) out[i] = v[i];
  return 0;
}

int gmo_update_queue(gmo_session *o, uint32_t *out, uint64_t cap, uint64_t *n_out) {
  Session &S = o->s;
  *n_out = S.uq.size();
  uint64_t i = 0;
  for (auto it = S.uq.begin(); it != S.uq.end() && i < cap; ++it, ++i) out[i] = *it;
  return 0;
}

int gmo_fuzzy_schedule(const uint32_t *pub_idx, const float *pub_dist, int64_t n, int32_t k,
                       int32_t euclidean, const int32_t *batch, int64_t nb, int32_t n_epochs,
                       float alpha, int32_t *coo_row, int32_t *coo_col, float *coo_val,
                       int32_t *t_row, int32_t *t_col, float *t_eps, float *sigma, float *rho,
                       int64_t *counts, float *scalars) {
  Embed E{pub_idx, pub_dist, (int)n, k, euclidean != 0};
  std::vector<int> bt(batch, batch + nb), cr, cc, tr, tc;
  std::vector<float> sg, rh, cv, te;
  int extras = 0;
  float mean = 0.0f, max_w = 0.0f, rounding = 1.0f;
  fuzzy_graph(E, bt, sg, rh, cr, cc, cv, extras, mean);
  const int md = schedule((int)n, cr, cc, cv, n_epochs, alpha, tr, tc, te, max_w, rounding);
  std::copy(cr.begin(), cr.end(), coo_row);
  std::copy(cc.begin(), cc.end(), coo_col);
  std::copy(cv.begin(), cv.end(), coo_val);
  std::copy(tr.begin(), tr.end(), t_row);
  std::copy(tc.begin(), tc.end(), t_col);
  std::copy(te.begin(), te.end(), t_eps);
  std::copy(sg.begin(), sg.end(), sigma);
  std::copy(rh.begin(), rh.end(), rho);
  counts[0] = (int64_t)cr.size();
  counts[1] = extras;
  counts[2] = (int64_t)tr.size();
  counts[3] = md;
  scalars[0] = mean;
  scalars[1] = max_w;
  scalars[2] = rounding;
  return 0;
}

int gmo_sgd(float *emb, int64_t n, const int32_t *head, const int32_t *tail, const float *eps,
            int64_t nnz, float rounding, float alpha0, float gamma, float a, float b,
            int32_t n_epochs, int32_t neg_rate, uint64_t seed) {
  sgd(emb, (int)n, head, tail, eps, (int)nnz, rounding, alpha0, gamma, a, b, n_epochs, neg_rate,
      seed);
  return 0;
}

// Runs the fixed push/pop script of oracle/ref_queue_driver.cpp through this
// file's queue rules and writes the same text; tests compare it with the
// reference's own output (tests/golden/queue_golden.txt).
int gmo_queue_script(char *out, uint64_t cap) {
  Session S;
  S.uq_in.assign(64, 0);
  std::deque<uint32_t> iq;
  std::string text;
  unsigned state = 12345u;
  auto next = [&]() {
    state = state * 1664525u + 1013904223u;
    return state >> 8;
  };
  char buf[64];
  for (int step = 0; step < 200; ++step) {
    const unsigned op = next() % 4u;
    if (op < 2) {
      const unsigned m = next() % 40u;
      std::vector<uint32_t> items;
      for (unsigned i = 0; i < m; ++i) items.push_back(next() % 64u);
      for (uint32_t v : items) uq_push(S, v);
      for (unsigned i = 0; i < m; ++i) iq.push_back(step * 100u + i);
      std::snprintf(buf, sizeof(buf), "push %u", m);
      text += buf;
      for (uint32_t v : items) {
        std::snprintf(buf, sizeof(buf), " %u", v);
        text += buf;
      }
      text += "\n";
    } else {
      const unsigned req = next() % 50u;
      auto a = uq_pop(S, req);
      std::snprintf(buf, sizeof(buf), "upop %u", req);
      text += buf;
      for (uint32_t v : a) {
        std::snprintf(buf, sizeof(buf), " %u", v);
        text += buf;
      }
      text += "\n";
      std::snprintf(buf, sizeof(buf), "ipop %u", req);
      text += buf;
      for (unsigned i = 0; i < req && !iq.empty(); ++i) {
        std::snprintf(buf, sizeof(buf), " %u", iq.front());
        text += buf;
        iq.pop_front();
      }
      text += "\n";
    }
  }
  std::snprintf(buf, sizeof(buf), "usize %zu\n", S.uq.size());
  text += buf;
  if (text.size() + 1 > cap) return -1;
  std::memcpy(out, text.c_str(), text.size() + 1);
  return (int)text.size();
}

float gmo_expf(float x) { return o_expf(x); }
float gmo_logf(float x) { return o_logf(x); }
float gmo_powf(float x, float y) { return o_powf(x, y); }
void gmo_philox(uint32_t ctr[4], uint32_t k0, uint32_t k1) { philox(ctr, k0, k1); }
uint32_t gmo_bloom_hash(int which, uint32_t v) { return which ? bh1(v) : bh0(v); }

}  // extern "C"
