// Shared device-side definitions for the GB300 progressive-UMAP engine:
// list widths, status bits, the counter-based RNG, bit-reproducible float
// math, the bounded per-node lock and the warp-cooperative 32-list merge.
//
// Every floating-point expression whose result feeds a comparison on the
// k-NN path is written with explicit round-to-nearest intrinsics and the
// library is compiled with -fmad=false, so the CPU oracle (which uses the same
// formulas with fmaf() and -ffp-contract=off) reproduces it bit for bit.
#pragma once

#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

namespace gm {

// List widths (the reference's buffers.cuh:17-22 values).
constexpr int kListW = 32;        // working neighbour list width (MAX_NEIGHBORS)
constexpr int kMaxCand = 256;     // insertion candidate slots (MAX_CANDIDATES)
constexpr int kSamples = 32;      // forward / reverse sample cap (NUM_SAMPLES)
constexpr int kJoinMax = 64;      // new or old join list cap (MAX_NUM_BI_SAMPLES)
constexpr int kInsertIters = 10;  // insertion NN-Descent iterations
constexpr int kWindowBatches = 3; // recent-window length in batches

constexpr int kIdSentinel = 0x7fffffff;       // INT_MAX: empty list slot
constexpr uint32_t kPubIdxSentinel = 0xffffffffu;

// Device error bits, OR-ed into the session's error word.
constexpr unsigned kDevErrLock = 1u;  // a per-node lock wait ran out
constexpr unsigned kDevErrSpin = 2u;  // another bounded wait ran out
constexpr unsigned kDevErrOverflow = 4u;  // a scratch pool would have overflowed (work skipped)

// Lock wait bound: about a second at the longest back-off.
constexpr uint32_t kLockSpinLimit = 1u << 20;

#define GM_HD __host__ __device__ __forceinline__
#define GM_D __device__ __forceinline__

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11,
// "Parallel random numbers: as easy as 1, 2, 3"): ten rounds of the 4x32
// multiply-xor round with a Weyl key schedule.  A stream is named by
// (key, stream id, purpose tag); draw i comes from block i/4, word i%4.
// ---------------------------------------------------------------------------
struct Philox {
  uint32_t k0, k1, stream, tag, block, pos;
  uint32_t buf[4];
};

GM_HD void philox_block(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                        uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

GM_HD void philox_init(Philox &g, uint64_t seed, uint32_t stream, uint32_t tag) {
  g.k0 = (uint32_t)seed;
  g.k1 = (uint32_t)(seed >> 32);
  g.stream = stream;
  g.tag = tag;
  g.block = 0;
  g.pos = 4;
}

GM_HD uint32_t philox_next(Philox &g) {
  if (g.pos == 4) {
    philox_block(g.stream, g.block, g.tag, 0u, g.k0, g.k1, g.buf);
    ++g.block;
    g.pos = 0;
  }
  return g.buf[g.pos++];
}

// Purpose tags (keep streams for different uses independent).
constexpr uint32_t kTagInitNeighbors = 0x11u;
constexpr uint32_t kTagInitEmbedding = 0x22u;
constexpr uint32_t kTagNegSample = 0x33u;
constexpr uint32_t kTagNoise = 0x44u;

// ---------------------------------------------------------------------------
// Bit-reproducible float32 exp / log / pow.
//   exp: Cody-Waite range reduction x = n*ln2 + r with a two-part ln2, then a
//        degree-7 Taylor polynomial for e^r on |r| <= ln2/2, scaled by 2^n.
//   log: frexp into m*2^e with m in [sqrt(1/2), sqrt(2)), then
//        log(m) = 2*atanh(s), s = (m-1)/(m+1), odd series to s^9.
// Each step is a correctly rounded IEEE operation, so CPU and GPU agree.
// ---------------------------------------------------------------------------
GM_D float gm_expf(float x) {
  if (x != x) return x;
  if (x > 88.72283f) return __int_as_float(0x7f800000);
  if (x < -87.33654f) return 0.0f;
  const float n = rintf(__fmul_rn(x, 1.44269504088896341f));
  float r = __fmaf_rn(-n, 0.693145751953125f, x);
  r = __fmaf_rn(-n, 1.428606765330187e-06f, r);
  float p = 1.0f / 5040.0f;
  p = __fmaf_rn(p, r, 1.0f / 720.0f);
  p = __fmaf_rn(p, r, 1.0f / 120.0f);
  p = __fmaf_rn(p, r, 1.0f / 24.0f);
  p = __fmaf_rn(p, r, 1.0f / 6.0f);
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  // p * 2^n: exponent-field add when the result stays normal (exact, the
  // same value ldexpf gives), ldexpf otherwise
  const int ni = (int)n;
  const unsigned pb = __float_as_uint(p);
  const int ef = (int)((pb >> 23) & 0xffu) + ni;
  if (ef >= 1 && ef <= 254) return __uint_as_float(pb + ((unsigned)ni << 23));
  return ldexpf(p, ni);
}

GM_D float gm_logf(float x) {
  if (!(x > 0.0f)) return (x == 0.0f) ? __int_as_float(0xff800000) : __int_as_float(0x7fc00000);
  if (x == __int_as_float(0x7f800000)) return x;
  // frexpf by bit fields: x = m * 2^e, m in [0.5, 1) (subnormals scaled by
  // 2^23 first, exactly)
  unsigned u = __float_as_uint(x);
  int e = 0;
  if (u < 0x00800000u) {
    u = __float_as_uint(__fmul_rn(x, 8388608.0f));
    e = -23;
  }
  e += (int)(u >> 23) - 126;
  float m = __uint_as_float((u & 0x007fffffu) | 0x3f000000u);
  if (m < 0.70710678f) {
    m = __fmul_rn(m, 2.0f);
    e -= 1;
  }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float s2 = __fmul_rn(s, s);
  float p = 1.0f / 9.0f;
  p = __fmaf_rn(p, s2, 1.0f / 7.0f);
  p = __fmaf_rn(p, s2, 1.0f / 5.0f);
  p = __fmaf_rn(p, s2, 1.0f / 3.0f);
  p = __fmaf_rn(p, s2, 1.0f);
  const float lm = __fmul_rn(__fmul_rn(2.0f, s), p);
  const float fe = (float)e;
  return __fmaf_rn(fe, 0.693145751953125f, __fmaf_rn(fe, 1.428606765330187e-06f, lm));
}

GM_D float gm_powf(float x, float y) {
  if (y == 0.0f) return 1.0f;
  if (x == 0.0f) return (y > 0.0f) ? 0.0f : __int_as_float(0x7f800000);
  return gm_expf(__fmul_rn(y, gm_logf(x)));
}

// Standard normal draw by the Marsaglia polar method (rejection, at most 16
// attempts; the fallback after 16 rejections has probability ~2e-11).
GM_D float gm_normal(Philox &g) {
  for (int a = 0; a < 16; ++a) {
    const float u1 = __fmaf_rn((float)(philox_next(g) >> 8), 1.0f / 16777216.0f, 0.5f / 16777216.0f);
    const float u2 = __fmaf_rn((float)(philox_next(g) >> 8), 1.0f / 16777216.0f, 0.5f / 16777216.0f);
    const float v1 = __fsub_rn(__fmul_rn(2.0f, u1), 1.0f);
    const float v2 = __fsub_rn(__fmul_rn(2.0f, u2), 1.0f);
    const float s = __fadd_rn(__fmul_rn(v1, v1), __fmul_rn(v2, v2));
    if (s > 0.0f && s < 1.0f) {
      const float f = __fsqrt_rn(__fdiv_rn(__fmul_rn(-2.0f, gm_logf(s)), s));
      return __fmul_rn(v1, f);
    }
  }
  return 0.0f;
}

// Canonical squared distance from a sequential fma dot product:
//   dist = max(0, (|a|^2 + |b|^2) - 2*dot)  (reference: insertion_kernel.cuh:400-403)
GM_D float canon_dist(float na, float nb, float dot) {
  const float v = __fsub_rn(__fadd_rn(na, nb), __fmul_rn(2.0f, dot));
  return v <= 0.0f ? 0.0f : v;  // also maps -0 to +0 (key order needs +0)
}

// Lexicographic (dist, id) order used by every neighbour list.
GM_HD bool item_less(float da, int ia, float db, int ib) {
  return (da < db) || (da == db && ia < ib);
}

// ---------------------------------------------------------------------------
// Bounded per-node lock.  Lane 0 spins with back-off; after kLockSpinLimit
// failed attempts it records kDevErrLock and reports failure.
// ---------------------------------------------------------------------------
GM_D bool warp_lock(int *lock, unsigned *err) {
  const int lane = threadIdx.x & 31;
  int ok = 0;
  if (lane == 0) {
    for (uint32_t it = 0; it < kLockSpinLimit; ++it) {
      if (atomicCAS(lock, 0, 1) == 0) {
        ok = 1;
        break;
      }
      __nanosleep(it < 64u ? 32u : 256u);
    }
    if (!ok) atomicOr(err, kDevErrLock);
  }
  // acquire: every lane is ordered after lane 0's successful CAS
  __syncwarp();
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __threadfence();
  return ok != 0;
}

GM_D void warp_unlock(int *lock) {
  // release: all lanes' list stores precede lane 0's fence and unlock
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    __threadfence();
    atomicExch(lock, 0);
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Working-list entries are 64-bit keys: high word = bits of the non-negative
// float distance, low word = id.  Unsigned key order is the lexicographic
// (dist, id) order, and an 8-byte load of one slot is never torn.
// A placeholder is an entry whose distance is FLT_MAX (a random initial
// neighbour); the empty slot is (FLT_MAX, INT_MAX).
// ---------------------------------------------------------------------------
typedef unsigned long long Key;
constexpr uint32_t kFltMaxBits = 0x7f7fffffu;
constexpr Key kEmptyKey = ((Key)kFltMaxBits << 32) | (Key)0x7fffffffu;

GM_HD Key make_key(float d, int id) {
#ifdef __CUDA_ARCH__
  const uint32_t b = __float_as_uint(d);
#else
  uint32_t b;
  __builtin_memcpy(&b, &d, 4);
#endif
  return ((Key)b << 32) | (Key)(uint32_t)id;
}
GM_HD int key_id(Key k) { return (int)(uint32_t)(k & 0xffffffffu); }
GM_D float key_dist(Key k) { return __uint_as_float((uint32_t)(k >> 32)); }
GM_HD bool key_is_placeholder(Key k) { return (uint32_t)(k >> 32) == kFltMaxBits; }

// Offers m candidate keys to node t's 32-wide sorted list under t's lock.
// Per candidate: if its id is listed with a finite distance, nothing
// happens; if its id is listed as a placeholder, the placeholder is removed
// and the candidate inserted; otherwise the candidate is inserted before the
// first entry it is smaller than, dropping the last entry.  (The reference,
// update_kernel.cuh:310-375, skips any listed id; whether a placeholder was
// evicted before its id is offered then depends on lock order.  Replacing
// the placeholder makes the final list independent of the order of offers.)
// Returns the smallest insert position (kListW if nothing changed, -1 if the
// lock wait ran out).
GM_D int warp_locked_merge(int t, const Key *cands, int m, Key *g_key, int *locks,
                           unsigned *err) {
  const int lane = threadIdx.x & 31;
  if (!warp_lock(&locks[t], err)) return -1;
  Key *row = g_key + (size_t)t * kListW;
  Key mine = __ldcg(&row[lane]);
  int minpos = kListW;
  for (int q = 0; q < m; ++q) {
    const Key ck = cands[q];
    const int cid = key_id(ck);
    const unsigned match = __ballot_sync(0xffffffffu, key_id(mine) == cid);
    if (match) {
      const int at = __ffs(match) - 1;
      const Key there = __shfl_sync(0xffffffffu, mine, at);
      if (!key_is_placeholder(there)) continue;
      const Key nxt = __shfl_down_sync(0xffffffffu, mine, 1);
      if (lane >= at) mine = (lane == kListW - 1) ? kEmptyKey : nxt;
    }
    const unsigned msk = __ballot_sync(0xffffffffu, ck < mine);
    if (msk == 0u) continue;
    const int pos = __ffs(msk) - 1;
    const Key prev = __shfl_up_sync(0xffffffffu, mine, 1);
    if (lane > pos) mine = prev;
    else if (lane == pos) mine = ck;
    minpos = min(minpos, pos);
  }
  if (minpos < kListW) __stcg(&row[lane], mine);
  warp_unlock(&locks[t]);
  return minpos;
}

}  // namespace gm
