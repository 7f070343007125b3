// Exact insertion (precision = 1): each insertion batch is compared with
// every inserted row.  Distances are first formed on the 5th-generation tensor
// cores (split-BF16 operands staged by TMA, FP32 accumulators in TMEM), then
// every pair that a rigorous error bound cannot rule out is re-scored with the
// canonical FP32 distance.  Resulting lists are the exact 32 nearest rows
// under the canonical distance, identical to a brute-force CPU computation.
//
// Split BF16: each FP32 value x is stored as hi = bf16(x) and lo = bf16(x - hi)
// (x - hi is exact in FP32), and a.b is formed as hi.hi + hi.lo + lo.hi in one
// FP32 accumulator: three BF16 products per element, relative operand error
// about 3 * 2^-16 instead of 2^-7 for plain BF16.
//
//  k_to_bf16     batch rows -> [hi | lo] shadow rows (each zero padded to dh, a multiple of 64)
//  k_exact_dist  approx D[m][j] = |x_m|^2 + |x_j|^2 - 2 (x_m . x_j)_split
//                (tcgen05.mma kind::f16, M=128 x N=256 x K=16 per instruction),
//                screened as the accumulators are drained (the tile is not
//                stored): per batch row, the columns that may be among its
//                32 nearest; per existing row, the batch rows that may enter
//                its list
//  k_row_threshold  per batch row: its exact threshold from the CTAs' heaps
//  k_row_dists / k_pair_dists   canonical FP32 re-score of the survivors
//  k_row_select / k_col_merge   exact top-32 merges
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <mutex>

#include "gm_common.cuh"
#include "gm_kernels.h"

namespace gm {

namespace {

constexpr int kTM = 128;                       // batch rows per tile (MMA M)
constexpr int kTN = 256;                       // columns per tile (MMA N)
constexpr int kTK = 64;                        // bf16 per K chunk = one 128-byte swizzle row
// A stage holds one K chunk of all four operand halves (A hi | A lo | B hi |
// B lo) and feeds all three products of the split (12 MMAs of K = 16), so a
// byte in flight carries 1.5x the work of one product per stage and B's hi
// half is fetched once instead of twice.
constexpr int kStages = 2;
constexpr int kABytes = kTM * kTK * 2;         // 16 KB
constexpr int kBBytes = kTN * kTK * 2;         // 32 KB
constexpr int kStageBytes = 2 * kABytes + 2 * kBBytes; // 96 KB
// Warp 0 TMA, warp 1 MMA, then the epilogue: one warp group (four warps, one
// per 32-row quarter of the tile) per column share of the tile.  The heap
// pass keeps one group (its per-row heaps cannot be shared); the others run
// four, each on 64 of the tile's 256 columns, so that every scheduler has
// four epilogue warps to hide their latencies with.
__host__ __device__ constexpr int exact_groups(int pass) { return pass == 1 ? 1 : 4; }
__host__ __device__ constexpr int exact_threads(int pass) { return 64 + 128 * exact_groups(pass); }
constexpr int kTmemCols = 512;                 // two 128 x 256 FP32 accumulators
constexpr uint32_t kWaitLimit = 1u << 24;      // bounded mbarrier waits
// epilogue column buffer: the 256 columns' squared norms, bound factors and
// list bars of a tile, double buffered (two tiles), then per buffer sixteen
// per-warp maxima of the norms and bound factors (float bits: both >= 0)
constexpr size_t kEpiBytes = (size_t)2 * 3 * kTN * sizeof(float) + (size_t)2 * 2 * 16 * sizeof(float);
constexpr int kListTop = 32;                   // list width the screen keeps exact
constexpr size_t kHeapBytes = (size_t)kListTop * kTM * sizeof(float);
constexpr size_t kExactSmem = (size_t)kStages * kStageBytes + 1024 + 256 + kEpiBytes + kHeapBytes;
static_assert(kExactSmem <= 232448, "k_exact_dist shared memory above the 227 KB per-CTA limit");

// Instruction descriptor, kind::f16: D=F32 (bits 4-5), A=B=BF16 (7-9, 10-12),
// both K-major (15, 16 = 0), N>>3 at 17-22, M>>4 at 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                            ((uint32_t)(kTN >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);

GM_D uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

GM_D void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
GM_D void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
GM_D void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Waits (bounded) until the phase with the given parity has completed.
GM_D bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

GM_D void tma_load_2d(const CUtensorMap *map, uint64_t *bar, void *dst, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
// The same with an L2 cache policy (createpolicy) for the lines it reads.
GM_D void tma_load_2d_hint(const CUtensorMap *map, uint64_t *bar, void *dst, int x, int y,
                           uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint "
      "[%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}
// Column tiles stream through L2 once per row tile while other kernels of
// the session (the embedding's SGD) work out of L2: their lines go first.
constexpr bool kStreamEvictFirst = true;

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row groups 1024 bytes apart (stride byte offset), descriptor version 1.
GM_D uint64_t sw128_desc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;            // version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

GM_D void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}
GM_D void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
GM_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
GM_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive columns of this thread's lane; the registers are valid after
// tmem_ld_wait (which names them, so that no read of them moves above it)
GM_D void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// One column of this thread's lane, waited for.
GM_D uint32_t tmem_ld1(uint32_t taddr) {
  uint32_t r;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r)
      : "r"(taddr)
      : "memory");
  return r;
}
GM_D void tmem_ld_wait(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

// Batch rows to split BF16 (both halves round to nearest): shadow row =
// hi[0..dh) | lo[0..dh), zero padded past d.
__global__ void k_to_bf16(const float *X, int ld, int d, int dh, int row0, int nrows,
                          __nv_bfloat16 *Xh) {
  const long total = (long)nrows * dh;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const int r = (int)(i / dh), c = (int)(i - (long)r * dh);
    const size_t row = (size_t)(row0 + r);
    const float v = c < d ? X[row * ld + c] : 0.0f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(hi)));
    Xh[row * 2 * dh + c] = hi;
    Xh[row * 2 * dh + dh + c] = lo;
  }
}

// Rigorous bound on |approx - canonical| for one pair, as coef * sqrt(na nb)
// + 2^-21 (na + nb), with coef from exact_bound_coef.  Both distances share
// fl(na + nb); they differ by 2 |v - dot_c| plus the final subtraction's
// rounding (2^-24 of |s - 2v| and of |s - 2 dot_c|, each below 2 (na + nb)
// for any pair within the bound).  sa, sb: sqrt(na), sqrt(nb) rounded up, so
// sa * sb (rounded up) >= sqrt(na nb).
GM_D float pair_bound(float coef, float sa, float sb, float na, float nb) {
  return __fadd_ru(__fmul_ru(coef, __fmul_ru(sa, sb)),
                   __fadd_ru(__fmul_ru(4.8e-7f, __fadd_ru(na, nb)), 1e-30f));
}


// Max-heap of the 32 smallest upper bounds of one row, in shared memory with
// stride kTM (element i of row r at h[i * kTM]).  Pushes x (the caller has
// checked x < the current threshold) and returns the new threshold: the
// largest of the 32 once the heap is full, +inf before.
GM_D float heap_push(float *h, int &cnt, float x) {
  if (cnt < kListTop) {
    int pos = cnt++;
    while (pos > 0) {
      const int up = (pos - 1) >> 1;
      const float pv = h[up * kTM];
      if (pv >= x) break;
      h[pos * kTM] = pv;
      pos = up;
    }
    h[pos * kTM] = x;
    return cnt < kListTop ? __int_as_float(0x7f800000) : h[0];
  }
  int pos = 0;
  for (;;) {
    int c = 2 * pos + 1;
    if (c >= kListTop) break;
    if (c + 1 < kListTop && h[(c + 1) * kTM] > h[c * kTM]) ++c;
    const float cv = h[c * kTM];
    if (cv <= x) break;
    h[pos * kTM] = cv;
    pos = c;
  }
  h[pos * kTM] = x;
  return h[0];
}

// Screen state of one block of batch rows (batch-local row m).
struct TileScreen {
  int tile_count;     // column tiles this pass visits: tile t is column tile t * tile_stride
  int tile_stride;
  float *heaps;       // (m * gridDim.x + CTA) * 32: each CTA's 32 smallest upper bounds of row m
  const float *seed;  // passes 1 and 3: per-row upper bounds from pass 0 (or null)
  float *mins;        // pass 0: m * mins_ld + 8 * t + c: smallest upper bound of row m over
  int mins_ld;        //   the 32 columns of chunk c of sampled tile t
  const float *row_t; // exact per-row thresholds (pass 2)
  int *cand;          // m * cand_ld + i: candidate columns of row m (pass 2)
  long cand_ld;
  int *row_cnt;       // candidates per row (zeroed before pass 2)
  int *pool_j, *pool_m;  // (existing row, batch row) pairs that may enter j's list
  int *pool_counter;
  long pool_cap;
  const Key *g_key;   // working lists (the 32nd entry of an existing row is its bar)
  int n_exist;        // rows [0, n_exist) are the existing rows
  float coef;
  // pass 3: the stored columns of row m seen by CTA c, packed (lower bound
  // bits << 32 | column) with their upper bounds in pre_ub, in segment
  // (m * gridDim.x + c) of pre_cap entries; pre_cnt holds each segment's
  // length and pre_over is set when one would exceed pre_cap
  unsigned long long *pre;
  float *pre_ub;
  int *pre_cnt;
  int pre_cap;
  int *pre_over;
  int col_test;       // pass 1: run the column test (off when pass 3 already did)
  const int *run_if;  // when set, the launch does nothing unless *run_if != 0
};

// Distances of a block of batch rows against all columns, screened as they
// leave the tensor memory (the tile itself is not stored).  grid.y: 128-row
// tiles of the batch; grid.x: CTAs sharing the column tiles.  For every pair
// (batch row m, column j) the epilogue forms D and the bound B (pair_bound);
// its upper bound is D + B and its lower bound D - B.  Past 32 column tiles:
//  Pass 0 (kPass == 0), on an evenly spaced sample of column tiles: per row
//    and 32-column chunk, the smallest upper bound (sc.mins).  The 32nd
//    smallest of a row's chunk minima (k_seed_select) is the largest upper
//    bound of 32 distinct columns, so it bounds the row's 32nd smallest
//    upper bound over all columns from above: the seed.
//  Pass 3 (kPass == 3), all column tiles: every column whose lower bound is
//    at most the seed is stored with its bounds.  Every column whose upper
//    bound is at most the row's exact threshold T (its 32nd smallest upper
//    bound) is among them, so k_pre_select finds T exactly from the stored
//    upper bounds, then keeps the stored columns with lower bound <= T.
//    Column side, for an existing row j: (j, m) goes to the pair pool when
//    D - B is at most the 32nd distance of j's list.
// Up to 32 column tiles, and for a block whose stored columns overflowed:
//  Pass 1 (kPass == 1), all column tiles: every CTA keeps, per row, a
//    max-heap of the 32 smallest upper bounds it sees (at or below the seed
//    when there is one) and stores it to sc.heaps; the 32nd smallest of
//    their union (k_row_threshold) is T, or the seed when smaller.  The
//    column test as in pass 3 (sc.col_test; off after a pass 3).
//  Pass 2 (kPass == 2): the same tiles again; j becomes a candidate of row m
//    when D - B <= T.
// Either way the candidates hold every column whose canonical distance can
// be among m's 32 smallest.  With kKeepD the tile is also written to D (ldD
// columns per row), for tests.
template <int kPass, bool kKeepD>
__global__ void __launch_bounds__(exact_threads(kPass), 1)
    k_exact_dist(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                 int arow0, int nb, int n, int kchunks, int dh, const float *norms,
                 const float *snorms, TileScreen sc, float *D, long ldD, unsigned *err) {
  // a gated launch (the fallback after a pass 3 whose stored columns did
  // not overflow) does nothing: the flag is read before any barrier or
  // tensor memory is set up, by every thread alike
  if (sc.run_if && *sc.run_if == 0) return;
  extern __shared__ __align__(1024) unsigned char raw[];
  unsigned char *base = (unsigned char *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(base + (size_t)kStages * kStageBytes);
  uint64_t *empty = full + kStages;
  uint64_t *tmem_full = empty + kStages;  // [2]: accumulator b holds a finished tile
  uint64_t *tmem_empty = tmem_full + 2;   // [2]: accumulator b has been drained
  uint32_t *tmem_slot = (uint32_t *)(tmem_empty + 2);
  float *epi = (float *)(base + (size_t)kStages * kStageBytes + 256);
  float *heaps = (float *)((unsigned char *)epi + kEpiBytes);

  constexpr int kGroups = exact_groups(kPass);
  constexpr int kEpi = 128 * kGroups;    // epilogue threads
  constexpr int kGroupCols = kTN / kGroups;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.y;
  const int m0 = mt * kTM;  // batch-local first row of this tile

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tmem_full[b], 1);
      mbar_init(&tmem_empty[b], kEpi);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t it = 0;
      uint64_t pol = 0;
      if (kStreamEvictFirst) asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
      for (int t = blockIdx.x; t < sc.tile_count && ok; t += gridDim.x) {
        const int ct = t * sc.tile_stride;
        // kchunks K chunks, each with the hi and lo halves of both operands
        // (x offsets are multiples of 64; lo halves start at x = dh)
        for (int kc = 0; kc < kchunks; ++kc, ++it) {
          const uint32_t s = it % kStages, use = it / kStages;
          if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1)) {
            ok = false;
            break;
          }
          const int kx = kc * kTK;
          unsigned char *a = base + (size_t)s * kStageBytes;
          mbar_expect_tx(&full[s], kStageBytes);
          tma_load_2d(&tm_a, &full[s], a, kx, arow0 + m0);
          tma_load_2d(&tm_a, &full[s], a + kABytes, dh + kx, arow0 + m0);
          if (kStreamEvictFirst) {
            tma_load_2d_hint(&tm_b, &full[s], a + 2 * kABytes, kx, ct * kTN, pol);
            tma_load_2d_hint(&tm_b, &full[s], a + 2 * kABytes + kBBytes, dh + kx, ct * kTN, pol);
          } else {
            tma_load_2d(&tm_b, &full[s], a + 2 * kABytes, kx, ct * kTN);
            tma_load_2d(&tm_b, &full[s], a + 2 * kABytes + kBBytes, dh + kx, ct * kTN);
          }
        }
      }
      if (!ok) atomicOr(err, kDevErrSpin);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // tile tc accumulates in TMEM columns [256 (tc & 1), +256): the MMAs of
      // the next tile run while the epilogue drains this one
      uint32_t it = 0, tc = 0;
      for (int t = blockIdx.x; t < sc.tile_count && ok; t += gridDim.x, ++tc) {
        const uint32_t b = tc & 1u, use = tc >> 1;
        if (use > 0 && !mbar_wait(&tmem_empty[b], (use - 1) & 1)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + b * (uint32_t)kTN;
        for (int kc = 0; kc < kchunks; ++kc, ++it) {
          const uint32_t s = it % kStages, u2 = it / kStages;
          if (!mbar_wait(&full[s], u2 & 1)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t ahi = smem_u32(base + (size_t)s * kStageBytes);
          const uint32_t alo = ahi + kABytes, bhi = ahi + 2 * kABytes, blo = bhi + kBBytes;
          // a.b = hi.hi + hi.lo + lo.hi, K = 16 at a time
#pragma unroll
          for (int k = 0; k < kTK / 16; ++k) {
            umma_bf16(acc, sw128_desc(ahi + k * 32), sw128_desc(bhi + k * 32), (kc | k) != 0 ? 1u : 0u);
            umma_bf16(acc, sw128_desc(ahi + k * 32), sw128_desc(blo + k * 32), 1u);
            umma_bf16(acc, sw128_desc(alo + k * 32), sw128_desc(bhi + k * 32), 1u);
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tmem_full[b]);
      }
      if (!ok) atomicOr(err, kDevErrSpin);
    }
    __syncwarp();
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (tile rows), one row
    // per thread, 16 columns per tcgen05.ld; warp group g = (w - 2) / 4
    // takes columns [g * kGroupCols, +kGroupCols) of each tile.  Each group
    // loads its columns' data (squared norms, bound factors, list bars) one
    // tile ahead into a double-buffered shared array that its lanes read by
    // broadcast; each tile begins with a barrier of the group's 128 threads
    // (named barrier 1 + g), executed the same number of times by each of
    // them, so that groups run on without waiting for one another.  Named
    // barrier 5 spans the whole epilogue (before the first tile and, in pass
    // 3, after the last).
    const int quarter = warp & 3;
    const int group = (warp - 2) >> 2;
    const int r = quarter * 32 + lane;
    const int m = m0 + r;
    const bool live = m < nb;
    const int row = arow0 + m;
    const int gt = threadIdx.x - 64 - 128 * group;  // 0..127 within the group
    const float nm = live ? norms[row] : 0.0f;
    const float sm = live ? snorms[row] : 0.0f;
    const float inf = __int_as_float(0x7f800000);
    float *heap = heaps + r;
    int hcnt = 0;
    float t_loc = inf;  // passes 0 and 1: the heap's largest once it holds 32
    const float t_row = (kPass == 2 && live) ? sc.row_t[m] : inf;
    const float seed = ((kPass == 1 || kPass == 3) && live && sc.seed) ? sc.seed[m] : inf;
    int *cand_m = sc.cand + (long)m * sc.cand_ld;
    // pass 3: the segment of stored columns of (row m, this CTA), filled by
    // the row's threads of every group through a shared-memory counter
    // (in the heap space, which pass 3 does not use)
    const size_t seg = ((size_t)m * gridDim.x + blockIdx.x) * (size_t)sc.pre_cap;
    int *scnt = reinterpret_cast<int *>(heaps);
    if (kPass == 3 && group == 0) scnt[r] = 0;
    asm volatile("bar.sync 5, %0;" ::"n"(kEpi) : "memory");
    const bool col_test = kPass == 3 || (kPass == 1 && sc.col_test);
    // this thread's columns of a tile: group * kGroupCols + gt + 128 h
    constexpr int kColsPer = (kGroupCols + 127) / 128;
    float cv[3 * kColsPer];
    auto load_cols = [&](int t) {
      const int c0 = t * sc.tile_stride * kTN;
#pragma unroll
      for (int h = 0; h < kColsPer; ++h) {
        const int gi = gt + h * 128;
        const int jj = group * kGroupCols + gi;
        const int j = c0 + jj;
        const bool in = gi < kGroupCols && j < n;
        cv[3 * h] = in ? norms[j] : 0.0f;
        cv[3 * h + 1] = in ? snorms[j] : 0.0f;
        cv[3 * h + 2] = ((kPass == 1 || kPass == 3) && gi < kGroupCols && j < sc.n_exist)
                            ? key_dist(sc.g_key[(size_t)j * kListW + kListW - 1])
                            : -inf;
      }
    };
    if ((int)blockIdx.x < sc.tile_count) load_cols(blockIdx.x);
    bool eok = true;
    uint32_t tc = 0;
    for (int t = blockIdx.x; t < sc.tile_count; t += gridDim.x, ++tc) {
      const uint32_t b = tc & 1u;
      float *cn = epi + (size_t)b * 3 * kTN;  // norms | bound factors | list bars
      // per-warp maxima of the column norms and factors: slot 4 g + q for
      // warp q of group g (0 where the warp has no columns)
      unsigned *mx = reinterpret_cast<unsigned *>(epi + 2 * 3 * kTN) + b * 2 * 16;
      {
        unsigned mn = 0, ms = 0;
#pragma unroll
        for (int h = 0; h < kColsPer; ++h) {
          const int gi = gt + h * 128;
          if (gi < kGroupCols) {
            const int jj = group * kGroupCols + gi;
            cn[jj] = cv[3 * h];
            cn[kTN + jj] = cv[3 * h + 1];
            cn[2 * kTN + jj] = cv[3 * h + 2];
            mn = max(mn, __float_as_uint(cv[3 * h]));
            ms = max(ms, __float_as_uint(cv[3 * h + 1]));
          }
        }
        mn = __reduce_max_sync(0xffffffffu, mn);
        ms = __reduce_max_sync(0xffffffffu, ms);
        if (lane == 0) {
          mx[4 * group + quarter] = mn;
          mx[16 + 4 * group + quarter] = ms;
        }
      }
      switch (group) {  // the barrier id is an immediate
        case 0: asm volatile("bar.sync 1, 128;" ::: "memory"); break;
        case 1: asm volatile("bar.sync 2, 128;" ::: "memory"); break;
        case 2: asm volatile("bar.sync 3, 128;" ::: "memory"); break;
        default: asm volatile("bar.sync 4, 128;" ::: "memory"); break;
      }
      // the largest pair bound of the row over this group's columns
      // (pair_bound is nondecreasing in the column's norm and factor)
      float bmax;
      {
        unsigned mn = 0, ms = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          mn = max(mn, mx[4 * group + q]);
          ms = max(ms, mx[16 + 4 * group + q]);
        }
        bmax = pair_bound(sc.coef, sm, __uint_as_float(ms), nm, __uint_as_float(mn));
      }
      if (t + (int)gridDim.x < sc.tile_count) load_cols(t + gridDim.x);
      if (eok && !mbar_wait(&tmem_full[b], (tc >> 1) & 1)) {
        if (lane == 0) atomicOr(err, kDevErrSpin);
        eok = false;
      }
      if (!eok) continue;
      tc_fence_after();
      const int ctile = t * sc.tile_stride * kTN;
      // passes 2 and 3: D - B of every column of the group is at least
      // RD(D - bmax); when that exceeds the row's limit and the column's list
      // bar in every lane, no test can pass for the column
      const float lim = kPass == 3 ? seed : t_row;
      float cmin = inf;    // pass 0: the 32-column chunk's smallest D over other columns
      unsigned hmask = 0;  // column test: the chunk's hit columns (bit i)
      // the exact tests of column c + i of the tile (chunk bit (c & 16) + i),
      // whose D is dv
      auto slow = [&](int i, float dv, int c) {
        const float nj = cn[c + i];
        const int j = ctile + c + i;
        const bool other = live && j < n && j != row;
        const float wj = (kPass == 1 || kPass == 3) ? cn[2 * kTN + c + i] : -inf;
        const float sj = cn[kTN + c + i];
        const float bnd = pair_bound(sc.coef, sm, sj, nm, nj);
        if (kPass == 1 && other) {
          const float ub = fmaxf(__fadd_ru(dv, bnd), 0.0f);
          if (ub < t_loc && ub <= seed) t_loc = heap_push(heap, hcnt, ub);
        }
        if (kPass == 3 && other) {
          const float lb = __fsub_rd(dv, bnd);
          if (lb <= seed) {
            const int q = atomicAdd(&scnt[r], 1);
            if (q < sc.pre_cap) {
              sc.pre[seg + q] = ((unsigned long long)__float_as_uint(lb) << 32) | (unsigned)j;
              sc.pre_ub[seg + q] = fmaxf(__fadd_ru(dv, bnd), 0.0f);
            }
          }
        }
        if (col_test) {
          if (live && j < sc.n_exist && __fsub_rd(dv, bnd) <= wj) hmask |= 1u << ((c & 16) + i);
        } else if (kPass == 2 && other && __fsub_rd(dv, bnd) <= t_row) {
          cand_m[atomicAdd(&sc.row_cnt[m], 1)] = j;
        }
      };
      // 16 columns from c (a half of a 32-column chunk), their accumulators
      // in v and at tensor-memory address tah
      auto half = [&](uint32_t(&v)[16], int c, uint32_t tah) {
        const int col0 = ctile + c;
        // fast phase: D of the 16 columns and, for passes 2 and 3, a
        // warp-uniform mask of the columns where some lane may pass a test;
        // 16 independent chains without branches
        unsigned need = 0u;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float dv = __fsub_rn(__fadd_rn(nm, cn[c + i]), __fmul_rn(2.0f, __uint_as_float(v[i])));
          if (kPass == 1) v[i] = __float_as_uint(dv);
          if (kKeepD && live && col0 + i < n) D[(long)m * ldD + col0 + i] = dv;
          if (kPass == 0 && live && col0 + i < n && col0 + i != row) cmin = fminf(cmin, dv);
          if (kPass == 2 || kPass == 3) {
            const float wj = kPass == 3 ? cn[2 * kTN + c + i] : -inf;
            if (__any_sync(0xffffffffu, __fsub_rd(dv, bmax) <= fmaxf(lim, wj))) need |= 1u << i;
          }
        }
        // slow phase, in column order: every column for the heap pass; for
        // passes 2 and 3 only the flagged ones, each accumulator read again
        // from tensor memory (D recomputed by the same operations), so that
        // nothing of the fast phase stays live across it
        if constexpr (kPass == 1) {
#pragma unroll
          for (int i = 0; i < 16; ++i) slow(i, __uint_as_float(v[i]), c);
        } else if constexpr (kPass == 2 || kPass == 3) {
          while (need) {  // warp-uniform
            const int i = __ffs(need) - 1;
            need &= need - 1;
            const float acc = __uint_as_float(tmem_ld1(tah + (uint32_t)i));
            slow(i, __fsub_rn(__fadd_rn(nm, cn[c + i]), __fmul_rn(2.0f, acc)), c);
          }
        }
      };
      // after both halves of the 32-column chunk at c
      auto chunk_end = [&](int c) {
        const int col0 = ctile + c;
        if (kPass == 0 && live)
          sc.mins[(size_t)m * sc.mins_ld + t * (kTN / 32) + c / 32] =
              cmin == inf ? inf : fmaxf(__fadd_ru(cmin, bmax), 0.0f);
        cmin = inf;
        if (col_test) {
          // the chunk's (existing row j, batch row m) pairs: one pool
          // reservation per warp, lanes in order
          const int cnt = __popc(hmask);
          int incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          const int total = __shfl_sync(0xffffffffu, incl, 31);
          if (total) {
            int base = 0;
            if (lane == 31) base = atomicAdd(sc.pool_counter, total);
            base = __shfl_sync(0xffffffffu, base, 31);
            long q = (long)base + incl - cnt;
            while (hmask) {
              const int i = __ffs(hmask) - 1;
              hmask &= hmask - 1;
              if (q < sc.pool_cap) {
                sc.pool_j[q] = col0 + i;
                sc.pool_m[q] = m;
              } else {
                atomicOr(err, kDevErrOverflow);
              }
              ++q;
            }
          }
          hmask = 0;
        }
      };
      // the group's columns 16 at a time, the next half's tensor-memory load
      // in flight while this half is screened
      constexpr int kHalves = kGroupCols / 16;
      const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + b * (uint32_t)kTN +
                          (uint32_t)(group * kGroupCols);
      uint32_t va[16], vb[16];
      tmem_ld16(ta, va);
#pragma unroll 1
      for (int h = 0; h < kHalves; h += 2) {
        tmem_ld_wait(va);
        tmem_ld16(ta + (uint32_t)(h + 1) * 16, vb);
        half(va, group * kGroupCols + h * 16, ta + (uint32_t)h * 16);
        tmem_ld_wait(vb);
        if (h + 2 < kHalves) tmem_ld16(ta + (uint32_t)(h + 2) * 16, va);
        half(vb, group * kGroupCols + (h + 1) * 16, ta + (uint32_t)(h + 1) * 16);
        chunk_end(group * kGroupCols + h * 16);
      }
      tc_fence_before();
      mbar_arrive(&tmem_empty[b]);
    }
    if (kPass == 1 && live) {
      float *out = sc.heaps + ((size_t)m * gridDim.x + blockIdx.x) * kListTop;
      for (int i = 0; i < kListTop; ++i) out[i] = i < hcnt ? heap[i * kTM] : inf;
    }
    if (kPass == 3) {
      // every group's stores to the row's counter are done
      asm volatile("bar.sync 5, %0;" ::"n"(kEpi) : "memory");
      if (group == 0 && live) {
        const int pcnt = scnt[r];
        sc.pre_cnt[(size_t)m * gridDim.x + blockIdx.x] = min(pcnt, sc.pre_cap);
        if (pcnt > sc.pre_cap) atomicOr(sc.pre_over, 1);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
}

// ---- screen: exact threshold, FP32 re-score, exact top-32 -----------------
//
// Around and after k_exact_dist, per block of batch rows (brow0 .. +nrows):
//  k_row_threshold  warp per batch row: T = 32nd smallest upper bound over all
//                columns, from the union of the CTAs' heaps (pass 1), for the
//                candidate test of pass 2
//  k_pool_count / k_pool_scatter   groups the column pairs by existing row
//                (counting sort; order inside a group is free)
//  k_row_dists   canonical distances of the row candidates
//  k_pair_dists  canonical distances of the column pairs
//  k_row_select  warp per batch row: exact top-32 keys of its candidates
//  k_col_merge   warp per existing row: merges its pairs into its list
// Both merges are order independent: a list ends as the 32 smallest keys of
// its old entries and every candidate, and keys are unique (distinct ids).
//
// Canonical distances are sequential FP32 fused multiply-add chains over the
// features; a warp forms 32 chains at once, one per lane, from feature rows
// staged 32 columns at a time in shared memory by coalesced loads (lane l
// reads tile row l at column i: bank (l * 33 + i) mod 32, conflict free).
// fmaf(a, b, c) = fmaf(b, a, c) exactly, so d(x, y) = d(y, x) bit for bit.

constexpr int kTile = 32;
constexpr int kTileLd = 33;
constexpr int kFinalWarps = 4;

// Merges each lane's value u into the warp's ascending top 32 (lane l holds
// the l-th smallest); values not below the current 32nd change nothing.
GM_D void top32_merge(float &top, float u, int lane) {
  unsigned pend = __ballot_sync(0xffffffffu, u < __shfl_sync(0xffffffffu, top, 31));
  while (pend) {
    const int src = __ffs(pend) - 1;
    pend &= pend - 1;
    const float x = __shfl_sync(0xffffffffu, u, src);
    const unsigned pos_mask = __ballot_sync(0xffffffffu, x < top);
    if (!pos_mask) continue;
    const int pos = __ffs(pos_mask) - 1;
    const float prev = __shfl_up_sync(0xffffffffu, top, 1);
    if (lane > pos) top = prev;
    else if (lane == pos) top = x;
  }
}

// The 32nd smallest of cnt values at v (inf when fewer than 32 are finite),
// one warp; eight 32-value chunks are loaded together, then merged.
GM_D float warp_32nd(const float *v, int cnt, int lane) {
  const float inf = __int_as_float(0x7f800000);
  float top = inf;
  for (int c0 = 0; c0 < cnt; c0 += 8 * 32) {
    float u[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = c0 + q * 32 + lane;
      u[q] = idx < cnt ? v[idx] : inf;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) top32_merge(top, u[q], lane);
  }
  return __shfl_sync(0xffffffffu, top, 31);
}

// Warp per batch row: T = the 32nd smallest of the union of the CTAs' heaps
// (pass 1), capped by the seed; both bound the row's 32nd smallest upper
// bound from above.  With run_if, only when *run_if != 0.
__global__ void __launch_bounds__(kFinalWarps * 32)
    k_row_threshold(const float *heaps, int ncta, int nrows, int n, const float *seed, float *row_t,
                    const int *run_if, unsigned long long *stat) {
  if (run_if && *run_if == 0) return;
  const int lane = threadIdx.x & 31;
  const int ml = blockIdx.x * kFinalWarps + (threadIdx.x >> 5);
  if (ml >= nrows) return;
  const float inf = __int_as_float(0x7f800000);
  const float T = fminf(warp_32nd(heaps + (size_t)ml * ncta * kListTop, ncta * kListTop, lane),
                        seed ? seed[ml] : inf);
  if (lane == 0) {
    // fewer than 32 other rows: every column is a candidate
    row_t[ml] = n - 1 < kListTop ? inf : T;
    if (stat) atomicAdd(&stat[5], (unsigned long long)n);
  }
}

// Warp per batch row: the seed, the 32nd smallest of the row's chunk minima
// from pass 0 (the largest upper bound of 32 distinct columns).
__global__ void __launch_bounds__(kFinalWarps * 32)
    k_seed_select(const float *mins, int mins_ld, int nrows, float *seed) {
  const int lane = threadIdx.x & 31;
  const int ml = blockIdx.x * kFinalWarps + (threadIdx.x >> 5);
  if (ml >= nrows) return;
  const float T = warp_32nd(mins + (size_t)ml * mins_ld, mins_ld, lane);
  if (lane == 0) seed[ml] = T;
}

// Warp per batch row, after pass 3: T = the 32nd smallest stored upper
// bound (exact: every column whose upper bound is at most T was stored),
// then the row's candidates, the stored columns with lower bound <= T.  Lane
// l walks segments l, l + 32, ... (a row tile has at least 19 CTAs on 152
// SMs with blocks of up to 1,024 rows); entry i of every lane's segment is
// handled together, four entries loaded ahead.  Does nothing when a segment
// overflowed (the heap passes then run instead).
__global__ void __launch_bounds__(kFinalWarps * 32)
    k_pre_select(const unsigned long long *pre, const float *pre_ub, const int *pre_cnt, int gx,
                 int cap, const int *pre_over, int nrows, int n, float *row_t, int *cand,
                 long cand_ld, int *row_cnt, unsigned long long *stat) {
  if (*pre_over) {
    if (stat && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stat[9], 1ull);
    return;
  }
  const int lane = threadIdx.x & 31;
  const int m = blockIdx.x * kFinalWarps + (threadIdx.x >> 5);
  if (m >= nrows) return;
  const float inf = __int_as_float(0x7f800000);
  float top = inf;
  for (int c0 = 0; c0 < gx; c0 += 32) {
    const int c = c0 + lane;
    const size_t seg = (size_t)m * gx + c;
    const int len = c < gx ? pre_cnt[seg] : 0;
    const float *u = pre_ub + seg * (size_t)cap;
    int maxlen = len;
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
    for (int i0 = 0; i0 < maxlen; i0 += 4) {
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = i0 + q < len ? u[i0 + q] : inf;
#pragma unroll
      for (int q = 0; q < 4; ++q) top32_merge(top, v[q], lane);
    }
  }
  // fewer than 32 other rows: every column is a candidate
  const float T = n - 1 < kListTop ? inf : __shfl_sync(0xffffffffu, top, 31);
  int *out = cand + (long)m * cand_ld;
  int cnt = 0;
  for (int c0 = 0; c0 < gx; c0 += 32) {
    const int c = c0 + lane;
    const size_t seg = (size_t)m * gx + c;
    const int len = c < gx ? pre_cnt[seg] : 0;
    const unsigned long long *e = pre + seg * (size_t)cap;
    int maxlen = len;
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
    for (int i0 = 0; i0 < maxlen; i0 += 4) {
      unsigned long long v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = i0 + q < len ? e[i0 + q] : 0ull;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool keep = i0 + q < len && __uint_as_float((unsigned)(v[q] >> 32)) <= T;
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (keep) out[cnt + __popc(bal & ((1u << lane) - 1u))] = (int)(unsigned)v[q];
        cnt += __popc(bal);
      }
    }
  }
  if (lane == 0) {
    row_t[m] = T;
    row_cnt[m] = cnt;
    if (stat) atomicAdd(&stat[5], (unsigned long long)n);
  }
}

__global__ void k_pool_count(const int *pool_j, const int *counter, long pool_cap, int *pcnt,
                             unsigned long long *stat) {
  const long total = min((long)*counter, pool_cap);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x)
    atomicAdd(&pcnt[pool_j[e]], 1);
  if (stat && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stat[6], (unsigned long long)total);
}
// pcnt: zeroed again before this launch (it serves as the fill cursor)
__global__ void k_pool_scatter(const int *pool_j, const int *pool_m, const int *counter,
                               long pool_cap, const int *poff, int *pcnt, int *pool_j2,
                               int *pool_m2) {
  const long total = min((long)*counter, pool_cap);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int j = pool_j[e];
    const int q = poff[j] + atomicAdd(&pcnt[j], 1);
    pool_j2[q] = j;
    pool_m2[q] = pool_m[e];
  }
}

// 32 canonical chains per warp, one per lane (pair ra, rb; dummies for idle
// lanes).  Feature chunks of 32 columns of the 64 rows are copied into a ring
// of kRing shared-memory slots by 4-byte cp.async (each lane copies column
// `lane` of every row: coalesced), kRing - 1 chunks ahead of the chain.
constexpr int kRing = 4;
constexpr int kPairWarps = 2;
struct PairTiles {
  float a[kRing][kTile][kTileLd];
  float b[kRing][kTile][kTileLd];
  int ra[kTile], rb[kTile];
};
constexpr size_t kPairSmem = sizeof(PairTiles) * kPairWarps;

GM_D void cp_async4(float *dst, const float *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
GM_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
GM_D void cp_async_wait_ring() {
  asm volatile("cp.async.wait_group %0;" ::"n"(kRing - 1) : "memory");
}

GM_D float warp_pair_dot(const float *X, int ld, int d, int ra, int rb, PairTiles &t) {
  const int lane = threadIdx.x & 31;
  t.ra[lane] = ra;
  t.rb[lane] = rb;
  __syncwarp();
  const int nch = (d + kTile - 1) / kTile;
  // one commit group per chunk index (empty past the last chunk), so that
  // "at most kRing - 1 groups pending" means chunk c has landed
  auto issue = [&](int c) {
    const int col = c * kTile + lane;
    if (c < nch && col < d) {
      const int slot = c % kRing;
#pragma unroll 8
      for (int r = 0; r < kTile; ++r) {
        cp_async4(&t.a[slot][r][lane], X + (size_t)t.ra[r] * ld + col);
        cp_async4(&t.b[slot][r][lane], X + (size_t)t.rb[r] * ld + col);
      }
    }
    cp_async_commit();
  };
  for (int c = 0; c < kRing - 1; ++c) issue(c);
  float dot = 0.0f;
  for (int c = 0; c < nch; ++c) {
    issue(c + kRing - 1);  // refills the slot the previous iteration consumed
    cp_async_wait_ring();
    __syncwarp();
    const int slot = c % kRing, lim = min(kTile, d - c * kTile);
    for (int i = 0; i < lim; ++i) dot = __fmaf_rn(t.a[slot][lane][i], t.b[slot][lane][i], dot);
    __syncwarp();
  }
  return dot;
}

__global__ void __launch_bounds__(kPairWarps * 32)
    k_pair_dists(const float *X, int ld, int d, const float *norms, int brow0, const int *pool_j,
                 const int *pool_m, float *pool_d, const int *counter, long pool_cap) {
  extern __shared__ __align__(16) unsigned char pair_smem[];
  PairTiles &t = reinterpret_cast<PairTiles *>(pair_smem)[threadIdx.x >> 5];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long total = min((long)*counter, pool_cap);
  const long nw = (long)gridDim.x * kPairWarps;
  for (long g = ((long)blockIdx.x * kPairWarps + w) * 32; g < total; g += nw * 32) {
    const long e = g + lane;
    const bool ok = e < total;
    const int a = ok ? pool_j[e] : 0;
    const int b = ok ? brow0 + pool_m[e] : 0;
    const float dot = warp_pair_dot(X, ld, d, a, b, t);
    if (ok) pool_d[e] = canon_dist(norms[a], norms[b], dot);
  }
}

// Row candidates: the batch row is common to the warp, so only the candidate
// rows go through the ring; lane l holds feature c0 + l of the batch row and
// hands it to every chain by a shuffle.
constexpr int kRowDistWarps = 4;
struct RowTiles {
  float b[kRing][kTile][kTileLd];
  float a[kRing][kTile];
  int rb[kTile];
};
constexpr size_t kRowSmem = sizeof(RowTiles) * kRowDistWarps;

__global__ void __launch_bounds__(kRowDistWarps * 32)
    k_row_dists(const float *X, int ld, int d, const float *norms, int brow0, const int *cand,
                long cand_ld, const int *row_cnt, float *cand_d) {
  extern __shared__ __align__(16) unsigned char row_smem[];
  RowTiles &t = reinterpret_cast<RowTiles *>(row_smem)[threadIdx.x >> 5];
  const int ml = blockIdx.x, row = brow0 + ml;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cnt = row_cnt[ml];
  const int *cl = cand + (long)ml * cand_ld;
  const float *xa = X + (size_t)row * ld;
  const int nch = (d + kTile - 1) / kTile;
  for (int g = w * 32; g < cnt; g += kRowDistWarps * 32) {
    const int c = g + lane;
    t.rb[lane] = c < cnt ? cl[c] : row;
    __syncwarp();
    auto issue = [&](int ch) {
      const int col = ch * kTile + lane;
      if (ch < nch && col < d) {
        const int slot = ch % kRing;
        cp_async4(&t.a[slot][lane], xa + col);
#pragma unroll 8
        for (int r = 0; r < kTile; ++r)
          cp_async4(&t.b[slot][r][lane], X + (size_t)t.rb[r] * ld + col);
      }
      cp_async_commit();
    };
    for (int ch = 0; ch < kRing - 1; ++ch) issue(ch);
    float dot = 0.0f;
    for (int ch = 0; ch < nch; ++ch) {
      issue(ch + kRing - 1);
      cp_async_wait_ring();
      __syncwarp();
      const int slot = ch % kRing, lim = min(kTile, d - ch * kTile);
      for (int i = 0; i < lim; ++i) dot = __fmaf_rn(t.a[slot][i], t.b[slot][lane][i], dot);
      __syncwarp();
    }
    if (c < cnt) cand_d[(long)ml * cand_ld + c] = canon_dist(norms[row], norms[t.rb[lane]], dot);
    __syncwarp();
  }
}

constexpr int kRowWarps = 4;
__global__ void k_row_select(const float *cand_d, int brow0, int nrows, const int *cand,
                             long cand_ld, const int *row_cnt, Key *g_key,
                             unsigned long long *stat) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ml = blockIdx.x * kRowWarps + warp;
  if (ml >= nrows) return;
  const int cnt = row_cnt[ml];
  const int *cl = cand + (long)ml * cand_ld;
  const float *dr = cand_d + (long)ml * cand_ld;
  Key mine = kEmptyKey;
  for (int c0 = 0; c0 < cnt; c0 += 32) {
    const int c = c0 + lane;
    const Key ck = c < cnt ? make_key(dr[c], cl[c]) : ~(Key)0;
    // insert the (up to) 32 new keys one at a time into the sorted warp list
    for (int src = 0; src < 32 && c0 + src < cnt; ++src) {
      const Key k = __shfl_sync(0xffffffffu, ck, src);
      const unsigned msk = __ballot_sync(0xffffffffu, k < mine);
      if (!msk) continue;
      const int pos = __ffs(msk) - 1;
      const Key prev = __shfl_up_sync(0xffffffffu, mine, 1);
      if (lane > pos) mine = prev;
      else if (lane == pos) mine = k;
    }
  }
  g_key[(size_t)(brow0 + ml) * kListW + lane] = mine;
  if (stat && lane == 0) atomicAdd(&stat[6], (unsigned long long)cnt);
}

// Warp per existing row j with pairs: lane l holds entry l of j's sorted list;
// each new key is inserted by a ballot on the lanes whose entry it precedes.
constexpr int kMergeWarps = 8;
__global__ void k_col_merge(int n_exist, int brow0, const int *poff, const int *pool_m,
                            const float *pool_d, Key *g_key, int *dirty) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * kMergeWarps + (threadIdx.x >> 5);
  if (j >= n_exist) return;
  const int base = poff[j], cnt = poff[j + 1] - poff[j];
  if (!cnt) return;
  Key *lst = g_key + (size_t)j * kListW;
  Key mine = lst[lane];
  bool changed = false;
  for (int c0 = 0; c0 < cnt; c0 += 32) {
    const int c = c0 + lane;
    const Key ck = c < cnt ? make_key(pool_d[base + c], brow0 + pool_m[base + c]) : ~(Key)0;
    for (int src = 0; src < 32 && c0 + src < cnt; ++src) {
      const Key k = __shfl_sync(0xffffffffu, ck, src);
      const unsigned msk = __ballot_sync(0xffffffffu, k < mine);
      if (!msk) continue;
      changed = true;
      const int pos = __ffs(msk) - 1;
      const Key prev = __shfl_up_sync(0xffffffffu, mine, 1);
      if (lane > pos) mine = prev;
      else if (lane == pos) mine = k;
    }
  }
  if (changed) {
    lst[lane] = mine;
    if (lane == 0) dirty[j] = 1;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

int exact_dh(int d) { return (d + kTK - 1) / kTK * kTK; }

// coef of pair_bound for d features (dh padded).  With S = sum |a_i b_i| <=
// |a||b| (Cauchy-Schwarz) and u = 2^-8 the BF16 unit roundoff:
//  * operands: a_i b_i - (hi hi + hi lo + lo hi) = lo lo + hi r + lo r + r hi + ...
//    with |lo| <= u|a_i|, |r| = |a_i - hi - lo| <= u^2 |a_i|: below 3.1 u^2 S;
//  * tensor-core accumulation of m = 3 dh exact products: every operand of
//    every internal addition (the products, and the running sum once per
//    K=16 instruction; m/4 allows for up to four internal stages each) is cut
//    by at most 2^-23 of the largest magnitude involved, itself at most the
//    products' magnitude sum (1 + u)^2 S + 2 u (1 + u) S < 1.02 S: below
//    (1.25 m + 1) 2^-23 * 1.02 S;
//  * canonical FP32 chain of d fused multiply-adds (round to nearest):
//    below d 2^-24 S (1 + d 2^-24);
//  times 2 for -2 dot, and 1 + d 2^-23 because sqrt(na nb) is formed from FP32
//  norms that may fall short of |a|^2 |b|^2 by that factor.
float exact_bound_coef(int d, int dh) {
  const double u = std::ldexp(1.0, -8);
  const double m = 3.0 * dh;
  const double op = 3.1 * u * u;
  const double acc = (1.25 * m + 1.0) * std::ldexp(1.0, -23) * 1.02;
  const double canon = d * std::ldexp(1.0, -24) * (1.0 + d * std::ldexp(1.0, -24));
  const double c = 2.0 * (op + acc + canon) * (1.0 + d * std::ldexp(1.0, -23)) * 1.001;
  return (float)(c * (1.0 + 1e-6));
}

bool make_row_maps(void *xh, int n_cap, int dh, ExactMaps *out) {
  auto enc = get_encode();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)dh * 2, (cuuint64_t)std::max(n_cap, 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)dh * 4};
  const cuuint32_t estr[2] = {1, 1};
  const cuuint32_t box_a[2] = {(cuuint32_t)kTK, (cuuint32_t)kTM};
  const cuuint32_t box_b[2] = {(cuuint32_t)kTK, (cuuint32_t)kTN};
  CUresult r1 = enc(reinterpret_cast<CUtensorMap *>(out->a), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, xh,
                    dims, strides, box_a, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  CUresult r2 = enc(reinterpret_cast<CUtensorMap *>(out->b), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, xh,
                    dims, strides, box_b, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r1 == CUDA_SUCCESS && r2 == CUDA_SUCCESS;
}

void launch_to_bf16(const DevState &st, void *xh, int dh, int row0, int nrows, cudaStream_t s) {
  if (nrows <= 0) return;
  const long total = (long)nrows * dh;
  k_to_bf16<<<std::min(cdiv(total, 256), 4096), 256, 0, s>>>(st.X, st.ld, st.d, dh, row0, nrows,
                                                           (__nv_bfloat16 *)xh);
  note_launch();
}

template <int kPass, bool kKeepD>
static void launch_tile(const DevState &st, const ExactMaps &maps, int dh, int row0, int blk0,
                        int nrows, int n, const ExactScreen &x, long ldD, int gx, int m_tiles,
                        int tile_count, int tile_stride, const float *seed, int pre_cap,
                        int mins_ld, int col_test, const int *run_if, cudaStream_t s) {
  // once per device (sessions on several host threads may launch at once)
  static std::atomic<unsigned> configured{0u};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 32 && !(configured.load() & (1u << dev))) {
    cudaFuncSetAttribute(k_exact_dist<kPass, kKeepD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kExactSmem);
    configured.fetch_or(1u << dev);
  }
  CUtensorMap ta, tb;
  memcpy(&ta, maps.a, sizeof(ta));
  memcpy(&tb, maps.b, sizeof(tb));
  TileScreen sc;
  sc.tile_count = tile_count;
  sc.tile_stride = tile_stride;
  sc.heaps = x.heaps;
  sc.seed = seed;
  sc.mins = x.mins;
  sc.mins_ld = mins_ld;
  sc.pre = x.pre;
  sc.pre_ub = x.pre_ub;
  sc.pre_cnt = x.pre_cnt;
  sc.pre_cap = pre_cap;
  sc.pre_over = x.pre_over;
  sc.col_test = col_test;
  sc.run_if = run_if;
  sc.row_t = x.row_t;
  sc.cand = x.cand;
  sc.cand_ld = ldD;
  sc.row_cnt = x.row_cnt;
  sc.pool_j = x.pool_j;
  sc.pool_m = x.pool_m;
  sc.pool_counter = x.counter;
  sc.pool_cap = x.pool_cap;
  sc.g_key = st.g_key;
  sc.n_exist = row0;
  sc.coef = exact_bound_coef(st.d, dh);
  k_exact_dist<kPass, kKeepD><<<dim3(gx, m_tiles), exact_threads(kPass), kExactSmem, s>>>(
      ta, tb, row0 + blk0, nrows, n, dh / kTK, dh, st.norms, st.snorms, sc, x.D, ldD, st.err);
  note_launch();
}

// Column tiles of the seed pass (evenly spaced over the columns): at least
// 16, and one in 16 of the block's tiles, so that the seed stays a low
// quantile of the row's upper bounds at any column count.
constexpr int kSeedTiles = 16;
constexpr int kSeedEvery = 16;

int exact_seed_tiles(int n_tiles) { return std::max(kSeedTiles, n_tiles / kSeedEvery); }

void launch_exact_dist(const DevState &st, const ExactMaps &maps, int dh, int row0, int blk0,
                       int nrows, int n, const ExactScreen &x, long ldD, bool keep_d, int sms,
                       cudaStream_t s) {
  const int n_tiles = cdiv(n, kTN);
  const int m_tiles = cdiv(nrows, kTM);
  // CTAs per row tile so that the grid covers the SMs once
  const int gx = std::max(1, std::min(n_tiles, std::max(1, sms / m_tiles)));
  const bool kd = keep_d && x.D;
  cudaMemsetAsync(x.row_cnt, 0, (size_t)nrows * sizeof(int), s);
  cudaMemsetAsync(x.counter, 0, sizeof(int), s);
  const int tiles = exact_seed_tiles(n_tiles);
  // entries per stored segment: the row's whole allocation shared by its
  // tile's CTAs (fewer CTAs per row tile, longer segments)
  const int cap = x.pre_fixed || gx > x.pre_gx ? x.pre_cap : (int)((long)x.pre_gx * x.pre_cap / gx);
  if (n_tiles > 2 * kSeedTiles && x.pre && cap > 0 && gx <= x.pre_gx &&
      tiles * (kTN / 32) <= x.mins_ld) {
    // seed pass over a spread sample of tiles, then the store pass
    const int stride = n_tiles / tiles;
    const int gx0 = std::max(1, std::min(tiles, std::max(1, sms / m_tiles)));
    const int mins_ld = tiles * (kTN / 32);
    launch_tile<0, false>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx0, m_tiles, tiles, stride,
                          nullptr, 0, mins_ld, 0, nullptr, s);
    k_seed_select<<<cdiv(nrows, kFinalWarps), kFinalWarps * 32, 0, s>>>(x.mins, mins_ld, nrows, x.seed);
    cudaMemsetAsync(x.pre_over, 0, sizeof(int), s);
    if (kd)
      launch_tile<3, true>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, x.seed,
                           cap, 0, 0, nullptr, s);
    else
      launch_tile<3, false>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, x.seed,
                            cap, 0, 0, nullptr, s);
    k_pre_select<<<cdiv(nrows, kFinalWarps), kFinalWarps * 32, 0, s>>>(
        x.pre, x.pre_ub, x.pre_cnt, gx, cap, x.pre_over, nrows, n, x.row_t, x.cand, ldD, x.row_cnt,
        st.stat);
    note_launch(2);
    // after an overflow only: the heap pass (seed-capped; its pairs were
    // already pooled), the threshold and the candidate pass
    launch_tile<1, false>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, x.seed, 0,
                          0, 0, x.pre_over, s);
    k_row_threshold<<<cdiv(nrows, kFinalWarps), kFinalWarps * 32, 0, s>>>(x.heaps, gx, nrows, n, x.seed,
                                                                          x.row_t, x.pre_over, st.stat);
    note_launch();
    launch_tile<2, false>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, nullptr, 0,
                          0, 0, x.pre_over, s);
    return;
  }
  if (kd)
    launch_tile<1, true>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, nullptr, 0,
                         0, 1, nullptr, s);
  else
    launch_tile<1, false>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, nullptr, 0,
                          0, 1, nullptr, s);
  k_row_threshold<<<cdiv(nrows, kFinalWarps), kFinalWarps * 32, 0, s>>>(x.heaps, gx, nrows, n, nullptr,
                                                                        x.row_t, nullptr, st.stat);
  note_launch();
  launch_tile<2, false>(st, maps, dh, row0, blk0, nrows, n, x, ldD, gx, m_tiles, n_tiles, 1, nullptr, 0,
                        0, 0, nullptr, s);
}

void launch_exact_screen(const DevState &st, int row0, int blk0, int nrows, int n,
                         const ExactScreen &x, long ldD, int sms, cudaStream_t s) {
  if (nrows <= 0 || n <= 0) return;
  const int brow0 = row0 + blk0;  // global first row of the block
  const int grid = 4 * std::max(sms, 1);
  if (row0 > 0) {
    cudaMemsetAsync(x.pcnt, 0, (size_t)row0 * sizeof(int), s);
    k_pool_count<<<grid, 256, 0, s>>>(x.pool_j, x.counter, x.pool_cap, x.pcnt, st.stat);
    note_launch();
    exclusive_scan(x.pcnt, x.poff, row0, x.tmp, s);
    cudaMemsetAsync(x.pcnt, 0, (size_t)row0 * sizeof(int), s);
    k_pool_scatter<<<grid, 256, 0, s>>>(x.pool_j, x.pool_m, x.counter, x.pool_cap, x.poff, x.pcnt,
                                        x.pool_j2, x.pool_m2);
    note_launch();
  }
  static std::atomic<unsigned> pair_configured{0u};
  {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(pair_configured.load() & (1u << dev))) {
      cudaFuncSetAttribute(k_row_dists, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRowSmem);
      cudaFuncSetAttribute(k_pair_dists, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPairSmem);
      pair_configured.fetch_or(1u << dev);
    }
  }
  k_row_dists<<<nrows, kRowDistWarps * 32, kRowSmem, s>>>(st.X, st.ld, st.d, st.norms, brow0,
                                                         x.cand, ldD, x.row_cnt, x.cand_d);
  note_launch();
  k_row_select<<<cdiv(nrows, kRowWarps), kRowWarps * 32, 0, s>>>(x.cand_d, brow0, nrows, x.cand,
                                                                 ldD, x.row_cnt, st.g_key, st.stat);
  note_launch();
  if (row0 > 0) {
    k_pair_dists<<<grid, kPairWarps * 32, kPairSmem, s>>>(
        st.X, st.ld, st.d, st.norms, brow0, x.pool_j2, x.pool_m2, x.pool_d, x.counter, x.pool_cap);
    note_launch();
    k_col_merge<<<cdiv(row0, kMergeWarps), kMergeWarps * 32, 0, s>>>(
        row0, brow0, x.poff, x.pool_m2, x.pool_d, st.g_key, st.dirty);
    note_launch();
  }
}

}  // namespace gm
