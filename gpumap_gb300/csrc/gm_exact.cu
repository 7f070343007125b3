// Exact insertion (precision = 1): each insertion batch is compared with
// every inserted row.  Distances are first formed on the 5th-generation tensor
// cores (BF16 operands staged by TMA, FP32 accumulators in TMEM), then every
// pair that a rigorous BF16 error bound cannot rule out is re-scored with the
// canonical FP32 distance.  Resulting lists are the exact 32 nearest rows
// under the canonical distance, identical to a brute-force CPU computation.
//
//  k_to_bf16     batch rows -> BF16 shadow rows (zero padded to a multiple of 64)
//  k_exact_dist  approx D[m][j] = |x_m|^2 + |x_j|^2 - 2 bf16(x_m).bf16(x_j)
//                (tcgen05.mma kind::f16, M=128 x N=256 x K=16 per instruction)
//  k_exact_rows  per batch row: bound, candidates, FP32 re-score, exact top-32
//  k_exact_cols  per existing row: batch rows that may enter its list
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "gm_common.cuh"
#include "gm_kernels.h"

namespace gm {

namespace {

constexpr int kTM = 128;                       // batch rows per tile (MMA M)
constexpr int kTN = 256;                       // columns per tile (MMA N)
constexpr int kTK = 64;                        // bf16 per K chunk = one 128-byte swizzle row
constexpr int kStages = 4;
constexpr int kABytes = kTM * kTK * 2;         // 16 KB
constexpr int kBBytes = kTN * kTK * 2;         // 32 KB
constexpr int kStageBytes = kABytes + kBBytes; // 48 KB
constexpr int kExactThreads = 192;             // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int kTmemCols = 256;                 // one 128 x 256 FP32 accumulator
constexpr uint32_t kWaitLimit = 1u << 24;      // bounded mbarrier waits
constexpr size_t kExactSmem = (size_t)kStages * kStageBytes + 1024 + 256;

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

GM_D void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Batch rows to BF16 (round to nearest), zero padded to dh columns.
__global__ void k_to_bf16(const float *X, int ld, int d, int dh, int row0, int nrows,
                          __nv_bfloat16 *Xh) {
  const long total = (long)nrows * dh;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const int r = (int)(i / dh), c = (int)(i - (long)r * dh);
    const size_t row = (size_t)(row0 + r);
    const float v = c < d ? X[row * ld + c] : 0.0f;
    Xh[row * dh + c] = __float2bfloat16_rn(v);
  }
}

// Approximate distances of a block of batch rows against all columns.
// grid.y: 128-row tiles of the batch; grid.x: CTAs sharing the column tiles.
__global__ void __launch_bounds__(kExactThreads, 1)
    k_exact_dist(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                 int arow0, int nb, int n, int kchunks, const float *norms, float *D, long ldD,
                 unsigned *err) {
  extern __shared__ __align__(1024) unsigned char raw[];
  unsigned char *base = (unsigned char *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(base + (size_t)kStages * kStageBytes);
  uint64_t *empty = full + kStages;
  uint64_t *tmem_full = empty + kStages;
  uint64_t *tmem_empty = tmem_full + 1;
  uint32_t *tmem_slot = (uint32_t *)(tmem_empty + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.y;
  const int m0 = mt * kTM;  // batch-local first row of this tile
  const int n_tiles = (n + kTN - 1) / kTN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tmem_full, 1);
    mbar_init(tmem_empty, 128);
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
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        for (int kc = 0; kc < kchunks; ++kc, ++it) {
          const uint32_t s = it % kStages, use = it / kStages;
          if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1)) {
            ok = false;
            break;
          }
          unsigned char *a = base + (size_t)s * kStageBytes;
          mbar_expect_tx(&full[s], kStageBytes);
          tma_load_2d(&tm_a, &full[s], a, kc * kTK, arow0 + m0);
          tma_load_2d(&tm_b, &full[s], a + kABytes, kc * kTK, t * kTN);
        }
      }
      if (!ok) atomicOr(err, kDevErrSpin);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t it = 0, tc = 0;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, ++tc) {
        if (tc > 0 && !mbar_wait(tmem_empty, (tc - 1) & 1)) {
          ok = false;
          break;
        }
        tc_fence_after();
        for (int kc = 0; kc < kchunks; ++kc, ++it) {
          const uint32_t s = it % kStages, use = it / kStages;
          if (!mbar_wait(&full[s], use & 1)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a = smem_u32(base + (size_t)s * kStageBytes);
          const uint32_t b = a + kABytes;
#pragma unroll
          for (int k = 0; k < kTK / 16; ++k)
            umma_bf16(tmem, sw128_desc(a + k * 32), sw128_desc(b + k * 32),
                      (kc | k) != 0 ? 1u : 0u);
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(tmem_full);
      }
      if (!ok) atomicOr(err, kDevErrSpin);
    }
    __syncwarp();
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (tile rows)
    const int quarter = warp & 3;
    const int r = quarter * 32 + lane;
    const int m = m0 + r;
    const bool row_ok = m < nb;
    const float nm = row_ok ? norms[arow0 + m] : 0.0f;
    uint32_t tc = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++tc) {
      if (!mbar_wait(tmem_full, tc & 1)) {
        if (lane == 0) atomicOr(err, kDevErrSpin);
        break;
      }
      tc_fence_after();
      for (int c = 0; c < kTN; c += 32) {
        uint32_t v[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
        const int col0 = t * kTN + c;
        if (row_ok) {
          float *out = D + (long)m * ldD + col0;
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int j = col0 + i;
            if (j < n)
              out[i] = __fsub_rn(__fadd_rn(nm, norms[j]),
                                 __fmul_rn(2.0f, __uint_as_float(v[i])));
          }
        }
      }
      tc_fence_before();
      mbar_arrive(tmem_empty);
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

// Rigorous bound on |approx - canonical| for one pair: BF16 rounding of both
// operands (2u + u^2 with u = 2^-9) plus FP32 accumulation of <= 2048 terms in
// the tensor core and in the canonical chain, times 2 (the distance carries
// -2 dot), applied to sum|a_i b_i| <= |a||b|; plus the rounding of the norm
// sums.  0.009 covers 2 * (0.0039101 + 2048 * 2^-23 + 2048 * 2^-24) = 0.00855.
GM_D float pair_bound(float na, float nb) {
  return __fadd_rn(__fmul_rn(0.009f, __fsqrt_ru(__fmul_ru(na, nb))),
                   __fadd_rn(__fmul_rn(1e-6f, __fadd_rn(na, nb)), 1e-30f));
}

GM_D float canon_pair(const float *X, int ld, int d, const float *norms, int a, int b) {
  const float *xa = X + (size_t)a * ld;
  const float *xb = X + (size_t)b * ld;
  float dot = 0.0f;
  for (int i = 0; i < d; ++i) dot = __fmaf_rn(xa[i], xb[i], dot);
  return canon_dist(norms[a], norms[b], dot);
}

// One warp per batch row: an upper bound T on its 32nd smallest distance (the
// largest of the 32 per-lane minima of the upper bounds: there are 32 distinct
// columns at or below it), every column whose lower bound reaches T, exact
// re-scoring of those, and the exact top-32 keys written as the row's list.
constexpr int kRowWarps = 4;
__global__ void k_exact_rows(const float *D, long ldD, int arow0, int mrow0, int nrows, int n,
                             const float *X, int ld, int d, const float *norms, Key *g_key,
                             int *cand, long cand_ld, unsigned long long *stat) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ml = blockIdx.x * kRowWarps + warp;
  if (ml >= nrows) return;
  const int m = mrow0 + ml;       // batch-local row
  const int row = arow0 + m;      // global row
  const float nm = norms[row];
  const float *Dr = D + (long)m * ldD;
  float lmin = __int_as_float(0x7f800000);
  for (int j = lane; j < n; j += 32) {
    if (j == row) continue;
    lmin = fminf(lmin, __fadd_ru(Dr[j], pair_bound(nm, norms[j])));
  }
  float T = lmin;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) T = fmaxf(T, __shfl_xor_sync(0xffffffffu, T, o));
  // fewer than 32 other columns: take them all
  if (n - 1 < 32) T = __int_as_float(0x7f800000);
  int *cl = cand + (long)ml * cand_ld;
  int cnt = 0;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    bool keep = false;
    if (j < n && j != row) keep = __fsub_rd(Dr[j], pair_bound(nm, norms[j])) <= T;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (keep) cl[cnt + __popc(bal & ((1u << lane) - 1u))] = j;
    cnt += __popc(bal);
  }
  __syncwarp();
  if (lane == 0 && stat) {
    atomicAdd(&stat[5], (unsigned long long)n);
    atomicAdd(&stat[6], (unsigned long long)cnt);
  }
  Key mine = kEmptyKey;
  for (int c0 = 0; c0 < cnt; c0 += 32) {
    const int c = c0 + lane;
    Key ck = ~(Key)0;
    if (c < cnt) {
      const int j = cl[c];
      ck = make_key(canon_pair(X, ld, d, norms, row, j), j);
    }
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
  g_key[(size_t)row * kListW + lane] = mine;
}

// One thread per existing row j < n_exist: batch rows of this block whose lower
// bound does not exceed j's current last entry are re-scored and merged into
// j's list (the thread owns the list; batch rows in ascending order).
__global__ void k_exact_cols(const float *D, long ldD, int n_exist, int brow0, int nrows,
                             const float *X, int ld, int d, const float *norms, Key *g_key,
                             int *dirty, unsigned long long *stat) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_exist) return;
  Key *lst = g_key + (size_t)j * kListW;
  Key worst = lst[kListW - 1];
  const float nj = norms[j];
  bool changed = false;
  unsigned rescored = 0;
  for (int ml = 0; ml < nrows; ++ml) {
    const float a = D[(long)ml * ldD + j];
    const int row = brow0 + ml;
    const float wd = key_dist(worst);
    if (__fsub_rd(a, pair_bound(nj, norms[row])) > wd) continue;
    const Key ck = make_key(canon_pair(X, ld, d, norms, j, row), row);
    ++rescored;
    if (!(ck < worst)) continue;
    int pos = kListW - 1;
    while (pos > 0 && ck < lst[pos - 1]) {
      lst[pos] = lst[pos - 1];
      --pos;
    }
    lst[pos] = ck;
    worst = lst[kListW - 1];
    changed = true;
  }
  if (changed) dirty[j] = 1;
  if (stat && rescored) atomicAdd(&stat[6], (unsigned long long)rescored);
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

bool make_row_maps(void *xh, int n_cap, int dh, ExactMaps *out) {
  auto enc = get_encode();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)dh, (cuuint64_t)std::max(n_cap, 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)dh * 2};
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

void launch_exact_dist(const DevState &st, const ExactMaps &maps, int dh, int row0, int blk0,
                       int nrows, int n, float *D, long ldD, int sms, cudaStream_t s) {
  if (nrows <= 0 || n <= 0) return;
  static unsigned configured = 0u;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 32 && !(configured & (1u << dev))) {
    cudaFuncSetAttribute(k_exact_dist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kExactSmem);
    configured |= (1u << dev);
  }
  const int m_tiles = cdiv(nrows, kTM);
  const int n_tiles = cdiv(n, kTN);
  const int gx = std::max(1, std::min(n_tiles, std::max(1, sms / m_tiles)));
  CUtensorMap ta, tb;
  memcpy(&ta, maps.a, sizeof(ta));
  memcpy(&tb, maps.b, sizeof(tb));
  k_exact_dist<<<dim3(gx, m_tiles), kExactThreads, kExactSmem, s>>>(
      ta, tb, row0 + blk0, nrows, n, dh / kTK, st.norms, D, ldD, st.err);
  note_launch();
}

void launch_exact_screen(const DevState &st, int row0, int blk0, int nrows, int n,
                         const float *D, long ldD, int *cand, long cand_ld, cudaStream_t s) {
  if (nrows <= 0 || n <= 0) return;
  const int brow0 = row0 + blk0;  // global first row of the block
  k_exact_rows<<<cdiv(nrows, kRowWarps), kRowWarps * 32, 0, s>>>(
      D, ldD, brow0, 0, nrows, n, st.X, st.ld, st.d, st.norms, st.g_key, cand, cand_ld, st.stat);
  note_launch();
  if (row0 > 0) {
    k_exact_cols<<<cdiv(row0, 128), 128, 0, s>>>(D, ldD, row0, brow0, nrows, st.X, st.ld, st.d,
                                                 st.norms, st.g_key, st.dirty, st.stat);
    note_launch();
  }
}

}  // namespace gm
