// Device-wide exclusive scan and order-preserving compaction.  Three passes
// (per-block totals, a single-block scan of the totals, per-block write);
// results are deterministic and keep ascending index order.
#include "gm_common.cuh"
#include "gm_kernels.h"

#include <algorithm>
#include <atomic>

namespace gm {

namespace {
std::atomic<uint64_t> g_launches{0};
}  // namespace

void note_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
uint64_t launch_counter() { return g_launches.load(std::memory_order_relaxed); }
void launch_counter_reset() { g_launches.store(0, std::memory_order_relaxed); }

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;  // 1024 items per block

// Inclusive scan of one int per thread across a 256-thread block.
__device__ __forceinline__ int block_inclusive_scan(int v, int *warp_tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) warp_tot[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v += warp_tot[warp - 1];
  __syncthreads();
  return v;
}

// Predicate value of item i for the three input kinds.
struct Pred {
  const int *vals;     // plain values (scan) or flags
  const int *list;     // optional indirection list
  const int *n_dev;    // optional device length of list
  int n_host;          // host length bound
  int select;          // -1: value != 0 ; >= 0: value == select ; -2: raw value
  __device__ __forceinline__ int len() const { return n_dev ? min(*n_dev, n_host) : n_host; }
  __device__ __forceinline__ int at(int i) const {
    const int src = list ? list[i] : i;
    const int v = vals[src];
    if (select == -2) return v;
    if (select == -1) return v != 0 ? 1 : 0;
    return v == select ? 1 : 0;
  }
  __device__ __forceinline__ int id(int i) const { return list ? list[i] : i; }
};

__global__ void __launch_bounds__(kScanThreads) k_block_totals(Pred p, int *tot) {
  __shared__ int wt[kScanThreads / 32];
  const int n = p.len();
  const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += p.at(base + i);
  s = block_inclusive_scan(s, wt);
  if (threadIdx.x == kScanThreads - 1) tot[blockIdx.x] = s;
}

// Exclusive scan of tot[0..nb) in place; tot[nb] = grand total.  One block.
__global__ void __launch_bounds__(kScanThreads) k_scan_totals(int *tot, int nb,
                                                              int *total_out) {
  __shared__ int wt[kScanThreads / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb; c0 += kScanBlock) {
    const int base = c0 + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      v[i] = (base + i < nb) ? tot[base + i] : 0;
      s += v[i];
    }
    const int incl = block_inclusive_scan(s, wt);
    int run = carry + incl - s;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      if (base + i < nb) tot[base + i] = run;
      run += v[i];
    }
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry = run;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    tot[nb] = carry;
    if (total_out) *total_out = carry;
  }
}

// mode 0: exclusive scan output out[i]; mode 1: compaction out[pos] = id(i).
__global__ void __launch_bounds__(kScanThreads) k_block_write(Pred p, const int *tot,
                                                              int *out, int mode,
                                                              int n_cap_out) {
  __shared__ int wt[kScanThreads / 32];
  const int n = p.len();
  const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? p.at(base + i) : 0;
    s += v[i];
  }
  const int incl = block_inclusive_scan(s, wt);
  int run = tot[blockIdx.x] + incl - s;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) {
      if (mode == 0) {
        out[base + i] = run;
      } else if (v[i] && run < n_cap_out) {
        out[run] = p.id(base + i);
      }
    }
    run += v[i];
  }
  if (mode == 0 && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = tot[gridDim.x];
}

inline int nblocks(int n) { return n <= 0 ? 1 : (n + kScanBlock - 1) / kScanBlock; }

void run_scan(const Pred &p, int n_max, int *out, int mode, int *count, int *tmp,
              cudaStream_t s) {
  const int nb = nblocks(n_max);
  k_block_totals<<<nb, kScanThreads, 0, s>>>(p, tmp);
  note_launch();
  k_scan_totals<<<1, kScanThreads, 0, s>>>(tmp, nb, count);
  note_launch();
  k_block_write<<<nb, kScanThreads, 0, s>>>(p, tmp, out, mode, n_max);
  note_launch();
}

}  // namespace

namespace {
__global__ void k_fill_u32(uint32_t *p, uint32_t v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}
__global__ void k_fill_u64(unsigned long long *p, unsigned long long v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}
}  // namespace

void fill_u64(void *p, unsigned long long v, size_t n, cudaStream_t s) {
  if (n == 0) return;
  const size_t blocks = std::min<size_t>((n + 255) / 256, 4096);
  k_fill_u64<<<(unsigned)blocks, 256, 0, s>>>((unsigned long long *)p, v, n);
  note_launch();
}

void fill_u32(void *p, uint32_t v, size_t n, cudaStream_t s) {
  if (n == 0) return;
  const size_t blocks = std::min<size_t>((n + 255) / 256, 4096);
  k_fill_u32<<<(unsigned)blocks, 256, 0, s>>>((uint32_t *)p, v, n);
  note_launch();
}

size_t scan_tmp_ints(int n) { return (size_t)nblocks(n) + 2; }
size_t compact_tmp_ints(int n) { return (size_t)nblocks(n) + 2; }

void exclusive_scan(const int *in, int *out, int n, int *tmp, cudaStream_t s) {
  Pred p{in, nullptr, nullptr, n, -2};
  run_scan(p, n, out, 0, nullptr, tmp, s);
}

void compact_flags(const int *flag, int n, int select, int *out, int *count,
                   int *tmp, cudaStream_t s) {
  Pred p{flag, nullptr, nullptr, n, select >= 0 ? select : -1};
  run_scan(p, n, out, 1, count, tmp, s);
}

void compact_flags_dev(const int *flag, const int *n_dev, int n_max, int *out,
                       int *count, int *tmp, cudaStream_t s) {
  Pred p{flag, nullptr, n_dev, n_max, -1};
  run_scan(p, n_max, out, 1, count, tmp, s);
}

void compact_list(const int *list, const int *n_dev, int n_max, const int *pred,
                  int *out, int *count, int *tmp, cudaStream_t s) {
  Pred p{pred, list, n_dev, n_max, -1};
  run_scan(p, n_max, out, 1, count, tmp, s);
}

}  // namespace gm
