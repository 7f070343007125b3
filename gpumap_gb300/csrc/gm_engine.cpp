// Session engine: host-side policy of the progressive cycle, all numeric
// state on the device.  The queue, cursor, seed and completion rules restate
// the reference's GPUMAP::Impl (impl.cuh:29-533); the O(n) host copies and
// host merges of the reference are replaced by device kernels, so per-cycle
// host work and PCIe/C2C traffic scale with the batch, not with n.
#include "gm_engine.h"

#include "gm_common.cuh"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <unordered_set>

namespace gm {

namespace {

using Clock = std::chrono::high_resolution_clock;

void ck(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return;
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation)
    throw Error(GM_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
  throw Error(GM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }

}  // namespace

template <typename... A>
void Session::log(const char *fmt, A... a) const {
  if (p_.verbose) {
    std::fprintf(stderr, fmt, a...);
    std::fflush(stderr);
  }
}

Session::Session(const gm_params &p) : p_(p) {
  if (p.n_components != 2)
    throw Error(GM_ERR_INVALID, "n_components must be 2");
  if (p.n_neighbors < 1 || p.n_neighbors > (uint64_t)kListW)
    throw Error(GM_ERR_INVALID, "n_neighbors must be in [1, 32]");
  if (p.n_features < 1) throw Error(GM_ERR_INVALID, "n_features must be >= 1");
  if (p.metric != GM_METRIC_EUCLIDEAN && p.metric != GM_METRIC_COSINE)
    throw Error(GM_ERR_INVALID, "unknown metric");
  if (p.precision != 0 && p.precision != 1)
    throw Error(GM_ERR_INVALID, "precision must be 0 (FP32 NN-Descent) or 1 (exact, BF16 tensor cores)");
  if (p.overlap != 0 && p.overlap != 1) throw Error(GM_ERR_INVALID, "overlap must be 0 or 1");
  if (p.n_instances > (uint64_t)(1u << 30))
    throw Error(GM_ERR_INVALID, "n_instances exceeds 2^30");
  if (p.n_features > (uint64_t)(1u << 24)) throw Error(GM_ERR_INVALID, "n_features too large");

  if (p.device >= 0) ck(cudaSetDevice(p.device), "cudaSetDevice");
  ck(cudaGetDevice(&device_), "cudaGetDevice");
  ck(cudaFree(nullptr), "CUDA context");
  ck(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  ck(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_), "attr");
  if (p.overlap) {
    // the embedding stream gets the higher priority: its cooperative SGD
    // launch is placed as soon as SMs free up
    int lo = 0, hi = 0;
    ck(cudaDeviceGetStreamPriorityRange(&lo, &hi), "stream priorities");
    ck(cudaStreamCreateWithPriority(&estream_, cudaStreamNonBlocking, hi), "cudaStreamCreate");
    ck(cudaStreamCreateWithPriority(&estream_alt_, cudaStreamNonBlocking, hi), "cudaStreamCreate");
    for (cudaEvent_t *e : {&ev_pub_, &ev_emb_, &ev_snap_, &ev_init_, &ev_hpin_, &ev_hpin_alt_})
      ck(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
  }

  const size_t N = p.n_instances, d = p.n_features, k = p.n_neighbors;
  st_.n_cap = (int)N;
  st_.d = (int)d;
  st_.ld = (int)round_up(d, 4);
  st_.k = (int)k;
  st_.cosine = p.metric == GM_METRIC_COSINE;
  const size_t Nm = std::max<size_t>(N, 1);

  auto dalloc = [&](size_t bytes) -> void * {
    void *ptr = nullptr;
    ck(cudaMalloc(&ptr, std::max<size_t>(bytes, 16)), "cudaMalloc");
    allocs_.push_back(ptr);
    fixed_bytes_ += std::max<size_t>(bytes, 16);
    return ptr;
  };
  try {
    st_.X = (float *)dalloc(Nm * st_.ld * sizeof(float));
    st_.norms = (float *)dalloc(Nm * sizeof(float));
    st_.snorms = (float *)dalloc(Nm * sizeof(float));
    st_.g_key = (unsigned long long *)dalloc(Nm * kListW * sizeof(unsigned long long));
    st_.locks = (int *)dalloc(Nm * sizeof(int));
    st_.dirty = (int *)dalloc(Nm * sizeof(int));
    st_.knn_ids = (int *)dalloc(Nm * k * sizeof(int));
    st_.knn_dists = (float *)dalloc(Nm * k * sizeof(float));
    st_.pub_idx = (uint32_t *)dalloc(Nm * (k + 1) * sizeof(uint32_t));
    st_.pub_dist = (float *)dalloc(Nm * (k + 1) * sizeof(float));
    st_.emb = (float *)dalloc(Nm * 2 * sizeof(float));
    st_.bloom = (uint32_t *)dalloc(Nm * 64 * sizeof(uint32_t));
    st_.err = (unsigned *)dalloc(16);
    d_stat_ = (unsigned long long *)dalloc(16 * sizeof(unsigned long long));
    st_.stat = d_stat_;

    us_.fwd_new = (int *)dalloc(Nm * kSamples * sizeof(int));
    us_.fwd_old = (int *)dalloc(Nm * kSamples * sizeof(int));
    us_.rev_new = (int *)dalloc(Nm * kSamples * sizeof(int));
    us_.rev_old = (int *)dalloc(Nm * kSamples * sizeof(int));
    us_.sizes = (int4 *)dalloc(Nm * sizeof(int4));
    us_.cnt = (int *)dalloc(Nm * sizeof(int));
    us_.off = (int *)dalloc((Nm + 1) * sizeof(int));
    us_.fill = (int *)dalloc(Nm * sizeof(int));
    us_.csr = (int *)dalloc(Nm * kSamples * sizeof(int));
    us_.hflag = (int *)dalloc(Nm * sizeof(int));

    d_rows_ = (int *)dalloc(Nm * sizeof(int));
    d_rows2_ = (int *)dalloc(Nm * sizeof(int));
    d_batch_ = (int *)dalloc(Nm * sizeof(int));
    d_cnt_ = (int *)dalloc(16 * sizeof(int));
    d_tmp_ = (int *)dalloc(std::max(scan_tmp_ints((int)Nm), compact_tmp_ints((int)Nm)) *
                           sizeof(int) + 64);

    // the embedding phase has its own batch, scan scratch, counters and
    // pinned staging, so that it can run beside the other phases (two sets
    // in overlap mode, one per side)
    auto alloc_side = [&](EmbedScratch &e, int *&cnt) {
      e.flag = (int *)dalloc(Nm * sizeof(int));
      e.unsel = (int *)dalloc(Nm * sizeof(int));
      e.sigma = (float *)dalloc(Nm * sizeof(float));
      e.rho = (float *)dalloc(Nm * sizeof(float));
      e.deg = (int *)dalloc(Nm * sizeof(int));
      e.snap = (float *)dalloc(Nm * 2 * sizeof(float));
      e.fscal = (float *)dalloc(16 * sizeof(float));
      e.iscal = (int *)dalloc(16 * sizeof(int));
      e.cap_partial = (Nm * k + 255) / 256 + 512;
      e.partial = (float *)dalloc(e.cap_partial * 2 * sizeof(float));
      e.ipartial = (int *)dalloc(e.cap_partial * sizeof(int));
      e.batch = (int *)dalloc(Nm * sizeof(int));
      e.tmp = (int *)dalloc(std::max(scan_tmp_ints((int)Nm), compact_tmp_ints((int)Nm)) *
                            sizeof(int) + 64);
      if (p.overlap) {
        e.pub_idx_snap = (uint32_t *)dalloc(Nm * (k + 1) * sizeof(uint32_t));
        e.pub_dist_snap = (float *)dalloc(Nm * (k + 1) * sizeof(float));
      }
      cnt = (int *)dalloc(16 * sizeof(int));
    };
    alloc_side(es_, es_cnt_);
    if (p.overlap) alloc_side(es_alt_, es_cnt_alt_);

    ck(cudaMallocHost((void **)&h_pin_, (Nm + 64) * sizeof(uint32_t)), "cudaMallocHost");
    ck(cudaMallocHost((void **)&h_emb_pin_, (Nm + 64) * sizeof(uint32_t)), "cudaMallocHost");
    if (p.overlap)
      ck(cudaMallocHost((void **)&h_emb_pin_alt_, (Nm + 64) * sizeof(uint32_t)), "cudaMallocHost");
    if (p.precision == 1) {
      // split-BF16 shadow rows (hi | lo, 2 x dh bf16 each) plus a block of
      // candidate / pair scratch for the worst case (every column a
      // candidate of every block row): 28 bytes per (block row, row).  The
      // block takes up to 1,024 rows (fewer, longer launches) within an
      // eighth of the device's memory and at most 32 GB, and at least 128
      dh_ = exact_dh((int)d);
      xh_ = dalloc(Nm * (size_t)dh_ * 4);
      size_t free_b = 0, total_b = 0;
      ck(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
      const size_t budget = std::min<size_t>(total_b / 8, (size_t)32 << 30);
      ex_block_ = (int)std::max<size_t>(128, std::min<size_t>(1024, budget / (Nm * 28)));
      ex_block_ = ex_block_ / 128 * 128;
      // the approximate tile itself is only stored on request (tests), in
      // a buffer allocated then
      ex_cand_ = (int *)dalloc((size_t)ex_block_ * Nm * sizeof(int));
      xs_.cand = ex_cand_;
      xs_.cand_d = (float *)dalloc((size_t)ex_block_ * Nm * sizeof(float));
      xs_.row_cnt = (int *)dalloc((size_t)ex_block_ * sizeof(int));
      xs_.pool_cap = (long)ex_block_ * (long)Nm;
      xs_.pool_j = (int *)dalloc((size_t)xs_.pool_cap * sizeof(int));
      xs_.pool_m = (int *)dalloc((size_t)xs_.pool_cap * sizeof(int));
      xs_.pool_d = (float *)dalloc((size_t)xs_.pool_cap * sizeof(float));
      xs_.pool_j2 = (int *)dalloc((size_t)xs_.pool_cap * sizeof(int));
      xs_.pool_m2 = (int *)dalloc((size_t)xs_.pool_cap * sizeof(int));
      xs_.row_t = (float *)dalloc((size_t)ex_block_ * sizeof(float));
      xs_.seed = (float *)dalloc((size_t)ex_block_ * sizeof(float));
      // pre-candidate segments: one per (block row, CTA of a row tile), for
      // every grid width a block can take (at most one CTA per column tile)
      xs_.pre_cap = pre_cap_alloc_ = 64;
      xs_.pre_gx = (int)std::min<size_t>(std::max(sms_, 1), (Nm + 255) / 256);
      xs_.pre = (unsigned long long *)dalloc((size_t)ex_block_ * xs_.pre_gx * xs_.pre_cap *
                                             sizeof(unsigned long long));
      xs_.pre_ub = (float *)dalloc((size_t)ex_block_ * xs_.pre_gx * xs_.pre_cap * sizeof(float));
      xs_.mins_ld = exact_seed_tiles((int)((Nm + 255) / 256)) * 8;
      xs_.mins = (float *)dalloc((size_t)ex_block_ * xs_.mins_ld * sizeof(float));
      xs_.pre_cnt = (int *)dalloc((size_t)ex_block_ * xs_.pre_gx * sizeof(int));
      xs_.pre_over = (int *)dalloc(sizeof(int));
      xs_.heaps = (float *)dalloc((size_t)ex_block_ * std::max(sms_, 1) * 32 * sizeof(float));
      xs_.pcnt = (int *)dalloc((Nm + 1) * sizeof(int));
      xs_.poff = (int *)dalloc((Nm + 1) * sizeof(int));
      xs_.tmp = (int *)dalloc(scan_tmp_ints((int)Nm) * sizeof(int));
      xs_.counter = (int *)dalloc(16 * sizeof(int));
    }
  } catch (...) {
    for (void *q : allocs_) cudaFree(q);
    allocs_.clear();
    if (h_pin_) cudaFreeHost(h_pin_);
    if (h_emb_pin_) cudaFreeHost(h_emb_pin_);
    if (h_emb_pin_alt_) cudaFreeHost(h_emb_pin_alt_);
    release_streams();
    throw;
  }

  // Initial contents: zero features (padding must stay zero), empty lists,
  // "no neighbour" published rows, zero embedding.
  cudaStream_t s = stream_;
  ck(cudaMemsetAsync(st_.X, 0, Nm * st_.ld * sizeof(float), s), "memset");
  ck(cudaMemsetAsync(st_.norms, 0, Nm * sizeof(float), s), "memset");
  ck(cudaMemsetAsync(st_.snorms, 0, Nm * sizeof(float), s), "memset");
  fill_u64(st_.g_key, kEmptyKey, Nm * kListW, s);
  ck(cudaMemsetAsync(st_.locks, 0, Nm * sizeof(int), s), "memset");
  ck(cudaMemsetAsync(st_.dirty, 0, Nm * sizeof(int), s), "memset");
  fill_u32(st_.knn_ids, (uint32_t)kIdSentinel, Nm * k, s);
  fill_u32(st_.knn_dists, kFltMaxBits, Nm * k, s);
  fill_u32(st_.pub_idx, kPubIdxSentinel, Nm * (k + 1), s);
  fill_u32(st_.pub_dist, kFltMaxBits, Nm * (k + 1), s);
  ck(cudaMemsetAsync(st_.emb, 0, Nm * 2 * sizeof(float), s), "memset");
  ck(cudaMemsetAsync(st_.bloom, 0, Nm * 64 * sizeof(uint32_t), s), "memset");
  ck(cudaMemsetAsync(st_.err, 0, 16, s), "memset");
  ck(cudaMemsetAsync(d_stat_, 0, 16 * sizeof(unsigned long long), s), "memset");
  ck(cudaMemsetAsync(us_.sizes, 0, Nm * sizeof(int4), s), "memset");
  for (EmbedScratch *e : {&es_, &es_alt_}) {
    if (!e->sigma) continue;
    ck(cudaMemsetAsync(e->sigma, 0, Nm * sizeof(float), s), "memset");
    ck(cudaMemsetAsync(e->rho, 0, Nm * sizeof(float), s), "memset");
    ck(cudaMemsetAsync(e->iscal, 0, 16 * sizeof(int), s), "memset");
    ck(cudaMemsetAsync(e->fscal, 0, 16 * sizeof(float), s), "memset");
  }
  if (xh_) ck(cudaMemsetAsync(xh_, 0, Nm * (size_t)dh_ * 4, s), "memset");
  ck(cudaGetLastError(), "init fill");
  ck(cudaStreamSynchronize(s), "init sync");
  if (xh_) {
    if (!make_row_maps(xh_, (int)Nm, dh_, &maps_)) {
      for (void *q : allocs_) cudaFree(q);
      allocs_.clear();
      cudaFreeHost(h_pin_);
      h_pin_ = nullptr;
      cudaFreeHost(h_emb_pin_);
      h_emb_pin_ = nullptr;
      if (h_emb_pin_alt_) cudaFreeHost(h_emb_pin_alt_);
      h_emb_pin_alt_ = nullptr;
      release_streams();
      throw Error(GM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable or failed");
    }
  }
  upd_q_.reset(N);
  ensure_embed(es_, 1);
  if (p.overlap) ensure_embed(es_alt_, 1);
}

void Session::release_streams() {
  for (cudaEvent_t *e : {&ev_pub_, &ev_emb_, &ev_snap_, &ev_init_, &ev_hpin_, &ev_hpin_alt_}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  for (cudaStream_t *q : {&estream_, &estream_alt_, &stream_}) {
    if (*q) cudaStreamDestroy(*q);
    *q = nullptr;
  }
}

// Waits for both embedding sides.
void Session::sync_embed_streams() {
  for (cudaStream_t q : {estream_, estream_alt_})
    if (q) ck(cudaStreamSynchronize(q), "cudaStreamSynchronize");
}

void Session::free_embed(EmbedScratch &e) {
  if (!e.coo_row) return;
  for (void *q : {(void *)e.coo_row, (void *)e.coo_col, (void *)e.coo_val, (void *)e.t_row,
                  (void *)e.t_col, (void *)e.flag_tail, (void *)e.t_val, (void *)e.next_s,
                  (void *)e.next_n, (void *)e.tmp2})
    cudaFree(q);
  e.coo_row = nullptr;
  e.cap_coo = 0;
}

Session::~Session() {
  for (cudaStream_t q : {stream_, estream_, estream_alt_})
    if (q) cudaStreamSynchronize(q);
  for (auto &e : ev_pool_) cudaEventDestroy(e);
  for (auto &pr : ev_pending_) {
    cudaEventDestroy(pr.a);
    cudaEventDestroy(pr.b);
  }
  for (void *q : allocs_) cudaFree(q);
  if (cand_) cudaFree(cand_);
  if (cand_cnt_) cudaFree(cand_cnt_);
  if (cand_dist_) cudaFree(cand_dist_);
  free_embed(es_);
  free_embed(es_alt_);
  if (h_pin_) cudaFreeHost(h_pin_);
  if (h_emb_pin_) cudaFreeHost(h_emb_pin_);
  if (h_emb_pin_alt_) cudaFreeHost(h_emb_pin_alt_);
  if (cstream_) cudaStreamSynchronize(cstream_);
  for (auto &slot : ring_) {
    if (slot.done) cudaEventDestroy(slot.done);
    if (slot.buf) cudaFreeHost(slot.buf);
  }
  if (cstream_) cudaStreamDestroy(cstream_);
  release_streams();
}

void Session::sync() { ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize"); }

// The consumer stream waits (on the device) for the work queued so far on
// the main and the embedding streams; the main stream already waits for
// every row transfer.
void Session::order_after(cudaStream_t consumer) const {
  for (cudaStream_t producer : {stream_, estream_, estream_alt_}) {
    if (!producer) continue;
    cudaEvent_t ev = nullptr;
    ck(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    const cudaError_t e1 = cudaEventRecord(ev, producer);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(consumer, ev, 0) : e1;
    cudaEventDestroy(ev);  // the wait keeps the recorded work
    ck(e2, "stream wait");
  }
}

// Waits for every phase in flight, the overlapped embedding included, and
// reports a device error bit raised meanwhile.
void Session::drain() {
  sync();
  sync_embed_streams();
  emb_pending_ = snap_pending_ = init_wait_ = false;
  check_device_error("embedding");
}

void Session::check_launch_error(const char *phase) {
  // a launch the runtime refused (resources, configuration) is reported
  // once, by the next query of the last error
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) ck(le, (std::string(phase) + " launch").c_str());
}

void Session::check_device_error(const char *phase) {
  check_launch_error(phase);
  unsigned e = 0;
  ck(cudaMemcpyAsync(&e, st_.err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream_), "err");
  sync();
  if (e != 0u) {
    cudaMemsetAsync(st_.err, 0, sizeof(unsigned), stream_);
    throw Error(GM_ERR_DEVICE, std::string(phase) + ": a bounded device wait ran out (bits " +
                                   std::to_string(e) + ")");
  }
}

void Session::ensure_cand(size_t rows) {
  if (rows <= cand_rows_) return;
  sync();
  if (cand_) cudaFree(cand_);
  if (cand_cnt_) cudaFree(cand_cnt_);
  if (cand_dist_) cudaFree(cand_dist_);
  cand_ = nullptr;
  cand_cnt_ = nullptr;
  cand_dist_ = nullptr;
  cand_rows_ = 0;
  const size_t r = std::max<size_t>(rows, 1024);
  ck(cudaMalloc(&cand_, r * kMaxCand * sizeof(int)), "cudaMalloc cand");
  ck(cudaMalloc(&cand_cnt_, r * sizeof(int)), "cudaMalloc cand");
  ck(cudaMalloc(&cand_dist_, r * kMaxCand * sizeof(float)), "cudaMalloc cand");
  cand_rows_ = r;
}

void Session::set_pre_cap(int cap) {
  drain();
  xs_.pre_cap = std::max(0, std::min(cap, pre_cap_alloc_));
  xs_.pre_fixed = true;
}

void Session::set_keep_tile(bool on) {
  if (on && p_.precision == 1 && !ex_D_) {
    drain();
    const size_t bytes = (size_t)ex_block_ * std::max<size_t>(p_.n_instances, 1) * sizeof(float);
    void *ptr = nullptr;
    ck(cudaMalloc(&ptr, bytes), "cudaMalloc tile");
    allocs_.push_back(ptr);
    fixed_bytes_ += bytes;
    ex_D_ = (float *)ptr;
    xs_.D = ex_D_;
  }
  keep_tile_ = on;
}

size_t Session::device_bytes() const {
  size_t b = fixed_bytes_;
  b += cand_rows_ * (size_t)kMaxCand * (sizeof(int) + sizeof(float)) + cand_rows_ * sizeof(int);
  for (const EmbedScratch *e : {&es_, &es_alt_})
    if (e->coo_row) b += e->cap_coo * 9 * 4 + (compact_tmp_ints((int)e->cap_coo) + 64) * sizeof(int);
  return b;
}

size_t Session::growth_bytes(uint32_t n_ins, uint32_t n_emb) const {
  size_t g = 0;
  if (p_.precision == 0 && n_ins > cand_rows_) {
    const size_t r = std::max<size_t>(n_ins, 1024);
    g += r * (size_t)kMaxCand * (sizeof(int) + sizeof(float)) + r * sizeof(int);
  }
  // an embedding batch takes the queued new rows plus the cursor's rows
  const size_t nb = std::max<size_t>(n_emb, n_inserted_ + n_ins - emb_new_head_);
  const size_t c = std::max<size_t>(2 * std::max<size_t>(nb, 1) * (size_t)st_.k, 4096);
  // (in overlap mode the next phase runs on the other side)
  const EmbedScratch &next = p_.overlap ? es_alt_ : es_;
  if (n_emb > 0 && c > next.cap_coo) g += c * 9 * 4 + (compact_tmp_ints((int)c) + 64) * sizeof(int);
  return g;
}

void Session::ensure_embed(EmbedScratch &e, size_t nb) {
  const size_t need = 2 * std::max<size_t>(nb, 1) * (size_t)st_.k;
  if (need <= e.cap_coo) return;
  sync();
  sync_embed_streams();
  free_embed(e);
  const size_t c = std::max(need, (size_t)4096);
  ck(cudaMalloc(&e.coo_row, c * sizeof(int)), "cudaMalloc coo");
  ck(cudaMalloc(&e.coo_col, c * sizeof(int)), "cudaMalloc coo");
  ck(cudaMalloc(&e.coo_val, c * sizeof(float)), "cudaMalloc coo");
  ck(cudaMalloc(&e.t_row, c * sizeof(int)), "cudaMalloc coo");
  ck(cudaMalloc(&e.t_col, c * sizeof(int)), "cudaMalloc coo");
  ck(cudaMalloc(&e.flag_tail, c * sizeof(int)), "cudaMalloc coo");
  ck(cudaMalloc(&e.t_val, c * sizeof(float)), "cudaMalloc coo");
  ck(cudaMalloc(&e.next_s, c * sizeof(float)), "cudaMalloc coo");
  ck(cudaMalloc(&e.next_n, c * sizeof(float)), "cudaMalloc coo");
  ck(cudaMalloc(&e.tmp2, (compact_tmp_ints((int)c) + 64) * sizeof(int)), "cudaMalloc coo");
  e.cap_coo = c;
}

// ---------------------------------------------------------------------------
// statistics: CUDA events around the launches of interest
// ---------------------------------------------------------------------------
void Session::timed_begin(int slot, cudaStream_t s) {
  if (!stats_on_) return;
  if (!s) s = stream_;
  cudaEvent_t a, b;
  if (ev_pool_.size() >= 2) {
    a = ev_pool_.back();
    ev_pool_.pop_back();
    b = ev_pool_.back();
    ev_pool_.pop_back();
  } else {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  cudaEventRecord(a, s);
  ev_pending_.push_back({a, b, slot});
}

void Session::timed_end(int slot, cudaStream_t s) {
  if (!stats_on_ || ev_pending_.empty()) return;
  (void)slot;
  cudaEventRecord(ev_pending_.back().b, s ? s : stream_);
}

// Accumulates the event pairs in order; without `block`, stops at the first
// pair still in flight (an overlapped embedding) and keeps the rest.
void Session::collect_timings(bool block) {
  if (ev_pending_.empty()) return;
  size_t done = 0;
  for (auto &pr : ev_pending_) {
    if (!block && cudaEventQuery(pr.b) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    ++done;
    float ms = 0.0f;
    if (cudaEventSynchronize(pr.b) == cudaSuccess && cudaEventElapsedTime(&ms, pr.a, pr.b) == cudaSuccess) {
      if (pr.slot == 0) {
        stats_.join_ms += ms;
        stats_.join_launches += 1;
      } else if (pr.slot == 1) {
        stats_.cand_ms += ms;
        stats_.cand_launches += 1;
      } else if (pr.slot == 2) {
        stats_.sgd_ms += ms;
        stats_.sgd_launches += 1;
      } else if (pr.slot == 3) {
        stats_.exact_ms += ms;
        stats_.exact_launches += 1;
      } else if (pr.slot == 4) {
        stats_.screen_ms += ms;
      }
    }
    ev_pool_.push_back(pr.a);
    ev_pool_.push_back(pr.b);
  }
  ev_pending_.erase(ev_pending_.begin(), ev_pending_.begin() + (long)done);
}

void Session::reset_stats() {
  sync();
  collect_timings();
  stats_ = gm_stats{};
  cudaMemsetAsync(d_stat_, 0, 16 * sizeof(unsigned long long), stream_);
  launch_counter_reset();
  sync();
}

void Session::get_stats(gm_stats *out) {
  sync();
  sync_embed_streams();
  collect_timings(true);
  unsigned long long h[16];
  ck(cudaMemcpy(h, d_stat_, sizeof(h), cudaMemcpyDeviceToHost), "stats");
  stats_.join_nodes = h[0];
  stats_.join_rows = h[1];
  stats_.join_pairs = h[2];
  stats_.join_merges = h[3];
  stats_.cand_rows = h[4];
  stats_.exact_pairs = h[5];
  stats_.exact_rescored = h[6];
  stats_.sgd_edges = h[7];
  stats_.sgd_negatives = h[8];
  stats_.exact_overflow_blocks = h[9];
  stats_.kernel_launches = launch_counter();
  *out = stats_;
}

// ---------------------------------------------------------------------------
// append (reference impl.cuh:77-101)
// ---------------------------------------------------------------------------
// Appends rows at [n_inserted, +n_rows) of X (row stride ld; reference
// append_host, matrix_utils.cuh:50-63, a cudaMemcpy2DAsync into stride d+1).
// Host rows go through the ingest ring: a copy stream and two pinned staging
// slots.  Rows already in page-locked memory are copied from where they are;
// pageable rows are first copied into the next slot (waiting only for that
// slot's previous transfer).  The main stream waits for the transfer on the
// device, so the host returns as soon as it is queued and the transfer of
// the next chunk overlaps the work still running (an overlapped embedding).
void Session::append(const float *rows, size_t n_rows, size_t n_cols, bool on_device) {
  if (closed_) throw Error(GM_ERR_CLOSED, "session is closed");
  if (n_rows == 0) return;
  if (n_cols != p_.n_features)
    throw Error(GM_ERR_RUNTIME, "n_features mismatch with numpy array second dimension.");
  if (rows == nullptr) throw Error(GM_ERR_RUNTIME, "null input rows");
  if (n_inserted_ + n_rows > p_.n_instances)
    throw Error(GM_ERR_CAPACITY, "Exceeding maximum number of rows in storage");
  float *dst = st_.X + n_inserted_ * (size_t)st_.ld;
  const size_t pitch = (size_t)st_.ld * sizeof(float), width = n_cols * sizeof(float);
  if (on_device) {
    ck(cudaMemcpy2DAsync(dst, pitch, rows, width, width, n_rows, cudaMemcpyDeviceToDevice, stream_),
       "append copy");
  } else {
    if (!cstream_) {
      ck(cudaStreamCreateWithFlags(&cstream_, cudaStreamNonBlocking), "cudaStreamCreate");
      for (auto &slot : ring_) ck(cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming), "cudaEventCreate");
    }
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, rows) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    RingSlot &slot = ring_[ring_next_];
    ring_next_ = (ring_next_ + 1) % kRingSlots;
    const float *src = rows;
    if (!pinned) {
      const size_t bytes = n_rows * width;
      ck(cudaEventSynchronize(slot.done), "ingest slot");  // its previous transfer
      if (slot.cap < bytes) {
        if (slot.buf) cudaFreeHost(slot.buf);
        slot.buf = nullptr;
        slot.cap = 0;
        ck(cudaMallocHost(&slot.buf, std::max<size_t>(bytes, (size_t)8 << 20)), "cudaMallocHost ingest");
        slot.cap = std::max<size_t>(bytes, (size_t)8 << 20);
      }
      std::memcpy(slot.buf, rows, bytes);
      src = (const float *)slot.buf;
    }
    ck(cudaMemcpy2DAsync(dst, pitch, src, width, width, n_rows, cudaMemcpyHostToDevice, cstream_),
       "append copy");
    ck(cudaEventRecord(slot.done, cstream_), "ingest event");
    ck(cudaStreamWaitEvent(stream_, slot.done, 0), "ingest wait");
    if (pinned) {
      // the caller's buffer is in use until the transfer ends: block here
      // rather than let the caller overwrite it (the slot event covers it)
      ck(cudaEventSynchronize(slot.done), "append copy");
    }
  }
  n_inserted_ += n_rows;
}

// ---------------------------------------------------------------------------
// run (reference impl.cuh:146-218)
// ---------------------------------------------------------------------------
gm_result Session::run(uint32_t n_ins, uint32_t n_upd, uint32_t n_emb) {
  if (closed_) throw Error(GM_ERR_CLOSED, "session is closed");
  gm_result r{};
  log("[GPUMAP] run() start: insert=%u update=%u embed=%u inserted=%zu\n", n_ins, n_upd, n_emb,
      n_inserted_);
  // overlap mode: with no update in between, the new rows' embedding moves to
  // the start of this run's embedding phase (it must follow the phase in
  // flight, which the insertion itself need not wait for)
  defer_init_ = p_.overlap && n_upd == 0 && n_emb != 0 && !emb_done_;
  if (!ins_done_) {
    const auto t0 = Clock::now();
    r.n_insertion_ops = insert(n_ins);
    sync();
    check_device_error("insertion");
    const auto t1 = Clock::now();
    r.insertion_time = std::chrono::duration<float>(t1 - t0).count();
    ins_done_ = (ins_head_ == n_inserted_) && n_inserted_ == p_.n_instances;
    log("[GPUMAP] insert done: actual=%u time=%.3fs\n", r.n_insertion_ops, r.insertion_time);
  }
  if (n_upd != 0 && !upd_done_) {
    size_t changed = 0;
    const auto t0 = Clock::now();
    r.n_update_ops = update(n_upd, changed);
    sync();
    check_device_error("update");
    const auto t1 = Clock::now();
    r.n_update_changed_edges = changed;
    r.update_time = std::chrono::duration<float>(t1 - t0).count();
    log("[GPUMAP] update done: actual=%u changed_edges=%zu time=%.3fs\n", r.n_update_ops,
        changed, r.update_time);
  }
  r.embedding_pending_edges = n_inserted_;
  if (n_emb != 0 && n_inserted_ != 0 && !emb_done_) {
    const auto t0 = Clock::now();
    r.n_embedding_ops = embed(n_emb);
    if (!p_.overlap) {
      sync();
      check_device_error("embedding");
    } else {
      check_launch_error("embedding");
    }
    const auto t1 = Clock::now();
    r.embedding_time = std::chrono::duration<float>(t1 - t0).count();
    log("[GPUMAP] embed done: actual=%u time=%.3fs\n", r.n_embedding_ops, r.embedding_time);
  }
  flush_init();
  defer_init_ = false;
  collect_timings(!p_.overlap);
  stats_.phase_s[0] += r.insertion_time;
  stats_.phase_s[1] += r.update_time;
  stats_.phase_s[2] += r.embedding_time;
  r.n_inserted_instances = n_inserted_;
  r.insertion_queue_size = n_inserted_ - ins_head_;
  r.update_queue_size = upd_q_.size();
  r.embedding_queue_size = r.embedding_pending_edges;
  r.insertion_completed = ins_done_;
  r.update_completed = upd_done_;
  r.embedding_completed = emb_done_;
  return r;
}

// ---------------------------------------------------------------------------
// insertion (reference impl.cuh:220-253, insertion_kernel.cuh:926-1095)
// ---------------------------------------------------------------------------
uint32_t Session::insert(uint32_t n_ops) {
  const size_t qsize = n_inserted_ - ins_head_;
  if (qsize == 0 || n_ops == 0) return 0;
  const size_t B = std::min<size_t>(n_ops, qsize);
  const int row0 = (int)ins_head_;
  ins_head_ += B;
  batch_hist_.push_back((uint32_t)row0);
  if ((int)batch_hist_.size() > kWindowBatches) batch_hist_.pop_front();
  const int window_start = (int)batch_hist_.front();
  const int seed_i = (int)(n_ops * 9973u + (uint32_t)n_inserted_ * 7919u);
  const uint64_t seed = (uint64_t)(int64_t)seed_i;
  const int n = (int)n_inserted_;
  const int nb = (int)B;
  cudaStream_t s = stream_;

  if (!bloom_clean_) {
    ck(cudaMemsetAsync(st_.bloom, 0, (size_t)st_.n_cap * 64 * sizeof(uint32_t), s), "bloom");
    bloom_clean_ = true;
  }
  ck(cudaMemsetAsync(st_.dirty, 0, (size_t)n * sizeof(int), s), "dirty");
  launch_row_norms(st_, row0, nb, s);
  // the previous insertion's rows get their embedding at the start of the
  // embedding phase that followed it, from their working lists: no list
  // changes before that has run
  auto wait_init = [&] {
    if (init_wait_) ck(cudaStreamWaitEvent(s, ev_init_, 0), "wait row embedding");
    init_wait_ = false;
  };
  if (p_.precision == 1) {
    // exact lists: every batch row against every inserted row on the tensor
    // cores, re-scored in FP32 where the split-BF16 bound cannot decide
    launch_to_bf16(st_, xh_, dh_, row0, nb, s);
    // columns: the rows inserted so far (rows appended but still queued have
    // no norms or shadow rows yet)
    const int ncol = row0 + nb;
    for (int b0 = 0; b0 < nb; b0 += ex_block_) {
      const int rows = std::min(ex_block_, nb - b0);
      timed_begin(3);
      launch_exact_dist(st_, maps_, dh_, row0, b0, rows, ncol, xs_, (long)ncol, keep_tile_, sms_, s);
      timed_end(3);
      wait_init();
      timed_begin(4);
      launch_exact_screen(st_, row0, b0, rows, ncol, xs_, (long)ncol, sms_, s);
      timed_end(4);
      // algorithmic work: three BF16 products per padded feature (hi.hi,
      // hi.lo, lo.hi) for every pair, once (the seed pass, and pass 2 after
      // an overflow, are overhead on the same pairs)
      const uint64_t flops = 6ull * (uint64_t)rows * (uint64_t)ncol * (uint64_t)dh_;
      stats_.exact_flops += (double)(stats_on_ ? flops : 0);
    }
  } else {
    ensure_cand(B);
    wait_init();
    launch_random_init(st_, row0, nb, n, window_start, seed, s);
    for (int it = 0; it < kInsertIters; ++it) {
      launch_sample_candidates(st_, row0, nb, n, cand_, cand_cnt_, s);
      timed_begin(1);
      launch_candidate_dists(st_, row0, nb, cand_, cand_cnt_, cand_dist_, s);
      timed_end(1);
      launch_forward_merge(st_, row0, nb, cand_, cand_cnt_, cand_dist_, s);
      if (row0 > 0) launch_reverse_insert(st_, row0, nb, cand_, cand_cnt_, cand_dist_, s);
    }
  }
  // existing rows whose list changed, ascending
  compact_flags(st_.dirty, row0, -1, d_rows_, d_cnt_, d_tmp_, s);
  // the embedding phase in flight reads the published table until its
  // snapshot (overlap mode) and the embedding until it ends
  if (snap_pending_) ck(cudaStreamWaitEvent(s, ev_snap_, 0), "wait snapshot");
  else if (emb_pending_) ck(cudaStreamWaitEvent(s, ev_emb_, 0), "wait embedding");
  launch_adopt_and_publish(st_, row0, nb, d_rows_, d_cnt_, row0, n, s);
  if (defer_init_) {
    // the new rows' embedding waits for the phase in flight; it runs at the
    // start of this run's embedding phase
    init_pending_ = nb > 0;
    init_row0_ = (int)row0;
    init_nb_ = nb;
    init_n_ = (int)n;
  } else {
    if (emb_pending_) ck(cudaStreamWaitEvent(s, ev_emb_, 0), "wait embedding");
    launch_embed_init(st_, row0, nb, n, s);
  }
  ck(cudaMemcpyAsync(h_pin_, d_cnt_, sizeof(int), cudaMemcpyDeviceToHost, s), "count");
  sync();
  if (!defer_init_) emb_pending_ = snap_pending_ = false;  // the stream waited for it above
  const int nd = (int)h_pin_[0];
  if (nd > 0) {
    ck(cudaMemcpyAsync(h_pin_, d_rows_, (size_t)nd * sizeof(int), cudaMemcpyDeviceToHost, s),
       "rows");
    sync();
  }
  // affected = batch rows then changed existing rows (insertion_kernel.cuh:1039-1089)
  for (int i = 0; i < nb; ++i) upd_q_.push((uint32_t)(row0 + i));
  for (int i = 0; i < nd; ++i) upd_q_.push(h_pin_[i]);
  return (uint32_t)B;
}

// ---------------------------------------------------------------------------
// update (reference impl.cuh:255-333)
// ---------------------------------------------------------------------------
uint32_t Session::update(uint32_t n_ops, size_t &changed) {
  changed = 0;
  const size_t n = n_inserted_;
  if (n_ops == 0 || upd_done_ || n == 0) return 0;
  // the update republishes rows the embedding in flight reads (until its
  // snapshot in overlap mode) and changes working lists
  if (snap_pending_) ck(cudaStreamWaitEvent(stream_, ev_snap_, 0), "wait snapshot");
  else if (emb_pending_) ck(cudaStreamWaitEvent(stream_, ev_emb_, 0), "wait embedding");
  if (init_wait_) ck(cudaStreamWaitEvent(stream_, ev_init_, 0), "wait row embedding");
  init_wait_ = false;
  const size_t threshold = (size_t)(0.0001f * (float)n);
  uint32_t left = n_ops;
  while (left > 0) {
    std::vector<uint32_t> batch;
    if ((size_t)left >= n) {
      upd_q_.pop_n(upd_q_.size());
      batch.resize(n);
      std::iota(batch.begin(), batch.end(), 0u);
    } else if ((size_t)left >= upd_q_.size()) {
      batch = upd_q_.pop_n(upd_q_.size());
      std::vector<char> seen(n, 0);
      for (uint32_t v : batch) seen[v] = 1;
      std::uniform_int_distribution<uint32_t> dist(0, (uint32_t)(n - 1));
      uint32_t start = dist(rng_);
      while (batch.size() < (size_t)left) {
        const uint32_t c = (start++) % (uint32_t)n;
        if (!seen[c]) {
          seen[c] = 1;
          batch.push_back(c);
        }
      }
    } else {
      batch = upd_q_.pop_n(left);
    }
    if (batch.empty()) break;
    const size_t raw = batch.size();
    std::vector<uint32_t> affected;
    changed += update_round(batch, affected);
    left -= (uint32_t)raw;
    for (uint32_t v : affected) upd_q_.push(v);
    if (upd_q_.size() < threshold) {
      upd_done_ = (n == p_.n_instances);
      break;
    }
  }
  return n_ops - left;
}

// One UpdateAlgo::run (update_kernel.cuh:913-1054) on a batch.
size_t Session::update_round(std::vector<uint32_t> &batch, std::vector<uint32_t> &affected) {
  std::sort(batch.begin(), batch.end());
  batch.erase(std::unique(batch.begin(), batch.end()), batch.end());
  const int nb = (int)batch.size();
  const int n = (int)n_inserted_;
  cudaStream_t s = stream_;
  std::memcpy(h_pin_, batch.data(), (size_t)nb * sizeof(uint32_t));
  ck(cudaMemcpyAsync(d_batch_, h_pin_, (size_t)nb * sizeof(int), cudaMemcpyHostToDevice, s),
     "batch");
  ck(cudaMemsetAsync(us_.sizes, 0, (size_t)n * sizeof(int4), s), "sizes");
  ck(cudaMemsetAsync(st_.dirty, 0, (size_t)n * sizeof(int), s), "dirty");
  launch_sample_graph(st_, us_, d_batch_, nb, n, s);
  bloom_clean_ = false;
  build_reverse(st_, us_, d_batch_, nb, n, 0, d_tmp_, s);
  build_reverse(st_, us_, d_batch_, nb, n, 1, d_tmp_, s);
  launch_join_flags(us_, n, us_.hflag, s);
  compact_flags(us_.hflag, n, -1, d_rows_, d_cnt_ + 3, d_tmp_, s);
  timed_begin(0);
  launch_local_join(st_, us_, d_rows_, d_cnt_ + 3, n, n, s);
  timed_end(0);
  ck(cudaMemsetAsync(d_cnt_ + 1, 0, sizeof(int), s), "edges");
  launch_merge_publish(st_, us_, nullptr, nullptr, n, n, d_cnt_ + 1, us_.hflag, s);
  compact_flags(us_.hflag, n, -1, d_rows_, d_cnt_ + 2, d_tmp_, s);
  ck(cudaMemcpyAsync(h_pin_, d_cnt_, 4 * sizeof(int), cudaMemcpyDeviceToHost, s), "counts");
  sync();
  const int edges = (int)h_pin_[1];
  const int na = (int)h_pin_[2];
  if (na > 0) {
    ck(cudaMemcpyAsync(h_pin_, d_rows_, (size_t)na * sizeof(int), cudaMemcpyDeviceToHost, s),
       "affected");
    sync();
    affected.assign(h_pin_, h_pin_ + na);
  }
  return (size_t)edges;
}

// ---------------------------------------------------------------------------
// embedding (reference impl.cuh:335-500)
// ---------------------------------------------------------------------------
uint32_t Session::embed(uint32_t n_ops) {
  const size_t n = n_inserted_;
  if (n_ops == 0 || n == 0) return 0;
  const size_t total_n = p_.n_instances;
  std::vector<uint32_t> batch;
  if ((size_t)n_ops >= n) {
    emb_new_head_ = n_inserted_;
    batch.resize(n);
    std::iota(batch.begin(), batch.end(), 0u);
    emb_cursor_ = n - 1;
    if (emb_cursor_ == total_n - 1 && upd_done_) ++sweeps_;
  } else {
    for (size_t v = emb_new_head_; v < n_inserted_; ++v) batch.push_back((uint32_t)v);
    emb_new_head_ = n_inserted_;
    size_t left = batch.size() >= (size_t)n_ops ? 0 : (size_t)n_ops - batch.size();
    if (left > 0) {
      std::vector<char> seen(n, 0);
      for (uint32_t v : batch) seen[v] = 1;
      size_t cursor = (emb_cursor_ == SIZE_MAX) ? 0 : (emb_cursor_ + 1) % n;
      for (size_t checked = 0; left > 0 && checked < n; ++checked) {
        if (!seen[cursor]) {
          seen[cursor] = 1;
          batch.push_back((uint32_t)cursor);
          emb_cursor_ = cursor;
          if (emb_cursor_ == total_n - 1 && upd_done_) ++sweeps_;
          --left;
        }
        cursor = (cursor + 1) % n;
      }
    }
  }
  log("[GPUMAP] embed batch_size=%zu cursor=%zu\n", batch.size(), emb_cursor_);
  const int nb = (int)batch.size();
  const int ni = (int)n;
  const int k = st_.k;
  cudaStream_t s = stream_;
  if (p_.overlap) {
    // this phase takes the other side (stream, scratch, staging); it reads
    // the table the insertion just published
    std::swap(estream_, estream_alt_);
    std::swap(es_, es_alt_);
    std::swap(es_cnt_, es_cnt_alt_);
    std::swap(h_emb_pin_, h_emb_pin_alt_);
    std::swap(ev_hpin_, ev_hpin_alt_);
    ck(cudaEventRecord(ev_pub_, stream_), "record publish");
    ck(cudaStreamWaitEvent(estream_, ev_pub_, 0), "wait publish");
    s = estream_;
    // the side's staging was last read by the upload two phases ago
    ck(cudaEventSynchronize(ev_hpin_), "staging");
  }
  ensure_embed(es_, (size_t)nb);
  std::memcpy(h_emb_pin_, batch.data(), (size_t)nb * sizeof(uint32_t));
  ck(cudaMemcpyAsync(es_.batch, h_emb_pin_, (size_t)nb * sizeof(int), cudaMemcpyHostToDevice, s),
     "batch");
  if (p_.overlap) ck(cudaEventRecord(ev_hpin_, s), "record staging");
  const int euclid = p_.metric == GM_METRIC_EUCLIDEAN;
  const double target = std::log2((double)(k - 1));
  launch_fuzzy_graph(st_.pub_idx, st_.pub_dist, ni, k, euclid, es_.batch, nb, target, es_, s);
  if (sweeps_ > 2) emb_done_ = upd_done_;
  const uint64_t noise_seed = 42ull ^ (uint64_t)sweeps_;
  const int nu = ni - nb;
  const uint32_t *heur_idx = st_.pub_idx;
  const float *heur_dist = st_.pub_dist;
  // the rows the reposition step moves (those not in the batch) and the
  // SGD's row count depend only on the batch: queued before the phase
  // waits for the previous one (after the schedule, whose compaction
  // shares the flag scratch)
  auto select_unsel = [&] {
    launch_set_int(es_.iscal + kIscalN, ni, s);
    if (nu <= 0) return;
    ck(cudaMemsetAsync(es_.flag, 0, (size_t)ni * sizeof(int), s), "flags");
    launch_mark_rows(es_.batch, nb, es_.flag, s);
    compact_flags(es_.flag, ni, 0, es_.unsel, es_cnt_, es_.tmp, s);
  };
  if (!p_.overlap) {
    launch_add_noise(st_.emb, ni, es_.batch, nb, 0.001f, noise_seed, es_, s);
    launch_schedule(ni, nb, k, p_.alpha, (int)p_.max_epoch, (int)p_.negative_sample_rate, es_, s);
    select_unsel();
  } else {
    // the fuzzy set and schedule read only the published table: they run
    // beside the previous phase's SGD.  The reposition step reads the table
    // as it is now (a snapshot: the next insertion may publish before it
    // runs).  Noise, the new rows' embedding and the SGD read the embedding
    // and wait for the previous phase.
    launch_schedule(ni, nb, k, p_.alpha, (int)p_.max_epoch, (int)p_.negative_sample_rate, es_, s);
    select_unsel();
    if (nu > 0) {
      const size_t w = (size_t)ni * (size_t)(k + 1);
      ck(cudaMemcpyAsync(es_.pub_idx_snap, st_.pub_idx, w * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                         s), "snapshot");
      ck(cudaMemcpyAsync(es_.pub_dist_snap, st_.pub_dist, w * sizeof(float), cudaMemcpyDeviceToDevice,
                         s), "snapshot");
      heur_idx = es_.pub_idx_snap;
      heur_dist = es_.pub_dist_snap;
    }
    ck(cudaEventRecord(ev_snap_, s), "record snapshot");
    snap_pending_ = true;
    if (emb_pending_) ck(cudaStreamWaitEvent(s, ev_emb_, 0), "wait embedding");
    if (init_pending_) {
      launch_embed_init(st_, init_row0_, init_nb_, init_n_, s);
      ck(cudaEventRecord(ev_init_, s), "record row embedding");
      init_pending_ = false;
      init_wait_ = true;
    }
    launch_add_noise(st_.emb, ni, es_.batch, nb, 0.001f, noise_seed, es_, s);
  }
  timed_begin(2, s);
  run_sgd(s);
  timed_end(2, s);
  if (nu > 0) launch_heuristic(heur_idx, heur_dist, ni, k, euclid, es_.unsel, nu, st_.emb, es_, s);
  if (p_.overlap) {
    ck(cudaEventRecord(ev_emb_, s), "record embedding");
    emb_pending_ = true;
  }
  return (uint32_t)nb;
}

// A deferred embedding of new rows whose phase did not run: on the main
// stream, after the phase in flight.
void Session::flush_init() {
  if (!init_pending_) return;
  if (emb_pending_) ck(cudaStreamWaitEvent(stream_, ev_emb_, 0), "wait embedding");
  launch_embed_init(st_, init_row0_, init_nb_, init_n_, stream_);
  init_pending_ = false;
}

// The max_epoch SGD epochs of one embedding call: one cooperative launch
// with a grid barrier between epochs (sizes are read from device scalars).
// t_col (free once the schedule is built) holds the edge grouping and
// ipartial its bins.
void Session::run_sgd(cudaStream_t s) {
  if (p_.max_epoch == 0) return;
  // overlapped: half the SMs, the other half stays free for the next cycle's
  // distance work (the per-epoch time does not depend on it)
  const int max_ctas = p_.overlap ? std::max(1, sms_ / 2) : 0;
  ck(launch_sgd_call(st_.emb, es_.t_row, es_.flag_tail, es_.t_val, es_.next_s, es_.next_n,
                     es_.iscal, es_.fscal, p_.alpha, 1.0f, p_.a, p_.b, (int)p_.max_epoch,
                     (int)p_.negative_sample_rate, 42ull, (unsigned *)(es_.iscal + kIscalBarrier),
                     st_.err, device_, s, st_.stat, max_ctas),
     "SGD launch");
}

void Session::close() {
  if (closed_) return;
  cudaStreamSynchronize(stream_);
  for (cudaStream_t q : {estream_, estream_alt_})
    if (q) cudaStreamSynchronize(q);
  emb_pending_ = snap_pending_ = init_wait_ = false;
  closed_ = true;
}

void Session::debug_scalars(int64_t *out, int cnt) const {
  int iscal[16] = {0};
  unsigned err = 0;
  cudaStreamSynchronize(stream_);
  for (cudaStream_t q : {estream_, estream_alt_})
    if (q) cudaStreamSynchronize(q);
  cudaMemcpy(iscal, es_.iscal, sizeof(iscal), cudaMemcpyDeviceToHost);
  cudaMemcpy(&err, st_.err, sizeof(err), cudaMemcpyDeviceToHost);
  int64_t v[11] = {(int64_t)n_inserted_,
                   (int64_t)ins_head_,
                   (int64_t)emb_new_head_,
                   emb_cursor_ == SIZE_MAX ? -1 : (int64_t)emb_cursor_,
                   (int64_t)sweeps_,
                   iscal[0],
                   iscal[1],
                   iscal[2],
                   iscal[3],
                   (int64_t)upd_q_.size(),
                   (int64_t)err};
  for (int i = 0; i < cnt && i < 11; ++i) out[i] = v[i];
}

}  // namespace gm
