// Session engine: the progressive UMAP cycle (insert -> update -> embed) on
// one GPU with all graph, queue-derived and embedding state resident in HBM.
// Host-side policy (queues, cursors, seeds, completion flags) follows the
// reference's GPUMAP::Impl (impl.cuh:29-533).
#pragma once

#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <deque>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "gm_kernels.h"
#include "../../include/gpumap_gb300.h"

namespace gm {

// Error carrying a C-ABI status code.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Deduplicating FIFO (reference UpdateQueue, queue.cuh:10-87): pushing an id
// already queued is a no-op.
class DedupQueue {
 public:
  void reset(size_t cap) {
    q_.clear();
    in_.assign(cap, 0);
  }
  size_t size() const { return q_.size(); }
  void push(uint32_t v) {
    if (v < in_.size() && !in_[v]) {
      in_[v] = 1;
      q_.push_back(v);
    }
  }
  std::vector<uint32_t> pop_n(size_t n) {
    const size_t m = std::min(n, q_.size());
    std::vector<uint32_t> out(q_.begin(), q_.begin() + (long)m);
    for (uint32_t v : out) in_[v] = 0;
    q_.erase(q_.begin(), q_.begin() + (long)m);
    return out;
  }
  const std::deque<uint32_t> &items() const { return q_; }

 private:
  std::deque<uint32_t> q_;
  std::vector<char> in_;
};

class Session {
 public:
  explicit Session(const gm_params &p);
  ~Session();
  Session(const Session &) = delete;
  Session &operator=(const Session &) = delete;

  void append(const float *rows, size_t n_rows, size_t n_cols, bool on_device);
  gm_result run(uint32_t n_ins, uint32_t n_upd, uint32_t n_emb);
  void close();

  const gm_params &params() const { return p_; }
  const DevState &state() const { return st_; }
  const EmbedScratch &embed_scratch() const { return es_; }
  size_t n_inserted() const { return n_inserted_; }
  cudaStream_t stream() const { return stream_; }
  int device() const { return device_; }
  void set_stats(bool on) { stats_on_ = on; }
  // device memory the session holds now, and what a run with these op
  // counts could add (its scratch grows on demand)
  size_t device_bytes() const;
  size_t growth_bytes(uint32_t n_ins, uint32_t n_emb) const;
  // keep each insertion block's approximate distance tile (tests)
  void set_keep_tile(bool on);
  void set_pre_cap(int cap);
  void drain();
  // consumer waits (on the device) for everything queued on this session
  void order_after(cudaStream_t consumer) const;
  void get_stats(gm_stats *out);
  void reset_stats();
  void debug_scalars(int64_t *out, int n) const;
  const DedupQueue &update_queue() const { return upd_q_; }
  const float *exact_scratch() const { return ex_D_; }
  uint64_t exact_scratch_bytes() const {
    return ex_D_ ? (uint64_t)ex_block_ * std::max<uint64_t>(p_.n_instances, 1) * 4 : 0;
  }

 private:
  uint32_t insert(uint32_t n_ops);
  uint32_t update(uint32_t n_ops, size_t &changed_edges);
  size_t update_round(std::vector<uint32_t> &batch, std::vector<uint32_t> &affected);
  uint32_t embed(uint32_t n_ops);
  void check_launch_error(const char *phase);
  void check_device_error(const char *phase);
  void ensure_cand(size_t rows);
  void ensure_embed(EmbedScratch &e, size_t nb);
  void free_embed(EmbedScratch &e);
  void sync_embed_streams();
  void flush_init();
  template <typename... A> void log(const char *fmt, A... a) const;
  void sync();
  void release_streams();
  void timed_begin(int slot, cudaStream_t s = nullptr);
  void timed_end(int slot, cudaStream_t s = nullptr);
  void collect_timings(bool block = true);
  void run_sgd(cudaStream_t s);

  gm_params p_;
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  // overlap mode: the embedding phase's stream, "table published" and
  // "embedding done" events, and whether an embedding is in flight.
  // Consecutive embedding phases alternate between two sides (stream,
  // scratch, pinned staging), so that a phase's fuzzy set and schedule are
  // built while the previous phase's SGD runs; "snapshot taken" marks the
  // point after which a phase no longer reads the published table.  The
  // insertion's embedding of its new rows runs at the start of the next
  // phase (after the previous SGD); the insertion after it waits for that
  // before it changes any working list.
  cudaStream_t estream_ = nullptr, estream_alt_ = nullptr;
  cudaEvent_t ev_pub_ = nullptr, ev_emb_ = nullptr, ev_snap_ = nullptr, ev_init_ = nullptr;
  cudaEvent_t ev_hpin_ = nullptr, ev_hpin_alt_ = nullptr;  // each side's batch upload
  bool emb_pending_ = false, snap_pending_ = false, init_wait_ = false;
  bool defer_init_ = false, init_pending_ = false;
  int init_row0_ = 0, init_nb_ = 0, init_n_ = 0;
  // ingest ring: host-to-device row transfers on their own stream, pageable
  // rows staged through two pinned slots
  static constexpr int kRingSlots = 2;
  struct RingSlot {
    void *buf = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
  };
  cudaStream_t cstream_ = nullptr;
  RingSlot ring_[kRingSlots];
  int ring_next_ = 0;
  DevState st_;
  UpdScratch us_;
  EmbedScratch es_, es_alt_;
  std::vector<void *> allocs_;
  size_t fixed_bytes_ = 0;

  // insertion candidates (grow on demand)
  int *cand_ = nullptr, *cand_cnt_ = nullptr;
  float *cand_dist_ = nullptr;
  size_t cand_rows_ = 0;

  // device row lists / counters
  int *d_rows_ = nullptr, *d_rows2_ = nullptr, *d_batch_ = nullptr;
  int *d_cnt_ = nullptr;  // [0] list count, [1] edges, [2] report count, [3] join count
  int *d_tmp_ = nullptr;
  uint32_t *h_pin_ = nullptr;      // pinned staging (n_cap + 16 words)
  uint32_t *h_emb_pin_ = nullptr;  // the embedding phase's pinned staging
  int *es_cnt_ = nullptr;          // the embedding phase's compaction counter
  uint32_t *h_emb_pin_alt_ = nullptr;  // the other side's (overlap mode)
  int *es_cnt_alt_ = nullptr;

  size_t n_inserted_ = 0;
  size_t ins_head_ = 0;      // insertion queue = [ins_head_, n_inserted_)
  size_t emb_new_head_ = 0;  // new-row embedding queue = [emb_new_head_, n_inserted_)
  DedupQueue upd_q_;
  size_t emb_cursor_ = SIZE_MAX;
  size_t sweeps_ = 0;
  std::deque<uint32_t> batch_hist_;
  std::mt19937 rng_{42};
  bool bloom_clean_ = true;
  bool ins_done_ = false, upd_done_ = false, emb_done_ = false;
  bool closed_ = false;

  // statistics
  bool stats_on_ = false;
  bool keep_tile_ = false;
  int pre_cap_alloc_ = 0;  // pre-candidate segment length allocated (precision 1)
  gm_stats stats_{};
  struct EvPair { cudaEvent_t a, b; int slot; };
  std::vector<EvPair> ev_pending_;
  std::vector<cudaEvent_t> ev_pool_;
  unsigned long long *d_stat_ = nullptr;

  // exact insertion (precision 1): BF16 shadow rows, TMA maps, block scratch
  void *xh_ = nullptr;
  int dh_ = 0;
  ExactMaps maps_{};
  float *ex_D_ = nullptr;
  int *ex_cand_ = nullptr;
  int ex_block_ = 0;
  ExactScreen xs_{};
  int sms_ = 0;
};

}  // namespace gm

// The C ABI's opaque session handle (include/gpumap_gb300.h).
struct gm_session {
  gm::Session *impl;
};
