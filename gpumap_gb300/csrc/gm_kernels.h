// Host-side launchers for the engine's CUDA kernels.  Every launcher is
// asynchronous on the given stream; sizes and pointers are plain.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace gm {

// Resident session state in HBM (all device pointers, capacity n_cap rows).
struct DevState {
  int n_cap = 0;  // n_instances
  int d = 0;      // n_features
  int ld = 0;     // row stride of X in floats (d rounded up to 4)
  int k = 0;      // n_neighbors
  int cosine = 0;
  float *X = nullptr;         // n_cap x ld, zero padded
  float *norms = nullptr;     // n_cap squared L2 norms
  float *snorms = nullptr;    // n_cap sqrt of norms rounded up (exact-mode bounds)
  unsigned long long *g_key = nullptr;  // n_cap x 32 working lists, (dist bits << 32 | id)
  int *locks = nullptr;       // n_cap per-node locks (0 = free)
  int *dirty = nullptr;       // n_cap device dirty flags (0/1/2)
  int *knn_ids = nullptr;     // n_cap x k authoritative list, old flag = sign
  float *knn_dists = nullptr; // n_cap x k
  uint32_t *pub_idx = nullptr; // n_cap x (k+1) published ids, col k = dirty
  float *pub_dist = nullptr;   // n_cap x (k+1) published distances
  float *emb = nullptr;        // n_cap x 2
  uint32_t *bloom = nullptr;   // n_cap x 64 words (4 sets x 512 bits)
  unsigned *err = nullptr;     // device error bits
  unsigned long long *stat = nullptr; // device counters for statistics (16)
};

// Update-phase scratch (capacity n_cap rows).
struct UpdScratch {
  int *fwd_new = nullptr;  // n_cap x 32
  int *fwd_old = nullptr;  // n_cap x 32
  int *rev_new = nullptr;  // n_cap x 32
  int *rev_old = nullptr;  // n_cap x 32
  int4 *sizes = nullptr;   // n_cap: (fwd new, rev new, fwd old, rev old)
  int *cnt = nullptr;      // n_cap reverse in-degree
  int *off = nullptr;      // n_cap + 1 exclusive offsets
  int *fill = nullptr;     // n_cap
  int *csr = nullptr;      // n_cap x 32 reverse sources
  int *hflag = nullptr;    // n_cap per-row host-side dirty state
  int *rowtmp = nullptr;   // n_cap row list scratch
  int *rowtmp2 = nullptr;  // n_cap row list scratch
  int *counters = nullptr; // small device counters
};

// ---- utilities (gm_kernels_util.cu) ----
// Count of kernels launched by this library (all sessions and operators).
void note_launch(int n = 1);
uint64_t launch_counter();
// Fills n 32-bit (64-bit) words at p with v.
void fill_u32(void *p, uint32_t v, size_t n, cudaStream_t s);
void fill_u64(void *p, unsigned long long v, size_t n, cudaStream_t s);
void launch_counter_reset();
// Exclusive scan of in[0..n) into out[0..n]; out[n] = total.  tmp needs
// scan_tmp_ints(n) ints.
size_t scan_tmp_ints(int n);
void exclusive_scan(const int *in, int *out, int n, int *tmp, cudaStream_t s);
// Ordered compaction of the ids i in [0, n) with flag[i] != 0 (or, when
// select >= 0, flag[i] == select) into out; *count receives the number.
size_t compact_tmp_ints(int n);
// As compact_flags, with the length read from device memory (bounded by n_max).
void compact_flags_dev(const int *flag, const int *n_dev, int n_max, int *out,
                       int *count, int *tmp, cudaStream_t s);
void compact_flags(const int *flag, int n, int select, int *out, int *count,
                   int *tmp, cudaStream_t s);
// Ordered compaction of list[i] (i < *n_dev) where pred[list[i]] != 0.
void compact_list(const int *list, const int *n_dev, int n_max, const int *pred,
                  int *out, int *count, int *tmp, cudaStream_t s);

// ---- insertion (gm_kernels_insert.cu) ----
void launch_row_norms(const DevState &st, int row0, int nrows, cudaStream_t s);
void launch_random_init(const DevState &st, int row0, int nrows, int n,
                        int window_start, uint64_t seed, cudaStream_t s);
void launch_sample_candidates(const DevState &st, int row0, int nrows, int n,
                              int *cand, int *cand_cnt, cudaStream_t s);
void launch_candidate_dists(const DevState &st, int row0, int nrows,
                            const int *cand, const int *cand_cnt,
                            float *cand_dist, cudaStream_t s);
void launch_forward_merge(const DevState &st, int row0, int nrows,
                          const int *cand, const int *cand_cnt,
                          const float *cand_dist, cudaStream_t s);
void launch_reverse_insert(const DevState &st, int row0, int nrows,
                           const int *cand, const int *cand_cnt,
                           const float *cand_dist, cudaStream_t s);
// Copies the first k working entries of rows [row0,row0+nrows) and of the
// listed rows into the authoritative list and publishes them.
void launch_adopt_and_publish(const DevState &st, int row0, int nrows,
                              const int *rows, const int *n_rows_dev, int n_rows_max,
                              int n, cudaStream_t s);
void launch_embed_init(const DevState &st, int row0, int nrows, int n,
                       cudaStream_t s);

// ---- exact insertion on tensor cores (gm_exact.cu) ----
// Two TMA descriptors over the BF16 shadow rows (boxes of 128 and 256 rows).
struct ExactMaps {
  alignas(64) unsigned char a[128];
  alignas(64) unsigned char b[128];
};
int exact_dh(int d);  // shadow row width: d rounded up to 64
bool make_row_maps(void *xh, int n_cap, int dh, ExactMaps *out);
void launch_to_bf16(const DevState &st, void *xh, int dh, int row0, int nrows, cudaStream_t s);
// Screen scratch of one block of batch rows (rows x n_cap where noted).
struct ExactScreen {
  float *D = nullptr;         // rows x ldD approximate distances (written only when kept)
  int *cand = nullptr;        // rows x ldD candidate columns per batch row
  float *cand_d = nullptr;    // rows x ldD: their approximate, then canonical distances
  int *row_cnt = nullptr;     // rows candidate counts
  float *heaps = nullptr;     // rows x CTAs x 32: per-CTA smallest upper bounds (pass 1)
  float *row_t = nullptr;     // rows exact thresholds
  float *seed = nullptr;      // rows thresholds from the seed pass
  float *mins = nullptr;       // rows x mins_ld chunk minima of the seed pass
  int mins_ld = 0;
  // stored columns of the store pass: per row pre_gx x pre_cap packed (lower
  // bound, column) entries and their upper bounds, split into one segment
  // per CTA of the row's tile (pre_gx x pre_cap / CTAs entries each, or
  // pre_cap when pre_fixed), the segments' lengths, and an overflow flag
  unsigned long long *pre = nullptr;
  float *pre_ub = nullptr;
  int *pre_cnt = nullptr;
  int pre_cap = 0, pre_gx = 0;
  bool pre_fixed = false;
  int *pre_over = nullptr;
  int *pool_j = nullptr, *pool_m = nullptr;    // column pairs as found
  int *pool_j2 = nullptr, *pool_m2 = nullptr;  // grouped by existing row
  float *pool_d = nullptr;    // their canonical distances
  int *pcnt = nullptr;        // n_cap + 1 pairs per existing row, then fill cursors
  int *poff = nullptr;        // n_cap + 1 group offsets
  int *tmp = nullptr;         // scan scratch, scan_tmp_ints(n_cap)
  int *counter = nullptr;     // pairs in the pool
  long pool_cap = 0;
};
// Distances of batch rows [row0+blk0, +nrows) against rows [0, n) on the
// tensor cores, screened as the accumulators drain, in two passes (the
// per-row exact threshold, then the candidates): candidate columns per batch
// row and (existing row, batch row) pairs land in x.  With keep_d the
// approximate tile is also written to x.D (nrows x ldD), for tests.
// Column tiles the seed pass samples out of n_tiles.
int exact_seed_tiles(int n_tiles);
void launch_exact_dist(const DevState &st, const ExactMaps &maps, int dh, int row0, int blk0,
                       int nrows, int n, const ExactScreen &x, long ldD, bool keep_d, int sms,
                       cudaStream_t s);
// Exact lists of those rows (threshold, FP32 re-score, top-32) and their
// offers to rows [0, row0).
void launch_exact_screen(const DevState &st, int row0, int blk0, int nrows, int n,
                         const ExactScreen &x, long ldD, int sms, cudaStream_t s);

// ---- update (gm_kernels_update.cu) ----
void launch_sample_graph(const DevState &st, const UpdScratch &u,
                         const int *batch, int nb, int n, cudaStream_t s);
// Builds rev[j] from fwd lists of the batch rows, keeping the 32 smallest
// source ids per target.  which = 0 new, 1 old.
void build_reverse(const DevState &st, const UpdScratch &u, const int *batch,
                   int nb, int n, int which, int *tmp, cudaStream_t s);
void launch_local_join(const DevState &st, const UpdScratch &u,
                       const int *join_nodes, const int *n_join_dev, int n_join_max,
                       int n, cudaStream_t s);
// Merges working lists into the authoritative lists for dirty rows,
// re-sorts them, publishes changed rows and flags rows to report.
void launch_join_flags(const UpdScratch &u, int n, int *flag, cudaStream_t s);
void launch_merge_publish(const DevState &st, const UpdScratch &u,
                          const int *rows, const int *n_rows_dev, int n_rows_max,
                          int n, int *edge_counter, int *report_flag,
                          cudaStream_t s);

// ---- embedding (gm_kernels_embed.cu) ----
struct EmbedScratch {
  int *batch = nullptr;     // batch ids
  int *unsel = nullptr;     // unselected ids
  int *flag = nullptr;      // n_cap scratch flags
  float *sigma = nullptr;   // n_cap
  float *rho = nullptr;     // n_cap
  int *coo_row = nullptr;   // 2*B*k
  int *coo_col = nullptr;
  float *coo_val = nullptr;
  int *t_row = nullptr;     // trimmed copies
  int *t_col = nullptr;
  int *flag_tail = nullptr; // trimmed tails
  float *t_val = nullptr;   // epochs_per_sample after scheduling
  float *next_s = nullptr;
  float *next_n = nullptr;
  int *deg = nullptr;       // n_cap
  float *snap = nullptr;    // n_cap x 2
  float *fscal = nullptr;   // float scalars (see gm_kernels_embed.cu)
  int *iscal = nullptr;     // int scalars
  float *partial = nullptr; // reduction partials
  int *ipartial = nullptr;
  int *tmp = nullptr;       // scan / compaction scratch (n_cap items)
  int *tmp2 = nullptr;      // scan / compaction scratch (cap_coo items)
  // overlap mode: the published table as the phase's fuzzy set saw it, for
  // its reposition step (the next cycle may publish meanwhile)
  uint32_t *pub_idx_snap = nullptr;
  float *pub_dist_snap = nullptr;
  size_t cap_coo = 0;
  size_t cap_partial = 0;
};

// Embed-time fuzzy simplicial set from the published k-NN (self prepended).
void launch_fuzzy_graph(const uint32_t *pub_idx, const float *pub_dist, int n,
                        int k, int euclidean, const int *batch, int nb,
                        double log2_target, EmbedScratch &e, cudaStream_t s);
// Edge scheduling + SGD epochs on the COO in e (nnz in e.iscal[0]).
void launch_optimize_layout(float *emb, int n, int nb, int k, float alpha0,
                            float gamma, float a, float b, int n_epochs,
                            int neg_rate, uint64_t seed, EmbedScratch &e,
                            cudaStream_t s);
// Edge scheduling only: max weight, trim, epochs_per_sample, degrees,
// rounding factor (results in e.t_row/e.flag_tail/e.t_val, e.iscal, e.fscal).
void launch_schedule(int n, int nb, int k, float alpha0, int n_epochs, int neg_rate,
                     EmbedScratch &e, cudaStream_t s);
void launch_mark_rows(const int *rows, int nr, int *flag, cudaStream_t s);
// SGD epochs on scheduled edges; next_s/next_n initialised; nnz in
// iscal[2], rows n in iscal[4], rounding factor in fscal[2].  grid blocks of
// 256 threads stride over the edges, so a fixed grid can be captured once.
void launch_sgd(float *emb, const int *head, const int *tail, const float *eps,
                float *next_s, float *next_n, const int *iscal, const float *fscal,
                int grid, float alpha0, float gamma, float a, float b, int n_epochs,
                int neg_rate, uint64_t seed, cudaStream_t s,
                unsigned long long *stat = nullptr);
// All n_epochs epochs in one cooperative launch (one CTA of 512 threads per
// SM, at most max_ctas CTAs when max_ctas > 0) with a bounded grid barrier
// between epochs; bar: 1 device word,
// cleared here; a barrier timeout sets kDevErrSpin in *err.  Edges run in
// the schedule's order, one per thread slot.
cudaError_t launch_sgd_persistent(float *emb, const int *head, const int *tail,
                                  const float *eps, float *next_s, float *next_n,
                                  const int *iscal, const float *fscal, float alpha0,
                                  float gamma, float a, float b, int n_epochs, int neg_rate,
                                  uint64_t seed, unsigned *bar, unsigned *err, int device,
                                  cudaStream_t s, unsigned long long *stat = nullptr,
                                  int max_ctas = 0);
// One embedding call's SGD (all epochs): launch_sgd_persistent.
cudaError_t launch_sgd_call(float *emb, const int *head, const int *tail, const float *eps,
                            float *next_s, float *next_n, const int *iscal, const float *fscal,
                            float alpha0, float gamma, float a, float b, int n_epochs, int neg_rate,
                            uint64_t seed, unsigned *bar, unsigned *err, int device,
                            cudaStream_t s, unsigned long long *stat = nullptr, int max_ctas = 0);
void launch_set_int(int *p, int v, cudaStream_t s);
constexpr int kIscalN = 4;
constexpr int kIscalBarrier = 8;  // iscal[8..9]: SGD grid-barrier words
void launch_epoch_init(const float *eps, int nnz, int neg_rate, float *next_s,
                       float *next_n, cudaStream_t s);
void launch_add_noise(float *emb, int n, const int *batch, int nb,
                      float noise_scale, uint64_t seed, EmbedScratch &e,
                      cudaStream_t s);
void launch_heuristic(const uint32_t *pub_idx, const float *pub_dist, int n,
                      int k, int euclidean, const int *unsel, int nu,
                      float *emb, EmbedScratch &e, cudaStream_t s);

}  // namespace gm
