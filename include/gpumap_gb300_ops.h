/*
 * gpumap_gb300 -- stage-level C ABI: internal-state copies and stateless
 * stage operators on caller-owned device buffers.  Used by the parity tests
 * to compare each stage with the CPU oracle on identical inputs.
 *
 * The reference exposes no such entry points; each operator below names the
 * reference function whose computation it performs.
 */
#ifndef GPUMAP_GB300_OPS_H
#define GPUMAP_GB300_OPS_H

#include "gpumap_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Internal buffers of a session (device -> host copies). */
#define GM_BUF_GRAPH_IDS 0   /* n_instances x 32 int32 working lists (graph_buffer_, buffers.cuh:416) */
#define GM_BUF_GRAPH_DISTS 1 /* n_instances x 32 float (dists_buffer_, buffers.cuh:419) */
#define GM_BUF_KNN_IDS 2     /* n_instances x k int32, old flag = -id-1 (h_graph, buffers.cuh:463) */
#define GM_BUF_KNN_DISTS 3   /* n_instances x k float (h_dists, buffers.cuh:465) */
#define GM_BUF_NORMS 4       /* n_instances float squared norms (data column d, storage.cuh:116) */
#define GM_BUF_BLOOM 5       /* n_instances x 64 uint32 (BloomFilter bits, buffers.cuh:35-137) */
#define GM_BUF_SIGMA 6       /* n float, last embedding call */
#define GM_BUF_RHO 7         /* n float, last embedding call */
#define GM_BUF_COO_ROW 8     /* nnz int32 fuzzy-union COO of the last embedding call */
#define GM_BUF_COO_COL 9
#define GM_BUF_COO_VAL 10
#define GM_BUF_SCHED_ROW 11  /* nnz2 int32 trimmed edges of the last embedding call */
#define GM_BUF_SCHED_COL 12
#define GM_BUF_SCHED_EPS 13  /* nnz2 float epochs_per_sample */
#define GM_BUF_X 14          /* n_instances x ld float feature rows (ld = n_features rounded up to 4) */
#define GM_BUF_PUB_IDX 15    /* n_instances x (k+1) uint32 published indices (neighbor_indices) */
#define GM_BUF_PUB_DIST 16   /* n_instances x (k+1) float published distances (neighbor_dists) */
#define GM_BUF_EMBEDDING 17  /* n_instances x 2 float embedding */
#define GM_BUF_EXACT_D 18    /* precision 1, while gm_debug_keep_tiles is on: approximate distances of the last insertion block,
                                block rows x (rows inserted so far), row-major */

/* Size in bytes of internal buffer `which`. */
int gm_debug_buffer_size(const struct gm_session *s, int which, uint64_t *bytes);
/* Copies `bytes` bytes of internal buffer `which` to host memory. */
int gm_debug_copy(const struct gm_session *s, int which, void *host, uint64_t bytes);
/* Precision 1: keep (on != 0) or stop keeping each insertion block's
 * approximate distance tile for GM_BUF_EXACT_D.  Off by default: the screen
 * runs as the tile leaves the tensor memory and the tile is not stored. */
int gm_debug_keep_tiles(struct gm_session *s, int on);
/* Precision 1: entries per segment of stored columns that the store pass
 * over the tiles may keep, fixed whatever the grid width (clamped to 64;
 * by default each of a row tile's CTAs gets an equal share of the row's
 * 64 x min(SMs, column tiles) entries; 0 runs the heap and candidate passes
 * instead, as for blocks of up to 32 column tiles).  A segment that would
 * exceed it makes the heap and candidate passes run for its block
 * (gm_stats.exact_overflow_blocks). */
int gm_debug_pre_capacity(struct gm_session *s, int cap);
/* Host and device scalars, out[0..n):
 *  0 n_inserted, 1 insertion-queue head, 2 new-row embedding-queue head,
 *  3 embedding cursor (-1 = none), 4 embedding sweeps, 5 last nnz,
 *  6 last extras, 7 last trimmed nnz, 8 last max degree, 9 update queue size,
 * 10 device error bits. */
int gm_debug_scalars(const struct gm_session *s, int64_t *out, int n);
/* Update-queue contents in FIFO order. */
int gm_debug_update_queue(const struct gm_session *s, uint32_t *out, uint64_t cap,
                          uint64_t *n_out);

/* Fuzzy simplicial set + edge scheduling on a published k-NN table
 * (reference compute_fuzzy_graph, embedding_kernel.cuh:650-716, and the
 * scheduling half of run_optimize_layout, :726-778).
 *   pub_idx/pub_dist: n x (k+1) device tables (column k ignored)
 *   batch: nb device int32 row ids
 *   coo_*: capacity 2*nb*k; t_*: capacity 2*nb*k; sigma/rho: n
 *   counts_out (host, 4): nnz, extras, trimmed nnz, max degree
 *   scalars_out (host, 3): mean distance, max weight, rounding factor */
int gm_op_fuzzy_schedule(const uint32_t *pub_idx, const float *pub_dist, int64_t n,
                         int32_t k, int32_t euclidean, const int32_t *batch, int64_t nb,
                         int32_t n_epochs, float alpha, int32_t *coo_row,
                         int32_t *coo_col, float *coo_val, int32_t *t_row, int32_t *t_col,
                         float *t_eps, float *sigma, float *rho, int64_t *counts_out,
                         float *scalars_out, void *stream);

/* SGD epochs on a scheduled edge list (reference optimize_batch_kernel loop,
 * embedding_kernel.cuh:509-589 and :780-797). emb: n x 2 device, updated,
 * 8-byte aligned (GM_ERR_INVALID otherwise). */
int gm_op_sgd(float *emb, int64_t n, const int32_t *head, const int32_t *tail,
              const float *eps, int64_t nnz, float rounding, float alpha0, float gamma,
              float a, float b, int32_t n_epochs, int32_t negative_sample_rate,
              uint64_t seed, void *stream);

/* Largest edge list gm_op_sgd_noalloc accepts. */
#define GM_SGD_NOALLOC_MAX_EDGES 1048576

/* gm_op_sgd without any device allocation, for callers that must not
 * allocate while they run: a host framework whose memory pool owns the GPU
 * (a cudaMalloc beside it can fail or fragment that pool) or a latency-bound
 * loop that cannot take cudaFree's device-wide synchronisation.  No
 * counterpart in the reference.  Same arguments as gm_op_sgd and the same
 * arithmetic per edge, but one kernel launch per epoch instead of
 * gm_op_sgd's single launch for all epochs: results equal gm_op_sgd's bit
 * for bit where no two edges of an epoch touch the same row (and for a single
 * edge, negative samples included); with Hogwild races they agree
 * statistically, as two runs of either operator do.
 *  - Scratch is one fixed device array of 8 MiB + 128 bytes inside this
 *    library, held by every GPU that loads it until the process exits;
 *    nnz above GM_SGD_NOALLOC_MAX_EDGES is rejected with GM_ERR_INVALID.
 *  - The first call on a device looks up the array's device address (with
 *    that device current); make that first call before any stream capture.
 *  - Every call shares the array and overwrites what it reads before use;
 *    calls that overlap on the GPU (different streams, or threads) race.
 *  - Returns once the work is queued on `stream`; kernel errors surface at
 *    the caller's next synchronisation of that stream. */
int gm_op_sgd_noalloc(float *emb, int64_t n, const int32_t *head, const int32_t *tail,
                      const float *eps, int64_t nnz, float rounding, float alpha0, float gamma,
                      float a, float b, int32_t n_epochs, int32_t negative_sample_rate,
                      uint64_t seed, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GPUMAP_GB300_OPS_H */
