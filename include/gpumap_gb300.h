/*
 * gpumap_gb300 -- C ABI of the GB300 progressive UMAP engine.
 *
 * Drop-in boundary for the reference's pybind11 module gpumap._core, whose
 * C++ surface is gpumap::GPUMAP (cpp/include/gpumap/gpumap.cuh:15-96) bound in
 * cpp/bindings/binding.cu:45-115.  Plain pointers and sizes only; no C++
 * exception crosses this boundary.  Every function returns 0 on success or a
 * negative GM_ERR_* code; gm_last_error() gives the calling thread's message.
 *
 * Threading: one session is single-threaded (calls on the same session must
 * not overlap); different sessions may be driven from different threads.
 */
#ifndef GPUMAP_GB300_H
#define GPUMAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GM_OK 0
#define GM_ERR_INVALID (-1)  /* bad argument or parameter (Python ValueError) */
#define GM_ERR_RUNTIME (-2)  /* bad input data / state (Python RuntimeError) */
#define GM_ERR_CAPACITY (-3) /* append beyond n_instances (Python RuntimeError) */
#define GM_ERR_OOM (-4)      /* device or pinned allocation failed (MemoryError) */
#define GM_ERR_CUDA (-5)     /* CUDA runtime error */
#define GM_ERR_DEVICE (-6)   /* a bounded device wait ran out; state unreliable */
#define GM_ERR_CLOSED (-7)   /* session already closed */

/* Metric (reference enum gpumap::Metric, gpumap.cuh:13). */
#define GM_METRIC_EUCLIDEAN 0
#define GM_METRIC_COSINE 1

/* View element types. */
#define GM_DTYPE_F32 0
#define GM_DTYPE_U32 1

/* Parameters (reference GPUMAPParams, gpumap.cuh:15-36). */
typedef struct gm_params {
  uint64_t n_neighbors;          /* k, 1..32 (default 15) */
  uint64_t n_components;         /* must be 2 (default 2) */
  float min_dist;                /* default 0.1; used by the caller's a,b fit */
  uint64_t negative_sample_rate; /* default 5 */
  uint64_t max_epoch;            /* SGD epochs per embedding call (default 200) */
  float a, b;                    /* curve parameters (default 1, 1) */
  float alpha;                   /* initial learning rate (default 1) */
  int32_t verbose;               /* log phase progress to stderr */
  int32_t metric;                /* GM_METRIC_* */
  uint64_t n_instances;          /* capacity in rows */
  uint64_t n_features;           /* columns per row */
  int32_t precision;             /* 0 = the reference's NN-Descent insertion, FP32 (default);
                                    1 = exact insertion: BF16 tensor-core distance tiles against
                                        every inserted row, FP32 re-score of the survivors */
  int32_t device;                /* CUDA device ordinal, -1 = current */
  int32_t overlap;               /* 0 = phases run one after another, as the reference (default);
                                    1 = a cycle's embedding runs on a second stream while the next
                                        cycle's distance work proceeds: gm_run returns once the
                                        embedding is queued (embedding_time is then the time to
                                        queue it), gm_get_embedding waits for it */
} gm_params;

/* Result of one cycle (reference GPUMAPResult, gpumap.cuh:38-56). */
typedef struct gm_result {
  uint32_t n_insertion_ops, n_update_ops, n_embedding_ops;
  float insertion_time, update_time, embedding_time; /* seconds */
  uint8_t insertion_completed, update_completed, embedding_completed;
  uint64_t n_inserted_instances;
  uint64_t n_update_changed_edges;
  uint64_t embedding_pending_edges;
  uint64_t insertion_queue_size;
  uint64_t update_queue_size;
  uint64_t embedding_queue_size;
} gm_result;

/* Borrowed device view, valid until gm_destroy (row-major). */
typedef struct gm_view {
  void *ptr;
  uint64_t rows, cols, row_stride_bytes;
  int32_t dtype; /* GM_DTYPE_* */
} gm_view;

/* Kernel statistics (filled when gm_set_stats(s, 1) is on). Times come from
 * CUDA events recorded on the session's stream around each launch. */
typedef struct gm_stats {
  uint64_t kernel_launches;   /* kernels launched by the engine */
  uint64_t join_launches;     /* local-join kernel launches */
  double join_ms;             /* summed local-join kernel time */
  uint64_t join_nodes;        /* nodes joined */
  uint64_t join_rows;         /* feature rows loaded by the join (sum over nodes) */
  uint64_t join_pairs;        /* distance pairs formed by the join */
  uint64_t join_merges;       /* locked list merges */
  uint64_t cand_launches;     /* insertion candidate-distance launches */
  double cand_ms;
  uint64_t cand_rows;         /* candidate feature rows loaded */
  uint64_t sgd_launches;
  double sgd_ms;
  uint64_t sgd_edges;         /* edge samples processed by the SGD epochs */
  uint64_t sgd_negatives;     /* negative samples drawn */
  uint64_t exact_launches;    /* tensor-core distance launches (precision 1) */
  double exact_ms;            /* their summed time */
  double exact_flops;         /* 6 x rows x columns x padded features (split BF16), summed */
  double screen_ms;           /* bound + FP32 re-score + top-32 kernels */
  uint64_t exact_pairs;       /* batch x column pairs formed on the tensor cores */
  uint64_t exact_rescored;    /* pairs re-scored in FP32 */
  double phase_s[3];          /* insertion / update / embedding seconds */
  uint64_t exact_overflow_blocks; /* insertion blocks whose stored candidates overflowed, so
                                     that the candidate pass over the tiles ran again */
} gm_stats;

/* Replaces GPUMAPParams() defaults (gpumap.cuh:15-30). */
int gm_params_default(gm_params *out);

/* Replaces GPUMAP::GPUMAP(params) (gpumap.cuh:73; impl.cuh:57-68). Allocates
 * all session state for n_instances rows on the device. */
int gm_create(const gm_params *params, struct gm_session **out);

/* Replaces GPUMAP::initialize (impl.cu:12-15): a no-op kept for parity. */
int gm_initialize(struct gm_session *s, uint64_t n_instances, uint64_t n_features);

/* Replaces GPUMAP::append_data (impl.cuh:77-101): copies n_rows x n_cols
 * row-major float32 HOST rows into the session and queues them. */
int gm_append(struct gm_session *s, const float *host_rows, uint64_t n_rows,
              uint64_t n_cols);

/* Same as gm_append for rows already in device memory. */
int gm_append_device(struct gm_session *s, const float *device_rows, uint64_t n_rows,
                     uint64_t n_cols);

/* Replaces GPUMAP::run (impl.cuh:146-218): one insert/update/embed cycle. */
int gm_run(struct gm_session *s, uint32_t n_insertion_ops, uint32_t n_update_ops,
           uint32_t n_embedding_ops, gm_result *out);

/* Replace GPUMAP::get_embedding / get_neighbor_indices / get_neighbor_dists
 * (impl.cuh:509-533): full-capacity views; index/dist rows are k+1 wide and
 * index column k holds the row's dirty flag. */
int gm_get_embedding(const struct gm_session *s, gm_view *out);
int gm_get_neighbor_indices(const struct gm_session *s, gm_view *out);
int gm_get_neighbor_dists(const struct gm_session *s, gm_view *out);

/* The session's CUDA stream (cudaStream_t) for stream-aware consumers. */
int gm_get_stream(const struct gm_session *s, void **stream_out);

/* Makes `consumer_stream` (a cudaStream_t; NULL is the legacy default
 * stream) wait on the device for every piece of work the session has
 * queued so far, on all of its streams, without blocking the host: reads of
 * the result views issued on that stream afterwards see the finished
 * values.  No counterpart in the reference, whose views carry no stream
 * (cpp/bindings/utils/cai_wrapper.cuh:39-62); the DLPack export of the
 * Python views calls it with the consumer's stream. */
int gm_stream_wait(const struct gm_session *s, void *consumer_stream);

/* The CUDA device the session's memory lives on. */
int gm_get_device(const struct gm_session *s, int32_t *device_out);

/* Replaces GPUMAP::close (impl.cuh:502-507). */
int gm_close(struct gm_session *s);

/* Frees the session (reference destructor). NULL is ignored. */
void gm_destroy(struct gm_session *s);

/* Thread-local message of the last failing call on this thread. */
const char *gm_last_error(void);

/* Kernel statistics. */
int gm_set_stats(struct gm_session *s, int enable);
int gm_get_stats(struct gm_session *s, gm_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* GPUMAP_GB300_H */
