/* gpumap_gb300 serving ABI: many progressive sessions on one GPU, driven by
 * insertion requests.
 *
 * No counterpart in the reference, which runs one session per process and
 * one cycle at a time (python/gpumap/gpumap.py:88-146 over
 * cpp/src/impl.cuh:146-218).  Here a server owns several sessions (each the
 * engine of include/gpumap_gb300.h, with its graph, lists and embedding
 * resident in device memory) and a request queue:
 *
 *  - a request appends rows to one session and runs one cycle on it
 *    (gm_run: insertion of those rows, update, embedding);
 *  - `slots` worker threads take requests in arrival order, one request per
 *    session at a time (a session's cycles stay in order), so the cycles of
 *    different sessions run concurrently on the GPU, each on its session's
 *    own streams; a request that arrives while the slots are busy starts as
 *    soon as one frees (continuous batching);
 *  - device memory is admitted against a byte budget: opening a session
 *    charges its footprint (GM_ERR_CAPACITY if the budget or the free device
 *    memory would be exceeded), and a request whose run could grow its
 *    session's scratch waits until the budget has room;
 *  - every request records its arrival, start and finish times, so the
 *    caller can form latency percentiles.
 *
 * Results of a session do not depend on what else runs: its k-NN lists are
 * the same alone and in any mix; its embedding differs only by the
 * order-dependent rounding of concurrent SGD updates, as between two runs
 * alone. */
#ifndef GPUMAP_GB300_SERVER_H
#define GPUMAP_GB300_SERVER_H

#include <stdint.h>

#include "gpumap_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gm_server gm_server;

typedef struct gm_server_params {
  int32_t device;         /* CUDA device of every session */
  int32_t slots;          /* requests running at once (worker threads), >= 1 */
  uint64_t hbm_budget;    /* device bytes all sessions may hold together */
} gm_server_params;

/* One finished (or failed) request. */
typedef struct gm_request_info {
  uint64_t request;       /* id from gm_server_submit */
  uint32_t session;
  int32_t status;         /* GM_OK or the run's error code */
  uint64_t rows;          /* rows appended */
  double t_arrive;        /* seconds on the server's steady clock */
  double t_start;         /* a slot took it */
  double t_end;           /* its cycle's device work finished */
  gm_result result;       /* the cycle's result (valid when status == GM_OK) */
} gm_request_info;

/* Server statistics over the requests finished so far. */
typedef struct gm_server_stats {
  uint64_t finished, failed, rows;
  uint64_t sessions_open;
  uint64_t bytes_in_use;  /* charged to open sessions */
  double first_arrive, last_end;
  double latency_p50, latency_p99, latency_max;  /* t_end - t_arrive, seconds */
  double service_p50, service_p99;               /* t_end - t_start */
} gm_server_stats;

int gm_server_create(const gm_server_params *p, gm_server **out);
/* Waits for every queued request, then stops the workers and frees every
 * session. */
void gm_server_destroy(gm_server *srv);

/* Opens a session (same parameters as gm_create; device is the server's)
 * and charges its footprint to the budget. */
int gm_server_open_session(gm_server *srv, const gm_params *p, uint32_t *session_out);
/* Closes a session once its queued requests have finished. */
int gm_server_close_session(gm_server *srv, uint32_t session);

/* Queues a request: `rows` host rows (n_cols == n_features, copied before
 * the call returns) appended to `session`, then one cycle
 * gm_run(rows, n_update_ops, n_embedding_ops).  GM_ERR_CAPACITY when the
 * session cannot take the rows. */
int gm_server_submit(gm_server *srv, uint32_t session, const float *host_rows, uint64_t rows,
                     uint64_t n_cols, uint32_t n_update_ops, uint32_t n_embedding_ops,
                     uint64_t *request_out);
/* Blocks until the request has finished; fills `out`. */
int gm_server_wait(gm_server *srv, uint64_t request, gm_request_info *out);
/* Blocks until every queued request has finished. */
int gm_server_drain(gm_server *srv);

/* The session's engine handle, for result views (gm_get_embedding, ...)
 * and debug copies; valid until the session is closed.  Read it only while
 * none of its requests is queued or running. */
int gm_server_session_handle(gm_server *srv, uint32_t session, gm_session **out);

int gm_server_get_stats(gm_server *srv, gm_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* GPUMAP_GB300_SERVER_H */
