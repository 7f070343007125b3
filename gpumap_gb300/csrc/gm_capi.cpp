// extern "C" boundary: status codes in, no exceptions out.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "gm_engine.h"
#include "../../include/gpumap_gb300.h"
#include "../../include/gpumap_gb300_ops.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

template <typename F>
int guarded(F &&f) {
  try {
    f();
    g_last_error.clear();
    return GM_OK;
  } catch (const gm::Error &e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc &) {
    return fail(GM_ERR_OOM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(GM_ERR_RUNTIME, e.what());
  } catch (...) {
    return fail(GM_ERR_RUNTIME, "unknown error");
  }
}

int ck(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return GM_OK;
  cudaGetLastError();
  return fail(e == cudaErrorMemoryAllocation ? GM_ERR_OOM : GM_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

namespace gm {
// Records `msg` as the calling thread's gm_last_error() (cleared for GM_OK)
// and returns `code`; for entry points defined outside this file.
int set_last_error(int code, const char *msg) {
  if (code == GM_OK) {
    g_last_error.clear();
    return GM_OK;
  }
  return fail(code, msg);
}
}  // namespace gm

extern "C" {

int gm_params_default(gm_params *out) {
  if (!out) return fail(GM_ERR_INVALID, "null params");
  std::memset(out, 0, sizeof(*out));
  out->n_neighbors = 15;
  out->n_components = 2;
  out->min_dist = 0.1f;
  out->negative_sample_rate = 5;
  out->max_epoch = 200;
  out->a = 1.0f;
  out->b = 1.0f;
  out->alpha = 1.0f;
  out->verbose = 0;
  out->metric = GM_METRIC_EUCLIDEAN;
  out->n_instances = 0;
  out->n_features = 0;
  out->precision = 0;
  out->overlap = 0;
  out->device = -1;
  return GM_OK;
}

int gm_create(const gm_params *params, gm_session **out) {
  if (!params || !out) return fail(GM_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] {
    auto *s = new gm_session{nullptr};
    try {
      s->impl = new gm::Session(*params);
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
  });
}

int gm_initialize(gm_session *s, uint64_t, uint64_t) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  return GM_OK;
}

int gm_append(gm_session *s, const float *host_rows, uint64_t n_rows, uint64_t n_cols) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  return guarded([&] { s->impl->append(host_rows, n_rows, n_cols, false); });
}

int gm_append_device(gm_session *s, const float *device_rows, uint64_t n_rows,
                     uint64_t n_cols) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  return guarded([&] { s->impl->append(device_rows, n_rows, n_cols, true); });
}

int gm_run(gm_session *s, uint32_t ni, uint32_t nu, uint32_t ne, gm_result *out) {
  if (!s || !out) return fail(GM_ERR_INVALID, "null argument");
  return guarded([&] { *out = s->impl->run(ni, nu, ne); });
}

int gm_get_embedding(const gm_session *s, gm_view *out) {
  if (!s || !out) return fail(GM_ERR_INVALID, "null argument");
  // an overlapped embedding may still be running: the view is complete
  // once it has finished
  const int rc = guarded([&] { s->impl->drain(); });
  if (rc != GM_OK) return rc;
  const auto &st = s->impl->state();
  out->ptr = st.emb;
  out->rows = s->impl->params().n_instances;
  out->cols = 2;
  out->row_stride_bytes = 2 * sizeof(float);
  out->dtype = GM_DTYPE_F32;
  return GM_OK;
}

int gm_get_neighbor_indices(const gm_session *s, gm_view *out) {
  if (!s || !out) return fail(GM_ERR_INVALID, "null argument");
  const auto &st = s->impl->state();
  out->ptr = st.pub_idx;
  out->rows = s->impl->params().n_instances;
  out->cols = (uint64_t)st.k + 1;
  out->row_stride_bytes = out->cols * sizeof(uint32_t);
  out->dtype = GM_DTYPE_U32;
  return GM_OK;
}

int gm_get_neighbor_dists(const gm_session *s, gm_view *out) {
  if (!s || !out) return fail(GM_ERR_INVALID, "null argument");
  const auto &st = s->impl->state();
  out->ptr = st.pub_dist;
  out->rows = s->impl->params().n_instances;
  out->cols = (uint64_t)st.k + 1;
  out->row_stride_bytes = out->cols * sizeof(float);
  out->dtype = GM_DTYPE_F32;
  return GM_OK;
}

int gm_get_stream(const gm_session *s, void **stream_out) {
  if (!s || !stream_out) return fail(GM_ERR_INVALID, "null argument");
  *stream_out = (void *)s->impl->stream();
  return GM_OK;
}

int gm_stream_wait(const gm_session *s, void *consumer_stream) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  return guarded([&] { s->impl->order_after((cudaStream_t)consumer_stream); });
}

int gm_get_device(const gm_session *s, int32_t *device_out) {
  if (!s || !device_out) return fail(GM_ERR_INVALID, "null argument");
  *device_out = s->impl->device();
  return GM_OK;
}

int gm_close(gm_session *s) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  return guarded([&] { s->impl->close(); });
}

void gm_destroy(gm_session *s) {
  if (!s) return;
  delete s->impl;
  delete s;
}

const char *gm_last_error(void) { return g_last_error.c_str(); }

int gm_set_stats(gm_session *s, int enable) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  return guarded([&] {
    s->impl->reset_stats();
    s->impl->set_stats(enable != 0);
  });
}

int gm_get_stats(gm_session *s, gm_stats *out) {
  if (!s || !out) return fail(GM_ERR_INVALID, "null argument");
  return guarded([&] { s->impl->get_stats(out); });
}

// ---------------------------------------------------------------------------
// stage-level entry points
// ---------------------------------------------------------------------------
int gm_debug_buffer_size(const gm_session *s, int which, uint64_t *bytes) {
  if (!s || !bytes) return fail(GM_ERR_INVALID, "null argument");
  const auto &st = s->impl->state();
  const uint64_t N = s->impl->params().n_instances, k = (uint64_t)st.k;
  int64_t sc[11];
  s->impl->debug_scalars(sc, 11);
  const uint64_t n = (uint64_t)sc[0], nnz = (uint64_t)sc[5], nnz2 = (uint64_t)sc[7];
  switch (which) {
    case GM_BUF_GRAPH_IDS: case GM_BUF_GRAPH_DISTS: *bytes = N * 32 * 4; break;
    case GM_BUF_KNN_IDS: case GM_BUF_KNN_DISTS: *bytes = N * k * 4; break;
    case GM_BUF_NORMS: *bytes = N * 4; break;
    case GM_BUF_BLOOM: *bytes = N * 64 * 4; break;
    case GM_BUF_SIGMA: case GM_BUF_RHO: *bytes = n * 4; break;
    case GM_BUF_COO_ROW: case GM_BUF_COO_COL: case GM_BUF_COO_VAL: *bytes = nnz * 4; break;
    case GM_BUF_SCHED_ROW: case GM_BUF_SCHED_COL: case GM_BUF_SCHED_EPS: *bytes = nnz2 * 4; break;
    case GM_BUF_X: *bytes = N * (uint64_t)st.ld * 4; break;
    case GM_BUF_PUB_IDX: case GM_BUF_PUB_DIST: *bytes = N * (k + 1) * 4; break;
    case GM_BUF_EMBEDDING: *bytes = N * 2 * 4; break;
    case GM_BUF_EXACT_D: *bytes = s->impl->exact_scratch_bytes(); break;
    default: return fail(GM_ERR_INVALID, "unknown buffer");
  }
  return GM_OK;
}

int gm_debug_copy(const gm_session *s, int which, void *host, uint64_t bytes) {
  if (!s || (!host && bytes)) return fail(GM_ERR_INVALID, "null argument");
  uint64_t cap = 0;
  int rc = gm_debug_buffer_size(s, which, &cap);
  if (rc) return rc;
  if (bytes > cap) return fail(GM_ERR_INVALID, "copy larger than buffer");
  rc = guarded([&] { s->impl->drain(); });
  if (rc != GM_OK) return rc;
  const auto &st = s->impl->state();
  const auto &es = s->impl->embed_scratch();
  const void *src = nullptr;
  switch (which) {
    case GM_BUF_GRAPH_IDS:
    case GM_BUF_GRAPH_DISTS: {
      // working lists are stored as packed (dist, id) keys; unpack on the host
      const uint64_t cnt = bytes / 4;
      std::vector<unsigned long long> keys(cnt);
      cudaStreamSynchronize(s->impl->stream());
      int rc2 = ck(cudaMemcpy(keys.data(), st.g_key, cnt * 8, cudaMemcpyDeviceToHost), "debug copy");
      if (rc2) return rc2;
      uint32_t *o = static_cast<uint32_t *>(host);
      for (uint64_t i = 0; i < cnt; ++i)
        o[i] = which == GM_BUF_GRAPH_IDS ? (uint32_t)(keys[i] & 0xffffffffu) : (uint32_t)(keys[i] >> 32);
      return GM_OK;
    }
    case GM_BUF_KNN_IDS: src = st.knn_ids; break;
    case GM_BUF_KNN_DISTS: src = st.knn_dists; break;
    case GM_BUF_NORMS: src = st.norms; break;
    case GM_BUF_BLOOM: src = st.bloom; break;
    case GM_BUF_SIGMA: src = es.sigma; break;
    case GM_BUF_RHO: src = es.rho; break;
    case GM_BUF_COO_ROW: src = es.coo_row; break;
    case GM_BUF_COO_COL: src = es.coo_col; break;
    case GM_BUF_COO_VAL: src = es.coo_val; break;
    case GM_BUF_SCHED_ROW: src = es.t_row; break;
    case GM_BUF_SCHED_COL: src = es.flag_tail; break;
    case GM_BUF_SCHED_EPS: src = es.t_val; break;
    case GM_BUF_X: src = st.X; break;
    case GM_BUF_PUB_IDX: src = st.pub_idx; break;
    case GM_BUF_PUB_DIST: src = st.pub_dist; break;
    case GM_BUF_EMBEDDING: src = st.emb; break;
    case GM_BUF_EXACT_D: src = s->impl->exact_scratch(); break;
    default: return fail(GM_ERR_INVALID, "unknown buffer");
  }
  if (bytes == 0) return GM_OK;
  cudaStreamSynchronize(s->impl->stream());
  return ck(cudaMemcpy(host, src, bytes, cudaMemcpyDeviceToHost), "debug copy");
}

int gm_debug_keep_tiles(gm_session *s, int on) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  s->impl->set_keep_tile(on != 0);
  return GM_OK;
}

int gm_debug_pre_capacity(gm_session *s, int cap) {
  if (!s) return fail(GM_ERR_INVALID, "null session");
  if (cap < 0) return fail(GM_ERR_INVALID, "negative capacity");
  return guarded([&] { s->impl->set_pre_cap(cap); });
}

int gm_debug_scalars(const gm_session *s, int64_t *out, int n) {
  if (!s || !out) return fail(GM_ERR_INVALID, "null argument");
  s->impl->debug_scalars(out, n);
  return GM_OK;
}

int gm_debug_update_queue(const gm_session *s, uint32_t *out, uint64_t cap, uint64_t *n_out) {
  if (!s || !n_out) return fail(GM_ERR_INVALID, "null argument");
  const auto &q = s->impl->update_queue().items();
  *n_out = q.size();
  uint64_t i = 0;
  for (auto it = q.begin(); it != q.end() && i < cap; ++it, ++i) out[i] = *it;
  return GM_OK;
}

int gm_op_fuzzy_schedule(const uint32_t *pub_idx, const float *pub_dist, int64_t n,
                         int32_t k, int32_t euclidean, const int32_t *batch, int64_t nb,
                         int32_t n_epochs, float alpha, int32_t *coo_row, int32_t *coo_col,
                         float *coo_val, int32_t *t_row, int32_t *t_col, float *t_eps,
                         float *sigma, float *rho, int64_t *counts_out, float *scalars_out,
                         void *stream) {
  if (n < 0 || nb < 0 || k < 1 || k > 32 || n_epochs < 1)
    return fail(GM_ERR_INVALID, "bad sizes");
  cudaStream_t s = (cudaStream_t)stream;
  return guarded([&] {
    gm::EmbedScratch e;
    std::vector<void *> al;
    auto dalloc = [&](size_t bytes) {
      void *p = nullptr;
      if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        for (void *q : al) cudaFree(q);
        throw gm::Error(GM_ERR_OOM, "cudaMalloc");
      }
      al.push_back(p);
      return p;
    };
    const size_t cap = (size_t)std::max<int64_t>(2 * nb * k, 1);
    const size_t N = (size_t)std::max<int64_t>(n, 1);
    e.coo_row = coo_row;
    e.coo_col = coo_col;
    e.coo_val = coo_val;
    e.t_row = t_row;
    e.flag_tail = t_col;
    e.t_val = t_eps;
    e.sigma = sigma;
    e.rho = rho;
    e.t_col = (int *)dalloc(cap * sizeof(int));
    e.next_s = (float *)dalloc(cap * sizeof(float));
    e.next_n = (float *)dalloc(cap * sizeof(float));
    e.deg = (int *)dalloc(N * sizeof(int));
    e.fscal = (float *)dalloc(16 * sizeof(float));
    e.iscal = (int *)dalloc(16 * sizeof(int));
    e.cap_partial = (N * (size_t)k + 255) / 256 + 512;
    e.partial = (float *)dalloc(e.cap_partial * 2 * sizeof(float));
    e.ipartial = (int *)dalloc(e.cap_partial * sizeof(int));
    e.tmp = (int *)dalloc((gm::compact_tmp_ints((int)N) + 64) * sizeof(int));
    e.tmp2 = (int *)dalloc((gm::compact_tmp_ints((int)cap) + 64) * sizeof(int));
    e.cap_coo = cap;
    cudaMemsetAsync(e.iscal, 0, 16 * sizeof(int), s);
    cudaMemsetAsync(e.fscal, 0, 16 * sizeof(float), s);
    const double target = std::log2((double)(k - 1));
    gm::launch_fuzzy_graph(pub_idx, pub_dist, (int)n, k, euclidean, batch, (int)nb, target, e, s);
    gm::launch_schedule((int)n, (int)nb, k, alpha, n_epochs, 5, e, s);
    int iscal[16];
    float fscal[16];
    cudaMemcpyAsync(iscal, e.iscal, sizeof(iscal), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(fscal, e.fscal, sizeof(fscal), cudaMemcpyDeviceToHost, s);
    const cudaError_t err = cudaStreamSynchronize(s);
    for (void *q : al) cudaFree(q);
    if (err != cudaSuccess) throw gm::Error(GM_ERR_CUDA, cudaGetErrorString(err));
    if (counts_out) {
      counts_out[0] = iscal[0];
      counts_out[1] = iscal[1];
      counts_out[2] = iscal[2];
      counts_out[3] = iscal[3];
    }
    if (scalars_out) {
      scalars_out[0] = fscal[0];
      scalars_out[1] = fscal[1];
      scalars_out[2] = fscal[2];
    }
  });
}

int gm_op_sgd(float *emb, int64_t n, const int32_t *head, const int32_t *tail,
              const float *eps, int64_t nnz, float rounding, float alpha0, float gamma,
              float a, float b, int32_t n_epochs, int32_t neg_rate, uint64_t seed,
              void *stream) {
  if (n < 1 || nnz < 0 || n_epochs < 0) return fail(GM_ERR_INVALID, "bad sizes");
  if ((uintptr_t)emb % 8 != 0) return fail(GM_ERR_INVALID, "emb must be 8-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  return guarded([&] {
    if (nnz == 0 || n_epochs == 0) return;
    void *ns = nullptr, *nn = nullptr, *sc = nullptr;
    if (cudaMalloc(&ns, (size_t)nnz * 4) != cudaSuccess || cudaMalloc(&nn, (size_t)nnz * 4) != cudaSuccess ||
        cudaMalloc(&sc, 128) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(ns);
      cudaFree(nn);
      cudaFree(sc);
      throw gm::Error(GM_ERR_OOM, "cudaMalloc");
    }
    int iscal[16] = {0};
    float fscal[16] = {0};
    iscal[2] = (int)nnz;
    iscal[gm::kIscalN] = (int)n;
    fscal[2] = rounding;
    cudaMemcpyAsync(sc, iscal, 64, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync((char *)sc + 64, fscal, 64, cudaMemcpyHostToDevice, s);
    gm::launch_epoch_init(eps, (int)nnz, neg_rate, (float *)ns, (float *)nn, s);
    int dev = 0;
    cudaGetDevice(&dev);
    // scalars: iscal[0..16) at sc, fscal at sc + 64; grid-barrier words in
    // iscal[8..9], device error word in iscal[10]
    int *isc = (int *)sc;
    const cudaError_t le = gm::launch_sgd_call(
        emb, head, tail, eps, (float *)ns, (float *)nn, isc, (const float *)((char *)sc + 64),
        alpha0, gamma, a, b, n_epochs, neg_rate, seed, (unsigned *)(isc + gm::kIscalBarrier),
        (unsigned *)(isc + 10), dev, s);
    unsigned dev_err = 0;
    if (le == cudaSuccess) cudaMemcpyAsync(&dev_err, isc + 10, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    const cudaError_t err = le != cudaSuccess ? le : cudaStreamSynchronize(s);
    if (le != cudaSuccess) cudaGetLastError();
    cudaFree(ns);
    cudaFree(nn);
    cudaFree(sc);
    if (err != cudaSuccess) throw gm::Error(GM_ERR_CUDA, cudaGetErrorString(err));
    if (dev_err) throw gm::Error(GM_ERR_DEVICE, "SGD grid barrier wait ran out");
  });
}

}  // extern "C"
