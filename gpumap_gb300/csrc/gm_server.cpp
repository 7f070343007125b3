// Serving: many progressive sessions on one GPU behind a request queue
// (include/gpumap_gb300_server.h).  Worker threads ("slots") take queued
// requests in arrival order, skipping those whose session is busy, so each
// session's cycles run in order while different sessions' cycles run at the
// same time on their own streams.  Device memory is charged to a byte
// budget: a session's footprint when it opens, and the scratch a request's
// run may add before that run starts.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gm_engine.h"
#include "../../include/gpumap_gb300.h"
#include "../../include/gpumap_gb300_server.h"

namespace gm {
int set_last_error(int code, const char *msg);
}

namespace {

double now_s() {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

struct Request {
  uint64_t id = 0;
  uint32_t session = 0;
  std::vector<float> rows;
  uint64_t n_rows = 0, n_cols = 0;
  uint32_t n_upd = 0, n_emb = 0;
  double t_arrive = 0, t_start = 0, t_end = 0;
  int status = GM_OK;
  gm_result result{};
  bool done = false;
  size_t charged = 0;  // scratch growth charged to the budget while it runs
};

struct Slot {
  gm_session *h = nullptr;
  size_t bytes = 0;       // charged to the budget
  uint64_t committed = 0; // rows inserted or queued
  uint64_t capacity = 0;  // n_instances
  uint64_t n_features = 0;
  int active = 0;         // requests queued or running
  bool busy = false;      // a request is running
  bool closing = false;
};

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  const size_t i = std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5));
  std::nth_element(v.begin(), v.begin() + (long)i, v.end());
  return v[i];
}

}  // namespace

struct gm_server {
  gm_server_params p{};
  std::mutex mu;
  std::condition_variable cv;  // every change of queue, slot or request state
  std::map<uint32_t, Slot> sessions;
  uint32_t next_session = 1;
  std::deque<Request *> pending;
  std::map<uint64_t, std::unique_ptr<Request>> requests;
  uint64_t next_request = 1;
  size_t bytes_in_use = 0;
  int running = 0;
  bool stopping = false;
  std::vector<std::thread> workers;
  // finished requests
  std::vector<double> latency, service;
  uint64_t finished = 0, failed = 0, rows = 0;
  double first_arrive = std::numeric_limits<double>::infinity(), last_end = 0.0;

  void work();
  Request *take(std::unique_lock<std::mutex> &lk);
};

// Next request a slot may run: the oldest whose session is idle and whose
// possible scratch growth fits the budget.  A request that cannot fit while
// nothing else runs (so nothing can free memory) fails with GM_ERR_CAPACITY.
Request *gm_server::take(std::unique_lock<std::mutex> &) {
  for (auto it = pending.begin(); it != pending.end(); ++it) {
    Request *r = *it;
    Slot &sl = sessions.at(r->session);
    if (sl.busy) continue;
    const size_t grow = sl.h->impl->growth_bytes((uint32_t)r->n_rows, r->n_emb);
    if (bytes_in_use + grow > p.hbm_budget) {
      if (running > 0) continue;
      pending.erase(it);
      r->status = GM_ERR_CAPACITY;
      r->t_start = r->t_end = now_s();
      r->done = true;
      sl.active -= 1;
      sl.committed -= r->n_rows;
      failed += 1;
      cv.notify_all();
      return nullptr;  // the caller rescans
    }
    pending.erase(it);
    sl.busy = true;
    r->charged = grow;
    bytes_in_use += grow;
    running += 1;
    return r;
  }
  return nullptr;
}

void gm_server::work() {
  cudaSetDevice(p.device);
  for (;;) {
    Request *r = nullptr;
    gm_session *h = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      for (;;) {
        if (stopping && pending.empty()) return;
        const size_t before = pending.size();
        r = take(lk);
        if (r) break;
        if (pending.size() != before) continue;  // one failed: look again
        cv.wait(lk);
      }
      h = sessions.at(r->session).h;
    }
    r->t_start = now_s();
    int rc = r->n_rows ? gm_append(h, r->rows.data(), r->n_rows, r->n_cols) : GM_OK;
    const bool appended = rc == GM_OK;
    if (rc == GM_OK) rc = gm_run(h, (uint32_t)r->n_rows, r->n_upd, r->n_emb, &r->result);
    if (rc == GM_OK) {
      // the cycle is finished once its (possibly overlapped) embedding is
      try {
        h->impl->drain();
      } catch (const gm::Error &e) {
        rc = gm::set_last_error(e.code, e.what());
      } catch (const std::exception &e) {
        rc = gm::set_last_error(GM_ERR_RUNTIME, e.what());
      }
    }
    r->t_end = now_s();
    std::vector<float>().swap(r->rows);
    {
      std::lock_guard<std::mutex> g(mu);
      Slot &sl = sessions.at(r->session);
      // the charge becomes what the session holds now
      const size_t now_bytes = h->impl->device_bytes();
      bytes_in_use = bytes_in_use - r->charged - sl.bytes + now_bytes;
      sl.bytes = now_bytes;
      sl.busy = false;
      sl.active -= 1;
      running -= 1;
      r->status = rc;
      r->done = true;
      if (rc == GM_OK) {
        finished += 1;
        rows += r->n_rows;
        latency.push_back(r->t_end - r->t_arrive);
        service.push_back(r->t_end - r->t_start);
        first_arrive = std::min(first_arrive, r->t_arrive);
        last_end = std::max(last_end, r->t_end);
      } else {
        failed += 1;
        if (!appended) sl.committed -= r->n_rows;  // the rows did not go in
      }
      cv.notify_all();
    }
  }
}

extern "C" {

int gm_server_create(const gm_server_params *p, gm_server **out) {
  if (!p || !out) return gm::set_last_error(GM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (p->slots < 1 || p->slots > 64) return gm::set_last_error(GM_ERR_INVALID, "slots must be in [1, 64]");
  if (p->hbm_budget == 0) return gm::set_last_error(GM_ERR_INVALID, "hbm_budget must be positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || p->device < 0 || p->device >= ndev) {
    cudaGetLastError();
    return gm::set_last_error(GM_ERR_INVALID, "no such CUDA device");
  }
  auto *s = new (std::nothrow) gm_server;
  if (!s) return gm::set_last_error(GM_ERR_OOM, "host allocation failed");
  s->p = *p;
  try {
    for (int i = 0; i < p->slots; ++i) s->workers.emplace_back([s] { s->work(); });
  } catch (const std::exception &e) {
    {
      std::lock_guard<std::mutex> g(s->mu);
      s->stopping = true;
    }
    s->cv.notify_all();
    for (auto &t : s->workers) t.join();
    delete s;
    return gm::set_last_error(GM_ERR_RUNTIME, e.what());
  }
  *out = s;
  return gm::set_last_error(GM_OK, "");
}

void gm_server_destroy(gm_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stopping = true;
  }
  s->cv.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto &kv : s->sessions) gm_destroy(kv.second.h);
  delete s;
}

int gm_server_open_session(gm_server *s, const gm_params *params, uint32_t *session_out) {
  if (!s || !params || !session_out) return gm::set_last_error(GM_ERR_INVALID, "null argument");
  gm_params q = *params;
  q.device = s->p.device;
  size_t free_b = 0, total_b = 0;
  if (cudaSetDevice(s->p.device) != cudaSuccess || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return gm::set_last_error(GM_ERR_CUDA, "cannot query device memory");
  }
  gm_session *h = nullptr;
  int rc = gm_create(&q, &h);
  if (rc != GM_OK) return rc;
  const size_t bytes = h->impl->device_bytes();
  std::lock_guard<std::mutex> g(s->mu);
  if (s->bytes_in_use + bytes > s->p.hbm_budget) {
    gm_destroy(h);
    return gm::set_last_error(GM_ERR_CAPACITY, ("session needs " + std::to_string(bytes) +
                                                " device bytes; the server's budget has " +
                                                std::to_string(s->p.hbm_budget - s->bytes_in_use) + " left")
                                                   .c_str());
  }
  const uint32_t id = s->next_session++;
  Slot sl;
  sl.h = h;
  sl.bytes = bytes;
  sl.capacity = q.n_instances;
  sl.n_features = q.n_features;
  s->sessions[id] = sl;
  s->bytes_in_use += bytes;
  *session_out = id;
  return gm::set_last_error(GM_OK, "");
}

int gm_server_close_session(gm_server *s, uint32_t session) {
  if (!s) return gm::set_last_error(GM_ERR_INVALID, "null server");
  gm_session *h = nullptr;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->sessions.find(session);
    if (it == s->sessions.end() || it->second.closing)
      return gm::set_last_error(GM_ERR_INVALID, "no such session");
    it->second.closing = true;
    s->cv.wait(lk, [&] { return it->second.active == 0; });
    h = it->second.h;
    s->bytes_in_use -= it->second.bytes;
    s->sessions.erase(it);
    s->cv.notify_all();
  }
  gm_destroy(h);
  return gm::set_last_error(GM_OK, "");
}

int gm_server_submit(gm_server *s, uint32_t session, const float *host_rows, uint64_t rows,
                     uint64_t n_cols, uint32_t n_update_ops, uint32_t n_embedding_ops,
                     uint64_t *request_out) {
  if (!s || !request_out || (rows > 0 && !host_rows))
    return gm::set_last_error(GM_ERR_INVALID, "null argument");
  auto r = std::make_unique<Request>();
  r->session = session;
  r->n_rows = rows;
  r->n_cols = n_cols;
  r->n_upd = n_update_ops;
  r->n_emb = n_embedding_ops;
  try {
    r->rows.assign(host_rows, host_rows + rows * n_cols);
  } catch (const std::bad_alloc &) {
    return gm::set_last_error(GM_ERR_OOM, "host allocation failed");
  }
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stopping) return gm::set_last_error(GM_ERR_CLOSED, "server is stopping");
  auto it = s->sessions.find(session);
  if (it == s->sessions.end() || it->second.closing) return gm::set_last_error(GM_ERR_INVALID, "no such session");
  Slot &sl = it->second;
  if (rows > 0 && n_cols != sl.n_features)
    return gm::set_last_error(GM_ERR_INVALID, "n_cols does not match the session's n_features");
  if (sl.committed + rows > sl.capacity)
    return gm::set_last_error(GM_ERR_CAPACITY, "the session cannot take these rows (n_instances reached)");
  sl.committed += rows;
  sl.active += 1;
  r->id = s->next_request++;
  r->t_arrive = now_s();
  *request_out = r->id;
  s->pending.push_back(r.get());
  s->requests[r->id] = std::move(r);
  s->cv.notify_all();
  return gm::set_last_error(GM_OK, "");
}

int gm_server_wait(gm_server *s, uint64_t request, gm_request_info *out) {
  if (!s || !out) return gm::set_last_error(GM_ERR_INVALID, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->requests.find(request);
  if (it == s->requests.end()) return gm::set_last_error(GM_ERR_INVALID, "no such request (or already waited for)");
  Request *r = it->second.get();
  s->cv.wait(lk, [&] { return r->done; });
  out->request = r->id;
  out->session = r->session;
  out->status = r->status;
  out->rows = r->n_rows;
  out->t_arrive = r->t_arrive;
  out->t_start = r->t_start;
  out->t_end = r->t_end;
  out->result = r->result;
  s->requests.erase(it);
  return gm::set_last_error(GM_OK, "");
}

int gm_server_drain(gm_server *s) {
  if (!s) return gm::set_last_error(GM_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv.wait(lk, [&] { return s->pending.empty() && s->running == 0; });
  return gm::set_last_error(GM_OK, "");
}

int gm_server_session_handle(gm_server *s, uint32_t session, gm_session **out) {
  if (!s || !out) return gm::set_last_error(GM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->sessions.find(session);
  if (it == s->sessions.end()) return gm::set_last_error(GM_ERR_INVALID, "no such session");
  *out = it->second.h;
  return gm::set_last_error(GM_OK, "");
}

int gm_server_get_stats(gm_server *s, gm_server_stats *out) {
  if (!s || !out) return gm::set_last_error(GM_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->finished = s->finished;
  out->failed = s->failed;
  out->rows = s->rows;
  out->sessions_open = s->sessions.size();
  out->bytes_in_use = s->bytes_in_use;
  out->first_arrive = s->finished ? s->first_arrive : 0.0;
  out->last_end = s->last_end;
  out->latency_p50 = percentile(s->latency, 0.50);
  out->latency_p99 = percentile(s->latency, 0.99);
  out->latency_max = s->latency.empty() ? 0.0 : *std::max_element(s->latency.begin(), s->latency.end());
  out->service_p50 = percentile(s->service, 0.50);
  out->service_p99 = percentile(s->service, 0.99);
  return gm::set_last_error(GM_OK, "");
}

}  // extern "C"
