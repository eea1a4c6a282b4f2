// server.cu -- the serving form of the C ABI: continuous admission of verification requests.
//
// Requests are copied at submit time (the caller's descriptor arrays may be freed afterwards) and
// admitted in arrival order while an in-flight slot is free and the device-memory pool can hold the
// request's initial store reservation. Each admitted request runs on its own worker thread and CUDA
// stream, so requests admitted while others run overlap with them on the device and a short request
// is not held back by a long one. A running request's passed/waiting stores stay resident across its
// BFS levels and grow by taking more from the shared pool; a request whose store needs more than the
// pool has left, or more than the server's per-request limit, stops with HORA_E_BUDGET. With a bounded
// queue, a request that arrives while the queue is full is rejected at submission. Destroying the
// server cancels the running requests at their next level.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "host.h"

namespace hgb {

struct Request {
  int64_t ticket = 0;
  OwnedNet net;
  uint64_t est_bytes = 0;
  int done = 0;
  int verdict = -1;
  hora_stats st{};
  BudgetPool limit;   // the request's growth beyond its reservation, inside the server's pool
  std::chrono::steady_clock::time_point t_submit;
};

}  // namespace hgb

// The serving loop: one worker thread per in-flight slot; each takes the oldest queued request whose
// reservation fits the pool, runs it, publishes the result and takes the next.
struct hora_server {
  hgb::BudgetPool pool;                // device memory of the admitted requests' stores
  int max_inflight = 0;
  int inflight = 0;
  uint64_t per_request = 0;            // a request's store may hold at most this much (0: no limit)
  int32_t max_queued = 0;              // submissions past this many waiting requests are rejected (0: none)
  int64_t next_ticket = 1;
  std::deque<std::unique_ptr<hgb::Request>> queue;
  std::set<int64_t> running;
  std::map<int64_t, std::unique_ptr<hgb::Request>> finished;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  volatile int32_t cancel = 0;         // set by destroy: running requests end at their next level
  std::vector<std::thread> workers;
  int device = 0;
};

using namespace hgb;

// A request's initial store reservation: 64 Ki zones of its dimension, or a slice of the pool when
// that is larger; the store grows from the pool as it needs.
static uint64_t reserve_bytes(const hora_server* s, const hora_net_desc* n) {
  const uint64_t d = (uint64_t)n->nclocks + 1;
  const uint64_t floor_bytes = (1ull << 16) * (d * d * 4 + 32) * 2;
  const uint64_t slice = s->pool.cap / (uint64_t)(4 * s->max_inflight);
  const uint64_t r = slice > floor_bytes ? slice : floor_bytes;
  return s->per_request && r > s->per_request ? s->per_request : r;
}

static void worker_main(hora_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    std::unique_ptr<Request> r;
    uint64_t per_request = 0;
    {
      std::unique_lock<std::mutex> g(s->mu);
      s->cv.wait(g, [&] {
        return s->stop || (!s->queue.empty() && s->inflight < s->max_inflight &&
                           s->pool.used.load() + s->queue.front()->est_bytes <= s->pool.cap);
      });
      if (s->stop) return;
      if (!s->pool.take(s->queue.front()->est_bytes)) continue;   // a running store just grew
      ++s->inflight;
      r = std::move(s->queue.front());
      s->queue.pop_front();
      s->running.insert(r->ticket);
      per_request = s->per_request;
    }
    int32_t verdict = -1;
    hora_stats st{};
    BudgetPool* grow = &s->pool;
    if (per_request) {
      // growth past the reservation must fit both the request's limit and the server's pool
      r->limit.cap = per_request > r->est_bytes ? per_request - r->est_bytes : 0;
      r->limit.parent = &s->pool;
      grow = &r->limit;
    }
    const int rc = run_batch(1, &r->net.d, &r->net.q, &verdict, &st, &s->cancel, (size_t)r->est_bytes, grow);
    const auto now = std::chrono::steady_clock::now();
    {
      std::lock_guard<std::mutex> g(s->mu);
      r->done = 1;
      r->verdict = (rc == HORA_OK || rc == HORA_E_CANCELLED) && st.status == HORA_OK ? verdict : -1;
      r->st = st;
      if (rc && rc != HORA_E_CANCELLED) r->st.status = rc;
      // time to verdict: submission to publication
      r->st.seconds = std::chrono::duration<double>(now - r->t_submit).count();
      s->pool.give(r->est_bytes);
      --s->inflight;
      s->running.erase(r->ticket);
      const int64_t t = r->ticket;
      s->finished[t] = std::move(r);
    }
    s->cv.notify_all();
  }
}

extern "C" {

int32_t hora_gb_server_create(uint64_t budget_bytes, int32_t max_inflight, hora_server** out) {
  if (!out || max_inflight <= 0) return HORA_E_INVALID;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return HORA_E_NO_DEVICE;
  hora_server* s = new hora_server;
  s->pool.cap = budget_bytes;
  s->max_inflight = max_inflight;
  cudaGetDevice(&s->device);
  const int nworkers = std::min(64, max_inflight);
  for (int w = 0; w < nworkers; ++w) s->workers.emplace_back(worker_main, s);
  *out = s;
  return HORA_OK;
}

int32_t hora_gb_server_submit(hora_server* s, const hora_net_desc* net, const hora_query_desc* q, int64_t* ticket) {
  if (!s || !net || !q || !ticket) return HORA_E_INVALID;
  const auto t_arrive = std::chrono::steady_clock::now();
  uint64_t est = 0;
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->max_queued > 0 && (int64_t)s->queue.size() >= s->max_queued) return HORA_E_BUDGET;   // queue full
    est = reserve_bytes(s, net);
  }
  if (est > s->pool.cap) return HORA_E_BUDGET;
  auto r = std::make_unique<Request>();
  r->net.copy(net, q);
  r->est_bytes = est;
  r->t_submit = t_arrive;
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->queue.push_back(std::move(r));
  }
  s->cv.notify_all();
  return HORA_OK;
}

int32_t hora_gb_server_set_limits(hora_server* s, uint64_t per_request_bytes, int32_t max_queued) {
  if (!s || max_queued < 0) return HORA_E_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  s->per_request = per_request_bytes;
  s->max_queued = max_queued;
  return HORA_OK;
}

int32_t hora_gb_server_step(hora_server* s, int32_t* active) {
  if (!s) return HORA_E_INVALID;
  std::unique_lock<std::mutex> g(s->mu);
  // the workers drive the device; waiting briefly for progress keeps a polling caller from spinning
  s->cv.wait_for(g, std::chrono::milliseconds(1));
  if (active) *active = (int32_t)s->queue.size() + s->inflight;
  return HORA_OK;
}

int32_t hora_gb_server_poll(hora_server* s, int64_t ticket, int32_t* done, int32_t* verdict, hora_stats* stats) {
  if (!s || !done) return HORA_E_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->finished.find(ticket);
  if (it == s->finished.end()) {
    if (ticket <= 0 || ticket >= s->next_ticket) return HORA_E_INVALID;
    bool pending = s->running.count(ticket) > 0;
    for (const auto& q : s->queue) pending |= q->ticket == ticket;
    if (!pending) return HORA_E_INVALID;    // already reported, and released
    *done = 0;
    return HORA_OK;
  }
  *done = 1;
  if (verdict) *verdict = it->second->verdict;
  if (stats) *stats = it->second->st;
  s->finished.erase(it);                    // a result is reported once; its copy is released
  return HORA_OK;
}

int32_t hora_gb_server_destroy(hora_server* s) {
  if (!s) return HORA_E_INVALID;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    s->cancel = 1;
  }
  s->cv.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
  return HORA_OK;
}

}  // extern "C"
