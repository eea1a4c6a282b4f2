// server.cu -- the serving form of the C ABI: continuous admission of verification requests.
//
// Requests are copied at submit time (the caller's descriptor arrays may be freed afterwards) and
// admitted in arrival order while a slot of the in-flight limit and its share of the device-memory
// budget are free. Each admitted request runs on its own worker thread and CUDA stream, so requests
// admitted while others are running overlap with them on the device, and a short request is not
// held back by a long one. A request whose passed store outgrows its share stops with
// HORA_E_BUDGET.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <map>
#include <memory>
#include <mutex>
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
  std::chrono::steady_clock::time_point t_submit;
};

}  // namespace hgb

// The serving loop: one worker thread per in-flight slot; each takes the oldest queued request whose
// budget share fits, runs it, publishes the result and takes the next.
struct hora_server {
  uint64_t budget = 0;
  uint64_t in_use = 0;                 // estimated bytes of the requests on the device
  int max_inflight = 0;
  int inflight = 0;
  int64_t next_ticket = 1;
  std::deque<std::unique_ptr<hgb::Request>> queue;
  std::map<int64_t, std::unique_ptr<hgb::Request>> finished;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  std::vector<std::thread> workers;
  int device = 0;
};

using namespace hgb;

// A request's share of the budget: an equal part per in-flight slot, but at least 64 Ki zones of its
// dimension.
static uint64_t share_bytes(const hora_server* s, const hora_net_desc* n) {
  const uint64_t d = (uint64_t)n->nclocks + 1;
  const uint64_t floor_bytes = (1ull << 16) * (d * d * 4 + 32);
  const uint64_t share = s->budget / (uint64_t)s->max_inflight;
  return share > floor_bytes ? share : floor_bytes;
}

static void worker_main(hora_server* s, int per_batch) {
  cudaSetDevice(s->device);
  for (;;) {
    std::vector<std::unique_ptr<Request>> batch;
    {
      std::unique_lock<std::mutex> g(s->mu);
      s->cv.wait(g, [&] {
        return s->stop || (!s->queue.empty() && s->inflight < s->max_inflight &&
                           s->in_use + s->queue.front()->est_bytes <= s->budget);
      });
      if (s->stop) return;
      while (!s->queue.empty() && (int)batch.size() < per_batch && s->inflight < s->max_inflight &&
             s->in_use + s->queue.front()->est_bytes <= s->budget) {
        s->in_use += s->queue.front()->est_bytes;
        ++s->inflight;
        batch.push_back(std::move(s->queue.front()));
        s->queue.pop_front();
      }
    }
    std::vector<hora_net_desc> nets;
    std::vector<hora_query_desc> qs;
    for (auto& r : batch) { nets.push_back(r->net.d); qs.push_back(r->net.q); }
    std::vector<int32_t> verdicts(batch.size());
    std::vector<hora_stats> st(batch.size());
    uint64_t share = 0;
    for (auto& r : batch) share += r->est_bytes;
    const int rc = run_batch((int32_t)batch.size(), nets.data(), qs.data(), verdicts.data(), st.data(), nullptr,
                             (size_t)share);
    const auto now = std::chrono::steady_clock::now();
    {
      std::lock_guard<std::mutex> g(s->mu);
      for (size_t k = 0; k < batch.size(); ++k) {
        Request& r = *batch[k];
        r.done = 1;
        r.verdict = rc == HORA_OK ? verdicts[k] : -1;
        r.st = st[k];
        if (rc) r.st.status = rc;
        // time to verdict: submission to publication
        r.st.seconds = std::chrono::duration<double>(now - r.t_submit).count();
        s->in_use -= r.est_bytes;
        --s->inflight;
        const int64_t t = r.ticket;
        s->finished[t] = std::move(batch[k]);
      }
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
  s->budget = budget_bytes;
  s->max_inflight = max_inflight;
  cudaGetDevice(&s->device);
  const int nworkers = std::min(64, max_inflight);
  const int per_batch = 1;
  for (int w = 0; w < nworkers; ++w) s->workers.emplace_back(worker_main, s, per_batch);
  *out = s;
  return HORA_OK;
}

int32_t hora_gb_server_submit(hora_server* s, const hora_net_desc* net, const hora_query_desc* q, int64_t* ticket) {
  if (!s || !net || !q || !ticket) return HORA_E_INVALID;
  const uint64_t est = share_bytes(s, net);
  if (est > s->budget) return HORA_E_BUDGET;
  auto r = std::make_unique<Request>();
  r->net.copy(net, q);
  r->est_bytes = est;
  r->t_submit = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->queue.push_back(std::move(r));
  }
  s->cv.notify_all();
  return HORA_OK;
}

int32_t hora_gb_server_step(hora_server* s, int32_t* active) {
  if (!s) return HORA_E_INVALID;
  std::unique_lock<std::mutex> g(s->mu);
  // wait briefly for progress so that a polling caller does not spin
  s->cv.wait_for(g, std::chrono::milliseconds(1));
  if (active) *active = (int32_t)s->queue.size() + s->inflight;
  return HORA_OK;
}

int32_t hora_gb_server_poll(hora_server* s, int64_t ticket, int32_t* done, int32_t* verdict, hora_stats* stats) {
  if (!s || !done) return HORA_E_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->finished.find(ticket);
  if (it == s->finished.end()) { *done = 0; return HORA_OK; }
  *done = 1;
  if (verdict) *verdict = it->second->verdict;
  if (stats) *stats = it->second->st;
  return HORA_OK;
}

int32_t hora_gb_server_destroy(hora_server* s) {
  if (!s) return HORA_E_INVALID;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
  return HORA_OK;
}

}  // extern "C"
