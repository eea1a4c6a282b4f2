// server.cu -- the serving form of the C ABI: a request queue drained into device batches.
//
// Requests are copied at submit time (the caller's descriptor arrays may be freed afterwards).
// Each hora_gb_server_step() admits queued requests in arrival order while their estimated
// passed/waiting-store footprint fits the budget and the in-flight limit allows, runs the admitted
// set as one batched level-synchronous search per DBM dimension, and publishes the results.
#include <cuda_runtime.h>

#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"

namespace hgb {

// Owned copy of a network descriptor and a query.
struct OwnedNet {
  std::vector<int32_t> chan_flags, int_lo, int_hi, int_init, proc_nlocs, proc_init, loc_flags, loc_inv_off,
      edge_proc, edge_src, edge_tgt, edge_chan, edge_dir, edge_guard_off, edge_iguard_off, edge_reset_off,
      edge_iupd_off, cons, iatoms, resets, iupds;
  std::vector<int32_t> p_loc, p_int, p_clk, q_loc, q_int, q_clk;
  hora_net_desc d{};
  hora_query_desc q{};
  void copy(const hora_net_desc* n, const hora_query_desc* qq) {
    int tot = 0;
    for (int p = 0; p < n->nprocs; ++p) tot += n->proc_nlocs[p];
    const int ne = n->nedges;
    auto cp = [](std::vector<int32_t>& v, const int32_t* s, size_t k) { v.assign(s, s + k); if (v.empty()) v.push_back(0); };
    cp(chan_flags, n->chan_flags, n->nchans);
    cp(int_lo, n->int_lo, n->nints); cp(int_hi, n->int_hi, n->nints); cp(int_init, n->int_init, n->nints);
    cp(proc_nlocs, n->proc_nlocs, n->nprocs); cp(proc_init, n->proc_init, n->nprocs);
    cp(loc_flags, n->loc_flags, tot); cp(loc_inv_off, n->loc_inv_off, tot + 1);
    cp(edge_proc, n->edge_proc, ne); cp(edge_src, n->edge_src, ne); cp(edge_tgt, n->edge_tgt, ne);
    cp(edge_chan, n->edge_chan, ne); cp(edge_dir, n->edge_dir, ne);
    cp(edge_guard_off, n->edge_guard_off, ne + 1); cp(edge_iguard_off, n->edge_iguard_off, ne + 1);
    cp(edge_reset_off, n->edge_reset_off, ne + 1); cp(edge_iupd_off, n->edge_iupd_off, ne + 1);
    const int ncons = std::max(ne ? n->edge_guard_off[ne] : 0, n->loc_inv_off[tot]);
    cp(cons, n->cons, 3 * (size_t)ncons);
    cp(iatoms, n->iatoms, ne ? 3 * (size_t)n->edge_iguard_off[ne] : 0);
    cp(resets, n->resets, ne ? (size_t)n->edge_reset_off[ne] : 0);
    cp(iupds, n->iupds, ne ? 2 * (size_t)n->edge_iupd_off[ne] : 0);
    d = *n;
    d.chan_flags = chan_flags.data(); d.int_lo = int_lo.data(); d.int_hi = int_hi.data(); d.int_init = int_init.data();
    d.proc_nlocs = proc_nlocs.data(); d.proc_init = proc_init.data(); d.loc_flags = loc_flags.data();
    d.loc_inv_off = loc_inv_off.data(); d.edge_proc = edge_proc.data(); d.edge_src = edge_src.data();
    d.edge_tgt = edge_tgt.data(); d.edge_chan = edge_chan.data(); d.edge_dir = edge_dir.data();
    d.edge_guard_off = edge_guard_off.data(); d.edge_iguard_off = edge_iguard_off.data();
    d.edge_reset_off = edge_reset_off.data(); d.edge_iupd_off = edge_iupd_off.data(); d.cons = cons.data();
    d.iatoms = iatoms.data(); d.resets = resets.data(); d.iupds = iupds.data();
    q = *qq;
    cp(p_loc, qq->p.loc_req, 2 * (size_t)qq->p.nloc); cp(p_int, qq->p.int_cond, 3 * (size_t)qq->p.nint);
    cp(p_clk, qq->p.clk_cond, 3 * (size_t)qq->p.nclk);
    cp(q_loc, qq->q.loc_req, 2 * (size_t)qq->q.nloc); cp(q_int, qq->q.int_cond, 3 * (size_t)qq->q.nint);
    cp(q_clk, qq->q.clk_cond, 3 * (size_t)qq->q.nclk);
    q.p.loc_req = p_loc.data(); q.p.int_cond = p_int.data(); q.p.clk_cond = p_clk.data();
    q.q.loc_req = q_loc.data(); q.q.int_cond = q_int.data(); q.q.clk_cond = q_clk.data();
  }
};

struct Request {
  int64_t ticket = 0;
  OwnedNet net;
  uint64_t est_bytes = 0;
  int done = 0;
  int verdict = -1;
  hora_stats st{};
};

}  // namespace hgb

struct hora_server {
  uint64_t budget = 0;
  int max_inflight = 0;
  int64_t next_ticket = 1;
  std::deque<std::unique_ptr<hgb::Request>> queue;
  std::map<int64_t, std::unique_ptr<hgb::Request>> finished;
  std::mutex mu;
};

using namespace hgb;

// A request's store estimate: a floor of 64 Ki zones of its dimension plus the hash table.
static uint64_t estimate_bytes(const hora_net_desc* n) {
  const uint64_t d = (uint64_t)n->nclocks + 1;
  return (1ull << 16) * (d * d * 4 + 32);
}

extern "C" {

int32_t hora_gb_server_create(uint64_t budget_bytes, int32_t max_inflight, hora_server** out) {
  if (!out || max_inflight <= 0) return HORA_E_INVALID;
  hora_server* s = new hora_server;
  s->budget = budget_bytes;
  s->max_inflight = max_inflight;
  *out = s;
  return HORA_OK;
}

int32_t hora_gb_server_submit(hora_server* s, const hora_net_desc* net, const hora_query_desc* q, int64_t* ticket) {
  if (!s || !net || !q || !ticket) return HORA_E_INVALID;
  const uint64_t est = estimate_bytes(net);
  if (est > s->budget) return HORA_E_BUDGET;
  auto r = std::make_unique<Request>();
  r->net.copy(net, q);
  r->est_bytes = est;
  std::lock_guard<std::mutex> g(s->mu);
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  s->queue.push_back(std::move(r));
  return HORA_OK;
}

int32_t hora_gb_server_step(hora_server* s, int32_t* active) {
  if (!s) return HORA_E_INVALID;
  std::vector<std::unique_ptr<Request>> batch;
  {
    std::lock_guard<std::mutex> g(s->mu);
    uint64_t used = 0;
    while (!s->queue.empty() && (int)batch.size() < s->max_inflight &&
           used + s->queue.front()->est_bytes <= s->budget) {
      used += s->queue.front()->est_bytes;
      batch.push_back(std::move(s->queue.front()));
      s->queue.pop_front();
    }
  }
  if (!batch.empty()) {
    std::vector<hora_net_desc> nets;
    std::vector<hora_query_desc> qs;
    for (auto& r : batch) { nets.push_back(r->net.d); qs.push_back(r->net.q); }
    std::vector<int32_t> verdicts(batch.size());
    std::vector<hora_stats> st(batch.size());
    const int rc = hora_gb_batch_run((int32_t)batch.size(), nets.data(), qs.data(), verdicts.data(), st.data());
    std::lock_guard<std::mutex> g(s->mu);
    for (size_t k = 0; k < batch.size(); ++k) {
      batch[k]->done = 1;
      batch[k]->verdict = rc == HORA_OK ? verdicts[k] : -1;
      batch[k]->st = st[k];
      if (rc) batch[k]->st.status = rc;
      const int64_t t = batch[k]->ticket;
      s->finished[t] = std::move(batch[k]);
    }
  }
  if (active) {
    std::lock_guard<std::mutex> g(s->mu);
    *active = (int32_t)s->queue.size();
  }
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
  delete s;
  return HORA_OK;
}

}  // extern "C"
