// host.h -- host-side model compilation and the per-dimension engine entry points.
#pragma once
#include <atomic>
#include <cstdint>
#include <chrono>
#include <string>
#include <vector>

#include "../../include/hora_gb300.h"
#include "engine.cuh"

namespace hgb {

// Device memory shared by the requests of a server: each request's store starts from the reservation
// it was admitted with and grows level by level while the pool has room (BudgetPool::take). A pool
// with a parent is one request's limit inside the server's pool: a take must fit both.
struct BudgetPool {
  std::atomic<uint64_t> used{0};
  uint64_t cap = 0;
  BudgetPool* parent = nullptr;
  bool take(uint64_t b) {
    uint64_t u = used.load();
    while (u + b <= cap) {
      if (used.compare_exchange_weak(u, u + b)) {
        if (!parent || parent->take(b)) return true;
        used.fetch_sub(b);
        return false;
      }
    }
    return false;
  }
  void give(uint64_t b) {
    used.fetch_sub(b);
    if (parent) parent->give(b);
  }
};


// One (network, query) instance compiled for the device: the descriptor's arrays re-indexed, the
// static analyses of src/model/network.cpp applied, and the query's constants folded in.
struct HostNet {
  int kind = 0;
  int nclocks = 0, dim = 0, nprocs = 0, nints = 0, nchans = 0, nedges = 0, nlocs = 0;
  int keybits = 0;
  int has_urgent_chan = 0;
  int t_never = 0;
  unsigned long long qmask = 0;
  std::vector<int32_t> chan_flags, int_lo, int_init, proc_init, loc_base, loc_flags, loc_inv_off, eloc_off,
      eloc, edge_tgt, edge_chan, edge_dir, edge_guard_off, edge_iguard_off, edge_reset_off, edge_iupd_off, cons,
      iatoms, resets, iupds, Lloc, Uloc, kshift, kwidth, L, U, Lq, Uq, t_loc, t_int, t_clk;
  std::vector<unsigned long long> act;
  // leads-to
  int av_on = 0, av_nclk = 0, av_psi = 0;
  int av_neg[3] = {0, 0, 0};
  std::vector<int32_t> av_loc, av_int, av_clk, p_loc, p_int, p_clk;
};

// Compile `net` for query `kind` (HORA_Q_*): `p` is the reach target or the left side of a
// leads-to, `q` its right side (both may be null when unused).
// Returns HORA_OK, HORA_E_INVALID or HORA_E_NOT_SUPPORTED with a message in `err`.
int compile_net(const hora_net_desc* net, int kind, const hora_pred_desc* p, const hora_pred_desc* q, HostNet& out,
                std::string& err);

// Device copy of one or more compiled instances: a blob per instance and the NetView array.
// Device memory of the engine comes from the stream-ordered allocator (cudaMallocAsync /
// cudaFreeAsync) on the stream of the search that owns it: freeing never synchronises the device,
// so concurrent searches (the batched and serving forms) do not stall one another, and the device's
// default pool keeps freed memory for reuse (up to a release threshold set once per device).
// g_alloc_stream is that stream for the calling thread (nullptr: the legacy default stream).
extern thread_local cudaStream_t g_alloc_stream;
void prepare_device_pool();

struct DeviceNets {
  cudaStream_t stream = nullptr;   // the stream the tables were allocated on (freed on it)
  std::vector<void*> blobs;
  std::vector<size_t> blob_bytes;
  NetView* views = nullptr;   // device array
  NetView* views_plain = nullptr;  // the same with the leads-to restriction off (reachability phases)
  std::vector<NetView> host_views;
  int* ok = nullptr;          // device array of per-instance "runnable" flags
  ~DeviceNets();
};
int upload_nets(const std::vector<const HostNet*>& nets, int inst_shift, DeviceNets& out, std::string& err);
void build_blob(const HostNet& H, std::vector<int32_t>& blob, std::vector<size_t>& offs);
NetView make_view(const HostNet& H, const int32_t* device_blob, const std::vector<size_t>& offs, int inst_shift);

// Owned copy of a network descriptor and a query: the caller's arrays may be freed afterwards
// (the serving queue and query handles keep their requests this way).
struct OwnedNet {
  std::vector<int32_t> chan_flags, int_lo, int_hi, int_init, proc_nlocs, proc_init, loc_flags, loc_inv_off,
      edge_proc, edge_src, edge_tgt, edge_chan, edge_dir, edge_guard_off, edge_iguard_off, edge_reset_off,
      edge_iupd_off, cons, iatoms, resets, iupds;
  std::vector<int32_t> p_loc, p_int, p_clk, q_loc, q_int, q_clk;
  hora_net_desc d{};
  hora_query_desc q{};
  void copy(const hora_net_desc* n, const hora_query_desc* qq);
};

// The batched form (hora_gb_batch_run) with an explicit store budget for the whole call, in bytes
// (0: three quarters of the free device memory).
int32_t run_batch(int32_t n, const hora_net_desc* nets, const hora_query_desc* queries, int32_t* verdicts,
                  hora_stats* stats, const volatile int32_t* cancel, size_t store_budget,
                  BudgetPool* pool = nullptr);

// Result of one instance.
struct InstResult {
  int status = HORA_OK;
  int verdict = 0;            // goal reached (reach: target reachable; deadlock: deadlock reachable)
  hora_stats st{};
};

// A witness of E[] psi read back from the exact zone graph: the states of a path from the root, each
// reached from the previous one by its emission ordinal, ending in a stop state (loop_to = -1) or
// closing a cycle into state loop_to by ordinal loop_ord.
struct Trace {
  std::vector<int32_t> ords, locs, ints, zones;
  int loop_to = -1, loop_ord = -1, nsteps = 0;
};

struct RunOptions {
  int blocks = 0;             // grid cap for the level kernels (0: derived from the SM count)
  const volatile int32_t* cancel = nullptr;
  size_t succ_cap0 = 1 << 16; // initial successor-buffer capacity
  size_t succ_budget_bytes = size_t(8) << 30;  // a level's successors beyond this run in instance chunks
  size_t store_budget_bytes = 0;  // 0: unbounded; else instances stop with HORA_E_BUDGET past it
  BudgetPool* pool = nullptr;     // when set, the store may grow past store_budget_bytes by taking
                                  // more from the pool (returned when the run ends)
  bool has_t_call = false;    // per-instance times count from t_call (the batch call) when set
  std::chrono::steady_clock::time_point t_call{};
  Trace* trace = nullptr;     // E[] psi, one instance: fill with a witness when it holds
  bool yield_wait = false;    // wait for the stream on a blocking-sync event (the host thread sleeps
                              // instead of spinning): for groups that share the host's cores
  int long_list = 4;          // the probe scans a key list longer than this with a whole warp
  bool long_list_env = false; // long_list came from the environment (it then overrides the tuning)
  int blocks_per_sm = 16;     // grid of the level kernels: this many blocks per SM (when blocks is 0)
};

// Run a group of instances that share the DBM dimension D (one level-synchronous BFS over all of
// them). Implemented per D in the generated units.
template <int D>
int run_group(const std::vector<const HostNet*>& nets, std::vector<InstResult>& res, const RunOptions& o,
              std::string& err);
template <int D>
int run_expand(const HostNet& net, int n, const int* locs, const int* ints, const int* zones, int emode,
               int64_t cap, int* out_src, int* out_ord, int* out_locs, int* out_ints, int* out_zones, int64_t* out_n,
               std::string& err);
template <int D>
int run_has_deadlock(const HostNet& net, int n, const int* locs, const int* ints, const int* zones, int* out,
                     std::string& err);

constexpr int kMinDim = 1;
constexpr int kMaxDim = 17;

}  // namespace hgb
