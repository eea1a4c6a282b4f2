// engine_run.cuh -- the host-side level loop for one dimension D (run_group<D>) and the
// host-buffer entry points (run_expand<D>, run_has_deadlock<D>). Included by the generated
// per-dimension units next to level_kernels_impl.cuh.
#pragma once
#include <chrono>
#include <cstring>
#include <algorithm>
#include <numeric>
#include <cuda_runtime.h>

#include "host.h"
#include "level_kernels.cuh"

namespace hgb {

#define HGB_CUDA(call)                                                             \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      err = std::string("CUDA: ") + #call + ": " + cudaGetErrorString(e_);         \
      if (e_ == cudaErrorMemoryAllocation) {  /* not sticky: the context lives on */ \
        (void)cudaGetLastError();                                                  \
        return HORA_E_NOMEM;                                                       \
      }                                                                            \
      return HORA_E_CUDA;                                                          \
    }                                                                              \
  } while (0)

// A device allocation that frees itself, stream-ordered on the stream it was allocated on (the
// calling thread's g_alloc_stream): work queued on that stream before the free still sees it, and
// freeing synchronises nothing. grow() keeps the first `keep` bytes.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  ~DBuf() { if (p) cudaFreeAsync(p, st); }
  cudaError_t alloc(size_t b) {
    if (p) { cudaFreeAsync(p, st); p = nullptr; }
    bytes = 0;
    st = g_alloc_stream;
    cudaError_t e = cudaMallocAsync(&p, b ? b : 16, st);
    if (e == cudaSuccess) bytes = b;
    else p = nullptr;
    return e;
  }
  cudaError_t grow(size_t b, size_t keep, cudaStream_t s) {
    if (b <= bytes) return cudaSuccess;
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, b, s);
    if (e != cudaSuccess) return e;
    if (p && keep) {
      e = cudaMemcpyAsync(q, p, std::min(keep, bytes), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) { cudaFreeAsync(q, s); return e; }
    }
    if (p) cudaFreeAsync(p, st == s ? s : st);
    p = q;
    st = s;
    bytes = b;
    return cudaSuccess;
  }
  void swap(DBuf& b) { std::swap(p, b.p); std::swap(bytes, b.bytes); std::swap(st, b.st); }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

static __global__ void k_rehash(const unsigned long long* okey, const long long* ooff, const int* olive,
                                unsigned long long ocap, unsigned long long* nkey, long long* noff, int* nlive,
                                unsigned long long nmask, unsigned* err) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ocap;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long k = okey[i];
    if (k == kEmptyKey) continue;
    unsigned long long h = hash_mix(k) & nmask;
    unsigned long long probe = 0;
    for (; probe <= nmask; ++probe) {
      if (atomicCAS(&nkey[h], kEmptyKey, k) == kEmptyKey) { noff[h] = ooff[i]; nlive[h] = olive[i]; break; }
      h = (h + 1) & nmask;
    }
    if (probe > nmask) atomicMax(err, 4u);
  }
}

// CUDA-event timing of each kernel family on the engine's stream. Events are collected after the
// host synchronises for the level's counters, so timing adds no synchronisation of its own.
struct KTimer {
  cudaEvent_t b[8], e[8];
  int kind[8];
  int n = 0;
  double sec[6] = {0, 0, 0, 0, 0, 0};
  unsigned long long calls[6] = {0, 0, 0, 0, 0, 0};
  bool ok = false;
  KTimer() {
    ok = true;
    for (int i = 0; i < 8; ++i) ok &= cudaEventCreate(&b[i]) == cudaSuccess && cudaEventCreate(&e[i]) == cudaSuccess;
  }
  ~KTimer() { for (int i = 0; i < 8; ++i) { cudaEventDestroy(b[i]); cudaEventDestroy(e[i]); } }
  void begin(cudaStream_t s) { if (n < 8) cudaEventRecord(b[n], s); }
  void end(cudaStream_t s, int k, int launches = 1) {
    calls[k] += launches;
    if (n < 8) { cudaEventRecord(e[n], s); kind[n++] = k; }
  }
  void collect() {   // call after the stream has been synchronised
    for (int i = 0; i < n; ++i) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, b[i], e[i]) == cudaSuccess) sec[kind[i]] += ms * 1e-3;
    }
    n = 0;
  }
};
enum { KT_EXPAND = 0, KT_PROBE = 1, KT_DEADLOCK = 2, KT_GROUP = 3, KT_MERGE = 4, KT_OTHER = 5 };

template <int D>
struct StoreBufs {
  DBuf hkey, pend, pend_base, klive, kloff;   // hash table
  DBuf arena;                                 // key lists
  DBuf nzone, ncol0, nlevel, ndead, ninst, nkey, npar, nraw;   // nodes
  unsigned long long hcap = 0;
  long long ncap = 0, acap = 0;
};

// The level-synchronous engine over a group of instances sharing the DBM dimension D. Store 0 is
// the a_LU passed store of reach / deadlock / leads-to phase 1; store 1 is the exact-zone graph of
// leads-to phase 2.
template <int D>
struct Engine {
  static constexpr long long Z2 = (long long)D * D;
  std::vector<const HostNet*> nets;
  int ninst = 0, inst_shift = 63;
  RunOptions o;
  std::string& err;
  cudaStream_t s = nullptr;
  // Destroys the stream after every later member (the device buffers, freed on it) is gone.
  struct StreamEnd {
    cudaStream_t* ps;
    cudaStream_t prev = nullptr;   // the thread's allocation stream before this search
    ~StreamEnd() {
      if (*ps) { cudaStreamSynchronize(*ps); cudaStreamDestroy(*ps); }
      if (*ps && g_alloc_stream == *ps) g_alloc_stream = prev;
    }
  } s_end{&s};
  int blocks = 0;
  DeviceNets dn;
  StoreBufs<D> S[2];
  DBuf skey, sparent, sord, sraw, sflag, spnode, sslot, srank, szone, ssurv, sseg, ssorted, stouched, sokh, sokl, sskh, sskl,
      sheavy, slight, slong;
  long long scap = 0;
  DBuf clist;
  long long ccap = 0;
  DBuf fkey[2], fnode[2], frank[2], finst[2];
  long long fcapb[2] = {0, 0};
  DBuf esrc, edst, eord, eraw;
  long long ecap = 0;
  int merge_blocks = 0;         // resident blocks of the merge kernel (it schedules keys itself)
  int pass_blocks = 0;          // grid of the heavy keys' sort and relation passes (256-thread blocks)
  bool merge_wide = false;      // a single query at D >= 9: the merge runs in 512-thread blocks
  DBuf hv_n, hv_a, hv_cb, hv_bm, hv_bounds, hv_pool, hv_prefix, hv_order;   // keys merged block-wide
  long long hv_cap = 0, pool_cap = 0, prefix_cap = 0;
  std::vector<int> h_hn, h_ha, h_order;
  std::vector<long long> h_hbm, h_prefix;
  DBuf zw;                      // exact-zone table of the graph store
  unsigned long long zcap = 0;
  DBuf ctl, emode, done, found, generated, gen_backup, nlive, nkeys, nfront, probes, hit_node, hit_raw, hit_key,
      hit_zone;
  Ctl hctl{};
  KTimer kt;
  unsigned long long launches = 0, h2d = 0, d2h = 0;
  std::vector<int> h_done, h_emode;
  std::vector<unsigned> h_found;
  std::vector<unsigned long long> h_nfront, h_nkeys, h_gen, explored, levels;
  std::vector<long long> h_nlive;
  std::vector<double> t_fin;   // per instance: seconds from the start to its verdict (-1: not yet)
  std::vector<char> h_budget;  // per instance: stopped because the group's store budget ran out
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_wait = nullptr;   // blocking-sync event (o.yield_wait)
  std::chrono::steady_clock::time_point t_start;

  Engine(const std::vector<const HostNet*>& n, const RunOptions& opt, std::string& e) : nets(n), o(opt), err(e) {}
  ~Engine() {
    if (o.pool && pool_taken) o.pool->give(pool_taken);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev_wait) cudaEventDestroy(ev_wait);
  }

  // Wait until the stream's work is done: spinning (lowest latency) or, when several searches share
  // the host's cores, sleeping on a blocking-sync event so the threads do not take turns on them.
  cudaError_t wait() {
    if (!ev_wait) return cudaStreamSynchronize(s);
    cudaError_t e = cudaEventRecord(ev_wait, s);
    return e == cudaSuccess ? cudaEventSynchronize(ev_wait) : e;
  }

  Store store(int k) {
    StoreBufs<D>& B = S[k];
    Store st;
    st.hkey = B.hkey.template as<unsigned long long>();
    st.pend = B.pend.template as<unsigned>(); st.pend_base = B.pend_base.template as<unsigned>();
    st.klive = B.klive.template as<int>(); st.kloff = B.kloff.template as<long long>();
    st.hmask = B.hcap - 1;
    st.arena = B.arena.template as<int>(); st.acap = B.acap;
    st.nzone = B.nzone.template as<int>(); st.ncol0 = B.ncol0.template as<int>();
    st.nlevel = B.nlevel.template as<int>(); st.ndead = B.ndead.template as<int>(); st.ninst = B.ninst.template as<int>();
    st.nkey = B.nkey.template as<unsigned long long>();
    st.npar = B.npar.template as<int>(); st.nraw = B.nraw.template as<int>();
    return st;
  }
  Succ succ() {
    Succ sc;
    sc.key = skey.template as<unsigned long long>(); sc.parent = sparent.template as<int>();
    sc.ord = sord.template as<int>(); sc.slot = sslot.template as<int>(); sc.rank = srank.template as<int>();
    sc.raw = sraw.template as<int>(); sc.flag = sflag.template as<int>(); sc.pnode = spnode.template as<int>();
    sc.zone = szone.template as<int>(); sc.surv = ssurv.template as<int>(); sc.seg = sseg.template as<int>();
    sc.sorted = ssorted.template as<int>(); sc.touched = stouched.template as<int>(); sc.cap = scap;
    sc.okh = sokh.template as<unsigned long long>(); sc.okl = sokl.template as<unsigned long long>();
    sc.heavy = sheavy.template as<int>(); sc.light = slight.template as<int>(); sc.longs = slong.template as<int>();
    sc.skh = sskh.template as<unsigned long long>(); sc.skl = sskl.template as<unsigned long long>();
    sc.clist = clist.template as<int>(); sc.ccap = ccap;
    sc.hv.n = hv_n.template as<int>(); sc.hv.a = hv_a.template as<int>();
    sc.hv.cb = hv_cb.template as<long long>(); sc.hv.bm = hv_bm.template as<long long>();
    sc.hv.bounds = hv_bounds.template as<int>(); sc.hv.pool = hv_pool.template as<unsigned>();
    return sc;
  }
  Front front(int b) {
    Front f;
    f.key = fkey[b].template as<unsigned long long>(); f.node = fnode[b].template as<int>();
    f.rank = frank[b].template as<int>(); f.inst = finst[b].template as<int>();
    return f;
  }
  Edges edges() {
    return Edges{esrc.template as<int>(), edst.template as<int>(), eord.template as<int>(), ecap, eraw.template as<int>()};
  }
  ZTab ztab() { return ZTab{zw.template as<unsigned long long>(), zcap - 1}; }
  InstState istate() {
    InstState is;
    is.emode = emode.template as<int>(); is.done = done.template as<int>(); is.found = found.template as<unsigned>();
    is.generated = generated.template as<unsigned long long>(); is.nlive = nlive.template as<long long>();
    is.nkeys = nkeys.template as<unsigned long long>(); is.nfront = nfront.template as<unsigned long long>();
    is.probes = probes.template as<unsigned long long>();
    is.hit_node = hit_node.template as<int>(); is.hit_raw = hit_raw.template as<int>();
    is.hit_key = hit_key.template as<unsigned long long>(); is.hit_zone = hit_zone.template as<int>();
    return is;
  }
  Ctl* dctl() { return ctl.template as<Ctl>(); }

  int read_ctl() {
    HGB_CUDA(cudaMemcpyAsync(&hctl, dctl(), sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    d2h += sizeof(Ctl);
    HGB_CUDA(wait());
    kt.collect();
    return HORA_OK;
  }
  int alloc_store(int k, unsigned long long hcap, long long ncap) {
    StoreBufs<D>& B = S[k];
    B.hcap = hcap;
    B.ncap = ncap;
    HGB_CUDA(B.hkey.alloc(hcap * 8)); HGB_CUDA(B.pend.alloc(hcap * 4));
    HGB_CUDA(B.pend_base.alloc(hcap * 4)); HGB_CUDA(B.klive.alloc(hcap * 4)); HGB_CUDA(B.kloff.alloc(hcap * 8));
    HGB_CUDA(cudaMemsetAsync(B.klive.p, 0, hcap * 4, s));
    HGB_CUDA(cudaMemsetAsync(B.hkey.p, 0xff, hcap * 8, s));
    HGB_CUDA(cudaMemsetAsync(B.pend.p, 0, hcap * 4, s));
    B.acap = std::max<long long>(1 << 16, 2 * ncap);
    HGB_CUDA(B.arena.alloc((size_t)B.acap * 4));
    HGB_CUDA(B.nzone.alloc(ncap * Z2 * 4)); HGB_CUDA(B.ncol0.alloc(ncap * D * 4)); HGB_CUDA(B.nlevel.alloc(ncap * 4));
    HGB_CUDA(B.ndead.alloc(ncap * 4)); HGB_CUDA(B.ninst.alloc(ncap * 4)); HGB_CUDA(B.nkey.alloc(ncap * 8));
    HGB_CUDA(B.npar.alloc(ncap * 4)); HGB_CUDA(B.nraw.alloc(ncap * 4));
    return HORA_OK;
  }
  int alloc_succ(long long cap) {
    scap = cap;
    HGB_CUDA(skey.alloc(cap * 8)); HGB_CUDA(sparent.alloc(cap * 4)); HGB_CUDA(sord.alloc(cap * 4));
    HGB_CUDA(sraw.alloc(cap * 4)); HGB_CUDA(sflag.alloc(cap * 4)); HGB_CUDA(spnode.alloc(cap * 4));
    HGB_CUDA(sslot.alloc(cap * 4)); HGB_CUDA(srank.alloc(cap * 4)); HGB_CUDA(szone.alloc(cap * Z2 * 4));
    HGB_CUDA(ssurv.alloc(cap * 4)); HGB_CUDA(sseg.alloc(cap * 4)); HGB_CUDA(ssorted.alloc(cap * 4));
    HGB_CUDA(stouched.alloc(cap * 4));
    HGB_CUDA(sokh.alloc(cap * 8)); HGB_CUDA(sokl.alloc(cap * 8));
    HGB_CUDA(sheavy.alloc(cap * 4)); HGB_CUDA(slight.alloc(cap * 4)); HGB_CUDA(slong.alloc(cap * 4));
    HGB_CUDA(sskh.alloc(cap * 8)); HGB_CUDA(sskl.alloc(cap * 8));
    return HORA_OK;
  }
  int alloc_front(int b, long long cap) {
    fcapb[b] = cap;
    HGB_CUDA(fkey[b].alloc(cap * 8)); HGB_CUDA(fnode[b].alloc(cap * 4));
    HGB_CUDA(frank[b].alloc(cap * 4)); HGB_CUDA(finst[b].alloc(cap * 4));
    return HORA_OK;
  }
  // Room in store k's hash table for `extra` more keys (load factor at most 1/2).
  int ensure_hash(int k, unsigned long long extra) {
    StoreBufs<D>& B = S[k];
    if ((hctl.nslots + extra) * 2 <= B.hcap) return HORA_OK;
    unsigned long long ncap = B.hcap;
    while ((hctl.nslots + extra) * 2 > ncap) ncap <<= 1;
    DBuf k2, o2, p2, pb2, l2;
    HGB_CUDA(k2.alloc(ncap * 8)); HGB_CUDA(o2.alloc(ncap * 8)); HGB_CUDA(p2.alloc(ncap * 4)); HGB_CUDA(pb2.alloc(ncap * 4));
    HGB_CUDA(l2.alloc(ncap * 4));
    HGB_CUDA(cudaMemsetAsync(l2.p, 0, ncap * 4, s));
    HGB_CUDA(cudaMemsetAsync(k2.p, 0xff, ncap * 8, s));
    HGB_CUDA(cudaMemsetAsync(p2.p, 0, ncap * 4, s));
    kt.begin(s);
    k_rehash<<<1024, 256, 0, s>>>(B.hkey.template as<unsigned long long>(), B.kloff.template as<long long>(),
                                 B.klive.template as<int>(), B.hcap, k2.template as<unsigned long long>(),
                                 o2.template as<long long>(), l2.template as<int>(), ncap - 1, &dctl()->err);
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    HGB_CUDA(wait());
    kt.collect();
    B.hkey.swap(k2);
    B.kloff.swap(o2);
    B.pend.swap(p2);
    B.pend_base.swap(pb2);
    B.klive.swap(l2);
    B.hcap = ncap;
    return HORA_OK;
  }
  // Room in store k's key-list arena for `extra` more entries; when full, the live lists are
  // copied into a fresh arena sized for twice the live zones plus the coming survivors.
  int ensure_arena(int k, long long extra) {
    StoreBufs<D>& B = S[k];
    if ((long long)hctl.arena_alloc + extra <= B.acap) return HORA_OK;
    const long long live = std::max<long long>(0, hctl.nlive);
    const long long cap = std::max<long long>(1 << 20, 2 * (live + extra));
    DBuf a2, n2;
    HGB_CUDA(a2.alloc((size_t)cap * 4));
    HGB_CUDA(n2.alloc(8));
    HGB_CUDA(cudaMemsetAsync(n2.p, 0, 8, s));
    kt.begin(s);
    k_arena_compact<<<1024, 256, 0, s>>>(store(k), a2.template as<int>(), cap, n2.template as<unsigned long long>(),
                                        dctl());
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    HGB_CUDA(cudaMemcpyAsync(&dctl()->arena_alloc, n2.p, 8, cudaMemcpyDeviceToDevice, s));
    HGB_CUDA(wait());
    B.arena.swap(a2);
    B.acap = cap;
    const int rc = read_ctl();
    if (rc) return rc;
    if (hctl.err) { err = "key-list arena overflow"; return (int)hctl.err; }
    return HORA_OK;
  }
  // Room in the exact-zone table of store k for `extra` more zones (load factor at most 1/2);
  // a larger table is refilled from the stored nodes.
  int ensure_ztab(int k, long long extra) {
    const unsigned long long need = 2ull * ((unsigned long long)hctl.nnodes + (unsigned long long)extra);
    if (need <= zcap) return HORA_OK;
    unsigned long long c = std::max<unsigned long long>(zcap, 1ull << 16);
    while (c < need) c <<= 1;
    if (c > (1ull << 31)) { err = "exact-zone table beyond 2^31 slots"; return HORA_E_NOMEM; }
    HGB_CUDA(zw.alloc(c * 8));
    HGB_CUDA(cudaMemsetAsync(zw.p, 0, c * 8, s));
    zcap = c;
    kt.begin(s);
    Level<D>::graph_rehash(store(k), (long long)hctl.nnodes, ztab(), dctl(), blocks, s);
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    return HORA_OK;
  }
  // One level of the exact-zone graph: dedup by zone hash, store the new zones, record the edges.
  int graph_level(const NetView* V, int k, int cur, long long nsucc, int level, bool roots) {
    int rc;
    InstState is = istate();
    if ((rc = ensure_ztab(k, nsucc))) return rc;
    if (nsucc > 0) {
      kt.begin(s);
      Level<D>::graph_probe(V, is, succ(), store(k), ztab(), dctl(), nsucc, blocks, s);
      kt.end(s, KT_PROBE);
      ++launches;
      HGB_CUDA(cudaGetLastError());
    }
    if ((rc = read_ctl())) return rc;
    if (hctl.err) { err = "device error in the graph probe"; return (int)hctl.err; }
    const long long nnew = (long long)hctl.nsurv;
    if ((rc = ensure_nodes(k, nnew))) return rc;
    if ((rc = grow_front(cur ^ 1, (long long)hctl.nfront, nnew))) return rc;
    const bool record = !roots;
    if (record && (rc = ensure_edges((long long)hctl.nedges + nsucc))) return rc;
    kt.begin(s);
    if (nnew > 0) {
      Level<D>::graph_store(V, is, succ(), store(k), ztab(), front(cur ^ 1), dctl(), nnew, level, blocks, s);
      ++launches;
    }
    if (record && nsucc > 0) {
      Level<D>::graph_edges(succ(), front(cur), edges(), dctl(), nsucc, s);
      ++launches;
    }
    kt.end(s, KT_MERGE, (nnew > 0 ? 1 : 0) + (record && nsucc > 0 ? 1 : 0));
    HGB_CUDA(cudaGetLastError());
    if ((rc = read_ctl())) return rc;
    if (hctl.err) { err = "device error in the graph store"; return (int)hctl.err; }
    return HORA_OK;
  }
  // One level of the subsumed leads-to graph: inclusion probe against the key's stored zones, the
  // maximal survivors of each key stored, every successor's edge to its covering node.
  int incl_level(const NetView* V, int k, int cur, long long nsucc, int level, bool roots) {
    int rc;
    InstState is = istate();
    if (nsucc > 0) {
      kt.begin(s);
      Level<D>::incl_probe(V, is, succ(), store(k), dctl(), nsucc, blocks, s);
      kt.end(s, KT_PROBE);
      ++launches;
      HGB_CUDA(cudaGetLastError());
    }
    if ((rc = read_ctl())) return rc;
    if (hctl.err) { err = "device error in the inclusion probe"; return (int)hctl.err; }
    const long long nsurv = (long long)hctl.nsurv, ntouched = (long long)hctl.ntouched;
    if ((rc = ensure_nodes(k, nsurv))) return rc;
    if ((rc = ensure_arena(k, std::max<long long>(0, hctl.nlive) + nsurv))) return rc;
    if ((rc = grow_front(cur ^ 1, (long long)hctl.nfront, nsurv))) return rc;
    const bool record = !roots;
    if (record && (rc = ensure_edges((long long)hctl.nedges + nsucc))) return rc;
    if (ntouched > 0) {
      kt.begin(s);
      Level<D>::incl_group(succ(), store(k), dctl(), nsucc, ntouched, s);
      kt.end(s, KT_GROUP, 2);
      kt.begin(s);
      Level<D>::incl_keep(succ(), store(k), dctl(), nsurv, blocks, s);
      Level<D>::incl_store(V, is, succ(), store(k), front(cur ^ 1), dctl(), nsurv, level, blocks, s);
      Level<D>::incl_cover(succ(), store(k), dctl(), nsurv, blocks, s);
      Level<D>::incl_lists(V, is, succ(), store(k), dctl(), ntouched, s);
      kt.end(s, KT_MERGE, 4);
      launches += 6;
      HGB_CUDA(cudaGetLastError());
    }
    if (record && nsucc > 0) {
      kt.begin(s);
      Level<D>::incl_edges(succ(), front(cur), edges(), dctl(), nsucc, s);
      kt.end(s, KT_MERGE);
      ++launches;
      HGB_CUDA(cudaGetLastError());
    }
    if ((rc = read_ctl())) return rc;
    if (hctl.err) { err = "device error in the inclusion store"; return (int)hctl.err; }
    return HORA_OK;
  }
  // The early witness of p --> q on the n phase-1 nodes of frontier b (leadsto_witness,
  // src/liveness/construction.cpp:786-826): an instance whose reachable p-zone, cut to !q, holds a
  // stop valuation is violated and stops.
  int leadsto_witness(int b, long long n) {
    bool any = false;
    for (int q = 0; q < ninst; ++q) any |= nets[q]->kind == HORA_Q_LEADSTO && !h_done[q];
    if (!any || n <= 0) return HORA_OK;
    InstState is = istate();
    Fix fx{};
    kt.begin(s);
    Level<D>::stop_fed(dn.views, is, store(0), 0, n, front(b).node, fx, dctl(), 1, blocks, s);
    kt.end(s, KT_DEADLOCK);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    int rc = read_ctl();
    if (rc) return rc;
    if (hctl.err) { err = "device error in the leads-to witness test"; return (int)hctl.err; }
    const size_t ni4 = (size_t)ninst * 4;
    HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(wait());
    d2h += ni4;
    bool changed = false;
    const double now = elapsed();
    for (int q = 0; q < ninst; ++q)
      if (!h_done[q] && h_found[q]) { h_done[q] = 1; changed = true; if (t_fin[q] < 0) t_fin[q] = now; }
    if (changed) {
      HGB_CUDA(cudaMemcpyAsync(is.done, h_done.data(), ni4, cudaMemcpyHostToDevice, s));
      h2d += ni4;
    }
    return HORA_OK;
  }
  // Bytes one stored node takes (zone, its column 0, level, dead flag, instance, key).
  static constexpr long long kNodeBytes = Z2 * 4 + D * 4 + 20;
  // Nodes the store budget allows (unbounded without a budget).
  long long budget_nodes() const {
    return o.store_budget_bytes ? (long long)((o.store_budget_bytes + pool_taken) / 2 / kNodeBytes) : (1LL << 40);
  }
  uint64_t pool_taken = 0;   // bytes this run took from the server's pool beyond its admission share
  // With a pool, room for `need` nodes is taken from it (at least doubling what the run holds); false
  // when the pool cannot provide it.
  bool grow_budget(long long need) {
    if (!o.pool || !o.store_budget_bytes) return false;
    const uint64_t want_total = (uint64_t)need * 2 * kNodeBytes * 2;
    const uint64_t have = o.store_budget_bytes + pool_taken;
    if (want_total <= have) return true;
    const uint64_t more = std::max<uint64_t>(want_total - have, have);
    if (o.pool->take(more)) { pool_taken += more; return true; }
    if (o.pool->take(want_total - have)) { pool_taken += want_total - have; return true; }
    return false;
  }
  int ensure_nodes(int k, long long extra) {
    StoreBufs<D>& B = S[k];
    const long long need = (long long)hctl.nnodes + extra;
    if (need <= B.ncap) return HORA_OK;
    long long nc = B.ncap;
    while (need > nc) nc *= 2;
    if (nc > budget_nodes()) nc = std::max(need, budget_nodes());   // no doubling past the budget
    const size_t used = hctl.nnodes;
    HGB_CUDA(B.nzone.grow(nc * Z2 * 4, used * Z2 * 4, s));
    HGB_CUDA(B.ncol0.grow(nc * D * 4, used * D * 4, s));
    HGB_CUDA(B.nlevel.grow(nc * 4, used * 4, s));
    HGB_CUDA(B.ndead.grow(nc * 4, used * 4, s));
    HGB_CUDA(B.ninst.grow(nc * 4, used * 4, s));
    HGB_CUDA(B.nkey.grow(nc * 8, used * 8, s));
    HGB_CUDA(B.npar.grow(nc * 4, used * 4, s));
    HGB_CUDA(B.nraw.grow(nc * 4, used * 4, s));
    B.ncap = nc;
    return HORA_OK;
  }
  int ensure_edges(long long need) {
    if (need <= ecap) return HORA_OK;
    long long c = std::max<long long>(ecap, 1 << 16);
    while (c < need) c *= 2;
    const size_t used = (size_t)std::min<unsigned long long>(hctl.nedges, (unsigned long long)ecap);
    HGB_CUDA(esrc.grow(c * 4, used * 4, s));
    HGB_CUDA(edst.grow(c * 4, used * 4, s));
    HGB_CUDA(eord.grow(c * 4, used * 4, s));
    HGB_CUDA(eraw.grow(c * 4, used * 4, s));
    ecap = c;
    return HORA_OK;
  }

  int setup() {
    t_start = o.has_t_call ? o.t_call : std::chrono::steady_clock::now();
    ninst = (int)nets.size();
    int instbits = 0;
    while ((1 << instbits) < ninst) ++instbits;
    inst_shift = 63 - instbits;
    for (int k = 0; k < ninst; ++k)
      if (nets[k]->keybits > inst_shift) { err = "discrete key too wide for the batch"; return HORA_E_NOT_SUPPORTED; }
    HGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    s_end.prev = g_alloc_stream;
    g_alloc_stream = s;   // this search's buffers are allocated and freed on its stream
    prepare_device_pool();
    if (o.yield_wait) HGB_CUDA(cudaEventCreateWithFlags(&ev_wait, cudaEventBlockingSync | cudaEventDisableTiming));
    int dev = 0, nsm = 0;
    HGB_CUDA(cudaGetDevice(&dev));
    HGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    blocks = o.blocks > 0 ? o.blocks : nsm * std::max(1, o.blocks_per_sm);
    merge_wide = ninst == 1 && Level<D>::merge_wide_pays();
    merge_blocks = nsm * std::max(1, Level<D>::merge_blocks_per_sm(merge_wide));
    pass_blocks = nsm * 2;
    int rc = upload_nets(nets, inst_shift, dn, err);
    if (rc) return rc;
    for (size_t k = 0; k < dn.blob_bytes.size(); ++k) h2d += dn.blob_bytes[k];
    h2d += sizeof(NetView) * (size_t)ninst;
    unsigned long long hcap = 1ull << 16;
    while (hcap < 4ull * ninst) hcap <<= 1;
    if ((rc = alloc_store(0, hcap, std::max<long long>(1 << 14, 2LL * ninst)))) return rc;
    if ((rc = alloc_succ((long long)std::max<size_t>(o.succ_cap0, 4 * (size_t)ninst)))) return rc;
    for (int b = 0; b < 2; ++b)
      if ((rc = alloc_front(b, std::max<long long>(1 << 14, 2LL * ninst)))) return rc;
    HGB_CUDA(ctl.alloc(sizeof(Ctl)));
    HGB_CUDA(cudaMemsetAsync(ctl.p, 0, sizeof(Ctl), s));
    const size_t ni4 = (size_t)ninst * 4, ni8 = (size_t)ninst * 8;
    HGB_CUDA(emode.alloc(ni4)); HGB_CUDA(done.alloc(ni4)); HGB_CUDA(found.alloc(ni4));
    HGB_CUDA(generated.alloc(ni8)); HGB_CUDA(gen_backup.alloc(ni8)); HGB_CUDA(nlive.alloc(ni8));
    HGB_CUDA(nkeys.alloc(ni8)); HGB_CUDA(nfront.alloc(ni8)); HGB_CUDA(probes.alloc(ni8));
    for (DBuf* b : {&emode, &done, &found, &generated, &nlive, &nkeys, &nfront, &probes})
      HGB_CUDA(cudaMemsetAsync(b->p, 0, b->bytes, s));
    HGB_CUDA(hit_node.alloc(ni4)); HGB_CUDA(hit_raw.alloc(ni4)); HGB_CUDA(hit_key.alloc(ni8));
    HGB_CUDA(hit_zone.alloc((size_t)ninst * Z2 * 4));
    HGB_CUDA(cudaMemsetAsync(hit_node.p, 0xff, ni4, s));   // -1: no goal state yet
    h_done.assign(ninst, 0); h_emode.assign(ninst, 0); h_found.assign(ninst, 0);
    h_nfront.assign(ninst, 0); h_nkeys.assign(ninst, 0); h_gen.assign(ninst, 0);
    h_nlive.assign(ninst, 0); explored.assign(ninst, 0); levels.assign(ninst, 0);
    t_fin.assign(ninst, -1.0);
    h_budget.assign(ninst, 0);
    HGB_CUDA(cudaEventCreate(&ev0));
    HGB_CUDA(cudaEventCreate(&ev1));
    HGB_CUDA(cudaEventRecord(ev0, s));
    return HORA_OK;
  }

  // Level 0 of store 0: every instance's initial state. Returns the frontier size in *nf.
  // Level 0 of store 0. For E[] psi the initial state is the psi-restricted network's (it becomes
  // the graph's root); otherwise the unrestricted network's.
  int init(long long* nf) {
    InstState is = istate();
    const bool eg = !nets.empty() && nets[0]->kind == HORA_Q_EG;
    kt.begin(s);
    Level<D>::init(eg ? dn.views : dn.views_plain, ninst, dn.ok, store(0), front(0), is, dctl(), s);
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    int rc = read_ctl();
    if (rc) return rc;
    if (hctl.err) { err = "device error in init"; return (int)hctl.err; }
    HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, (size_t)ninst * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_done.data(), is.done, (size_t)ninst * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(wait());
    *nf = (long long)hctl.nfront;
    return HORA_OK;
  }

  // BFS on store k from frontier buffer `cur` until it empties.
  //  mode 0: a_LU subsumption store with the reach / deadlock goals and the adaptive Extra_LU+;
  //  mode 1: exact-zone graph store recording edges. With roots_src set, the first step turns the
  //          frontier's store-0 zones into the graph's level-0 roots instead of expanding them.
  int run_levels(int k, int mode, int& cur, long long nf, int& level, const int* roots_src) {
    const size_t ni4 = (size_t)ninst * 4, ni8 = (size_t)ninst * 8;
    InstState is = istate();
    int rc;
    bool roots = roots_src != nullptr;
    const NetView* V = k == 0 ? dn.views_plain : dn.views;   // the !q restriction is for the graph only
    while (nf > 0) {
      if (o.cancel && *o.cancel) return HORA_E_CANCELLED;
      if (!roots) ++level;
      HGB_CUDA(cudaMemcpyAsync(h_nfront.data(), is.nfront, ni8, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemsetAsync(is.nfront, 0, ni8, s));
      HGB_CUDA(cudaMemsetAsync(&dctl()->nfront, 0, 8, s));
      HGB_CUDA(wait());
      if (!roots)
        for (int q = 0; q < ninst; ++q)
          if (!h_done[q] && h_nfront[q]) { explored[q] += h_nfront[q]; levels[q] = level; }
      if (mode == 0) {
        // a forward search whose frontier ran dry has its verdict: record when
        const double now = elapsed();
        for (int q = 0; q < ninst; ++q)
          if (!h_done[q] && !h_nfront[q] && t_fin[q] < 0 && nets[q]->kind != HORA_Q_LEADSTO) t_fin[q] = now;
      }
      // ---- the level in chunks of whole instances, so that one chunk's successors fit the budget;
      // an instance's level is never split, so its canonical insertion order is kept
      std::vector<int> cuts{0};
      {
        const double fan = std::max(8.0, 2.0 * (double)gen_total / (double)std::max<unsigned long long>(1, exp_total));
        const double budget = (double)o.succ_budget_bytes / (double)(Z2 * 4 + 96);
        double acc = 0;
        for (int q = 0; q < ninst; ++q) {
          const double e = (double)h_nfront[q] * fan;
          if (acc > 0 && acc + e > budget) { cuts.push_back(q); acc = 0; }
          acc += e;
        }
        cuts.push_back(ninst);
      }
      for (size_t c = 0; c + 1 < cuts.size(); ++c)
        if ((rc = run_chunk(k, mode, cur, nf, level, roots, roots_src, V, cuts[c], cuts[c + 1]))) return rc;
      // ---- end of level: goals and the adaptive extrapolation (store 0 only)
      if (mode == 0 && (rc = leadsto_witness(cur ^ 1, (long long)hctl.nfront))) return rc;
      if (mode == 0) {
        HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
        HGB_CUDA(cudaMemcpyAsync(h_nlive.data(), is.nlive, ni8, cudaMemcpyDeviceToHost, s));
        HGB_CUDA(cudaMemcpyAsync(h_nkeys.data(), is.nkeys, ni8, cudaMemcpyDeviceToHost, s));
        HGB_CUDA(wait());
        bool changed = false;
        const double now = elapsed();
        for (int q = 0; q < ninst; ++q) {
          if (h_done[q]) continue;
          if (h_found[q]) {
            h_done[q] = 1;
            changed = true;
            if (t_fin[q] < 0 && nets[q]->kind != HORA_Q_LEADSTO) t_fin[q] = now;
            continue;
          }
          // adaptive switch to Extra_LU+ (src/reachability/engine.cpp:2178-2184)
          if (h_emode[q] == 0 && h_nkeys[q] && (double)h_nlive[q] >= 4.0 * (double)h_nkeys[q]) { h_emode[q] = 1; changed = true; }
        }
        if (changed) {
          HGB_CUDA(cudaMemcpyAsync(is.done, h_done.data(), ni4, cudaMemcpyHostToDevice, s));
          HGB_CUDA(cudaMemcpyAsync(is.emode, h_emode.data(), ni4, cudaMemcpyHostToDevice, s));
          h2d += 2 * ni4;
        }
      }
      if ((rc = read_ctl())) return rc;
      if (o.store_budget_bytes && (rc = enforce_budget(mode))) return rc;
      nf = (long long)hctl.nfront;
      cur ^= 1;
      roots = false;
    }
    return HORA_OK;
  }
  unsigned long long gen_total = 0, exp_total = 0;   // successors / expanded states so far (fan-out)
  unsigned long long merge_surv = 0;                 // survivors handed to the merge (store 0)
  double last_fan = 0;                               // successors per frontier state, recent levels

  // The group's store may hold about store_budget_bytes (plus what it took from a server's pool): in a
  // group of several instances one past a quarter of it stops, and once the store is past it every
  // instance still running stops (status HORA_E_BUDGET, no verdict). The store grows by at most one
  // level past the check.
  int enforce_budget(int mode) {
    const size_t ni4 = (size_t)ninst * 4, ni8 = (size_t)ninst * 8;
    InstState is = istate();
    if (mode >= 1) {
      HGB_CUDA(cudaMemcpyAsync(h_nlive.data(), is.nlive, ni8, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(wait());
    }
    if (o.pool && (double)hctl.nnodes > (double)budget_nodes()) grow_budget((long long)hctl.nnodes);
    const double allowed = (double)budget_nodes();
    const bool all = (double)hctl.nnodes > allowed;
    // with a pool the group grows while the pool has room, so no instance is held to a fixed quarter
    const bool quarter = ninst > 1 && !o.pool;
    bool changed = false;
    for (int q = 0; q < ninst; ++q) {
      if (h_done[q]) continue;
      if (all || (quarter && (double)h_nlive[q] > allowed / 4)) { h_done[q] = 1; h_budget[q] = 1; changed = true; }
    }
    if (changed) {
      HGB_CUDA(cudaMemcpyAsync(is.done, h_done.data(), ni4, cudaMemcpyHostToDevice, s));
      h2d += ni4;
    }
    return HORA_OK;
  }

  // Room for `extra` more entries in frontier buffer b, keeping the `used` ones already there.
  int grow_front(int b, long long used, long long extra) {
    if (used + extra <= fcapb[b]) return HORA_OK;
    long long fc = std::max<long long>(fcapb[b], 1 << 14);
    while (used + extra > fc) fc *= 2;
    HGB_CUDA(fkey[b].grow(fc * 8, used * 8, s)); HGB_CUDA(fnode[b].grow(fc * 4, used * 4, s));
    HGB_CUDA(frank[b].grow(fc * 4, used * 4, s)); HGB_CUDA(finst[b].grow(fc * 4, used * 4, s));
    fcapb[b] = fc;
    return HORA_OK;
  }

  // Keys merged block-wide: sort and gather them, then precompute their pairwise relations.
  int heavy_relations(const NetView* V, int k) {
    const long long nh = (long long)hctl.nheavy;
    if (nh == 0) return HORA_OK;
    InstState is = istate();
    const long long need = (long long)hctl.bm_need;
    if (need > pool_cap) {
      long long c = std::max<long long>(pool_cap, 1 << 20);
      while (c < need) c *= 2;
      HGB_CUDA(hv_pool.alloc((size_t)c * 4));
      pool_cap = c;
    }
    h_hn.resize(nh); h_ha.resize(nh); h_hbm.resize(nh); h_prefix.resize(nh + 1);
    HGB_CUDA(cudaMemcpyAsync(h_hn.data(), hv_n.p, nh * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_ha.data(), hv_a.p, nh * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_hbm.data(), hv_bm.p, nh * 8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(wait());
    // Largest keys first: a key's ordered fold is serial, so the level's merge ends no earlier than
    // its longest key; started first, it runs alongside all the others.
    h_order.resize(nh);
    for (long long j = 0; j < nh; ++j) h_order[j] = (int)j;
    std::stable_sort(h_order.begin(), h_order.end(), [&](int x, int y) {
      return h_hn[x] != h_hn[y] ? h_hn[x] > h_hn[y] : h_ha[x] > h_ha[y];
    });
    HGB_CUDA(cudaMemcpyAsync(hv_order.p, h_order.data(), nh * 4, cudaMemcpyHostToDevice, s));
    h2d += nh * 4;
    kt.begin(s);
    Level<D>::heavy_prep(V, is, succ(), store(k), dctl(), nh, pass_blocks, hv_order.template as<int>(), s);
    kt.end(s, KT_MERGE);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    HGB_CUDA(wait());
    d2h += nh * 16;
    // tiles of 32 x 32 pairs: survivors x earlier survivors, survivors x old zones
    long long tot = 0;
    for (long long j = 0; j < nh; ++j) {
      h_prefix[j] = tot;
      if (h_hbm[j] < 0) continue;
      const long long bq = (h_hn[j] + 31) / 32, ba = (h_ha[j] + 31) / 32;
      tot += bq * (bq + 1) / 2 + bq * ba;
    }
    h_prefix[nh] = tot;
    if (tot > 0) {
      if (nh + 1 > prefix_cap) {
        long long c = std::max<long long>(prefix_cap, 1 << 12);
        while (c < nh + 1) c *= 2;
        HGB_CUDA(hv_prefix.alloc(c * 8));
        prefix_cap = c;
      }
      HGB_CUDA(cudaMemcpyAsync(hv_prefix.p, h_prefix.data(), (nh + 1) * 8, cudaMemcpyHostToDevice, s));
      h2d += (nh + 1) * 8;
      kt.begin(s);
      if (Level<D>::heavy_pairs(V, succ(), store(k), hv_prefix.template as<long long>(), nh, tot, pass_blocks * 4, s)) {
        err = "cannot size the relation pass's shared memory";
        return HORA_E_CUDA;
      }
      kt.end(s, KT_MERGE);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      HGB_CUDA(wait());   // the prefix buffer is host memory
    }
    return HORA_OK;
  }

  // One chunk of a level: the frontier entries of instances [i0, i1).
  int run_chunk(int k, int mode, int cur, long long nf, int level, bool roots, const int* roots_src,
                const NetView* V, int i0, int i1) {
    const size_t ni8 = (size_t)ninst * 8;
    InstState is = istate();
    int rc;
    // ---- expand; re-run with a larger buffer on overflow (it writes nothing persistent). The buffer
    // is first sized for the chunk's frontier at the last level's fan-out.
    const int* src = roots ? roots_src : S[k].nzone.template as<int>();
    if (!roots && last_fan > 0) {
      unsigned long long nfc = 0;
      for (int q = i0; q < i1; ++q) nfc += h_nfront[q];
      const long long want = (long long)((double)nfc * last_fan * 1.15) + 1024;
      if (want > scap && (rc = alloc_succ(want))) return rc;
    }
    for (;;) {
      HGB_CUDA(cudaMemsetAsync(dctl(), 0, kCtlChunkBytes, s));
      HGB_CUDA(cudaMemcpyAsync(gen_backup.p, is.generated, ni8, cudaMemcpyDeviceToDevice, s));
      kt.begin(s);
      Level<D>::expand(V, is, front(cur), (int)nf, src, succ(), dctl(), roots ? 1 : 0, i0, i1, blocks, s);
      kt.end(s, KT_EXPAND);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      if ((rc = read_ctl())) return rc;
      if (!hctl.overflow) break;
      HGB_CUDA(cudaMemcpyAsync(is.generated, gen_backup.p, ni8, cudaMemcpyDeviceToDevice, s));
      if ((rc = alloc_succ((long long)(hctl.nsucc + hctl.nsucc / 4 + 1024)))) return rc;
    }
    if (hctl.err) { err = "device error in expand"; return (int)hctl.err; }
    const long long nsucc = (long long)hctl.nsucc;
    if (!roots) {
      unsigned long long nfc = 0;
      for (int q = i0; q < i1; ++q) nfc += h_nfront[q];
      gen_total += (unsigned long long)nsucc;
      exp_total += nfc;
      if (nfc) last_fan = std::max(last_fan * 0.5, (double)nsucc / (double)nfc);
    }
    if ((rc = ensure_hash(k, (unsigned long long)nsucc))) return rc;
    if (mode == 1) return graph_level(V, k, cur, nsucc, level, roots);   // exact-zone graph
    if (mode == 2) return incl_level(V, k, cur, nsucc, level, roots);    // subsumed leads-to graph
    // ---- deadlock goal, on every successor before the probe: a successor the probe would drop lies
    // in a_M of a stored zone, whose valuations were all tested, and a_M is a bisimulation, so the
    // verdict and its level are those of testing the survivors only; an instance found here skips
    // the probe and merge of this level
    bool any_dl = false;
    for (int q = i0; q < i1; ++q) any_dl |= (nets[q]->kind == HORA_Q_DEADLOCK && !h_done[q]);
    if (any_dl && nsucc > 0) {
      kt.begin(s);
      Level<D>::deadlock(V, is, succ(), dctl(), nsucc, 1, blocks, s);
      kt.end(s, KT_DEADLOCK);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      if ((rc = read_ctl())) return rc;
      if (hctl.err) { err = "deadlock test exceeded its escape table"; return (int)hctl.err; }
    }
    // ---- probe
    if (nsucc > 0) {
      HGB_CUDA(cudaMemsetAsync(&dctl()->nlong, 0, 8, s));
      kt.begin(s);
      Level<D>::probe(V, is, succ(), store(k), dctl(), nsucc, o.long_list, blocks, s);
      Level<D>::probe_long(V, is, succ(), store(k), dctl(), blocks, s);   // reads the count on the device
      kt.end(s, KT_PROBE, 2);
      launches += 2;
      HGB_CUDA(cudaGetLastError());
    }
    if ((rc = read_ctl())) return rc;
    if (hctl.err) { err = "device error in probe"; return (int)hctl.err; }
    const long long nsurv = (long long)hctl.nsurv, ntouched = (long long)hctl.ntouched;
    merge_surv += (unsigned long long)nsurv;
    if (ntouched > hv_cap) {   // per-key arrays of the grouping pass
      long long c = std::max<long long>(hv_cap, 1 << 12);
      while (c < ntouched) c *= 2;
      HGB_CUDA(hv_n.alloc(c * 4)); HGB_CUDA(hv_a.alloc(c * 4)); HGB_CUDA(hv_cb.alloc(c * 8));
      HGB_CUDA(hv_order.alloc(c * 4));
      HGB_CUDA(hv_bm.alloc(c * 8)); HGB_CUDA(hv_bounds.alloc(c * 2 * D * 4));
      hv_cap = c;
    }
    // ---- room for the new nodes, their key lists and the next frontier; a chunk that would take
    // the store past its budget stops its instances instead (HORA_E_BUDGET)
    if (o.store_budget_bytes && (long long)hctl.nnodes + nsurv > budget_nodes() &&
        !grow_budget((long long)hctl.nnodes + nsurv)) {
      bool changed = false;
      for (int q = i0; q < i1; ++q)
        if (!h_done[q]) { h_done[q] = 1; h_budget[q] = 1; changed = true; }
      if (changed) {
        HGB_CUDA(cudaMemcpyAsync(is.done, h_done.data(), (size_t)ninst * 4, cudaMemcpyHostToDevice, s));
        h2d += (size_t)ninst * 4;
      }
      // their pending survivors are dropped: the merge skips finished instances and resets the slots
      if (ntouched > 0) {
        kt.begin(s);
        Level<D>::group(succ(), store(k), dctl(), nsucc, ntouched, s);
        kt.end(s, KT_GROUP, 2);
        Level<D>::merge(V, is, succ(), store(k), front(cur ^ 1), dctl(), ntouched, level, merge_blocks, merge_wide,
                        nullptr, s);
        launches += 3;
        HGB_CUDA(cudaGetLastError());
      }
      return read_ctl();
    }
    if ((rc = ensure_nodes(k, nsurv))) return rc;
    if ((rc = ensure_arena(k, std::max<long long>(0, hctl.nlive) + nsurv))) return rc;
    if ((rc = grow_front(cur ^ 1, (long long)hctl.nfront, nsurv))) return rc;
    const long long clneed = std::max<long long>(0, hctl.nlive) + nsurv;   // touched keys' lists + survivors
    if (clneed > ccap) {
      long long c = std::max<long long>(ccap, 1 << 16);
      while (clneed > c) c *= 2;
      HGB_CUDA(clist.alloc(c * 4));
      ccap = c;
    }
    // ---- group + merge
    if (ntouched > 0) {
      kt.begin(s);
      Level<D>::group(succ(), store(k), dctl(), nsucc, ntouched, s);
      kt.end(s, KT_GROUP, 2);
      launches += 2;
      HGB_CUDA(cudaGetLastError());
      if ((rc = read_ctl())) return rc;
      if ((rc = heavy_relations(V, k))) return rc;
      kt.begin(s);
      Level<D>::merge(V, is, succ(), store(k), front(cur ^ 1), dctl(), ntouched, level, merge_blocks, merge_wide,
                      hctl.nheavy ? hv_order.template as<int>() : nullptr, s);
      kt.end(s, KT_MERGE);
      launches += 1;
      HGB_CUDA(cudaGetLastError());
    }
    if ((rc = read_ctl())) return rc;
    if (hctl.err) { err = "device error in merge"; return (int)hctl.err; }
    return HORA_OK;
  }

  // Leads-to after phase 1: roots, the !q graph, stop sets and the greatest fixpoint -- the subsumed
  // graph with the federation sweep for p --> q, the exact-zone graph with node flags for E[] psi.
  int leadsto_phase2(int& cur) {
    int rc;
    InstState is = istate();
    const bool eg = nets[0]->kind == HORA_Q_EG;
    const long long n1 = (long long)hctl.nnodes;
    // counters of store 1 start from zero; phase 1's stay in the per-instance totals
    HGB_CUDA(cudaMemsetAsync(&dctl()->nnodes, 0, 8, s));
    HGB_CUDA(cudaMemsetAsync(&dctl()->nkeys, 0, 8, s));
    HGB_CUDA(cudaMemsetAsync(&dctl()->nslots, 0, 8, s));
    HGB_CUDA(cudaMemsetAsync(&dctl()->nlive, 0, 8, s));
    HGB_CUDA(cudaMemsetAsync(&dctl()->arena_alloc, 0, 8, s));
    HGB_CUDA(cudaMemsetAsync(is.nlive, 0, (size_t)ninst * 8, s));
    HGB_CUDA(cudaMemsetAsync(is.nkeys, 0, (size_t)ninst * 8, s));
    HGB_CUDA(cudaMemsetAsync(is.nfront, 0, (size_t)ninst * 8, s));
    std::vector<int> one(ninst, 1);
    HGB_CUDA(cudaMemcpyAsync(is.emode, one.data(), (size_t)ninst * 4, cudaMemcpyHostToDevice, s));
    for (int q = 0; q < ninst; ++q) h_emode[q] = 1;
    unsigned long long hcap = 1ull << 16;
    if ((rc = alloc_store(1, hcap, std::max<long long>(1 << 14, 2LL * ninst)))) return rc;
    // the p-nodes of phase 1 as a frontier
    if (n1 > fcapb[cur]) { if ((rc = alloc_front(cur, n1))) return rc; }
    HGB_CUDA(cudaMemsetAsync(dctl(), 0, kCtlChunkBytes, s));
    HGB_CUDA(cudaMemsetAsync(&dctl()->nfront, 0, 8, s));
    kt.begin(s);
    Level<D>::collect_p(dn.views_plain, store(0), n1, front(cur), dctl(), s);
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    if ((rc = read_ctl())) return rc;
    long long nf = (long long)hctl.nfront;
    int level = 0;
    // the reported level count is the graph's: per instance, its last level with a frontier
    for (int q = 0; q < ninst; ++q)
      if (!h_done[q]) levels[q] = 0;   // an instance decided in phase 1 keeps its level count
    if ((rc = run_levels(1, eg ? 1 : 2, cur, nf, level, S[0].nzone.template as<int>()))) return rc;
    if (!eg) return fed_sweep();
    // stop flags and the sweep
    const long long n2 = (long long)hctl.nnodes, ne = (long long)hctl.nedges;
    DBuf stop, W, F;
    HGB_CUDA(stop.alloc((size_t)std::max<long long>(n2, 1) * 4));
    HGB_CUDA(W.alloc((size_t)std::max<long long>(n2, 1) * 4));
    HGB_CUDA(F.alloc((size_t)std::max<long long>(n2, 1) * 4));
    HGB_CUDA(cudaMemsetAsync(stop.p, 0, stop.bytes, s));
    HGB_CUDA(cudaMemsetAsync(F.p, 0, F.bytes, s));
    std::vector<int> ones((size_t)std::max<long long>(n2, 1), 1);
    HGB_CUDA(cudaMemcpyAsync(W.p, ones.data(), (size_t)std::max<long long>(n2, 1) * 4, cudaMemcpyHostToDevice, s));
    if (n2 > 0) {
      kt.begin(s);
      Level<D>::stop(dn.views, store(1), n2, stop.template as<int>(), dctl(), blocks, s);
      kt.end(s, KT_DEADLOCK);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      if ((rc = read_ctl())) return rc;
      if (hctl.err) { err = "stop-set test exceeded its escape table"; return (int)hctl.err; }
    }
    unsigned long long iters = 0;
    for (long long guard = 0; guard <= n2 + 1; ++guard) {
      HGB_CUDA(cudaMemsetAsync(&dctl()->flag, 0, 4, s));
      kt.begin(s);
      Level<D>::gfp_pass(edges(), ne, n2, stop.template as<int>(), W.template as<int>(), F.template as<int>(), dctl(), s);
      kt.end(s, KT_MERGE, 2);
      launches += 2;
      ++iters;
      HGB_CUDA(cudaGetLastError());
      if ((rc = read_ctl())) return rc;
      if (!hctl.flag) break;
    }
    HGB_CUDA(cudaMemsetAsync(is.found, 0, (size_t)ninst * 4, s));
    kt.begin(s);
    Level<D>::gfp_verdict(dn.views, store(1), n2, W.template as<int>(), is, dctl(), s);
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    if ((rc = read_ctl())) return rc;
    gfp_iters = iters;
    pre_calls = (unsigned long long)ne;
    if (o.trace && ninst == 1 && nets[0]->kind == HORA_Q_EG)
      return extract_trace(n2, ne, W.template as<int>(), stop.template as<int>());
    return HORA_OK;
  }

  // The federation sweep of p --> q over the subsumed graph: stop sets, the edges by source, then
  // Jacobi rounds of W = W /\ (Stop \/ Pre(W)) over the nodes whose successors changed, until nothing
  // changes or every root is empty. A federation that outgrows its K zones restarts the sweep with
  // twice the room (up to kFedMax; past it the query reports HORA_E_OVERFLOW, the reference's
  // capped fixpoint).
  int fed_sweep() {
    int rc;
    InstState is = istate();
    const long long n2 = (long long)hctl.nnodes, ne = (long long)hctl.nedges;
    const Store st = store(1);
    const Edges ed = edges();
    // stop sets, re-run with a larger piece arena if they overflow it
    DBuf swhole, shead, snext, spiece, eoff, eidx, tmp, woff, wcnt, woff2, wcnt2, warena, dirty, dlist, chg, clst, scratch;
    const long long nn = std::max<long long>(n2, 1);
    HGB_CUDA(swhole.alloc(nn * 4)); HGB_CUDA(shead.alloc(nn * 4));
    Fix fx{};
    fx.swhole = swhole.template as<int>(); fx.shead = shead.template as<int>();
    long long scap = std::max<long long>(1 << 14, n2 / 4);
    for (;;) {
      HGB_CUDA(snext.alloc(scap * 4)); HGB_CUDA(spiece.alloc(scap * Z2 * 4));
      fx.snext = snext.template as<int>(); fx.spiece = spiece.template as<int>(); fx.scap = scap;
      HGB_CUDA(cudaMemsetAsync(&dctl()->spieces, 0, 8, s));
      HGB_CUDA(cudaMemsetAsync(&dctl()->stop_over, 0, 4, s));
      kt.begin(s);
      Level<D>::stop_fed(dn.views, is, st, 0, n2, nullptr, fx, dctl(), 0, blocks, s);
      kt.end(s, KT_DEADLOCK);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      if ((rc = read_ctl())) return rc;
      if (hctl.err) { err = "stop-set test exceeded its escape table"; return (int)hctl.err; }
      if (!hctl.stop_over) break;
      scap = 2 * (long long)hctl.spieces + 1024;
    }
    // edges by source
    const long long nb = (n2 + 1 + 1023) / 1024;
    HGB_CUDA(eoff.alloc((size_t)(n2 + 1) * 4)); HGB_CUDA(eidx.alloc((size_t)std::max<long long>(ne, 1) * 4));
    HGB_CUDA(tmp.alloc((size_t)std::max(nn, nb) * 4));
    HGB_CUDA(cudaMemsetAsync(eoff.p, 0, (size_t)(n2 + 1) * 4, s));
    kt.begin(s);
    Level<D>::edge_csr(ed, ne, n2, eoff.template as<int>(), eidx.template as<int>(), tmp.template as<int>(), s);
    kt.end(s, KT_OTHER, 5);
    launches += 5;
    HGB_CUDA(cudaGetLastError());
    fx.eoff = eoff.template as<int>(); fx.eidx = eidx.template as<int>();
    HGB_CUDA(woff.alloc(nn * 8)); HGB_CUDA(wcnt.alloc(nn * 4)); HGB_CUDA(woff2.alloc(nn * 8)); HGB_CUDA(wcnt2.alloc(nn * 4));
    HGB_CUDA(dirty.alloc(nn * 4)); HGB_CUDA(dlist.alloc(nn * 4)); HGB_CUDA(chg.alloc(nn * 4)); HGB_CUDA(clst.alloc(nn * 4));
    fx.woff = woff.template as<long long>(); fx.wcnt = wcnt.template as<int>();
    fx.woff2 = woff2.template as<long long>(); fx.wcnt2 = wcnt2.template as<int>();
    fx.dirty = dirty.template as<int>(); fx.dlist = dlist.template as<int>();
    fx.changed = chg.template as<int>(); fx.clist = clst.template as<int>();
    fx.ntiles = Level<D>::relax_tiles(blocks);
    unsigned long long rounds = 0, npre = 0;
    for (int K = 16;; K *= 2) {
      fx.K = K;
      HGB_CUDA(scratch.alloc((size_t)fx.ntiles * K * Z2 * 4));
      fx.scratch = scratch.template as<int>();
      long long wcap = std::max<long long>(1 << 16, 4 * n2);
      HGB_CUDA(warena.alloc((size_t)wcap * Z2 * 4));
      fx.warena = warena.template as<int>(); fx.wcap = wcap;
      kt.begin(s);
      Level<D>::gfp_init(fx, n2, dctl(), s);
      kt.end(s, KT_OTHER);
      ++launches;
      HGB_CUDA(cudaMemsetAsync(&dctl()->walloc, 0, 8, s));
      HGB_CUDA(cudaMemsetAsync(&dctl()->fed_over, 0, 4, s));
      long long ndirty = n2, live_roots = 1;
      while (ndirty > 0 && live_roots > 0) {
        if (o.cancel && *o.cancel) return HORA_E_CANCELLED;
        // room in the arena for this round's new values; otherwise copy the live values into a
        // fresh arena sized for them and the round
        if ((long long)hctl.walloc + ndirty * K > wcap) {
          const long long cap2 = std::max<long long>(wcap, 4 * ndirty * (long long)K);
          DBuf a2, na;
          HGB_CUDA(a2.alloc((size_t)cap2 * Z2 * 4)); HGB_CUDA(na.alloc(8));
          HGB_CUDA(cudaMemsetAsync(na.p, 0, 8, s));
          kt.begin(s);
          Level<D>::gfp_compact(fx, n2, a2.template as<int>(), na.template as<unsigned long long>(), s);
          kt.end(s, KT_OTHER);
          ++launches;
          HGB_CUDA(cudaMemcpyAsync(&dctl()->walloc, na.p, 8, cudaMemcpyDeviceToDevice, s));
          warena.swap(a2);
          wcap = cap2;
          fx.warena = warena.template as<int>(); fx.wcap = wcap;
          if ((rc = read_ctl())) return rc;
          if ((long long)hctl.walloc + ndirty * K > wcap) {   // still short: grow once more
            const long long cap3 = 2 * ((long long)hctl.walloc + ndirty * K);
            DBuf a3, nb3;
            HGB_CUDA(a3.alloc((size_t)cap3 * Z2 * 4)); HGB_CUDA(nb3.alloc(8));
            HGB_CUDA(cudaMemsetAsync(nb3.p, 0, 8, s));
            Level<D>::gfp_compact(fx, n2, a3.template as<int>(), nb3.template as<unsigned long long>(), s);
            ++launches;
            HGB_CUDA(cudaMemcpyAsync(&dctl()->walloc, nb3.p, 8, cudaMemcpyDeviceToDevice, s));
            warena.swap(a3);
            wcap = cap3;
            fx.warena = warena.template as<int>(); fx.wcap = wcap;
          }
        }
        HGB_CUDA(cudaMemsetAsync(&dctl()->nchanged, 0, 8, s));
        kt.begin(s);
        Level<D>::gfp_relax(dn.views, st, ed, fx, dctl(), ndirty, blocks, s);
        kt.end(s, KT_MERGE);
        kt.begin(s);
        Level<D>::gfp_round_end(ed, ne, n2, fx, S[1].nlevel.template as<int>(), dctl(), s);
        kt.end(s, KT_OTHER, 3);
        launches += 4;
        ++rounds;
        HGB_CUDA(cudaGetLastError());
        if ((rc = read_ctl())) return rc;
        if (hctl.err) { err = "device error in the federation sweep"; return (int)hctl.err; }
        if (hctl.fed_over) break;
        ndirty = (long long)hctl.ndirty;
        live_roots = (long long)hctl.nroots_live;
        if (rounds > 1000000ull) { err = "federation sweep did not settle"; return HORA_E_OVERFLOW; }
      }
      npre += hctl.npre;
      if (!hctl.fed_over) break;
      if (2 * K > kFedMax) { err = "a federation of the sweep outgrew its capacity"; return HORA_E_OVERFLOW; }
      HGB_CUDA(cudaMemsetAsync(&dctl()->npre, 0, 8, s));
    }
    // instances found by the phase-1 witness keep their flag: they have no roots here
    kt.begin(s);
    Level<D>::gfp_verdict_fed(dn.views, st, n2, fx, is, s);
    kt.end(s, KT_OTHER);
    ++launches;
    HGB_CUDA(cudaGetLastError());
    if ((rc = read_ctl())) return rc;
    gfp_iters = rounds;
    pre_calls = npre;
    if (o.trace && ninst == 1 && nets[0]->kind == HORA_Q_LEADSTO) return sweep_trace(n2, ne, fx);
    return HORA_OK;
  }

  // Counterexample of p --> q decided by the sweep: a root whose W is not empty, reached from the
  // initial state by the creation path of the phase-1 node whose p-part it is, then a path of the !q
  // graph through nodes whose W is not empty -- to the nearest node whose whole zone is a stop set,
  // else to the nearest node with a stop set, else around a cycle (every node of W without a stop set
  // has an edge into W, by the fixpoint). Steps: the phase-1 path (ords = transition index, the
  // initial state -1), the root (ords = -2: the previous state cut to p and !q, no transition), the
  // !q path (ords = the edge's transition index); loop_to / loop_ord close a cycle.
  int sweep_trace(long long n2, long long ne, const Fix& fx) {
    Trace& T = *o.trace;
    T = Trace{};
    if (n2 <= 0) return HORA_OK;
    std::vector<int> wc((size_t)n2), sw((size_t)n2), sh((size_t)n2), lev((size_t)n2), es((size_t)ne), ed((size_t)ne),
        er((size_t)ne);
    std::vector<unsigned long long> key((size_t)n2);
    HGB_CUDA(cudaMemcpyAsync(wc.data(), fx.wcnt, n2 * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(sw.data(), fx.swhole, n2 * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(sh.data(), fx.shead, n2 * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(lev.data(), S[1].nlevel.p, n2 * 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(key.data(), S[1].nkey.p, n2 * 8, cudaMemcpyDeviceToHost, s));
    if (ne > 0) {
      HGB_CUDA(cudaMemcpyAsync(es.data(), esrc.p, ne * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(ed.data(), edst.p, ne * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(er.data(), eraw.p, ne * 4, cudaMemcpyDeviceToHost, s));
    }
    HGB_CUDA(wait());
    d2h += (size_t)n2 * 24 + (size_t)ne * 12;
    int root = -1;
    for (long long u = 0; u < n2 && root < 0; ++u)
      if (wc[u] > 0 && lev[u] == 0) root = (int)u;
    if (root < 0) return HORA_OK;   // holds
    std::vector<long long> off((size_t)n2 + 1, 0);   // edges by source
    for (long long e = 0; e < ne; ++e) off[es[e] + 1]++;
    for (long long u = 0; u < n2; ++u) off[u + 1] += off[u];
    std::vector<long long> fill(off.begin(), off.end() - 1), byu((size_t)std::max<long long>(ne, 1));
    for (long long e = 0; e < ne; ++e) byu[fill[es[e]]++] = e;
    // breadth-first over the nodes of W from the root; the nearest whole stop set, else any stop set
    std::vector<long long> via((size_t)n2, -2);   // edge that reached the node (-1: the root)
    std::vector<int> q{root};
    via[root] = -1;
    int goal_whole = -1, goal_part = -1;
    for (size_t h = 0; h < q.size() && goal_whole < 0; ++h) {
      const int u = q[h];
      if (sw[u]) { goal_whole = u; break; }
      if (sh[u] >= 0 && goal_part < 0) goal_part = u;
      for (long long k = off[u]; k < off[u + 1]; ++k) {
        const long long e = byu[k];
        const int v = ed[e];
        if (wc[v] > 0 && via[v] == -2) { via[v] = e; q.push_back(v); }
      }
    }
    std::vector<int> path;        // !q graph nodes from the root
    std::vector<int> praw;        // transition index into each (-1 for the root)
    const int goal = goal_whole >= 0 ? goal_whole : goal_part;
    if (goal >= 0) {
      for (int u = goal; u != root; u = es[via[u]]) { path.push_back(u); praw.push_back(er[via[u]]); }
      path.push_back(root); praw.push_back(-1);
      std::reverse(path.begin(), path.end());
      std::reverse(praw.begin(), praw.end());
    } else {
      std::vector<int> seen((size_t)n2, -1);
      int u = root, raw = -1;
      for (;;) {
        seen[u] = (int)path.size();
        path.push_back(u);
        praw.push_back(raw);
        long long pick = -1;
        for (long long k = off[u]; k < off[u + 1] && pick < 0; ++k)
          if (wc[ed[byu[k]]] > 0) pick = byu[k];
        if (pick < 0) { err = "counterexample walk left the fixpoint"; return HORA_E_CUDA; }
        const int v = ed[pick];
        if (seen[v] >= 0) { T.loop_to = seen[v]; T.loop_ord = er[pick]; break; }
        u = v;
        raw = er[pick];
      }
    }
    // the phase-1 creation path of the root's source node
    int src = -1;
    HGB_CUDA(cudaMemcpyAsync(&src, S[1].npar.template as<int>() + root, 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(wait());
    std::vector<int> pre, preraw;
    std::vector<unsigned long long> prekey;
    for (int u = src; u >= 0;) {
      int par = -1, raw = -1;
      unsigned long long k = 0;
      HGB_CUDA(cudaMemcpyAsync(&par, S[0].npar.template as<int>() + u, 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(&raw, S[0].nraw.template as<int>() + u, 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(&k, S[0].nkey.template as<unsigned long long>() + u, 8, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(wait());
      pre.push_back(u); preraw.push_back(raw); prekey.push_back(k);
      if ((long long)pre.size() > S[0].ncap + 1) { err = "trace walk did not reach the initial state"; return HORA_E_CUDA; }
      u = par;
    }
    std::reverse(pre.begin(), pre.end());
    std::reverse(preraw.begin(), preraw.end());
    std::reverse(prekey.begin(), prekey.end());
    const HostNet& H = *nets[0];
    const int np = H.nprocs, ni = H.nints;
    const int n0 = (int)pre.size(), nsteps = n0 + (int)path.size();
    T.nsteps = nsteps;
    if (T.loop_to >= 0) T.loop_to += n0;
    T.ords.assign(nsteps, -1);
    T.locs.resize((size_t)nsteps * np);
    T.ints.resize((size_t)nsteps * std::max(ni, 0));
    T.zones.resize((size_t)nsteps * Z2);
    auto fill_step = [&](int i, unsigned long long k, const int* dz) -> int {
      HGB_CUDA(cudaMemcpyAsync(T.zones.data() + (size_t)i * Z2, dz, Z2 * 4, cudaMemcpyDeviceToHost, s));
      const unsigned long long kk = k & ((1ull << inst_shift) - 1);
      for (int p = 0; p < np; ++p) T.locs[(size_t)i * np + p] = (int)((kk >> H.kshift[p]) & ((1ull << H.kwidth[p]) - 1));
      for (int v = 0; v < ni; ++v)
        T.ints[(size_t)i * ni + v] = (int)((kk >> H.kshift[np + v]) & ((1ull << H.kwidth[np + v]) - 1)) + H.int_lo[v];
      return HORA_OK;
    };
    int rc;
    for (int i = 0; i < n0; ++i) {
      T.ords[i] = i == 0 ? -1 : preraw[i];
      if ((rc = fill_step(i, prekey[i], S[0].nzone.template as<int>() + (long long)pre[i] * Z2))) return rc;
    }
    for (size_t j = 0; j < path.size(); ++j) {
      T.ords[n0 + j] = j == 0 ? -2 : praw[j];
      if ((rc = fill_step(n0 + (int)j, key[path[j]], S[1].nzone.template as<int>() + (long long)path[j] * Z2))) return rc;
    }
    HGB_CUDA(wait());
    d2h += (size_t)nsteps * (Z2 * 4 + 16);
    return HORA_OK;
  }

  // E[] psi witness: from a surviving root, follow edges into W until a stop node or a node seen
  // before. Every node of W is a stop node or has an edge into W (the fixpoint), so the walk ends.
  int extract_trace(long long n2, long long ne, const int* dW, const int* dstop) {
    Trace& T = *o.trace;
    std::vector<int> hW((size_t)n2), hstop((size_t)n2), hlev((size_t)n2), es((size_t)ne), ed((size_t)ne), eo((size_t)ne);
    std::vector<unsigned long long> hkey((size_t)n2);
    if (n2 > 0) {
      HGB_CUDA(cudaMemcpyAsync(hW.data(), dW, n2 * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(hstop.data(), dstop, n2 * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(hlev.data(), S[1].nlevel.p, n2 * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(hkey.data(), S[1].nkey.p, n2 * 8, cudaMemcpyDeviceToHost, s));
    }
    if (ne > 0) {
      HGB_CUDA(cudaMemcpyAsync(es.data(), esrc.p, ne * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(ed.data(), edst.p, ne * 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(eo.data(), eord.p, ne * 4, cudaMemcpyDeviceToHost, s));
    }
    HGB_CUDA(wait());
    d2h += (size_t)n2 * 20 + (size_t)ne * 12;
    int root = -1;
    for (long long u = 0; u < n2 && root < 0; ++u)
      if (hW[u] && hlev[u] == 0) root = (int)u;
    T = Trace{};
    if (root < 0) return HORA_OK;
    std::vector<long long> off((size_t)n2 + 1, 0);   // edges by source
    for (long long e = 0; e < ne; ++e) off[es[e] + 1]++;
    for (long long u = 0; u < n2; ++u) off[u + 1] += off[u];
    std::vector<long long> fill(off.begin(), off.end() - 1), byu((size_t)ne);
    for (long long e = 0; e < ne; ++e) byu[fill[es[e]]++] = e;
    std::vector<int> path, pord;
    std::vector<int> seen((size_t)n2, -1);
    int u = root, ord = -1;
    for (;;) {
      seen[u] = (int)path.size();
      path.push_back(u);
      pord.push_back(ord);
      if (hstop[u]) break;
      long long pick = -1;
      for (long long k = off[u]; k < off[u + 1] && pick < 0; ++k)
        if (hW[ed[byu[k]]]) pick = byu[k];
      if (pick < 0) { err = "witness walk left the fixpoint"; return HORA_E_CUDA; }
      const int v = ed[pick];
      if (seen[v] >= 0) { T.loop_to = seen[v]; T.loop_ord = eo[pick]; break; }
      u = v;
      ord = eo[pick];
    }
    const HostNet& H = *nets[0];
    const int np = H.nprocs, ni = H.nints;
    T.nsteps = (int)path.size();
    T.ords = pord;
    T.locs.resize((size_t)T.nsteps * np);
    T.ints.resize((size_t)T.nsteps * std::max(ni, 0));
    T.zones.resize((size_t)T.nsteps * Z2);
    for (int i = 0; i < T.nsteps; ++i) {
      HGB_CUDA(cudaMemcpyAsync(T.zones.data() + (size_t)i * Z2, S[1].nzone.template as<int>() + (long long)path[i] * Z2,
                               Z2 * 4, cudaMemcpyDeviceToHost, s));
      const unsigned long long k = hkey[path[i]] & ((1ull << inst_shift) - 1);
      for (int p = 0; p < np; ++p)
        T.locs[(size_t)i * np + p] = (int)((k >> H.kshift[p]) & ((1ull << H.kwidth[p]) - 1));
      for (int v = 0; v < ni; ++v)
        T.ints[(size_t)i * ni + v] = (int)((k >> H.kshift[np + v]) & ((1ull << H.kwidth[np + v]) - 1)) + H.int_lo[v];
    }
    HGB_CUDA(wait());
    return HORA_OK;
  }
  unsigned long long gfp_iters = 0, pre_calls = 0;

  // Trace of a forward search that reached its goal (E<> target, a deadlocked state, or the leads-to
  // early witness): the creation path of the passed store from the initial state to the node whose
  // successor is the goal state, then that state. Step i > 0 is labelled with its transition index
  // (ords[i]); its zone is the stored zone, which contains the exact successor of step i-1's zone by
  // that transition (the stored zone may be extrapolated or a convex hull). Empty when the goal was
  // not reached, or when a leads-to violation was found only by the backward sweep.
  int hit_trace() {
    Trace& T = *o.trace;
    T = Trace{};
    int hn = -1, hr = -1;
    unsigned long long hk = 0;
    HGB_CUDA(cudaMemcpyAsync(&hn, hit_node.p, 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(&hr, hit_raw.p, 4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(&hk, hit_key.p, 8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(wait());
    if (hn == -1) return HORA_OK;
    std::vector<int> path;                       // nodes, the initial one first
    std::vector<int> raws;
    std::vector<unsigned long long> keys;
    for (int u = hn; u >= 0;) {
      int par = -1, raw = -1;
      unsigned long long k = 0;
      HGB_CUDA(cudaMemcpyAsync(&par, S[0].npar.template as<int>() + u, 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(&raw, S[0].nraw.template as<int>() + u, 4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaMemcpyAsync(&k, S[0].nkey.template as<unsigned long long>() + u, 8, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(wait());
      path.push_back(u); raws.push_back(raw); keys.push_back(k);
      if ((long long)path.size() > S[0].ncap + 1) { err = "trace walk did not reach the initial state"; return HORA_E_CUDA; }
      u = par;
    }
    std::reverse(path.begin(), path.end());
    std::reverse(raws.begin(), raws.end());
    std::reverse(keys.begin(), keys.end());
    const bool extra = hn >= 0 && hr >= 0;         // the goal is a successor of the last node
    const HostNet& H = *nets[0];
    const int np = H.nprocs, ni = H.nints;
    const int nsteps = hn == -2 ? 1 : (int)path.size() + (extra ? 1 : 0);
    T.nsteps = nsteps;
    T.ords.assign(nsteps, -1);
    T.locs.resize((size_t)nsteps * np);
    T.ints.resize((size_t)nsteps * std::max(ni, 0));
    T.zones.resize((size_t)nsteps * Z2);
    auto fill = [&](int i, unsigned long long key, const int* dz) -> int {
      HGB_CUDA(cudaMemcpyAsync(T.zones.data() + (size_t)i * Z2, dz, Z2 * 4, cudaMemcpyDeviceToHost, s));
      const unsigned long long kk = key & ((1ull << inst_shift) - 1);
      for (int p = 0; p < np; ++p) T.locs[(size_t)i * np + p] = (int)((kk >> H.kshift[p]) & ((1ull << H.kwidth[p]) - 1));
      for (int v = 0; v < ni; ++v)
        T.ints[(size_t)i * ni + v] = (int)((kk >> H.kshift[np + v]) & ((1ull << H.kwidth[np + v]) - 1)) + H.int_lo[v];
      return HORA_OK;
    };
    int rc;
    if (hn == -2) {
      if ((rc = fill(0, hk, hit_zone.template as<int>()))) return rc;
    } else {
      for (size_t i = 0; i < path.size(); ++i) {
        T.ords[i] = i == 0 ? -1 : raws[i];
        if ((rc = fill((int)i, keys[i], S[0].nzone.template as<int>() + (long long)path[i] * Z2))) return rc;
      }
      if (extra) {
        T.ords[path.size()] = hr;
        if ((rc = fill((int)path.size(), hk, hit_zone.template as<int>()))) return rc;
      }
    }
    HGB_CUDA(wait());
    d2h += (size_t)nsteps * (Z2 * 4 + 16);
    return HORA_OK;
  }

  double elapsed() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  }

  // Per-instance results. After a cancellation, forward-route instances that already had their
  // verdict (goal found, or frontier exhausted) report it with HORA_OK; the others report
  // HORA_E_CANCELLED. st.seconds is the time from the start of the run to the instance's verdict.
  int finish(std::vector<InstResult>& res, int status, bool leadsto) {
    const size_t ni4 = (size_t)ninst * 4, ni8 = (size_t)ninst * 8;
    InstState is = istate();
    HGB_CUDA(cudaEventRecord(ev1, s));
    HGB_CUDA(cudaEventSynchronize(ev1));
    float dev_ms = 0;
    HGB_CUDA(cudaEventElapsedTime(&dev_ms, ev0, ev1));
    HGB_CUDA(cudaMemcpyAsync(h_gen.data(), is.generated, ni8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_nlive.data(), is.nlive, ni8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_nkeys.data(), is.nkeys, ni8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(wait());
    d2h += 2 * ni8 + ni4 + ni8;
    const double wall = elapsed();
    res.assign(ninst, InstResult{});
    for (int k = 0; k < ninst; ++k) {
      InstResult& r = res[k];
      int ist = (status == HORA_E_CANCELLED && !leadsto && t_fin[k] >= 0) ? HORA_OK : status;
      if (h_budget[k] && (ist == HORA_OK || ist == HORA_E_CANCELLED)) ist = HORA_E_BUDGET;
      r.status = ist;
      // leads-to: a surviving root violates it; E[] psi: a surviving root is its witness
      const bool eg = nets[k]->kind == HORA_Q_EG;
      r.verdict = (leadsto && !eg) ? (h_found[k] ? 0 : 1) : (h_found[k] ? 1 : 0);
      r.st.explored = explored[k];
      r.st.expanded = explored[k];
      r.st.generated = h_gen[k];
      r.st.stored = (uint64_t)std::max<long long>(0, h_nlive[k]);
      r.st.keys = h_nkeys[k];
      r.st.levels = levels[k];
      r.st.probes = ninst == 1 ? hctl.probes : 0;
      r.st.probe_full = ninst == 1 ? hctl.probe_full : 0;
      r.st.merge_surv = ninst == 1 ? merge_surv : 0;
      r.st.merge_live = ninst == 1 ? hctl.merge_live : 0;
      r.st.nodes = ninst == 1 ? hctl.nnodes : 0;
      r.st.pre_calls = pre_calls;
      r.st.gfp_iters = gfp_iters;
      r.st.kernel_launches = launches;
      r.st.seconds = (ist == HORA_OK && t_fin[k] >= 0) ? t_fin[k] : wall;
      r.st.device_seconds = dev_ms * 1e-3;
      r.st.extrapolating = h_emode[k];
      r.st.status = ist;
      for (int q = 0; q < 6; ++q) { r.st.kernel_seconds[q] = kt.sec[q]; r.st.kernel_calls[q] = kt.calls[q]; }
      r.st.h2d_bytes = h2d;
      r.st.d2h_bytes = d2h;
    }
    return status;
  }
};

template <int D>
int run_group(const std::vector<const HostNet*>& nets, std::vector<InstResult>& res, const RunOptions& o,
              std::string& err) {
  Engine<D> E(nets, o, err);
  if (o.trace) *o.trace = Trace{};
  int rc = E.setup();
  if (rc) return rc;
  long long nf = 0;
  if ((rc = E.init(&nf))) return rc;
  int cur = 0, level = 0;
  const bool eg = !nets.empty() && nets[0]->kind == HORA_Q_EG;
  const bool leadsto = !nets.empty() && (nets[0]->kind == HORA_Q_LEADSTO || eg);
  // E[] psi has no reachability pass: its graph is rooted at the (restricted) initial state
  int status = eg ? HORA_OK : E.leadsto_witness(cur, nf);
  if (status == HORA_OK && !eg) status = E.run_levels(0, 0, cur, nf, level, nullptr);
  if (status == HORA_OK && leadsto) status = E.leadsto_phase2(cur);
  if (status != HORA_OK && status != HORA_E_CANCELLED) {
    E.finish(res, status, leadsto);
    return status;
  }
  // a forward search's goal; for leads-to, the early witness unless the sweep already left a trace
  if (status == HORA_OK && o.trace && nets.size() == 1 && nets[0]->kind != HORA_Q_EG && o.trace->nsteps == 0 &&
      (status = E.hit_trace())) {
    E.finish(res, status, leadsto);
    return status;
  }
  const int frc = E.finish(res, status, leadsto);
  return frc;
}


template <int D>
int run_expand(const HostNet& net, int n, const int* locs, const int* ints, const int* zones, int emode, int64_t cap,
               int* out_src, int* out_ord, int* out_locs, int* out_ints, int* out_zones, int64_t* out_n,
               std::string& err) {
  constexpr long long Z2 = (long long)D * D;
  cudaStream_t s;
  HGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  // declared first, so it ends last: the buffers below are freed on the stream before it goes
  struct StreamGuard {
    cudaStream_t s, prev;
    ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); g_alloc_stream = prev; }
  } sg{s, g_alloc_stream};
  g_alloc_stream = s;
  prepare_device_pool();
  DeviceNets dn;
  std::vector<const HostNet*> v{&net};
  int rc = upload_nets(v, 63, dn, err);
  if (rc) return rc;
  const int np = net.nprocs, ni = std::max(net.nints, 1);
  DBuf dl, di, dz, ctl;
  HGB_CUDA(dl.alloc((size_t)n * np * 4)); HGB_CUDA(di.alloc((size_t)n * ni * 4)); HGB_CUDA(dz.alloc((size_t)n * Z2 * 4));
  HGB_CUDA(ctl.alloc(sizeof(Ctl)));
  HGB_CUDA(cudaMemcpyAsync(dl.p, locs, (size_t)n * np * 4, cudaMemcpyHostToDevice, s));
  if (net.nints) HGB_CUDA(cudaMemcpyAsync(di.p, ints, (size_t)n * net.nints * 4, cudaMemcpyHostToDevice, s));
  HGB_CUDA(cudaMemcpyAsync(dz.p, zones, (size_t)n * Z2 * 4, cudaMemcpyHostToDevice, s));
  long long dcap = std::max<long long>(cap, 16);
  for (;;) {
    DBuf okey, osrc, oord, olocs, oints, oz;
    HGB_CUDA(okey.alloc(dcap * 8)); HGB_CUDA(osrc.alloc(dcap * 4)); HGB_CUDA(oord.alloc(dcap * 4));
    HGB_CUDA(olocs.alloc(dcap * np * 4)); HGB_CUDA(oints.alloc(dcap * ni * 4)); HGB_CUDA(oz.alloc(dcap * Z2 * 4));
    HGB_CUDA(cudaMemsetAsync(ctl.p, 0, sizeof(Ctl), s));
    Level<D>::expand_plain(dn.views, dl.as<int>(), di.as<int>(), dz.as<int>(), n, emode, okey.as<unsigned long long>(),
                           osrc.as<int>(), oord.as<int>(), olocs.as<int>(), oints.as<int>(), oz.as<int>(), dcap,
                           ctl.as<Ctl>(), s);
    HGB_CUDA(cudaGetLastError());
    Ctl h;
    HGB_CUDA(cudaMemcpyAsync(&h, ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaStreamSynchronize(s));
    if (h.err) { err = "broadcast receivers exceed the device tables"; return (int)h.err; }
    const long long total = (long long)h.nsucc;
    if (total > dcap && dcap < cap) { dcap = std::min<long long>(total, cap); continue; }
    const long long k = std::min<long long>(total, dcap);
    std::vector<unsigned long long> key(k);
    std::vector<int> src(k), ord(k), lo((size_t)k * np), in((size_t)k * ni), zz((size_t)k * Z2);
    HGB_CUDA(cudaMemcpy(key.data(), okey.p, k * 8, cudaMemcpyDeviceToHost));
    HGB_CUDA(cudaMemcpy(src.data(), osrc.p, k * 4, cudaMemcpyDeviceToHost));
    HGB_CUDA(cudaMemcpy(ord.data(), oord.p, k * 4, cudaMemcpyDeviceToHost));
    HGB_CUDA(cudaMemcpy(lo.data(), olocs.p, (size_t)k * np * 4, cudaMemcpyDeviceToHost));
    HGB_CUDA(cudaMemcpy(in.data(), oints.p, (size_t)k * ni * 4, cudaMemcpyDeviceToHost));
    HGB_CUDA(cudaMemcpy(zz.data(), oz.p, (size_t)k * Z2 * 4, cudaMemcpyDeviceToHost));
    std::vector<long long> perm(k);
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(), [&](long long a, long long b) { return key[a] < key[b]; });
    for (long long q = 0; q < k; ++q) {
      const long long a = perm[q];
      out_src[q] = src[a];
      out_ord[q] = ord[a];
      std::memcpy(out_locs + q * np, lo.data() + a * np, np * 4);
      if (net.nints) std::memcpy(out_ints + q * net.nints, in.data() + a * ni, net.nints * 4);
      std::memcpy(out_zones + q * Z2, zz.data() + a * Z2, Z2 * 4);
    }
    *out_n = total;
    return total > cap ? HORA_E_OVERFLOW : HORA_OK;
  }
}

template <int D>
int run_has_deadlock(const HostNet& net, int n, const int* locs, const int* ints, const int* zones, int* out,
                     std::string& err) {
  constexpr long long Z2 = (long long)D * D;
  cudaStream_t s;
  HGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  // declared first, so it ends last: the buffers below are freed on the stream before it goes
  struct StreamGuard {
    cudaStream_t s, prev;
    ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); g_alloc_stream = prev; }
  } sg{s, g_alloc_stream};
  g_alloc_stream = s;
  prepare_device_pool();
  DeviceNets dn;
  std::vector<const HostNet*> v{&net};
  int rc = upload_nets(v, 63, dn, err);
  if (rc) return rc;
  const int np = net.nprocs, ni = std::max(net.nints, 1);
  DBuf dl, di, dz, dout, ctl;
  HGB_CUDA(dl.alloc((size_t)n * np * 4)); HGB_CUDA(di.alloc((size_t)n * ni * 4));
  HGB_CUDA(dz.alloc((size_t)n * Z2 * 4)); HGB_CUDA(dout.alloc((size_t)n * 4)); HGB_CUDA(ctl.alloc(sizeof(Ctl)));
  HGB_CUDA(cudaMemcpyAsync(dl.p, locs, (size_t)n * np * 4, cudaMemcpyHostToDevice, s));
  if (net.nints) HGB_CUDA(cudaMemcpyAsync(di.p, ints, (size_t)n * net.nints * 4, cudaMemcpyHostToDevice, s));
  HGB_CUDA(cudaMemcpyAsync(dz.p, zones, (size_t)n * Z2 * 4, cudaMemcpyHostToDevice, s));
  HGB_CUDA(cudaMemsetAsync(ctl.p, 0, sizeof(Ctl), s));
  Level<D>::has_deadlock(dn.views, dl.as<int>(), di.as<int>(), dz.as<int>(), n, dout.as<int>(), ctl.as<Ctl>(), s);
  HGB_CUDA(cudaGetLastError());
  Ctl h;
  HGB_CUDA(cudaMemcpyAsync(&h, ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaMemcpyAsync(out, dout.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaStreamSynchronize(s));
  if (h.err) { err = "deadlock test exceeded its escape table"; return (int)h.err; }
  return HORA_OK;
}

}  // namespace hgb
