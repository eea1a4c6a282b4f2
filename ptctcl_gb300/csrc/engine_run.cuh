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
      return HORA_E_CUDA;                                                          \
    }                                                                              \
  } while (0)

// A device allocation that frees itself. grow() keeps the first `keep` bytes.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t b) {
    if (p) { cudaFree(p); p = nullptr; }
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b ? b : 16);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  cudaError_t grow(size_t b, size_t keep, cudaStream_t s) {
    if (b <= bytes) return cudaSuccess;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, b);
    if (e != cudaSuccess) return e;
    if (p && keep) {
      e = cudaMemcpyAsync(q, p, std::min(keep, bytes), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) { cudaFree(q); return e; }
      cudaStreamSynchronize(s);
    }
    if (p) cudaFree(p);
    p = q;
    bytes = b;
    return cudaSuccess;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

static __global__ void k_rehash(const unsigned long long* okey, const int* ohead, unsigned long long ocap,
                                unsigned long long* nkey, int* nhead, unsigned long long nmask, unsigned* err) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ocap;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long k = okey[i];
    if (k == kEmptyKey) continue;
    unsigned long long h = hash_mix(k) & nmask;
    unsigned long long probe = 0;
    for (; probe <= nmask; ++probe) {
      if (atomicCAS(&nkey[h], kEmptyKey, k) == kEmptyKey) { nhead[h] = ohead[i]; break; }
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
struct GroupBuffers {
  DBuf hkey, head, pend, pend_base;                         // hash table
  DBuf nzone, nnext, nlevel, ndead, ninst;                  // nodes
  DBuf skey, sparent, sord, sslot, srank, szone, ssurv, sseg, ssorted, stouched;   // successors
  DBuf fkey[2], fnode[2], frank[2], finst[2];               // frontiers
  DBuf ctl, nets_ok;
  DBuf emode, done, found, generated, gen_backup, nlive, nkeys, nfront, probes;
  unsigned long long hcap = 0;
  long long ncap = 0, scap = 0, fcapb[2] = {0, 0};
};

template <int D>
int run_group(const std::vector<const HostNet*>& nets, std::vector<InstResult>& res, const RunOptions& o,
              std::string& err) {
  const auto t_start = std::chrono::steady_clock::now();
  constexpr long long Z2 = (long long)D * D;
  const int ninst = (int)nets.size();
  res.assign(ninst, InstResult{});
  int instbits = 0;
  while ((1 << instbits) < ninst) ++instbits;
  const int inst_shift = 63 - instbits;
  for (int k = 0; k < ninst; ++k)
    if (nets[k]->keybits > inst_shift) { err = "discrete key too wide for the batch"; return HORA_E_NOT_SUPPORTED; }

  cudaStream_t s;
  HGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{s};
  int dev = 0, nsm = 0;
  HGB_CUDA(cudaGetDevice(&dev));
  HGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = o.blocks > 0 ? o.blocks : nsm * 16;

  DeviceNets dn;
  {
    int rc = upload_nets(nets, inst_shift, dn, err);
    if (rc) return rc;
  }
  GroupBuffers<D> B;
  // --- initial sizes
  B.hcap = 1ull << 16;
  while (B.hcap < 4ull * ninst) B.hcap <<= 1;
  B.ncap = std::max<long long>(1 << 14, 2LL * ninst);
  B.scap = (long long)std::max<size_t>(o.succ_cap0, 4 * (size_t)ninst);
  B.fcapb[0] = B.fcapb[1] = std::max<long long>(1 << 14, 2LL * ninst);
  auto alloc_table = [&](DBuf& k, DBuf& h, DBuf& p, DBuf& pb, unsigned long long cap) -> cudaError_t {
    cudaError_t e;
    if ((e = k.alloc(cap * 8)) || (e = h.alloc(cap * 4)) || (e = p.alloc(cap * 4)) || (e = pb.alloc(cap * 4))) return e;
    if ((e = cudaMemsetAsync(k.p, 0xff, cap * 8, s)) || (e = cudaMemsetAsync(h.p, 0xff, cap * 4, s)) ||
        (e = cudaMemsetAsync(p.p, 0, cap * 4, s)))
      return e;
    return cudaSuccess;
  };
  HGB_CUDA(alloc_table(B.hkey, B.head, B.pend, B.pend_base, B.hcap));
  HGB_CUDA(B.nzone.alloc(B.ncap * Z2 * 4));
  HGB_CUDA(B.nnext.alloc(B.ncap * 4));
  HGB_CUDA(B.nlevel.alloc(B.ncap * 4));
  HGB_CUDA(B.ndead.alloc(B.ncap * 4));
  HGB_CUDA(B.ninst.alloc(B.ncap * 4));
  auto alloc_succ = [&](long long cap) -> cudaError_t {
    cudaError_t e;
    if ((e = B.skey.alloc(cap * 8)) || (e = B.sparent.alloc(cap * 4)) || (e = B.sord.alloc(cap * 4)) ||
        (e = B.sslot.alloc(cap * 4)) || (e = B.srank.alloc(cap * 4)) || (e = B.szone.alloc(cap * Z2 * 4)) ||
        (e = B.ssurv.alloc(cap * 4)) || (e = B.sseg.alloc(cap * 4)) || (e = B.ssorted.alloc(cap * 4)) ||
        (e = B.stouched.alloc(cap * 4)))
      return e;
    return cudaSuccess;
  };
  HGB_CUDA(alloc_succ(B.scap));
  for (int b = 0; b < 2; ++b) {
    HGB_CUDA(B.fkey[b].alloc(B.fcapb[b] * 8));
    HGB_CUDA(B.fnode[b].alloc(B.fcapb[b] * 4));
    HGB_CUDA(B.frank[b].alloc(B.fcapb[b] * 4));
    HGB_CUDA(B.finst[b].alloc(B.fcapb[b] * 4));
  }
  HGB_CUDA(B.ctl.alloc(sizeof(Ctl)));
  HGB_CUDA(cudaMemsetAsync(B.ctl.p, 0, sizeof(Ctl), s));
  const size_t ni4 = (size_t)ninst * 4, ni8 = (size_t)ninst * 8;
  HGB_CUDA(B.emode.alloc(ni4)); HGB_CUDA(B.done.alloc(ni4)); HGB_CUDA(B.found.alloc(ni4));
  HGB_CUDA(B.generated.alloc(ni8)); HGB_CUDA(B.gen_backup.alloc(ni8)); HGB_CUDA(B.nlive.alloc(ni8));
  HGB_CUDA(B.nkeys.alloc(ni8)); HGB_CUDA(B.nfront.alloc(ni8)); HGB_CUDA(B.probes.alloc(ni8));
  for (DBuf* b : {&B.emode, &B.done, &B.found, &B.generated, &B.nlive, &B.nkeys, &B.nfront, &B.probes})
    HGB_CUDA(cudaMemsetAsync(b->p, 0, b->bytes, s));

  auto store = [&]() {
    Store st;
    st.hkey = B.hkey.template as<unsigned long long>(); st.head = B.head.template as<int>();
    st.pend = B.pend.template as<unsigned>(); st.pend_base = B.pend_base.template as<unsigned>();
    st.hmask = B.hcap - 1;
    st.nzone = B.nzone.template as<int>(); st.nnext = B.nnext.template as<int>();
    st.nlevel = B.nlevel.template as<int>(); st.ndead = B.ndead.template as<int>(); st.ninst = B.ninst.template as<int>();
    return st;
  };
  auto succ = [&]() {
    Succ sc;
    sc.key = B.skey.template as<unsigned long long>(); sc.parent = B.sparent.template as<int>();
    sc.ord = B.sord.template as<int>(); sc.slot = B.sslot.template as<int>(); sc.rank = B.srank.template as<int>();
    sc.zone = B.szone.template as<int>(); sc.surv = B.ssurv.template as<int>(); sc.seg = B.sseg.template as<int>();
    sc.sorted = B.ssorted.template as<int>(); sc.touched = B.stouched.template as<int>(); sc.cap = B.scap;
    return sc;
  };
  auto front = [&](int b) {
    Front f;
    f.key = B.fkey[b].template as<unsigned long long>(); f.node = B.fnode[b].template as<int>();
    f.rank = B.frank[b].template as<int>(); f.inst = B.finst[b].template as<int>();
    return f;
  };
  InstState is;
  is.emode = B.emode.template as<int>(); is.done = B.done.template as<int>(); is.found = B.found.template as<unsigned>();
  is.generated = B.generated.template as<unsigned long long>(); is.nlive = B.nlive.template as<long long>();
  is.nkeys = B.nkeys.template as<unsigned long long>(); is.nfront = B.nfront.template as<unsigned long long>();
  is.probes = B.probes.template as<unsigned long long>();
  Ctl* dctl = B.ctl.template as<Ctl>();
  Ctl hctl;
  unsigned long long launches = 0, h2d = 0, d2h = 0;
  for (const HostNet* hn : nets) (void)hn;
  for (size_t k = 0; k < dn.blob_bytes.size(); ++k) h2d += dn.blob_bytes[k];
  h2d += sizeof(NetView) * (size_t)ninst;
  KTimer kt;
  auto read_ctl = [&]() -> cudaError_t {
    cudaError_t e = cudaMemcpyAsync(&hctl, dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s);
    if (e) return e;
    d2h += sizeof(Ctl);
    e = cudaStreamSynchronize(s);
    kt.collect();
    return e;
  };
  // per-instance host mirrors
  std::vector<int> h_done(ninst, 0), h_emode(ninst, 0);
  std::vector<unsigned> h_found(ninst, 0);
  std::vector<unsigned long long> h_nfront(ninst, 0), h_nkeys(ninst, 0), h_gen(ninst, 0);
  std::vector<long long> h_nlive(ninst, 0);
  std::vector<unsigned long long> explored(ninst, 0), levels(ninst, 0);

  cudaEvent_t ev0, ev1;
  HGB_CUDA(cudaEventCreate(&ev0));
  HGB_CUDA(cudaEventCreate(&ev1));
  struct EvGuard { cudaEvent_t a, b; ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); } } eg{ev0, ev1};
  HGB_CUDA(cudaEventRecord(ev0, s));

  // --- level 0
  kt.begin(s);
  Level<D>::init(dn.views, ninst, dn.ok, store(), front(0), is, dctl, s);
  kt.end(s, KT_OTHER);
  ++launches;
  HGB_CUDA(cudaGetLastError());
  HGB_CUDA(read_ctl());
  if (hctl.err) { err = "device error in init"; return (int)hctl.err; }
  HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaMemcpyAsync(h_done.data(), is.done, ni4, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaStreamSynchronize(s));
  long long nfront = (long long)hctl.nfront;
  int cur = 0;
  int level = 0;
  int status = HORA_OK;
  while (nfront > 0) {
    if (o.cancel && *o.cancel) { status = HORA_E_CANCELLED; break; }
    ++level;
    // per-instance frontier sizes of this level
    HGB_CUDA(cudaMemcpyAsync(h_nfront.data(), is.nfront, ni8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemsetAsync(is.nfront, 0, ni8, s));
    HGB_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < ninst; ++k)
      if (!h_done[k] && h_nfront[k]) { explored[k] += h_nfront[k]; levels[k] = level; }
    // ---- expand (re-run with a larger buffer on overflow; expand writes nothing persistent)
    for (;;) {
      HGB_CUDA(cudaMemsetAsync(dctl, 0, kCtlLevelBytes, s));
      HGB_CUDA(cudaMemcpyAsync(B.gen_backup.p, is.generated, ni8, cudaMemcpyDeviceToDevice, s));
      kt.begin(s);
      Level<D>::expand(dn.views, is, front(cur), (int)nfront, store(), succ(), dctl, blocks, s);
      kt.end(s, KT_EXPAND);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      HGB_CUDA(read_ctl());
      if (!hctl.overflow) break;
      const long long need = (long long)(hctl.nsucc + hctl.nsucc / 4 + 1024);
      HGB_CUDA(cudaMemcpyAsync(is.generated, B.gen_backup.p, ni8, cudaMemcpyDeviceToDevice, s));
      B.scap = need;
      HGB_CUDA(alloc_succ(B.scap));
    }
    if (hctl.err) { status = (int)hctl.err; err = "device error in expand"; break; }
    const long long nsucc = (long long)hctl.nsucc;
    if (hctl.found) {
      HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaStreamSynchronize(s));
    }
    // ---- make room in the hash table for every possible new key
    if ((hctl.nslots + (unsigned long long)nsucc) * 2 > B.hcap) {
      unsigned long long ncap = B.hcap;
      while ((hctl.nslots + (unsigned long long)nsucc) * 2 > ncap) ncap <<= 1;
      DBuf k2, h2, p2, pb2;
      HGB_CUDA(alloc_table(k2, h2, p2, pb2, ncap));
      kt.begin(s);
      k_rehash<<<1024, 256, 0, s>>>(B.hkey.template as<unsigned long long>(), B.head.template as<int>(), B.hcap,
                                   k2.template as<unsigned long long>(), h2.template as<int>(), ncap - 1, &dctl->err);
      kt.end(s, KT_OTHER);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      HGB_CUDA(cudaStreamSynchronize(s));
      kt.collect();
      std::swap(B.hkey.p, k2.p); std::swap(B.hkey.bytes, k2.bytes);
      std::swap(B.head.p, h2.p); std::swap(B.head.bytes, h2.bytes);
      std::swap(B.pend.p, p2.p); std::swap(B.pend.bytes, p2.bytes);
      std::swap(B.pend_base.p, pb2.p); std::swap(B.pend_base.bytes, pb2.bytes);
      B.hcap = ncap;
    }
    // ---- probe
    if (nsucc > 0) {
      kt.begin(s);
      Level<D>::probe(dn.views, is, succ(), store(), dctl, nsucc, blocks, s);
      kt.end(s, KT_PROBE);
      ++launches;
      HGB_CUDA(cudaGetLastError());
    }
    HGB_CUDA(read_ctl());
    if (hctl.err) { status = (int)hctl.err; err = "device error in probe"; break; }
    const long long nsurv = (long long)hctl.nsurv, ntouched = (long long)hctl.ntouched;
    // ---- deadlock goal on the survivors
    bool any_dl = false;
    for (int k = 0; k < ninst; ++k) any_dl |= (nets[k]->kind == HORA_Q_DEADLOCK && !h_done[k]);
    if (any_dl && nsurv > 0) {
      kt.begin(s);
      Level<D>::deadlock(dn.views, is, succ(), dctl, nsurv, blocks, s);
      kt.end(s, KT_DEADLOCK);
      ++launches;
      HGB_CUDA(cudaGetLastError());
      HGB_CUDA(read_ctl());
      if (hctl.err) { status = (int)hctl.err; err = "deadlock test exceeded its escape table"; break; }
    }
    if (hctl.found) {
      HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
      HGB_CUDA(cudaStreamSynchronize(s));
    }
    // ---- room for the new nodes and the next frontier
    if ((long long)hctl.nnodes + nsurv > B.ncap) {
      long long nc = B.ncap;
      while ((long long)hctl.nnodes + nsurv > nc) nc *= 2;
      const size_t used = hctl.nnodes;
      HGB_CUDA(B.nzone.grow(nc * Z2 * 4, used * Z2 * 4, s));
      HGB_CUDA(B.nnext.grow(nc * 4, used * 4, s));
      HGB_CUDA(B.nlevel.grow(nc * 4, used * 4, s));
      HGB_CUDA(B.ndead.grow(nc * 4, used * 4, s));
      HGB_CUDA(B.ninst.grow(nc * 4, used * 4, s));
      B.ncap = nc;
    }
    if (nsurv > B.fcapb[cur ^ 1]) {   // the next frontier holds at most one entry per survivor
      const int nxt = cur ^ 1;
      long long fc = B.fcapb[nxt];
      while (nsurv > fc) fc *= 2;
      HGB_CUDA(B.fkey[nxt].alloc(fc * 8)); HGB_CUDA(B.fnode[nxt].alloc(fc * 4));
      HGB_CUDA(B.frank[nxt].alloc(fc * 4)); HGB_CUDA(B.finst[nxt].alloc(fc * 4));
      B.fcapb[nxt] = fc;
    }
    // ---- group + merge
    if (ntouched > 0) {
      kt.begin(s);
      Level<D>::group(succ(), store(), dctl, nsucc, ntouched, s);
      kt.end(s, KT_GROUP, 2);
      kt.begin(s);
      Level<D>::merge(dn.views, is, front(cur), succ(), store(), front(cur ^ 1), dctl, ntouched, level, blocks, s);
      kt.end(s, KT_MERGE);
      launches += 3;
      HGB_CUDA(cudaGetLastError());
    }
    HGB_CUDA(read_ctl());
    if (hctl.err) { status = (int)hctl.err; err = "device error in merge"; break; }
    // ---- end of level: goals, adaptive extrapolation, next frontier
    HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_nlive.data(), is.nlive, ni8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaMemcpyAsync(h_nkeys.data(), is.nkeys, ni8, cudaMemcpyDeviceToHost, s));
    HGB_CUDA(cudaStreamSynchronize(s));
    bool changed = false;
    for (int k = 0; k < ninst; ++k) {
      if (h_done[k]) continue;
      if (h_found[k]) { h_done[k] = 1; changed = true; continue; }
      // adaptive switch to Extra_LU+ (src/reachability/engine.cpp:2178-2184)
      if (h_emode[k] == 0 && h_nkeys[k] && (double)h_nlive[k] >= 4.0 * (double)h_nkeys[k]) { h_emode[k] = 1; changed = true; }
    }
    if (changed) {
      HGB_CUDA(cudaMemcpyAsync(is.done, h_done.data(), ni4, cudaMemcpyHostToDevice, s));
      HGB_CUDA(cudaMemcpyAsync(is.emode, h_emode.data(), ni4, cudaMemcpyHostToDevice, s));
    }
    nfront = (long long)hctl.nfront;
    cur ^= 1;
  }
  HGB_CUDA(cudaEventRecord(ev1, s));
  HGB_CUDA(cudaEventSynchronize(ev1));
  float dev_ms = 0;
  HGB_CUDA(cudaEventElapsedTime(&dev_ms, ev0, ev1));
  HGB_CUDA(cudaMemcpyAsync(h_gen.data(), is.generated, ni8, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaMemcpyAsync(h_found.data(), is.found, ni4, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaMemcpyAsync(h_nlive.data(), is.nlive, ni8, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaMemcpyAsync(h_nkeys.data(), is.nkeys, ni8, cudaMemcpyDeviceToHost, s));
  HGB_CUDA(cudaStreamSynchronize(s));
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  for (int k = 0; k < ninst; ++k) {
    InstResult& r = res[k];
    r.status = status;
    r.verdict = h_found[k] ? 1 : 0;
    r.st.explored = explored[k];
    r.st.expanded = explored[k];
    r.st.generated = h_gen[k];
    r.st.stored = (uint64_t)std::max<long long>(0, h_nlive[k]);
    r.st.keys = h_nkeys[k];
    r.st.levels = levels[k];
    r.st.probes = ninst == 1 ? hctl.probes : 0;
    r.st.kernel_launches = launches;
    r.st.seconds = wall;
    r.st.device_seconds = dev_ms * 1e-3;
    r.st.extrapolating = h_emode[k];
    r.st.status = status;
    for (int q = 0; q < 6; ++q) { r.st.kernel_seconds[q] = kt.sec[q]; r.st.kernel_calls[q] = kt.calls[q]; }
    r.st.h2d_bytes = h2d;
    r.st.d2h_bytes = d2h;
  }
  return status == HORA_E_CANCELLED ? HORA_E_CANCELLED : (status ? status : HORA_OK);
}

template <int D>
int run_expand(const HostNet& net, int n, const int* locs, const int* ints, const int* zones, int emode, int64_t cap,
               int* out_src, int* out_ord, int* out_locs, int* out_ints, int* out_zones, int64_t* out_n,
               std::string& err) {
  constexpr long long Z2 = (long long)D * D;
  DeviceNets dn;
  std::vector<const HostNet*> v{&net};
  int rc = upload_nets(v, 63, dn, err);
  if (rc) return rc;
  cudaStream_t s;
  HGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{s};
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
  DeviceNets dn;
  std::vector<const HostNet*> v{&net};
  int rc = upload_nets(v, 63, dn, err);
  if (rc) return rc;
  cudaStream_t s;
  HGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{s};
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
