// level_kernels_impl.cuh -- bodies of the level kernels. Included once per DBM dimension by the
// generated translation units (dim_<D>.cu), which instantiate hgb::Level<D>.
#pragma once
#include "level_kernels.cuh"

namespace hgb {

constexpr int kBlock = 128;   // threads per block: 4 warps, each holding floor(32/D) tiles

template <int D>
__device__ __forceinline__ long long tile_id() {
  constexpr int TPW = 32 / D;
  const int lane = threadIdx.x & 31;
  return ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * TPW + lane / D;
}
template <int D>
__device__ __forceinline__ long long tile_count() {
  return (long long)gridDim.x * (blockDim.x >> 5) * (32 / D);
}
__device__ __forceinline__ unsigned long long key_part(unsigned long long hk, int inst_shift) {
  return hk & ((1ull << inst_shift) - 1);
}

// Find or insert a hash key (atomic CAS, linear probing). Returns the slot, or -1 if the table
// is full; *inserted tells a fresh key from an existing one. Called by one lane.
inline __device__ long long slot_find_insert(const Store& st, unsigned long long hk, bool* inserted) {
  unsigned long long h = hash_mix(hk) & st.hmask;
  *inserted = false;
  for (unsigned long long probe = 0; probe <= st.hmask; ++probe) {
    const unsigned long long k = st.hkey[h];
    if (k == hk) return (long long)h;
    if (k == kEmptyKey) {
      const unsigned long long prev = atomicCAS(&st.hkey[h], kEmptyKey, hk);
      if (prev == kEmptyKey) { *inserted = true; return (long long)h; }
      if (prev == hk) return (long long)h;
    }
    h = (h + 1) & st.hmask;
  }
  return -1;
}

// ---------------------------------------------------------------------------------------------
// init: the initial symbolic state of every instance (initial_symbolic_state,
// src/reachability/engine.cpp:1322-1335), its goal test, and its insertion at level 0.
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock) k_init(const NetView* nets, int ninst, const int* ok, Store st,
                                                 Front out, InstState is, Ctl* ctl) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  DlScratch<D> S;
  for (long long w = tile_id<D>(); w < ninst; w += tile_count<D>()) {
    const int inst = (int)w;
    if (!ok[inst]) continue;
    const NetView& N = nets[inst];
    int locs[kMaxProcs], ints[kMaxInts];
    for (int p = 0; p < N.nprocs; ++p) locs[p] = N.proc_init[p];
    for (int v = 0; v < N.nints; ++v) ints[v] = N.int_init[v];
    int z[D];
    init_zero(z);
    if (!close_succ(N, t, z, locs, ints, 0) || is_empty(t, z)) {   // no initial state at all
      if (t.i == 0) is.done[inst] = 1;
      continue;
    }
    bool hit = false;
    if (N.kind == 0) hit = target_hit(N, t, z, locs, ints);
    else if (N.kind == 1) {
      const int r = state_has_deadlock(N, t, locs, ints, z, S);
      if (r < 0) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
      hit = r == 1;
    }
    if (hit) {
      if (t.i == 0) { is.found[inst] = 1; is.done[inst] = 1; atomicOr(&ctl->found, 1u); }
      continue;
    }
    const unsigned long long hk = key_encode(N, locs, ints) | ((unsigned long long)inst << N.inst_shift);
    long long slot = 0, node = 0;
    if (t.i == 0) {
      bool ins;
      slot = slot_find_insert(st, hk, &ins);
      if (slot >= 0) node = (long long)atomicAdd(&ctl->nnodes, 1ull);
    }
    slot = (long long)t.shfl64((unsigned long long)slot, 0);
    node = (long long)t.shfl64((unsigned long long)node, 0);
    if (slot < 0) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
    store_rows(t, z, st.nzone + node * D * D);
    if (t.i == 0) {
      st.nnext[node] = -1; st.nlevel[node] = 0; st.ndead[node] = 0; st.ninst[node] = inst; st.nkey[node] = hk;
      st.head[slot] = (int)node;
      const unsigned long long f = atomicAdd(&ctl->nfront, 1ull);
      out.key[f] = hk; out.node[f] = (int)node; out.rank[f] = 0; out.inst[f] = inst;
      is.nkeys[inst] = 1; is.nlive[inst] = 1; is.nfront[inst] = 1;
      atomicAdd(&ctl->nkeys, 1ull);
      atomicAdd(&ctl->nslots, 1ull);
      atomicAdd((unsigned long long*)&ctl->nlive, 1ull);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// expand: successors of every frontier state
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock) k_expand(const NetView* nets, InstState is, Front fr, int nfront,
                                                   const int* src_zone, Succ sc, Ctl* ctl, int roots) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  for (long long f = tile_id<D>(); f < nfront; f += tile_count<D>()) {
    const int inst = fr.inst[f];
    if (is.done[inst]) continue;
    const NetView& N = nets[inst];
    const unsigned long long hk = fr.key[f];
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, N.inst_shift), locs, ints);
    int src[D];
    load_rows(t, src, src_zone + (long long)fr.node[f] * D * D);
    const int emode = is.emode[inst];
    int ord = 0;
    bool hit = false;
    auto emit = [&](const int* tl, const int* ti, const int (&z)[D]) {
      unsigned long long idx = 0;
      if (t.i == 0) idx = atomicAdd(&ctl->nsucc, 1ull);
      idx = t.shfl64(idx, 0);
      if ((long long)idx < sc.cap) {
        store_rows(t, z, sc.zone + (long long)idx * D * D);
        if (t.i == 0) {
          sc.key[idx] = key_encode(N, tl, ti) | ((unsigned long long)inst << N.inst_shift);
          sc.parent[idx] = (int)f;
          sc.ord[idx] = ord;
          sc.okh[idx] = hk;
          sc.okl[idx] = ((unsigned long long)(unsigned)fr.rank[f] << 32) | (unsigned)ord;
        }
      } else if (t.i == 0) {
        ctl->overflow = 1;
      }
      ++ord;
      if (N.kind == 0 && !hit) hit = target_hit(N, t, z, tl, ti);
    };
    bool ok = true;
    if (roots) {
      // leads-to roots: the p-part of a phase-1 zone, cut to !q
      if (apply_cons(t, src, N.p_clk, 0, N.p_nclk) && avoid_cut(N, t, src, locs, ints) && !is_empty(t, src))
        emit(locs, ints, src);
    } else {
      ok = for_each_successor(N, t, locs, ints, src, emode, emit);
    }
    if (t.i == 0) {
      if (!ok) atomicMax(&ctl->err, 4u);
      if (ord && !roots) atomicAdd(&is.generated[inst], (unsigned long long)ord);
      if (hit) { is.found[inst] = 1; atomicOr(&ctl->found, 1u); }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// probe: drop successors a stored zone simulates; group the rest by hash slot
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock) k_probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl,
                                                  long long nsucc, int mode) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  for (long long s = tile_id<D>(); s < nsucc; s += tile_count<D>()) {
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    if (is.found[inst] || is.done[inst]) { if (t.i == 0) sc.slot[s] = -1; continue; }
    const NetView& N = nets[inst];
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    int Ly, U[D];
    key_bounds(N, t, locs, Ly, U);
    int z[D], z0[D];
    load_rows(t, z, sc.zone + s * D * D);
#pragma unroll
    for (int x = 0; x < D; ++x) z0[x] = t.shfl(z[x], 0);
    long long slot = 0;
    int inserted = 0;
    if (t.i == 0) {
      bool ins;
      slot = slot_find_insert(st, hk, &ins);
      inserted = ins;   // keys are counted when their first zone is stored (merge), not here
      if (ins) atomicAdd(&ctl->nslots, 1ull);
    }
    slot = (long long)t.shfl64((unsigned long long)slot, 0);
    inserted = t.shfl(inserted, 0);
    if (slot < 0) { if (t.i == 0) { atomicMax(&ctl->err, 4u); sc.slot[s] = -1; } continue; }
    bool killed = false;
    unsigned long long nprobe = 0;
    if (!inserted && mode == 0) {
      // the lanes take the stored zones of the chain in turn, each deciding a whole a_LU test
      int Lall[D];
#pragma unroll
      for (int x = 0; x < D; ++x) Lall[x] = t.shfl(Ly, x);
      const int* zs = sc.zone + s * D * D;
      bool mine = false;
      int pos = 0;
      for (int n = __ldg(st.head + slot); n >= 0; n = __ldg(st.nnext + n), ++pos) {
        const int lane_for = pos % D;
        if (lane_for == t.i && !mine && !__ldg(st.ndead + n)) {
          ++nprobe;
          mine = alu_le_lane<D>(zs, st.nzone + (long long)n * D * D, Lall, U);
        }
        if (lane_for == D - 1 && t.any(mine)) break;
      }
      killed = t.any(mine);
    }
    if (nprobe) atomicAdd(&ctl->probes, nprobe);
    if (t.i == 0) {
      if (killed) {
        sc.slot[s] = -1;
      } else {
        const unsigned r = atomicAdd(&st.pend[slot], 1u);
        if (r == 0) sc.touched[atomicAdd(&ctl->ntouched, 1ull)] = (int)slot;
        sc.slot[s] = (int)slot;
        sc.rank[s] = (int)r;
        sc.surv[atomicAdd(&ctl->nsurv, 1ull)] = (int)s;
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// deadlock: the goal test of the deadlock query, on the probe's survivors
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock) k_deadlock(const NetView* nets, InstState is, Succ sc, Ctl* ctl,
                                                     long long nsurv) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  DlScratch<D> S;
  const int ishift = nets[0].inst_shift;
  for (long long w = tile_id<D>(); w < nsurv; w += tile_count<D>()) {
    const int s = sc.surv[w];
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    if (N.kind != 1 || is.found[inst]) continue;
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    int z[D];
    load_rows(t, z, sc.zone + (long long)s * D * D);
    const int r = state_has_deadlock(N, t, locs, ints, z, S);
    if (t.i == 0) {
      if (r < 0) atomicMax(&ctl->err, 4u);
      else if (r == 1) { is.found[inst] = 1; atomicOr(&ctl->found, 1u); }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// group: one contiguous segment of survivors per touched slot
// ---------------------------------------------------------------------------------------------
static __global__ void k_seg_alloc(Succ sc, Store st, Ctl* ctl, long long ntouched) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < ntouched; j += (long long)gridDim.x * blockDim.x) {
    const int s = sc.touched[j];
    st.pend_base[s] = (unsigned)atomicAdd(&ctl->seg_alloc, (unsigned long long)st.pend[s]);
  }
}
static __global__ void k_seg_scatter(Succ sc, Store st, long long nsucc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nsucc; i += (long long)gridDim.x * blockDim.x) {
    const int s = sc.slot[i];
    if (s < 0) continue;
    const unsigned pos = st.pend_base[s] + sc.rank[i];
    sc.seg[pos] = (int)i;
    sc.skh[pos] = sc.okh[i];
    sc.skl[pos] = sc.okl[i];
  }
}

// ---------------------------------------------------------------------------------------------
// merge: NetPassedT::add folds (passed_set.hpp:287-444) per key, in canonical order
// ---------------------------------------------------------------------------------------------

template <int D>
__global__ void __launch_bounds__(kBlock) k_merge(const NetView* nets, InstState is, Front fr, Succ sc, Store st,
                                                  Front out, Ctl* ctl, long long ntouched, int level, int mode,
                                                  Edges ed, int record) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  volatile int* vhead = st.head;
  volatile int* vnext = st.nnext;
  volatile int* vdead = st.ndead;
  volatile int* vlevel = st.nlevel;
  for (long long j = tile_id<D>(); j < ntouched; j += tile_count<D>()) {
    const int s = sc.touched[j];
    const unsigned n = st.pend[s];
    const unsigned base = st.pend_base[s];
    const unsigned long long hk = st.hkey[s];
    const int inst = (int)(hk >> ishift);
    if (is.found[inst] || is.done[inst]) { t.sync(); if (t.i == 0) st.pend[s] = 0; continue; }
    const NetView& N = nets[inst];
    // canonical order: rank every pending survivor by (parent key, parent rank, ordinal)
    for (unsigned e = t.i; e < n; e += D) {
      const unsigned long long kh = sc.skh[base + e], kl = sc.skl[base + e];
      unsigned r = 0;
      for (unsigned q = 0; q < n; ++q) {
        const unsigned long long qh = sc.skh[base + q], ql = sc.skl[base + q];
        r += (qh < kh || (qh == kh && (ql < kl || (ql == kl && q < e)))) ? 1u : 0u;
      }
      sc.sorted[base + r] = sc.seg[base + e];
    }
    // the key's live zones, gathered once into a contiguous list: oldest first, so that the zones
    // this merge stores are appended and a backwards scan is the chain's newest-first order
    long long cb = 0;
    int clen = 0;
    if (t.i == 0) {
      int c = 0;
      for (int m = vhead[s]; m >= 0; m = vnext[m]) c += vdead[m] ? 0 : 1;
      cb = (long long)atomicAdd(&ctl->chain_alloc, (unsigned long long)(c + n));
      if (cb + c + n > sc.ccap) { atomicMax(&ctl->err, 4u); cb = -1; }
      else {
        int k = c;
        for (int m = vhead[s]; m >= 0; m = vnext[m])
          if (!vdead[m]) sc.clist[cb + (--k)] = m;
      }
      clen = c;
    }
    cb = (long long)t.shfl64((unsigned long long)cb, 0);
    clen = t.shfl(clen, 0);
    t.sync();
    if (cb < 0) continue;
    volatile int* cl = sc.clist + cb;
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    int Ly, U[D], Lall[D];
    key_bounds(N, t, locs, Ly, U);
#pragma unroll
    for (int x = 0; x < D; ++x) Lall[x] = t.shfl(Ly, x);
    long long dlive = 0;
    unsigned long long nprobe = 0;
    // store z as a new node of this key and append it to the list
    auto store_new = [&](const int (&z)[D]) -> int {
      long long node = 0;
      if (t.i == 0) node = (long long)atomicAdd(&ctl->nnodes, 1ull);
      node = (long long)t.shfl64((unsigned long long)node, 0);
      store_rows(t, z, st.nzone + node * D * D);
      t.sync();
      if (t.i == 0) {
        const int old_head = vhead[s];
        if (old_head < 0) { atomicAdd(&ctl->nkeys, 1ull); atomicAdd(&is.nkeys[inst], 1ull); }
        st.nnext[node] = old_head;
        st.nlevel[node] = level;
        st.ndead[node] = 0;
        st.ninst[node] = inst;
        st.nkey[node] = hk;
        cl[clen] = (int)node;
        __threadfence_block();
        vhead[s] = (int)node;
      }
      ++clen;
      ++dlive;
      t.sync();
      return (int)node;
    };
    for (unsigned q = 0; q < n; ++q) {
      const int a = ((volatile int*)sc.sorted)[base + q];
      const int* zs = sc.zone + (long long)a * D * D;
      int z[D], z0[D];
      load_rows(t, z, zs);
#pragma unroll
      for (int x = 0; x < D; ++x) z0[x] = t.shfl(z[x], 0);
      if (mode == 1) {
        // exact-zone graph: the lanes compare the list's zones in turn; at most one can be equal
        int mine = -1;
        for (int k = t.i; k < clen; k += D) {
          const int m = cl[k];
          const int* zp = st.nzone + (long long)m * D * D;
          bool eq = true;
          for (int e = 0; e < D * D && eq; ++e) eq = __ldcg(zp + e) == __ldg(zs + e);
          if (eq) { mine = m; break; }
        }
        int hit = -1;
#pragma unroll
        for (int l = 0; l < D; ++l) { const int v = t.shfl(mine, l); hit = v >= 0 ? v : hit; }
        if (hit < 0) hit = store_new(z);
        if (record && t.i == 0) {
          const unsigned long long e = atomicAdd(&ctl->nedges, 1ull);
          if ((long long)e < ed.cap) { ed.src[e] = fr.node[sc.parent[a]]; ed.dst[e] = hit; }
          else atomicMax(&ctl->err, 4u);
        }
        continue;
      }
      // (1)+(2): dropped if a stored zone simulates it. Every zone stored before this level was
      // already tested by the probe, and a stored zone is only ever retired by one that simulates
      // it, so only the zones stored at this level -- the list's tail -- can still drop it.
      bool drop = false;
      for (int k = clen - 1; k >= 0; --k) {
        const int m = cl[k];
        if (m < 0) continue;
        if (vlevel[m] != level) break;
        int zp[D];
        load_rows_rw(t, zp, st.nzone + (long long)m * D * D);
        ++nprobe;
        if (alu_le(t, z, zp, z0, Ly, U)) { drop = true; break; }
      }
      if (drop) continue;
      // (3): retire the stored zones the new one simulates; the lanes take the list in turn
      {
        int retired = 0;
        for (int k = t.i; k < clen; k += D) {
          const int m = cl[k];
          if (m < 0) continue;
          if (alu_le_lane<D>(st.nzone + (long long)m * D * D, zs, Lall, U)) {
            vdead[m] = 1;
            cl[k] = -1;
            ++retired;
          }
        }
        t.sync();
#pragma unroll
        for (int l = 0; l < D; ++l) dlive -= t.shfl(retired, l);
      }
      // (4): convex-union absorb within the newest kMergeScan live zones, restarting after each
      for (bool merged = true; merged;) {
        merged = false;
        int seen = 0;
        for (int k = clen - 1; k >= 0 && seen < kMergeScan; --k) {
          const int m = cl[k];
          if (m < 0) continue;
          ++seen;
          int zp[D];
          load_rows_rw(t, zp, st.nzone + (long long)m * D * D);
          if (try_union(t, z, zp)) {
            t.sync();
            if (t.i == 0) { vdead[m] = 1; cl[k] = -1; }
            --dlive;
            t.sync();
            merged = true;
            break;
          }
        }
      }
      // (5): prepend
      store_new(z);
    }
    // this key's zones stored at this level enter the next frontier, in chain order
    if (t.i == 0) {
      int r = 0;
      for (int k = clen - 1; k >= 0; --k) {
        const int m = cl[k];
        if (m < 0 || vlevel[m] != level) continue;
        const unsigned long long f = atomicAdd(&ctl->nfront, 1ull);
        out.key[f] = hk; out.node[f] = m; out.rank[f] = r++; out.inst[f] = inst;
      }
      if (r) atomicAdd(&is.nfront[inst], (unsigned long long)r);
      if (dlive) {
        atomicAdd((unsigned long long*)&ctl->nlive, (unsigned long long)dlive);
        atomicAdd((unsigned long long*)&is.nlive[inst], (unsigned long long)dlive);
      }
      st.pend[s] = 0;
    }
    if (nprobe) atomicAdd(&ctl->probes, nprobe);
    t.sync();
  }
}

// ---------------------------------------------------------------------------------------------
// leads-to: roots, end-of-run flags, greatest fixpoint
// ---------------------------------------------------------------------------------------------
// Phase-1 nodes whose discrete state satisfies p become the root frontier (one thread per node).
static __global__ void k_collect_p(const NetView* nets, Store st, long long nnodes, Front out, Ctl* ctl) {
  const int ishift = nets[0].inst_shift;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes; n += (long long)gridDim.x * blockDim.x) {
    if (st.ndead[n]) continue;
    const unsigned long long hk = st.nkey[n];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    if (N.kind != 2) continue;
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    if (!pred_disc(N.p_loc, N.p_nloc, N.p_int, N.p_nint, locs, ints)) continue;
    const unsigned long long f = atomicAdd(&ctl->nfront, 1ull);
    // the node id as rank keeps the order keys of one key's roots distinct
    out.key[f] = hk; out.node[f] = (int)n; out.rank[f] = (int)n; out.inst[f] = inst;
  }
}

// stop_set (src/liveness/construction.cpp:1200-1239) of every graph node, as a flag: the node holds
// a valuation whose run may end here.
template <int D>
__global__ void __launch_bounds__(kBlock) k_stop(const NetView* nets, Store st, long long nnodes, int* stop, Ctl* ctl) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  DlScratch<D> S;
  const int ishift = nets[0].inst_shift;
  for (long long n = tile_id<D>(); n < nnodes; n += tile_count<D>()) {
    const unsigned long long hk = st.nkey[n];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    int z[D];
    load_rows(t, z, st.nzone + n * D * D);
    int r = 0;
    if (N.av_nclk == 0) {
      // unrestricted: no successor at all, time divergence, or a deadlocked valuation
      NetView U = N;
      U.av_on = 0;
      int cnt = 0;
      const bool ok = for_each_successor(U, t, locs, ints, z, 1, [&](const int*, const int*, const int (&)[D]) { ++cnt; });
      if (!ok) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
      if (cnt == 0 || time_diverges(N, t, locs, ints, z, false)) r = 1;
      else {
        const int d = state_has_deadlock(N, t, locs, ints, z, S);
        if (d < 0) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
        r = d;
      }
    } else {
      // restricted: divergence inside !q, or a genuine timelock of the unrestricted system
      if (time_diverges(N, t, locs, ints, z, true)) r = 1;
      else if (orig_time_open(N, t, locs, ints)) r = 0;
      else {
        const int d = state_has_deadlock(N, t, locs, ints, z, S);
        if (d < 0) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
        r = d;
      }
    }
    if (t.i == 0) stop[n] = r;
  }
}

// One Jacobi pass of W = W /\ (stop \/ exists edge into W): mark sources with a successor in W...
static __global__ void k_gfp_mark(Edges ed, long long nedges, const int* W, int* F) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nedges; e += (long long)gridDim.x * blockDim.x)
    if (W[ed.dst[e]]) F[ed.src[e]] = 1;
}
// ... then keep a node only if it stops or kept such a successor.
static __global__ void k_gfp_update(long long nnodes, const int* stop, int* W, int* F, Ctl* ctl) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes; n += (long long)gridDim.x * blockDim.x) {
    const int w = W[n] && (stop[n] || F[n]);
    if (w != W[n]) { W[n] = w; ctl->flag = 1; }
    F[n] = 0;
  }
}
// Violated iff a root (a level-0 node of the graph) survives.
static __global__ void k_gfp_verdict(const NetView* nets, Store st, long long nnodes, const int* W, InstState is) {
  const int ishift = nets[0].inst_shift;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes; n += (long long)gridDim.x * blockDim.x)
    if (W[n] && st.nlevel[n] == 0) is.found[(int)(st.nkey[n] >> ishift)] = 1;
}

// ---------------------------------------------------------------------------------------------
// host-buffer entry points: successors and deadlock test of explicit states
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock) k_expand_plain(const NetView* nets, const int* locs_in, const int* ints_in,
                                                         const int* zones, int n, int emode,
                                                         unsigned long long* okey, int* osrc, int* oord, int* olocs,
                                                         int* oints, int* ozones, long long cap, Ctl* ctl) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const NetView& N = nets[0];
  for (long long f = tile_id<D>(); f < n; f += tile_count<D>()) {
    int locs[kMaxProcs], ints[kMaxInts];
    for (int p = 0; p < N.nprocs; ++p) locs[p] = locs_in[f * N.nprocs + p];
    for (int v = 0; v < N.nints; ++v) ints[v] = ints_in[f * N.nints + v];
    int src[D];
    load_rows(t, src, zones + f * D * D);
    int ord = 0;
    const bool ok = for_each_successor(N, t, locs, ints, src, emode, [&](const int* tl, const int* ti, const int (&z)[D]) {
      unsigned long long idx = 0;
      if (t.i == 0) idx = atomicAdd(&ctl->nsucc, 1ull);
      idx = t.shfl64(idx, 0);
      if ((long long)idx < cap) {
        store_rows(t, z, ozones + (long long)idx * D * D);
        if (t.i == 0) {
          okey[idx] = ((unsigned long long)f << 32) | (unsigned)ord;
          osrc[idx] = (int)f;
          oord[idx] = ord;
          for (int p = 0; p < N.nprocs; ++p) olocs[idx * N.nprocs + p] = tl[p];
          for (int v = 0; v < N.nints; ++v) oints[idx * N.nints + v] = ti[v];
        }
      } else if (t.i == 0) {
        ctl->overflow = 1;
      }
      ++ord;
    });
    if (!ok && t.i == 0) atomicMax(&ctl->err, 4u);
  }
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_has_deadlock(const NetView* nets, const int* locs_in, const int* ints_in,
                                                         const int* zones, int n, int* out, Ctl* ctl) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  DlScratch<D> S;
  const NetView& N = nets[0];
  for (long long f = tile_id<D>(); f < n; f += tile_count<D>()) {
    int locs[kMaxProcs], ints[kMaxInts];
    for (int p = 0; p < N.nprocs; ++p) locs[p] = locs_in[f * N.nprocs + p];
    for (int v = 0; v < N.nints; ++v) ints[v] = ints_in[f * N.nints + v];
    int z[D];
    load_rows(t, z, zones + f * D * D);
    const int r = is_empty(t, z) ? 0 : state_has_deadlock(N, t, locs, ints, z, S);
    if (t.i == 0) {
      out[f] = r;
      if (r < 0) atomicMax(&ctl->err, 4u);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
inline int grid_for(long long items, int tiles_per_block, int max_blocks) {
  long long b = (items + tiles_per_block - 1) / tiles_per_block;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

template <int D>
void Level<D>::init(const NetView* nets, int ninst, const int* ok, Store st, Front out, InstState is, Ctl* ctl,
                    cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_init<D><<<grid_for(ninst, TPB, 4096), kBlock, 0, s>>>(nets, ninst, ok, st, out, is, ctl);
}
template <int D>
void Level<D>::expand(const NetView* nets, InstState is, Front fr, int nfront, const int* src_zone, Succ sc,
                      Ctl* ctl, int roots, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_expand<D><<<grid_for(nfront, TPB, blocks), kBlock, 0, s>>>(nets, is, fr, nfront, src_zone, sc, ctl, roots);
}
template <int D>
void Level<D>::probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nsucc, int mode,
                     int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_probe<D><<<grid_for(nsucc, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, st, ctl, nsucc, mode);
}
template <int D>
void Level<D>::deadlock(const NetView* nets, InstState is, Succ sc, Ctl* ctl, long long nsurv, int blocks,
                        cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_deadlock<D><<<grid_for(nsurv, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, ctl, nsurv);
}
template <int D>
void Level<D>::group(Succ sc, Store st, Ctl* ctl, long long nsucc, long long ntouched, cudaStream_t s) {
  k_seg_alloc<<<grid_for(ntouched, 256, 1024), 256, 0, s>>>(sc, st, ctl, ntouched);
  k_seg_scatter<<<grid_for(nsucc, 256, 4096), 256, 0, s>>>(sc, st, nsucc);
}
template <int D>
void Level<D>::merge(const NetView* nets, InstState is, Front fr, Succ sc, Store st, Front out, Ctl* ctl,
                     long long ntouched, int level, int mode, Edges ed, int record, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_merge<D><<<grid_for(ntouched, TPB, blocks), kBlock, 0, s>>>(nets, is, fr, sc, st, out, ctl, ntouched, level,
                                                                mode, ed, record);
}
template <int D>
void Level<D>::collect_p(const NetView* nets, Store st, long long nnodes, Front out, Ctl* ctl, cudaStream_t s) {
  k_collect_p<<<grid_for(nnodes, 256, 4096), 256, 0, s>>>(nets, st, nnodes, out, ctl);
}
template <int D>
void Level<D>::stop(const NetView* nets, Store st, long long nnodes, int* stop, Ctl* ctl, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_stop<D><<<grid_for(nnodes, TPB, blocks), kBlock, 0, s>>>(nets, st, nnodes, stop, ctl);
}
template <int D>
void Level<D>::gfp_pass(Edges ed, long long nedges, long long nnodes, const int* stop, int* W, int* F, Ctl* ctl,
                        cudaStream_t s) {
  if (nedges > 0) k_gfp_mark<<<grid_for(nedges, 256, 8192), 256, 0, s>>>(ed, nedges, W, F);
  k_gfp_update<<<grid_for(nnodes, 256, 8192), 256, 0, s>>>(nnodes, stop, W, F, ctl);
}
template <int D>
void Level<D>::gfp_verdict(const NetView* nets, Store st, long long nnodes, const int* W, InstState is, Ctl* ctl,
                           cudaStream_t s) {
  (void)ctl;
  k_gfp_verdict<<<grid_for(nnodes, 256, 8192), 256, 0, s>>>(nets, st, nnodes, W, is);
}
template <int D>
void Level<D>::expand_plain(const NetView* nets, const int* locs, const int* ints, const int* zones, int n, int emode,
                            unsigned long long* okey, int* osrc, int* oord, int* olocs, int* oints, int* ozones,
                            long long cap, Ctl* ctl, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_expand_plain<D><<<grid_for(n, TPB, 4096), kBlock, 0, s>>>(nets, locs, ints, zones, n, emode, okey, osrc, oord,
                                                                olocs, oints, ozones, cap, ctl);
}
template <int D>
void Level<D>::has_deadlock(const NetView* nets, const int* locs, const int* ints, const int* zones, int n, int* out,
                            Ctl* ctl, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_has_deadlock<D><<<grid_for(n, TPB, 4096), kBlock, 0, s>>>(nets, locs, ints, zones, n, out, ctl);
}

}  // namespace hgb
