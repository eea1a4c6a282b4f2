// level_kernels_impl.cuh -- bodies of the level kernels. Included once per DBM dimension by the
// generated translation units (dim_<D>.cu), which instantiate hgb::Level<D>.
#pragma once
#include <cooperative_groups.h>

#include "level_kernels.cuh"

namespace hgb {

// One index from a shared counter for each calling thread. The threads of a warp that call it
// together take theirs with one atomic: an atomic per successor or survivor on one counter
// serialises in L2.
__device__ __forceinline__ unsigned long long take_index(unsigned long long* counter) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long b = 0;
  if (g.thread_rank() == 0) b = atomicAdd(counter, (unsigned long long)g.size());
  return g.shfl(b, 0) + g.thread_rank();
}


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

// The first goal state of an instance, kept for its trace: the node whose successor it is (or -2 for
// the initial state, or the node itself with raw -1), the transition index, its key and zone.
template <int D>
__device__ __forceinline__ void record_hit(const Tile<D>& t, const InstState& is, int inst, int node, int raw,
                                           unsigned long long hk, const int (&z)[D]) {
  if (!is.hit_node) return;
  int won = 0;
  if (t.i == 0) won = atomicCAS(&is.hit_node[inst], -1, node) == -1;
  won = t.shfl(won, 0);
  if (!won) return;
  store_rows(t, z, is.hit_zone + (long long)inst * D * D);
  if (t.i == 0) { is.hit_raw[inst] = raw; is.hit_key[inst] = hk; }
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
      record_hit(t, is, inst, -2, -1, key_encode(N, locs, ints) | ((unsigned long long)inst << N.inst_shift), z);
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
    st.ncol0[node * D + t.i] = z[0];
    if (t.i == 0) {
      st.nlevel[node] = 0; st.ndead[node] = 0; st.ninst[node] = inst; st.nkey[node] = hk;
      st.npar[node] = -1; st.nraw[node] = -1;
      const long long off = (long long)atomicAdd(&ctl->arena_alloc, 1ull);
      if (off < st.acap) { st.arena[off] = (int)node; st.kloff[slot] = off; st.klive[slot] = 1; }
      else atomicMax(&ctl->err, 4u);
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
                                                   const int* src_zone, Succ sc, Ctl* ctl, int roots, int i0, int i1) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  for (long long f = tile_id<D>(); f < nfront; f += tile_count<D>()) {
    const int inst = fr.inst[f];
    if (inst < i0 || inst >= i1 || is.done[inst]) continue;
    const NetView& N = nets[inst];
    const unsigned long long hk = fr.key[f];
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, N.inst_shift), locs, ints);
    int src[D];
    load_rows(t, src, src_zone + (long long)fr.node[f] * D * D);
    const int emode = is.emode[inst];
    int ord = 0;
    bool hit = false;
    auto emit = [&](const int* tl, const int* ti, const int (&z)[D], int raw) {
      unsigned long long idx = 0;
      if (t.i == 0) idx = take_index(&ctl->nsucc);
      idx = t.shfl64(idx, 0);
      if ((long long)idx < sc.cap) {
        store_rows(t, z, sc.zone + (long long)idx * D * D);
        if (t.i == 0) {
          sc.key[idx] = key_encode(N, tl, ti) | ((unsigned long long)inst << N.inst_shift);
          sc.parent[idx] = (int)f;
          sc.ord[idx] = ord;
          sc.raw[idx] = raw;
          sc.pnode[idx] = fr.node[f];
          sc.okh[idx] = hk;
          sc.okl[idx] = ((unsigned long long)(unsigned)fr.rank[f] << 32) | (unsigned)ord;
        }
      } else if (t.i == 0) {
        ctl->overflow = 1;
      }
      ++ord;
      if (N.kind == 0 && !hit) {
        hit = target_hit(N, t, z, tl, ti);
        if (hit) record_hit(t, is, inst, fr.node[f], raw,
                            key_encode(N, tl, ti) | ((unsigned long long)inst << N.inst_shift), z);
      }
    };
    bool ok = true;
    if (roots) {
      // leads-to roots: the p-part of a phase-1 zone, cut to !q
      if (apply_cons(t, src, N.p_clk, 0, N.p_nclk) && avoid_cut(N, t, src, locs, ints) && !is_empty(t, src))
        emit(locs, ints, src, -1);
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
// At most 64 registers (8 blocks of 128 threads per SM): the scan waits on dependent loads, and the
// extra resident warps hide more of that latency than the spills cost (19% faster on config 2).
template <int D>
__global__ void __launch_bounds__(kBlock, 8) k_probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl,
                                                  long long nsucc, int long_list) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  // the probe counters are summed per lane over the whole loop and added once per tile at the end:
  // one global atomic per lane and successor on the same two counters serialised in L2
  unsigned long long nprobe_sum = 0, nfull_sum = 0;
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
    if (!inserted && __ldg(st.klive + slot) > long_list) {
      // a long list: left to k_probe_long, whose warps test 32 list entries per round
      if (t.i == 0) { sc.slot[s] = (int)slot; sc.longs[take_index(&ctl->nlong)] = (int)s; }
      continue;
    }
    bool killed = false;
    unsigned long long nprobe = 0, nfull = 0;
    if (!inserted) {
      // the lanes take the key's live zones in turn, newest first, each deciding a whole a_LU test
      int Lall[D];
#pragma unroll
      for (int x = 0; x < D; ++x) Lall[x] = t.shfl(Ly, x);
      const int* zs = sc.zone + s * D * D;
      int zc0[D];   // column 0 of the successor: x_y - x_0 bounds
#pragma unroll
      for (int y = 0; y < D; ++y) zc0[y] = t.shfl(z[0], y);
      const int nl = __ldg(st.klive + slot);
      const int* lst = st.arena + __ldg(st.kloff + slot);
      bool mine = false;
      for (int k0 = nl - 1; k0 >= 0 && !killed; k0 -= D) {
        const int k = k0 - t.i;
        if (k >= 0) {
          ++nprobe;
          const int m = __ldg(lst + k);
          // most failing tests fail on column 0: decide those from the stored zone's column copy
          const bool col0_pass = !alu_col0_witness<D>(zc0, st.ncol0 + (long long)m * D, Lall);
          nfull += col0_pass;
          mine = col0_pass && alu_le_lane<D>(zs, st.nzone + (long long)m * D * D, Lall, U);
        }
        killed = t.any(mine);
      }
    }
    nprobe_sum += nprobe;
    nfull_sum += nfull;
    if (t.i == 0) {
      if (killed) {
        sc.slot[s] = -1;
      } else {
        const unsigned r = atomicAdd(&st.pend[slot], 1u);
        if (r == 0) sc.touched[atomicAdd(&ctl->ntouched, 1ull)] = (int)slot;
        sc.slot[s] = (int)slot;
        sc.rank[s] = (int)r;
        sc.surv[take_index(&ctl->nsurv)] = (int)s;
      }
    }
  }
  unsigned long long tp = 0, tf = 0;
#pragma unroll
  for (int l = 0; l < D; ++l) {
    tp += t.shfl64(nprobe_sum, l);
    tf += t.shfl64(nfull_sum, l);
  }
  if (t.i == 0) {
    if (tp) atomicAdd(&ctl->probes, tp);
    if (tf) atomicAdd(&ctl->probe_full, tf);
  }
}

// The probe of the successors whose key has more than long_list live zones, one warp each: the
// warp's 32 lanes take 32 list entries per round (a tile takes D), so a long scan needs a third to a
// sixteenth of the rounds and runs with every lane of the warp busy. Same decisions as k_probe: the
// successor is dropped iff some live zone simulates it; survivors get their rank in the slot's
// pending list. The count of such successors is read on the device (no host round trip).
template <int D>
__global__ void __launch_bounds__(kBlock) k_probe_long(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl) {
  const int lane = threadIdx.x & 31;
  const long long nlong = (long long)*(volatile unsigned long long*)&ctl->nlong;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const int ishift = nets[0].inst_shift;
  unsigned long long nprobe = 0, nfull = 0;
  for (long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nlong; w += nw) {
    const int s = sc.longs[w];
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    const long long slot = sc.slot[s];
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    // per-clock bounds: lane c < D computes clock c's (key_bounds' rule), then every lane takes all
    int l = kAluNegInf, u = kAluNegInf;
    if (lane == 0) {
      l = u = 0;
    } else if (lane < D) {
      for (int p = 0; p < N.nprocs; ++p) {
        const int gl = N.loc_base[p] + locs[p];
        l = max(l, N.Lloc[gl * N.dim + lane]);
        u = max(u, N.Uloc[gl * N.dim + lane]);
      }
      l = max(l, N.Lq[lane]);
      u = max(u, N.Uq[lane]);
    }
    int Lall[D], U[D], zc0[D];
    const int* zs = sc.zone + (long long)s * D * D;
#pragma unroll
    for (int x = 0; x < D; ++x) {
      Lall[x] = __shfl_sync(0xffffffffu, l, x);
      U[x] = __shfl_sync(0xffffffffu, u, x);
      zc0[x] = __ldg(zs + x * D);
    }
    const int nl = __ldg(st.klive + slot);
    const int* lst = st.arena + __ldg(st.kloff + slot);
    bool killed = false;
    for (int k0 = nl - 1; k0 >= 0 && !killed; k0 -= 32) {
      const int k = k0 - lane;
      bool mine = false;
      if (k >= 0) {
        ++nprobe;
        const int m = __ldg(lst + k);
        const bool col0_pass = !alu_col0_witness<D>(zc0, st.ncol0 + (long long)m * D, Lall);
        nfull += col0_pass;
        mine = col0_pass && alu_le_lane<D>(zs, st.nzone + (long long)m * D * D, Lall, U);
      }
      killed = __any_sync(0xffffffffu, mine);
    }
    if (lane == 0) {
      if (killed) {
        sc.slot[s] = -1;
      } else {
        const unsigned r = atomicAdd(&st.pend[slot], 1u);
        if (r == 0) sc.touched[atomicAdd(&ctl->ntouched, 1ull)] = (int)slot;
        sc.rank[s] = (int)r;
        sc.surv[take_index(&ctl->nsurv)] = s;
      }
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    nprobe += __shfl_xor_sync(0xffffffffu, nprobe, o);
    nfull += __shfl_xor_sync(0xffffffffu, nfull, o);
  }
  if (lane == 0) {
    if (nprobe) atomicAdd(&ctl->probes, nprobe);
    if (nfull) atomicAdd(&ctl->probe_full, nfull);
  }
}

// ---------------------------------------------------------------------------------------------
// deadlock: the goal test of the deadlock query, on every successor of the level (all = 1) or on
// the probe's survivors
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kBlock) k_deadlock(const NetView* nets, InstState is, Succ sc, Ctl* ctl,
                                                     long long n, int all) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  DlScratch<D> S;
  const int ishift = nets[0].inst_shift;
  for (long long w = tile_id<D>(); w < n; w += tile_count<D>()) {
    const int s = all ? (int)w : sc.surv[w];
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    if (N.kind != 1 || is.found[inst]) continue;
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    int z[D];
    load_rows(t, z, sc.zone + (long long)s * D * D);
    const int r = state_has_deadlock(N, t, locs, ints, z, S);
    if (r == 1) record_hit(t, is, inst, sc.pnode[s], sc.raw[s], hk, z);
    if (t.i == 0) {
      if (r < 0) atomicMax(&ctl->err, 4u);
      else if (r == 1) { is.found[inst] = 1; atomicOr(&ctl->found, 1u); }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// group: one contiguous segment of survivors per touched slot; keys whose merge is long (many
// survivors against a long antichain) go to the block-wide merge, the rest to the tile merge
// ---------------------------------------------------------------------------------------------
constexpr long long kHeavyMerge = 512;    // survivors x (live zones + survivors) of a block-wide key
constexpr int kRelMaxN = 1 << 16;         // larger keys fold without precomputed relations

// Words of a heavy key's relation block (layout at k_heavy_prep).
__device__ __forceinline__ long long rel_words(long long n, long long a) {
  return 3 * n + n * ((n + 31) / 32 + (a + 31) / 32);
}

static __global__ void k_seg_alloc(Succ sc, Store st, Ctl* ctl, long long ntouched) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < ntouched; j += (long long)gridDim.x * blockDim.x) {
    const int s = sc.touched[j];
    const unsigned n = st.pend[s];
    st.pend_base[s] = (unsigned)atomicAdd(&ctl->seg_alloc, (unsigned long long)n);
    const int a = st.klive[s];
    atomicAdd(&ctl->merge_live, (unsigned long long)a);
    if (n >= 2 && (long long)n * ((long long)a + n) >= kHeavyMerge) {
      const unsigned long long j = atomicAdd(&ctl->nheavy, 1ull);
      sc.heavy[j] = s;
      sc.hv.n[j] = (int)n;
      sc.hv.a[j] = a;
      sc.hv.cb[j] = -1;
      sc.hv.bm[j] = n <= (unsigned)kRelMaxN
                        ? (long long)atomicAdd(&ctl->bm_need, (unsigned long long)rel_words(n, a)) : -1;
    } else {
      sc.light[atomicAdd(&ctl->nlight, 1ull)] = s;
    }
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
//
// Per touched key: rank its survivors by the order key (parent key, parent rank, ordinal), gather
// its live zones into a list (oldest first; the zones this merge stores are appended, so a
// backwards scan is newest-first chain order), then for each survivor in order:
//   (1)+(2) drop it if a zone stored at this level simulates it -- every older zone was already
//           tried by the probe, and a stored zone is only retired by one that simulates it;
//   (3)     retire the stored zones it simulates;
//   (4)     absorb the newest convex-union partner among the newest kMergeScan live zones, and
//           repeat with the hull until none is left;
//   (5)     store it.
// Finally the key's zones stored at this level go to the next frontier in chain order and the
// key's chain is relinked through its live zones only.
// ---------------------------------------------------------------------------------------------
constexpr int kMergeBlock = 256;
constexpr int kMergeBlockWide = 512;
// A heavy key's fold tests its union window (kMergeScan candidates) and its open hulls on every tile
// of its block at once. Where a 256-thread block holds fewer tiles than the window (D >= 9: 3 or
// fewer tiles per warp), a single query's merge runs in blocks of 512 threads, one per SM, which
// cover the window in one round (config 2, D = 9: the merge 0.37 s -> 0.32 s per query). At D <= 8
// the 256-thread block already does, and twice the blocks keep twice the heavy keys folding (config
// 3, D = 7: 512 threads made the merge 1.5x slower); the batched form keeps 256-thread blocks.
template <int D>
constexpr bool wide_fold_pays() { return (kMergeBlock / 32) * (32 / D) < kMergeScan; }

// Z ≼_aLU Zp decided by one thread from whole matrices behind plain pointers (global or shared).
template <int D>
__device__ __forceinline__ bool alu_le_ptr(const int* Z, const int* Zp, const int (&L)[D], const int (&U)[D]) {
#pragma unroll
  for (int x = 0; x < D; ++x) {
    if (U[x] == kAluNegInf) continue;
    const int z0x = Z[x];
    if (z0x < r_le(-U[x])) continue;
#pragma unroll
    for (int y = 0; y < D; ++y) {
      if (y == x || L[y] == kAluNegInf) continue;
      const int zp = Zp[y * D + x];
      if (zp < Z[y * D + x] && r_add(zp, r_lt(-L[y])) < z0x) return false;
    }
  }
  return true;
}

// The x = 0 part of alu_le_ptr from the two zones' column 0 alone: true when it already shows that
// Z is not simulated by Zp (most failing tests end here, as in the probe).
template <int D>
__device__ __forceinline__ bool alu_col0_fails(const int (&z0c)[D], const int (&zp0c)[D], const int (&L)[D],
                                               const int (&U)[D]) {
  if (U[0] == kAluNegInf || z0c[0] < r_le(-U[0])) return false;
  bool w = false;
#pragma unroll
  for (int y = 1; y < D; ++y) {
    if (L[y] == kAluNegInf) continue;
    w |= zp0c[y] < z0c[y] && r_add(zp0c[y], r_lt(-L[y])) < z0c[0];
  }
  return w;
}

// Canonical rank of every survivor of a segment; threads [tid, n) step `stride`.
__device__ __forceinline__ void rank_segment(const Succ& sc, unsigned base, unsigned n, unsigned tid, unsigned stride) {
  for (unsigned e = tid; e < n; e += stride) {
    const unsigned long long kh = sc.skh[base + e], kl = sc.skl[base + e];
    unsigned r = 0;
    for (unsigned q = 0; q < n; ++q) {
      const unsigned long long qh = sc.skh[base + q], ql = sc.skl[base + q];
      r += (qh < kh || (qh == kh && (ql < kl || (ql == kl && q < e)))) ? 1u : 0u;
    }
    sc.sorted[base + r] = sc.seg[base + e];
  }
}

// Room in clist for the key's live zones and its survivors (one thread). Returns the offset, or -1
// on overflow; the caller copies the key's list there.
__device__ __forceinline__ long long alloc_clist(const Succ& sc, const Store& st, int s, unsigned n, Ctl* ctl) {
  const int c = st.klive[s];
  const long long cb = (long long)atomicAdd(&ctl->chain_alloc, (unsigned long long)(c + n));
  if (cb + c + n > sc.ccap) { atomicMax(&ctl->err, 4u); return -1; }
  return cb;
}

// End of a key's merge (one thread): frontier entries (contiguous, newest first), live-only chain,
// counters.
__device__ __forceinline__ void finish_key(const Succ& sc, const Store& st, const Front& out, const InstState& is,
                                           Ctl* ctl, int s, unsigned long long hk, int inst, const int* cl,
                                           int clen0, int clen, long long dlive) {
  int nnew = 0;
  for (int k = clen0; k < clen; ++k) nnew += cl[k] >= 0 ? 1 : 0;
  if (nnew) {
    const unsigned long long f0 = atomicAdd(&ctl->nfront, (unsigned long long)nnew);
    int r = 0;
    for (int k = clen - 1; k >= clen0; --k) {
      const int m = cl[k];
      if (m < 0) continue;
      const unsigned long long f = f0 + r;
      out.key[f] = hk; out.node[f] = m; out.rank[f] = r++; out.inst[f] = inst;
    }
    atomicAdd(&is.nfront[inst], (unsigned long long)nnew);
  }
  const bool was_empty = st.klive[s] == 0;
  int live = 0;
  for (int k = 0; k < clen; ++k) live += cl[k] >= 0 ? 1 : 0;
  const long long off = (long long)atomicAdd(&ctl->arena_alloc, (unsigned long long)live);
  if (off + live > st.acap) {
    atomicMax(&ctl->err, 4u);
  } else {
    int w = 0;
    for (int k = 0; k < clen; ++k)
      if (cl[k] >= 0) st.arena[off + (w++)] = cl[k];
    st.kloff[s] = off;
    st.klive[s] = live;
  }
  if (was_empty && live > 0) { atomicAdd(&ctl->nkeys, 1ull); atomicAdd(&is.nkeys[inst], 1ull); }
  if (dlive) {
    atomicAdd((unsigned long long*)&ctl->nlive, (unsigned long long)dlive);
    atomicAdd((unsigned long long*)&is.nlive[inst], (unsigned long long)dlive);
  }
  st.pend[s] = 0;
}

// New node for zone rows `z` of key hk (metadata only; the caller writes the zone).
__device__ __forceinline__ void node_meta(const Store& st, long long node, int level, int inst, unsigned long long hk,
                                          int par, int raw) {
  st.nlevel[node] = level;
  st.ndead[node] = 0;
  st.ninst[node] = inst;
  st.nkey[node] = hk;
  st.npar[node] = par;
  st.nraw[node] = raw;
}

// The heavy fold keeps the liveness of the newest kRing list positions in shared memory, so the
// scan for the union window reads no list entries from memory unless the window reaches further
// back.
constexpr int kRing = 256;
constexpr int kHullList = 1024;   // open hull tests one survivor decides tile-wide

template <int D>
struct MergeShared {
  int zbuf[2][D * D];   // the survivor being added (becomes the hull on a union), double-buffered
  long long node_base;  // node ids reserved for the key's stored zones
  int L[D], U[D];       // the key's per-clock bounds
  int win[kMergeScan];  // list positions of the newest live zones, newest first
  long long cb;
  int nw, best, node, retired, clen, job, unioned, nhull, nkeep;
  int hcomp;                   // hull count after the last compaction of the hull list
  int hl_n;                    // live hulls whose column 0 leaves a test with s_q open
  int hl_u[kHullList];         // their list positions (past the old zones)
  int hl_f[kHullList];         // bit 0: s_q <= hull open, bit 1: hull <= s_q open, bit 2: hull retired
  // The first kHC entries of the hull list (list positions and the zones' column 0), and the
  // liveness of every position this fold stores (bit u: position clen0 + u), so the hull screen
  // reads no memory outside the block.
  static constexpr int kHC = (16384 / (4 * (D + 1))) < 1024 ? (16384 / (4 * (D + 1))) : 1024;
  int hpos[kHC];
  int hcol[kHC * D];
  unsigned ulive[kRelMaxN / 32];
  unsigned lbits[kRing / 32];  // liveness of list positions [clen - kRing, clen), bit p % kRing
  int wsum[64];         // per-warp sums of the block-wide finish
  long long scal[4];    // its frontier base, arena offset, live and new counts
};

// ---------------------------------------------------------------------------------------------
// Keys merged block-wide ("heavy"): their pairwise a_LU relations are precomputed by a grid-wide
// pass, so the ordered fold reads its drop and retire decisions from bitmaps.
//
// Relation block of heavy key j at pool + hv.bm[j] (n survivors in canonical order, a live zones
// before the level):
//   drop[n]      1 if s_q ≼ s_q' for some q' < q
//   tpos[n]      list position (past the old zones) where s_q was stored unchanged, else -1
//   hull[n]      list positions of zones stored as convex hulls (the first nhull entries)
//   rt[n][rtw]   bit q' of row q: s_q' ≼ s_q, q' < q              (rtw = ceil(n / 32))
//   r0[n][r0w]   bit m of row q: old zone m ≼ s_q                  (r0w = ceil(a / 32))
// Why drop[] decides the fold's first test exactly: if s_q ≼ s_q' for an earlier q', then s_q'
// was stored (and a zone stored this level that simulates it is still live: zones only die when
// a later one simulates or contains them), or s_q' was dropped because such a zone simulated it;
// simulation is transitive, so s_q is dropped either way. Conversely a live zone stored this
// level that simulates s_q is either some s_q' stored unchanged (then drop[q] is set) or a hull,
// which the fold tests directly.
// ---------------------------------------------------------------------------------------------

// Canonical order of a long segment by one block: chunks of kSortChunk entries are bitonic-sorted in
// shared memory and written back in place (keys and successor indices), then every entry's final
// rank is its rank in its chunk plus, per other chunk, the number of smaller keys (binary search).
// The order keys of one segment are distinct (parent key, parent rank, emission ordinal).
constexpr int kSortChunk = 1024;

__device__ __forceinline__ bool ok_less(unsigned long long ah, unsigned long long al, unsigned long long bh,
                                        unsigned long long bl) {
  return ah < bh || (ah == bh && al < bl);
}

static __device__ void sort_segment_block(const Succ& sc, unsigned base, unsigned n) {
  __shared__ unsigned long long skh[kSortChunk], skl[kSortChunk];
  __shared__ int sv[kSortChunk];
  const unsigned nc = (n + kSortChunk - 1) / kSortChunk;
  for (unsigned c = 0; c < nc; ++c) {
    const unsigned c0 = c * kSortChunk, len = min((unsigned)kSortChunk, n - c0);
    for (unsigned e = threadIdx.x; e < kSortChunk; e += blockDim.x) {
      if (e < len) { skh[e] = sc.skh[base + c0 + e]; skl[e] = sc.skl[base + c0 + e]; sv[e] = sc.seg[base + c0 + e]; }
      else { skh[e] = ~0ull; skl[e] = ~0ull; sv[e] = -1; }
    }
    __syncthreads();
    for (unsigned k = 2; k <= (unsigned)kSortChunk; k <<= 1)
      for (unsigned jj = k >> 1; jj > 0; jj >>= 1) {
        for (unsigned i = threadIdx.x; i < (unsigned)kSortChunk; i += blockDim.x) {
          const unsigned l = i ^ jj;
          if (l > i) {
            const bool up = (i & k) == 0;
            const bool gt = ok_less(skh[l], skl[l], skh[i], skl[i]);
            if (gt == up) {
              const unsigned long long th = skh[i], tl = skl[i];
              const int tv = sv[i];
              skh[i] = skh[l]; skl[i] = skl[l]; sv[i] = sv[l];
              skh[l] = th; skl[l] = tl; sv[l] = tv;
            }
          }
        }
        __syncthreads();
      }
    for (unsigned e = threadIdx.x; e < len; e += blockDim.x) {
      sc.skh[base + c0 + e] = skh[e]; sc.skl[base + c0 + e] = skl[e]; sc.seg[base + c0 + e] = sv[e];
    }
    __syncthreads();
  }
  for (unsigned p = threadIdx.x; p < n; p += blockDim.x) {
    const unsigned c = p / kSortChunk;
    const unsigned long long kh = sc.skh[base + p], kl = sc.skl[base + p];
    unsigned r = p - c * kSortChunk;
    for (unsigned o = 0; o < nc; ++o) {
      if (o == c) continue;
      unsigned lo = o * kSortChunk, hi = min((o + 1) * kSortChunk, n);   // first entry not less than key
      while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (ok_less(sc.skh[base + mid], sc.skl[base + mid], kh, kl)) lo = mid + 1; else hi = mid;
      }
      r += lo - o * kSortChunk;
    }
    sc.sorted[base + r] = sc.seg[base + p];
  }
}

// Sort the key's survivors, gather its live list, its bounds, and clear its relation block.
template <int D>
__global__ void __launch_bounds__(kMergeBlock) k_heavy_prep(const NetView* nets, InstState is, Succ sc, Store st,
                                                            Ctl* ctl, long long nheavy, const int* order) {
  Tile<D> t;
  const bool in_tile = make_tile(t, threadIdx.x & 31);
  const int ishift = nets[0].inst_shift;
  for (long long jj = blockIdx.x; jj < nheavy; jj += gridDim.x) {
    const long long j = order ? order[jj] : jj;
    const int s = sc.heavy[j];
    const unsigned long long hk = st.hkey[s];
    const int inst = (int)(hk >> ishift);
    if (is.found[inst] || is.done[inst]) continue;
    const int n = sc.hv.n[j], a = sc.hv.a[j];
    const unsigned base = st.pend_base[s];
    if (n <= 128) rank_segment(sc, base, (unsigned)n, threadIdx.x, blockDim.x);
    else sort_segment_block(sc, base, (unsigned)n);
    __shared__ long long cb_sh;
    if (threadIdx.x == 0) { cb_sh = alloc_clist(sc, st, s, (unsigned)n, ctl); sc.hv.cb[j] = cb_sh; }
    __syncthreads();
    const long long cb = cb_sh;
    if (cb >= 0) {
      const int* lst = st.arena + st.kloff[s];
      for (int k = threadIdx.x; k < a; k += blockDim.x) sc.clist[cb + k] = lst[k];
    }
    if (threadIdx.x < 32 && in_tile && t.base == 0) {
      int locs[kMaxProcs], ints[kMaxInts];
      key_decode(nets[inst], key_part(hk, ishift), locs, ints);
      int Ly, U[D];
      key_bounds(nets[inst], t, locs, Ly, U);
      sc.hv.bounds[j * 2 * D + t.i] = Ly;
      sc.hv.bounds[j * 2 * D + D + t.i] = U[t.i];
    }
    const long long bm = sc.hv.bm[j];
    if (bm >= 0) {
      unsigned* R = sc.hv.pool + bm;
      const long long w = rel_words(n, a);
      for (long long k = threadIdx.x; k < w; k += blockDim.x) R[k] = (k >= n && k < 2LL * n) ? 0xffffffffu : 0u;
    }
    __syncthreads();
  }
}

// One 32 x 32 tile of pairs per block iteration: survivors x earlier survivors, or survivors x old
// zones. Zones are staged in shared memory (row stride made odd against bank conflicts); lane c of
// a warp tests column c against the warp's rows and a ballot writes the 32 relation bits at once.
template <int D>
__global__ void __launch_bounds__(kMergeBlock) k_heavy_pairs(const NetView* nets, Succ sc, Store st,
                                                             const long long* prefix, long long nheavy,
                                                             long long ntiles) {
  constexpr int Z2 = D * D;
  constexpr int P = (Z2 & 1) ? Z2 : Z2 + 1;
  extern __shared__ int smz[];
  int* A = smz;            // 32 survivors (rows)
  int* B = smz + 32 * P;   // 32 columns
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (long long tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
    long long lo = 0, hi = nheavy;   // prefix[lo] <= tt < prefix[lo + 1]
    while (hi - lo > 1) {
      const long long mid = (lo + hi) >> 1;
      if (prefix[mid] <= tt) lo = mid; else hi = mid;
    }
    const long long j = lo;
    const int n = sc.hv.n[j], a = sc.hv.a[j];
    const long long bm = sc.hv.bm[j], cb = sc.hv.cb[j];
    const int s = sc.heavy[j];
    const unsigned base = st.pend_base[s];
    const long long bq = (n + 31) / 32, ba = (a + 31) / 32, ss = bq * (bq + 1) / 2;
    const long long u = tt - prefix[j];
    long long bi, bj;
    const bool pairs_ss = u < ss;
    if (pairs_ss) {
      bi = (long long)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
      while (bi * (bi + 1) / 2 > u) --bi;
      while ((bi + 1) * (bi + 2) / 2 <= u) ++bi;
      bj = u - bi * (bi + 1) / 2;
    } else {
      const long long v = u - ss;
      bi = v / ba;
      bj = v % ba;
    }
    const bool skip = bm < 0 || cb < 0;
    if (!skip) {
      for (int e = threadIdx.x; e < 32 * Z2; e += blockDim.x) {
        const int r = e / Z2, k = e - r * Z2;
        const long long q = bi * 32 + r;
        if (q < n) A[r * P + k] = sc.zone[(long long)sc.sorted[base + q] * Z2 + k];
        const long long c = bj * 32 + r;
        if (pairs_ss) {
          if (c < n) B[r * P + k] = sc.zone[(long long)sc.sorted[base + c] * Z2 + k];
        } else if (c < a) {
          B[r * P + k] = st.nzone[(long long)sc.clist[cb + c] * Z2 + k];
        }
      }
    }
    __syncthreads();
    if (!skip) {
      int L[D], U[D];
#pragma unroll
      for (int x = 0; x < D; ++x) { L[x] = sc.hv.bounds[j * 2 * D + x]; U[x] = sc.hv.bounds[j * 2 * D + D + x]; }
      unsigned* R = sc.hv.pool + bm;
      const long long rtw = bq, r0w = ba;
      unsigned* drop = R;
      unsigned* rt = R + 3LL * n;
      unsigned* r0 = rt + (long long)n * rtw;
      for (int r = warp; r < 32; r += nwarps) {
        const long long q = bi * 32 + r;
        if (q >= n) continue;   // warp-uniform
        const long long c = bj * 32 + lane;
        if (pairs_ss) {
          const bool ok = c < q;
          const bool dq = ok && alu_le_ptr<D>(A + r * P, B + lane * P, L, U);   // s_q ≼ s_c
          const unsigned bd = __ballot_sync(0xffffffffu, dq);
          if (bd) {
            // s_q is dropped, so the fold never reads its retire row: the reverse tests are skipped
            if (lane == 0) drop[q] = 1u;
          } else {
            const bool rq = ok && alu_le_ptr<D>(B + lane * P, A + r * P, L, U);   // s_c ≼ s_q
            const unsigned br = __ballot_sync(0xffffffffu, rq);
            if (lane == 0 && br) rt[q * rtw + bj] = br;
          }
        } else {
          const bool rq = c < a && alu_le_ptr<D>(B + lane * P, A + r * P, L, U);   // old zone c ≼ s_q
          const unsigned br = __ballot_sync(0xffffffffu, rq);
          if (lane == 0 && br) r0[q * r0w + bj] = br;
        }
      }
    }
    __syncthreads();
  }
}

// End of a block-wide key merge, by the whole block: the key's zones stored at this level go to
// the frontier ranked newest first (contiguous, so the next expand sees a key's zones together),
// and its live zones (oldest first) to a fresh arena list.
static __device__ void finish_key_block(const Store& st, const Front& out, const InstState& is, Ctl* ctl, int s,
                                        unsigned long long hk, int inst, int clen0, int clen, long long dlive,
                                        const int* cl, int* wsum, long long* scal) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  int nall = 0, nnew = 0;
  for (int k = tid; k < clen; k += blockDim.x)
    if (cl[k] >= 0) { ++nall; nnew += k >= clen0 ? 1 : 0; }
  for (int o = 16; o; o >>= 1) {
    nall += __shfl_xor_sync(0xffffffffu, nall, o);
    nnew += __shfl_xor_sync(0xffffffffu, nnew, o);
  }
  if (lane == 0) { wsum[warp] = nall; wsum[32 + warp] = nnew; }
  __syncthreads();
  if (tid == 0) {
    int ta = 0, tn = 0;
    for (int w = 0; w < nwarp; ++w) { ta += wsum[w]; tn += wsum[32 + w]; }
    scal[0] = tn ? (long long)atomicAdd(&ctl->nfront, (unsigned long long)tn) : 0;
    if (tn) atomicAdd(&is.nfront[inst], (unsigned long long)tn);
    const bool was_empty = st.klive[s] == 0;
    const long long off = (long long)atomicAdd(&ctl->arena_alloc, (unsigned long long)ta);
    const bool ok = off + ta <= st.acap;
    if (!ok) atomicMax(&ctl->err, 4u);
    scal[1] = ok ? off : -1;
    scal[2] = ta;
    scal[3] = tn;
    if (ok) { st.kloff[s] = off; st.klive[s] = ta; }
    if (was_empty && ta > 0) { atomicAdd(&ctl->nkeys, 1ull); atomicAdd(&is.nkeys[inst], 1ull); }
    if (dlive) {
      atomicAdd((unsigned long long*)&ctl->nlive, (unsigned long long)dlive);
      atomicAdd((unsigned long long*)&is.nlive[inst], (unsigned long long)dlive);
    }
    st.pend[s] = 0;
  }
  __syncthreads();
  const long long f0 = scal[0], off = scal[1];
  const int ta = (int)scal[2], tn = (int)scal[3], nold = ta - tn;
  int carry = 0;   // live entries before the current chunk
  for (int c0 = 0; c0 < clen; c0 += blockDim.x) {
    const int k = c0 + tid;
    const int m = k < clen ? cl[k] : -1;
    const bool live = m >= 0;
    const unsigned b = __ballot_sync(0xffffffffu, live);
    if (lane == 0) wsum[warp] = __popc(b);
    __syncthreads();
    int before = carry + __popc(b & ((1u << lane) - 1u));
    for (int w = 0; w < nwarp; ++w) {
      if (w < warp) before += wsum[w];
      carry += wsum[w];
    }
    if (live) {
      if (off >= 0) st.arena[off + before] = m;
      if (k >= clen0) {
        const int r = tn - 1 - (before - nold);
        const long long f = f0 + r;
        out.key[f] = hk; out.node[f] = m; out.rank[f] = r; out.inst[f] = inst;
      }
    }
    __syncthreads();
  }
}

// One heavy key merged by a whole block, in canonical order (sorted and gathered by k_heavy_prep).
template <int D>
__device__ void merge_key_block(const NetView* nets, const InstState& is, const Succ& sc, const Store& st,
                                const Front& out, Ctl* ctl, long long j, int level, bool in_tile, const Tile<D>& t,
                                MergeShared<D>& sh) {
  constexpr int TPW = 32 / D;
  constexpr int DD = D * D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ishift = nets[0].inst_shift;
  const int s = sc.heavy[j];
  const unsigned base = st.pend_base[s];
  const unsigned long long hk = st.hkey[s];
  const int inst = (int)(hk >> ishift);
  if (is.found[inst] || is.done[inst]) {
    __syncthreads();
    if (tid == 0) st.pend[s] = 0;
    return;
  }
  const unsigned n = (unsigned)sc.hv.n[j];
  const int a = sc.hv.a[j];
  const long long cb = sc.hv.cb[j], bm = sc.hv.bm[j];
  if (cb < 0) { __syncthreads(); return; }
  if (tid == 0) { sh.clen = a; sh.retired = 0; sh.nhull = 0; sh.hcomp = 0; sh.hl_n = 0; }
  for (int w = tid; w < kRing / 32; w += blockDim.x) sh.lbits[w] = 0u;
  if (bm >= 0)
    for (int w = tid; w < (int)((n + 31) / 32); w += blockDim.x) sh.ulive[w] = 0u;
  // node ids for every survivor that can be stored (the relations' drops excluded), reserved at once
  if (warp == 0) {
    int keep = 0;
    for (unsigned q0 = 0; q0 < n; q0 += 32)
      keep += __popc(__ballot_sync(0xffffffffu, q0 + lane < n && !(bm >= 0 && sc.hv.pool[bm + q0 + lane])));
    if (lane == 0) sh.node_base = keep ? (long long)atomicAdd(&ctl->nnodes, (unsigned long long)keep) : 0;
    if (lane == 0) sh.nkeep = keep;
  }
  int Lr[D], Ur[D];
#pragma unroll
  for (int x = 0; x < D; ++x) { Lr[x] = sc.hv.bounds[j * 2 * D + x]; Ur[x] = sc.hv.bounds[j * 2 * D + D + x]; }
  __syncthreads();
  int* cl = sc.clist + cb;
  const int clen0 = a;
  for (int k = (a > kRing ? a - kRing : 0) + tid; k < a; k += blockDim.x)   // read after the first survivor's barrier
    if (cl[k] >= 0) atomicOr(&sh.lbits[(k & (kRing - 1)) >> 5], 1u << (k & 31));
  const bool rel = bm >= 0;
  unsigned* R = rel ? sc.hv.pool + bm : nullptr;
  const long long rtw = ((long long)n + 31) / 32, r0w = ((long long)a + 31) / 32;
  unsigned* drop = R;
  int* tpos = rel ? (int*)(R + n) : nullptr;
  int* hull = rel ? (int*)(R + 2LL * n) : nullptr;
  const unsigned* rt = rel ? R + 3LL * n : nullptr;
  const unsigned* r0 = rel ? rt + (long long)n * rtw : nullptr;
  long long dlive = 0;   // meaningful on thread 0
  const int tile_idx = warp * TPW + lane / D, ntiles = (blockDim.x >> 5) * TPW;
  const long long node_base = sh.node_base;
  int used = 0, cur = 0;
  // survivor q + 1's drop flag and successor index, loaded during survivor q
  unsigned pf_q = 0xffffffffu, pf_drop = 0;
  int pf_as = 0;
  for (unsigned q = 0; q < n; ++q) {
    unsigned dq;
    int a_s;
    if (q == pf_q) { dq = pf_drop; a_s = pf_as; }
    else { dq = rel ? drop[q] : 0u; a_s = sc.sorted[base + q]; }
    if (dq) continue;   // every thread reads the same word: uniform
    int* const zc = sh.zbuf[cur];
    cur ^= 1;
    for (int e = tid; e < DD; e += blockDim.x) zc[e] = sc.zone[(long long)a_s * DD + e];
    if (tid == 0) sh.unioned = 0;
    __syncthreads();
    if (q + 1 < n) {
      pf_q = q + 1;
      pf_drop = rel ? drop[q + 1] : 0u;
      pf_as = sc.sorted[base + q + 1];
    }
    const int clen = sh.clen;
    int nhull = sh.nhull;
    // The hull list only grows, and hulls die (retired, or absorbed into a newer hull): when it has
    // doubled since its last compaction, the block drops its dead entries (order kept).
    if (rel && nhull >= 256 && nhull >= 2 * sh.hcomp) {
      int carry = 0;
      for (int c0 = 0; c0 < nhull; c0 += blockDim.x) {
        const int h = c0 + tid;
        const int u = h < nhull ? (h < MergeShared<D>::kHC ? sh.hpos[h] : hull[h]) : 0;
        const bool live = h < nhull && ((sh.ulive[u >> 5] >> (u & 31)) & 1u);
        int col[D];
        if (live) {
#pragma unroll
          for (int y = 0; y < D; ++y)
            col[y] = h < MergeShared<D>::kHC ? sh.hcol[h * D + y] : __ldcg(st.ncol0 + (node_base + u) * D + y);
        }
        const unsigned b = __ballot_sync(0xffffffffu, live);
        if (lane == 0) sh.wsum[warp] = __popc(b);
        __syncthreads();
        int before = carry + __popc(b & ((1u << lane) - 1u));
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
          if (w < warp) before += sh.wsum[w];
          carry += sh.wsum[w];
        }
        __syncthreads();   // every entry of this chunk is read before any is overwritten
        if (live) {   // before <= h: entries of later chunks stay untouched
          hull[before] = u;
          if (before < MergeShared<D>::kHC) {
            sh.hpos[before] = u;
#pragma unroll
            for (int y = 0; y < D; ++y) sh.hcol[before * D + y] = col[y];
          }
        }
      }
      __syncthreads();
      if (tid == 0) { sh.nhull = carry; sh.hcomp = carry; }
      nhull = carry;
    }
    // (1)+(2): with relations only the hulls stored this level remain to test; without, every
    // zone stored this level
    bool dropped = false;
    // A zone stored at position clen0 + u of this fold has node id node_base + u, so a hull's zone,
    // column copy and liveness load without going through the list. Both directions against the
    // live hulls are decided before the barrier: s_q dropped by a hull, or (step 3) a hull that s_q
    // simulates. Nothing changes a hull's liveness between the two steps, so this is the same
    // decision as testing them one after the other. Stage A (a thread per hull entry) settles most
    // tests from the two column-0 copies and lists the live hulls where a direction stays open;
    // stage B (a tile per listed hull) loads its rows at once and decides the open directions. The
    // retire rows' first words load here too.
    unsigned w0 = 0, wt = 0;
    const long long wq = ((long long)q + 31) / 32;
    int nl = 0;
    if (rel) {
      if (tid < r0w) w0 = r0[(long long)q * r0w + tid];
      if (tid < wq) wt = rt[(long long)q * rtw + tid];
      if (nhull > 0) {
        int zq0[D];   // column 0 of s_q
#pragma unroll
        for (int y = 0; y < D; ++y) zq0[y] = zc[y * D];
        auto list_open = [&](int u, const int (&c)[D]) {
          const int f = (alu_col0_fails<D>(zq0, c, Lr, Ur) ? 0 : 1) | (alu_col0_fails<D>(c, zq0, Lr, Ur) ? 0 : 2);
          if (!f) return;
          const int e = atomicAdd(&sh.hl_n, 1);
          if (e < kHullList) { sh.hl_u[e] = u; sh.hl_f[e] = f; }
        };
        constexpr int kHC = MergeShared<D>::kHC;
        const int ncached = nhull < kHC ? nhull : kHC;
        for (int h = tid; h < ncached; h += blockDim.x) {   // cached entries: shared memory only
          const int u = sh.hpos[h];
          if (!((sh.ulive[u >> 5] >> (u & 31)) & 1u)) continue;
          int c[D];
#pragma unroll
          for (int y = 0; y < D; ++y) c[y] = sh.hcol[h * D + y];
          list_open(u, c);
        }
        for (int h = kHC + tid; h < nhull; h += blockDim.x) {   // the rest: positions and columns from memory
          const int u = hull[h];
          if (!((sh.ulive[u >> 5] >> (u & 31)) & 1u)) continue;
          int c[D];
#pragma unroll
          for (int y = 0; y < D; ++y) c[y] = __ldcg(st.ncol0 + (node_base + u) * D + y);
          list_open(u, c);
        }
        __syncthreads();
        nl = sh.hl_n;
        if (nl <= kHullList) {
          if (in_tile) {
            int z0q[D];   // row 0 of s_q
#pragma unroll
            for (int x = 0; x < D; ++x) z0q[x] = zc[x];
            const int Ly = sel(Lr, t.i);
            int za[D];
#pragma unroll
            for (int x = 0; x < D; ++x) za[x] = zc[t.i * D + x];
            auto decide = [&](int e, const int (&zb)[D]) {
              const int f = sh.hl_f[e];
              if ((f & 1) && alu_le(t, za, zb, z0q, Ly, Ur)) dropped = true;
              if (f & 2) {
                int z0h[D];
#pragma unroll
                for (int x = 0; x < D; ++x) z0h[x] = t.shfl(zb[x], 0);
                if (alu_le(t, zb, za, z0h, Ly, Ur) && t.i == 0) sh.hl_f[e] = f | 4;
              }
            };
            if constexpr (D <= 12) {
              // two listed hulls per tile per step, their rows loaded together
              for (int e0 = tile_idx; e0 < nl; e0 += 2 * ntiles) {
                const int e1 = e0 + ntiles;
                int zb0[D], zb1[D];
                load_rows_rw(t, zb0, st.nzone + (node_base + sh.hl_u[e0]) * DD);
                if (e1 < nl) load_rows_rw(t, zb1, st.nzone + (node_base + sh.hl_u[e1]) * DD);
                decide(e0, zb0);
                if (e1 < nl) decide(e1, zb1);
              }
            } else {
              for (int e = tile_idx; e < nl; e += ntiles) {
                int zb[D];
                load_rows_rw(t, zb, st.nzone + (node_base + sh.hl_u[e]) * DD);
                decide(e, zb);
              }
            }
          }
        } else {
          // more open tests than the list holds: each thread decides its own hulls' drop test
          for (int h = tid; h < nhull && !dropped; h += blockDim.x) {
            const long long m = node_base + hull[h];
            if (!st.ndead[m]) dropped = alu_le_ptr<D>(zc, st.nzone + m * DD, Lr, Ur);
          }
        }
      }
    } else {
      for (int k = clen0 + tid; k < clen && !dropped; k += blockDim.x) {
        const int m = cl[k];
        if (m >= 0) dropped = alu_le_ptr<D>(zc, st.nzone + (long long)m * DD, Lr, Ur);
      }
    }
    if (__syncthreads_or(dropped)) {
      if (tid == 0) sh.hl_n = 0;   // the list is read by no one before the next survivor's barrier
      continue;
    }
    // (3): retire the zones s_q simulates
    int ret = 0;
    auto kill = [&](int k) {
      const int m = cl[k];
      if (m >= 0) {
        st.ndead[m] = 1;
        cl[k] = -1;
        ++ret;
        if (k >= clen - kRing) atomicAnd(&sh.lbits[(k & (kRing - 1)) >> 5], ~(1u << (k & 31)));
        if (rel && k >= clen0) atomicAnd(&sh.ulive[(k - clen0) >> 5], ~(1u << ((k - clen0) & 31)));
      }
    };
    if (rel) {
      const unsigned* row0 = r0 + (long long)q * r0w;
      for (long long w = tid; w < r0w; w += blockDim.x)
        for (unsigned b = w == tid ? w0 : row0[w]; b; b &= b - 1) kill((int)(w * 32 + __ffs(b) - 1));
      const unsigned* rowt = rt + (long long)q * rtw;
      for (long long w = tid; w < wq; w += blockDim.x)
        for (unsigned b = w == tid ? wt : rowt[w]; b; b &= b - 1) {
          const int p = tpos[w * 32 + __ffs(b) - 1];
          if (p >= 0) kill(clen0 + p);
        }
      if (nl <= kHullList) {
        for (int e = tid; e < nl; e += blockDim.x)
          if (sh.hl_f[e] & 4) kill(clen0 + sh.hl_u[e]);
      } else {
        for (int h = tid; h < nhull; h += blockDim.x) {
          const int u = hull[h];
          const long long m = node_base + u;
          const bool live = !st.ndead[m];
          if (alu_le_ptr<D>(st.nzone + m * DD, zc, Lr, Ur) && live) kill(clen0 + u);
        }
      }
    } else {
      for (int k = tid; k < clen; k += blockDim.x) {
        const int m = cl[k];
        if (m >= 0 && alu_le_ptr<D>(st.nzone + (long long)m * DD, zc, Lr, Ur)) kill(k);
      }
    }
    if (ret) atomicAdd(&sh.retired, ret);
    // (4)
    for (;;) {
      __syncthreads();
      if (warp == 0) {
        int nw = 0;
        const int lo = clen > kRing ? clen - kRing : 0;   // positions [lo, clen): the liveness ring
        for (int top = clen - 1; top >= lo && nw < kMergeScan; top -= 32) {
          const int k = top - lane;
          const bool live = k >= lo && ((sh.lbits[(k & (kRing - 1)) >> 5] >> (k & 31)) & 1u);
          const unsigned b = __ballot_sync(0xffffffffu, live);
          const int before = __popc(b & ((1u << lane) - 1u));
          if (live && nw + before < kMergeScan) sh.win[nw + before] = k;
          nw += __popc(b);
        }
        for (int top = lo - 1; top >= 0 && nw < kMergeScan; top -= 32) {
          const int k = top - lane;
          const bool live = k >= 0 && cl[k] >= 0;
          const unsigned b = __ballot_sync(0xffffffffu, live);
          const int before = __popc(b & ((1u << lane) - 1u));
          if (live && nw + before < kMergeScan) sh.win[nw + before] = k;
          nw += __popc(b);
        }
        if (lane == 0) {
          sh.nw = nw < kMergeScan ? nw : kMergeScan;
          sh.best = 0x7fffffff;
          dlive -= sh.retired;
          sh.retired = 0;
        }
      }
      __syncthreads();
      const int nw = sh.nw;
      if (nw == 0) break;
      int mybest = 0x7fffffff;
      int hl[D];
      if (in_tile) {
        // a tile-uniform read: a partner found at a lower index makes later candidates irrelevant
        auto best_now = [&]() { return t.shfl(*(volatile int*)&sh.best, 0); };
        auto node_of = [&](int k) { return k >= clen0 ? node_base + (k - clen0) : (long long)cl[k]; };
        auto attempt = [&](int c, const int (&zb)[D]) {
          int za[D];
#pragma unroll
          for (int e = 0; e < D; ++e) za[e] = zc[t.i * D + e];
          if (!try_union(t, za, zb)) return false;
          mybest = c;
#pragma unroll
          for (int e = 0; e < D; ++e) hl[e] = za[e];
          if (t.i == 0) atomicMin(&sh.best, c);
          return true;
        };
        if constexpr (D <= 12) {
          // a tile's two candidates (c0, c0 + ntiles) have their rows loaded together
          for (int c0 = tile_idx; c0 < nw; c0 += 2 * ntiles) {
            if (c0 > best_now()) break;
            const int c1 = c0 + ntiles;
            const bool has1 = c1 < nw;
            int zb0[D], zb1[D];
            load_rows_rw(t, zb0, st.nzone + node_of(sh.win[c0]) * DD);
            if (has1) load_rows_rw(t, zb1, st.nzone + node_of(sh.win[c1]) * DD);
            if (attempt(c0, zb0)) break;
            if (has1 && c1 <= best_now() && attempt(c1, zb1)) break;
          }
        } else {
          for (int c = tile_idx; c < nw; c += ntiles) {
            if (c > best_now()) break;
            int zb[D];
            load_rows_rw(t, zb, st.nzone + node_of(sh.win[c]) * DD);
            if (attempt(c, zb)) break;
          }
        }
      }
      __syncthreads();
      const int best = sh.best;
      if (best == 0x7fffffff) break;
      if (in_tile && mybest == best) {
#pragma unroll
        for (int e = 0; e < D; ++e) zc[t.i * D + e] = hl[e];
      }
      if (tid == 0) {
        const int k = sh.win[best];
        st.ndead[cl[k]] = 1;
        cl[k] = -1;
        if (k >= clen - kRing) sh.lbits[(k & (kRing - 1)) >> 5] &= ~(1u << (k & 31));
        if (rel && k >= clen0) sh.ulive[(k - clen0) >> 5] &= ~(1u << ((k - clen0) & 31));
        --dlive;
        sh.unioned = 1;
      }
    }
    // (5): store under the next reserved id. No barrier: the next survivor fills the other buffer,
    // and this one is reused only after the next survivor's barriers.
    const long long node = node_base + used;
    ++used;
    if (tid == 0) {
      node_meta(st, node, level, inst, hk, sc.pnode[a_s], sc.raw[a_s]);
      cl[clen] = (int)node;
      sh.lbits[(clen & (kRing - 1)) >> 5] |= 1u << (clen & 31);   // the slot of position clen - kRing
      sh.hl_n = 0;
      if (rel) {
        const int u = clen - clen0;
        sh.ulive[u >> 5] |= 1u << (u & 31);
        if (sh.unioned) {
          const int h = sh.nhull++;
          hull[h] = u;
          if (h < MergeShared<D>::kHC) {
            sh.hpos[h] = u;
            for (int y = 0; y < D; ++y) sh.hcol[h * D + y] = zc[y * D];
          }
        } else {
          tpos[q] = u;
        }
      }
      sh.clen = clen + 1;
      ++dlive;
    }
    for (int e = tid; e < DD; e += blockDim.x) st.nzone[node * DD + e] = zc[e];
    if (tid < D) st.ncol0[node * D + tid] = zc[tid * D];
  }
  for (int u = used + tid; u < sh.nkeep; u += blockDim.x) {   // ids a drop by a hull left unused
    const long long node = node_base + u;
    st.ndead[node] = 1; st.nlevel[node] = -1; st.ninst[node] = inst; st.nkey[node] = hk;
  }
  __syncthreads();
  finish_key_block(st, out, is, ctl, s, hk, inst, clen0, sh.clen, tid == 0 ? dlive : 0, cl, sh.wsum, sh.scal);
}

// One key merged by one tile (keys with little work).
template <int D>
__device__ void merge_key_tile(const NetView* nets, const InstState& is, const Succ& sc, const Store& st,
                               const Front& out, Ctl* ctl, int s, int level, const Tile<D>& t) {
  const int ishift = nets[0].inst_shift;
  const unsigned n = st.pend[s];
  const unsigned base = st.pend_base[s];
  const unsigned long long hk = st.hkey[s];
  const int inst = (int)(hk >> ishift);
  if (is.found[inst] || is.done[inst]) { t.sync(); if (t.i == 0) st.pend[s] = 0; return; }
  const NetView& N = nets[inst];
  rank_segment(sc, base, n, t.i, D);
  long long cb = 0;
  if (t.i == 0) cb = alloc_clist(sc, st, s, n, ctl);
  cb = (long long)t.shfl64((unsigned long long)cb, 0);
  if (cb < 0) { t.sync(); return; }
  int clen = st.klive[s];
  {
    const int* lst = st.arena + st.kloff[s];
    for (int k = t.i; k < clen; k += D) sc.clist[cb + k] = lst[k];
  }
  t.sync();
  const int clen0 = clen;
  volatile int* cl = sc.clist + cb;
  volatile int* vdead = st.ndead;
  int locs[kMaxProcs], ints[kMaxInts];
  key_decode(N, key_part(hk, ishift), locs, ints);
  int Ly, U[D], Lall[D];
  key_bounds(N, t, locs, Ly, U);
#pragma unroll
  for (int x = 0; x < D; ++x) Lall[x] = t.shfl(Ly, x);
  long long dlive = 0;
  for (unsigned q = 0; q < n; ++q) {
    const int a = ((volatile int*)sc.sorted)[base + q];
    const int* zs = sc.zone + (long long)a * D * D;
    int z[D];
    load_rows(t, z, zs);
    // (1)+(2): the lanes take this level's zones in turn
    bool drop = false;
    for (int k = clen0 + t.i; k < clen && !drop; k += D) {
      const int m = cl[k];
      if (m >= 0) drop = alu_le_lane<D>(zs, st.nzone + (long long)m * D * D, Lall, U);
    }
    if (t.any(drop)) continue;
    // (3)
    int retired = 0;
    for (int k = t.i; k < clen; k += D) {
      const int m = cl[k];
      if (m >= 0 && alu_le_lane<D>(st.nzone + (long long)m * D * D, zs, Lall, U)) {
        vdead[m] = 1;
        cl[k] = -1;
        ++retired;
      }
    }
    t.sync();
#pragma unroll
    for (int l = 0; l < D; ++l) dlive -= t.shfl(retired, l);
    // (4)
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
    // (5)
    long long node = 0;
    if (t.i == 0) node = (long long)take_index(&ctl->nnodes);
    node = (long long)t.shfl64((unsigned long long)node, 0);
    store_rows(t, z, st.nzone + node * D * D);
    st.ncol0[node * D + t.i] = z[0];
    if (t.i == 0) {
      node_meta(st, node, level, inst, hk, sc.pnode[a], sc.raw[a]);
      cl[clen] = (int)node;
    }
    ++clen;
    ++dlive;
    t.sync();
  }
  if (t.i == 0) finish_key(sc, st, out, is, ctl, s, hk, inst, (const int*)cl, clen0, clen, dlive);
  t.sync();
}

template <int D, int NT>
__global__ void __launch_bounds__(NT, kMergeBlockWide / NT) k_merge(const NetView* nets, InstState is, Succ sc, Store st,
                                                          Front out, Ctl* ctl, int level, const int* order) {
  __shared__ MergeShared<D> sh;
  Tile<D> t;
  const bool in_tile = make_tile(t, threadIdx.x & 31);
  // keys with much work: one block each, taken in turn
  const long long nheavy = (long long)ctl->nheavy, nlight = (long long)ctl->nlight;
  for (;;) {
    if (threadIdx.x == 0) sh.job = (int)atomicAdd(&ctl->heavy_next, 1ull);
    __syncthreads();
    const long long jj = sh.job;
    __syncthreads();
    if (jj >= nheavy) break;
    const long long j = order ? order[jj] : jj;
    merge_key_block<D>(nets, is, sc, st, out, ctl, j, level, in_tile, t, sh);
  }
  // the rest: one tile each, taken in turn
  if (!in_tile) return;
  for (;;) {
    unsigned long long j = 0;
    if (t.i == 0) j = take_index(&ctl->light_next);
    j = t.shfl64(j, 0);
    if ((long long)j >= nlight) break;
    merge_key_tile<D>(nets, is, sc, st, out, ctl, sc.light[j], level, t);
  }
}

// Copy every key's list into a fresh arena (thread per slot), dropping the lists merges replaced.
static __global__ void k_arena_compact(Store st, int* narena, long long ncap, unsigned long long* nalloc, Ctl* ctl) {
  for (unsigned long long h = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; h <= st.hmask;
       h += (unsigned long long)gridDim.x * blockDim.x) {
    const int c = st.klive[h];
    if (c <= 0) continue;
    const long long off = (long long)atomicAdd(nalloc, (unsigned long long)c);
    if (off + c > ncap) { atomicMax(&ctl->err, 4u); continue; }
    const int* src = st.arena + st.kloff[h];
    for (int k = 0; k < c; ++k) narena[off + k] = src[k];
    st.kloff[h] = off;
  }
}

// ---------------------------------------------------------------------------------------------
// exact-zone graph store (leads-to graph mode): hash dedup instead of a per-key list scan
// ---------------------------------------------------------------------------------------------
// 32-bit hash of (hash key, zone), never 0: each lane mixes its row, lane 0 folds the rows in order.
template <int D>
__device__ __forceinline__ unsigned zone_hash(const Tile<D>& t, const int (&z)[D], unsigned long long hk) {
  unsigned long long r = 0x9e3779b97f4a7c15ull * (unsigned long long)(t.i + 1);
#pragma unroll
  for (int j = 0; j < D; ++j) r = hash_mix(r ^ (unsigned)z[j]);
  unsigned long long h = hash_mix(hk);
#pragma unroll
  for (int l = 0; l < D; ++l) h = hash_mix(h ^ t.shfl64(r, l));
  const unsigned v = (unsigned)(h >> 32);
  return v ? v : 1u;
}

// Per successor: find an equal stored zone, an equal successor of this level that claimed a slot
// first, or claim a free slot. Claimers are listed in sc.surv; sc.slot[s] = claimed slot (>= 0),
// -2 for a duplicate (sc.rank[s] = the slot word's ref), -1 when the instance is finished.
template <int D>
__global__ void __launch_bounds__(kBlock) k_graph_probe(const NetView* nets, InstState is, Succ sc, Store st, ZTab zt,
                                                        Ctl* ctl, long long nsucc) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  volatile unsigned long long* vw = zt.w;
  for (long long s = tile_id<D>(); s < nsucc; s += tile_count<D>()) {
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    if (is.found[inst] || is.done[inst]) { if (t.i == 0) sc.slot[s] = -1; continue; }
    int z[D];
    load_rows(t, z, sc.zone + s * D * D);
    const unsigned h = zone_hash(t, z, hk);
    const unsigned long long mine = ((unsigned long long)h << 32) | (kZRefSucc | (unsigned)s);
    unsigned long long pos = hash_mix(((unsigned long long)h << 32) ^ hk) & zt.mask;
    int result = -3;   // -3 searching, >= 0 claimed slot, -2 duplicate
    unsigned ref = 0;
    for (unsigned long long it = 0; it <= zt.mask && result == -3; ++it, pos = (pos + 1) & zt.mask) {
      unsigned long long w = 0;
      if (t.i == 0) {
        w = vw[pos];
        if (w == 0) w = atomicCAS(&zt.w[pos], 0ull, mine);   // 0: claimed
      }
      w = t.shfl64(w, 0);
      if (w == 0) { result = (int)pos; break; }
      if ((unsigned)(w >> 32) != h) continue;
      const unsigned r = (unsigned)w;
      const bool succ_ref = (r & kZRefSucc) != 0;
      const long long idx = (long long)(r & ~kZRefSucc);
      const unsigned long long okey = succ_ref ? sc.key[idx] : st.nkey[idx];
      if (okey != hk) continue;
      const int* oz = (succ_ref ? sc.zone : st.nzone) + idx * D * D;
      bool eq = true;
#pragma unroll
      for (int j = 0; j < D; ++j) eq &= __ldcg(oz + t.i * D + j) == z[j];
      if (t.all(eq)) { result = -2; ref = r; }
    }
    if (t.i == 0) {
      if (result == -3) {   // table full: the host sizes it at most half full, so this is an error
        atomicMax(&ctl->err, 4u);
        sc.slot[s] = -1;
      } else {
        sc.slot[s] = result;
        if (result == -2) sc.rank[s] = (int)ref;
        else sc.surv[take_index(&ctl->nsurv)] = (int)s;
        // keys are counted once, by the successor that first inserts the discrete key
        bool ins = false;
        const long long ks = slot_find_insert(st, hk, &ins);
        if (ks < 0) atomicMax(&ctl->err, 4u);
        else if (ins) { atomicAdd(&ctl->nslots, 1ull); atomicAdd(&ctl->nkeys, 1ull); atomicAdd(&is.nkeys[inst], 1ull); }
      }
    }
  }
}

// Store every claimer as a node of this level, point its slot at the node and put it in the next
// frontier; sc.rank[s] = its node id.
template <int D>
__global__ void __launch_bounds__(kBlock) k_graph_store(const NetView* nets, InstState is, Succ sc, Store st, ZTab zt,
                                                        Front out, Ctl* ctl, long long nnew, int level) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  for (long long w = tile_id<D>(); w < nnew; w += tile_count<D>()) {
    const int s = sc.surv[w];
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    long long node = 0;
    if (t.i == 0) node = (long long)take_index(&ctl->nnodes);
    node = (long long)t.shfl64((unsigned long long)node, 0);
    int z[D];
    load_rows(t, z, sc.zone + (long long)s * D * D);
    store_rows(t, z, st.nzone + node * D * D);
    st.ncol0[node * D + t.i] = z[0];
    if (t.i == 0) {
      st.nlevel[node] = level;
      st.ndead[node] = 0;
      st.ninst[node] = inst;
      st.nkey[node] = hk;
      const long long pos = sc.slot[s];
      zt.w[pos] = (zt.w[pos] & 0xffffffff00000000ull) | (unsigned)node;
      sc.rank[s] = (int)node;
      const unsigned long long f = atomicAdd(&ctl->nfront, 1ull);
      out.key[f] = hk; out.node[f] = (int)node; out.rank[f] = 0; out.inst[f] = inst;
      atomicAdd(&is.nfront[inst], 1ull);
      atomicAdd((unsigned long long*)&ctl->nlive, 1ull);
      atomicAdd((unsigned long long*)&is.nlive[inst], 1ull);
    }
  }
}

// One edge per successor, from its parent's node to the node holding its zone.
static __global__ void k_graph_edges(Succ sc, Front fr, Edges ed, Ctl* ctl, long long nsucc) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nsucc; s += (long long)gridDim.x * blockDim.x) {
    const int sl = sc.slot[s];
    if (sl == -1) continue;
    int node;
    if (sl >= 0) node = sc.rank[s];
    else {
      const unsigned r = (unsigned)sc.rank[s];
      node = (r & kZRefSucc) ? sc.rank[r & ~kZRefSucc] : (int)r;
    }
    const unsigned long long e = take_index(&ctl->nedges);
    if ((long long)e < ed.cap) { ed.src[e] = fr.node[sc.parent[s]]; ed.dst[e] = node; ed.ord[e] = sc.ord[s]; }
    else atomicMax(&ctl->err, 4u);
  }
}

// Re-insert every stored node into a fresh (larger) zone table.
template <int D>
__global__ void __launch_bounds__(kBlock) k_graph_rehash(Store st, long long nnodes, ZTab zt, Ctl* ctl) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  for (long long n = tile_id<D>(); n < nnodes; n += tile_count<D>()) {
    const unsigned long long hk = st.nkey[n];
    int z[D];
    load_rows(t, z, st.nzone + n * D * D);
    const unsigned h = zone_hash(t, z, hk);
    if (t.i == 0) {
      unsigned long long pos = hash_mix(((unsigned long long)h << 32) ^ hk) & zt.mask;
      unsigned long long it = 0;
      for (; it <= zt.mask; ++it, pos = (pos + 1) & zt.mask)
        if (atomicCAS(&zt.w[pos], 0ull, ((unsigned long long)h << 32) | (unsigned)n) == 0ull) break;
      if (it > zt.mask) atomicMax(&ctl->err, 4u);
    }
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
    if (N.kind != 2 && N.kind != 3) continue;   // leads-to p-nodes; E[]: the initial state
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
      const bool ok = for_each_successor(U, t, locs, ints, z, 1, [&](const int*, const int*, const int (&)[D], int) { ++cnt; });
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
    const bool ok = for_each_successor(N, t, locs, ints, src, emode, [&](const int* tl, const int* ti, const int (&z)[D], int) {
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
                      Ctl* ctl, int roots, int i0, int i1, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_expand<D><<<grid_for(nfront, TPB, blocks), kBlock, 0, s>>>(nets, is, fr, nfront, src_zone, sc, ctl, roots, i0, i1);
}
template <int D>
void Level<D>::probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nsucc, int long_list,
                     int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_probe<D><<<grid_for(nsucc, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, st, ctl, nsucc, long_list);
}
template <int D>
void Level<D>::probe_long(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, int blocks, cudaStream_t s) {
  k_probe_long<D><<<blocks, kBlock, 0, s>>>(nets, is, sc, st, ctl);
}
template <int D>
void Level<D>::deadlock(const NetView* nets, InstState is, Succ sc, Ctl* ctl, long long n, int all, int blocks,
                        cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_deadlock<D><<<grid_for(n, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, ctl, n, all);
}
template <int D>
void Level<D>::group(Succ sc, Store st, Ctl* ctl, long long nsucc, long long ntouched, cudaStream_t s) {
  k_seg_alloc<<<grid_for(ntouched, 256, 1024), 256, 0, s>>>(sc, st, ctl, ntouched);
  k_seg_scatter<<<grid_for(nsucc, 256, 4096), 256, 0, s>>>(sc, st, nsucc);
}
template <int D>
void Level<D>::heavy_prep(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nheavy,
                          int blocks, const int* order, cudaStream_t s) {
  const long long g = nheavy < blocks ? nheavy : blocks;
  if (g > 0) k_heavy_prep<D><<<(int)g, kMergeBlock, 0, s>>>(nets, is, sc, st, ctl, nheavy, order);
}
template <int D>
int Level<D>::heavy_pairs(const NetView* nets, Succ sc, Store st, const long long* prefix, long long nheavy,
                          long long ntiles, int blocks, cudaStream_t s) {
  constexpr int Z2 = D * D;
  constexpr int P = (Z2 & 1) ? Z2 : Z2 + 1;
  constexpr size_t smem = 2 * 32 * P * sizeof(int);
  static const bool attr_ok =
      cudaFuncSetAttribute(k_heavy_pairs<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
  if (!attr_ok) return 1;
  const long long g = ntiles < blocks ? ntiles : blocks;
  if (g > 0) k_heavy_pairs<D><<<(int)g, kMergeBlock, smem, s>>>(nets, sc, st, prefix, nheavy, ntiles);
  return 0;
}
template <int D>
bool Level<D>::merge_wide_pays() {
  return wide_fold_pays<D>();
}
template <int D>
int Level<D>::merge_blocks_per_sm(bool wide) {
  int n = 0;
  cudaError_t e;
  if constexpr (wide_fold_pays<D>()) {
    e = wide ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_merge<D, kMergeBlockWide>, kMergeBlockWide, 0)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_merge<D, kMergeBlock>, kMergeBlock, 0);
  } else {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_merge<D, kMergeBlock>, kMergeBlock, 0);
  }
  if (e != cudaSuccess) n = 1;
  return n;
}
template <int D>
void Level<D>::merge(const NetView* nets, InstState is, Succ sc, Store st, Front out, Ctl* ctl, long long ntouched,
                     int level, int blocks, bool wide, const int* order, cudaStream_t s) {
  const long long g = ntouched < blocks ? ntouched : blocks;
  if constexpr (wide_fold_pays<D>()) {
    if (wide) {
      k_merge<D, kMergeBlockWide><<<(int)(g > 0 ? g : 1), kMergeBlockWide, 0, s>>>(nets, is, sc, st, out, ctl, level, order);
      return;
    }
  }
  k_merge<D, kMergeBlock><<<(int)(g > 0 ? g : 1), kMergeBlock, 0, s>>>(nets, is, sc, st, out, ctl, level, order);
}template <int D>
void Level<D>::graph_probe(const NetView* nets, InstState is, Succ sc, Store st, ZTab zt, Ctl* ctl, long long nsucc,
                           int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_graph_probe<D><<<grid_for(nsucc, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, st, zt, ctl, nsucc);
}
template <int D>
void Level<D>::graph_store(const NetView* nets, InstState is, Succ sc, Store st, ZTab zt, Front out, Ctl* ctl,
                           long long nnew, int level, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_graph_store<D><<<grid_for(nnew, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, st, zt, out, ctl, nnew, level);
}
template <int D>
void Level<D>::graph_edges(Succ sc, Front fr, Edges ed, Ctl* ctl, long long nsucc, cudaStream_t s) {
  k_graph_edges<<<grid_for(nsucc, 256, 8192), 256, 0, s>>>(sc, fr, ed, ctl, nsucc);
}
template <int D>
void Level<D>::graph_rehash(Store st, long long nnodes, ZTab zt, Ctl* ctl, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  if (nnodes > 0) k_graph_rehash<D><<<grid_for(nnodes, TPB, blocks), kBlock, 0, s>>>(st, nnodes, zt, ctl);
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
