// subsumed_impl.cuh -- the subsumed leads-to graph and its federation-valued greatest fixpoint.
// Included by level_kernels_impl.cuh, so every kernel here is instantiated once per DBM dimension.
//
// Phase 2 of p --> q (leads_to_clocks, src/liveness/api.cpp:655-722) explores the !q-restricted
// network from the roots with Extra_M+ zones and INCLUSION covers: a successor is covered by a stored
// zone of its discrete key only when that zone contains it (the cover scan of online_intern,
// src/liveness/construction.cpp:194-215,480-684, with containment as the cover test). Per level and
// key, the survivors of the probe that no other survivor strictly contains (ties to the lower
// successor index) are stored, so the stored set depends only on the set of successor zones. Every
// successor records an edge to its covering node with its transition index, and the backward sweep
//     W[v] := W[v] /\ (Stop(v) \/ U_e Pre_e(W[tgt e]))
// (solve_greatest_fixpoint / relax, src/liveness/fixpoint.cpp:48-977,750-864) runs on federations
// with the exact predecessor (exact_predecessor, src/liveness/operators.cpp:257-306). Because each
// edge's target contains the exact successor, the fixpoint is exact on valuations.
#pragma once

namespace hgb {

// ---------------------------------------------------------------------------------------------
// inclusion probe, grouping, maximal survivors, store, key lists, covers, edges
// ---------------------------------------------------------------------------------------------
// Per successor: find or insert its key, and look for a stored zone of the key containing it (each
// lane decides whole tests of successive list entries; the first list position found wins).
template <int D>
__global__ void __launch_bounds__(kBlock) k_incl_probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl,
                                                       long long nsucc) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  unsigned long long nprobe_sum = 0;   // added once per tile at the end (one atomic per test serialises)
  for (long long s = tile_id<D>(); s < nsucc; s += tile_count<D>()) {
    const unsigned long long hk = sc.key[s];
    const int inst = (int)(hk >> ishift);
    if (is.found[inst] || is.done[inst]) { if (t.i == 0) sc.slot[s] = -1; continue; }
    long long slot = 0;
    int inserted = 0;
    if (t.i == 0) {
      bool ins;
      slot = slot_find_insert(st, hk, &ins);
      inserted = ins;
      if (ins) atomicAdd(&ctl->nslots, 1ull);
    }
    slot = (long long)t.shfl64((unsigned long long)slot, 0);
    inserted = t.shfl(inserted, 0);
    if (slot < 0) { if (t.i == 0) { atomicMax(&ctl->err, 4u); sc.slot[s] = -1; } continue; }
    int cover = -1;
    unsigned long long nprobe = 0;
    if (!inserted) {
      const int* zs = sc.zone + s * D * D;
      int zc0[D];
#pragma unroll
      for (int y = 0; y < D; ++y) zc0[y] = __ldg(zs + y * D);
      const int nl = __ldg(st.klive + slot);
      const int* lst = st.arena + __ldg(st.kloff + slot);
      for (int k0 = 0; k0 < nl && cover < 0; k0 += D) {
        const int k = k0 + t.i;
        int mine = -1;
        if (k < nl) {
          ++nprobe;
          const int m = __ldg(lst + k);
          const int* c0 = st.ncol0 + (long long)m * D;
          bool inc = true;
#pragma unroll
          for (int y = 0; y < D; ++y) inc &= __ldg(c0 + y) >= zc0[y];
          if (inc) {
            const int* zm = st.nzone + (long long)m * D * D;
            for (int a = 0; a < D && inc; ++a)
#pragma unroll
              for (int b = 1; b < D; ++b) inc &= __ldg(zm + a * D + b) >= __ldg(zs + a * D + b);
          }
          if (inc) mine = m;
        }
        const unsigned bal = __ballot_sync(t.mask, mine >= 0) & t.mask;
        if (bal) cover = t.shfl(mine, __ffs(bal) - 1 - t.base);
      }
    }
    nprobe_sum += nprobe;
    if (t.i == 0) {
      if (cover >= 0) {
        sc.slot[s] = -2;
        sc.rank[s] = cover;
      } else {
        const unsigned r = atomicAdd(&st.pend[slot], 1u);
        if (r == 0) sc.touched[atomicAdd(&ctl->ntouched, 1ull)] = (int)slot;
        sc.slot[s] = (int)slot;
        sc.rank[s] = (int)r;
        sc.surv[take_index(&ctl->nsurv)] = (int)s;
      }
    }
  }
  unsigned long long tp = 0;
#pragma unroll
  for (int l = 0; l < D; ++l) tp += t.shfl64(nprobe_sum, l);
  if (t.i == 0 && tp) atomicAdd(&ctl->probes, tp);
}

// One contiguous segment of survivors per touched key.
static __global__ void k_incl_seg(Succ sc, Store st, Ctl* ctl, long long ntouched) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < ntouched; j += (long long)gridDim.x * blockDim.x) {
    const int s = sc.touched[j];
    st.pend_base[s] = (unsigned)atomicAdd(&ctl->seg_alloc, (unsigned long long)st.pend[s]);
  }
}

// Row-parallel comparison of a zone in global memory with the tile's zone z: ge = it contains z,
// eq = it equals z.
template <int D>
__device__ __forceinline__ void cmp_rows(const Tile<D>& t, const int* other, const int (&z)[D], bool& ge, bool& eq) {
  const int* row = other + t.i * D;
  bool g = true, e = true;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    const int v = __ldg(row + j);
    g &= v >= z[j];
    e &= v == z[j];
  }
  ge = t.all(g);
  eq = t.all(e);
}

// A survivor is stored unless another survivor of its key contains it strictly, or equals it with
// a lower successor index.
template <int D>
__global__ void __launch_bounds__(kBlock) k_incl_keep(Succ sc, Store st, long long nsurv) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  for (long long w = tile_id<D>(); w < nsurv; w += tile_count<D>()) {
    const int s = sc.surv[w];
    const int slot = sc.slot[s];
    const unsigned base = st.pend_base[slot], n = st.pend[slot];
    int z[D];
    load_rows(t, z, sc.zone + (long long)s * D * D);
    bool keep = true;
    for (unsigned j = 0; j < n && keep; ++j) {
      const int sj = sc.seg[base + j];
      if (sj == s) continue;
      bool ge, eq;
      cmp_rows(t, sc.zone + (long long)sj * D * D, z, ge, eq);
      if (ge && (!eq || sj < s)) keep = false;
    }
    if (t.i == 0) sc.flag[s] = keep ? 1 : 0;
  }
}

// Store the kept survivors as nodes of this level and put them in the next frontier.
template <int D>
__global__ void __launch_bounds__(kBlock) k_incl_store(const NetView* nets, InstState is, Succ sc, Store st, Front out,
                                                       Ctl* ctl, long long nsurv, int level) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const int ishift = nets[0].inst_shift;
  for (long long w = tile_id<D>(); w < nsurv; w += tile_count<D>()) {
    const int s = sc.surv[w];
    if (!sc.flag[s]) continue;
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
      st.nlevel[node] = level; st.ndead[node] = 0; st.ninst[node] = inst; st.nkey[node] = hk;
      // the source node (for a root: the phase-1 node whose p-part it is) and the transition index,
      // read by a counterexample trace
      st.npar[node] = sc.pnode[s]; st.nraw[node] = sc.raw[s];
      sc.rank[s] = (int)node;
      const unsigned long long f = atomicAdd(&ctl->nfront, 1ull);
      out.key[f] = hk; out.node[f] = (int)node; out.rank[f] = 0; out.inst[f] = inst;
      atomicAdd(&is.nfront[inst], 1ull);
      atomicAdd((unsigned long long*)&ctl->nlive, 1ull);
      atomicAdd((unsigned long long*)&is.nlive[inst], 1ull);
    }
  }
}

// One warp per touched key: its list becomes the old list followed by the nodes stored this level,
// written at a fresh arena offset; the key's pending count is cleared.
static __global__ void k_incl_lists(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long ntouched) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const int ishift = nets[0].inst_shift;
  for (long long j = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); j < ntouched; j += nw) {
    const int slot = sc.touched[j];
    const unsigned n = st.pend[slot], base = st.pend_base[slot];
    int nk = 0;
    for (unsigned k = lane; k < n; k += 32) nk += sc.flag[sc.seg[base + k]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nk += __shfl_xor_sync(0xffffffffu, nk, o);
    if (nk > 0) {
      const int old = st.klive[slot];
      const long long ooff = st.kloff[slot];
      long long off = 0;
      if (lane == 0) off = (long long)atomicAdd(&ctl->arena_alloc, (unsigned long long)(old + nk));
      off = (long long)__shfl_sync(0xffffffffu, (unsigned long long)off, 0);
      if (off + old + nk > st.acap) {
        if (lane == 0) atomicMax(&ctl->err, 4u);
      } else {
        for (int k = lane; k < old; k += 32) st.arena[off + k] = st.arena[ooff + k];
        long long pos = off + old;
        for (unsigned k0 = 0; k0 < n; k0 += 32) {
          const unsigned k = k0 + lane;
          const int s = k < n ? sc.seg[base + k] : -1;
          const bool f = s >= 0 && sc.flag[s];
          const unsigned b = __ballot_sync(0xffffffffu, f);
          if (f) st.arena[pos + __popc(b & ((1u << lane) - 1u))] = sc.rank[s];
          pos += __popc(b);
        }
        if (lane == 0) {
          st.klive[slot] = old + nk;
          st.kloff[slot] = off;
          if (old == 0) {
            atomicAdd(&ctl->nkeys, 1ull);
            atomicAdd(&is.nkeys[(int)(st.hkey[slot] >> ishift)], 1ull);
          }
        }
      }
    }
    if (lane == 0) st.pend[slot] = 0;
  }
}

// A survivor not stored is covered by a stored survivor of its key containing it.
template <int D>
__global__ void __launch_bounds__(kBlock) k_incl_cover(Succ sc, Store st, Ctl* ctl, long long nsurv) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  for (long long w = tile_id<D>(); w < nsurv; w += tile_count<D>()) {
    const int s = sc.surv[w];
    if (sc.flag[s]) continue;
    const int slot = sc.slot[s];
    const unsigned base = st.pend_base[slot], n = st.pend[slot];
    int z[D];
    load_rows(t, z, sc.zone + (long long)s * D * D);
    int cov = -1;
    for (unsigned j = 0; j < n && cov < 0; ++j) {
      const int sj = sc.seg[base + j];
      if (!sc.flag[sj]) continue;
      bool ge, eq;
      cmp_rows(t, sc.zone + (long long)sj * D * D, z, ge, eq);
      if (ge) cov = sc.rank[sj];
    }
    if (t.i == 0) {
      if (cov < 0) atomicMax(&ctl->err, 4u);
      else sc.rank[s] = cov;
    }
  }
}

// One edge per successor, from its parent's node to its covering node, with the transition index.
static __global__ void k_incl_edges(Succ sc, Front fr, Edges ed, Ctl* ctl, long long nsucc) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nsucc; s += (long long)gridDim.x * blockDim.x) {
    if (sc.slot[s] == -1) continue;
    const unsigned long long e = take_index(&ctl->nedges);
    if ((long long)e < ed.cap) {
      ed.src[e] = fr.node[sc.parent[s]]; ed.dst[e] = sc.rank[s]; ed.ord[e] = sc.ord[s]; ed.raw[e] = sc.raw[s];
    } else {
      atomicMax(&ctl->err, 4u);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// stop sets (stop_set, src/liveness/construction.cpp:1200-1239) as federations
// ---------------------------------------------------------------------------------------------
// With `witness`, nodes[] lists phase-1 nodes: each p-part cut to !q is tested for a stop valuation
// (leadsto_witness, construction.cpp:786-826) and its instance is found when one exists. Otherwise
// nodes n0..n1-1 of the graph get swhole / their pieces, which are listed from shead through snext.
template <int D>
__global__ void __launch_bounds__(kBlock) k_stop_fed(const NetView* nets, InstState is, Store st, long long n0,
                                                     long long n1, const int* nodes, Fix fx, Ctl* ctl, int witness) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  DlScratch<D> S;
  const int ishift = nets[0].inst_shift;
  for (long long w = n0 + tile_id<D>(); w < n1; w += tile_count<D>()) {
    const long long n = nodes ? nodes[w] : w;
    const unsigned long long hk = st.nkey[n];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    if (witness && (N.kind != 2 || is.found[inst] || is.done[inst])) continue;   // 2: leads-to
    int locs[kMaxProcs], ints[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    int z[D];
    load_rows(t, z, st.nzone + n * D * D);
    int zn[D];   // the node's zone, recorded as the witness state
#pragma unroll
    for (int j = 0; j < D; ++j) zn[j] = z[j];
    if (witness) {
      if (!pred_disc(N.p_loc, N.p_nloc, N.p_int, N.p_nint, locs, ints)) continue;
      if (!apply_cons(t, z, N.p_clk, 0, N.p_nclk) || !avoid_cut(N, t, z, locs, ints) || is_empty(t, z)) continue;
    }
    bool whole = false, none = false;
    if (N.av_nclk == 0) {
      NetView U = N;
      U.av_on = 0;
      int cnt = 0;
      const bool ok = for_each_successor(U, t, locs, ints, z, 1, [&](const int*, const int*, const int (&)[D], int) { ++cnt; });
      if (!ok) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
      whole = cnt == 0 || time_diverges(N, t, locs, ints, z, false);
    } else {
      whole = time_diverges(N, t, locs, ints, z, true);
      none = !whole && orig_time_open(N, t, locs, ints);
    }
    int head = -1, npieces = 0;
    bool over = false;
    if (!whole && !none) {
      int Z[D], nw = 0;
      const int r = collect_escapes(N, t, locs, ints, z, S, Z, nw);
      if (r < 0) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
      if (r > 0)
        npieces = subtract_escapes(t, z, S, nw, [&](const int (&P)[D]) {
          if (witness) return false;
          long long slot = 0;
          if (t.i == 0) slot = (long long)atomicAdd(&ctl->spieces, 1ull);
          slot = (long long)t.shfl64((unsigned long long)slot, 0);
          if (slot >= fx.scap) { over = true; return false; }
          store_rows(t, P, fx.spiece + slot * D * D);
          if (t.i == 0) fx.snext[slot] = head;
          head = (int)slot;
          return true;
        });
    }
    if (witness && (whole || npieces > 0)) record_hit(t, is, inst, (int)n, -1, hk, zn);
    if (t.i == 0) {
      if (witness) {
        if (whole || npieces > 0) { is.found[inst] = 1; atomicOr(&ctl->found, 1u); }
      } else {
        if (over) ctl->stop_over = 1;
        fx.swhole[n] = whole ? 1 : 0;
        fx.shead[n] = head;
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// exact predecessor of one transition
// ---------------------------------------------------------------------------------------------
// The recipe of one transition (GfpTag, src/liveness/operators.cpp:55-206): participating local
// edges, sender first, and the abstaining broadcast receivers with their abstain options.
struct TransRec {
  int ne;
  int edge[kMaxProcs + 1];
  int nab;
  int ab_part[kMaxProcs];
  int ab_opt[kMaxProcs];
  BcastParts P;
};

// Transition `want` of (locs, ints) in for_each_successor's enumeration, rebuilt without zone work.
__device__ inline bool find_trans(const NetView& N, const int* locs, const int* ints, int want, TransRec& T) {
  bool src_c, src_u;
  frozen_flags(N, locs, ints, src_c, src_u);
  int raw = 0;
  T.ne = 0; T.nab = 0;
  for (int p = 0; p < N.nprocs; ++p) {
    if (src_c && !committed_at(N, p, locs[p])) continue;
    const int gp = N.loc_base[p] + locs[p];
    for (int k = N.eloc_off[gp]; k < N.eloc_off[gp + 1]; ++k) {
      const int e = N.eloc[k];
      if (N.edge_chan[e] >= 0 || !int_ok(N, e, ints)) continue;
      if (raw++ == want) { T.edge[0] = e; T.ne = 1; return true; }
    }
  }
  for (int i = 0; i < N.nprocs; ++i) {
    const int gi = N.loc_base[i] + locs[i];
    for (int k = N.eloc_off[gi]; k < N.eloc_off[gi + 1]; ++k) {
      const int se = N.eloc[k];
      const int ch = N.edge_chan[se];
      if (ch < 0 || N.edge_dir[se] != 1 || (N.chan_flags[ch] & 1)) continue;
      if (!int_ok(N, se, ints)) continue;
      const bool i_comm = committed_at(N, i, locs[i]);
      for (int j = 0; j < N.nprocs; ++j) {
        if (j == i) continue;
        const int gj = N.loc_base[j] + locs[j];
        for (int q = N.eloc_off[gj]; q < N.eloc_off[gj + 1]; ++q) {
          const int re = N.eloc[q];
          if (N.edge_chan[re] != ch || N.edge_dir[re] != -1) continue;
          if (src_c && !(i_comm || committed_at(N, j, locs[j]))) continue;
          if (!int_ok(N, re, ints)) continue;
          if (raw++ == want) { T.edge[0] = se; T.edge[1] = re; T.ne = 2; return true; }
        }
      }
    }
  }
  for (int i = 0; i < N.nprocs; ++i) {
    const int gi = N.loc_base[i] + locs[i];
    for (int k = N.eloc_off[gi]; k < N.eloc_off[gi + 1]; ++k) {
      const int se = N.eloc[k];
      const int ch = N.edge_chan[se];
      if (ch < 0 || N.edge_dir[se] != 1 || !(N.chan_flags[ch] & 1)) continue;
      if (!int_ok(N, se, ints)) continue;
      if (!build_parts(N, locs, ints, se, i, T.P)) return false;
      int pick[kMaxProcs];
      for (int q = 0; q < T.P.n; ++q) pick[q] = 0;
      for (;;) {
        bool part_comm = committed_at(N, i, locs[i]);
        for (int q = 0; q < T.P.n; ++q)
          if (pick[q] < T.P.ne[q] && committed_at(N, T.P.proc[q], locs[T.P.proc[q]])) part_comm = true;
        if (!src_c || part_comm) {
          if (raw++ == want) {
            T.edge[T.ne++] = se;
            for (int q = 0; q < T.P.n; ++q) {
              if (pick[q] < T.P.ne[q]) T.edge[T.ne++] = T.P.edge[q][pick[q]];
              else { T.ab_part[T.nab] = q; T.ab_opt[T.nab] = pick[q] - T.P.ne[q]; T.nab++; }
            }
            return true;
          }
        }
        if (T.P.n == 0) break;
        int q = 0;
        for (; q < T.P.n; ++q) {
          if (++pick[q] < T.P.ne[q] + T.P.nab[q]) break;
          pick[q] = 0;
        }
        if (q == T.P.n) break;
      }
    }
  }
  return false;
}

// Exact predecessor of the target valuations Y through T from (sl, si) to (tl, ti), in place
// (exact_predecessor, src/liveness/operators.cpp:257-306): undo the active-clock reduction at the
// target, its invariant and delay, the resets, the guards and abstain constraints, then the delay
// before the action. The !q restriction is adjoined to both invariants as close_succ adjoins it,
// and the source invariant holds at the action point too. False when nothing is left.
template <int D>
__device__ bool pre_step(const NetView& N, const Tile<D>& t, int (&Y)[D], const TransRec& T, const int* sl,
                         const int* si, const int* tl, const int* ti) {
  unsigned long long a = N.qmask;
  for (int p = 0; p < N.nprocs; ++p) a |= N.act[N.loc_base[p] + tl[p]];
  unsigned long long dead = ~a & (((1ull << N.nclocks) - 1) << 1);
  while (dead) {
    const int k = __ffsll((long long)dead) - 1;
    dead &= dead - 1;
    free_clock(t, Y, k);
  }
  if (!apply_inv(N, t, Y, tl) || !avoid_cut(N, t, Y, tl, ti)) return false;
  bool c, u;
  frozen_flags(N, tl, ti, c, u);
  if (!c && !u) {
    down(t, Y);
    if (!apply_inv(N, t, Y, tl) || !avoid_cut(N, t, Y, tl, ti)) return false;
  }
  for (int k = 0; k < T.ne; ++k) {
    const int e = T.edge[k];
    for (int q = N.edge_reset_off[e]; q < N.edge_reset_off[e + 1]; ++q) {
      const int x = N.resets[q];
      if (!constrain(t, Y, x, 0, kZeroLe) || !constrain(t, Y, 0, x, kZeroLe)) return false;
    }
  }
  for (int k = 0; k < T.ne; ++k) {
    const int e = T.edge[k];
    for (int q = N.edge_reset_off[e]; q < N.edge_reset_off[e + 1]; ++q) free_clock(t, Y, N.resets[q]);
  }
  for (int k = 0; k < T.ne; ++k) {
    const int e = T.edge[k];
    if (!apply_cons(t, Y, N.cons, N.edge_guard_off[e], N.edge_guard_off[e + 1])) return false;
  }
  for (int k = 0; k < T.nab; ++k)
    if (!apply_abstain(N, t, Y, T.P, T.ab_part[k], T.ab_opt[k])) return false;
  if (!apply_inv(N, t, Y, sl) || !avoid_cut(N, t, Y, sl, si)) return false;
  frozen_flags(N, sl, si, c, u);
  if (!c && !u) {
    down(t, Y);
    if (!apply_inv(N, t, Y, sl) || !avoid_cut(N, t, Y, sl, si)) return false;
  }
  return !is_empty(t, Y);
}

// ---------------------------------------------------------------------------------------------
// the sweep
// ---------------------------------------------------------------------------------------------
template <int D>
struct FedStack {   // depth-first subtraction stack for the "is a zone inside this federation" test
  int stack[kFedMax + 1][D];
  int sidx[kFedMax + 1];
  int spos[kFedMax + 1];
};

// Zone k of W[v], this lane's row.
template <int D>
__device__ __forceinline__ void load_w(const Tile<D>& t, const Fix& fx, const Store& st, long long v, int k,
                                       int (&r)[D]) {
  const long long o = fx.woff[v];
  load_rows(t, r, o < 0 ? st.nzone + v * D * D : fx.warena + (o + k) * D * D);
}
// Rows of the tile's own scratch federation (written and read by the same lanes).
template <int D>
__device__ __forceinline__ void fed_get(const Tile<D>& t, const int* F, int k, int (&r)[D]) {
  const int* row = F + (long long)k * D * D + t.i * D;
#pragma unroll
  for (int j = 0; j < D; ++j) r[j] = row[j];
}
template <int D>
__device__ __forceinline__ void fed_put(const Tile<D>& t, int* F, int k, const int (&r)[D]) {
  int* row = F + (long long)k * D * D + t.i * D;
#pragma unroll
  for (int j = 0; j < D; ++j) row[j] = r[j];
}
// Add the non-empty zone x to the federation F (n zones, at most K): dropped when a zone of F
// contains it; zones it contains are dropped; exact convex unions with zones of F are taken
// (fed_compact, src/liveness/operators.cpp:428). False when F would exceed K.
template <int D>
__device__ bool fed_add(const Tile<D>& t, int* F, int& n, int K, int (&x)[D]) {
  int f[D];
  for (int k = 0; k < n; ++k) {
    fed_get(t, F, k, f);
    if (includes(t, f, x)) return true;
  }
  for (bool merged = true; merged;) {
    merged = false;
    for (int k = 0; k < n;) {
      fed_get(t, F, k, f);
      if (includes(t, x, f)) {
        if (k != n - 1) { fed_get(t, F, n - 1, f); fed_put(t, F, k, f); }
        --n;
        continue;
      }
      ++k;
    }
    for (int k = 0; k < n; ++k) {
      fed_get(t, F, k, f);
      if (try_union(t, x, f)) {
        if (k != n - 1) { fed_get(t, F, n - 1, f); fed_put(t, F, k, f); }
        --n;
        merged = true;
        break;
      }
    }
  }
  if (n >= K) return false;
  fed_put(t, F, n, x);
  ++n;
  return true;
}

// One relaxation of every node on the dirty list (Jacobi: values are read from woff/wcnt and the
// new ones written to woff2/wcnt2). A node's zones covered whole by one candidate (a stop piece
// or a predecessor) survive unchanged; otherwise the candidates' intersections with its zones are
// collected into the tile's scratch federation, and the node changes when some zone is not
// covered by their union.
template <int D>
__global__ void __launch_bounds__(kBlock) k_gfp_relax(const NetView* nets, Store st, Edges ed, Fix fx, Ctl* ctl,
                                                      long long ndirty) {
  Tile<D> t;
  if (!make_tile(t, threadIdx.x & 31)) return;
  const long long tile = tile_id<D>();
  int* F = fx.scratch + tile * (long long)fx.K * D * D;
  FedStack<D> S;
  TransRec T;
  const int ishift = nets[0].inst_shift;
  unsigned long long npre = 0;
  for (long long w = tile; w < ndirty; w += tile_count<D>()) {
    const long long v = fx.dlist[w];
    const int nwv = fx.wcnt[v];
    if (nwv == 0 || fx.swhole[v]) continue;
    const unsigned long long hk = st.nkey[v];
    const int inst = (int)(hk >> ishift);
    const NetView& N = nets[inst];
    int locs[kMaxProcs], ints[kMaxInts], tl[kMaxProcs], ti[kMaxInts];
    key_decode(N, key_part(hk, ishift), locs, ints);
    const unsigned long long full = nwv >= 64 ? ~0ull : ((1ull << nwv) - 1);
    unsigned long long cov = 0;
    int nf = 0;
    bool over = false;
    auto offer = [&](const int (&Y)[D]) {
      for (int i = 0; i < nwv && !over; ++i) {
        int wz[D], x[D];
        load_w(t, fx, st, v, i, wz);
        bool inside = true;
#pragma unroll
        for (int j = 0; j < D; ++j) { x[j] = wz[j] < Y[j] ? wz[j] : Y[j]; inside &= wz[j] <= Y[j]; }
        close(t, x);
        if (is_empty(t, x)) continue;
        if (t.all(inside)) cov |= 1ull << i;
        if (!fed_add(t, F, nf, fx.K, x)) over = true;
      }
    };
    for (int sp = fx.shead[v]; sp >= 0 && cov != full && !over; sp = fx.snext[sp]) {
      int Y[D];
      load_rows(t, Y, fx.spiece + (long long)sp * D * D);
      offer(Y);
    }
    for (int k = fx.eoff[v]; k < fx.eoff[v + 1] && cov != full && !over; ++k) {
      const int e = fx.eidx[k];
      const int j = ed.dst[e];
      const int nj = fx.wcnt[j];
      if (nj == 0) continue;
      if (!find_trans(N, locs, ints, ed.raw[e], T)) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
      key_decode(N, key_part(st.nkey[j], ishift), tl, ti);
      for (int y = 0; y < nj && cov != full && !over; ++y) {
        int Y[D];
        load_w(t, fx, st, j, y, Y);
        ++npre;
        if (pre_step(N, t, Y, T, locs, ints, tl, ti)) offer(Y);
      }
    }
    if (over) { if (t.i == 0) ctl->fed_over = 1; continue; }
    if (cov == full) continue;
    bool changed = false;
    for (int i = 0; i < nwv && !changed; ++i) {
      if ((cov >> i) & 1) continue;
      int wz[D];
      load_w(t, fx, st, v, i, wz);
      changed = dfs_subtract(t, wz, S, nf, [&](int k, int (&W)[D]) { fed_get(t, F, k, W); },
                             [](const int (&)[D]) { return false; }) > 0;
    }
    if (!changed) continue;
    long long off = 0;
    if (t.i == 0) off = (long long)atomicAdd(&ctl->walloc, (unsigned long long)nf);
    off = (long long)t.shfl64((unsigned long long)off, 0);
    if (off + nf > fx.wcap) { if (t.i == 0) atomicMax(&ctl->err, 4u); continue; }
    for (int k = 0; k < nf; ++k) {
      int r[D];
      fed_get(t, F, k, r);
      store_rows(t, r, fx.warena + (off + k) * D * D);
    }
    if (t.i == 0) {
      fx.woff2[v] = off;
      fx.wcnt2[v] = nf;
      fx.changed[v] = 1;
      fx.clist[atomicAdd(&ctl->nchanged, 1ull)] = (int)v;
    }
  }
  if (t.i == 0 && npre) atomicAdd(&ctl->npre, npre);
}

static __global__ void k_gfp_init(Fix fx, long long nnodes) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nnodes; v += (long long)gridDim.x * blockDim.x) {
    fx.woff[v] = -1; fx.wcnt[v] = 1; fx.dirty[v] = 0; fx.changed[v] = 0; fx.dlist[v] = (int)v;
  }
}
static __global__ void k_gfp_commit(Fix fx, Ctl* ctl) {
  const long long n = (long long)ctl->nchanged;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int v = fx.clist[c];
    fx.woff[v] = fx.woff2[v];
    fx.wcnt[v] = fx.wcnt2[v];
  }
}
static __global__ void k_gfp_mark(Edges ed, long long nedges, Fix fx) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nedges; e += (long long)gridDim.x * blockDim.x)
    if (fx.changed[ed.dst[e]]) fx.dirty[ed.src[e]] = 1;
}
// The next round's dirty list; live roots (the level-0 nodes, ids below nroots) are counted.
static __global__ void k_gfp_collect(Fix fx, long long nnodes, const int* nlevel, Ctl* ctl) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nnodes; v += (long long)gridDim.x * blockDim.x) {
    fx.changed[v] = 0;
    if (fx.dirty[v]) { fx.dirty[v] = 0; fx.dlist[atomicAdd(&ctl->ndirty, 1ull)] = (int)v; }
    if (nlevel[v] == 0 && fx.wcnt[v] > 0) atomicAdd(&ctl->nroots_live, 1ull);
  }
}
// Copy every node's stored W into a fresh arena.
template <int D>
__global__ void k_gfp_compact(Fix fx, long long nnodes, int* narena, unsigned long long* nalloc) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nnodes; v += (long long)gridDim.x * blockDim.x) {
    const long long o = fx.woff[v];
    const int c = fx.wcnt[v];
    if (o < 0 || c == 0) continue;
    const long long no = (long long)atomicAdd(nalloc, (unsigned long long)c);
    for (long long k = 0; k < (long long)c * D * D; ++k) narena[no * D * D + k] = fx.warena[o * D * D + k];
    fx.woff[v] = no;
  }
}
// Violated iff a root keeps a non-empty W.
static __global__ void k_gfp_verdict_fed(const NetView* nets, Store st, long long nnodes, Fix fx, InstState is) {
  const int ishift = nets[0].inst_shift;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nnodes; v += (long long)gridDim.x * blockDim.x)
    if (st.nlevel[v] == 0 && fx.wcnt[v] > 0) is.found[(int)(st.nkey[v] >> ishift)] = 1;
}

// ---------------------------------------------------------------------------------------------
// CSR of the edges by source: counts, an inclusive scan, then placement
// ---------------------------------------------------------------------------------------------
static __global__ void k_csr_count(Edges ed, long long nedges, int* eoff) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nedges; e += (long long)gridDim.x * blockDim.x)
    atomicAdd(&eoff[ed.src[e] + 1], 1);
}
constexpr int kScanBlock = 1024;
// In-place inclusive scan of a[0..n): each block scans its 1024 entries and leaves its total in
// sums[block]; k_scan_sums scans the totals; k_scan_add adds each block's offset.
static __global__ void k_scan_local(int* a, long long n, int* sums) {
  __shared__ int sh[kScanBlock];
  const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
  int v = i < n ? a[i] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int add = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  if (i < n) a[i] = sh[threadIdx.x];
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = sh[threadIdx.x];
}
static __global__ void k_scan_sums(int* sums, long long nb) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int acc = 0;
    for (long long b = 0; b < nb; ++b) { const int x = sums[b]; sums[b] = acc; acc += x; }
  }
}
static __global__ void k_scan_add(int* a, long long n, const int* sums) {
  const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) a[i] += sums[blockIdx.x];
}
static __global__ void k_csr_fill(Edges ed, long long nedges, const int* eoff, int* eidx, int* fill) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nedges; e += (long long)gridDim.x * blockDim.x) {
    const int u = ed.src[e];
    eidx[eoff[u] + atomicAdd(&fill[u], 1)] = (int)e;
  }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
template <int D>
void Level<D>::incl_probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nsucc, int blocks,
                          cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_incl_probe<D><<<grid_for(nsucc, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, st, ctl, nsucc);
}
template <int D>
void Level<D>::incl_group(Succ sc, Store st, Ctl* ctl, long long nsucc, long long ntouched, cudaStream_t s) {
  k_incl_seg<<<grid_for(ntouched, 256, 1024), 256, 0, s>>>(sc, st, ctl, ntouched);
  k_seg_scatter<<<grid_for(nsucc, 256, 4096), 256, 0, s>>>(sc, st, nsucc);
}
template <int D>
void Level<D>::incl_keep(Succ sc, Store st, Ctl* ctl, long long nsurv, int blocks, cudaStream_t s) {
  (void)ctl;
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_incl_keep<D><<<grid_for(nsurv, TPB, blocks), kBlock, 0, s>>>(sc, st, nsurv);
}
template <int D>
void Level<D>::incl_store(const NetView* nets, InstState is, Succ sc, Store st, Front out, Ctl* ctl, long long nsurv,
                          int level, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_incl_store<D><<<grid_for(nsurv, TPB, blocks), kBlock, 0, s>>>(nets, is, sc, st, out, ctl, nsurv, level);
}
template <int D>
void Level<D>::incl_lists(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long ntouched,
                          cudaStream_t s) {
  k_incl_lists<<<grid_for(ntouched, 8, 4096), 256, 0, s>>>(nets, is, sc, st, ctl, ntouched);
}
template <int D>
void Level<D>::incl_cover(Succ sc, Store st, Ctl* ctl, long long nsurv, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  k_incl_cover<D><<<grid_for(nsurv, TPB, blocks), kBlock, 0, s>>>(sc, st, ctl, nsurv);
}
template <int D>
void Level<D>::incl_edges(Succ sc, Front fr, Edges ed, Ctl* ctl, long long nsucc, cudaStream_t s) {
  k_incl_edges<<<grid_for(nsucc, 256, 8192), 256, 0, s>>>(sc, fr, ed, ctl, nsucc);
}
template <int D>
void Level<D>::stop_fed(const NetView* nets, InstState is, Store st, long long n0, long long n1, const int* nodes,
                        Fix fx, Ctl* ctl, int witness, int blocks, cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  if (n1 > n0) k_stop_fed<D><<<grid_for(n1 - n0, TPB, blocks), kBlock, 0, s>>>(nets, is, st, n0, n1, nodes, fx, ctl, witness);
}
template <int D>
void Level<D>::edge_csr(Edges ed, long long nedges, long long nnodes, int* eoff, int* eidx, int* tmp, cudaStream_t s) {
  if (nedges > 0) k_csr_count<<<grid_for(nedges, 256, 8192), 256, 0, s>>>(ed, nedges, eoff);
  const long long n = nnodes + 1, nb = (n + kScanBlock - 1) / kScanBlock;
  k_scan_local<<<(unsigned)nb, kScanBlock, 0, s>>>(eoff, n, tmp);
  k_scan_sums<<<1, 32, 0, s>>>(tmp, nb);
  k_scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(eoff, n, tmp);
  cudaMemsetAsync(tmp, 0, (size_t)(nnodes > nb ? nnodes : nb) * 4, s);
  if (nedges > 0) k_csr_fill<<<grid_for(nedges, 256, 8192), 256, 0, s>>>(ed, nedges, eoff, eidx, tmp);
}
template <int D>
void Level<D>::gfp_init(Fix fx, long long nnodes, Ctl* ctl, cudaStream_t s) {
  (void)ctl;
  if (nnodes > 0) k_gfp_init<<<grid_for(nnodes, 256, 8192), 256, 0, s>>>(fx, nnodes);
}
template <int D>
long long Level<D>::relax_tiles(int blocks) {
  return (long long)blocks * (kBlock / 32) * (32 / D);
}
template <int D>
void Level<D>::gfp_relax(const NetView* nets, Store st, Edges ed, Fix fx, Ctl* ctl, long long ndirty, int blocks,
                         cudaStream_t s) {
  constexpr int TPB = (kBlock / 32) * (32 / D);
  if (ndirty > 0) k_gfp_relax<D><<<grid_for(ndirty, TPB, blocks), kBlock, 0, s>>>(nets, st, ed, fx, ctl, ndirty);
}
template <int D>
void Level<D>::gfp_round_end(Edges ed, long long nedges, long long nnodes, Fix fx, const int* nlevel, Ctl* ctl,
                             cudaStream_t s) {
  k_gfp_commit<<<4096, 256, 0, s>>>(fx, ctl);
  if (nedges > 0) k_gfp_mark<<<grid_for(nedges, 256, 8192), 256, 0, s>>>(ed, nedges, fx);
  cudaMemsetAsync(&ctl->ndirty, 0, 8, s);
  cudaMemsetAsync(&ctl->nroots_live, 0, 8, s);
  if (nnodes > 0) k_gfp_collect<<<grid_for(nnodes, 256, 8192), 256, 0, s>>>(fx, nnodes, nlevel, ctl);
}
template <int D>
void Level<D>::gfp_compact(Fix fx, long long nnodes, int* narena, unsigned long long* nalloc, cudaStream_t s) {
  if (nnodes > 0) k_gfp_compact<D><<<grid_for(nnodes, 256, 8192), 256, 0, s>>>(fx, nnodes, narena, nalloc);
}
template <int D>
void Level<D>::gfp_verdict_fed(const NetView* nets, Store st, long long nnodes, Fix fx, InstState is, cudaStream_t s) {
  if (nnodes > 0) k_gfp_verdict_fed<<<grid_for(nnodes, 256, 8192), 256, 0, s>>>(nets, st, nnodes, fx, is);
}

}  // namespace hgb
