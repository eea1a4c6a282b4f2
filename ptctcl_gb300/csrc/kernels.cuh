// kernels.cuh -- the level-step kernels of the zone-graph engine, templated on the DBM dimension D.
//
// One BFS level is:  expand -> probe -> (deadlock test) -> group -> merge.
//
//  * expand  : one tile per frontier state. Enumerates the transitions in the reference's emission
//              order (local edges, binary handshakes, broadcasts; src/liveness/operators.cpp:55-206)
//              and runs the successor pipeline of close_succ_zone (include/hora/detail/
//              semantics.hpp:522-568) on the zone held row-per-lane in registers.
//  * probe   : one tile per successor. Finds or inserts the discrete key in the device hash table
//              (atomic CAS) and drops the successor if a stored zone of that key simulates it
//              (a_LU, NetPassedT::probe_kill, include/hora/detail/passed_set.hpp:239-266).
//  * group   : the survivors of each key are gathered into one contiguous segment.
//  * merge   : one tile per touched key. Applies NetPassedT::add's folds (passed_set.hpp:287-444)
//              to the key's survivors in canonical order -- (parent key, parent rank, emission
//              ordinal) -- so the stored antichains do not depend on thread scheduling, then emits
//              the key's new zones into the next frontier.
//
// Memory: zones are dense row-major int32[D*D]; frontier, successor and node arrays are
// structure-of-arrays in HBM. Nothing here allocates; the host sizes every buffer.
#pragma once
#include "dbm_tile.cuh"
#include "engine.cuh"

namespace hgb {

// ---------------------------------------------------------------------------------------------
// Per-lane discrete state helpers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void key_decode(const NetView& N, unsigned long long key, int* locs, int* ints) {
  for (int p = 0; p < N.nprocs; ++p)
    locs[p] = (int)((key >> N.kshift[p]) & ((1ull << N.kwidth[p]) - 1));
  for (int v = 0; v < N.nints; ++v) {
    const int f = N.nprocs + v;
    ints[v] = (int)((key >> N.kshift[f]) & ((1ull << N.kwidth[f]) - 1)) + N.int_lo[v];
  }
}
__device__ __forceinline__ unsigned long long key_encode(const NetView& N, const int* locs, const int* ints) {
  unsigned long long k = 0;
  for (int p = 0; p < N.nprocs; ++p) k |= (unsigned long long)(unsigned)locs[p] << N.kshift[p];
  for (int v = 0; v < N.nints; ++v)
    k |= (unsigned long long)(unsigned)(ints[v] - N.int_lo[v]) << N.kshift[N.nprocs + v];
  return k;
}

__device__ __forceinline__ bool iatoms_ok(const int* a, int n, const int* ints) {
  for (int k = 0; k < n; ++k) {
    const int x = ints[a[3 * k]], op = a[3 * k + 1], v = a[3 * k + 2];
    bool r;
    switch (op) {
      case 0: r = x == v; break;
      case 1: r = x != v; break;
      case 2: r = x < v; break;
      case 3: r = x <= v; break;
      case 4: r = x > v; break;
      default: r = x >= v; break;
    }
    if (!r) return false;
  }
  return true;
}
__device__ __forceinline__ bool int_ok(const NetView& N, int e, const int* ints) {
  const int a0 = N.edge_iguard_off[e], a1 = N.edge_iguard_off[e + 1];
  return iatoms_ok(N.iatoms + 3 * a0, a1 - a0, ints);
}
__device__ __forceinline__ bool committed_at(const NetView& N, int p, int l) {
  return (N.loc_flags[N.loc_base[p] + l] & 2) != 0;
}
__device__ __forceinline__ void apply_iupd(const NetView& N, int e, int* ints) {
  for (int u = N.edge_iupd_off[e]; u < N.edge_iupd_off[e + 1]; ++u) ints[N.iupds[2 * u]] = N.iupds[2 * u + 1];
}
__device__ __forceinline__ unsigned long long reset_mask(const NetView& N, int e) {
  unsigned long long r = 0;
  for (int q = N.edge_reset_off[e]; q < N.edge_reset_off[e + 1]; ++q) r |= 1ull << N.resets[q];
  return r;
}

// urgent_sync_enabled (semantics.hpp:118-139)
inline __device__ bool urgent_sync_enabled(const NetView& N, const int* locs, const int* ints) {
  if (!N.has_urgent_chan) return false;
  for (int i = 0; i < N.nprocs; ++i) {
    const int gi = N.loc_base[i] + locs[i];
    for (int k = N.eloc_off[gi]; k < N.eloc_off[gi + 1]; ++k) {
      const int se = N.eloc[k];
      const int ch = N.edge_chan[se];
      if (ch < 0 || N.edge_dir[se] != 1 || !(N.chan_flags[ch] & 2)) continue;
      if (!int_ok(N, se, ints)) continue;
      if (N.chan_flags[ch] & 1) return true;
      for (int j = 0; j < N.nprocs; ++j) {
        if (j == i) continue;
        const int gj = N.loc_base[j] + locs[j];
        for (int q = N.eloc_off[gj]; q < N.eloc_off[gj + 1]; ++q) {
          const int re = N.eloc[q];
          if (N.edge_chan[re] == ch && N.edge_dir[re] == -1 && int_ok(N, re, ints)) return true;
        }
      }
    }
  }
  return false;
}
// frozen_flags (semantics.hpp:160-169)
__device__ __forceinline__ void frozen_flags(const NetView& N, const int* locs, const int* ints, bool& comm, bool& urg) {
  comm = urg = false;
  for (int p = 0; p < N.nprocs; ++p) {
    const int f = N.loc_flags[N.loc_base[p] + locs[p]];
    comm |= (f & 2) != 0;
    urg |= (f & 1) != 0;
  }
  if (!urg && urgent_sync_enabled(N, locs, ints)) urg = true;
}

// ---------------------------------------------------------------------------------------------
// Zone pipeline pieces on a tile
// ---------------------------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ bool apply_cons(const Tile<D>& t, int (&r)[D], const int* cons, int c0, int c1) {
  for (int c = c0; c < c1; ++c)
    if (!constrain(t, r, cons[3 * c], cons[3 * c + 1], cons[3 * c + 2])) return false;
  return true;
}
template <int D>
__device__ __forceinline__ bool apply_inv(const NetView& N, const Tile<D>& t, int (&r)[D], const int* locs) {
  for (int p = 0; p < N.nprocs; ++p) {
    const int gl = N.loc_base[p] + locs[p];
    if (!apply_cons(t, r, N.cons, N.loc_inv_off[gl], N.loc_inv_off[gl + 1])) return false;
  }
  return true;
}
template <int D>
__device__ __forceinline__ void apply_resets(const NetView& N, const Tile<D>& t, int (&r)[D], int e) {
  for (int q = N.edge_reset_off[e]; q < N.edge_reset_off[e + 1]; ++q) reset(t, r, N.resets[q]);
}
__device__ __forceinline__ bool pred_disc(const int* loc, int nloc, const int* ia, int nint, const int* locs,
                                          const int* ints) {
  for (int k = 0; k < nloc; ++k) {   // l >= 0: at location l; l < 0: anywhere but -l-1
    const int l = loc[2 * k + 1], at = locs[loc[2 * k]];
    if (l >= 0 ? at != l : at == -l - 1) return false;
  }
  return iatoms_ok(ia, nint, ints);
}
// Leads-to restriction to !q: where q's discrete part holds, cut the zone to the complement of
// q's clock atom (a single constraint, so the complement is convex and the cut exact). False when
// nothing is left -- including everywhere q is purely discrete.
template <int D>
__device__ __forceinline__ bool avoid_cut(const NetView& N, const Tile<D>& t, int (&r)[D], const int* tl,
                                          const int* ti) {
  if (N.av_on && N.av_psi) {   // E[] psi (exists_invariant_run.cpp:70-91)
    if (!pred_disc(N.av_loc, N.av_nloc, N.av_int, N.av_nint, tl, ti)) return false;
    return apply_cons(t, r, N.av_clk, 0, N.av_nclk);
  }
  if (!N.av_on || !pred_disc(N.av_loc, N.av_nloc, N.av_int, N.av_nint, tl, ti)) return true;
  if (N.av_nclk == 0) return false;
  return constrain(t, r, N.av_neg[0], N.av_neg[1], N.av_neg[2]);
}

// close_succ_zone (semantics.hpp:522-568), with the leads-to restriction adjoined to the target
// invariant when it is on. False when the target invariant is unsatisfiable; the caller tests
// emptiness afterwards.
template <int D>
__device__ bool close_succ(const NetView& N, const Tile<D>& t, int (&r)[D], const int* tl, const int* ti, int emode) {
  if (!apply_inv(N, t, r, tl)) return false;
  if (!avoid_cut(N, t, r, tl, ti)) return false;
  bool c, u;
  frozen_flags(N, tl, ti, c, u);
  if (!c && !u) {
    delay(t, r);
    apply_inv(N, t, r, tl);
    avoid_cut(N, t, r, tl, ti);
  }
  // reset_inactive (semantics.hpp:186-215)
  unsigned long long a = N.qmask;
  for (int p = 0; p < N.nprocs; ++p) a |= N.act[N.loc_base[p] + tl[p]];
  unsigned long long dead = ~a & (((1ull << N.nclocks) - 1) << 1);
  while (dead) {
    const int k = __ffsll((long long)dead) - 1;
    dead &= dead - 1;
    reset(t, r, k);
  }
  if (emode == 1) extrap_lu_plus(t, r, N.L, N.U);
  return true;
}

// NetTarget match (reachable_net's is_target, src/reachability/engine.cpp:2272-2279).
template <int D>
__device__ bool target_hit(const NetView& N, const Tile<D>& t, const int (&r)[D], const int* locs, const int* ints) {
  if (N.t_never) return false;
  for (int k = 0; k < N.t_nloc; ++k)
    if (N.t_loc[2 * k + 1] >= 0 ? locs[N.t_loc[2 * k]] != N.t_loc[2 * k + 1]
                                : locs[N.t_loc[2 * k]] == -N.t_loc[2 * k + 1] - 1) return false;
  if (!iatoms_ok(N.t_int, N.t_nint, ints)) return false;
  int z[D];
#pragma unroll
  for (int j = 0; j < D; ++j) z[j] = r[j];
  return apply_cons(t, z, N.t_clk, 0, N.t_nclk);
}

// ---------------------------------------------------------------------------------------------
// Transition enumeration (successors_net, src/reachability/engine.cpp:243-368): calls
// step(guard-applied zone path) in emission order. The functor receives the working zone after the
// guards (in `r`), and must apply resets/updates itself through the arguments it is given.
//
// Each emitted successor reaches `emit(tl, ti, r)` with r closed and non-empty.
// ---------------------------------------------------------------------------------------------
struct BcastParts {
  int n;
  int proc[kMaxProcs];
  int ne[kMaxProcs];                    // receive-edge options
  int nab[kMaxProcs];                   // abstain options
  int edge[kMaxProcs][kMaxRecvEdges];
};

// Build the receiver options of a broadcast send (build_broadcast_parts, semantics.hpp:275-303).
// Returns false when a process has more enabled receivers than the device tables hold.
inline __device__ bool build_parts(const NetView& N, const int* locs, const int* ints, int se, int sender, BcastParts& P) {
  P.n = 0;
  const int ch = N.edge_chan[se];
  for (int j = 0; j < N.nprocs; ++j) {
    if (j == sender) continue;
    const int gj = N.loc_base[j] + locs[j];
    int ne = 0, nab = 1;
    bool empty_guard = false;
    for (int q = N.eloc_off[gj]; q < N.eloc_off[gj + 1]; ++q) {
      const int re = N.eloc[q];
      if (N.edge_chan[re] == ch && N.edge_dir[re] == -1 && int_ok(N, re, ints)) {
        if (ne == kMaxRecvEdges) return false;
        P.edge[P.n][ne++] = re;
        const int len = N.edge_guard_off[re + 1] - N.edge_guard_off[re];
        if (len == 0) empty_guard = true;
        else nab *= len;
      }
    }
    if (ne == 0) continue;
    P.proc[P.n] = j;
    P.ne[P.n] = ne;
    P.nab[P.n] = empty_guard ? 0 : nab;
    P.n++;
  }
  return true;
}
// Apply abstain option k of part t: one negated atom per enabled receiver guard, the first guard
// varying slowest (the order build_broadcast_parts' cross product produces).
template <int D>
__device__ bool apply_abstain(const NetView& N, const Tile<D>& t, int (&r)[D], const BcastParts& P, int part, int k) {
  int rem = k;
  int idx[kMaxRecvEdges];
  for (int g = P.ne[part] - 1; g >= 0; --g) {
    const int e = P.edge[part][g];
    const int len = N.edge_guard_off[e + 1] - N.edge_guard_off[e];
    idx[g] = rem % len;
    rem /= len;
  }
  for (int g = 0; g < P.ne[part]; ++g) {
    const int c = N.edge_guard_off[P.edge[part][g]] + idx[g];
    if (!constrain(t, r, N.cons[3 * c + 1], N.cons[3 * c], r_negate(N.cons[3 * c + 2]))) return false;
  }
  return true;
}

// Enumerate the successors of (locs, ints, src). `emit(tl, ti, z, raw)` is called for each non-empty
// successor zone, in emission order; `raw` numbers the transition among every candidate the
// enumeration visits (integer guards and committed filter passed, zone not yet tested), so
// find_trans() rebuilds its recipe from the discrete state alone. Returns false if a broadcast
// exceeded the device tables.
template <int D, class Emit>
__device__ bool for_each_successor(const NetView& N, const Tile<D>& t, const int* locs, const int* ints,
                                   const int (&src)[D], int emode, Emit&& emit) {
  int tl[kMaxProcs], ti[kMaxInts];
  int z[D];
  bool src_c, src_u;
  frozen_flags(N, locs, ints, src_c, src_u);
  int raw = 0;
  // ---- local edges ----
  for (int p = 0; p < N.nprocs; ++p) {
    if (src_c && !committed_at(N, p, locs[p])) continue;
    const int gp = N.loc_base[p] + locs[p];
    for (int k = N.eloc_off[gp]; k < N.eloc_off[gp + 1]; ++k) {
      const int e = N.eloc[k];
      if (N.edge_chan[e] >= 0) continue;
      if (!int_ok(N, e, ints)) continue;
      const int rw = raw++;
#pragma unroll
      for (int j = 0; j < D; ++j) z[j] = src[j];
      if (!apply_cons(t, z, N.cons, N.edge_guard_off[e], N.edge_guard_off[e + 1])) continue;
      apply_resets(N, t, z, e);
      for (int q = 0; q < N.nprocs; ++q) tl[q] = locs[q];
      for (int v = 0; v < N.nints; ++v) ti[v] = ints[v];
      tl[p] = N.edge_tgt[e];
      apply_iupd(N, e, ti);
      if (!close_succ(N, t, z, tl, ti, emode)) continue;
      if (is_empty(t, z)) continue;
      emit(tl, ti, z, rw);
    }
  }
  // ---- binary synchronisation ----
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
          const int rw = raw++;
#pragma unroll
          for (int jj = 0; jj < D; ++jj) z[jj] = src[jj];
          if (!apply_cons(t, z, N.cons, N.edge_guard_off[se], N.edge_guard_off[se + 1])) continue;
          if (!apply_cons(t, z, N.cons, N.edge_guard_off[re], N.edge_guard_off[re + 1])) continue;
          apply_resets(N, t, z, se);
          apply_resets(N, t, z, re);
          for (int w = 0; w < N.nprocs; ++w) tl[w] = locs[w];
          for (int v = 0; v < N.nints; ++v) ti[v] = ints[v];
          tl[i] = N.edge_tgt[se];
          tl[j] = N.edge_tgt[re];
          apply_iupd(N, se, ti);
          apply_iupd(N, re, ti);
          if (!close_succ(N, t, z, tl, ti, emode)) continue;
          if (is_empty(t, z)) continue;
          emit(tl, ti, z, rw);
        }
      }
    }
  }
  // ---- broadcast synchronisation ----
  BcastParts P;
  for (int i = 0; i < N.nprocs; ++i) {
    const int gi = N.loc_base[i] + locs[i];
    for (int k = N.eloc_off[gi]; k < N.eloc_off[gi + 1]; ++k) {
      const int se = N.eloc[k];
      const int ch = N.edge_chan[se];
      if (ch < 0 || N.edge_dir[se] != 1 || !(N.chan_flags[ch] & 1)) continue;
      if (!int_ok(N, se, ints)) continue;
      if (!build_parts(N, locs, ints, se, i, P)) return false;
      int pick[kMaxProcs];
      for (int q = 0; q < P.n; ++q) pick[q] = 0;
      for (;;) {
        bool part_comm = committed_at(N, i, locs[i]);
        for (int q = 0; q < P.n; ++q)
          if (pick[q] < P.ne[q] && committed_at(N, P.proc[q], locs[P.proc[q]])) part_comm = true;
        if (!src_c || part_comm) {
          const int rw = raw++;
#pragma unroll
          for (int jj = 0; jj < D; ++jj) z[jj] = src[jj];
          bool ok = apply_cons(t, z, N.cons, N.edge_guard_off[se], N.edge_guard_off[se + 1]);
          for (int q = 0; ok && q < P.n; ++q) {
            if (pick[q] < P.ne[q]) {
              const int re = P.edge[q][pick[q]];
              ok = apply_cons(t, z, N.cons, N.edge_guard_off[re], N.edge_guard_off[re + 1]);
            } else {
              ok = apply_abstain(N, t, z, P, q, pick[q] - P.ne[q]);
            }
          }
          if (ok) {
            for (int w = 0; w < N.nprocs; ++w) tl[w] = locs[w];
            for (int v = 0; v < N.nints; ++v) ti[v] = ints[v];
            tl[i] = N.edge_tgt[se];
            apply_iupd(N, se, ti);
            apply_resets(N, t, z, se);
            for (int q = 0; q < P.n; ++q) {
              if (pick[q] >= P.ne[q]) continue;
              const int re = P.edge[q][pick[q]];
              tl[P.proc[q]] = N.edge_tgt[re];
              apply_iupd(N, re, ti);
              apply_resets(N, t, z, re);
            }
            if (close_succ(N, t, z, tl, ti, emode) && !is_empty(t, z)) emit(tl, ti, z, rw);
          }
        }
        if (P.n == 0) break;
        int q = 0;
        for (; q < P.n; ++q) {
          if (++pick[q] < P.ne[q] + P.nab[q]) break;
          pick[q] = 0;
        }
        if (q == P.n) break;
      }
    }
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Deadlock predicate (state_has_deadlock, src/reachability/deadlock.cpp:74-270)
//
// The escape regions are collected into per-lane local memory (one row per escape), and the final
// question "is Z covered by the union of the escapes?" is answered by a depth-first subtraction
// whose stack also lives in local memory: Z \ W_i splits into the disjoint pieces
// Z ∧ c_1 ∧ .. ∧ c_{m-1} ∧ ¬c_m over W_i's tightening constraints, each of which must be covered by
// the later escapes. Returns 1 (deadlock), 0 (none) or -1 (more escapes than kMaxEscapes).
// ---------------------------------------------------------------------------------------------
template <int D>
struct DlScratch {
  int w[kMaxEscapes][D];        // escape rows
  int stack[kMaxEscapes + 1][D];// pieces under test
  int sidx[kMaxEscapes + 1];    // escape index each piece is tested against
  int spos[kMaxEscapes + 1];    // next constraint position of the split
};

// Collect the escape regions of (locs, ints, zone): every enabled transition's guard region of
// the delay-closed zone Z (returned), pulled back through the target invariant (add_src,
// deadlock.cpp:106-149), then let down unless the state is frozen, into S.w[0..nw). Returns 0 when
// no valuation can deadlock (no concrete state, or one escape is all of Z), 1 when the escapes are
// collected, -1 when there are more than kMaxEscapes.
template <int D>
__device__ int collect_escapes(const NetView& N, const Tile<D>& t, const int* locs, const int* ints,
                               const int (&zone)[D], DlScratch<D>& S, int (&Z)[D], int& nw_out) {
  bool src_c, src_u;
  frozen_flags(N, locs, ints, src_c, src_u);
  const bool frozen = src_c || src_u;
  int g[D];
#pragma unroll
  for (int j = 0; j < D; ++j) Z[j] = zone[j];
  if (!frozen) delay(t, Z);
  if (!apply_inv(N, t, Z, locs)) return 0;
  int nw = 0;
  bool covered = false, overflow = false;
  int tl[kMaxProcs];
  // add_src (deadlock.cpp:106-149): pull the target invariant back through the resets
  auto add_src = [&](int (&gz)[D], unsigned long long rmask) {
    for (int p = 0; p < N.nprocs; ++p) {
      const int gl = N.loc_base[p] + tl[p];
      for (int c = N.loc_inv_off[gl]; c < N.loc_inv_off[gl + 1]; ++c) {
        int ci = N.cons[3 * c], cj = N.cons[3 * c + 1];
        const int b = N.cons[3 * c + 2];
        if ((rmask >> ci) & 1) ci = 0;
        if ((rmask >> cj) & 1) cj = 0;
        if (ci == cj) { if (b < kZeroLe) return; continue; }
        if (!constrain(t, gz, ci, cj, b)) return;
      }
    }
    bool same = true;
#pragma unroll
    for (int j = 0; j < D; ++j) same &= (gz[j] == Z[j]);
    if (t.all(same)) { covered = true; return; }
    if (nw == kMaxEscapes) { overflow = true; return; }
#pragma unroll
    for (int j = 0; j < D; ++j) S.w[nw][j] = gz[j];
    ++nw;
  };
  // local edges
  for (int p = 0; p < N.nprocs && !covered; ++p) {
    if (src_c && !committed_at(N, p, locs[p])) continue;
    const int gp = N.loc_base[p] + locs[p];
    for (int k = N.eloc_off[gp]; k < N.eloc_off[gp + 1] && !covered; ++k) {
      const int e = N.eloc[k];
      if (N.edge_chan[e] >= 0 || !int_ok(N, e, ints)) continue;
#pragma unroll
      for (int j = 0; j < D; ++j) g[j] = Z[j];
      if (!apply_cons(t, g, N.cons, N.edge_guard_off[e], N.edge_guard_off[e + 1])) continue;
      for (int q = 0; q < N.nprocs; ++q) tl[q] = locs[q];
      tl[p] = N.edge_tgt[e];
      add_src(g, reset_mask(N, e));
    }
  }
  // binary synchronisation
  for (int i = 0; i < N.nprocs && !covered; ++i) {
    const int gi = N.loc_base[i] + locs[i];
    for (int k = N.eloc_off[gi]; k < N.eloc_off[gi + 1] && !covered; ++k) {
      const int se = N.eloc[k];
      const int ch = N.edge_chan[se];
      if (ch < 0 || N.edge_dir[se] != 1 || (N.chan_flags[ch] & 1)) continue;
      if (!int_ok(N, se, ints)) continue;
      const bool i_comm = committed_at(N, i, locs[i]);
      for (int j = 0; j < N.nprocs && !covered; ++j) {
        if (j == i) continue;
        const int gj = N.loc_base[j] + locs[j];
        for (int q = N.eloc_off[gj]; q < N.eloc_off[gj + 1] && !covered; ++q) {
          const int re = N.eloc[q];
          if (N.edge_chan[re] != ch || N.edge_dir[re] != -1) continue;
          if (src_c && !(i_comm || committed_at(N, j, locs[j]))) continue;
          if (!int_ok(N, re, ints)) continue;
#pragma unroll
          for (int jj = 0; jj < D; ++jj) g[jj] = Z[jj];
          if (!apply_cons(t, g, N.cons, N.edge_guard_off[se], N.edge_guard_off[se + 1])) continue;
          if (!apply_cons(t, g, N.cons, N.edge_guard_off[re], N.edge_guard_off[re + 1])) continue;
          for (int w = 0; w < N.nprocs; ++w) tl[w] = locs[w];
          tl[i] = N.edge_tgt[se];
          tl[j] = N.edge_tgt[re];
          add_src(g, reset_mask(N, se) | reset_mask(N, re));
        }
      }
    }
  }
  // broadcast synchronisation
  BcastParts P;
  for (int i = 0; i < N.nprocs && !covered; ++i) {
    const int gi = N.loc_base[i] + locs[i];
    for (int k = N.eloc_off[gi]; k < N.eloc_off[gi + 1] && !covered; ++k) {
      const int se = N.eloc[k];
      const int ch = N.edge_chan[se];
      if (ch < 0 || N.edge_dir[se] != 1 || !(N.chan_flags[ch] & 1)) continue;
      if (!int_ok(N, se, ints)) continue;
      if (!build_parts(N, locs, ints, se, i, P)) return -1;
      int pick[kMaxProcs];
      for (int q = 0; q < P.n; ++q) pick[q] = 0;
      for (;;) {
        bool part_comm = committed_at(N, i, locs[i]);
        for (int q = 0; q < P.n; ++q)
          if (pick[q] < P.ne[q] && committed_at(N, P.proc[q], locs[P.proc[q]])) part_comm = true;
        if (!src_c || part_comm) {
#pragma unroll
          for (int jj = 0; jj < D; ++jj) g[jj] = Z[jj];
          bool ok = apply_cons(t, g, N.cons, N.edge_guard_off[se], N.edge_guard_off[se + 1]);
          unsigned long long rm = reset_mask(N, se);
          for (int w = 0; w < N.nprocs; ++w) tl[w] = locs[w];
          tl[i] = N.edge_tgt[se];
          for (int q = 0; ok && q < P.n; ++q) {
            if (pick[q] >= P.ne[q]) { ok = apply_abstain(N, t, g, P, q, pick[q] - P.ne[q]); continue; }
            const int re = P.edge[q][pick[q]];
            ok = apply_cons(t, g, N.cons, N.edge_guard_off[re], N.edge_guard_off[re + 1]);
            rm |= reset_mask(N, re);
            tl[P.proc[q]] = N.edge_tgt[re];
          }
          if (ok) add_src(g, rm);
          if (covered) break;
        }
        if (P.n == 0) break;
        int q = 0;
        for (; q < P.n; ++q) {
          if (++pick[q] < P.ne[q] + P.nab[q]) break;
          pick[q] = 0;
        }
        if (q == P.n) break;
      }
    }
  }
  if (covered) return 0;
  if (overflow) return -1;
  // down() each escape unless frozen; a single escape containing Z settles it
  for (int w = 0; w < nw; ++w) {
    int a[D];
#pragma unroll
    for (int j = 0; j < D; ++j) a[j] = S.w[w][j];
    if (!frozen) {
      down(t, a);
#pragma unroll
      for (int j = 0; j < D; ++j) S.w[w][j] = a[j];
    }
    if (includes(t, a, Z)) return 0;
  }
  nw_out = nw;
  return 1;
}

// Depth-first subtraction of zones W_0..W_{nw-1} (row i of W_k loaded by getw(k, rows)) from Z0:
// Z0 \ W_i splits into the disjoint pieces Z0 ∧ c_1 ∧ .. ∧ c_{m-1} ∧ ¬c_m over W_i's tightening
// constraints, each then taken against the later zones. `piece(R)` is called for every piece no W
// reaches; the walk stops early when it returns false. S provides a stack of nw + 1 rows (stack,
// sidx, spos). Returns the number of pieces reported (0: Z0 ⊆ ∪ W).
template <int D, class Stk, class GetW, class Piece>
__device__ int dfs_subtract(const Tile<D>& t, const int (&Z0)[D], Stk& S, int nw, GetW&& getw, Piece&& piece) {
  int npieces = 0;
  if (nw == 0) { ++npieces; piece(Z0); return npieces; }
  int sp = 0;
#pragma unroll
  for (int j = 0; j < D; ++j) S.stack[0][j] = Z0[j];
  S.sidx[0] = 0;
  S.spos[0] = -1;   // -1: escape index not yet settled for this piece
  while (sp >= 0) {
    int R[D];
#pragma unroll
    for (int j = 0; j < D; ++j) R[j] = S.stack[sp][j];
    int wi = S.sidx[sp];
    if (S.spos[sp] < 0) {
      // first escape from wi on that meets the piece
      int W[D];
      for (; wi < nw; ++wi) {
        getw(wi, W);
        if (intersects(t, R, W)) break;
      }
      if (wi == nw) {                            // a piece no escape reaches
        ++npieces;
        if (!piece(R)) return npieces;
        --sp;
        continue;
      }
      if (includes(t, W, R)) { --sp; continue; }  // piece covered
      S.sidx[sp] = wi;
      S.spos[sp] = 0;
    }
    int W[D];
    getw(wi, W);
    // next tightening constraint (a, b) of W at linear position >= spos
    const int pos0 = S.spos[sp];
    unsigned long long m = 0;   // bit j of this lane's row: W[i][j] < R[i][j]
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j != t.i && W[j] < R[j]) m |= 1ull << j;
    int found_pos = -1;
    for (int a = pos0 / D; a < D && found_pos < 0; ++a) {
      unsigned long long ma = t.shfl64(m, a);
      const int from = (a == pos0 / D) ? pos0 % D : 0;
      ma &= ~((1ull << from) - 1);
      if (ma) found_pos = a * D + (__ffsll((long long)ma) - 1);
    }
    if (found_pos < 0) { --sp; continue; }      // the remainder lies inside W: covered
    const int a = found_pos / D, b = found_pos % D;
    S.spos[sp] = found_pos + 1;
    const int wab = t.shfl(sel(W, b), a);
    int Pc[D];
#pragma unroll
    for (int j = 0; j < D; ++j) Pc[j] = R[j];
    const bool cut = constrain(t, Pc, b, a, r_negate(wab));
    const bool rest = constrain(t, R, a, b, wab);
    if (rest) {
#pragma unroll
      for (int j = 0; j < D; ++j) S.stack[sp][j] = R[j];
    } else {
      S.spos[sp] = D * D;                        // nothing left of this piece after the child
    }
    if (cut) {
      if (wi + 1 >= nw) {                        // the piece escapes every region
        ++npieces;
        if (!piece(Pc)) return npieces;
        continue;
      }
      ++sp;
#pragma unroll
      for (int j = 0; j < D; ++j) S.stack[sp][j] = Pc[j];
      S.sidx[sp] = wi + 1;
      S.spos[sp] = -1;
    }
  }
  return npieces;
}

// The escapes S.w[0..nw) subtracted from Z0 (dfs_subtract over the deadlock scratch).
template <int D, class Piece>
__device__ int subtract_escapes(const Tile<D>& t, const int (&Z0)[D], DlScratch<D>& S, int nw, Piece&& piece) {
  return dfs_subtract(t, Z0, S, nw,
                      [&](int k, int (&W)[D]) {
#pragma unroll
                        for (int j = 0; j < D; ++j) W[j] = S.w[k][j];
                      },
                      piece);
}

template <int D>
__device__ int state_has_deadlock(const NetView& N, const Tile<D>& t, const int* locs, const int* ints,
                                  const int (&zone)[D], DlScratch<D>& S) {
  int Z[D], nw = 0;
  const int r = collect_escapes(N, t, locs, ints, zone, S, Z, nw);
  if (r <= 0) return r;
  return subtract_escapes(t, Z, S, nw, [](const int (&)[D]) { return false; }) > 0 ? 1 : 0;
}

// ---------------------------------------------------------------------------------------------
// End-of-run tests of the leads-to sweep (src/liveness/construction.cpp:1097-1177)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ bool has_upper_invariant(const NetView& N, const int* locs) {
  for (int p = 0; p < N.nprocs; ++p) {
    const int gl = N.loc_base[p] + locs[p];
    for (int c = N.loc_inv_off[gl]; c < N.loc_inv_off[gl + 1]; ++c)
      if (N.cons[3 * c] > 0 && N.cons[3 * c + 1] == 0 && N.cons[3 * c + 2] < kInf) return true;
  }
  return false;
}
// time_diverges: every clock unbounded after a delay inside the invariant (and, `restricted`,
// inside !q too).
template <int D>
__device__ bool time_diverges(const NetView& N, const Tile<D>& t, const int* locs, const int* ints,
                              const int (&zone)[D], bool restricted) {
  if (N.nclocks == 0 || has_upper_invariant(N, locs)) return false;
  bool c, u;
  frozen_flags(N, locs, ints, c, u);
  if (c || u) return false;
  int z[D];
#pragma unroll
  for (int j = 0; j < D; ++j) z[j] = zone[j];
  delay(t, z);
  if (!apply_inv(N, t, z, locs) || is_empty(t, z)) return false;
  if (!t.all(t.i == 0 || z[0] >= kInf)) return false;
  if (restricted && N.av_on && pred_disc(N.av_loc, N.av_nloc, N.av_int, N.av_nint, locs, ints)) {
#pragma unroll
    for (int j = 0; j < D; ++j) z[j] = zone[j];
    if (!avoid_cut(N, t, z, locs, ints)) return false;
    delay(t, z);
    if (!apply_inv(N, t, z, locs) || !avoid_cut(N, t, z, locs, ints) || is_empty(t, z)) return false;
    return t.all(t.i == 0 || z[0] >= kInf);
  }
  return true;
}
// orig_time_open: can time run away at these locations in the unrestricted system?
template <int D>
__device__ bool orig_time_open(const NetView& N, const Tile<D>& t, const int* locs, const int* ints) {
  if (N.nclocks == 0 || has_upper_invariant(N, locs)) return false;
  bool c, u;
  frozen_flags(N, locs, ints, c, u);
  if (c || u) return false;
  int z[D];
#pragma unroll
  for (int j = 0; j < D; ++j) z[j] = (j == t.i || t.i == 0) ? kZeroLe : kInf;
  delay(t, z);
  if (!apply_inv(N, t, z, locs)) return false;
  return t.all(t.i == 0 || z[0] >= kInf);
}

// ---------------------------------------------------------------------------------------------
// Per-key a_LU bounds (the state_bounds lambda, src/reachability/engine.cpp:1457-1497): this
// lane's L[i], and U[x] for every x.
// ---------------------------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void key_bounds(const NetView& N, const Tile<D>& t, const int* locs, int& Ly, int (&U)[D]) {
  int l = kAluNegInf, u = kAluNegInf;
  const int c = t.i;
  if (c > 0) {
    for (int p = 0; p < N.nprocs; ++p) {
      const int gl = N.loc_base[p] + locs[p];
      l = max(l, N.Lloc[gl * N.dim + c]);
      u = max(u, N.Uloc[gl * N.dim + c]);
    }
    l = max(l, N.Lq[c]);
    u = max(u, N.Uq[c]);
  } else {
    l = u = 0;
  }
  Ly = l;
#pragma unroll
  for (int x = 0; x < D; ++x) U[x] = t.shfl(u, x);
}

__device__ __forceinline__ unsigned long long hash_mix(unsigned long long k) {
  k ^= k >> 30; k *= 0xbf58476d1ce4e5b9ull;
  k ^= k >> 27; k *= 0x94d049bb133111ebull;
  return k ^ (k >> 31);
}

}  // namespace hgb
