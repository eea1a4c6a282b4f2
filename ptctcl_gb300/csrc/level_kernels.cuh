// level_kernels.cuh -- __global__ kernels of one BFS level, templated on the DBM dimension D, and
// their launchers (struct Level<D>), explicitly instantiated once per D in generated units.
#pragma once
#include <cuda_runtime.h>
#include "kernels.cuh"

namespace hgb {

constexpr int kFedMax = 64;   // zones a federation of the leads-to sweep may hold (the sweep doubles K up to it)

// Device buffers the level kernels share. Plain pointers; sizes are the host's business.
struct Store {
  // hash table of discrete keys
  unsigned long long* hkey;   // [cap] key | instance << inst_shift, kEmptyKey when free
  unsigned* pend;             // [cap] survivors pending for this key in the current level
  unsigned* pend_base;        // [cap] their segment offset
  int* klive;                 // [cap] live zones of the key's antichain ...
  long long* kloff;           // [cap] ... listed oldest first at arena[kloff .. kloff + klive)
  unsigned long long hmask;   // cap - 1
  int* arena;                 // key lists; a merged key's list is rewritten at a fresh offset
  long long acap;
  // passed-store nodes
  int* nzone;                 // [ncap * D*D]
  int* ncol0;                 // [ncap * D] column 0 of each zone (the probe's first test)
  int* nlevel;                // [ncap]
  int* ndead;                 // [ncap]
  int* ninst;                 // [ncap]
  unsigned long long* nkey;   // [ncap] hash key of the node's discrete state
  int* npar;                  // [ncap] node whose successor created this one (-1: initial state)
  int* nraw;                  // [ncap] the creating transition's index (for_each_successor's raw)
};
struct Edges {                // zone-graph edges (leads-to graph mode)
  int* src;
  int* dst;
  int* ord;                   // emission ordinal of the successor the edge came from
  long long cap;
  int* raw;                   // its transition index (for_each_successor's raw), for the predecessor
};
// The federation-valued greatest fixpoint of the subsumed leads-to graph. W[v] (a union of zones
// inside node v's zone) lives in an append-only arena: wcnt[v] zones from warena + woff[v] * D*D,
// or the node's own zone when woff[v] < 0 (the seed is not copied). A round reads the current values
// and writes changed ones to woff2/wcnt2, committed after the round (Jacobi order).
struct Fix {
  const int* eoff;            // [nnodes+1] out-edges of each node (CSR over eidx)
  const int* eidx;            // edge ids grouped by source
  int* swhole;                // [nnodes] 1: every valuation of the zone may end a run
  int* shead;                 // [nnodes] first piece of the node's stop set, -1 when none
  int* snext;                 // [scap] next piece of the same node
  int* spiece;                // [scap * D*D] stop-set pieces
  long long scap;
  long long* woff;
  int* wcnt;
  long long* woff2;
  int* wcnt2;
  int* warena;                // [wcap * D*D]
  long long wcap;
  int* dirty;                 // [nnodes] flag: relax in the next round
  int* dlist;                 // [nnodes] nodes to relax this round
  int* changed;               // [nnodes] flag: W changed this round
  int* clist;                 // [nnodes] nodes whose W changed this round
  int* scratch;               // [ntiles * K * D*D] one federation under construction per tile
  int K;                      // zones a federation may hold
  long long ntiles;
};
struct HeavyKeys {            // per key merged block-wide (index j of Succ::heavy)
  int* n;                     // survivors
  int* a;                     // live zones before the level
  long long* cb;              // clist offset of the key's list
  long long* bm;              // offset of its relation block in pool, -1 when it has none
  int* bounds;                // [2*D] per key: L[] then U[]
  unsigned* pool;             // relation blocks
};
struct Succ {                 // successors of the current level
  unsigned long long* key;    // hash key
  int* parent;                // frontier index of the source
  int* ord;                   // emission ordinal within the source
  int* raw;                   // transition index within the source (for_each_successor's raw)
  int* pnode;                 // passed-store node of the source
  int* flag;                  // inclusion store: 1 when the survivor is stored
  int* slot;                  // hash slot after the probe, -1 when dropped
  int* rank;                  // position among the slot's pending survivors (arrival order)
  int* zone;                  // [cap * D*D]
  int* surv;                  // survivor list (indices), filled by the probe
  int* seg;                   // grouped survivors, one segment per touched slot
  int* sorted;                // the same segments in canonical order
  int* touched;               // touched slots
  int* heavy;                 // touched slots merged block-wide
  int* light;                 // touched slots merged by one tile
  int* longs;                 // successors whose key list is long (the probe's warp-wide pass)
  unsigned long long* okh;    // canonical order key of each successor: parent's hash key ...
  unsigned long long* okl;    // ... then (parent's rank << 32) | emission ordinal
  unsigned long long* skh;    // the same keys gathered at the successor's segment position
  unsigned long long* skl;
  long long cap;
  int* clist;                 // per touched key, its live zones gathered for the merge
  long long ccap;
  HeavyKeys hv;
};
struct ZTab {                 // exact-zone table of the graph store: one word per slot,
  unsigned long long* w;      // (32-bit zone hash << 32) | ref, 0 when free; ref = node id, or
  unsigned long long mask;    // kZRefSucc | successor index while a level is being inserted
};
constexpr unsigned kZRefSucc = 0x80000000u;
struct Front {                // one frontier
  unsigned long long* key;    // hash key
  int* node;                  // passed-store node
  int* rank;                  // rank among the key's new zones, chain order
  int* inst;                  // instance
};
struct InstState {            // per-instance device state (one entry per instance)
  int* emode;                 // 0 exact zones, 1 Extra_LU+
  int* done;                  // instance finished: its work is skipped
  unsigned* found;            // goal hit this level
  unsigned long long* generated;
  long long* nlive;
  unsigned long long* nkeys;
  unsigned long long* nfront;
  unsigned long long* probes;
  // the goal state of a finished forward search, for its trace: the node whose successor reached
  // the goal (-1 none yet; -2 the initial state itself; with hit_raw -1 the node itself is the goal,
  // the leads-to early witness), the transition index, and the goal state's key and zone
  int* hit_node;
  int* hit_raw;
  unsigned long long* hit_key;
  int* hit_zone;              // [ninst * D*D]
};

template <int D>
struct Level {
  // Store 0 is the a_LU subsumption store (reach, deadlock, leads-to phase 1) fed by probe, group and
  // merge; store 1 the exact-zone graph (leads-to phase 2, E[]) fed by the graph_* kernels.
  static void init(const NetView* nets, int ninst, const int* inst_dim_ok, Store st, Front out, InstState is,
                   Ctl* ctl, cudaStream_t s);
  // expands the frontier entries of instances [i0, i1)
  static void expand(const NetView* nets, InstState is, Front fr, int nfront, const int* src_zone, Succ sc, Ctl* ctl,
                     int roots, int i0, int i1, int blocks, cudaStream_t s);
  static void probe_long(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, int blocks, cudaStream_t s);
  static void probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nsucc, int long_list, int blocks,
                    cudaStream_t s);
  static void deadlock(const NetView* nets, InstState is, Succ sc, Ctl* ctl, long long n, int all, int blocks,
                       cudaStream_t s);
  static void group(Succ sc, Store st, Ctl* ctl, long long nsucc, long long ntouched, cudaStream_t s);
  // order: the heavy keys' merge order (largest first), or null for their index order
  static void merge(const NetView* nets, InstState is, Succ sc, Store st, Front out, Ctl* ctl, long long ntouched,
                    int level, int blocks, bool wide, const int* order, cudaStream_t s);
  static int merge_blocks_per_sm(bool wide);
  static bool merge_wide_pays();
  // keys merged block-wide: sort + gather + bounds, then their pairwise relations
  static void heavy_prep(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nheavy,
                         int blocks, const int* order, cudaStream_t s);
  static int heavy_pairs(const NetView* nets, Succ sc, Store st, const long long* prefix, long long nheavy,
                         long long ntiles, int blocks, cudaStream_t s);
  // exact-zone graph store (leads-to graph mode): deduplicate the successors against the store and
  // each other by zone hash, store the new zones, record one edge per successor
  static void graph_probe(const NetView* nets, InstState is, Succ sc, Store st, ZTab zt, Ctl* ctl, long long nsucc,
                          int blocks, cudaStream_t s);
  static void graph_store(const NetView* nets, InstState is, Succ sc, Store st, ZTab zt, Front out, Ctl* ctl,
                          long long nnew, int level, int blocks, cudaStream_t s);
  static void graph_edges(Succ sc, Front fr, Edges ed, Ctl* ctl, long long nsucc, cudaStream_t s);
  static void graph_rehash(Store st, long long nnodes, ZTab zt, Ctl* ctl, int blocks, cudaStream_t s);
  // leads-to: phase-1 nodes whose discrete state satisfies p, as a frontier
  static void collect_p(const NetView* nets, Store st, long long nnodes, Front out, Ctl* ctl, cudaStream_t s);
  // leads-to: end-of-run flags and the greatest-fixpoint sweep over the recorded graph
  static void stop(const NetView* nets, Store st, long long nnodes, int* stop, Ctl* ctl, int blocks, cudaStream_t s);
  static void gfp_pass(Edges ed, long long nedges, long long nnodes, const int* stop, int* W, int* F, Ctl* ctl,
                       cudaStream_t s);
  static void gfp_verdict(const NetView* nets, Store st, long long nnodes, const int* W, InstState is, Ctl* ctl,
                          cudaStream_t s);
  // Subsumed leads-to graph (store 1): a successor is covered by a stored zone of its key that
  // contains it; per level the maximal survivors of each key are stored (incl_*), and every
  // successor records one edge to its covering node.
  static void incl_probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nsucc, int blocks,
                         cudaStream_t s);
  static void incl_group(Succ sc, Store st, Ctl* ctl, long long nsucc, long long ntouched, cudaStream_t s);
  static void incl_keep(Succ sc, Store st, Ctl* ctl, long long nsurv, int blocks, cudaStream_t s);
  static void incl_store(const NetView* nets, InstState is, Succ sc, Store st, Front out, Ctl* ctl, long long nsurv,
                         int level, int blocks, cudaStream_t s);
  static void incl_lists(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long ntouched,
                         cudaStream_t s);
  static void incl_cover(Succ sc, Store st, Ctl* ctl, long long nsurv, int blocks, cudaStream_t s);
  static void incl_edges(Succ sc, Front fr, Edges ed, Ctl* ctl, long long nsucc, cudaStream_t s);
  // Stop sets of nodes [n0, n1) as federations; with `witness`, an instance whose node holds a stop
  // valuation of its p-part cut to !q is found (the early witness on phase-1 nodes, whose zones
  // are read from st; fx.swhole/shead are then not written).
  static void stop_fed(const NetView* nets, InstState is, Store st, long long n0, long long n1, const int* nodes,
                       Fix fx, Ctl* ctl, int witness, int blocks, cudaStream_t s);
  // CSR of the edges by source: eoff (nnodes+1, zeroed by the caller) and eidx; tmp holds nnodes ints.
  static void edge_csr(Edges ed, long long nedges, long long nnodes, int* eoff, int* eidx, int* tmp, cudaStream_t s);
  static void gfp_init(Fix fx, long long nnodes, Ctl* ctl, cudaStream_t s);
  static void gfp_relax(const NetView* nets, Store st, Edges ed, Fix fx, Ctl* ctl, long long ndirty, int blocks,
                        cudaStream_t s);
  static void gfp_round_end(Edges ed, long long nedges, long long nnodes, Fix fx, const int* nlevel, Ctl* ctl,
                            cudaStream_t s);
  static void gfp_compact(Fix fx, long long nnodes, int* narena, unsigned long long* nalloc, cudaStream_t s);
  static void gfp_verdict_fed(const NetView* nets, Store st, long long nnodes, Fix fx, InstState is, cudaStream_t s);
  static long long relax_tiles(int blocks);
  // Host-buffer successor pipeline (hora_gb_expand): states given as frontier + node zones.
  static void expand_plain(const NetView* nets, const int* locs, const int* ints, const int* zones, int n,
                           int emode, unsigned long long* okey, int* osrc, int* oord, int* olocs, int* oints,
                           int* ozones, long long cap, Ctl* ctl, cudaStream_t s);
  static void has_deadlock(const NetView* nets, const int* locs, const int* ints, const int* zones, int n,
                           int* out, Ctl* ctl, cudaStream_t s);
};

}  // namespace hgb
