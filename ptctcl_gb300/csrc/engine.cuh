// engine.cuh -- shared host/device declarations of the GB300 zone-graph engine.
#pragma once
#include <cstdint>

namespace hgb {

constexpr int kMaxProcs = 16;     // processes per network handled on the device
constexpr int kMaxInts = 16;      // integer variables per network
constexpr int kMaxRecvEdges = 8;  // enabled receivers of one process in one broadcast
constexpr int kMergeScan = 32;    // convex-union window, kMergeScan (detail/engine_config.hpp:52)
constexpr int kMaxEscapes = 48;   // escape regions one deadlock test may collect
constexpr unsigned long long kEmptyKey = ~0ull;

// Read-only view of one compiled (network, query) instance in device memory. Every array lives
// in the instance's blob; the pointers are device addresses.
struct NetView {
  int nclocks, dim, nprocs, nints, nchans, nedges, nlocs;
  int has_urgent_chan;
  int kind;                    // HORA_Q_*
  int inst_shift;              // hash key = key | (instance << inst_shift)
  const int* chan_flags;
  const int* int_lo;
  const int* int_init;         // [nints]
  const int* proc_init;        // [nprocs]
  const int* loc_base;         // [nprocs]
  const int* loc_flags;        // [nlocs]
  const int* loc_inv_off;      // [nlocs+1]
  const int* eloc_off;         // [nlocs+1] outgoing edges of each location
  const int* eloc;             // edge ids, edge order within a location
  const int* edge_tgt;         // local target
  const int* edge_chan;
  const int* edge_dir;
  const int* edge_guard_off;
  const int* edge_iguard_off;
  const int* edge_reset_off;
  const int* edge_iupd_off;
  const int* cons;             // (i, j, raw) triples
  const int* iatoms;           // (var, op, val) triples
  const int* resets;
  const int* iupds;            // (var, val) pairs
  const int* Lloc;             // [nlocs*dim] per-location a_LU lower bounds
  const int* Uloc;             // [nlocs*dim] per-location a_LU upper bounds
  const unsigned long long* act;  // [nlocs] active-clock masks
  const int* kshift;           // [nprocs+nints]
  const int* kwidth;           // [nprocs+nints]
  const int* L;                // [dim] Extra_LU+ bounds (global, widened by the query)
  const int* U;
  const int* Lq;               // [dim] query floors of the per-state a_LU bounds
  const int* Uq;
  unsigned long long qmask;    // clocks the query reads
  // target conjunction (reach queries)
  int t_never, t_nloc, t_nint, t_nclk;
  const int* t_loc;
  const int* t_int;
  const int* t_clk;
  // leads-to: restriction of the successor pipeline to !q, and p's conjunction
  int av_on;                   // 1: cut successors to !q where q's discrete part holds
  int av_nloc, av_nint, av_nclk;
  const int* av_loc;
  const int* av_int;
  int av_neg[3];               // complement of q's single clock atom
  int av_psi;                  // 1: E[] psi -- keep only psi: its discrete part must hold, its clock
                               // conjunction (av_clk, av_nclk atoms) is adjoined to the invariant
  const int* av_clk;
  int p_nloc, p_nint, p_nclk;
  const int* p_loc;
  const int* p_int;
  const int* p_clk;
};

// Device-side counters, read back with a single copy. The first block is reset before every
// expand (a level runs as one or more chunks of instances), nfront at every level.
struct Ctl {
  unsigned long long nsucc;      // successors produced by expand (may exceed capacity)
  unsigned long long nsurv;      // successors that passed the probe
  unsigned long long ntouched;   // hash slots with pending successors
  unsigned long long seg_alloc;  // grouping segment allocator
  unsigned long long chain_alloc;  // merge's chain-list allocator
  unsigned long long nheavy;     // touched keys merged block-wide ...
  unsigned long long nlight;     // ... and by one tile
  unsigned long long heavy_next; // merge work counters
  unsigned long long light_next;
  unsigned long long bm_need;    // words of the heavy keys' relation blocks
  unsigned int found;            // some instance hit its goal this level
  unsigned int overflow;         // expand output overflowed
  // per level
  unsigned long long nfront;     // next-frontier entries
  // cumulative
  unsigned long long nnodes;     // passed-store nodes allocated
  unsigned long long nkeys;      // distinct keys holding at least one stored zone
  unsigned long long nslots;     // occupied hash slots
  unsigned long long nedges;     // graph edges recorded (leads-to graph mode)
  unsigned long long probes;     // stored zones the probe tested (their column 0 read)
  unsigned long long arena_alloc;  // key-list arena in use
  long long nlive;               // live passed-store zones
  unsigned int err;              // HORA_E_* raised on the device (table full, escape overflow)
  unsigned int flag;             // set by a fixpoint pass that changed something
  // federation sweep of the subsumed leads-to graph
  unsigned long long spieces;    // stop-set pieces allocated
  unsigned long long walloc;     // W-arena zones allocated
  unsigned long long ndirty;     // nodes to relax in the next round
  unsigned long long nchanged;   // nodes whose W shrank this round
  unsigned long long npre;       // exact predecessors computed
  unsigned long long nroots_live; // roots whose W is not yet empty
  unsigned int fed_over;         // a federation outgrew its slots (the sweep restarts with more)
  unsigned int stop_over;        // the stop-set arena overflowed (the pass re-runs with more)
  unsigned long long probe_full; // stored zones the probe read whole (column 0 did not decide)
  unsigned long long merge_live; // live zones of the keys the merge folded into, before each merge
  unsigned long long nlong;      // successors whose key list is long, probed by a whole warp each
};
constexpr unsigned long long kCtlChunkBytes = 10 * 8 + 2 * 4;

}  // namespace hgb
