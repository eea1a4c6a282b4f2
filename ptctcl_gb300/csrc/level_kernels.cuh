// level_kernels.cuh -- __global__ kernels of one BFS level, templated on the DBM dimension D, and
// their launchers (struct Level<D>), explicitly instantiated once per D in generated units.
#pragma once
#include <cuda_runtime.h>
#include "kernels.cuh"

namespace hgb {

// Device buffers the level kernels share. Plain pointers; sizes are the host's business.
struct Store {
  // hash table of discrete keys
  unsigned long long* hkey;   // [cap] key | instance << inst_shift, kEmptyKey when free
  int* head;                  // [cap] newest node of the key's antichain, -1 when none
  unsigned* pend;             // [cap] survivors pending for this key in the current level
  unsigned* pend_base;        // [cap] their segment offset
  unsigned long long hmask;   // cap - 1
  // passed-store nodes
  int* nzone;                 // [ncap * D*D]
  int* nnext;                 // [ncap]
  int* nlevel;                // [ncap]
  int* ndead;                 // [ncap]
  int* ninst;                 // [ncap]
};
struct Succ {                 // successors of the current level
  unsigned long long* key;    // hash key
  int* parent;                // frontier index of the source
  int* ord;                   // emission ordinal within the source
  int* slot;                  // hash slot after the probe, -1 when dropped
  int* rank;                  // position among the slot's pending survivors (arrival order)
  int* zone;                  // [cap * D*D]
  int* surv;                  // survivor list (indices), filled by the probe
  int* seg;                   // grouped survivors, one segment per touched slot
  int* sorted;                // the same segments in canonical order
  int* touched;               // touched slots
  long long cap;
};
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
};

template <int D>
struct Level {
  static void init(const NetView* nets, int ninst, const int* inst_dim_ok, Store st, Front out, InstState is,
                   Ctl* ctl, cudaStream_t s);
  static void expand(const NetView* nets, InstState is, Front fr, int nfront, Store st, Succ sc, Ctl* ctl,
                     int blocks, cudaStream_t s);
  static void probe(const NetView* nets, InstState is, Succ sc, Store st, Ctl* ctl, long long nsucc,
                    int blocks, cudaStream_t s);
  static void deadlock(const NetView* nets, InstState is, Succ sc, Ctl* ctl, long long nsurv, int blocks,
                       cudaStream_t s);
  static void group(Succ sc, Store st, Ctl* ctl, long long nsucc, long long ntouched, cudaStream_t s);
  static void merge(const NetView* nets, InstState is, Front fr, Succ sc, Store st, Front out, Ctl* ctl,
                    long long ntouched, int level, int blocks, cudaStream_t s);
  // Host-buffer successor pipeline (hora_gb_expand): states given as frontier + node zones.
  static void expand_plain(const NetView* nets, const int* locs, const int* ints, const int* zones, int n,
                           int emode, unsigned long long* okey, int* osrc, int* oord, int* olocs, int* oints,
                           int* ozones, long long cap, Ctl* ctl, cudaStream_t s);
  static void has_deadlock(const NetView* nets, const int* locs, const int* ints, const int* zones, int n,
                           int* out, Ctl* ctl, cudaStream_t s);
};

}  // namespace hgb
