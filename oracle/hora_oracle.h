/*
 * hora_oracle.h -- CPU oracle for the zone-graph hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference algorithm, used to check the CUDA engine: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and the product library
 * (libhora_gb300.so) never links or calls it.
 *
 * Parity pinning. The reference cannot be compiled here (its zone algebra lives in the HDBM
 * submodule, an external library that is absent), so this restatement follows the in-tree written
 * spec of that algebra -- the Metal shader text in src/metal/netengine_metal.mm and
 * src/metal/engine_metal.mm -- and the C++ semantics in include/hora/detail/semantics.hpp,
 * src/liveness/operators.cpp, src/reachability/{engine,deadlock}.cpp,
 * include/hora/detail/passed_set.hpp and src/model/network.cpp. It is pinned against the
 * reference's own known answers (tests/dbm_tests.cpp) and verdict tables
 * (the tables under tests/uppaal-differential) by the tests in the oracle tests.
 */
#ifndef HORA_ORACLE_H
#define HORA_ORACLE_H

#include <stdint.h>
#include "../include/hora_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- raw bound encoding (src/metal/netengine_metal.mm:76-100) ---- */
#define ORC_INF (1 << 30)
#define ORC_ZERO_LE 1
#define ORC_ALU_NEG_INF (-(1 << 29))

/* ---- DBM primitives on dense row-major int32[dim*dim] ---- */
void    orc_dbm_init(int32_t* d, int32_t dim);               /* origin zone: every clock 0 */
int32_t orc_dbm_empty(const int32_t* d, int32_t dim);
void    orc_dbm_close(int32_t* d, int32_t dim);
int32_t orc_dbm_constrain(int32_t* d, int32_t dim, int32_t a, int32_t b, int32_t raw);
void    orc_dbm_reset(int32_t* d, int32_t dim, int32_t k);
void    orc_dbm_delay(int32_t* d, int32_t dim);
void    orc_dbm_down(int32_t* d, int32_t dim);
void    orc_dbm_free(int32_t* d, int32_t dim, int32_t k);
int32_t orc_dbm_includes(const int32_t* a, const int32_t* b, int32_t dim);    /* a ⊇ b */
int32_t orc_dbm_alu_le(const int32_t* z, const int32_t* zp, int32_t dim, const int32_t* L,
                       const int32_t* U);                                      /* z ≼_aLU zp */
void    orc_dbm_extrap_lu_plus(int32_t* d, int32_t dim, const int32_t* L, const int32_t* U);
int32_t orc_dbm_try_union(int32_t* a, const int32_t* b, int32_t dim);
/* Is z ⊆ w[0] ∪ ... ∪ w[k-1]?  (federation covering; z non-empty) */
int32_t orc_fed_covers(const int32_t* z, const int32_t* w, int32_t k, int32_t dim);

/* ---- static analyses (src/model/network.cpp) ---- */
/* Fills L,U [dim] (global Extra_LU bounds), Lloc,Uloc [total_locs*dim] (per-location a_LU bounds),
 * act [total_locs] (active-clock masks, bit c = clock c). Returns a status. */
int32_t orc_static_bounds(const hora_net_desc* net, int32_t* L, int32_t* U, int32_t* Lloc,
                          int32_t* Uloc, uint64_t* act);

/* ---- successor pipeline, deadlock predicate: same contracts as hora_gb_expand/has_deadlock ---- */
int32_t orc_expand(const hora_net_desc* net, int32_t n, const int32_t* locs, const int32_t* ints,
                   const int32_t* zones, const int32_t* L, const int32_t* U, const uint8_t* qmask,
                   int32_t emode, int64_t cap, int32_t* out_src, int32_t* out_ord,
                   int32_t* out_locs, int32_t* out_ints, int32_t* out_zones, int64_t* out_n);
int32_t orc_has_deadlock(const hora_net_desc* net, int32_t n, const int32_t* locs,
                         const int32_t* ints, const int32_t* zones, int32_t* out);
/* The exact successor of one state by transition `raw` (its index in the enumeration): 1 and the
 * out buffers filled when it is non-empty, else 0. The step check of the forward routes' traces. */
int32_t orc_successor_raw(const hora_net_desc* net, const uint8_t* qmask, const int32_t* locs, const int32_t* ints,
                          const int32_t* zone, int32_t raw, int32_t* out_locs, int32_t* out_ints, int32_t* out_zone);
/* Leads-to phase 2 (the network restricted to !q): the successor by transition index raw (0: none),
 * and the stop set of a state's zone (0 empty, 1 its deadlocked valuations, 2 the whole zone). */
int32_t orc_lt_successor_raw(const hora_net_desc* net, const hora_pred_desc* q, const uint8_t* qmask,
                             const int32_t* locs, const int32_t* ints, const int32_t* zone, int32_t raw,
                             int32_t* out_locs, int32_t* out_ints, int32_t* out_zone);
int32_t orc_lt_stop(const hora_net_desc* net, const hora_pred_desc* q, const uint8_t* qmask,
                    const int32_t* locs, const int32_t* ints, const int32_t* zone);

/* ---- whole queries (level-synchronous BFS in the canonical order the engine uses) ---- */
int32_t orc_reachable_net(const hora_net_desc* net, const hora_pred_desc* target, hora_stats* st,
                          int32_t* result);
int32_t orc_deadlock_reachable(const hora_net_desc* net, hora_stats* st, int32_t* result);
int32_t orc_leads_to(const hora_net_desc* net, const hora_pred_desc* p, const hora_pred_desc* q,
                     hora_stats* st, int32_t* result);
int32_t orc_exists_invariant(const hora_net_desc* net, const hora_pred_desc* psi, hora_stats* st,
                             int32_t* result);
/* Replay of an E[] psi witness: the restricted initial state, and a state's successors in the
 * restricted graph in emission order. */
int32_t orc_eg_initial(const hora_net_desc* net, const hora_pred_desc* psi, int32_t* locs, int32_t* ints,
                       int32_t* zone);
int32_t orc_eg_successors(const hora_net_desc* net, const hora_pred_desc* psi, const int32_t* locs,
                          const int32_t* ints, const int32_t* zone, int32_t cap, int32_t* out_locs,
                          int32_t* out_ints, int32_t* out_zones, int32_t* n);

/* Stop whole-query runs after the first BFS level that ends past `seconds` (0 = no limit); the run
 * then reports status HORA_E_TIMEOUT with the counters reached so far. Used to bound the CPU
 * baseline sample. */
void orc_set_time_limit(double seconds);
/* Host threads of the E<> / deadlock reachability route (1: the sequential loop). Returns the count
 * in effect (1 when the oracle was built without OpenMP). Results do not depend on it. */
int32_t orc_set_threads(int32_t n);

/* Initial symbolic state of the reach route (initial_symbolic_state,
 * src/reachability/engine.cpp:1322-1335): fills locs[nprocs], ints[nints], zone[dim*dim]. Returns 0
 * when the initial invariant is unsatisfiable. */
int32_t orc_initial_state(const hora_net_desc* net, const uint8_t* qmask, int32_t* locs,
                          int32_t* ints, int32_t* zone);

#ifdef __cplusplus
}
#endif
#endif
