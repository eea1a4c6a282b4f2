/*
 * hora_gb300.h -- C ABI of the GB300-native zone-graph engine (libhora_gb300.so).
 *
 * This is the drop-in boundary for HORA's zone-graph hot path: the frontier successor pipeline,
 * the passed-store subsumption probe and the backward greatest-fixpoint sweep. Every entry point
 * takes plain pointers and sizes, returns an integer status (never throws across the ABI) and
 * leaves a message for hora_gb_last_error() on failure.
 *
 * Reference interfaces each entry point stands in for (file:line within horaverify/PTCTCL):
 *   hora_gb_reachable_net      bool reachable_net(const Network&, const NetTarget&, Backend,
 *                              ReachStats*)                         include/hora/reachability.hpp:61-62
 *   hora_gb_deadlock_reachable bool deadlock_reachable(const Network&, Backend, ReachStats*,
 *                              const std::atomic<bool>* cancel)     include/hora/liveness.hpp:144-146
 *   hora_gb_leads_to           bool leads_to_clocks / leads_to_otf(const Network&, const DiscPred& p,
 *                              const DiscPred& q, GfpStats*)        include/hora/liveness.hpp:120-124
 *   hora_gb_exists_invariant   bool exists_invariant_run(const Network&, const std::vector<Constraint>&
 *                              psi_clocks, const DiscPred& nq, ReachStats*)  include/hora/liveness.hpp:35-46
 *   hora_gb_expand             NetGpuExpander::expand(...)          include/hora/gpu/network.hpp:52-58
 *   hora_gb_batch_run          no reference counterpart (the reference runs one query at a time);
 *                              same verdict contract as the three entry points above, per instance
 *   hora_gb_server_*           no reference counterpart (continuous-batching request loop)
 *
 * Network encoding. A network of timed automata is passed flattened (hora_net_desc). It carries
 * exactly what include/hora/network.hpp's Network/NProc/NEdge/Location hold for the fast path
 * (clock guards, `var OP const` integer guards, clock resets, `var := const` updates, binary and
 * broadcast channels, urgent/committed locations, location invariants). General-expression guards
 * and updates (NEdge::gen_guard / gen_update) are not representable; networks that need them are
 * out of scope for this engine, as they are for the reference's GPU encoder
 * (include/hora/gpu/encode.hpp:36-44).
 *
 * Clock constraints are triples (i, j, raw) meaning x_i - x_j <| bound with raw = (bound << 1) | weak,
 * clock 0 the constant-zero reference clock, exactly the HDBM encoding the reference uses
 * (src/metal/netengine_metal.mm:76-100).
 */
#ifndef HORA_GB300_H
#define HORA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HORA_GB_ABI_VERSION 2

#if defined(__GNUC__)
#define HORA_GB_API __attribute__((visibility("default")))
#else
#define HORA_GB_API
#endif

/* ---- status codes ------------------------------------------------------------------------- */
enum {
  HORA_OK = 0,
  HORA_E_INVALID = 1,        /* malformed descriptor or argument */
  HORA_E_NOT_SUPPORTED = 2,  /* network outside the engine's scope (diagonal constraints, more than
                                16 clocks, discrete key wider than 63 bits); the caller keeps its
                                own engine, as the reference does when make_net_gpu_cuda returns
                                nullptr (src/reachability/engine.cpp:1557-1561) */
  HORA_E_CUDA = 3,           /* a CUDA runtime call failed; message in hora_gb_last_error() */
  HORA_E_OVERFLOW = 4,       /* a fixed-capacity device structure overflowed (verdict unusable) */
  HORA_E_TIMEOUT = 5,        /* a bounded device-side wait gave up (verdict unusable) */
  HORA_E_BUDGET = 6,         /* request rejected: device-memory budget exceeded */
  HORA_E_NOMEM = 7,          /* device allocation failed */
  HORA_E_CANCELLED = 8,      /* cancelled through the cancel flag between BFS levels */
  HORA_E_NO_DEVICE = 9       /* no CUDA device visible */
};

/* Backend selector, same values and meaning as `enum class Backend { Seq, Omp, Cuda, Metal }`
 * (include/hora/reach.hpp:21). This library implements HORA_BACKEND_CUDA only; passing another
 * value returns HORA_E_NOT_SUPPORTED so that the caller keeps its own CPU engine. */
enum { HORA_BACKEND_SEQ = 0, HORA_BACKEND_OMP = 1, HORA_BACKEND_CUDA = 2, HORA_BACKEND_METAL = 3 };

/* Integer-atom operators, the order of `enum class IntOp { Eq, Ne, Lt, Le, Gt, Ge }`
 * (include/hora/network.hpp:23). */
enum { HORA_IOP_EQ = 0, HORA_IOP_NE = 1, HORA_IOP_LT = 2, HORA_IOP_LE = 3, HORA_IOP_GT = 4, HORA_IOP_GE = 5 };

/* Channel flags and location flags. */
enum { HORA_CHAN_BROADCAST = 1, HORA_CHAN_URGENT = 2 };
enum { HORA_LOC_URGENT = 1, HORA_LOC_COMMITTED = 2 };

/* Flattened network. Locations are numbered process-major: process p's location l has global id
 * loc_base(p) + l, where loc_base(p) = sum of proc_nlocs[0..p). Edges are grouped by process
 * (edge_proc non-decreasing); within a process, edge order is NProc::edges order, which fixes the
 * successor emission order (src/liveness/operators.cpp:55-206). */
typedef struct hora_net_desc {
  int32_t nclocks;              /* clocks, not counting the reference clock; DBM dim = nclocks+1 */
  int32_t nprocs;
  int32_t nints;
  int32_t nchans;
  const int32_t* chan_flags;    /* [nchans] HORA_CHAN_* bits */
  const int32_t* int_lo;        /* [nints] declared range and initial value */
  const int32_t* int_hi;
  const int32_t* int_init;
  const int32_t* proc_nlocs;    /* [nprocs] */
  const int32_t* proc_init;     /* [nprocs] initial location, local index */
  const int32_t* loc_flags;     /* [total locations] HORA_LOC_* bits */
  const int32_t* loc_inv_off;   /* [total locations + 1] invariant constraints, offsets into cons */
  int32_t nedges;
  const int32_t* edge_proc;     /* [nedges] */
  const int32_t* edge_src;      /* [nedges] local source location */
  const int32_t* edge_tgt;      /* [nedges] local target location */
  const int32_t* edge_chan;     /* [nedges] channel id or -1 */
  const int32_t* edge_dir;      /* [nedges] +1 send (a!), -1 receive (a?), 0 none */
  const int32_t* edge_guard_off;  /* [nedges+1] clock guard, offsets into cons */
  const int32_t* edge_iguard_off; /* [nedges+1] integer guard, offsets into iatoms (triples) */
  const int32_t* edge_reset_off;  /* [nedges+1] clock resets, offsets into resets */
  const int32_t* edge_iupd_off;   /* [nedges+1] integer updates, offsets into iupds (pairs) */
  const int32_t* cons;          /* constraint triples (i, j, raw) */
  const int32_t* iatoms;        /* integer atom triples (var, op, val) */
  const int32_t* resets;        /* clock indices in 1..nclocks */
  const int32_t* iupds;         /* update pairs (var, val) */
} hora_net_desc;

/* A conjunction of location, integer and clock atoms: NetTarget (include/hora/network.hpp:152-165)
 * for reachability, and DiscPred's plain conjunction (include/hora/predicate.hpp:39-84) for the
 * two sides of a leads-to. */
typedef struct hora_pred_desc {
  int32_t nloc;
  const int32_t* loc_req;       /* pairs (proc, l): location l, or for l < 0 any location but -l-1 */
  int32_t nint;
  const int32_t* int_cond;      /* triples (var, op, val) */
  int32_t nclk;
  const int32_t* clk_cond;      /* triples (i, j, raw) */
  int32_t never;                /* 1: the literal `false` (NetTarget::never) */
} hora_pred_desc;

/* Query kinds for the batched and serving entry points. */
enum {
  HORA_Q_REACH = 0,     /* E<> target  (A[] not target is its negation) */
  HORA_Q_DEADLOCK = 1,  /* is a deadlocked state reachable?  (A[] not deadlock is its negation) */
  HORA_Q_LEADSTO = 2,   /* p --> q */
  HORA_Q_EG = 3         /* E[] p  (A<> phi is not E[] not phi) */
};

typedef struct hora_query_desc {
  int32_t kind;
  hora_pred_desc p;             /* target for HORA_Q_REACH; p for HORA_Q_LEADSTO; psi for HORA_Q_EG */
  hora_pred_desc q;             /* q for HORA_Q_LEADSTO */
} hora_query_desc;

/* Counters, a superset of ReachStats (include/hora/reach.hpp:10-19) and the GfpStats fields the
 * leads-to route reports (include/hora/liveness.hpp:57-77). */
typedef struct hora_stats {
  uint64_t explored;     /* frontier states expanded, summed over BFS levels (ReachStats::explored) */
  uint64_t generated;    /* non-empty successor zones generated (ReachStats::generated) */
  uint64_t expanded;     /* same as explored for the forward routes */
  uint64_t stored;       /* live zones in the passed store at the end */
  uint64_t keys;         /* distinct discrete states in the passed store */
  uint64_t levels;       /* BFS levels run */
  uint64_t probes;       /* stored zones the subsumption probe tested (their column 0 read) */
  uint64_t pre_calls;    /* exact_predecessor evaluations in the backward sweep */
  uint64_t gfp_iters;    /* sweeps of the backward fixpoint */
  uint64_t kernel_launches;
  double   seconds;      /* wall time of the call */
  double   device_seconds; /* time on the device, CUDA events around the level loop */
  int32_t  extrapolating; /* 1 if the adaptive switch to Extra_LU+ fired */
  int32_t  status;       /* HORA_OK or an error code for this query */
  /* per kernel family, CUDA-event time on the engine's stream and launch count:
   * [0] expand, [1] probe, [2] deadlock test, [3] group, [4] merge, [5] other (init, rehash) */
  double   kernel_seconds[6];
  uint64_t kernel_calls[6];
  uint64_t h2d_bytes;    /* host-to-device bytes moved by the call (descriptor, counters) */
  uint64_t d2h_bytes;    /* device-to-host bytes moved by the call (counters, verdict) */
  /* work of the passed store, for the per-kernel algorithmic bytes (single-query calls):
   * probes (above) counts the stored zones whose column 0 the probe read; of those, probe_full were
   * read whole; merge_surv survivors were folded against merge_live live zones of their keys; nodes
   * zones were written to the store */
  uint64_t probe_full;
  uint64_t merge_surv;
  uint64_t merge_live;
  uint64_t nodes;
} hora_stats;

/* ---- errors and device ---------------------------------------------------------------------- */

/* Thread-local text of the last failure (empty string when none). */
HORA_GB_API const char* hora_gb_last_error(void);
/* ABI version compiled into the library. */
HORA_GB_API int32_t hora_gb_abi_version(void);
/* Number of visible CUDA devices (0 when none); returns a status. */
HORA_GB_API int32_t hora_gb_device_count(int32_t* count);

/* Process-wide tuning per DBM dimension D = clocks + 1 (entry D of each array; ndims entries,
 * at most 18). long_list[D]: the key-list length past which the passed-store probe scans a
 * successor's key with a whole warp instead of one DBM tile; group_max[D]: the most instances of
 * dimension D the batched form runs as one group; blocks_per_sm[D]: the grid of the level kernels,
 * in blocks per SM. A negative or zero entry, or a null array, keeps the built-in default (4, 64,
 * 16); each call replaces the whole table. No reference counterpart: like the reference's
 * process-global options (include/hora/config.hpp:4-6), set it before queries run. Verdicts and
 * counts do not depend on it. ptctcl_gb300/tuner.py measures the values on the device at hand. */
HORA_GB_API int32_t hora_gb_set_tuning(const int32_t* long_list, const int32_t* group_max,
                                       const int32_t* blocks_per_sm, int32_t ndims);

/* ---- single-query entry points ---------------------------------------------------------------- */

/* E<> target. On HORA_OK, *result = 1 iff a symbolic state matching target is reachable. */
HORA_GB_API int32_t hora_gb_reachable_net(const hora_net_desc* net, const hora_pred_desc* target, int32_t backend,
                              hora_stats* stats, int32_t* result);

/* Is a state with a deadlocked valuation reachable?  A[] not deadlock holds iff *result == 0.
 * `cancel` may be null; when non-null it is polled between BFS levels and a non-zero value ends the
 * search with HORA_E_CANCELLED. */
HORA_GB_API int32_t hora_gb_deadlock_reachable(const hora_net_desc* net, int32_t backend, hora_stats* stats,
                                   const volatile int32_t* cancel, int32_t* result);

/* p --> q. On HORA_OK, *result = 1 iff the property holds. */
HORA_GB_API int32_t hora_gb_leads_to(const hora_net_desc* net, const hora_pred_desc* p, const hora_pred_desc* q,
                         int32_t backend, hora_stats* stats, int32_t* result);

/* E[] psi, psi a conjunction of location (also "not at location"), integer and clock atoms. On
 * HORA_OK, *result = 1 iff the initial state admits a maximal run all of whose states satisfy psi.
 * A<> phi for a single atom phi is !E[] (not phi). */
HORA_GB_API int32_t hora_gb_exists_invariant(const hora_net_desc* net, const hora_pred_desc* psi, int32_t backend,
                                 hora_stats* stats, int32_t* result);

/* E[] psi with a witness when it holds. No reference counterpart (the reference emits no traces).
 * The witness is a path of symbolic states of the psi-restricted zone graph from the initial state:
 * step 0 is the initial state (ords[0] = -1), step i is the successor of step i-1 with emission
 * ordinal ords[i] (the order of hora_gb_expand with Extra_M+ under the query's bounds), and the run
 * either ends in a state where it may stop (*loop_to = -1: time diverges inside psi, or a deadlock)
 * or closes a cycle: the successor of the last step with ordinal *loop_ord is step *loop_to.
 * Buffers hold cap steps: ords[cap], locs[cap*nprocs], ints[cap*nints], zones[cap*dim*dim];
 * *nsteps is set (also on HORA_E_OVERFLOW, when the witness needs more). *nsteps = 0 when psi fails. */
HORA_GB_API int32_t hora_gb_exists_invariant_trace(const hora_net_desc* net, const hora_pred_desc* psi,
                                       int32_t backend, hora_stats* stats, int32_t* result, int32_t cap,
                                       int32_t* nsteps, int32_t* ords, int32_t* locs, int32_t* ints,
                                       int32_t* zones, int32_t* loop_to, int32_t* loop_ord);

/* Successor pipeline on host buffers, for differential testing against a CPU implementation.
 * Inputs: n source states (locs[n*nprocs], ints[n*nints], zones[n*dim*dim] canonical, non-empty),
 * the per-clock bounds L, U [dim] used by Extra_LU+, the query clock mask qmask [dim] (1 = the
 * active-clock reduction must keep that clock) and emode (0 none, 1 Extra_LU+).
 * Outputs, at most `cap` successors in (source, emission order): out_src[k] source index,
 * out_ord[k] emission ordinal within its source, out_locs, out_ints, out_zones. *out_n receives the
 * successor count; when it exceeds cap only the first cap are written and HORA_E_OVERFLOW is
 * returned. */
HORA_GB_API int32_t hora_gb_expand(const hora_net_desc* net, int32_t n, const int32_t* locs, const int32_t* ints,
                       const int32_t* zones, const int32_t* L, const int32_t* U, const uint8_t* qmask,
                       int32_t emode, int64_t cap, int32_t* out_src, int32_t* out_ord,
                       int32_t* out_locs, int32_t* out_ints, int32_t* out_zones, int64_t* out_n);

/* Deadlock predicate on host buffers (state_has_deadlock, src/reachability/deadlock.cpp:74-270):
 * out[k] = 1 iff state k contains a deadlocked valuation. */
HORA_GB_API int32_t hora_gb_has_deadlock(const hora_net_desc* net, int32_t n, const int32_t* locs,
                             const int32_t* ints, const int32_t* zones, int32_t* out);

/* Deadlock predicate for callers that cannot allocate device memory. No counterpart in the
 * reference: it exists for callers whose device memory is owned by another allocator (a framework
 * pool that reserved the device) or who cannot take cudaMalloc/cudaFree's implicit synchronisation.
 * The caller passes DEVICE buffers: d_locs[n*nprocs], d_ints[n*nints] (may be null when nints is
 * 0), d_zones[n*dim*dim] and d_out[n]; the call allocates nothing. The compiled network lives in
 * one static device array of 1 MiB (held by every GPU that loads the library until exit); a
 * network whose tables do not fit is rejected with HORA_E_INVALID. The array's device address is
 * fetched on the first call on each device, which should therefore come before any stream capture.
 * The array is shared by all calls and keeps the last call's contents (its counters are cleared on
 * every call): calls that overlap on the GPU race. Runs on the legacy default stream and returns
 * after the kernel has finished. The legacy default stream is not ordered against streams created
 * with cudaStreamNonBlocking (PyTorch's side streams are): a caller that fills d_locs, d_ints or
 * d_zones on such a stream must synchronise it (cudaStreamSynchronize) before the call. */
HORA_GB_API int32_t hora_gb_has_deadlock_noalloc(const hora_net_desc* net, int32_t n, const int32_t* d_locs,
                                                 const int32_t* d_ints, const int32_t* d_zones, int32_t* d_out);

/* ---- handle form ------------------------------------------------------------------------------- */

/* One (network, query) pair opened once and run on demand; no reference counterpart beyond the
 * single-query entry points above, which it routes to by the query's kind.
 * hora_gb_open validates and copies both descriptors (the caller's arrays may be freed afterwards):
 * out-of-scope input returns HORA_E_NOT_SUPPORTED or HORA_E_INVALID there, before any device is
 * touched. hora_gb_run runs the query on the CUDA backend; *verdict follows the single-query
 * convention of hora_gb_batch_run (reach: reachable; deadlock: deadlock reachable; leads-to and
 * E[]: holds). hora_gb_trace copies the trace of the last run, into the buffers of
 * hora_gb_exists_invariant_trace:
 *   E[] psi: the witness, with that function's conventions (*nsteps = 0 when psi fails);
 *   reach, deadlock, and a leads-to violation found by the early witness: a counterexample -- the path
 *     of the passed store from the initial state (step 0) to the goal: a state matching the target,
 *     a state holding a deadlocked valuation, or a reachable p-state whose part outside q holds a
 *     valuation where a maximal run that avoids q may stop. ords[i] (i > 0) is the index of the
 *     transition taken from step i-1 among those hora_gb_expand's enumeration visits (the candidate
 *     transitions whose integer guards and committed rules hold, in emission order, whether or not
 *     their zone is empty); zones[i] is the stored zone, which contains the exact successor of
 *     zones[i-1] by that transition (it may be extrapolated, or a convex union); *loop_to = -1.
 *     *nsteps = 0 when the goal was not reached;
 *   a leads-to violation found by the backward sweep: the same path of the passed store to the
 *     p-state a surviving root was cut from, then the root (ords = -2: that state restricted to p and
 *     !q, no transition), then a path of the !q graph through nodes whose fixpoint value is not empty,
 *     each step's zone containing the exact successor of the previous one in the network restricted
 *     to !q, ending at a node with a stop set (a whole zone where time may diverge inside !q
 *     preferred, else one holding deadlocked valuations) or closing a cycle back to step *loop_to by
 *     transition *loop_ord.
 * A handle that has not run returns HORA_E_INVALID. A handle is used by one thread at a time. */
typedef struct hora_handle_s* hora_handle;
HORA_GB_API int32_t hora_gb_open(const hora_net_desc* net, const hora_query_desc* q, hora_handle* out);
HORA_GB_API int32_t hora_gb_run(hora_handle h, int32_t* verdict, hora_stats* stats);
HORA_GB_API int32_t hora_gb_trace(hora_handle h, int32_t cap, int32_t* nsteps, int32_t* ords, int32_t* locs,
                                  int32_t* ints, int32_t* zones, int32_t* loop_to, int32_t* loop_ord);
HORA_GB_API int32_t hora_gb_close(hora_handle h);

/* ---- batched form ----------------------------------------------------------------------------- */

/* Run n independent (network, query) instances together on the device. verdicts[k] receives the
 * result in the single-query convention of the query's kind (reach: reachable; deadlock: deadlock
 * reachable; leads-to: holds); stats (may be null) one record per instance, whose seconds field is
 * the time from the start of the call to that instance's verdict. Returns HORA_OK when every
 * instance ran; per-instance failures are reported in stats[k].status and verdicts[k] = -1.
 * cancel (may be null) is polled between BFS levels: once it reads non-zero the call returns
 * HORA_E_CANCELLED, instances that already had their verdict keep it (status HORA_OK) and the
 * others report HORA_E_CANCELLED. Instances share three quarters of the free device memory; one
 * whose passed store outgrows its share stops with status HORA_E_BUDGET and no verdict. */
HORA_GB_API int32_t hora_gb_batch_run(int32_t n, const hora_net_desc* nets, const hora_query_desc* queries,
                          int32_t* verdicts, hora_stats* stats, const volatile int32_t* cancel);

/* ---- serving form ------------------------------------------------------------------------------ */

typedef struct hora_server hora_server;

/* budget_bytes: device memory the passed/waiting stores of the admitted requests may hold together
 * (a pool); max_inflight: requests on the device at once, each on its own worker thread and stream.
 * A request is admitted, in arrival order, when a slot is free and the pool can hold its initial store
 * reservation; while it runs its stores stay resident across BFS levels and grow by taking more from
 * the pool; a request whose store needs more than the pool has left stops with status HORA_E_BUDGET. */
HORA_GB_API int32_t hora_gb_server_create(uint64_t budget_bytes, int32_t max_inflight, hora_server** out);
/* Bounds a request's stores and the queue; call before the first submit (defaults: 0, 0 = no limit).
 * per_request_bytes: a request whose store outgrows this stops with status HORA_E_BUDGET, so every
 * admitted request ends in bounded time whatever its state space; max_queued: a submission that finds
 * this many requests waiting for admission is rejected with HORA_E_BUDGET (reject rather than queue). */
HORA_GB_API int32_t hora_gb_server_set_limits(hora_server* s, uint64_t per_request_bytes, int32_t max_queued);
/* Queue a request; the descriptors are copied. *ticket identifies it. A request whose initial
 * reservation exceeds the whole pool, or that finds the queue full (hora_gb_server_set_limits), is
 * rejected with HORA_E_BUDGET. */
HORA_GB_API int32_t hora_gb_server_submit(hora_server* s, const hora_net_desc* net, const hora_query_desc* q,
                              int64_t* ticket);
/* The worker threads admit and run requests on their own; this waits up to 1 ms for progress and sets
 * *active to the number of requests still queued or running. */
HORA_GB_API int32_t hora_gb_server_step(hora_server* s, int32_t* active);
/* Fetch a request's result: *done = 0 while it is queued or running; once it has finished, *done = 1
 * with verdict and stats filled (stats.seconds = submission to result), and the result is released:
 * a later poll of the same ticket returns HORA_E_INVALID. */
HORA_GB_API int32_t hora_gb_server_poll(hora_server* s, int64_t ticket, int32_t* done, int32_t* verdict,
                            hora_stats* stats);
/* Cancels the running requests at their next BFS level, waits for the workers and frees the server;
 * results not yet polled are dropped. */
HORA_GB_API int32_t hora_gb_server_destroy(hora_server* s);

#ifdef __cplusplus
}
#endif

#endif /* HORA_GB300_H */
