/*
 * hora_oracle.c -- CPU oracle for the zone-graph hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * See hora_oracle.h for what this is restating and how it is pinned. Each function cites the
 * reference file:line it follows. Everything is single-threaded, integer-exact C11.
 */
#include "hora_oracle.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ============================================================================================
 * Raw bounds: (value << 1) | weak, kInf = 1<<30 (src/metal/netengine_metal.mm:76-100)
 * ============================================================================================ */
static inline int32_t r_le(int32_t v) { return (int32_t)((uint32_t)v << 1) | 1; }
static inline int32_t r_lt(int32_t v) { return (int32_t)((uint32_t)v << 1); }
static inline int32_t r_bound(int32_t r) { return r >> 1; }
static inline int r_strict(int32_t r) { return (r & 1) == 0; }
static inline int32_t r_add(int32_t a, int32_t b) {
  if (a >= ORC_INF || b >= ORC_INF) return ORC_INF;
  int32_t v = r_bound(a) + r_bound(b);
  return (!r_strict(a) && !r_strict(b)) ? r_le(v) : r_lt(v);
}
static inline int32_t r_negate(int32_t r) {  /* complement of x_i-x_j <| v, as x_j-x_i <| -v */
  int32_t v = r_bound(r);
  return r_strict(r) ? r_le(-v) : r_lt(-v);
}
static inline int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

/* ============================================================================================
 * DBM primitives (netengine_metal.mm:101-124, 225-238; engine_metal.mm:80-93)
 * ============================================================================================ */
void orc_dbm_init(int32_t* d, int32_t dim) {
  for (int i = 0; i < dim * dim; ++i) d[i] = ORC_ZERO_LE;
}
int32_t orc_dbm_empty(const int32_t* d, int32_t dim) {
  for (int i = 0; i < dim; ++i) if (d[i * dim + i] < ORC_ZERO_LE) return 1;
  return 0;
}
void orc_dbm_close(int32_t* d, int32_t dim) {
  for (int k = 0; k < dim; ++k)
    for (int i = 0; i < dim; ++i) {
      int32_t ik = d[i * dim + k];
      if (ik >= ORC_INF) continue;
      for (int j = 0; j < dim; ++j) {
        int32_t s = r_add(ik, d[k * dim + j]);
        if (s < d[i * dim + j]) d[i * dim + j] = s;
      }
    }
}
/* Incremental closure after tightening x_a - x_b to `raw` (netengine_metal.mm:110-124). */
int32_t orc_dbm_constrain(int32_t* d, int32_t dim, int32_t a, int32_t b, int32_t raw) {
  if (raw >= d[a * dim + b]) return !orc_dbm_empty(d, dim);
  d[a * dim + b] = raw;
  for (int i = 0; i < dim; ++i) {
    int32_t via = r_add(d[i * dim + a], raw);
    if (via < d[i * dim + b]) d[i * dim + b] = via;
  }
  for (int i = 0; i < dim; ++i) {
    int32_t ib = d[i * dim + b];
    if (ib >= ORC_INF) continue;
    for (int k = 0; k < dim; ++k) {
      int32_t via = r_add(ib, d[b * dim + k]);
      if (via < d[i * dim + k]) d[i * dim + k] = via;
    }
  }
  return !orc_dbm_empty(d, dim);
}
void orc_dbm_reset(int32_t* d, int32_t dim, int32_t k) {
  for (int j = 0; j < dim; ++j) { d[k * dim + j] = d[0 * dim + j]; d[j * dim + k] = d[j * dim + 0]; }
  d[k * dim + k] = ORC_ZERO_LE;
}
void orc_dbm_delay(int32_t* d, int32_t dim) {
  for (int i = 1; i < dim; ++i) d[i * dim + 0] = ORC_INF;
}
/* Time predecessor (HDBM dbm_down, used by exact_predecessor src/liveness/operators.cpp:278-303
 * and state_has_deadlock src/reachability/deadlock.cpp:244): every lower bound relaxes to the
 * tightest bound any clock difference still imposes, and never below zero. */
void orc_dbm_down(int32_t* d, int32_t dim) {
  for (int j = 1; j < dim; ++j) {
    int32_t m = ORC_ZERO_LE;
    for (int i = 1; i < dim; ++i) if (d[i * dim + j] < m) m = d[i * dim + j];
    d[0 * dim + j] = m;
  }
}
/* Existentially quantify clock k (HDBM dbm_free): k becomes any value >= 0. */
void orc_dbm_free(int32_t* d, int32_t dim, int32_t k) {
  for (int i = 0; i < dim; ++i) {
    if (i == k) continue;
    d[k * dim + i] = ORC_INF;
    d[i * dim + k] = d[i * dim + 0];
  }
  d[k * dim + 0] = ORC_INF;
  d[0 * dim + k] = ORC_ZERO_LE;
  d[k * dim + k] = ORC_ZERO_LE;
}
int32_t orc_dbm_includes(const int32_t* a, const int32_t* b, int32_t dim) {
  for (int i = 0; i < dim * dim; ++i) if (b[i] > a[i]) return 0;
  return 1;
}
/* z ≼_aLU zp (netengine_metal.mm:240-252; passed_set.hpp:41-48). */
int32_t orc_dbm_alu_le(const int32_t* z, const int32_t* zp, int32_t dim, const int32_t* L,
                       const int32_t* U) {
  for (int x = 0; x < dim; ++x) {
    if (U[x] == ORC_ALU_NEG_INF) continue;
    if (z[0 * dim + x] < r_le(-U[x])) continue;
    for (int y = 0; y < dim; ++y) {
      if (x == y) continue;
      if (L[y] == ORC_ALU_NEG_INF) continue;
      if (zp[y * dim + x] < z[y * dim + x] && r_add(zp[y * dim + x], r_lt(-L[y])) < z[0 * dim + x])
        return 0;
    }
  }
  return 1;
}
/* Extra_LU+ then close (engine_metal.mm:80-93). */
void orc_dbm_extrap_lu_plus(int32_t* d, int32_t dim, const int32_t* L, const int32_t* U) {
  int32_t row0[64];
  for (int k = 0; k < dim; ++k) row0[k] = d[k];
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) {
      if (i == j) continue;
      int32_t e = d[i * dim + j];
      if (e >= ORC_INF) continue;
      if (r_bound(e) > L[i]) { d[i * dim + j] = ORC_INF; continue; }
      if (-r_bound(row0[i]) > L[i]) { d[i * dim + j] = ORC_INF; continue; }
      if (i != 0 && -r_bound(row0[j]) > U[j]) { d[i * dim + j] = ORC_INF; continue; }
      if (e < r_lt(-U[j])) d[i * dim + j] = r_lt(-U[j]);
    }
  orc_dbm_close(d, dim);
}
/* Exact convex union (netengine_metal.mm:310-335): a ∪ b is convex iff every region the hull
 * gains by relaxing one of a's constraints lies in b, and vice versa. Every tightening constraint
 * is tested, which decides the same set identity the minimal-graph filter decides (a redundant
 * constraint's complement is covered by the complements of the generating ones). */
int32_t orc_dbm_try_union(int32_t* a, const int32_t* b, int32_t dim) {
  int32_t H[64 * 64], R[64 * 64];
  const int d2 = dim * dim;
  for (int k = 0; k < d2; ++k) H[k] = a[k] > b[k] ? a[k] : b[k];
  for (int pass = 0; pass < 2; ++pass) {
    const int32_t* z = pass == 0 ? a : b;
    const int32_t* other = pass == 0 ? b : a;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) {
        if (i == j || z[i * dim + j] >= H[i * dim + j]) continue;
        memcpy(R, H, sizeof(int32_t) * d2);
        if (!orc_dbm_constrain(R, dim, j, i, r_negate(z[i * dim + j]))) continue;
        if (!orc_dbm_includes(other, R, dim)) return 0;
      }
  }
  memcpy(a, H, sizeof(int32_t) * d2);
  return 1;
}

/* Is z covered by the union of the k zones w? Depth-first subtraction: z \ w0 splits into disjoint
 * pieces z ∧ c_1 ∧ .. ∧ c_{m-1} ∧ ¬c_m over w0's tightening constraints c_m, and each piece must be
 * covered by w1..w{k-1} (fed_subtract semantics, src/reachability/deadlock.cpp:262-267). */
static int fed_covers_rec(const int32_t* z, const int32_t* w, int k, int dim) {
  const int d2 = dim * dim;
  int i = 0;
  int32_t t[64 * 64];
  for (; i < k; ++i) {
    /* skip w[i] that misses z entirely */
    memcpy(t, z, sizeof(int32_t) * d2);
    int ok = 1;
    for (int a = 0; a < dim && ok; ++a)
      for (int b = 0; b < dim && ok; ++b)
        if (a != b && w[i * d2 + a * dim + b] < t[a * dim + b])
          ok = orc_dbm_constrain(t, dim, a, b, w[i * d2 + a * dim + b]);
    if (ok) break;
  }
  if (i == k) return 0;
  const int32_t* wi = w + (size_t)i * d2;
  if (orc_dbm_includes(wi, z, dim)) return 1;
  int32_t* r = (int32_t*)malloc(sizeof(int32_t) * d2 * 2);
  int32_t* p = r + d2;
  memcpy(r, z, sizeof(int32_t) * d2);
  int res = 1;
  for (int a = 0; a < dim && res; ++a)
    for (int b = 0; b < dim && res; ++b) {
      if (a == b || wi[a * dim + b] >= r[a * dim + b]) continue;
      memcpy(p, r, sizeof(int32_t) * d2);
      if (orc_dbm_constrain(p, dim, b, a, r_negate(wi[a * dim + b])))
        if (!fed_covers_rec(p, w + (size_t)(i + 1) * d2, k - i - 1, dim)) res = 0;
      if (!res) break;
      if (!orc_dbm_constrain(r, dim, a, b, wi[a * dim + b])) { a = dim; break; }
    }
  free(r);
  return res;
}
int32_t orc_fed_covers(const int32_t* z, const int32_t* w, int32_t k, int32_t dim) {
  if (orc_dbm_empty(z, dim)) return 1;
  return fed_covers_rec(z, w, k, dim);
}

/* ============================================================================================
 * Compiled model: indices and the static analyses of src/model/network.cpp
 * ============================================================================================ */
typedef struct {
  const hora_net_desc* n;
  int dim, nlocs_total;
  int* loc_base;        /* [nprocs] */
  int* eloc_off;        /* [nlocs_total+1] edges of each (global) location, in edge order */
  int* eloc;            /* edge ids */
  int32_t *L, *U;       /* global Extra_LU bounds [dim] */
  int32_t *Lloc, *Uloc; /* per-location a_LU bounds [nlocs_total*dim] */
  uint64_t* act;        /* active masks [nlocs_total] */
  int* kshift;          /* [nprocs+nints] discrete-key field offsets */
  int* kwidth;          /* [nprocs+nints] discrete-key field widths */
  int keybits;
  int has_urgent_chan;
  int has_diag;
  /* optional restriction to !q (leads-to): at states matching q's discrete part the successor
     must stay outside q's clock region, which is a single atom (convex complement) */
  const hora_pred_desc* avoid;   /* q (leads-to) or psi (E[] psi), or NULL */
  int32_t avoid_neg[3];          /* complement of q's clock atom */
  int avoid_psi;                 /* 1: the run must stay in the conjunction psi (E[] psi) */
} Model;

static int ceil_log2(long n) { int b = 0; while ((1L << b) < n) ++b; return b; }

static void model_free(Model* m) {
  free(m->loc_base); free(m->eloc_off); free(m->eloc); free(m->L); free(m->U);
  free(m->Lloc); free(m->Uloc); free(m->act); free(m->kshift); free(m->kwidth);
}

/* compute_bounds (network.cpp:59-85), compute_loc_bounds (:105-182), compute_active (:184-232). */
static int model_build(const hora_net_desc* n, Model* m) {
  memset(m, 0, sizeof *m);
  m->n = n;
  if (n->nclocks < 0 || n->nclocks > 62 || n->nprocs <= 0) return HORA_E_INVALID;
  const int dim = n->nclocks + 1;
  m->dim = dim;
  m->loc_base = (int*)calloc(n->nprocs, sizeof(int));
  int tot = 0;
  for (int p = 0; p < n->nprocs; ++p) { m->loc_base[p] = tot; tot += n->proc_nlocs[p]; }
  m->nlocs_total = tot;
  m->eloc_off = (int*)calloc(tot + 1, sizeof(int));
  m->eloc = (int*)calloc(n->nedges > 0 ? n->nedges : 1, sizeof(int));
  for (int e = 0; e < n->nedges; ++e) m->eloc_off[m->loc_base[n->edge_proc[e]] + n->edge_src[e] + 1]++;
  for (int l = 0; l < tot; ++l) m->eloc_off[l + 1] += m->eloc_off[l];
  int* fill = (int*)calloc(tot, sizeof(int));
  for (int e = 0; e < n->nedges; ++e) {
    int gl = m->loc_base[n->edge_proc[e]] + n->edge_src[e];
    m->eloc[m->eloc_off[gl] + fill[gl]++] = e;
  }
  free(fill);
  /* diagonal / urgent-channel flags */
  for (int l = 0; l < tot; ++l)
    for (int c = n->loc_inv_off[l]; c < n->loc_inv_off[l + 1]; ++c)
      if (n->cons[3 * c] > 0 && n->cons[3 * c + 1] > 0) m->has_diag = 1;
  for (int e = 0; e < n->nedges; ++e)
    for (int c = n->edge_guard_off[e]; c < n->edge_guard_off[e + 1]; ++c)
      if (n->cons[3 * c] > 0 && n->cons[3 * c + 1] > 0) m->has_diag = 1;
  for (int ch = 0; ch < n->nchans; ++ch) if (n->chan_flags[ch] & HORA_CHAN_URGENT) m->has_urgent_chan = 1;
  /* global bounds */
  m->L = (int32_t*)calloc(dim, sizeof(int32_t));
  m->U = (int32_t*)calloc(dim, sizeof(int32_t));
#define SCAN_GLOBAL(c0, c1)                                                         \
  for (int c = (c0); c < (c1); ++c) {                                               \
    int i = n->cons[3 * c], j = n->cons[3 * c + 1], v = r_bound(n->cons[3 * c + 2]); \
    if (i > 0 && j == 0) { if (v > m->U[i]) m->U[i] = v; }                          \
    else if (i == 0 && j > 0) { if (-v > m->L[j]) m->L[j] = -v; }                   \
    else if (i > 0 && j > 0) {                                                      \
      int a = v < 0 ? -v : v;                                                       \
      m->U[i] = imax(m->U[i], a); m->U[j] = imax(m->U[j], a);                       \
      m->L[i] = imax(m->L[i], a); m->L[j] = imax(m->L[j], a);                       \
    }                                                                               \
  }
  for (int l = 0; l < tot; ++l) SCAN_GLOBAL(n->loc_inv_off[l], n->loc_inv_off[l + 1]);
  for (int e = 0; e < n->nedges; ++e) SCAN_GLOBAL(n->edge_guard_off[e], n->edge_guard_off[e + 1]);
#undef SCAN_GLOBAL
  m->L[0] = m->U[0] = 0;
  /* per-location a_LU bounds: backward least fixpoint within each process */
  m->Lloc = (int32_t*)malloc(sizeof(int32_t) * tot * dim);
  m->Uloc = (int32_t*)malloc(sizeof(int32_t) * tot * dim);
  for (int k = 0; k < tot * dim; ++k) m->Lloc[k] = m->Uloc[k] = ORC_ALU_NEG_INF;
  int32_t* Lc = (int32_t*)malloc(sizeof(int32_t) * dim);
  int32_t* Uc = (int32_t*)malloc(sizeof(int32_t) * dim);
  char* rst = (char*)malloc(dim);
#define SCAN_LOC(c0, c1)                                                            \
  for (int c = (c0); c < (c1); ++c) {                                               \
    int i = n->cons[3 * c], j = n->cons[3 * c + 1], v = r_bound(n->cons[3 * c + 2]); \
    if (i > 0 && j == 0) Uc[i] = imax(Uc[i], v);                                    \
    else if (i == 0 && j > 0) Lc[j] = imax(Lc[j], -v);                              \
    else if (i > 0 && j > 0) {                                                      \
      int a = v < 0 ? -v : v;                                                       \
      Uc[i] = imax(Uc[i], a); Uc[j] = imax(Uc[j], a);                               \
      Lc[i] = imax(Lc[i], a); Lc[j] = imax(Lc[j], a);                               \
    }                                                                               \
  }
  for (int p = 0; p < n->nprocs; ++p) {
    const int nl = n->proc_nlocs[p], base = m->loc_base[p];
    int changed = 1;
    while (changed) {
      changed = 0;
      for (int l = 0; l < nl; ++l) {
        for (int c = 0; c < dim; ++c) Lc[c] = Uc[c] = ORC_ALU_NEG_INF;
        SCAN_LOC(n->loc_inv_off[base + l], n->loc_inv_off[base + l + 1]);
        for (int k = m->eloc_off[base + l]; k < m->eloc_off[base + l + 1]; ++k) {
          const int e = m->eloc[k];
          SCAN_LOC(n->edge_guard_off[e], n->edge_guard_off[e + 1]);
          memset(rst, 0, dim);
          for (int r = n->edge_reset_off[e]; r < n->edge_reset_off[e + 1]; ++r) rst[n->resets[r]] = 1;
          const int tg = base + n->edge_tgt[e];
          for (int c = 1; c < dim; ++c)
            if (!rst[c]) {
              Lc[c] = imax(Lc[c], m->Lloc[tg * dim + c]);
              Uc[c] = imax(Uc[c], m->Uloc[tg * dim + c]);
            }
        }
        for (int c = 1; c < dim; ++c) {
          if (Lc[c] > m->Lloc[(base + l) * dim + c]) { m->Lloc[(base + l) * dim + c] = Lc[c]; changed = 1; }
          if (Uc[c] > m->Uloc[(base + l) * dim + c]) { m->Uloc[(base + l) * dim + c] = Uc[c]; changed = 1; }
        }
      }
    }
  }
#undef SCAN_LOC
  /* active clocks */
  m->act = (uint64_t*)calloc(tot, sizeof(uint64_t));
  for (int p = 0; p < n->nprocs; ++p) {
    const int nl = n->proc_nlocs[p], base = m->loc_base[p];
    int changed = 1;
    while (changed) {
      changed = 0;
      for (int l = 0; l < nl; ++l) {
        uint64_t A = 0;
        for (int c = n->loc_inv_off[base + l]; c < n->loc_inv_off[base + l + 1]; ++c) {
          if (n->cons[3 * c] > 0) A |= 1ull << n->cons[3 * c];
          if (n->cons[3 * c + 1] > 0) A |= 1ull << n->cons[3 * c + 1];
        }
        for (int k = m->eloc_off[base + l]; k < m->eloc_off[base + l + 1]; ++k) {
          const int e = m->eloc[k];
          for (int c = n->edge_guard_off[e]; c < n->edge_guard_off[e + 1]; ++c) {
            if (n->cons[3 * c] > 0) A |= 1ull << n->cons[3 * c];
            if (n->cons[3 * c + 1] > 0) A |= 1ull << n->cons[3 * c + 1];
          }
          uint64_t r = 0;
          for (int q = n->edge_reset_off[e]; q < n->edge_reset_off[e + 1]; ++q) r |= 1ull << n->resets[q];
          A |= m->act[base + n->edge_tgt[e]] & ~r;
        }
        A &= ~1ull;
        if (A & ~m->act[base + l]) { m->act[base + l] |= A; changed = 1; }
      }
    }
  }
  free(Lc); free(Uc); free(rst);
  /* discrete key layout (DiscKeyCodecT, src/reachability/engine.cpp:967-1026) */
  m->kshift = (int*)calloc(n->nprocs + n->nints + 1, sizeof(int));
  m->kwidth = (int*)calloc(n->nprocs + n->nints + 1, sizeof(int));
  int off = 0;
  for (int p = 0; p < n->nprocs; ++p) {
    m->kshift[p] = off; m->kwidth[p] = ceil_log2(n->proc_nlocs[p]); off += m->kwidth[p];
  }
  for (int v = 0; v < n->nints; ++v) {
    m->kshift[n->nprocs + v] = off;
    m->kwidth[n->nprocs + v] = ceil_log2((long)n->int_hi[v] - n->int_lo[v] + 1);
    off += m->kwidth[n->nprocs + v];
  }
  m->keybits = off;
  return HORA_OK;
}

int32_t orc_static_bounds(const hora_net_desc* net, int32_t* L, int32_t* U, int32_t* Lloc,
                          int32_t* Uloc, uint64_t* act) {
  Model m;
  int rc = model_build(net, &m);
  if (rc) { model_free(&m); return rc; }
  memcpy(L, m.L, sizeof(int32_t) * m.dim);
  memcpy(U, m.U, sizeof(int32_t) * m.dim);
  memcpy(Lloc, m.Lloc, sizeof(int32_t) * m.dim * m.nlocs_total);
  memcpy(Uloc, m.Uloc, sizeof(int32_t) * m.dim * m.nlocs_total);
  memcpy(act, m.act, sizeof(uint64_t) * m.nlocs_total);
  model_free(&m);
  return HORA_OK;
}

static uint64_t key_encode(const Model* m, const int32_t* locs, const int32_t* ints) {
  uint64_t k = 0;
  for (int p = 0; p < m->n->nprocs; ++p) k |= (uint64_t)(uint32_t)locs[p] << m->kshift[p];
  for (int v = 0; v < m->n->nints; ++v)
    k |= (uint64_t)(uint32_t)(ints[v] - m->n->int_lo[v]) << m->kshift[m->n->nprocs + v];
  return k;
}
static void key_decode(const Model* m, uint64_t k, int32_t* locs, int32_t* ints) {
  const hora_net_desc* n = m->n;
  for (int p = 0; p < n->nprocs; ++p)
    locs[p] = (int32_t)((k >> m->kshift[p]) & ((1ull << m->kwidth[p]) - 1));
  for (int v = 0; v < n->nints; ++v) {
    const int f = n->nprocs + v;
    ints[v] = (int32_t)((k >> m->kshift[f]) & ((1ull << m->kwidth[f]) - 1)) + n->int_lo[v];
  }
}

/* ============================================================================================
 * Transition semantics (include/hora/detail/semantics.hpp)
 * ============================================================================================ */
static int int_ok(const hora_net_desc* n, int e, const int32_t* ints) {  /* semantics.hpp:53-68 */
  for (int a = n->edge_iguard_off[e]; a < n->edge_iguard_off[e + 1]; ++a) {
    const int32_t x = ints[n->iatoms[3 * a]], op = n->iatoms[3 * a + 1], v = n->iatoms[3 * a + 2];
    int r = 0;
    switch (op) {
      case HORA_IOP_EQ: r = x == v; break;
      case HORA_IOP_NE: r = x != v; break;
      case HORA_IOP_LT: r = x < v; break;
      case HORA_IOP_LE: r = x <= v; break;
      case HORA_IOP_GT: r = x > v; break;
      case HORA_IOP_GE: r = x >= v; break;
    }
    if (!r) return 0;
  }
  return 1;
}
static int ints_ok(const int32_t* atoms, int na, const int32_t* ints) {
  for (int a = 0; a < na; ++a) {
    const int32_t x = ints[atoms[3 * a]], op = atoms[3 * a + 1], v = atoms[3 * a + 2];
    int r = 0;
    switch (op) {
      case HORA_IOP_EQ: r = x == v; break;
      case HORA_IOP_NE: r = x != v; break;
      case HORA_IOP_LT: r = x < v; break;
      case HORA_IOP_LE: r = x <= v; break;
      case HORA_IOP_GT: r = x > v; break;
      case HORA_IOP_GE: r = x >= v; break;
    }
    if (!r) return 0;
  }
  return 1;
}
static int apply_cons(int32_t* z, int dim, const int32_t* cons, int c0, int c1) {  /* apply_all */
  for (int c = c0; c < c1; ++c)
    if (!orc_dbm_constrain(z, dim, cons[3 * c], cons[3 * c + 1], cons[3 * c + 2])) return 0;
  return 1;
}
static int apply_inv(const Model* m, int32_t* z, const int32_t* locs) {  /* all_invariants+apply_all */
  const hora_net_desc* n = m->n;
  for (int p = 0; p < n->nprocs; ++p) {
    const int gl = m->loc_base[p] + locs[p];
    if (!apply_cons(z, m->dim, n->cons, n->loc_inv_off[gl], n->loc_inv_off[gl + 1])) return 0;
  }
  return 1;
}
static inline int loc_committed(const Model* m, int p, int l) {
  return (m->n->loc_flags[m->loc_base[p] + l] & HORA_LOC_COMMITTED) != 0;
}
/* urgent_sync_enabled (semantics.hpp:118-139) */
static int urgent_sync_enabled(const Model* m, const int32_t* locs, const int32_t* ints) {
  const hora_net_desc* n = m->n;
  if (!m->has_urgent_chan) return 0;
  for (int i = 0; i < n->nprocs; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1]; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1) continue;
      if (!(n->chan_flags[n->edge_chan[se]] & HORA_CHAN_URGENT)) continue;
      if (!int_ok(n, se, ints)) continue;
      if (n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST) return 1;
      for (int j = 0; j < n->nprocs; ++j) {
        if (j == i) continue;
        const int gj = m->loc_base[j] + locs[j];
        for (int q = m->eloc_off[gj]; q < m->eloc_off[gj + 1]; ++q) {
          const int re = m->eloc[q];
          if (n->edge_chan[re] != n->edge_chan[se] || n->edge_dir[re] != -1) continue;
          if (int_ok(n, re, ints)) return 1;
        }
      }
    }
  }
  return 0;
}
/* frozen_flags (semantics.hpp:160-169) */
static void frozen_flags(const Model* m, const int32_t* locs, const int32_t* ints, int* committed,
                         int* urgent) {
  *committed = *urgent = 0;
  for (int p = 0; p < m->n->nprocs; ++p) {
    int f = m->n->loc_flags[m->loc_base[p] + locs[p]];
    if (f & HORA_LOC_COMMITTED) *committed = 1;
    if (f & HORA_LOC_URGENT) *urgent = 1;
  }
  if (!*urgent && urgent_sync_enabled(m, locs, ints)) *urgent = 1;
}
/* reset_inactive (semantics.hpp:186-215) */
static void reset_inactive(const Model* m, const int32_t* locs, int32_t* z, const uint8_t* qmask) {
  uint64_t a = 0;
  for (int p = 0; p < m->n->nprocs; ++p) a |= m->act[m->loc_base[p] + locs[p]];
  for (int c = 1; c < m->dim; ++c) if (qmask && qmask[c]) a |= 1ull << c;
  uint64_t dead = ~a & (((1ull << m->n->nclocks) - 1) << 1);
  while (dead) {
    int c = __builtin_ctzll(dead);
    dead &= dead - 1;
    orc_dbm_reset(z, m->dim, c);
  }
}
/* close_succ_zone without the avoid-set (semantics.hpp:522-568). Returns 0 when the target
 * invariant is unsatisfiable; the caller tests emptiness. */
static int ints_ok(const int32_t* atoms, int na, const int32_t* ints);
static int disc_match(const hora_pred_desc* t, const int32_t* locs, const int32_t* ints);
/* Restrict z to the complement of q where q's discrete part holds (leads-to), or to psi (E[] psi:
 * psi's discrete part must hold and its clock conjunction is adjoined, exists_invariant_run.cpp:
 * 70-91); 0 when nothing is left. */
static int avoid_cut(const Model* m, int32_t* z, const int32_t* tl, const int32_t* ti) {
  if (m->avoid && m->avoid_psi) {
    if (!disc_match(m->avoid, tl, ti)) return 0;
    return apply_cons(z, m->dim, m->avoid->clk_cond, 0, m->avoid->nclk);
  }
  if (!m->avoid || !disc_match(m->avoid, tl, ti)) return 1;
  if (m->avoid->nclk == 0) return 0;   /* a purely discrete q: the whole state is in q */
  return orc_dbm_constrain(z, m->dim, m->avoid_neg[0], m->avoid_neg[1], m->avoid_neg[2]);
}
static int close_succ_zone(const Model* m, const int32_t* tl, const int32_t* ti, int32_t* z,
                           const uint8_t* qmask, const int32_t* L, const int32_t* U, int emode) {
  if (!apply_inv(m, z, tl)) return 0;
  if (!avoid_cut(m, z, tl, ti)) return 0;
  int c, u;
  frozen_flags(m, tl, ti, &c, &u);
  if (!c && !u) { orc_dbm_delay(z, m->dim); apply_inv(m, z, tl); avoid_cut(m, z, tl, ti); }
  reset_inactive(m, tl, z, qmask);
  if (emode == 1) orc_dbm_extrap_lu_plus(z, m->dim, L, U);
  return 1;
}

/* Broadcast receiver options (build_broadcast_parts, semantics.hpp:275-303). */
#define MAXOPT 128
#define MAXPART 64
typedef struct {
  int proc;
  int nopt;
  int edge[MAXOPT];        /* edge id, or -1 for an abstain option */
  int xoff[MAXOPT];        /* abstain option: offset into xcons (triples) */
  int xn[MAXOPT];          /* abstain option: constraint count */
} Part;
typedef struct {
  int nparts;
  Part parts[MAXPART];
  int32_t* xcons;
  int nx, capx;
} Parts;
static void xpush(Parts* P, int i, int j, int32_t raw) {
  if (P->nx + 1 > P->capx) {
    P->capx = P->capx ? P->capx * 2 : 256;
    P->xcons = (int32_t*)realloc(P->xcons, sizeof(int32_t) * 3 * P->capx);
  }
  P->xcons[3 * P->nx] = i; P->xcons[3 * P->nx + 1] = j; P->xcons[3 * P->nx + 2] = raw;
  P->nx++;
}
/* One broadcast-enumeration scratch block per thread, reused across calls. */
static Parts* parts_scratch(void) {
  static _Thread_local Parts* P = NULL;   /* one per thread: the multi-core port expands in parallel */
  if (!P) P = (Parts*)calloc(1, sizeof(Parts));
  return P;
}
static int build_broadcast_parts(const Model* m, const int32_t* locs, const int32_t* ints, int se,
                                 int sender, Parts* P) {
  const hora_net_desc* n = m->n;
  P->nparts = 0; P->nx = 0;
  for (int j = 0; j < n->nprocs; ++j) {
    if (j == sender) continue;
    Part* pt = &P->parts[P->nparts];
    pt->proc = j; pt->nopt = 0;
    int guards[MAXOPT], ng = 0;
    const int gj = m->loc_base[j] + locs[j];
    for (int q = m->eloc_off[gj]; q < m->eloc_off[gj + 1]; ++q) {
      const int re = m->eloc[q];
      if (n->edge_chan[re] == n->edge_chan[se] && n->edge_dir[re] == -1 && int_ok(n, re, ints)) {
        pt->edge[pt->nopt] = re; pt->xoff[pt->nopt] = 0; pt->xn[pt->nopt] = 0; pt->nopt++;
        guards[ng++] = re;
      }
    }
    if (pt->nopt == 0) continue;
    /* DNF of the complement of the disjunction of the enabled receivers' clock guards */
    int ndnf = 1, empty_guard = 0;
    for (int g = 0; g < ng; ++g) {
      int len = n->edge_guard_off[guards[g] + 1] - n->edge_guard_off[guards[g]];
      if (len == 0) { empty_guard = 1; break; }
      ndnf *= len;
    }
    if (!empty_guard) {
      if (pt->nopt + ndnf > MAXOPT) return 0;
      for (int t = 0; t < ndnf; ++t) {
        /* disjunct t picks atom index (t / prod of earlier lengths) % len of each guard, in the
           order the reference's cross product appends them (earlier guards vary slowest) */
        int o = pt->nopt++;
        pt->edge[o] = -1; pt->xoff[o] = P->nx; pt->xn[o] = ng;
        int rem = t;
        int idx[MAXOPT];
        for (int g = ng - 1; g >= 0; --g) {
          int len = n->edge_guard_off[guards[g] + 1] - n->edge_guard_off[guards[g]];
          idx[g] = rem % len; rem /= len;
        }
        for (int g = 0; g < ng; ++g) {
          int c = n->edge_guard_off[guards[g]] + idx[g];
          /* negate(c): x_i - x_j <| v  ->  x_j - x_i <|' -v */
          xpush(P, n->cons[3 * c + 1], n->cons[3 * c], r_negate(n->cons[3 * c + 2]));
        }
      }
    }
    if (++P->nparts > MAXPART) return 0;
  }
  return 1;
}

/* Successor generation (successors_net, src/reachability/engine.cpp:243-368; the same emission
 * order as tagged_successors, src/liveness/operators.cpp:55-206). Calls emit() per non-empty
 * successor in order. `raw` numbers the transition among every candidate the enumeration visits
 * (the combinations that pass the integer guards and the committed filter, whether or not their
 * zone turns out empty), so find_trans() can rebuild its recipe -- the tag of tagged_successors --
 * from the source's discrete state alone. */
typedef void (*emit_fn)(void* ctx, const int32_t* locs, const int32_t* ints, const int32_t* zone, int raw);
static int successors(const Model* m, const int32_t* locs, const int32_t* ints, const int32_t* zone,
                      const int32_t* L, const int32_t* U, const uint8_t* qmask, int emode,
                      emit_fn emit, void* ctx) {
  const hora_net_desc* n = m->n;
  const int dim = m->dim, d2 = dim * dim, np = n->nprocs, ni = n->nints;
  int32_t z1[64 * 64];
  int32_t tl[64], ti[64];
  int src_c, src_u, raw = 0;
  frozen_flags(m, locs, ints, &src_c, &src_u);
  /* local edges */
  for (int p = 0; p < np; ++p) {
    if (src_c && !loc_committed(m, p, locs[p])) continue;
    const int gp = m->loc_base[p] + locs[p];
    for (int k = m->eloc_off[gp]; k < m->eloc_off[gp + 1]; ++k) {
      const int e = m->eloc[k];
      if (n->edge_chan[e] >= 0) continue;
      if (!int_ok(n, e, ints)) continue;
      const int rw = raw++;
      memcpy(z1, zone, sizeof(int32_t) * d2);
      if (!apply_cons(z1, dim, n->cons, n->edge_guard_off[e], n->edge_guard_off[e + 1])) continue;
      for (int r = n->edge_reset_off[e]; r < n->edge_reset_off[e + 1]; ++r) orc_dbm_reset(z1, dim, n->resets[r]);
      memcpy(tl, locs, sizeof(int32_t) * np); tl[p] = n->edge_tgt[e];
      memcpy(ti, ints, sizeof(int32_t) * ni);
      for (int u = n->edge_iupd_off[e]; u < n->edge_iupd_off[e + 1]; ++u) ti[n->iupds[2 * u]] = n->iupds[2 * u + 1];
      if (!close_succ_zone(m, tl, ti, z1, qmask, L, U, emode)) continue;
      if (orc_dbm_empty(z1, dim)) continue;
      emit(ctx, tl, ti, z1, rw);
    }
  }
  /* binary synchronisation */
  for (int i = 0; i < np; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1]; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1) continue;
      if (n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST) continue;
      if (!int_ok(n, se, ints)) continue;
      const int i_comm = loc_committed(m, i, locs[i]);
      for (int j = 0; j < np; ++j) {
        if (j == i) continue;
        const int gj = m->loc_base[j] + locs[j];
        for (int q = m->eloc_off[gj]; q < m->eloc_off[gj + 1]; ++q) {
          const int re = m->eloc[q];
          if (n->edge_chan[re] != n->edge_chan[se] || n->edge_dir[re] != -1) continue;
          if (src_c && !(i_comm || loc_committed(m, j, locs[j]))) continue;
          if (!int_ok(n, re, ints)) continue;
          const int rw = raw++;
          memcpy(z1, zone, sizeof(int32_t) * d2);
          if (!apply_cons(z1, dim, n->cons, n->edge_guard_off[se], n->edge_guard_off[se + 1])) continue;
          if (!apply_cons(z1, dim, n->cons, n->edge_guard_off[re], n->edge_guard_off[re + 1])) continue;
          for (int r = n->edge_reset_off[se]; r < n->edge_reset_off[se + 1]; ++r) orc_dbm_reset(z1, dim, n->resets[r]);
          for (int r = n->edge_reset_off[re]; r < n->edge_reset_off[re + 1]; ++r) orc_dbm_reset(z1, dim, n->resets[r]);
          memcpy(tl, locs, sizeof(int32_t) * np); tl[i] = n->edge_tgt[se]; tl[j] = n->edge_tgt[re];
          memcpy(ti, ints, sizeof(int32_t) * ni);
          for (int u = n->edge_iupd_off[se]; u < n->edge_iupd_off[se + 1]; ++u) ti[n->iupds[2 * u]] = n->iupds[2 * u + 1];
          for (int u = n->edge_iupd_off[re]; u < n->edge_iupd_off[re + 1]; ++u) ti[n->iupds[2 * u]] = n->iupds[2 * u + 1];
          if (!close_succ_zone(m, tl, ti, z1, qmask, L, U, emode)) continue;
          if (orc_dbm_empty(z1, dim)) continue;
          emit(ctx, tl, ti, z1, rw);
        }
      }
    }
  }
  /* broadcast synchronisation */
  Parts* P = parts_scratch();
  int ok_all = 1;
  for (int i = 0; i < np && ok_all; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1]; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1 || !(n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST)) continue;
      if (!int_ok(n, se, ints)) continue;
      if (!build_broadcast_parts(m, locs, ints, se, i, P)) { ok_all = 0; break; }
      int pick[MAXPART];
      memset(pick, 0, sizeof pick);
      for (;;) {
        int part_comm = loc_committed(m, i, locs[i]);
        for (int t = 0; t < P->nparts; ++t) {
          const Part* pt = &P->parts[t];
          if (pt->edge[pick[t]] >= 0 && loc_committed(m, pt->proc, locs[pt->proc])) part_comm = 1;
        }
        if (!src_c || part_comm) {
          const int rw = raw++;
          memcpy(z1, zone, sizeof(int32_t) * d2);
          int ok = apply_cons(z1, dim, n->cons, n->edge_guard_off[se], n->edge_guard_off[se + 1]);
          for (int t = 0; ok && t < P->nparts; ++t) {
            const Part* pt = &P->parts[t];
            const int o = pick[t];
            if (pt->edge[o] >= 0)
              ok = apply_cons(z1, dim, n->cons, n->edge_guard_off[pt->edge[o]], n->edge_guard_off[pt->edge[o] + 1]);
            else
              ok = apply_cons(z1, dim, P->xcons, pt->xoff[o], pt->xoff[o] + pt->xn[o]);
          }
          if (ok) {
            memcpy(tl, locs, sizeof(int32_t) * np);
            memcpy(ti, ints, sizeof(int32_t) * ni);
            tl[i] = n->edge_tgt[se];
            for (int u = n->edge_iupd_off[se]; u < n->edge_iupd_off[se + 1]; ++u) ti[n->iupds[2 * u]] = n->iupds[2 * u + 1];
            for (int r = n->edge_reset_off[se]; r < n->edge_reset_off[se + 1]; ++r) orc_dbm_reset(z1, dim, n->resets[r]);
            for (int t = 0; t < P->nparts; ++t) {
              const Part* pt = &P->parts[t];
              const int re = pt->edge[pick[t]];
              if (re < 0) continue;
              tl[pt->proc] = n->edge_tgt[re];
              for (int u = n->edge_iupd_off[re]; u < n->edge_iupd_off[re + 1]; ++u) ti[n->iupds[2 * u]] = n->iupds[2 * u + 1];
              for (int r = n->edge_reset_off[re]; r < n->edge_reset_off[re + 1]; ++r) orc_dbm_reset(z1, dim, n->resets[r]);
            }
            if (close_succ_zone(m, tl, ti, z1, qmask, L, U, emode) && !orc_dbm_empty(z1, dim))
              emit(ctx, tl, ti, z1, rw);
          }
        }
        if (P->nparts == 0) break;
        int t = 0;
        for (; t < P->nparts; ++t) { if (++pick[t] < P->parts[t].nopt) break; pick[t] = 0; }
        if (t == P->nparts) break;
      }
    }
  }
  return ok_all;
}

/* ============================================================================================
 * Deadlock predicate (state_has_deadlock, src/reachability/deadlock.cpp:74-270)
 * ============================================================================================ */
typedef struct {
  int32_t* w;
  int nw, cap, dim;
  const int32_t* Z;
  int covered;
} Escapes;
static void esc_add(Escapes* E, const Model* m, int32_t* g, const int32_t* tl, const uint64_t rmask) {
  /* pull the target invariant back through the resets (deadlock.cpp:118-127) */
  const hora_net_desc* n = m->n;
  const int dim = m->dim, d2 = dim * dim;
  for (int p = 0; p < n->nprocs; ++p) {
    const int gl = m->loc_base[p] + tl[p];
    for (int c = n->loc_inv_off[gl]; c < n->loc_inv_off[gl + 1]; ++c) {
      int i = n->cons[3 * c], j = n->cons[3 * c + 1];
      const int32_t b = n->cons[3 * c + 2];
      if ((rmask >> i) & 1) i = 0;
      if ((rmask >> j) & 1) j = 0;
      if (i == j) { if (b < ORC_ZERO_LE) return; continue; }
      if (!orc_dbm_constrain(g, dim, i, j, b)) return;
    }
  }
  if (orc_dbm_empty(g, dim)) return;
  if (memcmp(g, E->Z, sizeof(int32_t) * d2) == 0) { E->covered = 1; return; }
  if (E->nw == E->cap) {
    E->cap = E->cap ? E->cap * 2 : 16;
    E->w = (int32_t*)realloc(E->w, sizeof(int32_t) * d2 * E->cap);
  }
  memcpy(E->w + (size_t)E->nw * d2, g, sizeof(int32_t) * d2);
  E->nw++;
}
static uint64_t reset_mask(const hora_net_desc* n, int e) {
  uint64_t r = 0;
  for (int q = n->edge_reset_off[e]; q < n->edge_reset_off[e + 1]; ++q) r |= 1ull << n->resets[q];
  return r;
}
/* The escape regions of a state: every transition's guard region of the delay-closed zone `Z`
 * (filled here), pulled back through the target invariant, then let down unless the state is
 * frozen. Returns 0 when the state has no concrete valuation (empty zone, or invariant
 * unsatisfiable); Eout->covered is set when one escape is all of Z. */
static int deadlock_escapes(const Model* m, const int32_t* locs, const int32_t* ints, const int32_t* zone,
                            Escapes* Eout, int32_t* Z, int* frozen_out) {
  const hora_net_desc* n = m->n;
  const int dim = m->dim, d2 = dim * dim, np = n->nprocs;
  if (orc_dbm_empty(zone, dim)) return 0;
  int src_c, src_u;
  frozen_flags(m, locs, ints, &src_c, &src_u);
  const int frozen = src_c || src_u;
  *frozen_out = frozen;
  int32_t g[64 * 64];
  int32_t tl[64];
  memcpy(Z, zone, sizeof(int32_t) * d2);
  if (!frozen) orc_dbm_delay(Z, dim);
  if (!apply_inv(m, Z, locs)) return 0;
  Escapes E = {0};
  E.dim = dim; E.Z = Z;
  for (int p = 0; p < np && !E.covered; ++p) {
    if (src_c && !loc_committed(m, p, locs[p])) continue;
    const int gp = m->loc_base[p] + locs[p];
    for (int k = m->eloc_off[gp]; k < m->eloc_off[gp + 1] && !E.covered; ++k) {
      const int e = m->eloc[k];
      if (n->edge_chan[e] >= 0) continue;
      if (!int_ok(n, e, ints)) continue;
      memcpy(g, Z, sizeof(int32_t) * d2);
      if (!apply_cons(g, dim, n->cons, n->edge_guard_off[e], n->edge_guard_off[e + 1])) continue;
      memcpy(tl, locs, sizeof(int32_t) * np); tl[p] = n->edge_tgt[e];
      esc_add(&E, m, g, tl, reset_mask(n, e));
    }
  }
  for (int i = 0; i < np && !E.covered; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1] && !E.covered; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1) continue;
      if (n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST) continue;
      if (!int_ok(n, se, ints)) continue;
      const int i_comm = loc_committed(m, i, locs[i]);
      for (int j = 0; j < np && !E.covered; ++j) {
        if (j == i) continue;
        const int gj = m->loc_base[j] + locs[j];
        for (int q = m->eloc_off[gj]; q < m->eloc_off[gj + 1] && !E.covered; ++q) {
          const int re = m->eloc[q];
          if (n->edge_chan[re] != n->edge_chan[se] || n->edge_dir[re] != -1) continue;
          if (src_c && !(i_comm || loc_committed(m, j, locs[j]))) continue;
          if (!int_ok(n, re, ints)) continue;
          memcpy(g, Z, sizeof(int32_t) * d2);
          if (!apply_cons(g, dim, n->cons, n->edge_guard_off[se], n->edge_guard_off[se + 1])) continue;
          if (!apply_cons(g, dim, n->cons, n->edge_guard_off[re], n->edge_guard_off[re + 1])) continue;
          memcpy(tl, locs, sizeof(int32_t) * np); tl[i] = n->edge_tgt[se]; tl[j] = n->edge_tgt[re];
          esc_add(&E, m, g, tl, reset_mask(n, se) | reset_mask(n, re));
        }
      }
    }
  }
  Parts* P = parts_scratch();
  for (int i = 0; i < np && !E.covered; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1] && !E.covered; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1 || !(n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST)) continue;
      if (!int_ok(n, se, ints)) continue;
      build_broadcast_parts(m, locs, ints, se, i, P);
      int pick[MAXPART];
      memset(pick, 0, sizeof pick);
      for (;;) {
        int part_comm = loc_committed(m, i, locs[i]);
        for (int t = 0; t < P->nparts; ++t) {
          const Part* pt = &P->parts[t];
          if (pt->edge[pick[t]] >= 0 && loc_committed(m, pt->proc, locs[pt->proc])) part_comm = 1;
        }
        if (!src_c || part_comm) {
          memcpy(g, Z, sizeof(int32_t) * d2);
          int ok = apply_cons(g, dim, n->cons, n->edge_guard_off[se], n->edge_guard_off[se + 1]);
          uint64_t rm = reset_mask(n, se);
          memcpy(tl, locs, sizeof(int32_t) * np); tl[i] = n->edge_tgt[se];
          for (int t = 0; ok && t < P->nparts; ++t) {
            const Part* pt = &P->parts[t];
            const int o = pick[t];
            if (pt->edge[o] < 0) { ok = apply_cons(g, dim, P->xcons, pt->xoff[o], pt->xoff[o] + pt->xn[o]); continue; }
            const int re = pt->edge[o];
            ok = apply_cons(g, dim, n->cons, n->edge_guard_off[re], n->edge_guard_off[re + 1]);
            rm |= reset_mask(n, re);
            tl[pt->proc] = n->edge_tgt[re];
          }
          if (ok) esc_add(&E, m, g, tl, rm);
          if (E.covered) break;
        }
        if (P->nparts == 0) break;
        int t = 0;
        for (; t < P->nparts; ++t) { if (++pick[t] < P->parts[t].nopt) break; pick[t] = 0; }
        if (t == P->nparts) break;
      }
    }
  }
  if (!E.covered && !frozen) for (int w = 0; w < E.nw; ++w) orc_dbm_down(E.w + (size_t)w * d2, dim);
  *Eout = E;
  return 1;
}
static int state_has_deadlock(const Model* m, const int32_t* locs, const int32_t* ints, const int32_t* zone) {
  const int dim = m->dim, d2 = dim * dim;
  int32_t Z[64 * 64];
  Escapes E = {0};
  int frozen = 0;
  if (!deadlock_escapes(m, locs, ints, zone, &E, Z, &frozen)) { free(E.w); return 0; }
  int dead;
  if (E.covered) dead = 0;
  else {
    dead = -1;
    for (int w = 0; w < E.nw; ++w)
      if (orc_dbm_includes(E.w + (size_t)w * d2, Z, dim)) { dead = 0; break; }
    if (dead < 0) dead = !orc_fed_covers(Z, E.w, E.nw, dim);
  }
  free(E.w);
  return dead;
}

/* ============================================================================================
 * Host-buffer entry points
 * ============================================================================================ */
typedef struct {
  int64_t cap, n;
  int src, ord;
  int np, ni, d2;
  int32_t *out_src, *out_ord, *out_locs, *out_ints, *out_zones;
} ExpCtx;
static void exp_emit(void* c, const int32_t* locs, const int32_t* ints, const int32_t* zone, int raw) {
  (void)raw;
  ExpCtx* x = (ExpCtx*)c;
  if (x->n < x->cap) {
    const int64_t k = x->n;
    x->out_src[k] = x->src; x->out_ord[k] = x->ord;
    memcpy(x->out_locs + k * x->np, locs, sizeof(int32_t) * x->np);
    if (x->ni) memcpy(x->out_ints + k * x->ni, ints, sizeof(int32_t) * x->ni);
    memcpy(x->out_zones + k * x->d2, zone, sizeof(int32_t) * x->d2);
  }
  x->n++;
  x->ord++;
}
int32_t orc_expand(const hora_net_desc* net, int32_t n, const int32_t* locs, const int32_t* ints,
                   const int32_t* zones, const int32_t* L, const int32_t* U, const uint8_t* qmask,
                   int32_t emode, int64_t cap, int32_t* out_src, int32_t* out_ord,
                   int32_t* out_locs, int32_t* out_ints, int32_t* out_zones, int64_t* out_n) {
  Model m;
  int rc = model_build(net, &m);
  if (rc) { model_free(&m); return rc; }
  ExpCtx x = {cap, 0, 0, 0, net->nprocs, net->nints, m.dim * m.dim,
              out_src, out_ord, out_locs, out_ints, out_zones};
  for (int s = 0; s < n; ++s) {
    x.src = s; x.ord = 0;
    successors(&m, locs + (size_t)s * net->nprocs, ints + (size_t)s * net->nints,
               zones + (size_t)s * x.d2, L, U, qmask, emode, exp_emit, &x);
  }
  *out_n = x.n;
  model_free(&m);
  return x.n > cap ? HORA_E_OVERFLOW : HORA_OK;
}
/* The successor of (locs, ints, zone) by transition `raw` (the index successors() gives it), exact
 * (no extrapolation), with the active-clock reduction under qmask. Returns 1 and fills the out
 * buffers when that transition yields a non-empty zone, 0 otherwise. Replays the traces of the
 * forward routes step by step. */
typedef struct { int want, hit; int np, ni, d2; int32_t *locs, *ints, *zone; } RawCtx;
static void raw_emit(void* c, const int32_t* locs, const int32_t* ints, const int32_t* zone, int raw) {
  RawCtx* x = (RawCtx*)c;
  if (raw != x->want || x->hit) return;
  x->hit = 1;
  memcpy(x->locs, locs, sizeof(int32_t) * x->np);
  if (x->ni) memcpy(x->ints, ints, sizeof(int32_t) * x->ni);
  memcpy(x->zone, zone, sizeof(int32_t) * x->d2);
}
int32_t orc_successor_raw(const hora_net_desc* net, const uint8_t* qmask, const int32_t* locs, const int32_t* ints,
                          const int32_t* zone, int32_t raw, int32_t* out_locs, int32_t* out_ints, int32_t* out_zone) {
  Model m;
  if (model_build(net, &m)) { model_free(&m); return 0; }
  uint8_t qm[64] = {0};
  if (qmask) memcpy(qm, qmask, (size_t)m.dim);
  RawCtx x = {raw, 0, net->nprocs, net->nints, m.dim * m.dim, out_locs, out_ints, out_zone};
  successors(&m, locs, ints, zone, m.L, m.U, qm, 0, raw_emit, &x);
  model_free(&m);
  return x.hit;
}

int32_t orc_has_deadlock(const hora_net_desc* net, int32_t n, const int32_t* locs,
                         const int32_t* ints, const int32_t* zones, int32_t* out) {
  Model m;
  int rc = model_build(net, &m);
  if (rc) { model_free(&m); return rc; }
  const int d2 = m.dim * m.dim;
  for (int s = 0; s < n; ++s)
    out[s] = state_has_deadlock(&m, locs + (size_t)s * net->nprocs, ints + (size_t)s * net->nints,
                                zones + (size_t)s * d2);
  model_free(&m);
  return HORA_OK;
}

/* ============================================================================================
 * Passed store (NetPassedT::add, include/hora/detail/passed_set.hpp:287-444)
 * ============================================================================================ */
typedef struct {
  int32_t* zones;   /* node zone storage */
  int* next; int* level; char* dead;
  int nn, capn;
  uint64_t* skey; int* shead; int* stouch;  /* open-addressing slots */
  uint64_t smask; int nkeys;
  int d2;
  long nlive;
} Store;
static uint64_t mix64(uint64_t k) { return k * 0x9e3779b97f4a7c15ULL; }
static void store_init(Store* S, int d2) {
  memset(S, 0, sizeof *S);
  S->d2 = d2;
  S->smask = 1023;
  S->skey = (uint64_t*)calloc(1024, sizeof(uint64_t));
  S->shead = (int*)malloc(sizeof(int) * 1024);
  S->stouch = (int*)calloc(1024, sizeof(int));
  for (int i = 0; i < 1024; ++i) S->shead[i] = -2;   /* -2 free, -1 key present with no live node */
}
static void store_free(Store* S) {
  free(S->zones); free(S->next); free(S->level); free(S->dead);
  free(S->skey); free(S->shead); free(S->stouch);
}
static uint64_t slot_of(const Store* S, uint64_t k) {
  uint64_t i = (mix64(k) >> 20) & S->smask;
  while (S->shead[i] != -2 && S->skey[i] != k) i = (i + 1) & S->smask;
  return i;
}
static void store_grow(Store* S) {
  uint64_t ncap = (S->smask + 1) * 2, nmask = ncap - 1;
  uint64_t* nk = (uint64_t*)calloc(ncap, sizeof(uint64_t));
  int* nh = (int*)malloc(sizeof(int) * ncap);
  int* nt = (int*)calloc(ncap, sizeof(int));
  for (uint64_t i = 0; i < ncap; ++i) nh[i] = -2;
  for (uint64_t i = 0; i <= S->smask; ++i)
    if (S->shead[i] != -2) {
      uint64_t j = (mix64(S->skey[i]) >> 20) & nmask;
      while (nh[j] != -2) j = (j + 1) & nmask;
      nk[j] = S->skey[i]; nh[j] = S->shead[i]; nt[j] = S->stouch[i];
    }
  free(S->skey); free(S->shead); free(S->stouch);
  S->skey = nk; S->shead = nh; S->stouch = nt; S->smask = nmask;
}
/* Room for `extra` more nodes without reallocation (the multi-core port reserves a level's worth
 * before inserting in parallel). */
static void store_reserve(Store* S, int extra) {
  if (S->nn + extra <= S->capn) return;
  int c = S->capn ? S->capn : 1024;
  while (S->nn + extra > c) c *= 2;
  S->capn = c;
  S->zones = (int32_t*)realloc(S->zones, sizeof(int32_t) * S->d2 * (size_t)S->capn);
  S->next = (int*)realloc(S->next, sizeof(int) * S->capn);
  S->level = (int*)realloc(S->level, sizeof(int) * S->capn);
  S->dead = (char*)realloc(S->dead, S->capn);
}
/* Node ids and the live count are updated atomically: in the multi-core port, threads insert into
 * disjoint keys of one store (capacity reserved beforehand). */
static int store_node(Store* S, const int32_t* z, int level, int next) {
  if (S->nn == S->capn) store_reserve(S, 1);
  const int id = __atomic_fetch_add(&S->nn, 1, __ATOMIC_RELAXED);
  memcpy(S->zones + (size_t)id * S->d2, z, sizeof(int32_t) * S->d2);
  S->next[id] = next; S->level[id] = level; S->dead[id] = 0;
  __atomic_fetch_add(&S->nlive, 1, __ATOMIC_RELAXED);
  return id;
}
#define MERGE_SCAN 32   /* kMergeScan, include/hora/detail/engine_config.hpp:52 */
/* Returns the new node id, or -1 when the zone was subsumed. `z` may be replaced by a hull. */
static int store_add(Store* S, uint64_t k, int32_t* z, int level, int dim, const int32_t* Ls,
                     const int32_t* Us, int64_t* probes) {
  if ((uint64_t)(S->nkeys + 1) * 10 >= (S->smask + 1) * 7) store_grow(S);
  const uint64_t si = slot_of(S, k);
  if (S->shead[si] == -2) {
    S->skey[si] = k;
    S->shead[si] = store_node(S, z, level, -1);
    S->nkeys++;
    return S->shead[si];
  }
  const int d2 = S->d2;
  /* live chain, newest first */
  int nlv = 0, cap = 64;
  int* live = (int*)malloc(sizeof(int) * cap);
  for (int i = S->shead[si]; i >= 0; i = S->next[i])
    if (!S->dead[i]) { if (nlv == cap) { cap *= 2; live = (int*)realloc(live, sizeof(int) * cap); } live[nlv++] = i; }
  /* (1)+(2): dropped when simulated by a stored zone (plain inclusion implies simulation) */
  for (int t = 0; t < nlv; ++t) {
    if (probes) (*probes)++;
    if (orc_dbm_alu_le(z, S->zones + (size_t)live[t] * d2, dim, Ls, Us)) { free(live); return -1; }
  }
  /* (3): retire stored zones simulated by z */
  int w = 0;
  for (int t = 0; t < nlv; ++t) {
    if (orc_dbm_alu_le(S->zones + (size_t)live[t] * d2, z, dim, Ls, Us)) { S->dead[live[t]] = 1; __atomic_fetch_sub(&S->nlive, 1, __ATOMIC_RELAXED); }
    else live[w++] = live[t];
  }
  nlv = w;
  /* (4): convex-union absorb within the newest MERGE_SCAN live zones, restarting after each */
  for (int merged = 1; merged;) {
    merged = 0;
    for (int t = 0; t < nlv && t < MERGE_SCAN; ++t) {
      if (orc_dbm_try_union(z, S->zones + (size_t)live[t] * d2, dim)) {
        S->dead[live[t]] = 1; __atomic_fetch_sub(&S->nlive, 1, __ATOMIC_RELAXED);
        memmove(live + t, live + t + 1, sizeof(int) * (nlv - t - 1));
        nlv--;
        merged = 1;
        break;
      }
    }
  }
  free(live);
  /* (5): prepend */
  const int id = store_node(S, z, level, S->shead[si]);
  S->shead[si] = id;
  return id;
}

/* ============================================================================================
 * Level-synchronous BFS (reach_engine, src/reachability/engine.cpp:1410-1497, 2045-2200)
 *
 * Canonical order: a level's frontier is sorted by discrete key, and within a key lists the live
 * zones stored at the previous level in chain order (newest first). Successors are inserted in
 * (frontier position, emission ordinal) order -- the order the reference's --deterministic mode
 * uses (engine.cpp:2148-2162) -- and the target test covers the whole level before the verdict.
 * ============================================================================================ */
typedef struct { uint64_t key; int node; } FItem;
static int fcmp(const void* a, const void* b) {
  const FItem* x = (const FItem*)a; const FItem* y = (const FItem*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return 0;   /* qsort is not stable: ties are resolved by construction below */
}

/* The next frontier in canonical order: keys touched at `level` ascending, and within a key its
 * live zones stored at `level` in chain order (newest first). */
static int collect_frontier(const Store* S, int level, FItem** frp, int* capp) {
  FItem* fr = *frp;
  int nfr = 0, capfr = *capp;
  for (uint64_t i = 0; i <= S->smask; ++i) {
    if (S->shead[i] == -2 || S->stouch[i] != level) continue;
    for (int nd = S->shead[i]; nd >= 0; nd = S->next[nd]) {
      if (S->dead[nd] || S->level[nd] != level) continue;
      if (nfr == capfr) { capfr = capfr ? capfr * 2 : 16; fr = (FItem*)realloc(fr, sizeof(FItem) * capfr); }
      fr[nfr].key = S->skey[i]; fr[nfr].node = nd; nfr++;
    }
  }
  /* one slot per key, so each key's entries form one contiguous run: sort the runs by key */
  int nr = 0;
  FItem* heads = (FItem*)malloc(sizeof(FItem) * (nfr ? nfr : 1));
  for (int f = 0; f < nfr; ++f)
    if (f == 0 || fr[f].key != fr[f - 1].key) { heads[nr].key = fr[f].key; heads[nr].node = f; nr++; }
  qsort(heads, nr, sizeof(FItem), fcmp);
  FItem* out = (FItem*)malloc(sizeof(FItem) * (nfr ? nfr : 1));
  int o = 0;
  for (int r = 0; r < nr; ++r)
    for (int f = heads[r].node; f < nfr && fr[f].key == heads[r].key; ++f) out[o++] = fr[f];
  if (nfr) memcpy(fr, out, sizeof(FItem) * nfr);
  free(out); free(heads);
  *frp = fr; *capp = capfr;
  return nfr;
}

typedef struct {
  int32_t* locs; int32_t* ints; int32_t* zones;
  int* raw; int* parent;         /* transition index and emitting node (phase-2 graph) */
  int n, cap, np, ni, d2;
  int cur_parent;
} SuccBuf;
static void sb_emit(void* c, const int32_t* locs, const int32_t* ints, const int32_t* zone, int raw) {
  SuccBuf* b = (SuccBuf*)c;
  if (b->n == b->cap) {
    b->cap = b->cap ? b->cap * 2 : 1024;
    b->locs = (int32_t*)realloc(b->locs, sizeof(int32_t) * b->np * (size_t)b->cap);
    b->ints = (int32_t*)realloc(b->ints, sizeof(int32_t) * (b->ni ? b->ni : 1) * (size_t)b->cap);
    b->zones = (int32_t*)realloc(b->zones, sizeof(int32_t) * b->d2 * (size_t)b->cap);
    b->raw = (int*)realloc(b->raw, sizeof(int) * (size_t)b->cap);
    b->parent = (int*)realloc(b->parent, sizeof(int) * (size_t)b->cap);
  }
  memcpy(b->locs + (size_t)b->n * b->np, locs, sizeof(int32_t) * b->np);
  if (b->ni) memcpy(b->ints + (size_t)b->n * b->ni, ints, sizeof(int32_t) * b->ni);
  memcpy(b->zones + (size_t)b->n * b->d2, zone, sizeof(int32_t) * b->d2);
  b->raw[b->n] = raw;
  b->parent[b->n] = b->cur_parent;
  b->n++;
}

typedef struct {
  int kind;                      /* 0 target, 1 deadlock */
  const hora_pred_desc* target;
} Goal;
static int goal_hit(const Model* m, const Goal* g, const int32_t* locs, const int32_t* ints,
                    const int32_t* zone) {
  if (g->kind == 1) return state_has_deadlock(m, locs, ints, zone);
  const hora_pred_desc* t = g->target;
  if (t->never) return 0;
  if (!disc_match(t, locs, ints)) return 0;
  int32_t z[64 * 64];
  memcpy(z, zone, sizeof(int32_t) * m->dim * m->dim);
  return apply_cons(z, m->dim, t->clk_cond, 0, t->nclk);
}

static double g_time_limit = 0.0;   /* seconds; 0 = none. Bounds a CPU-baseline sample. */
void orc_set_time_limit(double seconds) { g_time_limit = seconds; }
static int g_threads = 1;           /* host threads of the reachability route (orc_set_threads) */
int32_t orc_set_threads(int32_t n) {
#ifdef _OPENMP
  g_threads = n < 1 ? 1 : n;
#else
  g_threads = 1;
#endif
  return g_threads;
}

static double now_s(void) {
  struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + ts.tv_nsec * 1e-9;
}

/* True once a set time limit has passed since t0. Checked between BFS levels and every 256 items
 * of the loops inside one, so a sample ends close to its limit; a run stopped this way reports
 * HORA_E_TIMEOUT and the successors generated so far, and its verdict is not used. */
static int over_time(double t0, int i) {
  return g_time_limit > 0 && (i & 255) == 255 && now_s() - t0 > g_time_limit;
}

#ifdef _OPENMP
#include <omp.h>
/* One BFS level of run_reach on g_threads host threads, with the sequential level's results: the
 * frontier is expanded in contiguous chunks (a thread's successors keep frontier order), the goal is
 * tested on every successor, new keys are entered in successor order, and each thread then inserts
 * the successors of its own share of the keys in successor order -- the passed-store folds of one
 * key never interleave with another's, so every key sees the same insertion sequence as in the
 * sequential loop (the reference's omp backend likewise inserts under per-stripe locks,
 * src/reachability/engine.cpp:2045-2201). Node ids differ; the stored sets and the next frontier
 * (ordered by key, then chain order) do not. Returns 1 when the goal is found or the time limit
 * passed, else 0. */
static int reach_level_par(Model* m, const Goal* goal, Store* S, const FItem* fr, int nfr, int level, int emode,
                           const uint8_t* qmask, const int32_t* Lq, const int32_t* Uq, double t0, hora_stats* S0,
                           int* found, SuccBuf* TB) {
  const int T = g_threads, dim = m->dim, d2 = dim * dim, np = m->n->nprocs, ni = m->n->nints;
  for (int t = 0; t < T; ++t) TB[t].n = 0;
  int timed = 0;
  S0->explored += nfr;
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    const int f0 = (int)((long)nfr * t / T), f1 = (int)((long)nfr * (t + 1) / T);
    int32_t l[64], i[64];
    for (int f = f0; f < f1; ++f) {
      if (((f - f0) & 255) == 255 && g_time_limit > 0 && now_s() - t0 > g_time_limit) { timed = 1; break; }
      key_decode(m, fr[f].key, l, i);
      successors(m, l, i, S->zones + (size_t)fr[f].node * d2, m->L, m->U, qmask, emode, sb_emit, &TB[t]);
    }
  }
  long total = 0;
  for (int t = 0; t < T; ++t) total += TB[t].n;
  S0->generated += (uint64_t)total;
  if (timed) { S0->status = HORA_E_TIMEOUT; return 1; }
  int hit = 0;
#pragma omp parallel num_threads(T) reduction(|:hit)
  {
    const SuccBuf* b = &TB[omp_get_thread_num()];
    for (int j = 0; j < b->n && !hit; ++j)
      if (goal_hit(m, goal, b->locs + (size_t)j * np, b->ints + (size_t)j * ni, b->zones + (size_t)j * d2)) hit = 1;
  }
  if (hit) { *found = 1; return 1; }
  /* successor g -> (buffer, position); keys; new keys entered in successor order */
  uint64_t* K = (uint64_t*)malloc(sizeof(uint64_t) * (total ? total : 1));
  const int32_t** Z = (const int32_t**)malloc(sizeof(int32_t*) * (total ? total : 1));
  const int32_t** Lp = (const int32_t**)malloc(sizeof(int32_t*) * (total ? total : 1));
  {
    long g = 0;
    for (int t = 0; t < T; ++t)
      for (int j = 0; j < TB[t].n; ++j, ++g) {
        Z[g] = TB[t].zones + (size_t)j * d2;
        Lp[g] = TB[t].locs + (size_t)j * np;
        K[g] = key_encode(m, Lp[g], TB[t].ints + (size_t)j * ni);
      }
  }
  for (long g = 0; g < total; ++g) {
    if ((uint64_t)(S->nkeys + 1) * 10 >= (S->smask + 1) * 7) store_grow(S);
    const uint64_t si = slot_of(S, K[g]);
    if (S->shead[si] == -2) { S->skey[si] = K[g]; S->shead[si] = -1; S->nkeys++; }
  }
  if ((uint64_t)(S->nkeys + 1) * 10 >= (S->smask + 1) * 7) store_grow(S);
  store_reserve(S, (int)total);
  uint64_t probes = 0;
#pragma omp parallel num_threads(T) reduction(+:probes)
  {
    const int t = omp_get_thread_num();
    int32_t Ls[64], Us[64];
    int64_t pr = 0;
    for (long g = 0; g < total; ++g) {
      if ((int)((mix64(K[g]) >> 33) % (uint64_t)T) != t) continue;
      const int32_t* sl = Lp[g];
      for (int c = 1; c < dim; ++c) {
        int32_t lv = ORC_ALU_NEG_INF, uv = ORC_ALU_NEG_INF;
        for (int p = 0; p < np; ++p) {
          const int gl = m->loc_base[p] + sl[p];
          lv = imax(lv, m->Lloc[gl * dim + c]); uv = imax(uv, m->Uloc[gl * dim + c]);
        }
        Ls[c] = imax(lv, Lq[c]); Us[c] = imax(uv, Uq[c]);
      }
      Ls[0] = Us[0] = 0;
      int32_t zc[64 * 64];
      memcpy(zc, Z[g], sizeof(int32_t) * d2);
      const int id = store_add(S, K[g], zc, level, dim, Ls, Us, &pr);
      if (id >= 0) S->stouch[slot_of(S, K[g])] = level;
    }
    probes += (uint64_t)pr;
  }
  S0->probes += probes;
  free(K); free(Z); free(Lp);
  return 0;
}
#endif

/* The engine shared by E<> and deadlock. `collapse` selects the a_M bounds of deadlock_reachable
 * (engine.cpp:2363-2405, the HORA_DL_MODE=m route). */
static int32_t run_reach(const hora_net_desc* net, const Goal* goal, int collapse, hora_stats* st,
                         int32_t* result) {
  double t0 = now_s();
  Model m;
  int rc = model_build(net, &m);
  if (rc) { model_free(&m); return rc; }
  if (m.keybits > 63) { model_free(&m); return HORA_E_NOT_SUPPORTED; }
  const int dim = m.dim, d2 = dim * dim, np = net->nprocs, ni = net->nints;
  if (collapse) {
    for (int c = 0; c < dim; ++c) m.L[c] = m.U[c] = imax(m.L[c], m.U[c]);
    for (int k = 0; k < m.nlocs_total * dim; ++k) m.Lloc[k] = m.Uloc[k] = imax(m.Lloc[k], m.Uloc[k]);
  }
  /* query constants: extend_bounds (engine.cpp:1417-1419) and Lq/Uq, qmask (:1440-1455) */
  uint8_t qmask[64] = {0};
  int32_t Lq[64], Uq[64];
  for (int c = 0; c < dim; ++c) Lq[c] = Uq[c] = ORC_ALU_NEG_INF;
  if (goal->kind == 0) {
    const hora_pred_desc* t = goal->target;
    for (int k = 0; k < t->nclk; ++k) {
      const int i = t->clk_cond[3 * k], j = t->clk_cond[3 * k + 1], v = r_bound(t->clk_cond[3 * k + 2]);
      if (i > 0) qmask[i] = 1;
      if (j > 0) qmask[j] = 1;
      if (i > 0 && j == 0) { m.U[i] = imax(m.U[i], v); Uq[i] = imax(Uq[i], v); }
      else if (i == 0 && j > 0) { m.L[j] = imax(m.L[j], -v); Lq[j] = imax(Lq[j], -v); }
      else if (i > 0 && j > 0) {
        const int a = v < 0 ? -v : v;
        m.U[i] = imax(m.U[i], a); m.U[j] = imax(m.U[j], a); m.L[i] = imax(m.L[i], a); m.L[j] = imax(m.L[j], a);
        Uq[i] = imax(Uq[i], a); Uq[j] = imax(Uq[j], a); Lq[i] = imax(Lq[i], a); Lq[j] = imax(Lq[j], a);
      }
    }
  }
  m.L[0] = m.U[0] = 0;
  int emode = 0;
  hora_stats S0;
  memset(&S0, 0, sizeof S0);
  /* initial state */
  int32_t locs[64], ints[64], zone[64 * 64];
  for (int p = 0; p < np; ++p) locs[p] = net->proc_init[p];
  for (int v = 0; v < ni; ++v) ints[v] = net->int_init[v];
  orc_dbm_init(zone, dim);
  int found = 0;
  Store S;
  store_init(&S, d2);
  SuccBuf B = {0};
  B.np = np; B.ni = ni; B.d2 = d2;
  SuccBuf* TB = NULL;   /* per-thread successor buffers of the multi-core port */
  FItem* fr = NULL; int nfr = 0, capfr = 0;
  int32_t Ls[64], Us[64];
  if (!close_succ_zone(&m, locs, ints, zone, qmask, m.L, m.U, emode) || orc_dbm_empty(zone, dim)) {
    *result = 0;
    goto done;
  }
  if (goal_hit(&m, goal, locs, ints, zone)) { found = 1; goto done; }
  {
    const uint64_t k0 = key_encode(&m, locs, ints);
    int id = store_add(&S, k0, zone, 0, dim, m.L, m.U, NULL);
    capfr = 16; fr = (FItem*)malloc(sizeof(FItem) * capfr);
    fr[0].key = k0; fr[0].node = id; nfr = 1;
  }
  int level = 0;
  while (nfr > 0) {
#ifdef _OPENMP
    if (g_threads > 1) {
      if (!TB) {   /* one successor buffer per thread, for this network's shapes */
        TB = (SuccBuf*)calloc((size_t)g_threads, sizeof(SuccBuf));
        for (int t = 0; t < g_threads; ++t) { TB[t].np = np; TB[t].ni = ni; TB[t].d2 = d2; }
      }
      const int lr = reach_level_par(&m, goal, &S, fr, nfr, ++level, emode, qmask, Lq, Uq, t0, &S0, &found, TB);
      if (lr) { S0.levels = level; goto done; }     /* goal found or time limit */
      nfr = collect_frontier(&S, level, &fr, &capfr);
      if (g_time_limit > 0 && now_s() - t0 > g_time_limit) { S0.levels = level; S0.status = HORA_E_TIMEOUT; goto done; }
      if (emode == 0 && S.nkeys && (double)S.nlive >= 4.0 * (double)S.nkeys) { emode = 1; S0.extrapolating = 1; }
      S0.levels = level;
      continue;
    }
#endif
    S0.explored += nfr;
    ++level;
    B.n = 0;
    /* expand in frontier order; successor b's insertion order is its buffer position */
    for (int f = 0; f < nfr; ++f) {
      if (over_time(t0, f)) { S0.generated += B.n; S0.levels = level; S0.status = HORA_E_TIMEOUT; goto done; }
      key_decode(&m, fr[f].key, locs, ints);
      successors(&m, locs, ints, S.zones + (size_t)fr[f].node * d2, m.L, m.U, qmask, emode, sb_emit, &B);
    }
    S0.generated += B.n;
    for (int b = 0; b < B.n && !found; ++b) {
      if (over_time(t0, b)) { S0.levels = level; S0.status = HORA_E_TIMEOUT; goto done; }
      if (goal_hit(&m, goal, B.locs + (size_t)b * np, B.ints + (size_t)b * ni, B.zones + (size_t)b * d2)) found = 1;
    }
    if (found) { S0.levels = level; goto done; }
    /* insert in order */
    for (int b = 0; b < B.n; ++b) {
      if (over_time(t0, b)) { S0.levels = level; S0.status = HORA_E_TIMEOUT; goto done; }
      const int32_t* sl = B.locs + (size_t)b * np;
      const uint64_t k = key_encode(&m, sl, B.ints + (size_t)b * ni);
      for (int c = 1; c < dim; ++c) {
        int32_t lv = ORC_ALU_NEG_INF, uv = ORC_ALU_NEG_INF;
        for (int p = 0; p < np; ++p) {
          const int gl = m.loc_base[p] + sl[p];
          lv = imax(lv, m.Lloc[gl * dim + c]); uv = imax(uv, m.Uloc[gl * dim + c]);
        }
        Ls[c] = imax(lv, Lq[c]); Us[c] = imax(uv, Uq[c]);
      }
      Ls[0] = Us[0] = 0;
      const uint64_t si = slot_of(&S, k);
      int64_t pr = 0;
      int id = store_add(&S, k, B.zones + (size_t)b * d2, level, dim, Ls, Us, &pr);
      S0.probes += pr;
      (void)si;
      if (id >= 0) S.stouch[slot_of(&S, k)] = level;
    }
    /* next frontier: touched keys ascending, chain order within a key */
    nfr = collect_frontier(&S, level, &fr, &capfr);
    if (g_time_limit > 0 && now_s() - t0 > g_time_limit) { S0.levels = level; S0.status = HORA_E_TIMEOUT; goto done; }
    /* adaptive switch to Extra_LU+ (engine.cpp:2178-2184) */
    if (emode == 0 && S.nkeys && (double)S.nlive >= 4.0 * (double)S.nkeys) { emode = 1; S0.extrapolating = 1; }
    S0.levels = level;
  }
done:
  *result = found;
  S0.stored = (uint64_t)S.nlive;
  S0.keys = (uint64_t)S.nkeys;
  S0.expanded = S0.explored;
  S0.seconds = now_s() - t0;
  S0.probes += 0;
  if (st) *st = S0;
  free(fr); free(B.locs); free(B.ints); free(B.zones); free(B.raw); free(B.parent);
  for (int t = 0; TB && t < g_threads; ++t) {
    free(TB[t].locs); free(TB[t].ints); free(TB[t].zones); free(TB[t].raw); free(TB[t].parent);
  }
  free(TB);
  store_free(&S);
  model_free(&m);
  return HORA_OK;
}

int32_t orc_reachable_net(const hora_net_desc* net, const hora_pred_desc* target, hora_stats* st,
                          int32_t* result) {
  Goal g = {0, target};
  return run_reach(net, &g, 0, st, result);
}
int32_t orc_deadlock_reachable(const hora_net_desc* net, hora_stats* st, int32_t* result) {
  Goal g = {1, NULL};
  return run_reach(net, &g, 1, st, result);
}

int32_t orc_initial_state(const hora_net_desc* net, const uint8_t* qmask, int32_t* locs,
                          int32_t* ints, int32_t* zone) {
  Model m;
  if (model_build(net, &m)) { model_free(&m); return 0; }
  for (int p = 0; p < net->nprocs; ++p) locs[p] = net->proc_init[p];
  for (int v = 0; v < net->nints; ++v) ints[v] = net->int_init[v];
  orc_dbm_init(zone, m.dim);
  int ok = close_succ_zone(&m, locs, ints, zone, qmask, m.L, m.U, 0) && !orc_dbm_empty(zone, m.dim);
  model_free(&m);
  return ok;
}

/* ============================================================================================
 * Leads-to, p --> q  (leads_to_clocks / leads_to_otf, src/liveness/api.cpp:655-733)
 *
 * p --> q fails iff some reachable state satisfying p and not q starts a maximal run that never
 * satisfies q. This restatement decides that with the same three ingredients as the reference's
 * backward sweep (src/liveness/fixpoint.cpp:48-977): the region of !q-states, the end-of-run set
 * (stop_set, src/liveness/construction.cpp:1200-1239), and the greatest fixpoint
 * W = W /\ (NoSucc \/ Pre(W)):
 *
 *  1. the reachable states, explored with the deadlock-sound a_M bisimulation bounds (every query
 *     constant folded in), give the roots: their p-part, cut to !q;
 *  2. from the roots, the zone graph of the network restricted to !q (q's clock atom is a single
 *     constraint, so its complement is convex and is adjoined to the invariant exactly where q's
 *     discrete part holds) is built with Extra_M+ for finiteness and inclusion covers, and W is
 *     swept on federations with the exact predecessor (leadsto_subsumed below).
 * E[] psi keeps the exact-zone variant of step 2: exact-zone deduplication makes the graph
 * post-stable (every valuation of a node has a predecessor in each of its source nodes), so
 * node-level emptiness of W is exact there, and a witness is a path of nodes.
 * ============================================================================================ */
/* A location requirement (p, l) with l >= 0 asks for location l; l < 0 for any location but -l-1. */
static int disc_match(const hora_pred_desc* t, const int32_t* locs, const int32_t* ints) {
  for (int k = 0; k < t->nloc; ++k) {
    const int l = t->loc_req[2 * k + 1], at = locs[t->loc_req[2 * k]];
    if (l >= 0 ? at != l : at == -l - 1) return 0;
  }
  return ints_ok(t->int_cond, t->nint, ints);
}
static int has_upper_invariant(const Model* m, const int32_t* locs) {
  const hora_net_desc* n = m->n;
  for (int p = 0; p < n->nprocs; ++p) {
    const int gl = m->loc_base[p] + locs[p];
    for (int c = n->loc_inv_off[gl]; c < n->loc_inv_off[gl + 1]; ++c)
      if (n->cons[3 * c] > 0 && n->cons[3 * c + 1] == 0 && n->cons[3 * c + 2] < ORC_INF) return 1;
  }
  return 0;
}
static int all_unbounded(const int32_t* z, int dim) {
  for (int i = 1; i < dim; ++i) if (z[i * dim] != ORC_INF) return 0;
  return 1;
}
/* time_diverges (construction.cpp:1097-1136): every clock unbounded after a delay inside the
 * invariant -- and, when `restricted`, inside !q as well. */
static int time_diverges(const Model* m, const int32_t* locs, const int32_t* ints, const int32_t* zone, int restricted) {
  const int dim = m->dim;
  if (m->n->nclocks == 0 || has_upper_invariant(m, locs)) return 0;
  int c, u;
  frozen_flags(m, locs, ints, &c, &u);
  if (c || u) return 0;
  int32_t z[64 * 64];
  memcpy(z, zone, sizeof(int32_t) * dim * dim);
  orc_dbm_delay(z, dim);
  if (!apply_inv(m, z, locs) || orc_dbm_empty(z, dim) || !all_unbounded(z, dim)) return 0;
  if (restricted && m->avoid && disc_match(m->avoid, locs, ints)) {
    memcpy(z, zone, sizeof(int32_t) * dim * dim);
    if (!avoid_cut(m, z, locs, ints)) return 0;
    orc_dbm_delay(z, dim);
    if (!apply_inv(m, z, locs) || !avoid_cut(m, z, locs, ints) || orc_dbm_empty(z, dim)) return 0;
    return all_unbounded(z, dim);
  }
  return 1;
}
/* orig_time_open (construction.cpp:1163-1177): can time run away here in the unrestricted system? */
static int orig_time_open(const Model* m, const int32_t* locs, const int32_t* ints) {
  const int dim = m->dim;
  if (m->n->nclocks == 0 || has_upper_invariant(m, locs)) return 0;
  int c, u;
  frozen_flags(m, locs, ints, &c, &u);
  if (c || u) return 0;
  int32_t z[64 * 64];
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) z[i * dim + j] = (i == j || i == 0) ? ORC_ZERO_LE : ORC_INF;
  orc_dbm_delay(z, dim);
  if (!apply_inv(m, z, locs)) return 0;
  return all_unbounded(z, dim);
}

/* Exact-zone dedup insert: returns the node holding zone z under key k (new or existing). */
static int store_find_or_add_exact(Store* S, uint64_t k, const int32_t* z, int level, int* is_new) {
  if ((uint64_t)(S->nkeys + 1) * 10 >= (S->smask + 1) * 7) store_grow(S);
  const uint64_t si = slot_of(S, k);
  *is_new = 0;
  if (S->shead[si] == -2) {
    S->skey[si] = k;
    S->shead[si] = store_node(S, z, level, -1);
    S->nkeys++;
    *is_new = 1;
    return S->shead[si];
  }
  for (int i = S->shead[si]; i >= 0; i = S->next[i])
    if (memcmp(S->zones + (size_t)i * S->d2, z, sizeof(int32_t) * S->d2) == 0) return i;
  const int id = store_node(S, z, level, S->shead[si]);
  S->shead[si] = id;
  *is_new = 1;
  return id;
}

typedef struct { int* a; int n, cap; } IVec;
static void iv_push(IVec* v, int x) {
  if (v->n == v->cap) { v->cap = v->cap ? v->cap * 2 : 256; v->a = (int*)realloc(v->a, sizeof(int) * v->cap); }
  v->a[v->n++] = x;
}

typedef struct { IVec* succ_keys_unused; int count; } CountCtx;
static void count_emit(void* c, const int32_t* l, const int32_t* i, const int32_t* z, int raw) {
  (void)l; (void)i; (void)z; (void)raw;
  ((CountCtx*)c)->count++;
}

static int32_t leadsto_subsumed(Model* m, Store* R, const hora_pred_desc* p, const hora_pred_desc* q,
                                const uint8_t* qmask, hora_stats* S0, double t0, int* violated_out);
static int leadsto_witness_at(Model* m, const hora_pred_desc* p, const hora_pred_desc* q, const int32_t* locs,
                              const int32_t* ints, const int32_t* zone, const uint8_t* qmask);
/* p --> q (psi NULL), or E[] psi (p, q NULL): the two share the restricted exact zone graph, its
 * stop sets and the greatest fixpoint. E[] psi roots the graph at the initial state of the
 * psi-restricted network instead of at the p-states of a reachability pass. */
static int32_t liveness_core(const hora_net_desc* net, const hora_pred_desc* p, const hora_pred_desc* q,
                             const hora_pred_desc* psi, hora_stats* st, int32_t* result) {
  double t0 = now_s();
  if (!psi && q->nclk > 1) return HORA_E_NOT_SUPPORTED;   /* !q must be convex: at most one clock atom */
  Model m;
  int rc = model_build(net, &m);
  if (rc) { model_free(&m); return rc; }
  if (m.keybits > 63 || m.has_diag) { model_free(&m); return HORA_E_NOT_SUPPORTED; }
  const int dim = m.dim, d2 = dim * dim, np = net->nprocs, ni = net->nints;
  /* bounds: query constants folded in, then collapsed to a_M (L = U = max) */
  uint8_t qmask[64] = {0};
  int32_t Lq[64], Uq[64];
  for (int c = 0; c < dim; ++c) Lq[c] = Uq[c] = ORC_ALU_NEG_INF;
  const hora_pred_desc* preds[2] = {psi ? psi : p, psi ? psi : q};
  for (int w = 0; w < (psi ? 1 : 2); ++w)
    for (int k = 0; k < preds[w]->nclk; ++k) {
      const int i = preds[w]->clk_cond[3 * k], j = preds[w]->clk_cond[3 * k + 1];
      const int v = r_bound(preds[w]->clk_cond[3 * k + 2]);
      if (i > 0) qmask[i] = 1;
      if (j > 0) qmask[j] = 1;
      const int a = v < 0 ? -v : v;
      const int x = i > 0 ? i : j;
      m.L[x] = imax(m.L[x], a); m.U[x] = imax(m.U[x], a);
      Lq[x] = imax(Lq[x], a); Uq[x] = imax(Uq[x], a);
    }
  for (int c = 0; c < dim; ++c) { m.L[c] = m.U[c] = imax(m.L[c], m.U[c]); Lq[c] = Uq[c] = imax(Lq[c], Uq[c]); }
  for (int k = 0; k < m.nlocs_total * dim; ++k) m.Lloc[k] = m.Uloc[k] = imax(m.Lloc[k], m.Uloc[k]);
  m.L[0] = m.U[0] = 0;
  hora_stats S0;
  memset(&S0, 0, sizeof S0);
  int32_t locs[64], ints[64], zone[64 * 64], z2[64 * 64], Ls[64], Us[64];
  /* ---- phase 1: reachable states under a_M subsumption ---- */
  Store R;
  store_init(&R, d2);
  SuccBuf B = {0};
  B.np = np; B.ni = ni; B.d2 = d2;
  FItem* fr = NULL; int nfr = 0, capfr = 0;
  int emode = 0;
  for (int pp = 0; pp < np; ++pp) locs[pp] = net->proc_init[pp];
  for (int v = 0; v < ni; ++v) ints[v] = net->int_init[v];
  orc_dbm_init(zone, dim);
  int violated = 0;
  if (!psi && close_succ_zone(&m, locs, ints, zone, qmask, m.L, m.U, 0) && !orc_dbm_empty(zone, dim)) {
    const uint64_t k0 = key_encode(&m, locs, ints);
    int id = store_add(&R, k0, zone, 0, dim, m.L, m.U, NULL);
    capfr = 16; fr = (FItem*)malloc(sizeof(FItem) * capfr);
    fr[0].key = k0; fr[0].node = id; nfr = 1;
    if (leadsto_witness_at(&m, p, q, locs, ints, zone, qmask)) { violated = 1; nfr = 0; }
  }
  int level = 0;
  int timed_out = 0;
#ifdef _OPENMP
  SuccBuf* TB = NULL;   /* per-thread successor buffers of the multi-core phase 1 */
  const hora_pred_desc never = {0, NULL, 0, NULL, 0, NULL, 1};
  const Goal nogoal = {0, &never};
#endif
  while (nfr > 0) {
    if (g_time_limit > 0 && now_s() - t0 > g_time_limit) { timed_out = 1; break; }
#ifdef _OPENMP
    if (g_threads > 1 && !psi) {   /* the same level on every host thread (reach_level_par) */
      if (!TB) {
        TB = (SuccBuf*)calloc((size_t)g_threads, sizeof(SuccBuf));
        for (int t = 0; t < g_threads; ++t) { TB[t].np = np; TB[t].ni = ni; TB[t].d2 = d2; }
      }
      int unused = 0;
      const uint64_t pr0 = S0.probes;   /* phase 1's probes are not reported, as in the loop below */
      const int lr = reach_level_par(&m, &nogoal, &R, fr, nfr, ++level, emode, qmask, Lq, Uq, t0, &S0, &unused, TB);
      S0.probes = pr0;
      if (lr) { timed_out = 1; break; }
      S0.status = 0;
    } else
#endif
    {
    S0.explored += nfr;
    ++level;
    B.n = 0;
    for (int f = 0; f < nfr; ++f) {
      if (over_time(t0, f)) { timed_out = 1; break; }
      key_decode(&m, fr[f].key, locs, ints);
      successors(&m, locs, ints, R.zones + (size_t)fr[f].node * d2, m.L, m.U, qmask, emode, sb_emit, &B);
    }
    S0.generated += B.n;
    for (int b = 0; b < B.n && !timed_out; ++b) {
      if (over_time(t0, b)) { timed_out = 1; break; }
      const int32_t* sl = B.locs + (size_t)b * np;
      const uint64_t k = key_encode(&m, sl, B.ints + (size_t)b * ni);
      for (int c = 1; c < dim; ++c) {
        int32_t lv = ORC_ALU_NEG_INF;
        for (int pp = 0; pp < np; ++pp) lv = imax(lv, m.Lloc[(m.loc_base[pp] + sl[pp]) * dim + c]);
        Ls[c] = Us[c] = imax(lv, Lq[c]);
      }
      Ls[0] = Us[0] = 0;
      int id = store_add(&R, k, B.zones + (size_t)b * d2, level, dim, Ls, Us, NULL);
      if (id >= 0) R.stouch[slot_of(&R, k)] = level;
    }
    if (timed_out) break;
    }
    nfr = collect_frontier(&R, level, &fr, &capfr);
    if (emode == 0 && R.nkeys && (double)R.nlive >= 4.0 * (double)R.nkeys) emode = 1;
    /* p --> q: the early witness on every zone this level stored (leadsto_witness,
       construction.cpp:786-826); the search stops at the level that finds one */
    for (int f = 0; f < nfr && !psi && !violated; ++f) {
      key_decode(&m, fr[f].key, locs, ints);
      violated = leadsto_witness_at(&m, p, q, locs, ints, R.zones + (size_t)fr[f].node * d2, qmask);
    }
    if (violated) break;
  }
  /* ---- roots: the p-part of every stored zone, cut to !q; for E[] psi, the initial state ---- */
  m.avoid = psi ? psi : q;
  m.avoid_psi = psi != NULL;
  if (!psi && q->nclk == 1) {
    m.avoid_neg[0] = q->clk_cond[1]; m.avoid_neg[1] = q->clk_cond[0]; m.avoid_neg[2] = r_negate(q->clk_cond[2]);
  }
#ifdef _OPENMP
  for (int t = 0; TB && t < g_threads; ++t) {
    free(TB[t].locs); free(TB[t].ints); free(TB[t].zones); free(TB[t].raw); free(TB[t].parent);
  }
  free(TB);
#endif
  if (!psi) {   /* p --> q: the subsumed graph and the federation sweep */
    int viol = violated;
    if (timed_out) S0.status = HORA_E_TIMEOUT;
    else if (!viol) leadsto_subsumed(&m, &R, p, q, qmask, &S0, t0, &viol);
    else S0.levels = (uint64_t)level;
    store_free(&R);
    S0.expanded = S0.explored;
    S0.seconds = now_s() - t0;
    if (st) *st = S0;
    *result = !viol;
    free(fr); free(B.locs); free(B.ints); free(B.zones); free(B.raw); free(B.parent);
    model_free(&m);
    return HORA_OK;
  }
  Store G;
  store_init(&G, d2);
  IVec roots = {0}, efrom = {0}, eto = {0};
  nfr = 0;
  if (psi) {
    for (int pp = 0; pp < np; ++pp) locs[pp] = net->proc_init[pp];
    for (int v = 0; v < ni; ++v) ints[v] = net->int_init[v];
    orc_dbm_init(z2, dim);
    if (close_succ_zone(&m, locs, ints, z2, qmask, m.L, m.U, 0) && !orc_dbm_empty(z2, dim)) {
      int is_new;
      const uint64_t k0 = key_encode(&m, locs, ints);
      const int id = store_find_or_add_exact(&G, k0, z2, 0, &is_new);
      iv_push(&roots, id);
      capfr = capfr ? capfr : 16;
      fr = (FItem*)realloc(fr, sizeof(FItem) * capfr);
      fr[0].key = k0; fr[0].node = id; nfr = 1;
    }
  }
  for (uint64_t i = 0; !psi && i <= R.smask; ++i) {
    if (R.shead[i] == -2) continue;
    key_decode(&m, R.skey[i], locs, ints);
    if (!disc_match(p, locs, ints)) continue;
    for (int nd = R.shead[i]; nd >= 0; nd = R.next[nd]) {
      if (R.dead[nd]) continue;
      memcpy(z2, R.zones + (size_t)nd * d2, sizeof(int32_t) * d2);
      if (!apply_cons(z2, dim, p->clk_cond, 0, p->nclk)) continue;
      if (!avoid_cut(&m, z2, locs, ints) || orc_dbm_empty(z2, dim)) continue;
      int is_new;
      const int id = store_find_or_add_exact(&G, R.skey[i], z2, 0, &is_new);
      if (is_new) {
        iv_push(&roots, id);
        if (nfr == capfr) { capfr = capfr ? capfr * 2 : 16; fr = (FItem*)realloc(fr, sizeof(FItem) * capfr); }
        fr[nfr].key = R.skey[i]; fr[nfr].node = id; nfr++;
      }
    }
  }
  store_free(&R);
  /* ---- phase 2: exact zone graph of the !q-restricted network from the roots ---- */
  IVec nodekey_unused = {0};
  (void)nodekey_unused;
  uint64_t* nkey = NULL; int nkcap = 0;
  level = 0;
  while (nfr > 0 && !timed_out) {
    if (g_time_limit > 0 && now_s() - t0 > g_time_limit) { timed_out = 1; break; }
    S0.explored += nfr;
    ++level;
    FItem* nxt = NULL; int nn = 0, capn = 0;
    for (int f = 0; f < nfr; ++f) {
      if (over_time(t0, f)) { timed_out = 1; break; }
      key_decode(&m, fr[f].key, locs, ints);
      B.n = 0;
      successors(&m, locs, ints, G.zones + (size_t)fr[f].node * d2, m.L, m.U, qmask, 1, sb_emit, &B);
      S0.generated += B.n;
      for (int b = 0; b < B.n; ++b) {
        const uint64_t k = key_encode(&m, B.locs + (size_t)b * np, B.ints + (size_t)b * ni);
        int is_new;
        const int id = store_find_or_add_exact(&G, k, B.zones + (size_t)b * d2, level, &is_new);
        iv_push(&efrom, fr[f].node);
        iv_push(&eto, id);
        if (is_new) {
          if (nn == capn) { capn = capn ? capn * 2 : 16; nxt = (FItem*)realloc(nxt, sizeof(FItem) * capn); }
          nxt[nn].key = k; nxt[nn].node = id; nn++;
        }
      }
    }
    free(fr);
    fr = nxt; nfr = nn; capfr = capn;
  }
  /* node keys, for the stop sets (a timed-out run skips the sweep: its verdict is not used) */
  nkcap = timed_out ? 0 : G.nn;
  nkey = (uint64_t*)malloc(sizeof(uint64_t) * (nkcap ? nkcap : 1));
  for (uint64_t i = 0; i <= G.smask; ++i)
    if (G.shead[i] != -2)
      for (int nd = G.shead[i]; nd >= 0 && nkcap; nd = G.next[nd]) nkey[nd] = G.skey[i];
  /* ---- stop sets (stop_set, construction.cpp:1200-1239) ---- */
  char* stop = (char*)calloc(G.nn ? G.nn : 1, 1);
  char* inW = (char*)malloc(G.nn ? G.nn : 1);
  const hora_pred_desc* av = m.avoid;
  for (int u = 0; u < nkcap; ++u) {
    if (over_time(t0, u)) { timed_out = 1; break; }
    key_decode(&m, nkey[u], locs, ints);
    const int32_t* zu = G.zones + (size_t)u * d2;
    m.avoid = NULL;   /* deadlock and any-successor are judged in the unrestricted network */
    if ((psi ? psi->nclk : q->nclk) == 0) {
      CountCtx cc = {NULL, 0};
      successors(&m, locs, ints, zu, m.L, m.U, qmask, 1, count_emit, &cc);
      stop[u] = cc.count == 0 || time_diverges(&m, locs, ints, zu, 0) || state_has_deadlock(&m, locs, ints, zu);
    } else {
      m.avoid = av;
      if (time_diverges(&m, locs, ints, zu, 1)) stop[u] = 1;
      else if (orig_time_open(&m, locs, ints)) stop[u] = 0;
      else { m.avoid = NULL; stop[u] = state_has_deadlock(&m, locs, ints, zu) ? 1 : 0; }
    }
    m.avoid = av;
    inW[u] = 1;
  }
  /* ---- greatest fixpoint over the graph (CSR by source) ---- */
  int* off = (int*)calloc(G.nn + 1, sizeof(int));
  int* dst = (int*)malloc(sizeof(int) * (efrom.n ? efrom.n : 1));
  for (int e = 0; e < efrom.n; ++e) off[efrom.a[e] + 1]++;
  for (int u = 0; u < G.nn; ++u) off[u + 1] += off[u];
  {
    int* fill = (int*)calloc(G.nn ? G.nn : 1, sizeof(int));
    for (int e = 0; e < efrom.n; ++e) dst[off[efrom.a[e]] + fill[efrom.a[e]]++] = eto.a[e];
    free(fill);
  }
  for (int changed = !timed_out; changed;) {
    changed = 0;
    S0.gfp_iters++;
    for (int u = 0; u < G.nn; ++u) {
      if (!inW[u] || stop[u]) continue;
      int any = 0;
      for (int e = off[u]; e < off[u + 1] && !any; ++e) any = inW[dst[e]];
      if (!any) { inW[u] = 0; changed = 1; }
    }
  }
  for (int r = 0; r < roots.n && !violated && !timed_out; ++r) violated = inW[roots.a[r]];
  S0.stored = (uint64_t)G.nn;
  S0.keys = (uint64_t)G.nkeys;
  S0.levels = (uint64_t)level;
  S0.pre_calls = (uint64_t)efrom.n;
  S0.expanded = S0.explored;
  S0.seconds = now_s() - t0;
  if (timed_out) S0.status = HORA_E_TIMEOUT;
  if (st) *st = S0;
  *result = psi ? violated : !violated;   /* E[] psi holds iff its root keeps a maximal psi-run */
  free(off); free(dst); free(stop); free(inW); free(nkey);
  free(roots.a); free(efrom.a); free(eto.a); free(fr);
  free(B.locs); free(B.ints); free(B.zones); free(B.raw); free(B.parent);
  store_free(&G);
  model_free(&m);
  return HORA_OK;
}

/* ============================================================================================
 * Leads-to on the subsumed graph: inclusion covers and a federation-valued backward sweep
 * (online_intern / online_covers, src/liveness/construction.cpp:194-215,480-684;
 *  solve_greatest_fixpoint / relax, src/liveness/fixpoint.cpp:48-977,750-864;
 *  exact_predecessor, src/liveness/operators.cpp:257-306; stop_set, construction.cpp:1200-1239)
 *
 * Phase 2 of p --> q. From the roots (phase 1's p-zones cut to p's clock atoms and to !q), the
 * !q-restricted network is explored level by level with Extra_M+, and a successor is covered by a
 * stored zone of its discrete key only when that zone CONTAINS it. A level stores, per key, the
 * successors not contained in an earlier-level zone that are maximal among the level's own (a
 * successor strictly inside another, or equal to an earlier one, is covered by the first stored one
 * containing it). The stored set of a level is therefore a function of the set of successor zones
 * alone, independent of processing order. Every edge points at a zone containing the exact
 * successor, so the backward operator
 *     W[v] := W[v] /\ (Stop(v) \/ U_e Pre_e(W[tgt e]))
 * computed on federations with the exact predecessor is exact at the level of valuations: W[v] is
 * the set of valuations of Z_v that start a maximal !q-run. p --> q is violated iff a root keeps a
 * non-empty W. Early witness (leadsto_witness, construction.cpp:786-826): a root whose stop set is
 * non-empty already starts such a run, and the graph is not built.
 * ============================================================================================ */
typedef struct { int32_t* z; int n, cap, d2; } Fed;
static void fed_init(Fed* f, int d2) { f->z = NULL; f->n = f->cap = 0; f->d2 = d2; }
static void fed_free(Fed* f) { free(f->z); f->z = NULL; f->n = f->cap = 0; }
static void fed_push(Fed* f, const int32_t* z) {
  if (f->n == f->cap) {
    f->cap = f->cap ? f->cap * 2 : 4;
    f->z = (int32_t*)realloc(f->z, sizeof(int32_t) * f->d2 * (size_t)f->cap);
  }
  memcpy(f->z + (size_t)f->n * f->d2, z, sizeof(int32_t) * f->d2);
  f->n++;
}
static void fed_remove(Fed* f, int i) {   /* order is not kept */
  if (i != f->n - 1) memcpy(f->z + (size_t)i * f->d2, f->z + (size_t)(f->n - 1) * f->d2, sizeof(int32_t) * f->d2);
  f->n--;
}
/* out := a /\ b; 0 when empty */
static int dbm_intersect(int32_t* out, const int32_t* a, const int32_t* b, int dim) {
  const int d2 = dim * dim;
  for (int k = 0; k < d2; ++k) out[k] = a[k] < b[k] ? a[k] : b[k];
  orc_dbm_close(out, dim);
  return !orc_dbm_empty(out, dim);
}
/* Add z (non-empty) to f: dropped if a member contains it; members it contains are dropped; exact
 * convex unions with members are taken (fed_compact, src/liveness/operators.cpp:428). */
static void fed_add_compact(Fed* f, int32_t* z, int dim) {
  const int d2 = dim * dim;
  for (int i = 0; i < f->n; ++i) if (orc_dbm_includes(f->z + (size_t)i * d2, z, dim)) return;
  for (int merged = 1; merged;) {
    merged = 0;
    for (int i = 0; i < f->n;) {
      if (orc_dbm_includes(z, f->z + (size_t)i * d2, dim)) { fed_remove(f, i); continue; }
      ++i;
    }
    for (int i = 0; i < f->n; ++i)
      if (orc_dbm_try_union(z, f->z + (size_t)i * d2, dim)) { fed_remove(f, i); merged = 1; break; }
  }
  fed_push(f, z);
}
/* The pieces of z \ (w[0] U .. U w[k-1]) appended to out (disjoint pieces; fed_subtract). */
static void fed_subtract_rec(const int32_t* z, const int32_t* w, int k, int dim, Fed* out) {
  const int d2 = dim * dim;
  int32_t t[64 * 64];
  int i = 0;
  for (; i < k; ++i) if (dbm_intersect(t, z, w + (size_t)i * d2, dim)) break;
  if (i == k) { fed_push(out, z); return; }
  const int32_t* wi = w + (size_t)i * d2;
  if (orc_dbm_includes(wi, z, dim)) return;
  int32_t* r = (int32_t*)malloc(sizeof(int32_t) * d2 * 2);
  int32_t* p = r + d2;
  memcpy(r, z, sizeof(int32_t) * d2);
  int alive = 1;
  for (int a = 0; a < dim && alive; ++a)
    for (int b = 0; b < dim && alive; ++b) {
      if (a == b || wi[a * dim + b] >= r[a * dim + b]) continue;
      memcpy(p, r, sizeof(int32_t) * d2);
      if (orc_dbm_constrain(p, dim, b, a, r_negate(wi[a * dim + b])))
        fed_subtract_rec(p, w + (size_t)(i + 1) * d2, k - i - 1, dim, out);
      if (!orc_dbm_constrain(r, dim, a, b, wi[a * dim + b])) alive = 0;
    }
  free(r);
}

/* The recipe of one transition (GfpTag, src/liveness/operators.cpp:55-206): the participating
 * local edges, sender first, and the abstaining broadcast receivers' guard complements. */
#define TR_MAXAB 1024
typedef struct { int ne; int edge[64]; int nab; int32_t ab[3 * TR_MAXAB]; } Trans;
/* Rebuild the recipe of transition `want` (the raw index successors() gave it) of the discrete
 * state (locs, ints): the same enumeration with no zone work. Returns 0 if there is none. */
static int find_trans(const Model* m, const int32_t* locs, const int32_t* ints, int want, Trans* T) {
  const hora_net_desc* n = m->n;
  const int np = n->nprocs;
  int src_c, src_u, raw = 0;
  frozen_flags(m, locs, ints, &src_c, &src_u);
  T->ne = 0; T->nab = 0;
  for (int p = 0; p < np; ++p) {
    if (src_c && !loc_committed(m, p, locs[p])) continue;
    const int gp = m->loc_base[p] + locs[p];
    for (int k = m->eloc_off[gp]; k < m->eloc_off[gp + 1]; ++k) {
      const int e = m->eloc[k];
      if (n->edge_chan[e] >= 0 || !int_ok(n, e, ints)) continue;
      if (raw++ == want) { T->edge[T->ne++] = e; return 1; }
    }
  }
  for (int i = 0; i < np; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1]; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1) continue;
      if (n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST) continue;
      if (!int_ok(n, se, ints)) continue;
      const int i_comm = loc_committed(m, i, locs[i]);
      for (int j = 0; j < np; ++j) {
        if (j == i) continue;
        const int gj = m->loc_base[j] + locs[j];
        for (int q = m->eloc_off[gj]; q < m->eloc_off[gj + 1]; ++q) {
          const int re = m->eloc[q];
          if (n->edge_chan[re] != n->edge_chan[se] || n->edge_dir[re] != -1) continue;
          if (src_c && !(i_comm || loc_committed(m, j, locs[j]))) continue;
          if (!int_ok(n, re, ints)) continue;
          if (raw++ == want) { T->edge[0] = se; T->edge[1] = re; T->ne = 2; return 1; }
        }
      }
    }
  }
  Parts* P = parts_scratch();
  for (int i = 0; i < np; ++i) {
    const int gi = m->loc_base[i] + locs[i];
    for (int k = m->eloc_off[gi]; k < m->eloc_off[gi + 1]; ++k) {
      const int se = m->eloc[k];
      if (n->edge_chan[se] < 0 || n->edge_dir[se] != 1 || !(n->chan_flags[n->edge_chan[se]] & HORA_CHAN_BROADCAST)) continue;
      if (!int_ok(n, se, ints)) continue;
      if (!build_broadcast_parts(m, locs, ints, se, i, P)) return 0;
      int pick[MAXPART];
      memset(pick, 0, sizeof pick);
      for (;;) {
        int part_comm = loc_committed(m, i, locs[i]);
        for (int t = 0; t < P->nparts; ++t) {
          const Part* pt = &P->parts[t];
          if (pt->edge[pick[t]] >= 0 && loc_committed(m, pt->proc, locs[pt->proc])) part_comm = 1;
        }
        if (!src_c || part_comm) {
          if (raw++ == want) {
            T->edge[T->ne++] = se;
            for (int t = 0; t < P->nparts; ++t) {
              const Part* pt = &P->parts[t];
              const int o = pick[t];
              if (pt->edge[o] >= 0) { T->edge[T->ne++] = pt->edge[o]; continue; }
              for (int c = 0; c < pt->xn[o]; ++c) {
                if (T->nab == TR_MAXAB) return 0;
                memcpy(T->ab + 3 * T->nab, P->xcons + 3 * (pt->xoff[o] + c), sizeof(int32_t) * 3);
                T->nab++;
              }
            }
            return 1;
          }
        }
        if (P->nparts == 0) break;
        int t = 0;
        for (; t < P->nparts; ++t) { if (++pick[t] < P->parts[t].nopt) break; pick[t] = 0; }
        if (t == P->nparts) break;
      }
    }
  }
  return 0;
}
/* Exact predecessor of the target valuations Y through T, from (sl, si) to (tl, ti), in place
 * (exact_predecessor, src/liveness/operators.cpp:257-306): undo the active-clock reduction at the
 * target, the target invariant and delay, the resets, the guards and abstain constraints, then the
 * delay before the action. The !q restriction is adjoined to both invariants exactly as the
 * successor pipeline adjoins it, and the source invariant also holds at the action point itself, so
 * the result is the exact set of source valuations with a step into Y. Returns 0 when empty. */
static int pre_trans(const Model* m, const Trans* T, const int32_t* sl, const int32_t* si, const int32_t* tl,
                     const int32_t* ti, const uint8_t* qmask, int32_t* Y) {
  const hora_net_desc* n = m->n;
  const int dim = m->dim;
  uint64_t act = 0;
  for (int c = 1; c < dim; ++c) if (qmask[c]) act |= 1ull << c;
  for (int p = 0; p < n->nprocs; ++p) act |= m->act[m->loc_base[p] + tl[p]];
  for (int c = 1; c < dim; ++c) if (!((act >> c) & 1)) orc_dbm_free(Y, dim, c);
  if (!apply_inv(m, Y, tl) || !avoid_cut(m, Y, tl, ti) || orc_dbm_empty(Y, dim)) return 0;
  int fc, fu;
  frozen_flags(m, tl, ti, &fc, &fu);
  if (!fc && !fu) {
    orc_dbm_down(Y, dim);
    if (!apply_inv(m, Y, tl) || !avoid_cut(m, Y, tl, ti) || orc_dbm_empty(Y, dim)) return 0;
  }
  for (int k = 0; k < T->ne; ++k) {
    const int e = T->edge[k];
    for (int r = n->edge_reset_off[e]; r < n->edge_reset_off[e + 1]; ++r) {
      const int x = n->resets[r];
      if (!orc_dbm_constrain(Y, dim, x, 0, ORC_ZERO_LE) || !orc_dbm_constrain(Y, dim, 0, x, ORC_ZERO_LE)) return 0;
    }
  }
  for (int k = 0; k < T->ne; ++k) {
    const int e = T->edge[k];
    for (int r = n->edge_reset_off[e]; r < n->edge_reset_off[e + 1]; ++r) orc_dbm_free(Y, dim, n->resets[r]);
  }
  for (int k = 0; k < T->ne; ++k) {
    const int e = T->edge[k];
    if (!apply_cons(Y, dim, n->cons, n->edge_guard_off[e], n->edge_guard_off[e + 1])) return 0;
  }
  if (T->nab && !apply_cons(Y, dim, T->ab, 0, T->nab)) return 0;
  if (!apply_inv(m, Y, sl) || !avoid_cut(m, Y, sl, si) || orc_dbm_empty(Y, dim)) return 0;
  frozen_flags(m, sl, si, &fc, &fu);
  if (!fc && !fu) {
    orc_dbm_down(Y, dim);
    if (!apply_inv(m, Y, sl) || !avoid_cut(m, Y, sl, si) || orc_dbm_empty(Y, dim)) return 0;
  }
  return 1;
}
/* Stop(v) as a federation (stop_set, construction.cpp:1200-1239): the whole zone when time
 * diverges inside !q (or, for a purely discrete q, when the state has no successor at all);
 * nothing when q has a clock atom and the unrestricted location lets time run away; otherwise the
 * deadlocked valuations of the zone in the unrestricted network (state_has_deadlock's residue,
 * src/reachability/deadlock.cpp:262-267), as disjoint pieces. Returns 1 when it is the whole zone. */
static int stop_fed(Model* m, const hora_pred_desc* q, const int32_t* locs, const int32_t* ints,
                    const int32_t* zu, const uint8_t* qmask, Fed* out) {
  const hora_pred_desc* av = m->avoid;
  int whole = 0;
  out->n = 0;
  if (q->nclk == 0) {
    m->avoid = NULL;
    CountCtx cc = {NULL, 0};
    successors(m, locs, ints, zu, m->L, m->U, qmask, 1, count_emit, &cc);
    whole = cc.count == 0 || time_diverges(m, locs, ints, zu, 0);
  } else {
    whole = time_diverges(m, locs, ints, zu, 1);
    if (!whole && orig_time_open(m, locs, ints)) { m->avoid = av; return 0; }
    m->avoid = NULL;
  }
  if (whole) fed_push(out, zu);
  else {
    int32_t Z[64 * 64];
    Escapes E = {0};
    int frozen = 0;
    if (deadlock_escapes(m, locs, ints, zu, &E, Z, &frozen) && !E.covered)
      fed_subtract_rec(zu, E.w, E.nw, m->dim, out);
    free(E.w);
  }
  m->avoid = av;
  return whole;
}

/* Leads-to phase 2 for one state, for replaying a counterexample trace: the restricted model (the
 * network restricted to !q, !q adjoined to the invariants as close_succ_zone adjoins it). */
static int lt_model(const hora_net_desc* net, const hora_pred_desc* q, Model* m) {
  if (model_build(net, m)) return 0;
  m->avoid = q;
  m->avoid_psi = 0;
  if (q->nclk == 1) {
    m->avoid_neg[0] = q->clk_cond[1]; m->avoid_neg[1] = q->clk_cond[0]; m->avoid_neg[2] = r_negate(q->clk_cond[2]);
  }
  return 1;
}
int32_t orc_lt_successor_raw(const hora_net_desc* net, const hora_pred_desc* q, const uint8_t* qmask,
                             const int32_t* locs, const int32_t* ints, const int32_t* zone, int32_t raw,
                             int32_t* out_locs, int32_t* out_ints, int32_t* out_zone) {
  Model m;
  if (!lt_model(net, q, &m)) { model_free(&m); return 0; }
  uint8_t qm[64] = {0};
  if (qmask) memcpy(qm, qmask, (size_t)m.dim);
  RawCtx x = {raw, 0, net->nprocs, net->nints, m.dim * m.dim, out_locs, out_ints, out_zone};
  successors(&m, locs, ints, zone, m.L, m.U, qm, 0, raw_emit, &x);
  model_free(&m);
  return x.hit;
}
int32_t orc_lt_stop(const hora_net_desc* net, const hora_pred_desc* q, const uint8_t* qmask,
                    const int32_t* locs, const int32_t* ints, const int32_t* zone) {
  Model m;
  if (!lt_model(net, q, &m)) { model_free(&m); return -1; }
  uint8_t qm[64] = {0};
  if (qmask) memcpy(qm, qmask, (size_t)m.dim);
  Fed f;
  fed_init(&f, m.dim * m.dim);
  const int whole = stop_fed(&m, q, locs, ints, zone, qm, &f);
  const int32_t r = whole ? 2 : f.n > 0 ? 1 : 0;
  fed_free(&f);
  model_free(&m);
  return r;
}

/* The early witness of p --> q at a reachable zone (leadsto_witness, construction.cpp:786-826): its
 * p-part, cut to !q, holds a valuation where a maximal !q-run may stop (Stop above) -- that run
 * never meets q, so the property is violated. m->avoid is set for the test only (phase 1 explores
 * the unrestricted network). */
static int leadsto_witness_at(Model* m, const hora_pred_desc* p, const hora_pred_desc* q, const int32_t* locs,
                              const int32_t* ints, const int32_t* zone, const uint8_t* qmask) {
  if (!disc_match(p, locs, ints)) return 0;
  const int dim = m->dim;
  int32_t z[64 * 64];
  memcpy(z, zone, sizeof(int32_t) * dim * dim);
  if (!apply_cons(z, dim, p->clk_cond, 0, p->nclk)) return 0;
  const hora_pred_desc* av = m->avoid;
  const int ap = m->avoid_psi;
  int32_t an[3] = {m->avoid_neg[0], m->avoid_neg[1], m->avoid_neg[2]};
  m->avoid = q; m->avoid_psi = 0;
  if (q->nclk == 1) { m->avoid_neg[0] = q->clk_cond[1]; m->avoid_neg[1] = q->clk_cond[0]; m->avoid_neg[2] = r_negate(q->clk_cond[2]); }
  int hit = 0;
  if (avoid_cut(m, z, locs, ints) && !orc_dbm_empty(z, dim)) {
    Fed f;
    fed_init(&f, dim * dim);
    stop_fed(m, q, locs, ints, z, qmask, &f);
    hit = f.n > 0;
    fed_free(&f);
  }
  m->avoid = av; m->avoid_psi = ap;
  memcpy(m->avoid_neg, an, sizeof an);
  return hit;
}

typedef struct { uint64_t key; int idx; } KIdx;
static int kidx_cmp(const void* a, const void* b) {
  const KIdx* x = (const KIdx*)a; const KIdx* y = (const KIdx*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}
/* One level of the inclusion graph. Candidates c = 0..n-1 (key, zone); cov[c] receives the node
 * that covers c (an earlier-level node containing it, else the first stored candidate of the level
 * containing it, or its own new node). New nodes are appended to G (level `level`) in candidate
 * order; their ids are listed in *newids. */
static void incl_level(Store* G, uint64_t** nkey, int* nkcap, int nc, const uint64_t* ckey, const int32_t* cz,
                       int level, int dim, int* cov, IVec* newids, uint64_t* probes) {
  const int d2 = dim * dim;
  KIdx* sv = (KIdx*)malloc(sizeof(KIdx) * (nc ? nc : 1));
  int ns = 0;
  for (int c = 0; c < nc; ++c) {
    cov[c] = -1;
    const uint64_t si = slot_of(G, ckey[c]);
    if (G->shead[si] != -2)
      for (int nd = G->shead[si]; nd >= 0; nd = G->next[nd]) {
        if (probes) (*probes)++;
        if (orc_dbm_includes(G->zones + (size_t)nd * d2, cz + (size_t)c * d2, dim)) { cov[c] = nd; break; }
      }
    if (cov[c] < 0) { sv[ns].key = ckey[c]; sv[ns].idx = c; ns++; }
  }
  qsort(sv, ns, sizeof(KIdx), kidx_cmp);
  char* keep = (char*)calloc(nc ? nc : 1, 1);
  for (int a = 0; a < ns;) {
    int b = a;
    while (b < ns && sv[b].key == sv[a].key) ++b;
    for (int i = a; i < b; ++i) {
      const int32_t* zi = cz + (size_t)sv[i].idx * d2;
      int kept = 1;
      for (int j = a; j < b && kept; ++j) {
        if (j == i) continue;
        const int32_t* zj = cz + (size_t)sv[j].idx * d2;
        if (!orc_dbm_includes(zj, zi, dim)) continue;
        if (j < i || memcmp(zi, zj, sizeof(int32_t) * d2) != 0) kept = 0;
      }
      keep[sv[i].idx] = (char)kept;
    }
    a = b;
  }
  for (int c = 0; c < nc; ++c) {
    if (!keep[c]) continue;
    if ((uint64_t)(G->nkeys + 1) * 10 >= (G->smask + 1) * 7) store_grow(G);
    const uint64_t si = slot_of(G, ckey[c]);
    if (G->shead[si] == -2) { G->skey[si] = ckey[c]; G->shead[si] = -1; G->nkeys++; }
    const int id = store_node(G, cz + (size_t)c * d2, level, G->shead[si]);
    G->shead[si] = id;
    if (id >= *nkcap) { *nkcap = *nkcap ? *nkcap * 2 : 1024; *nkey = (uint64_t*)realloc(*nkey, sizeof(uint64_t) * *nkcap); }
    (*nkey)[id] = ckey[c];
    cov[c] = id;
    iv_push(newids, id);
  }
  /* a survivor not stored: the first stored survivor of its key (candidate order) containing it */
  for (int a = 0; a < ns;) {
    int b = a;
    while (b < ns && sv[b].key == sv[a].key) ++b;
    for (int i = a; i < b; ++i) {
      const int c = sv[i].idx;
      if (keep[c]) continue;
      for (int j = a; j < b; ++j)
        if (keep[sv[j].idx] && orc_dbm_includes(cz + (size_t)sv[j].idx * d2, cz + (size_t)c * d2, dim)) {
          cov[c] = cov[sv[j].idx];
          break;
        }
    }
    a = b;
  }
  free(keep); free(sv);
}

/* Phase 2 of p --> q on the subsumed graph, from phase 1's store R. */
static int32_t leadsto_subsumed(Model* m, Store* R, const hora_pred_desc* p, const hora_pred_desc* q,
                                const uint8_t* qmask, hora_stats* S0, double t0, int* violated_out) {
  const hora_net_desc* net = m->n;
  const int dim = m->dim, d2 = dim * dim, np = net->nprocs, ni = net->nints;
  int32_t locs[64], ints[64], z2[64 * 64];
  Store G;
  store_init(&G, d2);
  uint64_t* nkey = NULL; int nkcap = 0;
  IVec efrom = {0}, eto = {0}, eraw = {0}, roots = {0}, front = {0};
  int timed_out = 0, violated = 0;
  /* ---- roots ---- */
  {
    uint64_t* ck = NULL; int32_t* cz = NULL; int nc = 0, cc = 0;
    for (uint64_t i = 0; i <= R->smask; ++i) {
      if (R->shead[i] == -2) continue;
      key_decode(m, R->skey[i], locs, ints);
      if (!disc_match(p, locs, ints)) continue;
      for (int nd = R->shead[i]; nd >= 0; nd = R->next[nd]) {
        if (R->dead[nd]) continue;
        memcpy(z2, R->zones + (size_t)nd * d2, sizeof(int32_t) * d2);
        if (!apply_cons(z2, dim, p->clk_cond, 0, p->nclk)) continue;
        if (!avoid_cut(m, z2, locs, ints) || orc_dbm_empty(z2, dim)) continue;
        if (nc == cc) { cc = cc ? cc * 2 : 64; ck = (uint64_t*)realloc(ck, 8 * (size_t)cc); cz = (int32_t*)realloc(cz, sizeof(int32_t) * d2 * (size_t)cc); }
        ck[nc] = R->skey[i];
        memcpy(cz + (size_t)nc * d2, z2, sizeof(int32_t) * d2);
        nc++;
      }
    }
    int* cov = (int*)malloc(sizeof(int) * (nc ? nc : 1));
    incl_level(&G, &nkey, &nkcap, nc, ck, cz, 0, dim, cov, &roots, NULL);
    free(cov); free(ck); free(cz);
  }
  int level = 0;
  if (!violated) {
    for (int r = 0; r < roots.n; ++r) iv_push(&front, roots.a[r]);
    SuccBuf B = {0};
    B.np = np; B.ni = ni; B.d2 = d2;
    uint64_t* ck = NULL; int ckcap = 0;
    int* cov = NULL;
    while (front.n > 0 && !timed_out) {
      if (g_time_limit > 0 && now_s() - t0 > g_time_limit) { timed_out = 1; break; }
      S0->explored += front.n;
      ++level;
      B.n = 0;
      for (int f = 0; f < front.n; ++f) {
        if (over_time(t0, f)) { timed_out = 1; break; }
        key_decode(m, nkey[front.a[f]], locs, ints);
        B.cur_parent = front.a[f];
        successors(m, locs, ints, G.zones + (size_t)front.a[f] * d2, m->L, m->U, qmask, 1, sb_emit, &B);
      }
      if (timed_out) break;
      S0->generated += B.n;
      if (B.n > ckcap) { ckcap = B.n; ck = (uint64_t*)realloc(ck, 8 * (size_t)ckcap); cov = (int*)realloc(cov, sizeof(int) * ckcap); }
      for (int b = 0; b < B.n; ++b) ck[b] = key_encode(m, B.locs + (size_t)b * np, B.ints + (size_t)b * ni);
      IVec nxt = {0};
      incl_level(&G, &nkey, &nkcap, B.n, ck, B.zones, level, dim, cov, &nxt, &S0->probes);
      for (int b = 0; b < B.n; ++b) { iv_push(&efrom, B.parent[b]); iv_push(&eto, cov[b]); iv_push(&eraw, B.raw[b]); }
      free(front.a);
      front = nxt;
    }
    free(B.locs); free(B.ints); free(B.zones); free(B.raw); free(B.parent);
    free(ck); free(cov);
  }
  S0->stored = (uint64_t)G.nn;
  S0->keys = (uint64_t)G.nkeys;
  S0->levels = (uint64_t)level;
  /* ---- the backward sweep: a worklist of nodes whose successors' W changed ---- */
  if (!violated && !timed_out && G.nn > 0) {
    const int N = G.nn, E = efrom.n;
    int* off = (int*)calloc(N + 1, sizeof(int));        /* out-edges by source */
    int* eidx = (int*)malloc(sizeof(int) * (E ? E : 1));
    int* roff = (int*)calloc(N + 1, sizeof(int));       /* sources by target */
    int* rsrc = (int*)malloc(sizeof(int) * (E ? E : 1));
    for (int e = 0; e < E; ++e) { off[efrom.a[e] + 1]++; roff[eto.a[e] + 1]++; }
    for (int u = 0; u < N; ++u) { off[u + 1] += off[u]; roff[u + 1] += roff[u]; }
    {
      int* f1 = (int*)calloc(N + 1, sizeof(int));
      int* f2 = (int*)calloc(N + 1, sizeof(int));
      for (int e = 0; e < E; ++e) {
        eidx[off[efrom.a[e]] + f1[efrom.a[e]]++] = e;
        rsrc[roff[eto.a[e]] + f2[eto.a[e]]++] = efrom.a[e];
      }
      free(f1); free(f2);
    }
    Fed* W = (Fed*)malloc(sizeof(Fed) * N);
    Fed* ST = (Fed*)malloc(sizeof(Fed) * N);
    char* whole = (char*)calloc(N, 1);
    char* isroot = (char*)calloc(N, 1);
    for (int r = 0; r < roots.n; ++r) isroot[roots.a[r]] = 1;
    for (int u = 0; u < N; ++u) {
      fed_init(&W[u], d2); fed_init(&ST[u], d2);
      fed_push(&W[u], G.zones + (size_t)u * d2);
      if (timed_out || over_time(t0, u)) { timed_out = 1; continue; }
      key_decode(m, nkey[u], locs, ints);
      whole[u] = (char)stop_fed(m, q, locs, ints, G.zones + (size_t)u * d2, qmask, &ST[u]);
    }
    int* queue = (int*)malloc(sizeof(int) * N);
    char* inq = (char*)malloc(N);
    int qh = 0, qn = N;
    for (int u = 0; u < N; ++u) { queue[u] = N - 1 - u; inq[u] = 1; }   /* deepest first */
    int live_roots = roots.n;
    Fed nw;
    fed_init(&nw, d2);
    int32_t Y[64 * 64], X[64 * 64], tl[64], tlI[64];
    char* cov = NULL;
    int covcap = 0;
    Trans* Tp = (Trans*)malloc(sizeof(Trans));
    while (qn > 0 && !timed_out && live_roots > 0) {
      const int v = queue[qh];
      qh = (qh + 1) % N; qn--; inq[v] = 0;
      S0->gfp_iters++;
      if (over_time(t0, (int)S0->gfp_iters)) { timed_out = 1; break; }
      if (W[v].n == 0 || whole[v]) continue;
      key_decode(m, nkey[v], locs, ints);
      nw.n = 0;
      const int nwv = W[v].n;
      if (nwv > covcap) { covcap = nwv * 2; cov = (char*)realloc(cov, covcap); }
      memset(cov, 0, nwv);
      int ncov = 0;
      #define ORC_OFFER(CAND) do { \
          for (int i_ = 0; i_ < nwv; ++i_) { \
            const int32_t* w_ = W[v].z + (size_t)i_ * d2; \
            if (!dbm_intersect(X, w_, (CAND), dim)) continue; \
            if (!cov[i_] && orc_dbm_includes((CAND), w_, dim)) { cov[i_] = 1; ncov++; } \
            fed_add_compact(&nw, X, dim); \
          } } while (0)
      for (int c = 0; c < ST[v].n && ncov < nwv; ++c) ORC_OFFER(ST[v].z + (size_t)c * d2);
      for (int k = off[v]; k < off[v + 1] && ncov < nwv; ++k) {
        const int e = eidx[k], j = eto.a[e];
        if (W[j].n == 0) continue;
        if (!find_trans(m, locs, ints, eraw.a[e], Tp)) continue;
        key_decode(m, nkey[j], tl, tlI);
        for (int y = 0; y < W[j].n && ncov < nwv; ++y) {
          memcpy(Y, W[j].z + (size_t)y * d2, sizeof(int32_t) * d2);
          S0->pre_calls++;
          if (!pre_trans(m, Tp, locs, ints, tl, tlI, qmask, Y)) continue;
          ORC_OFFER(Y);
        }
      }
      #undef ORC_OFFER
      if (ncov == nwv) continue;                       /* every piece survives whole: unchanged */
      int changed = 0;
      for (int i = 0; i < nwv && !changed; ++i)
        if (!cov[i] && !orc_fed_covers(W[v].z + (size_t)i * d2, nw.z, nw.n, dim)) changed = 1;
      if (!changed) continue;
      Fed tmp = W[v]; W[v] = nw; nw = tmp;
      if (isroot[v] && W[v].n == 0) live_roots--;
      for (int k = roff[v]; k < roff[v + 1]; ++k) {
        const int u = rsrc[k];
        if (!inq[u]) { inq[u] = 1; queue[(qh + qn) % N] = u; qn++; }
      }
    }
    for (int r = 0; r < roots.n && !violated && !timed_out; ++r) violated = W[roots.a[r]].n > 0;
    fed_free(&nw);
    free(cov); free(Tp);
    for (int u = 0; u < N; ++u) { fed_free(&W[u]); fed_free(&ST[u]); }
    free(W); free(ST); free(whole); free(isroot); free(queue); free(inq);
    free(off); free(eidx); free(roff); free(rsrc);
  }
  free(nkey); free(efrom.a); free(eto.a); free(eraw.a); free(roots.a); free(front.a);
  store_free(&G);
  if (timed_out) S0->status = HORA_E_TIMEOUT;
  *violated_out = violated;
  return HORA_OK;
}

int32_t orc_leads_to(const hora_net_desc* net, const hora_pred_desc* p, const hora_pred_desc* q,
                     hora_stats* st, int32_t* result) {
  return liveness_core(net, p, q, NULL, st, result);
}

/* E[] psi (exists_invariant_run, include/hora/liveness.hpp:35-46): psi a conjunction of location,
 * integer and clock atoms; holds iff the initial state admits a maximal run whose states all
 * satisfy psi. */
int32_t orc_exists_invariant(const hora_net_desc* net, const hora_pred_desc* psi, hora_stats* st,
                             int32_t* result) {
  return liveness_core(net, NULL, NULL, psi, st, result);
}

/* ---- E[] psi witness replay: the psi-restricted model the E[] route explores ---- */
static int eg_model(const hora_net_desc* net, const hora_pred_desc* psi, Model* m, uint8_t* qmask) {
  int rc = model_build(net, m);
  if (rc) return rc;
  const int dim = m->dim;
  memset(qmask, 0, 64);
  for (int k = 0; k < psi->nclk; ++k) {
    const int i = psi->clk_cond[3 * k], j = psi->clk_cond[3 * k + 1], v = r_bound(psi->clk_cond[3 * k + 2]);
    if (i > 0) qmask[i] = 1;
    if (j > 0) qmask[j] = 1;
    const int a = v < 0 ? -v : v, x = i > 0 ? i : j;
    m->L[x] = imax(m->L[x], a); m->U[x] = imax(m->U[x], a);
  }
  for (int c = 0; c < dim; ++c) m->L[c] = m->U[c] = imax(m->L[c], m->U[c]);
  for (int k = 0; k < m->nlocs_total * dim; ++k) m->Lloc[k] = m->Uloc[k] = imax(m->Lloc[k], m->Uloc[k]);
  m->L[0] = m->U[0] = 0;
  m->avoid = psi;
  m->avoid_psi = 1;
  return HORA_OK;
}

/* Step 0 of an E[] psi witness: the psi-restricted initial state. Returns 1 when it exists. */
int32_t orc_eg_initial(const hora_net_desc* net, const hora_pred_desc* psi, int32_t* locs, int32_t* ints,
                       int32_t* zone) {
  Model m;
  uint8_t qmask[64];
  if (eg_model(net, psi, &m, qmask)) { model_free(&m); return 0; }
  for (int p = 0; p < net->nprocs; ++p) locs[p] = net->proc_init[p];
  for (int v = 0; v < net->nints; ++v) ints[v] = net->int_init[v];
  orc_dbm_init(zone, m.dim);
  const int ok = close_succ_zone(&m, locs, ints, zone, qmask, m.L, m.U, 0) && !orc_dbm_empty(zone, m.dim);
  model_free(&m);
  return ok;
}

/* The successors the E[] psi graph gives a state, in emission order (Extra_M+ under the query's
 * bounds, the psi restriction applied). Writes at most cap of them; *n = their number. */
int32_t orc_eg_successors(const hora_net_desc* net, const hora_pred_desc* psi, const int32_t* locs,
                          const int32_t* ints, const int32_t* zone, int32_t cap, int32_t* out_locs,
                          int32_t* out_ints, int32_t* out_zones, int32_t* n) {
  Model m;
  uint8_t qmask[64];
  int rc = eg_model(net, psi, &m, qmask);
  if (rc) { model_free(&m); return rc; }
  SuccBuf B = {0};
  B.np = net->nprocs; B.ni = net->nints; B.d2 = m.dim * m.dim;
  successors(&m, locs, ints, zone, m.L, m.U, qmask, 1, sb_emit, &B);
  *n = B.n;
  for (int k = 0; k < B.n && k < cap; ++k) {
    memcpy(out_locs + (size_t)k * B.np, B.locs + (size_t)k * B.np, sizeof(int32_t) * B.np);
    if (B.ni) memcpy(out_ints + (size_t)k * B.ni, B.ints + (size_t)k * B.ni, sizeof(int32_t) * B.ni);
    memcpy(out_zones + (size_t)k * B.d2, B.zones + (size_t)k * B.d2, sizeof(int32_t) * B.d2);
  }
  free(B.locs); free(B.ints); free(B.zones); free(B.raw); free(B.parent);
  model_free(&m);
  return HORA_OK;
}
