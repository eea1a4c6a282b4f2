// dbm_tile.cuh -- difference-bound matrices held row-per-lane in a tile of D lanes.
//
// One zone of dimension D (clocks + reference clock) lives in D consecutive lanes of a warp: lane
// i of the tile holds row i, `x_i - x_j <| r[j]`, in registers. A warp carries floor(32/D) tiles,
// i.e. several zones at once for small D. Row broadcasts go through __shfl_sync on the tile's own
// lane mask, so tiles of one warp may follow different control flow. Every branch below that a
// tile takes is tile-uniform: its condition is either a broadcast value or a ballot.
//
// Raw bound encoding (HDBM's, src/metal/netengine_metal.mm:76-100): r = (bound << 1) | weak,
// kInf = 1 << 30 for "no bound". The arithmetic is the same integer algebra as the reference's
// dbm_ops, so every canonical zone produced here is bit-identical to the reference's.
#pragma once
#include <cstdint>

namespace hgb {

constexpr int kInf = 1 << 30;
constexpr int kZeroLe = 1;
constexpr int kAluNegInf = -(1 << 29);

__device__ __forceinline__ int r_le(int v) { return (int)((unsigned)v << 1) | 1; }
__device__ __forceinline__ int r_lt(int v) { return (int)((unsigned)v << 1); }
__device__ __forceinline__ int r_bound(int r) { return r >> 1; }
// Sum of two bounds: values add, the result is weak iff both are weak; infinity absorbs.
__device__ __forceinline__ int r_add(int a, int b) {
  const int s = (int)((unsigned)a + (unsigned)b - (unsigned)((a | b) & 1));
  return (a >= kInf || b >= kInf) ? kInf : s;
}
// Complement of x_i - x_j <| v, written as x_j - x_i <|' -v.
__device__ __forceinline__ int r_negate(int r) {
  const int v = r_bound(r);
  return (r & 1) ? r_lt(-v) : r_le(-v);
}

template <int D>
struct Tile {
  unsigned mask;  // this tile's lanes
  int base;       // first lane of the tile
  int i;          // row held by this lane
  __device__ __forceinline__ int shfl(int v, int src) const { return __shfl_sync(mask, v, base + src); }
  __device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) const {
    return __shfl_sync(mask, v, base + src);
  }
  __device__ __forceinline__ bool any(bool p) const { return (__ballot_sync(mask, p) & mask) != 0; }
  __device__ __forceinline__ bool all(bool p) const { return (__ballot_sync(mask, p) & mask) == mask; }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
};

// Compute the tile a lane belongs to; returns false for the lanes left over past the last tile.
template <int D>
__device__ __forceinline__ bool make_tile(Tile<D>& t, int lane) {
  constexpr int TPW = 32 / D;
  const int k = lane / D;
  if (k >= TPW) return false;
  t.base = k * D;
  t.i = lane - t.base;
  t.mask = (D == 32 ? 0xffffffffu : ((1u << D) - 1u)) << t.base;
  return true;
}

// r[k] for a runtime k, without dynamic register indexing.
template <int D>
__device__ __forceinline__ int sel(const int (&r)[D], int k) {
  int v = r[0];
#pragma unroll
  for (int j = 1; j < D; ++j) v = (j == k) ? r[j] : v;
  return v;
}
template <int D>
__device__ __forceinline__ void put(int (&r)[D], int k, int v) {
#pragma unroll
  for (int j = 0; j < D; ++j) r[j] = (j == k) ? v : r[j];
}

template <int D>
__device__ __forceinline__ void load_rows(const Tile<D>& t, int (&r)[D], const int* z) {
  const int* row = z + t.i * D;
#pragma unroll
  for (int j = 0; j < D; ++j) r[j] = __ldg(row + j);
}
// Plain (coherent) load, for zones written earlier in the same kernel.
template <int D>
__device__ __forceinline__ void load_rows_rw(const Tile<D>& t, int (&r)[D], const int* z) {
  const volatile int* row = z + t.i * D;
#pragma unroll
  for (int j = 0; j < D; ++j) r[j] = row[j];
}
template <int D>
__device__ __forceinline__ void store_rows(const Tile<D>& t, const int (&r)[D], int* z) {
  int* row = z + t.i * D;
#pragma unroll
  for (int j = 0; j < D; ++j) row[j] = r[j];
}

// d[a][b], the same value on every lane of the tile.
template <int D>
__device__ __forceinline__ int get(const Tile<D>& t, const int (&r)[D], int a, int b) {
  return t.shfl(sel(r, b), a);
}

template <int D>
__device__ __forceinline__ bool is_empty(const Tile<D>& t, const int (&r)[D]) {
  return t.any(sel(r, t.i) < kZeroLe);
}

// Origin zone: every clock equal to 0.
template <int D>
__device__ __forceinline__ void init_zero(int (&r)[D]) {
#pragma unroll
  for (int j = 0; j < D; ++j) r[j] = kZeroLe;
}

// Tighten x_a - x_b to `raw` and re-close (dbm_constrain). The input must be canonical and
// non-empty. With one new edge (a,b) on a closed graph every new shortest path is
// d[i][a] + raw + d[b][j], so one O(D) pass per lane closes it. Returns false iff the zone empties.
template <int D>
__device__ __forceinline__ bool constrain(const Tile<D>& t, int (&r)[D], int a, int b, int raw) {
  const int dab = get(t, r, a, b);
  if (raw >= dab) return true;                 // no-op: the zone is unchanged, hence non-empty
  const int via = r_add(sel(r, a), raw);        // d[i][a] + raw
  int rb[D];
#pragma unroll
  for (int j = 0; j < D; ++j) rb[j] = t.shfl(r[j], b);   // row b
#pragma unroll
  for (int j = 0; j < D; ++j) {
    const int s = r_add(via, rb[j]);
    r[j] = s < r[j] ? s : r[j];
  }
  return !is_empty(t, r);
}

// x_k := 0 (dbm_reset): row k becomes row 0, column k becomes column 0.
template <int D>
__device__ __forceinline__ void reset(const Tile<D>& t, int (&r)[D], int k) {
  int r0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) r0[j] = t.shfl(r[j], 0);
  if (t.i == k) {
#pragma unroll
    for (int j = 0; j < D; ++j) r[j] = (j == k) ? kZeroLe : r0[j];
  } else {
    put(r, k, r[0]);
  }
}

// Let time pass (dbm_delay): drop every upper bound.
template <int D>
__device__ __forceinline__ void delay(const Tile<D>& t, int (&r)[D]) {
  if (t.i >= 1) r[0] = kInf;
}

// Full Floyd-Warshall closure (dbm_close), one broadcast row per pivot.
template <int D>
__device__ __forceinline__ void close(const Tile<D>& t, int (&r)[D]) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int ik = r[k];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const int kj = t.shfl(r[j], k);
      const int s = r_add(ik, kj);
      r[j] = s < r[j] ? s : r[j];
    }
  }
}

// Time predecessor (dbm_down): every lower bound relaxes to the tightest bound any clock
// difference still imposes on it, and never past zero.
template <int D>
__device__ __forceinline__ void down(const Tile<D>& t, int (&r)[D]) {
  int m[D];
#pragma unroll
  for (int j = 0; j < D; ++j) m[j] = kZeroLe;
#pragma unroll
  for (int i = 1; i < D; ++i) {
#pragma unroll
    for (int j = 1; j < D; ++j) {
      const int v = t.shfl(r[j], i);
      m[j] = v < m[j] ? v : m[j];
    }
  }
  if (t.i == 0) {
#pragma unroll
    for (int j = 1; j < D; ++j) r[j] = m[j];
  }
}

// Quantify clock k out (dbm_free): k becomes any non-negative value.
template <int D>
__device__ __forceinline__ void free_clock(const Tile<D>& t, int (&r)[D], int k) {
  if (t.i == k) {
#pragma unroll
    for (int j = 0; j < D; ++j) r[j] = (j == k) ? kZeroLe : kInf;
  } else {
    put(r, k, r[0]);
  }
}

// Extra_LU+ then close (engine_metal.mm:80-93). L and U hold the per-clock bounds, indexable
// by any lane (device memory, or a per-lane register copy through lu_of below).
template <int D>
__device__ __forceinline__ void extrap_lu_plus(const Tile<D>& t, int (&r)[D], const int* L, const int* U) {
  int r0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) r0[j] = t.shfl(r[j], 0);
  const int i = t.i;
  const int Li = L[i];
  const int mine0 = sel(r0, i);
#pragma unroll
  for (int j = 0; j < D; ++j) {
    if (j == i) continue;
    const int e = r[j];
    if (e >= kInf) continue;
    const int Uj = U[j];
    int v = e;
    if (r_bound(e) > Li) v = kInf;
    else if (-r_bound(mine0) > Li) v = kInf;
    else if (i != 0 && -r_bound(r0[j]) > Uj) v = kInf;
    else if (e < r_lt(-Uj)) v = r_lt(-Uj);
    r[j] = v;
  }
  close(t, r);
}

// a ⊇ b, where this lane holds row i of both.
template <int D>
__device__ __forceinline__ bool includes(const Tile<D>& t, const int (&a)[D], const int (&b)[D]) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < D; ++j) ok &= (b[j] <= a[j]);
  return t.all(ok);
}

// Z ≼_aLU Zp (dbm_is_alu_le; netengine_metal.mm:240-252), with z0 = row 0 of Z on every lane,
// Ly = L[i] for this lane's row and U[] the per-clock upper bounds on every lane.
template <int D>
__device__ __forceinline__ bool alu_le(const Tile<D>& t, const int (&z)[D], const int (&zp)[D],
                                       const int (&z0)[D], int Ly, const int (&U)[D]) {
  bool witness = false;
  if (Ly != kAluNegInf) {
    const int ly = r_lt(-Ly);
#pragma unroll
    for (int x = 0; x < D; ++x) {
      if (x == t.i) continue;
      if (U[x] == kAluNegInf) continue;
      if (z0[x] < r_le(-U[x])) continue;
      witness |= (zp[x] < z[x]) && (r_add(zp[x], ly) < z0[x]);
    }
  }
  return !t.any(witness);
}

// Z ≼_aLU Zp decided by ONE lane from whole matrices in global memory (row-major D*D, read through
// L2 so zones another lane of the tile just wrote are seen), with the per-clock bounds L[] and U[]
// in registers: the same test as alu_le, used where a tile spreads several stored zones over its
// lanes instead of one zone over its rows.
template <int D>
__device__ __forceinline__ bool alu_le_lane(const int* Z, const int* Zp, const int (&L)[D], const int (&U)[D]) {
#pragma unroll
  for (int x = 0; x < D; ++x) {
    if (U[x] == kAluNegInf) continue;
    const int z0x = __ldcg(Z + x);
    if (z0x < r_le(-U[x])) continue;
#pragma unroll
    for (int y = 0; y < D; ++y) {
      if (y == x || L[y] == kAluNegInf) continue;
      const int zp = __ldcg(Zp + y * D + x);
      if (zp < __ldcg(Z + y * D + x) && r_add(zp, r_lt(-L[y])) < z0x) return false;
    }
  }
  return true;
}

// True if column 0 alone shows Z is not simulated by Zp (the x = 0 case of the a_LU test, which
// decides most failing tests): some clock y has Zp[y][0] < Z[y][0] and Zp[y][0] - L_y < Z[0][0].
template <int D>
__device__ __forceinline__ bool alu_col0_witness(const int (&zc0)[D], const int* zpc0, const int (&L)[D]) {
  bool w = false;
#pragma unroll
  for (int y = 1; y < D; ++y) {
    if (L[y] == kAluNegInf) continue;
    const int zp = __ldg(zpc0 + y);
    w |= zp < zc0[y] && r_add(zp, r_lt(-L[y])) < zc0[0];
  }
  return w;
}

// Necessary condition for a convex union, from the clock bounds alone (netengine_metal.mm:455-465):
// if the projections of a and b on some clock are separated by a gap, a ∪ b is not convex.
template <int D>
__device__ __forceinline__ bool union_axis_gap(const Tile<D>& t, const int (&a)[D], const int (&b)[D]) {
  const int i = t.i;
  int a0[D], b0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) { a0[j] = t.shfl(a[j], 0); b0[j] = t.shfl(b[j], 0); }
  const int a0i = sel(a0, i), b0i = sel(b0, i);   // row 0 entry i: minus the lower bound of clock i
  bool gap = false;
  if (i > 0) {
    if (b[0] < kInf && a0i < kInf && -r_bound(a0i) > r_bound(b[0])) gap = true;
    if (a[0] < kInf && b0i < kInf && -r_bound(b0i) > r_bound(a[0])) gap = true;
  }
  return t.any(gap);
}

// One half of the exact convex-union test: does every region the hull h gains past one of z's
// constraints lie inside `other`?
template <int D>
__device__ __forceinline__ bool facets_inside(const Tile<D>& t, const int (&z)[D], const int (&other)[D],
                                              const int (&h)[D]) {
  unsigned m = 0;   // bit j: z[i][j] < h[i][j] on this lane's row i
#pragma unroll
  for (int j = 0; j < D; ++j)
    if (j != t.i && z[j] < h[j]) m |= 1u << j;
#pragma unroll 1
  for (int i = 0; i < D; ++i) {
    unsigned mi = (unsigned)t.shfl((int)m, i);
    while (mi) {
      const int j = __ffs(mi) - 1;
      mi &= mi - 1;
      int rr[D];
#pragma unroll
      for (int k = 0; k < D; ++k) rr[k] = h[k];
      const int zij = t.shfl(sel(z, j), i);
      if (!constrain(t, rr, j, i, r_negate(zij))) continue;   // crossing region empty
      bool inc = true;
#pragma unroll
      for (int k = 0; k < D; ++k) inc &= rr[k] <= other[k];
      if (!t.all(inc)) return false;
    }
  }
  return true;
}

// Exact convex union (dbm_try_union; netengine_metal.mm:310-335): a ∪ b is convex iff the hull
// h (entrywise max) holds no point outside both. facets_inside(a, b, h) decides exactly whether
// h \ a ⊆ b -- the part of h past a's loosened constraints is the union of the crossing regions it
// tests -- and h \ a ⊆ b, h ⊆ a ∪ b and h \ b ⊆ a are the same statement. The reference also
// tests the swapped direction, which can only agree; it is left out (the same answer, half the
// closures on a success). On success `a` becomes the hull (the entrywise max of two canonical
// DBMs is canonical).
template <int D>
__device__ __forceinline__ bool try_union(const Tile<D>& t, int (&a)[D], const int (&b)[D]) {
  if (union_axis_gap(t, a, b)) return false;
  int h[D];
#pragma unroll
  for (int j = 0; j < D; ++j) h[j] = a[j] > b[j] ? a[j] : b[j];
  if (!facets_inside(t, a, b, h)) return false;
#pragma unroll
  for (int j = 0; j < D; ++j) a[j] = h[j];
  return true;
}

// Non-empty intersection of two canonical zones: entrywise min, closed, diagonal non-negative.
template <int D>
__device__ __forceinline__ bool intersects(const Tile<D>& t, const int (&a)[D], const int (&b)[D]) {
  int m[D];
#pragma unroll
  for (int j = 0; j < D; ++j) m[j] = a[j] < b[j] ? a[j] : b[j];
  close(t, m);
  return !is_empty(t, m);
}

}  // namespace hgb
