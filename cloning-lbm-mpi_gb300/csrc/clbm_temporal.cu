// clbm_temporal.cu -- FP32 interval kernel with every clone resident on chip.
//
// One thread-block cluster per clone: the clone's H rows are split into CS
// bands of consecutive rows, given by the launch (an even split, or one
// balanced for the extra cost of the square's rows and the walls), each band
// in one CTA's shared memory (nine floats per node, node after node).  The T steps
// of the interval run without touching HBM except for the drag terms: P_0 is
// loaded once, S_T stored once.
//
// In-place update ("AA" pattern): one buffer A holds, alternately,
//   after a local step:  A[n][opp k] = P(n,k)        (post-collision, own node)
//   after a gather step: A[m][k]     = S_next(m,k)   (streamed, natural order)
// Step t with t even is a gather step: S(n,k) = A[n - c_k][opp k], or on a
// bounced slot A[n][k] (= P(n, opp k)); the collided P(n,k) is pushed to
// A[n + c_k][k], or to A[n][opp k] when slot (n, opp k) bounces back.  Step
// t odd is a local step: S(n,k) = A[n][k], P(n,k) -> A[n][opp k].  In both,
// the nine slots a node reads are exactly the nine it writes and no other
// node touches them, so a step needs no barrier inside; one cluster barrier
// separates steps.  These are the pull rules of clbm_step.cu (the reference's
// collide / push-stream / bounce-back / reset / swap sequence,
// src/mpi_LBM_GK_pops_perturb.cpp:426-443), so results are bit-identical to
// the streaming kernel.  Neighbours across a band edge are read and written
// in the adjacent CTA's shared memory (distributed shared memory).
#include <cooperative_groups.h>

#include <algorithm>

#include "clbm_internal.h"
#include "clbm_physics.cuh"
#include "clbm_reseed.cuh"

namespace cg = cooperative_groups;

namespace clbm {

// Distributed shared memory through 32-bit shared::cluster addresses: the
// address of this CTA's shared-memory offset `a` in the CTA of cluster rank
// `rank`, and FP32 loads / stores at such addresses.
__device__ __forceinline__ unsigned cluster_addr(unsigned a, int rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float ld_cluster(unsigned a) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void st_cluster(unsigned a, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// Geometry of one CTA's band.
struct Band {
  int cs, rank, clone, W, H, rows, row0, nb, rowstep;
  int rows_prev;  // rows of the previous band (its last row lies above this band's row 0)
  float *prev, *next;
  unsigned own_c, prev_c, next_c;  // shared::cluster byte addresses of A in this / previous / next CTA
  long long plane;
  const float *src;
  float *dst;
};

// One node of one step, any position: bounce-back, band edges (distributed
// shared memory), the square, walls.  i = band-local node index.
__device__ __forceinline__ void update_general(const TemporalArgs &a, const Band &b, float *A, int i,
                                               int t, bool gather, bool last, float *terms) {
  const RunDev &R = a.rd;
  const int W = b.W, H = b.H, rows = b.rows, rowstep = b.rowstep;
  const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * W, y = b.row0 + ly;
  const int cm = (x == 0 ? i + W - 1 : i - 1) * 9;
  const int c0 = i * 9;
  const int cp = (x == W - 1 ? i - (W - 1) : i + 1) * 9;
  const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  const int mask = (in_box || y == 0 || y == H - 1) ? bounce_mask(R, x, y) : 0;
  const long long n = (long long)y * W + x;
  if (mask & 512) {  // inside the square
    if (last) {
#pragma unroll
      for (int k = 0; k < 9; k++) b.dst[k * b.plane + n] = 0.0f;
    }
    return;
  }
  float S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    if (!gather || ((mask >> k) & 1)) {
      S[k] = A[c0 + k];
    } else {
      const int cx = cx_of(k), cy = cy_of(k);
      const int sxc = cx == 1 ? cm : (cx == -1 ? cp : c0);  // column, row ly
      const int sl = ly - cy;                                 // source row, band-local
      const float *base = sl < 0 ? b.prev : (sl >= rows ? b.next : A);
      const int roff = sl < 0 ? (b.rows_prev - 1 - ly) * rowstep : (sl >= rows ? -ly * rowstep : -cy * rowstep);
      S[k] = base[sxc + roff + opp_of(k)];
    }
  }
  if (in_box) store_drag_terms<false>(R, S, x, y, b.clone, terms);
  if (last) {
    float d = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      b.dst[k * b.plane + n] = S[k];
      d += S[k];
    }
    if (!(d > -1.0f)) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
    return;
  }
  const float *fm = (R.field_mode && t + 1 < R.field_steps && a.maps)
                        ? a.maps + R.map_base + (long long)b.clone * R.nodes + n
                        : nullptr;
  float P[9];
  const float drho = collide_f32_run(R, S, P, fm, R.f_field_eps);
  if (!(drho > -1.0f)) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int ok = opp_of(k);
    if (!gather || ((mask >> ok) & 1)) {
      A[c0 + ok] = P[k];
    } else {
      const int cx = cx_of(k), cy = cy_of(k);
      const int tx = cx == 1 ? (x == W - 1 ? 0 : x + 1) : (cx == -1 ? (x == 0 ? W - 1 : x - 1) : x);
      const int ty = y + cy;
      if (ty < 0 || ty >= H) continue;
      if (tx > R.xmin && tx < R.xmax && ty > R.ymin && ty < R.ymax) continue;  // into the square
      const int txc = cx == 1 ? cp : (cx == -1 ? cm : c0);
      const int tl = ly + cy;
      float *base = tl < 0 ? b.prev : (tl >= rows ? b.next : A);
      const int roff = tl < 0 ? (b.rows_prev - 1 - ly) * rowstep : (tl >= rows ? -ly * rowstep : cy * rowstep);
      base[txc + roff + k] = P[k];
    }
  }
}

// update_general for a gather step that is not the last: every slot the node
// reads is addressed once (32-bit shared::cluster address: this CTA, or the
// neighbour CTA across a band edge), and P(n,k) goes back to the slot S(n,
// opp k) came from -- the pull rules make the two the same slot (own slot opp
// k when that slot bounces, else (n + c_k, k)) -- unless the target row lies
// outside the channel or the target inside the square (the push is dropped,
// as in update_general).  PLAIN: a node off the walls and the square's box
// (a band-edge row): nothing bounces back and no push is dropped, only the
// neighbour rows may lie in the adjacent CTAs.  LOCAL: the node's row and
// both neighbour rows are in this CTA (1 <= ly <= rows - 2): the same slots
// through plain shared-memory indexing of A, which the compiler schedules
// freely (the shared::cluster accesses are ordered asm).
template <bool PLAIN = false, bool LOCAL = false>
__device__ __forceinline__ void update_general_gather(const TemporalArgs &a, const Band &b, int i, int t,
                                                      bool &bad, float *terms, float *A = nullptr) {
  const RunDev &R = a.rd;
  const int W = b.W, H = b.H, rows = b.rows, rs = b.rowstep;
  const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * W, y = b.row0 + ly;
  const int xm = x == 0 ? W - 1 : x - 1, xp = x == W - 1 ? 0 : x + 1;
  const bool in_box = !PLAIN && x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  const int mask = (!PLAIN && (in_box || y == 0 || y == H - 1)) ? bounce_mask(R, x, y) : 0;
  if (mask & 512) return;  // inside the square
  // byte addresses of column 0 of the rows y-1, y, y+1
  const unsigned rowC = b.own_c + 4u * (unsigned)(ly * rs);
  const unsigned rowU = ly == 0 ? b.prev_c + 4u * (unsigned)((b.rows_prev - 1) * rs) : rowC - 4u * (unsigned)rs;
  const unsigned rowD = ly == rows - 1 ? b.next_c : rowC + 4u * (unsigned)rs;
  const unsigned own = rowC + 36u * (unsigned)x;
  unsigned ad[9];
  float S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    if ((mask >> k) & 1) {
      ad[k] = own + 4u * k;
    } else {  // S(n,k) = A[n - c_k][opp k]
      const int cx = cx_of(k), cy = cy_of(k);
      const int sx = cx == 1 ? xm : (cx == -1 ? xp : x);
      const unsigned row = cy == 1 ? rowU : (cy == -1 ? rowD : rowC);
      ad[k] = row + 36u * (unsigned)sx + 4u * opp_of(k);
    }
    if (LOCAL)
      S[k] = A[(ad[k] - b.own_c) >> 2];
    else
      S[k] = ld_cluster(ad[k]);
  }
  if (in_box) store_drag_terms<false>(R, S, x, y, b.clone, terms);
  const long long n = (long long)y * W + x;
  const float *fm = (R.field_mode && t + 1 < R.field_steps && a.maps)
                        ? a.maps + R.map_base + (long long)b.clone * R.nodes + n
                        : nullptr;
  float P[9];
  const float drho = collide_f32_run(R, S, P, fm, R.f_field_eps);
  bad |= !(drho > -1.0f);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int ok = opp_of(k);
    if (!PLAIN && !((mask >> ok) & 1)) {
      const int cx = cx_of(k), cy = cy_of(k);
      const int tx = cx == 1 ? xp : (cx == -1 ? xm : x);
      const int ty = y + cy;
      if (ty < 0 || ty >= H) continue;
      if (tx > R.xmin && tx < R.xmax && ty > R.ymin && ty < R.ymax) continue;  // into the square
    }
    if (LOCAL)
      A[(ad[ok] - b.own_c) >> 2] = P[k];
    else
      st_cluster(ad[ok], P[k]);
  }
}

// update_general for a local step that is not the last: the node swaps its
// own slots; only the square's box needs more (drag terms, the interior).
__device__ __forceinline__ void update_general_local(const TemporalArgs &a, const Band &b, float *A, int i,
                                                     int t, bool &bad, float *terms) {
  const RunDev &R = a.rd;
  const int W = b.W;
  const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * W, y = b.row0 + ly;
  const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  if (in_box && (bounce_mask(R, x, y) & 512)) return;  // inside the square
  const int c0 = i * 9;
  float S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) S[k] = A[c0 + k];
  if (in_box) store_drag_terms<false>(R, S, x, y, b.clone, terms);
  const long long n = (long long)y * W + x;
  const float *fm = (R.field_mode && t + 1 < R.field_steps && a.maps)
                        ? a.maps + R.map_base + (long long)b.clone * R.nodes + n
                        : nullptr;
  float P[9];
  const float drho = collide_f32_run(R, S, P, fm, R.f_field_eps);
  bad |= !(drho > -1.0f);
#pragma unroll
  for (int k = 0; k < 9; k++) A[c0 + opp_of(k)] = P[k];
}

__device__ __forceinline__ Band make_band(const TemporalArgs &a, float *A, cg::cluster_group &cluster) {
  Band b;
  b.cs = (int)cluster.num_blocks();
  b.rank = (int)cluster.block_rank();
  b.clone = blockIdx.x / b.cs;
  b.W = a.rd.W;
  b.H = a.rd.H;
  b.row0 = a.band_row0[b.rank];
  b.rows = a.band_row0[b.rank + 1] - b.row0;
  b.rows_prev = b.rank > 0 ? b.row0 - a.band_row0[b.rank - 1] : b.rows;
  b.nb = b.rows * b.W;
  b.rowstep = b.W * 9;
  b.prev = b.rank > 0 ? cluster.map_shared_rank(A, b.rank - 1) : A;
  b.next = b.rank + 1 < b.cs ? cluster.map_shared_rank(A, b.rank + 1) : A;
  const unsigned a_cta = (unsigned)__cvta_generic_to_shared(A);
  b.own_c = cluster_addr(a_cta, b.rank);
  b.prev_c = b.rank > 0 ? cluster_addr(a_cta, b.rank - 1) : b.own_c;
  b.next_c = b.rank + 1 < b.cs ? cluster_addr(a_cta, b.rank + 1) : b.own_c;
  b.plane = a.rd.plane;
  const long long cb = a.rd.pop_base + (long long)b.clone * 9 * b.plane;
  b.src = a.src + cb;
  b.dst = a.dst + cb;
  return b;
}

// P_0 into the "after a local step" layout A[node*9 + opp k]
template <int THREADS>
__device__ __forceinline__ void load_band(const Band &b, float *A) {
  for (int i = threadIdx.x; i < b.nb; i += THREADS) {
    const long long n = (long long)b.row0 * b.W + i;
#pragma unroll
    for (int k = 0; k < 9; k++) A[i * 9 + opp_of(k)] = b.src[k * b.plane + n];
  }
}

// P_0 formed here from the previous interval's S (fused reseed: parent copy,
// perturbation, first collision; the same per-node function as the reseed
// kernel, so bit-identical), in the same layout.  Square-interior nodes get
// zeros: their slots are never read before the last step writes them.
template <int THREADS>
__device__ __forceinline__ void load_band_reseed(const TemporalArgs &a, const Band &b, float *A) {
  const RunDev &R = a.rd;
  for (int i = threadIdx.x; i < b.nb; i += THREADS) {
    const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * b.W, y = b.row0 + ly;
    float P[9];
    if (x > R.xmin && x < R.xmax && y > R.ymin && y < R.ymax) {
#pragma unroll
      for (int k = 0; k < 9; k++) P[k] = 0.0f;
    } else {
      reseed_node<false>(a.rs, R, a.run, b.clone, x, y, y * b.W + x, P);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) A[i * 9 + opp_of(k)] = P[k];
  }
}

// One node away from the square, not the last step of the interval.  C, U,
// D = the node's row and the rows above (y-1) and below (y+1); om, o0, op =
// the column offsets of x-1, x, x+1 (times 9).  GATHER: S(n,k) = A[n -
// c_k][opp k], P(n,k) -> A[n + c_k][k]; local step: S(n,k) = A[n][k], P(n,k)
// -> A[n][opp k].  WALL (gather step): 1 = the bottom wall y = 0, whose
// slots 2, 5, 6 bounce back (S(n,k) = A[n][k], and P(n, opp k) returns
// there); 2 = the top wall y = H - 1, slots 4, 7, 8; the row beyond the wall
// is not touched.  FIELD: beta scaled by (1 + feps * map[0]), feps = 0 once
// the field's steps are over (field_beta_f32 then returns beta exactly).  A
// density at or below zero sets `bad`.
template <bool GATHER, bool FIELD, int WALL = 0>
__device__ __forceinline__ void update_fast(const RunDev &R, float *C, float *U, float *D, int om, int o0,
                                            int op, const float *map, float feps, bool &bad) {
  float S[9];
  if (GATHER) {
    S[0] = C[o0 + 0];
    S[1] = C[om + 3];
    S[3] = C[op + 1];
    S[2] = WALL == 1 ? C[o0 + 2] : U[o0 + 4];
    S[5] = WALL == 1 ? C[o0 + 5] : U[om + 7];
    S[6] = WALL == 1 ? C[o0 + 6] : U[op + 8];
    S[4] = WALL == 2 ? C[o0 + 4] : D[o0 + 2];
    S[7] = WALL == 2 ? C[o0 + 7] : D[op + 5];
    S[8] = WALL == 2 ? C[o0 + 8] : D[om + 6];
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) S[k] = C[o0 + k];
  }
  float P[9];
  const float drho = collide_f32_run(R, S, P, FIELD ? map : nullptr, feps);
  bad |= !(drho > -1.0f);
  if (GATHER) {
    C[o0 + 0] = P[0];
    C[op + 1] = P[1];
    C[om + 3] = P[3];
    if (WALL == 2) {
      C[o0 + 4] = P[2];
      C[o0 + 7] = P[5];
      C[o0 + 8] = P[6];
    } else {
      D[o0 + 2] = P[2];
      D[op + 5] = P[5];
      D[om + 6] = P[6];
    }
    if (WALL == 1) {
      C[o0 + 2] = P[4];
      C[o0 + 5] = P[7];
      C[o0 + 6] = P[8];
    } else {
      U[o0 + 4] = P[4];
      U[om + 7] = P[7];
      U[op + 8] = P[8];
    }
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) C[o0 + opp_of(k)] = P[k];
  }
}

// A gather step of one node of a band-edge row (the band holds at least two
// rows): UP, the row above (y - 1) is the previous CTA's last row; else the
// row below (y + 1) is the next CTA's first row.  The remote row's slots are
// read and written at 32-bit shared::cluster addresses (Rc = that row's
// column 0), the node's own row C and the other neighbour row L in this CTA's
// shared memory; same slots and arithmetic as update_fast.
template <bool FIELD, bool UP>
__device__ __forceinline__ void update_edge(const RunDev &R, float *C, float *L, unsigned Rc, int om, int o0,
                                            int op, const float *map, float feps, bool &bad) {
  float S[9];
  S[0] = C[o0 + 0];
  S[1] = C[om + 3];
  S[3] = C[op + 1];
  if (UP) {
    S[4] = L[o0 + 2];
    S[7] = L[op + 5];
    S[8] = L[om + 6];
    S[2] = ld_cluster(Rc + 4u * (o0 + 4));
    S[5] = ld_cluster(Rc + 4u * (om + 7));
    S[6] = ld_cluster(Rc + 4u * (op + 8));
  } else {
    S[2] = L[o0 + 4];
    S[5] = L[om + 7];
    S[6] = L[op + 8];
    S[4] = ld_cluster(Rc + 4u * (o0 + 2));
    S[7] = ld_cluster(Rc + 4u * (op + 5));
    S[8] = ld_cluster(Rc + 4u * (om + 6));
  }
  float P[9];
  const float drho = collide_f32_run(R, S, P, FIELD ? map : nullptr, feps);
  bad |= !(drho > -1.0f);
  C[o0 + 0] = P[0];
  C[op + 1] = P[1];
  C[om + 3] = P[3];
  if (UP) {
    L[o0 + 2] = P[2];
    L[op + 5] = P[5];
    L[om + 6] = P[6];
    st_cluster(Rc + 4u * (o0 + 4), P[4]);
    st_cluster(Rc + 4u * (om + 7), P[7]);
    st_cluster(Rc + 4u * (op + 8), P[8]);
  } else {
    L[o0 + 4] = P[4];
    L[om + 7] = P[7];
    L[op + 8] = P[8];
    st_cluster(Rc + 4u * (o0 + 2), P[2]);
    st_cluster(Rc + 4u * (op + 5), P[5]);
    st_cluster(Rc + 4u * (om + 6), P[6]);
  }
}

__device__ __forceinline__ float field_eps(const TemporalArgs &a, int t) {
  return t + 1 < a.rd.field_steps ? a.rd.f_field_eps : 0.0f;
}

// Shared memory of one CTA: the band's populations, then the segment list,
// one class byte per 32-node segment and the five range ends of the list.
__host__ __device__ inline size_t temporal_smem(int nb) {
  const int nseg = (nb + 31) / 32;
  return sizeof(float) * 9 * (size_t)nb + 2 * (size_t)((nseg + 7) & ~7) + (size_t)((nseg + 15) & ~15) + 32;
}

// One step of every segment of the band (all but the interval's last step).
// The list holds the segments by class, in this order: the square's box (and
// a partial last segment, and wall or band-edge segments that span two rows
// at a wall), the wall rows, the band-edge rows, other segments spanning two
// rows at a band edge, the bulk segments with the periodic wrap and the
// interior bulk segments; range[c] = the end of the c-th range, and entry k
// of every range belongs to warp k % NW.  Gather step: the box range through
// the general path; wall rows through update_fast with the wall's bounce-back
// built in; band-edge rows with the neighbour row across the band edge at
// shared::cluster addresses and the rest in this CTA; rows spanning a band
// edge through the plain form of the general path (no bounce-back, every
// slot at a shared::cluster address); wrap segments with per-node column
// offsets; interior segments with their nine slots at constant offsets from
// the node's own (-9 / +9 floats for x -+ 1, -+ rowstep for y -+ 1).  Local
// step: a node touches only its own nine slots, so only the box range (drag
// terms, the interior) needs the general path.
// LOCAL_BOX: box segments whose rows all lie inside the band take the
// general gather through plain shared-memory indexing (compiled into the
// uniform-force kernels only: in the random-field ones it raised register
// spills).
template <int NW, bool GATHER, bool FIELD, bool LOCAL_BOX>
__device__ __forceinline__ void band_step(const TemporalArgs &a, const Band &b, float *A,
                                          const unsigned short *list, int nseg, const int *range,
                                          int warp, int lane, int t, const float *map, bool &bad) {
  const RunDev &R = a.rd;
  const float feps = FIELD ? field_eps(a, t) : 0.0f;
  float *terms = a.terms + (long long)t * a.term_slab + R.term_base;
  const int ngen = range[0];
  for (int k = warp; k < ngen; k += NW) {
    const int i = list[k] * 32 + lane;
    const int ly = (int)__umulhi((unsigned)i, R.div_w);
    const bool inner = LOCAL_BOX && __all_sync(0xffffffffu, i < b.nb && ly >= 1 && ly <= b.rows - 2);
    if (i >= b.nb) continue;
    if (GATHER) {
      if (inner)
        update_general_gather<false, true>(a, b, i, t, bad, terms, A);
      else
        update_general_gather(a, b, i, t, bad, terms);
    } else {
      update_general_local(a, b, A, i, t, bad, terms);
    }
  }
  if (!GATHER) {
    for (int k = ngen + ((warp - ngen) & (NW - 1)); k < nseg; k += NW) {
      const int i = list[k] * 32 + lane;
      float *C = A + i * 9;
      update_fast<false, FIELD>(R, C, C, C, 0, 0, 0, map + i, feps, bad);
    }
    return;
  }
  const int rs = b.rowstep;
  const int nwall = range[1], nedge = range[2], nspan = range[3], nwrap = range[4];
  for (int k = ngen + ((warp - ngen) & (NW - 1)); k < nwall; k += NW) {
    const int i = list[k] * 32 + lane;
    const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * b.W;
    const int o0 = x * 9, om = (x == 0 ? b.W - 1 : x - 1) * 9, op = (x == b.W - 1 ? 0 : x + 1) * 9;
    float *C = A + ly * rs;
    if (b.row0 + ly == 0)  // warp-uniform: a wall segment lies in one row
      update_fast<true, FIELD, 1>(R, C, C - rs, C + rs, om, o0, op, map + i, feps, bad);
    else
      update_fast<true, FIELD, 2>(R, C, C - rs, C + rs, om, o0, op, map + i, feps, bad);
  }
  for (int k = nwall + ((warp - nwall) & (NW - 1)); k < nedge; k += NW) {
    const int i = list[k] * 32 + lane;
    const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * b.W;
    const int o0 = x * 9, om = (x == 0 ? b.W - 1 : x - 1) * 9, op = (x == b.W - 1 ? 0 : x + 1) * 9;
    float *C = A + ly * rs;
    if (ly == 0)  // warp-uniform: an edge segment lies in one row
      update_edge<FIELD, true>(R, C, C + rs, b.prev_c + 4u * (unsigned)((b.rows_prev - 1) * rs), om, o0, op,
                               map + i, feps, bad);
    else
      update_edge<FIELD, false>(R, C, C - rs, b.next_c, om, o0, op, map + i, feps, bad);
  }
  for (int k = nedge + ((warp - nedge) & (NW - 1)); k < nspan; k += NW)
    update_general_gather<true>(a, b, list[k] * 32 + lane, t, bad, terms);
  for (int k = nspan + ((warp - nspan) & (NW - 1)); k < nwrap; k += NW) {
    const int i = list[k] * 32 + lane;
    const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * b.W;
    const int o0 = x * 9, om = (x == 0 ? b.W - 1 : x - 1) * 9, op = (x == b.W - 1 ? 0 : x + 1) * 9;
    float *C = A + ly * rs;
    update_fast<true, FIELD>(R, C, C - rs, C + rs, om, o0, op, map + i, feps, bad);
  }
  for (int k = nwrap + ((warp - nwrap) & (NW - 1)); k < nseg; k += NW) {
    const int i = list[k] * 32 + lane;
    float *C = A + i * 9;
    update_fast<true, FIELD>(R, C, C - rs, C + rs, -9, 0, 9, map + i, feps, bad);
  }
}

// Generic kernel: any W.  The band's nodes form 32-node segments; segments
// that cost more than a bulk segment (the square's box on the general path,
// then walls and band edges) are dealt out first, one per warp, and the bulk
// segments fill in after them: entry k of the list goes to warp k % NW.  The
// step time is that of the slowest warp (every step ends at a cluster
// barrier), which this keeps near the mean.  (Measured on a 256x64 channel,
// all slower than this: band-edge and wall rows through generic
// distributed-shared-memory pointers, a cost-weighted water-filling of the
// bulk segments over the warps, a fixed column per thread with compile-time
// shared-memory offsets, segments taken from a shared counter in one
// dispatch loop, the band geometry in shared memory.)
template <int THREADS, int MINB, bool FIELD>
__global__ void __launch_bounds__(THREADS, MINB) k_temporal_f32(TemporalArgs a) {
  // A[node * 9 + k]: a node's nine values together (stride 9 words: no bank
  // conflicts across a warp), so every access is a base register plus an
  // immediate offset
  extern __shared__ float A[];
  constexpr int NW = THREADS / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const Band b = make_band(a, A, cluster);
  const RunDev &R = a.rd;
  // (the fused load is compiled into the uniform-force kernels only: in the
  // random-field ones it raised register spills in the step loop)
  if (!FIELD && a.fused)
    load_band_reseed<THREADS>(a, b, A);
  else
    load_band<THREADS>(b, A);
  const int nseg = (b.nb + 31) / 32;
  unsigned short *list = (unsigned short *)(A + (size_t)9 * b.nb);
  unsigned char *cls = (unsigned char *)(list + ((nseg + 7) & ~7));
  int *count_s = (int *)(cls + ((nseg + 15) & ~15));
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  // segment classes: 5 touches the square's box, or past the band's end
  // (partial last segment), or a wall row that is not alone in its segment or
  // in its band; 4 a wall row (its neighbour row in this CTA); 3 a band-edge
  // row (neighbour row in another CTA, the other in this one); 2 other
  // segments touching a band-edge row (spanning two rows, or a one-row band);
  // 1 bulk with the periodic wrap; 0 interior bulk
  for (int sg = warp; sg < nseg; sg += NW) {
    const int i = sg * 32 + lane;
    const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * b.W, y = b.row0 + ly;
    const bool pad = i >= b.nb;
    const bool box = !pad && x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
    const bool wall = !pad && (y == 0 || y == b.H - 1);
    const bool edge = !pad && b.cs > 1 && (ly == 0 || ly == b.rows - 1);
    // (every lane takes part in the shuffle: it is not under the && below)
    const int ly0 = __shfl_sync(0xffffffffu, ly, 0);
    const bool one_row = __all_sync(0xffffffffu, !pad && ly == ly0) && b.rows > 1;
    const bool inner = __all_sync(0xffffffffu, !pad && x > 0 && x < b.W - 1);
    int c;
    if (__any_sync(0xffffffffu, box || pad))
      c = 5;
    else if (__any_sync(0xffffffffu, wall))
      c = one_row ? 4 : 5;
    else if (__any_sync(0xffffffffu, edge))
      c = one_row ? 3 : 2;
    else
      c = inner ? 0 : 1;
    if (lane == 0) cls[sg] = (unsigned char)c;
  }
  __syncthreads();
  if (warp == 0) {  // the list, class 5 first; range ends after classes 5, 4, 3, 2, 1
    const unsigned lower = (1u << lane) - 1u;
    int n = 0;
    for (int pass = 5; pass >= 0; pass--) {
      for (int c = 0; c < nseg; c += 32) {
        const bool take = c + lane < nseg && cls[c + lane] == pass;
        const unsigned m = __ballot_sync(0xffffffffu, take);
        if (take) list[n + __popc(m & lower)] = (unsigned short)(c + lane);
        n += __popc(m);
      }
      if (lane == 0 && pass >= 1) count_s[5 - pass] = n;
    }
  }
  __syncthreads();
  const int *range = count_s;  // read at each loop start: five registers fewer held across the steps
  const float *map = FIELD ? a.maps + R.map_base + (long long)b.clone * R.nodes + (long long)b.row0 * b.W : nullptr;
  bool bad = false;
  cluster.sync();
  // every step but the last
  // (steps past the field's run through the uniform-force path: with eps = 0
  // the field path computes the same beta and constants bit for bit)
  for (int t = 0; t + 1 < a.steps; t++) {
    const bool field = FIELD && t + 1 < R.field_steps;
    if ((t & 1) == 0) {
      if (field)
        band_step<NW, true, FIELD, !FIELD>(a, b, A, list, nseg, range, warp, lane, t, map, bad);
      else
        band_step<NW, true, false, !FIELD>(a, b, A, list, nseg, range, warp, lane, t, map, bad);
    } else {
      if (field)
        band_step<NW, false, FIELD, !FIELD>(a, b, A, list, nseg, range, warp, lane, t, map, bad);
      else
        band_step<NW, false, false, !FIELD>(a, b, A, list, nseg, range, warp, lane, t, map, bad);
    }
    cluster.sync();
  }
  // the last step stores S_T (one step in T: every node through update_general)
  {
    const int t = a.steps - 1;
    float *terms = a.terms + (long long)t * a.term_slab + R.term_base;
    for (int i = threadIdx.x; i < b.nb; i += THREADS) update_general(a, b, A, i, t, (t & 1) == 0, true, terms);
  }
  if (bad) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
  cluster.sync();  // no CTA leaves while a neighbour may still read its shared memory
}

typedef void (*TemporalFn)(TemporalArgs);

// shared memory a CTA may use
static constexpr size_t kSmemLimit = 227 * 1024;

int temporal_rows_limit(int W) {
  int r = 0;
  while (temporal_smem((r + 1) * W) <= kSmemLimit) r++;
  return r;
}

struct TemporalVariant {
  int threads;
  TemporalFn fn[2];  // [field]
};

#define GENERIC(T, M) {k_temporal_f32<T, M, false>, k_temporal_f32<T, M, true>}
static const TemporalVariant kTemporal[] = {{1024, GENERIC(1024, 1)}, {512, GENERIC(512, 2)}, {256, GENERIC(256, 4)}};
#undef GENERIC

int temporal_variant_count() { return (int)(sizeof(kTemporal) / sizeof(kTemporal[0])); }

// the kernel of a variant for this band shape, or nullptr when it cannot run it
static TemporalFn temporal_fn(int variant, int cs, int W, int rows_max, bool field) {
  if (variant < 0 || variant >= temporal_variant_count() || cs < 1 || cs > MAX_CLUSTER || rows_max < 1)
    return nullptr;
  if (temporal_smem(rows_max * W) > kSmemLimit) return nullptr;
  return kTemporal[variant].fn[field];
}

static cudaLaunchConfig_t temporal_config(int cs, int variant, int nclones, size_t smem, cudaStream_t s,
                                          cudaLaunchAttribute *attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs * nclones);
  cfg.blockDim = dim3(kTemporal[variant].threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

static cudaError_t prepare(TemporalFn fn, int cs, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && cs > 8) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

// Launch one run's interval with cluster size cs over the bands of
// a.band_row0 (every band at least one row).
cudaError_t launch_temporal(const TemporalArgs &a, int cs, int variant, int nclones, int W,
                            cudaStream_t s) {
  const bool field = a.rd.field_mode != 0 && a.maps != nullptr;
  if (cs < 1 || cs > MAX_CLUSTER || a.band_row0[0] != 0 || a.band_row0[cs] != a.rd.H)
    return cudaErrorInvalidConfiguration;
  int rows_max = 0;
  for (int b = 0; b < cs; b++) {
    const int rows = a.band_row0[b + 1] - a.band_row0[b];
    if (rows < 1) return cudaErrorInvalidConfiguration;
    rows_max = std::max(rows_max, rows);
  }
  TemporalFn fn = temporal_fn(variant, cs, W, rows_max, field);
  if (!fn || a.steps < 1) return cudaErrorInvalidConfiguration;
  const size_t smem = temporal_smem(rows_max * W);
  cudaError_t e = prepare(fn, cs, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = temporal_config(cs, variant, nclones, smem, s, attr);
  return cudaLaunchKernelEx(&cfg, fn, a);
}

// Whether the cluster shape can be resident at all (occupancy query, no launch).
int temporal_max_clusters(int cs, int variant, int W, int rows_max, bool field) {
  TemporalFn fn = temporal_fn(variant, cs, W, rows_max, field);
  if (!fn) return 0;
  const size_t smem = temporal_smem(rows_max * W);
  if (prepare(fn, cs, smem) != cudaSuccess) return 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = temporal_config(cs, variant, 64, smem, nullptr, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (void *)fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace clbm
