/*
 * clbm_oracle.c -- CPU restatement of the reference cloning-LBM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, by the smoke
 * entry point and by bench.py's CPU-baseline leg; the product library never
 * links or calls anything here.
 *
 * Compile with -ffp-contract=off: every FP64 expression below is written in
 * the reference's evaluation order, and a fused multiply-add would change the
 * rounding (GCC contracts by default on aarch64).
 *
 * Parity is pinned against the reference objects compiled in place
 * (oracle/Makefile -> oracle/_ref) by tests/test_oracle_vs_reference.py and
 * against the committed fixtures in tests/golden/.
 */
#include "clbm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* D2Q9 lattice: src/mpi_LBM_GK_pops_perturb.cpp:31-32, opposite map
 * src/lbm_src/square.cpp:8 */
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const double WK[9] = {4.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,
                             1.0 / 9.0,  1.0 / 9.0,  1.0 / 36.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
static const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

#define AOS(g, x, y, k) ((k) + 9 * ((y) + (g)->ny * (x)))
#define NODE(g, x, y) ((y) + (g)->ny * (x))

/* ------------------------------------------------------------------------ */
/* Stream-collide, uniform or spatial body force.
 * Follows src/lbm_src/streamCollCompute.cpp:7-48 (uniform) and :50-93
 * (spatial beta = (1 + eps*map)*beta0, :63): moments of fin, velocity shifted
 * by half the force (:28), BGK relaxation plus the forcing term written back
 * into fin (:34-37), push to the periodic neighbour (:39-40), and the
 * pre-streaming macroscopic fields (:44-45). */
static void stream_collide_impl(const orc_geom *g, double *fin, double *fout,
                                double *rho, double *ux, double *uy,
                                double beta0, const double *map, double tau,
                                double eps) {
  const double omega = 1. / tau;
  const double om1 = 1.0 - omega;
  const double cforce = 1.0 - 0.5 * omega;
  for (int x = 0; x < g->nx; x++) {
    for (int y = 0; y < g->ny; y++) {
      double beta = beta0;
      if (map) beta = (1.0 + eps * map[NODE(g, x, y)]) * beta0;
      double r = 0.0, jx = 0.0, jy = 0.0;
      for (int k = 0; k < 9; k++) {
        double f = fin[AOS(g, x, y, k)];
        r += f;
        jx += f * (double)CX[k];
        jy += f * (double)CY[k];
      }
      double vx = jx / r + 0.5 * beta / r;
      double vy = jy / r;
      double u2 = -1.5 * (vx * vx + vy * vy);
      for (int k = 0; k < 9; k++) {
        double cx = (double)CX[k], cy = (double)CY[k];
        double eu = cx * vx + cy * vy;
        double eueu = 4.5 * eu * eu;
        double feq = WK[k] * r * (1.0 + 3.0 * eu + eueu + u2);
        double drive = WK[k] * cforce * beta * (3. * (cx - vx) + 9. * cx * eu);
        double post = fin[AOS(g, x, y, k)] * om1 + feq * omega + drive;
        fin[AOS(g, x, y, k)] = post;
        int tx = (x + CX[k] + g->nx) % g->nx;
        int ty = (y + CY[k] + g->ny) % g->ny;
        fout[AOS(g, tx, ty, k)] = post;
      }
      if (ux) ux[NODE(g, x, y)] = vx;
      if (uy) uy[NODE(g, x, y)] = vy;
      if (rho) rho[NODE(g, x, y)] = r;
    }
  }
}

void orc_stream_collide(const orc_geom *g, double *fin, double *fout,
                        double *rho, double *ux, double *uy, double beta,
                        double tau) {
  stream_collide_impl(g, fin, fout, rho, ux, uy, beta, NULL, tau, 0.0);
}

void orc_stream_collide_spatial(const orc_geom *g, double *fin, double *fout,
                                double *rho, double *ux, double *uy,
                                double beta0, const double *map, double tau,
                                double eps) {
  stream_collide_impl(g, fin, fout, rho, ux, uy, beta0, map, tau, eps);
}

/* Half-way bounce-back on the channel walls y = 0 and y = Dy-1: the slots
 * pointing back into the fluid take the node's own post-collision opposite
 * population (src/lbm_src/domain_noSlipWalls.cpp:6-22). */
void orc_walls_bb(const orc_geom *g, double *fout, const double *fin) {
  const int top = g->ny - 1;
  static const int up[3] = {2, 5, 6};   /* cy = +1 */
  static const int down[3] = {4, 7, 8}; /* cy = -1 */
  for (int x = 0; x < g->nx; x++) {
    for (int i = 0; i < 3; i++) {
      fout[AOS(g, x, top, down[i])] = fin[AOS(g, x, top, OPP[down[i]])];
      fout[AOS(g, x, 0, up[i])] = fin[AOS(g, x, 0, OPP[up[i]])];
    }
  }
}

/* Half-way bounce-back on the square perimeter
 * (src/lbm_src/square.cpp:24-50, the live "_TEST" variant): three slots per
 * side node, one per corner. */
void orc_square_bb(const orc_geom *g, double *fout, const double *fin) {
  static const int bottom[3] = {7, 4, 8}, top[3] = {5, 2, 6};
  static const int left[3] = {6, 3, 7}, right[3] = {8, 1, 5};
  for (int x = g->xmin + 1; x < g->xmax; x++) {
    for (int i = 0; i < 3; i++) {
      fout[AOS(g, x, g->ymin, bottom[i])] =
          fin[AOS(g, x, g->ymin, OPP[bottom[i]])];
      fout[AOS(g, x, g->ymax, top[i])] = fin[AOS(g, x, g->ymax, OPP[top[i]])];
    }
  }
  for (int y = g->ymin + 1; y < g->ymax; y++) {
    for (int i = 0; i < 3; i++) {
      fout[AOS(g, g->xmin, y, left[i])] = fin[AOS(g, g->xmin, y, OPP[left[i]])];
      fout[AOS(g, g->xmax, y, right[i])] =
          fin[AOS(g, g->xmax, y, OPP[right[i]])];
    }
  }
  fout[AOS(g, g->xmin, g->ymin, 7)] = fin[AOS(g, g->xmin, g->ymin, 5)];
  fout[AOS(g, g->xmin, g->ymax, 6)] = fin[AOS(g, g->xmin, g->ymax, 8)];
  fout[AOS(g, g->xmax, g->ymax, 5)] = fin[AOS(g, g->xmax, g->ymax, 7)];
  fout[AOS(g, g->xmax, g->ymin, 8)] = fin[AOS(g, g->xmax, g->ymin, 6)];
}

/* Nodes strictly inside the square are reset to the rest equilibrium w[k]
 * after every step (src/mpi_LBM_GK_pops_perturb.cpp:430-439). */
void orc_interior_reset(const orc_geom *g, double *fout) {
  for (int x = g->xmin + 1; x < g->xmax; x++)
    for (int y = g->ymin + 1; y < g->ymax; y++)
      for (int k = 0; k < 9; k++) fout[AOS(g, x, y, k)] = WK[k];
}

/* Local moments with the UNshifted velocity (src/lbm_src/force.cpp:26-35) and
 * the non-equilibrium second moment sum_k fneq_k * a_k * b_k (:37-46). */
static void node_pi(const orc_geom *g, const double *f, int x, int y, int a,
                    double *rho_out, double *pi_out) {
  double r = 0.0, vx = 0.0, vy = 0.0;
  for (int k = 0; k < 9; k++) {
    double fk = f[AOS(g, x, y, k)];
    r += fk;
    vx += fk * (double)CX[k];
    vy += fk * (double)CY[k];
  }
  vy /= r;
  vx /= r;
  double pi = 0.0;
  double u2 = -1.5 * (vx * vx + vy * vy);
  for (int k = 0; k < 9; k++) {
    double cx = (double)CX[k], cy = (double)CY[k];
    double eu = cx * vx + cy * vy;
    double eueu = 4.5 * eu * eu;
    double feq = WK[k] * r * (1.0 + 3.0 * eu + eueu + u2);
    double fneq = f[AOS(g, x, y, k)] - feq;
    /* a == 0: Pi_xx weight cx*cx; a == 1: Pi_xy weight cx*cy */
    pi += fneq * cx * (a == 0 ? cx : cy);
  }
  *rho_out = r;
  *pi_out = pi;
}

/* x-drag on the square by stress integration over its perimeter
 * (src/lbm_src/force.cpp:8-144): West sum_y rho/3 + c*Pi_xx, East the
 * negative, North -c*Pi_xy, South +c*Pi_xy, c = 1 - omega/2; each side summed
 * sequentially, then West + East + North + South (:141). */
double orc_force_on_square(const orc_geom *g, const double *f, double omega) {
  const double third = 1. / 3.;
  const double c = 1.0 - .5 * omega;
  double r, pi;
  double west = 0.0, east = 0.0, north = 0.0, south = 0.0;
  for (int y = g->ymin; y < g->ymax + 1; y++) {
    node_pi(g, f, g->xmin, y, 0, &r, &pi);
    west += r * third + c * pi;
  }
  for (int y = g->ymin; y < g->ymax + 1; y++) {
    node_pi(g, f, g->xmax, y, 0, &r, &pi);
    east += -r * third - c * pi;
  }
  for (int x = g->xmin; x < g->xmax + 1; x++) {
    node_pi(g, f, x, g->ymax, 1, &r, &pi);
    north += -c * pi;
  }
  for (int x = g->xmin; x < g->xmax + 1; x++) {
    node_pi(g, f, x, g->ymin, 1, &r, &pi);
    south += +c * pi;
  }
  return west + east + north + south;
}

/* Momentum exchange (no counterpart in the reference; libclbm's
 * CLBM_DRAG_MOMENTUM).  A slot k the square bounces back holds the
 * post-collision population that left the node along c_{opp k}, reflected, so
 * the link hands the body -2 c_k f_k of momentum; x parts in k order. */
static double me_node(const orc_geom *g, const double *f, int x, int y) {
  const int m = orc_bounce_mask(g, x, y);
  double v = 0.0;
  for (int k = 1; k < 9; k++) {
    if (CX[k] == 0 || !((m >> k) & 1)) continue;
    const double s2 = f[AOS(g, x, y, k)] + f[AOS(g, x, y, k)];
    v = CX[k] < 0 ? v + s2 : v - s2;
  }
  return v;
}

double orc_force_momentum_exchange(const orc_geom *g, const double *f) {
  const int sy = g->ymax - g->ymin + 1, sx = g->xmax - g->xmin + 1;
  const int nt = 2 * sy + 2 * sx;
  double *term = (double *)malloc(sizeof(double) * nt);
  int i = 0;
  for (int y = g->ymin; y <= g->ymax; y++) term[i++] = me_node(g, f, g->xmin, y);
  for (int y = g->ymin; y <= g->ymax; y++) term[i++] = me_node(g, f, g->xmax, y);
  for (int x = g->xmin; x <= g->xmax; x++)
    term[i++] = (x == g->xmin || x == g->xmax) ? 0.0 : me_node(g, f, x, g->ymax);
  for (int x = g->xmin; x <= g->xmax; x++)
    term[i++] = (x == g->xmin || x == g->xmax) ? 0.0 : me_node(g, f, x, g->ymin);
  double lane[32], next[32];
  for (int l = 0; l < 32; l++) {
    lane[l] = 0.0;
    for (int j = l; j < nt; j += 32) lane[l] += term[j];
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int l = 0; l < 32; l++) next[l] = lane[l] + lane[l ^ o];
    memcpy(lane, next, sizeof lane);
  }
  free(term);
  return lane[0];
}

void orc_lbm_step(const orc_geom *g, double **state, double **scratch,
                  double *rho, double *ux, double *uy, double beta,
                  const double *map, double tau, double eps) {
  double *fin = *state, *fout = *scratch;
  stream_collide_impl(g, fin, fout, rho, ux, uy, beta, map, tau, eps);
  orc_walls_bb(g, fout, fin);
  orc_square_bb(g, fout, fin);
  orc_interior_reset(g, fout);
  *state = fout;
  *scratch = fin;
}

int orc_bounce_mask(const orc_geom *g, int x, int y) {
  int m = 0;
  if (y == g->ny - 1) m |= (1 << 4) | (1 << 7) | (1 << 8);
  if (y == 0) m |= (1 << 2) | (1 << 5) | (1 << 6);
  const int inx = x > g->xmin && x < g->xmax;
  const int iny = y > g->ymin && y < g->ymax;
  if (inx && y == g->ymin) m |= (1 << 7) | (1 << 4) | (1 << 8);
  if (inx && y == g->ymax) m |= (1 << 5) | (1 << 2) | (1 << 6);
  if (iny && x == g->xmin) m |= (1 << 6) | (1 << 3) | (1 << 7);
  if (iny && x == g->xmax) m |= (1 << 8) | (1 << 1) | (1 << 5);
  if (x == g->xmin && y == g->ymin) m |= 1 << 7;
  if (x == g->xmin && y == g->ymax) m |= 1 << 6;
  if (x == g->xmax && y == g->ymax) m |= 1 << 5;
  if (x == g->xmax && y == g->ymin) m |= 1 << 8;
  if (inx && iny) m |= 1 << 9;
  return m;
}

/* ------------------------------------------------------------------------ */
/* POSIX drand48: X <- (0x5DEECE66D X + 0xB) mod 2^48, value X/2^48 after the
 * step.  The reference never seeds it (src/mpi_LBM_GK_pops_perturb.cpp:517,
 * generatePerturbedState.cpp:15); glibc's never-seeded state is X0 = 0 (its
 * state block starts zeroed and only the multiplier and addend are filled in on
 * first use), so the first value is 11/2^48. */
#define D48_A 0x5DEECE66DULL
#define D48_C 0xBULL
#define D48_MASK ((1ULL << 48) - 1)

void orc_drand48_init_default(orc_drand48 *s) { s->x = 0; }

double orc_drand48_next(orc_drand48 *s) {
  s->x = (D48_A * s->x + D48_C) & D48_MASK;
  return ldexp((double)s->x, -48);
}

void orc_drand48_skip(orc_drand48 *s, uint64_t n) {
  /* compose the affine map X -> aX + c with itself n times */
  uint64_t am = 1, cm = 0, a = D48_A, c = D48_C;
  while (n) {
    if (n & 1) {
      am = (am * a) & D48_MASK;
      cm = (cm * a + c) & D48_MASK;
    }
    c = ((a + 1) * c) & D48_MASK;
    a = (a * a) & D48_MASK;
    n >>= 1;
  }
  s->x = (am * s->x + cm) & D48_MASK;
}

/* glibc rand() (TYPE_3 additive feedback generator), from its published
 * description: r0 = seed, r_i = 16807 r_{i-1} mod (2^31-1) for i < 31,
 * r_i = r_{i-31} for i = 31..33, r_i = r_{i-3} + r_{i-31} (mod 2^32) after
 * that, the k-th output being r_{k+344} >> 1.  The reference seeds it with
 * srand(rank+1) and discards 1000 values (pops driver :176-178). */
void orc_glibc_srand(orc_glibc_rand *s, uint32_t seed) {
  uint32_t r[344 + 34];
  if (seed == 0) seed = 1;
  r[0] = seed;
  for (int i = 1; i < 31; i++) {
    int64_t v = (16807LL * (int64_t)(int32_t)r[i - 1]) % 2147483647LL;
    if (v < 0) v += 2147483647LL;
    r[i] = (uint32_t)v;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 34; i < 344; i++) r[i] = r[i - 31] + r[i - 3];
  /* keep the last 34 values as a ring: next output uses r[i-31] + r[i-3] */
  for (int i = 0; i < 34; i++) s->r[i] = r[344 - 34 + i];
  s->i = 0;
}

int32_t orc_glibc_rand_next(orc_glibc_rand *s) {
  /* ring holds r_{n-34} .. r_{n-1} with r_{n-34} at index s->i */
  uint32_t a = s->r[(s->i + 34 - 31) % 34]; /* r_{n-31} */
  uint32_t b = s->r[(s->i + 34 - 3) % 34];  /* r_{n-3} */
  uint32_t v = a + b;
  s->r[s->i] = v;
  s->i = (s->i + 1) % 34;
  return (int32_t)(v >> 1);
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper:
 * ten rounds of two 32x32->64 multiplies with Weyl key bumps. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; round++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

double orc_philox_uniform(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2,
                          uint32_t c3) {
  uint32_t ctr[4] = {c0, c1, c2, c3};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  uint64_t m = ((uint64_t)(o[0] >> 5) << 26) | (uint64_t)(o[1] >> 6);
  return ldexp((double)m, -53);
}

/* ------------------------------------------------------------------------ */
/* Snapshot-mix perturbation (src/perturbation_routines/
 * generatePerturbedState.cpp:4-38): S = sum_n r_n snap_n accumulated in
 * snapshot order, weight = |f| / |S| over all n entries, then
 * f <- (f + eps*S*weight) / (1 + sum_n r_n * eps * weight).  The caller draws
 * the prefactors r_n (drand48 in the reference, :15). */
void orc_perturb_mix(double *fin, const double *snaps, int nsnap, int n,
                     double eps, const double *prefactors) {
  double *mix = (double *)calloc((size_t)n, sizeof(double));
  double sum_pref = 0.0;
  for (int s = 0; s < nsnap; s++) {
    double r = prefactors[s];
    sum_pref += r;
    const double *snap = snaps + (size_t)s * n;
    for (int i = 0; i < n; i++) mix[i] += r * snap[i];
  }
  double n0 = 0.0, n1 = 0.0;
  for (int i = 0; i < n; i++) {
    n0 += fin[i] * fin[i];
    n1 += mix[i] * mix[i];
  }
  n0 = sqrt(n0);
  n1 = sqrt(n1);
  double weight = n0 / n1;
  double a = 1.0 + sum_pref * eps * weight;
  double inv_a = 1. / a;
  for (int i = 0; i < n; i++) {
    fin[i] += eps * mix[i] * weight;
    fin[i] = fin[i] * inv_a;
  }
  free(mix);
}

/* Counter-based uniform multiplicative noise f <- f (1 + eps (2u - 1)), one
 * Philox draw per population, counter (aos index, clone, interval, run). */
void orc_perturb_uniform(double *fin, const orc_geom *g, double eps,
                         uint64_t seed, uint32_t run, uint32_t clone,
                         uint32_t interval) {
  const int n = 9 * g->nx * g->ny;
  for (int i = 0; i < n; i++) {
    double u = orc_philox_uniform(seed, (uint32_t)i, clone, interval,
                                  (run << 4) | 2u);
    fin[i] = fin[i] * (1.0 + eps * (2.0 * u - 1.0));
  }
}

/* Synthetic initial state: equilibrium at rho = 1, u = (u0, 0) in the fluid,
 * times (1 + noise (2u - 1)); w[k] inside the square. */
void orc_init_equilibrium(double *fin, const orc_geom *g, double u0,
                          double noise, uint64_t seed, uint32_t run,
                          uint32_t clone) {
  for (int x = 0; x < g->nx; x++) {
    for (int y = 0; y < g->ny; y++) {
      int solid = x > g->xmin && x < g->xmax && y > g->ymin && y < g->ymax;
      for (int k = 0; k < 9; k++) {
        int i = AOS(g, x, y, k);
        if (solid) {
          fin[i] = WK[k];
          continue;
        }
        double eu = (double)CX[k] * u0;
        double feq = WK[k] * (1.0 + 3.0 * eu + 4.5 * eu * eu + -1.5 * (u0 * u0));
        double u = orc_philox_uniform(seed, (uint32_t)i, clone, 0xFFFFFFFFu,
                                      (run << 4) | 1u);
        fin[i] = feq * (1.0 + noise * (2.0 * u - 1.0));
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Turn copy numbers into the copy table and labels: the m-th surplus copy (in
 * ascending parent order) fills the m-th lowest killed slot, which is what the
 * reference's restarted linear search yields
 * (src/mpi_LBM_GK_pops_perturb.cpp:590-619). */
static int build_table(int nc, int *n, int *labels, int *table) {
  int ncomm = 0, next_free = 0;
  for (int j = 0; j < nc; j++) labels[j] = j;
  for (int i = 0; i < nc; i++) {
    while (n[i] > 1) {
      while (next_free < nc && n[next_free] != 0) next_free++;
      if (next_free >= nc) return -1;
      table[2 * ncomm] = i;
      table[2 * ncomm + 1] = next_free;
      n[next_free] = -1;
      labels[next_free] = i;
      ncomm++;
      n[i]--;
    }
  }
  return ncomm;
}

/* Reference cloning step (pops driver :487-624): gather the mean weight over
 * ranks, draw n_j = floor(s_j/R + drand48()), then kill or duplicate uniformly
 * among the drawn copies with glibc rand() until sum n_j = Nc. */
orc_clone_result orc_clone_reference(int nc, int ranks, const double *s,
                                     orc_drand48 *master, orc_glibc_rand *rnd,
                                     int *copies_pre, int *copies_post,
                                     int *labels, int *table) {
  orc_clone_result res = {0.0, 0.0, 0, 0, 0};
  const int local = nc / ranks;
  double total = 0.0;
  for (int r = 0; r < ranks; r++) {
    double part = 0.0;
    for (int j = r * local; j < (r + 1) * local; j++) part += s[j];
    if (r == 0)
      total = part;
    else
      total += part;
  }
  total /= nc;
  res.rbar = total;
  res.logr = log(total);
  if (!isfinite(total) || !(total > 0.0)) {
    res.status = -3;
    return res;
  }
  int *n = (int *)malloc(sizeof(int) * nc);
  int *temp = (int *)malloc(sizeof(int) * (3 * nc + 2));
  int drawn = 0;
  for (int j = 0; j < nc; j++) {
    double a = orc_drand48_next(master);
    double v = floor(s[j] / total + a);
    if (!isfinite(v) || v > 2.0 * nc + 1) {
      res.status = -3;
      free(n);
      free(temp);
      return res;
    }
    n[j] = (int)v;
    drawn += n[j];
  }
  res.ncopies_drawn = drawn;
  if (copies_pre) memcpy(copies_pre, n, sizeof(int) * nc);
  int kk = 0;
  for (int j = 0; j < nc; j++)
    for (int i = 0; i < n[j]; i++) temp[kk++] = j;
  int delta = drawn - nc;
  if (delta > 0) {
    for (int i = 0; i < delta; i++) {
      int idx = orc_glibc_rand_next(rnd) % (drawn - i);
      int victim = temp[idx];
      temp[idx] = temp[drawn - i - 1];
      n[victim]--;
    }
  } else if (delta < 0) {
    if (drawn == 0) {
      res.status = -3;
      free(n);
      free(temp);
      return res;
    }
    for (int i = 0; i < -delta; i++) {
      int idx = orc_glibc_rand_next(rnd) % drawn;
      n[temp[idx]]++;
    }
  }
  if (copies_post) memcpy(copies_post, n, sizeof(int) * nc);
  res.ncomm = build_table(nc, n, labels, table);
  if (res.ncomm < 0) res.status = -3;
  free(n);
  free(temp);
  return res;
}

/* Systematic resampling (new mode, no reference counterpart): one uniform u,
 * c_j = (P_j / P_N) * Nc with P the prefix sum of exp(logw - max),
 * n_j = floor(c_j + u) - floor(c_{j-1} + u), which sums to Nc exactly. */
orc_clone_result orc_clone_systematic(int nc, const double *logw, double u,
                                      int *copies, int *labels, int *table) {
  orc_clone_result res = {0.0, 0.0, 0, 0, 0};
  double m = -INFINITY;
  for (int j = 0; j < nc; j++)
    if (logw[j] > m) m = logw[j];
  double *p = (double *)malloc(sizeof(double) * nc);
  int *n = (int *)malloc(sizeof(int) * nc);
  double acc = 0.0;
  for (int j = 0; j < nc; j++) {
    acc += exp(logw[j] - m);
    p[j] = acc;
  }
  res.logr = m + log(acc / nc);
  res.rbar = exp(res.logr);
  double prev = floor(u);
  for (int j = 0; j < nc; j++) {
    double c = (p[j] / acc) * nc;
    double cur = floor(c + u);
    n[j] = (int)(cur - prev);
    prev = cur;
  }
  res.ncopies_drawn = nc;
  if (copies) memcpy(copies, n, sizeof(int) * nc);
  res.ncomm = build_table(nc, n, labels, table);
  if (res.ncomm < 0) res.status = -3;
  free(p);
  free(n);
  return res;
}

/* ------------------------------------------------------------------------ */
/* The population-perturbation driver's loop (pops driver :387-701), run as
 * `ranks` virtual MPI ranks in one process: each rank owns a contiguous block
 * of clones and its own never-seeded drand48 stream, rank 0 also draws the copy
 * numbers and the glibc rand() corrections (srand(1) + 1000 discards).  New
 * clones are perturbed at the start of the next interval (_SMART_PERTURB).
 * Outputs (all optional): drag[t][j][tt] = F/F0 - shift, labels[t][j],
 * rvalues[t], logr[t] = log R_t, weights[t][j] = exp(alpha s_j),
 * copies[t][2][j]. */
int orc_run_sampler(const orc_sampler_cfg *cfg, double *states,
                    const double *snaps, double *drag, int *labels,
                    double *rvalues, double *logr, double *weights,
                    int *copies) {
  const orc_geom *g = &cfg->g;
  const int nc = cfg->nclones;
  const int n = 9 * g->nx * g->ny;
  const int ranks = cfg->ranks > 0 ? cfg->ranks : 1;
  if (nc % ranks) return -1;
  const int local = nc / ranks;
  const double omega = 1.0 / cfg->tau;
  orc_drand48 *d48 = (orc_drand48 *)malloc(sizeof(orc_drand48) * ranks);
  for (int r = 0; r < ranks; r++) orc_drand48_init_default(&d48[r]);
  orc_glibc_rand rnd;
  orc_glibc_srand(&rnd, 1);
  for (int i = 0; i < 1000; i++) orc_glibc_rand_next(&rnd);
  double *scratch = (double *)malloc(sizeof(double) * n);
  double *s = (double *)malloc(sizeof(double) * nc);
  double *logw = (double *)malloc(sizeof(double) * nc);
  int *mark = (int *)calloc(nc, sizeof(int));
  int *lab = (int *)malloc(sizeof(int) * nc);
  int *table = (int *)malloc(sizeof(int) * 2 * nc);
  int *pre = (int *)malloc(sizeof(int) * nc);
  int *post = (int *)malloc(sizeof(int) * nc);
  double pref[64];
  int status = 0;
  for (int t = 0; t < cfg->intervals && status == 0; t++) {
    for (int j = 0; j < nc; j++) {
      double *st = states + (size_t)j * n;
      if (mark[j]) {
        if (cfg->perturb_mode == ORC_PERTURB_MIX) {
          for (int q = 0; q < cfg->nsnap; q++)
            pref[q] = orc_drand48_next(&d48[j / local]);
          orc_perturb_mix(st, snaps, cfg->nsnap, n, cfg->eps, pref);
        } else if (cfg->perturb_mode == ORC_PERTURB_UNIFORM) {
          orc_perturb_uniform(st, g, cfg->eps, cfg->seed, cfg->run,
                              (uint32_t)j, (uint32_t)t);
        }
      }
      double acc = 0;
      double *cur = st, *tmp = scratch;
      for (int tt = 0; tt < cfg->steps; tt++) {
        orc_lbm_step(g, &cur, &tmp, NULL, NULL, NULL, cfg->beta, NULL,
                     cfg->tau, 0.0);
        double F = cfg->drag_mode == 1 ? orc_force_momentum_exchange(g, cur)
                                       : orc_force_on_square(g, cur, omega);
        F = F * cfg->force_scale;
        F = F - cfg->force_shift;
        if (drag) drag[((size_t)t * nc + j) * cfg->steps + tt] = F;
        acc += F;
      }
      if (cur != st) {
        memcpy(st, cur, sizeof(double) * n);
        scratch = cur;
      } else {
        scratch = tmp;
      }
      acc *= cfg->dt;
      logw[j] = cfg->alpha * acc;
      s[j] = exp(cfg->alpha * acc);
      if (weights) weights[(size_t)t * nc + j] = s[j];
    }
    orc_clone_result cr;
    if (cfg->resample_mode == ORC_RESAMPLE_SYSTEMATIC) {
      double u = orc_philox_uniform(cfg->seed, (uint32_t)t, 0, 0,
                                    (cfg->run << 4) | 3u);
      cr = orc_clone_systematic(nc, logw, u, pre, lab, table);
      memcpy(post, pre, sizeof(int) * nc);
    } else {
      cr = orc_clone_reference(nc, ranks, s, &d48[0], &rnd, pre, post, lab,
                               table);
    }
    if (cr.status) {
      status = cr.status;
      break;
    }
    if (rvalues) rvalues[t] = cr.rbar;
    if (logr) logr[t] = cr.logr;
    if (labels) memcpy(labels + (size_t)t * nc, lab, sizeof(int) * nc);
    if (copies) {
      memcpy(copies + (size_t)t * 2 * nc, pre, sizeof(int) * nc);
      memcpy(copies + (size_t)t * 2 * nc + nc, post, sizeof(int) * nc);
    }
    memset(mark, 0, sizeof(int) * nc);
    for (int i = 0; i < cr.ncomm; i++) {
      int src = table[2 * i], dst = table[2 * i + 1];
      memcpy(states + (size_t)dst * n, states + (size_t)src * n,
             sizeof(double) * n);
      mark[dst] = 1;
    }
  }
  free(d48);
  free(scratch);
  free(s);
  free(logw);
  free(mark);
  free(lab);
  free(table);
  free(pre);
  free(post);
  return status;
}

/* ------------------------------------------------------------------------ */
/* CPU baseline: the reference's per-clone hot loop (pops driver :424-460:
 * step, walls, square, reset, swap, drag) over nclones clones, the clones split
 * into contiguous blocks over nthreads threads the way MPI ranks split them. */
typedef struct {
  const orc_geom *g;
  int c0, c1, steps;
  double tau, beta, sum;
} bench_arg;

static void *bench_worker(void *p) {
  bench_arg *a = (bench_arg *)p;
  const int n = 9 * a->g->nx * a->g->ny;
  double *st = (double *)malloc(sizeof(double) * n);
  double *tmp = (double *)malloc(sizeof(double) * n);
  const double omega = 1.0 / a->tau;
  double sum = 0.0;
  for (int c = a->c0; c < a->c1; c++) {
    orc_init_equilibrium(st, a->g, 0.04, 1e-3, 12345, 0, (uint32_t)c);
    double *cur = st, *t2 = tmp;
    for (int s = 0; s < a->steps; s++) {
      orc_lbm_step(a->g, &cur, &t2, NULL, NULL, NULL, a->beta, NULL, a->tau,
                   0.0);
      sum += orc_force_on_square(a->g, cur, omega);
    }
    st = cur;
    tmp = t2;
  }
  free(st);
  free(tmp);
  a->sum = sum;
  return NULL;
}

double orc_bench_lbm(const orc_geom *g, int nclones, int steps, double tau,
                     double beta, int nthreads, double *checksum) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > nclones) nthreads = nclones;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  bench_arg *args = (bench_arg *)malloc(sizeof(bench_arg) * nthreads);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int i = 0; i < nthreads; i++) {
    args[i].g = g;
    args[i].c0 = (int)((long)nclones * i / nthreads);
    args[i].c1 = (int)((long)nclones * (i + 1) / nthreads);
    args[i].steps = steps;
    args[i].tau = tau;
    args[i].beta = beta;
    args[i].sum = 0.0;
    pthread_create(&th[i], NULL, bench_worker, &args[i]);
  }
  double sum = 0.0;
  for (int i = 0; i < nthreads; i++) {
    pthread_join(th[i], NULL);
    sum += args[i].sum;
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (checksum) *checksum = sum;
  free(th);
  free(args);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
