/*
 * ref_harness.cpp -- C entry points over the reference's own LBM objects,
 * compiled in place from the reference tree by oracle/Makefile into
 * oracle/_ref/libref_core.so.  TEST INFRASTRUCTURE ONLY: it lets the tests
 * call the reference functions with any channel geometry (the reference reads
 * its geometry from globals, src/lbm_src/global.h:11-15, which its drivers fix
 * to Dx = Dy = 4L+1) and time the reference hot loop as the CPU baseline.
 */
#include <cstdint>
#include <cstdlib>
#include <ctime>
#include <vector>

#include "boundaryConditions.h"
#include "force.h"
#include "streamCollCompute.h"

/* the globals the reference core reads (global.h:11-15); the lattice tables
 * must hold the same values as the drivers' (pops driver :31-32) */
int Dx, Dy, xmin, xmax, ymin, ymax;
int c[9][2] = {{0, 0}, {1, 0}, {0, 1}, {-1, 0}, {0, -1},
               {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
double w[9] = {4.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0, 1.0 / 9.0,
               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};

int generatePerturbedState(double *, double **, double, int, int);

extern "C" {

void ref_set_geom(int nx, int ny, int x0, int x1, int y0, int y1) {
  Dx = nx; Dy = ny; xmin = x0; xmax = x1; ymin = y0; ymax = y1;
}

void ref_stream_collide(double *fin, double *fout, double *rho, double *ux,
                        double *uy, double beta, double tau) {
  streamingAndCollisionComputeMacroBodyForce(fin, fout, rho, ux, uy, beta, tau);
}

void ref_stream_collide_spatial(double *fin, double *fout, double *rho,
                                double *ux, double *uy, double beta0,
                                double *map, double tau, double eps) {
  streamingAndCollisionComputeMacroBodyForceSpatial(fin, fout, rho, ux, uy,
                                                    beta0, map, tau, eps);
}

void ref_walls_bb(double *fout, double *fin) { computeDomainNoSlipWalls_BB(fout, fin); }

void ref_square_bb(double *fout, double *fin) { computeSquareBounceBack_TEST(fout, fin); }

double ref_force(double *f, double omega) { return computeForceOnSquare(f, omega); }

/* generatePerturbedState draws its prefactors from the process's drand48
 * stream; the caller positions that stream (seed48) before the call. */
void ref_perturb(double *fin, double *snaps, int nsnap, int n, double eps) {
  std::vector<double *> p(nsnap);
  for (int i = 0; i < nsnap; i++) p[i] = snaps + (size_t)i * n;
  generatePerturbedState(fin, p.data(), eps, nsnap, n);
}

/* The pops driver's per-step sequence (:426-445) on one clone, using the
 * reference functions; the interior reset and the swap are the driver's own
 * inline code, restated. */
static void one_step(double *&state, double *&scratch, double *rho, double *ux,
                     double *uy, double beta, double tau) {
  streamingAndCollisionComputeMacroBodyForce(state, scratch, rho, ux, uy, beta, tau);
  computeDomainNoSlipWalls_BB(scratch, state);
  computeSquareBounceBack_TEST(scratch, state);
  for (int x = xmin + 1; x < xmax; x++)
    for (int y = ymin + 1; y < ymax; y++)
      for (int k = 0; k < 9; k++) scratch[k + 9 * (y + Dy * x)] = w[k];
  double *t = state; state = scratch; scratch = t;
}

/* steps LB steps of one clone, drag after each: drag[steps] */
void ref_run_clone(double *state, int steps, double beta, double tau,
                   double *drag) {
  const int n = 9 * Dx * Dy;
  std::vector<double> scratch(n), rho(Dx * Dy), ux(Dx * Dy), uy(Dx * Dy);
  double *cur = state, *tmp = scratch.data();
  for (int s = 0; s < steps; s++) {
    one_step(cur, tmp, rho.data(), ux.data(), uy.data(), beta, tau);
    drag[s] = computeForceOnSquare(cur, 1.0 / tau);
  }
  if (cur != state)
    for (int i = 0; i < n; i++) state[i] = cur[i];
}

/* CPU baseline: nclones clones (state[nclones*n], prepared by the caller),
 * steps each, sequentially in this process; returns seconds. */
double ref_bench(double *states, int nclones, int steps, double beta,
                 double tau, double *checksum) {
  const int n = 9 * Dx * Dy;
  std::vector<double> scratch(n), rho(Dx * Dy), ux(Dx * Dy), uy(Dx * Dy);
  timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  double sum = 0.0;
  for (int j = 0; j < nclones; j++) {
    double *cur = states + (size_t)j * n, *tmp = scratch.data();
    for (int s = 0; s < steps; s++) {
      one_step(cur, tmp, rho.data(), ux.data(), uy.data(), beta, tau);
      sum += computeForceOnSquare(cur, 1.0 / tau);
    }
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (checksum) *checksum = sum;
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
}
