// refshim_harness.cpp -- a program written against the reference's function
// signatures, linked with libclbm_refshim.a (test infrastructure).
//
//   refshim_harness IN OUT
// IN: nx ny xmin xmax ymin ymax (int32), tau beta eps (FP64), f0 (9 nx ny),
//     map (nx ny).  OUT: the state after five LB steps as the reference's
//     drivers chain them (collide + stream, walls, square, interior reset,
//     swap; src/mpi_LBM_GK_pops_perturb.cpp:424-445) and the drag after each
//     step, then one spatial-force collision of f0: fin, fout, rho, ux, uy.
#include <cstdio>
#include <vector>

// the reference's signatures (src/lbm_src/streamCollCompute.h:1-2,
// boundaryConditions.h:1,5, force.h:1)
void streamingAndCollisionComputeMacroBodyForce(double *, double *, double *, double *, double *, double, double);
void streamingAndCollisionComputeMacroBodyForceSpatial(double *, double *, double *, double *, double *, double,
                                                       double *, double, double);
void computeDomainNoSlipWalls_BB(double *, double *);
void computeSquareBounceBack_TEST(double *, double *);
double computeForceOnSquare(double *, double);

// the globals the reference's functions read (src/lbm_src/global.h:11-13)
int Dx, Dy, xmin, xmax, ymin, ymax;

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 3;
  int gi[6];
  double p[3];
  if (std::fread(gi, sizeof(int), 6, in) != 6 || std::fread(p, sizeof(double), 3, in) != 3) return 4;
  Dx = gi[0], Dy = gi[1], xmin = gi[2], xmax = gi[3], ymin = gi[4], ymax = gi[5];
  const double tau = p[0], beta = p[1], eps = p[2];
  const size_t N = (size_t)9 * Dx * Dy, n = (size_t)Dx * Dy;
  std::vector<double> f0(N), map(n);
  if (std::fread(f0.data(), sizeof(double), N, in) != N || std::fread(map.data(), sizeof(double), n, in) != n) return 5;
  std::fclose(in);
  const double w[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
  std::vector<double> a(f0), b(N, 0.0), rho(n), ux(n), uy(n), drag(5);
  double *state = a.data(), *fout = b.data();
  for (int t = 0; t < 5; t++) {
    streamingAndCollisionComputeMacroBodyForce(state, fout, rho.data(), ux.data(), uy.data(), beta, tau);
    computeDomainNoSlipWalls_BB(fout, state);
    computeSquareBounceBack_TEST(fout, state);
    for (int x = xmin + 1; x < xmax; x++)
      for (int y = ymin + 1; y < ymax; y++)
        for (int k = 0; k < 9; k++) fout[k + 9 * (y + Dy * x)] = w[k];
    double *pivot = state;
    state = fout;
    fout = pivot;
    drag[t] = computeForceOnSquare(state, 1.0 / tau);
  }
  std::vector<double> sfin(f0), sfout(N, 0.0), srho(n), sux(n), suy(n);
  streamingAndCollisionComputeMacroBodyForceSpatial(sfin.data(), sfout.data(), srho.data(), sux.data(), suy.data(),
                                                    beta, map.data(), tau, eps);
  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 6;
  std::fwrite(state, sizeof(double), N, out);
  std::fwrite(drag.data(), sizeof(double), 5, out);
  for (const std::vector<double> *v : {&sfin, &sfout, &srho, &sux, &suy})
    std::fwrite(v->data(), sizeof(double), v->size(), out);
  std::fclose(out);
  return 0;
}
