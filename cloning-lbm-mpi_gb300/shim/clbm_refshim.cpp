// clbm_refshim.cpp -- the reference's LBM and perturbation functions with
// their own C++ signatures, computed by libclbm on the GPU.
//
// A program written against the reference's headers (src/lbm_src/
// streamCollCompute.h:1-2, boundaryConditions.h:1,5, force.h:1,
// src/perturbation.h:3,5) links against this archive instead of the
// reference's LBM objects, unchanged: same function names and argument
// meaning, geometry read from the program's own globals Dx, Dy, xmin, xmax,
// ymin, ymax (src/lbm_src/global.h:11-13), host arrays in the reference's
// AoS layout IDX(x,y,k) = k + 9*(y + Dy*x).  Each call copies its arrays to a
// device mirror, runs the libclbm function-level entry point (bit-identical
// to the reference function), and copies the arrays the function writes
// back.  That per-call traffic makes it a compatibility layer, not the fast
// path: the sampler API (clbm_ctx) keeps every clone on the device.
// The reference functions report no errors, so a libclbm error ends the
// program with a message.
#include <cstdio>
#include <cstdlib>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/clbm.h"

// the calling program's globals (the reference's drivers define them)
extern int Dx, Dy, xmin, xmax, ymin, ymax;

namespace {

void fatal(const char *where, const char *what) {
  std::fprintf(stderr, "clbm_refshim: %s: %s\n", where, what);
  std::abort();
}

void check(int status, const char *where) {
  if (status != CLBM_OK) fatal(where, clbm_last_error());
}

void check_cuda(cudaError_t e, const char *where) {
  if (e != cudaSuccess) fatal(where, cudaGetErrorString(e));
}

// One device buffer per host array the program passes, grown on demand and
// kept for the life of the process.
struct Mirrors {
  struct Buf {
    double *d = nullptr;
    size_t n = 0;
  };
  std::unordered_map<const void *, Buf> bufs;
  ~Mirrors() {
    for (auto &kv : bufs) cudaFree(kv.second.d);
  }
  double *get(const void *host, size_t n) {
    Buf &b = bufs[host];
    if (b.n < n) {
      if (b.d) cudaFree(b.d);
      b.d = nullptr;
      check_cuda(cudaMalloc((void **)&b.d, n * sizeof(double)), "cudaMalloc");
      b.n = n;
    }
    return b.d;
  }
};
Mirrors &mirrors() {
  static Mirrors m;
  return m;
}

double *to_device(const double *host, size_t n) {
  double *d = mirrors().get(host, n);
  check_cuda(cudaMemcpy(d, host, n * sizeof(double), cudaMemcpyHostToDevice), "copy to device");
  return d;
}

double *device_only(const double *host, size_t n) { return host ? mirrors().get(host, n) : nullptr; }

void to_host(double *host, const double *d, size_t n) {
  if (host) check_cuda(cudaMemcpy(host, d, n * sizeof(double), cudaMemcpyDeviceToHost), "copy to host");
}

clbm_geom geometry() { return clbm_geom{Dx, Dy, xmin, xmax, ymin, ymax}; }

size_t npop() { return (size_t)9 * Dx * Dy; }
size_t nnode() { return (size_t)Dx * Dy; }

}  // namespace

// streamCollCompute.h:1: collide fin in place, stream into fout, macroscopic
// fields into rho, ux, uy
void streamingAndCollisionComputeMacroBodyForce(double *fin, double *fout, double *rho, double *ux,
                                                double *uy, double beta, double tau) {
  const clbm_geom g = geometry();
  double *dfin = to_device(fin, npop()), *dfout = to_device(fout, npop());
  double *drho = device_only(rho, nnode()), *dux = device_only(ux, nnode()), *duy = device_only(uy, nnode());
  check(clbm_ref_stream_collide(&g, dfin, dfout, drho, dux, duy, beta, tau, nullptr),
        "streamingAndCollisionComputeMacroBodyForce");
  to_host(fin, dfin, npop());
  to_host(fout, dfout, npop());
  to_host(rho, drho, nnode());
  to_host(ux, dux, nnode());
  to_host(uy, duy, nnode());
}

// streamCollCompute.h:2: the same under the spatial body force
// beta(x,y) = (1 + eps map(x,y)) beta0
void streamingAndCollisionComputeMacroBodyForceSpatial(double *fin, double *fout, double *rho, double *ux,
                                                       double *uy, double beta0, double *map, double tau,
                                                       double eps) {
  const clbm_geom g = geometry();
  double *dfin = to_device(fin, npop()), *dfout = to_device(fout, npop());
  double *dmap = to_device(map, nnode());
  double *drho = device_only(rho, nnode()), *dux = device_only(ux, nnode()), *duy = device_only(uy, nnode());
  check(clbm_ref_stream_collide_spatial(&g, dfin, dfout, drho, dux, duy, beta0, dmap, tau, eps, nullptr),
        "streamingAndCollisionComputeMacroBodyForceSpatial");
  to_host(fin, dfin, npop());
  to_host(fout, dfout, npop());
  to_host(rho, drho, nnode());
  to_host(ux, dux, nnode());
  to_host(uy, duy, nnode());
}

// boundaryConditions.h:1: half-way bounce-back on the channel walls
void computeDomainNoSlipWalls_BB(double *fout, double *fin) {
  const clbm_geom g = geometry();
  double *dfout = to_device(fout, npop()), *dfin = to_device(fin, npop());
  check(clbm_ref_walls_bb(&g, dfout, dfin, nullptr), "computeDomainNoSlipWalls_BB");
  to_host(fout, dfout, npop());
}

// boundaryConditions.h:5: bounce-back on the square's perimeter
void computeSquareBounceBack_TEST(double *fout, double *fin) {
  const clbm_geom g = geometry();
  double *dfout = to_device(fout, npop()), *dfin = to_device(fin, npop());
  check(clbm_ref_square_bb(&g, dfout, dfin, nullptr), "computeSquareBounceBack_TEST");
  to_host(fout, dfout, npop());
}

// force.h:1: x-drag on the square by stress integration
double computeForceOnSquare(double *f, double omega) {
  const clbm_geom g = geometry();
  double *df = to_device(f, npop());
  double F = 0.0;
  check(clbm_ref_force_on_square(&g, df, omega, &F, nullptr), "computeForceOnSquare");
  return F;
}

// perturbation.h:5: fin <- (fin + eps w sum_q r_q snap_q) / a with the NN
// prefactors r_q drawn from the program's drand48() stream, in the
// reference's order (generatePerturbedState.cpp:15)
int generatePerturbedState(double *fin, double **popsForPerturb, double eps, int NN, int N) {
  std::vector<double> pre(NN);
  for (int q = 0; q < NN; q++) pre[q] = drand48();
  double *dfin = to_device(fin, (size_t)N);
  double *dsnap = mirrors().get(popsForPerturb, (size_t)NN * N);
  for (int q = 0; q < NN; q++)
    check_cuda(cudaMemcpy(dsnap + (size_t)q * N, popsForPerturb[q], (size_t)N * sizeof(double),
                          cudaMemcpyHostToDevice),
               "copy snapshots");
  check(clbm_ref_perturbed_state(dfin, dsnap, eps, NN, N, pre.data(), nullptr), "generatePerturbedState");
  to_host(fin, dfin, (size_t)N);
  return 0;
}

// perturbation.h:3: a Gaussian random field on the n x n lattice, covariance
// exp(-r^2 / (2 32^2)) (covariance_fctn.cpp:3-10), by circulant embedding;
// the normals come from libclbm's counter-based stream (seed 1, one draw per
// call), so the parity with the reference's rand() draws is statistical.
// error = 1 when the embedding had negative eigenvalues, as the reference.
void generate_random_field(int n, double *map_, int &error) {
  static int draw = 0;
  int negative = 0;
  check(clbm_ref_random_field(n, n, 32.0, 1ull, draw++, map_, &negative), "generate_random_field");
  error = negative > 0 ? 1 : 0;
}
