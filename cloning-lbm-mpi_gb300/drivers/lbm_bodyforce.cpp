// lbm_bodyforce.cpp -- LBM_BODYFORCE, the warm-up / snapshot generator over
// libclbm (the reference's stand-alone src/lbm_src/main_bodyforce.cpp).
//
// Reads input.datin: nbOfChunks nbOfTimeSteps L tau Ma folder inputPops
// facquVtk facquForce facquU (main_bodyforce.cpp:38-50; nbOfChunks is read and
// unused there too).  Runs one D2Q9 channel of Dx = Dy = 4L+1 with the square
// of side L and body force beta = 8 nu u0 / ((Dy-1)/2)^2, u0 = Ma/3, from the
// populations in file `inputPops`, or from the rest state w[k] when it is "0"
// (:95-110), and writes into folder/:
//   parameters.datout   (text)
//   data_force.datout   F after every step t with t % facquForce == 0 (raw)
//   ux_t.datout         ux at (Dx/4, Dy/4) of the state entering step t,
//                       t % facquU == 0
//   vtk_fluid/fluid_t<n>.vtk  rho-1 and (ux, uy) of the state entering step
//                       t, t % facquVtk == 0
//   pops.datout         the final populations (the clone initial condition the
//                       cloning drivers read, :179-182)
// Options before nothing (all optional): --fp32, --snapshots K --every M
// (after the run, K more states M steps apart as pops_<k>.datout plus a
// popfiles_list.dat naming them, the inputs of TLGK_LBM_POPS_PERTURB).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <numeric>
#include <string>
#include <vector>

#include "clbm.h"
#include "tlgk_io.h"
#include "vtk.h"

using namespace tlgk;

int main(int argc, char **argv) {
  int precision = CLBM_FP64, nsnap = 0, every = 0;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    if (a == "--fp32") precision = CLBM_FP32;
    else if (a == "--snapshots" && i + 1 < argc) nsnap = std::atoi(argv[++i]);
    else if (a == "--every" && i + 1 < argc) every = std::atoi(argv[++i]);
  }
  Log log("output_LBM.out");
  std::ifstream in("input.datin");
  int chunks = 0, steps = 0, L = 0, fvtk = 0, fforce = 0, fu = 0;
  double tau = 1.0, Ma = 1.0;
  std::string folder, inpops;
  if (!(in >> chunks >> steps >> L >> tau >> Ma >> folder >> inpops >> fvtk >> fforce >> fu)) {
    log.line("ERROR: could not read input.datin");
    return 1;
  }
  if (steps < 1 || fvtk < 1 || fforce < 1 || fu < 1 || (nsnap > 0 && every < 1)) {
    log.line("ERROR: steps and sampling periods must be >= 1");
    return 1;
  }
  const int Dy = 4 * L + 1, Dx = Dy;
  const int xmin = (Dx - 1) / 2, xmax = xmin + L, ymin = (Dy - 1) / 2 - L / 2, ymax = ymin + L;
  const double cs = 1. / std::sqrt(3);
  const double u0 = cs * cs * Ma;
  const double nu = 1. / 3 * (tau - 0.5);
  const double beta = 8 * nu * u0 / ((Dy - 1) / 2) / ((Dy - 1) / 2);
  make_dir(folder);
  make_dir(folder + "/vtk_fluid/");
  {
    std::ofstream p(folder + "/parameters.datout");
    p << "Number of timesteps : " << chunks << "X" << steps << "\nL : " << L << "\nDx : " << Dx
      << "\nDy : " << Dy << "\ntau : " << tau << "\nbeta : " << beta << "\n";
  }
  const size_t n = 9 * (size_t)Dx * Dy;
  std::vector<double> f(n);
  if (inpops != "0") {
    if (!read_pops(inpops, f, n, 0)) {
      log.line("ERROR: could not read " + inpops);
      return 1;
    }
  } else {
    const double w[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                         1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
    for (size_t i = 0; i < n; i++) f[i] = w[i % 9];
  }
  // the macro-field samples fall on multiples of facquU and facquVtk: run
  // the steps in chunks of their gcd and read the state between chunks
  const int chunk = std::max(1, std::min(steps, std::gcd(fu, fvtk)));
  clbm_run_desc d{};
  d.width = Dx;
  d.height = Dy;
  d.xmin = xmin;
  d.xmax = xmax;
  d.ymin = ymin;
  d.ymax = ymax;
  d.nclones = 1;
  d.ranks = 1;
  d.tau = tau;
  d.beta = beta;
  d.force_scale = 1.0;
  d.dt = 1.0;
  clbm_ctx *ctx = nullptr;
  int s = clbm_create(&d, 1, precision, std::max(chunk, every), 0, &ctx);
  if (s || (s = clbm_load_pops_aos_f64(ctx, 0, 0, f.data()))) {
    log.line(std::string("ERROR: ") + clbm_strerror(s) + ": " + clbm_last_error());
    return 1;
  }
  const std::string force_file = folder + "/data_force.datout", ux_file = folder + "/ux_t.datout";
  write_binary(force_file, nullptr, 0);
  write_binary(ux_file, nullptr, 0);
  std::vector<double> rho(Dx * Dy), ux(Dx * Dy), uy(Dx * Dy), drag(std::max(chunk, every));
  int tvtk = 0;
  for (int t0 = 0; t0 < steps; t0 += chunk) {
    const int m = std::min(chunk, steps - t0);
    if (t0 % fu == 0 || t0 % fvtk == 0) {
      if ((s = clbm_macro_fields(ctx, 0, 0, rho.data(), ux.data(), uy.data()))) break;
      if (t0 % fvtk == 0)
        write_fluid_vtk(folder + "/vtk_fluid/fluid_t" + std::to_string(tvtk++) + ".vtk", Dx, Dy, rho.data(),
                        ux.data(), uy.data());
      if (t0 % fu == 0) append_binary(ux_file, &ux[(Dy / 4) + Dy * (Dx / 4)], sizeof(double));
    }
    if ((s = clbm_run_interval(ctx, m)) || (s = clbm_get_drag(ctx, 0, drag.data()))) break;
    for (int i = 0; i < m; i++)
      if ((t0 + i) % fforce == 0) append_binary(force_file, &drag[i], sizeof(double));
  }
  if (!s) s = clbm_dump_pops_aos_f64(ctx, 0, 0, f.data());
  if (!s) write_binary(folder + "/pops.datout", f.data(), n * sizeof(double));
  if (!s && nsnap > 0) {
    std::ofstream list(folder + "/popfiles_list.dat");
    for (int k = 0; k < nsnap && !s; k++) {
      if ((s = clbm_run_interval(ctx, every)) || (s = clbm_dump_pops_aos_f64(ctx, 0, 0, f.data()))) break;
      const std::string name = "pops_" + std::to_string(k) + ".datout";
      write_binary(folder + "/" + name, f.data(), n * sizeof(double));
      list << name << "\n";
    }
  }
  if (s) {
    log.line(std::string("ERROR: ") + clbm_strerror(s) + ": " + clbm_last_error());
    return 1;
  }
  log.line("done: " + std::to_string(steps) + " steps, Dx = " + std::to_string(Dx));
  clbm_destroy(ctx);
  return 0;
}
