// tlgk_main.cpp -- the drop-in driver executables over libclbm's C ABI.
//
//   TLGK_LBM_POPS_PERTURB inputfile   (src/mpi_LBM_GK_pops_perturb.cpp)
//   TLGK_LBM [inputfile]              (src/mpi_LBM_GK.cpp)
//   TLGK_LBM_FORCING inputfile        (src/mpi_LBM_GK_forcing.cpp)
//
// They read the reference's input files and popfiles and write its binary
// outputs (labels.dat, rvalues.dat, clone_<j>/data_force.datout, and for the
// forcing variant weights_evolution_<t>, copies_evolution_<t>,
// clone_<j>/evolution_<t>_clone_<j>), so post_processing/ reads them
// unchanged.  All clones live on one GPU; there are no MPI ranks.  Options
// before the input file:
//   --ranks P        reproduce the random streams of an `mpirun -n P` run
//   --fp32           FP32 populations, interval kernel autotuned (default FP64, the
//                    reference's arithmetic)
//   --seed S         (forcing variant) seed of the random-field stream
//   --no-zero-mean   drag without the AVG = 1.775 shift (the Makefile sets
//                    ZERO_MEAN, so it is on by default)
//   --reconstruct    (pops variant) also write every final slot's lineage
//                    drag series to <parent>reconstructed/clone_<j>/data_force.datout,
//                    what post_processing/reconstruction.cpp assembles
//                    from labels.dat and the slot files
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "clbm.h"
#include "tlgk_io.h"

using namespace tlgk;

namespace {

struct Opts {
  int ranks = 1;
  int precision = CLBM_FP64;
  bool zero_mean = true;
  bool reconstruct = false;
  unsigned long long seed = 1;
  std::string input;
};

Opts parse(int argc, char **argv) {
  Opts o;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    if (a == "--ranks" && i + 1 < argc)
      o.ranks = std::atoi(argv[++i]);
    else if (a == "--fp32")
      o.precision = CLBM_FP32;
    else if (a == "--no-zero-mean")
      o.zero_mean = false;
    else if (a == "--reconstruct")
      o.reconstruct = true;
    else if (a == "--seed" && i + 1 < argc)
      o.seed = std::strtoull(argv[++i], nullptr, 10);
    else
      o.input = a;
  }
  return o;
}

// FP32 contexts: pick the fastest interval kernel for this workload (the
// streaming step's launch shapes or the cluster-resident kernel); the state
// is untouched and every choice gives the same bits.  FP64: nothing to pick.
int tune(clbm_ctx *ctx) {
  int best = 0;
  return clbm_autotune(ctx, 3, &best, nullptr, nullptr);
}

int die(Log &log, const std::string &msg, int status) {
  log.line("ERROR: " + msg);
  if (status) log.line(std::string("  libclbm: ") + clbm_strerror(status) + ": " + clbm_last_error());
  return 1;
}

std::string clone_dir(const std::string &parent, int j) { return parent + "clone_" + std::to_string(j) + "/"; }

// Population-perturbation driver (pops :35-733): perturbation of new clones
// from the snapshot mix, labels.dat, rvalues.dat, per-slot data_force.datout.
int run_pops(const Opts &o) {
  Log log("output_TLGK.out");
  Input in = read_input_pops(o.input);
  if (!in.ok) return die(log, "COULD NOT OPEN INPUT FILE " + o.input, 0);
  const Setup st = setup_from(in, false);
  const int NN = 10;
  if (o.ranks < 1 || in.nc % o.ranks) return die(log, "Nc must be a multiple of --ranks", 0);
  if (st.steps2 < 1 || st.intervals < 1) return die(log, "no LB step or no cloning step to run", 0);
  log.line("READ input file");
  log.line("  Nc = " + std::to_string(in.nc));
  log.line("  L = " + std::to_string(in.L) + " Dx = " + std::to_string(st.Dx) + " Dy = " + std::to_string(st.Dy));
  make_dir(in.parent);
  for (int j = 0; j < in.nc; j++) make_dir(clone_dir(in.parent, j));
  const std::string labels_file = in.parent + "labels.dat";
  write_binary(labels_file, nullptr, 0);

  // popfiles: with p ranks the master hands names nc/p.. to the other ranks
  // first, then reads its own (pops :273-293)
  const size_t n = 9 * (size_t)st.Dx * st.Dy;
  std::vector<std::string> names;
  if (!read_list(in.path + "popfiles_list.dat", names, std::max(in.nc, NN)))
    return die(log, "COULD NOT OPEN INDEX FILE " + in.path + "popfiles_list.dat", 0);
  const int local = in.nc / o.ranks;
  std::vector<double> states(n * in.nc), snaps(n * NN);
  for (int j = 0; j < in.nc; j++) {
    const int name_idx = (j >= local) ? j - local : in.nc - local + j;
    if (!read_pops(in.path + names[name_idx], states, n, n * j))
      return die(log, "could not read popfile " + names[name_idx], 0);
  }
  for (int q = 0; q < NN; q++)
    if (!read_pops(in.path + names[q], snaps, n, n * q))
      return die(log, "ERROR WITH READING OF POPULATIONS FOR PERTURB", 0);

  clbm_run_desc d{};
  d.width = st.Dx;
  d.height = st.Dy;
  d.xmin = st.xmin;
  d.xmax = st.xmax;
  d.ymin = st.ymin;
  d.ymax = st.ymax;
  d.nclones = in.nc;
  d.ranks = o.ranks;
  d.tau = in.tau;
  d.beta = st.beta0;
  d.alpha = in.alpha;
  d.force_scale = st.oneOvF0;
  d.force_shift = o.zero_mean ? 1.775 : 0.0;
  d.dt = st.delta_t;
  d.perturb_mode = CLBM_PERTURB_MIX;
  d.nsnap = NN;
  d.eps = in.eps;
  d.resample_mode = CLBM_RESAMPLE_REFERENCE;
  clbm_ctx *ctx = nullptr;
  int s = clbm_create(&d, 1, o.precision, st.steps2, 0, &ctx);
  if (s) return die(log, "clbm_create", s);
  if (o.reconstruct && (s = clbm_enable_history(ctx, st.intervals))) return die(log, "history", s);
  if ((s = clbm_load_run_aos_f64(ctx, 0, states.data())) ||
      (s = clbm_set_snapshots_aos_f64(ctx, 0, NN, snaps.data())))
    return die(log, "loading states", s);
  if ((s = tune(ctx))) return die(log, "autotune", s);

  std::vector<double> drag((size_t)in.nc * st.steps2), rrec(st.intervals);
  std::vector<int> labels(in.nc), post(in.nc);
  for (int t = 0; t < st.intervals; t++) {
    log.line("This is cloning step " + std::to_string(t));
    if ((s = clbm_run_interval(ctx, st.steps2)) || (s = clbm_get_drag(ctx, 0, drag.data())))
      return die(log, "interval", s);
    for (int j = 0; j < in.nc; j++)
      append_binary(clone_dir(in.parent, j) + "data_force.datout", &drag[(size_t)j * st.steps2],
                    sizeof(double) * st.steps2);
    if ((s = clbm_clone_step(ctx)) ||
        (s = clbm_get_clone_result(ctx, 0, labels.data(), &rrec[t], nullptr, nullptr, post.data())))
      return die(log, "cloning step", s);
    std::string line = "    nbCreatedCopies : ";
    for (int j = 0; j < in.nc; j++) line += std::to_string(j) + "|" + std::to_string(post[j]) + " ";
    log.line(line);
    append_binary(labels_file, labels.data(), sizeof(int) * in.nc);
  }
  write_binary(in.parent + "rvalues.dat", rrec.data(), sizeof(double) * st.intervals);
  if (o.reconstruct) {
    int n = 0;
    std::vector<double> lin((size_t)in.nc * st.intervals * st.steps2);
    if ((s = clbm_reconstruct_lineages(ctx, 0, &n, lin.data(), nullptr))) return die(log, "reconstruction", s);
    const std::string dir = in.parent + "reconstructed/";
    make_dir(dir);
    for (int j = 0; j < in.nc; j++) {
      make_dir(clone_dir(dir, j));
      write_binary(clone_dir(dir, j) + "data_force.datout", &lin[(size_t)j * n * st.steps2],
                   sizeof(double) * (size_t)n * st.steps2);
    }
  }
  clbm_destroy(ctx);
  return 0;
}

// Forcing driver (src/mpi_LBM_GK_forcing.cpp): every clone draws a Gaussian
// random field at the start of each interval and runs lbmTimeSteps1 steps
// under beta(x,y) = (1 + eps map(x,y)) beta0, then lbmTimeSteps2 plain steps
// (:333-395); no ZERO_MEAN shift, no perturbation of copies.  Outputs:
// clone_<j>/evolution_<t>_clone_<j> (F/F0 every step), weights_evolution_<t>
// (Nc doubles), copies_evolution_<t> (Nc int32 drawn, Nc int32 corrected),
// rvalues.dat.  The fields come from a counter-based stream instead of
// rand() (--seed S), so they are statistically, not bitwise, the reference's.
int run_forcing(const Opts &o) {
  Log log("output_TLGK.out");
  Input in = read_input_forcing(o.input);
  if (!in.ok) return die(log, "COULD NOT OPEN INPUT FILE " + o.input, 0);
  const Setup st = setup_from(in, true);
  if (o.ranks < 1 || in.nc % o.ranks) return die(log, "Nc must be a multiple of --ranks", 0);
  const int T = st.steps1 + st.steps2;
  if (T < 1 || st.intervals < 1 || st.steps1 < 0 || st.steps2 < 0)
    return die(log, "no LB step or no cloning step to run", 0);
  log.line("READ input file");
  log.line("  Nc = " + std::to_string(in.nc) + " L = " + std::to_string(in.L) + " Dx = " + std::to_string(st.Dx));
  make_dir(in.parent);
  for (int j = 0; j < in.nc; j++) make_dir(in.parent + "clone_" + std::to_string(j));
  const size_t n = 9 * (size_t)st.Dx * st.Dy;
  std::vector<std::string> names;
  if (!read_list(in.path + "popfiles_list.dat", names, in.nc))
    return die(log, "COULD NOT OPEN INDEX FILE " + in.path + "popfiles_list.dat", 0);
  const int local = in.nc / o.ranks;
  std::vector<double> states(n * in.nc);
  for (int j = 0; j < in.nc; j++) {
    const int name_idx = (j >= local) ? j - local : in.nc - local + j;
    if (!read_pops(in.path + names[name_idx], states, n, n * j))
      return die(log, "could not read popfile " + names[name_idx], 0);
  }
  clbm_run_desc d{};
  d.width = st.Dx;
  d.height = st.Dy;
  d.xmin = st.xmin;
  d.xmax = st.xmax;
  d.ymin = st.ymin;
  d.ymax = st.ymax;
  d.nclones = in.nc;
  d.ranks = o.ranks;
  d.tau = in.tau;
  d.beta = st.beta0;
  d.alpha = in.alpha;
  d.force_scale = st.oneOvF0;
  d.force_shift = 0.0;
  d.dt = st.delta_t;
  d.perturb_mode = CLBM_PERTURB_NONE;
  d.resample_mode = CLBM_RESAMPLE_REFERENCE;
  d.seed = o.seed;
  d.field_mode = 1;
  d.field_steps = st.steps1;
  d.field_eps = in.eps;
  d.field_sigma = 32.0;
  clbm_ctx *ctx = nullptr;
  int s = clbm_create(&d, 1, o.precision, T, 0, &ctx);
  if (s) return die(log, "clbm_create", s);
  if ((s = clbm_load_run_aos_f64(ctx, 0, states.data()))) return die(log, "loading states", s);
  if ((s = tune(ctx))) return die(log, "autotune", s);
  std::vector<double> drag((size_t)in.nc * T), rrec(st.intervals), w(in.nc);
  std::vector<int> pre(in.nc), post(in.nc);
  for (int t = 0; t < st.intervals; t++) {
    log.line("    This is cloning step " + std::to_string(t));
    if ((s = clbm_run_interval(ctx, T)) || (s = clbm_get_drag(ctx, 0, drag.data())))
      return die(log, "interval", s);
    if (t == 0) {
      int neg = 0;
      clbm_get_field_map(ctx, 0, 0, nullptr, &neg);
      if (neg) log.line("  random field: " + std::to_string(neg) + " negative embedding eigenvalues set to 0");
    }
    for (int j = 0; j < in.nc; j++)
      write_binary(in.parent + "clone_" + std::to_string(j) + "/evolution_" + std::to_string(t) + "_clone_" +
                       std::to_string(j),
                   &drag[(size_t)j * T], sizeof(double) * T);
    if ((s = clbm_clone_step(ctx)) ||
        (s = clbm_get_clone_result(ctx, 0, nullptr, &rrec[t], w.data(), pre.data(), post.data())))
      return die(log, "cloning step", s);
    write_binary(in.parent + "weights_evolution_" + std::to_string(t), w.data(), sizeof(double) * in.nc);
    std::vector<int> cp(pre);
    cp.insert(cp.end(), post.begin(), post.end());
    write_binary(in.parent + "copies_evolution_" + std::to_string(t), cp.data(), sizeof(int) * cp.size());
  }
  write_binary(in.parent + "rvalues.dat", rrec.data(), sizeof(double) * st.intervals);
  clbm_destroy(ctx);
  return 0;
}

// Plain driver (src/mpi_LBM_GK.cpp): hard-coded Nc = 2, T = dT = 1,
// alpha = 0.04 (:39-41, :61), parameters L tau Ma t0 from input_LBM.datin
// (:48-53), every clone starting from one control-run state (:133-149), drag
// not normalised (:192), no perturbation.  The reference's copy phase is
// broken (it copies pointers, :353); copies here are real.  Outputs (the
// reference writes none): labels.dat and rvalues.dat in the working directory.
int run_plain(const Opts &o) {
  Log log("output_TLGK.out");
  const std::string params = "input_LBM.datin";
  FILE *f = std::fopen(params.c_str(), "r");
  int L = 0;
  double tau = 1.0, Ma = 1.0, t0 = 1.0;
  if (!f || std::fscanf(f, "%d %lf %lf %lf", &L, &tau, &Ma, &t0) != 4) {
    if (f) std::fclose(f);
    return die(log, "could not read " + params, 0);
  }
  std::fclose(f);
  const int Nc = 2;
  const double T = 1, dT = 1, alpha = 0.04;
  const int Dy = 4 * L + 1, Dx = Dy;
  const int xmin = (Dx - 1) / 2, xmax = xmin + L, ymin = (Dy - 1) / 2 - L / 2, ymax = ymin + L;
  const double cs = 1. / std::sqrt(3);
  const double nu = 1. / 3. * (tau - 0.5);
  const double u0 = cs * cs * Ma;
  const double beta0 = 8 * nu * u0 / ((Dy - 1) / 2) / ((Dy - 1) / 2);
  const double delta_t = 1.0 / t0;
  const int steps = (int)std::floor(dT / delta_t);
  const int intervals = (int)std::floor(T / dT);
  const size_t n = 9 * (size_t)Dx * Dy;
  std::vector<double> one(n), states(n * Nc);
  const std::string ctrl = o.input.empty() ? "pops.datout" : o.input;
  if (!read_pops(ctrl, one, n, 0)) return die(log, "could not read control-run state " + ctrl, 0);
  for (int j = 0; j < Nc; j++) std::memcpy(&states[n * j], one.data(), n * sizeof(double));
  clbm_run_desc d{};
  d.width = Dx;
  d.height = Dy;
  d.xmin = xmin;
  d.xmax = xmax;
  d.ymin = ymin;
  d.ymax = ymax;
  d.nclones = Nc;
  d.ranks = 1;
  d.tau = tau;
  d.beta = beta0;
  d.alpha = alpha;
  d.force_scale = 1.0;
  d.force_shift = 0.0;
  d.dt = delta_t;
  d.perturb_mode = CLBM_PERTURB_NONE;
  d.resample_mode = CLBM_RESAMPLE_REFERENCE;
  if (steps < 1) return die(log, "t0 gives no LB step", 0);
  clbm_ctx *ctx = nullptr;
  int s = clbm_create(&d, 1, o.precision, steps, 0, &ctx);
  if (s) return die(log, "clbm_create", s);
  if ((s = clbm_load_run_aos_f64(ctx, 0, states.data()))) return die(log, "loading states", s);
  if ((s = tune(ctx))) return die(log, "autotune", s);
  std::vector<double> rrec(intervals);
  std::vector<int> labels(Nc);
  write_binary("labels.dat", nullptr, 0);
  for (int t = 0; t < intervals; t++) {
    if ((s = clbm_run_interval(ctx, steps)) || (s = clbm_clone_step(ctx)) ||
        (s = clbm_get_clone_result(ctx, 0, labels.data(), &rrec[t], nullptr, nullptr, nullptr)))
      return die(log, "interval", s);
    append_binary("labels.dat", labels.data(), sizeof(int) * Nc);
  }
  write_binary("rvalues.dat", rrec.data(), sizeof(double) * intervals);
  clbm_destroy(ctx);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  const Opts o = parse(argc, argv);
#if defined(CLBM_VARIANT_POPS)
  if (o.input.empty()) {
    std::fprintf(stderr, "usage: TLGK_LBM_POPS_PERTURB [--ranks P] [--fp32] [--no-zero-mean] inputfile\n");
    return 2;
  }
  return run_pops(o);
#elif defined(CLBM_VARIANT_PLAIN)
  return run_plain(o);
#else
  if (o.input.empty()) {
    std::fprintf(stderr, "usage: TLGK_LBM_FORCING [--ranks P] [--fp32] [--seed S] inputfile\n");
    return 2;
  }
  return run_forcing(o);
#endif
}
