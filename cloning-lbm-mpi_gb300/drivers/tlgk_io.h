// tlgk_io.h -- file-level boundary of the drop-in drivers: the reference's
// positional input files, the popfile list, and its raw little-endian binary
// outputs, so that post_processing/ reads them unchanged.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace tlgk {

// Positional tokens read with >> (src/mpi_LBM_GK_pops_perturb.cpp:66-81,
// src/mpi_LBM_GK_forcing.cpp:62-76, input_TEMPLATE:1-11).
struct Input {
  int nc = 0;
  double T = 1.0, dT = 1.0, dT0 = 1.0, eps = 1.0;
  int L = 0;
  double tau = 1.0, U0 = 1.0, alpha = 1.0;
  std::string path, parent;
  int facquVTK = 0;
  bool ok = false;
};
Input read_input_pops(const std::string &file);     // Nc T dT eps L tau U0 alpha path parent facquVTK
Input read_input_forcing(const std::string &file);  // Nc T dT dT0 eps L tau U0 alpha path parent

// Geometry and scalars exactly as the drivers derive them from L and U0
// (pops driver :131-151, forcing :125-144).
struct Setup {
  int Dx, Dy, xmin, xmax, ymin, ymax;
  double beta0, T0, F0, oneOvF0, delta_t;
  int steps2, steps1, intervals;
};
Setup setup_from(const Input &in, bool forcing);

// popfiles_list.dat names (pops driver :251-310, :321-364)
bool read_list(const std::string &path, std::vector<std::string> &names, int need);
bool read_pops(const std::string &file, std::vector<double> &dst, size_t n, size_t offset);

bool make_dir(const std::string &dir);
bool append_binary(const std::string &file, const void *data, size_t bytes);
bool write_binary(const std::string &file, const void *data, size_t bytes);

// output_TLGK.out, the run log (pops driver :88)
struct Log {
  explicit Log(const std::string &file);
  ~Log();
  void line(const std::string &s);
  void *f;
};

}  // namespace tlgk
