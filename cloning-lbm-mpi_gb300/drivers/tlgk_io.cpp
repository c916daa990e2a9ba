// tlgk_io.cpp -- input parsing, set-up scalars and binary outputs of the
// drop-in drivers (the reference's file-level interface).
#include "tlgk_io.h"

#include <sys/stat.h>
#include <sys/types.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <fstream>

namespace tlgk {

Input read_input_pops(const std::string &file) {
  Input in;
  std::ifstream f(file);
  if (!f.is_open()) return in;
  f >> in.nc >> in.T >> in.dT >> in.eps >> in.L >> in.tau >> in.U0 >> in.alpha >> in.path >>
      in.parent >> in.facquVTK;
  in.ok = !in.parent.empty();
  return in;
}

Input read_input_forcing(const std::string &file) {
  Input in;
  std::ifstream f(file);
  if (!f.is_open()) return in;
  f >> in.nc >> in.T >> in.dT >> in.dT0 >> in.eps >> in.L >> in.tau >> in.U0 >> in.alpha >>
      in.path >> in.parent;
  in.ok = !in.parent.empty();
  return in;
}

Setup setup_from(const Input &in, bool forcing) {
  Setup s{};
  const int L = in.L;
  s.Dy = 4 * L + 1;
  s.Dx = s.Dy;
  s.xmin = (s.Dx - 1) / 2;
  s.xmax = s.xmin + L;
  s.ymin = (s.Dy - 1) / 2 - L / 2;
  s.ymax = s.ymin + L;
  s.beta0 = (1. / (s.Dx - 1)) * ((double)L / (s.Dy - 1)) * in.U0 * in.U0;
  s.T0 = L / in.U0;
  s.F0 = (in.U0 * in.U0) * L * 0.5;
  s.oneOvF0 = 1. / s.F0;
  s.delta_t = 1.0 / s.T0;
  s.intervals = (int)std::floor(in.T / in.dT);
  if (forcing) {
    s.steps1 = (int)std::floor(in.dT0 * s.T0);
    s.steps2 = (int)std::floor((in.dT - in.dT0) * s.T0);
  } else {
    s.steps1 = 0;
    s.steps2 = (int)std::floor(in.dT * s.T0);
  }
  return s;
}

bool read_list(const std::string &path, std::vector<std::string> &names, int need) {
  std::ifstream f(path);
  if (!f.is_open()) return false;
  names.clear();
  std::string s;
  while ((int)names.size() < need && f >> s) names.push_back(s);
  return (int)names.size() >= need;
}

bool read_pops(const std::string &file, std::vector<double> &dst, size_t n, size_t offset) {
  std::ifstream f(file, std::ios::binary);
  if (!f.is_open()) return false;
  f.read(reinterpret_cast<char *>(dst.data() + offset), (std::streamsize)(n * sizeof(double)));
  return (size_t)f.gcount() == n * sizeof(double);
}

bool make_dir(const std::string &dir) {
  if (mkdir(dir.c_str(), 0755) == 0) return true;
  return errno == EEXIST;
}

bool append_binary(const std::string &file, const void *data, size_t bytes) {
  std::ofstream f(file, std::ios::binary | std::ios::app);
  if (!f.is_open()) return false;
  f.write(static_cast<const char *>(data), (std::streamsize)bytes);
  return f.good();
}

bool write_binary(const std::string &file, const void *data, size_t bytes) {
  std::ofstream f(file, std::ios::binary | std::ios::trunc);
  if (!f.is_open()) return false;
  f.write(static_cast<const char *>(data), (std::streamsize)bytes);
  return f.good();
}

Log::Log(const std::string &file) { f = std::fopen(file.c_str(), "w"); }
Log::~Log() {
  if (f) std::fclose(static_cast<FILE *>(f));
}
void Log::line(const std::string &s) {
  std::fprintf(stdout, "%s\n", s.c_str());
  if (f) {
    std::fprintf(static_cast<FILE *>(f), "%s\n", s.c_str());
    std::fflush(static_cast<FILE *>(f));
  }
}

}  // namespace tlgk
