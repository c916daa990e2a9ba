#include "vtk.h"

#include <fstream>

namespace tlgk {

bool write_fluid_vtk(const std::string &file, int Dx, int Dy, const double *rho, const double *ux,
                     const double *uy) {
  std::ofstream o(file);
  if (!o.is_open()) return false;
  o << "# vtk DataFile Version 3.0\nfluid_state\nASCII\nDATASET RECTILINEAR_GRID\n";
  o << "DIMENSIONS " << Dx << " " << Dy << " 1\n";
  o << "X_COORDINATES " << Dx << " float\n";
  for (int i = 0; i < Dx; ++i) o << i << " ";
  o << "\nY_COORDINATES " << Dy << " float\n";
  for (int j = 0; j < Dy; ++j) o << j << " ";
  o << "\nZ_COORDINATES 1 float\n0\n";
  o << "POINT_DATA " << Dx * Dy << "\n";
  o << "SCALARS density float 1\nLOOKUP_TABLE default\n";
  for (int y = 0; y < Dy; ++y)
    for (int x = 0; x < Dx; ++x) o << rho[y + Dy * x] - 1.0 << "\n";
  o << "VECTORS velocity_vector float\n";
  for (int y = 0; y < Dy; ++y)
    for (int x = 0; x < Dx; ++x) o << ux[y + Dy * x] << " " << uy[y + Dy * x] << " 0\n";
  return o.good();
}

}  // namespace tlgk
