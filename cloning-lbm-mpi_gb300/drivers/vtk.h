// vtk.h -- ASCII rectilinear-grid VTK of rho - 1 and (ux, uy), the format of
// the reference's write_fluid_vtk (src/lbm_src/write_vtk.cpp:8-53); fields
// in the reference's node order y + Dy*x.
#pragma once
#include <string>

namespace tlgk {
bool write_fluid_vtk(const std::string &file, int Dx, int Dy, const double *rho, const double *ux,
                     const double *uy);
}
