// vtk.h -- state output in the VTK ImageData (.vti) format of the reference's
// saveVTK (serial_ref/m_run.f90:653-720): interior cells only, one CellData
// array per conservative variable.
#pragma once
#include <string>

// Writes euler2d_<iStep, 8 digits>.vti into dir.  data is the host state in
// the Fortran layout A(isize, jsize, 4) of doubles (es = 8) or floats (es = 4).
// ascii = true reproduces the reference's ASCII file; false writes the same
// arrays as appended raw binary (smaller and faster to write).
std::string save_vtk(const std::string& dir, int iStep, const void* data, int nx, int ny, int es, bool ascii);
