// namelist.h -- reader for the reference's Fortran namelist parameter file.
//
// Groups and keys follow serial_ref/m_run.f90:71-73 (&RUN, &MESH, &HYDRO),
// the cuf variant's &OTHER implementationVersion (cuf/m_HydroParameters.cuf:90)
// and a trailing &GB300 group (riemann_solver = 'approx' | 'hllc',
// precision = 8 | 4) that the reference binaries never read: Fortran reads
// namelist groups by name, in file order, so the extra group is harmless.
#pragma once
#include <string>

#include "euler2d_gb300.h"

struct RunConfig {
  double tEnd = 0.0;
  int nStepmax = 0;
  int nOutput = 1;
  e2d_params p;
};

// Returns an empty string on success, else the error text.
std::string read_namelist(const std::string& path, RunConfig* cfg);
