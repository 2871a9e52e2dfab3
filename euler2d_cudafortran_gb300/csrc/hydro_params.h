// hydro_params.h -- the derived parameters of a run, on the host.
#pragma once
#include "../../include/euler2d_gb300.h"
#include "physics.cuh"

namespace e2d {

// Derived parameters exactly as serial_ref/m_run.f90:95-124 evaluates them in
// fp_kind (xmin=0, xmax=1), one rounding per operation (host code is built
// with -ffp-contract=off), plus the loop invariants gm1, entho and smallc2
// formed with the reference's own expressions.
template <typename Real>
inline Hydro<Real> make_hydro(const e2d_params& p) {
  Hydro<Real> h;
  const Real xmin = Real(0.0), xmax = Real(1.0);
  h.nx = p.nx;
  h.ny = p.ny;
  h.isize = p.nx + 4;
  h.jsize = p.ny + 4;
  h.dx = (xmax - xmin) / (Real)p.nx;
  h.dy = (xmax - xmin) / (Real)p.ny;
  h.gamma0 = (Real)p.gamma0;
  h.cfl = (Real)p.cfl;
  h.smallr = (Real)p.smallr;
  h.smallc = (Real)p.smallc;
  h.niter_riemann = p.niter_riemann;
  h.slope_type = p.slope_type;
  h.smallp = h.smallc * h.smallc / h.gamma0;
  h.smallpp = h.smallr * h.smallp;
  h.gamma6 = (h.gamma0 + Real(1.0)) / (Real(2.0) * h.gamma0);
  h.gm1 = h.gamma0 - Real(1.0);                 // eos, serial_ref/m_utils.f90:26
  h.entho = Real(1.0) / (h.gamma0 - Real(1.0));  // cmpflx :521, riemann_2d_hllc :560
  h.smallc2 = h.smallc * h.smallc;               // riemann_2d_hllc :584-585
  h.bc_xmin = p.boundary_type_xmin;
  h.bc_xmax = p.boundary_type_xmax;
  h.bc_ymin = p.boundary_type_ymin;
  h.bc_ymax = p.boundary_type_ymax;
  h.riemann = p.riemann_solver;
  return h;
}

}  // namespace e2d
