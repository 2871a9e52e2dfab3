// physics.cuh -- pointwise physics of the Euler-2D Godunov step, device side.
//
// Each routine states the serial_ref/m_utils.f90 routine it computes, with the
// same operations in the same order (Fortran's left-to-right association
// written as explicit parentheses).  The library is compiled with -fmad=false
// and IEEE division / square root, so every operation rounds exactly as the
// reference's double (or single) precision build does, and results are
// bitwise identical to it.
//
// Real = double (fp_kind = dp_kind) or float (fp_kind = sp_kind).  Fortran
// default-real literals stay single precision in both builds:
//   1e-6 (Newton tolerance, serial_ref/m_utils.f90:396) and 0.14
//   (init_implode, serial_ref/m_run.f90:548).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace e2d {

enum { ID = 0, IP = 1, IU = 2, IV = 3 };  // serial_ref/m_constants.f90:11-14, 0-based
enum { FACE_XMIN = 0, FACE_XMAX = 1, FACE_YMIN = 2, FACE_YMAX = 3 };
constexpr int GW = 2;  // ghostWidth, serial_ref/m_run.f90:28

// type HydroPar (serial_ref/m_parameters.f90:10-36) in the working precision.
template <typename Real>
struct Hydro {
  Real gamma0, gamma6, cfl, smallr, smallc, smallp, smallpp, dx, dy;
  int slope_type, niter_riemann, nx, ny, isize, jsize;
  int bc_xmin, bc_xmax, bc_ymin, bc_ymax, riemann;
};

// A pitched structure-of-arrays state: 4 planes of jsize rows of `pitch`
// elements; element (i, j, v) (0-based) at v*plane + j*pitch + i.
template <typename Real>
struct Field {
  Real* p;
  int pitch;
  long long plane;
  __host__ __device__ __forceinline__ Real& at(int v, int j, int i) const {
    return p[(long long)v * plane + (long long)j * pitch + i];
  }
};

template <typename Real> __device__ __forceinline__ Real rmax(Real a, Real b) { return fmax(a, b); }
template <typename Real> __device__ __forceinline__ Real rmin(Real a, Real b) { return fmin(a, b); }
template <typename Real> __device__ __forceinline__ Real rabs(Real a) { return fabs(a); }
template <typename Real> __device__ __forceinline__ Real rsqrt_ieee(Real a) { return sqrt(a); }

// eos + computePrimitives, serial_ref/m_utils.f90:15-29 and 35-64, without the
// sound speed (unused by every caller except compute_dt).
template <typename Real>
__device__ __forceinline__ void primitives(const Hydro<Real>& h, const Real u[4], Real q[4]) {
  q[ID] = rmax(u[ID], h.smallr);
  q[IU] = u[IU] / q[ID];
  q[IV] = u[IV] / q[ID];
  const Real eken = Real(0.5) * ((q[IU] * q[IU]) + (q[IV] * q[IV]));
  const Real e = (u[IP] / q[ID]) - eken;
  q[IP] = rmax(((h.gamma0 - Real(1.0)) * q[ID]) * e, q[ID] * h.smallp);
}

// Sound speed of eos (serial_ref/m_utils.f90:27) from primitive q.
template <typename Real>
__device__ __forceinline__ Real sound_speed(const Hydro<Real>& h, const Real q[4]) {
  return rsqrt_ieee((h.gamma0 * q[IP]) / q[ID]);
}

// The compute_dt term of one cell, serial_ref/m_run.f90:278-281.
template <typename Real>
__device__ __forceinline__ Real cell_invdt(const Hydro<Real>& h, const Real u[4]) {
  Real q[4];
  primitives(h, u, q);
  const Real c = sound_speed(h, q);
  const Real vx = c + rabs(q[IU]);
  const Real vy = c + rabs(q[IV]);
  return (vx / h.dx) + (vy / h.dy);
}

// One direction of slope_unsplit_hydro_2d, serial_ref/m_utils.f90:300-312.
template <typename Real>
__device__ __forceinline__ Real slope1(Real st, Real q, Real qp, Real qm) {
  const Real dlft = st * (q - qm);
  const Real drgt = st * (qp - q);
  const Real dcen = Real(0.5) * (qp - qm);
  const Real dsgn = (dcen >= Real(0.0)) ? Real(1.0) : Real(-1.0);
  const Real slop = rmin(rabs(dlft), rabs(drgt));
  const Real dlim = ((dlft * drgt) <= Real(0.0)) ? Real(0.0) : slop;
  return dsgn * rmin(dlim, rabs(dcen));
}

// slope_unsplit_hydro_2d, serial_ref/m_utils.f90:268-342.
template <typename Real>
__device__ __forceinline__ void slopes(const Hydro<Real>& h, const Real q[4], const Real qpx[4],
                                       const Real qmx[4], const Real qpy[4], const Real qmy[4],
                                       Real dqx[4], Real dqy[4]) {
  if (h.slope_type == 1 || h.slope_type == 2) {
    const Real st = Real(h.slope_type);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      dqx[v] = slope1(st, q[v], qpx[v], qmx[v]);
      dqy[v] = slope1(st, q[v], qpy[v], qmy[v]);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) { dqx[v] = Real(0.0); dqy[v] = Real(0.0); }
  }
}

// Source terms of trace_unsplit_2d_along_dir, serial_ref/m_utils.f90:213-216.
// They depend on the cell only, so a cell computes them once for its 4 faces.
template <typename Real>
__device__ __forceinline__ void trace_sources(const Hydro<Real>& h, const Real q[4], const Real dqx[4],
                                              const Real dqy[4], Real s[4]) {
  const Real r = q[ID], p = q[IP], u = q[IU], v = q[IV];
  s[ID] = ((-(u * dqx[ID])) - (v * dqy[ID])) - ((dqx[IU] + dqy[IV]) * r);
  s[IP] = ((-(u * dqx[IP])) - (v * dqy[IP])) - (((dqx[IU] + dqy[IV]) * h.gamma0) * p);
  s[IU] = ((-(u * dqx[IU])) - (v * dqy[IU])) - (dqx[IP] / r);
  s[IV] = ((-(u * dqx[IV])) - (v * dqy[IV])) - (dqy[IP] / r);
}

// Face state of trace_unsplit_2d_along_dir, serial_ref/m_utils.f90:218-252:
// qf = (q -/+ 0.5*dq_dir) + (s*dtd)*0.5, then rho floored at smallr.
// sign = -1 for the XMIN/YMIN faces, +1 for XMAX/YMAX; dq is the slope along
// the face normal, dtd = dtdx or dtdy.
template <typename Real, bool PLUS>
__device__ __forceinline__ void trace_face(const Hydro<Real>& h, const Real q[4], const Real dq[4],
                                           const Real s[4], Real dtd, Real qf[4]) {
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const Real a = PLUS ? (q[v] + (Real(0.5) * dq[v])) : (q[v] - (Real(0.5) * dq[v]));
    qf[v] = a + ((s[v] * dtd) * Real(0.5));
  }
  qf[ID] = rmax(h.smallr, qf[ID]);
}

// cmpflx, serial_ref/m_utils.f90:498-526.
template <typename Real>
__device__ __forceinline__ void cmpflx(const Hydro<Real>& h, const Real qg[4], Real flux[4]) {
  flux[ID] = qg[ID] * qg[IU];
  flux[IU] = (flux[ID] * qg[IU]) + qg[IP];
  flux[IV] = flux[ID] * qg[IV];
  const Real entho = Real(1.0) / (h.gamma0 - Real(1.0));
  const Real ekin = (Real(0.5) * qg[ID]) * ((qg[IU] * qg[IU]) + (qg[IV] * qg[IV]));
  const Real etot = (qg[IP] * entho) + ekin;
  flux[IP] = qg[IU] * (etot + qg[IP]);
}

// riemann_2d (two-shock approximate solver + cmpflx), serial_ref/m_utils.f90:349-492.
template <typename Real>
__device__ __forceinline__ void riemann_approx(const Hydro<Real>& h, const Real qleft[4],
                                               const Real qright[4], Real flux[4]) {
  const Real ONE = Real(1.0), ZERO = Real(0.0), H = Real(0.5);
  const Real tol = Real(1e-6f);
  const Real rl = rmax(qleft[ID], h.smallr);
  const Real ul = qleft[IU];
  const Real pl = rmax(qleft[IP], rl * h.smallp);
  const Real rr = rmax(qright[ID], h.smallr);
  const Real ur = qright[IU];
  const Real pr = rmax(qright[IP], rr * h.smallp);
  const Real cl = (h.gamma0 * pl) * rl;
  const Real cr = (h.gamma0 * pr) * rr;
  Real wl = rsqrt_ieee(cl);
  Real wr = rsqrt_ieee(cr);
  Real pold = rmax((((wr * pl) + (wl * pr)) + ((wl * wr) * (ul - ur))) / (wl + wr), ZERO);
  Real conv = ONE;
  int iter = 0;
  while (iter < h.niter_riemann && conv > tol) {
    const Real wwl = rsqrt_ieee(cl * (ONE + ((h.gamma6 * (pold - pl)) / pl)));
    const Real wwr = rsqrt_ieee(cr * (ONE + ((h.gamma6 * (pold - pr)) / pr)));
    const Real ql = (((Real(2.0) * wwl) * wwl) * wwl) / ((wwl * wwl) + cl);
    const Real qr = (((Real(2.0) * wwr) * wwr) * wwr) / ((wwr * wwr) + cr);
    const Real usl = ul - ((pold - pl) / wwl);
    const Real usr = ur + ((pold - pr) / wwr);
    const Real delp = rmax(((qr * ql) / (qr + ql)) * (usl - usr), -pold);
    pold = pold + delp;
    conv = rabs(delp / (pold + h.smallpp));
    iter = iter + 1;
  }
  const Real pstar = pold;
  wl = rsqrt_ieee(cl * (ONE + ((h.gamma6 * (pstar - pl)) / pl)));
  wr = rsqrt_ieee(cr * (ONE + ((h.gamma6 * (pstar - pr)) / pr)));
  const Real ustar = H * ((((ul + ((pl - pstar) / wl)) + ur) - ((pr - pstar) / wr)));
  const Real sgnm = (ustar >= ZERO) ? ONE : -ONE;
  Real ro, uo, po, wo;
  if (sgnm > ZERO) { ro = rl; uo = ul; po = pl; wo = wl; }
  else             { ro = rr; uo = ur; po = pr; wo = wr; }
  const Real co = rmax(h.smallc, rsqrt_ieee(rabs((h.gamma0 * po) / ro)));
  const Real rstar = rmax(ro / (ONE + ((ro * (po - pstar)) / (wo * wo))), h.smallr);
  const Real cstar = rmax(h.smallc, rsqrt_ieee(rabs((h.gamma0 * pstar) / rstar)));
  Real spout = co - (sgnm * uo);
  Real spin = cstar - (sgnm * ustar);
  const Real ushock = (wo / ro) - (sgnm * uo);
  if (pstar >= po) { spin = ushock; spout = ushock; }
  const Real scr = rmax(spout - spin, h.smallc + rabs(spout + spin));
  const Real frac = H * (ONE + ((spout + spin) / scr));
  Real qg[4];
  qg[ID] = (frac * rstar) + ((ONE - frac) * ro);
  qg[IU] = (frac * ustar) + ((ONE - frac) * uo);
  qg[IP] = (frac * pstar) + ((ONE - frac) * po);
  if (spout < ZERO) { qg[ID] = ro; qg[IU] = uo; qg[IP] = po; }
  if (spin > ZERO) { qg[ID] = rstar; qg[IU] = ustar; qg[IP] = pstar; }
  qg[IV] = (sgnm > ZERO) ? qleft[IV] : qright[IV];
  cmpflx(h, qg, flux);
}

// riemann_2d_hllc, serial_ref/m_utils.f90:534-644 (rcsum, unused there, is not formed).
template <typename Real>
__device__ __forceinline__ void riemann_hllc(const Hydro<Real>& h, const Real qleft[4],
                                             const Real qright[4], Real flux[4]) {
  const Real ONE = Real(1.0), ZERO = Real(0.0), H = Real(0.5);
  const Real entho = ONE / (h.gamma0 - ONE);
  const Real rl = rmax(qleft[ID], h.smallr);
  const Real pl = rmax(qleft[IP], rl * h.smallp);
  const Real ul = qleft[IU];
  Real ecinl = ((H * rl) * ul) * ul;
  ecinl = ecinl + (((H * rl) * qleft[IV]) * qleft[IV]);
  const Real etotl = (pl * entho) + ecinl;
  const Real ptotl = pl;
  const Real rr = rmax(qright[ID], h.smallr);
  const Real pr = rmax(qright[IP], rr * h.smallp);
  const Real ur = qright[IU];
  Real ecinr = ((H * rr) * ur) * ur;
  ecinr = ecinr + (((H * rr) * qright[IV]) * qright[IV]);
  const Real etotr = (pr * entho) + ecinr;
  const Real ptotr = pr;
  const Real cfastl = rsqrt_ieee(rmax((h.gamma0 * pl) / rl, h.smallc * h.smallc));
  const Real cfastr = rsqrt_ieee(rmax((h.gamma0 * pr) / rr, h.smallc * h.smallc));
  const Real SL = rmin(ul, ur) - rmax(cfastl, cfastr);
  const Real SR = rmax(ul, ur) + rmax(cfastl, cfastr);
  const Real rcl = rl * (ul - SL);
  const Real rcr = rr * (SR - ur);
  const Real ustar = (((rcr * ur) + (rcl * ul)) + (ptotl - ptotr)) / (rcr + rcl);
  const Real ptotstar = (((rcr * ptotl) + (rcl * ptotr)) + ((rcl * rcr) * (ul - ur))) / (rcr + rcl);
  Real ro, uo, ptoto, etoto;
  if (SL > ZERO) {
    ro = rl; uo = ul; ptoto = ptotl; etoto = etotl;
  } else if (ustar > ZERO) {
    ro = (rl * (SL - ul)) / (SL - ustar);
    uo = ustar; ptoto = ptotstar;
    etoto = ((((SL - ul) * etotl) - (ptotl * ul)) + (ptotstar * ustar)) / (SL - ustar);
  } else if (SR > ZERO) {
    ro = (rr * (SR - ur)) / (SR - ustar);
    uo = ustar; ptoto = ptotstar;
    etoto = ((((SR - ur) * etotr) - (ptotr * ur)) + (ptotstar * ustar)) / (SR - ustar);
  } else {
    ro = rr; uo = ur; ptoto = ptotr; etoto = etotr;
  }
  flux[ID] = ro * uo;
  flux[IU] = ((ro * uo) * uo) + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = (flux[ID] > ZERO) ? (flux[ID] * qleft[IV]) : (flux[ID] * qright[IV]);
}

template <typename Real>
__device__ __forceinline__ void riemann(const Hydro<Real>& h, const Real ql[4], const Real qr[4], Real flux[4]) {
  if (h.riemann == 2) riemann_hllc(h, ql, qr, flux);
  else riemann_approx(h, ql, qr, flux);
}

// Ordered-integer image of a non-negative float/double for atomicMax.
__device__ __forceinline__ unsigned long long ordered_bits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ unsigned int ordered_bits(float x) { return (unsigned int)__float_as_int(x); }

}  // namespace e2d
