// physics.cuh -- pointwise physics of the Euler-2D Godunov step, device side.
//
// Each routine states the serial_ref/m_utils.f90 routine it computes, with the
// same operations in the same order (Fortran's left-to-right association
// written as explicit parentheses).  The library is compiled with -fmad=false
// and IEEE division / square root, so every operation rounds exactly as the
// reference's double (or single) precision build does, and results are
// bitwise identical to it.
//
// The library's second build (-fmad=true, E2D_FMA=1) contracts multiply-adds
// and, where E2D_FMA_FORMS marks it, writes a few expressions in forms that
// fuse better (fewer FP64 instructions, different rounding), and rounds its
// double divisions and square roots faithfully: its results agree with
// serial_ref to the specified 1e-12 relative L1 and 1e-14 relative dt instead
// of bit for bit.
//
// Real = double (fp_kind = dp_kind) or float (fp_kind = sp_kind).  Fortran
// default-real literals stay single precision in both builds:
//   1e-6 (Newton tolerance, serial_ref/m_utils.f90:396) and 0.14
//   (init_implode, serial_ref/m_run.f90:548).
//
// Every division, square root, comparison, min/max, multiplication by 0.5 or
// 2 and sign flip goes through Ops<Real>.  For double these run on the
// integer and FP32 pipes (emul64.cuh) and return the same bits as the IEEE
// operations, which leaves the FP64 pipe -- the limit of this kernel on
// GB300 -- to the additions and multiplications.  Building with
// -DE2D_FP64_NATIVE selects the hardware FP64 operations instead.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "emul64.cuh"

#if defined(E2D_FMA) && E2D_FMA
#define E2D_FMA_FORMS 1
#else
#define E2D_FMA_FORMS 0
#endif
// The FMA build's division and square root are faithfully rounded (double:
// emul::div_fa, emul::sqrt_fa, a dozen fewer integer instructions on their
// dependent chains; float: emul::fdiv_fa, emul::fsqrt_fa, a correction of the
// hardware approximations by one fused residual): within one unit in the last
// place.  The exact build's round to nearest, as IEEE.
#ifndef E2D_FAITHFUL_DIVSQRT
#define E2D_FAITHFUL_DIVSQRT E2D_FMA_FORMS
#endif

namespace e2d {

// a*b + c rounded once.
__device__ __forceinline__ double fmx(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmx(float a, float b, float c) { return fmaf(a, b, c); }

enum { ID = 0, IP = 1, IU = 2, IV = 3 };  // serial_ref/m_constants.f90:11-14, 0-based
enum { FACE_XMIN = 0, FACE_XMAX = 1, FACE_YMIN = 2, FACE_YMAX = 3 };
constexpr int GW = 2;  // ghostWidth, serial_ref/m_run.f90:28

// type HydroPar (serial_ref/m_parameters.f90:10-36) in the working precision,
// plus three loop-invariant subexpressions of the reference evaluated once on
// the host with the same operations: gm1 = gamma0 - 1.0 (eos), entho =
// 1.0 / (gamma0 - 1.0) (cmpflx, riemann_2d_hllc), smallc2 = smallc * smallc.
template <typename Real>
struct Hydro {
  Real gamma0, gamma6, cfl, smallr, smallc, smallp, smallpp, dx, dy;
  Real gm1, entho, smallc2;
  int slope_type, niter_riemann, nx, ny, isize, jsize;
  int bc_xmin, bc_xmax, bc_ymin, bc_ymax, riemann;
};

template <typename Real> struct Ops;

// FP32: the hardware operations (the FP32 pipes are not the limit); in the
// FMA build, division and square root faithfully rounded (emul::fdiv_fa,
// emul::fsqrt_fa: shorter than the IEEE sequences, no slow path in range).
template <>
struct Ops<float> {
#if E2D_FAITHFUL_DIVSQRT
  static __device__ __forceinline__ float div(float a, float b) { return emul::fdiv_fa(a, b); }
  static __device__ __forceinline__ float sqrt(float a) { return emul::fsqrt_fa(a); }
#else
  static __device__ __forceinline__ float div(float a, float b) { return a / b; }
  static __device__ __forceinline__ float sqrt(float a) { return ::sqrtf(a); }
#endif
  static __device__ __forceinline__ float max(float a, float b) { return fmaxf(a, b); }
  static __device__ __forceinline__ float min(float a, float b) { return fminf(a, b); }
  static __device__ __forceinline__ bool gt0(float x) { return x > 0.0f; }
  static __device__ __forceinline__ bool ge0(float x) { return x >= 0.0f; }
  static __device__ __forceinline__ bool lt0(float x) { return x < 0.0f; }
  static __device__ __forceinline__ bool le0(float x) { return x <= 0.0f; }
  static __device__ __forceinline__ bool gt(float a, float b) { return a > b; }
  static __device__ __forceinline__ bool ge(float a, float b) { return a >= b; }
  static __device__ __forceinline__ float half(float x) { return 0.5f * x; }
  static __device__ __forceinline__ float twice(float x) { return 2.0f * x; }
  static __device__ __forceinline__ float neg_if(float x, bool n) { return n ? -x : x; }
};

#ifdef E2D_FP64_NATIVE
template <>
struct Ops<double> {
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ double sqrt(double a) { return ::sqrt(a); }
  static __device__ __forceinline__ double max(double a, double b) { return fmax(a, b); }
  static __device__ __forceinline__ double min(double a, double b) { return fmin(a, b); }
  static __device__ __forceinline__ bool gt0(double x) { return x > 0.0; }
  static __device__ __forceinline__ bool ge0(double x) { return x >= 0.0; }
  static __device__ __forceinline__ bool lt0(double x) { return x < 0.0; }
  static __device__ __forceinline__ bool le0(double x) { return x <= 0.0; }
  static __device__ __forceinline__ bool gt(double a, double b) { return a > b; }
  static __device__ __forceinline__ bool ge(double a, double b) { return a >= b; }
  static __device__ __forceinline__ double half(double x) { return 0.5 * x; }
  static __device__ __forceinline__ double twice(double x) { return 2.0 * x; }
  static __device__ __forceinline__ double neg_if(double x, bool n) { return n ? -x : x; }
};
#else
template <>
struct Ops<double> {
#if E2D_FAITHFUL_DIVSQRT
  static __device__ __forceinline__ double div(double a, double b) { return emul::div_fa(a, b); }
  static __device__ __forceinline__ double sqrt(double a) { return emul::sqrt_fa(a); }
#else
  static __device__ __forceinline__ double div(double a, double b) { return emul::div_rn(a, b); }
  static __device__ __forceinline__ double sqrt(double a) { return emul::sqrt_rn(a); }
#endif
  static __device__ __forceinline__ double max(double a, double b) { return emul::max_i(a, b); }
  static __device__ __forceinline__ double min(double a, double b) { return emul::min_i(a, b); }
  static __device__ __forceinline__ bool gt0(double x) { return emul::gt0(x); }
  static __device__ __forceinline__ bool ge0(double x) { return emul::ge0(x); }
  static __device__ __forceinline__ bool lt0(double x) { return emul::lt0(x); }
  static __device__ __forceinline__ bool le0(double x) { return emul::le0(x); }
  static __device__ __forceinline__ bool gt(double a, double b) { return emul::gt_i(a, b); }
  static __device__ __forceinline__ bool ge(double a, double b) { return emul::ge_i(a, b); }
  static __device__ __forceinline__ double half(double x) { return emul::half(x); }
  static __device__ __forceinline__ double twice(double x) { return emul::twice(x); }
  static __device__ __forceinline__ double neg_if(double x, bool n) { return emul::neg_if(x, n); }
};
#endif

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

// |a| (the sign bit cleared; for double on the integer pipe, like the other
// cheap operations of Ops<double>).
template <typename Real> __device__ __forceinline__ Real rabs(Real a) { return fabs(a); }
#ifndef E2D_FP64_NATIVE
template <> __device__ __forceinline__ double rabs<double>(double a) {
  return emul::from_bits(emul::bits(a) & 0x7fffffffffffffffull);
}
#endif

// max(a, b*c), the pressure floors of eos and the Riemann solvers (b a
// density, c = smallp).  For double, when a is a positive normal number with
// a >= 2^(ea-1023) >= 2^(eb+ec-2044) > b*c (ea, eb, ec the biased exponent
// fields; the bound holds for subnormal b or c too), the maximum is a whatever
// b*c rounds to, and the product is not formed: an exponent test on the
// integer pipe.  Other operands (a near the floor, zero, negative, NaN or
// infinite; b or c not finite) take the IEEE product and maximum.
#ifndef E2D_PFLOOR_EXP
#define E2D_PFLOOR_EXP 1
#endif
template <typename Real> __device__ __forceinline__ Real floor_prod(Real a, Real b, Real c) {
  return Ops<Real>::max(a, b * c);
}
#if !defined(E2D_FP64_NATIVE) && E2D_PFLOOR_EXP
template <> __device__ __forceinline__ double floor_prod<double>(double a, double b, double c) {
  const int ha = (int)(emul::bits(a) >> 32), hb = (int)(emul::bits(b) >> 32), hc = (int)(emul::bits(c) >> 32);
  const bool dominant = (unsigned)(ha - 0x00100000) < 0x7fe00000u && (unsigned)hb < 0x7ff00000u &&
                        (unsigned)hc < 0x7ff00000u && (ha >> 20) >= (hb >> 20) + (hc >> 20) - 1021;
  if (dominant) return a;
  return Ops<double>::max(a, b * c);
}
#endif

// The same maximum, also telling whether it returned a (the derivative then
// flows to a, else to b*c).
__device__ __forceinline__ double floor_pick(double a, double b, double c, bool& first) {
#if !defined(E2D_FP64_NATIVE) && E2D_PFLOOR_EXP
  const int ha = (int)(emul::bits(a) >> 32), hb = (int)(emul::bits(b) >> 32), hc = (int)(emul::bits(c) >> 32);
  if ((unsigned)(ha - 0x00100000) < 0x7fe00000u && (unsigned)hb < 0x7ff00000u && (unsigned)hc < 0x7ff00000u &&
      (ha >> 20) >= (hb >> 20) + (hc >> 20) - 1021) {
    first = true;
    return a;
  }
#endif
  const double bc = b * c;
  first = Ops<double>::gt(a, bc);
  return first ? a : bc;
}

// A new density that is not a positive finite number (the health check of the
// update; for double decided on the integer pipe).
__device__ __forceinline__ bool bad_density(float r) { return !(r > 0.0f) || !isfinite(r); }
__device__ __forceinline__ bool bad_density(double r) {
#ifdef E2D_FP64_NATIVE
  return !(r > 0.0) || !isfinite(r);
#else
  const long long b = (long long)emul::bits(r);
  return b <= 0 || b >= 0x7ff0000000000000ll;  // -0, negative, +0, or +inf / NaN
#endif
}

// eos + computePrimitives, serial_ref/m_utils.f90:15-29 and 35-64, without the
// sound speed (unused by every caller except compute_dt).
template <typename Real>
__device__ __forceinline__ void primitives(const Hydro<Real>& h, const Real u[4], Real q[4]) {
  using O = Ops<Real>;
  q[ID] = O::max(u[ID], h.smallr);
  q[IU] = O::div(u[IU], q[ID]);
  q[IV] = O::div(u[IV], q[ID]);
#if E2D_FMA_FORMS
  // a sum of two products written as one fused form, so that every kernel
  // rounds it alike (contraction alone may fuse either product); then
  // (gm1 rho) (E / rho - eken) as gm1 (E - rho eken): one fused form and a
  // product, no division
  const Real eken = O::half(fmx(q[IU], q[IU], q[IV] * q[IV]));
  q[IP] = floor_prod(h.gm1 * fmx(-q[ID], eken, u[IP]), q[ID], h.smallp);
#else
  const Real eken = O::half((q[IU] * q[IU]) + (q[IV] * q[IV]));
  const Real e = O::div(u[IP], q[ID]) - eken;
  q[IP] = floor_prod((h.gm1 * q[ID]) * e, q[ID], h.smallp);
#endif
}

// a and b the same number, bit for bit (an integer comparison).
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_int(a) == __float_as_int(b); }

// Sound speed of eos (serial_ref/m_utils.f90:27) from primitive q.
template <typename Real>
__device__ __forceinline__ Real sound_speed(const Hydro<Real>& h, const Real q[4]) {
  using O = Ops<Real>;
  return O::sqrt(O::div(h.gamma0 * q[IP], q[ID]));
}

// The compute_dt term of one cell, serial_ref/m_run.f90:278-281, from the
// cell's primitive variables q.
template <typename Real>
__device__ __forceinline__ Real cell_invdt_q(const Hydro<Real>& h, const Real q[4]) {
  using O = Ops<Real>;
  const Real c = sound_speed(h, q);
  const Real vx = c + rabs(q[IU]);
  const Real vy = c + rabs(q[IV]);
#if E2D_FMA_FORMS
  // square cells: (vx + vy) / dx as ((2c + |u|) + |v|) / dx, one division
  // and two additions (the FMA build's form)
  if (same_bits(h.dx, h.dy)) return O::div((O::twice(c) + rabs(q[IU])) + rabs(q[IV]), h.dx);
#endif
  return O::div(vx, h.dx) + O::div(vy, h.dy);
}

// The same from the conservative variables u.
template <typename Real>
__device__ __forceinline__ Real cell_invdt(const Hydro<Real>& h, const Real u[4]) {
  Real q[4];
  primitives(h, u, q);
  return cell_invdt_q(h, q);
}

// One direction of slope_unsplit_hydro_2d, serial_ref/m_utils.f90:300-312:
// dlft = st*(q-qm), drgt = st*(qp-q), dcen = 0.5*(qp-qm), dsgn = +-1 by
// dcen >= 0, dlim = 0 if dlft*drgt <= 0 else min(|dlft|,|drgt|), and the
// slope dsgn*min(dlim,|dcen|).  st is 1 or 2; the products by st, 0.5 and
// dsgn are exact scalings and sign flips.
template <typename Real>
__device__ __forceinline__ Real limiter_dlim(Real dlft, Real drgt, Real slop) {
  return Ops<Real>::le0(dlft * drgt) ? Real(0.0) : slop;
}

// dlft*drgt <= 0 for double, decided without the product: true when either
// factor is a zero or the signs differ; for same-sign nonzero normal factors
// with biased exponents ea, eb the exact product lies in
// [2^(ea+eb-2046), 2^(ea+eb-2044)), so it rounds to +0 when ea+eb <= 969 and
// to a nonzero value when ea+eb >= 972.  Exponent sums in between,
// subnormal factors, and infinite or NaN factors (0 * inf is NaN, and
// NaN <= 0 is false) set `amb`: the caller then takes the product.
#ifndef E2D_LIM_INT
#define E2D_LIM_INT 1
#endif
__device__ __forceinline__ bool prod_le0(double a, double b, bool& amb) {
#ifdef E2D_FP64_NATIVE
  return a * b <= 0.0;
#else
  const uint64_t ia = emul::bits(a), ib = emul::bits(b);
  const int ea = (int)(ia >> 52) & 0x7ff, eb = (int)(ib >> 52) & 0x7ff;
  const bool zero = ((ia << 1) == 0) | ((ib << 1) == 0);
  const bool neg = (int64_t)(ia ^ ib) < 0;
  const int e = ea + eb;
  amb |= (ea == 0x7ff) | (eb == 0x7ff) | (!zero & ((ea == 0) | (eb == 0) | ((unsigned)(e - 970) < 2u)));
  return zero | neg | (e <= 969);
#endif
}

// Limiter cases recorded for the adjoint (3 bits per slope): bits 0-1 the
// selection -- 0 limited to zero, 1 |dlft|, 2 |drgt|, 3 |dcen| -- and bit 2
// set when the selected one-sided difference has the sign opposite to dcen.
enum { LIM_ZERO = 0, LIM_LEFT = 1, LIM_RIGHT = 2, LIM_CENTRE = 3, LIM_FLIP = 4 };

template <typename Real, bool INT = false, bool CASE = false>
__device__ __forceinline__ Real slope1(bool mc, Real q, Real qp, Real qm, bool& amb, unsigned* cs = nullptr) {
  using O = Ops<Real>;
  const Real dl = q - qm, dr = qp - q;
  const Real dlft = mc ? O::twice(dl) : dl;
  const Real drgt = mc ? O::twice(dr) : dr;
  const Real dcen = O::half(qp - qm);
  const Real al = rabs(dlft), ar = rabs(drgt);
  const Real slop = O::min(al, ar);
  bool zero;
  if constexpr (INT) zero = prod_le0(dlft, drgt, amb);
  else zero = Ops<Real>::le0(dlft * drgt);
  const Real dlim = zero ? Real(0.0) : slop;
  const Real ac = rabs(dcen);
  if constexpr (CASE) {
    // the selections of O::min, which keeps its first argument when it is
    // strictly smaller (for double: in the integer order of emul::ord)
    const bool use_l = !O::ge(al, ar);
    const bool pick_slop = !O::ge(slop, ac);
    const Real x = use_l ? dlft : drgt;
    *cs = zero ? (unsigned)LIM_ZERO
               : pick_slop ? ((use_l ? (unsigned)LIM_LEFT : (unsigned)LIM_RIGHT) |
                              ((O::ge0(x) != O::ge0(dcen)) ? (unsigned)LIM_FLIP : 0u))
                           : (unsigned)LIM_CENTRE;
  }
  return O::neg_if(O::min(dlim, ac), !O::ge0(dcen));
}

// slope_unsplit_hydro_2d, serial_ref/m_utils.f90:268-342.  For double the
// limiter's sign test is decided from signs and exponents (prod_le0); a
// cell with a factor pair in the undecided band recomputes its slopes with
// the products, in a branch of its own -- a fallback product beside each
// test would be predicated into every path, and a predicated FP64
// instruction still takes its FP64 pipe slot.
// CASE: also return the limiter cases of the eight slopes in *cases (3 bits
// each, LIM_*: dqx[v] at bits 3v, dqy[v] at bits 12 + 3v; 0 when the slopes
// are not limited, slope_type 0).
template <typename Real, bool CASE = false>
__device__ __forceinline__ void slopes(const Hydro<Real>& h, const Real q[4], const Real qpx[4],
                                       const Real qmx[4], const Real qpy[4], const Real qmy[4],
                                       Real dqx[4], Real dqy[4], unsigned* cases = nullptr) {
  if (h.slope_type == 1 || h.slope_type == 2) {
    const bool mc = h.slope_type == 2;
    bool amb = false;
    constexpr bool INT = sizeof(Real) == 8 && E2D_LIM_INT;
    unsigned c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      dqx[v] = slope1<Real, INT, CASE>(mc, q[v], qpx[v], qmx[v], amb, &c[v]);
      dqy[v] = slope1<Real, INT, CASE>(mc, q[v], qpy[v], qmy[v], amb, &c[4 + v]);
    }
    if constexpr (INT) {
      if (amb) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          dqx[v] = slope1<Real, false, CASE>(mc, q[v], qpx[v], qmx[v], amb, &c[v]);
          dqy[v] = slope1<Real, false, CASE>(mc, q[v], qpy[v], qmy[v], amb, &c[4 + v]);
        }
      }
    }
    if constexpr (CASE) {
      unsigned w = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) w |= c[k] << (3 * k);
      *cases = w;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) { dqx[v] = Real(0.0); dqy[v] = Real(0.0); }
    if constexpr (CASE) *cases = 0u;
  }
}

// Source terms of trace_unsplit_2d_along_dir, serial_ref/m_utils.f90:213-216.
// They depend on the cell only, so a cell computes them once for its 4 faces.
template <typename Real>
__device__ __forceinline__ void trace_sources(const Hydro<Real>& h, const Real q[4], const Real dqx[4],
                                              const Real dqy[4], Real s[4]) {
  using O = Ops<Real>;
  const Real r = q[ID], p = q[IP], u = q[IU], v = q[IV];
#if E2D_FMA_FORMS
  // s = -(u*dqx + v*dqy + t) as one fused form (the form of trace_qs), so
  // that every kernel rounds it alike
  const Real dv = dqx[IU] + dqy[IV];
  Real t[4];
  t[ID] = dv * r;
  t[IP] = (dv * h.gamma0) * p;
  t[IU] = O::div(dqx[IP], r);
  t[IV] = O::div(dqy[IP], r);
#pragma unroll
  for (int k = 0; k < 4; ++k) s[k] = O::neg_if(fmx(u, dqx[k], fmx(v, dqy[k], t[k])), true);
#else
  s[ID] = ((-(u * dqx[ID])) - (v * dqy[ID])) - ((dqx[IU] + dqy[IV]) * r);
  s[IP] = ((-(u * dqx[IP])) - (v * dqy[IP])) - (((dqx[IU] + dqy[IV]) * h.gamma0) * p);
  s[IU] = ((-(u * dqx[IU])) - (v * dqy[IU])) - O::div(dqx[IP], r);
  s[IV] = ((-(u * dqx[IV])) - (v * dqy[IV])) - O::div(dqy[IP], r);
#endif
}

// The FMA build's cell value for its four face states on square cells:
// qs = q + (s*dtdx)*0.5 with the sources of trace_sources written as
// s = -(u*dqx + v*dqy + t), t the last term of each source, and
// qs = q - (dtdx/2)*(u*dqx + v*dqy + t), every step a fused multiply-add.
template <typename Real>
__device__ __forceinline__ void trace_qs(const Hydro<Real>& h, const Real q[4], const Real dqx[4], const Real dqy[4],
                                         Real hdt, Real qs[4]) {
  using O = Ops<Real>;
  const Real r = q[ID], p = q[IP], u = q[IU], v = q[IV];
  const Real dv = dqx[IU] + dqy[IV];
  Real t[4];
  t[ID] = dv * r;
  t[IP] = (dv * h.gamma0) * p;
  t[IU] = O::div(dqx[IP], r);
  t[IV] = O::div(dqy[IP], r);
#pragma unroll
  for (int k = 0; k < 4; ++k) qs[k] = fmx(-hdt, fmx(u, dqx[k], fmx(v, dqy[k], t[k])), q[k]);
}

// Face state of trace_unsplit_2d_along_dir, serial_ref/m_utils.f90:218-252:
// qf = (q -/+ 0.5*dq_dir) + (s*dtd)*0.5, then rho floored at smallr.
// PLUS selects the XMAX/YMAX faces; dq is the slope along the face normal,
// dtd = dtdx or dtdy.  PRE: s already holds (s*dtd)*0.5.
template <typename Real, bool PLUS, bool PRE = false>
__device__ __forceinline__ void trace_face(const Hydro<Real>& h, const Real q[4], const Real dq[4],
                                           const Real s[4], Real dtd, Real qf[4]) {
  using O = Ops<Real>;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const Real a = PLUS ? (q[v] + O::half(dq[v])) : (q[v] - O::half(dq[v]));
    qf[v] = a + (PRE ? s[v] : O::half(s[v] * dtd));
  }
  qf[ID] = O::max(h.smallr, qf[ID]);
}

// The same face state from qs = q + (s*dtd)*0.5 (the source term already
// added, once per cell for its four faces; the FMA build's form):
// qf = qs -/+ 0.5*dq, rho floored at smallr.
template <typename Real, bool PLUS>
__device__ __forceinline__ void trace_face_qs(const Hydro<Real>& h, const Real qs[4], const Real dq[4], Real qf[4]) {
#pragma unroll
  for (int v = 0; v < 4; ++v) qf[v] = fmx(PLUS ? Real(0.5) : Real(-0.5), dq[v], qs[v]);
  qf[ID] = Ops<Real>::max(h.smallr, qf[ID]);
}

// cmpflx, serial_ref/m_utils.f90:498-526.
template <typename Real>
__device__ __forceinline__ void cmpflx(const Hydro<Real>& h, const Real qg[4], Real flux[4]) {
  using O = Ops<Real>;
  flux[ID] = qg[ID] * qg[IU];
  flux[IU] = (flux[ID] * qg[IU]) + qg[IP];
  flux[IV] = flux[ID] * qg[IV];
#if E2D_FMA_FORMS
  const Real ekin = O::half(qg[ID]) * fmx(qg[IU], qg[IU], qg[IV] * qg[IV]);
#else
  const Real ekin = O::half(qg[ID]) * ((qg[IU] * qg[IU]) + (qg[IV] * qg[IV]));
#endif
  const Real etot = (qg[IP] * h.entho) + ekin;
  flux[IP] = qg[IU] * (etot + qg[IP]);
}

// riemann_2d (two-shock approximate solver + cmpflx), serial_ref/m_utils.f90:349-492.
template <typename Real>
__device__ __forceinline__ void riemann_approx(const Hydro<Real>& h, const Real qleft[4],
                                               const Real qright[4], Real flux[4]) {
  using O = Ops<Real>;
  const Real ONE = Real(1.0), ZERO = Real(0.0);
  const Real tol = Real(1e-6f);
  const Real rl = O::max(qleft[ID], h.smallr);
  const Real ul = qleft[IU];
  const Real pl = floor_prod(qleft[IP], rl, h.smallp);
  const Real rr = O::max(qright[ID], h.smallr);
  const Real ur = qright[IU];
  const Real pr = floor_prod(qright[IP], rr, h.smallp);
  const Real cl = (h.gamma0 * pl) * rl;
  const Real cr = (h.gamma0 * pr) * rr;
  Real wl = O::sqrt(cl);
  Real wr = O::sqrt(cr);
#if E2D_FMA_FORMS
  Real pold = O::max(O::div(fmx(wr, pl, fmx(wl, pr, (wl * wr) * (ul - ur))), wl + wr), ZERO);
#else
  Real pold = O::max(O::div(((wr * pl) + (wl * pr)) + ((wl * wr) * (ul - ur)), wl + wr), ZERO);
#endif
  Real conv = ONE;
  int iter = 0;
  while (iter < h.niter_riemann && O::gt(conv, tol)) {
    const Real wwl = O::sqrt(cl * (ONE + O::div(h.gamma6 * (pold - pl), pl)));
    const Real wwr = O::sqrt(cr * (ONE + O::div(h.gamma6 * (pold - pr), pr)));
    const Real ql = O::div((O::twice(wwl) * wwl) * wwl, (wwl * wwl) + cl);
    const Real qr = O::div((O::twice(wwr) * wwr) * wwr, (wwr * wwr) + cr);
    const Real usl = ul - O::div(pold - pl, wwl);
    const Real usr = ur + O::div(pold - pr, wwr);
    const Real delp = O::max(O::div(qr * ql, qr + ql) * (usl - usr), O::neg_if(pold, true));
    pold = pold + delp;
    conv = rabs(O::div(delp, pold + h.smallpp));
    iter = iter + 1;
  }
  const Real pstar = pold;
  wl = O::sqrt(cl * (ONE + O::div(h.gamma6 * (pstar - pl), pl)));
  wr = O::sqrt(cr * (ONE + O::div(h.gamma6 * (pstar - pr), pr)));
  const Real ustar = O::half(((ul + O::div(pl - pstar, wl)) + ur) - O::div(pr - pstar, wr));
  const bool left = O::ge0(ustar);  // sgnm = +1 (else -1)
  Real ro, uo, po, wo;
  if (left) { ro = rl; uo = ul; po = pl; wo = wl; }
  else      { ro = rr; uo = ur; po = pr; wo = wr; }
  const Real co = O::max(h.smallc, O::sqrt(rabs(O::div(h.gamma0 * po, ro))));
  const Real rstar = O::max(O::div(ro, ONE + O::div(ro * (po - pstar), wo * wo)), h.smallr);
  const Real cstar = O::max(h.smallc, O::sqrt(rabs(O::div(h.gamma0 * pstar, rstar))));
  const Real suo = O::neg_if(uo, !left), sust = O::neg_if(ustar, !left);  // sgnm*uo, sgnm*ustar
  Real spout = co - suo;
  Real spin = cstar - sust;
  const Real ushock = O::div(wo, ro) - suo;
  if (O::ge(pstar, po)) { spin = ushock; spout = ushock; }
  const Real scr = O::max(spout - spin, h.smallc + rabs(spout + spin));
  const Real frac = O::half(ONE + O::div(spout + spin, scr));
  Real qg[4];
#if E2D_FMA_FORMS
  const Real gfrac = ONE - frac;
  qg[ID] = fmx(frac, rstar, gfrac * ro);
  qg[IU] = fmx(frac, ustar, gfrac * uo);
  qg[IP] = fmx(frac, pstar, gfrac * po);
#else
  qg[ID] = (frac * rstar) + ((ONE - frac) * ro);
  qg[IU] = (frac * ustar) + ((ONE - frac) * uo);
  qg[IP] = (frac * pstar) + ((ONE - frac) * po);
#endif
  if (O::lt0(spout)) { qg[ID] = ro; qg[IU] = uo; qg[IP] = po; }
  if (O::gt0(spin)) { qg[ID] = rstar; qg[IU] = ustar; qg[IP] = pstar; }
  qg[IV] = left ? qleft[IV] : qright[IV];
  cmpflx(h, qg, flux);
}

// The FMA build's HLLC star pressure.  The reference's symmetric form
// (rcr pl + rcl pr + rcl rcr (ul - ur)) / (rcr + rcl) equals pl + rcl (ul -
// ustar) for the star velocity ustar = (rcr ur + rcl ul + pl - pr) / (rcr +
// rcl), identically in rcl, rcr, ul, ur, pl, pr: one fused multiply-add
// where the symmetric form takes four FP64 operations and a division (the
// same function, so its derivatives, which the adjoint takes in the
// symmetric form, are the same).  -DE2D_PSTAR_SYM builds the symmetric form
// instead (2.8 % slower on the 2048^2 step).
template <typename Real>
__device__ __forceinline__ Real hllc_pstar(Real rcl, Real rcr, Real ul, Real ur, Real pl, Real pr, Real ustar) {
#ifndef E2D_PSTAR_SYM
  return fmx(rcl, ul - ustar, pl);
#else
  return Ops<Real>::div(fmx(rcr, pl, rcl * fmx(rcr, ul - ur, pr)), rcr + rcl);
#endif
}

// riemann_2d_hllc, serial_ref/m_utils.f90:534-644 (rcsum, unused there, is not formed).
// The flux samples one side's state (left when SL > 0 or ustar > 0, else
// right: the reference's four branches), so the kinetic and total energy are
// formed for that side only, from the same operands: the same bits as the
// reference's etotl / etotr of the branch taken.
template <typename Real>
__device__ __forceinline__ void riemann_hllc(const Hydro<Real>& h, const Real qleft[4],
                                             const Real qright[4], Real flux[4]) {
  using O = Ops<Real>;
  const Real rl = O::max(qleft[ID], h.smallr);
  const Real pl = floor_prod(qleft[IP], rl, h.smallp);
  const Real ul = qleft[IU];
  const Real ptotl = pl;
  const Real rr = O::max(qright[ID], h.smallr);
  const Real pr = floor_prod(qright[IP], rr, h.smallp);
  const Real ur = qright[IU];
  const Real ptotr = pr;
  const Real cfastl = O::sqrt(O::max(O::div(h.gamma0 * pl, rl), h.smallc2));
  const Real cfastr = O::sqrt(O::max(O::div(h.gamma0 * pr, rr), h.smallc2));
  const Real cmax = O::max(cfastl, cfastr);
  const Real SL = O::min(ul, ur) - cmax;
  const Real SR = O::max(ul, ur) + cmax;
  const Real dsl = ul - SL, dsr = SR - ur;
  const Real rcl = rl * dsl;
  const Real rcr = rr * dsr;
#if E2D_FMA_FORMS
  const Real ustar = O::div(fmx(rcr, ur, fmx(rcl, ul, ptotl - ptotr)), rcr + rcl);
  const Real ptotstar = hllc_pstar(rcl, rcr, ul, ur, ptotl, ptotr, ustar);
#else
  const Real ustar = O::div(((rcr * ur) + (rcl * ul)) + (ptotl - ptotr), rcr + rcl);
  const Real ptotstar = O::div(((rcr * ptotl) + (rcl * ptotr)) + ((rcl * rcr) * (ul - ur)), rcr + rcl);
#endif
  // the sampled side (b1 / b2 of the reference: left; b3 / b4: right)
  const bool b1 = O::gt0(SL), lk = b1 || O::gt0(ustar);
  const Real rk = lk ? rl : rr, uk = lk ? ul : ur, vk = lk ? qleft[IV] : qright[IV], pk = lk ? pl : pr;
  const Real hrk = O::half(rk);
#if E2D_FMA_FORMS
  const Real ecink = hrk * fmx(uk, uk, vk * vk);
#else
  Real ecink = (hrk * uk) * uk;
  ecink = ecink + ((hrk * vk) * vk);
#endif
  const Real etotk = (pk * h.entho) + ecink;
  Real ro, uo, ptoto, etoto;
  if (b1 || !(lk || O::gt0(SR))) {  // supersonic: the side's own state
    ro = rk; uo = uk; ptoto = pk; etoto = etotk;
  } else {
    // the star state of the side, its operands chosen by selects: a warp
    // whose faces sample both star states issues it once
    uo = ustar; ptoto = ptotstar;
#if E2D_FMA_FORMS
    // rl (SL - ul) / (SL - ustar) = rcl / (ustar - SL), and so on
    const Real ps = ptotstar * ustar;
    const Real d = lk ? ustar - SL : SR - ustar;
    ro = O::div(lk ? rcl : rcr, d);
    etoto = O::div(fmx(lk ? dsl : dsr, etotk, fmx(O::neg_if(pk, !lk), uk, O::neg_if(ps, lk))), d);
#else
    // SL - ul is -(ul - SL) and rl (SL - ul) is -rcl, exactly (IEEE
    // differences and products are odd in each operand): the reference's
    // operands without forming them again
    const Real Sk = lk ? SL : SR;
    const Real sk = lk ? O::neg_if(dsl, true) : dsr;
    ro = O::div(lk ? O::neg_if(rcl, true) : rcr, Sk - ustar);
    etoto = O::div(((sk * etotk) - (pk * uk)) + (ptotstar * ustar), Sk - ustar);
#endif
  }
  flux[ID] = ro * uo;
  flux[IU] = ((ro * uo) * uo) + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = flux[ID] * (O::gt0(flux[ID]) ? qleft[IV] : qright[IV]);  // one product, either way
}

// The forward values of one HLLC solve that its reverse needs (the adjoint's
// face tape), in the order riemann_hllc_rec stores them.  HR_ETOTK is the
// total energy of the side the flux samples (left for branches 1-2, right
// for 3-4), HR_CA / HR_CF the sound speed squared and the sound speed of
// the side that gave cmax: the reverse needs no other side's.
enum {
  HR_QL = 0, HR_QR = 4, HR_PL = 8, HR_PR, HR_ETOTK, HR_CA, HR_CF, HR_SL, HR_SR, HR_RCL, HR_RCR, HR_USTAR,
  HR_PSTAR, HR_RO, HR_ETOTO, HR_FLUX, HR_N = HR_FLUX + 4
};
// flag bits: which operand each max/min, floor and branch of the solve took
enum {
  HF_PL_RAW = 1, HF_PR_RAW = 2, HF_CL_ACT = 4, HF_CR_ACT = 8, HF_CMAX_L = 16, HF_MIN_L = 32, HF_MAX_L = 64,
  HF_B1 = 128, HF_B2 = 256, HF_B3 = 512, HF_VLEFT = 1024
};

// riemann_hllc for double, recording its forward values into rec[HR_N] and
// flags (bit for bit the same flux: the same operations in the same order,
// with each max/min written as the selection it makes).
__device__ __forceinline__ void riemann_hllc_rec(const Hydro<double>& h, const double qleft[4],
                                                 const double qright[4], double rec[HR_N], unsigned& flags) {
  using O = Ops<double>;
  const auto pmax = [](double a, double b) { return emul::gt_i(a, b); };            // max(a, b) returns a
  const auto pmin = [](double a, double b) { return emul::ord(a) < emul::ord(b); };  // min(a, b) returns a
  bool pl_raw, pr_raw;
  const double rl = O::max(qleft[ID], h.smallr);
  const double pl = floor_pick(qleft[IP], rl, h.smallp, pl_raw);
  const double ul = qleft[IU];
  const double rr = O::max(qright[ID], h.smallr);
  const double pr = floor_pick(qright[IP], rr, h.smallp, pr_raw);
  const double ur = qright[IU];
  const double cal = O::div(h.gamma0 * pl, rl), car = O::div(h.gamma0 * pr, rr);
  const bool cl_act = pmax(cal, h.smallc2), cr_act = pmax(car, h.smallc2);
  const double cfastl = O::sqrt(cl_act ? cal : h.smallc2);
  const double cfastr = O::sqrt(cr_act ? car : h.smallc2);
  const bool cmax_l = pmax(cfastl, cfastr);
  const double cmax = cmax_l ? cfastl : cfastr;
  const bool min_l = pmin(ul, ur), max_l = pmax(ul, ur);
  const double SL = (min_l ? ul : ur) - cmax;
  const double SR = (max_l ? ul : ur) + cmax;
  const double dsl = ul - SL, dsr = SR - ur;
  const double rcl = rl * dsl;
  const double rcr = rr * dsr;
#if E2D_FMA_FORMS
  const double ustar = O::div(fmx(rcr, ur, fmx(rcl, ul, pl - pr)), rcr + rcl);
  const double ptotstar = hllc_pstar(rcl, rcr, ul, ur, pl, pr, ustar);
#else
  const double ustar = O::div(((rcr * ur) + (rcl * ul)) + (pl - pr), rcr + rcl);
  const double ptotstar = O::div(((rcr * pl) + (rcl * pr)) + ((rcl * rcr) * (ul - ur)), rcr + rcl);
#endif
  const bool b1 = O::gt0(SL), b2 = !b1 && O::gt0(ustar), b3 = !b1 && !b2 && O::gt0(SR);
  const bool lk = b1 || b2;  // the sampled side
  const double rk = lk ? rl : rr, uk = lk ? ul : ur, vk = lk ? qleft[IV] : qright[IV], pk = lk ? pl : pr;
  const double hrk = O::half(rk);
#if E2D_FMA_FORMS
  const double ecink = hrk * fmx(uk, uk, vk * vk);
#else
  double ecink = (hrk * uk) * uk;
  ecink = ecink + ((hrk * vk) * vk);
#endif
  const double etotk = (pk * h.entho) + ecink;
  double ro, uo, ptoto, etoto;
  if (!(b2 || b3)) {
    ro = rk; uo = uk; ptoto = pk; etoto = etotk;
  } else {
    uo = ustar; ptoto = ptotstar;
#if E2D_FMA_FORMS
    const double ps = ptotstar * ustar;
    const double d = lk ? ustar - SL : SR - ustar;
    ro = O::div(lk ? rcl : rcr, d);
    etoto = O::div(fmx(lk ? dsl : dsr, etotk, fmx(O::neg_if(pk, !lk), uk, O::neg_if(ps, lk))), d);
#else
    // SL - ul is -(ul - SL) and rl (SL - ul) is -rcl, exactly (IEEE
    // differences and products are odd in each operand): the reference's
    // operands without forming them again
    const double Sk = lk ? SL : SR;
    const double sk = lk ? O::neg_if(dsl, true) : dsr;
    ro = O::div(lk ? O::neg_if(rcl, true) : rcr, Sk - ustar);
    etoto = O::div(((sk * etotk) - (pk * uk)) + (ptotstar * ustar), Sk - ustar);
#endif
  }
  const double f0 = ro * uo;
  const bool vleft = O::gt0(f0);
#pragma unroll
  for (int v = 0; v < 4; ++v) { rec[HR_QL + v] = qleft[v]; rec[HR_QR + v] = qright[v]; }
  rec[HR_PL] = pl; rec[HR_PR] = pr; rec[HR_ETOTK] = etotk;
  rec[HR_CA] = cmax_l ? cal : car; rec[HR_CF] = cmax;
  rec[HR_SL] = SL; rec[HR_SR] = SR; rec[HR_RCL] = rcl; rec[HR_RCR] = rcr;
  rec[HR_USTAR] = ustar; rec[HR_PSTAR] = ptotstar; rec[HR_RO] = ro; rec[HR_ETOTO] = etoto;
  rec[HR_FLUX + ID] = f0;
  rec[HR_FLUX + IU] = ((ro * uo) * uo) + ptoto;
  rec[HR_FLUX + IP] = (etoto + ptoto) * uo;
  rec[HR_FLUX + IV] = f0 * (vleft ? qleft[IV] : qright[IV]);
  flags = (pl_raw ? HF_PL_RAW : 0u) | (pr_raw ? HF_PR_RAW : 0u) | (cl_act ? HF_CL_ACT : 0u) |
          (cr_act ? HF_CR_ACT : 0u) | (cmax_l ? HF_CMAX_L : 0u) | (min_l ? HF_MIN_L : 0u) |
          (max_l ? HF_MAX_L : 0u) | (b1 ? HF_B1 : 0u) | (b2 ? HF_B2 : 0u) | (b3 ? HF_B3 : 0u) |
          (vleft ? HF_VLEFT : 0u);
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
