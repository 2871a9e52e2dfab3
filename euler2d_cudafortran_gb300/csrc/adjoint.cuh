// adjoint.cuh -- hand-written reverse (adjoint) versions of the pointwise
// routines of physics.cuh, for the discrete adjoint of the FP64 step.
//
// Each *_rev routine recomputes what it needs of its forward routine (same
// operations, same branch decisions: limiter case, max/min selections, HLLC
// sampling branch, density and pressure floors) and accumulates the
// transposed Jacobian applied to the output adjoint into the input adjoints
// ("+=" semantics).  Ties in max/min follow the forward selection of Ops
// (the second argument wins a tie), so the derivative is a consistent
// one-sided derivative at those points.  Supported: the HLLC flux (the
// two-shock solver's Newton loop has no adjoint here).
#pragma once
#include "physics.cuh"

namespace e2d {
namespace adj {

using O = Ops<double>;

#ifndef E2D_REV_ONESTAR
#define E2D_REV_ONESTAR 1
#endif

__device__ __forceinline__ bool picks_first_max(double a, double b) { return emul::gt_i(a, b); }  // max(a,b) == a
__device__ __forceinline__ bool picks_first_min(double a, double b) { return emul::ord(a) < emul::ord(b); }

// computePrimitives (serial_ref/m_utils.f90:35-64) reverse: qb (adjoint of
// r, p, u, v) -> ub (adjoint of rho, E, rho u, rho v), given the forward
// primitives q of the same cell (r = q[ID], u = q[IU], v = q[IV]).
__device__ __forceinline__ void primitives_rev_q(const Hydro<double>& h, const double u[4], const double q[4],
                                                 const double qb[4], double ub[4]) {
  const double r = q[ID], uu = q[IU], vv = q[IV];
  const double eken = O::half(uu * uu + vv * vv);
  const double eu = O::div(u[IP], r);
  const double e = eu - eken;
  const double pa = (h.gm1 * r) * e, pb = r * h.smallp;
  double rb = qb[ID], eb = 0.0;
  if (picks_first_max(pa, pb)) {
    rb += qb[IP] * h.gm1 * e;
    eb = qb[IP] * h.gm1 * r;
  } else {
    rb += qb[IP] * h.smallp;
  }
  // e = E/r - 0.5 (u^2 + v^2)
  double ubu = qb[IU] - eb * uu;
  double ubv = qb[IV] - eb * vv;
  ub[IP] += O::div(eb, r);
  rb -= O::div(eb * eu, r);
  // u = (rho u)/r, v = (rho v)/r
  ub[IU] += O::div(ubu, r);
  ub[IV] += O::div(ubv, r);
  rb -= O::div(ubu * uu + ubv * vv, r);
  if (picks_first_max(u[ID], h.smallr)) ub[ID] += rb;
}

// The same, recomputing the primitives from u.
__device__ __forceinline__ void primitives_rev(const Hydro<double>& h, const double u[4], const double qb[4],
                                               double ub[4]) {
  const double r = O::max(u[ID], h.smallr);
  const double q[4] = {r, 0.0, O::div(u[IU], r), O::div(u[IV], r)};  // ID, IP (unused), IU, IV
  primitives_rev_q(h, u, q, qb, ub);
}

// The compute_dt term of one cell (serial_ref/m_run.f90:278-281) reverse.
__device__ __forceinline__ void cell_invdt_rev(const Hydro<double>& h, const double u[4], double tb, double ub[4]) {
  double q[4];
  primitives(h, u, q);
  const double c2 = O::div(h.gamma0 * q[IP], q[ID]);
  const double c = O::sqrt(c2);
  double qb[4] = {0.0, 0.0, 0.0, 0.0};
  const double cb = O::div(tb, h.dx) + O::div(tb, h.dy);
  qb[IU] = O::neg_if(O::div(tb, h.dx), !O::ge0(q[IU]));
  qb[IV] = O::neg_if(O::div(tb, h.dy), !O::ge0(q[IV]));
  const double c2b = O::div(cb, O::twice(c));
  qb[IP] += O::div(c2b * h.gamma0, q[ID]);
  qb[ID] -= O::div(c2b * c2, q[ID]);
  primitives_rev(h, u, qb, ub);
}

// One slope (slope_unsplit_hydro_2d, one variable and direction) reverse:
// adds d(slope)/d(q, qp, qm) * sb.
__device__ __forceinline__ void slope1_rev(bool mc, double q, double qp, double qm, double sb, double& qbar,
                                           double& qpbar, double& qmbar) {
  const double dl = q - qm, dr = qp - q;
  const double dlft = mc ? O::twice(dl) : dl;
  const double drgt = mc ? O::twice(dr) : dr;
  const double dcen = O::half(qp - qm);
  if (O::le0(dlft * drgt)) return;  // limited to zero
  const bool neg = !O::ge0(dcen);   // dsgn = -1
  const double al = rabs(dlft), ar = rabs(drgt), ac = rabs(dcen);
  const bool use_l = picks_first_min(al, ar);
  const double slop = use_l ? al : ar;
  if (picks_first_min(slop, ac)) {
    // slope = dsgn * |dlft| or dsgn * |drgt|
    const double x = use_l ? dlft : drgt;
    const double g = O::neg_if(sb, (!O::ge0(x)) != neg);  // dsgn * sign(x) * sb
    const double sg = mc ? O::twice(g) : g;              // st * g, st = 2 (MC) or 1
    if (use_l) { qbar += sg; qmbar -= sg; }
    else { qpbar += sg; qbar -= sg; }
  } else {
    // slope = dsgn * |dcen| = dcen
    const double g = O::half(O::neg_if(sb, (!O::ge0(dcen)) != neg));
    qpbar += g;
    qmbar -= g;
  }
}

// trace_sources reverse: sb -> (qb, dqxb, dqyb).
__device__ __forceinline__ void trace_sources_rev(const Hydro<double>& h, const double q[4], const double dqx[4],
                                                  const double dqy[4], const double sb[4], double qb[4],
                                                  double dqxb[4], double dqyb[4]) {
  const double r = q[ID], p = q[IP], u = q[IU], v = q[IV];
  const double div_ = dqx[IU] + dqy[IV];
  qb[IU] -= sb[ID] * dqx[ID] + sb[IP] * dqx[IP] + sb[IU] * dqx[IU] + sb[IV] * dqx[IV];
  qb[IV] -= sb[ID] * dqy[ID] + sb[IP] * dqy[IP] + sb[IU] * dqy[IU] + sb[IV] * dqy[IV];
  qb[ID] -= sb[ID] * div_;
  qb[ID] += O::div(O::div(sb[IU] * dqx[IP] + sb[IV] * dqy[IP], r), r);
  qb[IP] -= sb[IP] * div_ * h.gamma0;
  dqxb[ID] -= sb[ID] * u;
  dqyb[ID] -= sb[ID] * v;
  dqxb[IP] -= sb[IP] * u + O::div(sb[IU], r);
  dqyb[IP] -= sb[IP] * v + O::div(sb[IV], r);
  const double dd = sb[ID] * r + sb[IP] * h.gamma0 * p;
  dqxb[IU] -= dd + sb[IU] * u;
  dqyb[IU] -= sb[IU] * v;
  dqxb[IV] -= sb[IV] * u;
  dqyb[IV] -= dd + sb[IV] * v;
}

// trace_face reverse: qfb -> (qb, dqb, sb) and the dt/d adjoint dtdb.
// PRE: sh holds (s*dtd)*0.5 (dx == dy), and sb receives the adjoint of
// (s*dtd) per unit dtd -- the caller multiplies the cell's sum by dtd once.
template <bool PLUS, bool PRE = false>
__device__ __forceinline__ void trace_face_rev(const Hydro<double>& h, const double q[4], const double dq[4],
                                               const double s[4], const double* sh, double dtd,
                                               const double qfb_in[4], double qb[4], double dqb[4], double sb[4],
                                               double& dtdb) {
  double qfb[4] = {qfb_in[0], qfb_in[1], qfb_in[2], qfb_in[3]};
  const double a = PLUS ? (q[ID] + O::half(dq[ID])) : (q[ID] - O::half(dq[ID]));
  const double raw = a + (PRE ? sh[ID] : O::half(s[ID] * dtd));
  // max(smallr, raw) returns raw unless smallr > raw: no gradient through the floor
  if (emul::gt_i(h.smallr, raw)) qfb[ID] = 0.0;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double hq = O::half(qfb[v]);
    qb[v] += qfb[v];
    dqb[v] += O::neg_if(hq, !PLUS);
    sb[v] += PRE ? hq : dtd * hq;
    dtdb += s[v] * hq;
  }
}

// riemann_2d_hllc (serial_ref/m_utils.f90:534-644) reverse: fb -> (qlb, qrb).
// Also returns the forward flux (bit for bit riemann_hllc's) in flux[4].
__device__ __forceinline__ void riemann_hllc_rev(const Hydro<double>& h, const double ql[4], const double qr[4],
                                                 const double fb[4], double qlb[4], double qrb[4],
                                                 double flux[4]) {
  // ---- forward recomputation (same operations and branches as riemann_hllc)
  const double rl = O::max(ql[ID], h.smallr), rr = O::max(qr[ID], h.smallr);
  bool pl_raw, pr_raw;  // the pressure floors returned the face pressures
  const double pl = floor_pick(ql[IP], rl, h.smallp, pl_raw), pr = floor_pick(qr[IP], rr, h.smallp, pr_raw);
  const double ul = ql[IU], ur = qr[IU], vl = ql[IV], vr = qr[IV];
  const double hrl = O::half(rl), hrr = O::half(rr);
  const double etotl = (pl * h.entho) + (((hrl * ul) * ul) + ((hrl * vl) * vl));
  const double etotr = (pr * h.entho) + (((hrr * ur) * ur) + ((hrr * vr) * vr));
  const double cal = O::div(h.gamma0 * pl, rl), car = O::div(h.gamma0 * pr, rr);
  const bool cl_act = picks_first_max(cal, h.smallc2), cr_act = picks_first_max(car, h.smallc2);
  const double cfastl = O::sqrt(cl_act ? cal : h.smallc2), cfastr = O::sqrt(cr_act ? car : h.smallc2);
  const bool cmax_l = picks_first_max(cfastl, cfastr);
  const double cmax = cmax_l ? cfastl : cfastr;
  const bool min_l = picks_first_min(ul, ur), max_l = picks_first_max(ul, ur);
  const double SL = (min_l ? ul : ur) - cmax;
  const double SR = (max_l ? ul : ur) + cmax;
  const double rcl = rl * (ul - SL), rcr = rr * (SR - ur);
  const double den = rcr + rcl;
  const double ustar = O::div(((rcr * ur) + (rcl * ul)) + (pl - pr), den);
  const double ptotstar = O::div(((rcr * pl) + (rcl * pr)) + ((rcl * rcr) * (ul - ur)), den);
#if E2D_REV_ONESTAR
  // The sampled side K first (SL > 0: left state; ustar > 0: left star;
  // SR > 0: right star; else right state), then one star state from its
  // values: a warp whose faces sample both stars issues the arithmetic once.
  const bool b1 = O::gt0(SL), b2 = !b1 && O::gt0(ustar);
  const bool star = b2 || (!b1 && O::gt0(SR));
  const bool lside = b1 || b2;
  const double SK = lside ? SL : SR, rK = lside ? rl : rr, uK = lside ? ul : ur;
  const double eK = lside ? etotl : etotr, pK = lside ? pl : pr;
  double ro = rK, uo = uK, ptoto = pK, etoto = eK, d = 1.0, dS = 0.0;
  if (star) {
    dS = SK - uK;
    d = SK - ustar;
    ro = O::div(rK * dS, d); uo = ustar; ptoto = ptotstar;
    etoto = O::div((((dS * eK) - (pK * uK)) + (ptotstar * ustar)), d);
  }
#else
  int branch;
  double ro, uo, ptoto, etoto, d = 1.0, nE = 0.0;
  if (O::gt0(SL)) { branch = 1; ro = rl; uo = ul; ptoto = pl; etoto = etotl; }
  else if (O::gt0(ustar)) {
    branch = 2; d = SL - ustar;
    ro = O::div(rl * (SL - ul), d); uo = ustar; ptoto = ptotstar;
    nE = (((SL - ul) * etotl) - (pl * ul)) + (ptotstar * ustar); etoto = O::div(nE, d);
  } else if (O::gt0(SR)) {
    branch = 3; d = SR - ustar;
    ro = O::div(rr * (SR - ur), d); uo = ustar; ptoto = ptotstar;
    nE = (((SR - ur) * etotr) - (pr * ur)) + (ptotstar * ustar); etoto = O::div(nE, d);
  } else { branch = 4; ro = rr; uo = ur; ptoto = pr; etoto = etotr; }
#endif
  const double fr = ro * uo;
  const bool vleft = O::gt0(fr);
  flux[ID] = fr;
  flux[IU] = (fr * uo) + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = fr * (vleft ? vl : vr);

  // ---- reverse
  double rlb = 0, rrb = 0, plb = 0, prb = 0, ulb = 0, urb = 0, vlb = 0, vrb = 0, etotlb = 0, etotrb = 0;
  double SLb = 0, SRb = 0, ustarb = 0, ptotstarb = 0;
  // flux[IV] = fr * (vl or vr)
  double frb = fb[ID] + fb[IV] * (vleft ? vl : vr);
  if (vleft) vlb += fb[IV] * fr; else vrb += fb[IV] * fr;
  // flux[IU] = fr * uo + ptoto ; flux[IP] = (etoto + ptoto) * uo
  double uob = fb[IU] * fr + fb[IP] * (etoto + ptoto);
  frb += fb[IU] * uo;
  double ptotob = fb[IU] + fb[IP] * uo;
  double etotob = fb[IP] * uo;
  // fr = ro * uo
  double rob = frb * uo;
  uob += frb * ro;
#if E2D_REV_ONESTAR
  {
    double rKb = rob, uKb = uob, pKb = ptotob, eKb = etotob, SKb = 0.0;
    if (star) {
      ustarb += uob; ptotstarb += ptotob;
      const double rq = O::div(rob, d);
      rKb = rq * dS; SKb = rq * rK; uKb = O::neg_if(rq * rK, true);
      const double nEb = O::div(etotob, d);
      const double db = O::neg_if(rq * ro + nEb * etoto, true);
      SKb += nEb * eK; uKb -= nEb * eK; eKb = nEb * dS;
      pKb = O::neg_if(nEb * uK, true); uKb -= nEb * pK; ptotstarb += nEb * ustar; ustarb += nEb * ptotstar;
      SKb += db; ustarb -= db;
    }
    // the side's accumulators are all zero here: route by selection
    rlb = lside ? rKb : 0.0; rrb = lside ? 0.0 : rKb;
    ulb = lside ? uKb : 0.0; urb = lside ? 0.0 : uKb;
    plb = lside ? pKb : 0.0; prb = lside ? 0.0 : pKb;
    etotlb = lside ? eKb : 0.0; etotrb = lside ? 0.0 : eKb;
    SLb = lside ? SKb : 0.0; SRb = lside ? 0.0 : SKb;
  }
#else
  switch (branch) {
    case 1: rlb += rob; ulb += uob; plb += ptotob; etotlb += etotob; break;
    case 4: rrb += rob; urb += uob; prb += ptotob; etotrb += etotob; break;
    case 2: {
      ustarb += uob; ptotstarb += ptotob;
      const double rq = O::div(rob, d);
      rlb += rq * (SL - ul); SLb += rq * rl; ulb -= rq * rl;
      const double nEb = O::div(etotob, d);
      const double db = O::neg_if(rq * ro + nEb * etoto, true);  // d(ro, etoto)/d(d)
      SLb += nEb * etotl; ulb -= nEb * etotl; etotlb += nEb * (SL - ul);
      plb -= nEb * ul; ulb -= nEb * pl; ptotstarb += nEb * ustar; ustarb += nEb * ptotstar;
      SLb += db; ustarb -= db;
      break;
    }
    default: {  // 3
      ustarb += uob; ptotstarb += ptotob;
      const double rq = O::div(rob, d);
      rrb += rq * (SR - ur); SRb += rq * rr; urb -= rq * rr;
      const double nEb = O::div(etotob, d);
      const double db = O::neg_if(rq * ro + nEb * etoto, true);
      SRb += nEb * etotr; urb -= nEb * etotr; etotrb += nEb * (SR - ur);
      prb -= nEb * ur; urb -= nEb * pr; ptotstarb += nEb * ustar; ustarb += nEb * ptotstar;
      SRb += db; ustarb -= db;
      break;
    }
  }
#endif
  // ptotstar and ustar = num / den
  const double npb = O::div(ptotstarb, den), nub = O::div(ustarb, den);
  double denb = -npb * ptotstar - nub * ustar;
  double rcrb = npb * (pl + rcl * (ul - ur)) + nub * ur + denb;
  double rclb = npb * (pr + rcr * (ul - ur)) + nub * ul + denb;
  const double pa = npb * rcr + nub, pb = npb * rcl - nub;
  plb += pa;
  prb += pb;
  ulb += rcl * pa;   // npb rcl rcr + nub rcl
  urb -= rcr * pb;   // -npb rcl rcr + nub rcr
  // rcr = rr (SR - ur), rcl = rl (ul - SL)
  rrb += rcrb * (SR - ur); SRb += rcrb * rr; urb -= rcrb * rr;
  rlb += rclb * (ul - SL); ulb += rclb * rl; SLb -= rclb * rl;
  // SR = max(ul, ur) + cmax, SL = min(ul, ur) - cmax
  const double cmaxb = SRb - SLb;
  if (max_l) ulb += SRb; else urb += SRb;
  if (min_l) ulb += SLb; else urb += SLb;
  const double cfastlb = cmax_l ? cmaxb : 0.0, cfastrb = cmax_l ? 0.0 : cmaxb;
  if (cl_act) {
    const double cab = O::div(cfastlb, O::twice(cfastl));
    plb += O::div(cab * h.gamma0, rl);
    rlb -= O::div(cab * cal, rl);
  }
  if (cr_act) {
    const double cab = O::div(cfastrb, O::twice(cfastr));
    prb += O::div(cab * h.gamma0, rr);
    rrb -= O::div(cab * car, rr);
  }
  // etot = p entho + hr u u + hr v v, hr = rho / 2
  plb += etotlb * h.entho; prb += etotrb * h.entho;
  rlb += O::half(etotlb) * (ul * ul + vl * vl);
  rrb += O::half(etotrb) * (ur * ur + vr * vr);
  const double erl = etotlb * rl, err = etotrb * rr;  // 2 hr = rho
  ulb += erl * ul; vlb += erl * vl;
  urb += err * ur; vrb += err * vr;
  // pressure and density floors
  if (pl_raw) qlb[IP] += plb; else rlb += plb * h.smallp;
  if (pr_raw) qrb[IP] += prb; else rrb += prb * h.smallp;
  if (picks_first_max(ql[ID], h.smallr)) qlb[ID] += rlb;
  if (picks_first_max(qr[ID], h.smallr)) qrb[ID] += rrb;
  qlb[IU] += ulb; qlb[IV] += vlb;
  qrb[IU] += urb; qrb[IV] += vrb;
}

}  // namespace adj
}  // namespace e2d
