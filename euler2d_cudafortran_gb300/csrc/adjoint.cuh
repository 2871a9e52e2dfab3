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



__device__ __forceinline__ bool picks_first_max(double a, double b) { return emul::gt_i(a, b); }  // max(a,b) == a
__device__ __forceinline__ bool picks_first_min(double a, double b) { return emul::ord(a) < emul::ord(b); }

// computePrimitives (serial_ref/m_utils.f90:35-64) reverse: qb (adjoint of
// r, p, u, v) -> ub (adjoint of rho, E, rho u, rho v; written), given the forward
// primitives q of the same cell (all four: r = q[ID], p = q[IP], u = q[IU],
// v = q[IV]).  eos's pressure max((gm1 r) e, r smallp), e = E/r - eken,
// returned its first operand exactly when p > r smallp (it returned p; the
// floor would give p == r smallp), decided like floor_pick; unfloored,
// dp/dr = gm1 e = p / r and dp/de = gm1 r.
__device__ __forceinline__ void primitives_rev_q(const Hydro<double>& h, const double u[4], const double q[4],
                                                 const double qb[4], double ub[4]) {
  const double r = q[ID], uu = q[IU], vv = q[IV];
  const double eu = O::div(u[IP], r);
  bool raw;
  (void)floor_pick(q[IP], r, h.smallp, raw);
  double rb = qb[ID], eb = 0.0;
  if (raw) {
    rb += qb[IP] * O::div(q[IP], r);
    eb = qb[IP] * h.gm1 * r;
  } else {
    rb += qb[IP] * h.smallp;
  }
  // e = E/r - 0.5 (u^2 + v^2)
  double ubu = qb[IU] - eb * uu;
  double ubv = qb[IV] - eb * vv;
  ub[IP] = O::div(eb, r);
  rb -= O::div(eb * eu, r);
  // u = (rho u)/r, v = (rho v)/r
  ub[IU] = O::div(ubu, r);
  ub[IV] = O::div(ubv, r);
  rb -= O::div(ubu * uu + ubv * vv, r);
  ub[ID] = picks_first_max(u[ID], h.smallr) ? rb : 0.0;
}

// The same, recomputing the primitives from u, adding to ub.
__device__ __forceinline__ void primitives_rev(const Hydro<double>& h, const double u[4], const double qb[4],
                                               double ub[4]) {
  double q[4], t[4];
  primitives(h, u, q);
  primitives_rev_q(h, u, q, qb, t);
#pragma unroll
  for (int v = 0; v < 4; ++v) ub[v] += t[v];
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

// The same from the forward step's recorded limiter case (3 bits, LIM_*):
// nothing of the slope is recomputed.  It writes the neighbours' adjoints
// (qpbar, qmbar set, not accumulated) and adds the cell's own to qbar: no
// FP64 work for a slope limited to zero or a centred one, one addition for a
// one-sided one, where accumulating into zero slots costs two.
__device__ __forceinline__ void slope1_rev_case(bool mc, unsigned cs, double sb, double& qbar, double& qpbar,
                                                double& qmbar) {
  const unsigned sel = cs & 3u;
  qpbar = 0.0;
  qmbar = 0.0;
  if (sel == LIM_ZERO) return;
  if (sel == LIM_CENTRE) {  // slope = dcen = (qp - qm) / 2
    const double g = O::half(sb);
    qpbar = g;
    qmbar = O::neg_if(g, true);
    return;
  }
  const double g = O::neg_if(sb, (cs & LIM_FLIP) != 0u);  // dsgn * sign(x) * sb
  const double sg = mc ? O::twice(g) : g;                 // st * g
  const bool left = sel == LIM_LEFT;                      // else LIM_RIGHT
  qbar += O::neg_if(sg, !left);                           // one addition either way
  qpbar = left ? 0.0 : sg;
  qmbar = left ? O::neg_if(sg, true) : 0.0;
}

// trace_sources reverse: sb -> (qb, dqxb, dqyb); qb is written (the cell's
// adjoint starts here), dqxb and dqyb are added to.
__device__ __forceinline__ void trace_sources_rev(const Hydro<double>& h, const double q[4], const double dqx[4],
                                                  const double dqy[4], const double sb[4], double qb[4],
                                                  double dqxb[4], double dqyb[4]) {
  const double r = q[ID], p = q[IP], u = q[IU], v = q[IV];
  const double div_ = dqx[IU] + dqy[IV];
  qb[IU] = -(sb[ID] * dqx[ID] + sb[IP] * dqx[IP] + sb[IU] * dqx[IU] + sb[IV] * dqx[IV]);
  qb[IV] = -(sb[ID] * dqy[ID] + sb[IP] * dqy[IP] + sb[IU] * dqy[IU] + sb[IV] * dqy[IV]);
  qb[ID] = O::div(O::div(sb[IU] * dqx[IP] + sb[IV] * dqy[IP], r), r) - sb[ID] * div_;
  qb[IP] = -(sb[IP] * div_ * h.gamma0);
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

// trace_face reverse: qfb -> (qb, dqb, sb; written) and the dt/d adjoint
// dtdb (added to).
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
  for (int v = 0; v < 4; ++v) {  // qb, dqb, sb written (their slots start here)
    const double hq = O::half(qfb[v]);
    qb[v] = qfb[v];
    dqb[v] = O::neg_if(hq, !PLUS);
    sb[v] = PRE ? hq : dtd * hq;
    dtdb += s[v] * hq;
  }
}

// riemann_2d_hllc (serial_ref/m_utils.f90:534-644) reverse from the solve's
// recorded forward values (riemann_hllc_rec): fb -> (qlb, qrb), written.
__device__ __forceinline__ void riemann_hllc_rev_rec(const Hydro<double>& h, const double* rec, unsigned flags,
                                                     const double fb[4], double qlb[4], double qrb[4]) {
  const double ul = rec[HR_QL + IU], ur = rec[HR_QR + IU], vl = rec[HR_QL + IV], vr = rec[HR_QR + IV];
  const double rl = O::max(rec[HR_QL + ID], h.smallr), rr = O::max(rec[HR_QR + ID], h.smallr);
  const double pl = rec[HR_PL], pr = rec[HR_PR];
  const double eK = rec[HR_ETOTK], caC = rec[HR_CA], cfC = rec[HR_CF], SL = rec[HR_SL], SR = rec[HR_SR];
  const double rcl = rec[HR_RCL], rcr = rec[HR_RCR], ustar = rec[HR_USTAR], ptotstar = rec[HR_PSTAR];
  const double ro = rec[HR_RO], etoto = rec[HR_ETOTO], fr = rec[HR_FLUX + ID];
  const bool pl_raw = flags & HF_PL_RAW, pr_raw = flags & HF_PR_RAW;
  const bool cl_act = flags & HF_CL_ACT, cr_act = flags & HF_CR_ACT, cmax_l = flags & HF_CMAX_L;
  const bool min_l = flags & HF_MIN_L, max_l = flags & HF_MAX_L, vleft = flags & HF_VLEFT;
  const bool b1 = flags & HF_B1, b2 = flags & HF_B2, b3 = flags & HF_B3;
  const bool star = b2 || b3, lside = b1 || b2;  // sampled side K: left for branches 1, 2
  const double SK = lside ? SL : SR, rK = lside ? rl : rr, uK = lside ? ul : ur, vK = lside ? vl : vr;
  const double pK = lside ? pl : pr;
  const double uo = star ? ustar : uK, ptoto = star ? ptotstar : pK;
  const double den = rcr + rcl;
  const double dsl = ul - SL, dsr = SR - ur;  // rcl = rl dsl, rcr = rr dsr

  // (Every adjoint below is written on its first contribution, not added to
  // a zero: 0 + x costs an FP64 addition and gives the same bits, up to the
  // sign of a zero.)
  double rlb, rrb, plb, prb, ulb, urb, vlb, vrb, SLb, SRb, ustarb, ptotstarb;
  // flux[IV] = fr * (vl or vr)
  double frb = fb[ID] + fb[IV] * (vleft ? vl : vr);
  const double fvb = fb[IV] * fr;
  // flux[IU] = fr * uo + ptoto ; flux[IP] = (etoto + ptoto) * uo
  double uob = fb[IU] * fr + fb[IP] * (etoto + ptoto);
  frb += fb[IU] * uo;
  double ptotob = fb[IU] + fb[IP] * uo;
  double etotob = fb[IP] * uo;
  // fr = ro * uo
  double rob = frb * uo;
  uob += frb * ro;
  {
    // one star state for either side: a warp whose faces sample both issues it once
    double rKb = rob, uKb = uob, pKb = ptotob, eKb = etotob, SKb = 0.0;
    ustarb = 0.0;
    ptotstarb = 0.0;
    if (star) {
      const double dS = lside ? O::neg_if(dsl, true) : dsr, d = SK - ustar;  // SK - uK
      const double rq = O::div(rob, d);
      rKb = rq * dS; SKb = rq * rK; uKb = O::neg_if(rq * rK, true);
      const double nEb = O::div(etotob, d);
      const double db = O::neg_if(rq * ro + nEb * etoto, true);
      SKb += nEb * eK; uKb -= nEb * eK; eKb = nEb * dS;
      pKb = O::neg_if(nEb * uK, true); uKb -= nEb * pK;
      ptotstarb = ptotob + nEb * ustar;
      ustarb = (uob + nEb * ptotstar) - db;
      SKb += db;
    }
    // etot_K = pK entho + hrK (uK uK + vK vK), hrK = rK / 2 (the other
    // side's energy is not sampled: its adjoint is zero)
    pKb += eKb * h.entho;
    rKb += O::half(eKb) * (uK * uK + vK * vK);
    const double erK = eKb * rK;  // 2 hrK = rK
    uKb += erK * uK;
    const double vKb = erK * vK;
    rlb = lside ? rKb : 0.0; rrb = lside ? 0.0 : rKb;
    ulb = lside ? uKb : 0.0; urb = lside ? 0.0 : uKb;
    plb = lside ? pKb : 0.0; prb = lside ? 0.0 : pKb;
    SLb = lside ? SKb : 0.0; SRb = lside ? 0.0 : SKb;
    // flux[IV]'s share to the side vleft names, vKb to side K
    const double vsum = fvb + vKb;
    vlb = vleft ? (lside ? vsum : fvb) : (lside ? vKb : 0.0);
    vrb = vleft ? (lside ? 0.0 : vKb) : (lside ? fvb : vsum);
  }
  // ptotstar and ustar = num / den: d/drcr = (pl + rcl (ul - ur) - ptotstar,
  // ur - ustar) / den and d/drcl = (pr + rcr (ul - ur) - ptotstar, ul -
  // ustar) / den, where ptotstar = pl + rcl (ul - ustar) = pr + rcr (ustar -
  // ur) (the HLLC star pressure from either side) reduces the two to
  // (ustar - ur) pb and (ul - ustar) pa
  const double npb = O::div(ptotstarb, den), nub = O::div(ustarb, den);
  const double pa = npb * rcr + nub, pb = npb * rcl - nub;
  const double rcrb = (ustar - ur) * pb;
  const double rclb = (ul - ustar) * pa;
  {
    const double pKt = (lside ? plb : prb) + (lside ? pa : pb);  // side K's pressure adjoint
    plb = lside ? pKt : pa;
    prb = lside ? pb : pKt;
  }
  ulb += rcl * pa;   // npb rcl rcr + nub rcl
  urb -= rcr * pb;   // -npb rcl rcr + nub rcr
  // rcr = rr (SR - ur), rcl = rl (ul - SL)
  rrb += rcrb * dsr; SRb += rcrb * rr; urb -= rcrb * rr;
  rlb += rclb * dsl; ulb += rclb * rl; SLb -= rclb * rl;
  // SR = max(ul, ur) + cmax, SL = min(ul, ur) - cmax
  const double cmaxb = SRb - SLb;
  // (selected accumulators: one addition each, where branches cost a warp
  // holding both cases two)
  {
    const double t = (max_l ? ulb : urb) + SRb;
    ulb = max_l ? t : ulb; urb = max_l ? urb : t;
  }
  {
    const double t = (min_l ? ulb : urb) + SLb;
    ulb = min_l ? t : ulb; urb = min_l ? urb : t;
  }
  // cmax = the faster side C's sound speed sqrt(max(gamma p / rho, smallc2))
  if (cmax_l ? cl_act : cr_act) {
    const double rC = cmax_l ? rl : rr;
    const double cab = O::div(cmaxb, O::twice(cfC));
    const double pCb = O::div(cab * h.gamma0, rC), rCb = O::div(cab * caC, rC);
    const double pCt = (cmax_l ? plb : prb) + pCb, rCt = (cmax_l ? rlb : rrb) - rCb;
    plb = cmax_l ? pCt : plb; prb = cmax_l ? prb : pCt;
    rlb = cmax_l ? rCt : rlb; rrb = cmax_l ? rrb : rCt;
  }
  // pressure and density floors; the face-state adjoints are written
  if (!pl_raw) rlb += plb * h.smallp;
  if (!pr_raw) rrb += prb * h.smallp;
  qlb[IP] = pl_raw ? plb : 0.0;
  qrb[IP] = pr_raw ? prb : 0.0;
  qlb[ID] = emul::gt_i(rec[HR_QL + ID], h.smallr) ? rlb : 0.0;
  qrb[ID] = emul::gt_i(rec[HR_QR + ID], h.smallr) ? rrb : 0.0;
  qlb[IU] = ulb; qlb[IV] = vlb;
  qrb[IU] = urb; qrb[IV] = vrb;
}

// The same, recomputing the forward values from the face states; returns
// the forward flux (bit for bit riemann_hllc's) in flux[4].
__device__ __forceinline__ void riemann_hllc_rev(const Hydro<double>& h, const double ql[4], const double qr[4],
                                                 const double fb[4], double qlb[4], double qrb[4],
                                                 double flux[4]) {
  double rec[HR_N];
  unsigned flags;
  riemann_hllc_rec(h, ql, qr, rec, flags);
#pragma unroll
  for (int v = 0; v < 4; ++v) flux[v] = rec[HR_FLUX + v];
  riemann_hllc_rev_rec(h, rec, flags, fb, qlb, qrb);
}

}  // namespace adj
}  // namespace e2d
