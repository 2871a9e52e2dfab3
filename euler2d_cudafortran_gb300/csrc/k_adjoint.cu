// k_adjoint.cu -- reverse (adjoint) kernels of the FP64 step.
//
// k_step_rev: given the state U_n (ghosts filled) and the adjoint of the next
// state Ubar_{n+1} (interior cells), accumulates Ubar_n and the adjoint of the
// step's dt.  A CTA owns a 32 x 7 tile; it recomputes the forward values of
// its box (primitives, slopes, trace sources), then for each face it owns
// (the left / lower faces of its cells, plus the last wall faces) forms the
// flux adjoint from the update (F_i enters cell i with + and cell i-1 with -),
// runs the Riemann, trace, source, slope and primitive reverses, and adds the
// results into shared memory in passes where no two threads touch the same
// word (no shared atomics); ghost-cell adjoints are folded back to the
// interior cells make_boundaries copied them from (serial_ref/m_run.f90:
// 561-648) with global atomic adds, since neighbouring tiles overlap there.
// The 2x2 ghost corners are constants and receive nothing.
#include "adjoint.cuh"
#include "adjoint_launch.h"
#include "tile.cuh"

namespace e2d {

namespace {

// Reverse tile: 32 x E2D_REV_TY cells, E2D_REV_NT threads, E2D_REV_MINB CTAs
// per SM (shared memory and registers must allow that many).
#ifndef E2D_REV_TY
#define E2D_REV_TY 7
#endif
#ifndef E2D_REV_NT
#define E2D_REV_NT 128
#endif
#ifndef E2D_REV_MINB
#define E2D_REV_MINB 2
#endif
constexpr int ATX = 32, ATY = E2D_REV_TY, ANT = E2D_REV_NT;
constexpr int ABX = ATX + 4, ABY = ATY + 4, ARX = ATX + 2, ARY = ATY + 2;
constexpr int NBOX = ABX * ABY, NRING = ARX * ARY;
constexpr int NUB = (ATX + 1) * (ATY + 1);
// shared layout (doubles)
constexpr int Q_OFF = 0;                        // q box      [4][ABY][ABX]
constexpr int DQ_OFF = Q_OFF + 4 * NBOX;        // slopes     [8][ARY][ARX]
constexpr int S_OFF = DQ_OFF + 8 * NRING;       // sources    [4][ARY][ARX]
constexpr int UB_OFF = S_OFF + 4 * NRING;       // Ubar'      [4][ATY+1][ATX+1], cells (i0-1.., j0-1..)
constexpr int RA_OFF = UB_OFF + 4 * NUB;        // ring adj.  dqx[4] dqy[4] s[4]: [12][ARY][ARX]
constexpr int QB_OFF = RA_OFF + 12 * NRING;     // q adjoint  [4][ABY][ABX]
constexpr int SH_OFF = QB_OFF + 4 * NBOX;       // (s*dtd)/2  [4][ARY][ARX] (dx == dy only)
constexpr int N_SMEM = SH_OFF + 4 * NRING;
constexpr size_t SMEM_BYTES = (size_t)N_SMEM * sizeof(double) + 64;

// One 32 x 7 tile (bx, by) of the reverse step; sm is the dynamic shared area.
// ubz (if set) is the adjoint buffer of the following reverse step: the
// tile's interior cells of it are zeroed here (nothing reads it now).
// SQ (dx == dy, so dtdx == dtdy): the face source term (s*dtd)*0.5 is formed
// once per ring cell, and the source adjoints are summed per unit dtd and
// scaled once per ring cell.
// TAPE: the primitives of the box, the slopes and sources of the ring and
// each face's HLLC solve are read from the tape the forward step wrote
// (TapeOut, face records required), not recomputed.
template <bool SQ, bool TAPE = false>
__device__ __forceinline__ void step_rev_tile(const Hydro<double>& h, Field<double> un, Field<double> ubn1,
                                              Field<double> ubn, Field<double> ubz, double dt, double* dtbar,
                                              int bx, int by, double* sm, const TapeOut& tape = TapeOut()) {
  double* sq = sm + Q_OFF;
  double* sdq = sm + DQ_OFF;
  double* ss = sm + S_OFF;
  double* sub = sm + UB_OFF;
  double* sra = sm + RA_OFF;
  double* sqb = sm + QB_OFF;
  double* ssh = sm + SH_OFF;
  __shared__ double red[2][ANT / 32];
  const int tid = threadIdx.x;
  const int i0 = GW + bx * ATX, j0 = GW + by * ATY;
  // (the integer-pipe division: the same bits as dt / dx, without the FP64
  // instructions every thread would otherwise spend on it)
  const double dtdx = Ops<double>::div(dt, h.dx), dtdy = Ops<double>::div(dt, h.dy);
  if (ubz.p) {
    for (int k = tid; k < 4 * ATX * ATY; k += ANT) {
      const int v = k / (ATX * ATY), rem = k - v * (ATX * ATY), y = rem / ATX, x = rem - y * ATX;
      if (i0 + x <= h.nx + 1 && j0 + y <= h.ny + 1) ubz.at(v, j0 + y, i0 + x) = 0.0;
    }
  }

  // ---- load U box, Ubar' of cells [i0-1, i0+ATX) x [j0-1, j0+ATY), zero accumulators
  for (int k = tid; k < 4 * NBOX; k += ANT) {
    const int v = k / NBOX, rem = k - v * NBOX, y = rem / ABX, x = rem - y * ABX;
    const int gi = i0 - GW + x, gj = j0 - GW + y;
    if constexpr (TAPE) sq[k] = (gi < h.isize && gj < h.jsize) ? tape.at(tape.q, v, gj, gi) : 0.0;
    else sq[k] = (gi < h.isize && gj < h.jsize) ? un.at(v, gj, gi) : 0.0;
    sqb[k] = 0.0;
  }
  for (int k = tid; k < 12 * NRING; k += ANT) sra[k] = 0.0;
  for (int k = tid; k < 4 * NUB; k += ANT) {
    const int v = k / NUB, rem = k - v * NUB, y = rem / (ATX + 1), x = rem - y * (ATX + 1);
    const int gi = i0 - 1 + x, gj = j0 - 1 + y;
    const bool interior = gi >= GW && gi <= h.nx + 1 && gj >= GW && gj <= h.ny + 1;
    sub[k] = interior ? ubn1.at(v, gj, gi) : 0.0;
  }
  __syncthreads();
  auto Q = [&](int v, int y, int x) -> double { return sq[(v * ABY + y) * ABX + x]; };
  if constexpr (TAPE) {
    for (int k = tid; k < NRING; k += ANT) {
      const int gi = i0 - GW + k % ARX + 1, gj = j0 - GW + k / ARX + 1;
      const bool in = gi <= h.nx + 2 && gj <= h.ny + 2;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        sdq[v * NRING + k] = in ? tape.at(tape.dq, v, gj, gi) : 0.0;
        sdq[(4 + v) * NRING + k] = in ? tape.at(tape.dq, 4 + v, gj, gi) : 0.0;
        const double sv = in ? tape.at(tape.s, v, gj, gi) : 0.0;
        ss[v * NRING + k] = sv;
        if constexpr (SQ) ssh[v * NRING + k] = Ops<double>::half(sv * dtdx);
      }
    }
  } else {
  // ---- forward recomputation: primitives (box), slopes and sources (ring)
  for (int k = tid; k < NBOX; k += ANT) {
    double u[4], q[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) u[v] = sq[v * NBOX + k];
    primitives(h, u, q);
#pragma unroll
    for (int v = 0; v < 4; ++v) sq[v * NBOX + k] = q[v];
  }
  __syncthreads();
  for (int k = tid; k < NRING; k += ANT) {
    const int x = k % ARX + 1, y = k / ARX + 1;
    double qc[4], qe[4], qw[4], qn[4], qs[4], dqx[4], dqy[4], s[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qc[v] = Q(v, y, x); qe[v] = Q(v, y, x + 1); qw[v] = Q(v, y, x - 1);
      qn[v] = Q(v, y + 1, x); qs[v] = Q(v, y - 1, x);
    }
    slopes(h, qc, qe, qw, qn, qs, dqx, dqy);
    trace_sources(h, qc, dqx, dqy, s);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      sdq[v * NRING + k] = dqx[v];
      sdq[(4 + v) * NRING + k] = dqy[v];
      ss[v * NRING + k] = s[v];
      if constexpr (SQ) ssh[v * NRING + k] = Ops<double>::half(s[v] * dtdx);
    }
  }
  }
  __syncthreads();

  // ---- owned faces: flux adjoint -> Riemann, trace reverse
  double dtdxb = 0.0, dtdyb = 0.0;
  auto UB = [&](int v, int i, int j) -> double {  // Ubar' of absolute cell (i, j), zero outside the interior
    const int x = i - (i0 - 1), y = j - (j0 - 1);
    return (x >= 0 && x <= ATX && y >= 0 && y <= ATY) ? sub[(v * (ATY + 1) + y) * (ATX + 1) + x] : 0.0;
  };
  // Faces in four passes -- x faces with even, then odd f; y faces with even,
  // then odd g -- so that no two faces of a pass touch the same cell and the
  // adjoints are added into shared memory without atomics.  A pass has at
  // most ANT faces: one per thread.
  constexpr int NFX_EVEN = ATX / 2 + 1, NFX_ODD = (ATX + 1) / 2;       // f in [0, ATX]
  constexpr int NGY_EVEN = ATY / 2 + 1, NGY_ODD = (ATY + 1) / 2;       // g in [0, ATY]
  static_assert(NFX_EVEN * ATY <= ANT && NGY_EVEN * ATX <= ANT, "one face per thread per pass");
#pragma unroll 1
  for (int pass = 0; pass < 4; ++pass) {
    const bool xface = pass < 2;
    const int par = pass & 1;
    const int nfx = par ? NFX_ODD : NFX_EVEN;
    const int nf = xface ? nfx * ATY : (par ? NGY_ODD : NGY_EVEN) * ATX;
    int a = 0, b = 0;  // ring indices of the two cells (left/lower, right/upper)
    int ia = 0, ja = 0;
    int fi = 0, fj = 0;  // the face's cell to its right / above it
    double fb[4];
    bool valid = tid < nf;
    if (xface) {
      const int f = 2 * (tid % nfx) + par, r = tid / nfx;
      const int i = i0 + f, j = j0 + r;
      fi = i; fj = j;
      valid = valid && i <= h.nx + 2 && j <= h.ny + 1 && (f < ATX || i == h.nx + 2);
#pragma unroll
      for (int v = 0; v < 4; ++v) fb[v] = valid ? UB(v, i, j) - UB(v, i - 1, j) : 0.0;
      a = (r + 1) * ARX + f;
      b = a + 1;
      ia = f + 1; ja = r + 2;  // box coordinates of the left cell
    } else {
      const int c = tid % ATX, g = 2 * (tid / ATX) + par;
      const int i = i0 + c, j = j0 + g;
      fi = i; fj = j;
      valid = valid && i <= h.nx + 1 && j <= h.ny + 2 && (g < ATY || j == h.ny + 2);
#pragma unroll
      for (int v = 0; v < 4; ++v) fb[v] = valid ? UB(v, i, j) - UB(v, i, j - 1) : 0.0;
      a = g * ARX + (c + 1);
      b = a + ARX;
      ia = c + 2; ja = g + 1;  // box coordinates of the lower cell
    }
    if (valid) {
      const double dtd = xface ? dtdx : dtdy;
      const int nrm = xface ? 0 : 4;  // slope block of the face normal
      double qa[4], qb_[4], dqa[4], dqb[4], sa[4], sb[4], sha[4], shb[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        qa[v] = Q(v, ja, ia);
        qb_[v] = xface ? Q(v, ja, ia + 1) : Q(v, ja + 1, ia);
        dqa[v] = sdq[(nrm + v) * NRING + a]; dqb[v] = sdq[(nrm + v) * NRING + b];
        sa[v] = ss[v * NRING + a]; sb[v] = ss[v * NRING + b];
        if constexpr (SQ) { sha[v] = ssh[v * NRING + a]; shb[v] = ssh[v * NRING + b]; }
      }
      double rb[4];
      if (xface) {
#pragma unroll
        for (int v = 0; v < 4; ++v) rb[v] = fb[v] * dtd;
      } else {  // the stored y flux is the Riemann flux with IU and IV swapped back
        rb[ID] = fb[ID] * dtd; rb[IP] = fb[IP] * dtd; rb[IU] = fb[IV] * dtd; rb[IV] = fb[IU] * dtd;
      }
      double qlb[4] = {0, 0, 0, 0}, qrb[4] = {0, 0, 0, 0}, flux[4];
      if constexpr (TAPE) {  // the face's solve, recorded by the forward step
        double rec[HR_N];
        double* fr = xface ? tape.fx : tape.fy;
#pragma unroll
        for (int e = 0; e < HR_N; ++e) rec[e] = tape.at(fr, e, fj, fi);
        const unsigned fl = tape.flag(xface ? tape.flx : tape.fly, fj, fi);
        adj::riemann_hllc_rev_rec(h, rec, fl, rb, qlb, qrb);
#pragma unroll
        for (int v = 0; v < 4; ++v) flux[v] = rec[HR_FLUX + v];
      } else {
        double ql[4], qr[4];
        if constexpr (SQ) {
          trace_face<double, true, true>(h, qa, dqa, sha, dtd, ql);
          trace_face<double, false, true>(h, qb_, dqb, shb, dtd, qr);
        } else {
          trace_face<double, true>(h, qa, dqa, sa, dtd, ql);
          trace_face<double, false>(h, qb_, dqb, sb, dtd, qr);
        }
        if (!xface) {
          double t = ql[IU]; ql[IU] = ql[IV]; ql[IV] = t;
          t = qr[IU]; qr[IU] = qr[IV]; qr[IV] = t;
        }
        adj::riemann_hllc_rev(h, ql, qr, rb, qlb, qrb, flux);
      }
      if (xface) {
#pragma unroll
        for (int v = 0; v < 4; ++v) dtdxb += flux[v] * fb[v];
      } else {
        dtdyb += flux[ID] * fb[ID] + flux[IP] * fb[IP] + flux[IV] * fb[IU] + flux[IU] * fb[IV];
      }
      if (!xface) {
        double t = qlb[IU]; qlb[IU] = qlb[IV]; qlb[IV] = t;
        t = qrb[IU]; qrb[IU] = qrb[IV]; qrb[IV] = t;
      }
      double qab[4], dqab[4], sab[4], qbb[4], dqbb[4], sbb[4];
      // (a local accumulator: a reference selecting dtdxb or dtdyb would put
      // both in local memory)
      double dtdb = 0.0;
      adj::trace_face_rev<true, SQ>(h, qa, dqa, sa, sha, dtd, qlb, qab, dqab, sab, dtdb);
      adj::trace_face_rev<false, SQ>(h, qb_, dqb, sb, shb, dtd, qrb, qbb, dqbb, sbb, dtdb);
      if (xface) dtdxb += dtdb;
      else dtdyb += dtdb;
      const int ka = ja * ABX + ia;
      const int kb = xface ? ka + 1 : ka + ABX;
      // (pass 0 writes first to its cells' sums, x-slope and source slots,
      // pass 2 to its cells' y-slope slots: stores, not additions to zero)
      if (pass == 0) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          sqb[v * NBOX + ka] = qab[v];
          sqb[v * NBOX + kb] = qbb[v];
          sra[v * NRING + a] = dqab[v];
          sra[v * NRING + b] = dqbb[v];
          sra[(8 + v) * NRING + a] = sab[v];
          sra[(8 + v) * NRING + b] = sbb[v];
        }
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          sqb[v * NBOX + ka] += qab[v];
          sqb[v * NBOX + kb] += qbb[v];
          if (pass == 2) {
            sra[(nrm + v) * NRING + a] = dqab[v];
            sra[(nrm + v) * NRING + b] = dqbb[v];
          } else {
            sra[(nrm + v) * NRING + a] += dqab[v];
            sra[(nrm + v) * NRING + b] += dqbb[v];
          }
          sra[(8 + v) * NRING + a] += sab[v];
          sra[(8 + v) * NRING + b] += sbb[v];
        }
      }
    }
    __syncthreads();
  }

  // ---- ring cells: sources and slopes reverse.  A ring cell adds its own
  // (centre) adjoint to its box cell and leaves the adjoints of its four
  // limiter neighbours in its own slots -- east in the dq_x adjoint, west in
  // the dq_y adjoint, north in the source adjoint, south in the source
  // values, none of which anyone else reads now -- so no two threads write
  // the same word; the box pass below gathers them.
  const bool mc = h.slope_type == 2;
  const bool lim = h.slope_type == 1 || h.slope_type == 2;
  for (int k = tid; k < NRING; k += ANT) {
    const int x = k % ARX + 1, y = k / ARX + 1;
    double qc[4], dqx[4], dqy[4], sbar[4], dqxb[4], dqyb[4], qcb[4] = {0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qc[v] = Q(v, y, x);
      dqx[v] = sdq[v * NRING + k]; dqy[v] = sdq[(4 + v) * NRING + k];
      dqxb[v] = sra[v * NRING + k]; dqyb[v] = sra[(4 + v) * NRING + k];
      sbar[v] = sra[(8 + v) * NRING + k];
      if constexpr (SQ) sbar[v] = sbar[v] * dtdx;  // summed per unit dtd by the face pass
    }
    adj::trace_sources_rev(h, qc, dqx, dqy, sbar, qcb, dqxb, dqyb);
    const int kc = y * ABX + x;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double qe = 0, qw = 0, qn = 0, qs = 0;
      if (lim) {
        adj::slope1_rev(mc, qc[v], Q(v, y, x + 1), Q(v, y, x - 1), dqxb[v], qcb[v], qe, qw);
        adj::slope1_rev(mc, qc[v], Q(v, y + 1, x), Q(v, y - 1, x), dqyb[v], qcb[v], qn, qs);
      }
      sqb[v * NBOX + kc] += qcb[v];
      sra[v * NRING + k] = qe;
      sra[(4 + v) * NRING + k] = qw;
      sra[(8 + v) * NRING + k] = qn;
      ss[v * NRING + k] = qs;
    }
  }
  __syncthreads();

  // ---- box cells: gather the limiter neighbours' adjoints, primitives
  // reverse, fold ghosts back, identity part of the update
  auto ring_of = [&](int x, int y) -> int {  // ring index of box cell (x, y), -1 if not a ring cell
    return (x >= 1 && x <= ARX && y >= 1 && y <= ARY) ? (y - 1) * ARX + (x - 1) : -1;
  };
  for (int k = tid; k < NBOX; k += ANT) {
    const int y = k / ABX, x = k - y * ABX;
    const int gi = i0 - GW + x, gj = j0 - GW + y;
    if (gi >= h.isize || gj >= h.jsize) continue;
    const bool xin = gi >= GW && gi <= h.nx + 1, yin = gj >= GW && gj <= h.ny + 1;
    if (!xin && !yin) continue;  // corner: a constant
    double qb[4], u[4], ub[4] = {0, 0, 0, 0};
    const int rw = ring_of(x - 1, y), re = ring_of(x + 1, y), rs = ring_of(x, y - 1), rn = ring_of(x, y + 1);
    bool any = false;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double t = sqb[v * NBOX + k];
      if (rw >= 0) t += sra[v * NRING + rw];          // west neighbour's east adjoint
      if (re >= 0) t += sra[(4 + v) * NRING + re];    // east neighbour's west adjoint
      if (rs >= 0) t += sra[(8 + v) * NRING + rs];    // south neighbour's north adjoint
      if (rn >= 0) t += ss[v * NRING + rn];           // north neighbour's south adjoint
      qb[v] = t;
      any |= (emul::bits(t) << 1) != 0;  // t != 0, decided on the integer pipe
    }
    if (any) {
      double qf[4];  // the forward primitives, still in the box
#pragma unroll
      for (int v = 0; v < 4; ++v) { u[v] = un.at(v, gj, gi); qf[v] = sq[v * NBOX + k]; }
      adj::primitives_rev_q(h, u, qf, qb, ub);
    }
    if (xin && yin) {
      // own interior cells of this tile also carry Ubar' through U' = U + ...
      if (gi >= i0 && gi < i0 + ATX && gj >= j0 && gj < j0 + ATY) {
#pragma unroll
        for (int v = 0; v < 4; ++v) ub[v] += UB(v, gi, gj);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v)
        if ((emul::bits(ub[v]) << 1) != 0) atomicAdd(&ubn.at(v, gj, gi), ub[v]);
    } else if (any) {
      int si = gi, sj = gj, type, flip;
      if (!xin) {
        type = gi < GW ? h.bc_xmin : h.bc_xmax;
        si = ghost_source(gi, h.nx, type);
        flip = IU;
      } else {
        type = gj < GW ? h.bc_ymin : h.bc_ymax;
        sj = ghost_source(gj, h.ny, type);
        flip = IV;
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double g = Ops<double>::neg_if(ub[v], type == 1 && v == flip);
        if ((emul::bits(g) << 1) != 0) atomicAdd(&ubn.at(v, sj, si), g);  // g != 0
      }
    }
  }
  // ---- dt adjoint: dtdx = dt/dx, dtdy = dt/dy
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dtdxb += __shfl_xor_sync(0xffffffffu, dtdxb, o);
    dtdyb += __shfl_xor_sync(0xffffffffu, dtdyb, o);
  }
  if ((tid & 31) == 0) { red[0][tid >> 5] = dtdxb; red[1][tid >> 5] = dtdyb; }
  __syncthreads();
  if (tid == 0) {
    double sx = 0, sy = 0;
    for (int w = 0; w < ANT / 32; ++w) { sx += red[0][w]; sy += red[1][w]; }
    atomicAdd(dtbar, sx / h.dx + sy / h.dy);
  }
}

// ---- the reverse step of square cells reading a tape, in less shared memory
//
// With a tape and dx == dy the face pass needs neither the slopes nor the
// sources of its cells: the face states (and whether the density floor
// acted on them) are in the face's recorded solve, and the dt adjoint of the
// face source terms, sum over a cell's face states of s * (face adjoint)/2,
// is s times the cell's summed source adjoint, which the ring pass forms
// from the tape's s.  The ring pass reads the slopes and sources from the
// tape in global memory, and the slopes' reverse takes the limiter cases the
// forward step recorded (nothing of the slopes is recomputed).  Shared memory
// then holds the primitives box, the next adjoint, the ring and box adjoints
// and one scratch plane set: 73 KB, so three CTAs of 128 threads fit on an
// SM instead of two.
#ifndef E2D_REVT_MINB
#define E2D_REVT_MINB 3
#endif
constexpr int T_Q_OFF = 0;                    // q box      [4][ABY][ABX] (the tape's primitives)
constexpr int T_UB_OFF = T_Q_OFF + 4 * NBOX;  // Ubar'      [4][ATY+1][ATX+1]
constexpr int T_RA_OFF = T_UB_OFF + 4 * NUB;  // ring adj.  dqx[4] dqy[4] s[4]: [12][ARY][ARX]
constexpr int T_QB_OFF = T_RA_OFF + 12 * NRING;  // q adjoint  [4][ABY][ABX]
constexpr int T_SC_OFF = T_QB_OFF + 4 * NBOX;  // scratch    [4][ARY][ARX] (south limiter adjoints)
constexpr int T_N_SMEM = T_SC_OFF + 4 * NRING;
constexpr size_t T_SMEM_BYTES = (size_t)T_N_SMEM * sizeof(double) + 64;

__device__ __forceinline__ void step_rev_tile_tsq(const Hydro<double>& h, Field<double> un, Field<double> ubn1,
                                                  Field<double> ubn, Field<double> ubz, double dt, double* dtbar,
                                                  int bx, int by, double* sm, const TapeOut& tape) {
  double* sq = sm + T_Q_OFF;
  double* sub = sm + T_UB_OFF;
  double* sra = sm + T_RA_OFF;
  double* sqb = sm + T_QB_OFF;
  double* ssc = sm + T_SC_OFF;
  __shared__ double red[ANT / 32];
  const int tid = threadIdx.x;
  const int i0 = GW + bx * ATX, j0 = GW + by * ATY;
  const double dtdx = Ops<double>::div(dt, h.dx);  // == dt / dy
  if (ubz.p) {
    for (int k = tid; k < 4 * ATX * ATY; k += ANT) {
      const int v = k / (ATX * ATY), rem = k - v * (ATX * ATY), y = rem / ATX, x = rem - y * ATX;
      if (i0 + x <= h.nx + 1 && j0 + y <= h.ny + 1) ubz.at(v, j0 + y, i0 + x) = 0.0;
    }
  }
  for (int k = tid; k < 4 * NBOX; k += ANT) {
    const int v = k / NBOX, rem = k - v * NBOX, y = rem / ABX, x = rem - y * ABX;
    const int gi = i0 - GW + x, gj = j0 - GW + y;
    sq[k] = (gi < h.isize && gj < h.jsize) ? tape.at(tape.q, v, gj, gi) : 0.0;
    sqb[k] = 0.0;
  }
  // (the source adjoints, planes 8-11, are not accumulated by the faces: a
  // cell's is half its face states' summed adjoint, which sqb holds; the
  // ring pass writes those planes before anything reads them)
  for (int k = tid; k < 8 * NRING; k += ANT) sra[k] = 0.0;
  for (int k = tid; k < 4 * NUB; k += ANT) {
    const int v = k / NUB, rem = k - v * NUB, y = rem / (ATX + 1), x = rem - y * (ATX + 1);
    const int gi = i0 - 1 + x, gj = j0 - 1 + y;
    const bool interior = gi >= GW && gi <= h.nx + 1 && gj >= GW && gj <= h.ny + 1;
    sub[k] = interior ? ubn1.at(v, gj, gi) : 0.0;
  }
  __syncthreads();
  auto Q = [&](int v, int y, int x) -> double { return sq[(v * ABY + y) * ABX + x]; };
  auto UB = [&](int v, int i, int j) -> double {  // Ubar' of absolute cell (i, j), zero outside the interior
    const int x = i - (i0 - 1), y = j - (j0 - 1);
    return (x >= 0 && x <= ATX && y >= 0 && y <= ATY) ? sub[(v * (ATY + 1) + y) * (ATX + 1) + x] : 0.0;
  };

  // ---- owned faces (four conflict-free passes, as in step_rev_tile):
  // flux adjoint -> recorded Riemann solve reverse -> face-state adjoints
  // added to the cell, its normal slope and its (per unit dtdx) sources
  double dtb = 0.0;  // dt/dx adjoint of the fluxes
  constexpr int NFX_EVEN = ATX / 2 + 1, NFX_ODD = (ATX + 1) / 2;
  constexpr int NGY_EVEN = ATY / 2 + 1, NGY_ODD = (ATY + 1) / 2;
  static_assert(NFX_EVEN * ATY <= ANT && NGY_EVEN * ATX <= ANT, "one face per thread per pass");
#pragma unroll 1
  for (int pass = 0; pass < 4; ++pass) {
    const bool xface = pass < 2;
    const int par = pass & 1;
    const int nfx = par ? NFX_ODD : NFX_EVEN;
    const int nf = xface ? nfx * ATY : (par ? NGY_ODD : NGY_EVEN) * ATX;
    int a = 0, b = 0, ka = 0, kb = 0, fi = 0, fj = 0;
    double fb[4];
    bool valid = tid < nf;
    if (xface) {
      const int f = 2 * (tid % nfx) + par, r = tid / nfx;
      fi = i0 + f; fj = j0 + r;
      valid = valid && fi <= h.nx + 2 && fj <= h.ny + 1 && (f < ATX || fi == h.nx + 2);
#pragma unroll
      for (int v = 0; v < 4; ++v) fb[v] = valid ? UB(v, fi, fj) - UB(v, fi - 1, fj) : 0.0;
      a = (r + 1) * ARX + f;
      b = a + 1;
      ka = (r + 2) * ABX + (f + 1);
      kb = ka + 1;
    } else {
      const int c = tid % ATX, g = 2 * (tid / ATX) + par;
      fi = i0 + c; fj = j0 + g;
      valid = valid && fi <= h.nx + 1 && fj <= h.ny + 2 && (g < ATY || fj == h.ny + 2);
#pragma unroll
      for (int v = 0; v < 4; ++v) fb[v] = valid ? UB(v, fi, fj) - UB(v, fi, fj - 1) : 0.0;
      a = g * ARX + (c + 1);
      b = a + ARX;
      ka = (g + 1) * ABX + (c + 2);
      kb = ka + ABX;
    }
    if (valid) {
      double rb[4];
      if (xface) {
#pragma unroll
        for (int v = 0; v < 4; ++v) rb[v] = fb[v] * dtdx;
      } else {  // the stored y flux is the Riemann flux with IU and IV swapped back
        rb[ID] = fb[ID] * dtdx; rb[IP] = fb[IP] * dtdx; rb[IU] = fb[IV] * dtdx; rb[IV] = fb[IU] * dtdx;
      }
      double rec[HR_N];
      double* fr = xface ? tape.fx : tape.fy;
#pragma unroll
      for (int e = 0; e < HR_N; ++e) rec[e] = tape.at(fr, e, fj, fi);
      const unsigned fl = tape.flag(xface ? tape.flx : tape.fly, fj, fi);
      double qlb[4] = {0, 0, 0, 0}, qrb[4] = {0, 0, 0, 0};
      adj::riemann_hllc_rev_rec(h, rec, fl, rb, qlb, qrb);
      if (xface) {
#pragma unroll
        for (int v = 0; v < 4; ++v) dtb += rec[HR_FLUX + v] * fb[v];
      } else {
        dtb += rec[HR_FLUX + ID] * fb[ID] + rec[HR_FLUX + IP] * fb[IP] + rec[HR_FLUX + IV] * fb[IU] +
               rec[HR_FLUX + IU] * fb[IV];
        double t = qlb[IU]; qlb[IU] = qlb[IV]; qlb[IV] = t;
        t = qrb[IU]; qrb[IU] = qrb[IV]; qrb[IV] = t;
      }
      // density floor max(smallr, raw) of each face state, from the
      // recorded state: no gradient where it returned smallr
      if (!emul::gt_i(rec[HR_QL + ID], h.smallr)) qlb[ID] = 0.0;
      if (!emul::gt_i(rec[HR_QR + ID], h.smallr)) qrb[ID] = 0.0;
      const int nrm = xface ? 0 : 4;  // slope block of the face normal
      // The slots start at zero and the passes run in order: pass 0 (even x
      // faces) writes first to its cells' sums and x-slope slots, pass 2
      // (even y faces) first to its cells' y-slope slots, so those writes
      // are stores (0 + x is x: the same bits) and not additions.
      if (pass == 0) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          sqb[v * NBOX + ka] = qlb[v];
          sqb[v * NBOX + kb] = qrb[v];
          sra[v * NRING + a] = Ops<double>::half(qlb[v]);
          sra[v * NRING + b] = Ops<double>::neg_if(Ops<double>::half(qrb[v]), true);
        }
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const double hl = Ops<double>::half(qlb[v]), hr = Ops<double>::half(qrb[v]);
          sqb[v * NBOX + ka] += qlb[v];         // cell a's plus face (XMAX / YMAX)
          sqb[v * NBOX + kb] += qrb[v];         // cell b's minus face
          if (pass == 2) {
            sra[(nrm + v) * NRING + a] = hl;
            sra[(nrm + v) * NRING + b] = Ops<double>::neg_if(hr, true);
          } else {
            sra[(nrm + v) * NRING + a] += hl;
            sra[(nrm + v) * NRING + b] -= hr;
          }
        }
      }
    }
    __syncthreads();
  }

  // ---- ring cells: the dt adjoint of their face source terms, then
  // sources and slopes reverse (limiter neighbours' adjoints left in the
  // cell's own slots for the box pass, as in step_rev_tile)
  const bool mc = h.slope_type == 2;
  const bool lim = h.slope_type == 1 || h.slope_type == 2;
  double dts = 0.0;  // dt/dx adjoint of the source terms
  for (int k = tid; k < NRING; k += ANT) {
    const int x = k % ARX + 1, y = k / ARX + 1;
    const int gi = i0 - GW + x, gj = j0 - GW + y;
    const bool in = gi <= h.nx + 2 && gj <= h.ny + 2;
    const int kc = y * ABX + x;
    double qc[4], dqx[4], dqy[4], sbar[4], dqxb[4], dqyb[4], qcb[4] = {0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qc[v] = Q(v, y, x);
      dqx[v] = in ? tape.at(tape.dq, v, gj, gi) : 0.0;
      dqy[v] = in ? tape.at(tape.dq, 4 + v, gj, gi) : 0.0;
      const double sv = in ? tape.at(tape.s, v, gj, gi) : 0.0;
      dqxb[v] = sra[v * NRING + k]; dqyb[v] = sra[(4 + v) * NRING + k];
      // the source adjoint per unit dtdx: half the cell's face-state
      // adjoints, summed in sqb by the face pass (halving is exact, so this
      // is bit for bit the sum of the halves)
      const double sb = Ops<double>::half(sqb[v * NBOX + kc]);
      dts += sv * sb;
      sbar[v] = sb * dtdx;
    }
    adj::trace_sources_rev(h, qc, dqx, dqy, sbar, qcb, dqxb, dqyb);
    const unsigned cases = (in && lim) ? tape.flag(tape.lim, gj, gi) : 0u;  // the forward's limiter cases
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double qe, qw, qn, qs;
      adj::slope1_rev_case(mc, cases >> (3 * v), dqxb[v], qcb[v], qe, qw);
      adj::slope1_rev_case(mc, cases >> (12 + 3 * v), dqyb[v], qcb[v], qn, qs);
      sqb[v * NBOX + kc] += qcb[v];
      sra[v * NRING + k] = qe;
      sra[(4 + v) * NRING + k] = qw;
      sra[(8 + v) * NRING + k] = qn;
      ssc[v * NRING + k] = qs;
    }
  }
  __syncthreads();

  // ---- box cells: gather, primitives reverse, ghost folding, update identity
  auto ring_of = [&](int x, int y) -> int {
    return (x >= 1 && x <= ARX && y >= 1 && y <= ARY) ? (y - 1) * ARX + (x - 1) : -1;
  };
  for (int k = tid; k < NBOX; k += ANT) {
    const int y = k / ABX, x = k - y * ABX;
    const int gi = i0 - GW + x, gj = j0 - GW + y;
    if (gi >= h.isize || gj >= h.jsize) continue;
    const bool xin = gi >= GW && gi <= h.nx + 1, yin = gj >= GW && gj <= h.ny + 1;
    if (!xin && !yin) continue;  // corner: a constant
    double qb[4], u[4], ub[4] = {0, 0, 0, 0};
    const int rw = ring_of(x - 1, y), re = ring_of(x + 1, y), rs = ring_of(x, y - 1), rn = ring_of(x, y + 1);
    bool any = false;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double t = sqb[v * NBOX + k];
      if (rw >= 0) t += sra[v * NRING + rw];
      if (re >= 0) t += sra[(4 + v) * NRING + re];
      if (rs >= 0) t += sra[(8 + v) * NRING + rs];
      if (rn >= 0) t += ssc[v * NRING + rn];
      qb[v] = t;
      any |= (emul::bits(t) << 1) != 0;
    }
    if (any) {
      double qf[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) { u[v] = un.at(v, gj, gi); qf[v] = sq[v * NBOX + k]; }
      adj::primitives_rev_q(h, u, qf, qb, ub);
    }
    if (xin && yin) {
      if (gi >= i0 && gi < i0 + ATX && gj >= j0 && gj < j0 + ATY) {
#pragma unroll
        for (int v = 0; v < 4; ++v) ub[v] += UB(v, gi, gj);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v)
        if ((emul::bits(ub[v]) << 1) != 0) atomicAdd(&ubn.at(v, gj, gi), ub[v]);
    } else if (any) {
      int si = gi, sj = gj, type, flip;
      if (!xin) {
        type = gi < GW ? h.bc_xmin : h.bc_xmax;
        si = ghost_source(gi, h.nx, type);
        flip = IU;
      } else {
        type = gj < GW ? h.bc_ymin : h.bc_ymax;
        sj = ghost_source(gj, h.ny, type);
        flip = IV;
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double g = Ops<double>::neg_if(ub[v], type == 1 && v == flip);
        if ((emul::bits(g) << 1) != 0) atomicAdd(&ubn.at(v, sj, si), g);
      }
    }
  }
  // ---- dt adjoint: dtdx = dt/dx (== dt/dy)
  double d = dtb + dts;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if ((tid & 31) == 0) red[tid >> 5] = d;
  __syncthreads();
  if (tid == 0) {
    double sx = 0;
    for (int w = 0; w < ANT / 32; ++w) sx += red[w];
    atomicAdd(dtbar, sx / h.dx);
  }
}

__global__ void __launch_bounds__(ANT, E2D_REVT_MINB)
    k_step_rev_tsq(Hydro<double> h, Field<double> un, Field<double> ubn1, Field<double> ubn, Field<double> ubz,
                   const double* dt, double* dtbar, TapeOut tape) {
  extern __shared__ double sm[];
  step_rev_tile_tsq(h, un, ubn1, ubn, ubz, *dt, dtbar, blockIdx.x, blockIdx.y, sm, tape);
}

template <bool SQ, bool TAPE>
__global__ void __launch_bounds__(ANT, E2D_REV_MINB)
    k_step_rev(Hydro<double> h, Field<double> un, Field<double> ubn1, Field<double> ubn, Field<double> ubz,
               const double* dt, double* dtbar, TapeOut tape) {
  extern __shared__ double sm[];
  step_rev_tile<SQ, TAPE>(h, un, ubn1, ubn, ubz, *dt, dtbar, blockIdx.x, blockIdx.y, sm, tape);
}

// The 2x2 ghost corners are never written by a step, so a state keeps the
// corners of the buffer it lands in: the initial state's in u (even steps),
// zeros in u2 (odd steps).  Segment buffer j = 1..nseg-1 (state k0 + j)
// receives the corners of ping-pong buffer (k0 + j) & 1 before recomputation.
// 64 threads: var (4) x corner (4) x 2 x 2.
__device__ __forceinline__ void copy_corner(const double* src, double* dst, int pitch, long long plane, int isize,
                                            int jsize, int t) {
  const int v = t >> 4, c = (t >> 2) & 3, dy = (t >> 1) & 1, dx = t & 1;
  const int i = (c & 1) ? isize - 2 + dx : dx, jj = (c & 2) ? jsize - 2 + dy : dy;
  const long long o = v * plane + (long long)jj * pitch + i;
  dst[o] = src[o];
}

__global__ void k_seg_corners(double* pool, long long state_elems, int pitch, long long plane, int isize, int jsize,
                              int ping_index, int seg_index, int k0) {
  const int j = blockIdx.x + 1;
  if (threadIdx.x >= 64) return;
  copy_corner(pool + (long long)(ping_index + ((k0 + j) & 1)) * state_elems,
              pool + (long long)(seg_index + j) * state_elems, pitch, plane, isize, jsize, threadIdx.x);
}

// Does the running CFL maximum rise at state m?  (The maxima are logged with
// stride `stride`: one entry per problem and step.)
__device__ __forceinline__ bool max_rises(const double* inv_log, int m, int stride) {
  return m == 0 || inv_log[(long long)m * stride] > inv_log[(long long)(m - 1) * stride];
}

// Largest compute_dt term of a state and the cell (i + j*isize) that has it;
// on equal terms the lowest index wins.  CTA `part` of `nparts` takes every
// nparts-th row; 256 threads.
__device__ __forceinline__ void argmax_part(const Hydro<double>& h, Field<double> u, int part, int nparts, double* pv,
                                            long long* pi) {
  double best = -1.0;
  long long bi = 0x7fffffffffffffffll;
  for (int j = GW + part; j <= h.jsize - 4; j += nparts)
    for (int i = GW + threadIdx.x; i <= h.isize - 4; i += blockDim.x) {
      double uc[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) uc[v] = u.at(v, j, i);
      const double t = cell_invdt(h, uc);
      const long long idx = (long long)j * h.isize + i;
      if (t > best || (t == best && idx < bi)) { best = t; bi = idx; }
    }
  // (largest term, lowest index) is a total order: any reduction order gives
  // the same cell
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, best, o);
    const long long i2 = __shfl_xor_sync(0xffffffffu, bi, o);
    if (v2 > best || (v2 == best && i2 < bi)) { best = v2; bi = i2; }
  }
  __shared__ double sv[32];
  __shared__ long long si[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { sv[warp] = best; si[warp] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; ++w)
      if (sv[w] > best || (sv[w] == best && si[w] < bi)) { best = sv[w]; bi = si[w]; }
    pv[part] = best;
    pi[part] = bi;
  }
}

// If the running maximum rises at state m, the steps [m, n1) up to the next
// rise use the compute_dt term of the argmax cell of state m; their dt
// adjoints go to Ubar_m: dt_n = cfl / inv_n, d dt_n / d inv_n = -cfl / inv_n^2.
// One block of kDtThreads threads (all call it); logs have stride `stride`.
// The partial maxima, the search for n1 and the sum are spread over the
// block: the routing sits between two reverse steps, so its latency is the
// gradient's.
constexpr int kDtThreads = 256;
__device__ __forceinline__ void dt_route(const Hydro<double>& h, Field<double> u, Field<double> ub, const double* pv,
                                         const long long* pi, int nparts, const double* dtbar_log,
                                         const double* inv_log, int stride, int m, int nsteps) {
  constexpr int NW = kDtThreads / 32;
  __shared__ double sbest[NW], ssum[NW];
  __shared__ long long sidx[NW];
  __shared__ int sn1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // the argmax over the partial results (largest term, lowest index on ties)
  double best = -1.0;
  long long bi = 0x7fffffffffffffffll;
  for (int k = tid; k < nparts; k += kDtThreads)
    if (pv[k] > best || (pv[k] == best && pi[k] < bi)) { best = pv[k]; bi = pi[k]; }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, best, o);
    const long long i2 = __shfl_xor_sync(0xffffffffu, bi, o);
    if (v2 > best || (v2 == best && i2 < bi)) { best = v2; bi = i2; }
  }
  if (lane == 0) { sbest[warp] = best; sidx[warp] = bi; }
  if (tid == 0) sn1 = nsteps;
  __syncthreads();
  // n1: the next state after m where the maximum rises (or nsteps); a
  // thread's first rise is the smallest of its stride
  for (int n = m + 1 + tid; n < nsteps; n += kDtThreads)
    if (max_rises(inv_log, n, stride)) {
      atomicMin(&sn1, n);
      break;
    }
  __syncthreads();
  const int n1 = sn1;
  double sacc = 0.0;
  for (int n = m + tid; n < n1; n += kDtThreads) {
    const double inv = inv_log[(long long)n * stride];
    sacc += -h.cfl / (inv * inv) * dtbar_log[(long long)n * stride];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
  if (lane == 0) ssum[warp] = sacc;
  __syncthreads();
  if (tid != 0) return;
  best = sbest[0];
  bi = sidx[0];
  sacc = ssum[0];
  for (int w = 1; w < NW; ++w) {
    if (sbest[w] > best || (sbest[w] == best && sidx[w] < bi)) { best = sbest[w]; bi = sidx[w]; }
    sacc += ssum[w];
  }
  const int j = (int)(bi / h.isize), i = (int)(bi - (long long)j * h.isize);
  double uc[4], g[4] = {0, 0, 0, 0};
#pragma unroll
  for (int v = 0; v < 4; ++v) uc[v] = u.at(v, j, i);
  adj::cell_invdt_rev(h, uc, sacc, g);
#pragma unroll
  for (int v = 0; v < 4; ++v) ub.at(v, j, i) += g[v];
}

__global__ void k_argmax_partial(Hydro<double> h, Field<double> u, double* pv, long long* pi, const double* inv_log,
                                 int m) {
  if (!max_rises(inv_log, m, 1)) return;  // only states where the running maximum rises
  argmax_part(h, u, blockIdx.x, gridDim.x, pv, pi);
}

__global__ void k_dt_route(Hydro<double> h, Field<double> u, Field<double> ub, const double* pv,
                           const long long* pi, int nparts, const double* dtbar_log, const double* inv_log, int m,
                           int nsteps) {
  if (!max_rises(inv_log, m, 1)) return;  // uniform over the block
  dt_route(h, u, ub, pv, pi, nparts, dtbar_log, inv_log, 1, m, nsteps);
}

// J = sum over interior cells of rho^2 w(x, y), w a Gaussian of width sigma
// centred at (xc, yc), cell centres x = (i - 2 + 1/2) dx; and dJ/dU.
__device__ __forceinline__ double weight(const Hydro<double>& h, int i, int j, double xc, double yc, double sig) {
  const double x = (i - GW + 0.5) * h.dx, y = (j - GW + 0.5) * h.dy;
  return exp(-((x - xc) * (x - xc) + (y - yc) * (y - yc)) / (2.0 * sig * sig));
}

// Grid-stride over the interior with `nthreads` threads numbered `t`.
__device__ __forceinline__ void objective_part(const Hydro<double>& h, Field<double> u, double xc, double yc,
                                               double sig, double* J, Field<double> ub, long long t,
                                               long long nthreads) {
  double acc = 0.0;
  for (long long k = t; k < (long long)h.nx * h.ny; k += nthreads) {
    const int i = GW + (int)(k % h.nx), j = GW + (int)(k / h.nx);
    const double w = weight(h, i, j, xc, yc, sig);
    const double r = u.at(ID, j, i);
    acc += r * r * w;
    if (ub.p) {
      ub.at(ID, j, i) = 2.0 * r * w;
      ub.at(IP, j, i) = 0.0;
      ub.at(IU, j, i) = 0.0;
      ub.at(IV, j, i) = 0.0;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(J, acc);
}

__global__ void k_objective(Hydro<double> h, Field<double> u, double xc, double yc, double sig, double* J,
                            Field<double> ub) {
  objective_part(h, u, xc, yc, sig, J, ub, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                 (long long)gridDim.x * blockDim.x);
}

// ---- batched kernels: every problem of an ensemble in one launch ----------

__device__ __forceinline__ double* abuf(const AdjProb& P, int k) {
  return k < 0 ? P.u0 : P.base + (long long)k * P.state_elems;
}
__device__ __forceinline__ Field<double> afield(const AdjProb& P, int k) {
  return Field<double>{abuf(P, k), P.pitch, P.plane};
}

// Reverse step m of every problem: one CTA per 32 x 7 tile of the flattened
// tile list (problem p owns tiles [tile_begin, tile_begin + ntx * nty)).
template <bool SQ, bool TAPE>
__global__ void __launch_bounds__(ANT, E2D_REV_MINB)
    k_batch_step_rev(const AdjProb* __restrict__ probs, int nprob, const double* dt_log, double* dtbar_log, int un,
                     int ub_in, int ub_out, int ub_zero, int m, int tape_j) {
  extern __shared__ double sm[];
  __shared__ Hydro<double> sh;
  __shared__ int sp;
  const int t = blockIdx.x;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nprob - 1;  // last problem with tile_begin <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (probs[mid].tile_begin <= t) lo = mid;
      else hi = mid - 1;
    }
    sp = lo;
    sh = probs[lo].h;
  }
  __syncthreads();
  const AdjProb& P = probs[sp];
  const int tile = t - P.tile_begin;
  const long long row = (long long)m * nprob + sp;
  const TapeOut tp = TAPE ? tape_at(P.tape_base, tape_j, P.plane, P.pitch, false) : TapeOut();
  step_rev_tile<SQ, TAPE>(sh, afield(P, un), afield(P, ub_in), afield(P, ub_out),
                          ub_zero >= 0 ? afield(P, ub_zero) : Field<double>{nullptr, 0, 0}, dt_log[row],
                          dtbar_log + row, tile % P.ntx, tile / P.ntx, sm, tp);
}

// The batched reverse step of square cells reading the tape (see step_rev_tile_tsq).
__global__ void __launch_bounds__(ANT, E2D_REVT_MINB)
    k_batch_step_rev_tsq(const AdjProb* __restrict__ probs, int nprob, const double* dt_log, double* dtbar_log,
                         int un, int ub_in, int ub_out, int ub_zero, int m, int tape_j) {
  extern __shared__ double sm[];
  __shared__ Hydro<double> sh;
  __shared__ int sp;
  const int t = blockIdx.x;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nprob - 1;  // last problem with tile_begin <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (probs[mid].tile_begin <= t) lo = mid;
      else hi = mid - 1;
    }
    sp = lo;
    sh = probs[lo].h;
  }
  __syncthreads();
  const AdjProb& P = probs[sp];
  const int tile = t - P.tile_begin;
  const long long row = (long long)m * nprob + sp;
  step_rev_tile_tsq(sh, afield(P, un), afield(P, ub_in), afield(P, ub_out),
                    ub_zero >= 0 ? afield(P, ub_zero) : Field<double>{nullptr, 0, 0}, dt_log[row], dtbar_log + row,
                    tile % P.ntx, tile / P.ntx, sm, tape_at(P.tape_base, tape_j, P.plane, P.pitch, false));
}

__global__ void k_batch_argmax(const AdjProb* __restrict__ probs, int nprob, const double* inv_log, int un, int m,
                               double* pv, long long* pi) {
  const int p = blockIdx.y;
  if (!max_rises(inv_log + p, m, nprob)) return;
  const AdjProb& P = probs[p];
  argmax_part(P.h, afield(P, un), blockIdx.x, gridDim.x, pv + (long long)p * gridDim.x,
              pi + (long long)p * gridDim.x);
}

__global__ void k_batch_dt_route(const AdjProb* __restrict__ probs, int nprob, const double* pv, const long long* pi,
                                 int nparts, const double* dtbar_log, const double* inv_log, int un, int ub_out,
                                 int m, int nsteps) {
  const int p = blockIdx.x;
  if (!max_rises(inv_log + p, m, nprob)) return;  // uniform over the block
  const AdjProb& P = probs[p];
  dt_route(P.h, afield(P, un), afield(P, ub_out), pv + (long long)p * nparts, pi + (long long)p * nparts, nparts,
           dtbar_log + p, inv_log + p, nprob, m, nsteps);
}

__global__ void k_batch_objective(const AdjProb* __restrict__ probs, int un, double xc, double yc, double sig,
                                  double* J, int seed_ub) {
  const int p = blockIdx.y;
  const AdjProb& P = probs[p];
  Field<double> ub = seed_ub >= 0 ? afield(P, seed_ub) : Field<double>{nullptr, 0, 0};
  objective_part(P.h, afield(P, un), xc, yc, sig, J + p, ub, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                 (long long)gridDim.x * blockDim.x);
}

// Whole-buffer copy (src < 0: the initial state) or zero fill (src == dst);
// state_elems is a multiple of 32, so double2 accesses stay aligned.
__global__ void k_batch_copy(const AdjProb* __restrict__ probs, int src, int dst) {
  const AdjProb& P = probs[blockIdx.y];
  double2* d = reinterpret_cast<double2*>(abuf(P, dst));
  const double2* sp = reinterpret_cast<const double2*>(abuf(P, src));
  const long long n = P.state_elems / 2;
  const bool zero = src == dst;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    d[k] = zero ? make_double2(0.0, 0.0) : sp[k];
}

__global__ void k_batch_seg_corners(const AdjProb* __restrict__ probs, int ping, int seg, int k0) {
  const AdjProb& P = probs[blockIdx.y];
  const int j = blockIdx.x + 1;
  if (threadIdx.x >= 64) return;
  copy_corner(abuf(P, ping + ((k0 + j) & 1)), abuf(P, seg + j), P.pitch, P.plane, P.h.isize, P.h.jsize,
              threadIdx.x);
}

// Interior density adjoints of buffer ub into the packed output (i fastest).
__global__ void k_batch_extract(const AdjProb* __restrict__ probs, int ub, double* out) {
  const AdjProb& P = probs[blockIdx.y];
  const double* src = abuf(P, ub);
  const long long n = (long long)P.h.nx * P.h.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = GW + (int)(k % P.h.nx), j = GW + (int)(k / P.h.nx);
    out[P.grad_off + k] = src[(long long)j * P.pitch + i];
  }
}

}  // namespace

int step_rev_setup() {
  bool ok = true;
  for (auto f : {k_step_rev<false, false>, k_step_rev<true, false>, k_step_rev<false, true>, k_step_rev<true, true>})
    ok = ok && cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES) == cudaSuccess;
  ok = ok && cudaFuncSetAttribute(k_step_rev_tsq, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T_SMEM_BYTES) ==
                 cudaSuccess;
  return ok ? 0 : -1;
}

void launch_step_rev(const Hydro<double>& h, Field<double> un, Field<double> ubn1, Field<double> ubn,
                     Field<double> ubz, const double* dt, double* dtbar, cudaStream_t s, const TapeOut* tape) {
  dim3 g((h.nx + ATX - 1) / ATX, (h.ny + ATY - 1) / ATY);
  const TapeOut t = tape ? *tape : TapeOut();
  const bool sq = h.dx == h.dy;
  if (tape) {
    if (sq) k_step_rev_tsq<<<g, ANT, T_SMEM_BYTES, s>>>(h, un, ubn1, ubn, ubz, dt, dtbar, t);
    else k_step_rev<false, true><<<g, ANT, SMEM_BYTES, s>>>(h, un, ubn1, ubn, ubz, dt, dtbar, t);
  } else {
    if (sq) k_step_rev<true, false><<<g, ANT, SMEM_BYTES, s>>>(h, un, ubn1, ubn, ubz, dt, dtbar, t);
    else k_step_rev<false, false><<<g, ANT, SMEM_BYTES, s>>>(h, un, ubn1, ubn, ubz, dt, dtbar, t);
  }
}

void launch_seg_corners(const Hydro<double>& h, double* pool, size_t state_elems, size_t pitch, size_t plane,
                        int ping_index, int seg_index, int k0, int nseg, cudaStream_t s) {
  if (nseg > 1)
    k_seg_corners<<<nseg - 1, 64, 0, s>>>(pool, (long long)state_elems, (int)pitch, (long long)plane, h.isize,
                                          h.jsize, ping_index, seg_index, k0);
}

void launch_argmax(const Hydro<double>& h, Field<double> u, double* pv, long long* pi, int nparts,
                   const double* inv_log, int m, cudaStream_t s) {
  k_argmax_partial<<<nparts, 256, 0, s>>>(h, u, pv, pi, inv_log, m);
}

void launch_dt_route(const Hydro<double>& h, Field<double> u, Field<double> ub, const double* pv, const long long* pi,
                     int nparts, const double* dtbar_log, const double* inv_log, int m, int nsteps,
                     cudaStream_t s) {
  k_dt_route<<<1, kDtThreads, 0, s>>>(h, u, ub, pv, pi, nparts, dtbar_log, inv_log, m, nsteps);
}

void launch_objective(const Hydro<double>& h, Field<double> u, double xc, double yc, double sig, double* J,
                      Field<double> ub, cudaStream_t s) {
  k_objective<<<256, 256, 0, s>>>(h, u, xc, yc, sig, J, ub);
}

int batch_step_rev_setup() {
  bool ok = true;
  for (auto f : {k_batch_step_rev<false, false>, k_batch_step_rev<true, false>, k_batch_step_rev<false, true>,
                 k_batch_step_rev<true, true>})
    ok = ok && cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES) == cudaSuccess;
  ok = ok && cudaFuncSetAttribute(k_batch_step_rev_tsq, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)T_SMEM_BYTES) == cudaSuccess;
  return ok ? 0 : -1;
}

int rev_tile_shape(int* tx, int* ty) {
  *tx = ATX;
  *ty = ATY;
  return 0;
}

void launch_batch_step_rev(const AdjBatch& B, int un, int ub_in, int ub_out, int ub_zero, int m, cudaStream_t s,
                           int tape_j) {
  const auto args = [&](auto kern) {
    kern<<<B.total_tiles, ANT, SMEM_BYTES, s>>>(B.probs, B.nprob, B.dt_log, B.dtbar_log, un, ub_in, ub_out, ub_zero,
                                                m, tape_j);
  };
  if (tape_j >= 0) {
    if (B.square)
      k_batch_step_rev_tsq<<<B.total_tiles, ANT, T_SMEM_BYTES, s>>>(B.probs, B.nprob, B.dt_log, B.dtbar_log, un, ub_in,
                                                                   ub_out, ub_zero, m, tape_j);
    else args(k_batch_step_rev<false, true>);
  } else {
    if (B.square) args(k_batch_step_rev<true, false>);
    else args(k_batch_step_rev<false, false>);
  }
}

void launch_batch_argmax(const AdjBatch& B, int un, int m, cudaStream_t s) {
  k_batch_argmax<<<dim3(B.nparts, B.nprob), 256, 0, s>>>(B.probs, B.nprob, B.inv_log, un, m, B.part_v, B.part_i);
}

void launch_batch_dt_route(const AdjBatch& B, int un, int ub_out, int m, int nsteps, cudaStream_t s) {
  k_batch_dt_route<<<B.nprob, kDtThreads, 0, s>>>(B.probs, B.nprob, B.part_v, B.part_i, B.nparts, B.dtbar_log, B.inv_log, un,
                                          ub_out, m, nsteps);
}

void launch_batch_objective(const AdjBatch& B, int un, double xc, double yc, double sig, int seed_ub,
                            cudaStream_t s) {
  k_batch_objective<<<dim3(64, B.nprob), 256, 0, s>>>(B.probs, un, xc, yc, sig, B.J, seed_ub);
}

void launch_batch_copy(const AdjBatch& B, int src, int dst, cudaStream_t s) {
  k_batch_copy<<<dim3(64, B.nprob), 256, 0, s>>>(B.probs, src, dst);
}

void launch_batch_seg_corners(const AdjBatch& B, int ping, int seg, int k0, int nseg, cudaStream_t s) {
  if (nseg > 1) k_batch_seg_corners<<<dim3(nseg - 1, B.nprob), 64, 0, s>>>(B.probs, ping, seg, k0);
}

void launch_batch_extract(const AdjBatch& B, int ub, double* out, cudaStream_t s) {
  k_batch_extract<<<dim3(32, B.nprob), 256, 0, s>>>(B.probs, ub, out);
}

}  // namespace e2d
