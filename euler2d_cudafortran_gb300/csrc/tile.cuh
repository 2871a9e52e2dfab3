// tile.cuh -- the fused Godunov step of one tile, shared by the single-run
// kernel (k_fused.cu, TMA-loaded tiles) and the batched kernel (k_batch.cu).
//
// A CTA owns a TX x TY tile of interior cells whose conservative box
// [i0-2, i0+TX+2) x [j0-2, j0+TY+2) x 4 already sits in shared memory
// (outside the domain it holds zeros, as TMA zero fill gives).  tile_compute
//   - converts the box to primitives in place (computePrimitives),
//   - computes slopes (slope_unsplit_hydro_2d) and trace source terms once
//     per cell of the (TX+2) x (TY+2) ring,
//   - solves the (TX+1) x TY x-faces and TX x (TY+1) y-faces (face states of
//     trace_unsplit_2d_along_dir, the Riemann flux, times dt/dx or dt/dy),
//     warps claiming 32 faces at a time,
//   - applies updateHydro, writes the tile of the new state, the ghost cells
//     make_boundaries would copy from it (when asked), raises the health
//     flags, and returns the block maximum of the next step's CFL term.
#pragma once
#include "launch.h"

namespace e2d {

template <typename Real, int TX_, int TY_, int NT_>
struct TileCfg {
  static constexpr int TX = TX_, TY = TY_, NT = NT_;
  static constexpr int BXs = TX + 4, BYs = TY + 4;  // conservative box
  static constexpr int RX = TX + 2, RY = TY + 2;    // ring of cells with slopes
  static constexpr size_t q_off = 0;                              // [4][BYs][BXs]
  static constexpr size_t d_off = q_off + 4ull * BYs * BXs;       // [8][RY][RX]
  static constexpr size_t s_off = d_off + 8ull * RY * RX;         // [4][RY][RX]
  static constexpr size_t fx_off = s_off + 4ull * RY * RX;        // [4][TY][TX+1]
  static constexpr size_t fy_off = fx_off + 4ull * TY * (TX + 1); // [4][TY+1][TX]
  static constexpr size_t n_real = fy_off + 4ull * (TY + 1) * TX;
  // after the reals: mbarrier (8 B), face counter (8 B), warp maxima (32 reals), dt values (4 reals)
  static constexpr size_t bytes = n_real * sizeof(Real) + 16 + 36 * sizeof(Real) + 128;
  static constexpr uint32_t box_bytes = 4u * BYs * BXs * sizeof(Real);
  static_assert((n_real * sizeof(Real)) % 8 == 0, "mbarrier alignment");
};

// Source cell of ghost column/row g along one axis of n interior cells for
// boundary type `type` (serial_ref/m_run.f90:573-644), 0-based; g in
// {0, 1, n+2, n+3}.
__device__ __forceinline__ int ghost_source(int g, int n, int type) {
  if (g < 2) return (type == 1) ? 3 - g : (type == 2) ? 2 : n + g;
  return (type == 1) ? 2 * n + 3 - g : (type == 2) ? n + 1 : g - n;
}

template <typename Real>
__device__ __forceinline__ void atomic_max_slot_ptr(Real* slot, Real m);
template <>
__device__ __forceinline__ void atomic_max_slot_ptr<double>(double* slot, double m) {
  atomicMax(reinterpret_cast<unsigned long long*>(slot), ordered_bits(m));
}
template <>
__device__ __forceinline__ void atomic_max_slot_ptr<float>(float* slot, float m) {
  atomicMax(reinterpret_cast<unsigned int*>(slot), ordered_bits(m));
}

// Phases 2-5 for the tile at (i0, j0); all threads call it after the box is
// in base[q_off..].  *face_counter must be 0.  Returns, in thread 0, the
// block maximum of the CFL term of the new state (0 when !want_dt).
// A no-op for the after-faces hook of tile_compute.
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// The one tile of the domain partition that owns global index g (of n interior
// cells, first interior index GW) along one axis, for a tile starting at t0
// of width w; ghosts (and ring ghosts) go to the edge tiles.
__device__ __forceinline__ bool owns(int g, int t0, int w, int n) {
  const int end = t0 + w < n + GW ? t0 + w : n + GW;
  return (g >= t0 && g < end) || (t0 == GW && g < GW) || (t0 + w >= n + GW && g >= n + GW);
}

// after_faces: run by every thread right after the barrier that ends the face phase, after which no
// phase reads the box (a persistent caller loads the next box into the box
// region there; the carry below copies two ring rows of slopes and sources).
// SQ (only when dx == dy, so that dtdx == dtdy bit for bit): the source term
// of a face state, (s*dtdx)*0.5, is the same for the four faces of a cell;
// the ring pass forms it once and stores it in place of s.
// QIN: the box holds primitive variables already (the previous step wrote
// them beside its state); the update then writes the primitives of the new
// state, and of its ghost cells, to qout.  The primitives of a state are a
// function of its conservative values, so this changes no result.
// TAPE (FP64, !QIN): the step also writes its input's forward values to
// *tape (TapeOut).
// before_faces: run by every thread right after the barrier that ends the
// ring pass, before it claims faces (work there delays no barrier: the faces
// are claimed dynamically).
// carry (a CTA that walks a column of tiles upwards):
//   kCarryIn: the previous call of this CTA computed the tile below (j0 - TY)
//     and kCarryOut; its top two ring rows (slopes and face sources of the
//     tile rows -1 and 0 of this one) then sit in ring rows 0-1, and its top
//     y-face row (the faces below this tile's row 0) in sfy row TY.  Those
//     are not computed again: the same inputs and the same code give the
//     same bits.
//   kCarryOut: the next call computes the tile above with kCarryIn: after
//     the face phase, ring rows RY-2..RY-1 are copied to rows 0-1.  With
//     TAPE this call also records the ring row and y-face row that the tile
//     above owns but does not compute.
constexpr int kCarryIn = 1, kCarryOut = 2;
template <typename Real, class C, bool SQ = false, bool QIN = false, bool TAPE = false, class Hook = NoHook,
          class Hook2 = NoHook>
__device__ __forceinline__ Real tile_compute(const Hydro<Real>& h, Real* base, int* face_counter, Real* red,
                                             int i0, int j0, const Field<Real>& in, const Field<Real>& out,
                                             const Field<Real>& qout, Real dtdx, Real dtdy, bool fill_ghosts,
                                             bool want_dt, unsigned* health,
                                             Hook after_faces = Hook(), const TapeOut* tape = nullptr,
                                             Hook2 before_faces = Hook2(), int carry = 0) {
  static_assert(!TAPE || (sizeof(Real) == 8 && !QIN), "the tape is written by the FP64 conversion path");
  constexpr int TX = C::TX, TY = C::TY, NT = C::NT, BXs = C::BXs, BYs = C::BYs, RX = C::RX, RY = C::RY;
  static_assert(RY >= 4 && TX % 32 == 0, "carried ring rows do not overlap their copies; whole y-face chunks");
  Real* sq = base + C::q_off;
  Real* sdq = base + C::d_off;
  Real* ss = base + C::s_off;
  Real* sfx = base + C::fx_off;
  Real* sfy = base + C::fy_off;
  const int tid = threadIdx.x;
  // The FMA build on square cells (dtdx == dtdy) keeps the raw face fluxes
  // and applies dt/dx once per cell in the update, fused with the addition.
  constexpr bool kFluxRaw = SQ && E2D_FMA_FORMS;

  // ---- primitives of the whole box (computePrimitives), in place
  if constexpr (!QIN) {
    for (int k = tid; k < BXs * BYs; k += NT) {
      Real u[4], q[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) u[v] = sq[v * BXs * BYs + k];
      primitives(h, u, q);
#pragma unroll
      for (int v = 0; v < 4; ++v) sq[v * BXs * BYs + k] = q[v];
      if constexpr (TAPE) {
        const int gi = i0 - GW + k % BXs, gj = j0 - GW + k / BXs;
        if (gi < h.isize && gj < h.jsize && owns(gi, i0, TX, h.nx) && owns(gj, j0, TY, h.ny)) {
#pragma unroll
          for (int v = 0; v < 4; ++v) tape->at(tape->q, v, gj, gi) = q[v];
        }
      }
    }
    __syncthreads();
  }

  // ---- slopes and trace source terms of the ring cells (-1..TX, -1..TY)
  auto Q = [&](int v, int y, int x) -> Real { return sq[(v * BYs + y) * BXs + x]; };
  // carried in: the y-face row below tile row 0 is the previous tile's top
  // row (its update has read it: the caller's barrier ends that tile)
  const bool carried = (carry & kCarryIn) != 0;
  if (carried) {
    for (int k = tid; k < 4 * TX; k += NT) {
      const int v = k / TX, c = k % TX;
      sfy[(v * (TY + 1)) * TX + c] = sfy[(v * (TY + 1) + TY) * TX + c];
    }
  }
  // ring cells in warp-aligned rows: the first TX columns of every row, then
  // the last RX - TX columns (a warp then reads one row of consecutive words);
  // rows 0-1 are skipped when carried in
  static_assert(RX - TX == 2, "the ring is two columns wider than the tile");
  const int ys = carried ? 2 : 0, rows = RY - ys;
  for (int k = tid; k < RX * rows; k += NT) {
    const int x = k < TX * rows ? k % TX + 1 : TX + 1 + (k - TX * rows) % 2;  // box coordinates
    const int y = (k < TX * rows ? k / TX : (k - TX * rows) / 2) + 1 + ys;
    const int kr = (y - 1) * RX + (x - 1);                                 // ring index
    Real qc[4], qe[4], qw[4], qn[4], qs[4], dqx[4], dqy[4], s[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qc[v] = Q(v, y, x); qe[v] = Q(v, y, x + 1); qw[v] = Q(v, y, x - 1);
      qn[v] = Q(v, y + 1, x); qs[v] = Q(v, y - 1, x);
    }
    unsigned lim_cases = 0;
    slopes<Real, TAPE>(h, qc, qe, qw, qn, qs, dqx, dqy, &lim_cases);
#if E2D_FMA_FORMS
    // the FMA build on square cells forms q + (s*dtdx)*0.5 directly
    if constexpr (SQ && !TAPE) trace_qs(h, qc, dqx, dqy, Ops<Real>::half(dtdx), s);
    else trace_sources(h, qc, dqx, dqy, s);
#else
    trace_sources(h, qc, dqx, dqy, s);
#endif
    if constexpr (TAPE) {
      const int gi = i0 - GW + x, gj = j0 - GW + y;
      // (with kCarryOut also the top ring row, which the tile above owns but
      // takes over instead of computing)
      if (gi <= h.nx + 2 && gj <= h.ny + 2 && owns(gi, i0, TX, h.nx) &&
          (owns(gj, j0, TY, h.ny) || ((carry & kCarryOut) && y == RY && owns(gj, j0 + TY, TY, h.ny)))) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          tape->at(tape->dq, v, gj, gi) = dqx[v];
          tape->at(tape->dq, 4 + v, gj, gi) = dqy[v];
          tape->at(tape->s, v, gj, gi) = s[v];
        }
        tape->flag(tape->lim, gj, gi) = lim_cases;
      }
    }
    if constexpr (SQ) {
#if E2D_FMA_FORMS
      // the FMA build keeps q + (s*dtdx)*0.5 for the faces (formed above
      // unless the tape needed s itself).  trace_sources's s is -w and
      // trace_qs forms fma(-dtdx/2, w, q) for the same fused w, which is
      // fma(dtdx/2, s, q): the step without a tape's bits, from s
      if constexpr (TAPE) {
        const Real hdt = Ops<Real>::half(dtdx);
#pragma unroll
        for (int v = 0; v < 4; ++v) s[v] = fmx(hdt, s[v], qc[v]);
      }
#else
#pragma unroll
      for (int v = 0; v < 4; ++v) s[v] = Ops<Real>::half(s[v] * dtdx);
#endif
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      sdq[v * RX * RY + kr] = dqx[v];
      sdq[(4 + v) * RX * RY + kr] = dqy[v];
      ss[v * RX * RY + kr] = s[v];
    }
  }
  __syncthreads();

  // ---- Riemann fluxes of all faces of the tile, claimed 32 at a time per
  // warp.  The y faces start on a 32-face boundary, so no warp holds faces of
  // both directions: the two inlined solvers would both be issued for it
  // (every FP64 instruction a warp issues costs its FP64 pipe slots,
  // predicated or not).
  constexpr int NXF = (TX + 1) * TY, NYF = TX * (TY + 1);
  constexpr int Y0 = (NXF + 31) / 32 * 32;
  // carried in: y-face row 0 is not solved again (a whole number of chunks)
  const int yskip = carried ? TX : 0, NF = Y0 + NYF - yskip;
  const int lane = tid & 31;
  before_faces();
  while (true) {
    int chunk = 0;
    if (lane == 0) chunk = atomicAdd(face_counter, 32);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk >= NF) break;
    const int k = chunk + lane;
    if (k < NXF) {
      // x faces: the first TX of every row as warp-aligned blocks of TX (a
      // warp reads one row of consecutive words: no shared-memory bank
      // conflicts), then the last column, one face per row
      const int f = k < TX * TY ? k % TX : TX, r = k < TX * TY ? k / TX : k - TX * TY;  // between ring cells (f-1, r) and (f, r)
      if (i0 + f <= h.nx + 2 && j0 + r <= h.ny + 1) {
        const int kl = (r + 1) * RX + f, kr = kl + 1;
        Real qc[4], dq[4], s[4], ql[4], qr[4], flux[4];
        if constexpr (SQ && E2D_FMA_FORMS) {
#pragma unroll
          for (int v = 0; v < 4; ++v) { dq[v] = sdq[v * RX * RY + kl]; s[v] = ss[v * RX * RY + kl]; }
          trace_face_qs<Real, true>(h, s, dq, ql);
#pragma unroll
          for (int v = 0; v < 4; ++v) { dq[v] = sdq[v * RX * RY + kr]; s[v] = ss[v * RX * RY + kr]; }
          trace_face_qs<Real, false>(h, s, dq, qr);
        } else {
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, r + 2, f + 1); dq[v] = sdq[v * RX * RY + kl]; s[v] = ss[v * RX * RY + kl]; }
          trace_face<Real, true, SQ>(h, qc, dq, s, dtdx, ql);
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, r + 2, f + 2); dq[v] = sdq[v * RX * RY + kr]; s[v] = ss[v * RX * RY + kr]; }
          trace_face<Real, false, SQ>(h, qc, dq, s, dtdx, qr);
        }
        if constexpr (TAPE) {
          if (tape->fx) {
            double rec[HR_N];
            unsigned fl;
            riemann_hllc_rec(h, ql, qr, rec, fl);
#pragma unroll
            for (int v = 0; v < 4; ++v) flux[v] = rec[HR_FLUX + v];
            if (f < TX || i0 + TX == h.nx + 2) {  // the face at the left of cell (i0 + f, j0 + r)
#pragma unroll
              for (int e = 0; e < HR_N; ++e) tape->at(tape->fx, e, j0 + r, i0 + f) = rec[e];
              tape->flag(tape->flx, j0 + r, i0 + f) = fl;
            }
          } else {
            riemann(h, ql, qr, flux);
          }
        } else {
          riemann(h, ql, qr, flux);
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) sfx[(v * TY + r) * (TX + 1) + f] = kFluxRaw ? flux[v] : flux[v] * dtdx;
      }
    } else if (k >= Y0 && k < NF) {
      const int kk = k - Y0 + yskip;
      const int c = kk % TX, g = kk / TX;  // between ring cells (c, g-1) and (c, g)
      if (i0 + c <= h.nx + 1 && j0 + g <= h.ny + 2) {
        const int kl = g * RX + (c + 1), kr = kl + RX;
        Real qc[4], dq[4], s[4], ql[4], qr[4], flux[4];
        if constexpr (SQ && E2D_FMA_FORMS) {
#pragma unroll
          for (int v = 0; v < 4; ++v) { dq[v] = sdq[(4 + v) * RX * RY + kl]; s[v] = ss[v * RX * RY + kl]; }
          trace_face_qs<Real, true>(h, s, dq, ql);
#pragma unroll
          for (int v = 0; v < 4; ++v) { dq[v] = sdq[(4 + v) * RX * RY + kr]; s[v] = ss[v * RX * RY + kr]; }
          trace_face_qs<Real, false>(h, s, dq, qr);
        } else {
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, g + 1, c + 2); dq[v] = sdq[(4 + v) * RX * RY + kl]; s[v] = ss[v * RX * RY + kl]; }
          trace_face<Real, true, SQ>(h, qc, dq, s, dtdy, ql);
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, g + 2, c + 2); dq[v] = sdq[(4 + v) * RX * RY + kr]; s[v] = ss[v * RX * RY + kr]; }
          trace_face<Real, false, SQ>(h, qc, dq, s, dtdy, qr);
        }
        Real t = ql[IU]; ql[IU] = ql[IV]; ql[IV] = t;
        t = qr[IU]; qr[IU] = qr[IV]; qr[IV] = t;
        if constexpr (TAPE) {
          if (tape->fy) {
            double rec[HR_N];
            unsigned fl;
            riemann_hllc_rec(h, ql, qr, rec, fl);
#pragma unroll
            for (int v = 0; v < 4; ++v) flux[v] = rec[HR_FLUX + v];
            // the face below cell (i0 + c, j0 + g); with kCarryOut also the top
            // row, which the tile above owns but takes over
            if (g < TY || j0 + TY == h.ny + 2 || (carry & kCarryOut)) {
#pragma unroll
              for (int e = 0; e < HR_N; ++e) tape->at(tape->fy, e, j0 + g, i0 + c) = rec[e];
              tape->flag(tape->fly, j0 + g, i0 + c) = fl;
            }
          } else {
            riemann(h, ql, qr, flux);
          }
        } else {
          riemann(h, ql, qr, flux);
        }
        t = flux[IU]; flux[IU] = flux[IV]; flux[IV] = t;
#pragma unroll
        for (int v = 0; v < 4; ++v) sfy[(v * (TY + 1) + g) * TX + c] = kFluxRaw ? flux[v] : flux[v] * dtdy;
      }
    }
  }
  __syncthreads();
  after_faces();
  if (carry & kCarryOut) {  // ring rows RY-2..RY-1 -> rows 0-1 (read by no one until the next face phase)
    for (int k = tid; k < 12 * 2 * RX; k += NT) {
      const int pl = k / (2 * RX), e = k - pl * (2 * RX);
      Real* a = pl < 8 ? sdq + pl * RX * RY : ss + (pl - 8) * RX * RY;
      a[e] = a[(RY - 2) * RX + e];
    }
  }
  if constexpr (TAPE) {
    if (tape->only) return Real(0);
  }

  // ---- updateHydro + ghost copies + next-step CFL maximum
  Real m = Real(0);
  for (int k = tid; k < TX * TY; k += NT) {
    const int c = k % TX, r = k / TX;
    const int i = i0 + c, j = j0 + r;
    if (i > h.nx + 1 || j > h.ny + 1) continue;
    Real un[4], qn[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      Real flux_tot = sfx[(v * TY + r) * (TX + 1) + c] - sfx[(v * TY + r) * (TX + 1) + c + 1];
      flux_tot = (sfy[(v * (TY + 1) + r) * TX + c] - sfy[(v * (TY + 1) + r + 1) * TX + c]) + flux_tot;
      un[v] = kFluxRaw ? fmx(flux_tot, dtdx, in.at(v, j, i)) : in.at(v, j, i) + flux_tot;
      out.at(v, j, i) = un[v];
    }
    if constexpr (QIN) {
      primitives(h, un, qn);
#pragma unroll
      for (int v = 0; v < 4; ++v) qout.at(v, j, i) = qn[v];
    }
    // Ghost copies (reflective walls flip the normal momentum, and so the
    // normal velocity of the primitives: -m/rho is -(m/rho) exactly).
    if (fill_ghosts) {
      if (i <= 3 || i >= h.nx) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int g = (e < 2) ? e : h.nx + e;
          const int type = (e < 2) ? h.bc_xmin : h.bc_xmax;
          if (ghost_source(g, h.nx, type) == i) {
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              out.at(v, j, g) = Ops<Real>::neg_if(un[v], type == 1 && v == IU);  // reflective: flip u
              if constexpr (QIN) qout.at(v, j, g) = Ops<Real>::neg_if(qn[v], type == 1 && v == IU);
            }
          }
        }
      }
      if (j <= 3 || j >= h.ny) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int g = (e < 2) ? e : h.ny + e;
          const int type = (e < 2) ? h.bc_ymin : h.bc_ymax;
          if (ghost_source(g, h.ny, type) == j) {
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              out.at(v, g, i) = Ops<Real>::neg_if(un[v], type == 1 && v == IV);  // reflective: flip v
              if constexpr (QIN) qout.at(v, g, i) = Ops<Real>::neg_if(qn[v], type == 1 && v == IV);
            }
          }
        }
      }
    }
    if (bad_density(un[ID])) atomicOr(health, 2u);
    if (want_dt && i <= h.isize - 4 && j <= h.jsize - 4) {
      if constexpr (QIN) m = Ops<Real>::max(m, cell_invdt_q(h, qn));
      else m = Ops<Real>::max(m, cell_invdt(h, un));
    }
  }
  if (want_dt) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = Ops<Real>::max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red[tid >> 5] = m;
    __syncthreads();
    if (tid < 32) {
      m = (tid < NT / 32) ? red[tid] : Real(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = Ops<Real>::max(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
  }
  return m;
}

}  // namespace e2d
