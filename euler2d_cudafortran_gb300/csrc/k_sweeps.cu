// k_sweeps.cu -- whole-array sweeps of the Euler-2D step: initial condition,
// ghost cells, CFL reduction, primitives, and the two "stored intermediates"
// variants of the update (implementationVersion 1 and 2).
//
// All indices are 0-based: interior cells are i in [2, nx+1], j in [2, ny+1];
// the Fortran index of serial_ref is (i+1, j+1).
#include "launch.h"

namespace e2d {

namespace {

constexpr int BX = 32, BY = 8;  // block shape of the sweeps: one warp per row segment

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

template <typename Real>
__device__ __forceinline__ Real resolve_dt(const Hydro<Real>& h, const StepDt<Real>& sd, Ctl* ctl) {
  if (sd.dt_ptr) return *sd.dt_ptr;
  if (sd.from_slot) return Ops<Real>::div(h.cfl, *inv_slot<Real>(ctl, sd.rd_slot));
  return sd.dt_value;
}

template <typename Real>
__device__ __forceinline__ void atomic_max_slot(Ctl* ctl, int slot, Real m);
template <>
__device__ __forceinline__ void atomic_max_slot<double>(Ctl* ctl, int slot, double m) {
  atomicMax(&ctl->inv64[slot], ordered_bits(m));
}
template <>
__device__ __forceinline__ void atomic_max_slot<float>(Ctl* ctl, int slot, float m) {
  atomicMax(&ctl->inv32[slot], ordered_bits(m));
}

// Block-wide max of m, folded with inv[rd] (if rd >= 0) into inv[wr]; every
// thread of the block must call it.
template <typename Real>
__device__ void block_max_to_slot(Real m, Ctl* ctl, int rd, int wr) {
  __shared__ Real red[32];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nthreads = blockDim.x * blockDim.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((tid & 31) == 0) red[tid >> 5] = m;
  __syncthreads();
  if (tid < 32) {
    m = (tid < (nthreads + 31) / 32) ? red[tid] : Real(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (tid == 0) {
      if (rd >= 0) m = fmax(m, *inv_slot<Real>(ctl, rd));
      atomic_max_slot<Real>(ctl, wr, m);
    }
  }
}

template <typename Real>
__device__ __forceinline__ void load4(const Field<Real>& f, int j, int i, Real x[4]) {
#pragma unroll
  for (int v = 0; v < 4; ++v) x[v] = f.at(v, j, i);
}

template <typename Real>
__device__ __forceinline__ void store4(const Field<Real>& f, int j, int i, const Real x[4]) {
#pragma unroll
  for (int v = 0; v < 4; ++v) f.at(v, j, i) = x[v];
}

// init_implode generalised (serial_ref/m_run.f90:524-555); tmp is single precision.
template <typename Real>
__global__ void k_init_diagonal(Hydro<Real> h, Field<Real> u, double offset, double rho_hi, double p_hi,
                                double rho_lo, double p_lo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h.isize || j >= h.jsize) return;
  const float tmpf = ((1.0f * (float)(i - GW)) / (float)h.nx) + ((1.0f * (float)(j - GW)) / (float)h.ny);
  const Real tmp = (Real)tmpf;
  if (tmp > (Real)offset) {
    u.at(ID, j, i) = (Real)rho_hi;
    u.at(IP, j, i) = (Real)p_hi / (h.gamma0 - Real(1.0));
  } else {
    u.at(ID, j, i) = (Real)rho_lo;
    u.at(IP, j, i) = (Real)p_lo / (h.gamma0 - Real(1.0));
  }
  u.at(IU, j, i) = Real(0.0);
  u.at(IV, j, i) = Real(0.0);
}

// make_boundaries, serial_ref/m_run.f90:561-648.  One thread per ghost cell of
// the 4 edges (x edges over interior rows, y edges over interior columns);
// the corner blocks are never written.  w (when w.p is set): a second array
// of the same layout filled by the same rules in the same launch (the
// primitives kept beside a state: a reflective wall's flipped momentum is a
// flipped velocity).
template <typename Real>
__global__ void k_boundaries(Hydro<Real> h, Field<Real> u, Field<Real> w) {
  const int nx = h.nx, ny = h.ny;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nxe = 4 * ny, nye = 4 * nx;
  if (t < nxe) {
    const int g = t / ny, j = GW + t % ny;
    int i, i0, type;
    if (g < 2) {
      i = g; type = h.bc_xmin;
      i0 = (type == 1) ? 3 - i : (type == 2) ? 2 : nx + i;
    } else {
      i = nx + g; type = h.bc_xmax;
      i0 = (type == 1) ? 2 * nx + 3 - i : (type == 2) ? nx + 1 : i - nx;
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const Real dir = (type == 1 && v == IU) ? Real(-1.0) : Real(1.0);
      u.at(v, j, i) = u.at(v, j, i0) * dir;
      if (w.p) w.at(v, j, i) = w.at(v, j, i0) * dir;
    }
  } else if (t < nxe + nye) {
    const int tt = t - nxe;
    const int g = tt / nx, i = GW + tt % nx;
    int j, j0, type;
    if (g < 2) {
      j = g; type = h.bc_ymin;
      j0 = (type == 1) ? 3 - j : (type == 2) ? 2 : ny + j;
    } else {
      j = ny + g; type = h.bc_ymax;
      j0 = (type == 1) ? 2 * ny + 3 - j : (type == 2) ? ny + 1 : j - ny;
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const Real dir = (type == 1 && v == IV) ? Real(-1.0) : Real(1.0);
      u.at(v, j, i) = u.at(v, j0, i) * dir;
      if (w.p) w.at(v, j, i) = w.at(v, j0, i) * dir;
    }
  }
}

// compute_dt sweep, serial_ref/m_run.f90:269-281: cells i in [2, isize-4],
// j in [2, jsize-4] (the last interior row and column are excluded).
template <typename Real>
__global__ void k_dt_reduce(Hydro<Real> h, Field<Real> u, Ctl* ctl, int slot) {
  const int i = GW + blockIdx.x * blockDim.x + threadIdx.x;
  Real m = Real(0);
  if (i <= h.isize - 4) {
    for (int j = GW + blockIdx.y * blockDim.y + threadIdx.y; j <= h.jsize - 4; j += gridDim.y * blockDim.y) {
      Real uc[4];
      load4(u, j, i, uc);
      m = fmax(m, cell_invdt(h, uc));
    }
  }
  block_max_to_slot(m, ctl, -1, slot);
}

// convertToPrimitives, serial_ref/m_run.f90:317-358 (all cells).
template <typename Real>
__global__ void k_prim(Hydro<Real> h, Field<Real> u, Field<Real> q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h.isize || j >= h.jsize) return;
  Real uc[4], qc[4];
  load4(u, j, i, uc);
  primitives(h, uc, qc);
  store4(q, j, i, qc);
}

// computeAndStoreFluxes, serial_ref/m_run.f90:363-484: (i, j) in [2, size-2].
template <typename Real>
__global__ void k_fluxes_v2(Hydro<Real> h, Field<Real> q, StepDt<Real> sd, Ctl* ctl, Field<Real> fx,
                            Field<Real> fy) {
  const int i = GW + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = GW + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > h.isize - 2 || j > h.jsize - 2) return;
  const Real dt = resolve_dt(h, sd, ctl);
  const Real dtdx = Ops<Real>::div(dt, h.dx);
  const Real dtdy = Ops<Real>::div(dt, h.dy);
  Real qc[4], qe[4], qw[4], qn[4], qs[4], dqx[4], dqy[4], s[4];
  Real qN[4], qNe[4], qNw[4], qNn[4], qNs[4], dqNx[4], dqNy[4], sN[4];
  Real qleft[4], qright[4], flux[4];
  load4(q, j, i, qc); load4(q, j, i + 1, qe); load4(q, j, i - 1, qw); load4(q, j + 1, i, qn); load4(q, j - 1, i, qs);
  slopes(h, qc, qe, qw, qn, qs, dqx, dqy);
  trace_sources(h, qc, dqx, dqy, s);
  // left interface along X
  load4(q, j, i - 1, qN); load4(q, j, i, qNe); load4(q, j, i - 2, qNw); load4(q, j + 1, i - 1, qNn); load4(q, j - 1, i - 1, qNs);
  slopes(h, qN, qNe, qNw, qNn, qNs, dqNx, dqNy);
  trace_sources(h, qN, dqNx, dqNy, sN);
  trace_face<Real, false>(h, qc, dqx, s, dtdx, qright);
  trace_face<Real, true>(h, qN, dqNx, sN, dtdx, qleft);
  riemann(h, qleft, qright, flux);
#pragma unroll
  for (int v = 0; v < 4; ++v) fx.at(v, j, i) = flux[v] * dtdx;
  // left interface along Y
  load4(q, j - 1, i, qN); load4(q, j - 1, i + 1, qNe); load4(q, j - 1, i - 1, qNw); load4(q, j, i, qNn); load4(q, j - 2, i, qNs);
  slopes(h, qN, qNe, qNw, qNn, qNs, dqNx, dqNy);
  trace_sources(h, qN, dqNx, dqNy, sN);
  trace_face<Real, false>(h, qc, dqy, s, dtdy, qright);
  trace_face<Real, true>(h, qN, dqNy, sN, dtdy, qleft);
  Real t = qleft[IU]; qleft[IU] = qleft[IV]; qleft[IV] = t;
  t = qright[IU]; qright[IU] = qright[IV]; qright[IV] = t;
  riemann(h, qleft, qright, flux);
  t = flux[IU]; flux[IU] = flux[IV]; flux[IV] = t;
#pragma unroll
  for (int v = 0; v < 4; ++v) fy.at(v, j, i) = flux[v] * dtdy;
}

// Epilogue shared by the update kernels: CFL term of the new state (cells
// excluded from compute_dt contribute 0) and the health check.
template <typename Real>
__device__ __forceinline__ Real new_state_checks(const Hydro<Real>& h, int i, int j, const Real un[4], Ctl* ctl,
                                                 bool want_dt) {
  if (bad_density(un[ID])) atomicOr(&ctl->health, 2u);
  if (want_dt && i <= h.isize - 4 && j <= h.jsize - 4) return cell_invdt(h, un);
  return Real(0);
}

template <typename Real>
__device__ __forceinline__ void log_dt(const Hydro<Real>& h, const StepDt<Real>& sd, Ctl* ctl, Real dt) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    if (sd.dt_log) sd.dt_log[sd.log_index] = dt;
    if (sd.inv_log && sd.rd_slot >= 0) sd.inv_log[sd.log_index] = *inv_slot<Real>(ctl, sd.rd_slot);
    if (!isfinite(dt)) atomicOr(&ctl->health, 1u);
  }
}

// updateHydro, serial_ref/m_run.f90:489-518 (interior cells), plus the next
// step's CFL maximum when sd.wr_slot >= 0.
template <typename Real>
__global__ void k_update_v2(Hydro<Real> h, Field<Real> in, Field<Real> fx, Field<Real> fy, Field<Real> out,
                            StepDt<Real> sd, Ctl* ctl) {
  const int i = GW + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = GW + blockIdx.y * blockDim.y + threadIdx.y;
  Real m = Real(0);
  if (i <= h.nx + 1 && j <= h.ny + 1) {
    Real un[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      Real flux_tot = fx.at(v, j, i) - fx.at(v, j, i + 1);
      flux_tot = (fy.at(v, j, i) - fy.at(v, j + 1, i)) + flux_tot;
      un[v] = in.at(v, j, i) + flux_tot;
      out.at(v, j, i) = un[v];
    }
    m = new_state_checks(h, i, j, un, ctl, sd.wr_slot >= 0);
  }
  log_dt(h, sd, ctl, resolve_dt(h, sd, ctl));
  if (sd.wr_slot >= 0) block_max_to_slot(m, ctl, sd.rd_slot, sd.wr_slot);
}

// implementationVersion 1, trace stage: slopes and the four face states of
// every cell in [1, size-2] (trace_unsplit_2d_along_dir for FACE_XMIN,
// FACE_XMAX, FACE_YMIN, FACE_YMAX; serial_ref/m_utils.f90:177-254).
template <typename Real>
__global__ void k_trace_v1(Hydro<Real> h, Field<Real> q, StepDt<Real> sd, Ctl* ctl, Field<Real> qxm,
                           Field<Real> qxp, Field<Real> qym, Field<Real> qyp) {
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > h.isize - 2 || j > h.jsize - 2) return;
  const Real dt = resolve_dt(h, sd, ctl);
  const Real dtdx = Ops<Real>::div(dt, h.dx);
  const Real dtdy = Ops<Real>::div(dt, h.dy);
  Real qc[4], qe[4], qw[4], qn[4], qs[4], dqx[4], dqy[4], s[4], f[4];
  load4(q, j, i, qc); load4(q, j, i + 1, qe); load4(q, j, i - 1, qw); load4(q, j + 1, i, qn); load4(q, j - 1, i, qs);
  slopes(h, qc, qe, qw, qn, qs, dqx, dqy);
#if E2D_FMA_FORMS
  // the FMA build on square cells: qs = q + (s*dtdx)*0.5 in fused steps,
  // each face state one fused multiply-add per variable (as the fused step)
  if (h.dx == h.dy) {
    Real qsrc[4];
    trace_qs(h, qc, dqx, dqy, Ops<Real>::half(dtdx), qsrc);
    trace_face_qs<Real, false>(h, qsrc, dqx, f); store4(qxm, j, i, f);
    trace_face_qs<Real, true>(h, qsrc, dqx, f);  store4(qxp, j, i, f);
    trace_face_qs<Real, false>(h, qsrc, dqy, f); store4(qym, j, i, f);
    trace_face_qs<Real, true>(h, qsrc, dqy, f);  store4(qyp, j, i, f);
    return;
  }
#endif
  trace_sources(h, qc, dqx, dqy, s);
  // FP64 with dtdx == dtdy: the source term (s*dtd)*0.5 is the same for the
  // four faces (+0.8 %; the FP32 build, not bound by its FP pipes, is left as it is)
  if constexpr (sizeof(Real) == 8) {
    if (h.dx == h.dy) {
      Real sh[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) sh[v] = Ops<Real>::half(s[v] * dtdx);
      trace_face<Real, false, true>(h, qc, dqx, sh, dtdx, f); store4(qxm, j, i, f);
      trace_face<Real, true, true>(h, qc, dqx, sh, dtdx, f);  store4(qxp, j, i, f);
      trace_face<Real, false, true>(h, qc, dqy, sh, dtdy, f); store4(qym, j, i, f);
      trace_face<Real, true, true>(h, qc, dqy, sh, dtdy, f);  store4(qyp, j, i, f);
      return;
    }
  }
  trace_face<Real, false>(h, qc, dqx, s, dtdx, f); store4(qxm, j, i, f);
  trace_face<Real, true>(h, qc, dqx, s, dtdx, f);  store4(qxp, j, i, f);
  trace_face<Real, false>(h, qc, dqy, s, dtdy, f); store4(qym, j, i, f);
  trace_face<Real, true>(h, qc, dqy, s, dtdy, f);  store4(qyp, j, i, f);
}

// implementationVersion 1, flux + update stage: a 32 x 7 tile of interior
// cells solves the 33 x 7 x-faces and 32 x 8 y-faces it needs into shared
// memory, then applies updateHydro.  256 threads take the faces in two
// rounds, the y faces from a 32-face boundary (no warp issues both
// directions' solvers, and no round is left with a few faces).
constexpr int V1_TX = 32, V1_TY = 7, V1_NT = 256;
template <typename Real>
__global__ void __launch_bounds__(V1_NT) k_flux_update_v1(Hydro<Real> h, Field<Real> in, Field<Real> qxm,
                                                          Field<Real> qxp, Field<Real> qym, Field<Real> qyp,
                                                          Field<Real> out, StepDt<Real> sd, Ctl* ctl) {
  constexpr int TX = V1_TX, TY = V1_TY, NT = V1_NT;
  constexpr int NXF = (TX + 1) * TY, Y0 = (NXF + 31) / 32 * 32, NF = Y0 + TX * (TY + 1);
  static_assert(NF == 2 * NT && TX * TY <= NT, "two full rounds of faces, one round of cells");
  __shared__ Real sfx[4][TY][TX + 1];
  __shared__ Real sfy[4][TY + 1][TX];
  const int tid = threadIdx.x;
  const int i0 = GW + blockIdx.x * TX, j0 = GW + blockIdx.y * TY;
  const Real dt = resolve_dt(h, sd, ctl);
  const Real dtdx = Ops<Real>::div(dt, h.dx);
  const Real dtdy = Ops<Real>::div(dt, h.dy);
  // the FMA build on square cells keeps the raw fluxes and fuses dt/dx into
  // the update (as the fused step)
  const bool raw = E2D_FMA_FORMS && h.dx == h.dy;
  for (int k = tid; k < NF; k += NT) {
    if (k < NXF) {
      // x-faces: face f (0..TX) of row r sits between cells i0+f-1 and i0+f
      const int f = k % (TX + 1), r = k / (TX + 1);
      const int i = i0 + f, j = j0 + r;
      if (i <= h.nx + 2 && j <= h.ny + 1) {
        Real ql[4], qr[4], flux[4];
        load4(qxp, j, i - 1, ql);
        load4(qxm, j, i, qr);
        riemann(h, ql, qr, flux);
#pragma unroll
        for (int v = 0; v < 4; ++v) sfx[v][r][f] = raw ? flux[v] : flux[v] * dtdx;
      }
    } else if (k >= Y0) {
      // y-faces: face g (0..TY) of column c sits between cells j0+g-1 and j0+g
      const int c = (k - Y0) % TX, g = (k - Y0) / TX;
      const int i = i0 + c, j = j0 + g;
      if (i <= h.nx + 1 && j <= h.ny + 2) {
        Real ql[4], qr[4], flux[4];
        load4(qyp, j - 1, i, ql);
        load4(qym, j, i, qr);
        Real t = ql[IU]; ql[IU] = ql[IV]; ql[IV] = t;
        t = qr[IU]; qr[IU] = qr[IV]; qr[IV] = t;
        riemann(h, ql, qr, flux);
        t = flux[IU]; flux[IU] = flux[IV]; flux[IV] = t;
#pragma unroll
        for (int v = 0; v < 4; ++v) sfy[v][g][c] = raw ? flux[v] : flux[v] * dtdy;
      }
    }
  }
  __syncthreads();
  const int c = tid % TX, r = tid / TX;
  const int i = i0 + c, j = j0 + r;
  Real m = Real(0);
  if (r < TY && i <= h.nx + 1 && j <= h.ny + 1) {
    Real un[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      Real flux_tot = sfx[v][r][c] - sfx[v][r][c + 1];
      flux_tot = (sfy[v][r][c] - sfy[v][r + 1][c]) + flux_tot;
      un[v] = raw ? fmx(flux_tot, dtdx, in.at(v, j, i)) : in.at(v, j, i) + flux_tot;
      out.at(v, j, i) = un[v];
    }
    m = new_state_checks(h, i, j, un, ctl, sd.wr_slot >= 0);
  }
  log_dt(h, sd, ctl, dt);
  if (sd.wr_slot >= 0) block_max_to_slot(m, ctl, sd.rd_slot, sd.wr_slot);
}

}  // namespace

template <typename Real>
void launch_init_diagonal(const Hydro<Real>& h, Field<Real> u, double offset, double rho_hi, double p_hi,
                          double rho_lo, double p_lo, cudaStream_t s) {
  dim3 b(BX, BY), g(cdiv(h.isize, BX), cdiv(h.jsize, BY));
  k_init_diagonal<Real><<<g, b, 0, s>>>(h, u, offset, rho_hi, p_hi, rho_lo, p_lo);
}

namespace {

// Row copy between a packed array (rows of `width` words, e.g. a host state
// in the Fortran layout, read or written through its mapped address) and a
// pitched one: row r of `rows`, word c.  Consecutive threads take
// consecutive words of a row.
template <typename Word>
__global__ void k_repitch(const Word* __restrict__ src, long long src_pitch, Word* __restrict__ dst,
                          long long dst_pitch, int width, int rows) {
  const long long n = (long long)width * rows;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long r = k / width, c = k - r * width;
    dst[r * dst_pitch + c] = src[r * src_pitch + c];
  }
}

}  // namespace

void launch_repitch(const void* src, size_t src_pitch, void* dst, size_t dst_pitch, int width, int rows,
                    int word_bytes, cudaStream_t s) {
  const long long n = (long long)width * rows;
  const int grid = (int)std::min<long long>(cdiv(n, 256), 152LL * 8);
  if (word_bytes == 8)
    k_repitch<unsigned long long><<<grid, 256, 0, s>>>(static_cast<const unsigned long long*>(src), (long long)src_pitch,
                                                       static_cast<unsigned long long*>(dst), (long long)dst_pitch,
                                                       width, rows);
  else
    k_repitch<unsigned int><<<grid, 256, 0, s>>>(static_cast<const unsigned int*>(src), (long long)src_pitch,
                                                 static_cast<unsigned int*>(dst), (long long)dst_pitch, width, rows);
}

template <typename Real>
void launch_boundaries(const Hydro<Real>& h, Field<Real> u, cudaStream_t s) {
  const long long n = 4LL * h.nx + 4LL * h.ny;
  k_boundaries<Real><<<cdiv(n, 256), 256, 0, s>>>(h, u, Field<Real>{nullptr, 0, 0});
}

template <typename Real>
void launch_boundaries_pair(const Hydro<Real>& h, Field<Real> u, Field<Real> w, cudaStream_t s) {
  const long long n = 4LL * h.nx + 4LL * h.ny;
  k_boundaries<Real><<<cdiv(n, 256), 256, 0, s>>>(h, u, w);
}

template <typename Real>
void launch_dt_reduce(const Hydro<Real>& h, Field<Real> u, Ctl* ctl, int slot, cudaStream_t s) {
  const int ni = h.isize - 5, nj = h.jsize - 5;
  const unsigned gy = cdiv(nj, BY * 4);
  dim3 b(BX, BY), g(cdiv(ni, BX), gy < 1 ? 1 : gy);
  k_dt_reduce<Real><<<g, b, 0, s>>>(h, u, ctl, slot);
}

template <typename Real>
void launch_prim(const Hydro<Real>& h, Field<Real> u, Field<Real> q, cudaStream_t s) {
  dim3 b(BX, BY), g(cdiv(h.isize, BX), cdiv(h.jsize, BY));
  k_prim<Real><<<g, b, 0, s>>>(h, u, q);
}

template <typename Real>
void launch_fluxes_v2(const Hydro<Real>& h, Field<Real> q, StepDt<Real> sd, Ctl* ctl, Field<Real> fx,
                      Field<Real> fy, cudaStream_t s) {
  dim3 b(BX, BY), g(cdiv(h.isize - 3, BX), cdiv(h.jsize - 3, BY));
  k_fluxes_v2<Real><<<g, b, 0, s>>>(h, q, sd, ctl, fx, fy);
}

template <typename Real>
void launch_update_v2(const Hydro<Real>& h, Field<Real> in, Field<Real> fx, Field<Real> fy, Field<Real> out,
                      StepDt<Real> sd, Ctl* ctl, cudaStream_t s) {
  dim3 b(BX, BY), g(cdiv(h.nx, BX), cdiv(h.ny, BY));
  k_update_v2<Real><<<g, b, 0, s>>>(h, in, fx, fy, out, sd, ctl);
}

template <typename Real>
void launch_trace_v1(const Hydro<Real>& h, Field<Real> q, StepDt<Real> sd, Ctl* ctl, Field<Real> qxm,
                     Field<Real> qxp, Field<Real> qym, Field<Real> qyp, cudaStream_t s) {
  dim3 b(BX, BY), g(cdiv(h.isize - 2, BX), cdiv(h.jsize - 2, BY));
  k_trace_v1<Real><<<g, b, 0, s>>>(h, q, sd, ctl, qxm, qxp, qym, qyp);
}

template <typename Real>
void launch_flux_update_v1(const Hydro<Real>& h, Field<Real> in, Field<Real> qxm, Field<Real> qxp,
                           Field<Real> qym, Field<Real> qyp, Field<Real> out, StepDt<Real> sd, Ctl* ctl,
                           cudaStream_t s) {
  dim3 g(cdiv(h.nx, V1_TX), cdiv(h.ny, V1_TY));
  k_flux_update_v1<Real><<<g, V1_NT, 0, s>>>(h, in, qxm, qxp, qym, qyp, out, sd, ctl);
}

#define E2D_INSTANTIATE(Real)                                                                                  \
  template void launch_init_diagonal<Real>(const Hydro<Real>&, Field<Real>, double, double, double, double,    \
                                           double, cudaStream_t);                                              \
  template void launch_boundaries<Real>(const Hydro<Real>&, Field<Real>, cudaStream_t);                        \
  template void launch_boundaries_pair<Real>(const Hydro<Real>&, Field<Real>, Field<Real>, cudaStream_t);      \
  template void launch_dt_reduce<Real>(const Hydro<Real>&, Field<Real>, Ctl*, int, cudaStream_t);              \
  template void launch_prim<Real>(const Hydro<Real>&, Field<Real>, Field<Real>, cudaStream_t);                 \
  template void launch_fluxes_v2<Real>(const Hydro<Real>&, Field<Real>, StepDt<Real>, Ctl*, Field<Real>,       \
                                       Field<Real>, cudaStream_t);                                             \
  template void launch_update_v2<Real>(const Hydro<Real>&, Field<Real>, Field<Real>, Field<Real>, Field<Real>, \
                                       StepDt<Real>, Ctl*, cudaStream_t);                                      \
  template void launch_trace_v1<Real>(const Hydro<Real>&, Field<Real>, StepDt<Real>, Ctl*, Field<Real>,        \
                                      Field<Real>, Field<Real>, Field<Real>, cudaStream_t);                    \
  template void launch_flux_update_v1<Real>(const Hydro<Real>&, Field<Real>, Field<Real>, Field<Real>,         \
                                            Field<Real>, Field<Real>, Field<Real>, StepDt<Real>, Ctl*,         \
                                            cudaStream_t);
E2D_INSTANTIATE(double)
E2D_INSTANTIATE(float)

}  // namespace e2d
