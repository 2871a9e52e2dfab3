// k_fused.cu -- implementationVersion 0: the whole Godunov step of a tile in
// one kernel ("recompute" variant, cuf/m_HydroRun_gpu.cuf:1137-1293 in role,
// serial_ref/m_run.f90:210-243 in arithmetic).
//
// One CTA owns a TX x TY tile of interior cells.  It
//   1. loads the (TX+4) x (TY+4) x 4 conservative box (2-cell halo, ghosts
//      included) with one TMA 3D tile load into shared memory,
//   2. converts it in place to primitives (computePrimitives),
//   3. computes slopes (slope_unsplit_hydro_2d) and trace source terms once
//      per cell of the (TX+2) x (TY+2) ring,
//   4. solves the (TX+1) x TY x-faces and TX x (TY+1) y-faces (face states by
//      trace_unsplit_2d_along_dir, riemann_2d or riemann_2d_hllc, times
//      dt/dx or dt/dy) into shared memory, warps taking faces dynamically,
//   5. applies updateHydro to its cells and writes them, plus the ghost cells
//      that make_boundaries would copy from them at the next step, plus the
//      next step's CFL maximum (block max + atomic max into a run slot).
// Primitives, slopes, face states and fluxes never leave shared memory.
#include <cuda.h>
#include "launch.h"

namespace e2d {

struct FusedPlan {
  CUtensorMap tm[2];  // [0]: u, [1]: u2
};

namespace {

constexpr int NT = 256;  // threads per CTA
template <typename Real> struct Tile;
template <> struct Tile<double> { static constexpr int TX = 32, TY = 15, MINB = 2; };
template <> struct Tile<float> { static constexpr int TX = 32, TY = 15, MINB = 3; };

template <typename Real>
struct Smem {
  static constexpr int TX = Tile<Real>::TX, TY = Tile<Real>::TY;
  static constexpr int BXs = TX + 4, BYs = TY + 4;  // TMA box
  static constexpr int RX = TX + 2, RY = TY + 2;    // ring of cells with slopes
  static constexpr size_t q_off = 0;                                   // [4][BYs][BXs]
  static constexpr size_t d_off = q_off + 4ull * BYs * BXs;            // [8][RY][RX]
  static constexpr size_t s_off = d_off + 8ull * RY * RX;              // [4][RY][RX]
  static constexpr size_t fx_off = s_off + 4ull * RY * RX;             // [4][TY][TX+1]
  static constexpr size_t fy_off = fx_off + 4ull * TY * (TX + 1);      // [4][TY+1][TX]
  static constexpr size_t n_real = fy_off + 4ull * (TY + 1) * TX;
  static constexpr size_t bytes = n_real * sizeof(Real) + 256 /*mbarrier, counter, reduction, dt*/ + 128 /*align*/;
  static constexpr uint32_t tma_bytes = 4u * BYs * BXs * sizeof(Real);
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bounded wait on an mbarrier phase: gives up after ~2^31 SM cycles (about a
// second) and reports false, so a lost transfer cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
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

// Source cell of ghost column/row g along one axis of n interior cells for
// boundary type `type` (serial_ref/m_run.f90:573-644), 0-based; g in
// {0, 1, n+2, n+3}.
__device__ __forceinline__ int ghost_source(int g, int n, int type) {
  if (g < 2) return (type == 1) ? 3 - g : (type == 2) ? 2 : n + g;
  return (type == 1) ? 2 * n + 3 - g : (type == 2) ? n + 1 : g - n;
}

template <typename Real>
__global__ void __launch_bounds__(NT, Tile<Real>::MINB)
    k_fused(const __grid_constant__ CUtensorMap tm_in, Hydro<Real> h, Field<Real> in, Field<Real> out,
            StepDt<Real> sd, Ctl* ctl, int fill_ghosts) {
  using S = Smem<Real>;
  constexpr int TX = S::TX, TY = S::TY, BXs = S::BXs, BYs = S::BYs, RX = S::RX, RY = S::RY;
  extern __shared__ unsigned char smem_raw[];
  Real* base = reinterpret_cast<Real*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  Real* sq = base + S::q_off;
  Real* sd_ = base + S::d_off;
  Real* ss = base + S::s_off;
  Real* sfx = base + S::fx_off;
  Real* sfy = base + S::fy_off;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + S::n_real);
  int* face_counter = reinterpret_cast<int*>(bar + 1);
  Real* red = reinterpret_cast<Real*>(bar + 2);  // 8 warps
  Real* sdt = red + 8;                           // dt, dt/dx, dt/dy of this step

  const int tid = threadIdx.x;
  const int i0 = GW + blockIdx.x * TX;  // first interior cell of the tile
  const int j0 = GW + blockIdx.y * TY;

  // ---- 1. TMA load of the conservative box [i0-2, i0+TX+2) x [j0-2, j0+TY+2) x 4
  const uint32_t bar_a = smem_u32(bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    *face_counter = 0;
    // This step's dt (serial_ref/m_run.f90:308 when it comes from the running
    // maximum) and dt/dx, dt/dy (m_run.f90:384-385), once per CTA.
    const Real dt0 = sd.from_slot ? h.cfl / *inv_slot<Real>(ctl, sd.rd_slot) : sd.dt_value;
    sdt[0] = dt0;
    sdt[1] = dt0 / h.dx;
    sdt[2] = dt0 / h.dy;
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(S::tma_bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(sq)),
        "l"(reinterpret_cast<uint64_t>(&tm_in)), "r"(i0 - GW), "r"(j0 - GW), "r"(0), "r"(bar_a)
        : "memory");
  }
  const Real dt = sdt[0];
  const Real dtdx = sdt[1];
  const Real dtdy = sdt[2];
  const bool ok = mbar_wait(bar_a, 0);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicOr(&ctl->health, 4u);
    return;
  }

  // ---- 2. primitives of the whole box, in place (computePrimitives)
  for (int k = tid; k < BXs * BYs; k += NT) {
    Real u[4], q[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) u[v] = sq[v * BXs * BYs + k];
    primitives(h, u, q);
#pragma unroll
    for (int v = 0; v < 4; ++v) sq[v * BXs * BYs + k] = q[v];
  }
  __syncthreads();

  // ---- 3. slopes and trace source terms of the ring cells (-1..TX, -1..TY)
  auto Q = [&](int v, int y, int x) -> Real { return sq[(v * BYs + y) * BXs + x]; };
  for (int k = tid; k < RX * RY; k += NT) {
    const int rx = k % RX, ry = k / RX;  // ring coords; box coords are +1
    const int x = rx + 1, y = ry + 1;
    Real qc[4], qe[4], qw[4], qn[4], qs[4], dqx[4], dqy[4], s[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qc[v] = Q(v, y, x); qe[v] = Q(v, y, x + 1); qw[v] = Q(v, y, x - 1);
      qn[v] = Q(v, y + 1, x); qs[v] = Q(v, y - 1, x);
    }
    slopes(h, qc, qe, qw, qn, qs, dqx, dqy);
    trace_sources(h, qc, dqx, dqy, s);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      sd_[v * RX * RY + k] = dqx[v];
      sd_[(4 + v) * RX * RY + k] = dqy[v];
      ss[v * RX * RY + k] = s[v];
    }
  }
  __syncthreads();

  // ---- 4. Riemann fluxes of all faces of the tile, claimed 32 at a time per warp
  constexpr int NXF = (TX + 1) * TY, NYF = TX * (TY + 1), NF = NXF + NYF;
  const int lane = tid & 31;
  while (true) {
    int chunk = 0;
    if (lane == 0) chunk = atomicAdd(face_counter, 32);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk >= NF) break;
    const int k = chunk + lane;
    if (k < NF) {
      if (k < NXF) {
        const int f = k % (TX + 1), r = k / (TX + 1);  // between ring cells (f-1, r) and (f, r)
        if (i0 + f <= h.nx + 2 && j0 + r <= h.ny + 1) {
          const int kl = (r + 1) * RX + f, kr = kl + 1;  // ring indices of left/right cells
          Real qc[4], dq[4], s[4], ql[4], qr[4], flux[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, r + 2, f + 1); dq[v] = sd_[v * RX * RY + kl]; s[v] = ss[v * RX * RY + kl]; }
          trace_face<Real, true>(h, qc, dq, s, dtdx, ql);
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, r + 2, f + 2); dq[v] = sd_[v * RX * RY + kr]; s[v] = ss[v * RX * RY + kr]; }
          trace_face<Real, false>(h, qc, dq, s, dtdx, qr);
          riemann(h, ql, qr, flux);
#pragma unroll
          for (int v = 0; v < 4; ++v) sfx[(v * TY + r) * (TX + 1) + f] = flux[v] * dtdx;
        }
      } else {
        const int kk = k - NXF;
        const int c = kk % TX, g = kk / TX;  // between ring cells (c, g-1) and (c, g)
        if (i0 + c <= h.nx + 1 && j0 + g <= h.ny + 2) {
          const int kl = g * RX + (c + 1), kr = kl + RX;
          Real qc[4], dq[4], s[4], ql[4], qr[4], flux[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, g + 1, c + 2); dq[v] = sd_[(4 + v) * RX * RY + kl]; s[v] = ss[v * RX * RY + kl]; }
          trace_face<Real, true>(h, qc, dq, s, dtdy, ql);
#pragma unroll
          for (int v = 0; v < 4; ++v) { qc[v] = Q(v, g + 2, c + 2); dq[v] = sd_[(4 + v) * RX * RY + kr]; s[v] = ss[v * RX * RY + kr]; }
          trace_face<Real, false>(h, qc, dq, s, dtdy, qr);
          Real t = ql[IU]; ql[IU] = ql[IV]; ql[IV] = t;
          t = qr[IU]; qr[IU] = qr[IV]; qr[IV] = t;
          riemann(h, ql, qr, flux);
          t = flux[IU]; flux[IU] = flux[IV]; flux[IV] = t;
#pragma unroll
          for (int v = 0; v < 4; ++v) sfy[(v * (TY + 1) + g) * TX + c] = flux[v] * dtdy;
        }
      }
    }
  }
  __syncthreads();

  // ---- 5. updateHydro + ghost copies + next-step CFL maximum
  const bool want_dt = sd.wr_slot >= 0;
  Real m = Real(0);
  for (int k = tid; k < TX * TY; k += NT) {
    const int c = k % TX, r = k / TX;
    const int i = i0 + c, j = j0 + r;
    if (i > h.nx + 1 || j > h.ny + 1) continue;
    Real un[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      Real flux_tot = sfx[(v * TY + r) * (TX + 1) + c] - sfx[(v * TY + r) * (TX + 1) + c + 1];
      flux_tot = (sfy[(v * (TY + 1) + r) * TX + c] - sfy[(v * (TY + 1) + r + 1) * TX + c]) + flux_tot;
      un[v] = in.at(v, j, i) + flux_tot;
      out.at(v, j, i) = un[v];
    }
    if (fill_ghosts) {
      if (i <= 3 || i >= h.nx) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int g = (e < 2) ? e : h.nx + e;
          const int type = (e < 2) ? h.bc_xmin : h.bc_xmax;
          if (ghost_source(g, h.nx, type) == i) {
#pragma unroll
            for (int v = 0; v < 4; ++v)
              out.at(v, j, g) = un[v] * ((type == 1 && v == IU) ? Real(-1.0) : Real(1.0));
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
            for (int v = 0; v < 4; ++v)
              out.at(v, g, i) = un[v] * ((type == 1 && v == IV) ? Real(-1.0) : Real(1.0));
          }
        }
      }
    }
    if (!(un[ID] > Real(0)) || !isfinite(un[ID])) atomicOr(&ctl->health, 2u);
    if (want_dt && i <= h.isize - 4 && j <= h.jsize - 4) m = fmax(m, cell_invdt(h, un));
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) {
    if (sd.dt_log) sd.dt_log[sd.log_index] = dt;
    if (!isfinite(dt)) atomicOr(&ctl->health, 1u);
  }
  if (want_dt) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red[tid >> 5] = m;
    __syncthreads();
    if (tid < 32) {
      m = (tid < NT / 32) ? red[tid] : Real(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (tid == 0) {
        if (sd.rd_slot >= 0) m = fmax(m, *inv_slot<Real>(ctl, sd.rd_slot));
        atomic_max_slot<Real>(ctl, sd.wr_slot, m);
      }
    }
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 3D map over a pitched state: dims (isize, jsize, 4), zero fill outside.
template <typename Real>
bool encode_state_map(CUtensorMap* tm, const Hydro<Real>& h, Field<Real> f) {
  using S = Smem<Real>;
  EncodeTiledFn enc = get_encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)h.isize, (cuuint64_t)h.jsize, 4};
  const cuuint64_t strides[2] = {(cuuint64_t)f.pitch * sizeof(Real), (cuuint64_t)f.plane * sizeof(Real)};
  const cuuint32_t box[3] = {(cuuint32_t)S::BXs, (cuuint32_t)S::BYs, 4};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt =
      sizeof(Real) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  return enc(tm, dt, 3, f.p, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

template <typename Real>
FusedPlan* fused_plan_create(const Hydro<Real>& h, Field<Real> u, Field<Real> u2) {
  static_assert(Smem<Real>::BXs * sizeof(Real) % 16 == 0, "TMA inner box must be a multiple of 16 bytes");
  static_assert((Smem<Real>::TX * sizeof(Real)) % 16 == 0, "tile x origin must stay 16-byte aligned");
  FusedPlan* p = new FusedPlan;
  if (!encode_state_map<Real>(&p->tm[0], h, u) || !encode_state_map<Real>(&p->tm[1], h, u2)) {
    delete p;
    return nullptr;
  }
  if (cudaFuncSetAttribute(k_fused<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Smem<Real>::bytes) !=
      cudaSuccess) {
    delete p;
    return nullptr;
  }
  return p;
}

void fused_plan_destroy(FusedPlan* p) { delete p; }

template <typename Real>
void launch_fused(const Hydro<Real>& h, FusedPlan* plan, int in_is_u2, Field<Real> in, Field<Real> out,
                  StepDt<Real> sd, Ctl* ctl, bool fill_ghosts, cudaStream_t s) {
  using S = Smem<Real>;
  dim3 g((h.nx + S::TX - 1) / S::TX, (h.ny + S::TY - 1) / S::TY);
  k_fused<Real><<<g, NT, S::bytes, s>>>(plan->tm[in_is_u2 ? 1 : 0], h, in, out, sd, ctl, fill_ghosts ? 1 : 0);
}

template FusedPlan* fused_plan_create<double>(const Hydro<double>&, Field<double>, Field<double>);
template FusedPlan* fused_plan_create<float>(const Hydro<float>&, Field<float>, Field<float>);
template void launch_fused<double>(const Hydro<double>&, FusedPlan*, int, Field<double>, Field<double>,
                                   StepDt<double>, Ctl*, bool, cudaStream_t);
template void launch_fused<float>(const Hydro<float>&, FusedPlan*, int, Field<float>, Field<float>,
                                  StepDt<float>, Ctl*, bool, cudaStream_t);

}  // namespace e2d
