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

#include <algorithm>
#include "sync.cuh"
#include "tile.cuh"

namespace e2d {

struct FusedPlan {
  CUtensorMap tm[2];   // [0]: u, [1]: u2
  CUtensorMap tmq[2];  // primitives beside u and u2 (when has_q)
  CUtensorMap tmi[2];  // the interior tile of u and u2 (the L2 prefetch of what the update reads)
  bool has_q = false;
};

namespace {

// Tile of the single-run kernel, 256 threads (FP64: E2D_FUSED_NT64).  FP64: 32 x E2D_FUSED_TY64
// cells at E2D_FUSED_MINB64 CTAs per SM (shared memory and registers must
// allow that many); FP32: 32 x 15 cells at 4 CTAs per SM (64 registers, 4 x
// 55 KB of shared memory).  Both need the largest shared-memory carveout.
#ifndef E2D_FUSED_TX64
#define E2D_FUSED_TX64 32
#endif
#ifndef E2D_FUSED_TY64
#define E2D_FUSED_TY64 15
#endif
#ifndef E2D_FUSED_MINB64
#define E2D_FUSED_MINB64 2
#endif
#ifndef E2D_FUSED_NT64
#define E2D_FUSED_NT64 256
#endif
template <typename Real> struct FusedTile;
template <> struct FusedTile<double> { using C = TileCfg<double, E2D_FUSED_TX64, E2D_FUSED_TY64, E2D_FUSED_NT64>; };
template <> struct FusedTile<float> { using C = TileCfg<float, 32, 15, 256>; };

#ifndef E2D_PREFETCH_CONS
#define E2D_PREFETCH_CONS 1
#endif
#ifndef E2D_PREFETCH_CONS64
#define E2D_PREFETCH_CONS64 1
#endif

// Asks the TMA unit to bring a box of the map into L2 (no completion to wait for).
__device__ __forceinline__ void prefetch_box_l2(const CUtensorMap* tm, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(
                   reinterpret_cast<uint64_t>(tm)),
               "r"(x), "r"(y), "r"(0)
               : "memory");
}

// The tile (i0, j0)'s conservative values, which only the update reads,
// brought into L2 through an interior map (encode_state_map): x = i0 in FP64,
// the aligned i0 - 2 in FP32.
template <typename Real>
__device__ __forceinline__ void prefetch_cons(const CUtensorMap* tm, int i0, int j0) {
  prefetch_box_l2(tm, sizeof(Real) == 8 ? i0 : i0 - GW, j0);
}

// SQ: dx == dy (the shared face source term of tile_compute).  QIN: tm_in
// maps the primitives of the input state, and the primitives of the output
// go to qout (tile_compute); the tile's conservative values, which only the
// update reads, are prefetched into L2 through tm_cons when the box load is
// issued (FP32: +7 %; the FP64 persistent kernel, whose column-ordered walk
// finds fewer of them in L2: +0.9 %).
template <typename Real, bool SQ, bool QIN>
__global__ void __launch_bounds__(sizeof(Real) == 8 ? E2D_FUSED_NT64 : 256, sizeof(Real) == 8 ? E2D_FUSED_MINB64 : 4)
    k_fused(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_cons, Hydro<Real> h,
            Field<Real> in, Field<Real> out, Field<Real> qout, StepDt<Real> sd, Ctl* ctl, int fill_ghosts) {
  using C = typename FusedTile<Real>::C;
  extern __shared__ unsigned char smem_raw[];
  Real* base = reinterpret_cast<Real*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char* tail = reinterpret_cast<unsigned char*>(base + C::n_real);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tail);
  int* face_counter = reinterpret_cast<int*>(tail + 8);
  Real* red = reinterpret_cast<Real*>(tail + 16);
  Real* sdt = red + 32;  // dt, dt/dx, dt/dy of this step

  const int tid = threadIdx.x;
  const int i0 = GW + blockIdx.x * C::TX;  // first interior cell of the tile
  const int j0 = GW + blockIdx.y * C::TY;

  // ---- TMA load of the conservative box [i0-2, i0+TX+2) x [j0-2, j0+TY+2) x 4
  const uint32_t bar_a = smem_u32(bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    *face_counter = 0;
    // This step's dt (serial_ref/m_run.f90:308 when it comes from the running
    // maximum) and dt/dx, dt/dy (m_run.f90:384-385), once per CTA.
    const Real dt0 = sd.dt_ptr ? *sd.dt_ptr : sd.from_slot ? Ops<Real>::div(h.cfl, *inv_slot<Real>(ctl, sd.rd_slot)) : sd.dt_value;
    sdt[0] = dt0;
    sdt[1] = Ops<Real>::div(dt0, h.dx);  // (the integer-pipe division: the same bits)
    sdt[2] = Ops<Real>::div(dt0, h.dy);
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(C::box_bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(base + C::q_off)),
        "l"(reinterpret_cast<uint64_t>(&tm_in)), "r"(i0 - GW), "r"(j0 - GW), "r"(0), "r"(bar_a)
        : "memory");
    if (QIN && E2D_PREFETCH_CONS && sizeof(Real) == 4) prefetch_cons<Real>(&tm_cons, i0, j0);
  }
  const Real dt = sdt[0];
  const bool ok = mbar_wait(bar_a, 0, kTmaWaitCycles);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicOr(&ctl->health, 4u);
    return;
  }
  const bool want_dt = sd.wr_slot >= 0;
  Real m = tile_compute<Real, C, SQ, QIN>(h, base, face_counter, red, i0, j0, in, out, qout, sdt[1], sdt[2],
                                          fill_ghosts != 0, want_dt, &ctl->health);
  if (tid == 0) {
    if (blockIdx.x == 0 && blockIdx.y == 0) {
      if (sd.dt_log) sd.dt_log[sd.log_index] = dt;
      if (sd.inv_log && sd.rd_slot >= 0) sd.inv_log[sd.log_index] = *inv_slot<Real>(ctl, sd.rd_slot);
      if (!isfinite(dt)) atomicOr(&ctl->health, 1u);
    }
    if (want_dt) {
      if (sd.rd_slot >= 0) m = fmax(m, *inv_slot<Real>(ctl, sd.rd_slot));
      atomic_max_slot_ptr<Real>(inv_slot<Real>(ctl, sd.wr_slot), m);
    }
  }
}

// The FP64 step of the adjoint's forward sweeps: k_fused (conservative box)
// that also writes its input's primitives, slopes and trace sources to the
// tape the reverse step reads (tile_compute, TAPE); tape.only: just the tape.
template <bool SQ>
__global__ void __launch_bounds__(E2D_FUSED_NT64, E2D_FUSED_MINB64)
    k_fused_tape(const __grid_constant__ CUtensorMap tm_in, Hydro<double> h, Field<double> in, Field<double> out,
                 StepDt<double> sd, Ctl* ctl, TapeOut tape) {
  using C = typename FusedTile<double>::C;
  extern __shared__ unsigned char smem_raw[];
  double* base = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char* tail = reinterpret_cast<unsigned char*>(base + C::n_real);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tail);
  int* face_counter = reinterpret_cast<int*>(tail + 8);
  double* red = reinterpret_cast<double*>(tail + 16);
  double* sdt = red + 32;
  const int tid = threadIdx.x;
  const int i0 = GW + blockIdx.x * C::TX, j0 = GW + blockIdx.y * C::TY;
  const uint32_t bar_a = smem_u32(bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    *face_counter = 0;
    const double dt0 = sd.dt_ptr ? *sd.dt_ptr : sd.from_slot ? Ops<double>::div(h.cfl, *inv_slot<double>(ctl, sd.rd_slot)) : sd.dt_value;
    sdt[0] = dt0;
    sdt[1] = Ops<double>::div(dt0, h.dx);  // (the integer-pipe division: the same bits)
    sdt[2] = Ops<double>::div(dt0, h.dy);
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(C::box_bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(base + C::q_off)),
        "l"(reinterpret_cast<uint64_t>(&tm_in)), "r"(i0 - GW), "r"(j0 - GW), "r"(0), "r"(bar_a)
        : "memory");
  }
  const double dt = sdt[0];
  const bool ok = mbar_wait(bar_a, 0, kTmaWaitCycles);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicOr(&ctl->health, 4u);
    return;
  }
  const bool want_dt = sd.wr_slot >= 0 && !tape.only;
  double m = tile_compute<double, C, SQ, false, true>(h, base, face_counter, red, i0, j0, in, out, out, sdt[1],
                                                      sdt[2], true, want_dt, &ctl->health, NoHook(), &tape);
  if (tid == 0 && !tape.only) {
    if (blockIdx.x == 0 && blockIdx.y == 0) {
      if (sd.dt_log) sd.dt_log[sd.log_index] = dt;
      if (sd.inv_log && sd.rd_slot >= 0) sd.inv_log[sd.log_index] = *inv_slot<double>(ctl, sd.rd_slot);
      if (!isfinite(dt)) atomicOr(&ctl->health, 1u);
    }
    if (want_dt) {
      if (sd.rd_slot >= 0) m = Ops<double>::max(m, *inv_slot<double>(ctl, sd.rd_slot));
      atomic_max_slot_ptr<double>(inv_slot<double>(ctl, sd.wr_slot), m);
    }
  }
}

#ifndef E2D_FUSED_PERSISTENT
#define E2D_FUSED_PERSISTENT 1
#endif
// The taping step walks the tiles as the persistent step does (carry
// included); E2D_TAPE_PERSISTENT=0 launches one CTA per tile (k_fused_tape).
#ifndef E2D_TAPE_PERSISTENT
#define E2D_TAPE_PERSISTENT 1
#endif
// FP32 may take the persistent kernel too when its box is primitives (QIN:
// the next box lands in the 128-byte aligned primitives region); off, as
// measured: 19.4 against 19.7 Gcell/s for one CTA per tile at 2048^2 (FMA
// build; 20.6 against 21.6 with its faithful division and square root).
#ifndef E2D_FUSED_PERSISTENT32
#define E2D_FUSED_PERSISTENT32 0
#endif
template <typename Real, bool QIN>
constexpr bool use_persistent() {
  return sizeof(Real) == 8 ? E2D_FUSED_PERSISTENT != 0 : (E2D_FUSED_PERSISTENT32 != 0 && QIN);
}
#ifndef E2D_SQ_TRACE
#define E2D_SQ_TRACE 1
#endif

// Persistent variant (FP64, the default; E2D_FUSED_PERSISTENT=0 selects one
// CTA per tile): a grid of resident CTAs, each walking one contiguous run of
// the tiles in column order (up a column of tiles, then on to the next
// column; runs differ by at most one tile).  The box of a CTA's next tile is
// loaded by TMA into the box region as soon as the face phase of the current
// tile has ended (no later phase reads the box), so the load lands while the
// update phase runs.  One mbarrier, one phase per load; every wait is
// bounded.  A tile directly above the previous one takes over its top two
// ring rows and top y-face row (tile_compute's carry: 12 % fewer ring cells
// and 6 % fewer y faces at 32 x 15).
// TAPE (FP64, conservative boxes): the adjoint's forward step that also
// writes its input's forward values to `tape` (tape.only: just the tape).
#ifndef E2D_CARRY
#define E2D_CARRY 1
#endif
template <typename Real, bool SQ, bool QIN, bool TAPE = false>
__global__ void __launch_bounds__(sizeof(Real) == 8 ? E2D_FUSED_NT64 : 256, sizeof(Real) == 8 ? E2D_FUSED_MINB64 : 4)
    k_fused_persistent(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_cons,
                       Hydro<Real> h, Field<Real> in, Field<Real> out, Field<Real> qout, StepDt<Real> sd, Ctl* ctl,
                       int fill_ghosts, int nty, int ntiles, TapeOut tape) {
  static_assert(!TAPE || (sizeof(Real) == 8 && !QIN), "the tape is written by the FP64 conversion path");
  using C = typename FusedTile<Real>::C;
  extern __shared__ unsigned char smem_raw[];
  Real* base = reinterpret_cast<Real*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char* tail = reinterpret_cast<unsigned char*>(base + C::n_real);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tail);
  int* face_counter = reinterpret_cast<int*>(tail + 8);
  Real* red = reinterpret_cast<Real*>(tail + 16);
  Real* sdt = red + 32;
  Real* const dreg = base + C::q_off;  // where the next box lands (read by no phase after the faces)
  const int tid = threadIdx.x;
  const uint32_t bar_a = smem_u32(bar);
  // this CTA's run of tiles [t_begin, t_end); tile t is column t / nty, row t % nty
  const int per = ntiles / (int)gridDim.x, extra = ntiles % (int)gridDim.x, b = (int)blockIdx.x;
  const int t_begin = b * per + min(b, extra), t_end = t_begin + per + (b < extra ? 1 : 0);
  auto issue = [&](int t, Real* dst) {  // thread 0: the box of tile t into dst
    const int i0 = GW + (t / nty) * C::TX, j0 = GW + (t % nty) * C::TY;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(C::box_bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(&tm_in)), "r"(i0 - GW), "r"(j0 - GW), "r"(0), "r"(bar_a)
        : "memory");
    if (QIN && E2D_PREFETCH_CONS && (sizeof(Real) == 4 || E2D_PREFETCH_CONS64)) prefetch_cons<Real>(&tm_cons, i0, j0);
  };
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *face_counter = 0;
    const Real dt0 = sd.dt_ptr ? *sd.dt_ptr : sd.from_slot ? Ops<Real>::div(h.cfl, *inv_slot<Real>(ctl, sd.rd_slot)) : sd.dt_value;
    sdt[0] = dt0;
    sdt[1] = Ops<Real>::div(dt0, h.dx);  // (the integer-pipe division: the same bits)
    sdt[2] = Ops<Real>::div(dt0, h.dy);
    if (t_begin < t_end) issue(t_begin, base + C::q_off);
  }
  __syncthreads();
  const bool only = TAPE && tape.only;  // a tape-only pass: no update, no dt
  const bool want_dt = sd.wr_slot >= 0 && !only;
  Real mmax = Real(0);
  uint32_t parity = 0;
  bool first = true;
  for (int t = t_begin; t < t_end; ++t) {
    const bool ok = mbar_wait(bar_a, parity, kTmaWaitCycles);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(&ctl->health, 4u);
      return;
    }
    parity ^= 1;
    const int next = t + 1;
    const int i0 = GW + (t / nty) * C::TX, j0 = GW + (t % nty) * C::TY;
    auto prefetch = [&]() {
      if (tid == 0 && next < t_end) issue(next, dreg);
    };
    // the tile below was this CTA's previous one / the next one is the tile above
    const int carry = E2D_CARRY
                          ? ((!first && t % nty != 0) ? kCarryIn : 0) | ((next < t_end && next % nty != 0) ? kCarryOut : 0)
                          : 0;
    const Real m = tile_compute<Real, C, SQ, QIN, TAPE>(h, base, face_counter, red, i0, j0, in, out, qout,
                                                        sdt[1], sdt[2], fill_ghosts != 0, want_dt, &ctl->health,
                                                        prefetch, TAPE ? &tape : nullptr, NoHook(), carry);
    if (tid == 0) {
      mmax = Ops<Real>::max(mmax, m);
      *face_counter = 0;
    }
    __syncthreads();  // this tile's shared data consumed; the counter reset is visible
    first = false;
  }
  if (tid == 0 && !only) {
    const Real dt = sdt[0];
    if (blockIdx.x == 0) {
      if (sd.dt_log) sd.dt_log[sd.log_index] = dt;
      if (sd.inv_log && sd.rd_slot >= 0) sd.inv_log[sd.log_index] = *inv_slot<Real>(ctl, sd.rd_slot);
      if (!isfinite(dt)) atomicOr(&ctl->health, 1u);
    }
    if (want_dt) {
      if (sd.rd_slot >= 0) mmax = Ops<Real>::max(mmax, *inv_slot<Real>(ctl, sd.rd_slot));
      atomic_max_slot_ptr<Real>(inv_slot<Real>(ctl, sd.wr_slot), mmax);
    }
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Resident CTAs per SM x SMs of the current device (the persistent grid).
template <typename Real, bool SQ, bool QIN, bool TAPE = false>
int persistent_grid() {
  static int grid[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!grid[dev]) {
    using C = typename FusedTile<Real>::C;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_persistent<Real, SQ, QIN, TAPE>, C::NT,
                                                  C::bytes);
    grid[dev] = std::max(1, sms * std::max(1, per_sm));
  }
  return grid[dev];
}

// Dynamic shared memory of the tile, and the largest shared-memory carveout
// so that as many CTAs as the launch bounds ask for fit on an SM.
template <typename Real, bool SQ, bool QIN, bool TAPE = false>
bool set_persistent_attributes() {
  using C = typename FusedTile<Real>::C;
  return cudaFuncSetAttribute(k_fused_persistent<Real, SQ, QIN, TAPE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)C::bytes) == cudaSuccess &&
         cudaFuncSetAttribute(k_fused_persistent<Real, SQ, QIN, TAPE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                              (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess &&
         persistent_grid<Real, SQ, QIN, TAPE>() > 0;  // sized here, outside any stream capture
}

template <typename Real, bool SQ, bool QIN>
bool set_fused_attributes_sq() {
  using C = typename FusedTile<Real>::C;
  bool ok = cudaFuncSetAttribute(k_fused<Real, SQ, QIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)C::bytes) == cudaSuccess &&
            cudaFuncSetAttribute(k_fused<Real, SQ, QIN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess;
  if constexpr (use_persistent<Real, QIN>()) ok = ok && set_persistent_attributes<Real, SQ, QIN>();
  return ok;
}

template <typename Real>
bool set_fused_attributes() {
  bool ok = set_fused_attributes_sq<Real, false, false>() && set_fused_attributes_sq<Real, true, false>() &&
            set_fused_attributes_sq<Real, false, true>() && set_fused_attributes_sq<Real, true, true>();
  if constexpr (sizeof(Real) == 8) {
    using C = typename FusedTile<double>::C;
    ok = ok &&
         cudaFuncSetAttribute(k_fused_tape<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes) ==
             cudaSuccess &&
         cudaFuncSetAttribute(k_fused_tape<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes) ==
             cudaSuccess &&
         cudaFuncSetAttribute(k_fused_tape<false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                              (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess &&
         cudaFuncSetAttribute(k_fused_tape<true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                              (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess;
    if constexpr (E2D_FUSED_PERSISTENT && E2D_TAPE_PERSISTENT)
      ok = ok && set_persistent_attributes<double, false, false, true>() &&
           set_persistent_attributes<double, true, false, true>();
  }
  return ok;
}

template <typename Real, bool SQ, bool QIN>
void launch_fused_sq(const CUtensorMap& tm, const CUtensorMap& tmc, const Hydro<Real>& h, Field<Real> in,
                     Field<Real> out, Field<Real> qout, StepDt<Real> sd, Ctl* ctl, bool fill_ghosts,
                     cudaStream_t s) {
  using C = typename FusedTile<Real>::C;
  const int ntx = (h.nx + C::TX - 1) / C::TX, nty = (h.ny + C::TY - 1) / C::TY;
  if constexpr (use_persistent<Real, QIN>()) {
    const int grid = std::min(ntx * nty, persistent_grid<Real, SQ, QIN>());
    k_fused_persistent<Real, SQ, QIN><<<grid, C::NT, C::bytes, s>>>(tm, tmc, h, in, out, qout, sd, ctl,
                                                                    fill_ghosts ? 1 : 0, nty, ntx * nty,
                                                                    TapeOut{});
  } else {
    k_fused<Real, SQ, QIN><<<dim3(ntx, nty), C::NT, C::bytes, s>>>(tm, tmc, h, in, out, qout, sd, ctl,
                                                                   fill_ghosts ? 1 : 0);
  }
}

// dx == dy (a square domain of square cells, every benchmark grid) takes the
// instantiation that forms each cell's face source term once.  qout set: tm
// maps the input's primitives (QIN) and tmc its conservative values.
template <typename Real>
void launch_fused_tm(const CUtensorMap& tm, const CUtensorMap& tmc, const Hydro<Real>& h, Field<Real> in,
                     Field<Real> out, const Field<Real>* qout, StepDt<Real> sd, Ctl* ctl, bool fill_ghosts,
                     cudaStream_t s) {
  const Field<Real> qo = qout ? *qout : out;
#if E2D_SQ_TRACE
  if (h.dx == h.dy) {
    if (qout) launch_fused_sq<Real, true, true>(tm, tmc, h, in, out, qo, sd, ctl, fill_ghosts, s);
    else launch_fused_sq<Real, true, false>(tm, tmc, h, in, out, qo, sd, ctl, fill_ghosts, s);
    return;
  }
#endif
  if (qout) launch_fused_sq<Real, false, true>(tm, tmc, h, in, out, qo, sd, ctl, fill_ghosts, s);
  else launch_fused_sq<Real, false, false>(tm, tmc, h, in, out, qo, sd, ctl, fill_ghosts, s);
}

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

// 3D map over a pitched state: dims (isize, jsize, 4), zero fill outside;
// boxes of the tile with its 2-cell halo, or (interior) of the tile's rows
// alone -- in FP64 the tile itself (its first column i0 is 16-byte aligned),
// in FP32 the rows' 36 columns from the aligned column i0 - 2 (the TMA
// start rule: x times the element size a multiple of 16 bytes).  The
// interior maps serve prefetch_cons.
template <typename Real>
bool encode_state_map(CUtensorMap* tm, const Hydro<Real>& h, Field<Real> f, bool interior = false) {
  using S = typename FusedTile<Real>::C;
  EncodeTiledFn enc = get_encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)h.isize, (cuuint64_t)h.jsize, 4};
  const cuuint64_t strides[2] = {(cuuint64_t)f.pitch * sizeof(Real), (cuuint64_t)f.plane * sizeof(Real)};
  const cuuint32_t box[3] = {(cuuint32_t)(interior && sizeof(Real) == 8 ? S::TX : S::BXs),
                             (cuuint32_t)(interior ? S::TY : S::BYs), 4};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt =
      sizeof(Real) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  return enc(tm, dt, 3, f.p, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

template <typename Real>
FusedPlan* fused_plan_create(const Hydro<Real>& h, Field<Real> u, Field<Real> u2, const Field<Real>* q,
                             const Field<Real>* q2) {
  using C = typename FusedTile<Real>::C;
  static_assert(C::BXs * sizeof(Real) % 16 == 0, "TMA inner box must be a multiple of 16 bytes");
  static_assert((C::TX * sizeof(Real)) % 16 == 0, "tile x origin must stay 16-byte aligned");
  static_assert(sizeof(Real) != 8 || (GW * sizeof(Real)) % 16 == 0, "FP64 interior prefetch starts at column GW");
  FusedPlan* p = new FusedPlan;
  if (!encode_state_map<Real>(&p->tm[0], h, u) || !encode_state_map<Real>(&p->tm[1], h, u2) ||
      !encode_state_map<Real>(&p->tmi[0], h, u, true) || !encode_state_map<Real>(&p->tmi[1], h, u2, true)) {
    delete p;
    return nullptr;
  }
  if (q && q2) {
    if (!encode_state_map<Real>(&p->tmq[0], h, *q) || !encode_state_map<Real>(&p->tmq[1], h, *q2)) {
      delete p;
      return nullptr;
    }
    p->has_q = true;
  }
  if (!set_fused_attributes<Real>()) {
    cudaGetLastError();
    delete p;
    return nullptr;
  }
  return p;
}

void fused_plan_destroy(FusedPlan* p) { delete p; }

template <typename Real>
void launch_fused(const Hydro<Real>& h, FusedPlan* plan, int in_is_u2, Field<Real> in, Field<Real> out,
                  StepDt<Real> sd, Ctl* ctl, bool fill_ghosts, cudaStream_t s, const Field<Real>* qout) {
  const CUtensorMap& tmc = plan->tm[in_is_u2 ? 1 : 0];
  if (qout && plan->has_q)
    launch_fused_tm<Real>(plan->tmq[in_is_u2 ? 1 : 0], plan->tmi[in_is_u2 ? 1 : 0], h, in, out, qout, sd, ctl,
                          fill_ghosts, s);
  else
    launch_fused_tm<Real>(tmc, tmc, h, in, out, nullptr, sd, ctl, fill_ghosts, s);
}

template <typename Real>
bool fused_map_create(const Hydro<Real>& h, Field<Real> u, StateMap* out, bool interior) {
  static_assert(sizeof(StateMap) == sizeof(CUtensorMap), "descriptor size");
  using C = typename FusedTile<Real>::C;
  if (!set_fused_attributes<Real>()) {
    cudaGetLastError();
    return false;
  }
  return encode_state_map<Real>(reinterpret_cast<CUtensorMap*>(out->bytes), h, u, interior);
}

template <typename Real>
void launch_fused_map(const Hydro<Real>& h, const StateMap& map, Field<Real> in, Field<Real> out, StepDt<Real> sd,
                      Ctl* ctl, bool fill_ghosts, cudaStream_t s) {
  const CUtensorMap& tm = *reinterpret_cast<const CUtensorMap*>(map.bytes);
  launch_fused_tm<Real>(tm, tm, h, in, out, nullptr, sd, ctl, fill_ghosts, s);
}

template <bool SQ>
void launch_fused_tape_sq(const CUtensorMap& tm, const Hydro<double>& h, Field<double> in, Field<double> out,
                          StepDt<double> sd, Ctl* ctl, const TapeOut& tape, cudaStream_t s) {
  using C = typename FusedTile<double>::C;
  const int ntx = (h.nx + C::TX - 1) / C::TX, nty = (h.ny + C::TY - 1) / C::TY;
  if constexpr (E2D_FUSED_PERSISTENT && E2D_TAPE_PERSISTENT) {
    const int grid = std::min(ntx * nty, persistent_grid<double, SQ, false, true>());
    k_fused_persistent<double, SQ, false, true><<<grid, C::NT, C::bytes, s>>>(tm, tm, h, in, out, out, sd, ctl, 1,
                                                                              nty, ntx * nty, tape);
  } else {
    k_fused_tape<SQ><<<dim3(ntx, nty), C::NT, C::bytes, s>>>(tm, h, in, out, sd, ctl, tape);
  }
}

void launch_fused_tape(const Hydro<double>& h, const StateMap& map, Field<double> in, Field<double> out,
                       StepDt<double> sd, Ctl* ctl, const TapeOut& tape, cudaStream_t s) {
  const CUtensorMap& tm = *reinterpret_cast<const CUtensorMap*>(map.bytes);
  if (E2D_SQ_TRACE && h.dx == h.dy) launch_fused_tape_sq<true>(tm, h, in, out, sd, ctl, tape, s);
  else launch_fused_tape_sq<false>(tm, h, in, out, sd, ctl, tape, s);
}

void launch_fused_map_q(const Hydro<double>& h, const StateMap& qmap, const StateMap& imap, Field<double> in,
                        Field<double> out, Field<double> qout, StepDt<double> sd, Ctl* ctl, cudaStream_t s) {
  const CUtensorMap& tm = *reinterpret_cast<const CUtensorMap*>(qmap.bytes);
  const CUtensorMap& tmi = *reinterpret_cast<const CUtensorMap*>(imap.bytes);
  launch_fused_tm<double>(tm, tmi, h, in, out, &qout, sd, ctl, true, s);
}

template bool fused_map_create<double>(const Hydro<double>&, Field<double>, StateMap*, bool);
template bool fused_map_create<float>(const Hydro<float>&, Field<float>, StateMap*, bool);
template void launch_fused_map<double>(const Hydro<double>&, const StateMap&, Field<double>, Field<double>,
                                       StepDt<double>, Ctl*, bool, cudaStream_t);
template void launch_fused_map<float>(const Hydro<float>&, const StateMap&, Field<float>, Field<float>,
                                      StepDt<float>, Ctl*, bool, cudaStream_t);
template FusedPlan* fused_plan_create<double>(const Hydro<double>&, Field<double>, Field<double>,
                                              const Field<double>*, const Field<double>*);
template FusedPlan* fused_plan_create<float>(const Hydro<float>&, Field<float>, Field<float>, const Field<float>*,
                                             const Field<float>*);
template void launch_fused<double>(const Hydro<double>&, FusedPlan*, int, Field<double>, Field<double>,
                                   StepDt<double>, Ctl*, bool, cudaStream_t, const Field<double>*);
template void launch_fused<float>(const Hydro<float>&, FusedPlan*, int, Field<float>, Field<float>,
                                  StepDt<float>, Ctl*, bool, cudaStream_t, const Field<float>*);

}  // namespace e2d
