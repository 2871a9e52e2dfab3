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
#include "sync.cuh"
#include "tile.cuh"

namespace e2d {

struct FusedPlan {
  CUtensorMap tm[2];  // [0]: u, [1]: u2
};

namespace {

// Tile of the single-run kernel, 256 threads.  FP64: 32 x E2D_FUSED_TY64
// cells at E2D_FUSED_MINB64 CTAs per SM (shared memory and registers must
// allow that many); FP32: 32 x 15 cells at 4 CTAs per SM (64 registers, 4 x
// 55 KB of shared memory).  Both need the largest shared-memory carveout.
#ifndef E2D_FUSED_TY64
#define E2D_FUSED_TY64 15
#endif
#ifndef E2D_FUSED_MINB64
#define E2D_FUSED_MINB64 2
#endif
template <typename Real> struct FusedTile;
template <> struct FusedTile<double> { using C = TileCfg<double, 32, E2D_FUSED_TY64, 256>; };
template <> struct FusedTile<float> { using C = TileCfg<float, 32, 15, 256>; };

template <typename Real>
__global__ void __launch_bounds__(256, sizeof(Real) == 8 ? E2D_FUSED_MINB64 : 4)
    k_fused(const __grid_constant__ CUtensorMap tm_in, Hydro<Real> h, Field<Real> in, Field<Real> out,
            StepDt<Real> sd, Ctl* ctl, int fill_ghosts) {
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
    const Real dt0 = sd.dt_ptr ? *sd.dt_ptr : sd.from_slot ? h.cfl / *inv_slot<Real>(ctl, sd.rd_slot) : sd.dt_value;
    sdt[0] = dt0;
    sdt[1] = dt0 / h.dx;
    sdt[2] = dt0 / h.dy;
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
  const Real dt = sdt[0];
  const bool ok = mbar_wait(bar_a, 0, kTmaWaitCycles);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) atomicOr(&ctl->health, 4u);
    return;
  }
  const bool want_dt = sd.wr_slot >= 0;
  Real m = tile_compute<Real, C>(h, base, face_counter, red, i0, j0, in, out, sdt[1], sdt[2], fill_ghosts != 0,
                                 want_dt, &ctl->health);
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

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Dynamic shared memory of the tile, and the largest shared-memory carveout
// so that as many CTAs as the launch bounds ask for fit on an SM.
template <typename Real>
bool set_fused_attributes() {
  using C = typename FusedTile<Real>::C;
  return cudaFuncSetAttribute(k_fused<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes) ==
             cudaSuccess &&
         cudaFuncSetAttribute(k_fused<Real>, cudaFuncAttributePreferredSharedMemoryCarveout,
                              (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess;
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

// 3D map over a pitched state: dims (isize, jsize, 4), zero fill outside.
template <typename Real>
bool encode_state_map(CUtensorMap* tm, const Hydro<Real>& h, Field<Real> f) {
  using S = typename FusedTile<Real>::C;
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
  using C = typename FusedTile<Real>::C;
  static_assert(C::BXs * sizeof(Real) % 16 == 0, "TMA inner box must be a multiple of 16 bytes");
  static_assert((C::TX * sizeof(Real)) % 16 == 0, "tile x origin must stay 16-byte aligned");
  FusedPlan* p = new FusedPlan;
  if (!encode_state_map<Real>(&p->tm[0], h, u) || !encode_state_map<Real>(&p->tm[1], h, u2)) {
    delete p;
    return nullptr;
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
                  StepDt<Real> sd, Ctl* ctl, bool fill_ghosts, cudaStream_t s) {
  using C = typename FusedTile<Real>::C;
  dim3 g((h.nx + C::TX - 1) / C::TX, (h.ny + C::TY - 1) / C::TY);
  k_fused<Real><<<g, C::NT, C::bytes, s>>>(plan->tm[in_is_u2 ? 1 : 0], h, in, out, sd, ctl, fill_ghosts ? 1 : 0);
}

template <typename Real>
bool fused_map_create(const Hydro<Real>& h, Field<Real> u, StateMap* out) {
  static_assert(sizeof(StateMap) == sizeof(CUtensorMap), "descriptor size");
  using C = typename FusedTile<Real>::C;
  if (!set_fused_attributes<Real>()) {
    cudaGetLastError();
    return false;
  }
  return encode_state_map<Real>(reinterpret_cast<CUtensorMap*>(out->bytes), h, u);
}

template <typename Real>
void launch_fused_map(const Hydro<Real>& h, const StateMap& map, Field<Real> in, Field<Real> out, StepDt<Real> sd,
                      Ctl* ctl, bool fill_ghosts, cudaStream_t s) {
  using C = typename FusedTile<Real>::C;
  dim3 g((h.nx + C::TX - 1) / C::TX, (h.ny + C::TY - 1) / C::TY);
  k_fused<Real><<<g, C::NT, C::bytes, s>>>(*reinterpret_cast<const CUtensorMap*>(map.bytes), h, in, out, sd, ctl,
                                           fill_ghosts ? 1 : 0);
}

template bool fused_map_create<double>(const Hydro<double>&, Field<double>, StateMap*);
template bool fused_map_create<float>(const Hydro<float>&, Field<float>, StateMap*);
template void launch_fused_map<double>(const Hydro<double>&, const StateMap&, Field<double>, Field<double>,
                                       StepDt<double>, Ctl*, bool, cudaStream_t);
template void launch_fused_map<float>(const Hydro<float>&, const StateMap&, Field<float>, Field<float>,
                                      StepDt<float>, Ctl*, bool, cudaStream_t);
template FusedPlan* fused_plan_create<double>(const Hydro<double>&, Field<double>, Field<double>);
template FusedPlan* fused_plan_create<float>(const Hydro<float>&, Field<float>, Field<float>);
template void launch_fused<double>(const Hydro<double>&, FusedPlan*, int, Field<double>, Field<double>,
                                   StepDt<double>, Ctl*, bool, cudaStream_t);
template void launch_fused<float>(const Hydro<float>&, FusedPlan*, int, Field<float>, Field<float>,
                                  StepDt<float>, Ctl*, bool, cudaStream_t);

}  // namespace e2d
