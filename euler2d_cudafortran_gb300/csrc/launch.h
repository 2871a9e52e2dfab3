// launch.h -- host-side launchers shared by the translation units of the library.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "physics.cuh"

namespace e2d {

// Small device control block of a run: running CFL maxima (two slots, so a
// step can read one while its update kernel folds the next state's maximum
// into the other), health flags and the device dt log.
struct Ctl {
  unsigned long long inv64[2];  // FP64 runs: bit images of invDt (non-negative)
  unsigned int inv32[2];        // FP32 runs
  unsigned int health;          // E2D_HEALTH_* bits
  unsigned int pad;
};

template <typename Real> __host__ __device__ inline Real* inv_slot(Ctl* c, int s);
template <> __host__ __device__ inline double* inv_slot<double>(Ctl* c, int s) { return reinterpret_cast<double*>(&c->inv64[s]); }
template <> __host__ __device__ inline float* inv_slot<float>(Ctl* c, int s) { return reinterpret_cast<float*>(&c->inv32[s]); }

// Where a step kernel takes its dt from: a host value (godunov_unsplit called
// with dt, as serial_ref/main.f90:72) or the running maximum on the device
// (dt = cfl / invDt, serial_ref/m_run.f90:308), logged to dt_log[log_index].
template <typename Real>
struct StepDt {
  Real dt_value;
  const Real* dt_ptr;  // when set, dt is read from this device address (a logged dt)
  int from_slot;    // 1: dt = cfl / inv[rd_slot]
  int rd_slot;      // slot holding the running max for this step's dt
  int wr_slot;      // slot receiving max(inv[rd], max over the new state); -1: no reduction
  Real* dt_log;     // device; may be null
  int log_index;
  Real* inv_log = nullptr;  // device; if set, receives inv[rd_slot] (the running max this step's dt uses)
};

// ---- abi.cu ----
// Records msg as the text returned by e2d_last_error on this thread; returns code.
int set_error(int code, const std::string& msg);

// ---- k_sweeps.cu ----
template <typename Real> void launch_init_diagonal(const Hydro<Real>& h, Field<Real> u, double offset, double rho_hi,
                                                   double p_hi, double rho_lo, double p_lo, cudaStream_t s);
template <typename Real> void launch_boundaries(const Hydro<Real>& h, Field<Real> u, cudaStream_t s);
// Row copy between pitched arrays of 4- or 8-byte words (pitches in words);
// either side may be mapped pinned host memory (copies at the host link's
// rate without a staging buffer).
void launch_repitch(const void* src, size_t src_pitch, void* dst, size_t dst_pitch, int width, int rows,
                    int word_bytes, cudaStream_t s);
// make_boundaries on u and, in the same launch, on w (same layout and rules).
template <typename Real>
void launch_boundaries_pair(const Hydro<Real>& h, Field<Real> u, Field<Real> w, cudaStream_t s);
// Reduce the CFL maximum of u into ctl->inv[slot] (atomic max; running max kept).
template <typename Real> void launch_dt_reduce(const Hydro<Real>& h, Field<Real> u, Ctl* ctl, int slot, cudaStream_t s);
template <typename Real> void launch_prim(const Hydro<Real>& h, Field<Real> u, Field<Real> q, cudaStream_t s);
// implementationVersion 2: fluxes stored (serial_ref computeAndStoreFluxes + updateHydro)
template <typename Real> void launch_fluxes_v2(const Hydro<Real>& h, Field<Real> q, StepDt<Real> sd, Ctl* ctl,
                                               Field<Real> fx, Field<Real> fy, cudaStream_t s);
template <typename Real> void launch_update_v2(const Hydro<Real>& h, Field<Real> in, Field<Real> fx, Field<Real> fy,
                                               Field<Real> out, StepDt<Real> sd, Ctl* ctl, cudaStream_t s);
// implementationVersion 1: face states stored, then fluxes + update in one tiled kernel
template <typename Real> void launch_trace_v1(const Hydro<Real>& h, Field<Real> q, StepDt<Real> sd, Ctl* ctl,
                                              Field<Real> qxm, Field<Real> qxp, Field<Real> qym, Field<Real> qyp,
                                              cudaStream_t s);
template <typename Real> void launch_flux_update_v1(const Hydro<Real>& h, Field<Real> in, Field<Real> qxm,
                                                    Field<Real> qxp, Field<Real> qym, Field<Real> qyp,
                                                    Field<Real> out, StepDt<Real> sd, Ctl* ctl, cudaStream_t s);

// ---- k_fused.cu ---- implementationVersion 0: one fused kernel per step.
// Builds (once per state buffer) the TMA descriptor of a state, and of the
// primitive-variable arrays q, q2 kept beside u, u2 when they are given.
struct FusedPlan;
template <typename Real> FusedPlan* fused_plan_create(const Hydro<Real>& h, Field<Real> u, Field<Real> u2,
                                                      const Field<Real>* q = nullptr,
                                                      const Field<Real>* q2 = nullptr);
void fused_plan_destroy(FusedPlan* p);
// qout set (and the plan has q arrays): the step reads the primitives of its
// input from the q array beside it -- they must be current, ghosts and
// corners included -- and writes those of its output to *qout.
template <typename Real> void launch_fused(const Hydro<Real>& h, FusedPlan* plan, int in_is_u2, Field<Real> in,
                                           Field<Real> out, StepDt<Real> sd, Ctl* ctl, bool fill_ghosts,
                                           cudaStream_t s, const Field<Real>* qout = nullptr);
// A TMA descriptor for any pitched state (used for states outside a run's u/u2):
// boxes of a tile with its halo, or (interior) of the tile alone.
struct StateMap { alignas(64) unsigned char bytes[128]; };
template <typename Real>
bool fused_map_create(const Hydro<Real>& h, Field<Real> u, StateMap* out, bool interior = false);
// Where a forward step leaves the values of its input state that the reverse
// step recomputes otherwise (the adjoint's tape): the primitives of every
// cell, and the slopes and trace source terms of the cells the reverse's
// rings reach (i in [1, nx+2], j in [1, ny+2]), and optionally each face's
// HLLC solve.  Pitched like a state; each cell and face is written by exactly
// one tile.  only: stop before the update (a
// state whose step is not run).
struct TapeOut {
  double* q = nullptr;   // [4] planes
  double* dq = nullptr;  // [8] planes: dqx[4], dqy[4]
  double* s = nullptr;   // [4] planes
  // optional: the recorded HLLC solve of every face (physics.cuh, HR_*
  // planes and a plane of HF_* flags), x faces at the cell to their right,
  // y faces at the cell above them
  double* fx = nullptr;
  double* fy = nullptr;
  unsigned* flx = nullptr;
  unsigned* fly = nullptr;
  // the limiter cases of the ring cells' eight slopes (slopes<Real, true>)
  unsigned* lim = nullptr;
  int pitch = 0;
  long long plane = 0;
  int only = 0;
  __host__ __device__ __forceinline__ unsigned& flag(unsigned* b, int j, int i) const {
    return b[(long long)j * pitch + i];
  }
  __host__ __device__ __forceinline__ double& at(double* b, int v, int j, int i) const {
    return b[(long long)v * plane + (long long)j * pitch + i];
  }
};

// Planes of one tape: q 4, dq 8, s 4, x and y face records HR_N each, the
// two planes of 32-bit face flags in one plane of doubles, and the 32-bit
// limiter cases in one more.
constexpr int kTapePlanes = 4 + 8 + 4 + 2 * HR_N + 2;

// Tape j of a run of tapes at `base` (kTapePlanes planes each) of a state
// with `plane` elements per plane and row pitch `pitch`.
__host__ __device__ inline TapeOut tape_at(double* base, int j, long long plane, int pitch, bool only) {
  TapeOut t;
  double* b = base + (long long)j * kTapePlanes * plane;
  t.q = b;
  t.dq = b + 4 * plane;
  t.s = b + 12 * plane;
  t.fx = b + 16 * plane;
  t.fy = t.fx + HR_N * plane;
  t.flx = reinterpret_cast<unsigned*>(t.fy + HR_N * plane);
  t.fly = t.flx + plane;
  t.lim = t.fly + plane;
  t.pitch = pitch;
  t.plane = plane;
  t.only = only ? 1 : 0;
  return t;
}

// The adjoint's forward step: also writes its input's forward values to the
// tape; tape.only writes just those.
void launch_fused_tape(const Hydro<double>& h, const StateMap& map, Field<double> in, Field<double> out,
                       StepDt<double> sd, Ctl* ctl, const TapeOut& tape, cudaStream_t s);
// The step with primitives kept beside the states (as the run's advance):
// qmap maps the input's primitives (current, ghosts and corners included),
// imap the interior tiles of the input state (prefetched into L2 for the
// update); the output's primitives go to qout.  Ghosts of the output are filled.
void launch_fused_map_q(const Hydro<double>& h, const StateMap& qmap, const StateMap& imap, Field<double> in,
                        Field<double> out, Field<double> qout, StepDt<double> sd, Ctl* ctl, cudaStream_t s);
template <typename Real> void launch_fused_map(const Hydro<Real>& h, const StateMap& map, Field<Real> in,
                                               Field<Real> out, StepDt<Real> sd, Ctl* ctl, bool fill_ghosts,
                                               cudaStream_t s);

}  // namespace e2d
