// noalloc.cu -- one Godunov step that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host code whose GPU memory is owned
// by another runtime or memory pool (a Fortran code whose device arrays come
// from its own allocator, or a solver embedded in a framework that forbids
// allocations on its time-step path and hands the step only its input and
// output arrays).  For them this file offers e2d_godunov_unsplit_noalloc:
// the stored-fluxes variant of the step (make_boundaries, primitives, fluxes,
// update: the arithmetic of serial_ref/m_run.f90:210-243) whose work arrays
// (primitives q, fluxes fx and fy, and the control word of the kernels) live
// in the file-scope device array below instead of memory allocated per run.
//
// The array has a fixed size, E2D_NOALLOC_SCRATCH_BYTES (48 MiB); every GPU
// that loads this library reserves it until the process exits.  Grids whose
// three work arrays do not fit are rejected with E2D_ERR_INVALID_ARG.  All
// calls share the one array, which keeps the contents of the last call, so
// calls that may overlap on the GPU (different streams, different host
// threads) race with each other and must be serialised by the caller.
//
// The first call on a device looks up the device address of the array
// (cudaGetSymbolAddress, once per device and CUDA context, with that device
// current); make that first call before any stream capture begins.  The
// address is kept per device together with the identity of the context it
// was looked up in, so a call made after cudaDeviceReset (a new primary
// context, the module loaded again) looks it up again instead of using a
// stale address.
//
// Numerical health: the kernels raise the E2D_HEALTH_* bits of the step (a
// new density that is not a positive finite number) in the scratch's control
// word, cleared at the start of every call.  A caller that passes `health`
// receives them: the call then waits for its step to finish.
#include <cuda.h>
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/euler2d_gb300.h"
#include "hydro_params.h"
#include "launch.h"

using namespace e2d;

namespace {

constexpr size_t kCtlBytes = 256;  // control block, padded to keep the planes 256-byte aligned

// The scratch: the control block, then q, fx, fy (4 planes each, pitched).
static __device__ __align__(256) unsigned char g_noalloc_scratch[E2D_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_dev[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};

// Identity of the current CUDA context (cuCtxGetId, unique within the
// process), through the runtime's driver entry points; 0 when unavailable.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {  // called with g_mutex held
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
    resolved = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS) return id;
  return 0;
}

// Device address of the scratch array on the current device.  The host-side
// symbol g_noalloc_scratch is only a stand-in; the device address is looked up
// once per device and context, with that device current (when the context's
// identity cannot be read, on every call).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(E2D_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return set_error(E2D_ERR_INVALID_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (cudaSetDevice(dev) != cudaSuccess) {  // the same device: makes its primary context current
    cudaGetLastError();
    return set_error(E2D_ERR_NO_DEVICE, "no usable CUDA context on the current device");
  }
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_dev[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      return set_error(E2D_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    }
    g_scratch_dev[dev] = ptr;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_dev[dev];
  return E2D_OK;
}

template <typename Real>
int step(const e2d_params& p, void* u_in, void* u_out, size_t pitch, double dt, unsigned char* scratch,
         size_t work_pitch, cudaStream_t s, unsigned* health) {
  const Hydro<Real> h = make_hydro<Real>(p);
  const long long plane = (long long)pitch * h.jsize;
  const long long wplane = (long long)work_pitch * h.jsize;
  Field<Real> in{static_cast<Real*>(u_in), (int)pitch, plane};
  Field<Real> out{static_cast<Real*>(u_out), (int)pitch, plane};
  Ctl* ctl = reinterpret_cast<Ctl*>(scratch);
  Real* base = reinterpret_cast<Real*>(scratch + kCtlBytes);
  Field<Real> q{base, (int)work_pitch, wplane};
  Field<Real> fx{base + 4 * wplane, (int)work_pitch, wplane};
  Field<Real> fy{base + 8 * wplane, (int)work_pitch, wplane};
  StepDt<Real> sd;
  sd.dt_value = (Real)dt;
  sd.dt_ptr = nullptr;
  sd.from_slot = 0;
  sd.rd_slot = -1;
  sd.wr_slot = -1;
  sd.dt_log = nullptr;
  sd.log_index = 0;
  // The health word must start at zero; the work arrays are fully written
  // before they are read, so the previous call's contents need no clearing.
  if (cudaMemsetAsync(ctl, 0, sizeof(Ctl), s) != cudaSuccess) return set_error(E2D_ERR_CUDA, "cudaMemsetAsync failed");
  launch_boundaries<Real>(h, in, s);
  launch_prim<Real>(h, in, q, s);
  launch_fluxes_v2<Real>(h, q, sd, ctl, fx, fy, s);
  launch_update_v2<Real>(h, in, fx, fy, out, sd, ctl, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(E2D_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  if (health) {
    e = cudaMemcpyAsync(health, &ctl->health, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(E2D_ERR_CUDA, std::string("reading the health flags: ") + cudaGetErrorString(e));
    }
  }
  return E2D_OK;
}

}  // namespace

extern "C" int e2d_godunov_unsplit_noalloc(const e2d_params* p, void* u_in, void* u_out, size_t pitch_elems,
                                           double dt, void* stream, unsigned* health) {
  if (!p || !u_in || !u_out) return set_error(E2D_ERR_INVALID_ARG, "null arguments");
  if (p->nx < 2 || p->ny < 2 || p->nx > (1 << 20) || p->ny > (1 << 20) || (p->precision != 4 && p->precision != 8) ||
      (p->riemann_solver != E2D_RIEMANN_APPROX && p->riemann_solver != E2D_RIEMANN_HLLC) || !(p->gamma0 > 1.0) ||
      !(p->smallr > 0.0) || !(p->smallc > 0.0) || p->niter_riemann < 0)
    return set_error(E2D_ERR_INVALID_ARG, "invalid parameters");
  if (!(dt > 0.0) || !std::isfinite(dt)) return set_error(E2D_ERR_INVALID_ARG, "dt must be a positive finite number");
  const size_t isize = (size_t)p->nx + 4, jsize = (size_t)p->ny + 4, es = (size_t)p->precision;
  if (pitch_elems < isize) return set_error(E2D_ERR_INVALID_ARG, "pitch_elems must be at least nx + 4");
  if (pitch_elems > (size_t)INT_MAX) return set_error(E2D_ERR_INVALID_ARG, "pitch_elems must not exceed INT_MAX");
  // The two states must not share any byte: 4 planes of jsize rows each.
  const size_t state_bytes = 4 * jsize * pitch_elems * es;
  const uintptr_t a_in = reinterpret_cast<uintptr_t>(u_in), a_out = reinterpret_cast<uintptr_t>(u_out);
  if (a_in < a_out + state_bytes && a_out < a_in + state_bytes)
    return set_error(E2D_ERR_INVALID_ARG, "u_in and u_out overlap");
  const size_t work_pitch = (isize + 31) / 32 * 32;
  const size_t need = kCtlBytes + 3 * 4 * work_pitch * jsize * es;
  if (need > (size_t)E2D_NOALLOC_SCRATCH_BYTES)
    return set_error(E2D_ERR_INVALID_ARG, "grid too large for the no-allocation step: its work arrays need " +
                                              std::to_string(need) + " bytes, the static scratch holds " +
                                              std::to_string((size_t)E2D_NOALLOC_SCRATCH_BYTES));
  void* scratch = nullptr;
  if (int rc = scratch_address(&scratch)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* sc = static_cast<unsigned char*>(scratch);
  return p->precision == 8 ? step<double>(*p, u_in, u_out, pitch_elems, dt, sc, work_pitch, s, health)
                           : step<float>(*p, u_in, u_out, pitch_elems, dt, sc, work_pitch, s, health);
}
