// abi.cu -- the extern "C" boundary (include/euler2d_gb300.h): run handles,
// device memory, the per-call procedures of the HydroRun driver, and the
// graph-captured multi-step advance.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/euler2d_gb300.h"
#include "hydro_params.h"
#include "launch.h"
#include "nvtx_ranges.h"

using namespace e2d;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(E2D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define E2D_CK(call)                                   \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

}  // namespace

int e2d::set_error(int code, const std::string& msg) { return fail(code, msg); }

struct e2d_run {
  e2d_params p;
  int device = 0;
  int es = 8;  // element size
  Hydro<double> hd;
  Hydro<float> hf;
  int isize = 0, jsize = 0;
  size_t pitch = 0, plane = 0;  // elements
  void* u = nullptr;
  void* u2 = nullptr;
  void* work[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // implementationVersion 0: primitive variables beside u (qprim[0]) and u2
  // (qprim[1]), written by each fused step of e2d_advance / e2d_time_steps for
  // the next one; refreshed from u and u2 at the start of every such call.
  // Null when they could not be allocated (the step then converts its box).
  void* qprim[2] = {nullptr, nullptr};
  // q_valid[b]: qprim[b] holds the primitives of the interior (and, unless
  // the last writer was a per-call step, the ghosts) of buffer b.
  bool q_valid[2] = {false, false};
  Ctl* ctl = nullptr;
  void* dt_log = nullptr;  // device
  int dt_log_cap = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timed = false;
  FusedPlan* plan = nullptr;
  int cur_slot = 0;
  std::map<std::tuple<int, int, int, int>, cudaGraphExec_t> graphs;
  bool use_graphs = true;
  // folded[b]: the running CFL maximum (slot cur_slot) already includes the
  // current state of buffer b (0 = u, 1 = u2), so compute_dt on it needs no sweep.
  bool folded[2] = {false, false};
  // asynchronous output: a device snapshot of one state, copied to the host
  // on its own stream while later steps run on `stream`
  void* snapshot = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_copied = nullptr;
  bool download_pending = false;
  // pinned host word for compute_dt's read-back of the running maximum
  double* h_inv = nullptr;
};

namespace {

template <typename Real> const Hydro<Real>& hydro(const e2d_run* r);
template <> const Hydro<double>& hydro<double>(const e2d_run* r) { return r->hd; }
template <> const Hydro<float>& hydro<float>(const e2d_run* r) { return r->hf; }

template <typename Real>
Field<Real> field(const e2d_run* r, void* ptr) {
  return Field<Real>{static_cast<Real*>(ptr), (int)r->pitch, (long long)r->plane};
}

size_t state_dev_bytes(const e2d_run* r) { return 4 * r->plane * (size_t)r->es; }

int check_run(const e2d_run* r) {
  if (!r) return fail(E2D_ERR_INVALID_ARG, "null run handle");
  return E2D_OK;
}

int use_device(const e2d_run* r) {
  cudaError_t e = cudaSetDevice(r->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return E2D_OK;
}

// Launch the device work of one godunov step nStep (reading in, writing out).
// from_slot: dt comes from the running maximum; otherwise dt_value.
template <typename Real>
void enqueue_step(e2d_run* r, int nStep, Real dt_value, bool from_slot, int rd, int wr, int log_index,
                  bool boundaries_done, bool use_q = false) {
  const Hydro<Real>& h = hydro<Real>(r);
  const bool even = (nStep % 2) == 0;
  Field<Real> in = field<Real>(r, even ? r->u : r->u2);
  Field<Real> out = field<Real>(r, even ? r->u2 : r->u);
  StepDt<Real> sd;
  sd.dt_value = dt_value;
  sd.dt_ptr = nullptr;
  sd.from_slot = from_slot ? 1 : 0;
  sd.rd_slot = rd;
  sd.wr_slot = wr;
  sd.dt_log = from_slot ? static_cast<Real*>(r->dt_log) : nullptr;
  sd.log_index = log_index;
  cudaStream_t s = r->stream;
  if (!boundaries_done) {
    NvtxRange rg(NVTX_BOUNDARIES);
    launch_boundaries<Real>(h, in, s);
  }
  switch (r->p.implementation_version) {
    case 0: {
      // In the advance path the ghost cells of `out` are written by the
      // update epilogue (what make_boundaries does at the next step), and
      // with use_q the primitives of `out` beside it.
      const Field<Real> qout = field<Real>(r, r->qprim[even ? 1 : 0]);
      launch_fused<Real>(h, r->plan, even ? 0 : 1, in, out, sd, r->ctl, from_slot, s, use_q ? &qout : nullptr);
      break;
    }
    case 1: {
      // the reference's stages: primitives, then the traces and fluxes of
      // computeAndStoreFluxes, then (here fused with them) updateHydro
      Field<Real> q = field<Real>(r, r->work[0]);
      {
        NvtxRange rg(NVTX_PRIMITIVES);
        launch_prim<Real>(h, in, q, s);
      }
      NvtxRange rg(NVTX_FLUXES);
      launch_trace_v1<Real>(h, q, sd, r->ctl, field<Real>(r, r->work[1]), field<Real>(r, r->work[2]),
                            field<Real>(r, r->work[3]), field<Real>(r, r->work[4]), s);
      launch_flux_update_v1<Real>(h, in, field<Real>(r, r->work[1]), field<Real>(r, r->work[2]),
                                  field<Real>(r, r->work[3]), field<Real>(r, r->work[4]), out, sd, r->ctl, s);
      break;
    }
    default: {
      Field<Real> q = field<Real>(r, r->work[0]);
      {
        NvtxRange rg(NVTX_PRIMITIVES);
        launch_prim<Real>(h, in, q, s);
      }
      {
        NvtxRange rg(NVTX_FLUXES);
        launch_fluxes_v2<Real>(h, q, sd, r->ctl, field<Real>(r, r->work[1]), field<Real>(r, r->work[2]), s);
      }
      NvtxRange rg(NVTX_UPDATE);
      launch_update_v2<Real>(h, in, field<Real>(r, r->work[1]), field<Real>(r, r->work[2]), out, sd, r->ctl, s);
      break;
    }
  }
}

// The device work of e2d_advance: compute_dt on the state of nStep0, ghost
// fill, then nsteps steps with device-resident dt.
// implementationVersion 0 with primitive arrays: the primitives of the state
// of nStep0 (after its ghost fill) and of the other buffer (whose corners no
// step writes) are formed once; from then on each step writes those of its
// output.  Returns whether the steps may read them.
template <typename Real>
bool refresh_prims(e2d_run* r, int nStep0) {
  if (r->p.implementation_version != 0 || !r->qprim[0]) return false;
  const Hydro<Real>& h = hydro<Real>(r);
  const int b = nStep0 % 2;
  launch_prim<Real>(h, field<Real>(r, b ? r->u2 : r->u), field<Real>(r, r->qprim[b]), r->stream);
  launch_prim<Real>(h, field<Real>(r, b ? r->u : r->u2), field<Real>(r, r->qprim[b ^ 1]), r->stream);
  return true;
}

template <typename Real>
void enqueue_advance(e2d_run* r, int nStep0, int nsteps, int slot0, bool seed) {
  const Hydro<Real>& h = hydro<Real>(r);
  Field<Real> cur = field<Real>(r, (nStep0 % 2 == 0) ? r->u : r->u2);
  if (seed) launch_dt_reduce<Real>(h, cur, r->ctl, slot0, r->stream);
  launch_boundaries<Real>(h, cur, r->stream);
  const bool use_q = refresh_prims<Real>(r, nStep0);
  for (int k = 0; k < nsteps; ++k) {
    const int rd = slot0 ^ (k & 1);
    // implementationVersion 0 fills the ghosts of its output itself; the
    // stored variants run make_boundaries at the start of every step as the
    // reference does (serial_ref/m_run.f90:224).
    const bool bdone = (r->p.implementation_version == 0) || k == 0;
    enqueue_step<Real>(r, nStep0 + k, Real(0), true, rd, rd ^ 1, k, bdone, use_q);
  }
}

// The per-call step of implementationVersion 0 with primitive arrays: after
// the ghost fill of the input (enqueue_step), its primitives are made current
// -- their ghosts filled by the same rules, or both buffers' primitives formed
// when they are not valid -- and the step writes the output's interior ones.
template <typename Real>
void enqueue_percall_q(e2d_run* r, int nStep, Real dt) {
  const Hydro<Real>& h = hydro<Real>(r);
  const int b = nStep % 2;
  {
    NvtxRange rg(NVTX_BOUNDARIES);
    if (r->q_valid[b])
      launch_boundaries_pair<Real>(h, field<Real>(r, b ? r->u2 : r->u), field<Real>(r, r->qprim[b]), r->stream);
    else
      launch_boundaries<Real>(h, field<Real>(r, b ? r->u2 : r->u), r->stream);
  }
  if (!r->q_valid[b]) {
    NvtxRange rg(NVTX_PRIMITIVES);
    refresh_prims<Real>(r, nStep);
  }
  enqueue_step<Real>(r, nStep, dt, false, -1, r->cur_slot, 0, true, true);
  r->q_valid[0] = r->q_valid[1] = true;
}

// The device address of `bytes` of host memory the GPU can read and write
// directly (pinned and mapped: cudaMallocHost / cudaHostAlloc /
// e2d_host_alloc, torch's pin_memory), or null when the memory is pageable
// or the pinned mapping does not cover the last byte as well.
const void* mapped_host(const void* host, size_t bytes) {
  cudaPointerAttributes a, b;
  const char* last = static_cast<const char*>(host) + (bytes - 1);
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess || cudaPointerGetAttributes(&b, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer)
    return nullptr;
  if (static_cast<const char*>(b.devicePointer) != static_cast<const char*>(a.devicePointer) + (bytes - 1))
    return nullptr;
  return a.devicePointer;
}

template <typename Real>
int finish_dt(e2d_run* r, void* dt_out) {
  Real inv_local;
  Real* hp = r->h_inv ? reinterpret_cast<Real*>(r->h_inv) : &inv_local;  // pinned: a direct copy
  E2D_CK(cudaMemcpyAsync(hp, inv_slot<Real>(r->ctl, r->cur_slot), sizeof(Real), cudaMemcpyDeviceToHost,
                         r->stream));
  E2D_CK(cudaStreamSynchronize(r->stream));
  const Real inv = *hp;
  const Real dt = hydro<Real>(r).cfl / inv;
  *static_cast<Real*>(dt_out) = dt;
  return E2D_OK;
}

int ensure_dt_log(e2d_run* r, int nsteps) {
  if (nsteps <= r->dt_log_cap) return E2D_OK;
  E2D_CK(cudaStreamSynchronize(r->stream));
  for (auto& kv : r->graphs) cudaGraphExecDestroy(kv.second);  // they captured the old pointer
  r->graphs.clear();
  cudaFree(r->dt_log);
  r->dt_log = nullptr;
  r->dt_log_cap = 0;
  if (cudaMalloc(&r->dt_log, (size_t)nsteps * r->es) != cudaSuccess) {
    cudaGetLastError();
    return fail(E2D_ERR_OOM, "cudaMalloc of the dt log failed");
  }
  r->dt_log_cap = nsteps;
  return E2D_OK;
}

}  // namespace

extern "C" {

const char* e2d_last_error(void) { return g_err.c_str(); }

int e2d_default_params(e2d_params* p) {
  if (!p) return fail(E2D_ERR_INVALID_ARG, "null params");
  std::memset(p, 0, sizeof(*p));
  p->nx = 1024;
  p->ny = 1024;
  p->gamma0 = 1.666;
  p->cfl = 0.8;
  p->smallr = 1e-7;
  p->smallc = 1e-7;
  p->niter_riemann = 10;
  p->iorder = 2;
  p->slope_type = 2;
  p->boundary_type_xmin = p->boundary_type_xmax = p->boundary_type_ymin = p->boundary_type_ymax = 1;
  p->implementation_version = 0;
  p->riemann_solver = E2D_RIEMANN_APPROX;
  p->precision = 8;
  return E2D_OK;
}

int e2d_arithmetic(int* mode) {
  if (!mode) return fail(E2D_ERR_INVALID_ARG, "null argument");
#if defined(E2D_FMA) && E2D_FMA
  *mode = E2D_ARITH_FMA;
#else
  *mode = E2D_ARITH_EXACT;
#endif
  return E2D_OK;
}

int e2d_create(const e2d_params* p, e2d_run** out) {
  if (!p || !out) return fail(E2D_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (p->nx < 2 || p->ny < 2 || p->nx > (1 << 20) || p->ny > (1 << 20))
    return fail(E2D_ERR_INVALID_ARG, "nx and ny must be in [2, 2^20]");
  if (p->implementation_version < 0 || p->implementation_version > 2)
    return fail(E2D_ERR_INVALID_ARG, "The implementation version parameter should 0, 1 or 2");
  if (p->riemann_solver != E2D_RIEMANN_APPROX && p->riemann_solver != E2D_RIEMANN_HLLC)
    return fail(E2D_ERR_INVALID_ARG, "riemann_solver must be 0 (approx) or 2 (hllc)");
  if (p->precision != 4 && p->precision != 8) return fail(E2D_ERR_INVALID_ARG, "precision must be 4 or 8");
  if (!(p->gamma0 > 1.0) || !(p->cfl > 0.0) || !(p->smallr > 0.0) || !(p->smallc > 0.0))
    return fail(E2D_ERR_INVALID_ARG, "gamma0 > 1, cfl > 0, smallr > 0 and smallc > 0 are required");
  if (p->niter_riemann < 0) return fail(E2D_ERR_INVALID_ARG, "niter_riemann must be >= 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(E2D_ERR_NO_DEVICE, "no CUDA device");
  }
  e2d_run* r = new e2d_run;
  r->p = *p;
  cudaGetDevice(&r->device);
  r->es = p->precision;
  r->hd = make_hydro<double>(*p);
  r->hf = make_hydro<float>(*p);
  r->isize = p->nx + 4;
  r->jsize = p->ny + 4;
  r->pitch = ((size_t)r->isize + 31) / 32 * 32;
  r->plane = r->pitch * (size_t)r->jsize;
  if (const char* g = std::getenv("E2D_NO_GRAPH")) r->use_graphs = !(g[0] == '1');
  auto cleanup = [&](int code, const std::string& msg) {
    e2d_destroy(r);
    return fail(code, msg);
  };
  const size_t sb = state_dev_bytes(r);
  if (cudaMalloc(&r->u, sb) != cudaSuccess || cudaMalloc(&r->u2, sb) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(E2D_ERR_OOM, "cudaMalloc of the state arrays failed");
  }
  const int nwork = p->implementation_version == 1 ? 5 : p->implementation_version == 2 ? 3 : 0;
  for (int k = 0; k < nwork; ++k)
    if (cudaMalloc(&r->work[k], sb) != cudaSuccess) {
      cudaGetLastError();
      return cleanup(E2D_ERR_OOM, "cudaMalloc of the work arrays failed");
    }
  if (cudaMalloc(&r->ctl, sizeof(Ctl)) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(E2D_ERR_OOM, "cudaMalloc of the control block failed");
  }
  if (cudaStreamCreateWithFlags(&r->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&r->ev0) != cudaSuccess || cudaEventCreate(&r->ev1) != cudaSuccess)
    return cleanup(E2D_ERR_CUDA, "stream/event creation failed");
  r->stream = r->own_stream;
  if (cudaMallocHost(&r->h_inv, sizeof(double)) != cudaSuccess) {  // optional: a pageable copy otherwise
    cudaGetLastError();
    r->h_inv = nullptr;
  }
  cudaMemsetAsync(r->u, 0, sb, r->stream);
  cudaMemsetAsync(r->u2, 0, sb, r->stream);
  for (int k = 0; k < nwork; ++k) cudaMemsetAsync(r->work[k], 0, sb, r->stream);
  cudaMemsetAsync(r->ctl, 0, sizeof(Ctl), r->stream);
  if (p->implementation_version == 0) {
    // E2D_KEEP_PRIMS=0: no primitive arrays (every step converts its box;
    // primitives never leave shared memory)
    const char* kp = std::getenv("E2D_KEEP_PRIMS");
    const bool keep = !(kp && kp[0] == '0');
    if (keep && (cudaMalloc(&r->qprim[0], sb) != cudaSuccess || cudaMalloc(&r->qprim[1], sb) != cudaSuccess)) {
      cudaGetLastError();
      cudaFree(r->qprim[0]);
      r->qprim[0] = r->qprim[1] = nullptr;
    }
    if (p->precision == 8) {
      const Field<double> q0 = field<double>(r, r->qprim[0]), q1 = field<double>(r, r->qprim[1]);
      r->plan = fused_plan_create<double>(r->hd, field<double>(r, r->u), field<double>(r, r->u2),
                                          r->qprim[0] ? &q0 : nullptr, r->qprim[0] ? &q1 : nullptr);
    } else {
      const Field<float> q0 = field<float>(r, r->qprim[0]), q1 = field<float>(r, r->qprim[1]);
      r->plan = fused_plan_create<float>(r->hf, field<float>(r, r->u), field<float>(r, r->u2),
                                         r->qprim[0] ? &q0 : nullptr, r->qprim[0] ? &q1 : nullptr);
    }
    if (!r->plan) return cleanup(E2D_ERR_CUDA, "TMA descriptor / kernel attribute setup failed");
  }
  cudaError_t e = cudaStreamSynchronize(r->stream);
  if (e != cudaSuccess) return cleanup(E2D_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e));
  *out = r;
  return E2D_OK;
}

int e2d_destroy(e2d_run* r) {
  if (!r) return E2D_OK;
  cudaSetDevice(r->device);
  if (r->stream) cudaStreamSynchronize(r->stream);
  for (auto& kv : r->graphs) cudaGraphExecDestroy(kv.second);
  r->graphs.clear();
  if (r->plan) fused_plan_destroy(r->plan);
  cudaFree(r->u);
  cudaFree(r->u2);
  for (void* w : r->work) cudaFree(w);
  for (void* q : r->qprim) cudaFree(q);
  cudaFree(r->ctl);
  cudaFree(r->dt_log);
  if (r->ev0) cudaEventDestroy(r->ev0);
  if (r->ev1) cudaEventDestroy(r->ev1);
  if (r->copy_stream) {
    cudaStreamSynchronize(r->copy_stream);
    cudaStreamDestroy(r->copy_stream);
  }
  if (r->ev_snap) cudaEventDestroy(r->ev_snap);
  if (r->ev_copied) cudaEventDestroy(r->ev_copied);
  cudaFree(r->snapshot);
  if (r->h_inv) cudaFreeHost(r->h_inv);
  if (r->own_stream) cudaStreamDestroy(r->own_stream);
  delete r;
  return E2D_OK;
}

int e2d_get_sizes(const e2d_run* r, int* isize, int* jsize, size_t* state_bytes) {
  if (int rc = check_run(r)) return rc;
  if (isize) *isize = r->isize;
  if (jsize) *jsize = r->jsize;
  if (state_bytes) *state_bytes = (size_t)r->isize * r->jsize * 4 * r->es;
  return E2D_OK;
}

int e2d_set_stream(e2d_run* r, void* stream) {
  if (int rc = check_run(r)) return rc;
  cudaStreamSynchronize(r->stream);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (s != r->stream) {
    for (auto& kv : r->graphs) cudaGraphExecDestroy(kv.second);
    r->graphs.clear();
  }
  r->stream = s ? s : r->own_stream;
  return E2D_OK;
}

int e2d_synchronize(e2d_run* r) {
  if (int rc = check_run(r)) return rc;
  E2D_CK(cudaStreamSynchronize(r->stream));
  return E2D_OK;
}

int e2d_init_diagonal(e2d_run* r, double offset, double rho_hi, double p_hi, double rho_lo, double p_lo) {
  if (int rc = check_run(r)) return rc;
  if (int rc = use_device(r)) return rc;
  r->folded[0] = false;
  r->q_valid[0] = false;
  if (r->es == 8)
    launch_init_diagonal<double>(r->hd, field<double>(r, r->u), offset, rho_hi, p_hi, rho_lo, p_lo, r->stream);
  else
    launch_init_diagonal<float>(r->hf, field<float>(r, r->u), offset, rho_hi, p_hi, rho_lo, p_lo, r->stream);
  E2D_CK(cudaGetLastError());
  E2D_CK(cudaStreamSynchronize(r->stream));
  return E2D_OK;
}

int e2d_init_implode(e2d_run* r) {
  // data(ID)=1.0, data(IP)=1.0/(gamma0-1.0) where tmp > 0.5; else 0.125 and
  // 0.14/(gamma0-1.0) with 0.14 a default (single precision) real.
  return e2d_init_diagonal(r, 0.5, 1.0, 1.0, 0.125, (double)0.14f);
}

int e2d_upload_state(e2d_run* r, int which, const void* host) {
  if (int rc = check_run(r)) return rc;
  if (!host || (which != 0 && which != 1)) return fail(E2D_ERR_INVALID_ARG, "bad upload arguments");
  if (int rc = use_device(r)) return rc;
  const size_t w = (size_t)r->isize * r->es;
  r->folded[which] = false;
  r->q_valid[which] = false;
  if (const void* hd = mapped_host(host, w * 4 * r->jsize)) {  // pinned: rows repitched at the link's rate
    launch_repitch(hd, (size_t)r->isize, which ? r->u2 : r->u, r->pitch, r->isize, 4 * r->jsize, r->es, r->stream);
    E2D_CK(cudaGetLastError());
  } else {
    E2D_CK(cudaMemcpy2DAsync(which ? r->u2 : r->u, r->pitch * r->es, host, w, w, (size_t)4 * r->jsize,
                             cudaMemcpyHostToDevice, r->stream));
  }
  E2D_CK(cudaStreamSynchronize(r->stream));
  return E2D_OK;
}

int e2d_download_state(e2d_run* r, int which, void* host) {
  if (int rc = check_run(r)) return rc;
  if (!host || (which != 0 && which != 1)) return fail(E2D_ERR_INVALID_ARG, "bad download arguments");
  if (int rc = use_device(r)) return rc;
  const size_t w = (size_t)r->isize * r->es;
  if (void* hd = const_cast<void*>(mapped_host(host, w * 4 * r->jsize))) {
    launch_repitch(which ? r->u2 : r->u, r->pitch, hd, (size_t)r->isize, r->isize, 4 * r->jsize, r->es, r->stream);
    E2D_CK(cudaGetLastError());
  } else {
    E2D_CK(cudaMemcpy2DAsync(host, w, which ? r->u2 : r->u, r->pitch * r->es, w, (size_t)4 * r->jsize,
                             cudaMemcpyDeviceToHost, r->stream));
  }
  E2D_CK(cudaStreamSynchronize(r->stream));
  return E2D_OK;
}

int e2d_begin_download(e2d_run* r, int which, void* host) {
  if (int rc = check_run(r)) return rc;
  if (!host || (which != 0 && which != 1)) return fail(E2D_ERR_INVALID_ARG, "bad download arguments");
  if (int rc = use_device(r)) return rc;
  if (!r->snapshot) {
    if (cudaMalloc(&r->snapshot, state_dev_bytes(r)) != cudaSuccess) {
      cudaGetLastError();
      return fail(E2D_ERR_OOM, "cudaMalloc of the output snapshot failed");
    }
    E2D_CK(cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking));
    E2D_CK(cudaEventCreateWithFlags(&r->ev_snap, cudaEventDisableTiming));
    E2D_CK(cudaEventCreateWithFlags(&r->ev_copied, cudaEventDisableTiming));
  }
  if (r->download_pending) E2D_CK(cudaEventSynchronize(r->ev_copied));  // the snapshot is reused
  // snapshot in stream order (device to device), then to the host on the copy stream
  E2D_CK(cudaMemcpyAsync(r->snapshot, which ? r->u2 : r->u, state_dev_bytes(r), cudaMemcpyDeviceToDevice,
                         r->stream));
  E2D_CK(cudaEventRecord(r->ev_snap, r->stream));
  E2D_CK(cudaStreamWaitEvent(r->copy_stream, r->ev_snap, 0));
  const size_t w = (size_t)r->isize * r->es;
  E2D_CK(cudaMemcpy2DAsync(host, w, r->snapshot, r->pitch * r->es, w, (size_t)4 * r->jsize, cudaMemcpyDeviceToHost,
                           r->copy_stream));
  E2D_CK(cudaEventRecord(r->ev_copied, r->copy_stream));
  r->download_pending = true;
  return E2D_OK;
}

int e2d_wait_download(e2d_run* r) {
  if (int rc = check_run(r)) return rc;
  if (!r->download_pending) return E2D_OK;
  if (int rc = use_device(r)) return rc;
  E2D_CK(cudaEventSynchronize(r->ev_copied));
  r->download_pending = false;
  return E2D_OK;
}

int e2d_host_alloc(size_t bytes, void** ptr) {
  if (!ptr || bytes == 0) return fail(E2D_ERR_INVALID_ARG, "bad host allocation arguments");
  *ptr = nullptr;
  if (cudaMallocHost(ptr, bytes) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return fail(E2D_ERR_OOM, "cudaMallocHost failed");
  }
  return E2D_OK;
}

int e2d_host_free(void* ptr) {
  if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
    cudaGetLastError();
    return fail(E2D_ERR_CUDA, "cudaFreeHost failed");
  }
  return E2D_OK;
}

int e2d_compute_dt(e2d_run* r, int useU, void* dt) {
  NvtxRange rg(NVTX_COMPUTE_DT);
  if (int rc = check_run(r)) return rc;
  if (!dt || (useU != 0 && useU != 1)) return fail(E2D_ERR_INVALID_ARG, "bad compute_dt arguments");
  if (int rc = use_device(r)) return rc;
  // The max is idempotent: when the step that wrote this state already folded
  // its CFL maximum into the running maximum, a second sweep cannot change it.
  if (!r->folded[useU]) {
    if (r->es == 8)
      launch_dt_reduce<double>(r->hd, field<double>(r, useU ? r->u2 : r->u), r->ctl, r->cur_slot, r->stream);
    else
      launch_dt_reduce<float>(r->hf, field<float>(r, useU ? r->u2 : r->u), r->ctl, r->cur_slot, r->stream);
    E2D_CK(cudaGetLastError());
    r->folded[useU] = true;
  }
  return r->es == 8 ? finish_dt<double>(r, dt) : finish_dt<float>(r, dt);
}

int e2d_make_boundaries(e2d_run* r, int which) {
  NvtxRange rg(NVTX_BOUNDARIES);
  if (int rc = check_run(r)) return rc;
  if (which != 0 && which != 1) return fail(E2D_ERR_INVALID_ARG, "which must be 0 (u) or 1 (u2)");
  if (int rc = use_device(r)) return rc;
  // the primitives' ghosts follow in the same launch (a flipped momentum is a flipped velocity)
  if (r->es == 8) {
    const Field<double> w = field<double>(r, r->q_valid[which] ? r->qprim[which] : nullptr);
    launch_boundaries_pair<double>(r->hd, field<double>(r, which ? r->u2 : r->u), w, r->stream);
  } else {
    const Field<float> w = field<float>(r, r->q_valid[which] ? r->qprim[which] : nullptr);
    launch_boundaries_pair<float>(r->hf, field<float>(r, which ? r->u2 : r->u), w, r->stream);
  }
  E2D_CK(cudaGetLastError());
  return E2D_OK;
}


int e2d_godunov_unsplit(e2d_run* r, int nStep, double dt) {
  NvtxRange rg(NVTX_GODUNOV);
  if (int rc = check_run(r)) return rc;
  if (nStep < 0) return fail(E2D_ERR_INVALID_ARG, "nStep must be >= 0");
  if (int rc = use_device(r)) return rc;
  // dt comes from the caller; the update epilogue folds the CFL maximum of
  // the new state into the running maximum, which the next compute_dt reads.
  if (r->p.implementation_version == 0 && r->qprim[0]) {
    if (r->es == 8) enqueue_percall_q<double>(r, nStep, dt);
    else enqueue_percall_q<float>(r, nStep, (float)dt);
  } else if (r->es == 8) {
    enqueue_step<double>(r, nStep, dt, false, -1, r->cur_slot, 0, false);
  } else {
    enqueue_step<float>(r, nStep, (float)dt, false, -1, r->cur_slot, 0, false);
  }
  E2D_CK(cudaGetLastError());
  r->folded[(nStep % 2 == 0) ? 1 : 0] = true;
  return E2D_OK;
}

int e2d_advance(e2d_run* r, int nStep0, int nsteps, void* dt_log) {
  NvtxRange rg(NVTX_GODUNOV);  // nsteps steps: compute_dt and godunov_unsplit each, one graph
  if (int rc = check_run(r)) return rc;
  if (nStep0 < 0 || nsteps < 0) return fail(E2D_ERR_INVALID_ARG, "nStep0 and nsteps must be >= 0");
  if (int rc = use_device(r)) return rc;
  if (nsteps == 0) return E2D_OK;
  if (int rc = ensure_dt_log(r, nsteps)) return rc;
  const int slot0 = r->cur_slot;
  const int b0 = nStep0 % 2;
  const bool seed = !r->folded[b0];
  auto enqueue = [&]() {
    if (r->es == 8) enqueue_advance<double>(r, nStep0, nsteps, slot0, seed);
    else enqueue_advance<float>(r, nStep0, nsteps, slot0, seed);
  };
  cudaGraphExec_t exec = nullptr;
  if (r->use_graphs && r->stream != nullptr) {
    const auto key = std::make_tuple(b0, slot0, nsteps, seed ? 1 : 0);
    auto it = r->graphs.find(key);
    if (it != r->graphs.end()) {
      exec = it->second;
    } else {
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        enqueue();
        if (cudaStreamEndCapture(r->stream, &graph) == cudaSuccess && graph) {
          if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
          cudaGraphDestroy(graph);
        }
      }
      cudaGetLastError();
      if (exec) {
        cudaGraphUpload(exec, r->stream);
        r->graphs[key] = exec;
      }
    }
  }
  // Capture and instantiation happen before ev0, so the events bracket device work only.
  E2D_CK(cudaEventRecord(r->ev0, r->stream));
  if (exec) {
    E2D_CK(cudaGraphLaunch(exec, r->stream));
  } else {
    enqueue();
    E2D_CK(cudaGetLastError());
  }
  E2D_CK(cudaEventRecord(r->ev1, r->stream));
  r->timed = true;
  r->cur_slot = slot0 ^ (nsteps & 1);
  r->folded[0] = r->folded[1] = true;
  r->q_valid[0] = r->q_valid[1] = r->qprim[0] != nullptr && r->p.implementation_version == 0;
  if (dt_log) {
    E2D_CK(cudaMemcpyAsync(dt_log, r->dt_log, (size_t)nsteps * r->es, cudaMemcpyDeviceToHost, r->stream));
    E2D_CK(cudaStreamSynchronize(r->stream));
    unsigned health = 0;
    E2D_CK(cudaMemcpy(&health, &r->ctl->health, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (health & E2D_HEALTH_DT_NONFINITE) return fail(E2D_ERR_NUMERICS, "dt became non-finite");
  }
  return E2D_OK;
}

int e2d_time_steps(e2d_run* r, int nStep0, int nsteps, float* ms) {
  if (int rc = check_run(r)) return rc;
  if (nStep0 < 0 || nsteps <= 0 || !ms) return fail(E2D_ERR_INVALID_ARG, "bad time_steps arguments");
  if (int rc = use_device(r)) return rc;
  if (int rc = ensure_dt_log(r, nsteps)) return rc;
  std::vector<cudaEvent_t> ev(nsteps + 1, nullptr);
  for (auto& e : ev) E2D_CK(cudaEventCreate(&e));
  const int slot0 = r->cur_slot;
  const bool seed = !r->folded[nStep0 % 2];
  const bool v0 = r->p.implementation_version == 0;
  bool use_q = false;
  if (r->es == 8) {
    Field<double> cur = field<double>(r, (nStep0 % 2 == 0) ? r->u : r->u2);
    if (seed) launch_dt_reduce<double>(r->hd, cur, r->ctl, slot0, r->stream);
    launch_boundaries<double>(r->hd, cur, r->stream);
    use_q = refresh_prims<double>(r, nStep0);
  } else {
    Field<float> cur = field<float>(r, (nStep0 % 2 == 0) ? r->u : r->u2);
    if (seed) launch_dt_reduce<float>(r->hf, cur, r->ctl, slot0, r->stream);
    launch_boundaries<float>(r->hf, cur, r->stream);
    use_q = refresh_prims<float>(r, nStep0);
  }
  cudaEventRecord(ev[0], r->stream);
  for (int k = 0; k < nsteps; ++k) {
    const int rd = slot0 ^ (k & 1);
    if (r->es == 8) enqueue_step<double>(r, nStep0 + k, 0.0, true, rd, rd ^ 1, k, v0 || k == 0, use_q);
    else enqueue_step<float>(r, nStep0 + k, 0.0f, true, rd, rd ^ 1, k, v0 || k == 0, use_q);
    cudaEventRecord(ev[k + 1], r->stream);
  }
  cudaError_t e = cudaStreamSynchronize(r->stream);
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) e = cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(e, "e2d_time_steps");
  r->cur_slot = slot0 ^ (nsteps & 1);
  r->folded[0] = r->folded[1] = true;
  r->q_valid[0] = r->q_valid[1] = use_q;
  return E2D_OK;
}

int e2d_last_advance_ms(e2d_run* r, float* ms) {
  if (int rc = check_run(r)) return rc;
  if (!ms) return fail(E2D_ERR_INVALID_ARG, "null ms");
  if (!r->timed) return fail(E2D_ERR_INVALID_ARG, "no advance has been timed");
  E2D_CK(cudaEventSynchronize(r->ev1));
  E2D_CK(cudaEventElapsedTime(ms, r->ev0, r->ev1));
  return E2D_OK;
}

int e2d_get_invdt(e2d_run* r, double* invdt) {
  if (int rc = check_run(r)) return rc;
  if (!invdt) return fail(E2D_ERR_INVALID_ARG, "null invdt");
  E2D_CK(cudaStreamSynchronize(r->stream));
  if (r->es == 8) {
    E2D_CK(cudaMemcpy(invdt, inv_slot<double>(r->ctl, r->cur_slot), 8, cudaMemcpyDeviceToHost));
  } else {
    float f;
    E2D_CK(cudaMemcpy(&f, inv_slot<float>(r->ctl, r->cur_slot), 4, cudaMemcpyDeviceToHost));
    *invdt = f;
  }
  return E2D_OK;
}

int e2d_get_health(e2d_run* r, unsigned* flags) {
  if (int rc = check_run(r)) return rc;
  if (!flags) return fail(E2D_ERR_INVALID_ARG, "null flags");
  E2D_CK(cudaStreamSynchronize(r->stream));
  E2D_CK(cudaMemcpy(flags, &r->ctl->health, sizeof(unsigned), cudaMemcpyDeviceToHost));
  E2D_CK(cudaMemset(&r->ctl->health, 0, sizeof(unsigned)));
  return E2D_OK;
}

int e2d_device_state(e2d_run* r, int which, void** dptr, size_t* pitch_elems, size_t* plane_elems) {
  if (int rc = check_run(r)) return rc;
  if (which != 0 && which != 1) return fail(E2D_ERR_INVALID_ARG, "which must be 0 or 1");
  if (dptr) *dptr = which ? r->u2 : r->u;
  r->folded[0] = r->folded[1] = false;  // the caller may write the state directly
  r->q_valid[0] = r->q_valid[1] = false;
  if (pitch_elems) *pitch_elems = r->pitch;
  if (plane_elems) *plane_elems = r->plane;
  return E2D_OK;
}

}  // extern "C"
