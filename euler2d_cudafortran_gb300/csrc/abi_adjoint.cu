// abi_adjoint.cu -- the discrete adjoint of the FP64 HLLC step behind the C ABI
// (e2d_adjoint_*): gradient of J = sum rho^2 w(x, y) of the final state with
// respect to the initial density field.
//
// Forward: the N steps of the run (device-resident dt, as e2d_advance), with
// a checkpoint of the state every K = ceil(sqrt(N)) steps, the states of the
// last segment kept whole, and logs of dt_n and of the running CFL maximum
// inv_n.  Reverse: for each segment, last first, the reverse step kernel runs
// from the last state of the segment back to its first, while the previous
// segment's states are recomputed from its checkpoint with the logged dt (bit
// for bit the forward states) on a second stream into a second set of
// segment buffers.  When all N states and their tapes fit in half the free
// device memory, the forward sweep keeps them all instead and the reverse
// sweep recomputes nothing.  The whole gradient is one captured graph.  dt_mode 0 keeps every dt
// frozen; dt_mode 1 also differentiates dt_n = cfl / inv_n through the
// running maximum: the adjoint of inv_n goes to the cell whose compute_dt
// term set that maximum, in the state where it was first reached.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/euler2d_gb300.h"
#include "adjoint_launch.h"
#include "hydro_params.h"

using namespace e2d;

struct e2d_adjoint {
  e2d_params p;
  Hydro<double> h;
  int device = 0;
  size_t pitch = 0, plane = 0, state_elems = 0;
  double* pool = nullptr;  // states: 2 ping-pong, the checkpoints, 2 sets of K segment states
  // the forward values of each segment state (TapeOut: primitives, slopes,
  // sources, and the recorded HLLC solve of every face; kTapePlanes planes
  // each), written by the forward sweeps and read by the reverse steps; null
  // when they could not be allocated (the reverse recomputes them)
  double* tapes = nullptr;
  bool use_tape = true;  // E2D_NO_TAPE=1: the reverse recomputes (for comparisons)
  // primitives beside the two forward ping-pong states (the fast forward step
  // of e2d_advance: the step reads its input's and writes its output's);
  // null when they could not be allocated
  double* qping = nullptr;
  StateMap qmaps[2];
  StateMap imaps[2];  // the interior tiles of the ping-pong states (the fast step's L2 prefetch)
  std::map<std::tuple<int, double, double, double>, cudaGraphExec_t> fwd_graphs;
  int nchk = 0, kseg = 0, cap_steps = 0;
  bool cap_gradient = false;  // the buffers were laid out for a gradient (tapes considered)
  std::vector<StateMap> maps;  // one TMA descriptor per state buffer
  double* ub[3] = {nullptr, nullptr, nullptr};  // adjoint states, rotating: read, written, zeroed
  Ctl* ctl = nullptr;
  double* dt_log = nullptr;
  double* inv_log = nullptr;
  double* dtbar_log = nullptr;
  double* J = nullptr;
  double* part_v = nullptr;
  long long* part_i = nullptr;
  int nparts = 0;
  cudaStream_t stream = nullptr, stream2 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr, join = nullptr;
  float last_forward_ms = 0, last_gradient_ms = 0;
  std::map<std::tuple<int, int, double, double, double>, cudaGraphExec_t> graphs;
};

namespace {

int afail(int code, const std::string& m) { return set_error(code, m); }

#define A_CK(call)                                                                        \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return afail(E2D_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

Field<double> state(const e2d_adjoint* a, int k) {
  return Field<double>{a->pool + (size_t)k * a->state_elems, (int)a->pitch, (long long)a->plane};
}
Field<double> ubf(const e2d_adjoint* a, int k) { return Field<double>{a->ub[k], (int)a->pitch, (long long)a->plane}; }

// The tape of segment state j of set `set`.
TapeOut tape_of(const e2d_adjoint* a, int set, int j, bool only = false) {
  return tape_at(a->tapes, set * a->kseg + j, (long long)a->plane, (int)a->pitch, only);
}

Field<double> qpf(const e2d_adjoint* a, int k) {
  return Field<double>{a->qping + (size_t)k * a->state_elems, (int)a->pitch, (long long)a->plane};
}

void free_buffers(e2d_adjoint* a) {
  for (auto& kv : a->graphs) cudaGraphExecDestroy(kv.second);
  a->graphs.clear();
  for (auto& kv : a->fwd_graphs) cudaGraphExecDestroy(kv.second);
  a->fwd_graphs.clear();
  cudaFree(a->pool);
  a->pool = nullptr;
  cudaFree(a->tapes);
  a->tapes = nullptr;
  cudaFree(a->dt_log);
  cudaFree(a->inv_log);
  cudaFree(a->dtbar_log);
  a->dt_log = a->inv_log = a->dtbar_log = nullptr;
  a->maps.clear();
  a->cap_steps = 0;
  a->cap_gradient = false;
}

// Buffers for nsteps: 2 ping-pong states, ceil(N/K) checkpoints, and two
// sets of K segment states (one being reversed while the next is recomputed)
// with their tapes.  When every state and its tape fit in half the free
// device memory (and E2D_ADJ_FULL_TAPE is not 0), the run is one segment
// instead: K = N, one set, and the forward sweep keeps all N states and
// writes all N tapes, so the reverse sweep recomputes nothing.  A call for
// the objective alone (gradient false) lays out no tape; a later gradient
// lays the buffers out again.
int ensure(e2d_adjoint* a, int nsteps, bool gradient) {
  if (nsteps <= a->cap_steps && (a->cap_gradient || !gradient)) return E2D_OK;
  free_buffers(a);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const size_t full_bytes =
      ((size_t)nsteps * (kTapePlanes * a->plane + a->state_elems) + (size_t)3 * a->state_elems) * sizeof(double);
  const char* ft = std::getenv("E2D_ADJ_FULL_TAPE");
  bool full = gradient && a->use_tape && !(ft && ft[0] == '0') && full_bytes <= free_b / 2;
  for (;;) {
    const int K = full ? nsteps : std::max(1, (int)std::ceil(std::sqrt((double)nsteps)));
    const int nsets = full ? 1 : 2;
    const int nchk = (nsteps + K - 1) / K;
    const int nstates = 2 + nchk + nsets * K;
    if (cudaMalloc(&a->pool, (size_t)nstates * a->state_elems * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&a->dt_log, nsteps * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&a->inv_log, nsteps * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&a->dtbar_log, nsteps * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      free_buffers(a);
      if (full) {  // the segmented layout needs less
        full = false;
        continue;
      }
      return afail(E2D_ERR_OOM, "cudaMalloc of the adjoint checkpoints failed");
    }
    const size_t tape_bytes = (size_t)nsets * K * kTapePlanes * a->plane * sizeof(double);
    if (!gradient || !a->use_tape || cudaMalloc(&a->tapes, tape_bytes) != cudaSuccess) {
      cudaGetLastError();
      a->tapes = nullptr;
      if (full) {
        free_buffers(a);
        full = false;
        continue;
      }
    } else {
      A_CK(cudaMemsetAsync(a->tapes, 0, tape_bytes, a->stream));  // cells no tile writes read as zeros
    }
    A_CK(cudaMemsetAsync(a->pool, 0, (size_t)nstates * a->state_elems * sizeof(double), a->stream));
    a->maps.resize(nstates);
    for (int k = 0; k < nstates; ++k)
      if (!fused_map_create<double>(a->h, state(a, k), &a->maps[k]) ||
          (k < 2 && !fused_map_create<double>(a->h, state(a, k), &a->imaps[k], true)))
        return afail(E2D_ERR_CUDA, "TMA descriptor setup failed");
    a->kseg = K;
    a->nchk = nchk;
    a->cap_steps = nsteps;
    a->cap_gradient = gradient;
    return E2D_OK;
  }
}

constexpr int kPing = 0;  // states 0, 1: forward ping-pong
int chk_index(const e2d_adjoint*, int s) { return 2 + s; }
int seg_index(const e2d_adjoint* a, int set, int k) { return 2 + a->nchk + set * a->kseg + k; }

// Forward N steps from state 0 (u); J on the device and, for a gradient,
// checkpoints every K steps and the seed Ubar_N = dJ/dU_N.  Enqueued only:
// no host synchronisation.
void enqueue_forward(e2d_adjoint* a, int nsteps, double xc, double yc, double sig, bool with_adjoint_seed,
                     const double* dt_fixed) {
  const Hydro<double>& h = a->h;
  cudaStream_t s = a->stream;
  cudaMemsetAsync(a->ctl, 0, sizeof(Ctl), s);
  launch_dt_reduce<double>(h, state(a, kPing), a->ctl, 0, s);  // main.f90:42
  launch_boundaries<double>(h, state(a, kPing), s);            // main.f90:46
  if (a->qping) {  // the primitives of both ping-pong states (the second for its corners)
    launch_prim<double>(h, state(a, kPing), qpf(a, 0), s);
    launch_prim<double>(h, state(a, kPing + 1), qpf(a, 1), s);
  }
  const int K = a->kseg, last = (nsteps + K - 1) / K - 1;
  for (int k = 0; k < nsteps; ++k) {
    const int in = k & 1, out = in ^ 1;
    if (with_adjoint_seed) {  // checkpoints, and the last segment's states kept whole, for the reverse sweep
      if (k >= last * K)
        cudaMemcpyAsync(state(a, seg_index(a, last & 1, k - last * K)).p, state(a, in).p,
                        a->state_elems * sizeof(double), cudaMemcpyDeviceToDevice, s);
      else if (k % K == 0)
        cudaMemcpyAsync(state(a, chk_index(a, k / K)).p, state(a, in).p, a->state_elems * sizeof(double),
                        cudaMemcpyDeviceToDevice, s);
    }
    const int rd = k & 1;
    StepDt<double> sd;
    sd.inv_log = a->inv_log;
    sd.dt_value = dt_fixed ? dt_fixed[k] : 0.0;
    sd.dt_ptr = nullptr;
    sd.from_slot = dt_fixed ? 0 : 1;
    sd.rd_slot = rd;
    sd.wr_slot = rd ^ 1;
    sd.dt_log = a->dt_log;
    sd.log_index = k;
    // (the tape steps are the last segment's: no primitives-reading step follows them)
    if (with_adjoint_seed && a->tapes && k >= last * K)
      launch_fused_tape(h, a->maps[in], state(a, in), state(a, out), sd, a->ctl, tape_of(a, last & 1, k - last * K),
                        s);
    else if (a->qping)
      launch_fused_map_q(h, a->qmaps[in], a->imaps[in], state(a, in), state(a, out), qpf(a, out), sd, a->ctl, s);
    else
      launch_fused_map<double>(h, a->maps[in], state(a, in), state(a, out), sd, a->ctl, true, s);
  }
  cudaMemsetAsync(a->J, 0, sizeof(double), s);
  Field<double> seed = with_adjoint_seed ? ubf(a, 0) : Field<double>{nullptr, 0, 0};
  launch_objective(h, state(a, nsteps & 1), xc, yc, sig, a->J, seed, s);
}

// Recomputes segment sg's states (k0 .. k1-1) into segment set `set` from
// its checkpoint, with the logged dt (bit for bit the forward states).
void enqueue_recompute(e2d_adjoint* a, int sg, int set, int nsteps, cudaStream_t s) {
  const Hydro<double>& h = a->h;
  const int K = a->kseg, k0 = sg * K, k1 = std::min(k0 + K, nsteps);
  cudaMemcpyAsync(state(a, seg_index(a, set, 0)).p, state(a, chk_index(a, sg)).p, a->state_elems * sizeof(double),
                  cudaMemcpyDeviceToDevice, s);
  launch_seg_corners(h, a->pool, a->state_elems, a->pitch, a->plane, kPing, seg_index(a, set, 0), k0, k1 - k0, s);
  for (int m = k0; m < k1 - 1; ++m) {
    StepDt<double> sd;
    sd.dt_value = 0.0;
    sd.dt_ptr = a->dt_log + m;
    sd.from_slot = 0;
    sd.rd_slot = -1;
    sd.wr_slot = -1;
    sd.dt_log = nullptr;
    sd.log_index = 0;
    if (a->tapes)
      launch_fused_tape(h, a->maps[seg_index(a, set, m - k0)], state(a, seg_index(a, set, m - k0)),
                        state(a, seg_index(a, set, m - k0 + 1)), sd, a->ctl, tape_of(a, set, m - k0), s);
    else
      launch_fused_map<double>(h, a->maps[seg_index(a, set, m - k0)], state(a, seg_index(a, set, m - k0)),
                               state(a, seg_index(a, set, m - k0 + 1)), sd, a->ctl, true, s);
  }
  if (a->tapes) {  // the segment's last state has no step here: its tape alone
    const int j = k1 - 1 - k0;
    StepDt<double> sd;
    sd.dt_value = 0.0;
    sd.dt_ptr = a->dt_log + (k1 - 1);
    sd.from_slot = 0;
    sd.rd_slot = -1;
    sd.wr_slot = -1;
    sd.dt_log = nullptr;
    sd.log_index = 0;
    launch_fused_tape(h, a->maps[seg_index(a, set, j)], state(a, seg_index(a, set, j)),
                      state(a, seg_index(a, set, j)), sd, a->ctl, tape_of(a, set, j, true), s);
  }
}

// The reverse sweep: segments last first.  Segment sg is reversed on the
// main stream from segment set sg & 1 while segment sg - 1 is recomputed on
// the second stream into the other set, so the two overlap on the GPU; the
// last segment needs no recomputation (the forward sweep kept its states).  The
// running CFL maximum's rises are found on the device from the logged
// maxima.  The adjoint states rotate over three buffers: reverse step m
// reads one, accumulates into the next and zeroes the third for step m - 1.
// Leaves dJ/dU_0 in ub[final_ub(nsteps)].
void enqueue_reverse(e2d_adjoint* a, int nsteps, int dt_mode) {
  const Hydro<double>& h = a->h;
  cudaStream_t s = a->stream, s2 = a->stream2;
  cudaMemsetAsync(a->dtbar_log, 0, nsteps * sizeof(double), s);
  int cur = 0;  // ub[cur] holds Ubar of the state after the step being reversed
  cudaMemsetAsync(a->ub[1], 0, a->state_elems * sizeof(double), s);
  const int K = a->kseg, last = (nsteps + K - 1) / K - 1;
  // the last segment's states were kept by the forward sweep
  for (int sg = last; sg >= 0; --sg) {
    const int set = sg & 1, k0 = sg * K, k1 = std::min(k0 + K, nsteps);
    if (sg > 0) {  // the other set is free once segment sg + 1 has been reversed
      cudaEventRecord(a->fork, s);
      cudaStreamWaitEvent(s2, a->fork, 0);
      enqueue_recompute(a, sg - 1, set ^ 1, nsteps, s2);
      cudaEventRecord(a->join, s2);
    }
    for (int m = k1 - 1; m >= k0; --m) {
      const int nxt = (cur + 1) % 3, zro = (cur + 2) % 3;
      Field<double> um = state(a, seg_index(a, set, m - k0));
      const TapeOut tp = a->tapes ? tape_of(a, set, m - k0) : TapeOut();
      launch_step_rev(h, um, ubf(a, cur), ubf(a, nxt), m > 0 ? ubf(a, zro) : Field<double>{nullptr, 0, 0},
                      a->dt_log + m, a->dtbar_log + m, s, a->tapes ? &tp : nullptr);
      if (dt_mode == 1) {
        launch_argmax(h, um, a->part_v, a->part_i, a->nparts, a->inv_log, m, s);
        launch_dt_route(h, um, ubf(a, nxt), a->part_v, a->part_i, a->nparts, a->dtbar_log, a->inv_log, m, nsteps,
                        s);
      }
      cur = nxt;
    }
    if (sg > 0) cudaStreamWaitEvent(s, a->join, 0);  // segment sg - 1 recomputed
  }
}

int final_ub(int nsteps) { return nsteps % 3; }  // one rotation per reversed step

int check_health(e2d_adjoint* a) {
  unsigned health = 0;
  A_CK(cudaMemcpy(&health, &a->ctl->health, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (health & E2D_HEALTH_DT_NONFINITE) return afail(E2D_ERR_NUMERICS, "dt became non-finite");
  return E2D_OK;
}

int load_initial(e2d_adjoint* a, const void* u0) {
  A_CK(cudaMemsetAsync(state(a, 1).p, 0, a->state_elems * sizeof(double), a->stream));  // u2: fresh, zero
  if (u0) {
    const size_t w = (size_t)(a->p.nx + 4) * sizeof(double);
    A_CK(cudaMemcpy2DAsync(state(a, 0).p, a->pitch * sizeof(double), u0, w, w, (size_t)4 * (a->p.ny + 4),
                           cudaMemcpyHostToDevice, a->stream));
  } else {
    launch_init_diagonal<double>(a->h, state(a, 0), 0.5, 1.0, 1.0, 0.125, (double)0.14f, a->stream);
  }
  A_CK(cudaGetLastError());
  return E2D_OK;
}

}  // namespace

extern "C" {

int e2d_adjoint_create(const e2d_params* p, e2d_adjoint** out) {
  if (!p || !out) return afail(E2D_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (p->precision != 8 || p->riemann_solver != E2D_RIEMANN_HLLC)
    return afail(E2D_ERR_INVALID_ARG, "the adjoint is defined for FP64 and the HLLC flux");
  if (p->nx < 2 || p->ny < 2 || p->nx > (1 << 16) || p->ny > (1 << 16) || !(p->gamma0 > 1.0) || !(p->cfl > 0.0) ||
      !(p->smallr > 0.0) || !(p->smallc > 0.0))
    return afail(E2D_ERR_INVALID_ARG, "invalid parameters");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return afail(E2D_ERR_NO_DEVICE, "no CUDA device");
  }
  e2d_adjoint* a = new e2d_adjoint;
  a->p = *p;
  a->h = make_hydro<double>(*p);
  cudaGetDevice(&a->device);
  a->pitch = ((size_t)p->nx + 4 + 31) / 32 * 32;
  a->plane = a->pitch * (size_t)(p->ny + 4);
  a->state_elems = 4 * a->plane;
  a->nparts = std::min(1024, p->ny);
  if (const char* t = std::getenv("E2D_NO_TAPE")) a->use_tape = !(t[0] == '1');
  const size_t sb = a->state_elems * sizeof(double);
  if (cudaMalloc(&a->ub[0], sb) != cudaSuccess || cudaMalloc(&a->ub[1], sb) != cudaSuccess ||
      cudaMalloc(&a->ub[2], sb) != cudaSuccess ||
      cudaMalloc(&a->ctl, sizeof(Ctl)) != cudaSuccess || cudaMalloc(&a->J, sizeof(double)) != cudaSuccess ||
      cudaMalloc(&a->part_v, a->nparts * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&a->part_i, a->nparts * sizeof(long long)) != cudaSuccess) {
    cudaGetLastError();
    e2d_adjoint_destroy(a);
    return afail(E2D_ERR_OOM, "cudaMalloc of the adjoint state failed");
  }
  if (cudaMalloc(&a->qping, 2 * sb) != cudaSuccess) {
    cudaGetLastError();
    a->qping = nullptr;
  } else if (!fused_map_create<double>(a->h, qpf(a, 0), &a->qmaps[0]) ||
             !fused_map_create<double>(a->h, qpf(a, 1), &a->qmaps[1])) {
    cudaGetLastError();
    cudaFree(a->qping);
    a->qping = nullptr;
  }
  if (cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&a->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&a->e0) != cudaSuccess || cudaEventCreate(&a->e1) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->join, cudaEventDisableTiming) != cudaSuccess || step_rev_setup() != 0) {
    e2d_adjoint_destroy(a);
    return afail(E2D_ERR_CUDA, "stream/event/kernel setup failed");
  }
  *out = a;
  return E2D_OK;
}

int e2d_adjoint_destroy(e2d_adjoint* a) {
  if (!a) return E2D_OK;
  cudaSetDevice(a->device);
  if (a->stream) cudaStreamSynchronize(a->stream);
  free_buffers(a);
  cudaFree(a->ub[0]);
  cudaFree(a->ub[1]);
  cudaFree(a->ub[2]);
  cudaFree(a->qping);
  cudaFree(a->ctl);
  cudaFree(a->J);
  cudaFree(a->part_v);
  cudaFree(a->part_i);
  if (a->e0) cudaEventDestroy(a->e0);
  if (a->e1) cudaEventDestroy(a->e1);
  if (a->fork) cudaEventDestroy(a->fork);
  if (a->join) cudaEventDestroy(a->join);
  if (a->stream2) {
    cudaStreamSynchronize(a->stream2);
    cudaStreamDestroy(a->stream2);
  }
  if (a->stream) cudaStreamDestroy(a->stream);
  delete a;
  return E2D_OK;
}

int e2d_adjoint_objective(e2d_adjoint* a, const void* u0, int nsteps, double xc, double yc, double sigma,
                          const double* dt_fixed, double* J) {
  if (!a || !J || nsteps < 1 || !(sigma > 0.0)) return afail(E2D_ERR_INVALID_ARG, "bad objective arguments");
  cudaSetDevice(a->device);
  if (int rc = ensure(a, nsteps, false)) return rc;
  if (int rc = load_initial(a, u0)) return rc;
  // replayed from a captured graph on later calls with the same step count and
  // objective (not with given dt values)
  cudaGraphExec_t exec = nullptr;
  if (!dt_fixed) {
    const auto key = std::make_tuple(nsteps, xc, yc, sigma);
    auto it = a->fwd_graphs.find(key);
    if (it != a->fwd_graphs.end()) {
      exec = it->second;
    } else {
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(a->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        enqueue_forward(a, nsteps, xc, yc, sigma, false, nullptr);
        if (cudaStreamEndCapture(a->stream, &graph) == cudaSuccess && graph) {
          if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
          cudaGraphDestroy(graph);
        }
      }
      cudaGetLastError();
      if (exec) {
        cudaGraphUpload(exec, a->stream);
        a->fwd_graphs[key] = exec;
      }
    }
  }
  A_CK(cudaEventRecord(a->e0, a->stream));
  if (exec) A_CK(cudaGraphLaunch(exec, a->stream));
  else enqueue_forward(a, nsteps, xc, yc, sigma, false, dt_fixed);
  A_CK(cudaGetLastError());
  A_CK(cudaEventRecord(a->e1, a->stream));
  A_CK(cudaMemcpyAsync(J, a->J, sizeof(double), cudaMemcpyDeviceToHost, a->stream));
  A_CK(cudaStreamSynchronize(a->stream));
  cudaEventElapsedTime(&a->last_forward_ms, a->e0, a->e1);
  return check_health(a);
}

int e2d_adjoint_gradient(e2d_adjoint* a, const void* u0, int nsteps, int dt_mode, double xc, double yc,
                         double sigma, double* J, double* grad_rho0, double* dt_log) {
  if (!a || !J || !grad_rho0 || nsteps < 1 || (dt_mode != 0 && dt_mode != 1) || !(sigma > 0.0))
    return afail(E2D_ERR_INVALID_ARG, "bad gradient arguments");
  cudaSetDevice(a->device);
  if (int rc = ensure(a, nsteps, true)) return rc;
  if (int rc = load_initial(a, u0)) return rc;
  cudaStream_t s = a->stream;
  // The forward/backward pair is one captured graph, replayed on later calls
  // with the same step count, dt mode and objective.
  const auto key = std::make_tuple(nsteps, dt_mode, xc, yc, sigma);
  cudaGraphExec_t exec = nullptr;
  auto it = a->graphs.find(key);
  if (it != a->graphs.end()) {
    exec = it->second;
  } else {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      enqueue_forward(a, nsteps, xc, yc, sigma, true, nullptr);
      enqueue_reverse(a, nsteps, dt_mode);
      if (cudaStreamEndCapture(s, &graph) == cudaSuccess && graph) {
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
        cudaGraphDestroy(graph);
      }
    }
    cudaGetLastError();
    if (exec) {
      cudaGraphUpload(exec, s);
      a->graphs[key] = exec;
    }
  }
  A_CK(cudaEventRecord(a->e0, s));
  if (exec) {
    A_CK(cudaGraphLaunch(exec, s));
  } else {
    enqueue_forward(a, nsteps, xc, yc, sigma, true, nullptr);
    enqueue_reverse(a, nsteps, dt_mode);
    A_CK(cudaGetLastError());
  }
  A_CK(cudaEventRecord(a->e1, s));
  A_CK(cudaMemcpyAsync(J, a->J, sizeof(double), cudaMemcpyDeviceToHost, s));
  // dJ/d rho0 on the interior, Fortran order (i fastest)
  A_CK(cudaMemcpy2DAsync(grad_rho0, (size_t)a->p.nx * sizeof(double), a->ub[final_ub(nsteps)] + 2 * a->pitch + 2,
                         a->pitch * sizeof(double), (size_t)a->p.nx * sizeof(double), (size_t)a->p.ny,
                         cudaMemcpyDeviceToHost, s));
  if (dt_log) A_CK(cudaMemcpyAsync(dt_log, a->dt_log, nsteps * sizeof(double), cudaMemcpyDeviceToHost, s));
  A_CK(cudaStreamSynchronize(s));
  cudaEventElapsedTime(&a->last_gradient_ms, a->e0, a->e1);
  return check_health(a);
}

int e2d_adjoint_last_ms(e2d_adjoint* a, float* objective_ms, float* gradient_ms) {
  if (!a) return afail(E2D_ERR_INVALID_ARG, "null adjoint handle");
  if (objective_ms) *objective_ms = a->last_forward_ms;
  if (gradient_ms) *gradient_ms = a->last_gradient_ms;
  return E2D_OK;
}

int e2d_adjoint_layout(e2d_adjoint* a, int* segment_steps, int* tape) {
  if (!a) return afail(E2D_ERR_INVALID_ARG, "null adjoint handle");
  if (segment_steps) *segment_steps = a->kseg;
  if (tape) *tape = a->tapes ? 1 : 0;
  return E2D_OK;
}

}  // extern "C"
