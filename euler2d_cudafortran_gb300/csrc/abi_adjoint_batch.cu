// abi_adjoint_batch.cu -- the discrete adjoint of a whole ensemble
// (e2d_adjoint_batch_*): per-problem gradients of J_p = sum rho^2 w of the
// final state with respect to the initial density, for many independent FP64
// HLLC problems of uneven sizes, computed together.
//
// Every stage is one launch over all problems (all run the same number of
// steps): the forward step is the ensemble step kernel (k_batch.cu) with the
// running CFL maxima logged, the reverse step is the reverse tile kernel over
// the flattened tile list of all problems, and the argmax / dt routing /
// objective / checkpoint copies are batched kernels.  The forward/backward
// pair of one call is a single captured CUDA graph, replayed on later calls
// with the same step count, dt mode and objective.  Buffers of a problem
// (indices into its slab): 0, 1 forward ping-pong; 2.. checkpoints every
// K = ceil(sqrt(N)) steps; then two sets of K segment states (a segment is
// reversed on the main stream from one set while the next is recomputed on a
// second stream into the other); then 3 adjoint states (rotating: read,
// accumulated into, zeroed for the next reverse step).  The initial state
// lives in its own array so that a call can be replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <map>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/euler2d_gb300.h"
#include "adjoint_launch.h"
#include "batch.h"
#include "hydro_params.h"

using namespace e2d;

struct e2d_adjoint_batch {
  int nprob = 0, device = 0;
  std::vector<e2d_params> params;
  std::vector<Hydro<double>> hd;
  std::vector<size_t> pitch, plane, se;  // elements; se = one state (4 planes)
  std::vector<size_t> u0_off;            // offsets in the initial-state pool
  std::vector<long long> grad_off;
  long long grad_elems = 0;
  double* u0 = nullptr;
  // primitives beside the forward ping-pong states of every problem (the fast
  // forward step, as the ensemble's), at u0_off offsets, two pools; null when
  // they could not be allocated
  double* qping = nullptr;
  size_t q_total = 0;
  double* slab = nullptr;  // all problems' buffers, allocated by ensure()
  int kseg = 0, nchk = 0, cap_steps = 0;
  AdjProb* d_probs = nullptr;          // by problem index
  BatchProb<double>* d_fwd = nullptr;  // forward ping-pong, work-list order
  BatchProb<double>* d_seg = nullptr;  // [2][K - 1][nprob]: segment set, state j -> j + 1
  // The tape (one set of K segment states per problem, written by the
  // forward sweep's last segment and by each recomputation, read by the
  // reverse steps), when it fits in half the free memory and E2D_NO_TAPE is
  // not 1; the recomputation then follows each segment's reverse sweep
  // instead of overlapping it.
  double* tapes = nullptr;
  bool use_tape = true;
  BatchProb<double>* d_fwdtape = nullptr;  // [K][nprob]: forward steps of the last segment, with tapes
  BatchProb<double>* d_segonly = nullptr;  // [2][nprob]: the tape-only pass of a segment's last state
  int fwd_tiles = 0, fwd_grid = 0, rev_tiles = 0, nparts = 64;
  bool square = false;  // every problem has dx == dy
  Ctl* ctls = nullptr;
  double *dt_log = nullptr, *inv_log = nullptr, *dtbar_log = nullptr;
  double* J = nullptr;
  double* part_v = nullptr;
  long long* part_i = nullptr;
  double* grad = nullptr;
  cudaStream_t stream = nullptr, stream2 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr, join = nullptr;
  float last_forward_ms = 0, last_gradient_ms = 0;
  std::map<std::tuple<int, int, int, double, double, double>, cudaGraphExec_t> graphs;
};

namespace {

int abfail(int code, const std::string& m) { return set_error(code, m); }

#define AB_CK(call)                                                                                          \
  do {                                                                                                       \
    cudaError_t e_ = (call);                                                                                 \
    if (e_ != cudaSuccess) return abfail(E2D_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kPing = 0, kChk = 2;
int seg_base(const e2d_adjoint_batch* b) { return kChk + b->nchk; }
int ub_base(const e2d_adjoint_batch* b) { return kChk + b->nchk + 2 * b->kseg; }
int nbuf(const e2d_adjoint_batch* b) { return ub_base(b) + 3; }

void clear_graphs(e2d_adjoint_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

void free_slab(e2d_adjoint_batch* b) {
  clear_graphs(b);
  cudaFree(b->slab);
  cudaFree(b->d_probs);
  cudaFree(b->d_fwd);
  cudaFree(b->d_seg);
  cudaFree(b->tapes);
  cudaFree(b->d_fwdtape);
  cudaFree(b->d_segonly);
  b->tapes = nullptr;
  b->d_fwdtape = b->d_segonly = nullptr;
  cudaFree(b->dt_log);
  cudaFree(b->inv_log);
  cudaFree(b->dtbar_log);
  b->slab = nullptr;
  b->d_probs = nullptr;
  b->d_fwd = b->d_seg = nullptr;
  b->dt_log = b->inv_log = b->dtbar_log = nullptr;
  b->cap_steps = 0;
}

AdjBatch view(const e2d_adjoint_batch* b) {
  AdjBatch B;
  B.probs = b->d_probs;
  B.nprob = b->nprob;
  B.total_tiles = b->rev_tiles;
  B.nparts = b->nparts;
  B.square = b->square;
  B.dt_log = b->dt_log;
  B.inv_log = b->inv_log;
  B.dtbar_log = b->dtbar_log;
  B.J = b->J;
  B.part_v = b->part_v;
  B.part_i = b->part_i;
  return B;
}

// Buffers and work lists for nsteps steps.
int ensure(e2d_adjoint_batch* b, int nsteps) {
  if (nsteps <= b->cap_steps) return E2D_OK;
  AB_CK(cudaStreamSynchronize(b->stream));
  free_slab(b);
  const int K = std::max(1, (int)std::ceil(std::sqrt((double)nsteps)));
  b->kseg = K;
  b->nchk = (nsteps + K - 1) / K;
  const int nb = nbuf(b);
  std::vector<size_t> slab_off(b->nprob);
  size_t total = 0;
  for (int p = 0; p < b->nprob; ++p) {
    slab_off[p] = total;
    total += (size_t)nb * b->se[p];
  }
  const size_t nlog = (size_t)nsteps * b->nprob;
  if (cudaMalloc(&b->slab, total * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&b->d_probs, sizeof(AdjProb) * b->nprob) != cudaSuccess ||
      cudaMalloc(&b->d_fwd, sizeof(BatchProb<double>) * b->nprob) != cudaSuccess ||
      cudaMalloc(&b->d_seg, sizeof(BatchProb<double>) * b->nprob * 2 * std::max(1, K - 1)) != cudaSuccess ||
      cudaMalloc(&b->dt_log, nlog * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&b->inv_log, nlog * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&b->dtbar_log, nlog * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    free_slab(b);
    return abfail(E2D_ERR_OOM, "cudaMalloc of the batched adjoint checkpoints failed");
  }
  AB_CK(cudaMemsetAsync(b->slab, 0, total * sizeof(double), b->stream));
  // the tape: K tapes per problem, if they take at most half the free memory
  std::vector<size_t> tape_off(b->nprob);
  size_t tape_total = 0;
  for (int p = 0; p < b->nprob; ++p) {
    tape_off[p] = tape_total;
    tape_total += (size_t)K * kTapePlanes * b->plane[p];
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  if (b->use_tape && tape_total * sizeof(double) <= free_b / 2 &&
      cudaMalloc(&b->tapes, tape_total * sizeof(double)) == cudaSuccess &&
      cudaMalloc(&b->d_fwdtape, sizeof(BatchProb<double>) * b->nprob * K) == cudaSuccess &&
      cudaMalloc(&b->d_segonly, sizeof(BatchProb<double>) * b->nprob * 2) == cudaSuccess) {
    AB_CK(cudaMemsetAsync(b->tapes, 0, tape_total * sizeof(double), b->stream));  // unwritten cells read zeros
  } else {
    cudaGetLastError();
    cudaFree(b->tapes);
    cudaFree(b->d_fwdtape);
    cudaFree(b->d_segonly);
    b->tapes = nullptr;
    b->d_fwdtape = b->d_segonly = nullptr;
  }
  // reverse tiles by problem index
  int rtx, rty;
  rev_tile_shape(&rtx, &rty);
  std::vector<AdjProb> ap(b->nprob);
  int t = 0;
  for (int p = 0; p < b->nprob; ++p) {
    AdjProb& P = ap[p];
    P.h = b->hd[p];
    P.u0 = b->u0 + b->u0_off[p];
    P.base = b->slab + slab_off[p];
    P.state_elems = (long long)b->se[p];
    P.pitch = (int)b->pitch[p];
    P.plane = (long long)b->plane[p];
    P.ntx = (b->params[p].nx + rtx - 1) / rtx;
    P.nty = (b->params[p].ny + rty - 1) / rty;
    P.tile_begin = t;
    P.grad_off = b->grad_off[p];
    P.tape_base = b->tapes ? b->tapes + tape_off[p] : nullptr;
    t += P.ntx * P.nty;
  }
  b->rev_tiles = t;
  // forward work list (largest problems first), 32 x 15 tiles
  int ftx, fty, fnt;
  batch_tile_shape<double>(0, &ftx, &fty, &fnt);
  std::vector<int> order(b->nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (long long)b->params[x].nx * b->params[x].ny > (long long)b->params[y].nx * b->params[y].ny;
  });
  const size_t nseg_arr = (size_t)b->nprob * std::max(1, K - 1);
  std::vector<BatchProb<double>> fw(b->nprob), sg(2 * nseg_arr), fwt((size_t)K * b->nprob), so(2 * b->nprob);
  int ft = 0;
  for (int k = 0; k < b->nprob; ++k) {
    const int p = order[k];
    BatchProb<double>& F = fw[k];
    F.h = b->hd[p];
    F.u = ap[p].base + (size_t)kPing * b->se[p];
    F.u2 = ap[p].base + (size_t)(kPing + 1) * b->se[p];
    F.pitch = (int)b->pitch[p];
    F.plane = (long long)b->plane[p];
    F.ntx = (b->params[p].nx + ftx - 1) / ftx;
    F.nty = (b->params[p].ny + fty - 1) / fty;
    F.tile_begin = ft;
    F.id = p;
    F.q = b->qping ? b->qping + b->u0_off[p] : nullptr;
    F.q2 = b->qping ? b->qping + b->q_total + b->u0_off[p] : nullptr;
    ft += F.ntx * F.nty;
    const auto tape = [&](int j, bool only) {
      return b->tapes ? tape_at(b->tapes + tape_off[p], j, (long long)b->plane[p], (int)b->pitch[p], only)
                      : TapeOut();
    };
    for (int set = 0; set < 2; ++set) {
      for (int j = 0; j + 1 < K; ++j) {
        BatchProb<double>& S = sg[set * nseg_arr + (size_t)j * b->nprob + k];
        S = F;
        S.u = ap[p].base + (size_t)(seg_base(b) + set * K + j) * b->se[p];
        S.u2 = ap[p].base + (size_t)(seg_base(b) + set * K + j + 1) * b->se[p];
        S.tape = tape(j, false);
      }
      BatchProb<double>& O = so[(size_t)set * b->nprob + k];  // state K - 1 of the set, read at parity 0
      O = F;
      O.u = O.u2 = ap[p].base + (size_t)(seg_base(b) + set * K + (K - 1)) * b->se[p];
      O.tape = tape(K - 1, true);
    }
    for (int j = 0; j < K; ++j) {
      fwt[(size_t)j * b->nprob + k] = F;
      fwt[(size_t)j * b->nprob + k].tape = tape(j, false);
    }
  }
  b->fwd_tiles = ft;
  b->square = std::all_of(fw.begin(), fw.end(), [](const BatchProb<double>& F) { return F.h.dx == F.h.dy; });
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  b->fwd_grid = std::max(1, std::min(ft, sms * std::max(1, batch_resident_per_sm<double>(0))));
  AB_CK(cudaMemcpyAsync(b->d_probs, ap.data(), sizeof(AdjProb) * b->nprob, cudaMemcpyHostToDevice, b->stream));
  AB_CK(cudaMemcpyAsync(b->d_fwd, fw.data(), sizeof(BatchProb<double>) * b->nprob, cudaMemcpyHostToDevice,
                        b->stream));
  AB_CK(cudaMemcpyAsync(b->d_seg, sg.data(), sizeof(BatchProb<double>) * sg.size(), cudaMemcpyHostToDevice,
                        b->stream));
  if (b->tapes) {
    AB_CK(cudaMemcpyAsync(b->d_fwdtape, fwt.data(), sizeof(BatchProb<double>) * fwt.size(), cudaMemcpyHostToDevice,
                          b->stream));
    AB_CK(cudaMemcpyAsync(b->d_segonly, so.data(), sizeof(BatchProb<double>) * so.size(), cudaMemcpyHostToDevice,
                          b->stream));
  }
  AB_CK(cudaStreamSynchronize(b->stream));
  b->cap_steps = nsteps;
  return E2D_OK;
}

Field<double> field(const e2d_adjoint_batch* b, int p, double* base_ptr) {
  return Field<double>{base_ptr, (int)b->pitch[p], (long long)b->plane[p]};
}
double* host_buf(const e2d_adjoint_batch* b, int p, int k) {
  size_t off = 0;
  for (int q = 0; q < p; ++q) off += (size_t)nbuf(b) * b->se[q];
  return b->slab + off + (size_t)k * b->se[p];
}

BatchLaunch<double> step_launch(const e2d_adjoint_batch* b, const BatchProb<double>* probs) {
  BatchLaunch<double> L;
  L.probs = probs;
  L.nprob = b->nprob;
  L.total_tiles = b->fwd_tiles;
  L.grid = b->fwd_grid;
  L.ctls = b->ctls;
  L.parity = 0;
  L.rd = -1;
  L.wr = -1;
  L.dt_log = nullptr;
  L.square = b->square;
  return L;
}

// Forward: the initial states, then N ensemble steps (checkpoints every K
// steps when checkpointing), then J (and the adjoint seed).
void enqueue_forward(e2d_adjoint_batch* b, int nsteps, double xc, double yc, double sig, bool adjoint) {
  cudaStream_t s = b->stream;
  const AdjBatch B = view(b);
  launch_batch_copy(B, -1, kPing, s);
  cudaMemsetAsync(b->ctls, 0, sizeof(Ctl) * b->nprob, s);
  for (int p = 0; p < b->nprob; ++p) {
    Field<double> u = field(b, p, host_buf(b, p, kPing));
    launch_dt_reduce<double>(b->hd[p], u, &b->ctls[p], 0, s);  // main.f90:42
    launch_boundaries<double>(b->hd[p], u, s);                 // main.f90:46
    if (b->qping) {  // the primitives of both ping-pong states (the second for its corners)
      launch_prim<double>(b->hd[p], u, field(b, p, b->qping + b->u0_off[p]), s);
      launch_prim<double>(b->hd[p], field(b, p, host_buf(b, p, kPing + 1)),
                          field(b, p, b->qping + b->q_total + b->u0_off[p]), s);
    }
  }
  const int K = b->kseg, last = (nsteps + K - 1) / K - 1;
  for (int k = 0; k < nsteps; ++k) {
    if (adjoint) {  // checkpoints, and the last segment's states kept whole, for the reverse sweep
      if (k >= last * K) launch_batch_copy(B, kPing + (k & 1), seg_base(b) + (last & 1) * K + (k - last * K), s);
      else if (k % K == 0) launch_batch_copy(B, kPing + (k & 1), kChk + k / K, s);
    }
    const bool taping = adjoint && b->tapes && k >= last * K;
    BatchLaunch<double> L = step_launch(b, taping ? b->d_fwdtape + (size_t)(k - last * K) * b->nprob : b->d_fwd);
    L.parity = k & 1;
    L.rd = k & 1;
    L.wr = L.rd ^ 1;
    L.dt_log = b->dt_log + (size_t)k * b->nprob;
    L.inv_log = b->inv_log + (size_t)k * b->nprob;
    // (the taping steps are the last segment's: no primitives-reading step follows them)
    L.qin = !taping && b->qping != nullptr;
    if (taping) launch_batch_step_tape(L, s);
    else launch_batch_step<double>(0, L, s);
  }
  cudaMemsetAsync(b->J, 0, sizeof(double) * b->nprob, s);
  launch_batch_objective(B, kPing + (nsteps & 1), xc, yc, sig, adjoint ? ub_base(b) : -1, s);
}

// Recomputes segment sg of every problem into segment set `set` from its
// checkpoint with the logged dt.
void enqueue_recompute(e2d_adjoint_batch* b, int sg, int set, int nsteps, cudaStream_t s) {
  const AdjBatch B = view(b);
  const int K = b->kseg, k0 = sg * K, k1 = std::min(k0 + K, nsteps), sb = seg_base(b) + set * K;
  launch_batch_copy(B, kChk + sg, sb, s);
  launch_batch_seg_corners(B, kPing, sb, k0, k1 - k0, s);
  const size_t nseg_arr = (size_t)b->nprob * std::max(1, K - 1);
  for (int m = k0; m < k1 - 1; ++m) {
    BatchLaunch<double> L = step_launch(b, b->d_seg + set * nseg_arr + (size_t)(m - k0) * b->nprob);
    L.dt_src = b->dt_log + (size_t)m * b->nprob;
    if (b->tapes) launch_batch_step_tape(L, s);
    else launch_batch_step<double>(0, L, s);
  }
  if (b->tapes) {  // the segment's last state has no step here: its tape alone
    BatchLaunch<double> L = step_launch(b, b->d_segonly + (size_t)set * b->nprob);
    L.dt_src = b->dt_log + (size_t)(k1 - 1) * b->nprob;
    launch_batch_step_tape(L, s);
  }
}

// Reverse sweep, segment sg from set sg & 1 on the main stream while segment
// sg - 1 is recomputed into the other set on the second stream; dJ/dU_0 ends
// in buffer ub_base + (nsteps % 3).
void enqueue_reverse(e2d_adjoint_batch* b, int nsteps, int dt_mode) {
  cudaStream_t s = b->stream, s2 = b->stream2;
  const AdjBatch B = view(b);
  cudaMemsetAsync(b->dtbar_log, 0, sizeof(double) * nsteps * b->nprob, s);
  const int K = b->kseg, ub = ub_base(b), last = (nsteps + K - 1) / K - 1;
  int cur = 0;
  launch_batch_copy(B, ub + 1, ub + 1, s);  // zero
  // the last segment's states were kept by the forward sweep
  for (int sg = last; sg >= 0; --sg) {
    const int set = sg & 1, k0 = sg * K, k1 = std::min(k0 + K, nsteps), sb = seg_base(b) + set * K;
    if (sg > 0 && !b->tapes) {
      cudaEventRecord(b->fork, s);
      cudaStreamWaitEvent(s2, b->fork, 0);
      enqueue_recompute(b, sg - 1, set ^ 1, nsteps, s2);
      cudaEventRecord(b->join, s2);
    }
    for (int m = k1 - 1; m >= k0; --m) {
      const int nxt = (cur + 1) % 3, zro = (cur + 2) % 3;
      launch_batch_step_rev(B, sb + (m - k0), ub + cur, ub + nxt, m > 0 ? ub + zro : -1, m, s,
                            b->tapes ? m - k0 : -1);
      if (dt_mode == 1) {
        launch_batch_argmax(B, sb + (m - k0), m, s);
        launch_batch_dt_route(B, sb + (m - k0), ub + nxt, m, nsteps, s);
      }
      cur = nxt;
    }
    if (sg > 0) {
      if (b->tapes) enqueue_recompute(b, sg - 1, set ^ 1, nsteps, s);  // the one tape set is free now
      else cudaStreamWaitEvent(s, b->join, 0);
    }
  }
  launch_batch_extract(B, ub + cur, b->grad, s);
}

// Runs (capturing on first use) the forward or forward/backward graph.
int run(e2d_adjoint_batch* b, int nsteps, int dt_mode, bool adjoint, double xc, double yc, double sig) {
  cudaStream_t s = b->stream;
  const auto key = std::make_tuple(nsteps, adjoint ? dt_mode : -1, adjoint ? 1 : 0, xc, yc, sig);
  cudaGraphExec_t exec = nullptr;
  auto it = b->graphs.find(key);
  if (it != b->graphs.end()) {
    exec = it->second;
  } else {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      enqueue_forward(b, nsteps, xc, yc, sig, adjoint);
      if (adjoint) enqueue_reverse(b, nsteps, dt_mode);
      if (cudaStreamEndCapture(s, &graph) == cudaSuccess && graph) {
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
        cudaGraphDestroy(graph);
      }
    }
    cudaGetLastError();
    if (exec) {
      cudaGraphUpload(exec, s);
      b->graphs[key] = exec;
    }
  }
  AB_CK(cudaEventRecord(b->e0, s));
  if (exec) {
    AB_CK(cudaGraphLaunch(exec, s));
  } else {
    enqueue_forward(b, nsteps, xc, yc, sig, adjoint);
    if (adjoint) enqueue_reverse(b, nsteps, dt_mode);
    AB_CK(cudaGetLastError());
  }
  AB_CK(cudaEventRecord(b->e1, s));
  return E2D_OK;
}

int finish(e2d_adjoint_batch* b, float* ms) {
  AB_CK(cudaStreamSynchronize(b->stream));
  cudaEventElapsedTime(ms, b->e0, b->e1);
  std::vector<Ctl> c(b->nprob);
  AB_CK(cudaMemcpy(c.data(), b->ctls, sizeof(Ctl) * b->nprob, cudaMemcpyDeviceToHost));
  for (int p = 0; p < b->nprob; ++p)
    if (c[p].health & E2D_HEALTH_DT_NONFINITE)
      return abfail(E2D_ERR_NUMERICS, "dt became non-finite in problem " + std::to_string(p));
  return E2D_OK;
}

int check(const e2d_adjoint_batch* b) { return b ? E2D_OK : abfail(E2D_ERR_INVALID_ARG, "null handle"); }

}  // namespace

extern "C" {

int e2d_adjoint_batch_create(const e2d_params* base, int nprob, const int* nx, const int* ny, const int* bc,
                             e2d_adjoint_batch** out) {
  if (!base || !nx || !ny || !out || nprob < 1) return abfail(E2D_ERR_INVALID_ARG, "bad batched adjoint arguments");
  *out = nullptr;
  if (base->precision != 8 || base->riemann_solver != E2D_RIEMANN_HLLC)
    return abfail(E2D_ERR_INVALID_ARG, "the adjoint is defined for FP64 and the HLLC flux");
  if (!(base->gamma0 > 1.0) || !(base->cfl > 0.0) || !(base->smallr > 0.0) || !(base->smallc > 0.0))
    return abfail(E2D_ERR_INVALID_ARG, "gamma0 > 1, cfl > 0, smallr > 0, smallc > 0");
  for (int p = 0; p < nprob; ++p)
    if (nx[p] < 2 || ny[p] < 2 || nx[p] > (1 << 16) || ny[p] > (1 << 16))
      return abfail(E2D_ERR_INVALID_ARG, "every nx, ny must be in [2, 2^16]");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return abfail(E2D_ERR_NO_DEVICE, "no CUDA device");
  }
  e2d_adjoint_batch* b = new e2d_adjoint_batch;
  if (const char* t = std::getenv("E2D_NO_TAPE")) b->use_tape = !(t[0] == '1');
  b->nprob = nprob;
  cudaGetDevice(&b->device);
  size_t u0_total = 0;
  for (int p = 0; p < nprob; ++p) {
    e2d_params q = *base;
    q.nx = nx[p];
    q.ny = ny[p];
    if (bc) {
      q.boundary_type_xmin = bc[4 * p + 0];
      q.boundary_type_xmax = bc[4 * p + 1];
      q.boundary_type_ymin = bc[4 * p + 2];
      q.boundary_type_ymax = bc[4 * p + 3];
    }
    b->params.push_back(q);
    b->hd.push_back(make_hydro<double>(q));
    const size_t pitch = ((size_t)q.nx + 4 + 31) / 32 * 32;
    b->pitch.push_back(pitch);
    b->plane.push_back(pitch * (size_t)(q.ny + 4));
    b->se.push_back(4 * b->plane.back());
    b->u0_off.push_back(u0_total);
    u0_total += b->se.back();
    b->grad_off.push_back(b->grad_elems);
    b->grad_elems += (long long)q.nx * q.ny;
  }
  auto cleanup = [&](int code, const std::string& m) {
    e2d_adjoint_batch_destroy(b);
    return abfail(code, m);
  };
  if (cudaMalloc(&b->u0, u0_total * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&b->ctls, sizeof(Ctl) * nprob) != cudaSuccess ||
      cudaMalloc(&b->J, sizeof(double) * nprob) != cudaSuccess ||
      cudaMalloc(&b->part_v, sizeof(double) * nprob * b->nparts) != cudaSuccess ||
      cudaMalloc(&b->part_i, sizeof(long long) * nprob * b->nparts) != cudaSuccess ||
      cudaMalloc(&b->grad, sizeof(double) * b->grad_elems) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(E2D_ERR_OOM, "cudaMalloc of the batched adjoint state failed");
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess || batch_step_rev_setup() != 0)
    return cleanup(E2D_ERR_CUDA, "stream/event/kernel setup failed");
  cudaMemsetAsync(b->u0, 0, u0_total * sizeof(double), b->stream);
  if (cudaMalloc(&b->qping, 2 * u0_total * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    b->qping = nullptr;
  }
  b->q_total = u0_total;
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return cleanup(E2D_ERR_CUDA, "initialisation failed");
  *out = b;
  return E2D_OK;
}

int e2d_adjoint_batch_destroy(e2d_adjoint_batch* b) {
  if (!b) return E2D_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_slab(b);
  cudaFree(b->u0);
  cudaFree(b->qping);
  cudaFree(b->ctls);
  cudaFree(b->J);
  cudaFree(b->part_v);
  cudaFree(b->part_i);
  cudaFree(b->grad);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->stream2) {
    cudaStreamSynchronize(b->stream2);
    cudaStreamDestroy(b->stream2);
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return E2D_OK;
}

int e2d_adjoint_batch_init_diagonal(e2d_adjoint_batch* b, const double* offset, const double* rho_hi,
                                    const double* p_hi, const double* rho_lo, const double* p_lo) {
  if (int rc = check(b)) return rc;
  if (!offset || !rho_hi || !p_hi || !rho_lo || !p_lo) return abfail(E2D_ERR_INVALID_ARG, "null initial data");
  cudaSetDevice(b->device);
  for (int p = 0; p < b->nprob; ++p)
    launch_init_diagonal<double>(b->hd[p], field(b, p, b->u0 + b->u0_off[p]), offset[p], rho_hi[p], p_hi[p],
                                 rho_lo[p], p_lo[p], b->stream);
  AB_CK(cudaGetLastError());
  AB_CK(cudaStreamSynchronize(b->stream));
  return E2D_OK;
}

int e2d_adjoint_batch_upload_state(e2d_adjoint_batch* b, int prob, const void* host) {
  if (int rc = check(b)) return rc;
  if (prob < 0 || prob >= b->nprob || !host) return abfail(E2D_ERR_INVALID_ARG, "bad upload arguments");
  cudaSetDevice(b->device);
  const size_t w = (size_t)(b->params[prob].nx + 4) * sizeof(double);
  AB_CK(cudaMemcpy2DAsync(b->u0 + b->u0_off[prob], b->pitch[prob] * sizeof(double), host, w, w,
                          (size_t)4 * (b->params[prob].ny + 4), cudaMemcpyHostToDevice, b->stream));
  AB_CK(cudaStreamSynchronize(b->stream));
  return E2D_OK;
}

int e2d_adjoint_batch_objective(e2d_adjoint_batch* b, int nsteps, double xc, double yc, double sigma, double* J) {
  if (int rc = check(b)) return rc;
  if (!J || nsteps < 1 || !(sigma > 0.0)) return abfail(E2D_ERR_INVALID_ARG, "bad objective arguments");
  cudaSetDevice(b->device);
  if (int rc = ensure(b, nsteps)) return rc;
  if (int rc = run(b, nsteps, 0, false, xc, yc, sigma)) return rc;
  AB_CK(cudaMemcpyAsync(J, b->J, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost, b->stream));
  return finish(b, &b->last_forward_ms);
}

int e2d_adjoint_batch_gradient(e2d_adjoint_batch* b, int nsteps, int dt_mode, double xc, double yc, double sigma,
                               double* J, double* grad_rho0, double* dt_log) {
  if (int rc = check(b)) return rc;
  if (!J || !grad_rho0 || nsteps < 1 || (dt_mode != 0 && dt_mode != 1) || !(sigma > 0.0))
    return abfail(E2D_ERR_INVALID_ARG, "bad gradient arguments");
  cudaSetDevice(b->device);
  if (int rc = ensure(b, nsteps)) return rc;
  if (int rc = run(b, nsteps, dt_mode, true, xc, yc, sigma)) return rc;
  AB_CK(cudaMemcpyAsync(J, b->J, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost, b->stream));
  AB_CK(cudaMemcpyAsync(grad_rho0, b->grad, sizeof(double) * b->grad_elems, cudaMemcpyDeviceToHost, b->stream));
  if (dt_log)
    AB_CK(cudaMemcpyAsync(dt_log, b->dt_log, sizeof(double) * nsteps * b->nprob, cudaMemcpyDeviceToHost, b->stream));
  return finish(b, &b->last_gradient_ms);
}

int e2d_adjoint_batch_last_ms(e2d_adjoint_batch* b, float* objective_ms, float* gradient_ms) {
  if (int rc = check(b)) return rc;
  if (objective_ms) *objective_ms = b->last_forward_ms;
  if (gradient_ms) *gradient_ms = b->last_gradient_ms;
  return E2D_OK;
}

}  // extern "C"
