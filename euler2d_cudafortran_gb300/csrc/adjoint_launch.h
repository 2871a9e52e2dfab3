// adjoint_launch.h -- launchers of the reverse kernels (k_adjoint.cu).
#pragma once
#include "launch.h"

namespace e2d {

// One problem of a batched adjoint: its buffers (k >= 0 at base + k *
// state_elems, k = -1 the initial state u0) and its reverse-step tiles.
struct AdjProb {
  Hydro<double> h;
  double* u0;
  double* base;
  long long state_elems;
  int pitch;
  long long plane;
  int ntx, nty, tile_begin;  // 32 x 7 tiles; this problem's first tile in the flattened list
  long long grad_off;        // this problem's nx*ny gradient in the packed output
  double* tape_base;         // K tapes (kTapePlanes planes each) of the segment states; null: none
};

// The device-side view of a batched adjoint; logs are step-major
// ([step][problem]), partial argmax results problem-major ([problem][part]).
struct AdjBatch {
  const AdjProb* probs;  // device array, by problem index (tile_begin increasing)
  int nprob, total_tiles, nparts;
  double* dt_log;
  double* inv_log;
  double* dtbar_log;
  double* J;
  double* part_v;
  long long* part_i;
  bool square = false;  // every problem has dx == dy
};

int batch_step_rev_setup();
int rev_tile_shape(int* tx, int* ty);
// tape_j >= 0: every problem's reverse reads its tape tape_j (AdjProb::tape_base).
void launch_batch_step_rev(const AdjBatch& B, int un, int ub_in, int ub_out, int ub_zero, int m, cudaStream_t s,
                           int tape_j = -1);
void launch_batch_argmax(const AdjBatch& B, int un, int m, cudaStream_t s);
void launch_batch_dt_route(const AdjBatch& B, int un, int ub_out, int m, int nsteps, cudaStream_t s);
// J[p] += sum rho^2 w of buffer un; seed_ub >= 0: that buffer = dJ/dU on the interior.
void launch_batch_objective(const AdjBatch& B, int un, double xc, double yc, double sig, int seed_ub,
                            cudaStream_t s);
// Buffer copy src -> dst (src = -1: the initial state); src == dst zero-fills.
void launch_batch_copy(const AdjBatch& B, int src, int dst, cudaStream_t s);
void launch_batch_seg_corners(const AdjBatch& B, int ping, int seg, int k0, int nseg, cudaStream_t s);
void launch_batch_extract(const AdjBatch& B, int ub, double* out, cudaStream_t s);

int step_rev_setup();
// Ubar_n += reverse of one step (U_n with ghosts, Ubar_{n+1} interior); *dtbar += dJ/d dt.
// dt is read on the device (the logged dt of the step).  The interior of ubz
// (if ubz.p) is zeroed: the buffer the following reverse step accumulates into.
// tape (if set): the forward values of U_n the forward step left (launch_fused_tape).
void launch_step_rev(const Hydro<double>& h, Field<double> un, Field<double> ubn1, Field<double> ubn,
                     Field<double> ubz, const double* dt, double* dtbar, cudaStream_t s,
                     const TapeOut* tape = nullptr);
// Ghost corners of segment buffers seg_index + 1 .. seg_index + nseg - 1 (states k0 + j)
// from ping-pong buffer ping_index + ((k0 + j) & 1); buffers are state_elems apart in pool.
void launch_seg_corners(const Hydro<double>& h, double* pool, size_t state_elems, size_t pitch, size_t plane,
                        int ping_index, int seg_index, int k0, int nseg, cudaStream_t s);
// Argmax of the compute_dt term of state m, only when the running maximum rises at m.
void launch_argmax(const Hydro<double>& h, Field<double> u, double* pv, long long* pi, int nparts,
                   const double* inv_log, int m, cudaStream_t s);
// Routes the dt adjoints of the steps whose running maximum was set at state m into Ubar_m.
void launch_dt_route(const Hydro<double>& h, Field<double> u, Field<double> ub, const double* pv, const long long* pi,
                     int nparts, const double* dtbar_log, const double* inv_log, int m, int nsteps,
                     cudaStream_t s);
// *J += sum rho^2 w; if ub.p, ub = dJ/dU on the interior.
void launch_objective(const Hydro<double>& h, Field<double> u, double xc, double yc, double sig, double* J,
                      Field<double> ub, cudaStream_t s);

}  // namespace e2d
