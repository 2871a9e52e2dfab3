// batch.h -- device-side description of an ensemble of independent runs.
#pragma once
#include "launch.h"

namespace e2d {

template <typename Real>
struct BatchProb {
  Hydro<Real> h;   // this problem's parameters (size, boundaries, constants)
  Real* u;         // pitched states, as a single run's u and u2
  Real* u2;
  Real* q;         // primitives beside u and u2 (same layout), null when not kept
  Real* q2;
  int pitch;
  long long plane;
  int ntx, nty;    // tiles of the chosen shape
  int tile_begin;  // first index of this problem in the flattened tile list
  int id;          // problem index (its control block and dt-log column)
  TapeOut tape;    // (FP64 adjoint) where a taping step leaves its input's forward values
};

template <typename Real>
struct BatchLaunch {
  const BatchProb<Real>* probs;  // device array, in work-list order
  int nprob, total_tiles, parity, rd, wr, grid;
  Ctl* ctls;      // per-problem running CFL maxima and health flags, by problem index
  Real* dt_log;   // device, nprob entries for this step by problem index (may be null)
  const Real* dt_src = nullptr;  // if set: step with these logged dt (by problem index), no CFL fold
  Real* inv_log = nullptr;       // if set: receives each problem's running CFL maximum before the step
  bool square = false;           // every problem has dx == dy (selects the kernel that shares face sources)
  bool qin = false;              // the boxes are read from q/q2 (current), and the step writes the next ones
};

// (FP64, 32 x 15 tiles, conservative boxes) the step that also writes each
// problem's tape (BatchProb::tape; tape.only: just the tape).
void launch_batch_step_tape(const BatchLaunch<double>& L, cudaStream_t s);

// Tile shapes: variant 0 = 32 x 15 cells (256 threads), 1 = 32 x 7 (128 threads).
template <typename Real> int batch_tile_shape(int variant, int* tx, int* ty, int* nt);
template <typename Real> int batch_resident_per_sm(int variant);
template <typename Real> void launch_batch_step(int variant, const BatchLaunch<Real>& L, cudaStream_t s);

}  // namespace e2d
