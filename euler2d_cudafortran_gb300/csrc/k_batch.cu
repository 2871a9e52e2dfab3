// k_batch.cu -- one kernel launch advances a whole ensemble of independent
// problems of uneven sizes by one time step.
//
// The tiles of every problem form one flattened work list (problem p owns
// tiles [tile_begin[p], tile_begin[p+1]), column by column); a persistent
// grid of CTAs splits the list into contiguous runs, one per CTA.  Each tile
// is computed exactly as in the single-run kernel (tile.cuh) with its own
// problem's parameters, its own dt (from the problem's running CFL maximum)
// and its own ghost rules, and folds the next step's CFL maximum into the
// problem's own slot.  Boxes are copied with 16-byte asynchronous copies
// because every problem has its own array (a tensor map per problem would be
// a kernel argument per problem).
#include <algorithm>

#include "batch.h"
#include "sync.cuh"
#include "tile.cuh"

namespace e2d {

#ifndef E2D_BATCH_CARRY
#define E2D_BATCH_CARRY 1
#endif

namespace {

// 16-byte asynchronous copy global -> shared; the bytes past src_bytes (0, 8
// or 16) are zero-filled, what TMA zero fill gives outside the array.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// SQ: every problem of the launch has dx == dy (the shared face source term
// of tile_compute).  QIN: the boxes are read from the primitives kept beside
// the states, and the update writes those of the new state (tile_compute).
// A CTA walks one contiguous run of the flattened tiles (runs differ by at
// most one tile); within a problem the tiles are listed column by column, so
// that consecutive tiles of a run are mostly a tile and the one above it,
// which takes over the lower tile's top ring rows and y-face row
// (tile_compute's carry).  The box of the CTA's next tile is copied asynchronously
// (cp.async) into the box region as soon as the face phase of the current one
// ends (no later phase reads the box), so it lands while the update phase
// runs.  A problem's parameters and dt are loaded when the run enters it, not
// per tile.
// TAPE (FP64, !QIN): the step also writes each problem's tape (BatchProb::tape).
template <typename Real, class C, int MINB, bool SQ, bool QIN, bool TAPE = false>
__global__ void __launch_bounds__(C::NT, MINB)
    k_batch_step(const BatchProb<Real>* __restrict__ probs, int nprob, int total_tiles, int parity, int rd, int wr,
                 Ctl* ctls, Real* dt_log, const Real* dt_src, Real* inv_log) {
  extern __shared__ unsigned char smem_raw[];
  Real* base = reinterpret_cast<Real*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  unsigned char* tail = reinterpret_cast<unsigned char*>(base + C::n_real);
  int* face_counter = reinterpret_cast<int*>(tail + 8);
  Real* red = reinterpret_cast<Real*>(tail + 16);
  Real* sdt = red + 32;
  __shared__ Hydro<Real> sh;
  __shared__ int cur[3], nxt[3];  // problem (work-list order), problem index, tile within the problem
  const int tid = threadIdx.x;
  Real* const dreg = base + C::q_off;  // where a prefetched box lands (read by no phase after the faces)
  static_assert((C::q_off * sizeof(Real)) % 16 == 0 && (C::BXs * sizeof(Real)) % 16 == 0,
                "16-byte aligned copy destinations");

  auto lookup = [&](int t, int* info) {  // thread 0
    int lo = 0, hi = nprob - 1;  // last problem with tile_begin <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (probs[mid].tile_begin <= t) lo = mid;
      else hi = mid - 1;
    }
    info[0] = lo;
    info[1] = probs[lo].id;
    info[2] = t - probs[lo].tile_begin;
  };
  auto issue = [&](const int* info, Real* dst) {  // every thread: its part of the box of tile `info`
    const BatchProb<Real>& P = probs[info[0]];
    const int i0 = GW + (info[2] / P.nty) * C::TX, j0 = GW + (info[2] % P.nty) * C::TY;
    const Real* b = QIN ? (parity ? P.q2 : P.q) : (parity ? P.u2 : P.u);
    const int isize = P.h.isize, jsize = P.h.jsize;
    constexpr int CH = 16 / (int)sizeof(Real), NCH = C::BXs / CH;
    static_assert(C::BXs % CH == 0, "box rows of whole 16-byte chunks");
    for (int k = tid; k < 4 * C::BYs * NCH; k += C::NT) {
      const int v = k / (C::BYs * NCH), rem = k - v * (C::BYs * NCH);
      const int y = rem / NCH, c = rem - y * NCH;
      const int gi = i0 - GW + c * CH, gj = j0 - GW + y;
      const int n = gj < jsize ? max(0, min(isize - gi, CH)) : 0;
      const Real* src = n ? b + (long long)v * P.plane + (long long)gj * P.pitch + gi : b;
      cp_async16(smem_u32(dst + (v * C::BYs + y) * C::BXs + c * CH), src, n * (int)sizeof(Real));
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  // this CTA's run of the work list: [t_begin, t_end)
  const int per = total_tiles / (int)gridDim.x, extra = total_tiles % (int)gridDim.x, bid = (int)blockIdx.x;
  const int t_begin = bid * per + min(bid, extra), t_end = t_begin + per + (bid < extra ? 1 : 0);
  if (t_begin >= t_end) return;
  if (tid == 0) {
    lookup(t_begin, cur);
    *face_counter = 0;
  }
  __syncthreads();
  issue(cur, base + C::q_off);
  bool first = true;
  int loaded = -1;  // the work-list problem whose parameters and dt are in sh / sdt
  for (int t = t_begin; t < t_end; ++t) {
    if (tid == 0 && cur[0] != loaded) {
      loaded = cur[0];
      sh = probs[loaded].h;
      // (the integer-pipe division: the same bits as /, no FP64 pipe work)
      const Real dt0 = dt_src ? dt_src[cur[1]] : Ops<Real>::div(sh.cfl, *inv_slot<Real>(&ctls[cur[1]], rd));
      sdt[0] = dt0;
      sdt[1] = Ops<Real>::div(dt0, sh.dx);
      sdt[2] = Ops<Real>::div(dt0, sh.dy);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();  // every thread's copies, the problem's parameters and dt
    const int p = cur[0], id = cur[1], stile = cur[2];
    const BatchProb<Real>& P = probs[p];
    const int i0 = GW + (stile / P.nty) * C::TX, j0 = GW + (stile % P.nty) * C::TY;
    Field<Real> in{parity ? P.u2 : P.u, P.pitch, P.plane};
    Field<Real> out{parity ? P.u : P.u2, P.pitch, P.plane};
    const Field<Real> qout{QIN ? (parity ? P.q : P.q2) : out.p, P.pitch, P.plane};
    const int next = t + 1;
    const int ptiles = P.ntx * P.nty;
    // thread 0 names the next tile (this problem's next one, or the first of
    // the next problem in the work list) at the start of the face phase; the
    // barrier that ends the face phase publishes nxt to the prefetch
    auto find_next = [&]() {
      if (tid == 0 && next < t_end) {
        const bool same = stile + 1 < ptiles;
        nxt[0] = same ? p : p + 1;
        nxt[1] = same ? id : probs[p + 1].id;
        nxt[2] = same ? stile + 1 : 0;
      }
    };
    auto prefetch = [&]() {  // every thread, right after the face phase
      if (next < t_end) issue(nxt, dreg);
    };
    // the tile below was this CTA's previous one / the next one is the tile above
    const int carry = E2D_BATCH_CARRY
                          ? ((!first && stile % P.nty != 0) ? kCarryIn : 0) |
                                ((next < t_end && stile + 1 < ptiles && (stile + 1) % P.nty != 0) ? kCarryOut : 0)
                          : 0;
    const bool only = TAPE && P.tape.only;  // a tape-only pass: no update, no dt
    Real m = tile_compute<Real, C, SQ, QIN, TAPE>(sh, base, face_counter, red, i0, j0, in, out, qout, sdt[1],
                                                  sdt[2], true, wr >= 0 && !only, &ctls[id].health,
                                                  prefetch, &P.tape, find_next, carry);
    if (tid == 0 && !only) {
      if (stile == 0) {
        if (dt_log) dt_log[id] = sdt[0];
        if (inv_log) inv_log[id] = *inv_slot<Real>(&ctls[id], rd);
        if (!isfinite(sdt[0])) atomicOr(&ctls[id].health, 1u);
      }
      if (wr >= 0) {
        m = Ops<Real>::max(m, *inv_slot<Real>(&ctls[id], rd));
        atomic_max_slot_ptr<Real>(inv_slot<Real>(&ctls[id], wr), m);
      }
    }
    if (tid == 0) {
      *face_counter = 0;
      cur[0] = nxt[0];
      cur[1] = nxt[1];
      cur[2] = nxt[2];
    }
    __syncthreads();  // the tile's shared data consumed; the next tile named
    first = false;
  }
}

template <typename Real, class C, int MINB>
struct Variant {
  template <bool SQ, bool QIN>
  static int resident_sq() {
    int n = 0;
    if (cudaFuncSetAttribute(k_batch_step<Real, C, MINB, SQ, QIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)C::bytes) != cudaSuccess ||
        cudaFuncSetAttribute(k_batch_step<Real, C, MINB, SQ, QIN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_step<Real, C, MINB, SQ, QIN>, C::NT, C::bytes) !=
            cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return n;
  }
  // CTAs of any instantiation that fit on an SM (the persistent grid is sized
  // by it, so it must hold for the one launched).
  static int resident_per_sm() {
    return std::min(std::min(resident_sq<false, false>(), resident_sq<true, false>()),
                    std::min(resident_sq<false, true>(), resident_sq<true, true>()));
  }
  template <bool SQ, bool QIN>
  static void go(const BatchLaunch<Real>& L, cudaStream_t s) {
    k_batch_step<Real, C, MINB, SQ, QIN><<<L.grid, C::NT, C::bytes, s>>>(
        L.probs, L.nprob, L.total_tiles, L.parity, L.rd, L.wr, L.ctls, L.dt_log, L.dt_src, L.inv_log);
  }
  static void launch(const BatchLaunch<Real>& L, cudaStream_t s) {
    if (L.square) {
      if (L.qin) go<true, true>(L, s);
      else go<true, false>(L, s);
    } else {
      if (L.qin) go<false, true>(L, s);
      else go<false, false>(L, s);
    }
  }
};

// Tile shapes offered to the autotuner.
template <typename Real> using V32x15 = Variant<Real, TileCfg<Real, 32, 15, 256>, (sizeof(Real) == 8 ? 2 : 4)>;
template <typename Real> using V32x7 = Variant<Real, TileCfg<Real, 32, 7, 128>, (sizeof(Real) == 8 ? 4 : 6)>;

}  // namespace

void launch_batch_step_tape(const BatchLaunch<double>& L, cudaStream_t s) {
  using C = TileCfg<double, 32, 15, 256>;
  static bool attrs = false;
  if (!attrs) {  // dynamic shared memory and carveout, as for the other instantiations
    cudaFuncSetAttribute(k_batch_step<double, C, 2, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)C::bytes);
    cudaFuncSetAttribute(k_batch_step<double, C, 2, false, false, true>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes);
    cudaFuncSetAttribute(k_batch_step<double, C, 2, true, false, true>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_batch_step<double, C, 2, false, false, true>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    attrs = true;
  }
  if (L.square)
    k_batch_step<double, C, 2, true, false, true><<<L.grid, C::NT, C::bytes, s>>>(
        L.probs, L.nprob, L.total_tiles, L.parity, L.rd, L.wr, L.ctls, L.dt_log, L.dt_src, L.inv_log);
  else
    k_batch_step<double, C, 2, false, false, true><<<L.grid, C::NT, C::bytes, s>>>(
        L.probs, L.nprob, L.total_tiles, L.parity, L.rd, L.wr, L.ctls, L.dt_log, L.dt_src, L.inv_log);
}

template <typename Real>
int batch_tile_shape(int variant, int* tx, int* ty, int* nt) {
  switch (variant) {
    case 0: *tx = 32; *ty = 15; *nt = 256; return 0;
    case 1: *tx = 32; *ty = 7; *nt = 128; return 0;
    default: return -1;
  }
}

template <typename Real>
int batch_resident_per_sm(int variant) {
  return variant == 0 ? V32x15<Real>::resident_per_sm() : V32x7<Real>::resident_per_sm();
}

template <typename Real>
void launch_batch_step(int variant, const BatchLaunch<Real>& L, cudaStream_t s) {
  if (variant == 0) V32x15<Real>::launch(L, s);
  else V32x7<Real>::launch(L, s);
}

template int batch_tile_shape<double>(int, int*, int*, int*);
template int batch_tile_shape<float>(int, int*, int*, int*);
template int batch_resident_per_sm<double>(int);
template int batch_resident_per_sm<float>(int);
template void launch_batch_step<double>(int, const BatchLaunch<double>&, cudaStream_t);
template void launch_batch_step<float>(int, const BatchLaunch<float>&, cudaStream_t);

}  // namespace e2d
