/*
 * euler2d_gb300.h -- C ABI of the GB300 (sm_103a) Euler-2D explicit step.
 *
 * This is the drop-in boundary for the hot path of pkestene/euler2d_cudaFortran:
 * the CFL time-step reduction (compute_dt) and the unsplit second-order Godunov
 * update (make_boundaries, convertToPrimitives, computeAndStoreFluxes,
 * updateHydro).  Each entry point replaces one module procedure of
 * serial_ref/m_run.f90 (or cuf/m_HydroRun_gpu.cuf) called by the HydroRun
 * driver serial_ref/main.f90; the procedure it replaces is cited beside it.
 *
 * Conventions
 *  - Plain C types only; callable from Fortran through ISO_C_BINDING
 *    (bind(C), type(c_ptr) handles, real(c_double)/real(c_float) arrays).
 *  - Host state arrays use the Fortran layout A(isize, jsize, 4), column-major,
 *    isize = nx+4, jsize = ny+4, variables ID=rho, IP=E, IU=rho*u, IV=rho*v
 *    (serial_ref/m_constants.f90:11-14), element type double (precision 8) or
 *    float (precision 4).
 *  - The state pair u/u2 is selected by `which` / `useU`: 0 = u, 1 = u2, the
 *    ping-pong of serial_ref/m_run.f90:197-201 (even nStep reads u, writes u2).
 *  - Every function returns an int status (E2D_OK on success).  The reference
 *    has no error codes; it stops on a bad namelist (serial_ref/m_run.f90:77-82,
 *    cuf/m_HydroParameters.cuf:128-132), which maps to E2D_ERR_INVALID_ARG here.
 *  - All device work is issued on the run's stream (e2d_set_stream); calls that
 *    return host data synchronise that stream.
 */
#ifndef EULER2D_GB300_H
#define EULER2D_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define E2D_OK 0
#define E2D_ERR_INVALID_ARG 1
#define E2D_ERR_CUDA 2
#define E2D_ERR_OOM 3
#define E2D_ERR_NUMERICS 4 /* dt non-finite: the run has blown up */
#define E2D_ERR_NO_DEVICE 5

/* Health flags (e2d_get_health). */
#define E2D_HEALTH_DT_NONFINITE 1u
#define E2D_HEALTH_NEG_DENSITY 2u /* a new conservative density was <= 0 or non-finite */

#define E2D_RIEMANN_APPROX 0 /* riemann_2d, serial_ref/m_utils.f90:349 (the reference's choice) */
#define E2D_RIEMANN_HLLC 2   /* riemann_2d_hllc, serial_ref/m_utils.f90:534 */

/* Parameters: the &RUN-independent fields of type HydroPar
 * (serial_ref/m_parameters.f90:10-36) as read by initHydroParameters
 * (serial_ref/m_run.f90:48-128), plus the cuf namelist key
 * implementationVersion (cuf/m_HydroParameters.cuf:90) and two keys of the
 * trailing &GB300 namelist group. */
typedef struct e2d_params {
  int nx, ny;
  double gamma0, cfl, smallr, smallc;
  int niter_riemann, iorder, slope_type;
  int boundary_type_xmin, boundary_type_xmax, boundary_type_ymin, boundary_type_ymax;
  int implementation_version; /* 0 fused recompute, 1 stored prim + face states, 2 stored prim + fluxes */
  int riemann_solver;         /* E2D_RIEMANN_APPROX or E2D_RIEMANN_HLLC */
  int precision;              /* 8 = FP64 (fp_kind = dp_kind), 4 = FP32 (sp_kind) */
} e2d_params;

typedef struct e2d_run e2d_run; /* opaque run handle: owns u, u2 and work arrays on one GPU */

/* Fill *p with the reference defaults of serial_ref/test.nml and
 * serial_ref/m_parameters.f90 (niter_riemann=10, reflective walls), FP64,
 * implementationVersion 0, approximate Riemann solver. */
int e2d_default_params(e2d_params* p);

/* Arithmetic of this build of the library.  Two builds share this ABI:
 * libeuler2d_gb300.so (E2D_ARITH_EXACT: no multiply-add contraction, every
 * operation rounded as serial_ref's gfortran build rounds it, results bitwise
 * those of serial_ref's arithmetic) and libeuler2d_gb300_fma.so
 * (E2D_ARITH_FMA: multiply-adds fused, as nvfortran's default -O3 GPU builds
 * of cuf/ and stdpar/ do -- cuf/Makefile:22, stdpar/Makefile:8 --, results
 * within 1e-12 relative L1 and dt within 1e-14 of the exact build).  A host
 * picks one at link time (-leuler2d_gb300 or -leuler2d_gb300_fma). */
#define E2D_ARITH_EXACT 0
#define E2D_ARITH_FMA 1
int e2d_arithmetic(int* mode);

/* initHydroParameters + run_init allocation (serial_ref/m_run.f90:48-128,150-158;
 * cuf/m_HydroRun_gpu.cuf:83-118).  Validates p, allocates u, u2 (zeroed, as fresh
 * allocate() pages) and the work arrays of the chosen implementation version on
 * the current CUDA device.  The running CFL maximum starts at 0. */
int e2d_create(const e2d_params* p, e2d_run** out);

/* run_cleanup (serial_ref/m_run.f90:172-182). Accepts NULL. */
int e2d_destroy(e2d_run* h);

/* Sizes of the run: isize, jsize and bytes of one host state array. */
int e2d_get_sizes(const e2d_run* h, int* isize, int* jsize, size_t* state_bytes);

/* Issue all later device work on `stream` (a cudaStream_t); NULL selects the
 * run's own non-blocking stream (the default). */
int e2d_set_stream(e2d_run* h, void* stream);
int e2d_synchronize(e2d_run* h);

/* init_implode (serial_ref/m_run.f90:524-555) on the device into u. */
int e2d_init_implode(e2d_run* h);
/* Generalised diagonal interface (high state where tmp > offset); offset 0.5,
 * (1,1) / (0.125, (double)0.14f) is init_implode. */
int e2d_init_diagonal(e2d_run* h, double offset, double rho_hi, double p_hi, double rho_lo,
                      double p_lo);

/* Host <-> device copies of u (which=0) or u2 (which=1), full arrays incl. ghosts. */
int e2d_upload_state(e2d_run* h, int which, const void* host);
int e2d_download_state(e2d_run* h, int which, void* host);

/* compute_dt (serial_ref/m_run.f90:248-312; cuf/m_HydroRun_gpu.cuf:198-300):
 * folds max over [3, size-3]^2 of (c+|u|)/dx + (c+|v|)/dy of u (useU=0) or u2
 * (useU=1) into the run's running maximum and returns dt = cfl / max in *dt
 * (a double* for precision 8, a float* for precision 4). */
int e2d_compute_dt(e2d_run* h, int useU, void* dt);

/* make_boundaries (serial_ref/m_run.f90:561-648; cuf make_boundaries_gpu
 * cuf/m_HydroRun_gpu.cuf:1041-1130) on u (which=0) or u2 (which=1). */
int e2d_make_boundaries(e2d_run* h, int which);

/* godunov_unsplit (serial_ref/m_run.f90:187-243; cuf/m_HydroRun_gpu.cuf:305-450):
 * one step from u to u2 (nStep even) or u2 to u (odd) with the given dt, by the
 * run's implementation version. */
int e2d_godunov_unsplit(e2d_run* h, int nStep, double dt);

/* The inner loop of serial_ref/main.f90:53-76 for steps nStep0 .. nStep0+nsteps-1,
 * entirely on the device: dt of each step comes from the running maximum, the
 * next step's CFL maximum is reduced inside the update kernel, and no host
 * synchronisation happens between steps (steps are replayed from a captured
 * CUDA graph).  If dt_log is non-NULL it receives the nsteps dt values
 * (double or float by precision) and the call synchronises. */
int e2d_advance(e2d_run* h, int nStep0, int nsteps, void* dt_log);

/* Device time in milliseconds of the last e2d_advance call, measured with CUDA
 * events recorded on the run's stream around its launches (synchronises). */
int e2d_last_advance_ms(e2d_run* h, float* ms);

/* The same device work as e2d_advance(nStep0, nsteps), launched step by step
 * without a graph, with CUDA events on the run's stream around the device work
 * of each step; ms[k] receives the time of step k (synchronises).  Used to
 * time the step kernel for the roofline. */
int e2d_time_steps(e2d_run* h, int nStep0, int nsteps, float* ms);

/* Measures this GPU's FP64 throughput (independent DFMA per second and IEEE
 * double divisions per second) on the current device: the roof that binds
 * the FP64 step.  Not part of the reference; used by the benchmark. */
int e2d_measure_fp64_peak(double* dfma_per_s, double* ddiv_per_s);

/* Self-test of the library's integer-pipe double division (op 0) and square
 * root (op 1) against the hardware operations, and of its exponent-test
 * pressure floor max(a, b*c) (op 2) and limiter sign test a*b <= 0 (op 3)
 * against the product (and maximum), on n seeded inputs (mode 0 any bit
 * pattern, 1 exponents near 1, 2 exponents within +-400, 3 results next to
 * rounding boundaries -- for op 2, a within two binades of b*c; for op 3,
 * products next to the underflow to zero --, 4 signed zeros and small
 * integers): *mismatches
 * counts results that differ in any bit, first_bad[4] (optional) = a, b,
 * library, reference operation of the first one; ops 4 and 5 (double) and 6
 * and 7 (single precision) check the faithful division and square root of the
 * library's FMA build, which must equal the hardware result or one of its two
 * neighbours.  The two rates (optional, ops 0, 1, 4, 5) are chained
 * operations per second.  Not part of the reference; used by the tests. */
int e2d_selftest_arith(int op, int mode, long long n, unsigned long long seed, unsigned long long* mismatches,
                       double* first_bad, double* emulated_per_s, double* native_per_s);

/* Self-test of the bounded wait every kernel wait goes through (the step
 * kernels' TMA wait gives up after about a second and raises health flag 4):
 * one mbarrier that receives its arrival must complete (*arrived_completed =
 * 1), one that nothing arrives on must give up after limit_cycles SM cycles
 * (*silent_completed = 0, *waited_cycles about limit_cycles), with no copy in
 * flight and the context usable afterwards.  Not part of the reference; used
 * by the tests of failure detection. */
int e2d_selftest_wait(long long limit_cycles, int* arrived_completed, int* silent_completed,
                      long long* waited_cycles);

/* Current running maximum of 1/dt (double, whatever the precision). */
int e2d_get_invdt(e2d_run* h, double* invdt);

/* Asynchronous output (serial_ref/m_run.f90:653-720 writes the state
 * synchronously): e2d_begin_download copies state `which` (0 = u, 1 = u2)
 * into a device snapshot in stream order, after the steps already issued,
 * then to `host` (Fortran layout) on a separate copy stream, and returns;
 * steps issued afterwards run while the transfer proceeds.  `host` should
 * come from e2d_host_alloc (pinned) for the copy to overlap.  The snapshot is
 * reused: a second e2d_begin_download first waits for the previous copy.
 * e2d_wait_download blocks until the last copy has landed in `host`. */
int e2d_begin_download(e2d_run* h, int which, void* host);
int e2d_wait_download(e2d_run* h);
int e2d_host_alloc(size_t bytes, void** ptr);
int e2d_host_free(void* ptr);

/* Health flags accumulated by the kernels since the last call (cleared on read). */
int e2d_get_health(e2d_run* h, unsigned* flags);

/* Human-readable text of the last error on this thread. */
const char* e2d_last_error(void);

/* Device pointers to u / u2 (pitched SoA planes) for in-process callers that
 * keep the state resident, with the row pitch in elements and plane stride. */
int e2d_device_state(e2d_run* h, int which, void** dptr, size_t* pitch_elems,
                     size_t* plane_elems);

/* ---- Batched ensemble: many independent runs of uneven sizes ----
 * No counterpart in the reference (which runs one problem per process): the
 * step of each problem is the one of e2d_godunov_unsplit with
 * implementationVersion 0 arithmetic, each problem has its own dt, running
 * CFL maximum, boundary types and ping-pong pair, and one kernel launch
 * advances every problem by one step (the tiles of all problems form one
 * work list walked by a persistent grid).  Problem p's states are selected by
 * `prob`; layouts as for single runs. */
typedef struct e2d_batch e2d_batch;

/* nprob problems with sizes nx[p] x ny[p]; bc (optional) holds 4 boundary
 * types per problem (xmin, xmax, ymin, ymax); the other fields come from base. */
int e2d_batch_create(const e2d_params* base, int nprob, const int* nx, const int* ny, const int* bc,
                     e2d_batch** out);
int e2d_batch_destroy(e2d_batch* b);
/* Diagonal interface per problem (e2d_init_diagonal with per-problem arrays). */
int e2d_batch_init_diagonal(e2d_batch* b, const double* offset, const double* rho_hi, const double* p_hi,
                            const double* rho_lo, const double* p_lo);
int e2d_batch_upload_state(e2d_batch* b, int prob, int which, const void* host);
int e2d_batch_download_state(e2d_batch* b, int prob, int which, void* host);
/* e2d_advance for every problem at once; dt_log (optional) receives
 * nsteps x nprob values (step-major). */
int e2d_batch_advance(e2d_batch* b, int nStep0, int nsteps, void* dt_log);
int e2d_batch_last_advance_ms(e2d_batch* b, float* ms);
/* Schedule: variant 0 = 32x15-cell tiles, 1 = 32x7; grid_mult x resident CTAs
 * per SM x SMs persistent CTAs, each walking one contiguous run of the tiles
 * (grid_mult 0: one CTA per tile); order 0 = problem order, 1 = largest
 * first. */
int e2d_batch_set_schedule(e2d_batch* b, int variant, int grid_mult, int order);
int e2d_batch_get_schedule(e2d_batch* b, int* variant, int* grid_mult, int* order, int* grid);
/* Autotuner: times every schedule on `steps` steps of the current states
 * (restored afterwards) and keeps the fastest; with cache_path, reuses and
 * records choices per ensemble shape. */
int e2d_batch_tune(e2d_batch* b, int steps, const char* cache_path, float* best_ms);
int e2d_batch_get_health(e2d_batch* b, int prob, unsigned* flags);

/* ---- Discrete adjoint (FP64, HLLC flux) ----
 * No counterpart in the reference.  Gradient of J = sum over interior cells of
 * rho^2 w(x, y) after nsteps steps, w(x, y) = exp(-((x-xc)^2 + (y-yc)^2) /
 * (2 sigma^2)) at cell centres x = (i + 1/2) dx, with respect to the initial
 * density of the interior cells, by hand-written reverse kernels of every
 * stage of the step and ceil(sqrt(nsteps)) state checkpoints with
 * recomputation.  dt_mode 0 keeps the dt of every step frozen; 1 also
 * differentiates dt = cfl / (running CFL maximum).  u0 is the initial state
 * (Fortran layout, ghosts included) or NULL for init_implode. */
typedef struct e2d_adjoint e2d_adjoint;
int e2d_adjoint_create(const e2d_params* p, e2d_adjoint** out);
int e2d_adjoint_destroy(e2d_adjoint* a);
/* J only (the forward run), e.g. for finite differences; with dt_fixed
 * (nsteps values) step n uses dt_fixed[n] instead of the CFL dt. */
int e2d_adjoint_objective(e2d_adjoint* a, const void* u0, int nsteps, double xc, double yc, double sigma,
                          const double* dt_fixed, double* J);
/* J and dJ/d rho0 (nx*ny values, i fastest); dt_log (optional) gets the dt of each step. */
int e2d_adjoint_gradient(e2d_adjoint* a, const void* u0, int nsteps, int dt_mode, double xc, double yc,
                         double sigma, double* J, double* grad_rho0, double* dt_log);
/* Device times (ms) of the last objective and gradient calls. */
int e2d_adjoint_last_ms(e2d_adjoint* a, float* objective_ms, float* gradient_ms);
/* Memory layout of the last gradient call: *segment_steps = K, the steps
 * between checkpoints (K = N when every state and its tape were kept and
 * nothing was recomputed); *tape = 1 when the reverse steps read the forward
 * values from a tape, 0 when they recompute them.  Not in the reference. */
int e2d_adjoint_layout(e2d_adjoint* a, int* segment_steps, int* tape);

/* ---- Batched adjoint: the adjoint of many independent problems at once ----
 * No counterpart in the reference.  Problems of uneven sizes (FP64, HLLC),
 * each with its own initial state, boundaries, dt and running CFL maximum,
 * all advanced by the same number of steps; each stage of the forward and
 * reverse sweeps is one launch over every problem, and one call is one
 * captured CUDA graph.  J_p and dJ_p/d rho0_p are as for e2d_adjoint_gradient;
 * the gradients are packed problem after problem (nx[p]*ny[p] values each,
 * i fastest), dt_log (optional) gets nsteps x nprob values (step-major). */
typedef struct e2d_adjoint_batch e2d_adjoint_batch;
int e2d_adjoint_batch_create(const e2d_params* base, int nprob, const int* nx, const int* ny, const int* bc,
                             e2d_adjoint_batch** out);
int e2d_adjoint_batch_destroy(e2d_adjoint_batch* b);
/* Initial states: diagonal interfaces with per-problem data, or one problem's
 * full state (Fortran layout, ghosts included). */
int e2d_adjoint_batch_init_diagonal(e2d_adjoint_batch* b, const double* offset, const double* rho_hi,
                                    const double* p_hi, const double* rho_lo, const double* p_lo);
int e2d_adjoint_batch_upload_state(e2d_adjoint_batch* b, int prob, const void* host);
/* The forward runs only (no checkpoints): J[nprob]. */
int e2d_adjoint_batch_objective(e2d_adjoint_batch* b, int nsteps, double xc, double yc, double sigma, double* J);
int e2d_adjoint_batch_gradient(e2d_adjoint_batch* b, int nsteps, int dt_mode, double xc, double yc, double sigma,
                               double* J, double* grad_rho0, double* dt_log);
int e2d_adjoint_batch_last_ms(e2d_adjoint_batch* b, float* objective_ms, float* gradient_ms);

/* One godunov_unsplit step (the stored-fluxes variant, implementationVersion 2
 * arithmetic) that allocates no device memory.  No counterpart in the
 * reference: it serves callers that cannot call cudaMalloc (device arrays owned
 * by another allocator or memory pool, or a host framework that forbids
 * allocation on its time-step path).  u_in and u_out are device arrays in the
 * pitched layout of e2d_device_state (4 planes of ny+4 rows of pitch_elems
 * elements, nx+4 <= pitch_elems <= INT_MAX), owned by the caller, that must
 * not overlap; make_boundaries is applied to u_in first, as the reference
 * does, and only the interior of u_out is written.  dt must be positive and
 * finite.  The work arrays live in one static device array of
 * E2D_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
 * exit; grids whose three work arrays (primitives and two flux arrays) do not
 * fit are rejected with E2D_ERR_INVALID_ARG.  All calls share that array:
 * calls that overlap on the GPU race.  The first call on a device (and the
 * first after a device reset) looks up the array's device address and should
 * come before any stream capture.  Work is issued on `stream` (a
 * cudaStream_t, NULL = legacy default stream) and not synchronised, unless
 * `health` is not NULL: the call then waits for the step and stores its
 * E2D_HEALTH_* flags there. */
#define E2D_NOALLOC_SCRATCH_BYTES (48u * 1024u * 1024u)
int e2d_godunov_unsplit_noalloc(const e2d_params* p, void* u_in, void* u_out, size_t pitch_elems, double dt,
                                void* stream, unsigned* health);

#ifdef __cplusplus
}
#endif
#endif
