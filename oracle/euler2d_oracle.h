/*
 * euler2d_oracle.h -- CPU oracle for the Euler-2D explicit step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker against which the
 * CUDA path is compared.  Only the tests, the smoke check and the CPU-baseline
 * leg of bench.py may load it; the product library never links or calls it.
 *
 * It restates, routine by routine and expression by expression, the plain
 * Fortran serial version of pkestene/euler2d_cudaFortran (serial_ref/), built
 * with fp_kind = dp_kind (the _f64 entry points) or sp_kind (_f32).
 * Arrays use the Fortran layout A(isize, jsize, NBVAR), column-major:
 * element (i, j, v) (1-based) lives at ((v-1)*jsize + (j-1))*isize + (i-1),
 * with the variable order ID=1 (rho), IP=2 (E in u / p in q), IU=3, IV=4
 * (serial_ref/m_constants.f90:11-14).
 *
 * Parity status: the reference has no tests, golden vectors or fixtures, and
 * no Fortran compiler is available to run it, so this restatement is
 * "parity unpinned" against the reference binary; it is pinned instead by
 * hand-derived known-answer cases and invariants in tests/test_oracle.py.
 */
#ifndef EULER2D_ORACLE_H
#define EULER2D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Run parameters, as read from the &RUN/&MESH/&HYDRO namelist groups
 * (serial_ref/m_run.f90:71-92).  Derived values (smallp, smallpp, gamma6,
 * dx, dy, isize, jsize) are computed inside the oracle in the working
 * precision, as serial_ref/m_run.f90:103-124 does. */
typedef struct {
  int nx, ny;
  double gamma0, cfl, smallr, smallc;
  int niter_riemann, iorder, slope_type;
  int bc_xmin, bc_xmax, bc_ymin, bc_ymax; /* 1 reflective, 2 outflow, else periodic */
  int riemann;                            /* 0 two-shock approx (reference), 2 HLLC */
} oracle_params;

/* ---- whole-array sweeps (one call = one sweep of serial_ref/m_run.f90) ---- */
void oracle_init_implode_f64(const oracle_params* p, double* u);
void oracle_init_implode_f32(const oracle_params* p, float* u);
/* Generalised diagonal interface: high state where tmp > offset.  With
 * offset 0.5, (1, 1) and (0.125, (double)0.14f) it equals init_implode. */
void oracle_init_diagonal_f64(const oracle_params* p, double* u, double offset,
                              double rho_hi, double p_hi, double rho_lo, double p_lo);
void oracle_init_diagonal_f32(const oracle_params* p, float* u, double offset,
                              double rho_hi, double p_hi, double rho_lo, double p_lo);
void oracle_make_boundaries_f64(const oracle_params* p, double* u);
void oracle_make_boundaries_f32(const oracle_params* p, float* u);
/* compute_dt with the SAVEd running maximum passed explicitly in *invdt. */
void oracle_compute_dt_f64(const oracle_params* p, const double* u, double* invdt, double* dt, int nthreads);
void oracle_compute_dt_f32(const oracle_params* p, const float* u, float* invdt, float* dt, int nthreads);
void oracle_convert_to_primitives_f64(const oracle_params* p, const double* u, double* q, int nthreads);
void oracle_convert_to_primitives_f32(const oracle_params* p, const float* u, float* q, int nthreads);
void oracle_compute_and_store_fluxes_f64(const oracle_params* p, const double* q, double dt,
                                         double* fx, double* fy, int nthreads);
void oracle_compute_and_store_fluxes_f32(const oracle_params* p, const float* q, float dt,
                                         float* fx, float* fy, int nthreads);
void oracle_update_hydro_f64(const oracle_params* p, const double* in, const double* fx,
                             const double* fy, double* out, int nthreads);
void oracle_update_hydro_f32(const oracle_params* p, const float* in, const float* fx,
                             const float* fy, float* out, int nthreads);
/* One godunov_unsplit_cpu step (boundaries on `in`, primitives, fluxes, update). */
void oracle_godunov_step_f64(const oracle_params* p, double* in, double* out, double dt, int nthreads);
void oracle_godunov_step_f32(const oracle_params* p, float* in, float* out, float dt, int nthreads);

/* The HydroRun driver loop of serial_ref/main.f90:42-76 without I/O.
 * u holds the initial state on entry; u2 is used as given (callers zero it,
 * matching fresh allocate() pages).  *invdt carries the running maximum
 * (0 for a fresh run).  dt_log[n] receives the dt of step n (may be NULL).
 * After an even number of steps the final state is in u, else in u2. */
int oracle_run_f64(const oracle_params* p, int nsteps, double* u, double* u2,
                   double* invdt, double* dt_log, int nthreads);
int oracle_run_f32(const oracle_params* p, int nsteps, float* u, float* u2,
                   float* invdt, float* dt_log, int nthreads);

/* J = sum over interior cells of rho^2 w(x, y) (Gaussian w of width sig at (xc, yc)). */
double oracle_objective_f64(const oracle_params* p, const double* u, double xc, double yc, double sig);

/* euler2d_oracle.c also exports a complex-step (forward-mode tangent) build of
 * the same routines with the suffix _c128 (oracle_run_c128,
 * oracle_objective_c128, ...): arguments as for _f64 with every double array
 * or scalar of the state replaced by double complex; the imaginary parts
 * carry the directional derivatives. */

/* ---- pointwise routines (serial_ref/m_utils.f90), for unit tests ---- */
void oracle_primitives_f64(const oracle_params* p, const double u[4], double q[4], double* c);
void oracle_primitives_f32(const oracle_params* p, const float u[4], float q[4], float* c);
void oracle_slopes_f64(const oracle_params* p, const double q[4], const double qpx[4],
                       const double qmx[4], const double qpy[4], const double qmy[4],
                       double dqx[4], double dqy[4]);
void oracle_slopes_f32(const oracle_params* p, const float q[4], const float qpx[4],
                       const float qmx[4], const float qpy[4], const float qmy[4],
                       float dqx[4], float dqy[4]);
void oracle_trace_f64(const oracle_params* p, const double q[4], const double dqx[4],
                      const double dqy[4], double dtdx, double dtdy, int face, double qf[4]);
void oracle_trace_f32(const oracle_params* p, const float q[4], const float dqx[4],
                      const float dqy[4], float dtdx, float dtdy, int face, float qf[4]);
/* Riemann solvers; *niter (may be NULL) receives the Newton iteration count. */
void oracle_riemann_approx_f64(const oracle_params* p, const double ql[4], const double qr[4],
                               double flux[4], int* niter);
void oracle_riemann_approx_f32(const oracle_params* p, const float ql[4], const float qr[4],
                               float flux[4], int* niter);
void oracle_riemann_hllc_f64(const oracle_params* p, const double ql[4], const double qr[4],
                             double flux[4]);
void oracle_riemann_hllc_f32(const oracle_params* p, const float ql[4], const float qr[4],
                             float flux[4]);

#ifdef __cplusplus
}
#endif
#endif
