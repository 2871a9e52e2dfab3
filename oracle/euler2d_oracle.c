/*
 * euler2d_oracle.c -- CPU oracle for the Euler-2D explicit step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (see
 * euler2d_oracle.h).  Build with -ffp-contract=off (oracle/Makefile) so that
 * every multiply and add rounds separately, as gfortran does on x86-64.
 * OpenMP parallelises the outer j loops the way stdpar/m_run.f90:272,340,390,505
 * parallelises them with do concurrent; maxima and per-cell arithmetic are
 * order independent, so results are bitwise identical for any thread count.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stddef.h>
#include "euler2d_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

/* Variable indices, 0-based (serial_ref/m_constants.f90:11-14: ID=1, IP=2, IU=3, IV=4). */
enum { ID = 0, IP = 1, IU = 2, IV = 3 };

#define REAL double
#define SFX(name) name##_f64
#define RMAX(a, b) fmax((a), (b))
#define RMAXKEEP(a, b) ((b) > (a) ? (b) : (a))
#define RMIN(a, b) fmin((a), (b))
#define RABS(a) fabs(a)
#define RSQRT(a) sqrt(a)
#define RGT(a, b) ((a) > (b))
#define RGE(a, b) ((a) >= (b))
#define RLT(a, b) ((a) < (b))
#define RLE(a, b) ((a) <= (b))
#include "oracle_impl.inc"
#undef REAL
#undef SFX
#undef RMAX
#undef RMAXKEEP
#undef RMIN
#undef RABS
#undef RSQRT

#define REAL float
#define SFX(name) name##_f32
#define RMAX(a, b) fmaxf((a), (b))
#define RMAXKEEP(a, b) ((b) > (a) ? (b) : (a))
#define RMIN(a, b) fminf((a), (b))
#define RABS(a) fabsf(a)
#define RSQRT(a) sqrtf(a)
#include "oracle_impl.inc"
#undef REAL
#undef SFX
#undef RMAX
#undef RMAXKEEP
#undef RMIN
#undef RABS
#undef RSQRT
#undef RGT
#undef RGE
#undef RLT
#undef RLE

/* Complex-step instantiation (forward-mode tangent): every comparison, max,
 * min and |x| acts on the real part, so a state u + i h d (h tiny) carries
 * the directional derivative along d in its imaginary part through every
 * branch the real computation takes, including dt through the running max.
 * max/min of equal real parts return the second argument, with -0 ordered
 * below +0, which is the selection the library's kernels make, so the
 * derivative at ties is the one the adjoint uses. */
static inline long long ord_bits(double x) {
  long long b;
  memcpy(&b, &x, sizeof b);
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
#define REAL double complex
#define SFX(name) name##_c128
#define RMAX(a, b) (ord_bits(creal(a)) > ord_bits(creal(b)) ? (a) : (b))
#define RMAXKEEP(a, b) (creal(b) > creal(a) ? (b) : (a))
#define RMIN(a, b) (ord_bits(creal(a)) < ord_bits(creal(b)) ? (a) : (b))
#define RABS(a) (creal(a) < 0.0 ? -(a) : (a))
#define RSQRT(a) csqrt(a)
#define RGT(a, b) (creal(a) > creal(b))
#define RGE(a, b) (creal(a) >= creal(b))
#define RLT(a, b) (creal(a) < creal(b))
#define RLE(a, b) (creal(a) <= creal(b))
#include "oracle_impl.inc"

double oracle_objective_f64(const oracle_params* p, const double* u, double xc, double yc, double sig) {
  double out;
  oracle_objective_into_f64(p, u, xc, yc, sig, &out);
  return out;
}
