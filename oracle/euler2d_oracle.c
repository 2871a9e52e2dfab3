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
#include <math.h>
#include <stdlib.h>
#include <stddef.h>
#include "euler2d_oracle.h"

/* Variable indices, 0-based (serial_ref/m_constants.f90:11-14: ID=1, IP=2, IU=3, IV=4). */
enum { ID = 0, IP = 1, IU = 2, IV = 3 };

#define REAL double
#define SFX(name) name##_f64
#define RMAX(a, b) fmax((a), (b))
#define RMIN(a, b) fmin((a), (b))
#define RABS(a) fabs(a)
#define RSQRT(a) sqrt(a)
#include "oracle_impl.inc"
#undef REAL
#undef SFX
#undef RMAX
#undef RMIN
#undef RABS
#undef RSQRT

#define REAL float
#define SFX(name) name##_f32
#define RMAX(a, b) fmaxf((a), (b))
#define RMIN(a, b) fminf((a), (b))
#define RABS(a) fabsf(a)
#define RSQRT(a) sqrtf(a)
#include "oracle_impl.inc"
