// k_selftest.cu -- on-device check of the emulated double division and square
// root (emul64.cuh) against the hardware operations, bit for bit, plus their
// throughput, and of the exponent-test pressure floor (physics.cuh) against
// the product and maximum it stands for.  Exposed as e2d_selftest_arith for
// the GPU tests.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/euler2d_gb300.h"
#include "emul64.cuh"
#include "physics.cuh"
#include "sync.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Random double: mode 0 any finite/special bit pattern, mode 1 exponent within
// +-40 of 1, mode 2 exponent within +-400 of 1.
__device__ double rand_double(uint64_t r, int mode) {
  if (mode == 0) return __longlong_as_double((long long)r);
  const int span = mode == 1 ? 40 : 400;
  const uint64_t e = (uint64_t)(1023 - span + (int)((r >> 52) % (uint64_t)(2 * span + 1)));
  return __longlong_as_double((long long)((r & 0x800fffffffffffffull) | (e << 52)));
}

__device__ bool same(double x, double y) {
  const uint64_t a = (uint64_t)__double_as_longlong(x), b = (uint64_t)__double_as_longlong(y);
  if (x != x && y != y) return true;  // both NaN
  return a == b;
}

// op 0: division, op 1: square root (both bit for bit), op 4 / op 5: the
// faithful division and square root (equal to the hardware result or one of
// its two neighbours), op 6 / op 7: the same for single precision, op 2: the
// pressure floor max(a, b*c)
// (against the emulated maximum of the hardware product), op 3: the
// limiter's sign test dlft*drgt <= 0 from signs and exponents (the product
// taken where it reports the undecided band), against the product (mode 3:
// exponent sums next to the underflow band, either sign).  Modes 0-2 as
// rand_double; mode 4 signed zeros and small integers; mode 3 builds
// operands whose exact result lies within one part in 2^60 of a rounding
// boundary (quotient q + 1/2 ulp times b, or (q + 1/2 ulp)^2), and for op 2
// an a within two binades of b*c, either sign.
__global__ void k_check(int op, int mode, long long n, uint64_t seed, unsigned long long* bad, double* first) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const uint64_t r1 = mix64(seed ^ (uint64_t)k), r2 = mix64(r1 + 0x1234567ull);
    double a, b = 1.0;
    if (op == 2) {
      const uint64_t r3 = mix64(r2 + 0x7654321ull);
      b = rand_double(r2, mode == 0 ? 0 : mode == 4 ? 2 : 1);
      const double c = rand_double(r3, mode == 0 ? 0 : 2);
      if (mode == 3) {  // a = +-(b*c) with its exponent moved by -2..2 and a fresh mantissa
        const long long pb = __double_as_longlong(__dmul_rn(b, c));
        const long long e = ((pb >> 52) & 0x7ff) + (long long)(r1 % 5) - 2;
        a = (e > 0 && e < 2047) ? __longlong_as_double((long long)(r1 & 0x800fffffffffffffull) | (e << 52)) : 1.0;
      } else if (mode == 4) {
        a = (r1 & 2) ? 0.0 : rand_double(r1, 2);
        a = (r1 & 1) ? -a : a;
      } else {
        a = rand_double(r1, mode);
      }
      const double x = e2d::floor_prod<double>(a, b, c);
      const double y = e2d::emul::max_i(a, __dmul_rn(b, c));
      if (!same(x, y)) {
        if (atomicAdd(bad, 1ull) == 0) { first[0] = a; first[1] = b; first[2] = x; first[3] = y; }
      }
      continue;
    }
    if (op == 3) {
      a = rand_double(r1, mode == 3 ? 0 : mode == 4 ? 2 : mode);
      b = rand_double(r2, mode == 3 ? 0 : mode == 4 ? 0 : mode);
      if (mode == 3) {  // biased exponent sum within 966..975, subnormal and zero factors among them
        const long long ea = (long long)(r1 % 976);
        const long long eb = 966 + (long long)(r2 % 10) - ea;
        a = __longlong_as_double((long long)(r1 & 0x800fffffffffffffull) | (ea << 52));
        b = __longlong_as_double((long long)(r2 & 0x800fffffffffffffull) | ((eb < 0 ? 0 : eb > 2046 ? 2046 : eb) << 52));
      } else if (mode == 4) {
        a = (r1 & 2) ? ((r1 & 1) ? -0.0 : 0.0) : a;
      }
      bool amb = false;
      bool x = e2d::prod_le0(a, b, amb);
      if (amb) x = __dmul_rn(a, b) <= 0.0;
      const bool y = __dmul_rn(a, b) <= 0.0;
      if (x != y) {
        if (atomicAdd(bad, 1ull) == 0) { first[0] = a; first[1] = b; first[2] = x; first[3] = y; }
      }
      continue;
    }
    if (op >= 6) {  // single precision, faithful: 6 division, 7 square root
      float fa, fb = 1.0f;
      if (mode == 0) {
        fa = __uint_as_float((unsigned)r1); fb = __uint_as_float((unsigned)r2);
      } else if (mode == 1 || mode == 2) {  // exponents within +-20 (1) or +-100 (2) of 1
        const unsigned span = mode == 1 ? 20u : 100u;
        fa = __uint_as_float(((unsigned)r1 & 0x807fffffu) | ((127u - span + (unsigned)((r1 >> 40) % (2 * span + 1))) << 23));
        fb = __uint_as_float(((unsigned)r2 & 0x807fffffu) | ((127u - span + (unsigned)((r2 >> 40) % (2 * span + 1))) << 23));
      } else if (mode == 4) {  // signed zeros and small integers over random denominators
        fa = (r1 & 4) ? 0.0f : (float)(int)((r1 >> 8) & 7);
        fa = (r1 & 1) ? -fa : fa;
        fb = __uint_as_float(((unsigned)r2 & 0x807fffffu) | ((107u + (unsigned)((r2 >> 40) % 41)) << 23));
        if (op == 7) fa = fabsf(fa);
      } else {  // results next to a rounding boundary
        const float q = __uint_as_float(((unsigned)r1 & 0x007fffffu) | ((117u + (unsigned)((r1 >> 40) % 21)) << 23));
        const float h = 0.5f * (__uint_as_float(__float_as_uint(q) + 1) - q);
        if (op == 6) {
          fb = __uint_as_float(((unsigned)r2 & 0x807fffffu) | ((117u + (unsigned)((r2 >> 40) % 21)) << 23));
          fa = (float)((double)(q + h) * (double)fb);  // (q + half an ulp) * b, rounded once to float
        } else {
          fa = (float)((double)q * (double)q + (double)q * (double)(2.0f * h));  // ~ (q + h)^2
        }
        fa = __uint_as_float(__float_as_uint(fa) + (unsigned)(r2 & 3) - 1u);
      }
      const float fx = op == 6 ? e2d::emul::fdiv_fa(fa, fb) : e2d::emul::fsqrt_fa(fa);
      const float fy = op == 6 ? __fdiv_rn(fa, fb) : __fsqrt_rn(fa);
      const unsigned ix = __float_as_uint(fx), iy = __float_as_uint(fy);
      const bool ok = ix == iy || (fx != fx && fy != fy) ||
                      (fx == fx && fy == fy && ((ix ^ iy) >> 31) == 0 && (ix - iy == 1u || iy - ix == 1u));
      if (!ok) {
        if (atomicAdd(bad, 1ull) == 0) { first[0] = fa; first[1] = fb; first[2] = fx; first[3] = fy; }
      }
      continue;
    }
    const bool faithful = op >= 4;
    const int bop = faithful ? op - 4 : op;  // 0: division, 1: square root
    if (mode < 3) {
      a = rand_double(r1, mode);
      b = rand_double(r2, mode);
    } else if (mode == 4) {  // signed zeros and small integers over random denominators
      a = (r1 & 4) ? 0.0 : (double)(int)((r1 >> 8) & 7);
      a = (r1 & 1) ? -a : a;
      b = rand_double(r2, (r2 & 1) ? 0 : 2);
      if (bop == 1) a = (r1 & 4) ? a : (double)((r1 >> 8) & 7);
    } else if (bop == 0) {
      b = rand_double(r2, 1);
      const double q = rand_double(r1, 1);
      const double qm = q + 0.5 * (__longlong_as_double(__double_as_longlong(q) + 1) - q);  // rounds to a neighbour
      a = __dmul_rn(qm, b);
      a = __longlong_as_double(__double_as_longlong(a) + (long long)(r1 & 3) - 1);
    } else {
      const double q = fabs(rand_double(r1, 1));
      const double h = 0.5 * (__longlong_as_double(__double_as_longlong(q) + 1) - q);
      a = __dmul_rn(q + h, q + h);
      a = __longlong_as_double(__double_as_longlong(a) + (long long)(r2 & 3) - 1);
    }
    const double x = bop == 0 ? (faithful ? e2d::emul::div_fa(a, b) : e2d::emul::div_rn(a, b))
                              : (faithful ? e2d::emul::sqrt_fa(a) : e2d::emul::sqrt_rn(a));
    const double y = bop == 0 ? __ddiv_rn(a, b) : __dsqrt_rn(a);
    bool ok = same(x, y);
    if (!ok && faithful) {  // a neighbour of the correctly rounded result: patterns one apart, same sign
      const long long ix = __double_as_longlong(x), iy = __double_as_longlong(y);
      ok = x == x && y == y && (ix ^ iy) >= 0 && (ix - iy == 1 || iy - ix == 1);
    }
    if (!ok) {
      if (atomicAdd(bad, 1ull) == 0) { first[0] = a; first[1] = b; first[2] = x; first[3] = y; }
    }
  }
}

__global__ void k_rate(int op, int emulated, int iters, double* out) {
  double x0 = 1.0 + threadIdx.x * 1e-3, x1 = x0 + 0.25, x2 = x0 + 0.5, x3 = x0 + 0.75;
  const double c = 0.999;
  for (int i = 0; i < iters; ++i) {
    if (op == 4 && emulated) {
      x0 = e2d::emul::div_fa(c, x0) + 1.0; x1 = e2d::emul::div_fa(c, x1) + 1.0;
      x2 = e2d::emul::div_fa(c, x2) + 1.0; x3 = e2d::emul::div_fa(c, x3) + 1.0;
    } else if (op == 5 && emulated) {
      x0 = e2d::emul::sqrt_fa(x0) + 1.0; x1 = e2d::emul::sqrt_fa(x1) + 1.0;
      x2 = e2d::emul::sqrt_fa(x2) + 1.0; x3 = e2d::emul::sqrt_fa(x3) + 1.0;
    } else if (op == 0 || op == 4) {
      if (emulated) {
        x0 = e2d::emul::div_rn(c, x0) + 1.0; x1 = e2d::emul::div_rn(c, x1) + 1.0;
        x2 = e2d::emul::div_rn(c, x2) + 1.0; x3 = e2d::emul::div_rn(c, x3) + 1.0;
      } else {
        x0 = c / x0 + 1.0; x1 = c / x1 + 1.0; x2 = c / x2 + 1.0; x3 = c / x3 + 1.0;
      }
    } else {
      if (emulated) {
        x0 = e2d::emul::sqrt_rn(x0) + 1.0; x1 = e2d::emul::sqrt_rn(x1) + 1.0;
        x2 = e2d::emul::sqrt_rn(x2) + 1.0; x3 = e2d::emul::sqrt_rn(x3) + 1.0;
      } else {
        x0 = sqrt(x0) + 1.0; x1 = sqrt(x1) + 1.0; x2 = sqrt(x2) + 1.0; x3 = sqrt(x3) + 1.0;
      }
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

// The bounded mbarrier wait of the step kernels, exercised without any copy
// in flight: barrier A receives its single arrival and must complete at once;
// barrier B is never arrived on (a flag nothing sets) and the wait must give
// up after limit_cycles.  out[0] = A completed, out[1] = B completed,
// out[2] = cycles spent waiting on B.
__global__ void k_wait_probe(long long limit_cycles, long long* out) {
  __shared__ __align__(8) uint64_t bars[2];
  if (threadIdx.x != 0) return;
  const uint32_t a = e2d::smem_u32(&bars[0]), b = e2d::smem_u32(&bars[1]);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
  out[0] = e2d::mbar_wait(a, 0, limit_cycles) ? 1 : 0;
  const long long t0 = clock64();
  out[1] = e2d::mbar_wait(b, 0, limit_cycles) ? 1 : 0;
  out[2] = clock64() - t0;
}

}  // namespace

extern "C" int e2d_selftest_wait(long long limit_cycles, int* arrived_completed, int* silent_completed,
                                 long long* waited_cycles) {
  if (limit_cycles < 1 || limit_cycles > (1ll << 32) || !arrived_completed || !silent_completed)
    return E2D_ERR_INVALID_ARG;
  long long* d = nullptr;
  if (cudaMalloc(&d, 3 * sizeof(long long)) != cudaSuccess) {
    cudaGetLastError();
    return E2D_ERR_NO_DEVICE;
  }
  long long h[3] = {0, 0, 0};
  k_wait_probe<<<1, 32>>>(limit_cycles, d);
  const bool ok = cudaGetLastError() == cudaSuccess &&
                  cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok) return E2D_ERR_CUDA;
  *arrived_completed = (int)h[0];
  *silent_completed = (int)h[1];
  if (waited_cycles) *waited_cycles = h[2];
  return E2D_OK;
}

extern "C" int e2d_selftest_arith(int op, int mode, long long n, unsigned long long seed,
                                  unsigned long long* mismatches, double* first_bad, double* emulated_per_s,
                                  double* native_per_s) {
  if (op < 0 || op > 7 || mode < 0 || mode > 4 || n < 0 || !mismatches) return E2D_ERR_INVALID_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return E2D_ERR_NO_DEVICE;
  }
  unsigned long long* d_bad = nullptr;
  double* d_first = nullptr;
  double* d_out = nullptr;
  const int threads = 256, blocks = sms * 8;
  if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&d_first, 4 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_out, (size_t)threads * blocks * sizeof(double)) != cudaSuccess) {
    cudaFree(d_bad);
    cudaFree(d_first);
    cudaGetLastError();
    return E2D_ERR_OOM;
  }
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  cudaMemset(d_first, 0, 4 * sizeof(double));
  k_check<<<blocks, threads>>>(op, mode, n, seed, d_bad, d_first);
  cudaMemcpy(mismatches, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  if (first_bad) cudaMemcpy(first_bad, d_first, 4 * sizeof(double), cudaMemcpyDeviceToHost);
  if (emulated_per_s && native_per_s && (op < 2 || op == 4 || op == 5)) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = 400;
    for (int emulated = 0; emulated < 2; ++emulated) {
      k_rate<<<blocks, threads>>>(op, emulated, 8, d_out);
      cudaEventRecord(e0);
      k_rate<<<blocks, threads>>>(op, emulated, iters, d_out);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      const double rate = (double)threads * blocks * iters * 4 / (ms * 1e-3);
      *(emulated ? emulated_per_s : native_per_s) = rate;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(d_bad);
  cudaFree(d_first);
  cudaFree(d_out);
  return e == cudaSuccess ? E2D_OK : E2D_ERR_CUDA;
}
