// Host check of e2d::emul::mul_rn against the host's IEEE multiplication;
// built by tests/test_emul_host.py.  Prints "<bad> mismatches in <n>".
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "emul64.cuh"

using e2d::emul::mul_rn;

static uint64_t bits_of(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; }
static double of_bits(uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; }
static double with_exp(uint64_t r, int e) { return of_bits((r & 0x800fffffffffffffull) | ((uint64_t)e << 52)); }

int main(int argc, char** argv) {
  const long long per_mode = argc > 1 ? std::atoll(argv[1]) : 1000000;
  std::mt19937_64 g(20261203);
  long long bad = 0, n = 0;
  auto check = [&](double x, double y, const char* what) {
    const double e = mul_rn(x, y), h = x * y;
    ++n;
    if (!(bits_of(e) == bits_of(h) || (e != e && h != h))) {
      if (bad < 8) std::printf("%s: %a * %a = %a, IEEE %a\n", what, x, y, e, h);
      ++bad;
    }
  };
  for (long long k = 0; k < per_mode; ++k) {
    const uint64_t r1 = g(), r2 = g();
    check(of_bits(r1), of_bits(r2), "any bits");
    check(with_exp(r1, 983 + (int)((r1 >> 52) % 81)), with_exp(r2, 983 + (int)((r2 >> 52) % 81)), "near 1");
    check(with_exp(r1, 423 + (int)((r1 >> 52) % 1201)), with_exp(r2, 423 + (int)((r2 >> 52) % 1201)), "wide");
    check(of_bits((r1 & 0x800fffffc0000000ull) | ((uint64_t)(1000 + (r1 >> 52) % 48) << 52)),
          of_bits((r2 & 0x800ffffff8000000ull) | ((uint64_t)(1000 + (r2 >> 52) % 48) << 52)), "ties");
    double z = (r1 & 4) ? 0.0 : (double)(int)((r1 >> 8) & 7);
    if (r1 & 1) z = -z;
    check(z, of_bits(r2), "zeros");
    const int ex = 1 + (int)((r1 >> 52) % 2046);
    int ey = 3069 - ex + (int)(r2 >> 60) - 8;  // product near the overflow threshold
    ey = ey < 1 ? 1 : ey > 2046 ? 2046 : ey;
    check(with_exp(r1, ex), with_exp(r2, ey), "overflow edge");
    ey = 1024 - ex + (int)(r2 >> 60) - 8 + 1;  // product near the underflow threshold
    ey = ey < 1 ? 1 : ey > 2046 ? 2046 : ey;
    check(with_exp(r1, ex), with_exp(r2, ey), "underflow edge");
  }
  std::printf("%lld mismatches in %lld\n", bad, n);
  return bad != 0;
}
