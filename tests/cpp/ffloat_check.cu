// Host check of the float-float arithmetic of edgpu_internal.cuh (the vectors of the mixed mode's
// recurrences): sums, products, multiply-accumulate chains and renormalisation against long-double
// references on seeded random operands, including cancellations.  Prints the largest relative errors and
// exits non-zero when one exceeds its bound.  Built and run by tests/test_ffloat_cpu.py (host code only).
#include <cmath>
#include <cstdio>
#include <random>
#include "../../edlib_gb300/csrc/edgpu_internal.cuh"

using edgpu::ffloat;

static long double val(ffloat a) { return (long double)a.hi + (long double)a.lo; }

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-20, 20);
  double e_split = 0, e_add = 0, e_mul = 0, e_acc = 0, e_cancel = 0, e_renorm_rel = 0;
  for (int it = 0; it < 200000; ++it) {
    const double x = std::ldexp(u(rng), ex(rng)), y = std::ldexp(u(rng), ex(rng));
    const ffloat a(x), b(y);
    e_split = std::fmax(e_split, (double)(std::fabs(val(a) - (long double)x) / std::fabs((long double)x)));
    const long double s = (long double)x + (long double)y;
    if (s != 0) e_add = std::fmax(e_add, (double)(std::fabs(val(a + b) - s) / (std::fabs((long double)x) + std::fabs((long double)y))));
    const long double p = (long double)x * (long double)y;
    if (p != 0) e_mul = std::fmax(e_mul, (double)(std::fabs(val(a * b) - p) / std::fabs(p)));
    // a multiply-accumulate chain of 16 terms, as the operator sums an element
    ffloat acc(0.0);
    long double ref = 0, mag = 0;
    for (int k = 0; k < 16; ++k) {
      const double v = u(rng), w = std::ldexp(u(rng), ex(rng) / 4);
      acc += ffloat(v) * ffloat(w);
      ref += (long double)v * (long double)w;
      mag += std::fabs((long double)v * (long double)w);
    }
    e_acc = std::fmax(e_acc, (double)(std::fabs(val(acc) - ref) / mag));
    // cancellation: (x + d) - x, then renormalised
    const double d = std::ldexp(u(rng), -30) * std::fabs(x);
    const ffloat c = edgpu::renorm((ffloat(x) + ffloat(d)) - ffloat(x));
    if (d != 0) e_cancel = std::fmax(e_cancel, (double)(std::fabs(val(c) - (long double)d) / std::fabs((long double)x)));
    const ffloat r = edgpu::renorm(a * b);
    if (r.hi != 0) e_renorm_rel = std::fmax(e_renorm_rel, std::fabs((double)r.lo) / std::fabs((double)r.hi));
  }
  const double u48 = std::ldexp(1.0, -48);
  std::printf("split %.3g add %.3g mul %.3g mac16 %.3g cancel %.3g renorm |lo/hi| %.3g (2^-48 = %.3g)\n", e_split,
              e_add, e_mul, e_acc, e_cancel, e_renorm_rel, u48);
  const bool ok = e_split <= u48 && e_add <= 4 * u48 && e_mul <= 8 * u48 && e_acc <= 32 * u48 && e_cancel <= 4 * u48 &&
                  e_renorm_rel <= std::ldexp(1.0, -23);
  return ok ? 0 : 1;
}
