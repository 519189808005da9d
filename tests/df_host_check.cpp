// Host build of the double-float helpers (scale-dg-kernel-extraction_gb300/
// csrc/sdg_df.cuh), compiled with g++ -ffp-contract=off by test_df_host.py.
// Checks, over random doubles, that df_split carries x to 2^-48 relative in
// its documented range, that it agrees with the FP64-pipe split
// df_from_double to that accuracy, that f32_to_f64_bits widens exactly, and
// that the compensated dot product beats plain FP32 by the expected margin.
#include <cmath>
#include <cstdio>
#include <random>

#include "sdg_df.cuh"

using namespace sdg;

int main() {
  std::mt19937_64 g(20261203);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const double tol = std::ldexp(1.0, -48);
  long bad = 0;
  double worst = 0.0;
  for (long i = 0; i < 2000000; i++) {
    double x = U(g) * std::ldexp(1.0, (int)(g() % 140) - 70);
    if (i % 5 == 0) x = std::ldexp(std::floor(U(g) * 1e9), (int)(g() % 60) - 30);
    const dfl a = df_split(x);
    if ((double)a.hi != f32_to_f64_bits(a.hi) || (double)a.lo != f32_to_f64_bits(a.lo)) {
      std::printf("FAIL widen %a\n", x);
      return 1;
    }
    if (std::fabs(x) < std::ldexp(1.0, -74)) continue;
    const long double s = (long double)a.hi + (long double)a.lo;
    const double rel = (double)fabsl((s - (long double)x) / (long double)x);
    if (rel > worst) worst = rel;
    if (rel > tol) bad++;
    const dfl b = df_from_double(x);
    const long double sb = (long double)b.hi + (long double)b.lo;
    if ((double)fabsl((sb - s) / (long double)x) > 2 * tol) bad++;
  }
  // zero, signs and the flush range
  if (df_split(0.0).hi != 0.0f || df_split(-0.0).lo != 0.0f || df_split(1e-40).hi != 0.0f) {
    std::printf("FAIL specials\n");
    return 1;
  }
  // compensated dot product of an ill-conditioned sum (sum ~ 1e-6 of terms ~ 1)
  double worst_dot = 0.0;
  for (int t = 0; t < 20000; t++) {
    dacc A = dacc_zero();
    long double exact = 0.0L;
    for (int l = 0; l < 16; l++) {
      const double a = U(g), b = U(g);
      const dfl da = df_split(a), db = df_split(b);
      dacc_fma(A, da, db);
      exact += ((long double)da.hi + da.lo) * ((long double)db.hi + db.lo);
    }
    const dfl r = dacc_result(A);
    const long double got = (long double)r.hi + r.lo;
    const double err = (double)fabsl(got - exact);
    if (err > worst_dot) worst_dot = err;
  }
  std::printf("worst split rel %.3e, worst dot abs %.3e, bad %ld\n", worst, worst_dot, bad);
  return (bad == 0 && worst_dot < 1e-12) ? 0 : 1;
}
