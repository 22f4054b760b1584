// Host check of the division-free superbee slope of the fast binary64 step
// (rt_fast.cuh): superbee_slope64(Rj, up) must equal phi(up/Rj)*Rj exactly,
// where phi(r) = max(0, min(1,2r), min(2,r)) (superbee_fluxes.f90:10), and
// stay within rounding of the reference's division form
//   Cr = up/Rj (Rj /= 0), Cr = up*1.E20 (Rj == 0); phi(Cr)*Rj.
#include <cmath>
#include <cstdio>
#include <random>

#include "rt_fast.cuh"

using namespace rt;

// exact value from the case analysis with binary64 comparisons
static double exact_slope(double Rj, double up) {
  if (Rj == 0.0) return 0.0;
  if ((Rj > 0) != (up > 0) || up == 0.0) return 0.0;
  const double a = std::fabs(Rj), t = std::fabs(up);
  const double m = std::fmax(std::fmin(a, 2 * t), std::fmin(2 * a, t));
  return Rj > 0 ? m : -m;
}

static double reference_slope(double Rj, double up) {
  double Cr = Rj != 0.0 ? up / Rj : up * 1.0000000200408773e20;
  Cr = std::fmax(0.0, std::fmax(std::fmin(1.0, 2.0 * Cr), std::fmin(2.0, Cr)));
  return Cr * Rj;
}

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-60, 20);
  long fails = 0, n = 0;
  auto check = [&](double Rj, double up) {
    n++;
    const double got = superbee_slope64(Rj, up);
    const double want = exact_slope(Rj, up);
    if (!(got == want)) {
      if (fails < 20) std::printf("exact mismatch Rj=%.17g up=%.17g got=%.17g want=%.17g\n", Rj, up, got, want);
      fails++;
      return;
    }
    const double ref = reference_slope(Rj, up);
    const double scale = std::fabs(Rj) + std::fabs(up);
    if (std::fabs(got - ref) > 4e-16 * scale) {
      if (fails < 20) std::printf("reference mismatch Rj=%.17g up=%.17g got=%.17g ref=%.17g\n", Rj, up, got, ref);
      fails++;
    }
  };
  const double special[] = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0, 0.25, 3.0, 1e-300, -1e-300,
                            1e300, 4.9e-324, 1.5, -1.5, 0.75};
  for (double a : special)
    for (double b : special) check(a, b);
  for (int i = 0; i < 2000000; i++) {
    const double Rj = std::ldexp(u(rng), ex(rng));
    double up;
    switch (i % 5) {
      case 0: up = std::ldexp(u(rng), ex(rng)); break;
      case 1: up = Rj * 0.5; break;                     // r = 1/2: branch points
      case 2: up = Rj * 2.0; break;                     // r = 2
      case 3: up = Rj * (1.0 + 0.5 * u(rng)); break;    // r near 1
      default: up = Rj; break;                          // r = 1
    }
    check(Rj, up);
    check(Rj, -up);
  }
  std::printf("%ld cases, %ld failures\n", n, fails);
  return fails ? 1 : 0;
}
