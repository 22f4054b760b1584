// Host check of the stochastic rounding of the binary32 update (rt_step.cuh):
// upd32 returns one of the two binary32 neighbours of the exact sum
// e0 + x, and over the random words its mean equals the exact sum (zero
// mean error), also where the increment is far below half a unit in the
// last place of e0 (where round-to-nearest would lose it every time).
#include <cmath>
#include <cstdio>
#include <random>

#include "rt_step.cuh"

using namespace rt;

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  long fails = 0, n = 0;
  for (int t = 0; t < 2000; t++) {
    const float e0 = (float)std::ldexp(0.5 + u(rng), -10 - (int)(u(rng) * 20));
    // increments from 1e-3 ulp to 100 ulp of e0, both signs
    const double ulp = std::ldexp(1.0, std::ilogb(e0) - 23);
    const double xr = (u(rng) < 0.5 ? -1 : 1) * ulp * std::pow(10.0, -3.0 + 5.0 * u(rng));
    const float x = (float)xr;                 // the increment as the kernel holds it
    const double exact = (double)e0 + (double)x;
    const int N = 4096;
    double mean = 0.0;
    for (int k = 0; k < N; k++) {
      const unsigned rnd = sr_bits(k + 1000003LL * t, 12345u);
      const float r = upd32(e0, x, 0.f, 0.f, 0.f, rnd);   // mf = 0: E + x
      const double lo = std::nextafter((float)exact, -INFINITY), hi = std::nextafter((float)exact, INFINITY);
      if (!((double)r == (double)(float)exact || (double)r == lo || (double)r == hi)) fails++;
      if (std::fabs((double)r - exact) >= 2 * ulp) fails++;
      mean += r;
      n++;
    }
    mean /= N;
    // the mean error is within 5 standard errors of zero (std of one draw <= gap/2)
    const double se = ulp / std::sqrt((double)N);
    if (std::fabs(mean - exact) > 5 * se) {
      if (fails < 10) std::printf("biased: e0=%.9g x=%.9g mean-exact=%.3g se=%.3g\n", e0, x, mean - exact, se);
      fails++;
    }
  }
  // an exact sum stays exact
  if (upd32(1.0f, 0.5f, 0.f, 0.f, 0.f, 0xffffffffu) != 1.5f) fails++;
  std::printf("%ld cases, %ld failures\n", n, fails);
  return fails ? 1 : 0;
}
