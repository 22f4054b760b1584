// Host check of the invariant-divisor division of the fast binary64 step's
// index arithmetic (DivU32 / make_div in rt_fast.cuh): div(n) must equal
// n / d for every numerator below 2^31 the kernels can pass.  Every
// divisor up to 70000 (all extents and products of extents a field of
// fewer than 2^31 cells uses in practice) against the numerators at and
// around each multiple boundary that matters (0, d-1, d, d+1, 2^31-1 and
// the largest multiples of d below 2^31) plus random ones; then random
// divisors up to 2^31-1.
#include <cstdio>
#include <random>

#include "rt_fast.cuh"

using namespace rt;

int main() {
  std::mt19937_64 rng(20261204);
  const unsigned top = 0x7fffffffu;   // largest numerator: 2^31 - 1
  long fails = 0, n = 0;
  auto check = [&](const DivU32& D, unsigned x) {
    n++;
    const unsigned want = x / D.d, got = D.div(x);
    if (got != want) {
      if (fails < 20) std::printf("mismatch d=%u n=%u got=%u want=%u\n", D.d, x, got, want);
      fails++;
    }
  };
  auto probe = [&](unsigned d, int random) {
    const DivU32 D = make_div(d);
    const unsigned last = top / d * d;   // largest multiple of d not above 2^31 - 1
    const unsigned fixed[] = {0u, 1u, d - 1u, d, d + 1u, top, last, last - 1u, last > d ? last - d : 0u,
                              last > d ? last - d + 1u : 0u};
    for (unsigned x : fixed)
      if (x <= top) check(D, x);
    std::uniform_int_distribution<unsigned> u(0u, top);
    for (int i = 0; i < random; i++) check(D, u(rng));
  };
  for (unsigned d = 1; d <= 70000; d++) probe(d, 64);
  std::uniform_int_distribution<unsigned> ud(70001u, top);
  for (int i = 0; i < 20000; i++) probe(ud(rng), 64);
  std::printf("%ld cases, %ld failures\n", n, fails);
  return fails ? 1 : 0;
}
