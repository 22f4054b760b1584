// Check of the division-free superbee slope of the fast binary64 step
// (rt_fast.cuh): superbee_slope64(Rj, up) must equal phi(up/Rj)*Rj exactly
// (the host form; with --device also the device form, bit for bit),
// where phi(r) = max(0, min(1,2r), min(2,r)) (superbee_fluxes.f90:10), and
// stay within rounding of the reference's division form
//   Cr = up/Rj (Rj /= 0), Cr = up*1.E20 (Rj == 0); phi(Cr)*Rj.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

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

// the device form of superbee_slope64 (one block of integer PTX) over the
// same cases, compared bit for bit with the host form
__global__ void slope_kernel(const double* Rj, const double* up, double* out, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = superbee_slope64(Rj[i], up[i]);
}

static long device_check(const std::vector<double>& R, const std::vector<double>& U) {
  const long n = (long)R.size();
  double *dR = nullptr, *dU = nullptr, *dO = nullptr;
  if (cudaMalloc(&dR, n * sizeof(double)) != cudaSuccess || cudaMalloc(&dU, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dO, n * sizeof(double)) != cudaSuccess) {
    std::printf("device allocation failed\n");
    return -1;
  }
  cudaMemcpy(dR, R.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(dU, U.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  slope_kernel<<<304, 256>>>(dR, dU, dO, n);
  std::vector<double> got(n);
  const cudaError_t e = cudaMemcpy(got.data(), dO, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(dR);
  cudaFree(dU);
  cudaFree(dO);
  if (e != cudaSuccess) {
    std::printf("device run failed: %s\n", cudaGetErrorString(e));
    return -1;
  }
  long fails = 0;
  for (long i = 0; i < n; i++) {
    const double want = superbee_slope64(R[i], U[i]);
    if (std::memcmp(&got[i], &want, sizeof(double)) != 0) {
      if (fails < 20) std::printf("device mismatch Rj=%.17g up=%.17g got=%.17g want=%.17g\n", R[i], U[i], got[i], want);
      fails++;
    }
  }
  std::printf("device: %ld cases, %ld mismatches\n", n, fails);
  return fails;
}

int main(int argc, char** argv) {
  const bool device = argc > 1 && std::strcmp(argv[1], "--device") == 0;
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-60, 20);
  std::vector<double> R, U;
  long fails = 0, n = 0;
  auto check = [&](double Rj, double up) {
    n++;
    R.push_back(Rj);
    U.push_back(up);
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
  if (device) {
    const long d = device_check(R, U);
    if (d != 0) return 1;
  }
  return fails ? 1 : 0;
}
