// rt_fast.cuh -- arithmetic of the fast binary64 step (variant
// RT_VARIANT_FAST): the reference's superbee flux (superbee_fluxes.f90:
// 19-30) rewritten without a division and without a binary64 comparison.
//
// GB300 issues binary64 add / multiply / fma at a small fraction of its
// binary32 rate, and a correctly rounded binary64 division costs about ten
// of them.  The bit-exact form (flux_fp64u) spends two divisions per face
// flux (Cr = up/Rj; the divergence divides by the spacing) plus six
// comparisons.  This form keeps the same algebra and gives up only the
// reference's rounding sequence (results agree to a few units in the last
// place per step, far inside the 1e-12 relative bound of the plain form):
//
//   superbee slope   psi = phi(up/Rj) * Rj, phi(r) = max(0, min(1,2r), min(2,r))
//                        = s * max(0, min(2*min(a,t), max(a,t)))
//                    with s = sign(Rj), a = |Rj|, t = s*up.  Every candidate
//                    is Rj, up or twice one of them: psi is SELECTED, not
//                    computed, so it is exact.  For a, t >= 0 the order of
//                    binary64 values is the order of their bit patterns as
//                    unsigned integers, so the selection runs on the integer
//                    pipes; doubling adds one to the exponent field of a
//                    normal number and shifts the bits of a denormal (or
//                    zero) left by one, both exact.
//   centred + first diffusive part
//                    0.5*v*(Ec+Eb) - 0.5*|v|*Rj = v*E_up exactly
//                    (E_up = Eb for v > 0, else Ec)
//   flux             F = v*E_up + h*psi,  h = |v|/2 * (1 - |v dt/d|)
//                    (h is a constant of the face, cached like uCFL)
//
// Zero gradient (Rj == 0, the reference's 1.E20 branch): a = 0 and psi = 0,
// so the diffusive term vanishes as in the reference.
#pragma once
#include <cstdint>
#include <cstring>

namespace rt {

__host__ __device__ __forceinline__ unsigned long long f64_bits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  std::memcpy(&u, &x, sizeof u);
  return u;
#endif
}
__host__ __device__ __forceinline__ double f64_from_bits(unsigned long long u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, sizeof x);
  return x;
#endif
}

// v > 0 for a binary64 v that is not NaN, on the integer pipe: the bit
// pattern read as a signed integer is positive exactly for v > +0
__host__ __device__ __forceinline__ bool f64_pos(double v) { return (long long)f64_bits(v) > 0; }

// phi(up/Rj)*Rj of the superbee limiter, selected exactly (see above)
__host__ __device__ __forceinline__ double superbee_slope64(double Rj, double up) {
  const unsigned long long sbit = 0x8000000000000000ull;
  const unsigned long long rb = f64_bits(Rj);
  const unsigned long long s = rb & sbit;
  const unsigned long long a = rb ^ s;                  // |Rj|
  const unsigned long long t = f64_bits(up) ^ s;        // sign(Rj)*up
  const bool tpos = (long long)t > 0;                   // t > 0 (r > 0)
  const unsigned long long lo = a < t ? a : t;
  const unsigned long long hi = a < t ? t : a;
  const unsigned long long e1 = 0x0010000000000000ull;         // exponent field 1
  const unsigned long long lo2 = lo < e1 ? lo << 1 : lo + e1;  // 2*lo, exact
  unsigned long long m = lo2 < hi ? lo2 : hi;
  m = tpos ? m : 0ull;
  return f64_from_bits(m | s);
}

// p ? a : b formed on the integer pipes as b ^ ((a ^ b) & mask), the mask
// ANDed with `ones`, a kernel argument that is always all ones but unknown
// to the compilers: the upwind difference then stays one binary64
// subtraction of the selected operands.  A select the compilers can see
// becomes both differences and a select of them, a third binary64
// subtraction per face.
__device__ __forceinline__ double sel64(bool p, double a, double b, unsigned long long ones) {
  const unsigned long long m = (0ull - (unsigned long long)p) & ones;   // all ones when p
  const unsigned long long ua = f64_bits(a), ub = f64_bits(b);
  return f64_from_bits(ub ^ ((ua ^ ub) & m));
}

// binary64 face flux of the fast form, face between Eb = E0 and Ec = Ep1
// (E(f-1), E(f), E(f+1), E(f+2) = Em1, E0, Ep1, Ep2), v the face velocity
// and h its cached |v|/2*(1-|v dt/d|): two subtractions, one multiply, one
// fma on the binary64 pipe
__device__ __forceinline__ double flux_fast64(double v, double h, double Em1, double E0, double Ep1,
                                              double Ep2, unsigned long long ones) {
  const bool pos = f64_pos(v);
  const double Rj = __dsub_rn(Ep1, E0);
  const double up = __dsub_rn(sel64(pos, E0, Ep2, ones), sel64(pos, Em1, Ep1, ones));
  const double Eu = sel64(pos, E0, Ep1, ones);
  return __fma_rn(h, superbee_slope64(Rj, up), __dmul_rn(v, Eu));
}

}  // namespace rt
