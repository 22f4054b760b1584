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

// Division of a 32-bit index n < 2^31 by a divisor 1 <= d < 2^31 fixed
// for a launch: q = (n * m) >> S with S = 31 + ceil(log2 d) and
// m = ceil(2^S / d) < 2^32 (Granlund and Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994: the rounding error
// n*(m - 2^S/d)/2^S stays below 1/d for n < 2^31, so the quotient is
// exact).  One wide multiply and one shift instead of a generic division
// sequence per coordinate; checked on the host against n / d
// (tests/native/fastdiv_check.cu).
struct DivU32 {
  unsigned d, m, S;
  __host__ __device__ __forceinline__ unsigned div(unsigned n) const {
    return (unsigned)(((unsigned long long)n * m) >> S);
  }
};

inline DivU32 make_div(unsigned d) {
  unsigned k = 0;
  while ((1ull << k) < d) k++;
  const unsigned S = 31 + k;
  const unsigned long long m = ((1ull << S) + d - 1) / d;
  return DivU32{d, (unsigned)m, S};
}

// v > 0 for a binary64 v that is not NaN, on the integer pipe: the bit
// pattern read as a signed integer is positive exactly for v > +0
__host__ __device__ __forceinline__ bool f64_pos(double v) { return (long long)f64_bits(v) > 0; }

// phi(up/Rj)*Rj of the superbee limiter, selected exactly (see above).
// On the device the selection is one block of 64-bit integer PTX: written
// as C, its bit manipulations (sign extraction and flips, the doubling) are
// read back by the compilers as binary64 operations, and ncu counted about
// one more binary64-pipe instruction per face (the pipe this form is bound
// by: 83 ms against 96 ms per step at 32^6).  The host keeps the C form;
// both are checked against the case analysis on the host and on the GPU
// (tests/native/superbee_select_check.cu).
__host__ __device__ __forceinline__ double superbee_slope64(double Rj, double up) {
#ifdef __CUDA_ARCH__
  double r;
  asm("{\n\t"
      ".reg .b64 rb, ub, s, a, t, lo, hi, lo2, lo2a, lo2b, m;\n\t"
      ".reg .pred pt, pd;\n\t"
      "mov.b64 rb, %1;\n\t"
      "mov.b64 ub, %2;\n\t"
      "and.b64 s, rb, 0x8000000000000000;\n\t"     // sign of Rj
      "xor.b64 a, rb, s;\n\t"                      // |Rj|
      "xor.b64 t, ub, s;\n\t"                      // sign(Rj)*up
      "setp.gt.s64 pt, t, 0;\n\t"                  // t > 0
      "min.u64 lo, a, t;\n\t"
      "max.u64 hi, a, t;\n\t"
      "setp.lt.u64 pd, lo, 0x0010000000000000;\n\t"
      "shl.b64 lo2a, lo, 1;\n\t"                   // 2*lo: denormal or zero
      "add.u64 lo2b, lo, 0x0010000000000000;\n\t"  // 2*lo: normal
      "selp.b64 lo2, lo2a, lo2b, pd;\n\t"
      "min.u64 m, lo2, hi;\n\t"
      "selp.b64 m, m, 0, pt;\n\t"
      "or.b64 m, m, s;\n\t"
      "mov.b64 %0, m;\n\t"
      "}"
      : "=d"(r)
      : "d"(Rj), "d"(up));
  return r;
#else
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
#endif
}

// binary64 face flux of the fast form, face between Eb = E0 and Ec = Ep1
// (E(f-1), E(f), E(f+1), E(f+2) = Em1, E0, Ep1, Ep2), v the face velocity
// and h its cached |v|/2*(1-|v dt/d|): two subtractions, one multiply, one
// fma on the binary64 pipe (the operands of the upwind difference and the
// upwind value are selected before the arithmetic)
__device__ __forceinline__ double flux_fast64(double v, double h, double Em1, double E0, double Ep1,
                                              double Ep2) {
  const bool pos = f64_pos(v);
  const double Rj = __dsub_rn(Ep1, E0);
  const double up = __dsub_rn(pos ? E0 : Ep2, pos ? Em1 : Ep1);
  const double Eu = pos ? E0 : Ep1;
  return __fma_rn(h, superbee_slope64(Rj, up), __dmul_rn(v, Eu));
}

}  // namespace rt
