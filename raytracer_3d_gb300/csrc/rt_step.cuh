// rt_step.cuh -- the fused time step: superbee face fluxes
// (superbee_fluxes.f90:4-174), flux divergence (integrate.f90:105-200),
// mean-flow term (:202-252) and forward-Euler update (:255-268) in one
// sweep over E.  Fluxes, dE and meanfl are never stored.
#pragma once
#include <cstring>

#include "rt_common.cuh"

namespace rt {

// binary32 literal 1.E20 of superbee_fluxes.f90:26, widened to binary64
#define RT_LIT_1E20 1.0000000200408773e20

// ---- plain binary64 form: the reference's arithmetic, bit for bit -------
// Face flux at face f of one axis from E(f-1), E(f), E(f+1), E(f+2),
// superbee_fluxes.f90:19-30.
__device__ __forceinline__ double flux_fp64(double v, double dgrid, double dt, double Ea, double Eb,
                                            double Ec, double Ed) {
  const double uCFL = fabs(ddiv(dmul(v, dt), dgrid));
  const double Rjp = dsub(Ed, Ec);
  const double Rj = dsub(Ec, Eb);
  const double Rjm = dsub(Eb, Ea);
  const double up = v > 0 ? Rjm : Rjp;
  double Cr = (Rj != 0.0) ? ddiv(up, Rj) : dmul(up, RT_LIT_1E20);
  Cr = fmax2(0.0, fmax2(fmin2(1.0, dmul(2.0, Cr)), fmin2(2.0, Cr)));  // Limiter, :10
  const double adv = dmul(dmul(v, dadd(Ec, Eb)), 0.5);
  const double dif = dmul(dmul(dmul(fabs(v), dadd(dsub(1.0, Cr), dmul(uCFL, Cr))), Rj), 0.5);
  return dsub(adv, dif);
}

// The same flux with uCFL = |v*dt/d(f)| given: uCFL is a constant of the
// face (velocity, grid, dt), so the binary64 form computes it once, in the
// reference's operation order, and reuses it every step.
__device__ __forceinline__ double flux_fp64u(double v, double uCFL, double Ea, double Eb, double Ec,
                                             double Ed) {
  const double Rjp = dsub(Ed, Ec);
  const double Rj = dsub(Ec, Eb);
  const double Rjm = dsub(Eb, Ea);
  const double up = v > 0 ? Rjm : Rjp;
  double Cr = (Rj != 0.0) ? ddiv(up, Rj) : dmul(up, RT_LIT_1E20);
  Cr = fmax2(0.0, fmax2(fmin2(1.0, dmul(2.0, Cr)), fmin2(2.0, Cr)));
  const double adv = dmul(dmul(v, dadd(Ec, Eb)), 0.5);
  const double dif = dmul(dmul(dmul(fabs(v), dadd(dsub(1.0, Cr), dmul(uCFL, Cr))), Rj), 0.5);
  return dsub(adv, dif);
}

// ---- binary32 precision form -------------------------------------------
// Same flux, rearranged without a division.  With s = sign(Rj), t = s*up
// and a = |Rj|, the limited slope phi(r)*Rj (r = up/Rj) is
//   s * max(0, min(2*min(a, t), max(a, t)))
// (= s*max(0, min(a, 2t), min(2a, t)), the superbee form, exactly: the
// doubling is exact), and the centred part plus the first diffusive part,
// 0.5*(v*(Ec+Eb) - |v|*Rj), is the upwind value v*E_up exactly, so
//   F = v*E_up + |v|*(1/2 - |v|*dt/(2d)) * psi.
// For Rj == 0 psi = +-0 and the diffusive term vanishes as in the reference
// (it is multiplied by Rj there).  hcfl = dt/(2 d(f)).
__device__ __forceinline__ float flux_fp32(float v, float hcfl, float Ea, float Eb, float Ec, float Ed) {
  const float Rjp = Ed - Ec;
  const float Rj = Ec - Eb;
  const float Rjm = Eb - Ea;
  const bool pos = v > 0.f;
  const float up = pos ? Rjm : Rjp;
  const float Eu = pos ? Eb : Ec;
  // s = sign(Rj) applied by flipping the sign bit (one logic op each)
  const unsigned s = __float_as_uint(Rj) & 0x80000000u;
  const float a = fabsf(Rj);
  const float t = __uint_as_float(__float_as_uint(up) ^ s);
  const float ph = fmaxf(0.f, fminf(2.f * fminf(a, t), fmaxf(a, t)));
  const float psi = __uint_as_float(__float_as_uint(ph) ^ s);
  const float av = fabsf(v);
  const float h = av * fmaf(-hcfl, av, 0.5f);
  return fmaf(h, psi, v * Eu);
}

// ---- two cells at once: binary32 pairs on the packed f32x2 pipes --------
// sm_100+ executes add / sub / mul / fma on a pair of binary32 values held
// in a 64-bit register as one instruction, each lane rounded exactly as the
// scalar instruction would round it (round to nearest even), so a pair
// computed packed equals the two scalar results bit for bit.
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) {
  float2 d;
  asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b) {
  float2 d;
  asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b) {
  float2 d;
  asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
// a*b + c, one rounding per lane
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 pk_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 pk_abs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }

// Per-axis small tables of the binary32 form on the padded index range
// (Fortran index f at position f+1): 1/d(f) (the budget's divergence),
// dt/(2 d(f)) (the flux), and dt/d(f) as the unevaluated sum chi + clo of
// two binary32 numbers (the step's divergence).
struct Tab32 {
  const float* inv_d[6];
  const float* hcfl[6];
  const float* chi[6];
  const float* clo[6];
};

// Divergence and update of the binary32 step.  The step accumulates
// acc = dt * sum_a (F_l - F_r)/d_a and stores E + acc - dt*E*lambda.  Two
// sources of systematic error are removed, so that what remains averages
// out in the total energy:
//  * the constants dt/d_a and dt are carried as two-term binary32 sums
//    (about 48 bits): a single rounded binary32 constant would scale every
//    flux of an axis alike, so the energy leaving through the open
//    boundaries -- the only fluxes that do not cancel in the total -- and
//    the mean-flow exchange would carry one systematic relative error of up
//    to 2^-24 over a whole run;
//  * the sum E + increment is rounded stochastically: to one of the two
//    binary32 neighbours of the exact sum, the farther one with probability
//    (distance to the nearer) / (gap).  Round-to-nearest loses every
//    increment below half a unit in the last place of E, and where a cell's
//    increments keep one sign (slow exchange, weak gradients) those losses
//    add up over a run; stochastic rounding has zero mean error.  The random
//    word is a hash of the cell's index and a per-step seed that the step
//    kernels carry in device memory (seed_in / seed_out), so every binary32
//    schedule, and a member of a batch or a served request, draws the same
//    words and gives the same result bit for bit.
__device__ __forceinline__ float div32(float acc, float fr, float fl, float chi, float clo) {
  const float df = fl - fr;
  return fmaf(df, chi, fmaf(df, clo, acc));
}
__host__ __device__ __forceinline__ unsigned f32_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}
__host__ __device__ __forceinline__ float f32_from_bits(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}
// counter-based random word of a cell (linear index p) at the step with `seed`
__host__ __device__ __forceinline__ unsigned sr_bits(long long p, unsigned seed) {
  unsigned h = ((unsigned)p ^ ((unsigned)((unsigned long long)p >> 32) * 0x85EBCA6Bu)) + seed * 0x9E3779B1u;
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return h;
}
// s = RN(a + b) and err = a + b - s exactly (error-free transformation of
// the sum): the binary32 neighbour of s on the side of err with probability
// |err| / gap, using the top 24 bits of rnd
__host__ __device__ __forceinline__ float sr_round(float s, float err, unsigned rnd) {
  const unsigned sb = f32_bits(s);
  const unsigned nbits = ((err > 0.f) == ((sb >> 31) == 0u)) ? sb + 1u : sb - 1u;
  const float nb = f32_from_bits(nbits);
  const float gap = fabsf(nb - s);
  const float u = (float)(rnd >> 8) * 5.9604645e-08f;   // [0, 1) in steps of 2^-24
  return (u * gap < fabsf(err)) ? nb : s;               // err == 0: s
}
__host__ __device__ __forceinline__ float upd32(float e0, float acc, float mf, float dthi, float dtlo,
                                                unsigned rnd) {
  const float x = fmaf(-mf, dthi, fmaf(-mf, dtlo, acc));
  const float s = e0 + x;
  const float bp = s - e0;
  const float err = (e0 - (s - bp)) + (x - bp);
  return sr_round(s, err, rnd);
}

// The same per-cell arithmetic for two cells at once (flux_fp32, div32,
// upd32 lane by lane); PK selects the packed f32x2 instructions for the
// additions and products, the limiter's selections and min / max stay
// scalar.  Both settings give identical results.
template <bool PK>
__device__ __forceinline__ float2 flux2(float2 v, float2 hcfl, float2 Ea, float2 Eb, float2 Ec, float2 Ed) {
  if constexpr (!PK) {
    return make_float2(flux_fp32(v.x, hcfl.x, Ea.x, Eb.x, Ec.x, Ed.x), flux_fp32(v.y, hcfl.y, Ea.y, Eb.y, Ec.y, Ed.y));
  } else {
    const float2 Rjp = pk_sub(Ed, Ec), Rj = pk_sub(Ec, Eb), Rjm = pk_sub(Eb, Ea);
    const bool px = v.x > 0.f, py = v.y > 0.f;
    const float2 up = make_float2(px ? Rjm.x : Rjp.x, py ? Rjm.y : Rjp.y);
    const float2 Eu = make_float2(px ? Eb.x : Ec.x, py ? Eb.y : Ec.y);
    const unsigned sx = __float_as_uint(Rj.x) & 0x80000000u, sy = __float_as_uint(Rj.y) & 0x80000000u;
    const float ax = fabsf(Rj.x), ay = fabsf(Rj.y);
    const float tx = __uint_as_float(__float_as_uint(up.x) ^ sx), ty = __uint_as_float(__float_as_uint(up.y) ^ sy);
    const float2 mn = make_float2(fminf(ax, tx), fminf(ay, ty));
    const float2 mn2 = pk_mul(make_float2(2.f, 2.f), mn);
    const float phx = fmaxf(0.f, fminf(mn2.x, fmaxf(ax, tx))), phy = fmaxf(0.f, fminf(mn2.y, fmaxf(ay, ty)));
    const float2 psi = make_float2(__uint_as_float(__float_as_uint(phx) ^ sx), __uint_as_float(__float_as_uint(phy) ^ sy));
    const float2 av = pk_abs(v);
    const float2 h = pk_mul(av, pk_fma(pk_neg(hcfl), av, make_float2(0.5f, 0.5f)));
    return pk_fma(h, psi, pk_mul(v, Eu));
  }
}
template <bool PK>
__device__ __forceinline__ float2 div2(float2 acc, float2 fr, float2 fl, float2 chi, float2 clo) {
  if constexpr (!PK) {
    return make_float2(div32(acc.x, fr.x, fl.x, chi.x, clo.x), div32(acc.y, fr.y, fl.y, chi.y, clo.y));
  } else {
    const float2 df = pk_sub(fl, fr);
    return pk_fma(df, chi, pk_fma(df, clo, acc));
  }
}
template <bool PK>
__device__ __forceinline__ float2 upd2(float2 e0, float2 acc, float2 lam, float dthi, float dtlo, uint2 rnd) {
  if constexpr (!PK) {
    return make_float2(upd32(e0.x, acc.x, e0.x * lam.x, dthi, dtlo, rnd.x),
                       upd32(e0.y, acc.y, e0.y * lam.y, dthi, dtlo, rnd.y));
  } else {
    const float2 nmf = pk_neg(pk_mul(e0, lam));
    const float2 x = pk_fma(nmf, make_float2(dthi, dthi), pk_fma(nmf, make_float2(dtlo, dtlo), acc));
    const float2 s = pk_add(e0, x);
    const float2 bp = pk_sub(s, e0);
    const float2 err = pk_add(pk_sub(e0, pk_sub(s, bp)), pk_sub(x, bp));
    return make_float2(sr_round(s.x, err.x, rnd.x), sr_round(s.y, err.y, rnd.y));
  }
}

template <class T>
struct StepArgs {
  Dims d;
  Grid g;
  Tab32 t32;
  const T* E;          // state at the start of the step
  T* Enew;             // state after the step (ping-pong)
  const T* vel[6];     // right-face velocities
  const T* vlo[6];     // face-0 planes
  const T* lam[3];     // fp64: lambda_x/y/z; fp32: lam[0] = combined rate
  const T* uc[6];      // fp64: cached |v*dt/d| of the right faces (fp32: unused)
  const T* ucl[6];     // fp64: the same on the face-0 planes
  double dt;
  float dthi, dtlo;    // binary32 form: dt as the two-term sum dthi + dtlo
  // binary32 form: seed of this step's stochastic rounding (read), and the
  // next step's (written once per step by the thread that updates the
  // field's first item: seed + 1).  Two slots per handle, swapped with E.
  const unsigned* seed_in;
  unsigned* seed_out;
  int* status;         // device flag: bit 0 = a bounded wait timed out
};

// the next step's seed, written by thread 0 of the CTA that takes item 0 of
// a field (one writer per field and step; seed_in is not written by a step)
__device__ __forceinline__ void advance_seed(const unsigned* seed_in, unsigned* seed_out, long long item) {
  if (item == 0 && threadIdx.x == 0) *seed_out = *seed_in + 1u;
}

// Read E at cell p displaced by off along axis a from coordinate c,
// applying the ghost-cell map (returns the mapped linear index).
__device__ __forceinline__ long long nb_index(const Dims& d, long long p, int a, int c, int off,
                                              int cm) {
  int flip = 0;
  const int c2 = map_coord(d, a, c + off, flip);
  long long q = p + (long long)(c2 - c) * d.s[a];
  if (flip) q += (long long)((d.n[5] - 1 - cm) - cm) * d.s[5];
  return q;
}

// Per-cell tendency (everything but the update), shared by the step and the
// budget kernels so that both see bit-identical dE and meanfl.
template <class T>
struct CellTerms {
  T dE;        // -(flux divergence), before the mean-flow term
  T meanfl;
};

__device__ __forceinline__ long long plane_index(const Dims& d, int a, const int c[6]) {
  long long q = 0;
#pragma unroll
  for (int b = 0; b < 6; b++) q += (long long)c[b] * plane_stride(d, a, b);
  return q;
}

template <class T>
__device__ __forceinline__ CellTerms<T> cell_terms(const StepArgs<T>& A, long long p, const int c[6],
                                                   T e0);

template <>
__device__ __forceinline__ CellTerms<double> cell_terms<double>(const StepArgs<double>& A,
                                                                long long p, const int c[6],
                                                                double e0) {
  const Dims& d = A.d;
  double dE = 0.;
#pragma unroll
  for (int a = 0; a < 6; a++) {
    if (d.n[a] <= 1) continue;
    const int ca = c[a];
    const double Em2 = A.E[nb_index(d, p, a, ca, -2, c[5])];
    const double Em1 = A.E[nb_index(d, p, a, ca, -1, c[5])];
    const double Ep1 = A.E[nb_index(d, p, a, ca, +1, c[5])];
    const double Ep2 = A.E[nb_index(d, p, a, ca, +2, c[5])];
    const int F = ca + 1;  // Fortran index of the cell = its right face
    const double vr = A.vel[a][p];
    const double vl = ca > 0 ? A.vel[a][p - d.s[a]] : A.vlo[a][plane_index(d, a, c)];
    const double dr = A.g.d[a][pidx(F)];
    const double dl = A.g.d[a][pidx(F - 1)];
    const double fr = flux_fp64(vr, dr, A.dt, Em1, e0, Ep1, Ep2);
    const double fl = flux_fp64(vl, dl, A.dt, Em2, Em1, e0, Ep1);
    dE = dsub(dE, ddiv(dsub(fr, fl), dr));
  }
  double mf = 0.;
  if (d.n[0] > 1) mf = dadd(mf, dmul(e0, A.lam[0][p]));
  if (d.n[1] > 1) mf = dadd(mf, dmul(e0, A.lam[1][p]));
  if (d.n[2] > 1) mf = dadd(mf, dmul(e0, A.lam[2][p]));
  return {dE, mf};
}

template <>
__device__ __forceinline__ CellTerms<float> cell_terms<float>(const StepArgs<float>& A, long long p,
                                                              const int c[6], float e0) {
  const Dims& d = A.d;
  float dE = 0.f;
#pragma unroll
  for (int a = 0; a < 6; a++) {
    if (d.n[a] <= 1) continue;
    const int ca = c[a];
    const float Em2 = A.E[nb_index(d, p, a, ca, -2, c[5])];
    const float Em1 = A.E[nb_index(d, p, a, ca, -1, c[5])];
    const float Ep1 = A.E[nb_index(d, p, a, ca, +1, c[5])];
    const float Ep2 = A.E[nb_index(d, p, a, ca, +2, c[5])];
    const int F = ca + 1;
    const float vr = A.vel[a][p];
    const float vl = ca > 0 ? A.vel[a][p - d.s[a]] : A.vlo[a][plane_index(d, a, c)];
    const float fr = flux_fp32(vr, A.t32.hcfl[a][pidx(F)], Em1, e0, Ep1, Ep2);
    const float fl = flux_fp32(vl, A.t32.hcfl[a][pidx(F - 1)], Em2, Em1, e0, Ep1);
    dE -= (fr - fl) * A.t32.inv_d[a][pidx(F)];
  }
  const float mf = e0 * A.lam[0][p];
  return {dE, mf};
}

// the binary32 step of one cell (the one-thread-per-cell kernel): the same
// fluxes as cell_terms<float>, the step's divergence and update
__device__ __forceinline__ float cell_step32(const StepArgs<float>& A, long long p, const int c[6], float e0) {
  const Dims& d = A.d;
  float acc = 0.f;
#pragma unroll
  for (int a = 0; a < 6; a++) {
    if (d.n[a] <= 1) continue;
    const int ca = c[a];
    const float Em2 = A.E[nb_index(d, p, a, ca, -2, c[5])];
    const float Em1 = A.E[nb_index(d, p, a, ca, -1, c[5])];
    const float Ep1 = A.E[nb_index(d, p, a, ca, +1, c[5])];
    const float Ep2 = A.E[nb_index(d, p, a, ca, +2, c[5])];
    const int F = ca + 1;
    const float vr = A.vel[a][p];
    const float vl = ca > 0 ? A.vel[a][p - d.s[a]] : A.vlo[a][plane_index(d, a, c)];
    const float fr = flux_fp32(vr, A.t32.hcfl[a][pidx(F)], Em1, e0, Ep1, Ep2);
    const float fl = flux_fp32(vl, A.t32.hcfl[a][pidx(F - 1)], Em2, Em1, e0, Ep1);
    acc = div32(acc, fr, fl, A.t32.chi[a][pidx(F)], A.t32.clo[a][pidx(F)]);
  }
  return upd32(e0, acc, e0 * A.lam[0][p], A.dthi, A.dtlo, sr_bits(p, *A.seed_in));
}

}  // namespace rt
