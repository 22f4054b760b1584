// rt_coeff.cuh -- device restatement of calc_parameter.f90 without the
// padded temporaries.
//
// The reference builds omega_i/omega_e on every padded cell
// (calc_parameter.f90:13-27), averages omega_e along one axis of a pair and
// then OVERWRITES that average with the average along the partner axis
// (:34-40, :112-118, :188-194), and differences the result (:44-46, :69-71,
// ...).  Here every face velocity is evaluated directly from the dispersion
// relation at the four points it depends on; the arithmetic is the same
// binary64 sequence, so the values are bit-identical to the reference's
// arrays wherever the hot path reads them.
#pragma once
#include "rt_common.cuh"

namespace rt {

struct Phys {
  double f0;     // Coriolis parameter (main_module.f90:24)
  double sgn;    // sign_of_omega_i (main_module.f90:26)
  double dt;     // time step (main_module.f90:20)
};

__device__ __forceinline__ long long bg_idx(const Background& bg, int i, int j, int k) {
  return (long long)pidx(i) + (long long)bg.px * (pidx(j) + (long long)bg.py * pidx(k));
}

// omega_i, calc_parameter.f90:19-20 (Fortran indices, ghosts allowed)
__device__ __forceinline__ double omega_i_at(const Background& bg, const Grid& g, const Phys& ph,
                                             int i, int j, int k, int l, int n, int m) {
  const double ktv = g.kt[pidx(l)], ltv = g.lt[pidx(n)], mtv = g.mt[pidx(m)];
  const double kh2 = dadd(dmul(ltv, ltv), dmul(ktv, ktv));
  const double m2 = dmul(mtv, mtv);
  const double Nq = bg.Nsqr[bg_idx(bg, i, j, k)];
  const double num = dadd(dmul(Nq, kh2), dmul(dmul(ph.f0, ph.f0), m2));
  const double den = dadd(m2, kh2);
  return dmul(ph.sgn, __dsqrt_rn(ddiv(num, den)));
}

// omega_e, calc_parameter.f90:21
__device__ __forceinline__ double omega_e_at(const Background& bg, const Grid& g, const Phys& ph,
                                             int i, int j, int k, int l, int n, int m) {
  const long long q = bg_idx(bg, i, j, k);
  const double oi = omega_i_at(bg, g, ph, i, j, k, l, n, m);
  return dadd(dadd(oi, dmul(g.kt[pidx(l)], bg.U[q])), dmul(g.lt[pidx(n)], bg.V[q]));
}

// the pair-average "aloc" of the reference: average of omega_e over index
// q and q+1 along the SECOND axis of the pair (k for x/k, l for y/l,
// m for z/m), calc_parameter.f90:38-40, :116-118, :192-194.
// c[] holds Fortran indices of x,y,z,k,l,m.
__device__ __forceinline__ double aloc_at(const Background& bg, const Grid& g, const Phys& ph,
                                          const int c[6], int axis2) {
  int c2[6] = {c[0], c[1], c[2], c[3], c[4], c[5]};
  const double a = omega_e_at(bg, g, ph, c2[0], c2[1], c2[2], c2[3], c2[4], c2[5]);
  c2[axis2] += 1;
  const double b = omega_e_at(bg, g, ph, c2[0], c2[1], c2[2], c2[3], c2[4], c2[5]);
  return dmul(0.5, dadd(a, b));
}

// analytic velocity of a collapsed pair, calc_parameter.f90:98 (x) / :176 (y)
__device__ __forceinline__ double analytic_vel(const Background& bg, const Grid& g, const Phys& ph,
                                               const int c[6], int which) {
  const long long q = bg_idx(bg, c[0], c[1], c[2]);
  const double ktv = g.kt[pidx(c[3])], ltv = g.lt[pidx(c[4])], mtv = g.mt[pidx(c[5])];
  const double kh2 = dadd(dmul(ltv, ltv), dmul(ktv, ktv));
  const double oi = omega_i_at(bg, g, ph, c[0], c[1], c[2], c[3], c[4], c[5]);
  const double m2 = dmul(mtv, mtv);
  const double den = dadd(m2, kh2);
  double t = ddiv(dsub(bg.Nsqr[q], dmul(ph.f0, ph.f0)), oi);
  t = dmul(t, m2);
  t = ddiv(t, dmul(den, den));
  if (which == 0) return dadd(bg.U[q], dmul(t, ktv));
  return dadd(bg.V[q], dmul(t, ltv));
}

// Face velocity of axis a at the face with Fortran index c[a] (0..n_a),
// all other indices interior.  Pairs: x<->k, y<->l, z<->m.
//   spatial velocity (x,y,z):  (aloc(q) - aloc(q-1)) / d_partner(q) over
//                              the partner axis (:44-46, :122-124, :198-200)
//   spectral velocity (k,l,m): -(aloc(f) - aloc(f-1)) / d_partner(f) over
//                              the spatial partner (:69-71, :147-149, :219-221)
// then the outflow-only clamps at faces 0 and n (:55-66, :76-87, :133-144,
// :154-165, :204-216, :226-237).
static __device__ __noinline__ double face_velocity(const Dims& d, const Background& bg, const Grid& g,
                                             const Phys& ph, int a, const int cin[6]) {
  const int spatial = a < 3 ? a : a - 3;     // pair index 0:x/k 1:y/l 2:z/m
  const int sa = spatial, wa = spatial + 3;  // spatial axis, wavenumber axis
  const bool full = (spatial == 2) || (d.n[sa] > 1 && d.n[wa] > 1);
  const int f = cin[a];
  const int n = d.n[a];
  if (!full) {
    // collapsed x/k or y/l pair: analytic spatial velocity on interior
    // cells only; spectral velocity and boundary faces stay 0
    if (a < 3 && f >= 1 && f <= n) return analytic_vel(bg, g, ph, cin, spatial);
    return 0.0;
  }
  int c[6] = {cin[0], cin[1], cin[2], cin[3], cin[4], cin[5]};
  double v;
  if (a < 3) {
    // difference along the wavenumber partner at index q = c[wa]
    const double hi = aloc_at(bg, g, ph, c, wa);
    c[wa] -= 1;
    const double lo = aloc_at(bg, g, ph, c, wa);
    v = ddiv(dsub(hi, lo), g.d[wa][pidx(cin[wa])]);
    bool clamp_hi = true, clamp_lo = true;
    if (a == 2) { clamp_hi = !d.upper_refl; clamp_lo = !d.lower_refl; }
    if (f == n && clamp_hi) v = fmax2(0.0, v);
    if (f == 0 && clamp_lo) v = -fmax2(0.0, -v);
  } else {
    // difference along the spatial partner at index q = c[sa]
    const double hi = aloc_at(bg, g, ph, c, wa);
    c[sa] -= 1;
    const double lo = aloc_at(bg, g, ph, c, wa);
    v = -ddiv(dsub(hi, lo), g.d[sa][pidx(cin[sa])]);
    if (f == n) v = fmax2(0.0, v);
    if (f == 0) v = -fmax2(0.0, -v);
  }
  return v;
}

// Mean-flow growth rates on an interior cell, calc_parameter.f90:246-254.
// xd, yd, zd are the cell's own (right-face) velocities.
__device__ __forceinline__ void growth_rates(const Background& bg, const Grid& g, const Phys& ph,
                                             const int c[6], double xd, double yd, double zd,
                                             double& lx, double& ly, double& lz) {
  const int i = c[0], j = c[1], k = c[2];
  const long long q = bg_idx(bg, i, j, k);
  const double Uq = bg.U[q], Vq = bg.V[q];
  const double ktv = g.kt[pidx(c[3])], ltv = g.lt[pidx(c[4])];
  const double oi = omega_i_at(bg, g, ph, c[0], c[1], c[2], c[3], c[4], c[5]);
  const double inv = ddiv(1.0, oi);
  const double dxt2 = dmul(2.0, g.d[0][pidx(i)]);
  const double dyt2 = dmul(2.0, g.d[1][pidx(j)]);
  const double dzt2 = dmul(2.0, g.d[2][pidx(k)]);
  const double dUx = dsub(bg.U[bg_idx(bg, i + 1, j, k)], bg.U[bg_idx(bg, i - 1, j, k)]);
  const double dVx = dsub(bg.V[bg_idx(bg, i + 1, j, k)], bg.V[bg_idx(bg, i - 1, j, k)]);
  const double dUy = dsub(bg.U[bg_idx(bg, i, j + 1, k)], bg.U[bg_idx(bg, i, j - 1, k)]);
  const double dVy = dsub(bg.V[bg_idx(bg, i, j + 1, k)], bg.V[bg_idx(bg, i, j - 1, k)]);
  const double dUz = dsub(bg.U[bg_idx(bg, i, j, k + 1)], bg.U[bg_idx(bg, i, j, k - 1)]);
  const double dVz = dsub(bg.V[bg_idx(bg, i, j, k + 1)], bg.V[bg_idx(bg, i, j, k - 1)]);
  const double xu = dsub(xd, Uq), yv = dsub(yd, Vq);
  lx = dmul(dmul(inv, ktv), dadd(ddiv(dmul(xu, dUx), dxt2), ddiv(dmul(yv, dVx), dxt2)));
  ly = dmul(dmul(inv, ltv), dadd(ddiv(dmul(xu, dUy), dyt2), ddiv(dmul(yv, dVy), dyt2)));
  lz = dmul(dmul(inv, zd), dadd(ddiv(dmul(ktv, dUz), dzt2), ddiv(dmul(ltv, dVz), dzt2)));
}

}  // namespace rt
