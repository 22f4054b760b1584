/*
 * rt_oracle.c -- CPU restatement of the raytracer_3D time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See rt_oracle.h for the layout
 * and for the parity status ("parity unpinned": the Fortran reference cannot
 * be built here and has no tests or golden vectors; the restatement is
 * pinned by math known-answer tests instead).
 *
 * Every routine follows one reference subroutine loop by loop and keeps its
 * floating-point operation order (left-to-right evaluation of Fortran
 * expressions, x**2 as x*x, default-real literals such as 1.E20 widened from
 * binary32).  Compile with -O2 -ffp-contract=off.
 */
#include "rt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ONX 2

struct orc_state {
  int n[6];          /* nx ny nz nk nl nm */
  long long P[6];    /* padded extents n+2*onx */
  long long S[6];    /* strides of padded 6D arrays */
  long long len6, len3;
  double dt, f0, sign_of_omega_i, k_fixed, l_fixed, m_fixed;
  int upper_refl, lower_refl;
  double* f6[ORC_N6D];
  double* f3[3 + 8];
  double* g1[24];
  int forcing;       /* ORC_FORCING_* */
  double* force;     /* padded 5D (x,y,k,l,m) forcing field */
};

/* Fortran index f (1-onx..n+onx) -> 0-based padded position */
#define PO(f) ((long long)(f) + ONX - 1)

static inline long long i6(const orc_state* s, int i, int j, int k, int l, int n, int m) {
  return PO(i) * s->S[0] + PO(j) * s->S[1] + PO(k) * s->S[2] + PO(l) * s->S[3] +
         PO(n) * s->S[4] + PO(m) * s->S[5];
}
static inline long long i3(const orc_state* s, int i, int j, int k) {
  return PO(i) + s->P[0] * (PO(j) + s->P[1] * PO(k));
}

/* gfortran MAX/MIN of two reals: a > b ? a : b (b returned on ties) */
static inline double fmax2(double a, double b) { return a > b ? a : b; }
static inline double fmin2(double a, double b) { return a < b ? a : b; }

/* default-real (binary32) literals of the reference, widened to binary64 */
#define LIT_1E20 ((double)1.E20f)   /* superbee_fluxes.f90:26 */
#define LIT_1EM12 ((double)1e-12f)  /* diagnose.f90:56 */

orc_state* orc_create(int nx, int ny, int nz, int nk, int nl, int nm) {
  orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
  if (!s) return NULL;
  int nn[6] = {nx, ny, nz, nk, nl, nm};
  long long st = 1;
  for (int a = 0; a < 6; a++) {
    s->n[a] = nn[a];
    s->P[a] = nn[a] + 2 * ONX;
    s->S[a] = st;
    st *= s->P[a];
  }
  s->len6 = st;
  s->len3 = s->P[0] * s->P[1] * s->P[2];
  s->sign_of_omega_i = 1.0;
  s->f0 = 1e-4;
  s->upper_refl = s->lower_refl = 1;
  /* allocate_main_module (main_module.f90:131-232): everything zeroed */
  for (int f = 0; f < ORC_N6D; f++) {
    s->f6[f] = (double*)calloc((size_t)s->len6, sizeof(double));
    if (!s->f6[f]) { orc_destroy(s); return NULL; }
  }
  for (int f = 0; f < 11; f++) {
    s->f3[f] = (double*)calloc((size_t)s->len3, sizeof(double));
    if (!s->f3[f]) { orc_destroy(s); return NULL; }
  }
  for (int f = 0; f < 24; f++) {
    s->g1[f] = (double*)calloc((size_t)s->P[f / 4], sizeof(double));
    if (!s->g1[f]) { orc_destroy(s); return NULL; }
  }
  return s;
}

/* grids, background and scalars only (no 6D fields): the context of the
 * per-cell restatement below, for fields too large for the whole-array
 * oracle */
orc_state* orc_create_light(int nx, int ny, int nz, int nk, int nl, int nm) {
  orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
  if (!s) return NULL;
  int nn[6] = {nx, ny, nz, nk, nl, nm};
  long long st = 1;
  for (int a = 0; a < 6; a++) {
    s->n[a] = nn[a];
    s->P[a] = nn[a] + 2 * ONX;
    s->S[a] = st;
    st *= s->P[a];
  }
  s->len6 = st;
  s->len3 = s->P[0] * s->P[1] * s->P[2];
  s->sign_of_omega_i = 1.0;
  s->f0 = 1e-4;
  s->upper_refl = s->lower_refl = 1;
  for (int f = 0; f < 11; f++) {
    s->f3[f] = (double*)calloc((size_t)s->len3, sizeof(double));
    if (!s->f3[f]) { orc_destroy(s); return NULL; }
  }
  for (int f = 0; f < 24; f++) {
    s->g1[f] = (double*)calloc((size_t)s->P[f / 4], sizeof(double));
    if (!s->g1[f]) { orc_destroy(s); return NULL; }
  }
  return s;
}

void orc_destroy(orc_state* s) {
  if (!s) return;
  for (int f = 0; f < ORC_N6D; f++) free(s->f6[f]);
  for (int f = 0; f < 11; f++) free(s->f3[f]);
  for (int f = 0; f < 24; f++) free(s->g1[f]);
  free(s->force);
  free(s);
}

double* orc_field(orc_state* s, int id) {
  if (id >= 0 && id < ORC_N6D) return s->f6[id];
  if (id >= ORC_NSQR && id < ORC_NSQR + 11) return s->f3[id - ORC_NSQR];
  if (id >= ORC_GRID && id < ORC_GRID + 24) return s->g1[id - ORC_GRID];
  return NULL;
}

long long orc_field_len(orc_state* s, int id) {
  if (id >= 0 && id < ORC_N6D) return s->len6;
  if (id >= ORC_NSQR && id < ORC_NSQR + 11) return s->len3;
  if (id >= ORC_GRID && id < ORC_GRID + 24) return s->P[(id - ORC_GRID) / 4];
  return 0;
}

void orc_set_scalars(orc_state* s, double dt, double f0, double sign_of_omega_i,
                     int upper, int lower, double k_fixed, double l_fixed, double m_fixed) {
  s->dt = dt; s->f0 = f0; s->sign_of_omega_i = sign_of_omega_i;
  s->upper_refl = upper; s->lower_refl = lower;
  s->k_fixed = k_fixed; s->l_fixed = l_fixed; s->m_fixed = m_fixed;
}

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* calc_grid.f90                                                             */
/* ------------------------------------------------------------------------ */

/* u_centered_grid, calc_grid.f90:300-322 (arrays 0-based here, length n) */
static void u_centered_grid(const double* dyt, double* dyu, double* yt, double* yu, int n) {
  yu[0] = 0;
  for (int i = 1; i < n; i++) yu[i] = yu[i - 1] + dyt[i];
  yt[0] = yu[0] - dyt[0] * 0.5;
  for (int i = 1; i < n; i++) yt[i] = 2 * yu[i - 1] - yt[i - 1];
  for (int i = 0; i < n - 1; i++) dyu[i] = yt[i + 1] - yt[i];
  int im = (n - 1 > 1 ? n - 1 : 1);
  dyu[n - 1] = 2 * dyt[n - 1] - dyu[im - 1];
}

int orc_calc_grid(orc_state* s) {
  for (int a = 0; a < 6; a++) {
    int n = s->n[a];
    int P = (int)s->P[a];
    double* t = s->g1[4 * a + 0];
    double* u = s->g1[4 * a + 1];
    double* d = s->g1[4 * a + 2];
    double* du = s->g1[4 * a + 3];
    /* ghost widths, calc_grid.f90:104-111 */
    for (int i = 1; i <= ONX; i++) {
      d[PO(n + i)] = d[PO(n)];
      d[PO(1 - i)] = d[PO(1)];
    }
    u_centered_grid(d, du, t, u, P);
    double sh;
    switch (a) {
      case 0: case 1:               /* calc_grid.f90:115, :124 */
        sh = du[PO(1)];
        for (int i = 0; i < P; i++) { t[i] = t[i] - sh; u[i] = u[i] - sh; }
        break;
      case 2:                       /* calc_grid.f90:133 */
        sh = u[PO(n)];
        for (int i = 0; i < P; i++) { t[i] = t[i] - sh; u[i] = u[i] - sh; }
        break;
      default: {                    /* calc_grid.f90:142-146, :155-159, :168-172 */
        double fixed = (a == 3 ? s->k_fixed : a == 4 ? s->l_fixed : s->m_fixed);
        if (n > 1) {
          sh = u[PO(n / 2)];
          for (int i = 0; i < P; i++) { t[i] = t[i] - sh; u[i] = u[i] - sh; }
        } else {
          for (int i = 0; i < P; i++) { t[i] = fixed; u[i] = fixed; }
        }
      }
    }
  }
  /* monotonicity checks, calc_grid.f90:260-293 (1-based global indices) */
  {
    const double* dzu = s->g1[4 * 2 + 3]; const double* dzt = s->g1[4 * 2 + 2];
    for (int i = 2; i <= s->n[2]; i++)
      if (dzu[PO(i)] - dzu[PO(i - 1)] > 1e-12 || dzt[PO(i)] - dzt[PO(i - 1)] > 1e-12) return 1;
    const double* dmu = s->g1[4 * 5 + 3]; const double* dmt = s->g1[4 * 5 + 2];
    for (int i = 2; i <= s->n[5] / 2; i++)
      if (dmu[PO(i)] - dmu[PO(i - 1)] > 1e-12 || dmt[PO(i)] - dmt[PO(i - 1)] > 1e-12) return 2;
    const double* dlu = s->g1[4 * 4 + 3]; const double* dlt = s->g1[4 * 4 + 2];
    for (int i = 2; i <= s->n[4] / 2; i++)
      if (dlu[PO(i)] - dlu[PO(i - 1)] > 1e-12 || dlt[PO(i)] - dlt[PO(i - 1)] > 1e-12) return 3;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* calc_parameter.f90                                                        */
/* ------------------------------------------------------------------------ */

/* Visit every padded position p with its Fortran index f along axis a:
 * p = (outer*P + pos)*S + inner, f = pos - onx + 1. */
#define FOR_AXIS(s, a, p, f)                                                  \
  for (long long outer_ = 0, S_ = (s)->S[a], P_ = (s)->P[a],                  \
                 NO_ = (s)->len6 / (S_ * P_); outer_ < NO_; outer_++)          \
    for (long long pos_ = 0; pos_ < P_; pos_++)                                \
      for (long long inner_ = 0, f = pos_ - ONX + 1; inner_ < S_; inner_++)   \
        for (long long p = (outer_ * P_ + pos_) * S_ + inner_, once_ = 1; once_; once_ = 0)

/* dst(f along a) = 0.5*(src(f) + src(f+1)) for f in [lo,hi], all other indices */
static void avg_along(const orc_state* s, double* dst, const double* src, int a, int lo, int hi) {
  const long long S = s->S[a];
  FOR_AXIS(s, a, p, f) {
    if (f >= lo && f <= hi) dst[p] = 0.5 * (src[p] + src[p + S]);
  }
}

/* v(f along a) = sgn*((al(f) - al(f-1))/d(f)) for f in [lo,hi] */
static void diff_along(const orc_state* s, double* v, const double* al, int a, int lo, int hi,
                       const double* d, int negate) {
  const long long S = s->S[a];
  FOR_AXIS(s, a, p, f) {
    if (f >= lo && f <= hi) {
      double q = (al[p] - al[p - S]) / d[PO(f)];
      v[p] = negate ? -q : q;
    }
  }
}

/* outflow-only clamp of a face velocity at the domain boundary
 * (calc_parameter.f90:55-66 and the five copies of it) */
static void clamp_faces(const orc_state* s, double* v, int a, int clamp_hi, int clamp_lo) {
  const int n = s->n[a];
  FOR_AXIS(s, a, p, f) {
    if (f == n && clamp_hi) v[p] = fmax2(0.0, v[p]);
    if (f == 0 && clamp_lo) v[p] = -fmax2(0.0, -v[p]);
  }
  const long long S = s->S[a];
  FOR_AXIS(s, a, p, f) {
    if (f > n && f <= n + ONX) v[p] = v[p - (f - n) * S];     /* v(n+i) = v(n)  */
    if (f < 0 && f >= 1 - ONX) v[p] = v[p + (0 - f) * S];     /* v(0-i) = v(0)  */
  }
}

void orc_calc_parameter(orc_state* s) {
  const int nx = s->n[0], ny = s->n[1], nz = s->n[2], nk = s->n[3], nl = s->n[4], nm = s->n[5];
  const double* kt = s->g1[4 * 3 + 0];
  const double* lt = s->g1[4 * 4 + 0];
  const double* mt = s->g1[4 * 5 + 0];
  const double* dxt = s->g1[4 * 0 + 2]; const double* dyt = s->g1[4 * 1 + 2];
  const double* dzt = s->g1[4 * 2 + 2]; const double* dkt = s->g1[4 * 3 + 2];
  const double* dlt = s->g1[4 * 4 + 2]; const double* dmt = s->g1[4 * 5 + 2];
  const double* Nsqr = s->f3[0]; const double* U = s->f3[1]; const double* V = s->f3[2];
  double* om_i = s->f6[ORC_OMEGA_I]; double* om_e = s->f6[ORC_OMEGA_E];
  double* xdot = s->f6[ORC_XDOT]; double* ydot = s->f6[ORC_YDOT]; double* zdot = s->f6[ORC_ZDOT];
  double* kdot = s->f6[ORC_KDOT]; double* ldot = s->f6[ORC_LDOT]; double* mdot = s->f6[ORC_MDOT];
  const double f0 = s->f0;

  /* automatic array aloc (calc_parameter.f90:7-8); -finit-real=nan in make.inc:30 */
  double* aloc = (double*)malloc((size_t)s->len6 * sizeof(double));
  for (long long p = 0; p < s->len6; p++) aloc[p] = NAN;

  /* dispersion relation on all padded points, calc_parameter.f90:13-27 */
  for (int m = 1 - ONX; m <= nm + ONX; m++)
  for (int n = 1 - ONX; n <= nl + ONX; n++)
  for (int l = 1 - ONX; l <= nk + ONX; l++)
  for (int k = 1 - ONX; k <= nz + ONX; k++)
  for (int j = 1 - ONX; j <= ny + ONX; j++)
  for (int i = 1 - ONX; i <= nx + ONX; i++) {
    double kh2 = lt[PO(n)] * lt[PO(n)] + kt[PO(l)] * kt[PO(l)];
    long long p = i6(s, i, j, k, l, n, m), q = i3(s, i, j, k);
    om_i[p] = s->sign_of_omega_i *
              sqrt((Nsqr[q] * kh2 + f0 * f0 * (mt[PO(m)] * mt[PO(m)])) / (mt[PO(m)] * mt[PO(m)] + kh2));
    om_e[p] = om_i[p] + kt[PO(l)] * U[q] + lt[PO(n)] * V[q];
  }

  /* x/k pair, calc_parameter.f90:31-105 */
  if (nx > 1 && nk > 1) {
    avg_along(s, aloc, om_e, 0, 1 - ONX, nx + ONX - 1);
    avg_along(s, aloc, om_e, 3, 1 - ONX, nk + ONX - 1);     /* overwrites the x average */
    diff_along(s, xdot, aloc, 3, 2 - ONX, nk + ONX, dkt, 0);
    clamp_faces(s, xdot, 0, 1, 1);
    diff_along(s, kdot, aloc, 0, 2 - ONX, nx + ONX, dxt, 1);
    clamp_faces(s, kdot, 3, 1, 1);
  } else {
    for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
    for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
      double kh2 = lt[PO(n)] * lt[PO(n)] + kt[PO(l)] * kt[PO(l)];
      long long p = i6(s, i, j, k, l, n, m), q = i3(s, i, j, k);
      double m2 = mt[PO(m)] * mt[PO(m)];
      double den = m2 + kh2;
      xdot[p] = U[q] + (Nsqr[q] - f0 * f0) / om_i[p] * m2 / (den * den) * kt[PO(l)];
    }
  }

  /* y/l pair, calc_parameter.f90:109-183 */
  if (ny > 1 && nl > 1) {
    avg_along(s, aloc, om_e, 1, 1 - ONX, ny + ONX - 1);
    avg_along(s, aloc, om_e, 4, 1 - ONX, nl + ONX - 1);
    diff_along(s, ydot, aloc, 4, 2 - ONX, nl + ONX, dlt, 0);
    clamp_faces(s, ydot, 1, 1, 1);
    diff_along(s, ldot, aloc, 1, 2 - ONX, ny + ONX, dyt, 1);
    clamp_faces(s, ldot, 4, 1, 1);
  } else {
    for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
    for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
      double kh2 = lt[PO(n)] * lt[PO(n)] + kt[PO(l)] * kt[PO(l)];
      long long p = i6(s, i, j, k, l, n, m), q = i3(s, i, j, k);
      double m2 = mt[PO(m)] * mt[PO(m)];
      double den = m2 + kh2;
      ydot[p] = V[q] + (Nsqr[q] - f0 * f0) / om_i[p] * m2 / (den * den) * lt[PO(n)];
    }
  }

  /* z/m pair (no degenerate branch), calc_parameter.f90:187-237 */
  avg_along(s, aloc, om_e, 2, 1 - ONX, nz + ONX - 1);
  avg_along(s, aloc, om_e, 5, 1 - ONX, nm + ONX - 1);
  diff_along(s, zdot, aloc, 5, 2 - ONX, nm + ONX, dmt, 0);
  clamp_faces(s, zdot, 2, !s->upper_refl, !s->lower_refl);   /* ghost copies always */
  diff_along(s, mdot, aloc, 2, 2 - ONX, nz + ONX, dzt, 1);
  clamp_faces(s, mdot, 5, 1, 1);

  /* mean-flow growth rates, calc_parameter.f90:240-260 */
  double* lx = s->f6[ORC_LAMBDA_X]; double* ly = s->f6[ORC_LAMBDA_Y]; double* lz = s->f6[ORC_LAMBDA_Z];
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    long long p = i6(s, i, j, k, l, n, m), q = i3(s, i, j, k);
    double oi = om_i[p];
    lx[p] = 1. / oi * kt[PO(l)] *
            ((xdot[p] - U[q]) * (U[i3(s, i + 1, j, k)] - U[i3(s, i - 1, j, k)]) / (2 * dxt[PO(i)]) +
             (ydot[p] - V[q]) * (V[i3(s, i + 1, j, k)] - V[i3(s, i - 1, j, k)]) / (2 * dxt[PO(i)]));
    ly[p] = 1. / oi * lt[PO(n)] *
            ((xdot[p] - U[q]) * (U[i3(s, i, j + 1, k)] - U[i3(s, i, j - 1, k)]) / (2 * dyt[PO(j)]) +
             (ydot[p] - V[q]) * (V[i3(s, i, j + 1, k)] - V[i3(s, i, j - 1, k)]) / (2 * dyt[PO(j)]));
    lz[p] = 1. / oi * zdot[p] *
            (kt[PO(l)] * (U[i3(s, i, j, k + 1)] - U[i3(s, i, j, k - 1)]) / (2 * dzt[PO(k)]) +
             lt[PO(n)] * (V[i3(s, i, j, k + 1)] - V[i3(s, i, j, k - 1)]) / (2 * dzt[PO(k)]));
  }
  free(aloc);
}

/* ------------------------------------------------------------------------ */
/* integrate.f90 + reflection_condition + superbee_fluxes.f90                */
/* ------------------------------------------------------------------------ */

/* Loop helpers: iterate interior (j..m) with i innermost, pointer offsets.
 * The outer m loop is the one split across OpenMP threads; no loop here has
 * a cross-iteration dependence, so threading does not change any result. */

/* reflection_condition, serial branch: parallel_mpi.f90:837-841, :867-871 */
static void reflection_condition(orc_state* s, double* E) {
  const int nx = s->n[0], ny = s->n[1], nz = s->n[2], nk = s->n[3], nl = s->n[4], nm = s->n[5];
  if (s->upper_refl) {
    for (int ii = 1; ii <= ONX; ii++)
      for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
      for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++)
        E[i6(s, i, j, nz + ii, l, n, m)] = E[i6(s, i, j, nz - ii + 1, l, n, nm + 1 - m)];
  }
  if (s->lower_refl) {
    for (int ii = 1; ii <= ONX; ii++)
      for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
      for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++)
        E[i6(s, i, j, 1 - ii, l, n, m)] = E[i6(s, i, j, 1 + ii - 1, l, n, nm + 1 - m)];
  }
}

/* E(n+i) = E(n), E(1-i) = E(1) along axis a, other axes interior
 * (integrate.f90:23-94) */
static void outflow_fill(orc_state* s, double* E, int a) {
  const int n_a = s->n[a];
  int lo[6], hi[6];
  for (int b = 0; b < 6; b++) { lo[b] = 1; hi[b] = s->n[b]; }
  lo[a] = hi[a] = 1;  /* the axis itself is handled below */
  const long long S = s->S[a];
  for (int m = lo[5]; m <= hi[5]; m++) for (int n = lo[4]; n <= hi[4]; n++)
  for (int l = lo[3]; l <= hi[3]; l++) for (int k = lo[2]; k <= hi[2]; k++)
  for (int j = lo[1]; j <= hi[1]; j++) for (int i = lo[0]; i <= hi[0]; i++) {
    long long p1 = i6(s, i, j, k, l, n, m);            /* index 1 along a */
    long long pn = p1 + (long long)(n_a - 1) * S;      /* index n along a */
    for (int ii = 1; ii <= ONX; ii++) {
      E[pn + ii * S] = E[pn];
      E[p1 - ii * S] = E[p1];
    }
  }
}

/* Limiter(Cr) statement function, superbee_fluxes.f90:10 */
static inline double limiter(double Cr) {
  return fmax2(0.0, fmax2(fmin2(1.0, 2.0 * Cr), fmin2(2.0, Cr)));
}

/* one axis of superbee_fluxes.f90 (x :12-37, y :39-64, z :66-91, k :93-118,
 * l :120-145, m :147-172): faces f = 0..n along a, other axes interior */
static void superbee_axis(orc_state* s, int a, const double* vel, const double* dgrid, double* flux) {
  const double* E = s->f6[ORC_E];
  const long long S = s->S[a];
  const double dt = s->dt;
  const int nm = s->n[5];
  int lo[6], hi[6];
  for (int b = 0; b < 6; b++) { lo[b] = 1; hi[b] = s->n[b]; }
  lo[a] = 0;
  int mlo = lo[5], mhi = hi[5];
  (void)nm;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int m = mlo; m <= mhi; m++)
  for (int n = lo[4]; n <= hi[4]; n++) for (int l = lo[3]; l <= hi[3]; l++)
  for (int k = lo[2]; k <= hi[2]; k++) for (int j = lo[1]; j <= hi[1]; j++)
  for (int i = lo[0]; i <= hi[0]; i++) {
    int f = (a == 0 ? i : a == 1 ? j : a == 2 ? k : a == 3 ? l : a == 4 ? n : m);
    long long p = i6(s, i, j, k, l, n, m);
    double v = vel[p];
    double uCFL = fabs(v * dt / dgrid[PO(f)]);
    double Rjp = E[p + 2 * S] - E[p + S];
    double Rj = E[p + S] - E[p];
    double Rjm = E[p] - E[p - S];
    double Cr;
    if (Rj != 0.) {
      if (v > 0) Cr = Rjm / Rj; else Cr = Rjp / Rj;
    } else {
      if (v > 0) Cr = Rjm * LIT_1E20; else Cr = Rjp * LIT_1E20;
    }
    Cr = limiter(Cr);
    flux[p] = v * (E[p + S] + E[p]) * 0.5 - fabs(v) * ((1. - Cr) + uCFL * Cr) * Rj * 0.5;
  }
}

/* dE -= (flux(f) - flux(f-1))/d(f), interior (integrate.f90:106-200) */
static void divergence_axis(orc_state* s, int a, const double* flux, const double* dgrid) {
  double* dE = s->f6[ORC_DE];
  const long long S = s->S[a];
  const int nx = s->n[0], ny = s->n[1], nz = s->n[2], nk = s->n[3], nl = s->n[4], nm = s->n[5];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int m = 1; m <= nm; m++)
  for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++) for (int k = 1; k <= nz; k++)
  for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    int f = (a == 0 ? i : a == 1 ? j : a == 2 ? k : a == 3 ? l : a == 4 ? n : m);
    long long p = i6(s, i, j, k, l, n, m);
    dE[p] = dE[p] - (flux[p] - flux[p - S]) / dgrid[PO(f)];
  }
}

void orc_integrate(orc_state* s) {
  const int nx = s->n[0], ny = s->n[1], nz = s->n[2], nk = s->n[3], nl = s->n[4], nm = s->n[5];
  double* E = s->f6[ORC_E];
  double* dE = s->f6[ORC_DE];
  double* meanfl = s->f6[ORC_MEANFL];
  /* border_exchg(E) is a no-op on one rank (parallel_mpi.f90:506-618) */
  reflection_condition(s, E);                        /* integrate.f90:20 */
  if (nx > 1) outflow_fill(s, E, 0);                 /* integrate.f90:24-33 */
  if (ny > 1) outflow_fill(s, E, 1);                 /* :36-45 */
  {                                                  /* :48-57, no n>1 guard */
    const long long S = s->S[2];
    for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
    for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
      long long p1 = i6(s, i, j, 1, l, n, m), pn = i6(s, i, j, nz, l, n, m);
      for (int ii = 1; ii <= ONX; ii++) {
        if (!s->upper_refl) E[pn + ii * S] = E[pn];
        if (!s->lower_refl) E[p1 - ii * S] = E[p1];
      }
    }
  }
  if (nk > 1) outflow_fill(s, E, 3);                 /* :61-70 */
  if (nl > 1) outflow_fill(s, E, 4);                 /* :73-82 */
  if (nm > 1) outflow_fill(s, E, 5);                 /* :85-94 */

  /* superbee_fluxes, integrate.f90:99 */
  const int vid[6] = {ORC_XDOT, ORC_YDOT, ORC_ZDOT, ORC_KDOT, ORC_LDOT, ORC_MDOT};
  for (int a = 0; a < 6; a++)
    if (s->n[a] > 1) superbee_axis(s, a, s->f6[vid[a]], s->g1[4 * a + 2], s->f6[ORC_FLUX_X + a]);

  /* time tendency, integrate.f90:105-200 */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int m = 1; m <= nm; m++)
  for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++) for (int k = 1; k <= nz; k++)
  for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) dE[i6(s, i, j, k, l, n, m)] = 0.;
  for (int a = 0; a < 6; a++)
    if (s->n[a] > 1) divergence_axis(s, a, s->f6[ORC_FLUX_X + a], s->g1[4 * a + 2]);

  /* mean-flow interaction, integrate.f90:202-252, then update :255-268 */
  const double* lam[3] = {s->f6[ORC_LAMBDA_X], s->f6[ORC_LAMBDA_Y], s->f6[ORC_LAMBDA_Z]};
  const int use[3] = {nx > 1, ny > 1, nz > 1};
  const double dt = s->dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int m = 1; m <= nm; m++)
  for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++) for (int k = 1; k <= nz; k++)
  for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    long long p = i6(s, i, j, k, l, n, m);
    double mf = 0.;
    for (int c = 0; c < 3; c++)
      if (use[c]) mf = mf + E[p] * lam[c][p];
    meanfl[p] = mf;
    dE[p] = dE[p] - meanfl[p];
    E[p] = E[p] + dt * dE[p];
  }
}

/* ------------------------------------------------------------------------ */
/* set_forcing of the forced configurations (called before integrate,         */
/* main.f90:69-70); both act on the bottom z plane (Fortran k = 1) only        */
/* ------------------------------------------------------------------------ */

static long long len5(const orc_state* s) { return s->P[0] * s->P[1] * s->P[3] * s->P[4] * s->P[5]; }

/* F(i,j,l,n,m) of a padded 5D array with axes x,y,k,l,m */
static inline long long i5(const orc_state* s, int i, int j, int l, int n, int m) {
  return PO(i) + s->P[0] * (PO(j) + s->P[1] * (PO(l) + s->P[3] * (PO(n) + s->P[4] * PO(m))));
}

int orc_set_forcing(orc_state* s, int kind, const double* F) {
  if (kind != ORC_FORCING_NONE && kind != ORC_FORCING_FLUX && kind != ORC_FORCING_RELAX) return 1;
  if (kind != ORC_FORCING_NONE && !F) return 1;
  free(s->force);
  s->force = NULL;
  s->forcing = ORC_FORCING_NONE;
  if (kind == ORC_FORCING_NONE) return 0;
  s->force = (double*)malloc((size_t)len5(s) * sizeof(double));
  if (!s->force) return 2;
  memcpy(s->force, F, (size_t)len5(s) * sizeof(double));
  s->forcing = kind;
  return 0;
}

void orc_apply_forcing(orc_state* s) {
  if (s->forcing == ORC_FORCING_NONE) return;
  const int nx = s->n[0], ny = s->n[1], nk = s->n[3], nl = s->n[4], nm = s->n[5];
  double* E = s->f6[ORC_E];
  const double* zdot = s->f6[ORC_ZDOT];
  const double dz = s->g1[4 * 2 + 2][PO(1)];   /* dzt(1) */
  const double dt = s->dt;
  const int k = 1;
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    const long long p = i6(s, i, j, k, l, n, m);
    const double f = s->force[i5(s, i, j, l, n, m)];
    if (s->forcing == ORC_FORCING_FLUX)
      E[p] = E[p] + dt * f / dz;                                   /* lee1.f90:206 */
    else
      E[p] = E[p] - dt * fmax2(0., zdot[p]) * (E[p] - f) / dz;     /* critical_gm1.f90:132-133 */
  }
}

void orc_integrate_n(orc_state* s, int nsteps) {
  for (int t = 0; t < nsteps; t++) {
    orc_apply_forcing(s);
    orc_integrate(s);
  }
}

/* ------------------------------------------------------------------------ */
/* diagnose.f90 (energy budget; NetCDF output is out of the path)            */
/* ------------------------------------------------------------------------ */

void orc_diagnose(orc_state* s, orc_budget* o) {
  const int nx = s->n[0], ny = s->n[1], nz = s->n[2], nk = s->n[3], nl = s->n[4], nm = s->n[5];
  const double* dxt = s->g1[2]; const double* dyt = s->g1[6]; const double* dzt = s->g1[10];
  const double* dkt = s->g1[14]; const double* dlt = s->g1[18]; const double* dmt = s->g1[22];
  const double* E = s->f6[ORC_E]; const double* dE = s->f6[ORC_DE]; const double* meanfl = s->f6[ORC_MEANFL];
  const double* xdot = s->f6[ORC_XDOT]; const double* ydot = s->f6[ORC_YDOT]; const double* zdot = s->f6[ORC_ZDOT];
  const double* kdot = s->f6[ORC_KDOT]; const double* ldot = s->f6[ORC_LDOT]; const double* mdot = s->f6[ORC_MDOT];
  const double *fx = s->f6[ORC_FLUX_X], *fy = s->f6[ORC_FLUX_Y], *fz = s->f6[ORC_FLUX_Z];
  const double *fk = s->f6[ORC_FLUX_K], *fl = s->f6[ORC_FLUX_L], *fm = s->f6[ORC_FLUX_M];
  double* E_int = s->f3[3]; double* meanfl_int = s->f3[4];
  double* diss_ks = s->f3[5]; double* diss_ke = s->f3[6]; double* diss_ls = s->f3[7];
  double* diss_le = s->f3[8]; double* diss_ms = s->f3[9]; double* diss_me = s->f3[10];

  double umax = 0, vmax = 0, wmax = 0, kmax = 0, lmax = 0, mmax = 0, eint = 0, mflint = 0, mfl_max = 0;
  /* diagnose.f90:46-68 */
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    long long p = i6(s, i, j, k, l, n, m);
    double fxa = dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
    eint = eint + dE[p] * fxa;
    mflint = mflint + meanfl[p] * fxa;
    mfl_max = fmax2(mfl_max, fabs(meanfl[p]) / fmax2(LIT_1EM12, E[p]));
    umax = fmax2(umax, fabs(xdot[p]));
    vmax = fmax2(vmax, fabs(ydot[p]));
    wmax = fmax2(wmax, fabs(zdot[p]));
    kmax = fmax2(kmax, fabs(kdot[p]));
    lmax = fmax2(lmax, fabs(ldot[p]));
    mmax = fmax2(mmax, fabs(mdot[p]));
  }
  /* E_int, meanfl_int: diagnose.f90:84-98 */
  for (long long q = 0; q < s->len3; q++) { E_int[q] = 0.; meanfl_int[q] = 0; }
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    long long p = i6(s, i, j, k, l, n, m), q = i3(s, i, j, k);
    E_int[q] = E_int[q] + E[p] * dlt[PO(n)] * dmt[PO(m)] * dkt[PO(l)];
    meanfl_int[q] = meanfl_int[q] + meanfl[p] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  }
  double bfl_xs = 0, bfl_xe = 0, bfl_ys = 0, bfl_ye = 0, bfl_zs = 0, bfl_ze = 0;
  double bfl_ks = 0, bfl_ke = 0, bfl_ls = 0, bfl_le = 0, bfl_ms = 0, bfl_me = 0;
  /* x boundaries, diagnose.f90:103-128 */
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++)
    bfl_xs = bfl_xs + fx[i6(s, 0, j, k, l, n, m)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++)
    bfl_xe = bfl_xe + fx[i6(s, nx, j, k, l, n, m)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  /* y boundaries, :131-156 */
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int i = 1; i <= nx; i++)
    bfl_ys = bfl_ys + fy[i6(s, i, 0, k, l, n, m)] * dxt[PO(i)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int i = 1; i <= nx; i++)
    bfl_ye = bfl_ye + fy[i6(s, i, ny, k, l, n, m)] * dxt[PO(i)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  /* z boundaries, :159-184 */
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++)
    bfl_zs = bfl_zs + fz[i6(s, i, j, 0, l, n, m)] * dxt[PO(i)] * dyt[PO(j)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++)
    bfl_ze = bfl_ze + fz[i6(s, i, j, nz, l, n, m)] * dxt[PO(i)] * dyt[PO(j)] * dkt[PO(l)] * dlt[PO(n)] * dmt[PO(m)];
  /* k boundaries, :186-215 */
  for (long long q = 0; q < s->len3; q++) { diss_ks[q] = 0; diss_ke[q] = 0.; }
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    double fl0 = fk[i6(s, i, j, k, 0, n, m)];
    bfl_ks = bfl_ks + fl0 * dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dlt[PO(n)] * dmt[PO(m)];
    diss_ks[i3(s, i, j, k)] = diss_ks[i3(s, i, j, k)] + fl0 * dlt[PO(n)] * dmt[PO(m)];
  }
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    double fl1 = fk[i6(s, i, j, k, nk, n, m)];
    bfl_ke = bfl_ke + fl1 * dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dlt[PO(n)] * dmt[PO(m)];
    diss_ke[i3(s, i, j, k)] = diss_ke[i3(s, i, j, k)] + fl1 * dlt[PO(n)] * dmt[PO(m)];
  }
  /* l boundaries, :217-246 */
  for (long long q = 0; q < s->len3; q++) { diss_ls[q] = 0; diss_le[q] = 0.; }
  for (int m = 1; m <= nm; m++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    double fl0 = fl[i6(s, i, j, k, l, 0, m)];
    bfl_ls = bfl_ls + fl0 * dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dmt[PO(m)];
    diss_ls[i3(s, i, j, k)] = diss_ls[i3(s, i, j, k)] + fl0 * dkt[PO(l)] * dmt[PO(m)];
  }
  for (int m = 1; m <= nm; m++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    double fl1 = fl[i6(s, i, j, k, l, nl, m)];
    bfl_le = bfl_le + fl1 * dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dmt[PO(m)];
    diss_le[i3(s, i, j, k)] = diss_le[i3(s, i, j, k)] + fl1 * dkt[PO(l)] * dmt[PO(m)];
  }
  /* m boundaries, :248-277 */
  for (long long q = 0; q < s->len3; q++) { diss_ms[q] = 0.; diss_me[q] = 0.; }
  for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    double fl0 = fm[i6(s, i, j, k, l, n, 0)];
    bfl_ms = bfl_ms + fl0 * dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)];
    diss_ms[i3(s, i, j, k)] = diss_ms[i3(s, i, j, k)] + fl0 * dkt[PO(l)] * dlt[PO(n)];
  }
  for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    double fl1 = fm[i6(s, i, j, k, l, n, nm)];
    bfl_me = bfl_me + fl1 * dxt[PO(i)] * dyt[PO(j)] * dzt[PO(k)] * dkt[PO(l)] * dlt[PO(n)];
    diss_me[i3(s, i, j, k)] = diss_me[i3(s, i, j, k)] + fl1 * dkt[PO(l)] * dlt[PO(n)];
  }
  /* CFL, diagnose.f90:295-313 */
  double cfl[6] = {0, 0, 0, 0, 0, 0};
  const double vmx[6] = {umax, vmax, wmax, kmax, lmax, mmax};
  for (int a = 0; a < 6; a++) {
    const double* d = s->g1[4 * a + 2];
    for (int i = 1; i <= s->n[a]; i++) cfl[a] = fmax2(cfl[a], vmx[a] * s->dt / d[PO(i)]);
  }
  o->eint = eint; o->mflint = mflint; o->mfl_max = mfl_max;
  o->umax = umax; o->vmax = vmax; o->wmax = wmax; o->kmax = kmax; o->lmax = lmax; o->mmax = mmax;
  o->bfl_xs = bfl_xs; o->bfl_xe = bfl_xe; o->bfl_ys = bfl_ys; o->bfl_ye = bfl_ye;
  o->bfl_zs = bfl_zs; o->bfl_ze = bfl_ze; o->bfl_ks = bfl_ks; o->bfl_ke = bfl_ke;
  o->bfl_ls = bfl_ls; o->bfl_le = bfl_le; o->bfl_ms = bfl_ms; o->bfl_me = bfl_me;
  o->cfl_x = cfl[0]; o->cfl_y = cfl[1]; o->cfl_z = cfl[2];
  o->cfl_k = cfl[3]; o->cfl_l = cfl[4]; o->cfl_m = cfl[5];
  /* diagnose.f90:327-328 */
  o->residual = eint + mflint + bfl_xe + bfl_ye + bfl_ze + bfl_ke + bfl_le + bfl_me
                - bfl_xs - bfl_ys - bfl_zs - bfl_ks - bfl_ls - bfl_ms;
}

double orc_max_rate(orc_state* s) {
  const int vid[6] = {ORC_XDOT, ORC_YDOT, ORC_ZDOT, ORC_KDOT, ORC_LDOT, ORC_MDOT};
  const int nx = s->n[0], ny = s->n[1], nz = s->n[2], nk = s->n[3], nl = s->n[4], nm = s->n[5];
  double best = 0;
  for (int m = 1; m <= nm; m++) for (int n = 1; n <= nl; n++) for (int l = 1; l <= nk; l++)
  for (int k = 1; k <= nz; k++) for (int j = 1; j <= ny; j++) for (int i = 1; i <= nx; i++) {
    const int f[6] = {i, j, k, l, n, m};
    long long p = i6(s, i, j, k, l, n, m);
    double r = 0;
    for (int a = 0; a < 6; a++) {
      if (s->n[a] <= 1) continue;
      const double* v = s->f6[vid[a]];
      double vm = fmax2(fabs(v[p - s->S[a]]), fabs(v[p]));
      r = r + vm / s->g1[4 * a + 2][PO(f[a])];
    }
    best = fmax2(best, r);
  }
  return best;
}

/* ------------------------------------------------------------------------ */
/* Per-cell restatement (spot checks of fields too large for the arrays      */
/* above): the state after one step at one interior cell, from the pre-step  */
/* interior state, the grids and the background.  Every value is formed by   */
/* the same expressions, in the same order, as orc_calc_parameter (the       */
/* dispersion relation, the pair averages with the overwritten aloc, the     */
/* clamps), the boundary fill of orc_integrate and superbee_axis /           */
/* divergence_axis / the update, so it is bit-identical to the whole-array   */
/* oracle (checked on small cases by the tests).                             */
/* ------------------------------------------------------------------------ */

/* om_e (and om_i) at a padded point, calc_parameter.f90:13-27 */
static double pt_om(const orc_state* s, const int x[6], double* om_i_out) {
  const double* kt = s->g1[4 * 3 + 0];
  const double* lt = s->g1[4 * 4 + 0];
  const double* mt = s->g1[4 * 5 + 0];
  const double* Nsqr = s->f3[0]; const double* U = s->f3[1]; const double* V = s->f3[2];
  const double f0 = s->f0;
  const int l = x[3], n = x[4], m = x[5];
  double kh2 = lt[PO(n)] * lt[PO(n)] + kt[PO(l)] * kt[PO(l)];
  long long q = i3(s, x[0], x[1], x[2]);
  double oi = s->sign_of_omega_i *
              sqrt((Nsqr[q] * kh2 + f0 * f0 * (mt[PO(m)] * mt[PO(m)])) / (mt[PO(m)] * mt[PO(m)] + kh2));
  if (om_i_out) *om_i_out = oi;
  return oi + kt[PO(l)] * U[q] + lt[PO(n)] * V[q];
}

/* the pair average aloc(t along b) = 0.5*(om_e(t) + om_e(t+1)) at point x */
static double pt_avg(const orc_state* s, const int x[6], int b, int t) {
  int y[6];
  memcpy(y, x, sizeof y);
  y[b] = t;
  double e0 = pt_om(s, y, NULL);
  y[b] = t + 1;
  double e1 = pt_om(s, y, NULL);
  return 0.5 * (e0 + e1);
}

/* face velocity of axis a at face index f (Fortran), the other indices
 * those of `cell` (interior) */
static double pt_vel(const orc_state* s, int a, const int cell[6], int f) {
  int x[6];
  memcpy(x, cell, sizeof x);
  x[a] = f;
  const double f0 = s->f0;
  if (a == 0 || a == 1) {                 /* xdot / ydot: difference along k / l */
    const int b = a + 3;
    if (s->n[a] > 1 && s->n[b] > 1) {
      const double* d = s->g1[4 * b + 2];
      double q = (pt_avg(s, x, b, x[b]) - pt_avg(s, x, b, x[b] - 1)) / d[PO(x[b])];
      if (f == s->n[a]) q = fmax2(0.0, q);
      if (f == 0) q = -fmax2(0.0, -q);
      return q;
    }
    if (f < 1 || f > s->n[a]) return 0.0;   /* the analytic branch fills the interior only */
    const double* kt = s->g1[4 * 3 + 0];
    const double* lt = s->g1[4 * 4 + 0];
    const double* mt = s->g1[4 * 5 + 0];
    const double* Nsqr = s->f3[0];
    const double* UV = a == 0 ? s->f3[1] : s->f3[2];
    double oi;
    pt_om(s, x, &oi);
    double kh2 = lt[PO(x[4])] * lt[PO(x[4])] + kt[PO(x[3])] * kt[PO(x[3])];
    long long q = i3(s, x[0], x[1], x[2]);
    double m2 = mt[PO(x[5])] * mt[PO(x[5])];
    double den = m2 + kh2;
    return UV[q] + (Nsqr[q] - f0 * f0) / oi * m2 / (den * den) * (a == 0 ? kt[PO(x[3])] : lt[PO(x[4])]);
  }
  if (a == 3 || a == 4) {                 /* kdot / ldot: difference along x / y */
    const int b = a - 3;
    if (!(s->n[b] > 1 && s->n[a] > 1)) return 0.0;
    const double* d = s->g1[4 * b + 2];
    int xm[6];
    memcpy(xm, x, sizeof xm);
    xm[b] = x[b] - 1;
    double q = (pt_avg(s, x, a, f) - pt_avg(s, xm, a, f)) / d[PO(x[b])];
    double v = -q;
    if (f == s->n[a]) v = fmax2(0.0, v);
    if (f == 0) v = -fmax2(0.0, -v);
    return v;
  }
  if (a == 2) {                           /* zdot: difference along m, no analytic branch */
    const double* d = s->g1[4 * 5 + 2];
    double q = (pt_avg(s, x, 5, x[5]) - pt_avg(s, x, 5, x[5] - 1)) / d[PO(x[5])];
    if (f == s->n[2] && !s->upper_refl) q = fmax2(0.0, q);
    if (f == 0 && !s->lower_refl) q = -fmax2(0.0, -q);
    return q;
  }
  {                                       /* mdot: difference along z */
    const double* d = s->g1[4 * 2 + 2];
    int xm[6];
    memcpy(xm, x, sizeof xm);
    xm[2] = x[2] - 1;
    double q = (pt_avg(s, x, 5, f) - pt_avg(s, xm, 5, f)) / d[PO(x[2])];
    double v = -q;
    if (f == s->n[5]) v = fmax2(0.0, v);
    if (f == 0) v = -fmax2(0.0, -v);
    return v;
  }
}

/* E at `cell` with index t along axis a after the boundary fill of
 * orc_integrate (reflection with m reversed, else the edge cell); E0 is
 * the interior, x fastest */
static double pt_E(const orc_state* s, const double* E0, const int cell[6], int a, int t) {
  int x[6];
  memcpy(x, cell, sizeof x);
  const int n = s->n[a];
  if (t >= 1 && t <= n) {
    x[a] = t;
  } else if (a == 2 && t > n && s->upper_refl) {
    x[2] = 2 * n + 1 - t;
    x[5] = s->n[5] + 1 - x[5];
  } else if (a == 2 && t < 1 && s->lower_refl) {
    x[2] = 1 - t;
    x[5] = s->n[5] + 1 - x[5];
  } else {
    x[a] = t < 1 ? 1 : n;
  }
  long long p = 0;
  for (int b = 5; b >= 0; b--) p = p * s->n[b] + (x[b] - 1);
  return E0[p];
}

/* superbee flux at face f of axis a (superbee_fluxes.f90:19-30) */
static double pt_flux(const orc_state* s, const double* E0, const int cell[6], int a, int f) {
  const double* dgrid = s->g1[4 * a + 2];
  const double dt = s->dt;
  double v = pt_vel(s, a, cell, f);
  double uCFL = fabs(v * dt / dgrid[PO(f)]);
  double Ep2 = pt_E(s, E0, cell, a, f + 2), Ep1 = pt_E(s, E0, cell, a, f + 1);
  double Ef = pt_E(s, E0, cell, a, f), Em1 = pt_E(s, E0, cell, a, f - 1);
  double Rjp = Ep2 - Ep1;
  double Rj = Ep1 - Ef;
  double Rjm = Ef - Em1;
  double Cr;
  if (Rj != 0.) {
    if (v > 0) Cr = Rjm / Rj; else Cr = Rjp / Rj;
  } else {
    if (v > 0) Cr = Rjm * LIT_1E20; else Cr = Rjp * LIT_1E20;
  }
  Cr = limiter(Cr);
  return v * (Ep1 + Ef) * 0.5 - fabs(v) * ((1. - Cr) + uCFL * Cr) * Rj * 0.5;
}

/* growth rates at an interior cell, calc_parameter.f90:240-260 */
static void pt_lambda(const orc_state* s, const int c[6], double lam[3]) {
  const double* kt = s->g1[4 * 3 + 0];
  const double* lt = s->g1[4 * 4 + 0];
  const double* dxt = s->g1[4 * 0 + 2]; const double* dyt = s->g1[4 * 1 + 2];
  const double* dzt = s->g1[4 * 2 + 2];
  const double* U = s->f3[1]; const double* V = s->f3[2];
  const int i = c[0], j = c[1], k = c[2], l = c[3], n = c[4];
  double oi;
  pt_om(s, c, &oi);
  long long q = i3(s, i, j, k);
  double xd = pt_vel(s, 0, c, i), yd = pt_vel(s, 1, c, j), zd = pt_vel(s, 2, c, k);
  lam[0] = 1. / oi * kt[PO(l)] *
           ((xd - U[q]) * (U[i3(s, i + 1, j, k)] - U[i3(s, i - 1, j, k)]) / (2 * dxt[PO(i)]) +
            (yd - V[q]) * (V[i3(s, i + 1, j, k)] - V[i3(s, i - 1, j, k)]) / (2 * dxt[PO(i)]));
  lam[1] = 1. / oi * lt[PO(n)] *
           ((xd - U[q]) * (U[i3(s, i, j + 1, k)] - U[i3(s, i, j - 1, k)]) / (2 * dyt[PO(j)]) +
            (yd - V[q]) * (V[i3(s, i, j + 1, k)] - V[i3(s, i, j - 1, k)]) / (2 * dyt[PO(j)]));
  lam[2] = 1. / oi * zd *
           (kt[PO(l)] * (U[i3(s, i, j, k + 1)] - U[i3(s, i, j, k - 1)]) / (2 * dzt[PO(k)]) +
            lt[PO(n)] * (V[i3(s, i, j, k + 1)] - V[i3(s, i, j, k - 1)]) / (2 * dzt[PO(k)]));
}

/* E after one step (integrate.f90:105-268) at the interior cells
 * cells[6*q .. 6*q+5] (Fortran indices), from the interior pre-step state
 * E0 (x fastest); needs the grids, background and scalars of s */
void orc_point_steps(const orc_state* s, const double* E0, const int* cells, long long count, double* out) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (long long q = 0; q < count; q++) {
    const int* c = cells + 6 * q;
    double dE = 0.;
    for (int a = 0; a < 6; a++) {
      if (s->n[a] <= 1) continue;
      const double* dgrid = s->g1[4 * a + 2];
      const int f = c[a];
      double fr = pt_flux(s, E0, c, a, f);
      double fl = pt_flux(s, E0, c, a, f - 1);
      dE = dE - (fr - fl) / dgrid[PO(f)];
    }
    double lam[3];
    pt_lambda(s, c, lam);
    const int use[3] = {s->n[0] > 1, s->n[1] > 1, s->n[2] > 1};
    const double e = pt_E(s, E0, c, 0, c[0]);
    double mf = 0.;
    for (int cc = 0; cc < 3; cc++)
      if (use[cc]) mf = mf + e * lam[cc];
    dE = dE - mf;
    out[q] = e + s->dt * dE;
  }
}
