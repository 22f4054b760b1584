/*
 * rt_oracle.h -- CPU restatement of the raytracer_3D time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * library (libraytracer_gb300.so).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference legs may load it.  The product
 * path never calls it.
 *
 * Parity status: UNPINNED by reference outputs.  The reference
 * (Fortran 90 + MPI + NetCDF) cannot be compiled here (no gfortran, no MPI,
 * no netcdf-fortran) and ships no tests, fixtures or golden vectors.  The
 * restatement is pinned instead by known-answer tests derived from the
 * mathematics of the scheme (tests/test_oracle_kat.py) and by golden vectors
 * generated from this oracle with the generating script committed
 * (tests/golden/make_golden.py).
 *
 * Arrays follow the reference layout exactly: Fortran column-major order,
 * x fastest, every axis padded by onx=2 ghost cells on both sides
 * (for_src/main_module.f90:114, :131-238).  A 6D field has
 * (nx+4)(ny+4)(nz+4)(nk+4)(nl+4)(nm+4) doubles; Fortran index f of an axis
 * lives at 0-based position f+1 (lbound 1-onx = -1).
 * All arithmetic is IEEE binary64 in the reference's operation order; build
 * with -ffp-contract=off so that no multiply-add is fused.
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

/* field identifiers for orc_field() */
enum {
  ORC_E = 0, ORC_DE, ORC_XDOT, ORC_YDOT, ORC_ZDOT, ORC_KDOT, ORC_LDOT, ORC_MDOT,
  ORC_OMEGA_I, ORC_OMEGA_E, ORC_FLUX_X, ORC_FLUX_Y, ORC_FLUX_Z, ORC_FLUX_K,
  ORC_FLUX_L, ORC_FLUX_M, ORC_LAMBDA_X, ORC_LAMBDA_Y, ORC_LAMBDA_Z, ORC_MEANFL,
  ORC_N6D,                                   /* number of 6D fields (20) */
  ORC_NSQR = 32, ORC_U, ORC_V,               /* padded 3D background */
  ORC_E_INT, ORC_MEANFL_INT, ORC_DISS_KS, ORC_DISS_KE, ORC_DISS_LS,
  ORC_DISS_LE, ORC_DISS_MS, ORC_DISS_ME,     /* padded 3D diagnostics */
  /* padded 1D grids: axis a (0..5 = x,y,z,k,l,m) at ORC_GRID + 4*a + {0:t,1:u,2:dt,3:du} */
  ORC_GRID = 64
};

typedef struct {
  double eint, mflint, mfl_max;              /* diagnose.f90:46-68 */
  double umax, vmax, wmax, kmax, lmax, mmax;
  double bfl_xs, bfl_xe, bfl_ys, bfl_ye, bfl_zs, bfl_ze;   /* diagnose.f90:102-277 */
  double bfl_ks, bfl_ke, bfl_ls, bfl_le, bfl_ms, bfl_me;
  double cfl_x, cfl_y, cfl_z, cfl_k, cfl_l, cfl_m;         /* diagnose.f90:295-313 */
  double residual;                                         /* diagnose.f90:327-328 */
} orc_budget;

orc_state* orc_create(int nx, int ny, int nz, int nk, int nl, int nm);
void orc_destroy(orc_state* s);
double* orc_field(orc_state* s, int id);
long long orc_field_len(orc_state* s, int id);
void orc_set_scalars(orc_state* s, double dt, double f0, double sign_of_omega_i,
                     int enable_upper_reflection, int enable_lower_reflection,
                     double k_fixed, double l_fixed, double m_fixed);

/* calc_grid.f90:4-295 on one rank; reads the interior of the dXt arrays.
 * Returns 0, or 1/2/3 when the z/m/l monotonicity check fails (:260-293). */
int orc_calc_grid(orc_state* s);
/* calc_parameter.f90:2-264 */
void orc_calc_parameter(orc_state* s);
/* integrate.f90:4-271 (+ reflection_condition, parallel_mpi.f90:798-876,
 * and superbee_fluxes.f90:4-174); one forward-Euler step */
void orc_integrate(orc_state* s);
/* nsteps of the main loop body (main.f90:69-70): set_forcing, then integrate */
void orc_integrate_n(orc_state* s, int nsteps);

/* set_forcing of the forced configurations, on the bottom z plane k = 1:
 * FLUX  E += dt*F/dzt(1)                    (lee1.f90:193-212, F = flux_lee)
 * RELAX E -= dt*max(0,zdot)*(E-F)/dzt(1)    (critical_gm1.f90:119-139, F = E_gm)
 * F is a padded 5D array with axes x,y,k,l,m (the reference's allocatable
 * flux_lee / E_gm, onx ghosts on every axis); it is copied.  NONE switches
 * the forcing off.  Returns 0, 1 for a bad argument, 2 when out of memory. */
enum { ORC_FORCING_NONE = 0, ORC_FORCING_FLUX = 1, ORC_FORCING_RELAX = 2 };
int orc_set_forcing(orc_state* s, int kind, const double* F);
/* one application of the forcing (no-op when NONE) */
void orc_apply_forcing(orc_state* s);
/* budget part of diagnose.f90:20-329; fills orc_budget and the 3D fields */
void orc_diagnose(orc_state* s, orc_budget* out);
/* dt helper for the CFL-defined configs: max over interior cells of
 * sum_a max(|v_a(I-1)|,|v_a(I)|)/d_a(I) over axes with n_a>1 */
double orc_max_rate(orc_state* s);
/* OpenMP threads used by the step (1 when built without OpenMP) */
int orc_threads(void);

/* Per-cell restatement for fields too large for the arrays above.
 * orc_create_light allocates grids, background and scalars only (no 6D
 * field; orc_calc_parameter / orc_integrate / orc_diagnose must not be
 * called on it).  orc_point_steps writes to out[q] the state after one step
 * at the interior cell cells[6q..6q+5] (Fortran indices i,j,k,l,n,m), from
 * the interior pre-step state E0 (nx*ny*nz*nk*nl*nm doubles, x fastest),
 * with the expressions and operation order of orc_calc_parameter and
 * orc_integrate: bit-identical to the whole-array oracle. */
orc_state* orc_create_light(int nx, int ny, int nz, int nk, int nl, int nm);
void orc_point_steps(const orc_state* s, const double* E0, const int* cells, long long count, double* out);

#ifdef __cplusplus
}
#endif
#endif
