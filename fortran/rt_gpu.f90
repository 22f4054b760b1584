! rt_gpu.f90 -- ISO_C_BINDING interface of libraytracer_gb300.so (the GB300
! time-stepping path) for the Fortran driver of raytracer_3D.
!
! Each interface mirrors one declaration of include/rt_gb300.h.  Handles are
! type(c_ptr); 6D / 3D / 1D arrays are passed as the reference's padded,
! column-major module arrays (onx = 2 ghost cells per side), so the actual
! arguments are the module arrays themselves (E, dE, meanfl, Nsqr, U, V,
! dxt..dmt, kt, lt, mt of main_module).  Strings are C strings: append
! c_null_char.  Every function returns 0 or a negative RT_ERR_* code;
! rt_check turns a nonzero code into halt_stop, the reference's fatal-error
! path (parallel_mpi.f90:223-236).
!
! Compile with the driver (for_config/Makefile:9-16), e.g.
!   mpif90 -c rt_gpu.f90 && mpif90 ... rt_gpu.o -L$REPO/raytracer_3d_gb300 \
!       -lraytracer_gb300 -Wl,-rpath,$REPO/raytracer_3d_gb300
module rt_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: RT_FP64 = 0, RT_FP32 = 1
  integer(c_int), parameter :: RT_FORCING_NONE = 0, RT_FORCING_FLUX = 1, RT_FORCING_RELAX = 2
  ! rt_set_tuning variants (the binary64 ones; all give results within the
  ! plain form's bound, tma and split bit-identical to the reference)
  integer(c_int), parameter :: RT_VARIANT_TMA = 2, RT_VARIANT_SPLIT = 15, RT_VARIANT_FAST = 16

  type, bind(C) :: rt_dims
     integer(c_int) :: nx, ny, nz, nk, nl, nm, onx
  end type rt_dims

  type, bind(C) :: rt_params
     real(c_double) :: dt, f0, sign_of_omega_i
     integer(c_int) :: enable_upper_reflection, enable_lower_reflection, precision
  end type rt_params

  type, bind(C) :: rt_budget
     real(c_double) :: eint, mflint, mfl_max, umax, vmax, wmax, kmax, lmax, mmax
     real(c_double) :: bfl_xs, bfl_xe, bfl_ys, bfl_ye, bfl_zs, bfl_ze
     real(c_double) :: bfl_ks, bfl_ke, bfl_ls, bfl_le, bfl_ms, bfl_me
     real(c_double) :: cfl_x, cfl_y, cfl_z, cfl_k, cfl_l, cfl_m, residual
  end type rt_budget

  ! the driver's one handle (allocate_main_module's device side)
  type(c_ptr), save :: rt_h = c_null_ptr

  interface
    integer(c_int) function rt_create(d, p, h) bind(C, name="rt_create")
      import :: c_int, c_ptr, rt_dims, rt_params
      type(rt_dims), intent(in) :: d
      type(rt_params), intent(in) :: p
      type(c_ptr), intent(out) :: h
    end function rt_create

    integer(c_int) function rt_destroy(h) bind(C, name="rt_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function rt_destroy

    type(c_ptr) function rt_last_error(h) bind(C, name="rt_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function rt_last_error

    integer(c_int) function rt_set_grid(h, dxt, dyt, dzt, dkt, dlt, dmt, kt, lt, mt) bind(C, name="rt_set_grid")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: dxt(*), dyt(*), dzt(*), dkt(*), dlt(*), dmt(*), kt(*), lt(*), mt(*)
    end function rt_set_grid

    integer(c_int) function rt_set_background(h, Nsqr, U, V) bind(C, name="rt_set_background")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: Nsqr(*), U(*), V(*)
    end function rt_set_background

    integer(c_int) function rt_calc_parameter(h) bind(C, name="rt_calc_parameter")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function rt_calc_parameter

    integer(c_int) function rt_max_rate(h, rate) bind(C, name="rt_max_rate")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: rate
    end function rt_max_rate

    integer(c_int) function rt_set_dt(h, dt) bind(C, name="rt_set_dt")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), value :: dt
    end function rt_set_dt

    integer(c_int) function rt_set_state(h, E) bind(C, name="rt_set_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: E(*)
    end function rt_set_state

    integer(c_int) function rt_get_state(h, E) bind(C, name="rt_get_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(inout) :: E(*)
    end function rt_get_state

    integer(c_int) function rt_set_forcing(h, kind, F) bind(C, name="rt_set_forcing")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: kind
      real(c_double), intent(in) :: F(*)
    end function rt_set_forcing

    integer(c_int) function rt_integrate(h, nsteps) bind(C, name="rt_integrate")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function rt_integrate

    integer(c_int) function rt_integrate_host(h, E) bind(C, name="rt_integrate_host")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(inout) :: E(*)
    end function rt_integrate_host

    integer(c_int) function rt_set_host_access(h, direct) bind(C, name="rt_set_host_access")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: direct
    end function rt_set_host_access

    integer(c_int) function rt_diagnose(h, b, E_int, meanfl_int, diss_ks, diss_ke, diss_ls, diss_le, &
                                        diss_ms, diss_me) bind(C, name="rt_diagnose")
      import :: c_int, c_ptr, c_double, rt_budget
      type(c_ptr), value :: h
      type(rt_budget), intent(out) :: b
      real(c_double), intent(inout) :: E_int(*), meanfl_int(*), diss_ks(*), diss_ke(*), diss_ls(*), &
                                       diss_le(*), diss_ms(*), diss_me(*)
    end function rt_diagnose

    integer(c_int) function rt_get_tendency(h, dE, meanfl) bind(C, name="rt_get_tendency")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(inout) :: dE(*), meanfl(*)
    end function rt_get_tendency

    integer(c_int) function rt_set_tuning(h, variant, band, threads) bind(C, name="rt_set_tuning")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: variant, band, threads
    end function rt_set_tuning

    integer(c_int) function rt_sync(h) bind(C, name="rt_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function rt_sync

    integer(c_int) function rt_tic(h, name) bind(C, name="rt_tic")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: name(*)
    end function rt_tic

    integer(c_int) function rt_toc(h, name) bind(C, name="rt_toc")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: name(*)
    end function rt_toc

    integer(c_int) function rt_timing_secs(h, name, secs, calls) bind(C, name="rt_timing_secs")
      import :: c_int, c_ptr, c_char, c_double, c_long_long
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: name(*)
      real(c_double), intent(out) :: secs
      integer(c_long_long), intent(out) :: calls
    end function rt_timing_secs

    integer(c_int) function rt_selftest_wait_timeout(status, completed) bind(C, name="rt_selftest_wait_timeout")
      import :: c_int
      integer(c_int), intent(out) :: status, completed
    end function rt_selftest_wait_timeout
  end interface

contains

  ! nonzero return code of a library call: the reference's fatal-error path
  subroutine rt_check(rc)
    integer(c_int), intent(in) :: rc
    if (rc /= 0) call halt_stop(' GPU call failed (rt_last_error(rt_h) has the reason)')
  end subroutine rt_check

end module rt_gpu
