! rt_gpu_driver.f90 -- the bodies that replace the reference's calc_parameter
! (for_src/calc_parameter.f90:2-264, called at main.f90:47) and integrate
! (for_src/integrate.f90:4-271, called at main.f90:70), and the budget part
! of diagnose (diagnose.f90:46-329, main.f90:74), on libraytracer_gb300.so
! through the rt_gpu module.  Built in place of calc_parameter.f90 and
! integrate.f90; the driver's grids, configs, NetCDF output and restart
! code stay as they are.
!
! The device keeps the state between steps: E crosses to the host only in
! gpu_fetch_state (before diagnose's output, write_restart or the end of the
! run) and gpu_push_state (after read_restart).

subroutine calc_parameter
  use main_module
  use rt_gpu
  implicit none
  type(rt_dims) :: d
  type(rt_params) :: p
  integer :: up, lo
  up = 0
  lo = 0
  if (enable_upper_reflection) up = 1
  if (enable_lower_reflection) lo = 1
  d = rt_dims(nx, ny, nz, nk, nl, nm, onx)
  p = rt_params(dt, f0, sign_of_omega_i, up, lo, RT_FP64)
  if (c_associated(rt_h)) call rt_check(rt_destroy(rt_h))
  call rt_check(rt_create(d, p, rt_h))
  call rt_check(rt_set_grid(rt_h, dxt, dyt, dzt, dkt, dlt, dmt, kt, lt, mt))
  call rt_check(rt_set_background(rt_h, Nsqr, U, V))
  call rt_check(rt_calc_parameter(rt_h))
  ! the two-pass step: every face flux once, the reference's arithmetic bit
  ! for bit; RT_VARIANT_FAST trades bit identity for speed (within 1e-12
  ! relative per step)
  call rt_check(rt_set_tuning(rt_h, RT_VARIANT_SPLIT, 8, 256))
  call rt_check(rt_set_state(rt_h, E))
end subroutine calc_parameter

subroutine integrate
  use main_module
  use rt_gpu
  implicit none
  call rt_check(rt_integrate(rt_h, 1))
end subroutine integrate

! the budget of the last step: called at the top of diagnose
! (diagnose.f90:20) with its local 3D arrays (diagnose.f90:29-31), it fills
! them and the scalars of b, and brings E back for the output; the prints
! and NetCDF writes of diagnose follow unchanged, reading eint = b%eint,
! mflint = b%mflint, bfl_xs = b%bfl_xs, ...
subroutine gpu_budget(b, E_int, meanfl_int, diss_ks, diss_ke, diss_ls, diss_le, diss_ms, diss_me)
  use main_module
  use rt_gpu
  implicit none
  type(rt_budget), intent(out) :: b
  real*8 :: E_int(*), meanfl_int(*), diss_ks(*), diss_ke(*), diss_ls(*), diss_le(*), diss_ms(*), diss_me(*)
  call rt_check(rt_diagnose(rt_h, b, E_int, meanfl_int, diss_ks, diss_ke, diss_ls, diss_le, diss_ms, diss_me))
  call rt_check(rt_get_state(rt_h, E))
end subroutine gpu_budget

subroutine gpu_fetch_state
  use main_module
  use rt_gpu
  implicit none
  call rt_check(rt_get_state(rt_h, E))
  call rt_check(rt_get_tendency(rt_h, dE, meanfl))
end subroutine gpu_fetch_state

subroutine gpu_push_state
  use main_module
  use rt_gpu
  implicit none
  call rt_check(rt_set_state(rt_h, E))
end subroutine gpu_push_state
