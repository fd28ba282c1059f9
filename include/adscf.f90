! adscf.f90 -- iso_c_binding interface of include/adscf.h for ADSCF's
! Fortran 90 drivers.
!
! One module, `adscf`, declares the bind(C) mirror of the ABI structs and
! the interfaces of the entry points a Fortran driver calls.  The shim
! modules in adscf_shim.f90 build on it to keep the reference's own module
! and procedure names.  The derived types must keep the member order of the
! C structs (checked against the header by tests/test_capi_abi.py).
!
! Array arguments are passed as the reference passes them: a Fortran
! (gridx,gridy,gridz,monomer_types) array is the C [species][z][y][x] array.
module adscf
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: ADSCF_OK = 0, ADSCF_E_ARG = 1, ADSCF_E_CUDA = 2, &
       ADSCF_E_PIVOT = 3, ADSCF_E_NONFINITE = 4, ADSCF_E_TIMEOUT = 5, ADSCF_E_OOM = 6, &
       ADSCF_E_STATE = 7, ADSCF_E_TOO_LARGE = 8
  integer(c_int), parameter :: ADSCF_BULK = 0, ADSCF_FILM_1D = 1, ADSCF_FILM_3D = 2, &
       ADSCF_BRUSH = 3
  integer(c_int), parameter :: ADSCF_FP64 = 0, ADSCF_SPLIT = 1
  integer(c_int), parameter :: ADSCF_MIX_SIMPLE = 1, ADSCF_MIX_LAMBDA = 2, &
       ADSCF_MIX_ANDERSON = 3

  ! layout of adscf_params (include/adscf.h), member for member
  type, bind(C) :: adscf_params
     integer(c_int)  :: geometry
     integer(c_int)  :: gx, gy, gz
     real(c_double)  :: sizex, sizey, sizez
     real(c_double)  :: ds
     type(c_ptr)     :: dss
     integer(c_int)  :: ns
     integer(c_int)  :: n_a
     real(c_double)  :: block_length(2)
     integer(c_int)  :: ensemble
     real(c_double)  :: rho, mu
     real(c_double)  :: kappa, chi
     real(c_double)  :: monomer_volume(2)
     integer(c_int)  :: precision
     integer(c_int)  :: mixing_type
     integer(c_int)  :: mixing_dim
     real(c_double)  :: lambda
     real(c_double)  :: lam_warm
     integer(c_int)  :: warm_iters
     type(c_ptr)     :: dz
     integer(c_int)  :: int_scheme
     integer(c_int)  :: int_span
     type(c_ptr)     :: ext_potential
     real(c_double)  :: ww
     type(c_ptr)     :: graft
     integer(c_int)  :: nblocks
     type(c_ptr)     :: blocks
     type(c_ptr)     :: block_types
  end type adscf_params

  type, bind(C) :: adscf_chain_result
     real(c_double) :: Qsum, logQ, mu, rho, energy
  end type adscf_chain_result

  type, bind(C) :: adscf_iter_result
     real(c_double) :: accuracy, free_energy, Qsum, logQ, mu, rho, lambda
     integer(c_int) :: iter, status
  end type adscf_iter_result

  interface
     integer(c_int) function adscf_ctx_create(p, ctx) bind(C, name="adscf_ctx_create")
       import :: c_int, c_ptr, adscf_params
       type(adscf_params), intent(in) :: p
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function adscf_ctx_destroy(ctx) bind(C, name="adscf_ctx_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     type(c_ptr) function adscf_last_error(ctx) bind(C, name="adscf_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function adscf_propagate_diblock(ctx, field, density, res) &
          bind(C, name="adscf_propagate_diblock")
       import :: c_int, c_ptr, c_double, adscf_chain_result
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: field(*)
       real(c_double), intent(out) :: density(*)
       type(adscf_chain_result), intent(out) :: res
     end function
     integer(c_int) function adscf_propagate_homopolymer(ctx, field, density, res) &
          bind(C, name="adscf_propagate_homopolymer")
       import :: c_int, c_ptr, c_double, adscf_chain_result
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: field(*)
       real(c_double), intent(out) :: density(*)
       type(adscf_chain_result), intent(out) :: res
     end function
     integer(c_int) function adscf_propagate_step(ctx, prop, aux, ds) &
          bind(C, name="adscf_propagate_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: prop(*)
       real(c_double), intent(in) :: aux(*)
       real(c_double), value :: ds
     end function
     integer(c_int) function adscf_integrator(ctx, integrand, integral) &
          bind(C, name="adscf_integrator")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: integrand(*)
       real(c_double), intent(out) :: integral
     end function
     integer(c_int) function adscf_mean_fields(ctx, density, field) &
          bind(C, name="adscf_mean_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: density(*)
       real(c_double), intent(out) :: field(*)
     end function
     integer(c_int) function adscf_update_solvent(ctx, field, ensemble, rho, mu, qsum, energy, &
          density, distribution) bind(C, name="adscf_update_solvent")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: field(*)
       integer(c_int), value :: ensemble
       real(c_double), intent(inout) :: rho, mu
       real(c_double), intent(out) :: qsum, energy
       real(c_double), intent(out) :: density(*), distribution(*)
     end function
     integer(c_int) function adscf_mix(ctx, field, dfield, iter) bind(C, name="adscf_mix")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: field(*)
       real(c_double), intent(in) :: dfield(*)
       integer(c_int), value :: iter
     end function
     integer(c_int) function adscf_mix_reset(ctx) bind(C, name="adscf_mix_reset")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function adscf_set_field(ctx, field) bind(C, name="adscf_set_field")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: field(*)
     end function
     integer(c_int) function adscf_scf_iteration(ctx, field, density, res) &
          bind(C, name="adscf_scf_iteration")
       import :: c_int, c_ptr, c_double, adscf_iter_result
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: field(*)
       real(c_double), intent(out) :: density(*)
       type(adscf_iter_result), intent(out) :: res
     end function
     integer(c_int) function adscf_scf_run(ctx, n_iter, tol, res) bind(C, name="adscf_scf_run")
       import :: c_int, c_ptr, c_double, adscf_iter_result
       type(c_ptr), value :: ctx
       integer(c_int), value :: n_iter
       real(c_double), value :: tol
       type(adscf_iter_result), intent(out) :: res
     end function
     integer(c_int) function adscf_forward(ctx, field, free_energy) bind(C, name="adscf_forward")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: field(*)
       real(c_double), intent(out) :: free_energy
     end function
     integer(c_int) function adscf_backward(ctx, grad) bind(C, name="adscf_backward")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: grad(4)
     end function
     integer(c_int) function adscf_propagate_step_noalloc(gx, gy, gz, lx, ly, lz, ds, &
          d_prop, d_expfield, stream) bind(C, name="adscf_propagate_step_noalloc")
       import :: c_int, c_ptr, c_double
       integer(c_int), value :: gx, gy, gz
       real(c_double), value :: lx, ly, lz, ds
       type(c_ptr), value :: d_prop, d_expfield, stream
     end function
  end interface

contains

  ! adscf_last_error as a Fortran string (for the drivers' error prints)
  function adscf_error_text(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=256) :: msg
    character(kind=c_char), pointer :: chars(:)
    type(c_ptr) :: p
    integer :: i
    msg = ' '
    p = adscf_last_error(ctx)
    if (.not. c_associated(p)) return
    call c_f_pointer(p, chars, [256])
    do i = 1, 256
      if (chars(i) == c_null_char) exit
      msg(i:i) = chars(i)
    end do
  end function adscf_error_text

  ! stop the driver with the library's message on a non-zero status, the
  ! way the reference's routines print and stop
  subroutine adscf_check(ctx, rc, where)
    type(c_ptr), intent(in) :: ctx
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: where
    if (rc /= ADSCF_OK) then
      print *, 'adscf error ', rc, ' in ', where, ': ', trim(adscf_error_text(ctx))
      stop 1
    end if
  end subroutine adscf_check

end module adscf
