! adscf_shim_brush.f90 -- drop-in line step and integrator for ADSCF's
! polymer-brush driver (Brush_CK_AD).
!
! Module RealSpace_adscf keeps the signatures of the brush's
! Propagate_Step(prop, field, ds) (Brush_CK_AD/Geometry_Modules/
! mod_realspace.f90:26-79: one Crank-Nicolson step with the caller's step
! size) and integrator(integrand, integral) (Brush_CK_AD/Adaptive_Modules/
! mod_adaptive.f90:124-143); the bodies call the GB300 library through
! `adscf` (adscf.f90) and the shared contexts of adscf_shim_state.f90.
! Build: list adscf.f90, adscf_shim_state.f90 and this file after
! mod_global.f90, and have Molecule_Homopolymer (mod_homopolymer.f90) use
! RealSpace_adscf for these two procedures; the adaptive mesh and contour
! set-up (generate_mesh, Initialize_Homopolymer) stay Fortran.  A whole
! Propagate_Homopolymer in one call is adscf_propagate_homopolymer on an
! ADSCF_BRUSH context (adscf.h).

module RealSpace_adscf
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use Global
  implicit none
  private
  public :: Propagate_Step, integrator
contains

  subroutine Propagate_Step(prop, field, ds_step)
    double precision, dimension(gridx, gridy, 0:gridz), intent(inout) :: prop
    double precision, dimension(gridx, gridy, 0:gridz), intent(in) :: field
    double precision, intent(in) :: ds_step
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    ctx = shim_film_context(ADSCF_FILM_1D, 1, dz, int_scheme)
    rc = adscf_propagate_step(ctx, prop, field, ds_step)
    call adscf_check(ctx, rc, 'Propagate_Step (brush)')
  end subroutine Propagate_Step

  subroutine integrator(integrand, integral)
    double precision, dimension(gridx, gridy, 0:gridz), intent(in) :: integrand
    double precision, intent(out) :: integral
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    ctx = shim_film_context(ADSCF_FILM_1D, 1, dz, int_scheme)
    rc = adscf_integrator(ctx, integrand, integral)
    call adscf_check(ctx, rc, 'integrator (brush)')
  end subroutine integrator

end module RealSpace_adscf
