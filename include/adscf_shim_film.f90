! adscf_shim_film.f90 -- drop-in replacements for the compute modules of
! ADSCF's film drivers (Film_CK_AD/Film_1D and Film_CK_AD/Film_3D).
!
! The modules keep the names, public types and procedure signatures of the
! reference modules they replace; the bodies call the GB300 library through
! `adscf` (adscf.f90) and the shared contexts of adscf_shim_state.f90.
! Build: list adscf.f90, adscf_shim_state.f90 and this file (after
! mod_global.f90) in place of the replaced source files and link
! -ladscf_gb300.  A driver whose Global grid is one line (gridx = gridy = 1)
! runs the Film_1D Crank-Nicolson step and the Film_1D integrator (interior
! intervals); any other grid runs the Film_3D Douglas ADI step and the
! Film_3D integrator, as the two reference trees do.
!
!   replaced file (Film_CK_AD/Film_*)                  module here
!   Polymer_Modules/mod_diblock.f90                    Molecule_Diblock_Copolymer
!   Geometry_Modules/mod_realspace.f90                 RealSpace_adscf, used beside
!     (Propagate_Step, integrator)                     RealSpace, whose generate_mesh and
!                                                      calculate_Volume stay
! The drivers' mixing (Iterate) stays Fortran: film fields pack only the
! interior planes, which the bulk mixing shim does not.

! ---------------------------------------------------------------------------
! RealSpace_adscf (Film_CK_AD/Film_3D/Geometry_Modules/mod_realspace.f90:
! 22-140,267-281; Film_CK_AD/Film_1D/Geometry_Modules/mod_realspace.f90:
! 24-79 and its integrator)
module RealSpace_adscf
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use Global
  implicit none
  private
  public :: Propagate_Step, integrator, film_geometry, film_span
contains

  ! the reference tree this driver's grid belongs to
  integer function film_geometry()
    if (gridx * gridy == 1) then
      film_geometry = ADSCF_FILM_1D
    else
      film_geometry = ADSCF_FILM_3D
    end if
  end function film_geometry

  ! integrator span: 1 (interior intervals, Film_1D), 0 (all planes, Film_3D)
  integer function film_span()
    if (gridx * gridy == 1) then
      film_span = 1
    else
      film_span = 0
    end if
  end function film_span

  subroutine Propagate_Step(prop, field)
    double precision, dimension(gridx, gridy, 0:gridz), intent(inout) :: prop
    double precision, dimension(gridx, gridy, 0:gridz), intent(in) :: field
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    ctx = shim_film_context(film_geometry(), film_span(), dz, int_scheme)
    rc = adscf_propagate_step(ctx, prop, field, ds)
    call adscf_check(ctx, rc, 'Propagate_Step (film)')
  end subroutine Propagate_Step

  subroutine integrator(integrand, integral)
    double precision, dimension(gridx, gridy, 0:gridz), intent(in) :: integrand
    double precision, intent(out) :: integral
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    ctx = shim_film_context(film_geometry(), film_span(), dz, int_scheme)
    rc = adscf_integrator(ctx, integrand, integral)
    call adscf_check(ctx, rc, 'integrator')
  end subroutine integrator

end module RealSpace_adscf

! ---------------------------------------------------------------------------
! Molecule_Diblock_Copolymer (Film_CK_AD/Film_1D/Polymer_Modules/
! mod_diblock.f90:19-195; the Film_3D module has the same members and steps)
module Molecule_Diblock_Copolymer
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use RealSpace_adscf, only: film_geometry, film_span
  use Global
  implicit none
  private
  integer, parameter :: block_number = 2

  ! same members as the reference's type (Film_1D mod_diblock.f90:19-32)
  type diblock_copolymer
    integer :: label
    integer, dimension(block_number) :: monomer_type
    double precision, dimension(block_number) :: block_length
    integer :: ensemble
    double precision :: rho
    double precision :: mu
    double precision :: energy
    integer, dimension(block_number) :: block_segments
    integer :: segments
    double precision :: Qsum
    double precision, dimension(gridx, gridy, 0:gridz, block_number) :: distribution
    double precision, dimension(gridx, gridy, 0:gridz, block_number) :: density
  end type diblock_copolymer

  public :: diblock_copolymer, Initialize_Diblock, Propagate_Diblock
contains

  ! chain set-up with the reference's semantics (Film_1D mod_diblock.f90:
  ! 46-88): nint(f/ds) segments per block, flat initial block densities
  ! rho * segments * ds
  subroutine Initialize_Diblock(copolymer, label, monomer_type, block_length, ensemble, rho, mu)
    integer, intent(in) :: label, ensemble
    double precision, intent(in) :: rho, mu
    double precision, dimension(block_number), intent(in) :: block_length
    integer, dimension(block_number), intent(in) :: monomer_type
    type(diblock_copolymer), intent(out) :: copolymer
    integer :: b
    if (ensemble /= 1 .and. ensemble /= 2) print *, 'Invalid Ensemble'
    copolymer%label = label
    copolymer%monomer_type = monomer_type
    copolymer%block_length = block_length
    copolymer%ensemble = ensemble
    copolymer%rho = rho
    copolymer%mu = mu
    copolymer%block_segments = nint(block_length / ds)
    copolymer%segments = sum(copolymer%block_segments)
    copolymer%energy = 0d0
    copolymer%Qsum = 0d0
    copolymer%distribution = 0d0
    do b = 1, block_number
      copolymer%density(:, :, :, b) = rho * copolymer%block_segments(b) * ds
    end do
  end subroutine Initialize_Diblock

  ! both chains, Q (the geometry's integrator), the block densities and the
  ! ensemble closure on the GPU (Film_1D mod_diblock.f90:110-195)
  subroutine Propagate_Diblock(copolymer, field)
    type(diblock_copolymer), intent(inout) :: copolymer
    double precision, dimension(gridx, gridy, 0:gridz, monomer_types), intent(in) :: field
    double precision, dimension(gridx, gridy, 0:gridz, monomer_types) :: dens
    type(adscf_chain_result) :: res
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    integer :: b
    if (copolymer%monomer_type(1) == copolymer%monomer_type(2)) then
      print *, 'Propagate_Diblock: the blocks must have distinct monomer types'
      stop 1
    end if
    ctx = shim_film_chain_context(film_geometry(), film_span(), dz, int_scheme, &
                                  copolymer%block_length, copolymer%monomer_type, &
                                  copolymer%ensemble, copolymer%rho, copolymer%mu)
    rc = adscf_propagate_diblock(ctx, field, dens, res)
    call adscf_check(ctx, rc, 'Propagate_Diblock (film)')
    do b = 1, block_number
      copolymer%density(:, :, :, b) = dens(:, :, :, copolymer%monomer_type(b))
    end do
    copolymer%Qsum = res%Qsum
    copolymer%mu = res%mu
    copolymer%rho = res%rho
    copolymer%energy = res%energy
    if (copolymer%ensemble == 1) then
      copolymer%distribution = copolymer%density * copolymer%Qsum / (copolymer%rho * volume)
    else
      copolymer%distribution = copolymer%density * exp(-copolymer%mu)
    end if
  end subroutine Propagate_Diblock

end module Molecule_Diblock_Copolymer
