! adscf_shim.f90 -- drop-in replacements for the compute modules of ADSCF's
! bulk drivers (Bulk_3D_FFT).
!
! Each module below has the name, public types and procedure signatures of
! the reference module it replaces, so the reference's Main_* programs
! compile unchanged against it; the bodies call the GB300 library through
! the `adscf` binding module (adscf.f90) and the shared contexts of
! adscf_shim_state.f90.  Build: list adscf.f90, adscf_shim_state.f90 and this
! file (after mod_global.f90) in place of the replaced source files and link
! -ladscf_gb300.  Film drivers use adscf_shim_film.f90, the brush driver
! adscf_shim_brush.f90.
!
!   replaced file (Bulk_3D_FFT)                      module here
!   General_Routines/mod_propagate.f90               Propagate
!   Polymer_Modules/mod_diblock.f90                  Molecule_Diblock_Copolymer
!   Polymer_Modules/mod_solvent.f90                  Molecule_Solvent
!   General_Routines/mod_iterate.f90 (Mixing_*)      Iterate

! ---------------------------------------------------------------------------
! Propagate (Bulk_3D_FFT/General_Routines/mod_propagate.f90:22-68)
module Propagate
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use Global
  implicit none
contains

  ! expfield = exp(-ds w / 2), on the host as in the reference (:22-32)
  subroutine Calculate_Expfield(field, expfield)
    double precision, dimension(gridx, gridy, gridz, monomer_types), intent(in) :: field
    double precision, dimension(gridx, gridy, gridz, monomer_types), intent(out) :: expfield
    expfield = exp(-0.5d0 * ds * field)
  end subroutine Calculate_Expfield

  ! prop <- E IFFT(exp(-ds k^2) FFT(E prop)) on the GPU (:40-68)
  subroutine Propagate_Step(prop, expfield)
    double precision, dimension(gridx, gridy, gridz), intent(in) :: expfield
    double precision, dimension(gridx, gridy, gridz), intent(inout) :: prop
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    ctx = shim_bulk_context([0.5d0, 0.5d0], [1, 2], 1, 1d0, 0d0)
    rc = adscf_propagate_step(ctx, prop, expfield, 0d0)
    call adscf_check(ctx, rc, 'Propagate_Step')
  end subroutine Propagate_Step

end module Propagate

! ---------------------------------------------------------------------------
! Molecule_Diblock_Copolymer (Bulk_3D_FFT/Polymer_Modules/mod_diblock.f90)
module Molecule_Diblock_Copolymer
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use Global
  implicit none
  private
  integer, parameter :: block_number = 2

  ! same members as the reference's type (mod_diblock.f90:19-33)
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
    double precision, dimension(gridx, gridy, gridz, block_number) :: distribution
    double precision, dimension(gridx, gridy, gridz, block_number) :: density
  end type diblock_copolymer

  public :: diblock_copolymer, Initialize_Diblock, Propagate_Diblock
contains

  ! chain set-up with the reference's semantics (mod_diblock.f90:46-88):
  ! nint(f/ds) segments per block and the flat initial block densities
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
      copolymer%density(:, :, :, b) = rho * copolymer%block_segments(b) * ds * volume / dvol &
                                      / dble(gridx * gridy * gridz)
    end do
  end subroutine Initialize_Diblock

  ! both chains, Q, the block densities and the ensemble closure on the GPU
  ! (mod_diblock.f90:100-173).  The library takes the field w, recovered
  ! here from expfield = exp(-ds w / 2) (relative error ~1e-15).
  subroutine Propagate_Diblock(copolymer, expfield)
    type(diblock_copolymer), intent(inout) :: copolymer
    double precision, dimension(gridx, gridy, gridz, monomer_types), intent(in) :: expfield
    double precision, dimension(gridx, gridy, gridz, monomer_types) :: field, dens
    type(adscf_chain_result) :: res
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    integer :: b
    if (copolymer%monomer_type(1) == copolymer%monomer_type(2)) then
      print *, 'Propagate_Diblock: the blocks must have distinct monomer types'
      stop 1
    end if
    field = -2d0 * log(expfield) / ds
    ctx = shim_bulk_context(copolymer%block_length, copolymer%monomer_type, &
                            copolymer%ensemble, copolymer%rho, copolymer%mu)
    rc = adscf_propagate_diblock(ctx, field, dens, res)
    call adscf_check(ctx, rc, 'Propagate_Diblock')
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

! ---------------------------------------------------------------------------
! Molecule_Solvent (Bulk_3D_FFT/Polymer_Modules/mod_solvent.f90)
module Molecule_Solvent
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use Global
  implicit none
  private

  ! same members as the reference's type (mod_solvent.f90:19-28)
  type monomeric_solvent
    integer :: label
    integer :: monomer_type
    integer :: ensemble
    double precision :: rho
    double precision :: mu
    double precision :: energy
    double precision :: Qsum
    double precision, dimension(gridx, gridy, gridz) :: distribution
    double precision, dimension(gridx, gridy, gridz) :: density
  end type monomeric_solvent

  public :: monomeric_solvent, Initialize_Solvent, Update_Solvent
contains

  ! set-up with the reference's semantics (mod_solvent.f90:41-76)
  subroutine Initialize_Solvent(solvent, label, monomer_type, ensemble, rho, mu)
    integer, intent(in) :: label, ensemble, monomer_type
    double precision, intent(in) :: rho, mu
    type(monomeric_solvent), intent(out) :: solvent
    if (ensemble /= 1 .and. ensemble /= 2) print *, 'Invalid Ensemble'
    solvent%label = label
    solvent%monomer_type = monomer_type
    solvent%ensemble = ensemble
    solvent%rho = rho
    solvent%mu = mu
    solvent%energy = 0d0
    solvent%Qsum = 0d0
    solvent%distribution = 0d0
    solvent%density = solvent%rho * volume / dvol / dble(gridx * gridy * gridz)
  end subroutine Initialize_Solvent

  ! distribution, Qsum, density and energy on the GPU (mod_solvent.f90:85-110)
  subroutine Update_Solvent(solvent, field)
    type(monomeric_solvent), intent(inout) :: solvent
    double precision, dimension(gridx, gridy, gridz), intent(in) :: field
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    ctx = shim_grid_context()
    rc = adscf_update_solvent(ctx, field, int(solvent%ensemble, c_int), solvent%rho, solvent%mu, &
                              solvent%Qsum, solvent%energy, solvent%density, solvent%distribution)
    call adscf_check(ctx, rc, 'Update_Solvent')
  end subroutine Update_Solvent

end module Molecule_Solvent

! ---------------------------------------------------------------------------
! Iterate (Bulk_3D_FFT/General_Routines/mod_iterate.f90:13,27-150): the
! mixing history lives on the GPU, so only column 0 of field/dfield is read
! (x_k, r_k) and column 0 of field receives x_{k+1}.
module Iterate
  use iso_c_binding
  use adscf
  use adscf_shim_state
  use Global
  implicit none
  integer, parameter :: mixing_dim = 2
contains

  subroutine mix_on_device(mixing_type, field, dfield, fieldsize, lambda, iter)
    integer, intent(in) :: mixing_type, fieldsize, iter
    double precision, intent(in) :: lambda
    double precision, dimension(fieldsize, 0:mixing_dim), intent(inout) :: field, dfield
    double precision, dimension(fieldsize) :: x
    type(c_ptr) :: ctx
    integer(c_int) :: rc
    if (fieldsize /= 2 * gridx * gridy * gridz) then
      print *, 'Mixing: fieldsize must be 2*gridx*gridy*gridz'
      stop 1
    end if
    ctx = shim_mix_context(mixing_type, lambda)
    x = field(:, 0)
    rc = adscf_mix(ctx, x, dfield(:, 0), iter)
    call adscf_check(ctx, rc, 'Mixing')
    field(:, 0) = x
  end subroutine mix_on_device

  subroutine Mixing_Simple(field, dfield, fieldsize, lambda, iter)
    double precision, intent(in) :: lambda
    integer, intent(in) :: fieldsize, iter
    double precision, dimension(fieldsize, 0:mixing_dim), intent(inout) :: field, dfield
    call mix_on_device(ADSCF_MIX_SIMPLE, field, dfield, fieldsize, lambda, iter)
  end subroutine Mixing_Simple

  subroutine Mixing_Lambda(field, dfield, fieldsize, lambda, iter)
    double precision, intent(in) :: lambda
    integer, intent(in) :: fieldsize, iter
    double precision, dimension(fieldsize, 0:mixing_dim), intent(inout) :: field, dfield
    call mix_on_device(ADSCF_MIX_LAMBDA, field, dfield, fieldsize, lambda, iter)
  end subroutine Mixing_Lambda

  subroutine Mixing_Anderson(field, dfield, fieldsize, lam_mix, iter)
    double precision, intent(in) :: lam_mix
    integer, intent(in) :: fieldsize, iter
    double precision, dimension(fieldsize, 0:mixing_dim), intent(inout) :: field, dfield
    call mix_on_device(ADSCF_MIX_ANDERSON, field, dfield, fieldsize, lam_mix, iter)
  end subroutine Mixing_Anderson

end module Iterate


