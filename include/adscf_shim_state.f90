! adscf_shim_state.f90 -- library contexts shared by the drop-in modules of
! adscf_shim.f90 (bulk), adscf_shim_film.f90 (Film_1D, Film_3D) and
! adscf_shim_brush.f90 (brush).  It uses only the Global members every
! driver family declares (gridx, gridy, gridz, sizex, sizey, sizez, ds), so
! it compiles against any of their mod_global.f90.  One context per use,
! created on first use and made again when its parameters change; a non-zero
! library status prints the library's message and stops, as the reference's
! routines do on their own errors.
module adscf_shim_state
  use iso_c_binding
  use adscf
  use Global
  implicit none
  private
  type(c_ptr), save :: bulk_ctx = c_null_ptr    ! propagation (Propagate, Molecule_*)
  type(c_ptr), save :: mix_ctx = c_null_ptr     ! mixing (Iterate)
  type(c_ptr), save :: film_ctx = c_null_ptr    ! film / brush-line steps and integrator
  type(c_ptr), save :: chain_ctx = c_null_ptr   ! film chains (film Molecule_Diblock_Copolymer)
  type(c_ptr), save :: grid_ctx = c_null_ptr    ! grid-only routines (Molecule_Solvent)
  ! the chain the bulk context was created for
  real(c_double), save :: cur_len(2) = -1d0, cur_rho = -1d0, cur_mu = 0d0
  integer(c_int), save :: cur_types(2) = -1, cur_ens = -1
  integer, save :: cur_mix = -1
  real(c_double), save :: cur_lam = -1d0
  public :: shim_bulk_context, shim_mix_context, shim_film_context, shim_film_chain_context
  public :: shim_grid_context
contains

  subroutine base_params(p)
    type(adscf_params), intent(out) :: p
    p%geometry = ADSCF_BULK
    p%gx = gridx; p%gy = gridy; p%gz = gridz
    p%sizex = sizex; p%sizey = sizey; p%sizez = sizez
    p%ds = ds
    p%dss = c_null_ptr; p%ns = 0; p%n_a = 0
    p%block_length = [0.5d0, 0.5d0]
    p%ensemble = 1
    p%rho = 1d0; p%mu = 0d0
    p%kappa = 0d0; p%chi = 0d0
    p%monomer_volume = [1d0, 1d0]
    p%precision = ADSCF_FP64
    p%mixing_type = ADSCF_MIX_LAMBDA
    p%mixing_dim = 2
    p%lambda = 0.1d0
    p%lam_warm = 1d-3
    p%warm_iters = 2
    p%dz = c_null_ptr
    p%int_scheme = 1; p%int_span = 0
    p%ext_potential = c_null_ptr
    p%ww = 0d0
    p%graft = c_null_ptr
    p%nblocks = 0
    p%blocks = c_null_ptr
    p%block_types = c_null_ptr
  end subroutine base_params

  ! bulk context for a two-block chain of the given block lengths, monomer
  ! types (1-based, as the reference's monomer_type) and ensemble; made
  ! again when the chain changes
  function shim_bulk_context(block_length, monomer_type, ensemble, rho, mu) result(ctx)
    real(c_double), intent(in) :: block_length(2), rho, mu
    integer, intent(in) :: monomer_type(2), ensemble
    type(c_ptr) :: ctx
    type(adscf_params) :: p
    real(c_double), target, save :: blocks(2)
    integer(c_int), target, save :: types(2)
    integer(c_int) :: rc
    if (c_associated(bulk_ctx)) then
      if (all(cur_len == block_length) .and. all(cur_types == monomer_type) .and. &
          cur_ens == ensemble .and. cur_rho == rho .and. cur_mu == mu) then
        ctx = bulk_ctx
        return
      end if
      rc = adscf_ctx_destroy(bulk_ctx)
      bulk_ctx = c_null_ptr
    end if
    call base_params(p)
    blocks = block_length
    types = monomer_type - 1
    p%nblocks = 2
    p%blocks = c_loc(blocks)
    p%block_types = c_loc(types)
    p%block_length = block_length
    p%ensemble = ensemble
    p%rho = rho; p%mu = mu
    rc = adscf_ctx_create(p, bulk_ctx)
    call adscf_check(bulk_ctx, rc, 'adscf_ctx_create (bulk)')
    cur_len = block_length; cur_types = monomer_type
    cur_ens = ensemble; cur_rho = rho; cur_mu = mu
    ctx = bulk_ctx
  end function shim_bulk_context

  ! bulk context of the Global grid and box, for routines that use only them
  function shim_grid_context() result(ctx)
    type(c_ptr) :: ctx
    type(adscf_params) :: p
    integer(c_int) :: rc
    if (.not. c_associated(grid_ctx)) then
      call base_params(p)
      rc = adscf_ctx_create(p, grid_ctx)
      call adscf_check(grid_ctx, rc, 'adscf_ctx_create (grid)')
    end if
    ctx = grid_ctx
  end function shim_grid_context

  ! bulk context that holds the mixing history of one mixing scheme
  function shim_mix_context(mixing_type, lambda) result(ctx)
    integer, intent(in) :: mixing_type
    real(c_double), intent(in) :: lambda
    type(c_ptr) :: ctx
    type(adscf_params) :: p
    integer(c_int) :: rc
    if (c_associated(mix_ctx)) then
      if (cur_mix == mixing_type .and. cur_lam == lambda) then
        ctx = mix_ctx
        return
      end if
      rc = adscf_ctx_destroy(mix_ctx)
      mix_ctx = c_null_ptr
    end if
    call base_params(p)
    p%ds = 0.5d0            ! two contour steps: the context only mixes
    p%mixing_type = mixing_type
    p%lambda = lambda
    rc = adscf_ctx_create(p, mix_ctx)
    call adscf_check(mix_ctx, rc, 'adscf_ctx_create (mixing)')
    cur_mix = mixing_type; cur_lam = lambda
    ctx = mix_ctx
  end function shim_mix_context

  ! film or brush-line context (geometry ADSCF_FILM_3D or ADSCF_FILM_1D, the
  ! integrator span of that geometry) on the mesh zmesh(0:gridz), for steps
  ! and integrals; made again when the geometry or the mesh changes
  function shim_film_context(geometry, span, zmesh, scheme) result(ctx)
    integer, intent(in) :: geometry, span, scheme
    real(c_double), intent(in) :: zmesh(0:)
    type(c_ptr) :: ctx
    type(adscf_params) :: p
    real(c_double), allocatable, target, save :: dzc(:)
    integer, save :: cur_geom = -1, cur_span = -1, cur_scheme = -1
    integer(c_int) :: rc
    if (c_associated(film_ctx)) then
      if (cur_geom == geometry .and. cur_span == span .and. cur_scheme == scheme .and. &
          all(dzc == zmesh)) then
        ctx = film_ctx
        return
      end if
      rc = adscf_ctx_destroy(film_ctx)
      film_ctx = c_null_ptr
      deallocate(dzc)
    end if
    call base_params(p)
    allocate(dzc(0:size(zmesh) - 1))
    dzc = zmesh
    p%geometry = geometry
    p%dz = c_loc(dzc)
    p%int_scheme = scheme
    p%int_span = span
    rc = adscf_ctx_create(p, film_ctx)
    call adscf_check(film_ctx, rc, 'adscf_ctx_create (film)')
    cur_geom = geometry; cur_span = span; cur_scheme = scheme
    ctx = film_ctx
  end function shim_film_context

  ! film context for a two-block chain (block lengths, 1-based monomer types,
  ! ensemble, rho, mu) on the mesh zmesh(0:gridz); the chain is passed A block
  ! first (a B-A chain is the same molecule read backwards)
  function shim_film_chain_context(geometry, span, zmesh, scheme, block_length, monomer_type, &
                                   ensemble, rho, mu) result(ctx)
    integer, intent(in) :: geometry, span, scheme, monomer_type(2), ensemble
    real(c_double), intent(in) :: zmesh(0:), block_length(2), rho, mu
    type(c_ptr) :: ctx
    type(adscf_params) :: p
    real(c_double), allocatable, target, save :: dzc(:)
    real(c_double), save :: c_len(2) = -1d0, c_rho = -1d0, c_mu = 0d0
    integer, save :: c_types(2) = -1, c_ens = -1, c_geom = -1, c_span = -1, c_scheme = -1
    integer(c_int) :: rc
    if (c_associated(chain_ctx)) then
      if (all(c_len == block_length) .and. all(c_types == monomer_type) .and. c_ens == ensemble &
          .and. c_rho == rho .and. c_mu == mu .and. c_geom == geometry .and. c_span == span &
          .and. c_scheme == scheme .and. all(dzc == zmesh)) then
        ctx = chain_ctx
        return
      end if
      rc = adscf_ctx_destroy(chain_ctx)
      chain_ctx = c_null_ptr
      deallocate(dzc)
    end if
    call base_params(p)
    allocate(dzc(0:size(zmesh) - 1))
    dzc = zmesh
    p%geometry = geometry
    p%dz = c_loc(dzc)
    p%int_scheme = scheme
    p%int_span = span
    if (monomer_type(1) == 1) then
      p%block_length = block_length
    else
      p%block_length = [block_length(2), block_length(1)]
    end if
    p%ensemble = ensemble
    p%rho = rho; p%mu = mu
    rc = adscf_ctx_create(p, chain_ctx)
    call adscf_check(chain_ctx, rc, 'adscf_ctx_create (film chain)')
    c_len = block_length; c_types = monomer_type; c_ens = ensemble
    c_rho = rho; c_mu = mu; c_geom = geometry; c_span = span; c_scheme = scheme
    ctx = chain_ctx
  end function shim_film_chain_context

end module adscf_shim_state
