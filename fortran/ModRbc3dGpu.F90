!-----------------------------------------------------------------------
! ModRbc3dGpu -- ISO_C_BINDING interface to the GB300 library
! (librbc3d_gb300.so, C ABI in include/rbc3d_gpu.h).
!
! The derived types below are bind(C) copies of the C structs
! rbc3d_params, rbc3d_counts, rbc3d_solve_opts and rbc3d_solve_stats; the
! interface block declares every entry point with the C argument passing
! (value for scalars, arrays by address).  Module state: one context per
! process (gpu_ctx) and the arithmetic of the matvec and of the solves.
!
! Host helpers marshal RBC3D's module data (ModData: rbcs, walls,
! tlist_rbc, tlist_wall; ModConf: Lb, alpha_Ewd, rc_Ewd, ...) into the flat
! arrays of the ABI:
!   cell point p = (icell-1)*nlat*nlon + (ilon-1)*nlat + ilat, x(p, 1:3),
!   the order of SourceList_UpdateCoord (common/ModSourceList.F90:92);
!   spline tables per cell u, u1, u2, u12 of t_spline back to back.
! Status codes other than RBC3D_OK stop the program with the library's
! message (the reference stops on errors as well).
!-----------------------------------------------------------------------
module ModRbc3dGpu

  use iso_c_binding

  implicit none

  integer(c_int), parameter :: RBC3D_OK = 0, RBC3D_ERR_ARG = 1, RBC3D_ERR_CUDA = 2, &
                               RBC3D_ERR_TIMEOUT = 3, RBC3D_ERR_NOCONV = 4, &
                               RBC3D_ERR_OVERFLOW = 5, RBC3D_ERR_STATE = 6, RBC3D_ERR_NOMEM = 7
  integer(c_int), parameter :: RBC3D_FP64 = 0, RBC3D_FP32C = 1, RBC3D_FP32M = 2, RBC3D_FP32D = 3
  integer(c_int), parameter :: RBC3D_TLIST_RBC = 0, RBC3D_TLIST_WALL = 1, RBC3D_TLIST_RAW = 2
  integer(c_int), parameter :: RBC3D_TERM_REAL = 1, RBC3D_TERM_CORR = 2, RBC3D_TERM_LINEAR = 4, &
                               RBC3D_TERM_PME = 8, RBC3D_TERM_WALLS = 16, RBC3D_TERM_ALL = 31
  integer, parameter :: RBC3D_MAX_CELLTYPES = 8

  ! rbc3d_params (include/rbc3d_gpu.h)
  type, bind(C) :: rbc3d_params
    real(c_double) :: Lb(3)
    real(c_double) :: alpha
    real(c_double) :: rc
    real(c_double) :: eps
    integer(c_int) :: Nb(3)
    integer(c_int) :: P
    integer(c_int) :: nlat
    integer(c_int) :: nlon
    integer(c_int) :: ncelltypes
    real(c_double) :: viscRat(RBC3D_MAX_CELLTYPES)
    real(c_double) :: vBkg(3)
  end type rbc3d_params

  ! rbc3d_counts
  type, bind(C) :: rbc3d_counts
    integer(c_long_long) :: pairs_within_rc
    integer(c_long_long) :: nbr_items
    integer(c_long_long) :: nearsing_items
    integer(c_long_long) :: self_items
    integer(c_long_long) :: wall_pairs
    integer(c_long_long) :: wall_duffy
    integer(c_int) :: nbr_overflow
    integer(c_long_long) :: kernel_launches
    integer(c_long_long) :: screen_misses
    integer(c_long_long) :: near_replays
    integer(c_long_long) :: near_projections
  end type rbc3d_counts

  ! rbc3d_solve_opts
  type, bind(C) :: rbc3d_solve_opts
    real(c_double) :: rtol
    integer(c_int) :: max_it
    integer(c_int) :: restart
    integer(c_int) :: prec
    integer(c_int) :: guess
  end type rbc3d_solve_opts

  ! rbc3d_solve_stats
  type, bind(C) :: rbc3d_solve_stats
    integer(c_int) :: iterations
    integer(c_int) :: converged
    real(c_double) :: rnorm0
    real(c_double) :: rnorm
    real(c_double) :: bnorm
    real(c_double) :: ms
    integer(c_int) :: matvecs
    integer(c_int) :: refinements
  end type rbc3d_solve_stats

  interface
    integer(c_int) function rbc3d_abi_version() bind(C, name="rbc3d_abi_version")
      import
    end function
    integer(c_int) function rbc3d_ewald_prms(alpha, eps, Lb, P, rc, Nb) bind(C, name="rbc3d_ewald_prms")
      import
      real(c_double), value :: alpha, eps
      real(c_double), intent(in) :: Lb(3)
      integer(c_int), value :: P
      real(c_double), intent(out) :: rc
      integer(c_int), intent(out) :: Nb(3)
    end function
    integer(c_int) function rbc3d_create(prm, ctx) bind(C, name="rbc3d_create")
      import
      type(rbc3d_params), intent(in) :: prm
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function rbc3d_destroy(ctx) bind(C, name="rbc3d_destroy")
      import
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function rbc3d_last_error(ctx) bind(C, name="rbc3d_last_error")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function rbc3d_set_cell_grid(ctx, th, phi, w) bind(C, name="rbc3d_set_cell_grid")
      import
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: th(*), phi(*), w(*)
    end function
    integer(c_int) function rbc3d_set_cells(ctx, ncell, celltype, x, a3, detJ, area, meshSize, &
                                            spl_x, spl_a3, spl_detJ) bind(C, name="rbc3d_set_cells")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncell
      integer(c_int), intent(in) :: celltype(*)
      real(c_double), intent(in) :: x(*), a3(*), detJ(*), area(*), meshSize(*)
      real(c_double), intent(in) :: spl_x(*), spl_a3(*), spl_detJ(*)
    end function
    integer(c_int) function rbc3d_set_cell_density(ctx, f, g, spl_FdetJ, spl_GdetJ) &
        bind(C, name="rbc3d_set_cell_density")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: f, g, spl_FdetJ, spl_GdetJ   ! c_loc(...) or c_null_ptr
    end function
    integer(c_int) function rbc3d_set_walls(ctx, nvert, nele, x, e2v, indxVertGlb) bind(C, name="rbc3d_set_walls")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: nvert, nele
      real(c_double), intent(in) :: x(*)
      integer(c_int), intent(in) :: e2v(*), indxVertGlb(*)
    end function
    integer(c_int) function rbc3d_set_wall_density(ctx, f) bind(C, name="rbc3d_set_wall_density")
      import
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: f(*)
    end function
    integer(c_int) function rbc3d_get_wall_density(ctx, f) bind(C, name="rbc3d_get_wall_density")
      import
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: f(*)
    end function
    integer(c_int) function rbc3d_set_raw_targets(ctx, n, x) bind(C, name="rbc3d_set_raw_targets")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: n
      real(c_double), intent(in) :: x(*)
    end function
    integer(c_int) function rbc3d_num_targets(ctx, tlist) bind(C, name="rbc3d_num_targets")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: tlist
    end function
    integer(c_int) function rbc3d_add_int_on_rbcs(ctx, tlist, c1, c2, prec, v) bind(C, name="rbc3d_add_int_on_rbcs")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: tlist, prec
      real(c_double), value :: c1, c2
      real(c_double), intent(inout) :: v(*)
    end function
    integer(c_int) function rbc3d_add_int_on_walls(ctx, tlist, c1, prec, v) bind(C, name="rbc3d_add_int_on_walls")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: tlist, prec
      real(c_double), value :: c1
      real(c_double), intent(inout) :: v(*)
    end function
    integer(c_int) function rbc3d_prepare_sing_int_on_wall(ctx) bind(C, name="rbc3d_prepare_sing_int_on_wall")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function rbc3d_pme_distrib_source(ctx, c1, c2, cells, walls, prec) &
        bind(C, name="rbc3d_pme_distrib_source")
      import
      type(c_ptr), value :: ctx
      real(c_double), value :: c1, c2
      integer(c_int), value :: cells, walls, prec
    end function
    integer(c_int) function rbc3d_pme_transform(ctx) bind(C, name="rbc3d_pme_transform")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function rbc3d_pme_add_interp_vel(ctx, tlist, v) bind(C, name="rbc3d_pme_add_interp_vel")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: tlist
      real(c_double), intent(inout) :: v(*)
    end function
    integer(c_int) function rbc3d_matvec(ctx, tlist, c1, c2, terms, prec, v) bind(C, name="rbc3d_matvec")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: tlist, terms, prec
      real(c_double), value :: c1, c2
      real(c_double), intent(inout) :: v(*)
    end function
    integer(c_int) function rbc3d_compute_wall_residual_vel(ctx, prec, v) &
        bind(C, name="rbc3d_compute_wall_residual_vel")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: prec
      real(c_double), intent(out) :: v(*)
    end function
    integer(c_int) function rbc3d_wall_matmult(ctx, prec, u, y) bind(C, name="rbc3d_wall_matmult")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: prec
      real(c_double), intent(in) :: u(*)
      real(c_double), intent(out) :: y(*)
    end function
    integer(c_int) function rbc3d_no_slip_wall(ctx, opt, guess, st) bind(C, name="rbc3d_no_slip_wall")
      import
      type(c_ptr), value :: ctx
      type(rbc3d_solve_opts), intent(in) :: opt
      type(c_ptr), value :: guess                         ! c_null_ptr: zero increment
      type(rbc3d_solve_stats), intent(out) :: st
    end function
    integer(c_int) function rbc3d_calc_velocity_field(ctx, tlist, prec, v) bind(C, name="rbc3d_calc_velocity_field")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: tlist, prec
      real(c_double), intent(out) :: v(*)
    end function
    integer(c_int) function rbc3d_get_counts(ctx, c) bind(C, name="rbc3d_get_counts")
      import
      type(c_ptr), value :: ctx
      type(rbc3d_counts), intent(out) :: c
    end function
    integer(c_int) function rbc3d_cell_dof(ctx, nlat0) bind(C, name="rbc3d_cell_dof")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: nlat0
    end function
    integer(c_int) function rbc3d_solve_rbc_vel(ctx, opt, nlat0, sol, v, st) bind(C, name="rbc3d_solve_rbc_vel")
      import
      type(c_ptr), value :: ctx
      type(rbc3d_solve_opts), intent(in) :: opt
      integer(c_int), value :: nlat0
      real(c_double), intent(inout) :: sol(*)
      real(c_double), intent(out) :: v(*)
      type(rbc3d_solve_stats), intent(out) :: st
    end function
    integer(c_int) function rbc3d_set_ref_cells(ctx, ntypes, xref, ES, ED, EB) bind(C, name="rbc3d_set_ref_cells")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: ntypes
      real(c_double), intent(in) :: xref(*), ES(*), ED(*), EB(*)
    end function
    integer(c_int) function rbc3d_cell_geometry(ctx, ncell, x, a3, detJ, area, vol) bind(C, name="rbc3d_cell_geometry")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncell
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(out) :: a3(*), detJ(*), area(*), vol(*)
    end function
    integer(c_int) function rbc3d_shell_res_force(ctx, ncell, celltype, x, f) bind(C, name="rbc3d_shell_res_force")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncell
      integer(c_int), intent(in) :: celltype(*)
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(out) :: f(*)
    end function
    integer(c_int) function rbc3d_intra_cell_repulsion(ctx, ncell, x, a3, area, force_coef, f, count) &
        bind(C, name="rbc3d_intra_cell_repulsion")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncell
      real(c_double), intent(in) :: x(*), a3(*), area(*)
      real(c_double), value :: force_coef
      real(c_double), intent(inout) :: f(*)
      integer(c_int), intent(out) :: count
    end function
    integer(c_int) function rbc3d_set_cells_x(ctx, ncell, celltype, nlat0, x) bind(C, name="rbc3d_set_cells_x")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncell, nlat0
      integer(c_int), intent(in) :: celltype(*)
      real(c_double), intent(in) :: x(*)
    end function
    integer(c_int) function rbc3d_set_cell_density_x(ctx, nlat0, f, g) bind(C, name="rbc3d_set_cell_density_x")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: nlat0
      type(c_ptr), value :: f, g                          ! c_loc(...) or c_null_ptr
    end function
    integer(c_int) function rbc3d_inter_cell_repulsion(ctx, epsDist, viscRatThresh, rigidsep, x, distMin, nmoved) &
        bind(C, name="rbc3d_inter_cell_repulsion")
      import
      type(c_ptr), value :: ctx
      real(c_double), value :: epsDist, viscRatThresh
      integer(c_int), value :: rigidsep
      real(c_double), intent(out) :: x(*)
      real(c_double), intent(out) :: distMin
      integer(c_int), intent(out) :: nmoved
    end function
    integer(c_int) function rbc3d_wall_rhs(ctx, prec, b) bind(C, name="rbc3d_wall_rhs")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: prec
      real(c_double), intent(out) :: b(*)
    end function
    integer(c_int) function rbc3d_wall_spectral_init(ctx, nring, tau, record) bind(C, name="rbc3d_wall_spectral_init")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: nring, record
      real(c_double), value :: tau
    end function
    integer(c_int) function rbc3d_wall_spectral_add(ctx, x, added) bind(C, name="rbc3d_wall_spectral_add")
      import
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: x(*)
      integer(c_int), intent(out) :: added
    end function
    integer(c_int) function rbc3d_wall_spectral_predict(ctx, b, x0, rem) bind(C, name="rbc3d_wall_spectral_predict")
      import
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: b(*)
      real(c_double), intent(out) :: x0(*), rem(*)
    end function
    integer(c_int) function rbc3d_wall_spectral_size(ctx, nmodes, nbasis, pairs) bind(C, name="rbc3d_wall_spectral_size")
      import
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: nmodes
      integer(c_int), intent(out) :: nbasis(*)
      integer(c_long_long), intent(out) :: pairs
    end function
    integer(c_int) function rbc3d_min_dist_to_tri(xtar, x, s0, t0, x0, dist) bind(C, name="rbc3d_min_dist_to_tri")
      import
      real(c_double), intent(in) :: xtar(3), x(9)
      real(c_double), intent(out) :: s0, t0, x0(3), dist
    end function
  end interface

  ! The context of this process and the arithmetic of each use
  type(c_ptr), save :: gpu_ctx = c_null_ptr
  integer(c_int), save :: gpu_matvec_prec = RBC3D_FP32D  ! AddIntOnRbcs, PME_*, residual velocities
  integer(c_int), save :: gpu_solve_prec = RBC3D_FP64    ! NoSlipWall, Solve_RBC_Vel operators
  ! .true.: Rbc3dGpu_SyncCells sends positions and raw densities only, and the
  ! library derives the geometry and the spline tables on the device
  ! (rbc3d_set_cells_x / rbc3d_set_cell_density_x, degree < nlat0)
  logical, save :: gpu_cells_from_positions = .false.



contains

  ! Stops with the library's message unless ierr is RBC3D_OK.
  subroutine rbc3d_check(ierr, where)
    integer(c_int), intent(in) :: ierr
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    character(len=256) :: text
    integer :: i

    if (ierr == RBC3D_OK) return
    text = ''
    if (c_associated(gpu_ctx)) then
      call c_f_pointer(rbc3d_last_error(gpu_ctx), msg, [256])
      do i = 1, 256
        if (msg(i) == c_null_char) exit
        text(i:i) = msg(i)
      end do
    end if
    write (*, '(A,A,A,I0,A,A)') 'rbc3d_gb300: ', where, ' returned status ', ierr, ': ', trim(text)
    stop 1
  end subroutine rbc3d_check

end module ModRbc3dGpu
