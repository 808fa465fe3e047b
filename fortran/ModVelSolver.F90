!-----------------------------------------------------------------------
! Drop-in ModVelSolver: Solve_RBC_Vel(v) of common/ModVelSolver.F90:44 on
! the GB300 library (deflation off, as the reference's default).  The
! right-hand side (Compute_Rhs), the operator (MyMatMult: g from the
! spherical-harmonic coefficients, its spline rebuilt, the double layer)
! and Glob_Sph_Trans run on the GPU; the coefficient vector persists
! between calls as the reference's vec_sol and warm-starts the next solve
! (KSPSetInitialGuessNonzero).  rtol 1e-11 and 200 iterations as the
! reference configures the KSP; arithmetic gpu_solve_prec.
!-----------------------------------------------------------------------
module ModVelSolver

  use iso_c_binding
  use ModDataTypes
  use ModDataStruct
  use ModConf
  use ModData
  use ModRbc3dGpu
  use ModRbc3dSync

  implicit none

  private

  real(c_double), allocatable, save :: sol(:)

  public :: Solve_RBC_Vel

contains

  subroutine Solve_RBC_Vel(v)
    real(WP) :: v(:, :)

    type(rbc3d_solve_opts) :: opt
    type(rbc3d_solve_stats) :: st
    real(c_double), allocatable :: vv(:)
    integer(c_int) :: ierr, nlat0
    integer :: n

    if (nrbc == 0) return
    nlat0 = rbcs(1)%nlat0
    call Rbc3dGpu_SyncCells(.true., .true., .false.)
    if (nwall > 0) call Rbc3dGpu_SyncWall
    if (.not. allocated(sol)) then
      allocate (sol(rbc3d_cell_dof(gpu_ctx, nlat0)))
      sol = 0.
    end if
    opt%rtol = 1.D-11
    opt%max_it = 200
    opt%restart = 30
    opt%prec = gpu_solve_prec
    opt%guess = 1
    n = size(v, 1)
    allocate (vv(3*n))
    ierr = rbc3d_solve_rbc_vel(gpu_ctx, opt, nlat0, sol, vv, st)
    if (ierr /= RBC3D_ERR_NOCONV) call rbc3d_check(ierr, 'rbc3d_solve_rbc_vel')
    v(1:n, 1:3) = reshape(vv, [n, 3])
    deallocate (vv)
    if (rootWorld) then
      write (*, '(A,I5,A,ES12.2)') 'niter = ', st%iterations, ' residual = ', st%rnorm
    end if
  end subroutine Solve_RBC_Vel

end module ModVelSolver
