!-----------------------------------------------------------------------
! Drop-in ModNoSlip (common/ModNoSlip.F90:32-34): NoSlipWall and
! Compute_Wall_Residual_Vel(v) on the GB300 library.  NoSlipWall solves
! for the wall-density increment with the device GMRES (PCNONE, the
! reference's KSP settings: rtol eps_Ewd, restart 30; max_it below) from a
! zero increment and updates walls(1)%f; Compute_Wall_Residual_Vel returns
! the residual wall velocity (cells + walls + PME + background velocity)
! at the wall vertices.  The cells' state is pushed first.
! Arithmetic: gpu_solve_prec (RBC3D_FP64, or an FP32 mode for the
! mixed-precision solve judged on the FP64 residual).
! NoSlipWall_Rings > 0 (the wall a uniform stack of that many rings along
! z, as the tube meshes) switches on the learned spectral operator: every
! converged solve teaches it its exact pair (A x, x), and each solve starts
! from its prediction with the operator as GMRES's right preconditioner
! (guess mode 5); the stopping test stays ||b - A x|| < rtol ||b||.  0 (the
! default) is the reference's solve from a zero increment.
!-----------------------------------------------------------------------
module ModNoSlip

  use iso_c_binding
  use ModDataTypes
  use ModDataStruct
  use ModConf
  use ModData
  use ModRbc3dGpu
  use ModRbc3dSync

  implicit none

  private

  integer, save, public :: NoSlipWall_MaxIt = 60      ! KSPSetTolerances max_it of NoSlipWall
  integer, save, public :: NoSlipWall_Restart = 30    ! KSPGMRESSetRestart (PETSc default)
  integer, save, public :: NoSlipWall_Rings = 0       ! > 0: learned spectral preconditioner
  logical, save :: spectral_ready = .false.

  public :: NoSlipWall, &
            Compute_Wall_Residual_Vel

contains

  subroutine NoSlipWall
    type(rbc3d_solve_opts) :: opt
    type(rbc3d_solve_stats) :: st
    real(c_double), allocatable :: fw(:)
    integer(c_int) :: ierr

    if (nwall == 0) return
    call Rbc3dGpu_SyncCells(.true., .true., .true.)
    call Rbc3dGpu_SyncWall
    opt%rtol = eps_Ewd
    opt%max_it = NoSlipWall_MaxIt
    opt%restart = NoSlipWall_Restart
    opt%prec = gpu_solve_prec
    opt%guess = 0
    if (NoSlipWall_Rings > 0) then
      if (.not. spectral_ready) then
        call rbc3d_check(rbc3d_wall_spectral_init(gpu_ctx, int(NoSlipWall_Rings, c_int), 1.0e-7_c_double, 1_c_int), &
                         'rbc3d_wall_spectral_init')
        spectral_ready = .true.
      end if
      opt%guess = 5
    end if
    ierr = rbc3d_no_slip_wall(gpu_ctx, opt, c_null_ptr, st)
    if (ierr /= RBC3D_ERR_NOCONV) call rbc3d_check(ierr, 'rbc3d_no_slip_wall')  ! KSP returns at max_it too
    allocate (fw(3*walls(1)%nvert))
    call rbc3d_check(rbc3d_get_wall_density(gpu_ctx, fw), 'rbc3d_get_wall_density')
    walls(1)%f = reshape(fw, [walls(1)%nvert, 3])
    deallocate (fw)
    if (rootWorld) then
      write (*, '(A)') 'Wall iteration:'
      write (*, '(A,I5,A,ES12.2)') 'niter = ', st%iterations, ' residual = ', st%rnorm
    end if
  end subroutine NoSlipWall

  subroutine Compute_Wall_Residual_Vel(v)
    real(WP) :: v(:, :)

    real(c_double), allocatable :: vv(:)
    integer :: n

    n = walls(1)%nvert
    call Rbc3dGpu_SyncCells(.true., .true., .true.)
    call Rbc3dGpu_SyncWall
    allocate (vv(3*n))
    call rbc3d_check(rbc3d_compute_wall_residual_vel(gpu_ctx, gpu_matvec_prec, vv), &
                     'rbc3d_compute_wall_residual_vel')
    v(1:n, 1:3) = reshape(vv, [n, 3])
    deallocate (vv)
  end subroutine Compute_Wall_Residual_Vel

end module ModNoSlip
