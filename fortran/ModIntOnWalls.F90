!-----------------------------------------------------------------------
! Drop-in ModIntOnWalls (common/ModIntOnWalls.F90:37,136,181,480) on the
! GB300 library: AddIntOnWalls(c1, tlist, v), SingIntOnWall(c1, wall, v),
! PrepareSingIntOnWall(wall) and MinDistToTri(xTar, x, s0, t0, x0).
! PrepareSingIntOnWall assembles the self-wall operator on the GPU (once);
! AddIntOnWalls pushes the wall density and adds the wall single layer at
! the points of tlist.  MinDistToTri stays public for the repulsion
! routines (common/ModRepulsion.F90:600) and runs on the host
! (rbc3d_min_dist_to_tri).  The triangle rules Tri_Int_Regular /
! Tri_Int_Duffy have no callers outside the module and are not exported.
!-----------------------------------------------------------------------
module ModIntOnWalls

  use iso_c_binding
  use ModDataTypes
  use ModDataStruct
  use ModData
  use ModRbc3dGpu
  use ModRbc3dSync

  implicit none

  private

  public :: AddIntOnWalls, &
            SingIntOnWall, &
            PrepareSingIntOnWall, &
            MinDistToTri

contains

  subroutine AddIntOnWalls(c1, tlist, v)
    real(WP) :: c1
    type(t_TargetList), target :: tlist
    real(WP) :: v(:, :)

    real(c_double), allocatable :: vv(:)
    integer(c_int) :: which
    integer :: n

    if (nwall == 0) return
    call Rbc3dGpu_SyncWall
    which = Rbc3dGpu_WhichList(tlist)
    n = tlist%nPoint
    allocate (vv(3*n))
    vv = reshape(v(1:n, 1:3), [3*n])
    call rbc3d_check(rbc3d_add_int_on_walls(gpu_ctx, which, c1, gpu_matvec_prec, vv), 'rbc3d_add_int_on_walls')
    v(1:n, 1:3) = reshape(vv, [n, 3])
    deallocate (vv)
  end subroutine AddIntOnWalls

  ! v(1:nvert,:) += the self-wall operator applied to wall%f (c1 = 1/(4 pi)
  ! as the reference's callers use it): the wall-target part of
  ! AddIntOnWalls with the wall's own density.
  subroutine SingIntOnWall(c1, wall, v)
    real(WP) :: c1
    type(t_Wall) :: wall
    real(WP) :: v(:, :)

    real(c_double), allocatable :: vv(:)
    integer :: n

    n = wall%nvert
    call Rbc3dGpu_SyncWall
    allocate (vv(3*n))
    vv = reshape(v(1:n, 1:3), [3*n])
    call rbc3d_check(rbc3d_add_int_on_walls(gpu_ctx, RBC3D_TLIST_WALL, c1, RBC3D_FP64, vv), 'SingIntOnWall')
    v(1:n, 1:3) = reshape(vv, [n, 3])
    deallocate (vv)
  end subroutine SingIntOnWall

  subroutine PrepareSingIntOnWall(wall)
    type(t_wall) :: wall
    call Rbc3dGpu_Init
    call rbc3d_check(rbc3d_prepare_sing_int_on_wall(gpu_ctx), 'rbc3d_prepare_sing_int_on_wall')
  end subroutine PrepareSingIntOnWall

  function MinDistToTri(xTar, x, s0, t0, x0)
    real(WP) :: MinDistToTri
    real(WP) :: xTar(3), x(3, 3)
    real(WP), optional :: s0, t0, x0(3)

    real(c_double) :: s, t, xp(3), d

    call rbc3d_check(rbc3d_min_dist_to_tri(xTar, reshape(x, [9]), s, t, xp, d), 'rbc3d_min_dist_to_tri')
    MinDistToTri = d
    if (present(s0)) s0 = s
    if (present(t0)) t0 = t
    if (present(x0)) x0 = xp
  end function MinDistToTri

end module ModIntOnWalls
