!-----------------------------------------------------------------------
! Drop-in ModIntOnRbcs: AddIntOnRbcs(c1, c2, tlist, v) of
! common/ModIntOnRbcs.F90:25 on the GB300 library.  Same public name and
! argument meaning: v(:,1:3) += the real-space Stokeslet / stresslet sums
! over the cell surfaces (with the same-cell mask), the own-cell and
! near-singular polar-patch corrections and the linear double-layer term,
! at the points of tlist.  The cells' state is pushed to the GPU first
! (positions, geometry, densities and spline tables of rbcs(:)).
!-----------------------------------------------------------------------
module ModIntOnRbcs

  use iso_c_binding
  use ModDataTypes
  use ModDataStruct
  use ModData
  use ModRbc3dGpu
  use ModRbc3dSync

  implicit none

  private

  public :: AddIntOnRbcs

contains

  subroutine AddIntOnRbcs(c1, c2, tlist, v)
    real(WP) :: c1, c2
    type(t_TargetList), target :: tlist
    real(WP) :: v(:, :)

    real(c_double), allocatable :: vv(:)
    integer(c_int) :: which
    integer :: n

    if (nrbc == 0) return
    call Rbc3dGpu_SyncCells(.true., c1 /= 0., c2 /= 0.)
    which = Rbc3dGpu_WhichList(tlist)
    n = tlist%nPoint
    allocate (vv(3*n))
    vv = reshape(v(1:n, 1:3), [3*n])
    call rbc3d_check(rbc3d_add_int_on_rbcs(gpu_ctx, which, c1, c2, gpu_matvec_prec, vv), 'rbc3d_add_int_on_rbcs')
    v(1:n, 1:3) = reshape(vv, [n, 3])
    deallocate (vv)
  end subroutine AddIntOnRbcs

end module ModIntOnRbcs
