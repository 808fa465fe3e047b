!-----------------------------------------------------------------------
! Drop-in ModPME (common/ModPME.F90:44-48): PME_Init, PME_Finalize,
! PME_Distrib_Source(c1, c2, cells, walls), PME_Transform and
! PME_Add_Interp_Vel(tlist, v) on the GB300 library.  The mesh, the
! B-spline factors and the FFT plans live in the GPU context
! (rbc3d_create), so PME_Init creates the context and PME_Finalize
! destroys it.  PME_Distrib_Source pushes the cells' and the wall's
! state first; the velocity grid stays on the GPU between the calls.
!-----------------------------------------------------------------------
module ModPME

  use iso_c_binding
  use ModDataTypes
  use ModDataStruct
  use ModData
  use ModRbc3dGpu
  use ModRbc3dSync

  implicit none

  private

  public :: PME_Init, &
            PME_Finalize, &
            PME_Distrib_Source, &
            PME_Transform, &
            PME_Add_Interp_Vel

contains

  subroutine PME_Init
    call Rbc3dGpu_Init
  end subroutine PME_Init

  subroutine PME_Finalize
    call Rbc3dGpu_Finalize
  end subroutine PME_Finalize

  subroutine PME_Distrib_Source(c1, c2, cells, walls)
    real(WP) :: c1, c2
    type(t_rbc), optional :: cells(:)
    type(t_wall), optional :: walls(:)

    integer(c_int) :: use_cells, use_walls

    use_cells = 0
    use_walls = 0
    if (present(cells)) then
      use_cells = 1
      call Rbc3dGpu_SyncCells(.true., c1 /= 0., c2 /= 0.)
    end if
    if (present(walls)) then
      use_walls = 1
      call Rbc3dGpu_SyncWall
    end if
    call rbc3d_check(rbc3d_pme_distrib_source(gpu_ctx, c1, c2, use_cells, use_walls, gpu_matvec_prec), &
                     'rbc3d_pme_distrib_source')
  end subroutine PME_Distrib_Source

  subroutine PME_Transform
    call rbc3d_check(rbc3d_pme_transform(gpu_ctx), 'rbc3d_pme_transform')
  end subroutine PME_Transform

  subroutine PME_Add_Interp_Vel(tlist, v)
    type(t_TargetList), target :: tlist
    real(WP) :: v(:, :)

    real(c_double), allocatable :: vv(:)
    integer(c_int) :: which
    integer :: n

    which = Rbc3dGpu_WhichList(tlist)
    n = tlist%nPoint
    allocate (vv(3*n))
    vv = reshape(v(1:n, 1:3), [3*n])
    call rbc3d_check(rbc3d_pme_add_interp_vel(gpu_ctx, which, vv), 'rbc3d_pme_add_interp_vel')
    v(1:n, 1:3) = reshape(vv, [n, 3])
    deallocate (vv)
  end subroutine PME_Add_Interp_Vel

end module ModPME
