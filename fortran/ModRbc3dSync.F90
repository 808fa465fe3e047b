!-----------------------------------------------------------------------
! ModRbc3dSync -- keeps the GPU context in step with RBC3D's module data.
!
! RBC3D refreshes its source and target lists where positions or densities
! change (SourceList_UpdateCoord / SourceList_UpdateDensity /
! TargetList_Update, e.g. common/ModTimeInt.F90:744-745,770,790).  Those CPU
! lists stay as they are (the repulsion routines read them); the drop-in
! modules in this directory push the same state to the GPU at their entry:
!   Rbc3dGpu_Init         once, from TimeInt_Init's PrepareSingIntOnWall or
!                         PME_Init (context, cell grid, wall mesh)
!   Rbc3dGpu_SyncCells    positions, geometry and spline tables of rbcs(:)
!                         (rbc3d_set_cells) and their densities
!                         (rbc3d_set_cell_density)
!   Rbc3dGpu_SyncWall     the wall density walls(1)%f
!   Rbc3dGpu_WhichList    tlist_rbc / tlist_wall / a raw list
! Layouts: cell point p = (icell-1)*nlat*nlon + (ilon-1)*nlat + ilat and
! x(p, 1:3), the order of SourceList_UpdateCoord; t_spline tables u, u1, u2,
! u12 back to back per cell.  One wall (walls(1)), as the C ABI.
!-----------------------------------------------------------------------
module ModRbc3dSync

  use iso_c_binding
  use ModDataTypes
  use ModDataStruct
  use ModConf
  use ModData
  use ModRbc3dGpu

  implicit none

  private

  public :: Rbc3dGpu_Init, &
            Rbc3dGpu_Finalize, &
            Rbc3dGpu_SyncCells, &
            Rbc3dGpu_SyncWall, &
            Rbc3dGpu_WhichList

contains

  subroutine Rbc3dGpu_Init
    type(rbc3d_params) :: prm
    type(t_wall), pointer :: wall
    integer(c_int), allocatable :: e2v(:)
    real(c_double), allocatable :: xw(:)
    integer :: l

    if (c_associated(gpu_ctx)) return
    prm%Lb = Lb
    prm%alpha = alpha_Ewd
    prm%rc = rc_Ewd
    prm%eps = eps_Ewd
    prm%Nb = Nb_Ewd
    prm%P = PBspln_Ewd
    prm%nlat = 0
    prm%nlon = 0
    if (nrbc > 0) then
      prm%nlat = rbcs(1)%nlat
      prm%nlon = rbcs(1)%nlon
    end if
    if (nCellTypes > RBC3D_MAX_CELLTYPES) call rbc3d_check(RBC3D_ERR_ARG, 'Rbc3dGpu_Init: nCellTypes')
    prm%ncelltypes = max(1, nCellTypes)
    prm%viscRat = 1.
    do l = 1, nCellTypes
      prm%viscRat(l) = viscRat(l)
    end do
    prm%vBkg = vBkg
    call rbc3d_check(rbc3d_create(prm, gpu_ctx), 'rbc3d_create')
    if (nrbc > 0) call rbc3d_check(rbc3d_set_cell_grid(gpu_ctx, rbcs(1)%th, rbcs(1)%phi, rbcs(1)%w), &
                                   'rbc3d_set_cell_grid')
    if (nwall > 1) call rbc3d_check(RBC3D_ERR_ARG, 'Rbc3dGpu_Init: one wall')
    if (nwall == 1) then
      wall => walls(1)
      allocate (xw(3*wall%nvert), e2v(3*wall%nele))
      xw = reshape(wall%x, [3*wall%nvert])
      e2v = reshape(wall%e2v, [3*wall%nele])
      call rbc3d_check(rbc3d_set_walls(gpu_ctx, wall%nvert, wall%nele, xw, e2v, wall%indxVertGlb), &
                       'rbc3d_set_walls')
      call Rbc3dGpu_SyncWall
      deallocate (xw, e2v)
    end if
  end subroutine Rbc3dGpu_Init

  subroutine Rbc3dGpu_Finalize
    integer(c_int) :: ierr
    if (.not. c_associated(gpu_ctx)) return
    ierr = rbc3d_destroy(gpu_ctx)
    gpu_ctx = c_null_ptr
  end subroutine Rbc3dGpu_Finalize

  ! Cell geometry (geom), single-layer density (fFlag) and double-layer
  ! density (gFlag) of rbcs(:) to the GPU.
  subroutine Rbc3dGpu_SyncCells(geom, fFlag, gFlag)
    logical, intent(in) :: geom, fFlag, gFlag
    integer :: irbc, nv, npt, ns, ip, is, k
    type(t_rbc), pointer :: rbc
    integer(c_int), allocatable :: ct(:)
    real(c_double), allocatable, target :: x(:, :), a3(:, :), detJ(:), area(:), msz(:)
    real(c_double), allocatable, target :: sx(:), sa(:), sd(:), f(:, :), g(:, :), sf(:), sg(:)
    type(c_ptr) :: pf, pg, psf, psg

    if (nrbc == 0) return
    nv = rbcs(1)%nlat*rbcs(1)%nlon
    npt = nrbc*nv
    if (gpu_cells_from_positions) then
      call sync_cells_raw(geom, fFlag, gFlag, nv, npt)
      return
    end if
    if (geom) then
      allocate (ct(nrbc), x(npt, 3), a3(npt, 3), detJ(npt), area(nrbc), msz(nrbc))
      ns = spline_size(rbcs(1)%spln_x)
      allocate (sx(nrbc*ns), sa(nrbc*ns), sd(nrbc*spline_size(rbcs(1)%spln_detJ)))
      do irbc = 1, nrbc
        rbc => rbcs(irbc)
        ip = (irbc - 1)*nv
        do k = 1, 3
          x(ip + 1:ip + nv, k) = reshape(rbc%x(:, :, k), [nv])
          a3(ip + 1:ip + nv, k) = reshape(rbc%a3(:, :, k), [nv])
        end do
        detJ(ip + 1:ip + nv) = reshape(rbc%detJ, [nv])
        area(irbc) = rbc%area
        msz(irbc) = rbc%meshSize
        ct(irbc) = rbc%celltype - 1
        call pack_spline(rbc%spln_x, sx, (irbc - 1)*ns)
        call pack_spline(rbc%spln_a3, sa, (irbc - 1)*ns)
        call pack_spline(rbc%spln_detJ, sd, (irbc - 1)*spline_size(rbc%spln_detJ))
      end do
      call rbc3d_check(rbc3d_set_cells(gpu_ctx, nrbc, ct, x, a3, detJ, area, msz, sx, sa, sd), 'rbc3d_set_cells')
      deallocate (ct, x, a3, detJ, area, msz, sx, sa, sd)
    end if
    if (fFlag .or. gFlag) then
      pf = c_null_ptr; pg = c_null_ptr; psf = c_null_ptr; psg = c_null_ptr
      ns = spline_size(rbcs(1)%spln_FdetJ)
      if (fFlag) then
        allocate (f(npt, 3), sf(nrbc*ns))
        do irbc = 1, nrbc
          ip = (irbc - 1)*nv
          do k = 1, 3
            f(ip + 1:ip + nv, k) = reshape(rbcs(irbc)%f(:, :, k), [nv])
          end do
          call pack_spline(rbcs(irbc)%spln_FdetJ, sf, (irbc - 1)*ns)
        end do
        pf = c_loc(f); psf = c_loc(sf)
      end if
      if (gFlag) then
        is = spline_size(rbcs(1)%spln_GdetJ)
        allocate (g(npt, 3), sg(nrbc*is))
        do irbc = 1, nrbc
          ip = (irbc - 1)*nv
          do k = 1, 3
            g(ip + 1:ip + nv, k) = reshape(rbcs(irbc)%g(:, :, k), [nv])
          end do
          call pack_spline(rbcs(irbc)%spln_GdetJ, sg, (irbc - 1)*is)
        end do
        pg = c_loc(g); psg = c_loc(sg)
      end if
      call rbc3d_check(rbc3d_set_cell_density(gpu_ctx, pf, pg, psf, psg), 'rbc3d_set_cell_density')
      if (allocated(f)) deallocate (f, sf)
      if (allocated(g)) deallocate (g, sg)
    end if
  end subroutine Rbc3dGpu_SyncCells

  ! Positions and raw densities only; the library derives a3, detJ, area,
  ! meshSize and the spline tables (RBC_ComputeGeometry and
  ! Rbc_BuildSurfaceSource at degree < nlat0) on the device.
  subroutine sync_cells_raw(geom, fFlag, gFlag, nv, npt)
    logical, intent(in) :: geom, fFlag, gFlag
    integer, intent(in) :: nv, npt
    integer :: irbc, ip, k
    integer(c_int), allocatable :: ct(:)
    real(c_double), allocatable, target :: x(:, :), f(:, :), g(:, :)
    type(c_ptr) :: pf, pg
    integer(c_int) :: nlat0

    nlat0 = int(rbcs(1)%nlat0, c_int)
    if (geom) then
      allocate (ct(nrbc), x(npt, 3))
      do irbc = 1, nrbc
        ip = (irbc - 1)*nv
        do k = 1, 3
          x(ip + 1:ip + nv, k) = reshape(rbcs(irbc)%x(:, :, k), [nv])
        end do
        ct(irbc) = rbcs(irbc)%celltype - 1
      end do
      call rbc3d_check(rbc3d_set_cells_x(gpu_ctx, int(nrbc, c_int), ct, nlat0, x), 'rbc3d_set_cells_x')
      deallocate (ct, x)
    end if
    if (fFlag .or. gFlag) then
      pf = c_null_ptr; pg = c_null_ptr
      if (fFlag) then
        allocate (f(npt, 3))
        do irbc = 1, nrbc
          ip = (irbc - 1)*nv
          do k = 1, 3
            f(ip + 1:ip + nv, k) = reshape(rbcs(irbc)%f(:, :, k), [nv])
          end do
        end do
        pf = c_loc(f)
      end if
      if (gFlag) then
        allocate (g(npt, 3))
        do irbc = 1, nrbc
          ip = (irbc - 1)*nv
          do k = 1, 3
            g(ip + 1:ip + nv, k) = reshape(rbcs(irbc)%g(:, :, k), [nv])
          end do
        end do
        pg = c_loc(g)
      end if
      call rbc3d_check(rbc3d_set_cell_density_x(gpu_ctx, nlat0, pf, pg), 'rbc3d_set_cell_density_x')
      if (allocated(f)) deallocate (f)
      if (allocated(g)) deallocate (g)
    end if
  end subroutine sync_cells_raw

  subroutine Rbc3dGpu_SyncWall
    real(c_double), allocatable :: fw(:)
    if (nwall == 0) return
    allocate (fw(3*walls(1)%nvert))
    fw = reshape(walls(1)%f, [3*walls(1)%nvert])
    call rbc3d_check(rbc3d_set_wall_density(gpu_ctx, fw), 'rbc3d_set_wall_density')
    deallocate (fw)
  end subroutine Rbc3dGpu_SyncWall

  ! RBC3D_TLIST_RBC, RBC3D_TLIST_WALL, or RBC3D_TLIST_RAW after uploading the
  ! list's points (TargetList_CreateFromRaw lists of the post-processing).
  integer(c_int) function Rbc3dGpu_WhichList(tlist) result(which)
    type(t_TargetList), target, intent(in) :: tlist
    real(c_double), allocatable :: xr(:)

    if (c_associated(c_loc(tlist), c_loc(tlist_rbc))) then
      which = RBC3D_TLIST_RBC
    else if (c_associated(c_loc(tlist), c_loc(tlist_wall))) then
      which = RBC3D_TLIST_WALL
    else
      allocate (xr(3*tlist%nPoint))
      xr = reshape(tlist%x(:, 1:3), [3*tlist%nPoint])
      call rbc3d_check(rbc3d_set_raw_targets(gpu_ctx, tlist%nPoint, xr), 'rbc3d_set_raw_targets')
      deallocate (xr)
      which = RBC3D_TLIST_RAW
    end if
  end function Rbc3dGpu_WhichList

  integer function spline_size(s)
    type(t_spline), intent(in) :: s
    spline_size = 4*size(s%u)
  end function spline_size

  subroutine pack_spline(s, buf, off)
    type(t_spline), intent(in) :: s
    real(c_double), intent(inout) :: buf(:)
    integer, intent(in) :: off
    integer :: n
    n = size(s%u)
    buf(off + 1:off + n) = reshape(s%u, [n])
    buf(off + n + 1:off + 2*n) = reshape(s%u1, [n])
    buf(off + 2*n + 1:off + 3*n) = reshape(s%u2, [n])
    buf(off + 3*n + 1:off + 4*n) = reshape(s%u12, [n])
  end subroutine pack_spline

end module ModRbc3dSync
