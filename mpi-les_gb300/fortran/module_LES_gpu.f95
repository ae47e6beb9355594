! module_LES_gpu.f95 -- Fortran binding of the GB300 solver library (include/les_gpu.h).
!
! A drop-in for MPI-LES's solver calls: the subroutines below keep the names and
! argument lists of the reference's velnw (velnw.f95:5), bondv1 (bondv1.f95:5),
! velfg (velFG.f95:6-8), feedbf (feedbf.f95:5-6), les (les.f95:6-7), adam
! (adam.f95:5), press (press.f95:9-10), boundp1/boundp2 (boundp.f95:28,7), and work on
! the device-resident copy of the state.  The host arrays are read only by
! initialise_LES_gpu and written only by sync_LES_gpu (the sync points); in between
! their contents are ignored.  run_LES_gpu(n, nmax) is the whole step on the device
! (the counterpart of run_LES_kernel, main.f95:251).
!
! main.f95 selects it with the macro that switches the OpenCL path today
! (main.f95:14-27, 228-234, 250-251), e.g.
!
!   #ifdef _CUDA_LES
!         use module_LES_gpu
!         call initialise_LES_gpu(p,u,v,w,usum,vsum,wsum,f,g,h,fold,gold,hold, &
!              bmask1,cmask1,dmask1,cn1,cn2l,cn2s,cn3l,cn3s,cn4l,cn4s,dxs,dys,dzs,dx1,dy1, &
!              dzn,z2,dt,im,jm,km)
!         ...
!         do n = n0, nmax
!           call run_LES_gpu(n, nmax)
!         end do
!         call sync_LES_gpu(u,v,w,p,usum,vsum,wsum,fold,gold,hold,im,jm,km)
!   #endif
!
! Link with -L<repo>/mpi-les_gb300/_build -llesgpu.  Built with the reference's own
! Fortran flags; requires a Fortran 2003 compiler (ISO_C_BINDING).
module module_LES_gpu
  use, intrinsic :: iso_c_binding
  implicit none
  private
  public :: initialise_LES_gpu, run_LES_gpu, sync_LES_gpu, finalise_LES_gpu
  public :: velnw, bondv1, velfg, feedbf, les, adam, press, boundp1, boundp2
  public :: ifdata_out, read_restart_LES_gpu, aveflow

  ! field ids of include/les_gpu.h
  integer(c_int), parameter :: LES_FIELD_U = 1, LES_FIELD_V = 2, LES_FIELD_W = 3, LES_FIELD_P = 4
  integer(c_int), parameter :: LES_FIELD_F = 5, LES_FIELD_G = 6, LES_FIELD_H = 7
  integer(c_int), parameter :: LES_FIELD_FOLD = 8, LES_FIELD_GOLD = 9, LES_FIELD_HOLD = 10
  integer(c_int), parameter :: LES_FIELD_USUM = 11, LES_FIELD_VSUM = 12, LES_FIELD_WSUM = 13
  integer(c_int), parameter :: LES_FIELD_BMASK1 = 16, LES_FIELD_CMASK1 = 17, LES_FIELD_DMASK1 = 18
  integer(c_int), parameter :: LES_FIELD_CN1 = 20
  integer(c_int), parameter :: LES_FIELD_DX1 = 32, LES_FIELD_DY1 = 33, LES_FIELD_DZN = 34, LES_FIELD_DZS = 35
  integer(c_int), parameter :: LES_FIELD_DXS = 36, LES_FIELD_DYS = 37, LES_FIELD_Z2 = 38
  integer(c_int), parameter :: LES_FIELD_CN2L = 39, LES_FIELD_CN2S = 40, LES_FIELD_CN3L = 41
  integer(c_int), parameter :: LES_FIELD_CN3S = 42, LES_FIELD_CN4L = 43, LES_FIELD_CN4S = 44
  integer(c_int), parameter :: LES_FIELD_UIN = 53, LES_FIELD_VIN = 54, LES_FIELD_WIN = 55

  type, bind(C) :: les_dims
    integer(c_int) :: im, jm, km
  end type
  type, bind(C) :: les_params
    real(c_float) :: dt, ro, vn, alpha, beta, omega, pjuge
    integer(c_int) :: nmaxp, sor_fixed, sor_ksplit
  end type

  type(c_ptr), save :: les_h = c_null_ptr

  interface
    integer(c_int) function les_gpu_create(dims, prm, h) bind(C, name='les_gpu_create')
      import :: c_int, c_ptr, les_dims, les_params
      type(les_dims), intent(in) :: dims
      type(les_params), intent(in) :: prm
      type(c_ptr), intent(out) :: h
    end function
    integer(c_int) function les_gpu_destroy(h) bind(C, name='les_gpu_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_upload(h, field, host, lb, ub) bind(C, name='les_gpu_upload')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: h
      integer(c_int), value :: field
      real(c_float), intent(in) :: host(*)
      integer(c_int), intent(in) :: lb(3), ub(3)
    end function
    integer(c_int) function les_gpu_download(h, field, host, lb, ub) bind(C, name='les_gpu_download')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: h
      integer(c_int), value :: field
      real(c_float), intent(inout) :: host(*)
      integer(c_int), intent(in) :: lb(3), ub(3)
    end function
    integer(c_int) function les_gpu_sync(h) bind(C, name='les_gpu_sync')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_download_async(h, field, host, lb, ub, ticket) &
        bind(C, name='les_gpu_download_async')
      import :: c_int, c_ptr, c_float, c_long_long
      type(c_ptr), value :: h
      integer(c_int), value :: field
      real(c_float), intent(inout) :: host(*)
      integer(c_int), intent(in) :: lb(3), ub(3)
      integer(c_long_long), intent(out) :: ticket
    end function
    integer(c_int) function les_gpu_download_wait(h, ticket) bind(C, name='les_gpu_download_wait')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h
      integer(c_long_long), value :: ticket
    end function
    integer(c_int) function les_gpu_aveflow(h, n, n1, nmax) bind(C, name='les_gpu_aveflow')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: n, n1, nmax
    end function
    integer(c_int) function les_gpu_write_data20(h, path, flags) bind(C, name='les_gpu_write_data20')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: path
      integer(c_int), value :: flags
    end function
    integer(c_int) function les_gpu_write_data10(h, path, flags) bind(C, name='les_gpu_write_data10')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: path
      integer(c_int), value :: flags
    end function
    integer(c_int) function les_gpu_write_data11(h, path, flags) bind(C, name='les_gpu_write_data11')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: path
      integer(c_int), value :: flags
    end function
    integer(c_int) function les_gpu_write_data21(h, path, flags) bind(C, name='les_gpu_write_data21')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: path
      integer(c_int), value :: flags
    end function
    integer(c_int) function les_gpu_ifdata_out(h, dir, n, n1, nmax, time, flags, written) &
        bind(C, name='les_gpu_ifdata_out')
      import :: c_int, c_ptr, c_char, c_float
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: dir
      integer(c_int), value :: n, n1, nmax, flags
      real(c_float), value :: time
      integer(c_int) :: written
    end function
    integer(c_int) function les_gpu_read_restart(h, data30, data31, n, time) bind(C, name='les_gpu_read_restart')
      import :: c_int, c_ptr, c_char, c_float
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: data30, data31
      integer(c_int) :: n
      real(c_float) :: time
    end function
    integer(c_int) function les_gpu_commit_setup(h) bind(C, name='les_gpu_commit_setup')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_velnw(h) bind(C, name='les_gpu_velnw')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_bondv1(h, n) bind(C, name='les_gpu_bondv1')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: n
    end function
    integer(c_int) function les_gpu_velfg(h) bind(C, name='les_gpu_velfg')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_feedbf(h) bind(C, name='les_gpu_feedbf')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_les(h) bind(C, name='les_gpu_les')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_adam(h) bind(C, name='les_gpu_adam')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_press(h, n, nmax) bind(C, name='les_gpu_press')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: n, nmax
    end function
    integer(c_int) function les_gpu_boundp1(h) bind(C, name='les_gpu_boundp1')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_boundp2(h) bind(C, name='les_gpu_boundp2')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    integer(c_int) function les_gpu_step(h, n, nmax) bind(C, name='les_gpu_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: n, nmax
    end function
    integer(c_int) function les_gpu_last_error(h, buf, length) bind(C, name='les_gpu_last_error')
      import :: c_int, c_ptr, c_char, c_size_t
      type(c_ptr), value :: h
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_size_t), value :: length
    end function
  end interface

contains

  subroutine check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    character(kind=c_char) :: buf(512)
    integer(c_int) :: r2
    integer :: q
    character(len=512) :: msg
    if (rc == 0) return
    r2 = les_gpu_last_error(les_h, buf, int(512, c_size_t))
    msg = ' '
    do q = 1, 512
      if (buf(q) == c_null_char) exit
      msg(q:q) = buf(q)
    end do
    print *, 'les_gpu: ', what, ' failed (', rc, '): ', trim(msg)
    stop 1
  end subroutine

  subroutine put3(field, a, l1, u1, l2, u2, l3, u3)
    integer(c_int), intent(in) :: field
    integer, intent(in) :: l1, u1, l2, u2, l3, u3
    real(4), intent(in) :: a(l1:u1, l2:u2, l3:u3)
    call check(les_gpu_upload(les_h, field, a, [l1, l2, l3], [u1, u2, u3]), 'upload')
  end subroutine

  subroutine get3(field, a, l1, u1, l2, u2, l3, u3)
    integer(c_int), intent(in) :: field
    integer, intent(in) :: l1, u1, l2, u2, l3, u3
    real(4), intent(inout) :: a(l1:u1, l2:u2, l3:u3)
    call check(les_gpu_download(les_h, field, a, [l1, l2, l3], [u1, u2, u3]), 'download')
  end subroutine

  subroutine put1(field, a, l1, u1)
    integer(c_int), intent(in) :: field
    integer, intent(in) :: l1, u1
    real(4), intent(in) :: a(l1:u1)
    call check(les_gpu_upload(les_h, field, a, [l1, 0, 0], [u1, 0, 0]), 'upload')
  end subroutine

  ! Upload the state, grid, coefficients, masks and the inflow profile of
  ! bondv1.f95:33-54 (5 m/s up to k = 78, u(77) above, v = w = 0), then commit.
  ! Replaces initialise_LES_kernel (main.f95:229-233).  press leaves its SOR loop
  ! once sor < pjuge (press.f95:119-121), as the reference does; the optional
  ! fixed_sor = .true. always runs nmaxp = 50 iterations instead (throughput runs).
  subroutine initialise_LES_gpu(p, u, v, w, usum, vsum, wsum, f, g, h, fold, gold, hold, &
                                bmask1, cmask1, dmask1, cn1, cn2l, cn2s, cn3l, cn3s, cn4l, cn4s, &
                                dxs, dys, dzs, dx1, dy1, dzn, z2, dt, im, jm, km, fixed_sor)
    integer, intent(in) :: im, jm, km
    logical, intent(in), optional :: fixed_sor
    real(4), intent(in) :: dt
    real(4), intent(in) :: p(0:im+2, 0:jm+2, 0:km+1)
    real(4), intent(in) :: u(0:im+1, -1:jm+1, 0:km+1), v(0:im+1, -1:jm+1, 0:km+1)
    real(4), intent(in) :: w(0:im+1, -1:jm+1, -1:km+1)
    real(4), intent(in) :: usum(0:im, 0:jm, 0:km), vsum(0:im, 0:jm, 0:km), wsum(0:im, 0:jm, 0:km)
    real(4), intent(in) :: f(0:im, 0:jm, 0:km), g(0:im, 0:jm, 0:km), h(0:im, 0:jm, 0:km)
    real(4), intent(in) :: fold(im, jm, km), gold(im, jm, km), hold(im, jm, km)
    real(4), intent(in) :: bmask1(-1:im+1, 0:jm+1, 0:km+1), cmask1(0:im+1, -1:jm+1, 0:km+1)
    real(4), intent(in) :: dmask1(0:im+1, 0:jm+1, 0:km+1)
    real(4), intent(in) :: cn1(im, jm, km), cn2l(im), cn2s(im), cn3l(jm), cn3s(jm), cn4l(km), cn4s(km)
    real(4), intent(in) :: dxs(0:im), dys(0:jm), dzs(-1:km+2), dx1(-1:im+1), dy1(0:jm+1), dzn(-1:km+2)
    real(4), intent(in) :: z2(0:km+2)
    type(les_dims) :: dims
    type(les_params) :: prm
    real(4), allocatable :: inflow(:, :), zero(:, :)
    integer :: k
    integer(c_int) :: sor_fixed
    sor_fixed = 0
    if (present(fixed_sor)) then
      if (fixed_sor) sor_fixed = 1
    end if
    dims = les_dims(im, jm, km)
    ! set.f95:89-95 (dt, ro, vn, alpha, beta) and press.f95:43-45 (omega, pjuge,
    ! nmaxp); sor_fixed = 0 is press.f95:119-121's exit on sor < pjuge
    prm = les_params(dt, 1.1763, 15.83 * 10.**(-6.), -10., -1., 1., 0.0001, 50, sor_fixed, 0)
    call check(les_gpu_create(dims, prm, les_h), 'create')
    call put3(LES_FIELD_P, p, 0, im + 2, 0, jm + 2, 0, km + 1)
    call put3(LES_FIELD_U, u, 0, im + 1, -1, jm + 1, 0, km + 1)
    call put3(LES_FIELD_V, v, 0, im + 1, -1, jm + 1, 0, km + 1)
    call put3(LES_FIELD_W, w, 0, im + 1, -1, jm + 1, -1, km + 1)
    call put3(LES_FIELD_USUM, usum, 0, im, 0, jm, 0, km)
    call put3(LES_FIELD_VSUM, vsum, 0, im, 0, jm, 0, km)
    call put3(LES_FIELD_WSUM, wsum, 0, im, 0, jm, 0, km)
    call put3(LES_FIELD_F, f, 0, im, 0, jm, 0, km)
    call put3(LES_FIELD_G, g, 0, im, 0, jm, 0, km)
    call put3(LES_FIELD_H, h, 0, im, 0, jm, 0, km)
    call put3(LES_FIELD_FOLD, fold, 1, im, 1, jm, 1, km)
    call put3(LES_FIELD_GOLD, gold, 1, im, 1, jm, 1, km)
    call put3(LES_FIELD_HOLD, hold, 1, im, 1, jm, 1, km)
    call put3(LES_FIELD_BMASK1, bmask1, -1, im + 1, 0, jm + 1, 0, km + 1)
    call put3(LES_FIELD_CMASK1, cmask1, 0, im + 1, -1, jm + 1, 0, km + 1)
    call put3(LES_FIELD_DMASK1, dmask1, 0, im + 1, 0, jm + 1, 0, km + 1)
    call put3(LES_FIELD_CN1, cn1, 1, im, 1, jm, 1, km)
    call put1(LES_FIELD_DX1, dx1, -1, im + 1)
    call put1(LES_FIELD_DY1, dy1, 0, jm + 1)
    call put1(LES_FIELD_DZN, dzn, -1, km + 2)
    call put1(LES_FIELD_DZS, dzs, -1, km + 2)
    call put1(LES_FIELD_DXS, dxs, 0, im)
    call put1(LES_FIELD_DYS, dys, 0, jm)
    call put1(LES_FIELD_Z2, z2, 0, km + 2)
    call put1(LES_FIELD_CN2L, cn2l, 1, im)
    call put1(LES_FIELD_CN2S, cn2s, 1, im)
    call put1(LES_FIELD_CN3L, cn3l, 1, jm)
    call put1(LES_FIELD_CN3S, cn3s, 1, jm)
    call put1(LES_FIELD_CN4L, cn4l, 1, km)
    call put1(LES_FIELD_CN4S, cn4s, 1, km)
    allocate(inflow(jm, km), zero(jm, km))
    zero = 0.0
    do k = 1, km
      inflow(:, k) = 5.0
    end do
    if (km >= 79) then
      do k = 79, km
        inflow(:, k) = inflow(:, 77)
      end do
    end if
    call check(les_gpu_upload(les_h, LES_FIELD_UIN, inflow, [1, 1, 0], [jm, km, 0]), 'upload uin')
    call check(les_gpu_upload(les_h, LES_FIELD_VIN, zero, [1, 1, 0], [jm, km, 0]), 'upload vin')
    call check(les_gpu_upload(les_h, LES_FIELD_WIN, zero, [1, 1, 0], [jm, km, 0]), 'upload win')
    deallocate(inflow, zero)
    call check(les_gpu_commit_setup(les_h), 'commit_setup')
  end subroutine

  ! One whole time step on the device (velnw .. press, main.f95:260-296).
  subroutine run_LES_gpu(n, nmax)
    integer, intent(in) :: n, nmax
    call check(les_gpu_step(les_h, int(n, c_int), int(nmax, c_int)), 'step')
  end subroutine

  ! Copy the device state back into the host arrays (before output, averaging or a
  ! restart write: the routines of main.f95:311-327 read the host arrays).
  subroutine sync_LES_gpu(u, v, w, p, usum, vsum, wsum, fold, gold, hold, im, jm, km)
    integer, intent(in) :: im, jm, km
    real(4), intent(inout) :: u(0:im+1, -1:jm+1, 0:km+1), v(0:im+1, -1:jm+1, 0:km+1)
    real(4), intent(inout) :: w(0:im+1, -1:jm+1, -1:km+1), p(0:im+2, 0:jm+2, 0:km+1)
    real(4), intent(inout) :: usum(0:im, 0:jm, 0:km), vsum(0:im, 0:jm, 0:km), wsum(0:im, 0:jm, 0:km)
    real(4), intent(inout) :: fold(im, jm, km), gold(im, jm, km), hold(im, jm, km)
    ! the steps since the last sync finished (a kernel's bounded wait that gave up is
    ! reported here and stops the run, like any other failed call)
    call check(les_gpu_sync(les_h), 'sync')
    call get3(LES_FIELD_U, u, 0, im + 1, -1, jm + 1, 0, km + 1)
    call get3(LES_FIELD_V, v, 0, im + 1, -1, jm + 1, 0, km + 1)
    call get3(LES_FIELD_W, w, 0, im + 1, -1, jm + 1, -1, km + 1)
    call get3(LES_FIELD_P, p, 0, im + 2, 0, jm + 2, 0, km + 1)
    call get3(LES_FIELD_USUM, usum, 0, im, 0, jm, 0, km)
    call get3(LES_FIELD_VSUM, vsum, 0, im, 0, jm, 0, km)
    call get3(LES_FIELD_WSUM, wsum, 0, im, 0, jm, 0, km)
    call get3(LES_FIELD_FOLD, fold, 1, im, 1, jm, 1, km)
    call get3(LES_FIELD_GOLD, gold, 1, im, 1, jm, 1, km)
    call get3(LES_FIELD_HOLD, hold, 1, im, 1, jm, 1, km)
  end subroutine

  subroutine finalise_LES_gpu()
    integer(c_int) :: rc
    if (c_associated(les_h)) rc = les_gpu_destroy(les_h)
    les_h = c_null_ptr
  end subroutine

  ! ---- per-subroutine drop-ins: the reference's argument lists (host arrays unused)
  subroutine velnw(km, jm, im, p, ro, dxs, u, dt, f, dys, v, g, dzs, w, h)
    integer, intent(in) :: km, jm, im
    real(4), intent(in) :: ro, dt
    real(4) :: p(*), dxs(*), u(*), f(*), dys(*), v(*), g(*), dzs(*), w(*), h(*)
    call check(les_gpu_velnw(les_h), 'velnw')
  end subroutine

  subroutine bondv1(jm, u, z2, dzn, v, w, km, n, im, dt, dxs)
    integer, intent(in) :: jm, km, n, im
    real(4), intent(in) :: dt
    real(4) :: u(*), z2(*), dzn(*), v(*), w(*), dxs(*)
    call check(les_gpu_bondv1(les_h, int(n, c_int)), 'bondv1')
  end subroutine

  subroutine velfg(km, jm, im, dx1, cov1, cov2, cov3, dfu1, diu1, diu2, dy1, diu3, dzn, vn, f, cov4, &
                   cov5, cov6, dfv1, diu4, diu5, diu6, g, cov7, cov8, cov9, dfw1, diu7, diu8, diu9, dzs, h, &
                   nou1, u, nou5, v, nou9, w, nou2, nou3, nou4, nou6, nou7, nou8, uspd, vspd)
    integer, intent(in) :: km, jm, im
    real(4), intent(in) :: vn
    real(4) :: dx1(*), cov1(*), cov2(*), cov3(*), dfu1(*), diu1(*), diu2(*), dy1(*), diu3(*), dzn(*), f(*)
    real(4) :: cov4(*), cov5(*), cov6(*), dfv1(*), diu4(*), diu5(*), diu6(*), g(*), cov7(*), cov8(*)
    real(4) :: cov9(*), dfw1(*), diu7(*), diu8(*), diu9(*), dzs(*), h(*), nou1(*), u(*), nou5(*), v(*)
    real(4) :: nou9(*), w(*), nou2(*), nou3(*), nou4(*), nou6(*), nou7(*), nou8(*), uspd(*), vspd(*)
    call check(les_gpu_velfg(les_h), 'velfg')
  end subroutine

  subroutine feedbf(km, jm, im, usum, u, bmask1, vsum, v, cmask1, wsum, w, dmask1, alpha, dt, beta, &
                    fx, fy, fz, f, g, h)
    integer, intent(in) :: km, jm, im
    real(4), intent(in) :: alpha, dt, beta
    real(4) :: usum(*), u(*), bmask1(*), vsum(*), v(*), cmask1(*), wsum(*), w(*), dmask1(*)
    real(4) :: fx(*), fy(*), fz(*), f(*), g(*), h(*)
    call check(les_gpu_feedbf(les_h), 'feedbf')
  end subroutine

  subroutine les(km, delx1, dx1, dy1, dzn, jm, im, diu1, diu2, diu3, diu4, diu5, diu6, diu7, diu8, diu9, &
                 sm, f, g, h, uspd, vspd, dxs, dys)
    integer, intent(in) :: km, jm, im
    real(4) :: delx1(*), dx1(*), dy1(*), dzn(*), diu1(*), diu2(*), diu3(*), diu4(*), diu5(*), diu6(*)
    real(4) :: diu7(*), diu8(*), diu9(*), sm(*), f(*), g(*), h(*), uspd(*), vspd(*), dxs(*), dys(*)
    call check(les_gpu_les(les_h), 'les')
  end subroutine

  ! adam writes data21 (fold, gold, hold, fghold) when mod(n,1000) == 0 or n == nmax
  ! (adam.f95:20-27), from the device state, big-endian like the reference's build.
  subroutine adam(n, nmax, data21, fold, im, jm, km, gold, hold, fghold, f, g, h)
    integer, intent(in) :: n, nmax, im, jm, km
    character(len=*) :: data21
    real(4) :: fold(*), gold(*), hold(*), fghold(*), f(*), g(*), h(*)
    call check(les_gpu_adam(les_h), 'adam')
#if !defined(NO_IO) && !defined(MPI)
    if (mod(n, 1000) == 0 .or. n == nmax) then
      call check(les_gpu_write_data21(les_h, trim(data21)//c_null_char, 0_c_int), 'adam: data21')
    end if
#endif
  end subroutine

  subroutine press(km, jm, im, rhs, u, dx1, v, dy1, w, dzn, f, g, h, dt, cn1, cn2l, p, cn2s, cn3l, cn3s, &
                   cn4l, cn4s, n, nmax, data20, usum, vsum, wsum)
    integer, intent(in) :: km, jm, im, n, nmax
    real(4), intent(in) :: dt
    character(len=*) :: data20
    real(4) :: rhs(*), u(*), dx1(*), v(*), dy1(*), w(*), dzn(*), f(*), g(*), h(*), cn1(*), cn2l(*)
    real(4) :: p(*), cn2s(*), cn3l(*), cn3s(*), cn4l(*), cn4s(*), usum(*), vsum(*), wsum(*)
    call check(les_gpu_press(les_h, int(n, c_int), int(nmax, c_int)), 'press')
    ! press.f95:197-216: data20 (u, v, w, p, usum, vsum, wsum) every 1000 steps and at nmax
#if !defined(NO_IO) && !defined(MPI)
    if (mod(n, 1000) == 0 .or. n == nmax) then
      call check(les_gpu_write_data20(les_h, trim(data20)//c_null_char, 0_c_int), 'press: data20')
    end if
#endif
  end subroutine

  ! aveflow of aveflow.f95:5 (called after every step, main.f95:320): the averages stay on
  ! the device; at n == nmax data10 and data11 are written from them (aveflow.f95:209-344).
  subroutine aveflow(n, n1, km, jm, im, aveu, avev, avew, avep, avel, aveuu, avevv, aveww, &
                     avesm, avesmsm, uwfx, avesu, avesv, avesw, avesuu, avesvv, avesww, u, v, w, p, sm, &
                     nmax, uwfxs, data10, time, data11, data13, data14, amask1)
    integer, intent(in) :: n, n1, km, jm, im, nmax
    real, intent(in) :: time
    character(len=*) :: data10, data11, data13, data14
    real(4) :: aveu(*), avev(*), avew(*), avep(*), avel(*), aveuu(*), avevv(*), aveww(*)
    real(4) :: avesm(*), avesmsm(*), uwfx(*), avesu(*), avesv(*), avesw(*), avesuu(*), avesvv(*)
    real(4) :: avesww(*), u(*), v(*), w(*), p(*), sm(*), uwfxs(*), amask1(*)
    call check(les_gpu_aveflow(les_h, int(n, c_int), int(n1, c_int), int(nmax, c_int)), 'aveflow')
    if (n == nmax) then
      call check(les_gpu_write_data10(les_h, trim(data10)//c_null_char, 0_c_int), 'aveflow: data10')
      call check(les_gpu_write_data11(les_h, trim(data11)//c_null_char, 0_c_int), 'aveflow: data11')
    end if
  end subroutine

  ! ifdata_out of anime.f95:326 (called after every step, main.f95:318): data30NNNNNN.dat
  ! and data31NNNNNN.dat in the working directory at n == n1-1 and n == nmax.
  subroutine ifdata_out(n, n0, n1, nmax, time, km, jm, im, u, w, v, p, usum, vsum, wsum, f, g, h, &
                        fold, gold, hold)
    integer, intent(in) :: n, n0, n1, nmax, km, jm, im
    real, intent(in) :: time
    real(4) :: u(*), w(*), v(*), p(*), usum(*), vsum(*), wsum(*), f(*), g(*), h(*)
    real(4) :: fold(*), gold(*), hold(*)
    integer(c_int) :: written
    call check(les_gpu_ifdata_out(les_h, '.'//c_null_char, int(n, c_int), int(n1, c_int), &
                                  int(nmax, c_int), real(time, c_float), 0_c_int, written), 'ifdata_out')
  end subroutine

  ! The restart read of ifdata (ifdata.f95:252-480, ical == 1), into the device state:
  ! n and time from data30, the interiors of the 13 state fields from data30/data31.
  ! The reference reads 'data30048000.dat' and 'data31048000.dat'.
  subroutine read_restart_LES_gpu(data30, data31, n, time)
    character(len=*), intent(in) :: data30, data31
    integer, intent(out) :: n
    real, intent(out) :: time
    integer(c_int) :: nc
    real(c_float) :: tc
    call check(les_gpu_read_restart(les_h, trim(data30)//c_null_char, trim(data31)//c_null_char, nc, tc), &
               'read_restart')
    n = nc
    time = tc
  end subroutine

  subroutine boundp1(km, jm, p, im)
    integer, intent(in) :: km, jm, im
    real(4) :: p(*)
    call check(les_gpu_boundp1(les_h), 'boundp1')
  end subroutine

  subroutine boundp2(jm, im, p, km)
    integer, intent(in) :: jm, im, km
    real(4) :: p(*)
    call check(les_gpu_boundp2(les_h), 'boundp2')
  end subroutine

end module module_LES_gpu
