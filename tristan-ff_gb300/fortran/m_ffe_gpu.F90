! m_ffe_gpu — iso_c_binding bindings of libffe_gb300 (include/ffe.h) and
! wrappers with the names of the reference's field-solver procedures, so that
! src/tristanmainloop.F90 and the user files keep their calls.
!
! Written against include/ffe.h; not compiled here (the build image has no
! Fortran compiler).  Link with -lffe_gb300 -lcudart.
!
! Use: after initializeFields and userInitialize (the fields are on the host),
! call ffeInitialize(setup_id, params); from then on the fields live on the
! GPU.  writeOutput calls ffeOutput(istep, nodes) for its twelve datasets.
module m_ffe_gpu
  use iso_c_binding
  use m_globalnamespace, only: CC
  use m_domain
  use m_fields
  implicit none

  integer(c_int32_t), parameter :: FFE_EX = 0, FFE_EY = 1, FFE_EZ = 2, FFE_BX = 3, FFE_BY = 4, FFE_BZ = 5
  integer(c_int32_t), parameter :: FFE_B0X = 6, FFE_B0Y = 7, FFE_B0Z = 8

  type, bind(C) :: ffe_grid_desc
    integer(c_int32_t) :: sx, sy, sz, x0, y0, z0, gsx, gsy, gsz
    integer(c_int32_t) :: boundary(3), absorb_buff, precision, setup, path, flags, reserved
    real(c_double)     :: cc
    real(c_double)     :: params(8)
    type(c_ptr)        :: stream
  end type

  interface
    integer(c_int) function ffe_desc_default(d, sx, sy, sz) bind(C, name="ffe_desc_default")
      import; type(ffe_grid_desc) :: d; integer(c_int32_t), value :: sx, sy, sz
    end function
    integer(c_int) function ffe_create(h, d) bind(C, name="ffe_create")
      import; type(c_ptr) :: h; type(ffe_grid_desc) :: d
    end function
    integer(c_int) function ffe_destroy(h) bind(C, name="ffe_destroy")
      import; type(c_ptr), value :: h
    end function
    integer(c_int) function ffe_last_error(h, buf, n) bind(C, name="ffe_last_error")
      import; type(c_ptr), value :: h; character(kind=c_char) :: buf(*); integer(c_size_t), value :: n
    end function
    integer(c_int) function ffe_upload(h, f, a, n) bind(C, name="ffe_upload")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: f
      type(c_ptr), value :: a; integer(c_size_t), value :: n
    end function
    integer(c_int) function ffe_download(h, f, a, n) bind(C, name="ffe_download")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: f
      type(c_ptr), value :: a; integer(c_size_t), value :: n
    end function
    integer(c_int) function ffe_init_rk_step(h) bind(C, name="ffe_init_rk_step")
      import; type(c_ptr), value :: h
    end function
    integer(c_int) function ffe_rk3_stage(h, c1, c2, c3) bind(C, name="ffe_rk3_stage")
      import; type(c_ptr), value :: h; real(c_double), value :: c1, c2, c3
    end function
    integer(c_int) function ffe_clean_epar(h) bind(C, name="ffe_clean_epar")
      import; type(c_ptr), value :: h
    end function
    integer(c_int) function ffe_exchange_fields(h, b0) bind(C, name="ffe_exchange_fields")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: b0
    end function
    integer(c_int) function ffe_user_bc(h, step) bind(C, name="ffe_user_bc")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: step
    end function
    integer(c_int) function ffe_step(h, n, step0) bind(C, name="ffe_step")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: n, step0
    end function
    integer(c_int) function ffe_synchronize(h) bind(C, name="ffe_synchronize")
      import; type(c_ptr), value :: h
    end function
    integer(c_int) function ffe_output_dims(h, istep, dims) bind(C, name="ffe_output_dims")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: istep; integer(c_int32_t) :: dims(3)
    end function
    integer(c_int) function ffe_output(h, istep, buf, n) bind(C, name="ffe_output")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: istep
      type(c_ptr), value :: buf; integer(c_size_t), value :: n
    end function
  end interface

  type(c_ptr) :: ffe_h = c_null_ptr

contains

  subroutine ffeCheck(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    character(kind=c_char) :: buf(256)
    integer(c_int) :: st
    integer :: i
    if (rc .eq. 0) return
    st = ffe_last_error(ffe_h, buf, int(256, c_size_t))
    write (*, '(A, A, I0, A)', advance='no') what, ': status ', rc, ': '
    do i = 1, 256
      if (buf(i) .eq. c_null_char) exit
      write (*, '(A)', advance='no') buf(i)
    end do
    write (*, *)
    stop
  end subroutine ffeCheck

  ! after initializeFields and userInitialize: descriptor, device state, fields
  subroutine ffeInitialize(setup_id, params)
    integer, intent(in) :: setup_id
    real(c_double), intent(in) :: params(8)
    type(ffe_grid_desc) :: d
    call ffeCheck(ffe_desc_default(d, int(this_meshblock % ptr % sx, c_int32_t), &
                                   int(this_meshblock % ptr % sy, c_int32_t), &
                                   int(this_meshblock % ptr % sz, c_int32_t)), "ffe_desc_default")
    d % x0 = this_meshblock % ptr % x0; d % y0 = this_meshblock % ptr % y0; d % z0 = this_meshblock % ptr % z0
    d % gsx = global_mesh % sx; d % gsy = global_mesh % sy; d % gsz = global_mesh % sz
    d % boundary = (/boundary_x, boundary_y, boundary_z/)
    d % absorb_buff = absorb_buff
    d % precision = merge(0, 1, kind(ex) .eq. 8)        ! FFE_FP64 for a -fdefault-real-8 build
    d % setup = setup_id
    d % params = params
    d % cc = CC
    call ffeCheck(ffe_create(ffe_h, d), "ffe_create")
    call ffePut(FFE_EX, ex); call ffePut(FFE_EY, ey); call ffePut(FFE_EZ, ez)
    call ffePut(FFE_BX, bx); call ffePut(FFE_BY, by); call ffePut(FFE_BZ, bz)
    call ffePut(FFE_B0X, b0x); call ffePut(FFE_B0Y, b0y); call ffePut(FFE_B0Z, b0z)
  end subroutine ffeInitialize

  ! c_loc needs a contiguous array: the reference's field arrays are whole
  ! allocatable arrays, and the contiguous attribute (Fortran 2008) makes the
  ! compiler pass them (or a contiguous copy of any other actual) as such
  subroutine ffePut(f, a)
    integer(c_int32_t), intent(in) :: f
    real, target, contiguous, intent(in) :: a(:, :, :)
    call ffeCheck(ffe_upload(ffe_h, f, c_loc(a), int(size(a), c_size_t)), "ffe_upload")
  end subroutine ffePut

  subroutine ffeGet(f, a)
    integer(c_int32_t), intent(in) :: f
    real, target, contiguous, intent(inout) :: a(:, :, :)
    call ffeCheck(ffe_download(ffe_h, f, c_loc(a), int(size(a), c_size_t)), "ffe_download")
  end subroutine ffeGet

  ! the reference's procedure names (src/algorithms/field_solver.F90)
  subroutine initRKstep()
    call ffeCheck(ffe_init_rk_step(ffe_h), "initRKstep")
  end subroutine initRKstep

  subroutine rk3Step(c1, c2, c3)
    real, intent(in) :: c1, c2, c3
    call ffeCheck(ffe_rk3_stage(ffe_h, real(c1, c_double), real(c2, c_double), real(c3, c_double)), "rk3Step")
  end subroutine rk3Step

  subroutine cleanEpar()
    call ffeCheck(ffe_clean_epar(ffe_h), "cleanEpar")
  end subroutine cleanEpar

  subroutine exchangeFields(exchangeB0)               ! one meshblock per GPU: on-device ghost fill
    logical, optional, intent(in) :: exchangeB0
    integer(c_int32_t) :: b0
    b0 = 0
    if (present(exchangeB0)) then
      if (exchangeB0) b0 = 1
    end if
    call ffeCheck(ffe_exchange_fields(ffe_h, b0), "exchangeFields")
  end subroutine exchangeFields

  subroutine userFieldBoundaryConditions(step)        ! the device version of the setup's BC
    integer, optional, intent(in) :: step
    integer(c_int32_t) :: s
    s = 0
    if (present(step)) s = step
    call ffeCheck(ffe_user_bc(ffe_h, s), "userFieldBoundaryConditions")
  end subroutine userFieldBoundaryConditions

  ! the whole main-loop body of tristanmainloop.F90:50-84 for one timestep
  subroutine ffeStep(timestep)
    integer, intent(in) :: timestep
    call ffeCheck(ffe_step(ffe_h, 1_c_int32_t, int(timestep, c_int32_t)), "ffe_step")
  end subroutine ffeStep

  ! writeOutput's twelve node datasets (ex ey ez bx by bz var1 var2 var3 xx yy zz)
  subroutine ffeOutput(istep, nodes)
    integer, intent(in) :: istep
    real, allocatable, target, intent(out) :: nodes(:, :, :, :)
    integer(c_int32_t) :: dims(3)
    call ffeCheck(ffe_output_dims(ffe_h, int(istep, c_int32_t), dims), "ffe_output_dims")
    allocate (nodes(0:dims(1) - 1, 0:dims(2) - 1, 0:dims(3) - 1, 12))
    call ffeCheck(ffe_output(ffe_h, int(istep, c_int32_t), c_loc(nodes), int(size(nodes), c_size_t)), "ffe_output")
  end subroutine ffeOutput

  subroutine ffeFinalize()
    integer(c_int) :: rc
    rc = ffe_destroy(ffe_h)
    ffe_h = c_null_ptr
  end subroutine ffeFinalize
end module m_ffe_gpu
