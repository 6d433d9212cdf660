! bgk_gpu.F90 -- ISO_C_BINDING interface of BGK2D's Fortran driver to libbgk2d_gb300.so.
!
! To be compiled with the reference's SRC/ (it uses `module storage` for the population
! arrays) and linked with -lbgk2d_gb300.  Every interface below binds one entry point of
! include/bgk2d_gb300.h; the derived type bgk_case_desc mirrors the C struct of the same name
! field by field (interoperable kinds, same order), so gfortran lays it out as the C compiler
! does.  tests/test_fortran_binding.py checks the names, argument lists, constants and field
! offsets of this file against the header on every CPU test run.
!
! The time loop that replaces SRC/bgk2d.F90:92-113 is in bgk_gpu_loop.F90.
module bgk_gpu
  use iso_c_binding
  implicit none

  ! status codes
  integer(c_int), parameter :: BGK_OK = 0, BGK_E_INVALID = 1, BGK_E_NOMEM = 2, BGK_E_CUDA = 3, &
                               BGK_E_UNSUPPORTED = 4, BGK_E_NUMERIC = 5, BGK_E_TIMEOUT = 7, &
                               BGK_E_TOOLARGE = 9
  ! storage and arithmetic kinds (SRC/precision.F90: mystorage / mykind)
  integer(c_int), parameter :: BGK_STORE_F32 = 0, BGK_STORE_F64 = 1, BGK_STORE_F16 = 2, BGK_STORE_BF16 = 3
  integer(c_int), parameter :: BGK_COMPUTE_F32 = 0, BGK_COMPUTE_F64 = 1
  integer(c_int), parameter :: BGK_SCHEME_PINGPONG = 0, BGK_SCHEME_AA = 1, BGK_SCHEME_ORIGINAL = 2
  ! the compile-time case flags of SRC/Makefile
  integer(c_int), parameter :: BGK_CASE_LDC = 0, BGK_CASE_TGV = 1, BGK_CASE_POF = 2, &
                               BGK_CASE_VKS = 3, BGK_CASE_COU = 4, BGK_CASE_BFS = 5, &
                               BGK_CASE_MYV = 6
  integer(c_int), parameter :: BGK_OBS_NONE = 0, BGK_OBS_CIRCLE = 1, BGK_OBS_SQUARE = 2, &
                               BGK_OBS_HALF_CIRCLE = 3
  integer(c_int), parameter :: BGK_INIT_REST = 0, BGK_INIT_TGV_REF = 1
  integer(c_int), parameter :: BGK_DIAGNO_ALL = 0, BGK_DIAGNO_FLUID = 1, BGK_DIAGNO_REFERENCE = 2

  ! mirror of bgk_case_desc; wall_u(2,4) is the C array wall_u[4][2]
  type, bind(c) :: bgk_case_desc
     integer(c_int)  :: lx, ly, ipad, jpad
     integer(c_int)  :: storage, compute, scheme, tcase
     integer(c_int)  :: faces(4)
     real(c_double)  :: wall_u(2,4)
     real(c_double)  :: svisc, u0, omega, u_inflow
     integer(c_int)  :: inflow_profile, obstacle, radius, obs_icoord, obs_jcoord
     type(c_ptr)     :: obs_mask
     integer(c_int)  :: init_v
     real(c_double)  :: tgv_u0
     integer(c_int)  :: device
     integer(c_int)  :: les
     real(c_double)  :: cte_s
     integer(c_int)  :: trick1
     integer(c_int)  :: noshift
     integer(c_int)  :: force_y
     integer(c_int)  :: reserved(1)
  end type bgk_case_desc

  interface
     integer(c_int) function bgk_default_desc(d) bind(c, name="bgk_default_desc")
       import :: c_int, bgk_case_desc
       type(bgk_case_desc), intent(out) :: d
     end function bgk_default_desc

     integer(c_int) function bgk_create(d, h) bind(c, name="bgk_create")
       import :: c_int, c_ptr, bgk_case_desc
       type(bgk_case_desc), intent(in) :: d
       type(c_ptr), intent(out) :: h
     end function bgk_create

     integer(c_int) function bgk_destroy(h) bind(c, name="bgk_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function bgk_destroy

     integer(c_int) function bgk_upload(h, pops, ld) bind(c, name="bgk_upload")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h
       type(c_ptr), intent(in) :: pops(9)
       integer(c_int64_t), value :: ld
     end function bgk_upload

     integer(c_int) function bgk_download(h, pops, ld) bind(c, name="bgk_download")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h
       type(c_ptr), intent(in) :: pops(9)
       integer(c_int64_t), value :: ld
     end function bgk_download

     integer(c_int) function bgk_advance_host(h, pin, pout, ld, nsteps) bind(c, name="bgk_advance_host")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h
       type(c_ptr), intent(in) :: pin(9), pout(9)
       integer(c_int64_t), value :: ld
       integer(c_int), value :: nsteps
     end function bgk_advance_host

     integer(c_int) function bgk_boundaries(h) bind(c, name="bgk_boundaries")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function bgk_boundaries

     integer(c_int) function bgk_propagation(h) bind(c, name="bgk_propagation")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function bgk_propagation

     integer(c_int) function bgk_collision(h, itime) bind(c, name="bgk_collision")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: itime
     end function bgk_collision

     integer(c_int) function bgk_step(h, nsteps) bind(c, name="bgk_step")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: nsteps
     end function bgk_step

     integer(c_int) function bgk_sync(h) bind(c, name="bgk_sync")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function bgk_sync

     integer(c_int) function bgk_diagno(h, mode, out) bind(c, name="bgk_diagno")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: mode
       real(c_double), intent(out) :: out(4)
     end function bgk_diagno

     integer(c_int) function bgk_draglift(h, out) bind(c, name="bgk_draglift")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), intent(out) :: out(2)
     end function bgk_draglift

     integer(c_int) function bgk_draglift_reference(h, out) bind(c, name="bgk_draglift_reference")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), intent(out) :: out(2)
     end function bgk_draglift_reference

     integer(c_int) function bgk_residual(h, out) bind(c, name="bgk_residual")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), intent(out) :: out
     end function bgk_residual

     ! the profile readers of prof_i / prof_j / varm / probe computed on the device, for a loop
     ! that writes those files without downloading the populations
     integer(c_int) function bgk_prof_i(h, jcoord, u, v, den) bind(c, name="bgk_prof_i")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: jcoord
       real(c_double), intent(out) :: u(*), v(*), den(*)
     end function bgk_prof_i

     integer(c_int) function bgk_prof_j(h, icoord, u, v, den) bind(c, name="bgk_prof_j")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: icoord
       real(c_double), intent(out) :: u(*), v(*), den(*)
     end function bgk_prof_j

     integer(c_int) function bgk_varm(h, u, w, den) bind(c, name="bgk_varm")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), intent(out) :: u(*), w(*), den(*)
     end function bgk_varm

     integer(c_int) function bgk_probe(h, i0, j0, out) bind(c, name="bgk_probe")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: i0, j0
       real(c_double), intent(out) :: out(3)
     end function bgk_probe

     integer(c_int) function bgk_vtk_fields(h, u, w, rho, vort, stream) bind(c, name="bgk_vtk_fields")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: h
       real(c_float), intent(out) :: u(*), w(*), rho(*), vort(*), stream(*)
     end function bgk_vtk_fields

     integer(c_int) function bgk_diagno_noalloc(pops, ld, lx, ly, storage, out) bind(c, name="bgk_diagno_noalloc")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), intent(in) :: pops(9)
       integer(c_int64_t), value :: ld
       integer(c_int), value :: lx, ly, storage
       real(c_double), intent(out) :: out(4)
     end function bgk_diagno_noalloc

     integer(c_int) function bgk_last_error(h, buf, n) bind(c, name="bgk_last_error")
       import :: c_int, c_ptr, c_char, c_size_t
       type(c_ptr), value :: h
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_size_t), value :: n
     end function bgk_last_error
  end interface

  ! the case this process runs (one domain per process, as the reference)
  type(c_ptr) :: bgk_h = c_null_ptr

contains

  ! host addresses of the nine module arrays, in the reference's direction order.  Under FUSED
  ! they are pointers already; under ORIGINAL their declarations need the `target` attribute.
  subroutine bgk_pops(p)
    use storage
    type(c_ptr), intent(out) :: p(9)
    p(1) = c_loc(a01(0,0)); p(2) = c_loc(a03(0,0)); p(3) = c_loc(a05(0,0))
    p(4) = c_loc(a08(0,0)); p(5) = c_loc(a10(0,0)); p(6) = c_loc(a12(0,0))
    p(7) = c_loc(a14(0,0)); p(8) = c_loc(a17(0,0)); p(9) = c_loc(a19(0,0))
  end subroutine bgk_pops

  ! stop with the library's message when a call fails (the reference reports errors by `stop`)
  subroutine bgk_check(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    character(kind=c_char) :: buf(256)
    integer(c_int) :: ignored
    integer :: k
    if (rc /= BGK_OK) then
       buf = c_null_char
       if (c_associated(bgk_h)) ignored = bgk_last_error(bgk_h, buf, int(size(buf), c_size_t))
       write(6,*) "ERROR: ", what, " returned ", rc, ": ", (buf(k), k = 1, size(buf))
       stop
    endif
  end subroutine bgk_check
end module bgk_gpu
