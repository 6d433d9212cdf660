! bgk_gpu_loop.F90 -- BGK2D's time loop on libbgk2d_gb300.so.
!
! Replaces the loop of SRC/bgk2d.F90:92-113, which calls boundaries, propagation, collision and
! diagnostic once per step, in a build whose populations live on the GPU behind the library.
! The driver keeps everything else: `initialize` still fills the module arrays (init or
! restore_raw), and `diagnostic`, `profile` and the final diagno/varm/prof calls still run on
! the host arrays.  In SRC/bgk2d.F90:
!   - after `call initialize(...)`:           call bgk_gpu_start(BGK_STORE_F32, BGK_COMPUTE_F32, BGK_CASE_LDC)
!     (the storage/compute kinds of the SINGLE, DOUBLE or MIXED2 build, and its case flag);
!   - in place of the `do itime=itstart+1,itfin ... enddo` loop:
!                                             call bgk_gpu_time_loop(itstart, itfin, ivtim, icheck, itsave, isignal)
!   - before `call finalize(...)`:            call bgk_gpu_stop()
! and add bgk_gpu.F90 and this file to the Makefile's object list, linking -lbgk2d_gb300.
module bgk_gpu_loop
  use bgk_gpu
  implicit none

contains

  ! create the device case from the scalars that initialize has set, and upload the host state
  subroutine bgk_gpu_start(storage_kind, compute_kind, tcase)
    use storage
    integer(c_int), intent(in) :: storage_kind, compute_kind, tcase
    type(bgk_case_desc) :: d
    type(c_ptr) :: p(9)
    call bgk_check(bgk_default_desc(d), "bgk_default_desc")
    d%lx = l
    d%ly = m
    d%ipad = ipad
    d%jpad = jpad
    d%storage = storage_kind
    d%compute = compute_kind
    d%tcase = tcase
    d%svisc = svisc
    d%u0 = u0 + u00          ! build_bcond moved a lid speed from u0 to u00; the library splits it again
    d%radius = radius
    d%init_v = BGK_INIT_REST ! the populations come from the host arrays, uploaded next
    call bgk_check(bgk_create(d, bgk_h), "bgk_create")
    call bgk_pops(p)
    call bgk_check(bgk_upload(bgk_h, p, int(l + 2 + ipad, c_int64_t)), "bgk_upload")
  end subroutine bgk_gpu_start

  ! first step after itime at which `diagnostic` or `profile` does something (a multiple of
  ! ivtim, icheck, itsave or isignal), or itfin
  integer function bgk_gpu_next_stop(itime, itfin, ivtim, icheck, itsave, isignal)
    integer, intent(in) :: itime, itfin, ivtim, icheck, itsave, isignal
    bgk_gpu_next_stop = min(itfin, next_multiple(ivtim), next_multiple(icheck), next_multiple(itsave), &
                            next_multiple(isignal))
  contains
    integer function next_multiple(every)
      integer, intent(in) :: every
      next_multiple = (itime / every + 1) * every
    end function next_multiple
  end function bgk_gpu_next_stop

  ! the time loop: the steps between two diagnostic stops run on the GPU in one call (replayed
  ! from CUDA graphs); the host arrays are refreshed only where `diagnostic` reads them, and at
  ! the end for the final diagno/varm/prof calls.  `diagnostic` acts only at multiples of ivtim,
  ! icheck and itsave (SRC/diagnostic.F90), so calling it at the stops alone changes no output.
  subroutine bgk_gpu_time_loop(itstart, itfin, ivtim, icheck, itsave, isignal)
    use storage
    integer, intent(in) :: itstart, itfin, ivtim, icheck, itsave, isignal
    type(c_ptr) :: p(9)
    integer :: itime, stop_at
    integer(c_int64_t) :: ld
    ld = int(l + 2 + ipad, c_int64_t)
    call bgk_pops(p)
    itime = itstart
    do while (itime < itfin)
       stop_at = bgk_gpu_next_stop(itime, itfin, ivtim, icheck, itsave, isignal)
       call bgk_check(bgk_step(bgk_h, int(stop_at - itime, c_int)), "bgk_step")
       itime = stop_at
       if (mod(itime, ivtim) == 0 .or. mod(itime, icheck) == 0 .or. mod(itime, itsave) == 0 &
           .or. itime == itfin) then
          call bgk_check(bgk_download(bgk_h, p, ld), "bgk_download")   ! synchronises
       end if
       call diagnostic(itime, ivtim, icheck, itsave)
       if (mod(itime, isignal) == 0) then
          call bgk_check(bgk_sync(bgk_h), "bgk_sync")                  ! timings cover the steps
          if (myrank == 0) call profile(itime, itfin, isignal)
       end if
    end do
  end subroutine bgk_gpu_time_loop

  subroutine bgk_gpu_stop()
    call bgk_check(bgk_destroy(bgk_h), "bgk_destroy")
    bgk_h = c_null_ptr
  end subroutine bgk_gpu_stop
end module bgk_gpu_loop
