! wpic_shim2d.f90 -- drop-in replacements for WumingPIC's 2D hot-path modules
! (particle, field, sort, boundary_periodic, boundary_reconnection, boundary_shock, mom_calc)
! that forward to the GB300 library
! through ISO_C_BINDING.  Link these objects instead of the corresponding objects
! of libwuming2d_common.a; the drivers ({2d}/proj/*/app.f90) stay unchanged.
!
! Coherence: the first particle__solv uploads the host state (up, uf, cumcnt;
! np2 = cumcnt(nxe+1,:,:)).  Afterwards the device state is authoritative and the
! host arrays are refreshed only where the drivers read them: on entry to
! mom_calc__accl (the diagnostic block: mom_calc__accl, mom_calc__nvt, bc__mom,
! io__mom and energy_history read up, uf, cumcnt and np2; np2 is handed back in
! mom_calc__nvt) and in the I/O routines io__ptcl, io__orb, io__mom and io__output,
! which this file's wuming2d module wraps (2d/proj/weibel/app.f90:108-125, 571).
! io__input marks the host state as the newer one, so the next call uploads it.
! Between those points no particle or field array crosses the host link.
! wpic_shim_set_sync(n) (n >= 1) refreshes the host arrays every n steps instead,
! for drivers that read them elsewhere; the shock driver, which edits the host state
! every step, gets n = 1 and an upload every step from boundary_shock__init.
! The environment variable WPIC_PRECISION chooses the arithmetic without a driver change:
! 'mixed' runs the mixed-precision step (particle__solv requests the push, field__fdtd_i runs
! the fused step, the boundary and sort calls find their work done), 'fp64_exact' the
! reference-order FP64 build, anything else FP64.
!
! The three boundary routines that field__fdtd_i receives as procedure arguments
! are accepted and ignored: the library applies the boundary of the kind chosen
! at init (periodic here).
module wpic_capi
  use iso_c_binding
  implicit none

  type, bind(C) :: wpic_params
     integer(c_int) :: ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye
     real(c_double) :: delx, delt, c, gfac
     real(c_double) :: q(2), r(2)
     integer(c_int) :: bc_kind, precision, device_cap
  end type wpic_params

  interface
     integer(c_int) function wpic_init_2d(ctx, p, stream) bind(C, name="wpic_init_2d")
       import :: c_int, c_ptr, wpic_params
       type(c_ptr), intent(out) :: ctx
       type(wpic_params), intent(in) :: p
       type(c_ptr), value :: stream
     end function wpic_init_2d
     integer(c_int) function wpic_put_particles(ctx, which, up, np2, cumcnt) bind(C, name="wpic_put_particles")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: which
       real(c_double), intent(in) :: up(*)
       integer(c_int), intent(in) :: np2(*), cumcnt(*)
     end function wpic_put_particles
     integer(c_int) function wpic_get_particles(ctx, which, up, np2, cumcnt) bind(C, name="wpic_get_particles")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: which
       real(c_double), intent(inout) :: up(*)
       integer(c_int), intent(inout) :: np2(*), cumcnt(*)
     end function wpic_get_particles
     integer(c_int) function wpic_put_fields(ctx, uf) bind(C, name="wpic_put_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: uf(*)
     end function wpic_put_fields
     integer(c_int) function wpic_get_fields(ctx, uf) bind(C, name="wpic_get_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: uf(*)
     end function wpic_get_fields
     integer(c_int) function wpic_mom_calc_nvt(ctx, from_gp) bind(C, name="wpic_mom_calc_nvt")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: from_gp
     end function wpic_mom_calc_nvt
     integer(c_int) function wpic_get_mom(ctx, mom) bind(C, name="wpic_get_mom")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: mom(*)
     end function wpic_get_mom
     integer(c_int) function wpic_set_window(ctx, nxs, nxe) bind(C, name="wpic_set_window")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: nxs, nxe
     end function wpic_set_window
     integer(c_int) function wpic_bc_injection(ctx, u0) bind(C, name="wpic_bc_injection")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: u0
     end function wpic_bc_injection
     integer(c_int) function wpic_mom_calc_accl(ctx) bind(C, name="wpic_mom_calc_accl")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic_mom_calc_accl
     integer(c_int) function wpic_bc_mom(ctx) bind(C, name="wpic_bc_mom")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic_bc_mom
     integer(c_int) function wpic_call(ctx) bind(C)
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic_call
  end interface

  ! one device context per process (one MPI rank holding the whole domain)
  type(c_ptr), save :: wpic_ctx = c_null_ptr
  type(wpic_params), save :: wpic_prm
  logical, save :: wpic_uploaded = .false.
  logical, save :: wpic_bc_set = .false.           ! a boundary module's __init chose the kind
  logical, save :: wpic_upload_each_step = .false. ! drivers that edit up/uf/cumcnt between steps
  integer, save :: wpic_win_s = -1, wpic_win_e = -1
  integer, save :: wpic_sync_every = 0, wpic_step_count = 0  ! 0: refresh at the read points only
  integer, save :: wpic_synced_at = -1      ! step count of the host arrays' last refresh
  integer(c_int), allocatable, save :: wpic_np2_dev(:,:), wpic_cc_dev(:,:,:)

  procedure(wpic_call), pointer :: p_solv => null(), p_fdtd => null(), p_bcx => null(), &
       p_bcy => null(), p_sort => null(), p_solv_vay => null()

contains

  ! The arithmetic of the context, chosen without a driver change by the environment variable
  ! WPIC_PRECISION: 'mixed' (WPIC_MIXED: the staged calls run the fused mixed step; the grid's
  ! nx and ny, and nz in 3D, must be multiples of the tile edge), 'fp64_exact' (the reference's
  ! operation order), anything else or unset: FP64.
  integer(c_int) function wpic_env_precision()
    character(len=32) :: val
    integer :: n, stat
    wpic_env_precision = 0
    call get_environment_variable('WPIC_PRECISION', val, n, stat)
    if (stat /= 0 .or. n < 1) return
    if (val(1:n) == 'mixed') wpic_env_precision = 2
    if (val(1:n) == 'fp64_exact') wpic_env_precision = 1
  end function wpic_env_precision

  subroutine wpic_check(st, where)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    if (st /= 0) then
       write(0,*) 'wumingpic_gb300: ', where, ' failed with status ', st
       stop
    endif
  end subroutine wpic_check

  ! The shock driver adds particles and sets upstream fields on the host between steps
  ! (inject, relocate: 2d/proj/shock/app.f90:615-852); with upload on, every particle__solv
  ! sends the host state to the device first.
  subroutine wpic_shim_set_upload(flag)
    logical, intent(in) :: flag
    wpic_upload_each_step = flag
  end subroutine wpic_shim_set_upload

  ! the active window nxs..nxe that the driver passes to every module call
  subroutine wpic_apply_window(nxs, nxe)
    integer, intent(in) :: nxs, nxe
    if (nxs /= wpic_win_s .or. nxe /= wpic_win_e) then
       call wpic_check(wpic_set_window(wpic_ctx, int(nxs, c_int), int(nxe, c_int)), 'window')
       wpic_win_s = nxs; wpic_win_e = nxe
    endif
  end subroutine wpic_apply_window

  ! up, uf and cumcnt to the device; cumcnt beyond the window (stale in the drivers) is
  ! completed with the row totals, which is what the library keeps there
  subroutine wpic_upload_state(up, uf, cumcnt, nxe)
    real(8), intent(in) :: up(*), uf(*)
    integer, intent(in) :: cumcnt(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer, intent(in) :: nxe
    integer(c_int) :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer(c_int) :: cc(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer :: i
    cc(:,:,:) = cumcnt(:,:,:)
    do i = nxe+2, wpic_prm%nxge+1
       cc(i,:,:) = cumcnt(nxe+1,:,:)
    enddo
    np2(:,:) = cumcnt(nxe+1,:,:)
    call wpic_check(wpic_put_particles(wpic_ctx, 0_c_int, up, np2, cc), 'put up')
    call wpic_check(wpic_put_fields(wpic_ctx, uf), 'put uf')
    wpic_uploaded = .true.
  end subroutine wpic_upload_state

  subroutine wpic_shim_set_sync(n)
    integer, intent(in) :: n
    wpic_sync_every = max(0, n)
  end subroutine wpic_shim_set_sync

  ! The host arrays brought up to date with the device (once per step): the sorted state up,
  ! uf, and, when present, np2 and cumcnt.  Before the first upload the host is the newer side
  ! and nothing is copied.
  subroutine wpic_sync_host(up, uf, np2, cumcnt)
    real(8), intent(inout) :: up(*), uf(*)
    integer, intent(inout), optional :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer, intent(inout), optional :: cumcnt(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    if (.not. wpic_uploaded) return
    if (.not. allocated(wpic_np2_dev)) then
       allocate(wpic_np2_dev(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp))
       allocate(wpic_cc_dev(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp))
    endif
    if (wpic_synced_at /= wpic_step_count) then
       call wpic_check(wpic_get_particles(wpic_ctx, 0_c_int, up, wpic_np2_dev, wpic_cc_dev), 'get up')
       call wpic_check(wpic_get_fields(wpic_ctx, uf), 'get uf')
       wpic_synced_at = wpic_step_count
    endif
    if (present(np2)) np2(:,:) = wpic_np2_dev(:,:)
    if (present(cumcnt)) cumcnt(:,:,:) = wpic_cc_dev(:,:,:)
  end subroutine wpic_sync_host

  ! uf alone brought up to date (io__mom receives uf only)
  subroutine wpic_sync_fields(uf)
    real(8), intent(inout) :: uf(*)
    if (.not. wpic_uploaded) return
    if (wpic_synced_at /= wpic_step_count) call wpic_check(wpic_get_fields(wpic_ctx, uf), 'get uf')
  end subroutine wpic_sync_fields

  ! np2 of the last refresh (mom_calc__nvt receives np2 after mom_calc__accl refreshed up)
  subroutine wpic_sync_np2(np2)
    integer, intent(inout) :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    if (wpic_uploaded .and. allocated(wpic_np2_dev) .and. wpic_synced_at == wpic_step_count) &
         np2(:,:) = wpic_np2_dev(:,:)
  end subroutine wpic_sync_np2

  subroutine wpic_bind_procedures()
    interface
       integer(c_int) function wpic_particle_solv(ctx) bind(C, name="wpic_particle_solv")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
       end function
       integer(c_int) function wpic_particle_solv_vay(ctx) bind(C, name="wpic_particle_solv_vay")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
       end function
       integer(c_int) function wpic_field_fdtd_i(ctx) bind(C, name="wpic_field_fdtd_i")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
       end function
       integer(c_int) function wpic_bc_particle_x(ctx) bind(C, name="wpic_bc_particle_x")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
       end function
       integer(c_int) function wpic_bc_particle_y(ctx) bind(C, name="wpic_bc_particle_y")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
       end function
       integer(c_int) function wpic_sort_bucket(ctx) bind(C, name="wpic_sort_bucket")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
       end function
    end interface
    p_solv => wpic_particle_solv
    p_solv_vay => wpic_particle_solv_vay
    p_fdtd => wpic_field_fdtd_i
    p_bcx => wpic_bc_particle_x
    p_bcy => wpic_bc_particle_y
    p_sort => wpic_sort_bucket
  end subroutine wpic_bind_procedures

  subroutine wpic_ensure_ctx()
    if (.not. c_associated(wpic_ctx)) then
       call wpic_check(wpic_init_2d(wpic_ctx, wpic_prm, c_null_ptr), 'wpic_init_2d')
       call wpic_bind_procedures()
    endif
  end subroutine wpic_ensure_ctx

end module wpic_capi


module particle
  use wpic_capi
  implicit none
  private
  public :: particle__init, particle__solv, particle__solv_vay
contains
  subroutine particle__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in, &
                            delx_in,delt_in,c_in,q_in,r_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
    real(8), intent(in) :: delx_in, delt_in, c_in, q_in(nsp_in), r_in(nsp_in)
    wpic_prm%ndim = ndim_in; wpic_prm%np = np_in; wpic_prm%nsp = nsp_in
    wpic_prm%nxgs = nxgs_in; wpic_prm%nxge = nxge_in; wpic_prm%nygs = nygs_in; wpic_prm%nyge = nyge_in
    wpic_prm%nys = nys_in; wpic_prm%nye = nye_in
    wpic_prm%delx = delx_in; wpic_prm%delt = delt_in; wpic_prm%c = c_in
    wpic_prm%q(1:nsp_in) = q_in; wpic_prm%r(1:nsp_in) = r_in
    if (.not. wpic_bc_set) wpic_prm%bc_kind = 0
    wpic_prm%precision = wpic_env_precision(); wpic_prm%device_cap = 0
  end subroutine particle__init

  subroutine particle__solv(gp,up,uf,cumcnt,nxs,nxe)
    integer, intent(in)  :: nxs, nxe
    integer, intent(in)  :: cumcnt(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    real(8), intent(in)  :: up(*), uf(*)
    real(8), intent(out) :: gp(*)
    call wpic_ensure_ctx()
    call wpic_apply_window(nxs, nxe)
    if (.not. wpic_uploaded .or. wpic_upload_each_step) call wpic_upload_state(up, uf, cumcnt, nxe)
    call wpic_check(p_solv(wpic_ctx), 'particle__solv')
  end subroutine particle__solv

  subroutine particle__solv_vay(gp,up,uf,cumcnt,nxs,nxe)
    integer, intent(in)  :: nxs, nxe
    integer, intent(in)  :: cumcnt(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    real(8), intent(in)  :: up(*), uf(*)
    real(8), intent(out) :: gp(*)
    call wpic_ensure_ctx()
    call wpic_apply_window(nxs, nxe)
    if (.not. wpic_uploaded .or. wpic_upload_each_step) call wpic_upload_state(up, uf, cumcnt, nxe)
    call wpic_check(p_solv_vay(wpic_ctx), 'particle__solv_vay')
  end subroutine particle__solv_vay
end module particle


module field
  use wpic_capi
  implicit none
  private
  public :: field__init, field__fdtd_i
contains
  subroutine field__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in, &
                         mnpr_in,ncomw_in,opsum_in,nerr_in,delx_in,delt_in,c_in,q_in,r_in,gfac_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
    integer, intent(in) :: mnpr_in, ncomw_in, opsum_in, nerr_in
    real(8), intent(in) :: delx_in, delt_in, c_in, q_in(nsp_in), r_in(nsp_in), gfac_in
    wpic_prm%gfac = gfac_in
  end subroutine field__init

  subroutine field__fdtd_i(uf,up,gp,cumcnt,nxs,nxe,set_boundary_dfield,set_boundary_curre,set_boundary_phi)
    integer, intent(in)    :: nxs, nxe
    integer, intent(in)    :: cumcnt(*)
    real(8), intent(in)    :: up(*), gp(*)
    real(8), intent(inout) :: uf(*)
    external :: set_boundary_dfield, set_boundary_curre, set_boundary_phi
    call wpic_apply_window(nxs, nxe)
    call wpic_check(p_fdtd(wpic_ctx), 'field__fdtd_i')
    if (wpic_sync_every > 0) then
       if (mod(wpic_step_count + 1, wpic_sync_every) == 0) &
            call wpic_check(wpic_get_fields(wpic_ctx, uf), 'get uf')
    endif
  end subroutine field__fdtd_i
end module field


module sort
  use wpic_capi
  implicit none
  private
  public :: sort__init, sort__bucket
contains
  subroutine sort__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
  end subroutine sort__init

  ! np2 is intent(in) in the reference; here it is refreshed together with the
  ! sorted state at the sync points, so it is declared intent(inout)
  subroutine sort__bucket(gp,up,cumcnt,np2,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    integer, intent(inout) :: np2(wpic_prm%nye-wpic_prm%nys+1, wpic_prm%nsp)
    integer, intent(inout) :: cumcnt(*)
    real(8), intent(in)    :: up(*)
    real(8), intent(inout) :: gp(*)
    integer(c_int) :: np2_dev(wpic_prm%nye-wpic_prm%nys+1, wpic_prm%nsp)
    call wpic_ensure_ctx()
    call wpic_apply_window(nxs, nxe)
    if (.not. wpic_uploaded) then
       ! the restart path (2d/proj/weibel/app.f90:351-352): io__input filled the host 'up' (this
       ! routine's up dummy) and np2; they are sorted on the device and handed back, and the next
       ! particle__solv uploads the whole host state
       np2_dev(:,:) = np2(:,:)
       ! (cumcnt is not read for the gp state; np2 stands in for it)
       call wpic_check(wpic_put_particles(wpic_ctx, 1_c_int, up, np2_dev, np2_dev), 'put gp')
       call wpic_check(p_sort(wpic_ctx), 'sort__bucket')
       call wpic_check(wpic_get_particles(wpic_ctx, 0_c_int, gp, np2_dev, cumcnt), 'get up')
       np2(:,:) = np2_dev(:,:)
       return
    endif
    call wpic_check(p_sort(wpic_ctx), 'sort__bucket')
    wpic_step_count = wpic_step_count + 1
    if (wpic_sync_every > 0) then
       if (mod(wpic_step_count, wpic_sync_every) == 0) then
          ! the sorted state ('gp' dummy = the driver's up) with its np2 and cumcnt
          call wpic_check(wpic_get_particles(wpic_ctx, 0_c_int, gp, np2_dev, cumcnt), 'get up')
          np2(:,:) = np2_dev(:,:)
          wpic_synced_at = wpic_step_count
       endif
    endif
  end subroutine sort__bucket
end module sort


module boundary_periodic
  use wpic_capi
  implicit none
  private
  public :: boundary_periodic__init, boundary_periodic__dfield, boundary_periodic__particle_x, &
       boundary_periodic__particle_y, boundary_periodic__curre, boundary_periodic__phi, boundary_periodic__mom
contains
  subroutine boundary_periodic__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in, &
                                     nup_in,ndown_in,mnpi_in,mnpr_in,ncomw_in,nerr_in,nstat_in,delx_in,delt_in,c_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
    integer, intent(in) :: nup_in, ndown_in, mnpi_in, mnpr_in, ncomw_in, nerr_in, nstat_in(:)
    real(8), intent(in) :: delx_in, delt_in, c_in
  end subroutine boundary_periodic__init

  subroutine boundary_periodic__particle_x(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    call wpic_check(p_bcx(wpic_ctx), 'bc__particle_x')
  end subroutine boundary_periodic__particle_x

  subroutine boundary_periodic__particle_y(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(inout) :: np2(*)
    call wpic_check(p_bcy(wpic_ctx), 'bc__particle_y')
  end subroutine boundary_periodic__particle_y

  ! applied inside the library; present so that field__fdtd_i's arguments type-check
  subroutine boundary_periodic__dfield(df,nxs,nxe,nys,nye,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nxgs, nxge
    real(8), intent(inout) :: df(*)
  end subroutine boundary_periodic__dfield
  subroutine boundary_periodic__curre(uj,nxs,nxe,nys,nye,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nxgs, nxge
    real(8), intent(inout) :: uj(*)
  end subroutine boundary_periodic__curre
  subroutine boundary_periodic__phi(phi,nxs,nxe,nys,nye,l)
    integer, intent(in)    :: nxs, nxe, nys, nye, l
    real(8), intent(inout) :: phi(*)
  end subroutine boundary_periodic__phi

  ! the fold runs on the device copy of mom that mom_calc__nvt left there; the host array
  ! is refreshed from it
  subroutine boundary_periodic__mom(mom)
    real(8), intent(inout) :: mom(*)
    call wpic_check(wpic_bc_mom(wpic_ctx), 'bc__mom')
    call wpic_check(wpic_get_mom(wpic_ctx, mom), 'get mom')
  end subroutine boundary_periodic__mom
end module boundary_periodic


! mom_calc (2d/common/mom_calc.f90) on the device: mom_calc__accl writes the device gp,
! mom_calc__nvt deposits from it (the driver passes gp) and copies mom to the host.
module mom_calc
  use wpic_capi
  implicit none
  private
  public :: mom_calc__init, mom_calc__accl, mom_calc__nvt
contains
  subroutine mom_calc__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in, &
                            delx_in,delt_in,c_in,q_in,r_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
    real(8), intent(in) :: delx_in, delt_in, c_in, q_in(nsp_in), r_in(nsp_in)
  end subroutine mom_calc__init

  ! the start of every driver's diagnostic block: the host up, uf and cumcnt are refreshed here
  ! (intent(in) in the reference; the drivers pass their own arrays)
  subroutine mom_calc__accl(gp,up,uf,cumcnt,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    integer, intent(inout) :: cumcnt(wpic_prm%nxgs:wpic_prm%nxge+1,wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    real(8), intent(inout) :: up(*), uf(*)
    real(8), intent(out)   :: gp(*)
    call wpic_ensure_ctx()
    call wpic_sync_host(up, uf, cumcnt=cumcnt)
    call wpic_check(wpic_mom_calc_accl(wpic_ctx), 'mom_calc__accl')
  end subroutine mom_calc__accl

  ! np2 comes back with the state refreshed in mom_calc__accl (energy_history reads it next)
  subroutine mom_calc__nvt(mom,up,np2)
    integer, intent(inout) :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    real(8), intent(in)    :: up(*)
    real(8), intent(out)   :: mom(*)
    call wpic_ensure_ctx()
    call wpic_sync_np2(np2)
    call wpic_check(wpic_mom_calc_nvt(wpic_ctx, 1_c_int), 'mom_calc__nvt')
    call wpic_check(wpic_get_mom(wpic_ctx, mom), 'get mom')
  end subroutine mom_calc__nvt
end module mom_calc


! boundary_reconnection (2d/proj/reconnection/boundary_reconnection.f90): conducting walls in x
module boundary_reconnection
  use wpic_capi
  implicit none
  private
  public :: boundary_reconnection__init, boundary_reconnection__dfield, boundary_reconnection__particle_x, &
       boundary_reconnection__particle_y, boundary_reconnection__curre, boundary_reconnection__phi, &
       boundary_reconnection__mom
contains
  subroutine boundary_reconnection__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in, &
                                         nup_in,ndown_in,mnpi_in,mnpr_in,ncomw_in,nerr_in,nstat_in,delx_in,delt_in,c_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
    integer, intent(in) :: nup_in, ndown_in, mnpi_in, mnpr_in, ncomw_in, nerr_in, nstat_in(:)
    real(8), intent(in) :: delx_in, delt_in, c_in
    wpic_prm%bc_kind = 1; wpic_bc_set = .true.
  end subroutine boundary_reconnection__init

  subroutine boundary_reconnection__particle_x(up,np2,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    call wpic_apply_window(nxs, nxe)
    call wpic_check(p_bcx(wpic_ctx), 'bc__particle_x')
  end subroutine boundary_reconnection__particle_x

  subroutine boundary_reconnection__particle_y(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(inout) :: np2(*)
    call wpic_check(p_bcy(wpic_ctx), 'bc__particle_y')
  end subroutine boundary_reconnection__particle_y

  ! applied inside the library; present so that field__fdtd_i's arguments type-check
  subroutine boundary_reconnection__dfield(df,nxs,nxe,nys,nye,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nxgs, nxge
    real(8), intent(inout) :: df(*)
  end subroutine boundary_reconnection__dfield
  subroutine boundary_reconnection__curre(uj,nxs,nxe,nys,nye,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nxgs, nxge
    real(8), intent(inout) :: uj(*)
  end subroutine boundary_reconnection__curre
  subroutine boundary_reconnection__phi(phi,nxs,nxe,nys,nye,l)
    integer, intent(in)    :: nxs, nxe, nys, nye, l
    real(8), intent(inout) :: phi(*)
  end subroutine boundary_reconnection__phi

  subroutine boundary_reconnection__mom(mom)
    real(8), intent(inout) :: mom(*)
    call wpic_check(wpic_bc_mom(wpic_ctx), 'bc__mom')
    call wpic_check(wpic_get_mom(wpic_ctx, mom), 'get mom')
  end subroutine boundary_reconnection__mom
end module boundary_reconnection


! boundary_shock (2d/proj/shock/boundary_shock.f90): reflecting wall at nxs, injection
! boundary at nxe of the window.  The shock driver edits up, uf and cumcnt on the host
! (inject, relocate), so its init switches the per-step upload on.
module boundary_shock
  use wpic_capi
  implicit none
  private
  public :: boundary_shock__init, boundary_shock__dfield, boundary_shock__particle_x, &
       boundary_shock__particle_y, boundary_shock__injection, boundary_shock__curre, boundary_shock__phi, &
       boundary_shock__mom
contains
  subroutine boundary_shock__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nys_in,nye_in, &
                                  nup_in,ndown_in,mnpi_in,mnpr_in,ncomw_in,nerr_in,nstat_in,delx_in,delt_in,c_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nys_in, nye_in
    integer, intent(in) :: nup_in, ndown_in, mnpi_in, mnpr_in, ncomw_in, nerr_in, nstat_in(:)
    real(8), intent(in) :: delx_in, delt_in, c_in
    wpic_prm%bc_kind = 2; wpic_bc_set = .true.
    call wpic_shim_set_upload(.true.)
    call wpic_shim_set_sync(1)
  end subroutine boundary_shock__init

  subroutine boundary_shock__particle_x(up,np2,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    call wpic_apply_window(nxs, nxe)
    call wpic_check(p_bcx(wpic_ctx), 'bc__particle_x')
  end subroutine boundary_shock__particle_x

  subroutine boundary_shock__particle_y(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(inout) :: np2(*)
    call wpic_check(p_bcy(wpic_ctx), 'bc__particle_y')
  end subroutine boundary_shock__particle_y

  subroutine boundary_shock__injection(up,np2,nxs,nxe,u0)
    integer, intent(in)    :: nxs, nxe
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    real(8), intent(in)    :: u0
    call wpic_apply_window(nxs, nxe)
    call wpic_check(wpic_bc_injection(wpic_ctx, real(u0, c_double)), 'bc__injection')
  end subroutine boundary_shock__injection

  ! applied inside the library; present so that field__fdtd_i's arguments type-check
  subroutine boundary_shock__dfield(df,nxs,nxe,nys,nye,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nxgs, nxge
    real(8), intent(inout) :: df(*)
  end subroutine boundary_shock__dfield
  subroutine boundary_shock__curre(uj,nxs,nxe,nys,nye,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nxgs, nxge
    real(8), intent(inout) :: uj(*)
  end subroutine boundary_shock__curre
  subroutine boundary_shock__phi(phi,nxs,nxe,nys,nye,l)
    integer, intent(in)    :: nxs, nxe, nys, nye, l
    real(8), intent(inout) :: phi(*)
  end subroutine boundary_shock__phi

  subroutine boundary_shock__mom(mom)
    real(8), intent(inout) :: mom(*)
    call wpic_check(wpic_bc_mom(wpic_ctx), 'bc__mom')
    call wpic_check(wpic_get_mom(wpic_ctx, mom), 'get mom')
  end subroutine boundary_shock__mom
end module boundary_shock


! The I/O routines that read the host state (paraio, 2d/common/paraio.f90:93-741, the drivers'
! io__* through wuming2d) refresh it from the device first; io__input marks the host state as
! the newer one, so the next particle__solv or sort__bucket uploads it.
module wpic_io
  use wpic_capi
  use paraio
  implicit none
  private
  public :: io__input, io__output, io__mom, io__ptcl, io__orb
contains
  subroutine io__input(up,uf,np2,nxs,nxe,it,filename)
    real(8), intent(out)         :: up(*), uf(*)
    integer, intent(out)         :: np2(*), nxs, nxe, it
    character(len=*), intent(in) :: filename
    call paraio__input(up, uf, np2, nxs, nxe, it, filename)
    wpic_uploaded = .false.
  end subroutine io__input

  subroutine io__output(up,uf,np2,nxs,nxe,it,filename)
    real(8), intent(inout)       :: up(*), uf(*)
    integer, intent(inout)       :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer, intent(in)          :: nxs, nxe, it
    character(len=*), intent(in) :: filename
    call wpic_sync_host(up, uf, np2=np2)
    call paraio__output(up, uf, np2, nxs, nxe, it, filename)
  end subroutine io__output

  subroutine io__mom(mom,uf,it)
    real(8), intent(inout) :: mom(*), uf(*)
    integer, intent(in)    :: it
    call wpic_sync_fields(uf)
    call paraio__mom(mom, uf, it)
  end subroutine io__mom

  subroutine io__ptcl(up,uf,np2,it)
    real(8), intent(inout) :: up(*), uf(*)
    integer, intent(inout) :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer, intent(in)    :: it
    call wpic_sync_host(up, uf, np2=np2)
    call paraio__ptcl(up, uf, np2, it)
  end subroutine io__ptcl

  subroutine io__orb(up,uf,np2,it)
    real(8), intent(inout) :: up(*), uf(*)
    integer, intent(inout) :: np2(wpic_prm%nys:wpic_prm%nye,wpic_prm%nsp)
    integer, intent(in)    :: it
    call wpic_sync_host(up, uf, np2=np2)
    call paraio__orb(up, uf, np2, it)
  end subroutine io__orb
end module wpic_io


! wuming2d (2d/common/wuming2d.f90) with the paraio I/O routines of the drivers' calls routed
! through wpic_io; everything else it exports is unchanged
module wuming2d
  use json_module
  use jsonio
  use mpiio
  use field
  use particle
  use mom_calc
  use sort
  use mpi_set
  use fio
  use h5io
  use paraio, &
       & io__init     => paraio__init,     &
       & io__finalize => paraio__finalize, &
       & io__param    => paraio__param
  use wpic_io
  implicit none
end module wuming2d
