! wpic_shim3d.f90 -- drop-in replacements for WumingPIC's 3D hot-path modules
! (particle, field, sort, boundary_periodic, mom_calc) that forward to the GB300 library's
! wpic3d_* entry points through ISO_C_BINDING.  Link these objects instead of the
! corresponding objects of libwuming3d_common.a; the drivers (3d/proj/*/app.f90)
! stay unchanged.  Coherence follows the 2D shim: the first particle__solv uploads
! the host state, the device state is authoritative afterwards, and the host arrays
! are refreshed only where the drivers read them -- on entry to mom_calc__accl (np2
! handed back in mom_calc__nvt) and in io__ptcl, io__orb, io__mom and io__output, which
! this file's wuming3d module wraps (3d/proj/weibel/app.f90 loop and diagnostic block);
! io__input makes the host the newer side.  wpic3d_shim_set_sync(n) (n >= 1) adds a
! refresh every n steps; the shock driver gets n = 1 from boundary_shock__init.
! The environment variable WPIC_PRECISION chooses the arithmetic without a driver change:
! 'mixed' runs the mixed-precision step (particle__solv requests the push, field__fdtd_i runs
! the fused step, the boundary and sort calls find their work done), 'fp64_exact' the
! reference-order FP64 build, anything else FP64.
module wpic3d_capi
  use iso_c_binding
  implicit none

  type, bind(C) :: wpic_params3d
     integer(c_int) :: ndim, np, nsp, nxgs, nxge, nygs, nyge, nzgs, nzge, nys, nye, nzs, nze
     real(c_double) :: delx, delt, c, gfac
     real(c_double) :: q(2), r(2)
     integer(c_int) :: precision, device_cap, bc_kind
  end type wpic_params3d

  interface
     integer(c_int) function wpic3d_init(ctx, p, stream) bind(C, name="wpic3d_init")
       import :: c_int, c_ptr, wpic_params3d
       type(c_ptr), intent(out) :: ctx
       type(wpic_params3d), intent(in) :: p
       type(c_ptr), value :: stream
     end function wpic3d_init
     integer(c_int) function wpic3d_put_particles(ctx, which, up, np2, cumcnt) bind(C, name="wpic3d_put_particles")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: which
       real(c_double), intent(in) :: up(*)
       integer(c_int), intent(in) :: np2(*), cumcnt(*)
     end function wpic3d_put_particles
     integer(c_int) function wpic3d_get_particles(ctx, which, up, np2, cumcnt) bind(C, name="wpic3d_get_particles")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: which
       real(c_double), intent(inout) :: up(*)
       integer(c_int), intent(inout) :: np2(*), cumcnt(*)
     end function wpic3d_get_particles
     integer(c_int) function wpic3d_set_window(ctx, nxs, nxe) bind(C, name="wpic3d_set_window")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: nxs, nxe
     end function wpic3d_set_window
     integer(c_int) function wpic3d_bc_injection(ctx, u0) bind(C, name="wpic3d_bc_injection")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: u0
     end function wpic3d_bc_injection
     integer(c_int) function wpic3d_put_fields(ctx, uf) bind(C, name="wpic3d_put_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: uf(*)
     end function wpic3d_put_fields
     integer(c_int) function wpic3d_mom_calc_accl(ctx) bind(C, name="wpic3d_mom_calc_accl")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_mom_calc_accl
     integer(c_int) function wpic3d_mom_calc_nvt(ctx, from_gp) bind(C, name="wpic3d_mom_calc_nvt")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: from_gp
     end function wpic3d_mom_calc_nvt
     integer(c_int) function wpic3d_bc_mom(ctx) bind(C, name="wpic3d_bc_mom")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_bc_mom
     integer(c_int) function wpic3d_get_mom(ctx, mom) bind(C, name="wpic3d_get_mom")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: mom(*)
     end function wpic3d_get_mom
     integer(c_int) function wpic3d_get_fields(ctx, uf) bind(C, name="wpic3d_get_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(inout) :: uf(*)
     end function wpic3d_get_fields
     integer(c_int) function wpic3d_particle_solv(ctx) bind(C, name="wpic3d_particle_solv")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_particle_solv
     integer(c_int) function wpic3d_particle_solv_vay(ctx) bind(C, name="wpic3d_particle_solv_vay")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_particle_solv_vay
     integer(c_int) function wpic3d_field_fdtd_i(ctx) bind(C, name="wpic3d_field_fdtd_i")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_field_fdtd_i
     integer(c_int) function wpic3d_bc_particle_x(ctx) bind(C, name="wpic3d_bc_particle_x")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_bc_particle_x
     integer(c_int) function wpic3d_bc_particle_yz(ctx) bind(C, name="wpic3d_bc_particle_yz")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_bc_particle_yz
     integer(c_int) function wpic3d_sort_bucket(ctx) bind(C, name="wpic3d_sort_bucket")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function wpic3d_sort_bucket
  end interface

  type(c_ptr), save :: wpic3_ctx = c_null_ptr
  type(wpic_params3d), save :: wpic3_prm
  logical, save :: wpic3_uploaded = .false.
  logical, save :: wpic3_bc_set = .false.  ! a boundary module's __init chose the kind
  logical, save :: wpic3_upload_each_step = .false.  ! the shock driver edits up/uf/cumcnt between steps
  integer, save :: wpic3_win_s = -huge(1), wpic3_win_e = -huge(1)
  integer, save :: wpic3_sync_every = 0, wpic3_step_count = 0  ! 0: refresh at the read points only
  integer, save :: wpic3_synced_at = -1      ! step count of the host arrays' last refresh
  integer(c_int), allocatable, save :: wpic3_np2_dev(:,:,:), wpic3_cc_dev(:,:,:,:)

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


  subroutine wpic3_check(st, where)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    if (st /= 0) then
       write(0,*) 'wumingpic_gb300: ', where, ' failed with status ', st
       stop
    endif
  end subroutine wpic3_check

  subroutine wpic3d_shim_set_sync(n)
    integer, intent(in) :: n
    wpic3_sync_every = max(0, n)
  end subroutine wpic3d_shim_set_sync

  ! the host arrays brought up to date with the device (once per step): up, uf and, when
  ! present, np2 and cumcnt; before the first upload the host is the newer side
  subroutine wpic3_sync_host(up, uf, np2, cumcnt)
    real(8), intent(inout) :: up(*), uf(*)
    integer, intent(inout), optional :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer, intent(inout), optional :: cumcnt(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                                               wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    if (.not. wpic3_uploaded) return
    if (.not. allocated(wpic3_np2_dev)) then
       allocate(wpic3_np2_dev(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp))
       allocate(wpic3_cc_dev(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                             wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp))
    endif
    if (wpic3_synced_at /= wpic3_step_count) then
       call wpic3_check(wpic3d_get_particles(wpic3_ctx, 0_c_int, up, wpic3_np2_dev, wpic3_cc_dev), 'get up')
       call wpic3_check(wpic3d_get_fields(wpic3_ctx, uf), 'get uf')
       wpic3_synced_at = wpic3_step_count
    endif
    if (present(np2)) np2(:,:,:) = wpic3_np2_dev(:,:,:)
    if (present(cumcnt)) cumcnt(:,:,:,:) = wpic3_cc_dev(:,:,:,:)
  end subroutine wpic3_sync_host

  subroutine wpic3_sync_fields(uf)
    real(8), intent(inout) :: uf(*)
    if (.not. wpic3_uploaded) return
    if (wpic3_synced_at /= wpic3_step_count) call wpic3_check(wpic3d_get_fields(wpic3_ctx, uf), 'get uf')
  end subroutine wpic3_sync_fields

  subroutine wpic3_sync_np2(np2)
    integer, intent(inout) :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    if (wpic3_uploaded .and. allocated(wpic3_np2_dev) .and. wpic3_synced_at == wpic3_step_count) &
         np2(:,:,:) = wpic3_np2_dev(:,:,:)
  end subroutine wpic3_sync_np2

  subroutine wpic3_ensure_ctx()
    if (.not. c_associated(wpic3_ctx)) call wpic3_check(wpic3d_init(wpic3_ctx, wpic3_prm, c_null_ptr), 'wpic3d_init')
  end subroutine wpic3_ensure_ctx

  ! the active window nxs..nxe that the driver passes to every module call (a shock run widens it)
  subroutine wpic3_apply_window(nxs, nxe)
    integer, intent(in) :: nxs, nxe
    call wpic3_ensure_ctx()
    if (nxs /= wpic3_win_s .or. nxe /= wpic3_win_e) then
       call wpic3_check(wpic3d_set_window(wpic3_ctx, int(nxs, c_int), int(nxe, c_int)), 'window')
       wpic3_win_s = nxs; wpic3_win_e = nxe
    endif
  end subroutine wpic3_apply_window

  ! up, uf and cumcnt to the device; cumcnt beyond the window (stale in the drivers) is completed
  ! with the row totals, which is what the library keeps there
  subroutine wpic3_upload_state(up, uf, cumcnt, nxe)
    real(8), intent(in) :: up(*), uf(*)
    integer, intent(in) :: cumcnt(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                                  wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer, intent(in) :: nxe
    integer(c_int) :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer(c_int) :: cc(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                         wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer :: i
    cc(:,:,:,:) = cumcnt(:,:,:,:)
    do i = nxe+2, wpic3_prm%nxge+1
       cc(i,:,:,:) = cumcnt(nxe+1,:,:,:)
    enddo
    np2(:,:,:) = cumcnt(nxe+1,:,:,:)
    call wpic3_check(wpic3d_put_particles(wpic3_ctx, 0_c_int, up, np2, cc), 'put up')
    call wpic3_check(wpic3d_put_fields(wpic3_ctx, uf), 'put uf')
    wpic3_uploaded = .true.
  end subroutine wpic3_upload_state

end module wpic3d_capi


module particle
  use wpic3d_capi
  implicit none
  private
  public :: particle__init, particle__solv, particle__solv_vay
contains
  subroutine particle__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in,nzge_in,nys_in,nye_in, &
                            nzs_in,nze_in,delx_in,delt_in,c_in,q_in,r_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in
    integer, intent(in) :: nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in, nys_in, nye_in, nzs_in, nze_in
    real(8), intent(in) :: delx_in, delt_in, c_in, q_in(nsp_in), r_in(nsp_in)
    wpic3_prm%ndim = ndim_in; wpic3_prm%np = np_in; wpic3_prm%nsp = nsp_in
    wpic3_prm%nxgs = nxgs_in; wpic3_prm%nxge = nxge_in; wpic3_prm%nygs = nygs_in; wpic3_prm%nyge = nyge_in
    wpic3_prm%nzgs = nzgs_in; wpic3_prm%nzge = nzge_in
    wpic3_prm%nys = nys_in; wpic3_prm%nye = nye_in; wpic3_prm%nzs = nzs_in; wpic3_prm%nze = nze_in
    wpic3_prm%delx = delx_in; wpic3_prm%delt = delt_in; wpic3_prm%c = c_in
    wpic3_prm%q(1:nsp_in) = q_in; wpic3_prm%r(1:nsp_in) = r_in
    wpic3_prm%precision = wpic_env_precision(); wpic3_prm%device_cap = 0
    if (.not. wpic3_bc_set) wpic3_prm%bc_kind = 0
  end subroutine particle__init

  subroutine particle__solv(gp,up,uf,cumcnt,nxs,nxe)
    integer, intent(in)  :: nxs, nxe
    integer, intent(in)  :: cumcnt(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                                   wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    real(8), intent(in)  :: up(*), uf(*)
    real(8), intent(out) :: gp(*)
    call wpic3_apply_window(nxs, nxe)
    if (.not. wpic3_uploaded .or. wpic3_upload_each_step) call wpic3_upload_state(up, uf, cumcnt, nxe)
    call wpic3_check(wpic3d_particle_solv(wpic3_ctx), 'particle__solv')
  end subroutine particle__solv

  subroutine particle__solv_vay(gp,up,uf,cumcnt,nxs,nxe)
    integer, intent(in)  :: nxs, nxe
    integer, intent(in)  :: cumcnt(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                                   wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    real(8), intent(in)  :: up(*), uf(*)
    real(8), intent(out) :: gp(*)
    call wpic3_apply_window(nxs, nxe)
    if (.not. wpic3_uploaded .or. wpic3_upload_each_step) call wpic3_upload_state(up, uf, cumcnt, nxe)
    call wpic3_check(wpic3d_particle_solv_vay(wpic3_ctx), 'particle__solv_vay')
  end subroutine particle__solv_vay
end module particle


module field
  use wpic3d_capi
  implicit none
  private
  public :: field__init, field__fdtd_i
contains
  subroutine field__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in,nzge_in,nys_in,nye_in, &
                         nzs_in,nze_in,mnpr_in,ncomw_in,opsum_in,nerr_in,delx_in,delt_in,c_in,q_in,r_in,gfac_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in
    integer, intent(in) :: nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in, nys_in, nye_in, nzs_in, nze_in
    integer, intent(in) :: mnpr_in, ncomw_in, opsum_in, nerr_in
    real(8), intent(in) :: delx_in, delt_in, c_in, q_in(nsp_in), r_in(nsp_in), gfac_in
    wpic3_prm%gfac = gfac_in
  end subroutine field__init

  subroutine field__fdtd_i(uf,up,gp,cumcnt,nxs,nxe,set_boundary_dfield,set_boundary_curre,set_boundary_phi)
    integer, intent(in)    :: nxs, nxe
    integer, intent(in)    :: cumcnt(*)
    real(8), intent(in)    :: up(*), gp(*)
    real(8), intent(inout) :: uf(*)
    external :: set_boundary_dfield, set_boundary_curre, set_boundary_phi
    call wpic3_apply_window(nxs, nxe)
    call wpic3_check(wpic3d_field_fdtd_i(wpic3_ctx), 'field__fdtd_i')
    if (wpic3_sync_every > 0) then
       if (mod(wpic3_step_count + 1, wpic3_sync_every) == 0) &
            call wpic3_check(wpic3d_get_fields(wpic3_ctx, uf), 'get uf')
    endif
  end subroutine field__fdtd_i
end module field


module sort
  use wpic3d_capi
  implicit none
  private
  public :: sort__init, sort__bucket
contains
  subroutine sort__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in,nzge_in,nys_in,nye_in,nzs_in,nze_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in
    integer, intent(in) :: nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in, nys_in, nye_in, nzs_in, nze_in
  end subroutine sort__init

  ! np2 is intent(in) in the reference; it is refreshed with the sorted state at the sync points
  subroutine sort__bucket(gp,up,cumcnt,np2,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    integer, intent(inout) :: np2(wpic3_prm%nye-wpic3_prm%nys+1, wpic3_prm%nze-wpic3_prm%nzs+1, wpic3_prm%nsp)
    integer, intent(inout) :: cumcnt(*)
    real(8), intent(in)    :: up(*)
    real(8), intent(inout) :: gp(*)
    integer(c_int) :: np2_dev(wpic3_prm%nye-wpic3_prm%nys+1, wpic3_prm%nze-wpic3_prm%nzs+1, wpic3_prm%nsp)
    call wpic3_apply_window(nxs, nxe)
    if (.not. wpic3_uploaded) then
       ! the restart path: io__input filled the host state; it is sorted on the device and handed
       ! back, and the next particle__solv uploads the whole host state (cumcnt is not read for
       ! the gp state; np2 stands in for it)
       np2_dev(:,:,:) = np2(:,:,:)
       call wpic3_check(wpic3d_put_particles(wpic3_ctx, 1_c_int, up, np2_dev, np2_dev), 'put gp')
       call wpic3_check(wpic3d_sort_bucket(wpic3_ctx), 'sort__bucket')
       call wpic3_check(wpic3d_get_particles(wpic3_ctx, 0_c_int, gp, np2_dev, cumcnt), 'get up')
       np2(:,:,:) = np2_dev(:,:,:)
       return
    endif
    call wpic3_check(wpic3d_sort_bucket(wpic3_ctx), 'sort__bucket')
    wpic3_step_count = wpic3_step_count + 1
    if (wpic3_sync_every > 0) then
       if (mod(wpic3_step_count, wpic3_sync_every) == 0) then
          call wpic3_check(wpic3d_get_particles(wpic3_ctx, 0_c_int, gp, np2_dev, cumcnt), 'get up')
          np2(:,:,:) = np2_dev(:,:,:)
          wpic3_synced_at = wpic3_step_count
       endif
    endif
  end subroutine sort__bucket
end module sort


module boundary_periodic
  use wpic3d_capi
  implicit none
  private
  public :: boundary_periodic__init, boundary_periodic__dfield, boundary_periodic__particle_x, &
       boundary_periodic__particle_yz, boundary_periodic__curre, boundary_periodic__phi, boundary_periodic__mom
contains
  subroutine boundary_periodic__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in, &
                                     nzge_in,nys_in,nye_in,nzs_in,nze_in,jup_in,jdown_in,kup_in,kdown_in,mnpi_in, &
                                     mnpr_in,ncomw_in,nerr_in,nstat_in,delx_in,delt_in,c_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in
    integer, intent(in) :: nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in, nys_in, nye_in, nzs_in, nze_in
    integer, intent(in) :: jup_in, jdown_in, kup_in, kdown_in, mnpi_in, mnpr_in, ncomw_in, nerr_in, nstat_in(:)
    real(8), intent(in) :: delx_in, delt_in, c_in
  end subroutine boundary_periodic__init

  subroutine boundary_periodic__particle_x(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    call wpic3_check(wpic3d_bc_particle_x(wpic3_ctx), 'bc__particle_x')
  end subroutine boundary_periodic__particle_x

  subroutine boundary_periodic__particle_yz(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(inout) :: np2(*)
    call wpic3_check(wpic3d_bc_particle_yz(wpic3_ctx), 'bc__particle_yz')
  end subroutine boundary_periodic__particle_yz

  ! applied inside the library; present so that field__fdtd_i's arguments type-check
  subroutine boundary_periodic__dfield(df,nxs,nxe,nys,nye,nzs,nze,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, nxgs, nxge
    real(8), intent(inout) :: df(*)
  end subroutine boundary_periodic__dfield
  subroutine boundary_periodic__curre(uj,nxs,nxe,nys,nye,nzs,nze,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, nxgs, nxge
    real(8), intent(inout) :: uj(*)
  end subroutine boundary_periodic__curre
  subroutine boundary_periodic__phi(phi,nxs,nxe,nys,nye,nzs,nze,l)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, l
    real(8), intent(inout) :: phi(*)
  end subroutine boundary_periodic__phi

  ! the fold runs on the device copy of mom that mom_calc__nvt left there
  subroutine boundary_periodic__mom(mom)
    real(8), intent(inout) :: mom(*)
    call wpic3_check(wpic3d_bc_mom(wpic3_ctx), 'bc__mom')
    call wpic3_check(wpic3d_get_mom(wpic3_ctx, mom), 'get mom')
  end subroutine boundary_periodic__mom
end module boundary_periodic


! boundary_reconnection (3d/proj/reconnection/boundary_reconnection.f90): conducting walls in x,
! periodic in y and z.  Its init selects the wall rules of the library's boundary kernels; the
! reflection runs in bc__particle_x, the other rules inside field__fdtd_i and bc__mom.
module boundary_reconnection
  use wpic3d_capi
  implicit none
  private
  public :: boundary_reconnection__init, boundary_reconnection__dfield, boundary_reconnection__particle_x, &
       boundary_reconnection__particle_yz, boundary_reconnection__curre, boundary_reconnection__phi, &
       boundary_reconnection__mom
contains
  subroutine boundary_reconnection__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in, &
                                         nzge_in,nys_in,nye_in,nzs_in,nze_in,jup_in,jdown_in,kup_in,kdown_in, &
                                         mnpi_in,mnpr_in,ncomw_in,nerr_in,nstat_in,delx_in,delt_in,c_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in
    integer, intent(in) :: nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in, nys_in, nye_in, nzs_in, nze_in
    integer, intent(in) :: jup_in, jdown_in, kup_in, kdown_in, mnpi_in, mnpr_in, ncomw_in, nerr_in, nstat_in(:)
    real(8), intent(in) :: delx_in, delt_in, c_in
    wpic3_prm%bc_kind = 1; wpic3_bc_set = .true.
  end subroutine boundary_reconnection__init

  subroutine boundary_reconnection__particle_x(up,np2,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    call wpic3_check(wpic3d_bc_particle_x(wpic3_ctx), 'bc__particle_x')
  end subroutine boundary_reconnection__particle_x

  subroutine boundary_reconnection__particle_yz(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(inout) :: np2(*)
    call wpic3_check(wpic3d_bc_particle_yz(wpic3_ctx), 'bc__particle_yz')
  end subroutine boundary_reconnection__particle_yz

  ! applied inside the library; present so that field__fdtd_i's arguments type-check
  subroutine boundary_reconnection__dfield(df,nxs,nxe,nys,nye,nzs,nze,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, nxgs, nxge
    real(8), intent(inout) :: df(*)
  end subroutine boundary_reconnection__dfield
  subroutine boundary_reconnection__curre(uj,nxs,nxe,nys,nye,nzs,nze,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, nxgs, nxge
    real(8), intent(inout) :: uj(*)
  end subroutine boundary_reconnection__curre
  subroutine boundary_reconnection__phi(phi,nxs,nxe,nys,nye,nzs,nze,l)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, l
    real(8), intent(inout) :: phi(*)
  end subroutine boundary_reconnection__phi

  subroutine boundary_reconnection__mom(mom)
    real(8), intent(inout) :: mom(*)
    call wpic3_check(wpic3d_bc_mom(wpic3_ctx), 'bc__mom')
    call wpic3_check(wpic3d_get_mom(wpic3_ctx, mom), 'get mom')
  end subroutine boundary_reconnection__mom
end module boundary_reconnection


! boundary_shock (3d/proj/shock/boundary_shock.f90): reflecting wall at nxs, injection boundary
! at nxe of the window.  The shock driver edits up, uf and cumcnt on the host (inject, relocate,
! 3d/proj/shock/app.f90:120-124), so its init switches the per-step upload on.
module boundary_shock
  use wpic3d_capi
  implicit none
  private
  public :: boundary_shock__init, boundary_shock__dfield, boundary_shock__particle_yz, &
       boundary_shock__injection, boundary_shock__curre, boundary_shock__phi, boundary_shock__mom
contains
  subroutine boundary_shock__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in, &
                                  nzge_in,nys_in,nye_in,nzs_in,nze_in,jup_in,jdown_in,kup_in,kdown_in, &
                                  mnpi_in,mnpr_in,ncomw_in,nerr_in,nstat_in,delx_in,delt_in,c_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in
    integer, intent(in) :: nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in, nys_in, nye_in, nzs_in, nze_in
    integer, intent(in) :: jup_in, jdown_in, kup_in, kdown_in, mnpi_in, mnpr_in, ncomw_in, nerr_in, nstat_in(:)
    real(8), intent(in) :: delx_in, delt_in, c_in
    wpic3_prm%bc_kind = 2; wpic3_bc_set = .true.
    wpic3_upload_each_step = .true.
    call wpic3d_shim_set_sync(1)
  end subroutine boundary_shock__init

  subroutine boundary_shock__particle_yz(up,np2)
    real(8), intent(inout) :: up(*)
    integer, intent(inout) :: np2(*)
    call wpic3_check(wpic3d_bc_particle_yz(wpic3_ctx), 'bc__particle_yz')
  end subroutine boundary_shock__particle_yz

  subroutine boundary_shock__injection(up,np2,nxs,nxe,u0)
    integer, intent(in)    :: nxs, nxe
    real(8), intent(inout) :: up(*)
    integer, intent(in)    :: np2(*)
    real(8), intent(in)    :: u0
    call wpic3_apply_window(nxs, nxe)
    call wpic3_check(wpic3d_bc_injection(wpic3_ctx, real(u0, c_double)), 'bc__injection')
  end subroutine boundary_shock__injection

  ! applied inside the library; present so that field__fdtd_i's arguments type-check
  subroutine boundary_shock__dfield(df,nxs,nxe,nys,nye,nzs,nze,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, nxgs, nxge
    real(8), intent(inout) :: df(*)
  end subroutine boundary_shock__dfield
  subroutine boundary_shock__curre(uj,nxs,nxe,nys,nye,nzs,nze,nxgs,nxge)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, nxgs, nxge
    real(8), intent(inout) :: uj(*)
  end subroutine boundary_shock__curre
  subroutine boundary_shock__phi(phi,nxs,nxe,nys,nye,nzs,nze,l)
    integer, intent(in)    :: nxs, nxe, nys, nye, nzs, nze, l
    real(8), intent(inout) :: phi(*)
  end subroutine boundary_shock__phi

  subroutine boundary_shock__mom(mom)
    real(8), intent(inout) :: mom(*)
    call wpic3_check(wpic3d_bc_mom(wpic3_ctx), 'bc__mom')
    call wpic3_check(wpic3d_get_mom(wpic3_ctx, mom), 'get mom')
  end subroutine boundary_shock__mom
end module boundary_shock


! mom_calc (3d/common/mom_calc.f90) on the device, as in the 2D shim
module mom_calc
  use wpic3d_capi
  implicit none
  private
  public :: mom_calc__init, mom_calc__accl, mom_calc__nvt
contains
  subroutine mom_calc__init(ndim_in,np_in,nsp_in,nxgs_in,nxge_in,nygs_in,nyge_in,nzgs_in,nzge_in,nys_in,nye_in, &
                            nzs_in,nze_in,delx_in,delt_in,c_in,q_in,r_in)
    integer, intent(in) :: ndim_in, np_in, nsp_in, nxgs_in, nxge_in, nygs_in, nyge_in, nzgs_in, nzge_in
    integer, intent(in) :: nys_in, nye_in, nzs_in, nze_in
    real(8), intent(in) :: delx_in, delt_in, c_in, q_in(nsp_in), r_in(nsp_in)
  end subroutine mom_calc__init

  ! the start of every driver's diagnostic block: the host up, uf and cumcnt are refreshed here
  subroutine mom_calc__accl(gp,up,uf,cumcnt,nxs,nxe)
    integer, intent(in)    :: nxs, nxe
    integer, intent(inout) :: cumcnt(wpic3_prm%nxgs:wpic3_prm%nxge+1,wpic3_prm%nys:wpic3_prm%nye, &
                                     wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    real(8), intent(inout) :: up(*), uf(*)
    real(8), intent(out)   :: gp(*)
    call wpic3_ensure_ctx()
    call wpic3_sync_host(up, uf, cumcnt=cumcnt)
    call wpic3_check(wpic3d_mom_calc_accl(wpic3_ctx), 'mom_calc__accl')
  end subroutine mom_calc__accl

  ! np2 comes back with the state refreshed in mom_calc__accl (energy_history reads it next)
  subroutine mom_calc__nvt(mom,up,np2)
    integer, intent(inout) :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    real(8), intent(in)    :: up(*)
    real(8), intent(out)   :: mom(*)
    call wpic3_ensure_ctx()
    call wpic3_sync_np2(np2)
    call wpic3_check(wpic3d_mom_calc_nvt(wpic3_ctx, 1_c_int), 'mom_calc__nvt')
    call wpic3_check(wpic3d_get_mom(wpic3_ctx, mom), 'get mom')
  end subroutine mom_calc__nvt
end module mom_calc


! The paraio routines that read the host state (3d/common/paraio.f90:102-866, the drivers' io__*
! through wuming3d) refresh it from the device first; io__input makes the host the newer side.
module wpic3_io
  use wpic3d_capi
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
    wpic3_uploaded = .false.
  end subroutine io__input

  subroutine io__output(up,uf,np2,nxs,nxe,it,filename)
    real(8), intent(inout)       :: up(*), uf(*)
    integer, intent(inout)       :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer, intent(in)          :: nxs, nxe, it
    character(len=*), intent(in) :: filename
    call wpic3_sync_host(up, uf, np2=np2)
    call paraio__output(up, uf, np2, nxs, nxe, it, filename)
  end subroutine io__output

  subroutine io__mom(mom,uf,it)
    real(8), intent(inout) :: mom(*), uf(*)
    integer, intent(in)    :: it
    call wpic3_sync_fields(uf)
    call paraio__mom(mom, uf, it)
  end subroutine io__mom

  subroutine io__ptcl(up,uf,np2,it)
    real(8), intent(inout) :: up(*), uf(*)
    integer, intent(inout) :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer, intent(in)    :: it
    call wpic3_sync_host(up, uf, np2=np2)
    call paraio__ptcl(up, uf, np2, it)
  end subroutine io__ptcl

  subroutine io__orb(up,uf,np2,it)
    real(8), intent(inout) :: up(*), uf(*)
    integer, intent(inout) :: np2(wpic3_prm%nys:wpic3_prm%nye,wpic3_prm%nzs:wpic3_prm%nze,wpic3_prm%nsp)
    integer, intent(in)    :: it
    call wpic3_sync_host(up, uf, np2=np2)
    call paraio__orb(up, uf, np2, it)
  end subroutine io__orb
end module wpic3_io


! wuming3d (3d/common/wuming3d.f90) with the drivers' io__* routed through wpic3_io
module wuming3d
  use json_module
  use jsonio
  use mpiio
  use field
  use particle
  use mom_calc
  use sort
  use mpi_set
  use paraio, &
       & io__init     => paraio__init,     &
       & io__finalize => paraio__finalize, &
       & io__param    => paraio__param
  use wpic3_io
  implicit none
end module wuming3d
