!> ISO_C_BINDING interface of librg (include/rg_api.h) for a Fortran engine:
!> the counterpart of the reference's GPU shell binding
!> (engine/source/elements/shell/coque/shell_gpu_mod.F90:292-713), widened to
!> every entry point of the C ABI.  Context and batch handles are opaque
!> type(c_ptr); arrays are passed as the engine holds them (X(3,NUMNOD),
!> IXS(11,NUMELS), ...); arguments the C side accepts as NULL are
!> type(c_ptr), value (pass c_null_ptr or c_loc(array)).  Every function
!> returns RG_OK (0) or a negative RG_E_* code; rg_error_message turns the
!> context's last error into a Fortran string.
!>
!> Built only on request (RG_FORTRAN=1 with a Fortran compiler, see
!> openradioss_gb300/build.py: build_fortran); nothing in the library needs it.
module rg_api_mod
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: RG_OK = 0, RG_E_ARG = -1, RG_E_STATE = -2, &
       RG_E_CUDA = -3, RG_E_UNSUP = -4, RG_E_DEVICE = -5, RG_E_MEM = -6, RG_E_SIZE = -7
  integer(c_int), parameter :: RG_ST_NEGVOL = 1, RG_ST_NAN = 2, RG_ST_SLOT = 4, &
       RG_ST_DTMIN = 8, RG_ST_BARRIER = 16, RG_ST_NODSTIF = 32
  integer(c_int), parameter :: RG_PREC_FP64 = 0, RG_PREC_MIXED = 1
  integer(c_int), parameter :: RG_PART_NQ = 7

  interface
    ! ---- context ---------------------------------------------------------
    integer(c_int) function rg_ctx_create(device, ctx) bind(c, name='rg_ctx_create')
      import :: c_int, c_ptr
      integer(c_int), value :: device
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function rg_ctx_destroy(ctx) bind(c, name='rg_ctx_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function rg_last_error(ctx) bind(c, name='rg_last_error')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function rg_set_precision(ctx, mode) bind(c, name='rg_set_precision')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: mode
    end function
    ! ---- model set-up ------------------------------------------------------
    integer(c_int) function rg_mesh_upload(ctx, numnod, x, v, ms, in, icodt) &
         bind(c, name='rg_mesh_upload')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: numnod
      real(c_double), intent(in) :: x(*), v(*), ms(*)
      type(c_ptr), value :: in, icodt
    end function
    integer(c_int) function rg_hexa_group_add(ctx, nel, ixs, mtn, pm, geo, uparam, iparam, &
         ismstr, jhbe, jcvt) bind(c, name='rg_hexa_group_add')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nel, mtn, ismstr, jhbe, jcvt
      integer(c_int), intent(in) :: ixs(*)
      real(c_double), intent(in) :: pm(*), geo(*)
      type(c_ptr), value :: uparam, iparam
    end function
    integer(c_int) function rg_shell_group_add(ctx, nel, ixc, npt, pm, geo, uparam, iparam, &
         thk0, ismstr, ithk) bind(c, name='rg_shell_group_add')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nel, npt, ismstr, ithk
      integer(c_int), intent(in) :: ixc(*), iparam(*)
      real(c_double), intent(in) :: pm(*), geo(*), uparam(*), thk0(*)
    end function
    integer(c_int) function rg_rwall_add(ctx, p0, nrm, dsearch) bind(c, name='rg_rwall_add')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: p0(3), nrm(3)
      real(c_double), value :: dsearch
    end function
    integer(c_int) function rg_rlink_add(ctx, nsn, nodes, ic, icr) bind(c, name='rg_rlink_add')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nsn, ic, icr
      integer(c_int), intent(in) :: nodes(*)
    end function
    integer(c_int) function rg_rlink_set_active(ctx, link, active) &
         bind(c, name='rg_rlink_set_active')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: link, active
    end function
    integer(c_int) function rg_set_nodal_dt(ctx, dtfac, dtmin) bind(c, name='rg_set_nodal_dt')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: dtfac, dtmin
    end function
    integer(c_int) function rg_set_shell_frame(ctx, ishfram) bind(c, name='rg_set_shell_frame')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: ishfram
    end function
    integer(c_int) function rg_skyline_set(ctx, adsky, iads, iadc) bind(c, name='rg_skyline_set')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(in) :: adsky(*)
      type(c_ptr), value :: iads, iadc
    end function
    integer(c_int) function rg_finalize(ctx, dtfac_solid, dtfac_shell, dtmx, dt2old) &
         bind(c, name='rg_finalize')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: dtfac_solid, dtfac_shell, dtmx, dt2old
    end function
    integer(c_int) function rg_skyline_get(ctx, adsky, iads, iadc, lsky) &
         bind(c, name='rg_skyline_get')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, adsky, iads, iadc, lsky
    end function
    ! ---- cycles ------------------------------------------------------------
    integer(c_int) function rg_cycle(ctx, ncycle) bind(c, name='rg_cycle')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncycle
    end function
    integer(c_int) function rg_synchronize(ctx) bind(c, name='rg_synchronize')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function rg_forint_step(ctx, x, v, vr, dt1, f, stifn, fr, stifr, dt2t, &
         neltst) bind(c, name='rg_forint_step')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: x(*), v(*)
      type(c_ptr), value :: vr, f, stifn, fr, stifr
      real(c_double), value :: dt1
      real(c_double), intent(out) :: dt2t
      integer(c_int), intent(out) :: neltst
    end function
    integer(c_int) function rg_cycle_host(ctx, x, v, vr, x_out, v_out, vr_out, d_out, dt2) &
         bind(c, name='rg_cycle_host')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, x, v, vr, x_out, v_out, vr_out, d_out
      real(c_double), intent(out) :: dt2
    end function
    integer(c_int) function rg_host_register(ctx, ptr, bytes) bind(c, name='rg_host_register')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: ctx, ptr
      integer(c_long_long), value :: bytes
    end function
    integer(c_int) function rg_host_unregister(ctx, ptr) bind(c, name='rg_host_unregister')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, ptr
    end function
    ! ---- results -----------------------------------------------------------
    integer(c_int) function rg_download_nodes(ctx, x, v, d, vr) bind(c, name='rg_download_nodes')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, x, v, d, vr
    end function
    integer(c_int) function rg_download_forces(ctx, f, stifn, fr) &
         bind(c, name='rg_download_forces')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, f, stifn, fr
    end function
    integer(c_int) function rg_download_hexa_state(ctx, which, out) &
         bind(c, name='rg_download_hexa_state')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: which
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function rg_download_shell_state(ctx, which, out) &
         bind(c, name='rg_download_shell_state')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: which
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function rg_get_time(ctx, tt, dt1, dt2, ncycle, neltst) &
         bind(c, name='rg_get_time')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: tt, dt1, dt2
      integer(c_int), intent(out) :: ncycle, neltst
    end function
    integer(c_int) function rg_energy(ctx, eint, ekin, ekinr, ehour) bind(c, name='rg_energy')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: eint, ekin, ekinr, ehour
    end function
    integer(c_int) function rg_set_dtmin(ctx, kind, idtmin, dtmin) bind(c, name='rg_set_dtmin')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: kind, idtmin
      real(c_double), value :: dtmin
    end function
    integer(c_int) function rg_energy_balance(ctx, out, n) bind(c, name='rg_energy_balance')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out(*)
      integer(c_int), value :: n
    end function
    ! ---- per-part sums (SBILAN / CBILAN PARTSAV, /TH/PART) ------------------
    integer(c_int) function rg_set_parts(ctx, npart, hexa_part, shell_part) &
        bind(c, name='rg_set_parts')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: npart
      integer(c_int), intent(in) :: hexa_part(*), shell_part(*)
    end function
    integer(c_int) function rg_part_count(ctx, npart) bind(c, name='rg_part_count')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: npart
    end function
    integer(c_int) function rg_part_sums_due(ctx) bind(c, name='rg_part_sums_due')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function rg_part_sums(ctx, out, npart) bind(c, name='rg_part_sums')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out(*)
      integer(c_int), value :: npart
    end function
    integer(c_int) function rg_status(ctx) bind(c, name='rg_status')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    ! ---- checkpoint / restart ------------------------------------------------
    integer(c_int) function rg_snapshot_size(ctx, bytes) bind(c, name='rg_snapshot_size')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: ctx
      integer(c_long_long), intent(out) :: bytes
    end function
    integer(c_int) function rg_snapshot(ctx, buf, bytes) bind(c, name='rg_snapshot')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: ctx, buf
      integer(c_long_long), value :: bytes
    end function
    integer(c_int) function rg_restore(ctx, buf, bytes) bind(c, name='rg_restore')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: ctx, buf
      integer(c_long_long), value :: bytes
    end function
    ! ---- inspection / benchmarking -------------------------------------------
    integer(c_int) function rg_info(ctx, numnod, numels, numelc, lsky, device_bytes) &
         bind(c, name='rg_info')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: numnod, numels, numelc, lsky
      integer(c_long_long), intent(out) :: device_bytes
    end function
    integer(c_int) function rg_set_timing(ctx, on) bind(c, name='rg_set_timing')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function
    integer(c_int) function rg_kernel_times(ctx, ms4) bind(c, name='rg_kernel_times')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: ms4(4)
    end function
    integer(c_int) function rg_time_cycles(ctx, ncycle, ms) bind(c, name='rg_time_cycles')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncycle
      real(c_double), intent(out) :: ms
    end function
    integer(c_int) function rg_time_cycles_cold(ctx, ncycle, flush_bytes, ms) &
         bind(c, name='rg_time_cycles_cold')
      import :: c_int, c_ptr, c_double, c_long_long
      type(c_ptr), value :: ctx
      integer(c_int), value :: ncycle
      integer(c_long_long), value :: flush_bytes
      real(c_double), intent(out) :: ms
    end function
    integer(c_int) function rg_kinetic_energy_noalloc(device, numnod, d_v, d_ms, ekin) &
         bind(c, name='rg_kinetic_energy_noalloc')
      import :: c_int, c_ptr, c_double
      integer(c_int), value :: device, numnod
      type(c_ptr), value :: d_v, d_ms
      real(c_double), intent(out) :: ekin
    end function
    integer(c_int) function rg_fp64_peak(device, fma_per_s) bind(c, name='rg_fp64_peak')
      import :: c_int, c_double
      integer(c_int), value :: device
      real(c_double), intent(out) :: fma_per_s
    end function
    ! ---- batched jobs --------------------------------------------------------
    integer(c_int) function rg_batch_create(device, b) bind(c, name='rg_batch_create')
      import :: c_int, c_ptr
      integer(c_int), value :: device
      type(c_ptr), intent(out) :: b
    end function
    integer(c_int) function rg_batch_destroy(b) bind(c, name='rg_batch_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
    end function
    type(c_ptr) function rg_batch_last_error(b) bind(c, name='rg_batch_last_error')
      import :: c_ptr
      type(c_ptr), value :: b
    end function
    integer(c_int) function rg_batch_add(b, job, target_ncycle) bind(c, name='rg_batch_add')
      import :: c_int, c_ptr
      type(c_ptr), value :: b, job
      integer(c_int), value :: target_ncycle
    end function
    integer(c_int) function rg_batch_remove(b, slot) bind(c, name='rg_batch_remove')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: slot
    end function
    integer(c_int) function rg_batch_set_target(b, slot, target_ncycle) &
         bind(c, name='rg_batch_set_target')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: slot, target_ncycle
    end function
    integer(c_int) function rg_batch_set_config(b, ktile, knode, blocks_per_sm, schedule) &
         bind(c, name='rg_batch_set_config')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: ktile, knode, blocks_per_sm, schedule
    end function
    integer(c_int) function rg_batch_get_config(b, cfg5) bind(c, name='rg_batch_get_config')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), intent(out) :: cfg5(5)
    end function
    integer(c_int) function rg_batch_cycle(b, ncycle) bind(c, name='rg_batch_cycle')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: ncycle
    end function
    integer(c_int) function rg_batch_synchronize(b) bind(c, name='rg_batch_synchronize')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
    end function
    integer(c_int) function rg_batch_time_cycles(b, ncycle, ms) &
         bind(c, name='rg_batch_time_cycles')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: ncycle
      real(c_double), intent(out) :: ms
    end function
    integer(c_int) function rg_batch_progress(b, ncycle, nslots, bstatus) &
         bind(c, name='rg_batch_progress')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), intent(out) :: ncycle(*)
      integer(c_int), value :: nslots
      integer(c_int), intent(out) :: bstatus
    end function
    integer(c_int) function rg_batch_job_status(b, status, nslots) &
         bind(c, name='rg_batch_job_status')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), intent(out) :: status(*)
      integer(c_int), value :: nslots
    end function
    integer(c_int) function rg_batch_set_barrier_test(b, spin_limit, late_block, late_us) &
         bind(c, name='rg_batch_set_barrier_test')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: spin_limit, late_block, late_us
    end function
    integer(c_int) function rg_batch_autotune(b, trial_cycles, cand, ncand, best5) &
         bind(c, name='rg_batch_autotune')
      import :: c_int, c_ptr
      type(c_ptr), value :: b, cand
      integer(c_int), value :: trial_cycles, ncand
      integer(c_int), intent(out) :: best5(5)
    end function
  end interface

contains

  !> The context's last error message as a Fortran string.
  function rg_error_message(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: p(:)
    type(c_ptr) :: cp
    integer :: n
    interface
      integer(c_size_t) function c_strlen(s) bind(c, name='strlen')
        import :: c_ptr, c_size_t
        type(c_ptr), value :: s
      end function
    end interface
    cp = rg_last_error(ctx)
    if (.not. c_associated(cp)) then
      msg = ''
      return
    end if
    n = int(c_strlen(cp))
    call c_f_pointer(cp, p, [n])
    allocate(character(len=n) :: msg)
    msg = transfer(p(1:n), msg)
  end function

end module rg_api_mod
