! sesp_mod.f90 - ISO_C_BINDING interface to the GB300 engine (include/sesp.h)
! for the reference's Fortran driver src/mybox.f90.  A driver that keeps
! program mybox as the host replaces the force section and the move_*_a /
! move_*_b calls with the bindings below (see the integration notes shipped
! with the engine).  All arrays are (3, n_sites) real(c_double) in the
! reference's site order and reduced units.
module sesp_mod
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SESP_PLAIN_FP64 = 0, SESP_MIXED = 1, SESP_MIXED_FP32C = 2, SESP_MIXED_COMP = 3
  integer(c_int), parameter :: SESP_T_ALL = 1023
  integer(c_int), parameter :: SESP_PRESET_REFERENCE = 0, SESP_PRESET_CONFIG = 1

  type, bind(C) :: sesp_params
    integer(c_int) :: n_cells(3)
    integer(c_int) :: precision
    integer(c_int) :: rebuild_interval
    integer(c_int) :: graphite_on
    real(c_double) :: tr
    real(c_double) :: tau_steps
    real(c_double) :: shake_tol
    integer(c_int) :: shake_maxit
    integer(c_int) :: device
    integer(c_int) :: max_cell_sites
    integer(c_int) :: preset           ! SESP_PRESET_REFERENCE (0) or SESP_PRESET_CONFIG (1)
  end type sesp_params

  interface
    integer(c_int) function sesp_abi_version() bind(C, name="sesp_abi_version")
      import :: c_int
    end function
    integer(c_int) function sesp_last_error(buf, len) bind(C, name="sesp_last_error")
      import :: c_int, c_char, c_size_t
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_size_t), value :: len
    end function
    integer(c_int) function sesp_default_params(p) bind(C, name="sesp_default_params")
      import :: c_int, sesp_params
      type(sesp_params), intent(out) :: p
    end function
    integer(c_int) function sesp_default_config_params(p) bind(C, name="sesp_default_config_params")
      import :: c_int, sesp_params
      type(sesp_params), intent(out) :: p
    end function
    integer(c_int) function sesp_create(p, ctx) bind(C, name="sesp_create")
      import :: c_int, c_ptr, sesp_params
      type(sesp_params), intent(in) :: p
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function sesp_destroy(ctx) bind(C, name="sesp_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_upload_state(ctx, n_water, n_surf, pos, vel, n_carbon, carbons) &
        bind(C, name="sesp_upload_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: n_water, n_surf, n_carbon
      real(c_double), intent(in) :: pos(*), vel(*), carbons(*)
    end function
    integer(c_int) function sesp_download_state(ctx, pos, vel, acc) bind(C, name="sesp_download_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: pos(*), vel(*), acc(*)
    end function
    integer(c_int) function sesp_set_state(ctx, pos, vel, acc, eta) bind(C, name="sesp_set_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: pos(*), vel(*), acc(*)
      real(c_double), value :: eta
    end function
    integer(c_int) function sesp_force(ctx, rebuild) bind(C, name="sesp_force")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: rebuild
    end function
    integer(c_int) function sesp_force_terms(ctx, rebuild, terms) bind(C, name="sesp_force_terms")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: rebuild, terms
    end function
    integer(c_int) function sesp_download_forces(ctx, f) bind(C, name="sesp_download_forces")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: f(*)
    end function
    integer(c_int) function sesp_init_accel(ctx) bind(C, name="sesp_init_accel")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_move_a(ctx) bind(C, name="sesp_move_a")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_move_b(ctx) bind(C, name="sesp_move_b")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_step(ctx, kb) bind(C, name="sesp_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: kb
    end function
    integer(c_int) function sesp_run(ctx, kb0, nsteps) bind(C, name="sesp_run")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: kb0, nsteps
    end function
    integer(c_int) function sesp_run_async(ctx, kb0, nsteps) bind(C, name="sesp_run_async")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: kb0, nsteps
    end function
    integer(c_int) function sesp_sync(ctx) bind(C, name="sesp_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_temperature(ctx, t) bind(C, name="sesp_temperature")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: t
    end function
    integer(c_int) function sesp_get_eta(ctx, eta) bind(C, name="sesp_get_eta")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: eta
    end function
    integer(c_int) function sesp_set_eta(ctx, eta) bind(C, name="sesp_set_eta")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: eta
    end function
    integer(c_int) function sesp_energies(ctx, e) bind(C, name="sesp_energies")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: e(8)
    end function
    integer(c_int) function sesp_autotune(ctx, out) bind(C, name="sesp_autotune")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: out(3)
    end function
    integer(c_int) function sesp_tuning(ctx, out) bind(C, name="sesp_tuning")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: out(3)
    end function
    integer(c_int) function sesp_set_tuning(ctx, tile, ctas_per_sm) bind(C, name="sesp_set_tuning")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: tile, ctas_per_sm
    end function
    integer(c_int) function sesp_set_constraint_tuning(ctx, surf_warps, mols_per_warp) &
        bind(C, name="sesp_set_constraint_tuning")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: surf_warps, mols_per_warp
    end function
    integer(c_int) function sesp_constraint_tuning(ctx, out) bind(C, name="sesp_constraint_tuning")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: out(4)
    end function
    ! sesp_energies without allocating (fixed scratch; at most 131072 sites)
    integer(c_int) function sesp_energies_static(ctx, e) bind(C, name="sesp_energies_static")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: e(8)
    end function
    integer(c_int) function sesp_counters(ctx, c) bind(C, name="sesp_counters")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), intent(out) :: c(8)
    end function
    ! get_molecule_count and computeOnm4 checks, 8 values per replica
    integer(c_int) function sesp_checks(ctx, c) bind(C, name="sesp_checks")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: c(*)
    end function
    integer(c_int) function sesp_check_flags(c) bind(C, name="sesp_check_flags")
      import :: c_int, c_double
      real(c_double), intent(in) :: c(7)
    end function
    ! compute_temperature_rescale: v = sqrt(target / T) v (the reference's target is 3.9)
    integer(c_int) function sesp_rescale_temperature(ctx, target, t_before) bind(C, name="sesp_rescale_temperature")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: target
      real(c_double), intent(out) :: t_before
    end function
    integer(c_int) function sesp_kernel_times(ctx, t, reset) bind(C, name="sesp_kernel_times")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: t(8)
      integer(c_int), value :: reset
    end function
    integer(c_int) function sesp_enable_timing(ctx, on) bind(C, name="sesp_enable_timing")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function
    integer(c_int) function sesp_run_timed(ctx, kb0, nsteps, flush_l2, step_ms) bind(C, name="sesp_run_timed")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: kb0, nsteps, flush_l2
      real(c_double), intent(out) :: step_ms(*)
    end function
    integer(c_int) function sesp_pair_counts(ctx, c) bind(C, name="sesp_pair_counts")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), intent(out) :: c(2)
    end function
    integer(c_int) function sesp_upload_batch(ctx, n_rep, n_water, n_surf, n_cells, pos, vel, n_carbon, carbons) &
        bind(C, name="sesp_upload_batch")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: n_rep
      integer(c_int), intent(in) :: n_water(*), n_surf(*), n_cells(*), n_carbon(*)
      real(c_double), intent(in) :: pos(*), vel(*), carbons(*)
    end function
    integer(c_int) function sesp_replica_count(ctx) bind(C, name="sesp_replica_count")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_get_eta_batch(ctx, eta) bind(C, name="sesp_get_eta_batch")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: eta(*)
    end function
    integer(c_int) function sesp_set_eta_batch(ctx, eta) bind(C, name="sesp_set_eta_batch")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: eta(*)
    end function
    integer(c_int) function sesp_failures_batch(ctx, fails) bind(C, name="sesp_failures_batch")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), intent(out) :: fails(*)
    end function
    integer(c_int) function sesp_query(ctx) bind(C, name="sesp_query")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function sesp_device_bytes(ctx, bytes) bind(C, name="sesp_device_bytes")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), intent(out) :: bytes
    end function
    integer(c_int) function sesp_fp32_peak(device, tflops) bind(C, name="sesp_fp32_peak")
      import :: c_int, c_double
      integer(c_int), value :: device
      real(c_double), intent(out) :: tflops
    end function
  end interface
end module sesp_mod
