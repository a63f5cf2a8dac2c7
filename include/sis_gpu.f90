! ISO_C_BINDING interface module of libsisgpu (include/sis_gpu.h) for the
! Fortran host of SIS.  Each interface binds one C entry point by name, with
! the header's argument order and kinds; the derived types mirror the C
! structs field by field.  tests/test_abi.py checks both against the header.
! (No Fortran compiler is available where this library is built and tested,
! so the module is checked textually, not compiled.)
module sis_gpu_mod
  use, intrinsic :: iso_c_binding
  implicit none
  integer(c_int), parameter :: SIS_OK = 0
  ! include/sis_gpu.h status codes
  integer(c_int), parameter :: SIS_ERR_ARG = -1, SIS_ERR_CUDA = -2, SIS_ERR_LIST_OVERFLOW = -3, &
                               SIS_ERR_NONFINITE = -4, SIS_ERR_NOMEM = -5, SIS_ERR_STATE = -6, &
                               SIS_ERR_TIMEOUT = -7
  integer(c_int32_t), parameter :: SIS_PREC_FP64 = 0, SIS_PREC_MIXED = 1
  integer(c_int32_t), parameter :: SIS_LIST_WCA = 0, SIS_LIST_ELE = 1, SIS_LIST_BP = 2
  integer(c_int32_t), parameter :: SIS_LIST_WCA_INNER = 3, SIS_LIST_ELE_INNER = 4

  ! include/sis_gpu.h struct sis_params, field by field
  type, bind(C) :: sis_params
    real(c_double)     :: bond_k, bond_r0
    integer(c_int32_t) :: angl_reb
    real(c_double)     :: angl_k, angl_t0
    integer(c_int32_t) :: dih_type
    real(c_double)     :: dih_k, dih_w, dih_p0
    real(c_double)     :: wca_sigma, wca_eps
    integer(c_int32_t) :: bp_model, bp_min_loop, bp_jnext_compat
    real(c_double)     :: bp_cutoff_energy
    real(c_double)     :: bp_ff(15, 3)          ! C bp_ff[3][15]: GC, AU, GU
    real(c_double)     :: nn_dH(21), nn_dS(21)
    real(c_double)     :: dH0, dS0
    integer(c_int32_t) :: nnend
    real(c_double)     :: nnend_dH(6), nnend_dS(6), dHend0, dSend0
    integer(c_int32_t) :: flg_ele, ele_cutoff_type
    real(c_double)     :: ele_cutoff_inp, length_per_charge
    integer(c_int32_t) :: ele_excl_bond, ele_excl_angle, temp_independent
    real(c_double)     :: tempK_ref
    integer(c_int32_t) :: integrator
    real(c_double)     :: dt, viscosity_Pas, nl_margin
    integer(c_int32_t) :: nstep_bp_mc, max_bp_per_nt
    integer(c_int32_t) :: precision
    integer(c_int64_t) :: seed                  ! uint64_t in C
    integer(c_int32_t) :: nbr_cap, bp_cap
  end type

  type, bind(C) :: sis_topology
    integer(c_int32_t) :: n_inst
    type(c_ptr) :: inst_chain_off, chain_len, chain_moltype, seq, has_charge
    type(c_ptr) :: tempK, ionic_strength, box, stream
  end type

  type, bind(C) :: sis_stats
    integer(c_int64_t) :: steps, rebuilds, pair_entries, wca_pairs, ele_pairs, bp_pairs
    integer(c_int32_t) :: error_flags, n_beads, n_inst, lanes_per_bead
    integer(c_int64_t) :: capped
    integer(c_int32_t) :: bp_blocks, overlap, small_blocks, small_threads
    integer(c_int64_t) :: cluster_pairs
    integer(c_int32_t) :: i_clusters, reserved
  end type

  interface
    integer(c_int) function sis_gpu_create(top, par, ctx) bind(C, name="sis_gpu_create")
      import :: c_int, c_ptr, sis_topology, sis_params
      type(sis_topology), intent(in) :: top
      type(sis_params), intent(in) :: par
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function sis_gpu_get_stats(ctx, st) bind(C, name="sis_gpu_get_stats")
      import :: c_int, c_ptr, sis_stats
      type(c_ptr), value :: ctx
      type(sis_stats), intent(out) :: st
    end function
    subroutine sis_gpu_destroy(ctx) bind(C, name="sis_gpu_destroy")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    integer(c_int) function sis_gpu_set_state(ctx, inst, xyz, velos, accels) bind(C, name="sis_gpu_set_state")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
      type(c_ptr), value :: xyz, velos, accels   ! c_loc(...) or c_null_ptr
    end function
    integer(c_int) function sis_gpu_get_state(ctx, inst, xyz, velos, accels) bind(C, name="sis_gpu_get_state")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
      type(c_ptr), value :: xyz, velos, accels
    end function
    integer(c_int) function sis_gpu_neighbor_list(ctx, inst) bind(C, name="sis_gpu_neighbor_list")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
    end function
    integer(c_int) function sis_gpu_force(ctx, inst, forces) bind(C, name="sis_gpu_force")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
      real(c_double), intent(out) :: forces(3, *)
    end function
    integer(c_int) function sis_gpu_energy_sumup(ctx, inst, tempK, energies) bind(C, name="sis_gpu_energy_sumup")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
      real(c_double), value :: tempK
      real(c_double), intent(out) :: energies(0:10)
    end function
    integer(c_int) function sis_gpu_energy_kinetic(ctx, inst, ekin) bind(C, name="sis_gpu_energy_kinetic")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
      real(c_double), intent(out) :: ekin
    end function
    integer(c_int) function sis_gpu_step(ctx, nsteps, noise) bind(C, name="sis_gpu_step")
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: nsteps
      type(c_ptr), value :: noise                ! c_null_ptr: device Philox noise
    end function
    integer(c_int) function sis_gpu_set_condition(ctx, inst, tempK, ionic) bind(C, name="sis_gpu_set_condition")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst
      real(c_double), value :: tempK, ionic
    end function
    integer(c_int) function sis_gpu_set_temperature(ctx, inst, tempK) bind(C, name="sis_gpu_set_temperature")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst           ! -1: every instance
      real(c_double), value :: tempK
    end function
    integer(c_int) function sis_gpu_set_frozen(ctx, inst, beads, n) bind(C, name="sis_gpu_set_frozen")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, n
      integer(c_int32_t), intent(in) :: beads(*)  ! [Freeze] bead numbers (1-based)
    end function
    integer(c_int) function sis_gpu_set_ss_pairs(ctx, inst, n, pairs) bind(C, name="sis_gpu_set_ss_pairs")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, n
      integer(c_int32_t), intent(in) :: pairs(2, *)  ! bp_map pairs (imp, jmp) of read_ss, 1-based
    end function
    integer(c_int) function sis_gpu_set_bias_ss(ctx, on, force) bind(C, name="sis_gpu_set_bias_ss")
      import :: c_int, c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: on              ! flg_bias_ss
      real(c_double), value :: force               ! bias_ss_force (kcal/mol/A)
    end function
    integer(c_int) function sis_gpu_set_small(ctx, mode) bind(C, name="sis_gpu_set_small")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: mode
    end function
    integer(c_int) function sis_gpu_get_list(ctx, inst, kind, out, cap, n_out) bind(C, name="sis_gpu_get_list")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, kind, cap
      type(c_ptr), value :: out                  ! int32 (2|7, cap), 1-based bead indices
      integer(c_int32_t), intent(out) :: n_out
    end function
    integer(c_int) function sis_gpu_set_stage(ctx, sigma, eps) bind(C, name="sis_gpu_set_stage")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: sigma, eps
    end function
    integer(c_int) function sis_gpu_set_rg_bias(ctx, inst, pott, k, rg0) bind(C, name="sis_gpu_set_rg_bias")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, pott
      real(c_double), value :: k, rg0
    end function
    integer(c_int) function sis_gpu_set_bias_items(ctx, inst, n, kind_ij, par) bind(C, name="sis_gpu_set_bias_items")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, n
      integer(c_int32_t), intent(in) :: kind_ij(3, *)  ! kind, i, j (1-based)
      real(c_double), intent(in) :: par(14, *)
    end function
    integer(c_int) function sis_gpu_remd_init(ctx, temps) bind(C, name="sis_gpu_remd_init")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: temps(*)     ! the ladder by label
    end function
    integer(c_int) function sis_gpu_remd_init_vars(ctx, nvar, kinds, values) bind(C, name="sis_gpu_remd_init_vars")
      import :: c_int, c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nvar
      integer(c_int32_t), intent(in) :: kinds(*)    ! REPT%TEMP, %ION, %TWZDCF, %RG
      real(c_double), intent(in) :: values(*)       ! (nvar, nrep_all): lab2val
    end function
    integer(c_int) function sis_gpu_remd_exchange(ctx, parity, uniforms, rep2lab, n_accepted) &
        bind(C, name="sis_gpu_remd_exchange")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: parity         ! 0: pairs 1-2, 3-4, ...; 1: pairs 2-3, 4-5, ...
      type(c_ptr), value :: uniforms             ! c_null_ptr: device uniforms; else random0
      integer(c_int32_t), intent(out) :: rep2lab(*)   ! 0-based labels
      integer(c_int32_t), intent(out) :: n_accepted
    end function
    integer(c_int) function sis_gpu_bp_mc(ctx, inst, draws, n_draws) bind(C, name="sis_gpu_bp_mc")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, n_draws
      type(c_ptr), value :: draws                ! c_null_ptr: device uniforms
    end function
    integer(c_int) function sis_gpu_get_bp_status(ctx, inst, out, cap, n_out) bind(C, name="sis_gpu_get_bp_status")
      import :: c_int, c_int32_t, c_int8_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, cap
      integer(c_int8_t), intent(out) :: out(*)   ! 1 = formed, in the order of SIS_LIST_BP
      integer(c_int32_t), intent(out) :: n_out
    end function
    integer(c_int) function sis_gpu_get_bp_energies(ctx, inst, out, cap, n_out) bind(C, name="sis_gpu_get_bp_energies")
      import :: c_int, c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: inst, cap
      real(c_double), intent(out) :: out(*)      ! ene_bp, in the order of SIS_LIST_BP
      integer(c_int32_t), intent(out) :: n_out
    end function
    integer(c_int) function sis_gpu_step_noise_static(ctx, nsteps, noise) bind(C, name="sis_gpu_step_noise_static")
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: nsteps
      type(c_ptr), value :: noise                ! 3*nmp*nsteps doubles, step-major
    end function
    integer(c_int) function sis_gpu_probe_barrier_timeout(ctx) bind(C, name="sis_gpu_probe_barrier_timeout")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function sis_gpu_last_error(ctx) bind(C, name="sis_gpu_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
  end interface
end module sis_gpu_mod
