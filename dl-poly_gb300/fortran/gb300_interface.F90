!> ISO_C_BINDING interface of libdlpoly_gb300.so for the DL_POLY driver.
!>
!> Each procedure binds one entry point of include/gb300_dlpoly.h.  The call
!> sites in the reference keep their signatures; a shim at the top of each
!> replaced routine calls the device path and returns.
!> Status codes are DL_POLY error numbers: the shim passes them to error().
Module gb300_interface
  Use, Intrinsic :: iso_c_binding, Only: c_int, c_int32_t, c_int64_t, c_double, c_ptr, c_char

  Implicit None

  Private

  !> mirror of gb_params (field order and kinds as in the C header)
  Type, Bind(C), Public :: gb_params
    Real(c_double)    :: cell(9)
    Real(c_double)    :: rcut, rpad, rvdw, alpha, epsq, tstep, shake_tol, pdplnc
    Integer(c_int32_t) :: kmax(3)
    Integer(c_int32_t) :: nsplines, spline_pad, vdw_direct, shake_maxit, max_list, max_exclude, mxatms
    Integer(c_int32_t) :: precision, ntypes, device
    Integer(c_int32_t) :: mxnode               ! comm%mxnode: gb_init refuses more than one rank
    Integer(c_int32_t) :: reserved(5)
  End Type gb_params

  !> mirror of gb_step_stats
  Type, Bind(C), Public :: gb_step_stats
    Real(c_double) :: engcpe_rc, vircpe_rc, engcpe_rl, vircpe_rl, engcpe_ex, vircpe_ex, engvdw, virvdw
    Real(c_double) :: engke, vircon
    Real(c_double) :: stress(9), strkin(9), strcon(9)
    Real(c_double) :: consv
    Real(c_double) :: engmet, virmet
    Integer(c_int32_t) :: list_rebuilt, shake_iters, rattle_iters, mts_full
  End Type gb_step_stats

  Logical, Public :: gb_active = .false.

  Public :: gb_init, gb_upload_parts, gb_download_parts, gb_relocate, gb_list_build, gb_vnl_check, &
            gb_refresh, gb_forces, gb_spme, gb_vv, gb_constraints_tags, gb_shake, gb_rattle, gb_md_run, gb_mts_config, gb_mts_stats, &
            gb_set_precision, gb_set_overlap, gb_set_ensemble, gb_set_step, gb_thermostat_state, &
            gb_set_thermostat_state, gb_set_metal_eam, gb_metal_energies, gb_finalize

  Interface
    Integer(c_int) Function gb_init(prm, natms, ltype, chge, weight, lfrzn, vdw_prm, ntcons, listcon, &
                                    prmcon, list_excl) Bind(C, name="gb_init")
      Import :: c_int, c_int32_t, c_double, gb_params
      Type(gb_params), Intent(In) :: prm
      Integer(c_int), Value :: natms, ntcons
      Integer(c_int32_t), Intent(In) :: ltype(*), lfrzn(*), listcon(*), list_excl(*)
      Real(c_double), Intent(In) :: chge(*), weight(*), vdw_prm(*), prmcon(*)
    End Function gb_init

    Integer(c_int) Function gb_upload_parts(parts, vx, vy, vz) Bind(C, name="gb_upload_parts")
      Import :: c_int, c_ptr, c_double
      Type(c_ptr), Value :: parts               ! c_loc(config%parts(1)), 64-byte corePart records
      Real(c_double), Intent(In) :: vx(*), vy(*), vz(*)
    End Function gb_upload_parts

    Integer(c_int) Function gb_download_parts(parts, vx, vy, vz) Bind(C, name="gb_download_parts")
      Import :: c_int, c_ptr, c_double
      Type(c_ptr), Value :: parts
      Real(c_double), Intent(Out) :: vx(*), vy(*), vz(*)
    End Function gb_download_parts

    Integer(c_int) Function gb_relocate() Bind(C, name="gb_relocate")
      Import :: c_int
    End Function gb_relocate

    Integer(c_int) Function gb_list_build(list_out, ldlist, max_list_io) Bind(C, name="gb_list_build")
      Import :: c_int, c_int32_t, c_ptr
      Type(c_ptr), Value :: list_out            ! c_loc(neigh%list(-3,1)) or c_null_ptr
      Integer(c_int), Value :: ldlist
      Integer(c_int32_t), Intent(InOut) :: max_list_io
    End Function gb_list_build

    Integer(c_int) Function gb_vnl_check(update) Bind(C, name="gb_vnl_check")
      Import :: c_int, c_int32_t
      Integer(c_int32_t), Intent(Out) :: update
    End Function gb_vnl_check

    Integer(c_int) Function gb_refresh(update) Bind(C, name="gb_refresh")
      Import :: c_int, c_int32_t
      Integer(c_int32_t), Intent(Out) :: update
    End Function gb_refresh

    Integer(c_int) Function gb_forces(eng_out, stress_out) Bind(C, name="gb_forces")
      Import :: c_int, c_double
      Real(c_double), Intent(Out) :: eng_out(8), stress_out(9)
    End Function gb_forces

    Integer(c_int) Function gb_spme(eng_rc, vir_rc, stress_out) Bind(C, name="gb_spme")
      Import :: c_int, c_double
      Real(c_double), Intent(Out) :: eng_rc, vir_rc, stress_out(9)
    End Function gb_spme

    Integer(c_int) Function gb_vv(stage, strkin, engke, iters, vircon, strcon) Bind(C, name="gb_vv")
      Import :: c_int, c_int32_t, c_double
      Integer(c_int), Value :: stage
      Real(c_double), Intent(Out) :: strkin(9), engke, vircon, strcon(9)
      Integer(c_int32_t), Intent(Out) :: iters
    End Function gb_vv

    Integer(c_int) Function gb_constraints_tags() Bind(C, name="gb_constraints_tags")
      Import :: c_int
    End Function gb_constraints_tags

    Integer(c_int) Function gb_shake(iters, vircon, strcon) Bind(C, name="gb_shake")
      Import :: c_int, c_int32_t, c_double
      Integer(c_int32_t), Intent(Out) :: iters
      Real(c_double), Intent(Out) :: vircon, strcon(9)
    End Function gb_shake

    Integer(c_int) Function gb_rattle(iters) Bind(C, name="gb_rattle")
      Import :: c_int, c_int32_t
      Integer(c_int32_t), Intent(Out) :: iters
    End Function gb_rattle

    Integer(c_int) Function gb_md_run(nsteps, stats) Bind(C, name="gb_md_run")
      Import :: c_int, gb_step_stats
      Integer(c_int), Value :: nsteps
      Type(gb_step_stats), Intent(Out) :: stats(*)
    End Function gb_md_run

    Integer(c_int) Function gb_mts_config(k, tol, train_steps) Bind(C, name="gb_mts_config")
      Import :: c_int, c_double
      Integer(c_int), Value :: k, train_steps
      Real(c_double), Value :: tol
    End Function gb_mts_config

    Integer(c_int) Function gb_mts_stats(out, n) Bind(C, name="gb_mts_stats")
      Import :: c_int, c_double
      Real(c_double), Intent(Out) :: out(*)
      Integer(c_int), Value :: n
    End Function gb_mts_stats

    Integer(c_int) Function gb_set_precision(precision) Bind(C, name="gb_set_precision")
      Import :: c_int
      Integer(c_int), Value :: precision
    End Function gb_set_precision

    Integer(c_int) Function gb_set_overlap(enable) Bind(C, name="gb_set_overlap")
      Import :: c_int
      Integer(c_int), Value :: enable
    End Function gb_set_overlap

    Integer(c_int) Function gb_set_ensemble(kind, temp, tau_t, chi, seed, degfre) &
        Bind(C, name="gb_set_ensemble")
      Import :: c_int, c_int32_t, c_double
      Integer(c_int), Value :: kind
      Real(c_double), Value :: temp, tau_t, chi, degfre
      Integer(c_int32_t), Intent(In) :: seed(3)
    End Function gb_set_ensemble

    Integer(c_int) Function gb_set_step(nstep) Bind(C, name="gb_set_step")
      Import :: c_int, c_int32_t
      Integer(c_int32_t), Value :: nstep
    End Function gb_set_step

    Integer(c_int) Function gb_thermostat_state(chi_t, cint, consv) Bind(C, name="gb_thermostat_state")
      Import :: c_int, c_double
      Real(c_double), Intent(Out) :: chi_t, cint, consv
    End Function gb_thermostat_state

    Integer(c_int) Function gb_set_thermostat_state(chi_t, cint) Bind(C, name="gb_set_thermostat_state")
      Import :: c_int, c_double
      Real(c_double), Value :: chi_t, cint
    End Function gb_set_thermostat_state

    Integer(c_int) Function gb_set_metal_eam(ntab, kind, t1, t2, ngrid, start, finish, values, listed) &
        Bind(C, name="gb_set_metal_eam")
      Import :: c_int, c_int32_t, c_double
      Integer(c_int), Value :: ntab
      Integer(c_int32_t), Intent(In) :: kind(*), t1(*), t2(*), ngrid(*), listed(*)
      Real(c_double), Intent(In) :: start(*), finish(*), values(*)
    End Function gb_set_metal_eam

    Integer(c_int) Function gb_metal_energies(out4) Bind(C, name="gb_metal_energies")
      Import :: c_int, c_double
      Real(c_double), Intent(Out) :: out4(4)
    End Function gb_metal_energies

    Subroutine gb_finalize() Bind(C, name="gb_finalize")
    End Subroutine gb_finalize
  End Interface

End Module gb300_interface
