/*
 * gb300_dlpoly.h - C-ABI of the GB300 (sm_103a) per-timestep force and update
 * path of DL_POLY 5: link-cell Verlet list, real-space vdW + erfc-Coulomb
 * pairs, SPME reciprocal space, NVE velocity Verlet and SHAKE/RATTLE.
 *
 * The library keeps one device context (one GPU, one CUDA stream), exactly as
 * a serial DL_POLY rank keeps one configuration.  Positions, velocities,
 * forces, halo images, the Verlet list and the SPME grids stay resident in HBM
 * between calls; host arrays are borrowed only for the duration of a call.
 *
 * Conventions shared with the Fortran side (ISO_C_BINDING):
 *   - every array is a plain pointer plus a size, column-major where the
 *     Fortran array is 2-D, and index VALUES are 1-based (the Verlet list
 *     stores Fortran atom indices, list_excl stores global atom ids);
 *   - every entry point returns an int status: 0 = success, a positive value
 *     is the DL_POLY error code the caller passes to error(kode)
 *     (source/errors_warnings.F90:840), a negative value is a library error
 *     described by gb_strerror();
 *   - no exception, exit or device trap crosses the boundary.
 */
#ifndef GB300_DLPOLY_H
#define GB300_DLPOLY_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* DL_POLY error codes returned through the ABI (errors_warnings.F90). */
#define GB_OK 0
#define GB_ERR_CUTOFF_CELL 95     /* cutoff_extended >= half cell width (neighbours.F90:410) */
#define GB_ERR_SHAKE 105          /* SHAKE did not converge (constraints.F90:996) */
#define GB_ERR_LIST_OVERFLOW 106  /* Verlet list overflow (neighbours.F90:1193) */
#define GB_ERR_LINK_CELLS 307     /* fewer than one link cell per direction (neighbours.F90:428) */
#define GB_ERR_UNSAFE 505         /* unsafe pair/grid state (two_body.F90:751) */
#define GB_ERR_RATTLE 515         /* RATTLE did not converge (constraints.F90:748) */
#define GB_ERR_HALO 56            /* halo larger than mxatms (deport_data.F90:1870) */
#define GB_ERR_METAL_TABLE 506    /* metal table read below its first point (metal.F90:946) */
#define GB_ERR_METAL_DENSITY 507  /* local density outside its embedding table (metal.F90:1245) */
/* library errors */
#define GB_ERR_NOT_INIT (-1)
#define GB_ERR_CUDA (-2)
#define GB_ERR_ARG (-3)
#define GB_ERR_NO_DEVICE (-4)
#define GB_ERR_NONFINITE (-5)
#define GB_ERR_TOO_LARGE (-6)  /* size beyond a fixed scratch limit (gb_kinstress_noalloc) */
#define GB_ERR_RNG (-7)        /* a Gaussian deviate's rejection loop hit its iteration cap */
#define GB_ERR_MULTI_RANK (-8) /* gb_params.mxnode > 1: a multi-rank run cannot use the device path */
#define GB_ERR_DEVICE_WAIT (-9) /* a kernel's wait on its tensor-core completion hit its iteration limit */

/* Precision forms of the force path. */
#define GB_FP64 0   /* plain: FP64 accuracy; pair loop and SPME in double-float (pairs of FP32) */
#define GB_MIXED 1  /* FP32 pair/spline/FFT arithmetic, int64 fixed-point forces (2^40) */
#define GB_FP64_NATIVE 2  /* the FP64 form with the pair loop and SPME in native FP64 */

/* Ensembles of the VV stages (thermo%ensemble, drivers.F90:1132-1175) */
#define GB_NVE 0              /* nve_0_vv */
#define GB_NVT_BERENDSEN 1    /* nvt_b0_vv */
#define GB_NVT_NOSE_HOOVER 2  /* nvt_h0_vv */
#define GB_NVT_LANGEVIN 3     /* nvt_l0_vv */

/*
 * Run parameters.  Mirrors the CONTROL/FIELD-derived scalars the reference
 * keeps in neigh%, ewld%, electro%, vdws%, cons% and thermo%.
 */
typedef struct gb_params {
  double cell[9];       /* config%cell(1:9), cell vectors as rows (configuration.F90) */
  double rcut;          /* neigh%cutoff: real-space Coulomb cutoff */
  double rpad;          /* neigh%padding: Verlet skin */
  double rvdw;          /* vdws%cutoff */
  double alpha;         /* ewld%alpha (1/Angstrom) */
  double epsq;          /* electro%eps, relative dielectric constant */
  double tstep;         /* thermo%tstep (ps) */
  double shake_tol;     /* cons%tolerance (Angstrom) */
  double pdplnc;        /* neigh%pdplnc, sub-celling threshold density (default 50) */
  int32_t kmax[3];      /* ewld%kspace%k_vec_dim, SPME grid */
  int32_t nsplines;     /* ewld%bspline%num_splines, B-spline order p */
  int32_t spline_pad;   /* ewld%bspline%num_spline_pad (halo width for SPME) */
  int32_t vdw_direct;   /* 0 = tabulated vdW (default, vdw.F90:1790), 1 = direct (vdw.F90:1578) */
  int32_t shake_maxit;  /* cons%max_iter_shake (default 250) */
  int32_t max_list;     /* neigh%max_list */
  int32_t max_exclude;  /* neigh%max_exclude */
  int32_t mxatms;       /* config%mxatms: capacity for local + halo atoms */
  int32_t precision;    /* GB_FP64, GB_MIXED or GB_FP64_NATIVE */
  int32_t ntypes;       /* sites%ntype_atom */
  int32_t device;       /* CUDA device ordinal this context uses (one GPU per process) */
  int32_t mxnode;       /* comm%mxnode, MPI ranks of the run: gb_init returns GB_ERR_MULTI_RANK when > 1
                           (one rank drives one GPU; there is no domain decomposition, comms.F90) */
  int32_t reserved[5];
} gb_params;

/* Per-step scalars returned by the resident MD loop. */
typedef struct gb_step_stats {
  double engcpe_rc, vircpe_rc;  /* SPME reciprocal + self energy, virial */
  double engcpe_rl, vircpe_rl;  /* real-space Ewald */
  double engcpe_ex, vircpe_ex;  /* exclusion correction */
  double engvdw, virvdw;        /* van der Waals (without long-range correction) */
  double engke;                 /* kinetic energy (kinetics.F90:218) */
  double vircon;                /* constraint virial */
  double stress[9];             /* configurational stress (two-body + SPME) */
  double strkin[9];             /* kinetic stress */
  double strcon[9];             /* constraint stress of the SHAKE stage (stats%strcon) */
  double consv;                 /* thermostat's conserved-energy term (stats%consv; Nose-Hoover) */
  double engmet, virmet;        /* metal energy and virial: pair + embedding (engmet + engden) */
  int32_t list_rebuilt;         /* 1 if the Verlet list was rebuilt this step */
  int32_t shake_iters, rattle_iters;
  int32_t mts_full;             /* 1 if full SPME ran this step (learned-MTS form) */
} gb_step_stats;

/*
 * Replaces the start-up sequence molecular_dynamics_initialise ->
 * set_halo_particles (source/meta.F90:324-427) for the data the hot path
 * needs: uploads topology, builds the erfc and vdW interpolation tables
 * (electrostatic.F90:88, vdw.F90:1397), the SPME |b(m)|^2 table
 * (bspline.F90:73) and the self-interaction energy (spme.F90:159).
 *   ltype[natms]     1-based atom type (config%ltype)
 *   chge/weight      charge (e) and mass (amu) per atom
 *   lfrzn[natms]     frozen flag
 *   vdw_prm[3*nkey]  per type-pair key ai*(ai-1)/2+aj: (kind 0=none,1=lj, epsilon [internal units], sigma)
 *   listcon[3*ntcons] (type, global i, global j) as cons%listcon(0:2,k)
 *   prmcon[ntcontypes] constraint bond lengths (cons%prmcon)
 *   list_excl[(max_exclude+1)*natms] neigh%list_excl, column-major, sorted global ids
 */
int gb_init(const gb_params* prm, int natms, const int32_t* ltype, const double* chge,
            const double* weight, const int32_t* lfrzn, const double* vdw_prm, int ntcons,
            const int32_t* listcon, const double* prmcon, const int32_t* list_excl);

/* Upload positions (x,y,z) and velocities for the natms local atoms.
 * Replaces the host copies read by read_config (configuration.F90:846). */
int gb_upload_state(const double* x, const double* y, const double* z, const double* vx,
                    const double* vy, const double* vz);

/* Same, from the reference's 64-byte corePart records (particle.F90:13-19):
 * xxx,yyy,zzz,fxx,fyy,fzz,chge (f64) + 2 x int32 pad.  Forces are ignored. */
int gb_upload_parts(const void* parts, const double* vx, const double* vy, const double* vz);

/* Download positions, velocities and forces of the local atoms (any pointer may be NULL). */
int gb_download_state(double* x, double* y, double* z, double* vx, double* vy, double* vz,
                      double* fx, double* fy, double* fz);

/* Download into corePart records (positions, forces, charge). */
int gb_download_parts(void* parts, double* vx, double* vy, double* vz);

/*
 * relocate_particles + set_halo_particles in serial form
 * (deport_data.F90:2870 -> numerics.F90:1851 pbcshift; halo.F90:153) and
 * vnl_set_check (neighbours.F90:305): wrap into the cell, rebuild the halo
 * images on the device, set the displacement checkpoint.
 */
int gb_relocate(void);

/*
 * link_cell_pairs (neighbours.F90:356-1414) on the device: half-shell Verlet
 * list with sub-celling, nir bypass cells, frozen and excluded reordering.
 * If list_out != NULL the list is copied back in the reference layout
 * list(-3:max_list, 1:natms) column-major (ldlist must be max_list+4).
 * On overflow returns 106 and writes the needed max_list into *max_list_io.
 */
int gb_list_build(int32_t* list_out, int ldlist, int32_t* max_list_io);

/* vnl_check (neighbours.F90:123): sets *update = 1 when the largest
 * displacement since the last rebuild reaches half the padding. */
int gb_vnl_check(int32_t* update);

/* refresh_mappings (drivers.F90:1009) serial form: vnl_check, then either
 * relocate + halo rebuild (update) or refresh_halo_positions (halo.F90:47). */
int gb_refresh(int32_t* update);

/*
 * calculate_forces force part (drivers.F90:655-786): zero forces, SPME
 * reciprocal (ewald_spme_forces_coul, ewald_spole.F90:244), then the
 * two_body_forces pair loop (two_body.F90:339-606).
 *   eng_out[8] = engcpe_rc, vircpe_rc, engcpe_rl, vircpe_rl, engcpe_ex, vircpe_ex, engvdw, virvdw
 *   stress_out[9] configurational stress
 */
int gb_forces(double* eng_out, double* stress_out);

/* ewald_spme_forces_coul alone (forces zeroed first); for component tests. */
int gb_spme(double* eng_rc, double* vir_rc, double* stress_out);

/* two_body pair loop alone (forces zeroed first, no SPME); for component tests.
 * eng_out[6] = engcpe_rl, vircpe_rl, engcpe_ex, vircpe_ex, engvdw, virvdw */
int gb_real(double* eng_out, double* stress_out);

/* nve_0_vv (nve.F90:38): stage 1 = half kick + drift + SHAKE (apply_shake,
 * constraints.F90:1071); stage 2 = half kick + RATTLE (apply_rattle,
 * constraints.F90:1032) + kinstress (kinetics.F90:218).  With an NVT ensemble
 * set (gb_set_ensemble) the stages are those of nvt_b0_vv, nvt_h0_vv or
 * nvt_l0_vv instead. */
int gb_vv(int stage, double* strkin, double* engke, int32_t* iters, double* vircon,
          double* strcon);

/* The constraint parts of the VV stages on their own, for a driver that runs its own
 * stage update (another ensemble's Fortran stage) and calls apply_shake / apply_rattle
 * itself; gb_vv calls the same code.  They act on the resident state (gb_upload_state
 * first when the host changed it):
 *   gb_constraints_tags  constraints_tags (constraints.F90:438-586): the old bond vectors
 *                        from the current positions; call before the stage-1 drift.
 *   gb_shake             apply_shake (constraints.F90:1071-1200): the current positions are
 *                        the unconstrained ones; SHAKE (constraints_shake_vv :777-1030), then
 *                        the velocity and force corrections; returns 105 when SHAKE does not
 *                        converge in shake_maxit sweeps.
 *   gb_rattle            apply_rattle with kit = 1 (constraints.F90:1032-1069 ->
 *                        constraints_rattle :587-775) on the current velocities; returns 515
 *                        when RATTLE does not converge. */
int gb_constraints_tags(void);
int gb_shake(int32_t* iters, double* vircon, double* strcon);
int gb_rattle(int32_t* iters);

/* Resident MD loop (md_vv, drivers.F90:2059-2288): nsteps of VV1+SHAKE,
 * refresh, forces, VV2+RATTLE with no host round trip; stats[nsteps] may be NULL.
 * Each step first advances the step counter (gb_set_step).  In NVE without
 * constraints, thermostat, metals or learned MTS, a call of 3 or more steps replays
 * each step as CUDA graphs captured inside the call (same kernels and results). */
int gb_md_run(int nsteps, gb_step_stats* stats);

/* Ensemble of the VV stages: the dispatch on thermo%ensemble (drivers.F90:1132-1175)
 * for the non-rigid-body ensembles
 *   GB_NVE               nve_0_vv (nve.F90:38)
 *   GB_NVT_BERENDSEN     nvt_b0_vv (nvt_berendsen.F90:39), tau_t [ps]
 *   GB_NVT_NOSE_HOOVER   nvt_h0_vv (nvt_nose_hoover.F90), tau_t [ps]
 *   GB_NVT_LANGEVIN      nvt_l0_vv (nvt_langevin.F90), chi = friction [1/ps]
 * temp [K] is thermo%temp; seed[3] the 'random_seed' shifts of sarurnd
 * (numerics.F90:458; NULL = no shift); degfre the degrees of freedom
 * (config%degfre; <= 0 computes 3*(free atoms) - 3 - constraints,
 * temperature.F90:109-143).  Resets chi_t and cint to zero. */
int gb_set_ensemble(int kind, double temp, double tau_t, double chi, const int32_t* seed,
                    double degfre);

/* flow%step used by the next stage-1 call (the Langevin random forces are keyed
 * on it, langevin.F90:57); gb_md_run increments it before each step. */
int gb_set_step(int32_t nstep);

/* Thermostat state thermo%chi_t, thermo%cint and stats%consv (Nose-Hoover:
 * 0.5*qmass*chi_t^2 + ceng*cint, else 0); the setter restores chi_t and cint
 * (REVIVE, system.F90:1831). */
int gb_thermostat_state(double* chi_t, double* cint, double* consv);
int gb_set_thermostat_state(double chi_t, double cint);

/* Test hook: the generator of the Langevin forces on the device.  mode 0: out[i] =
 * sarurnd(a[i], b[i], c[i]) (numerics.F90:458); mode 1: out[3i..3i+2] =
 * box_mueller_saru3(a[i], b[i]) with its counter starting at c[i] (numerics.F90:745). */
int gb_rng_eval(int mode, int n, const int64_t* a, const int64_t* b, const int64_t* c, double* out);

/* Tabulated EAM metals ('metal ... eam' in FIELD with a TABEAM file: metal.F90 tab = 1).
 * ntab tables in TABEAM order: kind[k] 1 = pair (types t1[k], t2[k]), 2 = density of
 * type t1[k], 3 = embedding of type t1[k]; ngrid[k] points from start[k] to finish[k];
 * values concatenated, energies already in internal units (metal_table_read,
 * metal.F90:1489).  listed[nkey] (may be NULL = all) marks the type pairs the FIELD
 * 'metal' directive lists; unlisted pairs exert no metal force (keypot -1).  Each force
 * evaluation then runs metal_ld_compute (metal.F90:897) and metal_forces (:193) on the
 * Verlet list; their energies go to gb_step_stats.engmet/virmet and gb_metal_energies.
 * FP64 form only; ntab = 0 removes the metal terms. */
int gb_set_metal_eam(int ntab, const int32_t* kind, const int32_t* t1, const int32_t* t2,
                     const int32_t* ngrid, const double* start, const double* finish,
                     const double* values, const int32_t* listed);

/* engmet, virmet, engden, virden of the last force evaluation (two_body.F90:780-781). */
int gb_metal_energies(double* out4);

/* F'(rho_i) per local atom after the last force evaluation (met%rho after
 * metal_ld_compute); test hook. */
int gb_metal_rho(double* out);

/* Learned multiple-time-step form (no counterpart in the reference: its
 * electro%nstfce key is parsed but SPME runs every step, two_body.F90:298-302).
 * A time-reversible impulse split: every step integrates the real-space force
 * plus S = (reciprocal force on a coarse grid) + (a per-atom MLP's correction of
 * that grid's error); every k-th step runs SPME and its force carries the impulse
 * k (F_SPME - S).  The first train_steps MD steps run SPME every step and train
 * the network online on F_SPME - C; afterwards every k-th step compares S with
 * SPME and runs plain SPME every step (no impulses) while
 * RMS(S - SPME) / RMS(total force) > tol.  Needs GB_MIXED; each call restarts
 * from fresh weights.  k = 1 disables. */
int gb_mts_config(int k, double tol, int train_steps);

/* Learned-MTS counters, up to n of: [0] last checked relative error,
 * [1] full steps, [2] inner steps, [3] fallback entries, [4] last training
 * loss, [5] optimiser steps, [6] largest checked error, [7] 1 while in
 * fallback, [8] checks made, [9] MD steps seen, [10] error of the same check
 * without the network (coarse-grid force alone), [11] error of the reciprocal
 * force of the previous full step held unchanged, [12] coarse grid points along x. */
int gb_mts_stats(double* out, int n);

/* Test hooks of the learned form (no reference counterpart).
 * gb_mts_features: the current scaled network inputs of the first n atoms
 *   (n x 51 floats) and the 51 input scales + force scale (52 floats).
 * gb_mlp_param_count: length of the FP32 parameter vector
 *   W1[51][128] b1[128] W2[128][128] b2[128] W3[128][3] b3[3].
 * gb_mlp_train_eval: the training kernel's forward + MSE + backward on nb rows
 *   x[nb][51] with labels target[nb][3]: loss, grad[param_count], y[nb][3].
 * gb_mlp_infer_eval: the inference kernel's output y[nb][3] for x[nb][51]. */
int gb_mts_features(float* x, int n, float* scales);
/* Ablation switch for tests: 1 = S is the coarse-grid force alone (the same
 * impulse schedule without the network, which is then not trained). */
int gb_mts_ablation(int no_network);
int gb_mlp_param_count(void);
int gb_mlp_train_eval(int nb, const float* x, const float* target, const float* params, float* loss,
                      float* grad, float* y);
int gb_mlp_infer_eval(int nb, const float* x, const float* params, float* y);

/* Switch the force path between GB_FP64, GB_MIXED and GB_FP64_NATIVE after gb_init. */
int gb_set_precision(int precision);

/* Device time (ms) of the last gb_md_run per region, CUDA events on the
 * library stream: [0] list+halo, [1] real-space, [2] SPME, [3] integrate,
 * [4] total.  n = number of slots to copy. */
int gb_last_timings(double* ms, int n);

/* Number of kernels the library launched since gb_init (its own count). */
int64_t gb_kernel_launches(void);

/* Per-kernel CUDA-event timing on the library stream (the CHRONO timers of
 * timer.F90:335-476 as device events).  gb_profile(1) starts collecting and
 * clears the totals; gb_profile_read copies, for up to max entries, the
 * kernel name (32 bytes each), total milliseconds and launch count. */
int gb_profile(int enable);
int gb_profile_read(char* names, double* ms, int64_t* launches, int max);

/* Reciprocal-space sum on a second stream, of higher priority, while the pair kernel runs
 * (1, the default; GB_OVERLAP=0 in the environment at gb_init starts with 0) or both on
 * one stream (0).  The results are the same bits either way; 0 gives each kernel the
 * whole GPU, which the per-kernel timings of gb_profile want.  No reference counterpart. */
int gb_set_overlap(int enable);

/* Work counters of the last force evaluation and list build: [0] half-list entries,
 * [1] unique pairs inside rc, [2] list-build candidates tested in exact FP64,
 * [3] list entries with a halo image from the forward half shell, [4] from the
 * backward halo pass (equal when every such pair is listed from both atoms),
 * [5] 1 when the pair kernels walked the sorted-position list, [6] list-build
 * tiles of the second (larger shared memory) launch, [7] link cells per tile along x. */
int gb_pair_counts(int64_t* out, int n);

/* FP64 FMA throughput of this device in TFLOP/s, measured by a register-
 * resident DFMA loop (the FP64 roofline denominator; not used by the path). */
double gb_fp64_peak_tflops(void);

/*
 * Kinetic stress of n atoms (the sum kinstress forms) for callers that cannot
 * allocate device memory: a host program whose device memory belongs to a
 * pool it does not control, or that must not allocate once a run is under
 * way.  This entry point has no counterpart in the reference.
 *   vx, vy, vz, weight, lfrzn (may be NULL: no frozen atoms) and strkin_out
 *   (9 doubles, the symmetric 3x3 tensor) are DEVICE pointers; stream may be
 *   NULL (the default stream).  The call only enqueues work: synchronise the
 *   stream before reading strkin_out.  It needs no gb_init.
 * It allocates nothing.  Its scratch is a fixed array of 4096 x 6 doubles
 * (196,608 bytes) in the library's device memory, held on every GPU that loads
 * the library until the process exits, so n is limited to 1,048,576 atoms;
 * larger n returns GB_ERR_TOO_LARGE and launches nothing.  The first call on
 * each device looks up the address of that array; make that first call before
 * any stream capture.  All calls share the one array: calls that overlap on
 * the GPU (concurrent streams, or another host thread) race and give wrong
 * results, so serialise them.
 */
int gb_kinstress_noalloc(const double* vx, const double* vy, const double* vz, const double* weight,
                         const int32_t* lfrzn, int n, double* strkin_out, void* stream);

/* Release device memory; gb_init may be called again afterwards. */
void gb_finalize(void);

/* Human-readable text for a status code. */
const char* gb_strerror(int status);

#ifdef __cplusplus
}
#endif

#endif /* GB300_DLPOLY_H */
