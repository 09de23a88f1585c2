/*
 * sesp.h - C ABI of the GB300 engine for the per-timestep force-and-integrate
 * path of jhalverson/surfactant_enhanced_spreading (water / trisiloxane
 * surfactant nanodroplets on graphite).
 *
 * The reference is a Fortran 90 + MPI program whose driver (src/mybox.f90)
 * calls, every step, the velocity-Verlet first halves, the force section and
 * the second halves.  Its subroutines take one integer (the rank) and move
 * all data through COMMON blocks (src/mybox.cmns:207-259), so there is no
 * binary interface to keep; this header is the boundary a Fortran driver
 * binds through ISO_C_BINDING (include/sesp_mod.f90) and that the Python
 * host layer binds through ctypes.  Each entry point names the reference
 * call sequence it replaces.
 *
 * Conventions: every function returns 0 on success or a positive SESP_E*
 * code; sesp_last_error() returns the message of the last failure of the
 * calling thread.  State arrays are host-owned (n_sites, 3) row-major
 * doubles in the reference's order (waters O,H,H first, then 29-site
 * surfactants, src/read_config.f90:16-38) and reduced units (sigma = 3.166 A,
 * epsilon = 650.2 J/mol, mass of O; velocities are displacements per step).
 * The engine copies them to its own device state, which persists between
 * calls.  Calls are synchronous unless named *_async.  One context is bound
 * to one GPU; contexts are independent and may be used from different
 * threads, one thread per context at a time.
 */
#ifndef SESP_H
#define SESP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SESP_ABI_VERSION 2

/* error codes */
#define SESP_OK 0
#define SESP_EINVAL 1      /* bad argument                                   */
#define SESP_ECUDA 2       /* CUDA runtime failure                           */
#define SESP_ENOMEM 3      /* device allocation failed                       */
#define SESP_ESTATE 4      /* call out of order (e.g. step before upload)    */
#define SESP_ECAPACITY 5   /* a cell or list exceeded its capacity           */
#define SESP_ESHAKE 6      /* SHAKE/RATTLE did not converge (state is kept)  */
#define SESP_EBUDGET 7     /* request exceeds the memory budget (serving)    */

/* precision of the force path */
#define SESP_PLAIN_FP64 0  /* every force term in FP64                       */
#define SESP_MIXED 1       /* FP32 pair, multipole and bonded arithmetic; FP64
                              for the constraint iterations, thermostat,
                              kinetic sums, positions and energy sums         */
#define SESP_MIXED_FP32C 2 /* SESP_MIXED with the constraint iterations in
                              FP32 (FP64 state and predictors, FP64 decisions
                              near the tolerance threshold)                   */
#define SESP_MIXED_COMP 3  /* SESP_MIXED with compensated (Kahan) FP32 sums of
                              the pair terms per site, in the pair field and
                              over its nine row partials                      */

/* force terms (bit mask for sesp_force_terms) */
#define SESP_T_NEAR 1        /* short-range LJ + Coulomb, src/eval[wS]*.f90   */
#define SESP_T_FAR 2         /* FMA local expansion, src/evalLjk4.f90         */
#define SESP_T_VALENCE 4     /* src/eval_valence.f90                          */
#define SESP_T_DIHEDRAL 8    /* src/eval_dihedral.f90                         */
#define SESP_T_BERENDSEN 16  /* src/eval_dihedral_berendsen.f90               */
#define SESP_T_INTERNAL 32   /* src/eval_surfactant_internal.f90              */
#define SESP_T_SUBTRACT 64   /* src/eval_subtract_fma.f90                     */
#define SESP_T_WALL 128      /* src/eval_wall.f90                             */
#define SESP_T_GRAPHITE 256  /* src/eval_graphite.f90                         */
#define SESP_T_BOND 512      /* harmonic chain bonds (configuration preset)   */
#define SESP_T_ALL 1023

/* force field and boundaries (sesp_params.preset) */
#define SESP_PRESET_REFERENCE 0  /* the reference's: SPC/E water, 29-site
                                    trisiloxane surfactants with rigid bonds,
                                    closed box with walls (src/init_arrays.f90,
                                    src/eval_wall.f90)                       */
#define SESP_PRESET_CONFIG 1     /* the benchmark configurations': SPC water
                                    (O -0.82 / H +0.41), 12-bead united-atom
                                    chains with harmonic bonds (1.53 A), 112
                                    degree angles and triple-cosine dihedrals,
                                    graphite with Lorentz-Berthelot carbon
                                    parameters (sigma 3.4 A, eps 0.23 kJ/mol)
                                    on every LJ site of the bottom cell
                                    layers, box periodic in x and y (far field
                                    over the 3 x 3 supercell of images), walls
                                    at the z faces only.  Cells: multiples of
                                    4, at least 8 in x and y.  Surfactants are
                                    the 12-bead chains; the constraint count
                                    per chain is 0.                          */

typedef struct sesp_ctx sesp_ctx;

typedef struct {
    int n_cells[3];        /* L4 cells per axis, multiples of 4; the reference
                              uses 12 x 12 x 12 (3 x 3 x 3 ranks of 4^3 cells,
                              src/mybox.cmns:55-57, src/init_box_dimensions.f90) */
    int precision;         /* SESP_PLAIN_FP64, SESP_MIXED or SESP_MIXED_FP32C */
    int rebuild_interval;  /* steps between list / far-field rebuilds; ifar = 10
                              (src/mybox.f90:24)                               */
    int graphite_on;       /* apply src/eval_graphite.f90                     */
    double tr;             /* thermostat target temperature, 3.81087
                              (src/mybox.f90:48)                               */
    double tau_steps;      /* thermostat relaxation time in steps, 7.5
                              (src/mybox.f90:49)                               */
    double shake_tol;      /* 1e-4 (src/move_w1_a.f90:19)                     */
    int shake_maxit;       /* 100 (src/move_w1_a.f90:20)                      */
    int device;            /* CUDA device ordinal                             */
    int max_cell_sites;    /* capacity of one cell, 0 = default (1024)        */
    int preset;            /* SESP_PRESET_REFERENCE (default) or
                              SESP_PRESET_CONFIG; sesp_default_config_params
                              fills the configuration preset's settings       */
} sesp_params;

/* library and error handling */
int sesp_abi_version(void);
int sesp_last_error(char *buf, size_t len);
int sesp_default_params(sesp_params *p);
/* the configuration preset's defaults: n_cells 8 x 8 x 8, target 300 K
 * (3.8363 reduced), Nose-Hoover relaxation 0.1 ps (50 steps), SHAKE / RATTLE
 * tolerance 1e-8, 100 iterations */
int sesp_default_config_params(sesp_params *p);

/* lifecycle.  sesp_create allocates nothing that depends on the system size;
 * sesp_upload_state sizes the device state for the system.
 * Replaces: src/mybox.f90:19-60 (init_box_dimensions, init_arrays,
 * read_config, read_graphite; velocities as given, init_temp is host side). */
int sesp_create(const sesp_params *p, sesp_ctx **out);
int sesp_destroy(sesp_ctx *ctx);
int sesp_upload_state(sesp_ctx *ctx, int n_water, int n_surf, const double *pos, const double *vel,
                      int n_carbon, const double *carbons);
/* any of pos / vel / acc may be NULL */
int sesp_download_state(sesp_ctx *ctx, double *pos, double *vel, double *acc);
/* velocities and accelerations in, e.g. to resume a saved state; eta is
 * given to every replica (sesp_set_eta_batch sets them one by one) */
int sesp_set_state(sesp_ctx *ctx, const double *pos, const double *vel, const double *acc, double eta);

/* several independent systems ("replicas") in one context, laid out back to
 * back and advanced together by every launch (batched ensembles).  Per
 * replica q: n_water[q], n_surf[q], its cells n_cells[3q..3q+2] and n_carbon[q];
 * pos / vel hold the replicas' sites one after the other, carbons their
 * carbons.  Each replica keeps its own thermostat variable.  Every other
 * entry point then acts on all replicas; state arrays are concatenated. */
int sesp_upload_batch(sesp_ctx *ctx, int n_rep, const int *n_water, const int *n_surf, const int *n_cells,
                      const double *pos, const double *vel, const int *n_carbon, const double *carbons);
/* number of replicas in the context (negative on error) */
int sesp_replica_count(sesp_ctx *ctx);
/* the thermostat variable of every replica */
int sesp_get_eta_batch(sesp_ctx *ctx, double *eta);
/* set it per replica (sesp_replica_count values), e.g. when a run moves
 * into another batched context at a rebuild boundary */
int sesp_set_eta_batch(sesp_ctx *ctx, const double *eta);
/* SHAKE / RATTLE non-convergences since upload, per replica (the split of
 * sesp_counters' [0]) */
int sesp_failures_batch(sesp_ctx *ctx, int64_t *out);

/* the force section.  rebuild = 1 replaces src/mybox.f90:142-152 (molecule
 * re-keying), :163-175 (list builders, multipoles and translations) and
 * :183-223 (all force kernels); rebuild = 0 replaces src/mybox.f90:179-223
 * (up_downSR_isr's intra-cell kernels, evalLjk4 and the 33 neighbour
 * kernels) with the lists and local expansions frozen at the last rebuild. */
int sesp_force(sesp_ctx *ctx, int rebuild);
/* the same with only the terms in `terms` (SESP_T_* mask); for tests */
int sesp_force_terms(sesp_ctx *ctx, int rebuild, int terms);
int sesp_download_forces(sesp_ctx *ctx, double *f);

/* src/init_accel.f90: a = F dt^2 / (2 m) after the first force call */
int sesp_init_accel(sesp_ctx *ctx);
/* move_surfactant_a, move_w1_a, move_w2_a (src/move_*_a.f90): Nose-Hoover
 * scaled predictor, SHAKE, kinetic sums and the eta update of
 * src/move_w2_a.f90:145-157 */
int sesp_move_a(sesp_ctx *ctx);
/* move_surfactant_b, move_w1_b, move_w2_b (src/move_*_b.f90): RATTLE */
int sesp_move_b(sesp_ctx *ctx);

/* one pass of the step loop body src/mybox.f90:136-227 for step number kb
 * (rebuild when kb mod rebuild_interval == 0) */
int sesp_step(sesp_ctx *ctx, int kb);
/* nsteps passes starting at kb0, launched as captured CUDA graphs of
 * rebuild_interval steps where possible */
int sesp_run(sesp_ctx *ctx, int kb0, int nsteps);
/* the same without waiting for completion; sesp_sync waits */
int sesp_run_async(sesp_ctx *ctx, int kb0, int nsteps);
int sesp_sync(sesp_ctx *ctx);
/* 0 when all work launched on the context has finished, 1 while some is
 * still running, negative on error (never blocks) */
int sesp_query(sesp_ctx *ctx);
/* device memory held by the context's state, in bytes */
int sesp_device_bytes(sesp_ctx *ctx, int64_t *bytes);

/* nsteps passes like sesp_run, each timed with CUDA events recorded on the
 * engine's stream around the step's graph launch.  With flush_l2 != 0 a
 * 256 MB buffer is written between steps, outside the timed intervals, so
 * every step starts with a cold L2.  step_ms receives nsteps durations. */
int sesp_run_timed(sesp_ctx *ctx, int kb0, int nsteps, int flush_l2, double *step_ms);

/* diagnostics */
/* ordered near-field site pairs and LJ-active pairs within rc of the current
 * state and lists (sizes the pair kernel's algorithmic flop count) */
int sesp_pair_counts(sesp_ctx *ctx, int64_t out[2]);
/* src/compute_temperature.f90:240-242: sum m v^2 / dt^2 / dof over every
 * replica, dof = 3 sites - constraints; an FP64 reduction on the device in
 * a fixed order (64 slices per replica, then their sum), then one double per
 * replica to the host (the reference reduces per rank and adds with an allreduce,
 * src/compute_temperature.f90:239-242) */
int sesp_temperature(sesp_ctx *ctx, double *t);
int sesp_get_eta(sesp_ctx *ctx, double *eta);
int sesp_set_eta(sesp_ctx *ctx, double eta);
/* energies (the reference computes none; these integrate its force laws):
 * [0] near Coulomb, [1] near LJ, [2] far field incl. the intramolecular
 * correction, [3] intramolecular pairs, [4] angles + dihedrals, [5] walls,
 * [6] graphite, [7] kinetic */
int sesp_energies(sesp_ctx *ctx, double out[8]);
/* Launch shape of the pair field: target sites per work item (32 or 64, or
 * 128 on the mixed paths, up to 4 per lane) and CTAs per SM of its
 * persistent kernel (default: 64 at the largest CTAs per SM).  The shape
 * changes no result, only the time.  sesp_autotune times every candidate on the current state
 * (a force call must have built the cell lists) and keeps the fastest:
 * out = {tile, ctas_per_sm, largest ctas_per_sm}.  New for the GPU build (the
 * reference has no launch shapes). */
int sesp_autotune(sesp_ctx *ctx, int out[3]);
int sesp_tuning(sesp_ctx *ctx, int out[3]);
int sesp_set_tuning(sesp_ctx *ctx, int tile, int ctas_per_sm);
/* Launch shape of the constraint halves on the mixed paths: surfactant warps
 * per CTA (1..4) and surfactants per such warp (1..2 on SESP_MIXED, whose
 * FP64 sweeps take 12 lanes per molecule, 1..8 on SESP_MIXED_FP32C).  The
 * surfactants'
 * FP64 sweep chains start on the first
 * ceil(n_surf / (mols_per_warp surf_warps)) CTAs (one CTA per SM), waters
 * fill every other warp.  The shape changes no result, only the time;
 * sesp_autotune picks it on the mixed paths (restoring the state its trials
 * change).  out = {surf_warps, mols_per_warp, largest surf_warps, largest
 * mols_per_warp}.  New for the GPU build. */
int sesp_set_constraint_tuning(sesp_ctx *ctx, int surf_warps, int mols_per_warp);
int sesp_constraint_tuning(sesp_ctx *ctx, int out[4]);
/* The energies of sesp_energies, bit for bit, without allocating: no
 * cudaMalloc or cudaFree (sesp_energies does both on every call, and cudaFree
 * waits for every stream on the device).  For callers that share the GPU with
 * runs they must not stall, or that have handed out all device memory.  Its
 * scratch is one fixed array in the library (6.1 MiB on every GPU that loads
 * it); contexts above SESP_NOALLOC_MAX_SITES sites or SESP_NOALLOC_MAX_SURF
 * surfactants get SESP_EINVAL.  The first call on a device looks up the
 * array's device address, so make it before any stream capture; the address is
 * kept for the life of the process, so do not call it after a reset of the
 * device's primary context (cudaDeviceReset).  A call first waits for the work
 * already queued on its context; calls on one device then share the array and
 * take turns under a lock.  No counterpart in the
 * reference, which computes no energies. */
#define SESP_NOALLOC_MAX_SITES 131072
#define SESP_NOALLOC_MAX_SURF 4096
int sesp_energies_static(sesp_ctx *ctx, double out[8]);
/* counts: [0] SHAKE/RATTLE non-convergences since upload, [1] capacity
 * overflows, [2] sites in no cell, [3] steps done, [4] max sites in a cell,
 * [5] near-field ordered pairs of the last rebuild, [6] LJ-eligible pairs,
 * [7] molecule-list entries that failed their bounds check and were skipped
 * (always 0 unless device memory was corrupted) */
int sesp_counters(sesp_ctx *ctx, int64_t out[8]);
/* The reference's consistency checks, from the cell lists of the last force
 * call, 8 values per replica (out holds 8 x sesp_replica_count):
 *   [0] molecules whose sites all lie in a cell, [1] molecules uploaded,
 *   [2] total charge of the sites in cells, [3] water O in cells,
 *   [4] water H in cells, [5] waters uploaded, [6] sites in no cell,
 *   [7] the warning bits of sesp_check_flags.
 * Replaces the counts and messages of get_molecule_count
 * (src/get_molecule_count.f90:16-57: "MOLECULES LOST") and of computeOnm4
 * (src/computeOnm4.f90:18-212: total charge, O:H ratio, missing oxygen),
 * which print and carry on. */
int sesp_checks(sesp_ctx *ctx, double *out);
#define SESP_CHECK_MOLECULES_LOST 1   /* [0] != [1] */
#define SESP_CHECK_CHARGE 2           /* [2]^2 > 0.001 */
#define SESP_CHECK_OH_RATIO 4         /* integer [4] / [3] != 2 (H without O counts too) */
#define SESP_CHECK_MISSING_OXYGEN 8   /* [3] != [5] */
/* Warning bits of one replica's counts c[0..6] (layout of sesp_checks); a
 * host function, no GPU needed (src/get_molecule_count.f90:57,
 * src/computeOnm4.f90:210-212). */
int sesp_check_flags(const double c[7]);
/* Velocities scaled by sqrt(target / T), T the temperature of
 * sesp_temperature before the call (returned in t_before unless null);
 * src/compute_temperature.f90's rescaling variant
 * (src/compute_temperature_rescale.f90:242-276) with its target 3.9 as
 * SESP_RESCALE_TARGET.  SESP_EINVAL unless target > 0 and T > 0. */
#define SESP_RESCALE_TARGET 3.9
int sesp_rescale_temperature(sesp_ctx *ctx, double target, double *t_before);
/* average device time in ms per launch of each kernel family since the last
 * reset, measured with CUDA events on the engine's stream:
 * [0] near field, [1] local-expansion force, [2] move_a, [3] move_b,
 * [4] intramolecular + external, [5] rebuild (sort + lists), [6] far-field build */
int sesp_kernel_times(sesp_ctx *ctx, double out[8], int reset);
/* The FP32 fused multiply-add throughput of a device in TFLOP/s: a loop of
 * independent FMA chains over (SMs x 8) CTAs, best of 5 launches timed with
 * CUDA events.  The ceiling the FP32 pair field is measured against (the
 * reference has no counterpart; a diagnostic of the GPU build). */
int sesp_fp32_peak(int device, double *tflops);
int sesp_enable_timing(sesp_ctx *ctx, int on);

#ifdef __cplusplus
}
#endif

#endif
