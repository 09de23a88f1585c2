/*
 * sesp_common.h - COMMON-block compatibility layer of the GB300 engine.
 *
 * The reference keeps its state in per-rank COMMON arrays
 * (src/mybox.cmns:125-200 declarations, :207-259 blocks): each of the
 * 3 x 3 x 3 MPI ranks owns a domain of 4 x 4 x 4 L4 cells and stores
 *   - water positions in rxw1(nw3, 216) ("w1", all three sites in the same
 *     L4 cell of the domain; 6^3 cells = the 4^3 central cells and one cell
 *     of halo) or rxw2(nw3, 512) ("w2", the others; 8^3 cells, two of halo),
 *   - surfactant positions in rxs(ns29, 1000) (10^3 cells, three of halo),
 *   - velocities and accelerations of the central cells in vxw1(nw3, 64) ...,
 *   - forces in fxw1(nw3, 216), fxw2(nw3, 512), fxs(ns29, 1000),
 *   - molecule counts per cell in ictw1(216), ictw2(512), icts(1000),
 *   - the thermostat scalars in /cmn50/ (tr, pnh1, pnh2, eta, ...),
 * a molecule's sites in consecutive slots k of its cell's column (Fortran
 * column-major: rxw1(k, c) is element (c - 1) nw3 + k - 1).
 *
 * This layer converts between that layout and the engine's molecule order,
 * and exports the step loop's calls under their gfortran names
 * (init_accel_, move_surfactant_a_, move_w1_a_, move_w2_a_, evalforces_,
 * move_surfactant_b_, move_w1_b_, move_w2_b_) so that a driver written
 * against the COMMON arrays keeps reading and writing them.  It is host code
 * over the public C ABI of sesp.h; the engine's device state stays the
 * authoritative copy and the COMMON arrays are its mirror:
 *   - after sesp_cmn_attach: the engine holds the COMMON contents;
 *   - after init_accel_: accelerations written back;
 *   - after move_surfactant_a_: positions, velocities and eta written back;
 *     on rebuild steps (kb mod rebuild_interval == 0) every molecule is first
 *     re-assigned to the domain, class and cell that src/read_config.f90:45-175
 *     gives for its new positions (what delete_* / add_* do in the reference);
 *   - after evalforces_: total forces written to the central cells' slots;
 *   - after move_surfactant_b_: velocities and accelerations written back.
 * The w1 / w2 / surfactant calls of one half are one engine call: the first
 * of them (move_surfactant_*_) does the work, the other two only check the
 * order.  Halo cells are not mirrored: their counts are set to 0 (the engine
 * needs no ghost copies; the reference's halo exchange and ghost-force
 * routines have nothing left to do).  Writes the driver makes into the
 * COMMON arrays reach the engine only through sesp_cmn_reload (e.g. after a
 * velocity rescale done in Fortran).
 *
 * Domains: n_cells (multiples of 4) give (n_cells[0] / 4) x (n_cells[1] / 4)
 * x (n_cells[2] / 4) domains, numbered d = ix + dx (iy + dy iz) like ibox2
 * (src/ibox.f90:128-139); the reference's 12 x 12 x 12 cells give its 27
 * ranks.  All domains' arrays are passed to this layer at once: one process
 * drives the one GPU.  An MPI driver keeps its per-rank COMMON and gathers
 * the ranks' 64 central columns of each array, and the counts, to that
 * process (one mpi_gatherv per array), scattering them back after each call.
 *
 * Engine molecule order set by sesp_cmn_attach: waters first, by domain,
 * then central cell (ix + 4 iy + 16 iz), then w1 before w2, then slot; then
 * surfactants by domain, central cell and slot.
 *
 * The reference's force field only (29-site surfactants): a context of the
 * configuration preset is rejected.
 *
 * Error convention: the C functions return 0 or a SESP_E* code (message in
 * sesp_last_error's buffer for engine errors, sesp_cmn_last_error for this
 * layer's own).  The gfortran-named subroutines return nothing, like the
 * reference's: on failure they print the message to stderr, skip their
 * work, and keep the first failure's code for sesp_cmn_status.
 */
#ifndef SESP_COMMON_H
#define SESP_COMMON_H

#include "sesp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* column heights of the reference build: nw3 = 3 nw, nw = 100 waters per
 * cell; ns29 = 29 ns, ns = 20 surfactants per cell (src/mybox.cmns:50-54) */
#define SESP_CMN_NW3 300
#define SESP_CMN_NS29 580
#define SESP_CMN_W1_CELLS 216      /* 6^3 */
#define SESP_CMN_W2_CELLS 512      /* 8^3 */
#define SESP_CMN_S_CELLS 1000      /* 10^3 */
#define SESP_CMN_CENTRAL 64        /* 4^3 */
#define SESP_CMN_NH 10             /* /cmn50/: tr pnh1 pnh2 eta sv1 sv2 w1v1 w1v2 w2v1 w2v2 */

/* molecule classes */
#define SESP_CMN_W1 0
#define SESP_CMN_W2 1
#define SESP_CMN_SURF 2

/* One domain's COMMON arrays (all pointers into caller-owned memory, laid
 * out exactly as the Fortran declarations; [3] = x, y, z arrays).  nh may be
 * NULL (eta is then not mirrored); force arrays may be NULL (forces are
 * then not mirrored). */
typedef struct {
    int nw3, ns29;     /* leading dimensions (SESP_CMN_NW3, SESP_CMN_NS29) */
    double *rw1[3];    /* /cmn05/ rxw1 ryw1 rzw1 (nw3, 216)  */
    double *rw2[3];    /* /cmn06/ rxw2 ryw2 rzw2 (nw3, 512)  */
    double *vw1[3];    /* /cmn07/ vxw1 vyw1 vzw1 (nw3, 64)   */
    double *vw2[3];    /* /cmn08/ vxw2 vyw2 vzw2 (nw3, 64)   */
    double *fw1[3];    /* /cmn09/ fxw1 fyw1 fzw1 (nw3, 216)  */
    double *fw2[3];    /* /cmn99/ fxw2 fyw2 fzw2 (nw3, 512)  */
    double *aw1[3];    /* /cmn10/ axw1 ayw1 azw1 (nw3, 64)   */
    double *aw2[3];    /* /cmn11/ axw2 ayw2 azw2 (nw3, 64)   */
    double *rs[3];     /* /cmn12/ rxs rys rzs (ns29, 1000)   */
    double *vs[3];     /* /cmn13/ vxs vys vzs (ns29, 64)     */
    double *as[3];     /* /cmn14/ axs ays azs (ns29, 64)     */
    double *fs[3];     /* /cmn15/ fxs fys fzs (ns29, 1000)   */
    int *ictw1;        /* /cmn16/ ictw1(216) */
    int *ictw2;        /* /cmn16/ ictw2(512) */
    int *icts;         /* /cmn16/ icts(1000) */
    double *nh;        /* /cmn50/ (SESP_CMN_NH doubles) or NULL */
} sesp_cmn_domain;

typedef struct sesp_cmn_map sesp_cmn_map;

/* ---- layout conversion (host only, no GPU) ---- */

/* number of domains of a cell grid (SESP_EINVAL unless every n_cells is a
 * positive multiple of 4) */
int sesp_cmn_domain_count(const int n_cells[3], int *ndom);
/* A map whose molecules are the ones in the domains' central cells, in the
 * engine order above; pos and vel (n_sites x 3, engine order) receive their
 * positions and velocities (either may be NULL; velocities of a domain that
 * binds no velocity arrays are left as the caller's buffer holds them). */
int sesp_cmn_map_from_domains(const sesp_cmn_domain *doms, const int n_cells[3], sesp_cmn_map **out,
                              int *n_water, int *n_surf, double *pos, double *vel);
int sesp_cmn_map_destroy(sesp_cmn_map *m);
/* re-assign every molecule from positions (engine order) by the rule of
 * src/read_config.f90:45-175: a water goes to the domain of its O; it is w1
 * when its three sites lie in that domain and in one L4 cell, else w2 in
 * the cell of its O; a surfactant goes to the cell of its 14th site.
 * SESP_EINVAL for a key site outside the box, SESP_ECAPACITY for a cell
 * beyond nw3 / 3 waters of a class or ns29 / 29 surfactants. */
int sesp_cmn_assign(sesp_cmn_map *m, const double *pos);
/* write the arrays given (any may be NULL) into the assigned slots; with
 * pos given, also set every cell count (central cells from the map, halo
 * cells 0) */
int sesp_cmn_scatter(const sesp_cmn_map *m, sesp_cmn_domain *doms, const double *pos, const double *vel,
                     const double *acc, const double *force);
/* read the arrays asked for (any may be NULL) from the assigned slots; a
 * molecule whose domain does not bind an array (NULL pointer) leaves that
 * output as it was */
int sesp_cmn_gather(const sesp_cmn_map *m, const sesp_cmn_domain *doms, double *pos, double *vel, double *acc);
/* where engine molecule `mol` sits: out = {domain, class, central cell, slot} */
int sesp_cmn_slot(const sesp_cmn_map *m, int mol, int out[4]);

/* ---- the attached job (one per process, like the COMMON blocks) ---- */

/* Create a context from p (reference preset), take the molecules of the
 * domains' central cells (positions, velocities; accelerations stay zero
 * until init_accel_) and the carbons, upload them, and make the domains the
 * mirror of the engine state.  kb0 is the number of the first step the
 * driver will take (99101 in src/mybox.f90:130).  The domains must stay
 * valid until sesp_cmn_detach. */
int sesp_cmn_attach(const sesp_params *p, sesp_cmn_domain *doms, int n_carbon, const double *carbons, int kb0);
int sesp_cmn_detach(void);
/* the attached job's context (NULL when none), e.g. for sesp_energies */
sesp_ctx *sesp_cmn_context(void);
/* the attached job's map (NULL when none) */
const sesp_cmn_map *sesp_cmn_current_map(void);
/* positions, velocities and accelerations read back from the COMMON
 * arrays into the engine (after the driver changed them); arrays the
 * domains do not bind keep the engine's values */
int sesp_cmn_reload(void);
/* first failure of a gfortran-named subroutine since attach (0 = none) */
int sesp_cmn_status(void);
/* message of this layer's last failure */
int sesp_cmn_last_error(char *buf, size_t len);

/* gfortran-named subroutines of the step loop (src/mybox.f90:125-227);
 * each takes the rank number by reference and ignores it (all domains are
 * attached) */
void init_accel_(int *my3d);
void move_surfactant_a_(int *my3d);
void move_w1_a_(int *my3d);
void move_w2_a_(int *comm3d, int *my3d);
/* the force section src/mybox.f90:161-223 (list builders and multipoles on
 * rebuild steps, the 33 pair kernels, evalLjk4, ghost forces) */
void evalforces_(int *my3d);
void move_surfactant_b_(int *my3d);
void move_w1_b_(int *my3d);
void move_w2_b_(int *my3d);
/* sesp_cmn_reload for a Fortran caller */
void sesp_cmn_reload_(int *my3d);

#ifdef __cplusplus
}
#endif

#endif
