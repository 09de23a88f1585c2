/*
 * TEST INFRASTRUCTURE ONLY - the CPU oracle.
 *
 * A plain-C, FP64 restatement of the reference's per-timestep
 * force-and-integrate path (jhalverson/surfactant_enhanced_spreading,
 * Fortran 90 + MPI).  The 27-rank 3x3x3 domain decomposition is collapsed
 * onto one global cell grid: every rank-local array of the reference is a
 * window of the global arrays held here, and halo copies are the global
 * entries themselves.  Each function cites the reference file:line it
 * follows.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load this library; the product path never does.
 *
 * Parity status: UNPINNED.  The reference ships no tests, fixtures or golden
 * vectors, and it cannot be compiled in this image (no Fortran compiler, no
 * MPI), so this restatement is checked only against hand-computable cases and
 * physical invariants (Newton's third law, finite-difference energies,
 * constraint residuals).
 *
 * Units are the reference's reduced units: length sigma = 3.166 A, energy
 * epsilon = 650.2 J/mol, mass m_O; velocities are displacements per step and
 * accelerations are F dt^2 / (2 m) (src/mybox.cmns:36-44).
 */
#ifndef ORC_H
#define ORC_H

#include <complex.h>
#include <stddef.h>
#include <stdint.h>

#define ORC_P 4
#define ORC_LP 25            /* p*p + 2p + 1, src/mybox.cmns:49-50 */
#define ORC_NSURF_SITE 29

/* An entry of a per-cell atom list, the global form of the reference's
 * 4-integer records (key cell, molecule, slot, site type), src/buildW2.f90:43-46. */
typedef struct {
    int key;    /* key (storage) cell of the molecule, global L4 index       */
    int mol;    /* global molecule index                                     */
    int gsite;  /* global site index                                         */
    int type;   /* site type within its molecule, 1-based as the reference   */
} orc_ent;

typedef struct {
    orc_ent *e;
    int n, cap;
} orc_list;

typedef struct {
    int *m;     /* molecule indices */
    int n, cap;
} orc_mlist;

typedef struct orc_sys {
    /* sizes */
    int nw, ns, nmol, nsite;
    int ncx, ncy, ncz, ncell;          /* global L4 grid (multiples of 4)   */
    int nrx, nry, nrz, nrank;          /* 4x4x4-cell "ranks"                */
    /* box, src/init_box_dimensions.f90:1-23 */
    double rs, rsdx, rsdy, rsdz, rhsx, rhsy, rhsz;
    /* state, site order: waters (O,H,H) then surfactants (29 sites) */
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *fx, *fy, *fz;
    /* per molecule */
    int *key;                          /* global L4 key cell                */
    int *w1;                           /* water: 1 = w1 (all sites in key cell) */
    /* per cell molecule storage (w1, w2, surfactant), by key cell */
    orc_mlist *cw1, *cw2, *cs;
    /* per cell atom lists (src/mybox.cmns:152-167) */
    orc_list *W2C, *W226, *W2nC, *W2n26, *W2nn;
    orc_list *SC, *S26, *SnC, *Sn26, *SnnC, *Snn26, *Snnn;
    /* isub: per surfactant site 28 slots, 0-terminated (src/mybox.cmns:187) */
    int *isub;
    /* FMA coefficients (src/mybox.cmns:189-190) */
    double complex *cO4, *cO3, *cO2, *cL4, *cL3, *cL2;
    /* graphite (fixed carbons) */
    int nc;
    double *gx, *gy, *gz;
    int graphite_on;
    /* thermostat, src/mybox.f90:44-52 */
    double eta, tr, pnh1, pnh2;
    double sv1, sv2, w1v1, w1v2, w2v1, w2v2;
    /* diagnostics */
    int shake_fail, rattle_fail;
    int64_t npair_coul, npair_lj;      /* pair counts of the last force call */
} orc_sys;

/* force-field tables, src/init_arrays.f90:88-840 */
typedef struct {
    double emw[4], ems[30];
    double rqw[4], rqs[30];
    double dsqw[4], dsqs[29];
    double th[37], rkth[37], dva[31], dvb[31], dvc[31];
    double sgss6[30][30], epss[30][30], sgws6[4][30], epws[4][30];
    double sgcs6[30], epcs[30];
    double rifact[34];
    int iself[43], jself[43], ibond[29], jbond[29];
    int iang[37], jang[37], kang[37];
    int idv[31], jdv[31], kdv[31], ldv[31];
} orc_tables;

extern orc_tables ORC_T;
extern const double ORC_SIGMA, ORC_EPSILON, ORC_RC, ORC_DELTA, ORC_RS, ORC_XPI;
extern const double ORC_DT, ORC_DTSQ, ORC_DTSQ2;

void orc_init_tables(void);

/* geometry helpers (src/ibox.f90, src/init_box_dimensions.f90) */
int orc_rank_of(const orc_sys *s, double x, double y, double z);          /* ibox2-1 */
void orc_rank_xyz(const orc_sys *s, int rank, int *rx, int *ry, int *rz);
void orc_rcen2(const orc_sys *s, int rank, double *cx, double *cy, double *cz);
int orc_local64(const orc_sys *s, int rank, double x, double y, double z); /* ibox64-1 */
int orc_keycell(const orc_sys *s, double x, double y, double z);
void orc_cell_xyz(const orc_sys *s, int c, int *ix, int *iy, int *iz);
int orc_cell_id(const orc_sys *s, int ix, int iy, int iz);                /* -1 if outside */
void orc_rcen4(const orc_sys *s, int c, double *cx, double *cy, double *cz);
int orc_isCentral(double x, double y, double z, double cx, double cy, double cz);
int orc_isNearest(double x, double y, double z, double cx, double cy, double cz);
extern const int ORC_KMID[26][3];

/* migration + list builders (src/delete_*.f90, src/build*.f90) */
void orc_classify(orc_sys *s);
void orc_build_lists(orc_sys *s);
void orc_buildinternal(orc_sys *s);

/* pair kernels (src/eval[wS]*.f90) */
int orc_threads(void);                       /* OpenMP threads of the pair kernels and the FMA (1 without OpenMP) */
void orc_eval_pairs_intracell(orc_sys *s);   /* called from src/up_downSR_isr.f90:324-329 */
void orc_eval_pairs_neighbour(orc_sys *s);   /* src/mybox.f90:185-217 */

/* FMA (src/computeOnm*.f90, src/computeLjk*.f90, src/shiftLjk*.f90, src/evalLjk4.f90) */
void orc_fma_build(orc_sys *s);
void orc_evalLjk4(orc_sys *s);
double orc_fma_energy(const orc_sys *s);
/* single expansion operations of the same formulas (used by orc_cfg.c) */
void orc_p2m_add(double complex *O, double q, double dx, double dy, double dz);
void orc_m2m_apply(const double complex *O, double dx, double dy, double dz, double complex *Op);
void orc_m2l_apply(const double complex *O, double dx, double dy, double dz, double complex *L);
void orc_l2l_apply(const double complex *L, double dx, double dy, double dz, double complex *Lc);
void orc_l2p_apply(const double complex *L, double rx, double ry, double rz, double rqq, double *fx, double *fy,
                   double *fz, double *phi);
double orc_legendre(int l, int m, double x);

/* intramolecular, external (src/eval_valence.f90 ... src/eval_graphite.f90) */
void orc_eval_valence(orc_sys *s);
void orc_eval_dihedral(orc_sys *s, int berendsen);
void orc_eval_surfactant_internal(orc_sys *s);
void orc_eval_subtract_fma(orc_sys *s);
void orc_eval_wall(orc_sys *s);
void orc_eval_graphite(orc_sys *s);

/* integrator (src/move_*.f90, src/nh_*.f90, src/init_accel.f90) */
void orc_move_a(orc_sys *s);
void orc_move_b(orc_sys *s);
void orc_init_accel(orc_sys *s);
double orc_temperature(const orc_sys *s);

/* list helpers */
void orc_list_push(orc_list *l, int key, int mol, int gsite, int type);
void orc_mlist_push(orc_mlist *l, int m);

static inline int orc_site_type(const orc_sys *s, int gsite) {
    return gsite < 3 * s->nw ? (gsite % 3) + 1 : ((gsite - 3 * s->nw) % ORC_NSURF_SITE) + 1;
}
static inline int orc_is_water(const orc_sys *s, int gsite) { return gsite < 3 * s->nw; }
static inline int orc_mol_of(const orc_sys *s, int gsite) {
    return gsite < 3 * s->nw ? gsite / 3 : s->nw + (gsite - 3 * s->nw) / ORC_NSURF_SITE;
}
static inline int orc_first_site(const orc_sys *s, int mol) {
    return mol < s->nw ? 3 * mol : 3 * s->nw + ORC_NSURF_SITE * (mol - s->nw);
}

#endif
