/*
 * TEST INFRASTRUCTURE ONLY (CPU oracle; parity unpinned - see orc.h).
 * Driver of the restated step (src/mybox.f90:130-241), energies, and a
 * second, independent near-field evaluation by the located-cell rule the
 * reference's 39 list kernels add up to, used to cross-check the two.
 * Exported with C linkage for ctypes.
 */
#include "orc.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define T ORC_T
#define LP ORC_LP

/* force terms, bit mask (the same bits the GPU engine's debug entry uses) */
enum {
    ORC_T_NEAR = 1, ORC_T_FAR = 2, ORC_T_VALENCE = 4, ORC_T_DIHEDRAL = 8, ORC_T_BERENDSEN = 16,
    ORC_T_INTERNAL = 32, ORC_T_SUBTRACT = 64, ORC_T_WALL = 128, ORC_T_GRAPHITE = 256, ORC_T_ALL = 511
};

static void *xcalloc(size_t n, size_t sz) { void *p = calloc(n ? n : 1, sz); return p; }

orc_sys *orc_create(int nw, int ns, int ncx, int ncy, int ncz, const double *pos, const double *vel,
                    int nc, const double *carbons, int graphite_on) {
    static int tables_done = 0;
    if (!tables_done) { orc_init_tables(); tables_done = 1; }
    if (ncx % 4 || ncy % 4 || ncz % 4 || ncx <= 0 || ncy <= 0 || ncz <= 0) return NULL;
    orc_sys *s = (orc_sys *)xcalloc(1, sizeof(orc_sys));
    s->nw = nw; s->ns = ns; s->nmol = nw + ns; s->nsite = 3 * nw + ORC_NSURF_SITE * ns;
    s->ncx = ncx; s->ncy = ncy; s->ncz = ncz; s->ncell = ncx * ncy * ncz;
    s->nrx = ncx / 4; s->nry = ncy / 4; s->nrz = ncz / 4; s->nrank = s->nrx * s->nry * s->nrz;
    s->rs = ORC_RS;
    s->rsdx = ncx * ORC_RS; s->rsdy = ncy * ORC_RS; s->rsdz = ncz * ORC_RS;
    s->rhsx = s->rsdx / 2.0; s->rhsy = s->rsdy / 2.0; s->rhsz = s->rsdz / 2.0;
    int N = s->nsite;
    double **arrs[12] = {&s->x, &s->y, &s->z, &s->vx, &s->vy, &s->vz, &s->ax, &s->ay, &s->az, &s->fx, &s->fy, &s->fz};
    for (int i = 0; i < 12; i++) *arrs[i] = (double *)xcalloc(N, sizeof(double));
    for (int g = 0; g < N; g++) {
        s->x[g] = pos[3 * g]; s->y[g] = pos[3 * g + 1]; s->z[g] = pos[3 * g + 2];
        if (vel) { s->vx[g] = vel[3 * g]; s->vy[g] = vel[3 * g + 1]; s->vz[g] = vel[3 * g + 2]; }
    }
    s->key = (int *)xcalloc(s->nmol, sizeof(int));
    s->w1 = (int *)xcalloc(s->nmol, sizeof(int));
    s->cw1 = (orc_mlist *)xcalloc(s->ncell, sizeof(orc_mlist));
    s->cw2 = (orc_mlist *)xcalloc(s->ncell, sizeof(orc_mlist));
    s->cs = (orc_mlist *)xcalloc(s->ncell, sizeof(orc_mlist));
    orc_list **ls[12] = {&s->W2C, &s->W226, &s->W2nC, &s->W2n26, &s->W2nn, &s->SC, &s->S26,
                         &s->SnC, &s->Sn26, &s->SnnC, &s->Snn26, &s->Snnn};
    for (int i = 0; i < 12; i++) *ls[i] = (orc_list *)xcalloc(s->ncell, sizeof(orc_list));
    s->isub = (int *)xcalloc((size_t)28 * ORC_NSURF_SITE * (ns ? ns : 1), sizeof(int));
    int n3 = s->ncell / 8;
    s->cO4 = (double complex *)xcalloc((size_t)LP * s->ncell, sizeof(double complex));
    s->cL4 = (double complex *)xcalloc((size_t)LP * s->ncell, sizeof(double complex));
    s->cO3 = (double complex *)xcalloc((size_t)LP * n3, sizeof(double complex));
    s->cL3 = (double complex *)xcalloc((size_t)LP * n3, sizeof(double complex));
    s->cO2 = (double complex *)xcalloc((size_t)LP * s->nrank, sizeof(double complex));
    s->cL2 = (double complex *)xcalloc((size_t)LP * s->nrank, sizeof(double complex));
    s->nc = nc;
    s->gx = (double *)xcalloc(nc, sizeof(double)); s->gy = (double *)xcalloc(nc, sizeof(double)); s->gz = (double *)xcalloc(nc, sizeof(double));
    for (int j = 0; j < nc; j++) { s->gx[j] = carbons[3 * j]; s->gy[j] = carbons[3 * j + 1]; s->gz[j] = carbons[3 * j + 2]; }
    s->graphite_on = graphite_on;
    /* src/mybox.f90:44-52 with the system's own site and constraint counts */
    int np = 3 * nw + ORC_NSURF_SITE * ns, ncon = 3 * nw + 28 * ns, df = 3 * np - ncon;
    s->tr = 3.81087;
    double rlx = 7.5 * ORC_DT;
    s->pnh1 = ORC_DT / df / s->tr / (rlx * rlx);
    s->pnh2 = -2.0 * df * s->tr;
    s->eta = 0.0;
    return s;
}

void orc_destroy(orc_sys *s) {
    if (!s) return;
    double *arrs[12] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->ax, s->ay, s->az, s->fx, s->fy, s->fz};
    for (int i = 0; i < 12; i++) free(arrs[i]);
    for (int c = 0; c < s->ncell; c++) {
        free(s->cw1[c].m); free(s->cw2[c].m); free(s->cs[c].m);
        orc_list *ls[12] = {s->W2C, s->W226, s->W2nC, s->W2n26, s->W2nn, s->SC, s->S26, s->SnC, s->Sn26, s->SnnC, s->Snn26, s->Snnn};
        for (int i = 0; i < 12; i++) free(ls[i][c].e);
    }
    free(s->cw1); free(s->cw2); free(s->cs);
    free(s->W2C); free(s->W226); free(s->W2nC); free(s->W2n26); free(s->W2nn); free(s->SC); free(s->S26);
    free(s->SnC); free(s->Sn26); free(s->SnnC); free(s->Snn26); free(s->Snnn);
    free(s->key); free(s->w1); free(s->isub);
    free(s->cO4); free(s->cL4); free(s->cO3); free(s->cL3); free(s->cO2); free(s->cL2);
    free(s->gx); free(s->gy); free(s->gz);
    free(s);
}

/* the force section of one step, src/mybox.f90:140-223 (rebuild = kb mod 10 == 0).
 * Only the terms selected in mask are added; forces are zeroed first. */
void orc_force_terms(orc_sys *s, int rebuild, int mask) {
    for (int g = 0; g < s->nsite; g++) { s->fx[g] = 0.0; s->fy[g] = 0.0; s->fz[g] = 0.0; }
    s->npair_coul = 0; s->npair_lj = 0;
    if (rebuild) {
        orc_classify(s);        /* delete_* / add_*, src/mybox.f90:142-152 */
        orc_build_lists(s);     /* buildW2, buildS, build*n*, src/up_downSR_isr_update.f90:324-325 */
        orc_buildinternal(s);   /* src/up_downSR_isr_update.f90:326 */
    }
    if (mask & ORC_T_NEAR) orc_eval_pairs_intracell(s);
    if (mask & ORC_T_VALENCE) orc_eval_valence(s);
    if (mask & ORC_T_DIHEDRAL) orc_eval_dihedral(s, 0);
    if (mask & ORC_T_BERENDSEN) orc_eval_dihedral(s, 1);
    if (mask & ORC_T_INTERNAL) orc_eval_surfactant_internal(s);
    if (mask & ORC_T_SUBTRACT) orc_eval_subtract_fma(s);
    if (mask & ORC_T_WALL) orc_eval_wall(s);
    if (mask & ORC_T_GRAPHITE) orc_eval_graphite(s);
    if (rebuild) orc_fma_build(s);  /* src/mybox.f90:171-175 */
    if (mask & ORC_T_FAR) orc_evalLjk4(s);
    if (mask & ORC_T_NEAR) orc_eval_pairs_neighbour(s);
}

void orc_force(orc_sys *s, int rebuild) { orc_force_terms(s, rebuild, ORC_T_ALL); }
void orc_move_a_api(orc_sys *s) { orc_move_a(s); }
void orc_move_b_api(orc_sys *s) { orc_move_b(s); }
void orc_init_accel_api(orc_sys *s) { orc_init_accel(s); }
double orc_temperature_api(orc_sys *s) { return orc_temperature(s); }

/* one pass of the step loop body, src/mybox.f90:136-227 */
void orc_step(orc_sys *s, int kb) {
    orc_move_a(s);
    orc_force(s, kb % 10 == 0);
    orc_move_b(s);
}

void orc_run(orc_sys *s, int kb0, int nsteps) {
    for (int k = 0; k < nsteps; k++) orc_step(s, kb0 + k);
}

/* which: 0 positions, 1 velocities, 2 accelerations, 3 forces; (nsite, 3) */
void orc_get(const orc_sys *s, int which, double *out) {
    const double *a[4][3] = {{s->x, s->y, s->z}, {s->vx, s->vy, s->vz}, {s->ax, s->ay, s->az}, {s->fx, s->fy, s->fz}};
    for (int g = 0; g < s->nsite; g++)
        for (int d = 0; d < 3; d++) out[3 * g + d] = a[which][d][g];
}
void orc_set(orc_sys *s, int which, const double *in) {
    double *a[4][3] = {{s->x, s->y, s->z}, {s->vx, s->vy, s->vz}, {s->ax, s->ay, s->az}, {s->fx, s->fy, s->fz}};
    for (int g = 0; g < s->nsite; g++)
        for (int d = 0; d < 3; d++) a[which][d][g] = in[3 * g + d];
}
double orc_get_eta(const orc_sys *s) { return s->eta; }
void orc_set_eta(orc_sys *s, double eta) { s->eta = eta; }
int orc_fail_count(const orc_sys *s) { return s->shake_fail + s->rattle_fail; }
void orc_pair_counts(const orc_sys *s, int64_t *out) { out[0] = s->npair_coul; out[1] = s->npair_lj; }
void orc_get_key(const orc_sys *s, int *key, int *w1) {
    for (int m = 0; m < s->nmol; m++) { key[m] = s->key[m]; w1[m] = s->w1[m]; }
}
void orc_get_fma(const orc_sys *s, int which, double *out) {
    const double complex *src = which == 0 ? s->cO4 : s->cL4;
    for (size_t i = 0; i < (size_t)LP * s->ncell; i++) { out[2 * i] = creal(src[i]); out[2 * i + 1] = cimag(src[i]); }
}

/* Located cell of every site at the last rebuild: a w1 water's sites sit in
 * its key cell, every other site in the cell whose Central test it passes.
 * -1 for a site in no list the near-field kernels visit as i side. */
void orc_located(const orc_sys *s, int *loc) {
    for (int g = 0; g < s->nsite; g++) loc[g] = -1;
    for (int c = 0; c < s->ncell; c++) {
        for (int a = 0; a < s->cw1[c].n; a++)
            for (int t = 0; t < 3; t++) loc[3 * s->cw1[c].m[a] + t] = c;
        const orc_list *L[5] = {&s->W2C[c], &s->W2nC[c], &s->SC[c], &s->SnC[c], &s->SnnC[c]};
        for (int l = 0; l < 5; l++)
            for (int a = 0; a < L[l]->n; a++) loc[L[l]->e[a].gsite] = c;
    }
}

/* LJ parameters of a site pair by site kind: water O-O (1), water O with a
 * surfactant site or surfactant-surfactant (2, tabulated), none (0) */
static int lj_of(const orc_sys *s, int gi, int gj, double *eps, double *sg6) {
    int wi = orc_is_water(s, gi), wj = orc_is_water(s, gj);
    int ti = orc_site_type(s, gi), tj = orc_site_type(s, gj);
    if (wi && wj) return (ti == 1 && tj == 1) ? 1 : 0;
    if (wi && !wj) { if (ti != 1) return 0; *eps = T.epws[1][tj]; *sg6 = T.sgws6[1][tj]; return 2; }
    if (!wi && wj) { if (tj != 1) return 0; *eps = T.epws[1][ti]; *sg6 = T.sgws6[1][ti]; return 2; }
    *eps = T.epss[ti][tj]; *sg6 = T.sgss6[ti][tj]; return 2;
}
static inline double charge_of(const orc_sys *s, int g) {
    return orc_is_water(s, g) ? T.rqw[orc_site_type(s, g)] : T.rqs[orc_site_type(s, g)];
}

/* Near field by the located-cell rule: every site gets the Coulomb force of
 * all sites of other molecules located in the 27 cells around its own cell,
 * plus truncated LJ by site kind.  Writes forces (nsite,3) and the pair
 * energies e[0] Coulomb, e[1] LJ (each unordered pair once). */
void orc_near_generic(const orc_sys *s, double *f, double *e) {
    int *loc = (int *)malloc(sizeof(int) * s->nsite);
    orc_located(s, loc);
    int *cnt = (int *)calloc(s->ncell + 1, sizeof(int));
    for (int g = 0; g < s->nsite; g++) if (loc[g] >= 0) cnt[loc[g] + 1]++;
    for (int c = 0; c < s->ncell; c++) cnt[c + 1] += cnt[c];
    int *fill = (int *)calloc((size_t)s->ncell + 1, sizeof(int));
    int *bin = (int *)malloc(sizeof(int) * (s->nsite ? s->nsite : 1));
    for (int g = 0; g < s->nsite; g++) if (loc[g] >= 0) bin[cnt[loc[g]] + fill[loc[g]]++] = g;
    double ec = 0.0, el = 0.0;
    for (int g = 0; g < s->nsite; g++) {
        f[3 * g] = f[3 * g + 1] = f[3 * g + 2] = 0.0;
        if (loc[g] < 0) continue;
        int ix, iy, iz;
        orc_cell_xyz(s, loc[g], &ix, &iy, &iz);
        int mi = orc_mol_of(s, g);
        double qi = charge_of(s, g) * ORC_XPI;
        double fx = 0, fy = 0, fz = 0;
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int c = orc_cell_id(s, ix + dx, iy + dy, iz + dz);
                    if (c < 0) continue;
                    for (int b = cnt[c]; b < cnt[c + 1]; b++) {
                        int h = bin[b];
                        if (orc_mol_of(s, h) == mi) continue;
                        double xij = s->x[g] - s->x[h], yij = s->y[g] - s->y[h], zij = s->z[g] - s->z[h];
                        double rsq = xij * xij + yij * yij + zij * zij, r = sqrt(rsq);
                        double qq = qi * charge_of(s, h);
                        double ft = qq / (r * r * r);
                        ec += 0.5 * qq / r;
                        double eps = 0, sg6 = 0;
                        int lj = lj_of(s, g, h, &eps, &sg6);
                        if (lj && r <= ORC_RC) {
                            double rsi = 1.0 / rsq, r6 = rsi * rsi * rsi;
                            if (lj == 1) { eps = 1.0; sg6 = 1.0; }
                            ft += 48.0 * eps * sg6 * r6 * (sg6 * r6 - 0.5) * rsi;
                            el += 0.5 * 4.0 * eps * (sg6 * sg6 * r6 * r6 - sg6 * r6);
                        }
                        fx += xij * ft; fy += yij * ft; fz += zij * ft;
                    }
                }
        f[3 * g] = fx; f[3 * g + 1] = fy; f[3 * g + 2] = fz;
    }
    if (e) { e[0] = ec; e[1] = el; }
    free(loc); free(cnt); free(fill); free(bin);
}

void orc_intra_energies(orc_sys *s, double *out);

/* energies of the current state with the lists and cL4 of the last force
 * call: [0] near Coulomb, [1] near LJ, [2] far field incl. the intramolecular
 * correction, [3] intramolecular pairs, [4] angles + dihedrals, [5] walls,
 * [6] graphite, [7] kinetic (1/2 sum m v^2 / dt^2) */
void orc_energies(orc_sys *s, double *out) {
    double *f = (double *)malloc(sizeof(double) * 3 * (s->nsite ? s->nsite : 1));
    double en[2];
    orc_near_generic(s, f, en);
    free(f);
    double ei[5];
    orc_intra_energies(s, ei);
    double kin = 0.0;
    for (int g = 0; g < s->nsite; g++) {
        double m = orc_is_water(s, g) ? T.emw[orc_site_type(s, g)] : T.ems[orc_site_type(s, g)];
        kin += 0.5 * m * (s->vx[g] * s->vx[g] + s->vy[g] * s->vy[g] + s->vz[g] * s->vz[g]);
    }
    out[0] = en[0]; out[1] = en[1];
    out[2] = orc_fma_energy(s) + ei[2];
    out[3] = ei[1]; out[4] = ei[0]; out[5] = ei[3]; out[6] = ei[4];
    out[7] = kin / ORC_DTSQ;
}

/* reference constants for the host side of the tests */
void orc_constants(double *out) {
    orc_init_tables();
    out[0] = ORC_SIGMA; out[1] = ORC_EPSILON; out[2] = ORC_RC; out[3] = ORC_RS; out[4] = ORC_XPI;
    out[5] = ORC_DT; out[6] = T.dsqw[1]; out[7] = T.dsqw[2];
}
void orc_table_dsqs(double *out) { orc_init_tables(); for (int i = 0; i < 28; i++) out[i] = T.dsqs[i + 1]; }
void orc_table_bonds(int *out) { orc_init_tables(); for (int i = 0; i < 28; i++) { out[2 * i] = T.ibond[i + 1]; out[2 * i + 1] = T.jbond[i + 1]; } }
