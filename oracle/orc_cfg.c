/*
 * TEST INFRASTRUCTURE ONLY - the CPU oracle of the configuration preset.
 *
 * The workloads of the benchmark configurations (SPC water, 12-bead
 * united-atom surfactant chains with harmonic bonds, angles and OPLS-style
 * dihedrals, graphite with Lorentz-Berthelot carbon parameters, periodic in x
 * and y) are not the reference's force field, so nothing of the reference can
 * be compared with them directly.  This file states that preset as plainly
 * as possible, in FP64, with the reference's algorithms where the preset
 * keeps them:
 *
 *  * near field: every site interacts with all sites of other molecules in
 *    the 27 cells (12 A, periodic in x and y) around the cell it was found in
 *    at the last rebuild: Coulomb uncut, LJ within rc, as the 39 list kernels
 *    of the reference add up to (src/evalw1w1n.f90:86-108);
 *  * far field: the reference's order-4 expansions (P2M, M2M, M2L, L2L, L2P of
 *    src/computeOnm4.f90, src/computeLjk4.f90, src/shiftLjk3.f90,
 *    src/evalLjk4.f90, through orc_fma.c) on the L4 / L3 / L2 hierarchy,
 *    with interaction lists wrapped in x and y; at L2 every (source box,
 *    image) pair with image shift in {-1, 0, 1}^2 that is not adjacent to the
 *    target, i.e. the charges of the 3 x 3 supercell of periodic images;
 *  * the intramolecular correction of src/eval_subtract_fma.f90 for
 *    same-molecule pairs in non-adjacent (unwrapped) cells;
 *  * chains: harmonic bonds, the harmonic angles of src/eval_valence.f90,
 *    triple-cosine dihedrals in the convention of src/eval_dihedral.f90
 *    (trans at 180 degrees), LJ + Coulomb without cutoff for pairs four or
 *    more bonds apart (src/eval_surfactant_internal.f90:33-66);
 *  * walls at the two z faces only (src/eval_wall.f90:17-23 form);
 *  * water SHAKE / RATTLE and the Nose-Hoover friction of
 *    src/move_w1_a.f90 / src/move_w1_b.f90 / src/move_w2_a.f90:145-157;
 *    chains advance by plain velocity Verlet with the same friction.
 *
 * The dihedral forces here follow the textbook gradient of the torsion angle
 * (atan2 form), an independent derivation from the reference's cosine
 * algebra that the GPU engine keeps, so the two cross-check each other.
 *
 * Units are the reference's reduced units (sigma = 3.166 A, epsilon =
 * 650.2 J/mol, mass of O, velocities as displacements per step).
 */
#include "orc.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define LP ORC_LP
#define NB 12          /* beads per chain                 */
#define NTY 14         /* 0 water O, 1 water H, 2..13 beads */
#define NCB (NB - 1)   /* bonds                          */
#define NCA (NB - 2)   /* angles                         */
#define NCD (NB - 3)   /* dihedrals                      */

enum {
    OCF_T_NEAR = 1, OCF_T_FAR = 2, OCF_T_VALENCE = 4, OCF_T_DIHEDRAL = 8, OCF_T_INTERNAL = 32,
    OCF_T_SUBTRACT = 64, OCF_T_WALL = 128, OCF_T_GRAPHITE = 256, OCF_T_BOND = 512
};

/* ---------------------------------------------------------------- preset tables */

typedef struct {
    double q[NTY], mass[NTY], e48[NTY][NTY], s6[NTY][NTY];  /* LJ pair (48 eps sg^6, sg^6), 0 without LJ */
    double ge48[NTY], gs6[NTY];                               /* with carbon                            */
    double kb, r0, kth, th0, dva, dvb, dvc;
    double dsqw[3];                                           /* water constraint lengths^2             */
} ocf_tables;

static ocf_tables CT;

static void ocf_init_tables(void) {
    static int done = 0;
    if (done) return;
    orc_init_tables();   /* the factorial table of the expansion formulas */
    const double sig = 3.166, eps = 650.2, kj = 1000.0 / eps;
    const double mO = 15.9994, mH = 1.00794;
    const double pi180 = 4.0 * atan(1.0) / 180.0;
    memset(&CT, 0, sizeof CT);
    /* masses (relative to O), charges */
    CT.mass[0] = 1.0; CT.mass[1] = mH / mO;
    CT.q[0] = -0.82; CT.q[1] = 0.41;
    const double hm[4] = {15.035, 15.9994, 14.027, 15.9994}, hq[4] = {0.40, -0.60, 0.60, -0.40};
    const double hs[4] = {3.75, 2.80, 3.95, 2.80}, he[4] = {0.815, 0.457, 0.382, 0.457};
    double sg[NTY], ep[NTY];
    sg[0] = 3.166 / sig; ep[0] = 0.650 * kj;
    sg[1] = 0.0; ep[1] = 0.0;
    for (int b = 0; b < NB; b++) {
        const int t = 2 + b;
        CT.mass[t] = (b < 4 ? hm[b] : 14.027) / mO;
        CT.q[t] = b < 4 ? hq[b] : 0.0;
        sg[t] = (b < 4 ? hs[b] : 3.9) / sig;
        ep[t] = (b < 4 ? he[b] : 0.38) * kj;
    }
    for (int a = 0; a < NTY; a++)
        for (int b = 0; b < NTY; b++) {
            if (a == 1 || b == 1) continue;
            const double s = (sg[a] + sg[b]) / 2.0, s2 = s * s, s6 = s2 * s2 * s2;
            CT.e48[a][b] = 48.0 * sqrt(ep[a] * ep[b]) * s6;
            CT.s6[a][b] = s6;
        }
    const double sgc = 3.4 / sig, epc = 0.23 * kj;
    for (int a = 0; a < NTY; a++) {
        if (a == 1) continue;
        const double s = (sg[a] + sgc) / 2.0, s2 = s * s, s6 = s2 * s2 * s2;
        CT.ge48[a] = 48.0 * sqrt(ep[a] * epc) * s6;
        CT.gs6[a] = s6;
    }
    CT.kb = 2000.0 * kj * sig * sig;   /* U = kb/2 (r - r0)^2, 2000 kJ/mol/A^2 */
    CT.r0 = 1.53 / sig;
    CT.kth = 519.7 * kj;               /* U = kth/2 (th - th0)^2 per rad^2    */
    CT.th0 = 112.0 * pi180;
    CT.dva = 2951.7 / eps;             /* a (1 + cos) + b (1 - cos 2) + c (1 + cos 3) */
    CT.dvb = -566.9 / eps;
    CT.dvc = 6579.0 / eps;
    const double hh = 2.0 * sin(109.47 * pi180 / 2.0);
    CT.dsqw[0] = 1.0 / (sig * sig); CT.dsqw[1] = hh * hh / (sig * sig); CT.dsqw[2] = 1.0 / (sig * sig);
    done = 1;
}

/* ---------------------------------------------------------------- system */

typedef struct ocf_sys {
    int nw, ns, nmol, nsite;
    int nc[3], ncell;
    double L[3], rhs[3];
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *fx, *fy, *fz;
    int *type, *mol, *first;
    /* frozen at the last rebuild: cell, image (x, y), extended cell index */
    int *cell, *imx, *imy, *ex, *ey, *ez;
    int *cstart, *cslot;              /* sites per cell, in site order */
    uint32_t *isub;                   /* per chain site: same-molecule sites to subtract */
    double complex *O4, *L4, *O3, *L3, *O2, *L2;
    int ncarb;
    double *gx, *gy, *gz;
    int *ccol_start, *ccol;           /* carbons binned by bottom-layer column */
    int graphite_on, igz;
    double eta, tr, pnh1, pnh2, tol;
    int maxit, fails;
    int64_t npair, nlj;
} ocf_sys;

static void *zc(size_t n, size_t s) { return calloc(n ? n : 1, s); }
static int fdiv(int a, int b) { int q = a / b; if ((a % b) != 0 && ((a < 0) != (b < 0))) q--; return q; }
static int wrapi(int a, int n) { int r = a % n; return r < 0 ? r + n : r; }

static double cen(const ocf_sys *s, int a, int i, double size) { return -s->rhs[a] + (i + 0.5) * size; }

ocf_sys *ocf_create(int nw, int ns, int ncx, int ncy, int ncz, const double *pos, const double *vel, int ncarb,
                    const double *carb, int graphite_on, double tr, double tau_steps, double tol) {
    ocf_init_tables();
    if (ncx % 4 || ncy % 4 || ncz % 4 || ncx < 8 || ncy < 8 || ncz <= 0) return NULL;
    ocf_sys *s = (ocf_sys *)zc(1, sizeof(ocf_sys));
    s->nw = nw; s->ns = ns; s->nmol = nw + ns; s->nsite = 3 * nw + NB * ns;
    s->nc[0] = ncx; s->nc[1] = ncy; s->nc[2] = ncz; s->ncell = ncx * ncy * ncz;
    for (int a = 0; a < 3; a++) { s->L[a] = s->nc[a] * ORC_RS; s->rhs[a] = s->L[a] / 2.0; }
    const int N = s->nsite;
    double **arr[12] = {&s->x, &s->y, &s->z, &s->vx, &s->vy, &s->vz, &s->ax, &s->ay, &s->az, &s->fx, &s->fy, &s->fz};
    for (int i = 0; i < 12; i++) *arr[i] = (double *)zc(N, sizeof(double));
    int **iarr[9] = {&s->type, &s->mol, &s->cell, &s->imx, &s->imy, &s->ex, &s->ey, &s->ez, &s->cslot};
    for (int i = 0; i < 9; i++) *iarr[i] = (int *)zc(N, sizeof(int));
    s->first = (int *)zc(s->nmol, sizeof(int));
    s->cstart = (int *)zc(s->ncell + 1, sizeof(int));
    s->isub = (uint32_t *)zc((size_t)NB * ns, sizeof(uint32_t));
    for (int g = 0; g < N; g++) {
        s->x[g] = pos[3 * g]; s->y[g] = pos[3 * g + 1]; s->z[g] = pos[3 * g + 2];
        if (vel) { s->vx[g] = vel[3 * g]; s->vy[g] = vel[3 * g + 1]; s->vz[g] = vel[3 * g + 2]; }
        if (g < 3 * nw) { s->type[g] = g % 3 == 0 ? 0 : 1; s->mol[g] = g / 3; }
        else { s->type[g] = 2 + (g - 3 * nw) % NB; s->mol[g] = nw + (g - 3 * nw) / NB; }
    }
    for (int m = 0; m < s->nmol; m++) s->first[m] = m < nw ? 3 * m : 3 * nw + NB * (m - nw);
    const int n3 = s->ncell / 8, n2 = s->ncell / 64;
    s->O4 = (double complex *)zc((size_t)LP * s->ncell, sizeof(double complex));
    s->L4 = (double complex *)zc((size_t)LP * s->ncell, sizeof(double complex));
    s->O3 = (double complex *)zc((size_t)LP * n3, sizeof(double complex));
    s->L3 = (double complex *)zc((size_t)LP * n3, sizeof(double complex));
    s->O2 = (double complex *)zc((size_t)LP * n2, sizeof(double complex));
    s->L2 = (double complex *)zc((size_t)LP * n2, sizeof(double complex));
    /* carbons binned by bottom-layer column (x, y periodic) */
    s->ncarb = ncarb;
    s->gx = (double *)zc(ncarb, sizeof(double)); s->gy = (double *)zc(ncarb, sizeof(double));
    s->gz = (double *)zc(ncarb, sizeof(double));
    s->ccol_start = (int *)zc((size_t)ncx * ncy + 1, sizeof(int));
    s->ccol = (int *)zc(ncarb, sizeof(int));
    const double irs = 1.0 / ORC_RS;
    int *colof = (int *)zc(ncarb, sizeof(int));
    double ztop = -1e300;
    for (int k = 0; k < ncarb; k++) {
        s->gx[k] = carb[3 * k]; s->gy[k] = carb[3 * k + 1]; s->gz[k] = carb[3 * k + 2];
        const int bx = wrapi((int)floor((s->gx[k] + s->rhs[0]) * irs), ncx);
        const int by = wrapi((int)floor((s->gy[k] + s->rhs[1]) * irs), ncy);
        colof[k] = bx + ncx * by;
        s->ccol_start[colof[k] + 1]++;
        if (s->gz[k] > ztop) ztop = s->gz[k];
    }
    for (int c = 0; c < ncx * ncy; c++) s->ccol_start[c + 1] += s->ccol_start[c];
    int *fill = (int *)zc((size_t)ncx * ncy, sizeof(int));
    for (int k = 0; k < ncarb; k++) s->ccol[s->ccol_start[colof[k]] + fill[colof[k]]++] = k;
    free(fill); free(colof);
    s->graphite_on = graphite_on && ncarb > 0;
    /* graphite acts on LJ sites in cell layers up to the one holding the
     * top carbon plane + rs (rc plus the 2 A list skin) */
    s->igz = -1;
    if (s->graphite_on) {
        int iz = (int)floor((ztop + ORC_RS + s->rhs[2]) * irs);
        s->igz = iz < 0 ? 0 : (iz >= ncz ? ncz - 1 : iz);
    }
    /* thermostat (src/mybox.f90:44-52): df = 3 N - constraints (3 per water) */
    const int df = 3 * N - 3 * nw;
    const double rlx = tau_steps * ORC_DT;
    s->tr = tr;
    s->pnh1 = ORC_DT / df / tr / (rlx * rlx);
    s->pnh2 = -2.0 * df * tr;
    s->tol = tol;
    s->maxit = 100;
    return s;
}

void ocf_destroy(ocf_sys *s) {
    if (!s) return;
    double *arr[12] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->ax, s->ay, s->az, s->fx, s->fy, s->fz};
    for (int i = 0; i < 12; i++) free(arr[i]);
    int *iarr[9] = {s->type, s->mol, s->cell, s->imx, s->imy, s->ex, s->ey, s->ez, s->cslot};
    for (int i = 0; i < 9; i++) free(iarr[i]);
    free(s->first); free(s->cstart); free(s->isub);
    free(s->O4); free(s->L4); free(s->O3); free(s->L3); free(s->O2); free(s->L2);
    free(s->gx); free(s->gy); free(s->gz); free(s->ccol_start); free(s->ccol);
    free(s);
}

/* ---------------------------------------------------------------- rebuild */

/* Every 10 steps: each site's cell from floor((r + rhs) / rs) (x and y
 * wrapped into the box with the integer image kept, z unwrapped: a site
 * outside the z range is in no cell), cell lists in site order, and the
 * intramolecular-correction masks from the unwrapped cells. */
static void ocf_rebuild(ocf_sys *s) {
    const double irs = 1.0 / ORC_RS;
    const int N = s->nsite;
    memset(s->cstart, 0, sizeof(int) * (s->ncell + 1));
    for (int g = 0; g < N; g++) {
        const int ex = (int)floor((s->x[g] + s->rhs[0]) * irs);
        const int ey = (int)floor((s->y[g] + s->rhs[1]) * irs);
        const int ez = (int)floor((s->z[g] + s->rhs[2]) * irs);
        s->ex[g] = ex; s->ey[g] = ey; s->ez[g] = ez;
        s->imx[g] = fdiv(ex, s->nc[0]); s->imy[g] = fdiv(ey, s->nc[1]);
        const int cx = ex - s->imx[g] * s->nc[0], cy = ey - s->imy[g] * s->nc[1];
        s->cell[g] = (ez < 0 || ez >= s->nc[2]) ? -1 : cx + s->nc[0] * (cy + s->nc[1] * ez);
        if (s->cell[g] >= 0) s->cstart[s->cell[g] + 1]++;
    }
    for (int c = 0; c < s->ncell; c++) s->cstart[c + 1] += s->cstart[c];
    int *fill = (int *)zc(s->ncell, sizeof(int));
    for (int g = 0; g < N; g++)
        if (s->cell[g] >= 0) s->cslot[s->cstart[s->cell[g]] + fill[s->cell[g]]++] = g;
    free(fill);
    for (int q = 0; q < s->ns; q++) {
        const int g0 = s->first[s->nw + q];
        for (int j = 0; j < NB; j++) {
            uint32_t m = 0;
            for (int k = 0; k < NB; k++) {
                if (k == j) continue;
                const int a = g0 + j, b = g0 + k;
                if (abs(s->ex[a] - s->ex[b]) > 1 || abs(s->ey[a] - s->ey[b]) > 1 || abs(s->ez[a] - s->ez[b]) > 1)
                    m |= 1u << k;
            }
            s->isub[(size_t)q * NB + j] = m;
        }
    }
}

/* the site's position wrapped by its frozen image */
static inline void wpos(const ocf_sys *s, int g, double *p) {
    p[0] = s->x[g] - s->imx[g] * s->L[0];
    p[1] = s->y[g] - s->imy[g] * s->L[1];
    p[2] = s->z[g];
}

/* ---------------------------------------------------------------- near field */

/* force (and energies) on site i from the 27 periodic neighbour cells */
static void near_site(ocf_sys *s, int i, double *f, double *ec, double *el, int64_t *np, int64_t *nl) {
    f[0] = f[1] = f[2] = 0.0;
    *ec = *el = 0.0;
    *np = *nl = 0;
    const int c = s->cell[i];
    if (c < 0) return;
    const int cx = c % s->nc[0], cy = (c / s->nc[0]) % s->nc[1], cz = c / (s->nc[0] * s->nc[1]);
    double pi[3];
    wpos(s, i, pi);
    const int ti = s->type[i], mi = s->mol[i];
    const double qi = CT.q[ti] * ORC_XPI, rc2 = ORC_RC * ORC_RC;
    for (int dz = -1; dz <= 1; dz++) {
        const int jz = cz + dz;
        if (jz < 0 || jz >= s->nc[2]) continue;
        for (int dy = -1; dy <= 1; dy++) {
            const int jyu = cy + dy, jy = wrapi(jyu, s->nc[1]);
            const double sy = (double)fdiv(jyu, s->nc[1]) * s->L[1];
            for (int dx = -1; dx <= 1; dx++) {
                const int jxu = cx + dx, jx = wrapi(jxu, s->nc[0]);
                const double sx = (double)fdiv(jxu, s->nc[0]) * s->L[0];
                const int cn = jx + s->nc[0] * (jy + s->nc[1] * jz);
                for (int k = s->cstart[cn]; k < s->cstart[cn + 1]; k++) {
                    const int j = s->cslot[k];
                    if (s->mol[j] == mi) continue;
                    double pj[3];
                    wpos(s, j, pj);
                    const double dxv = pi[0] - (pj[0] + sx), dyv = pi[1] - (pj[1] + sy), dzv = pi[2] - pj[2];
                    const double r2 = dxv * dxv + dyv * dyv + dzv * dzv, ir2 = 1.0 / r2, ir = sqrt(ir2);
                    const int tj = s->type[j];
                    const double qq = qi * CT.q[tj];
                    double ft = qq * ir * ir2;
                    *ec += 0.5 * qq * ir;
                    (*np)++;
                    if (r2 <= rc2 && CT.e48[ti][tj] != 0.0) {
                        const double r6 = ir2 * ir2 * ir2, e48 = CT.e48[ti][tj], s6 = CT.s6[ti][tj];
                        ft += e48 * r6 * (s6 * r6 - 0.5) * ir2;
                        *el += 0.5 * (e48 / 12.0) * (s6 * r6 * r6 - r6);
                        (*nl)++;
                    }
                    f[0] += dxv * ft; f[1] += dyv * ft; f[2] += dzv * ft;
                }
            }
        }
    }
}

static void ocf_near(ocf_sys *s, double *e) {
    double ec = 0.0, el = 0.0;
    int64_t np = 0, nl = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : np, nl)
    for (int i = 0; i < s->nsite; i++) {
        double f[3], a, b;
        int64_t p, l;
        near_site(s, i, f, &a, &b, &p, &l);
        s->fx[i] += f[0]; s->fy[i] += f[1]; s->fz[i] += f[2];
        np += p; nl += l;
    }
    if (e) {
        for (int i = 0; i < s->nsite; i++) {
            double f[3], a, b;
            int64_t p, l;
            near_site(s, i, f, &a, &b, &p, &l);
            ec += a; el += b;
        }
        e[0] = ec; e[1] = el;
    }
    s->npair = np;
    s->nlj = nl;
}

/* ---------------------------------------------------------------- far field */

static void ocf_fma(ocf_sys *s) {
    const int n4[3] = {s->nc[0], s->nc[1], s->nc[2]};
    const int n3[3] = {n4[0] / 2, n4[1] / 2, n4[2] / 2}, n2[3] = {n4[0] / 4, n4[1] / 4, n4[2] / 4};
    const int N4 = s->ncell, N3 = N4 / 8, N2 = N4 / 64;
    const double s4 = ORC_RS, s3 = 2.0 * ORC_RS, s2 = 4.0 * ORC_RS;
    memset(s->O4, 0, sizeof(double complex) * LP * N4); memset(s->L4, 0, sizeof(double complex) * LP * N4);
    memset(s->O3, 0, sizeof(double complex) * LP * N3); memset(s->L3, 0, sizeof(double complex) * LP * N3);
    memset(s->O2, 0, sizeof(double complex) * LP * N2); memset(s->L2, 0, sizeof(double complex) * LP * N2);
    /* P2M */
#pragma omp parallel for schedule(dynamic, 8)
    for (int c = 0; c < N4; c++) {
        const int ix = c % n4[0], iy = (c / n4[0]) % n4[1], iz = c / (n4[0] * n4[1]);
        const double cc[3] = {cen(s, 0, ix, s4), cen(s, 1, iy, s4), cen(s, 2, iz, s4)};
        for (int k = s->cstart[c]; k < s->cstart[c + 1]; k++) {
            const int g = s->cslot[k];
            double p[3];
            wpos(s, g, p);
            orc_p2m_add(&s->O4[(size_t)LP * c], CT.q[s->type[g]], p[0] - cc[0], p[1] - cc[1], p[2] - cc[2]);
        }
    }
    /* M2M: L4 -> L3 -> L2 */
    for (int lev = 3; lev >= 2; lev--) {
        const int *np_ = lev == 3 ? n3 : n2, *nch = lev == 3 ? n4 : n3;
        const double sp = lev == 3 ? s3 : s2, sc = lev == 3 ? s4 : s3;
        double complex *Op = lev == 3 ? s->O3 : s->O2;
        const double complex *Oc = lev == 3 ? s->O4 : s->O3;
        const int NP = np_[0] * np_[1] * np_[2];
#pragma omp parallel for schedule(static)
        for (int b = 0; b < NP; b++) {
            const int px = b % np_[0], py = (b / np_[0]) % np_[1], pz = b / (np_[0] * np_[1]);
            for (int ch = 0; ch < 8; ch++) {
                const int cx = 2 * px + (ch & 1), cy = 2 * py + ((ch >> 1) & 1), cz = 2 * pz + ((ch >> 2) & 1);
                const int ci = cx + nch[0] * (cy + nch[1] * cz);
                orc_m2m_apply(&Oc[(size_t)LP * ci], cen(s, 0, cx, sc) - cen(s, 0, px, sp), cen(s, 1, cy, sc) - cen(s, 1, py, sp),
                              cen(s, 2, cz, sc) - cen(s, 2, pz, sp), &Op[(size_t)LP * b]);
            }
        }
    }
    /* M2L at L2: every (source, image) of the 3 x 3 image supercell not adjacent to the target */
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < N2; t++) {
        const int tx = t % n2[0], ty = (t / n2[0]) % n2[1], tz = t / (n2[0] * n2[1]);
        for (int sb = 0; sb < N2; sb++) {
            const int sx = sb % n2[0], sy = (sb / n2[0]) % n2[1], sz = sb / (n2[0] * n2[1]);
            for (int iy = -1; iy <= 1; iy++)
                for (int ix = -1; ix <= 1; ix++) {
                    const int ux = sx + ix * n2[0], uy = sy + iy * n2[1];
                    if (abs(ux - tx) <= 1 && abs(uy - ty) <= 1 && abs(sz - tz) <= 1) continue;
                    orc_m2l_apply(&s->O2[(size_t)LP * sb], cen(s, 0, sx, s2) + ix * s->L[0] - cen(s, 0, tx, s2),
                                  cen(s, 1, sy, s2) + iy * s->L[1] - cen(s, 1, ty, s2), cen(s, 2, sz, s2) - cen(s, 2, tz, s2),
                                  &s->L2[(size_t)LP * t]);
                }
        }
    }
    /* L2L then M2L at L3 and L4: children of the parent's (periodic)
     * neighbours that are not adjacent to the target */
    for (int lev = 3; lev <= 4; lev++) {
        const int *nt = lev == 3 ? n3 : n4, *npa = lev == 3 ? n2 : n3;
        const double st = lev == 3 ? s3 : s4, sp = lev == 3 ? s2 : s3;
        double complex *Lt = lev == 3 ? s->L3 : s->L4;
        const double complex *Lp = lev == 3 ? s->L2 : s->L3, *Os = lev == 3 ? s->O3 : s->O4;
        const int NT = nt[0] * nt[1] * nt[2];
#pragma omp parallel for schedule(dynamic, 4)
        for (int t = 0; t < NT; t++) {
            const int tx = t % nt[0], ty = (t / nt[0]) % nt[1], tz = t / (nt[0] * nt[1]);
            const int px = tx / 2, py = ty / 2, pz = tz / 2;
            const int pi = px + npa[0] * (py + npa[1] * pz);
            orc_l2l_apply(&Lp[(size_t)LP * pi], cen(s, 0, px, sp) - cen(s, 0, tx, st), cen(s, 1, py, sp) - cen(s, 1, ty, st),
                          cen(s, 2, pz, sp) - cen(s, 2, tz, st), &Lt[(size_t)LP * t]);
            for (int ez = -1; ez <= 1; ez++) {
                const int qz = pz + ez;
                if (qz < 0 || qz >= npa[2]) continue;
                for (int ey = -1; ey <= 1; ey++)
                    for (int ex = -1; ex <= 1; ex++)
                        for (int ch = 0; ch < 8; ch++) {
                            const int ux = 2 * (px + ex) + (ch & 1), uy = 2 * (py + ey) + ((ch >> 1) & 1);
                            const int uz = 2 * qz + ((ch >> 2) & 1);
                            if (abs(ux - tx) <= 1 && abs(uy - ty) <= 1 && abs(uz - tz) <= 1) continue;
                            const int wx = wrapi(ux, nt[0]), wy = wrapi(uy, nt[1]);
                            const double shx = (double)fdiv(ux, nt[0]) * s->L[0], shy = (double)fdiv(uy, nt[1]) * s->L[1];
                            const int si = wx + nt[0] * (wy + nt[1] * uz);
                            orc_m2l_apply(&Os[(size_t)LP * si], cen(s, 0, wx, st) + shx - cen(s, 0, tx, st),
                                          cen(s, 1, wy, st) + shy - cen(s, 1, ty, st), cen(s, 2, uz, st) - cen(s, 2, tz, st),
                                          &Lt[(size_t)LP * t]);
                        }
            }
        }
    }
}

/* L2P force (and potential energy) of every located site */
static void ocf_l2p(ocf_sys *s, double *e) {
    double ef = 0.0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : ef)
    for (int c = 0; c < s->ncell; c++) {
        const int ix = c % s->nc[0], iy = (c / s->nc[0]) % s->nc[1], iz = c / (s->nc[0] * s->nc[1]);
        const double cc[3] = {cen(s, 0, ix, ORC_RS), cen(s, 1, iy, ORC_RS), cen(s, 2, iz, ORC_RS)};
        for (int k = s->cstart[c]; k < s->cstart[c + 1]; k++) {
            const int g = s->cslot[k];
            double p[3], phi = 0.0;
            wpos(s, g, p);
            const double qx = CT.q[s->type[g]] * ORC_XPI;
            orc_l2p_apply(&s->L4[(size_t)LP * c], p[0] - cc[0], p[1] - cc[1], p[2] - cc[2], qx, &s->fx[g], &s->fy[g],
                          &s->fz[g], &phi);
            ef += 0.5 * qx * phi;
        }
    }
    if (e) e[0] = ef;
}

/* ---------------------------------------------------------------- chains */

static inline void sub3(const double *a, const double *b, double *o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }
static inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1]; o[1] = a[2] * b[0] - a[0] * b[2]; o[2] = a[0] * b[1] - a[1] * b[0];
}

/* one chain's bonded and intramolecular terms; energies e[0] bonds, e[1]
 * angles, e[2] dihedrals, e[3] pairs, e[4] far-field correction */
static void chain_terms(ocf_sys *s, int q, int terms, double *e) {
    const int g0 = s->first[s->nw + q];
    double r[NB][3], f[NB][3];
    for (int i = 0; i < NB; i++) {
        r[i][0] = s->x[g0 + i]; r[i][1] = s->y[g0 + i]; r[i][2] = s->z[g0 + i];
        f[i][0] = f[i][1] = f[i][2] = 0.0;
    }
    double eb = 0, ea = 0, ed = 0, ep = 0, es = 0;
    if (terms & OCF_T_BOND)
        for (int b = 0; b < NCB; b++) {
            double d[3];
            sub3(r[b], r[b + 1], d);
            const double rr = sqrt(dot3(d, d)), dr = rr - CT.r0, fm = -CT.kb * dr / rr;
            for (int a = 0; a < 3; a++) { f[b][a] += fm * d[a]; f[b + 1][a] -= fm * d[a]; }
            eb += 0.5 * CT.kb * dr * dr;
        }
    if (terms & OCF_T_VALENCE)
        for (int t = 0; t < NCA; t++) {
            const int i = t, j = t + 1, k = t + 2;
            double a[3], b[3];
            sub3(r[i], r[j], a);
            sub3(r[k], r[j], b);
            const double la = sqrt(dot3(a, a)), lb = sqrt(dot3(b, b)), c = dot3(a, b) / (la * lb);
            const double th = acos(c), dth = th - CT.th0, g = CT.kth * dth / sin(th);   /* -dU/dcos */
            for (int x = 0; x < 3; x++) {
                const double fi = g * (b[x] / (la * lb) - c * a[x] / (la * la));
                const double fk = g * (a[x] / (la * lb) - c * b[x] / (lb * lb));
                f[i][x] += fi; f[k][x] += fk; f[j][x] -= fi + fk;
            }
            ea += 0.5 * CT.kth * dth * dth;
        }
    if (terms & OCF_T_DIHEDRAL)
        for (int t = 0; t < NCD; t++) {
            const int i = t, j = t + 1, k = t + 2, l = t + 3;
            double b1[3], b2[3], b3[3], m[3], n[3], mn[3];
            sub3(r[j], r[i], b1); sub3(r[k], r[j], b2); sub3(r[l], r[k], b3);
            cross3(b1, b2, m); cross3(b2, b3, n); cross3(m, n, mn);
            const double lb2 = sqrt(dot3(b2, b2)), m2 = dot3(m, m), n2 = dot3(n, n);
            const double phi = atan2(dot3(mn, b2) / lb2, dot3(m, n));
            ed += CT.dva * (1.0 + cos(phi)) + CT.dvb * (1.0 - cos(2.0 * phi)) + CT.dvc * (1.0 + cos(3.0 * phi));
            const double dU = -CT.dva * sin(phi) + 2.0 * CT.dvb * sin(2.0 * phi) - 3.0 * CT.dvc * sin(3.0 * phi);
            /* gradients of phi (Blondel & Karplus, J. Comput. Chem. 17, 1132
             * (1996), with F = -b1, G = -b2, H = b3, so A = m and B = n); the
             * four sum to zero */
            const double p12 = dot3(b1, b2) / (lb2 * lb2), p32 = dot3(b3, b2) / (lb2 * lb2);
            for (int x = 0; x < 3; x++) {
                const double gi = -lb2 * m[x] / m2, gl = lb2 * n[x] / n2;
                const double gj = -(1.0 + p12) * gi + p32 * gl, gk = p12 * gi - (1.0 + p32) * gl;
                f[i][x] -= dU * gi; f[j][x] -= dU * gj; f[k][x] -= dU * gk; f[l][x] -= dU * gl;
            }
        }
    if (terms & OCF_T_INTERNAL)
        for (int a = 0; a < NB; a++)
            for (int b = a + 4; b < NB; b++) {
                double d[3];
                sub3(r[a], r[b], d);
                const double r2 = dot3(d, d), ir2 = 1.0 / r2, ir = sqrt(ir2), r6 = ir2 * ir2 * ir2;
                const int ta = 2 + a, tb = 2 + b;
                const double qq = CT.q[ta] * CT.q[tb] * ORC_XPI, e48 = CT.e48[ta][tb], s6 = CT.s6[ta][tb];
                const double ft = qq * ir * ir2 + e48 * r6 * (s6 * r6 - 0.5) * ir2;
                for (int x = 0; x < 3; x++) { f[a][x] += ft * d[x]; f[b][x] -= ft * d[x]; }
                ep += qq * ir + (e48 / 12.0) * (s6 * r6 * r6 - r6);
            }
    if (terms & OCF_T_SUBTRACT)
        for (int j = 0; j < NB; j++) {
            uint32_t bits = s->isub[(size_t)q * NB + j];
            for (int k = 0; k < NB; k++) {
                if (!(bits >> k & 1u)) continue;
                double d[3];
                sub3(r[j], r[k], d);
                const double rr = sqrt(dot3(d, d)), qq = CT.q[2 + j] * CT.q[2 + k] * ORC_XPI;
                const double fel = qq / (rr * rr * rr);
                for (int x = 0; x < 3; x++) f[j][x] -= d[x] * fel;
                es -= 0.5 * qq / rr;
            }
        }
    for (int i = 0; i < NB; i++) { s->fx[g0 + i] += f[i][0]; s->fy[g0 + i] += f[i][1]; s->fz[g0 + i] += f[i][2]; }
    if (e) { e[0] += eb; e[1] += ea; e[2] += ed; e[3] += ep; e[4] += es; }
}

/* ---------------------------------------------------------------- external */

static inline double p13(double v) { double v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4 * v; }
static inline double p12(double v) { double v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4; }

static void ocf_walls(ocf_sys *s, double *e) {
    double ew = 0.0;
    for (int g = 0; g < s->nsite; g++) {
        const double z = s->z[g], h = s->rhs[2];
        s->fz[g] += 48.0 / p13(z - h);
        s->fz[g] += 48.0 / p13(h + z);
        ew += 4.0 / p12(z - h) + 4.0 / p12(h + z);
    }
    if (e) e[0] = ew;
}

/* graphite LJ on the LJ sites of the bottom cell layers (x, y periodic) */
static void ocf_graphite(ocf_sys *s, double *e) {
    if (!s->graphite_on) { if (e) e[0] = 0.0; return; }
    double eg = 0.0;
    const double rc2 = ORC_RC * ORC_RC;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : eg)
    for (int g = 0; g < s->nsite; g++) {
        const int c = s->cell[g], t = s->type[g];
        if (c < 0 || CT.ge48[t] == 0.0) continue;
        const int cx = c % s->nc[0], cy = (c / s->nc[0]) % s->nc[1], cz = c / (s->nc[0] * s->nc[1]);
        if (cz > s->igz) continue;
        double p[3];
        wpos(s, g, p);
        double fx = 0, fy = 0, fz = 0;
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int ux = cx + dx, uy = cy + dy, wx = wrapi(ux, s->nc[0]), wy = wrapi(uy, s->nc[1]);
                const double shx = (double)fdiv(ux, s->nc[0]) * s->L[0], shy = (double)fdiv(uy, s->nc[1]) * s->L[1];
                const int col = wx + s->nc[0] * wy;
                for (int k = s->ccol_start[col]; k < s->ccol_start[col + 1]; k++) {
                    const int cb = s->ccol[k];
                    const double xij = p[0] - (s->gx[cb] + shx), yij = p[1] - (s->gy[cb] + shy), zij = p[2] - s->gz[cb];
                    const double r2 = xij * xij + yij * yij + zij * zij;
                    if (r2 > rc2) continue;
                    const double rsi = 1.0 / r2, r6 = rsi * rsi * rsi, e48 = CT.ge48[t], s6 = CT.gs6[t];
                    const double flj = e48 * r6 * (s6 * r6 - 0.5) * rsi;
                    fx += xij * flj; fy += yij * flj; fz += zij * flj;
                    eg += (e48 / 12.0) * (s6 * r6 * r6 - r6);
                }
            }
        s->fx[g] += fx; s->fy[g] += fy; s->fz[g] += fz;
    }
    if (e) e[0] = eg;
}

/* ---------------------------------------------------------------- force section */

void ocf_force_terms(ocf_sys *s, int rebuild, int terms) {
    if (rebuild) {
        ocf_rebuild(s);
        ocf_fma(s);
    }
    for (int g = 0; g < s->nsite; g++) { s->fx[g] = 0.0; s->fy[g] = 0.0; s->fz[g] = 0.0; }
    if (terms & OCF_T_NEAR) ocf_near(s, NULL);
    if (terms & OCF_T_FAR) ocf_l2p(s, NULL);
    for (int q = 0; q < s->ns; q++) chain_terms(s, q, terms, NULL);
    if (terms & OCF_T_WALL) ocf_walls(s, NULL);
    if (terms & OCF_T_GRAPHITE) ocf_graphite(s, NULL);
}

/* energies of the current lists and expansions (a force call must have
 * rebuilt them): [0] near Coulomb, [1] near LJ, [2] far field incl. the
 * intramolecular correction, [3] intramolecular pairs, [4] bonds + angles +
 * dihedrals, [5] walls, [6] graphite, [7] kinetic; forces are left as the
 * full force of the current state */
void ocf_energies(ocf_sys *s, double *out) {
    for (int g = 0; g < s->nsite; g++) { s->fx[g] = 0.0; s->fy[g] = 0.0; s->fz[g] = 0.0; }
    double e2[2], e1;
    ocf_near(s, e2);
    out[0] = e2[0]; out[1] = e2[1];
    ocf_l2p(s, &e1);
    double ch[5] = {0, 0, 0, 0, 0};
    for (int q = 0; q < s->ns; q++) chain_terms(s, q, 0x7fffffff, ch);
    out[2] = e1 + ch[4];
    out[3] = ch[3];
    out[4] = ch[0] + ch[1] + ch[2];
    ocf_walls(s, &out[5]);
    ocf_graphite(s, &out[6]);
    double ek = 0.0;
    for (int g = 0; g < s->nsite; g++)
        ek += 0.5 * CT.mass[s->type[g]] * (s->vx[g] * s->vx[g] + s->vy[g] * s->vy[g] + s->vz[g] * s->vz[g]) / ORC_DTSQ;
    out[7] = ek;
}

/* ---------------------------------------------------------------- integrator */

static double ocf_ke(const ocf_sys *s) {
    double k = 0.0;
    for (int g = 0; g < s->nsite; g++)
        k += CT.mass[s->type[g]] * (s->vx[g] * s->vx[g] + s->vy[g] * s->vy[g] + s->vz[g] * s->vz[g]);
    return k;
}

/* predictor + SHAKE of one water (src/move_w1_a.f90:36-134), bonds O-H1,
 * H1-H2, H2-O in that order */
static int water_shake(ocf_sys *s, int g0, double escale) {
    double rx[3], ry[3], rz[3], px[3], py[3], pz[3], vx[3], vy[3], vz[3], mass[3];
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        mass[i] = CT.mass[i == 0 ? 0 : 1];
        rx[i] = s->x[g]; ry[i] = s->y[g]; rz[i] = s->z[g];
        px[i] = s->x[g] + s->vx[g] * escale + s->ax[g];
        py[i] = s->y[g] + s->vy[g] * escale + s->ay[g];
        pz[i] = s->z[g] + s->vz[g] * escale + s->az[g];
        vx[i] = s->vx[g] * escale + s->ax[g];
        vy[i] = s->vy[g] * escale + s->ay[g];
        vz[i] = s->vz[g] * escale + s->az[g];
    }
    const double tol2 = 2.0 * s->tol;
    int it = 0, ldone = 0;
    while (!ldone && it <= s->maxit) {
        ldone = 1;
        for (int b = 0; b < 3; b++) {
            const int i = b, j = b == 2 ? 0 : b + 1;
            double pxab = px[i] - px[j], pyab = py[i] - py[j], pzab = pz[i] - pz[j];
            double pabsq = pxab * pxab + pyab * pyab + pzab * pzab;
            double rabsq = CT.dsqw[b];
            double diffsq = rabsq - pabsq;
            if (fabs(diffsq) > rabsq * tol2) {
                double rxab = rx[i] - rx[j], ryab = ry[i] - ry[j], rzab = rz[i] - rz[j];
                double rpab = rxab * pxab + ryab * pyab + rzab * pzab;
                double rma = 1.0 / mass[i], rmb = 1.0 / mass[j];
                double gab = diffsq / (2.0 * (rma + rmb) * rpab);
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                px[i] = px[i] + rma * dx; py[i] = py[i] + rma * dy; pz[i] = pz[i] + rma * dz;
                px[j] = px[j] - rmb * dx; py[j] = py[j] - rmb * dy; pz[j] = pz[j] - rmb * dz;
                vx[i] = vx[i] + rma * dx; vy[i] = vy[i] + rma * dy; vz[i] = vz[i] + rma * dz;
                vx[j] = vx[j] - rmb * dx; vy[j] = vy[j] - rmb * dy; vz[j] = vz[j] - rmb * dz;
                ldone = 0;
            }
        }
        it++;
    }
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        s->x[g] = px[i]; s->y[g] = py[i]; s->z[g] = pz[i];
        s->vx[g] = vx[i]; s->vy[g] = vy[i]; s->vz[g] = vz[i];
    }
    return ldone ? 0 : 1;
}

/* RATTLE of one water (src/move_w1_b.f90:30-119) */
static int water_rattle(ocf_sys *s, int g0, double escale) {
    double rx[3], ry[3], rz[3], vx[3], vy[3], vz[3], mass[3];
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        mass[i] = CT.mass[i == 0 ? 0 : 1];
        rx[i] = s->x[g]; ry[i] = s->y[g]; rz[i] = s->z[g];
        s->ax[g] = s->fx[g] * ORC_DTSQ2 / mass[i];
        s->ay[g] = s->fy[g] * ORC_DTSQ2 / mass[i];
        s->az[g] = s->fz[g] * ORC_DTSQ2 / mass[i];
        vx[i] = escale * (s->vx[g] + s->ax[g]);
        vy[i] = escale * (s->vy[g] + s->ay[g]);
        vz[i] = escale * (s->vz[g] + s->az[g]);
    }
    int it = 0, ldone = 0;
    while (!ldone && it <= s->maxit) {
        ldone = 1;
        for (int b = 0; b < 3; b++) {
            const int i = b, j = b == 2 ? 0 : b + 1;
            double vxab = vx[i] - vx[j], vyab = vy[i] - vy[j], vzab = vz[i] - vz[j];
            double rxab = rx[i] - rx[j], ryab = ry[i] - ry[j], rzab = rz[i] - rz[j];
            double rvab = rxab * vxab + ryab * vyab + rzab * vzab;
            double rma = 1.0 / mass[i], rmb = 1.0 / mass[j];
            rvab = rvab / ORC_DT;
            double gab = -rvab / ((rma + rmb) * CT.dsqw[b]);
            if (fabs(gab) > s->tol) {
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                vx[i] = vx[i] + rma * dx * ORC_DT; vy[i] = vy[i] + rma * dy * ORC_DT; vz[i] = vz[i] + rma * dz * ORC_DT;
                vx[j] = vx[j] - rmb * dx * ORC_DT; vy[j] = vy[j] - rmb * dy * ORC_DT; vz[j] = vz[j] - rmb * dz * ORC_DT;
                ldone = 0;
            }
        }
        it++;
    }
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        s->vx[g] = vx[i]; s->vy[g] = vy[i]; s->vz[g] = vz[i];
    }
    return ldone ? 0 : 1;
}

void ocf_move_a(ocf_sys *s) {
    const double escale = 1.0 - s->eta * ORC_DT / 2.0;
    const double k1 = ocf_ke(s);
    for (int m = 0; m < s->nw; m++) s->fails += water_shake(s, 3 * m, escale);
    for (int g = 3 * s->nw; g < s->nsite; g++) {
        s->x[g] = s->x[g] + s->vx[g] * escale + s->ax[g];
        s->y[g] = s->y[g] + s->vy[g] * escale + s->ay[g];
        s->z[g] = s->z[g] + s->vz[g] * escale + s->az[g];
        s->vx[g] = s->vx[g] * escale + s->ax[g];
        s->vy[g] = s->vy[g] * escale + s->ay[g];
        s->vz[g] = s->vz[g] * escale + s->az[g];
    }
    const double k2 = ocf_ke(s);
    s->eta = s->eta + s->pnh1 * (k1 / ORC_DTSQ + s->pnh2 + k2 / ORC_DTSQ);
    for (int g = 0; g < s->nsite; g++) { s->fx[g] = 0.0; s->fy[g] = 0.0; s->fz[g] = 0.0; }
}

void ocf_move_b(ocf_sys *s) {
    const double escale = 2.0 / (2.0 + s->eta * ORC_DT);
    for (int m = 0; m < s->nw; m++) s->fails += water_rattle(s, 3 * m, escale);
    for (int g = 3 * s->nw; g < s->nsite; g++) {
        const double mi = CT.mass[s->type[g]];
        s->ax[g] = s->fx[g] * ORC_DTSQ2 / mi;
        s->ay[g] = s->fy[g] * ORC_DTSQ2 / mi;
        s->az[g] = s->fz[g] * ORC_DTSQ2 / mi;
        s->vx[g] = escale * (s->vx[g] + s->ax[g]);
        s->vy[g] = escale * (s->vy[g] + s->ay[g]);
        s->vz[g] = escale * (s->vz[g] + s->az[g]);
    }
}

void ocf_init_accel(ocf_sys *s) {
    for (int g = 0; g < s->nsite; g++) {
        const double m = CT.mass[s->type[g]];
        s->ax[g] = s->fx[g] * ORC_DTSQ2 / m;
        s->ay[g] = s->fy[g] * ORC_DTSQ2 / m;
        s->az[g] = s->fz[g] * ORC_DTSQ2 / m;
    }
}

double ocf_temperature(const ocf_sys *s) { return ocf_ke(s) / ORC_DTSQ / (3 * s->nsite - 3 * s->nw); }

void ocf_step(ocf_sys *s, int kb) {
    ocf_move_a(s);
    ocf_force_terms(s, kb % 10 == 0, 0x7fffffff);
    ocf_move_b(s);
}

void ocf_run(ocf_sys *s, int kb0, int n) {
    for (int k = 0; k < n; k++) ocf_step(s, kb0 + k);
}

/* ---------------------------------------------------------------- accessors */

/* which: 0 positions, 1 velocities, 2 accelerations, 3 forces; (n, 3) arrays */
void ocf_get(const ocf_sys *s, int which, double *out) {
    const double *a[4][3] = {{s->x, s->y, s->z}, {s->vx, s->vy, s->vz}, {s->ax, s->ay, s->az}, {s->fx, s->fy, s->fz}};
    for (int g = 0; g < s->nsite; g++)
        for (int k = 0; k < 3; k++) out[3 * g + k] = a[which][k][g];
}
void ocf_set(ocf_sys *s, int which, const double *in) {
    double *a[4][3] = {{s->x, s->y, s->z}, {s->vx, s->vy, s->vz}, {s->ax, s->ay, s->az}, {s->fx, s->fy, s->fz}};
    for (int g = 0; g < s->nsite; g++)
        for (int k = 0; k < 3; k++) a[which][k][g] = in[3 * g + k];
}
double ocf_get_eta(const ocf_sys *s) { return s->eta; }
void ocf_set_eta(ocf_sys *s, double v) { s->eta = v; }
int ocf_fail_count(const ocf_sys *s) { return s->fails; }
void ocf_pair_counts(const ocf_sys *s, int64_t *out) { out[0] = s->npair; out[1] = s->nlj; }
int ocf_graphite_layer(const ocf_sys *s) { return s->igz; }
/* the preset's per-type tables: q[14], mass[14] */
void ocf_type_tables(double *q, double *mass) {
    ocf_init_tables();
    for (int t = 0; t < NTY; t++) { q[t] = CT.q[t]; mass[t] = CT.mass[t]; }
}

/* Coulomb force on every site from the charges of other molecules in the
 * 3 x 3 supercell of periodic images (x, y), by direct summation, minus the
 * near field's 27-cell share: the exact counterpart of the far field.
 * O(N^2); for small accuracy checks. */
void ocf_direct_far(const ocf_sys *s, double *out) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < s->nsite; i++) {
        double pi[3], f[3] = {0, 0, 0};
        wpos(s, i, pi);
        const double qi = CT.q[s->type[i]] * ORC_XPI;
        for (int j = 0; j < s->nsite; j++) {
            if (s->cell[j] < 0 || s->cell[i] < 0) continue;
            double pj[3];
            wpos(s, j, pj);
            const int cxi = s->ex[i] - s->imx[i] * s->nc[0], cyi = s->ey[i] - s->imy[i] * s->nc[1];
            const int cxj = s->ex[j] - s->imx[j] * s->nc[0], cyj = s->ey[j] - s->imy[j] * s->nc[1];
            for (int iy = -1; iy <= 1; iy++)
                for (int ix = -1; ix <= 1; ix++) {
                    /* a molecule's own sites sit at the image that keeps it whole */
                    const int same = s->mol[j] == s->mol[i] && ix == s->imx[j] - s->imx[i] && iy == s->imy[j] - s->imy[i];
                    const int ux = cxj + ix * s->nc[0], uy = cyj + iy * s->nc[1];
                    const int adj = abs(ux - cxi) <= 1 && abs(uy - cyi) <= 1 && abs(s->ez[j] - s->ez[i]) <= 1;
                    if (same || adj) continue;
                    const double dx = pi[0] - (pj[0] + ix * s->L[0]), dy = pi[1] - (pj[1] + iy * s->L[1]), dz = pi[2] - pj[2];
                    const double r2 = dx * dx + dy * dy + dz * dz, ir = 1.0 / sqrt(r2);
                    const double ft = qi * CT.q[s->type[j]] * ir * ir * ir;
                    f[0] += dx * ft; f[1] += dy * ft; f[2] += dz * ft;
                }
        }
        out[3 * i] = f[0]; out[3 * i + 1] = f[1]; out[3 * i + 2] = f[2];
    }
}
