/*
 * TEST INFRASTRUCTURE ONLY (CPU oracle; parity unpinned - see orc.h).
 * Force-field tables, box geometry, molecule classification (migration) and
 * the per-cell atom-list builders, restated on one global cell grid.
 */
#include "orc.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

orc_tables ORC_T;

/* src/mybox.cmns:36-44.  xpi is written as a default-kind (single precision)
 * literal in the reference, so its double value is the float 675.05. */
const double ORC_SIGMA = 3.166;
const double ORC_EPSILON = 650.2;
const double ORC_RC = 10.0 / 3.166;
const double ORC_DELTA = 2.0 / 3.166;
const double ORC_RS = 10.0 / 3.166 + 2.0 / 3.166;
const double ORC_XPI = (double)675.05f;
const double ORC_DT = 0.00127362;
const double ORC_DTSQ = 0.00127362 * 0.00127362;
const double ORC_DTSQ2 = 0.00127362 * 0.00127362 / 2.0;

static double pow6(double v) { double v3 = v * v * v; return v3 * v3; }

/* src/init_arrays.f90:88-840 */
void orc_init_tables(void) {
    orc_tables *T = &ORC_T;
    memset(T, 0, sizeof(*T));
    const double pi180 = 4.0 * atan(1.0) / 180.0;
    const double sigma = ORC_SIGMA, epsilon = ORC_EPSILON;

    /* factorial table, src/init_arrays.f90:91-123 (rifact(n+1) = n!) */
    T->rifact[1] = 1.0;
    for (int n = 1; n <= 32; n++) T->rifact[n + 1] = T->rifact[n] * n;

    /* intramolecular nonbonded pairs, src/init_arrays.f90:127-220 */
    {
        static const int pairs[42][2] = {
            {16, 21}, {16, 22}, {16, 23}, {16, 24}, {16, 26}, {16, 27}, {16, 28}, {16, 29},
            {17, 22}, {17, 23}, {17, 24}, {17, 27}, {17, 28}, {17, 29},
            {19, 22}, {19, 23}, {19, 24}, {19, 27}, {19, 28}, {19, 29},
            {20, 27}, {20, 28}, {20, 29},
            {21, 26}, {21, 27}, {21, 28}, {21, 29},
            {22, 25}, {22, 26}, {22, 27}, {22, 28}, {22, 29},
            {23, 25}, {23, 26}, {23, 27}, {23, 28}, {23, 29},
            {24, 25}, {24, 26}, {24, 27}, {24, 28}, {24, 29}};
        for (int k = 0; k < 42; k++) { T->iself[k + 1] = pairs[k][0]; T->jself[k + 1] = pairs[k][1]; }
    }
    /* bonds, src/init_arrays.f90:229-264 */
    for (int i = 1; i <= 18; i++) { T->ibond[i] = i; T->jbond[i] = i + 1; }
    {
        static const int b[10][2] = {{18, 20}, {20, 21}, {21, 22}, {21, 23}, {21, 24},
                                     {18, 25}, {25, 26}, {26, 27}, {26, 28}, {26, 29}};
        for (int k = 0; k < 10; k++) { T->ibond[19 + k] = b[k][0]; T->jbond[19 + k] = b[k][1]; }
    }
    /* masses, src/init_arrays.f90:266-312 */
    const double hy = 1.00794, carbon = 12.011, oxygen = 15.9994, si = 28.0855;
    const double me = carbon + 2.0 * hy, methyl = carbon + 3.0 * hy;
    {
        const double m[30] = {0, hy, oxygen, me, me, oxygen, me, me, oxygen, me, me,
                              oxygen, me, me, oxygen, me, me, me, si, methyl, oxygen,
                              si, methyl, methyl, methyl, oxygen, si, methyl, methyl, methyl};
        for (int i = 1; i <= 29; i++) T->ems[i] = m[i] / oxygen;
        T->emw[1] = oxygen / oxygen; T->emw[2] = hy / oxygen; T->emw[3] = hy / oxygen;
    }
    /* LJ parameters and charges, src/init_arrays.f90:314-474 */
    double sgs[30], eps[30], sgw[4], epw[4];
    {
        const double s_ahy = 2.6, e_ahy = 33.5, s_aox = 3.07, e_aox = 711.76;
        const double s_ome = 3.983, e_ome = 478.12, s_oox = 3.047, e_oox = 817.67;
        const double s_tme = 3.95, e_tme = 382.47, s_bsi = 3.385, e_bsi = 2448.0;
        const double s_box = 2.955, e_box = 849.3, s_bme = 3.786, e_bme = 753.2;
        const double S[30] = {0, s_ahy, s_aox, s_ome, s_ome, s_oox, s_ome, s_ome, s_oox, s_ome, s_ome,
                              s_oox, s_ome, s_ome, s_oox, s_ome, s_tme, s_tme, s_bsi, s_bme, s_box,
                              s_bsi, s_bme, s_bme, s_bme, s_box, s_bsi, s_bme, s_bme, s_bme};
        const double E[30] = {0, e_ahy, e_aox, e_ome, e_ome, e_oox, e_ome, e_ome, e_oox, e_ome, e_ome,
                              e_oox, e_ome, e_ome, e_oox, e_ome, e_tme, e_tme, e_bsi, e_bme, e_box,
                              e_bsi, e_bme, e_bme, e_bme, e_box, e_bsi, e_bme, e_bme, e_bme};
        const double Q[30] = {0, 0.435, -0.700, 0.265, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29, 0.29,
                              -0.58, 0.29, 0.29, -0.58, 0.29, 0.0, 0.0, 0.3, 0.0, -0.3,
                              0.15, 0.0, 0.0, 0.0, -0.3, 0.15, 0.0, 0.0, 0.0};
        for (int i = 1; i <= 29; i++) { sgs[i] = S[i] / sigma; eps[i] = E[i] / epsilon; T->rqs[i] = Q[i]; }
        sgw[1] = sigma / sigma; epw[1] = epsilon / epsilon; T->rqw[1] = -0.8476;
        sgw[2] = 0.0; epw[2] = 0.0; T->rqw[2] = 0.4238;
        sgw[3] = 0.0; epw[3] = 0.0; T->rqw[3] = 0.4238;
    }
    /* combined parameters, src/init_arrays.f90:476-507 */
    for (int i = 1; i <= 29; i++)
        for (int j = 1; j <= 29; j++) {
            T->sgss6[i][j] = pow6((sgs[i] + sgs[j]) / 2.0);
            T->epss[i][j] = sqrt(eps[i] * eps[j]);
        }
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 29; j++) {
            T->sgws6[i][j] = pow6((sgw[i] + sgs[j]) / 2.0);
            T->epws[i][j] = sqrt(epw[i] * eps[j]);
        }
    for (int i = 1; i <= 29; i++) {
        T->sgcs6[i] = pow6((3.19 / sigma + sgs[i]) / 2.0);
        T->epcs[i] = sqrt((392.0 / epsilon) * eps[i]);
    }
    /* squared constraint lengths, src/init_arrays.f90:509-574 */
    {
        const double ahox = 0.945, aoxme = 1.430, omeme = 1.516, omeox = 1.410, ooxme = 1.410;
        const double tmeme = 1.540, bsiox = 1.60, boxsi = 1.60, bsime = 1.88, bmesi = 1.88;
        const double d[29] = {0, ahox, aoxme, omeme, omeox, ooxme, omeme, omeox, ooxme, omeme, omeox,
                              ooxme, omeme, omeox, ooxme, omeme, tmeme, bmesi, bsime, bsiox, boxsi,
                              bsime, bsime, bsime, bsiox, boxsi, bsime, bsime, bsime};
        for (int i = 1; i <= 28; i++) T->dsqs[i] = d[i] * d[i] / (sigma * sigma);
        T->dsqw[1] = 1.0; T->dsqw[2] = 2.0 * sin(109.47 * pi180 / 2.0); T->dsqw[3] = 1.0;
        for (int i = 1; i <= 3; i++) T->dsqw[i] = T->dsqw[i] * T->dsqw[i] / (sigma * sigma);
    }
    /* angles, src/init_arrays.f90:576-695 */
    {
        const double a1 = 108.5, oxmeme = 108.0, meoxme = 112.0, memeox = 108.0, tri = 114.0;
        const double tet = 109.5, sios = 144.0;
        const double th[37] = {0, a1, oxmeme, memeox, meoxme, oxmeme, memeox, meoxme, oxmeme, memeox,
                               meoxme, oxmeme, memeox, meoxme, oxmeme, tri, tet, tet, tet, tet, tet,
                               tet, sios, sios, tet, tet, tet, tet, tet, tet, tet, tet, tet, tet, tet, tet, tet};
        for (int i = 1; i <= 36; i++) T->th[i] = th[i] * pi180;
        const double k5 = 519700.0, ksos = 118400.0, koso = 791200.0, kosm = 418400.0;
        const double kmso = 418400.0, kmsm = 418400.0;
        const double k[37] = {0, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5, k5,
                              kmsm, kmso, kmso, kmso, kmso, ksos, ksos, kosm, kosm, kosm, kmsm, kmsm,
                              kmsm, kosm, kosm, kosm, kmsm, kmsm, kmsm, koso};
        for (int i = 1; i <= 36; i++) T->rkth[i] = k[i] / epsilon;
        for (int i = 1; i <= 17; i++) { T->iang[i] = i; T->jang[i] = i + 1; T->kang[i] = i + 2; }
        /* angle triples, src/eval_valence.f90:13-95 */
        static const int a[19][3] = {{17, 18, 20}, {17, 18, 25}, {19, 18, 20}, {19, 18, 25}, {18, 25, 26},
                                     {18, 20, 21}, {20, 21, 22}, {20, 21, 23}, {20, 21, 24}, {22, 21, 24},
                                     {22, 21, 23}, {23, 21, 24}, {25, 26, 27}, {25, 26, 28}, {25, 26, 29},
                                     {27, 26, 28}, {27, 26, 29}, {28, 26, 29}, {20, 18, 25}};
        for (int q = 0; q < 19; q++) { T->iang[18 + q] = a[q][0]; T->jang[18 + q] = a[q][1]; T->kang[18 + q] = a[q][2]; }
    }
    /* dihedrals, src/init_arrays.f90:697-836 and quadruples src/eval_dihedral.f90:23-100 */
    {
        const double al[3] = {3490.0, -486.0, 3130.0};
        const double ommo[3] = {2940.0, -888.0, 12810.0};
        const double mmom[3] = {19860.0, -5853.0, 8956.0};
        const double momm[3] = {19860.0, -5853.0, 8956.0};
        const double aomm[3] = {2940.0, -888.0, 12810.0};
        const double tr[3] = {5903.8, -1134.0, 13159.0};
        const double *c[19] = {0, al, ommo, mmom, momm, ommo, mmom, momm, ommo, mmom, momm,
                               ommo, mmom, momm, aomm, tr, tr, tr, tr};
        for (int i = 1; i <= 18; i++) { T->dva[i] = c[i][0]; T->dvb[i] = c[i][1]; T->dvc[i] = c[i][2]; }
        for (int i = 19; i <= 30; i++) { T->dva[i] = 3770.0; T->dvb[i] = 0.0; T->dvc[i] = 0.0; }
        for (int i = 1; i <= 18; i++) { T->dva[i] /= 2.0; T->dvb[i] /= 2.0; T->dvc[i] /= 2.0; }
        for (int i = 1; i <= 30; i++) { T->dva[i] /= epsilon; T->dvb[i] /= epsilon; T->dvc[i] /= epsilon; }
        for (int i = 1; i <= 16; i++) { T->idv[i] = i; T->jdv[i] = i + 1; T->kdv[i] = i + 2; T->ldv[i] = i + 3; }
        static const int d[14][4] = {{16, 17, 18, 20}, {16, 17, 18, 25}, {17, 18, 20, 21}, {17, 18, 25, 26},
                                     {19, 18, 20, 21}, {19, 18, 25, 26}, {18, 20, 21, 22}, {18, 20, 21, 23},
                                     {18, 20, 21, 24}, {18, 25, 26, 27}, {18, 25, 26, 28}, {18, 25, 26, 29},
                                     {20, 18, 25, 26}, {21, 20, 18, 25}};
        for (int q = 0; q < 14; q++) {
            T->idv[17 + q] = d[q][0]; T->jdv[17 + q] = d[q][1]; T->kdv[17 + q] = d[q][2]; T->ldv[17 + q] = d[q][3];
        }
    }
}

/* ---------------- geometry: src/ibox.f90, src/init_box_dimensions.f90 ---------------- */

void orc_rank_xyz(const orc_sys *s, int rank, int *rx, int *ry, int *rz) {
    *rx = rank % s->nrx; *ry = (rank / s->nrx) % s->nry; *rz = rank / (s->nrx * s->nry);
}

/* ibox2 - 1, src/ibox.f90:127-139 */
int orc_rank_of(const orc_sys *s, double x, double y, double z) {
    int ix = (int)((x + s->rhsx) * s->nrx / s->rsdx);
    int iy = (int)((y + s->rhsy) * s->nry / s->rsdy);
    int iz = (int)((z + s->rhsz) * s->nrz / s->rsdz);
    if (ix < 0) ix = 0; if (ix >= s->nrx) ix = s->nrx - 1;
    if (iy < 0) iy = 0; if (iy >= s->nry) iy = s->nry - 1;
    if (iz < 0) iz = 0; if (iz >= s->nrz) iz = s->nrz - 1;
    return ix + s->nrx * (iy + s->nry * iz);
}

/* rcen2xtmp, src/init_box_dimensions.f90:40-42 */
void orc_rcen2(const orc_sys *s, int rank, double *cx, double *cy, double *cz) {
    int rx, ry, rz;
    orc_rank_xyz(s, rank, &rx, &ry, &rz);
    double bx = s->nrx, by = s->nry, bz = s->nrz;
    *cx = s->rsdx * (rx + 1) / bx - s->rhsx - s->rsdx / bx / 2.0;
    *cy = s->rsdy * (ry + 1) / by - s->rhsy - s->rsdy / by / 2.0;
    *cz = s->rsdz * (rz + 1) / bz - s->rhsz - s->rsdz / bz / 2.0;
}

static int clamp4(int v) { return v < 0 ? 0 : (v > 3 ? 3 : v); }

/* ibox64 - 1, src/ibox.f90:172-186 (result clamped to the rank's 4x4x4 cells) */
int orc_local64(const orc_sys *s, int rank, double x, double y, double z) {
    double cx, cy, cz;
    orc_rcen2(s, rank, &cx, &cy, &cz);
    double rap = x - cx + 2.0 * s->rs, rbp = y - cy + 2.0 * s->rs, rcp = z - cz + 2.0 * s->rs;
    return clamp4((int)(rap / s->rs)) + clamp4((int)(rbp / s->rs)) * 4 + clamp4((int)(rcp / s->rs)) * 16;
}

void orc_cell_xyz(const orc_sys *s, int c, int *ix, int *iy, int *iz) {
    *ix = c % s->ncx; *iy = (c / s->ncx) % s->ncy; *iz = c / (s->ncx * s->ncy);
}

int orc_cell_id(const orc_sys *s, int ix, int iy, int iz) {
    if (ix < 0 || iy < 0 || iz < 0 || ix >= s->ncx || iy >= s->ncy || iz >= s->ncz) return -1;
    return ix + s->ncx * (iy + s->ncy * iz);
}

/* key cell of a position: ibox2 selects the rank, ibox64 the cell in it
 * (src/read_config.f90:59-76, src/delete_w1.f90:54-66) */
int orc_keycell(const orc_sys *s, double x, double y, double z) {
    int r = orc_rank_of(s, x, y, z);
    int l = orc_local64(s, r, x, y, z);
    int rx, ry, rz;
    orc_rank_xyz(s, r, &rx, &ry, &rz);
    return orc_cell_id(s, 4 * rx + (l % 4), 4 * ry + (l / 4) % 4, 4 * rz + l / 16);
}

/* rcen4x(l), src/init_box_dimensions.f90:79-94, evaluated by the cell's own rank */
void orc_rcen4(const orc_sys *s, int c, double *cx, double *cy, double *cz) {
    int ix, iy, iz;
    orc_cell_xyz(s, c, &ix, &iy, &iz);
    int rank = (ix / 4) + s->nrx * ((iy / 4) + s->nry * (iz / 4));
    double c2x, c2y, c2z;
    orc_rcen2(s, rank, &c2x, &c2y, &c2z);
    double rs = s->rs;
    int i = ix % 4 + 1, j = iy % 4 + 1, k = iz % 4 + 1;
    *cx = 4.0 * rs * i / 4.0 - 2.0 * rs - 4.0 * rs / 8.0 + c2x;
    *cy = 4.0 * rs * j / 4.0 - 2.0 * rs - 4.0 * rs / 8.0 + c2y;
    *cz = 4.0 * rs * k / 4.0 - 2.0 * rs - 4.0 * rs / 8.0 + c2z;
}

/* src/ibox.f90:101-124 */
int orc_isCentral(double x, double y, double z, double cx, double cy, double cz) {
    double rs2 = ORC_RS / 2.0;
    return (x < cx + rs2 && x >= cx - rs2) && (y < cy + rs2 && y >= cy - rs2) && (z < cz + rs2 && z >= cz - rs2);
}

/* src/ibox.f90:75-98 */
int orc_isNearest(double x, double y, double z, double cx, double cy, double cz) {
    double r15 = 1.5 * ORC_RS;
    return (x < cx + r15 && x >= cx - r15) && (y < cy + r15 && y >= cy - r15) && (z < cz + r15 && z >= cz - r15);
}

/* neighbour order kmid(1..26), src/buildW2n.f90:24-37 */
const int ORC_KMID[26][3] = {
    {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {-1, 1, 0}, {-1, 0, 0}, {-1, -1, 0}, {0, -1, 0}, {1, -1, 0},
    {1, 0, 1}, {1, 1, 1}, {0, 1, 1}, {-1, 1, 1}, {-1, 0, 1}, {-1, -1, 1}, {0, -1, 1}, {1, -1, 1},
    {1, 0, -1}, {1, 1, -1}, {0, 1, -1}, {-1, 1, -1}, {-1, 0, -1}, {-1, -1, -1}, {0, -1, -1}, {1, -1, -1},
    {0, 0, 1}, {0, 0, -1}};

/* cell order of the (2R+1)^3 - (2R-1)^3 shell: lower and upper planes, then
 * south/north rows and west/east columns of each middle plane
 * (src/buildW2nn.f90:28-225, src/buildSnnn.f90:26-226) */
static int shell_offsets(int R, int out[][3]) {
    int n = 0;
    for (int dz = -R; dz <= R; dz += 2 * R)
        for (int dy = -R; dy <= R; dy++)
            for (int dx = -R; dx <= R; dx++) { out[n][0] = dx; out[n][1] = dy; out[n][2] = dz; n++; }
    for (int dz = -(R - 1); dz <= R - 1; dz++) {
        for (int dx = -R; dx <= R; dx++) { out[n][0] = dx; out[n][1] = -R; out[n][2] = dz; n++; }
        for (int dx = -R; dx <= R; dx++) { out[n][0] = dx; out[n][1] = R; out[n][2] = dz; n++; }
        for (int dy = -(R - 1); dy <= R - 1; dy++) { out[n][0] = -R; out[n][1] = dy; out[n][2] = dz; n++; }
        for (int dy = -(R - 1); dy <= R - 1; dy++) { out[n][0] = R; out[n][1] = dy; out[n][2] = dz; n++; }
    }
    return n;
}

void orc_list_push(orc_list *l, int key, int mol, int gsite, int type) {
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 16;
        l->e = (orc_ent *)realloc(l->e, sizeof(orc_ent) * l->cap);
    }
    orc_ent *e = &l->e[l->n++];
    e->key = key; e->mol = mol; e->gsite = gsite; e->type = type;
}

void orc_mlist_push(orc_mlist *l, int m) {
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 16;
        l->m = (int *)realloc(l->m, sizeof(int) * l->cap);
    }
    l->m[l->n++] = m;
}

/* Re-key every molecule to the cell of its key atom and split waters into w1
 * (all three sites in the key cell of the same rank) and w2.  This is the
 * global outcome of src/read_config.f90:44-175 and of the delete/add pairs
 * (src/delete_w1.f90:28-224, src/delete_w2.f90, src/delete_s.f90:33-43 with
 * the key atom at site 14). */
void orc_classify(orc_sys *s) {
    for (int c = 0; c < s->ncell; c++) { s->cw1[c].n = 0; s->cw2[c].n = 0; s->cs[c].n = 0; }
    for (int m = 0; m < s->nw; m++) {
        int g = 3 * m;
        double xO = s->x[g], yO = s->y[g], zO = s->z[g];
        int ibO = orc_rank_of(s, xO, yO, zO);
        int ibG = orc_rank_of(s, s->x[g + 1], s->y[g + 1], s->z[g + 1]);
        int ibH = orc_rank_of(s, s->x[g + 2], s->y[g + 2], s->z[g + 2]);
        int w1 = 0;
        if (ibO == ibG && ibO == ibH) {
            int lO = orc_local64(s, ibO, xO, yO, zO);
            int lG = orc_local64(s, ibO, s->x[g + 1], s->y[g + 1], s->z[g + 1]);
            int lH = orc_local64(s, ibO, s->x[g + 2], s->y[g + 2], s->z[g + 2]);
            w1 = (lO == lG && lO == lH);
        }
        s->key[m] = orc_keycell(s, xO, yO, zO);
        s->w1[m] = w1;
        orc_mlist_push(w1 ? &s->cw1[s->key[m]] : &s->cw2[s->key[m]], m);
    }
    for (int q = 0; q < s->ns; q++) {
        int m = s->nw + q;
        int g = orc_first_site(s, m) + 13; /* site 14 */
        s->key[m] = orc_keycell(s, s->x[g], s->y[g], s->z[g]);
        s->w1[m] = 0;
        orc_mlist_push(&s->cs[s->key[m]], m);
    }
}

static void scan_w2_cell(orc_sys *s, int i, int k, double cx, double cy, double cz,
                         orc_list *central, orc_list *n26, int central_too) {
    orc_mlist *ml = &s->cw2[k];
    for (int a = 0; a < ml->n; a++) {
        int m = ml->m[a];
        for (int t = 0; t < 3; t++) {
            int g = 3 * m + t;
            int bc = orc_isCentral(s->x[g], s->y[g], s->z[g], cx, cy, cz);
            if (central_too && bc) orc_list_push(central, k, m, g, t + 1);
            int bn = orc_isNearest(s->x[g], s->y[g], s->z[g], cx, cy, cz);
            if (central_too) {
                if (bn && !bc) orc_list_push(n26, k, m, g, t + 1);
            } else if (bn) {
                orc_list_push(n26, k, m, g, t + 1);
            }
        }
    }
    (void)i;
}

static void scan_s_cell(orc_sys *s, int k, double cx, double cy, double cz,
                        orc_list *central, orc_list *n26, int central_too) {
    orc_mlist *ml = &s->cs[k];
    for (int a = 0; a < ml->n; a++) {
        int m = ml->m[a];
        int g0 = orc_first_site(s, m);
        for (int t = 0; t < ORC_NSURF_SITE; t++) {
            int g = g0 + t;
            int bc = orc_isCentral(s->x[g], s->y[g], s->z[g], cx, cy, cz);
            if (central_too && bc) orc_list_push(central, k, m, g, t + 1);
            int bn = orc_isNearest(s->x[g], s->y[g], s->z[g], cx, cy, cz);
            if (central_too) {
                if (bn && !bc) orc_list_push(n26, k, m, g, t + 1);
            } else if (bn) {
                orc_list_push(n26, k, m, g, t + 1);
            }
        }
    }
}

/* src/buildW2.f90, src/buildW2n.f90, src/buildW2nn.f90, src/buildS.f90,
 * src/buildSn.f90, src/buildSnn.f90, src/buildSnnn.f90 */
void orc_build_lists(orc_sys *s) {
    static int sh2[98][3], sh3[218][3];
    int n2 = shell_offsets(2, sh2), n3 = shell_offsets(3, sh3);
    for (int i = 0; i < s->ncell; i++) {
        s->W2C[i].n = s->W226[i].n = s->W2nC[i].n = s->W2n26[i].n = s->W2nn[i].n = 0;
        s->SC[i].n = s->S26[i].n = s->SnC[i].n = s->Sn26[i].n = 0;
        s->SnnC[i].n = s->Snn26[i].n = s->Snnn[i].n = 0;
    }
    for (int i = 0; i < s->ncell; i++) {
        double cx, cy, cz;
        orc_rcen4(s, i, &cx, &cy, &cz);
        int ix, iy, iz;
        orc_cell_xyz(s, i, &ix, &iy, &iz);
        /* buildW2: src/buildW2.f90:16-71 */
        scan_w2_cell(s, i, i, cx, cy, cz, &s->W2C[i], &s->W226[i], 1);
        /* buildS: src/buildS.f90:15-70 */
        scan_s_cell(s, i, cx, cy, cz, &s->SC[i], &s->S26[i], 1);
        /* buildW2n / buildSn: 26 neighbours in kmid order */
        for (int j = 0; j < 26; j++) {
            int k = orc_cell_id(s, ix + ORC_KMID[j][0], iy + ORC_KMID[j][1], iz + ORC_KMID[j][2]);
            if (k < 0) continue;
            scan_w2_cell(s, i, k, cx, cy, cz, &s->W2nC[i], &s->W2n26[i], 1);
        }
        for (int j = 0; j < 26; j++) {
            int k = orc_cell_id(s, ix + ORC_KMID[j][0], iy + ORC_KMID[j][1], iz + ORC_KMID[j][2]);
            if (k < 0) continue;
            scan_s_cell(s, k, cx, cy, cz, &s->SnC[i], &s->Sn26[i], 1);
        }
        /* buildW2nn: src/buildW2nn.f90:18-229 (isNearest only) */
        for (int j = 0; j < n2; j++) {
            int k = orc_cell_id(s, ix + sh2[j][0], iy + sh2[j][1], iz + sh2[j][2]);
            if (k < 0) continue;
            scan_w2_cell(s, i, k, cx, cy, cz, NULL, &s->W2nn[i], 0);
        }
        /* buildSnn: src/buildSnn.f90:16-315 */
        for (int j = 0; j < n2; j++) {
            int k = orc_cell_id(s, ix + sh2[j][0], iy + sh2[j][1], iz + sh2[j][2]);
            if (k < 0) continue;
            scan_s_cell(s, k, cx, cy, cz, &s->SnnC[i], &s->Snn26[i], 1);
        }
        /* buildSnnn: src/buildSnnn.f90:16-227 (isNearest only) */
        for (int j = 0; j < n3; j++) {
            int k = orc_cell_id(s, ix + sh3[j][0], iy + sh3[j][1], iz + sh3[j][2]);
            if (k < 0) continue;
            scan_s_cell(s, k, cx, cy, cz, NULL, &s->Snnn[i], 0);
        }
    }
}

/* src/buildinternal.f90:13-63: per surfactant site, the sites of its own
 * molecule outside the 27-cell block of the site's cell (10^3 grid of the
 * key rank, ibox1000 and rcen1000 at src/ibox.f90:206-220,
 * src/init_box_dimensions.f90:155-170). */
void orc_buildinternal(orc_sys *s) {
    memset(s->isub, 0, sizeof(int) * 28 * ORC_NSURF_SITE * (size_t)s->ns);
    for (int q = 0; q < s->ns; q++) {
        int m = s->nw + q;
        int g0 = orc_first_site(s, m);
        int kx, ky, kz;
        orc_cell_xyz(s, s->key[m], &kx, &ky, &kz);
        int rank = (kx / 4) + s->nrx * ((ky / 4) + s->nry * (kz / 4));
        double c2x, c2y, c2z;
        orc_rcen2(s, rank, &c2x, &c2y, &c2z);
        double rs = s->rs;
        for (int j = 0; j < ORC_NSURF_SITE; j++) {
            double xm = s->x[g0 + j], ym = s->y[g0 + j], zm = s->z[g0 + j];
            int li = (int)((xm - c2x + 5.0 * rs) / rs) + 1;
            int lj = (int)((ym - c2y + 5.0 * rs) / rs) + 1;
            int lk = (int)((zm - c2z + 5.0 * rs) / rs) + 1;
            double cx = 10.0 * rs * li / 10.0 - 10.0 * rs / 2.0 - 10.0 * rs / 20.0 + c2x;
            double cy = 10.0 * rs * lj / 10.0 - 10.0 * rs / 2.0 - 10.0 * rs / 20.0 + c2y;
            double cz = 10.0 * rs * lk / 10.0 - 10.0 * rs / 2.0 - 10.0 * rs / 20.0 + c2z;
            int *out = &s->isub[((size_t)q * ORC_NSURF_SITE + j) * 28];
            int n = 0;
            for (int k = 0; k < ORC_NSURF_SITE; k++) {
                if (k == j) continue;
                if (!orc_isNearest(s->x[g0 + k], s->y[g0 + k], s->z[g0 + k], cx, cy, cz)) out[n++] = k + 1;
            }
        }
    }
}
