/*
 * TEST INFRASTRUCTURE ONLY (CPU oracle; parity unpinned - see orc.h).
 * The reference's order-4 fast multipole far field: P2M at the 12-reduced-A
 * L4 cells, M2M to L3 and L2, M2L at L2 (non-adjacent L2 boxes), L3 and L4
 * (children of the parent's neighbours that are not adjacent), L2L down to
 * L4 and the L2P force at every located site.  Geometry of every pass follows
 * the reference's rank-relative centre formulas.
 */
#include "orc.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define T ORC_T
#define LP ORC_LP

/* igetIndex(n,m) - 1, src/ifma.f90:1-9 */
static inline int gidx(int n, int m) { return n * (n + 1) + m; }
static inline double fact(int n) { return T.rifact[n + 1]; }
static inline double neg1pow(int n) { return (n % 2 == 0) ? 1.0 : -1.0; }

/* binomial coefficient C(n, k) from the factorial table */
static inline double binom(int n, int k) { return fact(n) / (fact(k) * fact(n - k)); }

/* Associated Legendre function P_l^m(x) with the Condon-Shortley phase, from
 * the explicit polynomial that Rodrigues' formula gives when the m-th
 * derivative of P_l(x) = 2^-l sum_k (-1)^k C(l,k) C(2l-2k,l) x^(l-2k) is taken
 * term by term (Abramowitz & Stegun 8.6.6 with 22.3.8):
 *   P_l^m(x) = (-1)^m (1-x^2)^(m/2) 2^-l
 *              sum_{k=0}^{(l-m)/2} (-1)^k C(l,k) C(2l-2k,l) (l-2k)! / (l-2k-m)! x^(l-2k-m).
 * The reference's edge conventions are kept (src/rLegendreP.f90:11-19):
 * P(-1,0) = 1 and P(l,m) = 0 for m > l.  Orders here stay at l <= 2p = 8,
 * where the sum has at most 5 terms. */
static double legendre(int l, int m, double x) {
    if (l == -1 && m == 0) return 1.0;
    if (m > l) return 0.0;
    double sum = 0.0;
    for (int k = 0; 2 * k <= l - m; k++) {
        const int p = l - 2 * k - m;
        double xp = 1.0;
        for (int i = 0; i < p; i++) xp *= x;
        const double c = binom(l, k) * binom(2 * l - 2 * k, l) * fact(l - 2 * k) / fact(p);
        sum += (k % 2 ? -c : c) * xp;
    }
    double w = 1.0;   /* (1 - x^2)^(m/2) */
    const double s = sqrt((1.0 - x) * (1.0 + x));
    for (int i = 0; i < m; i++) w *= s;
    double two_l = 1.0;
    for (int i = 0; i < l; i++) two_l *= 2.0;
    return (m % 2 ? -w : w) * sum / two_l;
}

/* Ylm, src/ifma.f90:12-26 */
static double complex Ylm(int n, int m, double alpha, double beta) {
    int am = abs(m);
    double r = sqrt(fact(n - am) / fact(n + am)) * legendre(n, am, cos(alpha));
    return r * (cos(m * beta) + I * sin(m * beta));
}
/* rfctr, src/ifma.f90:29-38 */
static inline double rfctr(int n, int m) { return sqrt(fact(n - abs(m)) / fact(n + abs(m))); }
/* rAnm, src/ifma.f90:41-52 */
static inline double rAnm(int n, int m) { return neg1pow(n) / sqrt(fact(n - m) * fact(n + m)); }
/* iIkm1..3, src/ifma.f90:55-85 */
static inline double iIkm1(int k, int m) { return neg1pow(abs((abs(k) - abs(m) - abs(k - m)) / 2)); }
static inline double iIkm2(int k, int m) { return neg1pow(abs((abs(k - m) - abs(k) - abs(m)) / 2)); }
static inline double iIkm3(int k, int m) { return neg1pow(abs((abs(m) - abs(m - k) - abs(k)) / 2)); }

static inline double ipow(double x, int n) {
    double r = 1.0;
    if (n >= 0) { for (int i = 0; i < n; i++) r *= x; return r; }
    for (int i = 0; i < -n; i++) r *= x;
    return 1.0 / r;
}
static inline double complex cpowi(double complex z, int n) {
    double complex r = 1.0;
    for (int i = 0; i < abs(n); i++) r *= z;
    return n >= 0 ? r : 1.0 / r;
}

static void sph(double x, double y, double z, double *rho, double *alpha, double *beta) {
    *rho = sqrt(x * x + y * y + z * z);
    *alpha = acos(z / *rho);
    *beta = atan2(y, x);
}

/* rank-relative centres, src/init_box_dimensions.f90:62-132 */
static void rcen3_local(const orc_sys *s, int rank, int i, int j, int k, double *c) {
    double c2[3];
    orc_rcen2(s, rank, &c2[0], &c2[1], &c2[2]);
    int q[3] = {i, j, k};
    for (int d = 0; d < 3; d++) c[d] = 4.0 * s->rs * q[d] / 2.0 - 2.0 * s->rs - 4.0 * s->rs / 4.0 + c2[d];
}
static void rcen3Ljk3(const orc_sys *s, int rank, int i, int j, int k, double *c) {
    double c2[3];
    orc_rcen2(s, rank, &c2[0], &c2[1], &c2[2]);
    int q[3] = {i, j, k};
    for (int d = 0; d < 3; d++) c[d] = 12.0 * s->rs * q[d] / 6.0 - 6.0 * s->rs - 12.0 * s->rs / 12.0 + c2[d];
}
static void rcen4Ljk4(const orc_sys *s, int rank, int i, int j, int k, double *c) {
    double c2[3];
    orc_rcen2(s, rank, &c2[0], &c2[1], &c2[2]);
    int q[3] = {i, j, k};
    for (int d = 0; d < 3; d++) c[d] = 8.0 * s->rs * q[d] / 8.0 - 8.0 * s->rs / 2.0 - 8.0 * s->rs / 16.0 + c2[d];
}

/* iterate the atoms located in L4 cell c in the reference's P2M/L2P order
 * (w1, W2Central, SCentral, W2nCentral, SnCentral, SnnCentral,
 * src/computeOnm4.f90:36-138).  Returns the count; fills site and charge. */
static int located_atoms(const orc_sys *s, int c, int *site, double *q) {
    int n = 0;
    const orc_mlist *L = &s->cw1[c];
    for (int a = 0; a < L->n; a++)
        for (int t = 1; t <= 3; t++) { site[n] = 3 * L->m[a] + t - 1; q[n] = T.rqw[t]; n++; }
    const orc_list *lists[5] = {&s->W2C[c], &s->SC[c], &s->W2nC[c], &s->SnC[c], &s->SnnC[c]};
    for (int li = 0; li < 5; li++) {
        const orc_list *Ls = lists[li];
        for (int b = 0; b < Ls->n; b++) {
            site[n] = Ls->e[b].gsite;
            int ty = Ls->e[b].type;
            q[n] = (li == 0) ? T.rqw[ty] : (li == 2 ? T.rqw[2] : T.rqs[ty]);
            n++;
        }
    }
    return n;
}

static int max_located(const orc_sys *s) {
    int mx = 0;
    for (int c = 0; c < s->ncell; c++) {
        int n = 3 * s->cw1[c].n + s->W2C[c].n + s->SC[c].n + s->W2nC[c].n + s->SnC[c].n + s->SnnC[c].n;
        if (n > mx) mx = n;
    }
    return mx;
}

/* M2L from source coefficients O at vector d (source - target) into L,
 * src/computeLjk4.f90:130-158 */
static void m2l(const double complex *O, double dx, double dy, double dz, double complex *L) {
    double rho, al, be;
    sph(dx, dy, dz, &rho, &al, &be);
    for (int j = 0; j <= ORC_P; j++)
        for (int k = 0; k <= j; k++) {
            int ic = gidx(j, k);
            double rAjk = rAnm(j, k);
            for (int n = 0; n <= ORC_P; n++)
                for (int m = -n; m <= n; m++) {
                    double complex ctmp = O[gidx(n, m)] * Ylm(j + n, m - k, al, be);
                    double rtmp = iIkm2(k, m) * rAjk * rAnm(n, m) / (neg1pow(n) * rAnm(j + n, m - k) * ipow(rho, j + n + 1));
                    L[ic] += rtmp * ctmp;
                }
            if (k > 0) L[gidx(j, -k)] = conj(L[ic]);
        }
}

/* M2M of child coefficients O at vector d (child centre - parent centre)
 * into the parent's Op, src/computeOnm3.f90:47-94 */
static void m2m(const double complex *O, double dx, double dy, double dz, double complex *Op) {
    double rho, al, be;
    sph(dx, dy, dz, &rho, &al, &be);
    for (int j = 0; j <= ORC_P; j++)
        for (int k = 0; k <= j; k++) {
            int ic = gidx(j, k);
            double rAjk = rAnm(j, k);
            for (int n = 0; n <= j; n++)
                for (int m = -n; m <= n; m++) {
                    if (j - n - abs(k - m) < 0) continue;
                    double complex ctmp = O[gidx(j - n, k - m)] * Ylm(n, -m, al, be);
                    double rtmp = iIkm1(k, m) * rAnm(n, m) * rAnm(j - n, k - m) * ipow(rho, n) / rAjk;
                    Op[ic] += rtmp * ctmp;
                }
            if (k > 0) Op[gidx(j, -k)] = conj(Op[ic]);
        }
}

/* L2L of parent coefficients L at vector d (parent centre - child centre)
 * into the child's Lc, src/shiftLjk3.f90:44-87 */
static void l2l(const double complex *L, double dx, double dy, double dz, double complex *Lc) {
    double rho, al, be;
    sph(dx, dy, dz, &rho, &al, &be);
    for (int j = 0; j <= ORC_P; j++)
        for (int k = 0; k <= j; k++) {
            int ic = gidx(j, k);
            double rAjk = rAnm(j, k);
            for (int n = 0; n <= ORC_P; n++)
                for (int m = -n; m <= n; m++) {
                    if (n - j - abs(m - k) < 0) continue;
                    double complex ctmp = L[gidx(n, m)] * Ylm(n - j, m - k, al, be);
                    double rtmp = iIkm3(k, m) * rAnm(n - j, m - k) * rAjk * ipow(rho, n - j) / (neg1pow(n + j) * rAnm(n, m));
                    Lc[ic] += rtmp * ctmp;
                }
            if (k > 0) Lc[gidx(j, -k)] = conj(Lc[ic]);
        }
}

void orc_fma_build(orc_sys *s) {
    const int n4x = s->ncx, n4y = s->ncy, n4z = s->ncz;
    const int n3x = n4x / 2, n3y = n4y / 2, n3z = n4z / 2;
    const int n3 = n3x * n3y * n3z;
    memset(s->cO4, 0, sizeof(double complex) * LP * s->ncell);
    memset(s->cO3, 0, sizeof(double complex) * LP * n3);
    memset(s->cO2, 0, sizeof(double complex) * LP * s->nrank);
    memset(s->cL2, 0, sizeof(double complex) * LP * s->nrank);
    memset(s->cL3, 0, sizeof(double complex) * LP * n3);
    memset(s->cL4, 0, sizeof(double complex) * LP * s->ncell);

    /* P2M, src/computeOnm4.f90:24-162 (cells in parallel, scratch per thread) */
    const int mx = max_located(s) + 1;
#pragma omp parallel
    {
    int *site = (int *)malloc(sizeof(int) * mx);
    double *q = (double *)malloc(sizeof(double) * mx);
    double *rho = (double *)malloc(sizeof(double) * mx), *al = (double *)malloc(sizeof(double) * mx), *be = (double *)malloc(sizeof(double) * mx);
#pragma omp for schedule(dynamic, 4)
    for (int c = 0; c < s->ncell; c++) {
        double cx, cy, cz;
        orc_rcen4(s, c, &cx, &cy, &cz);
        int n = located_atoms(s, c, site, q);
        for (int a = 0; a < n; a++) sph(s->x[site[a]] - cx, s->y[site[a]] - cy, s->z[site[a]] - cz, &rho[a], &al[a], &be[a]);
        double complex *O = &s->cO4[(size_t)LP * c];
        for (int nn = 0; nn <= ORC_P; nn++)
            for (int m = 0; m <= nn; m++) {
                int ic = gidx(nn, m);
                for (int a = 0; a < n; a++) O[ic] += q[a] * ipow(rho[a], nn) * Ylm(nn, -m, al[a], be[a]);
                if (m > 0) O[gidx(nn, -m)] = conj(O[ic]);
            }
    }
    free(site); free(q); free(rho); free(al); free(be);
    }

    /* M2M L4 -> L3, src/computeOnm3.f90:27-98 (each parent on its own) */
#pragma omp parallel for schedule(static)
    for (int z3 = 0; z3 < n3z; z3++)
        for (int y3 = 0; y3 < n3y; y3++)
            for (int x3 = 0; x3 < n3x; x3++) {
                int rank = (x3 / 2) + s->nrx * ((y3 / 2) + s->nry * (z3 / 2));
                double c3[3];
                rcen3_local(s, rank, x3 % 2 + 1, y3 % 2 + 1, z3 % 2 + 1, c3);
                double complex *Op = &s->cO3[(size_t)LP * (x3 + n3x * (y3 + n3y * z3))];
                for (int jj = 0; jj < 8; jj++) {
                    int cx4 = 2 * x3 + (jj & 1), cy4 = 2 * y3 + ((jj >> 1) & 1), cz4 = 2 * z3 + ((jj >> 2) & 1);
                    int c = orc_cell_id(s, cx4, cy4, cz4);
                    double c4[3];
                    orc_rcen4(s, c, &c4[0], &c4[1], &c4[2]);
                    m2m(&s->cO4[(size_t)LP * c], -c3[0] + c4[0], -c3[1] + c4[1], -c3[2] + c4[2], Op);
                }
            }
    /* M2M L3 -> L2, src/computeOnm2.f90:13-62 */
#pragma omp parallel for schedule(dynamic, 1)
    for (int rank = 0; rank < s->nrank; rank++) {
        int rx, ry, rz;
        orc_rank_xyz(s, rank, &rx, &ry, &rz);
        double c2[3];
        orc_rcen2(s, rank, &c2[0], &c2[1], &c2[2]);
        for (int kk = 0; kk < 8; kk++) {
            int i = kk & 1, j = (kk >> 1) & 1, k = (kk >> 2) & 1;
            double c3[3];
            rcen3_local(s, rank, i + 1, j + 1, k + 1, c3);
            int l3 = (2 * rx + i) + n3x * ((2 * ry + j) + n3y * (2 * rz + k));
            m2m(&s->cO3[(size_t)LP * l3], -c2[0] + c3[0], -c2[1] + c3[1], -c2[2] + c3[2], &s->cO2[(size_t)LP * rank]);
        }
    }
    /* M2L at L2 over non-adjacent L2 boxes, src/computeLjk2.f90:17-72 */
#pragma omp parallel for schedule(dynamic, 1)
    for (int rank = 0; rank < s->nrank; rank++) {
        int rx, ry, rz;
        orc_rank_xyz(s, rank, &rx, &ry, &rz);
        double c2[3];
        orc_rcen2(s, rank, &c2[0], &c2[1], &c2[2]);
        for (int kk = 0; kk < s->nrz; kk++)
            for (int jj = 0; jj < s->nry; jj++)
                for (int ii = 0; ii < s->nrx; ii++) {
                    if (!(abs(ii - rx) > 1 || abs(jj - ry) > 1 || abs(kk - rz) > 1)) continue;
                    int l = ii + s->nrx * (jj + s->nry * kk);
                    double cl[3];
                    orc_rcen2(s, l, &cl[0], &cl[1], &cl[2]);
                    m2l(&s->cO2[(size_t)LP * l], cl[0] - c2[0], cl[1] - c2[1], cl[2] - c2[2], &s->cL2[(size_t)LP * rank]);
                }
    }
    /* L2L L2 -> L3, src/shiftLjk2.f90:16-60 */
#pragma omp parallel for schedule(dynamic, 1)
    for (int rank = 0; rank < s->nrank; rank++) {
        int rx, ry, rz;
        orc_rank_xyz(s, rank, &rx, &ry, &rz);
        double c2[3];
        orc_rcen2(s, rank, &c2[0], &c2[1], &c2[2]);
        for (int kk = 0; kk < 8; kk++) {
            int i = kk & 1, j = (kk >> 1) & 1, k = (kk >> 2) & 1;
            double c3[3];
            rcen3_local(s, rank, i + 1, j + 1, k + 1, c3);
            int l3 = (2 * rx + i) + n3x * ((2 * ry + j) + n3y * (2 * rz + k));
            l2l(&s->cL2[(size_t)LP * rank], c2[0] - c3[0], c2[1] - c3[1], c2[2] - c3[2], &s->cL3[(size_t)LP * l3]);
        }
    }
    /* M2L at L3 over the 6^3 window, src/computeLjk3.f90:45-102 */
#pragma omp parallel for schedule(dynamic, 1)
    for (int rank = 0; rank < s->nrank; rank++) {
        int rx, ry, rz;
        orc_rank_xyz(s, rank, &rx, &ry, &rz);
        for (int ib = 0; ib < 8; ib++) {
            int bi = ib & 1, bj = (ib >> 1) & 1, bk = (ib >> 2) & 1;
            int ip[3] = {3 + bi, 3 + bj, 3 + bk};
            double c3[3];
            rcen3_local(s, rank, bi + 1, bj + 1, bk + 1, c3);
            int l3t = (2 * rx + bi) + n3x * ((2 * ry + bj) + n3y * (2 * rz + bk));
            for (int kk = 1; kk <= 6; kk++)
                for (int jj = 1; jj <= 6; jj++)
                    for (int ii = 1; ii <= 6; ii++) {
                        if (!(abs(ii - ip[0]) > 1 || abs(jj - ip[1]) > 1 || abs(kk - ip[2]) > 1)) continue;
                        int gx = 2 * rx + ii - 3, gy = 2 * ry + jj - 3, gz = 2 * rz + kk - 3;
                        if (gx < 0 || gy < 0 || gz < 0 || gx >= n3x || gy >= n3y || gz >= n3z) continue;
                        double cl[3];
                        rcen3Ljk3(s, rank, ii, jj, kk, cl);
                        m2l(&s->cO3[(size_t)LP * (gx + n3x * (gy + n3y * gz))], cl[0] - c3[0], cl[1] - c3[1], cl[2] - c3[2],
                            &s->cL3[(size_t)LP * l3t]);
                    }
        }
    }
    /* L2L L3 -> L4, src/shiftLjk3.f90:27-91 */
#pragma omp parallel for schedule(static)
    for (int z3 = 0; z3 < n3z; z3++)
        for (int y3 = 0; y3 < n3y; y3++)
            for (int x3 = 0; x3 < n3x; x3++) {
                int rank = (x3 / 2) + s->nrx * ((y3 / 2) + s->nry * (z3 / 2));
                double c3[3];
                rcen3_local(s, rank, x3 % 2 + 1, y3 % 2 + 1, z3 % 2 + 1, c3);
                double complex *Lp = &s->cL3[(size_t)LP * (x3 + n3x * (y3 + n3y * z3))];
                for (int jj = 0; jj < 8; jj++) {
                    int c = orc_cell_id(s, 2 * x3 + (jj & 1), 2 * y3 + ((jj >> 1) & 1), 2 * z3 + ((jj >> 2) & 1));
                    double c4[3];
                    orc_rcen4(s, c, &c4[0], &c4[1], &c4[2]);
                    l2l(Lp, c3[0] - c4[0], c3[1] - c4[1], c3[2] - c4[2], &s->cL4[(size_t)LP * c]);
                }
            }
    /* M2L at L4 over the 6^3 window of each L3 parent, src/computeLjk4.f90:58-172
     * (every target cell on its own, in parallel) */
#pragma omp parallel for schedule(dynamic, 4)
    for (int c = 0; c < s->ncell; c++) {
        int ix, iy, iz;
        orc_cell_xyz(s, c, &ix, &iy, &iz);
        int rank = (ix / 4) + s->nrx * ((iy / 4) + s->nry * (iz / 4));
        /* 8-grid coordinates (1-based) of this cell and of its parent's window */
        int jp[3] = {ix % 4 + 3, iy % 4 + 3, iz % 4 + 3};
        int lo[3] = {((ix % 4) / 2) * 2 + 1, ((iy % 4) / 2) * 2 + 1, ((iz % 4) / 2) * 2 + 1};
        double c4[3];
        orc_rcen4(s, c, &c4[0], &c4[1], &c4[2]);
        int rx, ry, rz;
        orc_rank_xyz(s, rank, &rx, &ry, &rz);
        for (int kk = lo[2]; kk <= lo[2] + 5; kk++)
            for (int jj = lo[1]; jj <= lo[1] + 5; jj++)
                for (int ii = lo[0]; ii <= lo[0] + 5; ii++) {
                    if (!(abs(ii - jp[0]) > 1 || abs(jj - jp[1]) > 1 || abs(kk - jp[2]) > 1)) continue;
                    int sc = orc_cell_id(s, 4 * rx + ii - 3, 4 * ry + jj - 3, 4 * rz + kk - 3);
                    if (sc < 0) continue;
                    double cl[3];
                    rcen4Ljk4(s, rank, ii, jj, kk, cl);
                    m2l(&s->cO4[(size_t)LP * sc], cl[0] - c4[0], cl[1] - c4[1], cl[2] - c4[2], &s->cL4[(size_t)LP * c]);
                }
    }
}

/* potential and force of the local expansion at relative position (x,y,z),
 * src/evalLjk4.f90:38-66.  phi = sum Re[L rfctr P_j^|k| e^{ik phi} r^j]. */
static void l2p(const double complex *L, double rx, double ry, double rz, double rqq,
                double *fx, double *fy, double *fz, double *phi) {
    const double complex zn = I;
    double rr = sqrt(rx * rx + ry * ry + rz * rz);
    double rp1 = rz / rr;
    double complex rp2 = (rx + ry * zn) / sqrt(rx * rx + ry * ry);
    double rp3 = 1.0 / (rx * rx + ry * ry);
    double ph = 0.0;
    for (int j = 0; j <= ORC_P; j++)
        for (int k = -j; k <= j; k++) {
            int ic = gidx(j, k);
            double complex rq0 = L[ic] * rfctr(j, k) * cpowi(rp2, k) * ipow(rr, j - 1);
            double rq1 = (j + abs(k)) * legendre(j - 1, abs(k), rp1);
            double rq2 = legendre(j, abs(k), rp1);
            double rq3 = rx * rz * rq1;
            double complex rq4 = (zn * k * ry - j * rx) * rr * rq2;
            double rq5 = ry * rz * rq1;
            double complex rq6 = -(zn * k * rx + j * ry) * rr * rq2;
            *fx += creal(rqq * rp3 * rq0 * (rq3 + rq4));
            *fy += creal(rqq * rp3 * rq0 * (rq5 + rq6));
            *fz -= creal(rqq * rq0 * rq1);
            ph += creal(rq0 * rr * rq2);
        }
    if (phi) *phi = ph;
}

void orc_evalLjk4(orc_sys *s) {
    const int mx = max_located(s) + 1;
#pragma omp parallel
    {
    int *site = (int *)malloc(sizeof(int) * mx);
    double *q = (double *)malloc(sizeof(double) * mx);
#pragma omp for schedule(dynamic, 4)
    for (int c = 0; c < s->ncell; c++) {
        double cx, cy, cz;
        orc_rcen4(s, c, &cx, &cy, &cz);
        int n = located_atoms(s, c, site, q);
        for (int a = 0; a < n; a++) {
            int g = site[a];
            l2p(&s->cL4[(size_t)LP * c], s->x[g] - cx, s->y[g] - cy, s->z[g] - cz, q[a] * ORC_XPI,
                &s->fx[g], &s->fy[g], &s->fz[g], NULL);
        }
    }
    free(site); free(q);
    }
}

/* far-field energy 1/2 sum_i q_i xpi phi(r_i) (the reference computes none) */
double orc_fma_energy(const orc_sys *s) {
    int mx = max_located(s) + 1;
    int *site = (int *)malloc(sizeof(int) * mx);
    double *q = (double *)malloc(sizeof(double) * mx);
    double e = 0.0;
    for (int c = 0; c < s->ncell; c++) {
        double cx, cy, cz;
        orc_rcen4(s, c, &cx, &cy, &cz);
        int n = located_atoms(s, c, site, q);
        for (int a = 0; a < n; a++) {
            int g = site[a];
            double fx = 0, fy = 0, fz = 0, phi = 0;
            l2p(&s->cL4[(size_t)LP * c], s->x[g] - cx, s->y[g] - cy, s->z[g] - cz, q[a] * ORC_XPI, &fx, &fy, &fz, &phi);
            e += 0.5 * q[a] * ORC_XPI * phi;
        }
    }
    free(site); free(q);
    return e;
}

/* ---- single-operation entry points for the configuration-preset oracle
 * (orc_cfg.c), which builds its own periodic interaction lists on top of
 * the same expansion formulas. */

/* P2M of one charge at (dx, dy, dz) from the cell centre,
 * src/computeOnm4.f90:142-162: O_n^m += q rho^n Y(n, -m) */
void orc_p2m_add(double complex *O, double q, double dx, double dy, double dz) {
    double rho, al, be;
    sph(dx, dy, dz, &rho, &al, &be);
    for (int nn = 0; nn <= ORC_P; nn++)
        for (int m = 0; m <= nn; m++) {
            double complex v = q * ipow(rho, nn) * Ylm(nn, -m, al, be);
            O[gidx(nn, m)] += v;
            if (m > 0) O[gidx(nn, -m)] += conj(v);
        }
}
void orc_m2m_apply(const double complex *O, double dx, double dy, double dz, double complex *Op) { m2m(O, dx, dy, dz, Op); }
void orc_m2l_apply(const double complex *O, double dx, double dy, double dz, double complex *L) { m2l(O, dx, dy, dz, L); }
void orc_l2l_apply(const double complex *L, double dx, double dy, double dz, double complex *Lc) { l2l(L, dx, dy, dz, Lc); }
void orc_l2p_apply(const double complex *L, double rx, double ry, double rz, double rqq, double *fx, double *fy,
                   double *fz, double *phi) {
    l2p(L, rx, ry, rz, rqq, fx, fy, fz, phi);
}
/* the associated Legendre function above (exported for its test) */
double orc_legendre(int l, int m, double x) {
    if (T.rifact[1] == 0.0) orc_init_tables();
    return legendre(l, m, x);
}
