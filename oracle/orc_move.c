/*
 * TEST INFRASTRUCTURE ONLY (CPU oracle; parity unpinned - see orc.h).
 * Velocity-Verlet halves with SHAKE / RATTLE and the Nose-Hoover friction.
 * Waters (w1 and split) share one restatement: src/move_w1_a.f90 and
 * src/move_w2_a.f90 differ only in where the molecule is stored.
 */
#include "orc.h"

#include <math.h>

#define T ORC_T
#define NS ORC_NSURF_SITE

static const double TOL = 0.0001;   /* src/move_w1_a.f90:19-20 */
static const int MAXIT = 100;

static inline double site_mass(const orc_sys *s, int g) {
    return orc_is_water(s, g) ? T.emw[orc_site_type(s, g)] : T.ems[orc_site_type(s, g)];
}

/* sum m v^2 by species, src/nh_water1.f90:12-40, src/nh_surfactant.f90:12-199 */
static void ke_sums(const orc_sys *s, double *kw, double *ks) {
    double w = 0.0, q = 0.0;
    for (int g = 0; g < s->nsite; g++) {
        double v2 = s->vx[g] * s->vx[g] + s->vy[g] * s->vy[g] + s->vz[g] * s->vz[g];
        if (orc_is_water(s, g)) w += site_mass(s, g) * v2; else q += site_mass(s, g) * v2;
    }
    *kw = w; *ks = q;
}

/* predictor + SHAKE for one molecule, src/move_w1_a.f90:36-134 and
 * src/move_surfactant_a.f90:36-134 */
static int shake_mol(orc_sys *s, int g0, int nsite, int nb, const int *ia, const int *ja, const double *dsq,
                     const double *mass, double escale) {
    double rx[NS], ry[NS], rz[NS], px[NS], py[NS], pz[NS], vx[NS], vy[NS], vz[NS];
    for (int i = 0; i < nsite; i++) {
        int g = g0 + i;
        rx[i] = s->x[g]; ry[i] = s->y[g]; rz[i] = s->z[g];
        px[i] = s->x[g] + s->vx[g] * escale + s->ax[g];
        py[i] = s->y[g] + s->vy[g] * escale + s->ay[g];
        pz[i] = s->z[g] + s->vz[g] * escale + s->az[g];
        vx[i] = s->vx[g] * escale + s->ax[g];
        vy[i] = s->vy[g] * escale + s->ay[g];
        vz[i] = s->vz[g] * escale + s->az[g];
    }
    const double tol2 = 2.0 * TOL;
    int it = 0, ldone = 0;
    while (!ldone && it <= MAXIT) {
        ldone = 1;
        for (int b = 0; b < nb; b++) {
            int i = ia[b], j = ja[b];
            double pxab = px[i] - px[j], pyab = py[i] - py[j], pzab = pz[i] - pz[j];
            double pabsq = pxab * pxab + pyab * pyab + pzab * pzab;
            double rabsq = dsq[b];
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
    for (int i = 0; i < nsite; i++) {
        int g = g0 + i;
        s->x[g] = px[i]; s->y[g] = py[i]; s->z[g] = pz[i];
        s->vx[g] = vx[i]; s->vy[g] = vy[i]; s->vz[g] = vz[i];
    }
    return ldone ? 0 : 1;
}

/* RATTLE for one molecule, src/move_w1_b.f90:30-119, src/move_surfactant_b.f90:30-118 */
static int rattle_mol(orc_sys *s, int g0, int nsite, int nb, const int *ia, const int *ja, const double *dsq,
                      const double *mass, double escale) {
    double rx[NS], ry[NS], rz[NS], vx[NS], vy[NS], vz[NS];
    for (int i = 0; i < nsite; i++) {
        int g = g0 + i;
        rx[i] = s->x[g]; ry[i] = s->y[g]; rz[i] = s->z[g];
        s->ax[g] = s->fx[g] * ORC_DTSQ2 / mass[i];
        s->ay[g] = s->fy[g] * ORC_DTSQ2 / mass[i];
        s->az[g] = s->fz[g] * ORC_DTSQ2 / mass[i];
        vx[i] = escale * (s->vx[g] + s->ax[g]);
        vy[i] = escale * (s->vy[g] + s->ay[g]);
        vz[i] = escale * (s->vz[g] + s->az[g]);
    }
    int it = 0, ldone = 0;
    while (!ldone && it <= MAXIT) {
        ldone = 1;
        for (int b = 0; b < nb; b++) {
            int i = ia[b], j = ja[b];
            double vxab = vx[i] - vx[j], vyab = vy[i] - vy[j], vzab = vz[i] - vz[j];
            double rxab = rx[i] - rx[j], ryab = ry[i] - ry[j], rzab = rz[i] - rz[j];
            double rvab = rxab * vxab + ryab * vyab + rzab * vzab;
            rvab = rvab / ORC_DT;
            double rma = 1.0 / mass[i], rmb = 1.0 / mass[j];
            double gab = -rvab / ((rma + rmb) * dsq[b]);
            if (fabs(gab) > TOL) {
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                vx[i] = vx[i] + rma * dx * ORC_DT; vy[i] = vy[i] + rma * dy * ORC_DT; vz[i] = vz[i] + rma * dz * ORC_DT;
                vx[j] = vx[j] - rmb * dx * ORC_DT; vy[j] = vy[j] - rmb * dy * ORC_DT; vz[j] = vz[j] - rmb * dz * ORC_DT;
                ldone = 0;
            }
        }
        it++;
    }
    for (int i = 0; i < nsite; i++) {
        int g = g0 + i;
        s->vx[g] = vx[i]; s->vy[g] = vy[i]; s->vz[g] = vz[i];
    }
    return ldone ? 0 : 1;
}

static void topo(int water, int *nb, int *ia, int *ja, double *dsq, double *mass) {
    if (water) {
        *nb = 3;
        for (int i = 0; i < 3; i++) { ia[i] = i; ja[i] = (i + 1) % 3; dsq[i] = T.dsqw[i + 1]; mass[i] = T.emw[i + 1]; }
    } else {
        *nb = 28;
        for (int b = 0; b < 28; b++) { ia[b] = T.ibond[b + 1] - 1; ja[b] = T.jbond[b + 1] - 1; dsq[b] = T.dsqs[b + 1]; }
        for (int i = 0; i < NS; i++) mass[i] = T.ems[i + 1];
    }
}

/* move_surfactant_a, move_w1_a, move_w2_a (with the eta update of
 * src/move_w2_a.f90:145-157); forces are zeroed as at src/move_w1_a.f90:142-144 */
void orc_move_a(orc_sys *s) {
    double escale = 1.0 - s->eta * ORC_DT / 2.0;
    double kw1, ks1, kw2, ks2;
    ke_sums(s, &kw1, &ks1);
    int nb, ia[28], ja[28];
    double dsq[28], mass[NS];
    topo(0, &nb, ia, ja, dsq, mass);
    for (int q = 0; q < s->ns; q++) s->shake_fail += shake_mol(s, orc_first_site(s, s->nw + q), NS, nb, ia, ja, dsq, mass, escale);
    topo(1, &nb, ia, ja, dsq, mass);
    for (int m = 0; m < s->nw; m++) s->shake_fail += shake_mol(s, 3 * m, 3, nb, ia, ja, dsq, mass, escale);
    ke_sums(s, &kw2, &ks2);
    s->sv1 = ks1; s->sv2 = ks2; s->w1v1 = kw1; s->w1v2 = kw2; s->w2v1 = 0.0; s->w2v2 = 0.0;
    double sum1 = (s->sv1 + s->w1v1 + s->w2v1) / (ORC_DT * ORC_DT);
    double sum2 = (s->sv2 + s->w1v2 + s->w2v2) / (ORC_DT * ORC_DT);
    s->eta = s->eta + s->pnh1 * (sum1 + s->pnh2 + sum2);
    for (int g = 0; g < s->nsite; g++) { s->fx[g] = 0.0; s->fy[g] = 0.0; s->fz[g] = 0.0; }
}

/* move_surfactant_b, move_w1_b, move_w2_b */
void orc_move_b(orc_sys *s) {
    double escale = 2.0 / (2.0 + s->eta * ORC_DT);
    int nb, ia[28], ja[28];
    double dsq[28], mass[NS];
    topo(0, &nb, ia, ja, dsq, mass);
    for (int q = 0; q < s->ns; q++) s->rattle_fail += rattle_mol(s, orc_first_site(s, s->nw + q), NS, nb, ia, ja, dsq, mass, escale);
    topo(1, &nb, ia, ja, dsq, mass);
    for (int m = 0; m < s->nw; m++) s->rattle_fail += rattle_mol(s, 3 * m, 3, nb, ia, ja, dsq, mass, escale);
}

/* src/init_accel.f90:10-46 */
void orc_init_accel(orc_sys *s) {
    for (int g = 0; g < s->nsite; g++) {
        double m = site_mass(s, g);
        s->ax[g] = s->fx[g] * ORC_DTSQ2 / m;
        s->ay[g] = s->fy[g] * ORC_DTSQ2 / m;
        s->az[g] = s->fz[g] * ORC_DTSQ2 / m;
    }
}

/* src/compute_temperature.f90:240-242 */
double orc_temperature(const orc_sys *s) {
    double kw, ks;
    ke_sums(s, &kw, &ks);
    int np = 3 * s->nw + NS * s->ns, nc = 3 * s->nw + 28 * s->ns;
    return (kw + ks) / ORC_DTSQ / (3 * np - nc);
}
