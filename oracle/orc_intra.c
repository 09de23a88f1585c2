/*
 * TEST INFRASTRUCTURE ONLY (CPU oracle; parity unpinned - see orc.h).
 * Surfactant bonded terms, intramolecular nonbonded pairs, the far-field
 * correction for intramolecular pairs, the box walls and the graphite sheet.
 * Energies are not computed by the reference; the *_energy functions here
 * integrate the reference's force laws (checked by finite differences).
 */
#include "orc.h"

#include <math.h>

#define T ORC_T
#define NS ORC_NSURF_SITE

static inline void addf(orc_sys *s, int g, double fx, double fy, double fz) {
    s->fx[g] += fx; s->fy[g] += fy; s->fz[g] += fz;
}

/* src/eval_valence.f90:97-158 */
static double valence_mol(orc_sys *s, int g0, int do_force) {
    double e = 0.0;
    for (int i = 1; i <= 36; i++) {
        int ig = g0 + T.iang[i] - 1, jg = g0 + T.jang[i] - 1, kg = g0 + T.kang[i] - 1;
        double rxji = s->x[ig] - s->x[jg], ryji = s->y[ig] - s->y[jg], rzji = s->z[ig] - s->z[jg];
        double rxki = s->x[kg] - s->x[jg], ryki = s->y[kg] - s->y[jg], rzki = s->z[kg] - s->z[jg];
        double dp = rxji * rxki + ryji * ryki + rzji * rzki;
        double rjin = sqrt(rxji * rxji + ryji * ryji + rzji * rzji);
        double rkin = sqrt(rxki * rxki + ryki * ryki + rzki * rzki);
        double thjik = acos(dp / rjin / rkin);
        double costh = cos(thjik);
        e += 0.5 * T.rkth[i] * (thjik - T.th[i]) * (thjik - T.th[i]);
        if (!do_force) continue;
        double r1 = T.rkth[i] * (thjik - T.th[i]) / sin(thjik);
        double fjx = rxki / rjin / rkin - costh * rxji / (rjin * rjin);
        double fjy = ryki / rjin / rkin - costh * ryji / (rjin * rjin);
        double fjz = rzki / rjin / rkin - costh * rzji / (rjin * rjin);
        double fkx = rxji / rjin / rkin - costh * rxki / (rkin * rkin);
        double fky = ryji / rjin / rkin - costh * ryki / (rkin * rkin);
        double fkz = rzji / rjin / rkin - costh * rzki / (rkin * rkin);
        addf(s, ig, r1 * fjx, r1 * fjy, r1 * fjz);
        addf(s, jg, -r1 * (fjx + fkx), -r1 * (fjy + fky), -r1 * (fjz + fkz));
        addf(s, kg, r1 * fkx, r1 * fky, r1 * fkz);
    }
    return e;
}

void orc_eval_valence(orc_sys *s) {
    for (int q = 0; q < s->ns; q++) valence_mol(s, orc_first_site(s, s->nw + q), 1);
}

/* src/eval_dihedral.f90:102-294 (dihedrals 1-18, triple cosine) and
 * src/eval_dihedral_berendsen.f90 (dihedrals 19-30, cos 3 phi) */
static double dihedral_mol(orc_sys *s, int g0, int berendsen, int do_force) {
    double e = 0.0;
    int i0 = berendsen ? 19 : 1, i1 = berendsen ? 30 : 18;
    double clampv = berendsen ? 0.999999 : 0.99999999999;
    for (int i = i0; i <= i1; i++) {
        int iv = g0 + T.idv[i] - 1, jv = g0 + T.jdv[i] - 1, kv = g0 + T.kdv[i] - 1, lv = g0 + T.ldv[i] - 1;
        double rxji = s->x[jv] - s->x[iv], ryji = s->y[jv] - s->y[iv], rzji = s->z[jv] - s->z[iv];
        double rxkj = s->x[kv] - s->x[jv], rykj = s->y[kv] - s->y[jv], rzkj = s->z[kv] - s->z[jv];
        double rxnk = s->x[lv] - s->x[kv], rynk = s->y[lv] - s->y[kv], rznk = s->z[lv] - s->z[kv];
        double cpjikjx = rxji * rykj - ryji * rxkj;
        double cpjikjy = rxji * rzkj - rzji * rxkj;
        double cpjikjz = ryji * rzkj - rzji * rykj;
        double cpkjnkx = rxkj * rynk - rykj * rxnk;
        double cpkjnky = rxkj * rznk - rzkj * rxnk;
        double cpkjnkz = rykj * rznk - rzkj * rynk;
        double cpjikjn = sqrt(cpjikjx * cpjikjx + cpjikjy * cpjikjy + cpjikjz * cpjikjz);
        double cpkjnkn = sqrt(cpkjnkx * cpkjnkx + cpkjnky * cpkjnky + cpkjnkz * cpkjnkz);
        double dp = cpjikjx * cpkjnkx + cpjikjy * cpkjnky + cpjikjz * cpkjnkz;
        double arg = dp / cpjikjn / cpkjnkn;
        if (arg <= -1.0) arg = -clampv;
        if (arg >= 1.0) arg = clampv;
        double th = acos(arg);
        double costh = cos(th), sinth = sin(th);
        double r1;
        if (berendsen) {
            r1 = -3.0 * T.dva[i] * sin(3.0 * th) / sinth;
            e += T.dva[i] * (1.0 + cos(3.0 * th));
        } else {
            r1 = -T.dva[i] + 2.0 * T.dvb[i] * sin(2.0 * th) / sinth - 3.0 * T.dvc[i] * sin(3.0 * th) / sinth;
            e += T.dva[i] * (1.0 + cos(th)) + T.dvb[i] * (1.0 - cos(2.0 * th)) + T.dvc[i] * (1.0 + cos(3.0 * th));
        }
        if (!do_force) continue;
        double n12 = cpjikjn * cpjikjn, n22 = cpkjnkn * cpkjnkn;
        /* particle i */
        double fix = rxkj * (-rykj * rynk - rzkj * rznk) + rxnk * (rykj * rykj + rzkj * rzkj);
        double fiy = rykj * (-rxkj * rxnk - rzkj * rznk) + rynk * (rxkj * rxkj + rzkj * rzkj);
        double fiz = rzkj * (-rxkj * rxnk - rykj * rynk) + rznk * (rxkj * rxkj + rykj * rykj);
        fix = fix / cpjikjn / cpkjnkn; fiy = fiy / cpjikjn / cpkjnkn; fiz = fiz / cpjikjn / cpkjnkn;
        double fix2 = 2.0 * rxji * (-rykj * rykj - rzkj * rzkj) + 2.0 * rxkj * (ryji * rykj + rzji * rzkj);
        double fiy2 = 2.0 * ryji * (-rxkj * rxkj - rzkj * rzkj) + 2.0 * rykj * (rxji * rxkj + rzji * rzkj);
        double fiz2 = 2.0 * rzji * (-rxkj * rxkj - rykj * rykj) + 2.0 * rzkj * (rxji * rxkj + ryji * rykj);
        fix2 /= n12; fiy2 /= n12; fiz2 /= n12;
        double fxi = r1 * (fix - 0.5 * costh * fix2), fyi = r1 * (fiy - 0.5 * costh * fiy2), fzi = r1 * (fiz - 0.5 * costh * fiz2);
        /* particle j */
        double fjx = rxji * (-rykj * rynk - rzkj * rznk) + rxkj * (rykj * rynk + rzkj * rznk);
        double fjy = ryji * (-rxkj * rxnk - rzkj * rznk) + rykj * (rxkj * rxnk + rzkj * rznk);
        double fjz = rzji * (-rxkj * rxnk - rykj * rynk) + rzkj * (rxkj * rxnk + rykj * rynk);
        double fjx1 = rxnk * (-ryji * rykj - rzji * rzkj - rykj * rykj - rzkj * rzkj);
        double fjy1 = rynk * (-rxji * rxkj - rzji * rzkj - rxkj * rxkj - rzkj * rzkj);
        double fjz1 = rznk * (-rxji * rxkj - ryji * rykj - rxkj * rxkj - rykj * rykj);
        double fjx2 = 2.0 * rxkj * (ryji * rynk + rzji * rznk);
        double fjy2 = 2.0 * rykj * (rxji * rxnk + rzji * rznk);
        double fjz2 = 2.0 * rzkj * (rxji * rxnk + ryji * rynk);
        fjx = (fjx + fjx1 + fjx2) / cpjikjn / cpkjnkn;
        fjy = (fjy + fjy1 + fjy2) / cpjikjn / cpkjnkn;
        fjz = (fjz + fjz1 + fjz2) / cpjikjn / cpkjnkn;
        double fjx3 = 2.0 * rxji * (rykj * rykj + rzkj * rzkj + ryji * rykj + rzji * rzkj);
        double fjy3 = 2.0 * ryji * (rxkj * rxkj + rzkj * rzkj + rxji * rxkj + rzji * rzkj);
        double fjz3 = 2.0 * rzji * (rxkj * rxkj + rykj * rykj + rxji * rxkj + ryji * rykj);
        double fjx4 = 2.0 * rxkj * (-ryji * ryji - rzji * rzji - ryji * rykj - rzji * rzkj);
        double fjy4 = 2.0 * rykj * (-rxji * rxji - rzji * rzji - rxji * rxkj - rzji * rzkj);
        double fjz4 = 2.0 * rzkj * (-rxji * rxji - ryji * ryji - rxji * rxkj - ryji * rykj);
        fjx3 = (fjx3 + fjx4) / n12; fjy3 = (fjy3 + fjy4) / n12; fjz3 = (fjz3 + fjz4) / n12;
        double fjx5 = 2.0 * rxnk * (rykj * rynk + rzkj * rznk) + 2.0 * rxkj * (-rynk * rynk - rznk * rznk);
        double fjy5 = 2.0 * rynk * (rxkj * rxnk + rzkj * rznk) + 2.0 * rykj * (-rxnk * rxnk - rznk * rznk);
        double fjz5 = 2.0 * rznk * (rxkj * rxnk + rykj * rynk) + 2.0 * rzkj * (-rxnk * rxnk - rynk * rynk);
        fjx5 /= n22; fjy5 /= n22; fjz5 /= n22;
        double fxj = r1 * (fjx - 0.5 * costh * (fjx3 + fjx5));
        double fyj = r1 * (fjy - 0.5 * costh * (fjy3 + fjy5));
        double fzj = r1 * (fjz - 0.5 * costh * (fjz3 + fjz5));
        /* particle k */
        double fkx = rxji * (rykj * rykj + rzkj * rzkj + rykj * rynk + rzkj * rznk);
        double fky = ryji * (rxkj * rxkj + rzkj * rzkj + rxkj * rxnk + rzkj * rznk);
        double fkz = rzji * (rxkj * rxkj + rykj * rykj + rxkj * rxnk + rykj * rynk);
        double fkx2 = rxkj * (-ryji * rykj - rzji * rzkj);
        double fky2 = rykj * (-rxji * rxkj - rzji * rzkj);
        double fkz2 = rzkj * (-rxji * rxkj - ryji * rykj);
        double fkx3 = rxnk * (ryji * rykj + rzji * rzkj) + 2.0 * rxkj * (-ryji * rynk - rzji * rznk);
        double fky3 = rynk * (rxji * rxkj + rzji * rzkj) + 2.0 * rykj * (-rxji * rxnk - rzji * rznk);
        double fkz3 = rznk * (rxji * rxkj + ryji * rykj) + 2.0 * rzkj * (-rxji * rxnk - ryji * rynk);
        fkx = (fkx + fkx2 + fkx3) / cpjikjn / cpkjnkn;
        fky = (fky + fky2 + fky3) / cpjikjn / cpkjnkn;
        fkz = (fkz + fkz2 + fkz3) / cpjikjn / cpkjnkn;
        double fkx4 = 2.0 * rxji * (-ryji * rykj - rzji * rzkj) + 2.0 * rxkj * (ryji * ryji + rzji * rzji);
        double fky4 = 2.0 * ryji * (-rxji * rxkj - rzji * rzkj) + 2.0 * rykj * (rxji * rxji + rzji * rzji);
        double fkz4 = 2.0 * rzji * (-rxji * rxkj - ryji * rykj) + 2.0 * rzkj * (rxji * rxji + ryji * ryji);
        fkx4 /= n12; fky4 /= n12; fkz4 /= n12;
        double fkx5 = 2.0 * rxnk * (-rykj * rykj - rzkj * rzkj - rykj * rynk - rzkj * rznk);
        double fky5 = 2.0 * rynk * (-rxkj * rxkj - rzkj * rzkj - rxkj * rxnk - rzkj * rznk);
        double fkz5 = 2.0 * rznk * (-rxkj * rxkj - rykj * rykj - rxkj * rxnk - rykj * rynk);
        double fkx6 = 2.0 * rxkj * (rynk * rynk + rznk * rznk + rykj * rynk + rzkj * rznk);
        double fky6 = 2.0 * rykj * (rxnk * rxnk + rznk * rznk + rxkj * rxnk + rzkj * rznk);
        double fkz6 = 2.0 * rzkj * (rxnk * rxnk + rynk * rynk + rxkj * rxnk + rykj * rynk);
        fkx5 = (fkx5 + fkx6) / n22; fky5 = (fky5 + fky6) / n22; fkz5 = (fkz5 + fkz6) / n22;
        double fxk = r1 * (fkx - 0.5 * costh * (fkx4 + fkx5));
        double fyk = r1 * (fky - 0.5 * costh * (fky4 + fky5));
        double fzk = r1 * (fkz - 0.5 * costh * (fkz4 + fkz5));
        /* particle n */
        double fnx = rxji * (-rykj * rykj - rzkj * rzkj) + rxkj * (ryji * rykj + rzji * rzkj);
        double fny = ryji * (-rxkj * rxkj - rzkj * rzkj) + rykj * (rxji * rxkj + rzji * rzkj);
        double fnz = rzji * (-rxkj * rxkj - rykj * rykj) + rzkj * (rxji * rxkj + ryji * rykj);
        fnx = fnx / cpjikjn / cpkjnkn; fny = fny / cpjikjn / cpkjnkn; fnz = fnz / cpjikjn / cpkjnkn;
        double fnx2 = 2.0 * rxnk * (rykj * rykj + rzkj * rzkj) + 2.0 * rxkj * (-rykj * rynk - rzkj * rznk);
        double fny2 = 2.0 * rynk * (rxkj * rxkj + rzkj * rzkj) + 2.0 * rykj * (-rxkj * rxnk - rzkj * rznk);
        double fnz2 = 2.0 * rznk * (rxkj * rxkj + rykj * rykj) + 2.0 * rzkj * (-rxkj * rxnk - rykj * rynk);
        fnx2 /= n22; fny2 /= n22; fnz2 /= n22;
        double fxn = r1 * (fnx - 0.5 * costh * fnx2), fyn = r1 * (fny - 0.5 * costh * fny2), fzn = r1 * (fnz - 0.5 * costh * fnz2);
        addf(s, iv, fxi, fyi, fzi);
        addf(s, jv, fxj, fyj, fzj);
        addf(s, kv, fxk, fyk, fzk);
        addf(s, lv, fxn, fyn, fzn);
    }
    return e;
}

void orc_eval_dihedral(orc_sys *s, int berendsen) {
    for (int q = 0; q < s->ns; q++) dihedral_mol(s, orc_first_site(s, s->nw + q), berendsen, 1);
}

static inline double intra_pair(orc_sys *s, int gj, int gk, int jt, int kt, int do_force) {
    double x = s->x[gj] - s->x[gk], y = s->y[gj] - s->y[gk], z = s->z[gj] - s->z[gk];
    double rsq = x * x + y * y + z * z;
    double rctr = sqrt(rsq);
    double qq = T.rqs[jt] * T.rqs[kt] * ORC_XPI;
    double rsi = 1.0 / rsq, r6 = rsi * rsi * rsi;
    double eps = T.epss[jt][kt], sg6 = T.sgss6[jt][kt];
    if (do_force) {
        double fel = qq / (rctr * rctr * rctr);
        double rpl = 48.0 * eps * sg6 * r6 * (sg6 * r6 - 0.5);
        double ft = fel + rpl * rsi;
        addf(s, gj, x * ft, y * ft, z * ft);
        addf(s, gk, -x * ft, -y * ft, -z * ft);
    }
    return qq / rctr + 4.0 * eps * (sg6 * sg6 * r6 * r6 - sg6 * r6);
}

/* src/eval_surfactant_internal.f90:17-110: sites j = 1..15 with k >= j+4,
 * then the 42 listed pairs; LJ without cutoff */
static double internal_mol(orc_sys *s, int g0, int do_force) {
    double e = 0.0;
    for (int j = 1; j <= 15; j++)
        for (int k = j + 4; k <= 29; k++) e += intra_pair(s, g0 + j - 1, g0 + k - 1, j, k, do_force);
    for (int k = 1; k <= 42; k++) {
        int m = T.iself[k], n = T.jself[k];
        e += intra_pair(s, g0 + m - 1, g0 + n - 1, m, n, do_force);
    }
    return e;
}

void orc_eval_surfactant_internal(orc_sys *s) {
    for (int q = 0; q < s->ns; q++) internal_mol(s, orc_first_site(s, s->nw + q), 1);
}

/* src/eval_subtract_fma.f90:10-55 */
static double subtract_mol(orc_sys *s, int q, int do_force) {
    double e = 0.0;
    int g0 = orc_first_site(s, s->nw + q);
    for (int j = 1; j <= NS; j++) {
        const int *lst = &s->isub[((size_t)q * NS + (j - 1)) * 28];
        int m = g0 + j - 1;
        for (int c = 0; c < 28 && lst[c] != 0; c++) {
            int k = lst[c];
            int n = g0 + k - 1;
            double xmn = s->x[m] - s->x[n], ymn = s->y[m] - s->y[n], zmn = s->z[m] - s->z[n];
            double rmn = sqrt(xmn * xmn + ymn * ymn + zmn * zmn);
            double qq = T.rqs[j] * T.rqs[k] * ORC_XPI;
            if (do_force) {
                double fel = qq / (rmn * rmn * rmn);
                addf(s, m, -xmn * fel, -ymn * fel, -zmn * fel);
            }
            e -= 0.5 * qq / rmn;
        }
    }
    return e;
}

void orc_eval_subtract_fma(orc_sys *s) {
    for (int q = 0; q < s->ns; q++) subtract_mol(s, q, 1);
}

/* src/eval_wall.f90:1-59: 48/d^13 from the six faces on every mobile site */
static inline double p13(double v) { double v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4 * v; }
static inline double p12(double v) { double v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4; }
void orc_eval_wall(orc_sys *s) {
    for (int g = 0; g < s->nsite; g++) {
        s->fx[g] += 48.0 / p13(s->x[g] - s->rhsx); s->fx[g] += 48.0 / p13(s->rhsx + s->x[g]);
        s->fy[g] += 48.0 / p13(s->y[g] - s->rhsy); s->fy[g] += 48.0 / p13(s->rhsy + s->y[g]);
        s->fz[g] += 48.0 / p13(s->z[g] - s->rhsz); s->fz[g] += 48.0 / p13(s->rhsz + s->z[g]);
    }
}
static double wall_energy(const orc_sys *s) {
    double e = 0.0;
    for (int g = 0; g < s->nsite; g++)
        e += 4.0 / p12(s->x[g] - s->rhsx) + 4.0 / p12(s->rhsx + s->x[g]) + 4.0 / p12(s->y[g] - s->rhsy) +
             4.0 / p12(s->rhsy + s->y[g]) + 4.0 / p12(s->z[g] - s->rhsz) + 4.0 / p12(s->rhsz + s->z[g]);
    return e;
}

/* src/eval_graphite.f90:13-132: LJ against the fixed carbons within rc, for
 * water O (w1 and split) and for surfactant sites Central in their own key
 * cell, only in the bottom layer of cells.  Carbons are taken per cell column
 * as src/read_graphite.f90:9-35 pre-filters them. */
static double graphite_site(orc_sys *s, int g, double eps, double sg6, double cx, double cy, int do_force) {
    double e = 0.0;
    double rcut = (ORC_RC + sqrt(2.0) * ORC_RS / 2.0);
    rcut = rcut * rcut;
    for (int j = 0; j < s->nc; j++) {
        double dxc = s->gx[j] - cx, dyc = s->gy[j] - cy;
        if (dxc * dxc + dyc * dyc > rcut) continue;
        double xij = s->x[g] - s->gx[j], yij = s->y[g] - s->gy[j], zij = s->z[g] - s->gz[j];
        double rijsq = xij * xij + yij * yij + zij * zij;
        double rij = sqrt(rijsq);
        if (rij <= ORC_RC) {
            double rsi = 1.0 / rijsq, r6 = rsi * rsi * rsi;
            double rpl = 48.0 * eps * sg6 * r6 * (sg6 * r6 - 0.5);
            double flj = rpl * rsi;
            if (do_force) addf(s, g, xij * flj, yij * flj, zij * flj);
            e += 4.0 * eps * (sg6 * sg6 * r6 * r6 - sg6 * r6);
        }
    }
    return e;
}

static double graphite_all(orc_sys *s, int do_force) {
    if (!s->graphite_on) return 0.0;
    double e = 0.0;
    double sgcw6 = pow(3.19 / ORC_SIGMA, 6), epcw = 392.0 / ORC_EPSILON;
    for (int c = 0; c < s->ncell; c++) {
        int ix, iy, iz;
        orc_cell_xyz(s, c, &ix, &iy, &iz);
        if (iz != 0) continue;
        double cx, cy, cz;
        orc_rcen4(s, c, &cx, &cy, &cz);
        orc_mlist *L = &s->cw1[c];
        for (int a = 0; a < L->n; a++) e += graphite_site(s, 3 * L->m[a], epcw, sgcw6, cx, cy, do_force);
        orc_list *W = &s->W2C[c];
        for (int a = 0; a < W->n; a++)
            if (W->e[a].type == 1) e += graphite_site(s, W->e[a].gsite, epcw, sgcw6, cx, cy, do_force);
        orc_list *S = &s->SC[c];
        for (int a = 0; a < S->n; a++) {
            int ni = S->e[a].type;
            e += graphite_site(s, S->e[a].gsite, T.epcs[ni], T.sgcs6[ni], cx, cy, do_force);
        }
    }
    return e;
}

void orc_eval_graphite(orc_sys *s) { graphite_all(s, 1); }

/* energies of the terms in this file: out[0] bonded (angles + dihedrals),
 * out[1] intramolecular pairs, out[2] far-field correction, out[3] wall,
 * out[4] graphite */
void orc_intra_energies(orc_sys *s, double *out) {
    double eb = 0, ei = 0, es = 0;
    for (int q = 0; q < s->ns; q++) {
        int g0 = orc_first_site(s, s->nw + q);
        eb += valence_mol(s, g0, 0) + dihedral_mol(s, g0, 0, 0) + dihedral_mol(s, g0, 1, 0);
        ei += internal_mol(s, g0, 0);
        es += subtract_mol(s, q, 0);
    }
    out[0] = eb; out[1] = ei; out[2] = es; out[3] = wall_energy(s); out[4] = graphite_all(s, 0);
}
