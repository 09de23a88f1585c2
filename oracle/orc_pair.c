/*
 * TEST INFRASTRUCTURE ONLY (CPU oracle; parity unpinned - see orc.h).
 * The reference's 39 short-range pair kernels, one C function each, over the
 * global cell grid.  Every kernel keeps the reference's loop structure: which
 * list is the i side, which is the j side, whether the j side is updated
 * (Newton's third law inside a cell) or only the i side, the charge each side
 * is given and the condition under which the truncated LJ term is added.
 *
 * Pair term (e.g. src/evalw1w1n.f90:86-104, src/evalSS.f90:38-56):
 *   fel = qq / r^3 (no cutoff),  flj = 48 eps sg6 r^-6 (sg6 r^-6 - 1/2) / r^2 if r <= rc,
 *   f_i += d_ij (fel + flj), and f_j -= d_ij (fel + flj) for third-law pairs.
 */
#include "orc.h"

#include <math.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define T ORC_T

/* Forces and pair counts accumulate per thread (the kernels' cell loops are
 * shared among the threads of an OpenMP team, statically, so every thread
 * sees the same cells on every call) and are added in thread order after
 * the kernels: deterministic for a given thread count. */
static _Thread_local double *tl_f;        /* [3 * nsite]: x, y, z interleaved */
static _Thread_local int64_t tl_nc, tl_nl;

/* ljmode: 0 none, 1 water O-O (48 r6 (r6 - 1/2)), 2 tabulated (eps, sg6) */
static inline void pterm(orc_sys *s, int gi, int gj, double qq, int ljmode, double eps, double sg6, int n3l) {
    double xij = s->x[gi] - s->x[gj];
    double yij = s->y[gi] - s->y[gj];
    double zij = s->z[gi] - s->z[gj];
    double rijsq = xij * xij + yij * yij + zij * zij;
    double rij = sqrt(rijsq);
    double fel = qq / (rij * rij * rij);
    double flj = 0.0;
    tl_nc += n3l ? 2 : 1;
    if (ljmode && rij <= ORC_RC) {
        double rsi = 1.0 / rijsq;
        double r6 = rsi * rsi * rsi;
        double rpl = ljmode == 1 ? 48.0 * r6 * (r6 - 0.5) : 48.0 * eps * sg6 * r6 * (sg6 * r6 - 0.5);
        flj = rpl * rsi;
        tl_nl += n3l ? 2 : 1;
    }
    double ft = fel + flj;
    double *fi = tl_f + 3 * (size_t)gi;
    fi[0] += xij * ft; fi[1] += yij * ft; fi[2] += zij * ft;
    if (n3l) { double *fj = tl_f + 3 * (size_t)gj; fj[0] -= xij * ft; fj[1] -= yij * ft; fj[2] -= zij * ft; }
}

static inline double qw(int t) { return T.rqw[t]; }
static inline double qs(int t) { return T.rqs[t]; }

/* neighbour cell k of cell c by kmid index, -1 outside */
static inline int nbr(const orc_sys *s, int c, int j) {
    int ix, iy, iz;
    orc_cell_xyz(s, c, &ix, &iy, &iz);
    return orc_cell_id(s, ix + ORC_KMID[j][0], iy + ORC_KMID[j][1], iz + ORC_KMID[j][2]);
}

/* ---- water (w1) i side ---- */

/* src/evalw1w1.f90:28-245: 9 site pairs per molecule pair, third law */
static void evalw1w1(orc_sys *s) {
    double qq[4][4];
    double qOqO = T.rqw[1] * T.rqw[1] * ORC_XPI, qOqH = T.rqw[1] * T.rqw[2] * ORC_XPI, qHqH = T.rqw[2] * T.rqw[3] * ORC_XPI;
    qq[1][1] = qOqO; qq[1][2] = qq[1][3] = qq[2][1] = qq[3][1] = qOqH; qq[2][2] = qq[2][3] = qq[3][2] = qq[3][3] = qHqH;
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_mlist *L = &s->cw1[c];
        for (int a = 0; a < L->n; a++)
            for (int b = a + 1; b < L->n; b++)
                for (int ti = 1; ti <= 3; ti++)
                    for (int tj = 1; tj <= 3; tj++)
                        pterm(s, 3 * L->m[a] + ti - 1, 3 * L->m[b] + tj - 1, qq[ti][tj], (ti == 1 && tj == 1), 0, 0, 1);
    }
}

/* src/evalw1w1n.f90:29-231: i side only, 26 neighbour cells */
static void evalw1w1n(orc_sys *s) {
    double qq[4][4];
    double qOqO = T.rqw[1] * T.rqw[1] * ORC_XPI, qOqH = T.rqw[1] * T.rqw[2] * ORC_XPI, qHqH = T.rqw[2] * T.rqw[3] * ORC_XPI;
    qq[1][1] = qOqO; qq[1][2] = qq[1][3] = qq[2][1] = qq[3][1] = qOqH; qq[2][2] = qq[2][3] = qq[3][2] = qq[3][3] = qHqH;
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_mlist *L = &s->cw1[c];
        for (int a = 0; a < L->n; a++)
            for (int j = 0; j < 26; j++) {
                int k = nbr(s, c, j);
                if (k < 0) continue;
                orc_mlist *M = &s->cw1[k];
                for (int b = 0; b < M->n; b++)
                    for (int ti = 1; ti <= 3; ti++)
                        for (int tj = 1; tj <= 3; tj++)
                            pterm(s, 3 * L->m[a] + ti - 1, 3 * M->m[b] + tj - 1, qq[ti][tj], (ti == 1 && tj == 1), 0, 0, 0);
            }
    }
}

/* w1 i side against one atom list.  cmode: 0 actual water charge, 1 water H
 * charge; ljw: LJ only O(i)-O(j) water pairs; ljs: LJ O(i)-surfactant */
static void w1_vs_list(orc_sys *s, int c, orc_list *J, int jwater, int qH, int n3l) {
    orc_mlist *L = &s->cw1[c];
    for (int a = 0; a < L->n; a++)
        for (int ti = 1; ti <= 3; ti++) {
            int gi = 3 * L->m[a] + ti - 1;
            double rqq = qw(ti) * ORC_XPI;
            for (int b = 0; b < J->n; b++) {
                orc_ent *e = &J->e[b];
                if (jwater) {
                    double qj = qH ? qw(2) : qw(e->type);
                    int lj = (!qH && ti == 1 && e->type == 1) ? 1 : 0;
                    pterm(s, gi, e->gsite, rqq * qj, lj, 0, 0, n3l);
                } else {
                    int lj = ti == 1 ? 2 : 0;
                    pterm(s, gi, e->gsite, rqq * qs(e->type), lj, T.epws[1][e->type], T.sgws6[1][e->type], n3l);
                }
            }
        }
}

/* src/evalw1w2.f90:13-86 */
static void evalw1w2(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        /* per i atom: W2Central (third law) then W226 (i side, H charge) */
        orc_mlist *L = &s->cw1[c];
        for (int a = 0; a < L->n; a++)
            for (int ti = 1; ti <= 3; ti++) {
                int gi = 3 * L->m[a] + ti - 1;
                double rqq = qw(ti) * ORC_XPI;
                orc_list *J = &s->W2C[c];
                for (int b = 0; b < J->n; b++)
                    pterm(s, gi, J->e[b].gsite, rqq * qw(J->e[b].type), ti == 1 && J->e[b].type == 1, 0, 0, 1);
                J = &s->W226[c];
                for (int b = 0; b < J->n; b++) pterm(s, gi, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 0);
            }
    }
}

/* src/evalw1w2n.f90:13-87 */
static void evalw1w2n(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_mlist *L = &s->cw1[c];
        for (int a = 0; a < L->n; a++)
            for (int ti = 1; ti <= 3; ti++) {
                int gi = 3 * L->m[a] + ti - 1;
                double rqq = qw(ti) * ORC_XPI;
                orc_list *J = &s->W2nC[c];
                for (int b = 0; b < J->n; b++) pterm(s, gi, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 1);
                J = &s->W2n26[c];
                for (int b = 0; b < J->n; b++)
                    pterm(s, gi, J->e[b].gsite, rqq * qw(J->e[b].type), ti == 1 && J->e[b].type == 1, 0, 0, 0);
            }
    }
}

/* src/evalw1w2nn.f90:12-49 */
static void evalw1w2nn(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) w1_vs_list(s, c, &s->W2nn[c], 1, 1, 0);
}

/* src/evalw1s.f90:13-98, src/evalw1sn.f90, src/evalw1snn.f90: Central lists
 * with third law, 26 lists i side; src/evalw1snnn.f90 i side only */
static void evalw1s_family(orc_sys *s, orc_list *C, orc_list *N26) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_mlist *L = &s->cw1[c];
        for (int a = 0; a < L->n; a++)
            for (int ti = 1; ti <= 3; ti++) {
                int gi = 3 * L->m[a] + ti - 1;
                double rqq = qw(ti) * ORC_XPI;
                if (C) {
                    orc_list *J = &C[c];
                    for (int b = 0; b < J->n; b++) {
                        int n = J->e[b].type;
                        pterm(s, gi, J->e[b].gsite, rqq * qs(n), ti == 1 ? 2 : 0, T.epws[1][n], T.sgws6[1][n], 1);
                    }
                }
                orc_list *J = &N26[c];
                for (int b = 0; b < J->n; b++) {
                    int n = J->e[b].type;
                    pterm(s, gi, J->e[b].gsite, rqq * qs(n), ti == 1 ? 2 : 0, T.epws[1][n], T.sgws6[1][n], 0);
                }
            }
    }
}
static void evalw1s(orc_sys *s) { evalw1s_family(s, s->SC, s->S26); }
static void evalw1sn(orc_sys *s) { evalw1s_family(s, s->SnC, s->Sn26); }
static void evalw1snn(orc_sys *s) { evalw1s_family(s, s->SnnC, s->Snn26); }
static void evalw1snnn(orc_sys *s) { evalw1s_family(s, NULL, s->Snnn); }

/* ---- atom-list i side against the w1 molecules of the 26 neighbours ----
 * src/evalw2w1n.f90:15-112 (LJ if i is water O), src/evalw2nw1n.f90 (no LJ),
 * src/evalSw1n.f90, src/evalSnw1n.f90, src/evalSnnw1n.f90 (LJ with the O) */
static void list_vs_w1n(orc_sys *s, orc_list *IL, int iwater, int qHi) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &IL[c];
        for (int a = 0; a < L->n; a++) {
            orc_ent *ei = &L->e[a];
            int ni = ei->type;
            double rqq = (iwater ? (qHi ? qw(2) : qw(ni)) : qs(ni)) * ORC_XPI;
            for (int j = 0; j < 26; j++) {
                int k = nbr(s, c, j);
                if (k < 0) continue;
                orc_mlist *M = &s->cw1[k];
                for (int b = 0; b < M->n; b++)
                    for (int tj = 1; tj <= 3; tj++) {
                        int lj = 0;
                        double eps = 0, sg6 = 0;
                        if (tj == 1) {
                            if (iwater) lj = (!qHi && ni == 1) ? 1 : 0;
                            else { lj = 2; eps = T.epws[1][ni]; sg6 = T.sgws6[1][ni]; }
                        }
                        pterm(s, ei->gsite, 3 * M->m[b] + tj - 1, rqq * qw(tj), lj, eps, sg6, 0);
                    }
            }
        }
    }
}

/* exclusion of same-molecule pairs (mli/mlj, mni/mnj in the reference) */
static inline int same_mol(const orc_ent *a, const orc_ent *b) { return a->mol == b->mol; }

/* ---- split water (w2) i side ---- */

/* src/evalw2w2.f90:14-112 */
static void evalw2w2(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2C[c];
        for (int a = 0; a + 1 < L->n; a++) {
            orc_ent *ei = &L->e[a];
            double rqq = qw(ei->type) * ORC_XPI;
            for (int b = a + 1; b < L->n; b++) {
                orc_ent *ej = &L->e[b];
                if (same_mol(ei, ej)) continue;
                pterm(s, ei->gsite, ej->gsite, rqq * qw(ej->type), ei->type == 1 && ej->type == 1, 0, 0, 1);
            }
        }
        for (int a = 0; a < L->n; a++) {
            orc_ent *ei = &L->e[a];
            double rqq = qw(ei->type) * ORC_XPI;
            orc_list *J = &s->W226[c];
            for (int b = 0; b < J->n; b++) {
                if (same_mol(ei, &J->e[b])) continue;
                pterm(s, ei->gsite, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 0);
            }
        }
    }
}

/* src/evalw2w2n.f90: W2Central x W2nCentral (third law, H charge), W2Central
 * x W2n26 (LJ O-O), W2nCentral x W226 */
static void evalw2w2n(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2C[c];
        for (int a = 0; a < L->n; a++) {
            orc_ent *ei = &L->e[a];
            double rqq = qw(ei->type) * ORC_XPI;
            orc_list *J = &s->W2nC[c];
            for (int b = 0; b < J->n; b++) pterm(s, ei->gsite, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 1);
            J = &s->W2n26[c];
            for (int b = 0; b < J->n; b++)
                pterm(s, ei->gsite, J->e[b].gsite, rqq * qw(J->e[b].type), ei->type == 1 && J->e[b].type == 1, 0, 0, 0);
        }
        L = &s->W2nC[c];
        for (int a = 0; a < L->n; a++) {
            orc_ent *ei = &L->e[a];
            double rqq = qw(2) * ORC_XPI;
            orc_list *J = &s->W226[c];
            for (int b = 0; b < J->n; b++) pterm(s, ei->gsite, J->e[b].gsite, rqq * qw(J->e[b].type), 0, 0, 0, 0);
        }
    }
}

/* src/evalw2w2nn.f90 */
static void evalw2w2nn(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2C[c];
        for (int a = 0; a < L->n; a++) {
            orc_ent *ei = &L->e[a];
            double rqq = qw(ei->type) * ORC_XPI;
            orc_list *J = &s->W2nn[c];
            for (int b = 0; b < J->n; b++) pterm(s, ei->gsite, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 0);
        }
    }
}

/* src/evalw2s.f90, src/evalw2sn.f90, src/evalw2snn.f90: W2Central x
 * (Central third law, 26 i side) with LJ for water O; surfactant Central x
 * W226 (H charge).  src/evalw2snnn.f90: W2Central x Snnn only. */
static void evalw2s_family(orc_sys *s, orc_list *C, orc_list *N26, orc_list *SI) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2C[c];
        for (int a = 0; a < L->n; a++) {
            orc_ent *ei = &L->e[a];
            double rqq = qw(ei->type) * ORC_XPI;
            if (C) {
                orc_list *J = &C[c];
                for (int b = 0; b < J->n; b++) {
                    int n = J->e[b].type;
                    pterm(s, ei->gsite, J->e[b].gsite, rqq * qs(n), ei->type == 1 ? 2 : 0, T.epws[1][n], T.sgws6[1][n], 1);
                }
            }
            orc_list *J = &N26[c];
            for (int b = 0; b < J->n; b++) {
                int n = J->e[b].type;
                pterm(s, ei->gsite, J->e[b].gsite, rqq * qs(n), ei->type == 1 ? 2 : 0, T.epws[1][n], T.sgws6[1][n], 0);
            }
        }
        if (SI) {
            orc_list *L2 = &SI[c];
            for (int a = 0; a < L2->n; a++) {
                orc_ent *ei = &L2->e[a];
                double rqq = qs(ei->type) * ORC_XPI;
                orc_list *J = &s->W226[c];
                for (int b = 0; b < J->n; b++) pterm(s, ei->gsite, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 0);
            }
        }
    }
}
static void evalw2s(orc_sys *s) { evalw2s_family(s, s->SC, s->S26, s->SC); }
static void evalw2sn(orc_sys *s) { evalw2s_family(s, s->SnC, s->Sn26, s->SnC); }
static void evalw2snn(orc_sys *s) { evalw2s_family(s, s->SnnC, s->Snn26, s->SnnC); }
static void evalw2snnn(orc_sys *s) { evalw2s_family(s, NULL, s->Snnn, NULL); }

/* src/evalw2nw2n.f90: W2nCentral pairs (third law) and x W2n26 */
static void evalw2nw2n(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2nC[c];
        double rqq = qw(2) * ORC_XPI;
        for (int a = 0; a + 1 < L->n; a++)
            for (int b = a + 1; b < L->n; b++) {
                if (same_mol(&L->e[a], &L->e[b])) continue;
                pterm(s, L->e[a].gsite, L->e[b].gsite, rqq * qw(2), 0, 0, 0, 1);
            }
        for (int a = 0; a < L->n; a++) {
            orc_list *J = &s->W2n26[c];
            for (int b = 0; b < J->n; b++) {
                if (same_mol(&L->e[a], &J->e[b])) continue;
                pterm(s, L->e[a].gsite, J->e[b].gsite, rqq * qw(J->e[b].type), 0, 0, 0, 0);
            }
        }
    }
}

/* src/evalw2nw2nn.f90 */
static void evalw2nw2nn(orc_sys *s) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2nC[c];
        double rqq = qw(2) * ORC_XPI;
        for (int a = 0; a < L->n; a++) {
            orc_list *J = &s->W2nn[c];
            for (int b = 0; b < J->n; b++) pterm(s, L->e[a].gsite, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 0);
        }
    }
}

/* src/evalw2nS.f90, src/evalw2nSn.f90, src/evalw2nSnn.f90: W2nCentral x
 * (Central third law, 26 i side), Coulomb only; surfactant Central x W2n26
 * with LJ against the water O.  src/evalw2nSnnn.f90: W2nCentral x Snnn. */
static void evalw2nS_family(orc_sys *s, orc_list *C, orc_list *N26, orc_list *SI) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &s->W2nC[c];
        double rqq = qw(2) * ORC_XPI;
        for (int a = 0; a < L->n; a++) {
            if (C) {
                orc_list *J = &C[c];
                for (int b = 0; b < J->n; b++) pterm(s, L->e[a].gsite, J->e[b].gsite, rqq * qs(J->e[b].type), 0, 0, 0, 1);
            }
            orc_list *J = &N26[c];
            for (int b = 0; b < J->n; b++) pterm(s, L->e[a].gsite, J->e[b].gsite, rqq * qs(J->e[b].type), 0, 0, 0, 0);
        }
        if (SI) {
            orc_list *L2 = &SI[c];
            for (int a = 0; a < L2->n; a++) {
                int ni = L2->e[a].type;
                double rq2 = qs(ni) * ORC_XPI;
                orc_list *J = &s->W2n26[c];
                for (int b = 0; b < J->n; b++) {
                    int nj = J->e[b].type;
                    pterm(s, L2->e[a].gsite, J->e[b].gsite, rq2 * qw(nj), nj == 1 ? 2 : 0, T.epws[1][ni], T.sgws6[1][ni], 0);
                }
            }
        }
    }
}
static void evalw2nS(orc_sys *s) { evalw2nS_family(s, s->SC, s->S26, s->SC); }
static void evalw2nSn(orc_sys *s) { evalw2nS_family(s, s->SnC, s->Sn26, s->SnC); }
static void evalw2nSnn(orc_sys *s) { evalw2nS_family(s, s->SnnC, s->Snn26, s->SnnC); }
static void evalw2nSnnn(orc_sys *s) { evalw2nS_family(s, NULL, s->Snnn, NULL); }

/* ---- surfactant i side ---- */

/* surfactant list x W2nn (Coulomb, H charge): src/evalSw2nn.f90,
 * src/evalSnw2nn.f90, src/evalSnnw2nn.f90 */
static void s_vs_w2nn(orc_sys *s, orc_list *IL) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &IL[c];
        for (int a = 0; a < L->n; a++) {
            double rqq = qs(L->e[a].type) * ORC_XPI;
            orc_list *J = &s->W2nn[c];
            for (int b = 0; b < J->n; b++) pterm(s, L->e[a].gsite, J->e[b].gsite, rqq * qw(2), 0, 0, 0, 0);
        }
    }
}

static inline void ss_term(orc_sys *s, orc_ent *ei, orc_ent *ej, int n3l) {
    int ni = ei->type, nj = ej->type;
    pterm(s, ei->gsite, ej->gsite, qs(ni) * ORC_XPI * qs(nj), 2, T.epss[ni][nj], T.sgss6[ni][nj], n3l);
}

/* same-cell pairs of one Central list with third law, then the list against
 * its 26 partner list, both excluding same-molecule pairs:
 * src/evalSS.f90:13-124, src/evalSnSn.f90, src/evalSnnSnn.f90 */
static void ss_same(orc_sys *s, orc_list *C, orc_list *N26) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &C[c];
        for (int a = 0; a + 1 < L->n; a++)
            for (int b = a + 1; b < L->n; b++)
                if (!same_mol(&L->e[a], &L->e[b])) ss_term(s, &L->e[a], &L->e[b], 1);
        for (int a = 0; a < L->n; a++) {
            orc_list *J = &N26[c];
            for (int b = 0; b < J->n; b++)
                if (!same_mol(&L->e[a], &J->e[b])) ss_term(s, &L->e[a], &J->e[b], 0);
        }
    }
}

/* Central list A against Central list B (third law) and B's 26 list, then
 * B's Central list against A's 26 list: src/evalSSn.f90:13-148,
 * src/evalSSnn.f90, src/evalSnSnn.f90 */
static void ss_cross(orc_sys *s, orc_list *AC, orc_list *BC, orc_list *B26, orc_list *A26) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &AC[c];
        for (int a = 0; a < L->n; a++) {
            orc_list *J = &BC[c];
            for (int b = 0; b < J->n; b++) ss_term(s, &L->e[a], &J->e[b], 1);
            J = &B26[c];
            for (int b = 0; b < J->n; b++) ss_term(s, &L->e[a], &J->e[b], 0);
        }
        L = &BC[c];
        for (int a = 0; a < L->n; a++) {
            orc_list *J = &A26[c];
            for (int b = 0; b < J->n; b++) ss_term(s, &L->e[a], &J->e[b], 0);
        }
    }
}

/* Central list against Snnn, i side: src/evalSSnnn.f90, src/evalSnSnnn.f90,
 * src/evalSnnSnnn.f90 */
static void ss_nnn(orc_sys *s, orc_list *AC) {
    #pragma omp for schedule(static, 1)
    for (int c = 0; c < s->ncell; c++) {
        orc_list *L = &AC[c];
        for (int a = 0; a < L->n; a++) {
            orc_list *J = &s->Snnn[c];
            for (int b = 0; b < J->n; b++) ss_term(s, &L->e[a], &J->e[b], 0);
        }
    }
}

static void evalSS(orc_sys *s) { ss_same(s, s->SC, s->S26); }
static void evalSSn(orc_sys *s) { ss_cross(s, s->SC, s->SnC, s->Sn26, s->S26); }
static void evalSSnn(orc_sys *s) { ss_cross(s, s->SC, s->SnnC, s->Snn26, s->S26); }
static void evalSSnnn(orc_sys *s) { ss_nnn(s, s->SC); }
static void evalSnSn(orc_sys *s) { ss_same(s, s->SnC, s->Sn26); }
static void evalSnSnn(orc_sys *s) { ss_cross(s, s->SnC, s->SnnC, s->Snn26, s->Sn26); }
static void evalSnSnnn(orc_sys *s) { ss_nnn(s, s->SnC); }
static void evalSnnSnn(orc_sys *s) { ss_same(s, s->SnnC, s->Snn26); }
static void evalSnnSnnn(orc_sys *s) { ss_nnn(s, s->SnnC); }
static void evalw2w1n(orc_sys *s) { list_vs_w1n(s, s->W2C, 1, 0); }
static void evalw2nw1n(orc_sys *s) { list_vs_w1n(s, s->W2nC, 1, 1); }
static void evalSw1n(orc_sys *s) { list_vs_w1n(s, s->SC, 0, 0); }
static void evalSnw1n(orc_sys *s) { list_vs_w1n(s, s->SnC, 0, 0); }
static void evalSnnw1n(orc_sys *s) { list_vs_w1n(s, s->SnnC, 0, 0); }
static void evalSw2nn(orc_sys *s) { s_vs_w2nn(s, s->SC); }
static void evalSnw2nn(orc_sys *s) { s_vs_w2nn(s, s->SnC); }
static void evalSnnw2nn(orc_sys *s) { s_vs_w2nn(s, s->SnnC); }

/* intra-cell kernels in the order of src/up_downSR_isr.f90:324-329 */
static void intracell_kernels(orc_sys *s) {
    evalw1w1(s);
    evalw1w2(s);
    evalw1s(s);
    evalw2w2(s);
    evalw2s(s);
    evalSS(s);
}

/* neighbour kernels in the order of src/mybox.f90:185-217 */
static void neighbour_kernels(orc_sys *s) {
    evalw1w1n(s);
    evalw1w2n(s);
    evalw1w2nn(s);
    evalw1sn(s);
    evalw1snn(s);
    evalw1snnn(s);
    evalw2w1n(s);
    evalw2w2n(s);
    evalw2w2nn(s);
    evalw2sn(s);
    evalw2snn(s);
    evalw2snnn(s);
    evalw2nw1n(s);
    evalw2nw2n(s);
    evalw2nw2nn(s);
    evalw2nS(s);
    evalw2nSn(s);
    evalw2nSnn(s);
    evalw2nSnnn(s);
    evalSw1n(s);
    evalSw2nn(s);
    evalSSn(s);
    evalSSnn(s);
    evalSSnnn(s);
    evalSnw1n(s);
    evalSnw2nn(s);
    evalSnSn(s);
    evalSnSnn(s);
    evalSnSnnn(s);
    evalSnnw1n(s);
    evalSnnw2nn(s);
    evalSnnSnn(s);
    evalSnnSnnn(s);
}

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* run a group of kernels in an OpenMP team with per-thread force buffers,
 * then add the buffers to the forces in thread order */
static void run_team(orc_sys *s, void (*kernels)(orc_sys *)) {
    const int nt = orc_threads();
    const size_t n3 = 3 * (size_t)s->nsite;
    double *buf = (double *)calloc(n3 * nt + 1, sizeof(double));
    int64_t *cnt = (int64_t *)calloc(2 * (size_t)nt, sizeof(int64_t));
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        tl_f = buf + n3 * t;
        tl_nc = tl_nl = 0;
        kernels(s);
        cnt[2 * t] = tl_nc;
        cnt[2 * t + 1] = tl_nl;
#pragma omp barrier
#pragma omp for schedule(static)
        for (int g = 0; g < s->nsite; g++)
            for (int u = 0; u < nt; u++) {
                const double *f = buf + n3 * u + 3 * (size_t)g;
                s->fx[g] += f[0]; s->fy[g] += f[1]; s->fz[g] += f[2];
            }
        tl_f = NULL;
    }
    for (int u = 0; u < nt; u++) { s->npair_coul += cnt[2 * u]; s->npair_lj += cnt[2 * u + 1]; }
    free(buf);
    free(cnt);
}

void orc_eval_pairs_intracell(orc_sys *s) { run_team(s, intracell_kernels); }
void orc_eval_pairs_neighbour(orc_sys *s) { run_team(s, neighbour_kernels); }
