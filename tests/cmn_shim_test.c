/*
 * C-level test of the COMMON-block layer (include/sesp_common.h), driven by
 * tests/test_common_shim.py.
 *
 * The program plays the reference driver: it allocates every domain's COMMON
 * arrays with the reference's dimensions, fills them from a state file by a
 * loop-for-loop transcription of src/read_config.f90:45-175 (with ibox2 and
 * ibox64 of src/ibox.f90:128-185), and then calls the layer.
 *
 *   cmn_shim_test 0 in.bin          layout only (host, no GPU): map, slot
 *                                   agreement with the transcription,
 *                                   scatter / gather round trips,
 *                                   re-assignment, error paths
 *   cmn_shim_test 1 in.bin out.bin  the step loop through the gfortran-named
 *                                   subroutines on the GPU; writes the first
 *                                   forces and the final state in file order
 *
 * in.bin: int32 n_water, n_surf, n_cells[3], n_carbon, nsteps, precision;
 * then float64 positions and velocities (n_sites x 3) and carbons.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sesp_common.h"

#define NW3 SESP_CMN_NW3
#define NS29 SESP_CMN_NS29

static int g_fail = 0;
#define CHECK(c, ...)                                                 \
    do {                                                              \
        if (!(c)) {                                                   \
            fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__);      \
            fprintf(stderr, __VA_ARGS__);                             \
            fprintf(stderr, "\n");                                    \
            g_fail++;                                                 \
        }                                                             \
    } while (0)

/* ---- the reference's box geometry (src/mybox.cmns, init_box_dimensions) ---- */
static double rs_, rsdx, rsdy, rsdz, rhsx, rhsy, rhsz;
static int ibdx2, ibdy2, ibdz2;

static void init_box(const int nc[3]) {
    rs_ = 10.0 / 3.166 + 2.0 / 3.166;
    ibdx2 = nc[0] / 4;
    ibdy2 = nc[1] / 4;
    ibdz2 = nc[2] / 4;
    rsdx = nc[0] * rs_;
    rsdy = nc[1] * rs_;
    rsdz = nc[2] * rs_;
    rhsx = rsdx / 2.0;
    rhsy = rsdy / 2.0;
    rhsz = rsdz / 2.0;
}

/* src/ibox.f90:128-139, 1-based */
static int ibox2(double x, double y, double z) {
    int b = 1 + (int)((x + rhsx) * ibdx2 / rsdx);
    b = b + (int)((y + rhsy) * ibdy2 / rsdy) * ibdx2;
    b = b + (int)((z + rhsz) * ibdz2 / rsdz) * ibdx2 * ibdy2;
    return b;
}

/* get_box_center (src/init_box_dimensions.f90:37-39) for 0-based rank iaq */
static void box_center(int iaq, double c[3]) {
    int ix = iaq % ibdx2, iy = iaq / ibdx2 % ibdy2, iz = iaq / (ibdx2 * ibdy2);
    c[0] = rsdx * (ix + 1) / (double)ibdx2 - rhsx - rsdx / (double)ibdx2 / 2.0;
    c[1] = rsdy * (iy + 1) / (double)ibdy2 - rhsy - rsdy / (double)ibdy2 / 2.0;
    c[2] = rsdz * (iz + 1) / (double)ibdz2 - rhsz - rsdz / (double)ibdz2 / 2.0;
}

/* src/ibox.f90:172-185, 1-based */
static int ibox64(double x, double y, double z, const double c[3]) {
    double a = x - c[0] + 2.0 * rs_, b = y - c[1] + 2.0 * rs_, d = z - c[2] + 2.0 * rs_;
    return 1 + (int)(a / rs_) + (int)(b / rs_) * 4 + (int)(d / rs_) * 4 * 4;
}

/* src/ibox.f90:1-44 */
static int ib64to(int iaq, int base, int w) {
    int k = (iaq - 1) / 16, m = (iaq - 16 * k - 1) / 4, r = iaq - 16 * k - 4 * m;
    return base + w * w * k + w * m + r;
}
#define IB216(i) ib64to(i, 43, 6)
#define IB512(i) ib64to(i, 146, 8)
#define IB1000(i) ib64to(i, 333, 10)

/* ---- COMMON arrays of every domain ---- */
static double *alloc_d(size_t n) { return (double *)calloc(n, sizeof(double)); }

static void alloc_domain(sesp_cmn_domain *D, int with_nh) {
    memset(D, 0, sizeof *D);
    D->nw3 = NW3;
    D->ns29 = NS29;
    for (int a = 0; a < 3; a++) {
        D->rw1[a] = alloc_d((size_t)NW3 * 216);
        D->rw2[a] = alloc_d((size_t)NW3 * 512);
        D->vw1[a] = alloc_d((size_t)NW3 * 64);
        D->vw2[a] = alloc_d((size_t)NW3 * 64);
        D->fw1[a] = alloc_d((size_t)NW3 * 216);
        D->fw2[a] = alloc_d((size_t)NW3 * 512);
        D->aw1[a] = alloc_d((size_t)NW3 * 64);
        D->aw2[a] = alloc_d((size_t)NW3 * 64);
        D->rs[a] = alloc_d((size_t)NS29 * 1000);
        D->vs[a] = alloc_d((size_t)NS29 * 64);
        D->as[a] = alloc_d((size_t)NS29 * 64);
        D->fs[a] = alloc_d((size_t)NS29 * 1000);
    }
    D->ictw1 = (int *)calloc(216, sizeof(int));
    D->ictw2 = (int *)calloc(512, sizeof(int));
    D->icts = (int *)calloc(1000, sizeof(int));
    D->nh = with_nh ? alloc_d(SESP_CMN_NH) : NULL;
}

static void free_domain(sesp_cmn_domain *D) {
    for (int a = 0; a < 3; a++) {
        free(D->rw1[a]); free(D->rw2[a]); free(D->vw1[a]); free(D->vw2[a]);
        free(D->fw1[a]); free(D->fw2[a]); free(D->aw1[a]); free(D->aw2[a]);
        free(D->rs[a]); free(D->vs[a]); free(D->as[a]); free(D->fs[a]);
    }
    free(D->ictw1); free(D->ictw2); free(D->icts); free(D->nh);
}

/* where the transcription put each molecule (file order): domain (0-based),
 * class, Fortran column (1-based), central cell ib64 (1-based), slot (0-based) */
typedef struct { int d, cls, col, ib64, slot; } slot_t;

/* src/read_config.f90:40-171 over every rank iaq; returns 0 or -1 on overflow */
static int read_config(sesp_cmn_domain *doms, int ndom, int nw, int ns, const double *pos, const double *vel,
                       slot_t *where) {
    for (int m = 0; m < nw + ns; m++) where[m].d = -1;
    for (int iaq = 0; iaq < ndom; iaq++) {
        sesp_cmn_domain *D = &doms[iaq];
        double cen[3];
        box_center(iaq, cen);
        for (int w = 0; w < nw; w++) {
            const double *O = pos + 9 * w, *G = O + 3, *H = O + 6;
            int ibO = ibox2(O[0], O[1], O[2]), ibG = ibox2(G[0], G[1], G[2]), ibH = ibox2(H[0], H[1], H[2]);
            if (ibO != iaq + 1) continue;
            int ib64O = ibox64(O[0], O[1], O[2], cen);
            int w1 = 0;
            if (ibO == ibG && ibO == ibH) {
                int ib64G = ibox64(G[0], G[1], G[2], cen), ib64H = ibox64(H[0], H[1], H[2], cen);
                w1 = ib64O == ib64G && ib64O == ib64H;
            }
            int col = w1 ? IB216(ib64O) : IB512(ib64O);
            int *ict = w1 ? &D->ictw1[col - 1] : &D->ictw2[col - 1];
            if (*ict >= NW3 / 3) return -1;
            *ict += 1;
            for (int j = 0; j < 3; j++) {
                int k = (*ict - 1) * 3 + j + 1;
                for (int a = 0; a < 3; a++) {
                    (w1 ? D->rw1 : D->rw2)[a][(size_t)(col - 1) * NW3 + k - 1] = pos[9 * w + 3 * j + a];
                    (w1 ? D->vw1 : D->vw2)[a][(size_t)(ib64O - 1) * NW3 + k - 1] = vel[9 * w + 3 * j + a];
                }
            }
            where[w] = (slot_t){iaq, w1 ? SESP_CMN_W1 : SESP_CMN_W2, col, ib64O, *ict - 1};
        }
        for (int s = 0; s < ns; s++) {
            const double *S0 = pos + 9 * nw + 87 * s;
            const double *K = S0 + 3 * 13;
            if (ibox2(K[0], K[1], K[2]) != iaq + 1) continue;
            int ib64O = ibox64(K[0], K[1], K[2], cen);
            int col = IB1000(ib64O);
            if (D->icts[col - 1] >= NS29 / 29) return -1;
            D->icts[col - 1] += 1;
            for (int j = 0; j < 29; j++) {
                int k = (D->icts[col - 1] - 1) * 29 + j + 1;
                for (int a = 0; a < 3; a++) {
                    D->rs[a][(size_t)(col - 1) * NS29 + k - 1] = S0[3 * j + a];
                    D->vs[a][(size_t)(ib64O - 1) * NS29 + k - 1] = vel[9 * nw + 87 * s + 3 * j + a];
                }
            }
            where[nw + s] = (slot_t){iaq, SESP_CMN_SURF, col, ib64O, D->icts[col - 1] - 1};
        }
    }
    return 0;
}

static int sites_before(int m, int nw) { return m < nw ? 3 * m : 3 * nw + 29 * (m - nw); }
static int sites_of(int m, int nw) { return m < nw ? 3 : 29; }

/* engine molecule -> file molecule, from the layer's slots and the transcription's */
static int build_perm(const sesp_cmn_map *map, int nmol, const slot_t *where, int *perm) {
    for (int e = 0; e < nmol; e++) {
        int s[4];
        if (sesp_cmn_slot(map, e, s)) return -1;
        perm[e] = -1;
        for (int f = 0; f < nmol; f++)
            if (where[f].d == s[0] && where[f].cls == s[1] && where[f].ib64 == s[2] + 1 && where[f].slot == s[3]) {
                perm[e] = f;
                break;
            }
        if (perm[e] < 0) return -1;
    }
    return 0;
}

static int cmp_arrays(const sesp_cmn_domain *A, const sesp_cmn_domain *B, int nd) {
    int bad = 0;
    for (int d = 0; d < nd; d++) {
        bad += memcmp(A[d].ictw1, B[d].ictw1, 216 * sizeof(int)) != 0;
        bad += memcmp(A[d].ictw2, B[d].ictw2, 512 * sizeof(int)) != 0;
        bad += memcmp(A[d].icts, B[d].icts, 1000 * sizeof(int)) != 0;
        for (int a = 0; a < 3; a++) {
            bad += memcmp(A[d].rw1[a], B[d].rw1[a], (size_t)NW3 * 216 * 8) != 0;
            bad += memcmp(A[d].rw2[a], B[d].rw2[a], (size_t)NW3 * 512 * 8) != 0;
            bad += memcmp(A[d].rs[a], B[d].rs[a], (size_t)NS29 * 1000 * 8) != 0;
            bad += memcmp(A[d].vw1[a], B[d].vw1[a], (size_t)NW3 * 64 * 8) != 0;
            bad += memcmp(A[d].vw2[a], B[d].vw2[a], (size_t)NW3 * 64 * 8) != 0;
            bad += memcmp(A[d].vs[a], B[d].vs[a], (size_t)NS29 * 64 * 8) != 0;
        }
    }
    return bad;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s mode in.bin [out.bin]\n", argv[0]);
        return 2;
    }
    int mode = atoi(argv[1]);
    FILE *fi = fopen(argv[2], "rb");
    if (!fi) return 2;
    int hdr[8];
    if (fread(hdr, sizeof(int), 8, fi) != 8) return 2;
    int nw = hdr[0], ns = hdr[1], nc[3] = {hdr[2], hdr[3], hdr[4]}, ncarb = hdr[5], nsteps = hdr[6], prec = hdr[7];
    int nmol = nw + ns, nsite = 3 * nw + 29 * ns;
    double *pos = alloc_d(3 * (size_t)nsite), *vel = alloc_d(3 * (size_t)nsite), *carb = alloc_d(3 * (size_t)ncarb + 3);
    if (fread(pos, 8, 3 * (size_t)nsite, fi) != 3 * (size_t)nsite || fread(vel, 8, 3 * (size_t)nsite, fi) != 3 * (size_t)nsite ||
        fread(carb, 8, 3 * (size_t)ncarb, fi) != 3 * (size_t)ncarb)
        return 2;
    fclose(fi);

    int ndom = 0;
    CHECK(sesp_cmn_domain_count(nc, &ndom) == 0, "domain count");
    init_box(nc);
    CHECK(ndom == ibdx2 * ibdy2 * ibdz2, "ndom %d", ndom);
    sesp_cmn_domain *doms = (sesp_cmn_domain *)calloc(ndom, sizeof *doms);
    for (int d = 0; d < ndom; d++) alloc_domain(&doms[d], 1);
    slot_t *where = (slot_t *)calloc(nmol, sizeof *where);
    if (read_config(doms, ndom, nw, ns, pos, vel, where)) {
        fprintf(stderr, "a cell overflows the reference's columns\n");
        return 2;
    }
    for (int m = 0; m < nmol; m++) CHECK(where[m].d >= 0, "molecule %d in no domain", m);
    int *perm = (int *)calloc(nmol, sizeof(int));

    if (mode == 0) {
        sesp_cmn_map *map = NULL;
        int gw = -1, gs = -1;
        double *pe = alloc_d(3 * (size_t)nsite), *ve = alloc_d(3 * (size_t)nsite);
        CHECK(sesp_cmn_map_from_domains(doms, nc, &map, &gw, &gs, pe, ve) == 0, "map");
        CHECK(gw == nw && gs == ns, "molecule counts %d %d", gw, gs);
        CHECK(build_perm(map, nmol, where, perm) == 0, "every engine molecule sits in a transcribed slot");
        /* bijection, and the documented engine order */
        int *seen = (int *)calloc(nmol, sizeof(int));
        int prev[4] = {-1, -1, -1, -1};
        for (int e = 0; e < nmol; e++) {
            seen[perm[e]]++;
            CHECK((e < nw) == (perm[e] < nw), "waters first");
            int s[4];
            sesp_cmn_slot(map, e, s);
            if (e == nw) prev[0] = prev[1] = prev[2] = prev[3] = -1;
            long key = (((long)s[0] * 64 + s[2]) * 3 + s[1]) * 4096 + s[3];
            long pkey = (((long)prev[0] * 64 + prev[2]) * 3 + prev[1]) * 4096 + prev[3];
            CHECK(prev[0] < 0 || key > pkey, "engine order at %d", e);
            memcpy(prev, s, sizeof prev);
            int f = perm[e];
            for (int t = 0; t < 3 * sites_of(e, nw); t++) {
                CHECK(pe[3 * sites_before(e, nw) + t] == pos[3 * sites_before(f, nw) + t], "position of %d", e);
                CHECK(ve[3 * sites_before(e, nw) + t] == vel[3 * sites_before(f, nw) + t], "velocity of %d", e);
            }
        }
        for (int f = 0; f < nmol; f++) CHECK(seen[f] == 1, "file molecule %d taken %d times", f, seen[f]);
        /* the layer's rule agrees with the transcription on every molecule */
        CHECK(sesp_cmn_assign(map, pe) == 0, "assign");
        int *perm2 = (int *)calloc(nmol, sizeof(int));
        CHECK(build_perm(map, nmol, where, perm2) == 0 && memcmp(perm, perm2, nmol * sizeof(int)) == 0,
              "re-assignment keeps every slot");
        /* scatter into fresh arrays reproduces read_config's arrays bit for bit */
        sesp_cmn_domain *fresh = (sesp_cmn_domain *)calloc(ndom, sizeof *fresh);
        for (int d = 0; d < ndom; d++) alloc_domain(&fresh[d], 0);
        double *acc = alloc_d(3 * (size_t)nsite), *frc = alloc_d(3 * (size_t)nsite);
        for (int i = 0; i < 3 * nsite; i++) {
            acc[i] = 0.5 * ve[i] + 1.0;
            frc[i] = -2.0 * pe[i];
        }
        CHECK(sesp_cmn_scatter(map, fresh, pe, ve, acc, frc) == 0, "scatter");
        CHECK(cmp_arrays(doms, fresh, ndom) == 0, "scattered arrays differ from read_config's");
        for (int e = 0; e < nmol; e++) {
            slot_t w = where[perm[e]];
            int n = sites_of(e, nw);
            for (int t = 0; t < n; t++)
                for (int a = 0; a < 3; a++) {
                    size_t k = (size_t)w.slot * n + t;
                    double fv = w.cls == SESP_CMN_SURF ? fresh[w.d].fs[a][(size_t)(w.col - 1) * NS29 + k]
                                : w.cls == SESP_CMN_W1 ? fresh[w.d].fw1[a][(size_t)(w.col - 1) * NW3 + k]
                                                       : fresh[w.d].fw2[a][(size_t)(w.col - 1) * NW3 + k];
                    double av = w.cls == SESP_CMN_SURF ? fresh[w.d].as[a][(size_t)(w.ib64 - 1) * NS29 + k]
                                : w.cls == SESP_CMN_W1 ? fresh[w.d].aw1[a][(size_t)(w.ib64 - 1) * NW3 + k]
                                                       : fresh[w.d].aw2[a][(size_t)(w.ib64 - 1) * NW3 + k];
                    CHECK(fv == frc[3 * (sites_before(e, nw) + t) + a], "force slot of %d", e);
                    CHECK(av == acc[3 * (sites_before(e, nw) + t) + a], "acceleration slot of %d", e);
                }
        }
        double *pg = alloc_d(3 * (size_t)nsite), *vg = alloc_d(3 * (size_t)nsite), *ag = alloc_d(3 * (size_t)nsite);
        CHECK(sesp_cmn_gather(map, fresh, pg, vg, ag) == 0, "gather");
        CHECK(memcmp(pg, pe, 24 * (size_t)nsite) == 0 && memcmp(vg, ve, 24 * (size_t)nsite) == 0 &&
                  memcmp(ag, acc, 24 * (size_t)nsite) == 0,
              "gather returns what scatter wrote");
        /* a w1 water whose H crosses into the next cell becomes w2 in its O's cell;
         * a surfactant whose key site moves by a domain changes domain */
        int wv = -1;
        for (int e = 0; e < nw && wv < 0; e++) {
            int s[4];
            sesp_cmn_slot(map, e, s);
            if (s[1] == SESP_CMN_W1) wv = e;
        }
        CHECK(wv >= 0, "a w1 water");
        if (wv >= 0) {
            int s0[4], s1[4];
            sesp_cmn_slot(map, wv, s0);
            double *pm = alloc_d(3 * (size_t)nsite);
            memcpy(pm, pe, 24 * (size_t)nsite);
            double *H = pm + 9 * wv + 6;
            H[0] += (H[0] < 0 ? 1.0 : -1.0) * rs_;
            CHECK(sesp_cmn_assign(map, pm) == 0, "assign moved");
            sesp_cmn_slot(map, wv, s1);
            CHECK(s1[1] == SESP_CMN_W2 && s1[0] == s0[0] && s1[2] == s0[2], "moved water: class %d", s1[1]);
            if (ns > 0) {
                int se = nw, d0[4], d1[4];
                sesp_cmn_slot(map, se, d0);
                double *S0 = pm + 9 * nw;
                double shift = (S0[3 * 13 + 2] < 0 ? 4.0 : -4.0) * rs_;
                for (int t = 0; t < 29; t++) S0[3 * t + 2] += shift;
                CHECK(sesp_cmn_assign(map, pm) == 0, "assign moved surfactant");
                sesp_cmn_slot(map, se, d1);
                int dz0 = d0[0] / (ibdx2 * ibdy2), dz1 = d1[0] / (ibdx2 * ibdy2);
                CHECK(d1[1] == SESP_CMN_SURF && abs(dz1 - dz0) == 1 && d1[2] == d0[2], "moved surfactant");
            }
            /* a key site outside the box is an error and leaves the map as it was */
            pm[0] = rhsx + 1.0;
            sesp_cmn_slot(map, 0, s0);
            CHECK(sesp_cmn_assign(map, pm) == SESP_EINVAL, "outside the box");
            sesp_cmn_slot(map, 0, s1);
            CHECK(memcmp(s0, s1, sizeof s0) == 0, "map unchanged after a failed assign");
            char msg[256];
            sesp_cmn_last_error(msg, sizeof msg);
            CHECK(strstr(msg, "outside") != NULL, "message: %s", msg);
            free(pm);
        }
        /* a count above the column height is refused */
        sesp_cmn_map *bad = NULL;
        int keep = doms[0].ictw1[IB216(1) - 1];
        doms[0].ictw1[IB216(1) - 1] = NW3 / 3 + 1;
        CHECK(sesp_cmn_map_from_domains(doms, nc, &bad, NULL, NULL, NULL, NULL) == SESP_ECAPACITY && bad == NULL,
              "capacity");
        doms[0].ictw1[IB216(1) - 1] = keep;
        int badnc[3] = {12, 10, 12};
        CHECK(sesp_cmn_domain_count(badnc, &ndom) == SESP_EINVAL, "n_cells not multiples of 4");
        /* the subroutines refuse to run with no job attached */
        int r = 0;
        evalforces_(&r);
        CHECK(sesp_cmn_status() == SESP_ESTATE, "no job");
        sesp_cmn_map_destroy(map);
        if (g_fail == 0) printf("OK layout: %d waters, %d surfactants, %d domains\n", nw, ns, ndom);
        return g_fail ? 1 : 0;
    }

    /* mode 1: the step loop on the GPU */
    sesp_params p;
    sesp_default_params(&p);
    p.n_cells[0] = nc[0];
    p.n_cells[1] = nc[1];
    p.n_cells[2] = nc[2];
    p.precision = prec;
    p.graphite_on = ncarb > 0;
    int rc = sesp_cmn_attach(&p, doms, ncarb, carb, 99101);
    if (rc) {
        char msg[512];
        sesp_cmn_last_error(msg, sizeof msg);
        fprintf(stderr, "attach: %d %s\n", rc, msg);
        return 1;
    }
    CHECK(build_perm(sesp_cmn_current_map(), nmol, where, perm) == 0, "perm");
    int my3d = 0, comm3d = 0;
    evalforces_(&my3d);
    double *f0 = alloc_d(3 * (size_t)nsite);
    for (int f = 0; f < nmol; f++) {
        slot_t w = where[f];
        int n = sites_of(f, nw);
        for (int t = 0; t < n; t++)
            for (int a = 0; a < 3; a++) {
                size_t k = (size_t)w.slot * n + t;
                f0[3 * (sites_before(f, nw) + t) + a] =
                    w.cls == SESP_CMN_SURF ? doms[w.d].fs[a][(size_t)(w.col - 1) * NS29 + k]
                    : w.cls == SESP_CMN_W1 ? doms[w.d].fw1[a][(size_t)(w.col - 1) * NW3 + k]
                                           : doms[w.d].fw2[a][(size_t)(w.col - 1) * NW3 + k];
            }
    }
    init_accel_(&my3d);
    for (int kb = 0; kb < nsteps; kb++) {
        move_surfactant_a_(&my3d);
        move_w1_a_(&my3d);
        move_w2_a_(&comm3d, &my3d);
        evalforces_(&my3d);
        move_surfactant_b_(&my3d);
        move_w1_b_(&my3d);
        move_w2_b_(&my3d);
    }
    CHECK(sesp_cmn_status() == 0, "status %d", sesp_cmn_status());
    /* the mirror holds the device state bit for bit */
    double *pm = alloc_d(3 * (size_t)nsite), *vm = alloc_d(3 * (size_t)nsite), *am = alloc_d(3 * (size_t)nsite);
    double *pd = alloc_d(3 * (size_t)nsite), *vd = alloc_d(3 * (size_t)nsite), *ad = alloc_d(3 * (size_t)nsite);
    const sesp_cmn_map *map = sesp_cmn_current_map();
    CHECK(sesp_cmn_gather(map, doms, pm, vm, am) == 0, "gather");
    CHECK(sesp_download_state(sesp_cmn_context(), pd, vd, ad) == 0, "download");
    CHECK(memcmp(pm, pd, 24 * (size_t)nsite) == 0, "mirrored positions");
    CHECK(memcmp(vm, vd, 24 * (size_t)nsite) == 0, "mirrored velocities");
    CHECK(memcmp(am, ad, 24 * (size_t)nsite) == 0, "mirrored accelerations");
    double eta = 0.0;
    sesp_get_eta(sesp_cmn_context(), &eta);
    CHECK(doms[0].nh[3] == eta && doms[ndom - 1].nh[3] == eta, "eta mirrored");
    /* after a rebuild step the mirror's classes and cells are read_config's
     * for the current positions */
    if (nsteps % 10 == 0) {
        double *pf = alloc_d(3 * (size_t)nsite), *vf = alloc_d(3 * (size_t)nsite);
        for (int e = 0; e < nmol; e++)
            for (int t = 0; t < 3 * sites_of(e, nw); t++) {
                pf[3 * sites_before(perm[e], nw) + t] = pd[3 * sites_before(e, nw) + t];
                vf[3 * sites_before(perm[e], nw) + t] = vd[3 * sites_before(e, nw) + t];
            }
        sesp_cmn_domain *ref = (sesp_cmn_domain *)calloc(ndom, sizeof *ref);
        for (int d = 0; d < ndom; d++) alloc_domain(&ref[d], 0);
        slot_t *w2 = (slot_t *)calloc(nmol, sizeof *w2);
        CHECK(read_config(ref, ndom, nw, ns, pf, vf, w2) == 0, "transcription after the run");
        int moved = 0;
        for (int e = 0; e < nmol; e++) {
            int s[4];
            sesp_cmn_slot(map, e, s);
            slot_t w = w2[perm[e]];
            CHECK(w.d == s[0] && w.cls == s[1] && w.ib64 == s[2] + 1, "molecule %d placed as read_config would", e);
            slot_t w0 = where[perm[e]];
            moved += w0.d != w.d || w0.cls != w.cls || w0.ib64 != w.ib64;
        }
        for (int d = 0; d < ndom; d++) {
            CHECK(memcmp(ref[d].ictw1, doms[d].ictw1, 216 * sizeof(int)) == 0, "ictw1 of domain %d", d);
            CHECK(memcmp(ref[d].ictw2, doms[d].ictw2, 512 * sizeof(int)) == 0, "ictw2 of domain %d", d);
            CHECK(memcmp(ref[d].icts, doms[d].icts, 1000 * sizeof(int)) == 0, "icts of domain %d", d);
        }
        printf("molecules that changed domain, class or cell: %d\n", moved);
    }
    /* sesp_cmn_reload: a velocity rescale done in the COMMON arrays reaches
     * the engine; positions and accelerations stay the engine's */
    {
        double *vh = alloc_d(3 * (size_t)nsite), *p2 = alloc_d(3 * (size_t)nsite), *v2 = alloc_d(3 * (size_t)nsite),
               *a2 = alloc_d(3 * (size_t)nsite);
        for (int i = 0; i < 3 * nsite; i++) vh[i] = 0.5 * vd[i];
        CHECK(sesp_cmn_scatter(map, doms, NULL, vh, NULL, NULL) == 0, "scatter halved velocities");
        sesp_cmn_reload_(&my3d);
        CHECK(sesp_cmn_status() == 0, "reload status %d", sesp_cmn_status());
        CHECK(sesp_download_state(sesp_cmn_context(), p2, v2, a2) == 0, "download after reload");
        CHECK(memcmp(v2, vh, 24 * (size_t)nsite) == 0, "reloaded velocities");
        CHECK(memcmp(p2, pd, 24 * (size_t)nsite) == 0, "positions kept");
        CHECK(memcmp(a2, ad, 24 * (size_t)nsite) == 0, "accelerations kept");
        /* put the run's velocities back for the output below */
        CHECK(sesp_cmn_scatter(map, doms, NULL, vd, NULL, NULL) == 0, "scatter velocities");
        sesp_cmn_reload_(&my3d);
        free(vh); free(p2); free(v2); free(a2);
    }
    if (argc > 3) {
        FILE *fo = fopen(argv[3], "wb");
        fwrite(f0, 8, 3 * (size_t)nsite, fo);
        for (int e = 0; e < nmol; e++) {
            /* back to file order */
            int f = perm[e];
            for (int t = 0; t < 3 * sites_of(e, nw); t++) {
                pm[3 * sites_before(f, nw) + t] = pd[3 * sites_before(e, nw) + t];
                vm[3 * sites_before(f, nw) + t] = vd[3 * sites_before(e, nw) + t];
            }
        }
        fwrite(pm, 8, 3 * (size_t)nsite, fo);
        fwrite(vm, 8, 3 * (size_t)nsite, fo);
        fwrite(&eta, 8, 1, fo);
        fclose(fo);
    }
    CHECK(sesp_cmn_detach() == 0, "detach");
    for (int d = 0; d < ndom; d++) free_domain(&doms[d]);
    if (g_fail == 0) printf("OK steps: %d\n", nsteps);
    return g_fail ? 1 : 0;
}
