// COMMON-block compatibility layer (include/sesp_common.h): the reference's
// per-rank COMMON arrays (src/mybox.cmns:125-259) as a mirror of the engine
// state, and the step loop's calls under their gfortran names.  Host code over
// the public C ABI only.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sesp_common.h"

namespace {

constexpr double SIGMA_A = 3.166;
constexpr double RS = 10.0 / SIGMA_A + 2.0 / SIGMA_A;   // rc + delta, src/mybox.cmns:36-40
constexpr int NSS = 29;                                   // surfactant sites
constexpr int KEY_SITE = 13;                              // surfactant site keyed to a cell (14th)

thread_local std::string g_cmn_err;

int fail(int code, const std::string &msg) {
    g_cmn_err = msg;
    return code;
}

}  // namespace

struct sesp_cmn_map {
    int nw = 0, ns = 0;
    int nc[3] = {0, 0, 0};
    int nd[3] = {0, 0, 0};
    int ndom = 0;
    double rsd[3] = {0, 0, 0}, rhs[3] = {0, 0, 0}, cen[3][64] = {};   // box sizes, domain centres per axis
    std::vector<int> dom, cls, cell, slot;                            // per molecule
    std::vector<int> count;                                           // [domain][class][central cell]
};

namespace {

// columns of a central cell c = ix + 4 iy + 16 iz in the 6^3 / 8^3 / 10^3 arrays:
// halo widths 1, 2, 3 (the index maps of src/ibox.f90:1-44)
inline int col_w1(int c) { return (c / 16 + 1) * 36 + (c / 4 % 4 + 1) * 6 + (c % 4 + 1); }
inline int col_w2(int c) { return (c / 16 + 2) * 64 + (c / 4 % 4 + 2) * 8 + (c % 4 + 2); }
inline int col_s(int c) { return (c / 16 + 3) * 100 + (c / 4 % 4 + 3) * 10 + (c % 4 + 3); }

bool setup(sesp_cmn_map &m, const int n_cells[3]) {
    for (int a = 0; a < 3; a++) {
        if (n_cells[a] <= 0 || n_cells[a] % 4 != 0 || n_cells[a] / 4 > 64) return false;
        m.nc[a] = n_cells[a];
        m.nd[a] = n_cells[a] / 4;
        // src/init_box_dimensions.f90:14-20 and the domain centres of
        // src/init_box_dimensions.f90:37-39 (get_box_center), same operation order
        m.rsd[a] = m.nc[a] * RS;
        m.rhs[a] = m.rsd[a] / 2.0;
        double rd = (double)m.nd[a];
        for (int i = 0; i < m.nd[a]; i++) m.cen[a][i] = m.rsd[a] * (i + 1) / rd - m.rhs[a] - m.rsd[a] / rd / 2.0;
    }
    m.ndom = m.nd[0] * m.nd[1] * m.nd[2];
    return true;
}

// src/ibox.f90:128-139 (ibox2) per axis; -1 outside the box
inline int domain_axis(const sesp_cmn_map &m, int a, double x) {
    double t = (x + m.rhs[a]) * (double)m.nd[a] / m.rsd[a];
    if (!(t >= 0.0)) return -1;
    int i = (int)t;
    return i < m.nd[a] ? i : -1;
}

inline int domain_of(const sesp_cmn_map &m, const double *r) {
    int i = domain_axis(m, 0, r[0]), j = domain_axis(m, 1, r[1]), k = domain_axis(m, 2, r[2]);
    if (i < 0 || j < 0 || k < 0) return -1;
    return i + m.nd[0] * (j + m.nd[1] * k);
}

// src/ibox.f90:172-185 (ibox64) relative to domain d's centre; an index that
// rounding puts one past the domain's edge is held at the edge cell
inline int cell_of(const sesp_cmn_map &m, int d, const double *r) {
    int di[3] = {d % m.nd[0], d / m.nd[0] % m.nd[1], d / (m.nd[0] * m.nd[1])};
    int c[3];
    for (int a = 0; a < 3; a++) {
        double p = r[a] - m.cen[a][di[a]] + 2.0 * RS;
        int i = (int)(p / RS);
        c[a] = i < 0 ? 0 : (i > 3 ? 3 : i);
    }
    return c[0] + 4 * c[1] + 16 * c[2];
}

inline int site_of(const sesp_cmn_map &m, int mol) { return mol < m.nw ? 3 * mol : 3 * m.nw + NSS * (mol - m.nw); }
inline int sites_in(const sesp_cmn_map &m, int mol) { return mol < m.nw ? 3 : NSS; }

// (pointer triple, column, leading dimension) of a molecule's slot for one array kind
enum Kind { POS, VEL, ACC, FRC };

bool locate(const sesp_cmn_domain &D, int cls, int cell, int kind, double *const **arr, int *col, int *ld) {
    if (cls == SESP_CMN_SURF) {
        *ld = D.ns29;
        switch (kind) {
            case POS: *arr = D.rs; *col = col_s(cell); break;
            case VEL: *arr = D.vs; *col = cell; break;
            case ACC: *arr = D.as; *col = cell; break;
            default: *arr = D.fs; *col = col_s(cell); break;
        }
    } else {
        bool w1 = cls == SESP_CMN_W1;
        *ld = D.nw3;
        switch (kind) {
            case POS: *arr = w1 ? D.rw1 : D.rw2; *col = w1 ? col_w1(cell) : col_w2(cell); break;
            case VEL: *arr = w1 ? D.vw1 : D.vw2; *col = cell; break;
            case ACC: *arr = w1 ? D.aw1 : D.aw2; *col = cell; break;
            default: *arr = w1 ? D.fw1 : D.fw2; *col = w1 ? col_w1(cell) : col_w2(cell); break;
        }
    }
    return (*arr)[0] && (*arr)[1] && (*arr)[2];
}

void copy_out(const sesp_cmn_map &m, sesp_cmn_domain *doms, const double *src, int kind) {
    for (int mol = 0; mol < m.nw + m.ns; mol++) {
        double *const *arr;
        int col, ld;
        if (!locate(doms[m.dom[mol]], m.cls[mol], m.cell[mol], kind, &arr, &col, &ld)) continue;
        int n = sites_in(m, mol), s0 = site_of(m, mol);
        size_t base = (size_t)col * ld + (size_t)m.slot[mol] * n;
        for (int t = 0; t < n; t++)
            for (int a = 0; a < 3; a++) arr[a][base + t] = src[3 * (s0 + t) + a];
    }
}

// (a molecule whose domain does not bind this array keeps what dst holds)
void copy_in(const sesp_cmn_map &m, const sesp_cmn_domain *doms, double *dst, int kind) {
    for (int mol = 0; mol < m.nw + m.ns; mol++) {
        double *const *arr;
        int col, ld;
        int n = sites_in(m, mol), s0 = site_of(m, mol);
        if (!locate(doms[m.dom[mol]], m.cls[mol], m.cell[mol], kind, &arr, &col, &ld)) continue;
        size_t base = (size_t)col * ld + (size_t)m.slot[mol] * n;
        for (int t = 0; t < n; t++)
            for (int a = 0; a < 3; a++) dst[3 * (s0 + t) + a] = arr[a][base + t];
    }
}

bool domain_ok(const sesp_cmn_domain &D) {
    return D.nw3 >= 3 && D.ns29 >= NSS && D.ictw1 && D.ictw2 && D.icts && D.rw1[0] && D.rw1[1] && D.rw1[2] &&
           D.rw2[0] && D.rw2[1] && D.rw2[2] && D.rs[0] && D.rs[1] && D.rs[2];
}

}  // namespace

extern "C" {

int sesp_cmn_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return SESP_EINVAL;
    std::snprintf(buf, len, "%s", g_cmn_err.c_str());
    return SESP_OK;
}

int sesp_cmn_domain_count(const int n_cells[3], int *ndom) {
    sesp_cmn_map m;
    if (!n_cells || !ndom || !setup(m, n_cells)) return fail(SESP_EINVAL, "n_cells must be positive multiples of 4");
    *ndom = m.ndom;
    return SESP_OK;
}

int sesp_cmn_map_from_domains(const sesp_cmn_domain *doms, const int n_cells[3], sesp_cmn_map **out, int *n_water,
                              int *n_surf, double *pos, double *vel) {
    if (!doms || !n_cells || !out) return fail(SESP_EINVAL, "null argument");
    auto *m = new sesp_cmn_map;
    if (!setup(*m, n_cells)) {
        delete m;
        return fail(SESP_EINVAL, "n_cells must be positive multiples of 4");
    }
    // enumerate the central cells: waters (w1 before w2 in each cell), then surfactants
    for (int pass = 0; pass < 2; pass++) {
        for (int d = 0; d < m->ndom; d++) {
            const sesp_cmn_domain &D = doms[d];
            if (!domain_ok(D)) {
                delete m;
                return fail(SESP_EINVAL, "domain " + std::to_string(d) + ": missing array or bad leading dimension");
            }
            for (int c = 0; c < 64; c++) {
                for (int cls = (pass ? 2 : 0); cls < (pass ? 3 : 2); cls++) {
                    int n = cls == 0 ? D.ictw1[col_w1(c)] : cls == 1 ? D.ictw2[col_w2(c)] : D.icts[col_s(c)];
                    int cap = cls == 2 ? D.ns29 / NSS : D.nw3 / 3;
                    if (n < 0 || n > cap) {
                        delete m;
                        return fail(SESP_ECAPACITY, "domain " + std::to_string(d) + " cell " + std::to_string(c + 1) +
                                                        ": molecule count " + std::to_string(n) + " outside 0.." +
                                                        std::to_string(cap));
                    }
                    for (int k = 0; k < n; k++) {
                        m->dom.push_back(d);
                        m->cls.push_back(cls);
                        m->cell.push_back(c);
                        m->slot.push_back(k);
                    }
                }
            }
        }
        if (pass == 0) m->nw = (int)m->dom.size();
    }
    m->ns = (int)m->dom.size() - m->nw;
    m->count.assign((size_t)m->ndom * 3 * 64, 0);
    for (int mol = 0; mol < m->nw + m->ns; mol++) m->count[((size_t)m->dom[mol] * 3 + m->cls[mol]) * 64 + m->cell[mol]]++;
    if (pos) copy_in(*m, doms, pos, POS);
    if (vel) copy_in(*m, doms, vel, VEL);
    if (n_water) *n_water = m->nw;
    if (n_surf) *n_surf = m->ns;
    *out = m;
    return SESP_OK;
}

int sesp_cmn_map_destroy(sesp_cmn_map *m) {
    delete m;
    return SESP_OK;
}

int sesp_cmn_assign(sesp_cmn_map *m, const double *pos) {
    if (!m || !pos) return fail(SESP_EINVAL, "null argument");
    const int nmol = m->nw + m->ns;
    std::vector<int> dom(nmol), cls(nmol), cell(nmol), slot(nmol);
    std::vector<int> count((size_t)m->ndom * 3 * 64, 0);
    for (int mol = 0; mol < nmol; mol++) {
        const double *r = pos + 3 * site_of(*m, mol);
        if (mol < m->nw) {
            // src/read_config.f90:55-132: the O's domain; w1 when O and both H
            // share it and one L4 cell, else w2 in the O's cell
            int dO = domain_of(*m, r), dG = domain_of(*m, r + 3), dH = domain_of(*m, r + 6);
            if (dO < 0) return fail(SESP_EINVAL, "water " + std::to_string(mol) + ": O outside the box");
            int cO = cell_of(*m, dO, r);
            int c = SESP_CMN_W2;
            if (dO == dG && dO == dH && cO == cell_of(*m, dO, r + 3) && cO == cell_of(*m, dO, r + 6)) c = SESP_CMN_W1;
            dom[mol] = dO;
            cls[mol] = c;
            cell[mol] = cO;
        } else {
            // src/read_config.f90:137-171: the cell of the 14th site
            const double *k = r + 3 * KEY_SITE;
            int d = domain_of(*m, k);
            if (d < 0) return fail(SESP_EINVAL, "surfactant " + std::to_string(mol - m->nw) + ": key site outside the box");
            dom[mol] = d;
            cls[mol] = SESP_CMN_SURF;
            cell[mol] = cell_of(*m, d, k);
        }
        int &n = count[((size_t)dom[mol] * 3 + cls[mol]) * 64 + cell[mol]];
        slot[mol] = n++;
    }
    m->dom.swap(dom);
    m->cls.swap(cls);
    m->cell.swap(cell);
    m->slot.swap(slot);
    m->count.swap(count);
    return SESP_OK;
}

int sesp_cmn_scatter(const sesp_cmn_map *m, sesp_cmn_domain *doms, const double *pos, const double *vel,
                     const double *acc, const double *force) {
    if (!m || !doms) return fail(SESP_EINVAL, "null argument");
    for (int d = 0; d < m->ndom; d++)
        if (!domain_ok(doms[d])) return fail(SESP_EINVAL, "domain " + std::to_string(d) + ": missing array");
    for (int d = 0; d < m->ndom; d++)
        for (int c = 0; c < 3; c++)
            for (int cell = 0; cell < 64; cell++) {
                int n = m->count[((size_t)d * 3 + c) * 64 + cell];
                int cap = c == 2 ? doms[d].ns29 / NSS : doms[d].nw3 / 3;
                if (n > cap)
                    return fail(SESP_ECAPACITY, "domain " + std::to_string(d) + " cell " + std::to_string(cell + 1) +
                                                    ": " + std::to_string(n) + " molecules of class " +
                                                    std::to_string(c) + " exceed " + std::to_string(cap));
            }
    if (pos) {
        for (int d = 0; d < m->ndom; d++) {
            sesp_cmn_domain &D = doms[d];
            std::memset(D.ictw1, 0, sizeof(int) * SESP_CMN_W1_CELLS);
            std::memset(D.ictw2, 0, sizeof(int) * SESP_CMN_W2_CELLS);
            std::memset(D.icts, 0, sizeof(int) * SESP_CMN_S_CELLS);
            for (int cell = 0; cell < 64; cell++) {
                D.ictw1[col_w1(cell)] = m->count[((size_t)d * 3 + 0) * 64 + cell];
                D.ictw2[col_w2(cell)] = m->count[((size_t)d * 3 + 1) * 64 + cell];
                D.icts[col_s(cell)] = m->count[((size_t)d * 3 + 2) * 64 + cell];
            }
        }
        copy_out(*m, doms, pos, POS);
    }
    if (vel) copy_out(*m, doms, vel, VEL);
    if (acc) copy_out(*m, doms, acc, ACC);
    if (force) copy_out(*m, doms, force, FRC);
    return SESP_OK;
}

int sesp_cmn_gather(const sesp_cmn_map *m, const sesp_cmn_domain *doms, double *pos, double *vel, double *acc) {
    if (!m || !doms) return fail(SESP_EINVAL, "null argument");
    if (pos) copy_in(*m, doms, pos, POS);
    if (vel) copy_in(*m, doms, vel, VEL);
    if (acc) copy_in(*m, doms, acc, ACC);
    return SESP_OK;
}

int sesp_cmn_slot(const sesp_cmn_map *m, int mol, int out[4]) {
    if (!m || !out || mol < 0 || mol >= m->nw + m->ns) return fail(SESP_EINVAL, "molecule out of range");
    out[0] = m->dom[mol];
    out[1] = m->cls[mol];
    out[2] = m->cell[mol];
    out[3] = m->slot[mol];
    return SESP_OK;
}

}  // extern "C"

// ---- the attached job ----

namespace {

struct Job {
    sesp_ctx *ctx = nullptr;
    sesp_cmn_map *map = nullptr;
    sesp_cmn_domain *doms = nullptr;
    int interval = 10;
    int kb = 0;            // number of the current step
    int phase = 0;         // 0 before the first step; 1 after move_a; 2 after the force; 3 after move_b
    bool forced = false;   // a force call has been made
    int status = 0;
    std::vector<double> pos, vel, acc, frc;
};

Job g_job;

int engine_fail(int code, const char *what) {
    char buf[512];
    sesp_last_error(buf, sizeof buf);
    return fail(code, std::string(what) + ": " + buf);
}

void report(const char *name, int code) {
    if (code == SESP_OK) return;
    if (g_job.status == 0) g_job.status = code;
    std::fprintf(stderr, "sesp: %s failed (%d): %s\n", name, code, g_cmn_err.c_str());
}

int need_job() {
    if (!g_job.ctx) return fail(SESP_ESTATE, "no job attached (sesp_cmn_attach)");
    return SESP_OK;
}

int do_init_accel() {
    int rc = need_job();
    if (rc) return rc;
    if (!g_job.forced) return fail(SESP_ESTATE, "init_accel before the first evalforces");
    if ((rc = sesp_init_accel(g_job.ctx))) return engine_fail(rc, "sesp_init_accel");
    if ((rc = sesp_download_state(g_job.ctx, nullptr, nullptr, g_job.acc.data()))) return engine_fail(rc, "download");
    return sesp_cmn_scatter(g_job.map, g_job.doms, nullptr, nullptr, g_job.acc.data(), nullptr);
}

int do_move_a() {
    int rc = need_job();
    if (rc) return rc;
    if (!g_job.forced) return fail(SESP_ESTATE, "move_a before the first evalforces");
    if (g_job.phase == 1) return fail(SESP_ESTATE, "move_a twice without evalforces / move_b");
    if (g_job.phase != 0) g_job.kb++;
    if ((rc = sesp_move_a(g_job.ctx))) return engine_fail(rc, "sesp_move_a");
    g_job.phase = 1;
    if ((rc = sesp_download_state(g_job.ctx, g_job.pos.data(), g_job.vel.data(), nullptr))) return engine_fail(rc, "download");
    // src/mybox.f90:141-153: on rebuild steps molecules move to the cells of their new positions
    if (g_job.kb % g_job.interval == 0 && (rc = sesp_cmn_assign(g_job.map, g_job.pos.data()))) return rc;
    if ((rc = sesp_cmn_scatter(g_job.map, g_job.doms, g_job.pos.data(), g_job.vel.data(), nullptr, nullptr))) return rc;
    double eta;
    if ((rc = sesp_get_eta(g_job.ctx, &eta))) return engine_fail(rc, "sesp_get_eta");
    for (int d = 0; d < g_job.map->ndom; d++)
        if (g_job.doms[d].nh) g_job.doms[d].nh[3] = eta;
    return SESP_OK;
}

int do_force() {
    int rc = need_job();
    if (rc) return rc;
    if (g_job.forced && g_job.phase != 1) return fail(SESP_ESTATE, "evalforces outside a step (after move_a)");
    int rebuild = !g_job.forced || g_job.kb % g_job.interval == 0;
    if ((rc = sesp_force(g_job.ctx, rebuild))) return engine_fail(rc, "sesp_force");
    g_job.forced = true;
    if (g_job.phase == 1) g_job.phase = 2;
    if ((rc = sesp_download_forces(g_job.ctx, g_job.frc.data()))) return engine_fail(rc, "download");
    return sesp_cmn_scatter(g_job.map, g_job.doms, nullptr, nullptr, nullptr, g_job.frc.data());
}

int do_move_b() {
    int rc = need_job();
    if (rc) return rc;
    if (g_job.phase != 2) return fail(SESP_ESTATE, "move_b before this step's evalforces");
    if ((rc = sesp_move_b(g_job.ctx))) return engine_fail(rc, "sesp_move_b");
    g_job.phase = 3;
    if ((rc = sesp_download_state(g_job.ctx, nullptr, g_job.vel.data(), g_job.acc.data()))) return engine_fail(rc, "download");
    return sesp_cmn_scatter(g_job.map, g_job.doms, nullptr, g_job.vel.data(), g_job.acc.data(), nullptr);
}

int check_order(int want_phase, const char *what) {
    int rc = need_job();
    if (rc) return rc;
    if (g_job.phase != want_phase) return fail(SESP_ESTATE, std::string(what) + " called out of order");
    return SESP_OK;
}

}  // namespace

extern "C" {

int sesp_cmn_attach(const sesp_params *p, sesp_cmn_domain *doms, int n_carbon, const double *carbons, int kb0) {
    if (!p || !doms || n_carbon < 0 || (n_carbon > 0 && !carbons)) return fail(SESP_EINVAL, "null argument");
    if (g_job.ctx) return fail(SESP_ESTATE, "a job is already attached");
    if (p->preset != SESP_PRESET_REFERENCE) return fail(SESP_EINVAL, "the COMMON layout is the reference preset's");
    if (p->rebuild_interval <= 0) return fail(SESP_EINVAL, "rebuild_interval must be positive");
    sesp_cmn_map *m = nullptr;
    int nw = 0, ns = 0;
    int rc = sesp_cmn_map_from_domains(doms, p->n_cells, &m, &nw, &ns, nullptr, nullptr);
    if (rc) return rc;
    size_t n3 = 3 * ((size_t)3 * nw + (size_t)NSS * ns);
    std::vector<double> pos(n3), vel(n3);
    sesp_cmn_gather(m, doms, pos.data(), vel.data(), nullptr);
    sesp_ctx *ctx = nullptr;
    if ((rc = sesp_create(p, &ctx))) {
        sesp_cmn_map_destroy(m);
        return engine_fail(rc, "sesp_create");
    }
    if ((rc = sesp_upload_state(ctx, nw, ns, pos.data(), vel.data(), n_carbon, carbons))) {
        engine_fail(rc, "sesp_upload_state");
        sesp_destroy(ctx);
        sesp_cmn_map_destroy(m);
        return rc;
    }
    g_job = Job();
    g_job.ctx = ctx;
    g_job.map = m;
    g_job.doms = doms;
    g_job.interval = p->rebuild_interval;
    g_job.kb = kb0;
    g_job.pos.swap(pos);
    g_job.vel.swap(vel);
    g_job.acc.assign(n3, 0.0);
    g_job.frc.assign(n3, 0.0);
    return SESP_OK;
}

int sesp_cmn_detach(void) {
    if (!g_job.ctx) return fail(SESP_ESTATE, "no job attached");
    int rc = sesp_destroy(g_job.ctx);
    sesp_cmn_map_destroy(g_job.map);
    g_job = Job();
    return rc;
}

sesp_ctx *sesp_cmn_context(void) { return g_job.ctx; }

const sesp_cmn_map *sesp_cmn_current_map(void) { return g_job.map; }

int sesp_cmn_reload(void) {
    int rc = need_job();
    if (rc) return rc;
    // start from the engine's state, so arrays the domains do not bind keep it
    if ((rc = sesp_download_state(g_job.ctx, g_job.pos.data(), g_job.vel.data(), g_job.acc.data())))
        return engine_fail(rc, "download");
    sesp_cmn_gather(g_job.map, g_job.doms, g_job.pos.data(), g_job.vel.data(), g_job.acc.data());
    double eta;
    if ((rc = sesp_get_eta(g_job.ctx, &eta))) return engine_fail(rc, "sesp_get_eta");
    if ((rc = sesp_set_state(g_job.ctx, g_job.pos.data(), g_job.vel.data(), g_job.acc.data(), eta)))
        return engine_fail(rc, "sesp_set_state");
    return SESP_OK;
}

int sesp_cmn_status(void) { return g_job.status; }

void init_accel_(int *) { report("init_accel", do_init_accel()); }
void move_surfactant_a_(int *) { report("move_surfactant_a", do_move_a()); }
void move_w1_a_(int *) { report("move_w1_a", check_order(1, "move_w1_a")); }
void move_w2_a_(int *, int *) { report("move_w2_a", check_order(1, "move_w2_a")); }
void evalforces_(int *) { report("evalforces", do_force()); }
void move_surfactant_b_(int *) { report("move_surfactant_b", do_move_b()); }
void move_w1_b_(int *) { report("move_w1_b", check_order(3, "move_w1_b")); }
void move_w2_b_(int *) { report("move_w2_b", check_order(3, "move_w2_b")); }
void sesp_cmn_reload_(int *) { report("sesp_cmn_reload", sesp_cmn_reload()); }

}  // extern "C"
