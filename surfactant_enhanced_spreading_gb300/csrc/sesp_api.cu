// C ABI of the GB300 engine (declared in include/sesp.h): context, device
// state, host-side force-field tables and multipole translation operators,
// and the per-step launch sequence (captured into CUDA graphs by sesp_run).
#include <algorithm>
#include <chrono>
#include <atomic>
#include <thread>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "k_launch.cuh"

using namespace sesp;

namespace sesp {
// surfactant site LJ sigma (reduced) and epsilon (reduced), src/init_arrays.f90:314-474
void surf_lj(double *sgs, double *eps) {
    const double s_ahy = 2.6, e_ahy = 33.5, s_aox = 3.07, e_aox = 711.76, s_ome = 3.983, e_ome = 478.12;
    const double s_oox = 3.047, e_oox = 817.67, s_tme = 3.95, e_tme = 382.47, s_bsi = 3.385, e_bsi = 2448.0;
    const double s_box = 2.955, e_box = 849.3, s_bme = 3.786, e_bme = 753.2;
    const double S[NSURF] = {s_ahy, s_aox, s_ome, s_ome, s_oox, s_ome, s_ome, s_oox, s_ome, s_ome, s_oox, s_ome, s_ome, s_oox, s_ome,
                             s_tme, s_tme, s_bsi, s_bme, s_box, s_bsi, s_bme, s_bme, s_bme, s_box, s_bsi, s_bme, s_bme, s_bme};
    const double E[NSURF] = {e_ahy, e_aox, e_ome, e_ome, e_oox, e_ome, e_ome, e_oox, e_ome, e_ome, e_oox, e_ome, e_ome, e_oox, e_ome,
                             e_tme, e_tme, e_bsi, e_bme, e_box, e_bsi, e_bme, e_bme, e_bme, e_box, e_bsi, e_bme, e_bme, e_bme};
    for (int i = 0; i < NSURF; i++) { sgs[i] = S[i] / SIGMA; eps[i] = E[i] / EPSILON; }
}
}  // namespace sesp

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(SESP_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// ------------------------------------------------------------------ tables (src/init_arrays.f90)

double fact(int n) { double f = 1.0; for (int i = 2; i <= n; i++) f *= i; return f; }

Tables make_tables() {
    Tables T;
    memset(&T, 0, sizeof T);
    const double sigma = SIGMA, epsilon = EPSILON;
    const double pi180 = 4.0 * atan(1.0) / 180.0;
    const double hy = 1.00794, carbon = 12.011, oxygen = 15.9994, si = 28.0855;
    const double me = carbon + 2.0 * hy, methyl = carbon + 3.0 * hy;
    // masses (src/init_arrays.f90:266-312)
    const double ms[NSURF] = {hy, oxygen, me, me, oxygen, me, me, oxygen, me, me, oxygen, me, me, oxygen, me, me, me,
                              si, methyl, oxygen, si, methyl, methyl, methyl, oxygen, si, methyl, methyl, methyl};
    T.mass[0] = oxygen / oxygen;
    T.mass[1] = hy / oxygen;
    for (int i = 0; i < NSURF; i++) T.mass[2 + i] = ms[i] / oxygen;
    // charges (src/init_arrays.f90:340-474)
    const double qs[NSURF] = {0.435, -0.700, 0.265, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29,
                              0.0, 0.0, 0.3, 0.0, -0.3, 0.15, 0.0, 0.0, 0.0, -0.3, 0.15, 0.0, 0.0, 0.0};
    T.q[0] = -0.8476;
    T.q[1] = 0.4238;
    for (int i = 0; i < NSURF; i++) T.q[2 + i] = qs[i];
    // surfactant constraints (src/init_arrays.f90:229-264, 509-565)
    for (int b = 0; b < 18; b++) { T.bi[b] = b; T.bj[b] = b + 1; }
    const int bx[10][2] = {{18, 20}, {20, 21}, {21, 22}, {21, 23}, {21, 24}, {18, 25}, {25, 26}, {26, 27}, {26, 28}, {26, 29}};
    for (int b = 0; b < 10; b++) { T.bi[18 + b] = bx[b][0] - 1; T.bj[18 + b] = bx[b][1] - 1; }
    const double bl[NBOND] = {0.945, 1.430, 1.516, 1.410, 1.410, 1.516, 1.410, 1.410, 1.516, 1.410, 1.410, 1.516, 1.410, 1.410,
                              1.516, 1.540, 1.88, 1.88, 1.60, 1.60, 1.88, 1.88, 1.88, 1.60, 1.60, 1.88, 1.88, 1.88};
    for (int b = 0; b < NBOND; b++) T.dsqs[b] = bl[b] * bl[b] / (sigma * sigma);
    double w[3] = {1.0, 2.0 * sin(109.47 * pi180 / 2.0), 1.0};
    for (int i = 0; i < 3; i++) T.dsqw[i] = w[i] * w[i] / (sigma * sigma);
    // angles (src/eval_valence.f90:13-95, src/init_arrays.f90:576-695)
    const int ang[NANGLE][3] = {{1, 2, 3}, {2, 3, 4}, {3, 4, 5}, {4, 5, 6}, {5, 6, 7}, {6, 7, 8}, {7, 8, 9}, {8, 9, 10}, {9, 10, 11},
                                {10, 11, 12}, {11, 12, 13}, {12, 13, 14}, {13, 14, 15}, {14, 15, 16}, {15, 16, 17}, {16, 17, 18},
                                {17, 18, 19}, {17, 18, 20}, {17, 18, 25}, {19, 18, 20}, {19, 18, 25}, {18, 25, 26}, {18, 20, 21},
                                {20, 21, 22}, {20, 21, 23}, {20, 21, 24}, {22, 21, 24}, {22, 21, 23}, {23, 21, 24}, {25, 26, 27},
                                {25, 26, 28}, {25, 26, 29}, {27, 26, 28}, {27, 26, 29}, {28, 26, 29}, {20, 18, 25}};
    const double th[NANGLE] = {108.5, 108.0, 108.0, 112.0, 108.0, 108.0, 112.0, 108.0, 108.0, 112.0, 108.0, 108.0, 112.0, 108.0,
                               114.0, 109.5, 109.5, 109.5, 109.5, 109.5, 109.5, 144.0, 144.0, 109.5, 109.5, 109.5, 109.5, 109.5,
                               109.5, 109.5, 109.5, 109.5, 109.5, 109.5, 109.5, 109.5};
    const double kth[NANGLE] = {519700, 519700, 519700, 519700, 519700, 519700, 519700, 519700, 519700, 519700, 519700, 519700,
                                519700, 519700, 519700, 519700, 418400, 418400, 418400, 418400, 418400, 118400, 118400, 418400,
                                418400, 418400, 418400, 418400, 418400, 418400, 418400, 418400, 418400, 418400, 418400, 791200};
    for (int i = 0; i < NANGLE; i++) {
        T.ai[i] = ang[i][0] - 1; T.aj[i] = ang[i][1] - 1; T.ak[i] = ang[i][2] - 1;
        T.th[i] = th[i] * pi180;
        T.rkth[i] = kth[i] / epsilon;
    }
    // dihedrals (src/eval_dihedral.f90:23-100, src/init_arrays.f90:697-836)
    const int dh[NDIH][4] = {{1, 2, 3, 4}, {2, 3, 4, 5}, {3, 4, 5, 6}, {4, 5, 6, 7}, {5, 6, 7, 8}, {6, 7, 8, 9}, {7, 8, 9, 10},
                             {8, 9, 10, 11}, {9, 10, 11, 12}, {10, 11, 12, 13}, {11, 12, 13, 14}, {12, 13, 14, 15},
                             {13, 14, 15, 16}, {14, 15, 16, 17}, {15, 16, 17, 18}, {16, 17, 18, 19}, {16, 17, 18, 20},
                             {16, 17, 18, 25}, {17, 18, 20, 21}, {17, 18, 25, 26}, {19, 18, 20, 21}, {19, 18, 25, 26},
                             {18, 20, 21, 22}, {18, 20, 21, 23}, {18, 20, 21, 24}, {18, 25, 26, 27}, {18, 25, 26, 28},
                             {18, 25, 26, 29}, {20, 18, 25, 26}, {21, 20, 18, 25}};
    const double al[3] = {3490.0, -486.0, 3130.0}, ommo[3] = {2940.0, -888.0, 12810.0};
    const double mmom[3] = {19860.0, -5853.0, 8956.0}, tr[3] = {5903.8, -1134.0, 13159.0};
    const double *cf[18] = {al, ommo, mmom, mmom, ommo, mmom, mmom, ommo, mmom, mmom, ommo, mmom, mmom, ommo, tr, tr, tr, tr};
    for (int i = 0; i < NDIH; i++) {
        T.di[i] = dh[i][0] - 1; T.dj[i] = dh[i][1] - 1; T.dk[i] = dh[i][2] - 1; T.dl[i] = dh[i][3] - 1;
        if (i < 18) {
            T.dva[i] = cf[i][0] / 2.0 / epsilon; T.dvb[i] = cf[i][1] / 2.0 / epsilon; T.dvc[i] = cf[i][2] / 2.0 / epsilon;
        } else {
            T.dva[i] = 3770.0 / epsilon; T.dvb[i] = 0.0; T.dvc[i] = 0.0;
        }
    }
    // intramolecular listed pairs (src/init_arrays.f90:127-220)
    const int sp[NSELF][2] = {{16, 21}, {16, 22}, {16, 23}, {16, 24}, {16, 26}, {16, 27}, {16, 28}, {16, 29}, {17, 22}, {17, 23},
                              {17, 24}, {17, 27}, {17, 28}, {17, 29}, {19, 22}, {19, 23}, {19, 24}, {19, 27}, {19, 28}, {19, 29},
                              {20, 27}, {20, 28}, {20, 29}, {21, 26}, {21, 27}, {21, 28}, {21, 29}, {22, 25}, {22, 26}, {22, 27},
                              {22, 28}, {22, 29}, {23, 25}, {23, 26}, {23, 27}, {23, 28}, {23, 29}, {24, 25}, {24, 26}, {24, 27},
                              {24, 28}, {24, 29}};
    for (int k = 0; k < NSELF; k++) { T.si[k] = sp[k][0] - 1; T.sj[k] = sp[k][1] - 1; }
    // graphite (src/eval_graphite.f90:10-11, src/init_arrays.f90:512-515)
    double sgs[NSURF], eps[NSURF];
    surf_lj(sgs, eps);
    for (int i = 0; i < NSURF; i++) {
        double s = (3.19 / sigma + sgs[i]) / 2.0;
        T.sgcs6[i] = s * s * s * s * s * s;
        T.epcs[i] = sqrt((392.0 / epsilon) * eps[i]);
    }
    double sw = 3.19 / sigma;
    T.sgcw6 = sw * sw * sw * sw * sw * sw;
    T.epcw = 392.0 / epsilon;
    for (int n = 0; n <= P; n++)
        for (int m = -n; m <= n; m++) T.rfctr[n * (n + 1) + m] = sqrt(fact(n - abs(m)) / fact(n + abs(m)));
    for (int k = 0; k < LP; k++) T.rfctr32[k] = (float)T.rfctr[k];
    return T;
}

// The configuration preset's force field (the benchmark configurations'
// water and chains, see SESP_PRESET_CONFIG in sesp.h), in reduced units:
// per-kind charges, masses, LJ sigma / epsilon and the chains' bonded
// constants.  Kinds: 0 water O, 1 water H, 2 + b bead b of a chain.
struct CfgField {
    double q[NTYPE], mass[NTYPE], sg[NTYPE], ep[NTYPE];
    ChainTables ch;
};
CfgField make_cfg_field() {
    CfgField F;
    memset(&F, 0, sizeof F);
    const double sig = SIGMA, eps = EPSILON, kj = 1000.0 / eps;
    const double mO = 15.9994, mH = 1.00794;
    const double pi180 = 4.0 * atan(1.0) / 180.0;
    F.mass[0] = 1.0; F.mass[1] = mH / mO;
    F.q[0] = -0.82; F.q[1] = 0.41;
    // head beads 1-4 (charges summing to zero), then the CH2 tail
    const double hm[4] = {15.035, 15.9994, 14.027, 15.9994}, hq[4] = {0.40, -0.60, 0.60, -0.40};
    const double hs[4] = {3.75, 2.80, 3.95, 2.80}, he[4] = {0.815, 0.457, 0.382, 0.457};
    F.sg[0] = 3.166 / sig; F.ep[0] = 0.650 * kj;
    for (int b = 0; b < NCH; b++) {
        const int t = 2 + b;
        F.mass[t] = (b < 4 ? hm[b] : 14.027) / mO;
        F.q[t] = b < 4 ? hq[b] : 0.0;
        F.sg[t] = (b < 4 ? hs[b] : 3.9) / sig;
        F.ep[t] = (b < 4 ? he[b] : 0.38) * kj;
    }
    F.ch.kb = 2000.0 * kj * sig * sig;   // 2000 kJ/mol/A^2
    F.ch.r0 = 1.53 / sig;
    F.ch.kth = 519.7 * kj;               // per rad^2
    F.ch.th0 = 112.0 * pi180;
    F.ch.dva = 2951.7 / eps;
    F.ch.dvb = -566.9 / eps;
    F.ch.dvc = 6579.0 / eps;
    return F;
}
// carbon LJ of the configuration preset: sigma 3.4 A, epsilon 0.23 kJ/mol
constexpr double CFG_SG_C = 3.4 / SIGMA, CFG_EP_C = 0.23 * (1000.0 / EPSILON);

}  // namespace


namespace {

// per site kind (sqrt(48 eps), sigma / 2) for the FP32 pair kernel, which
// combines them by the Lorentz-Berthelot rule of src/init_arrays.f90:476-502:
// 48 eps_ij = sqrt(48 eps_i) sqrt(48 eps_j), sigma_ij = sigma_i/2 + sigma_j/2
// contribution table of the intramolecular kernel: term slots per site.
// Layout (matches IntraMap in k_force.cu): short off[30], short list[852],
// uchar pa[312], uchar pb[312].  Slots: angle a -> 3a + {i, vertex, k};
// dihedral i -> 108 + 4i + {i, j, k, l}; pair q -> 228 + 2q + {a, b}.
std::vector<unsigned char> make_intra_map(const Tables &T) {
    const int npair = 270 + NSELF, nslot = NANGLE * 3 + NDIH * 4 + npair * 2;
    std::vector<int> pa, pb;
    for (int j = 0; j < 15; j++)
        for (int k = j + 4; k < NSURF; k++) { pa.push_back(j); pb.push_back(k); }
    for (int k = 0; k < NSELF; k++) { pa.push_back(T.si[k]); pb.push_back(T.sj[k]); }
    std::vector<std::vector<short>> per(NSURF);
    for (int a = 0; a < NANGLE; a++) {
        per[T.ai[a]].push_back((short)(3 * a)); per[T.aj[a]].push_back((short)(3 * a + 1)); per[T.ak[a]].push_back((short)(3 * a + 2));
    }
    for (int i = 0; i < NDIH; i++) {
        int b = NANGLE * 3 + 4 * i;
        per[T.di[i]].push_back((short)b); per[T.dj[i]].push_back((short)(b + 1));
        per[T.dk[i]].push_back((short)(b + 2)); per[T.dl[i]].push_back((short)(b + 3));
    }
    for (int q = 0; q < npair; q++) {
        int b = NANGLE * 3 + NDIH * 4 + 2 * q;
        per[pa[q]].push_back((short)b); per[pb[q]].push_back((short)(b + 1));
    }
    std::vector<short> off(NSURF + 1, 0), list;
    for (int s = 0; s < NSURF; s++) { off[s] = (short)list.size(); for (short v : per[s]) list.push_back(v); }
    off[NSURF] = (short)list.size();
    std::vector<unsigned char> out(intra_map_size(), 0);
    memcpy(out.data(), off.data(), sizeof(short) * (NSURF + 1));
    memcpy(out.data() + sizeof(short) * (NSURF + 1), list.data(), sizeof(short) * nslot);
    size_t o = sizeof(short) * (NSURF + 1 + nslot);
    for (int q = 0; q < npair; q++) { out[o + q] = (unsigned char)pa[q]; out[o + npair + q] = (unsigned char)pb[q]; }
    return out;
}

// LJ pair table (48 eps sg6, sg6) over the 31 site kinds; zero where the
// reference adds no LJ (water H with anything)
std::vector<double2> make_lj_table() {
    double sgs[NSURF], eps[NSURF];
    surf_lj(sgs, eps);
    std::vector<double2> t(NTYPE * NTYPE, make_double2(0.0, 0.0));
    auto sg = [&](int k) { return k == 0 ? 1.0 : sgs[k - 2]; };
    auto ep = [&](int k) { return k == 0 ? 1.0 : eps[k - 2]; };
    for (int a = 0; a < NTYPE; a++)
        for (int b = 0; b < NTYPE; b++) {
            if (a == 1 || b == 1) continue;
            double s = (sg(a) + sg(b)) / 2.0;
            double s6 = s * s * s * s * s * s;
            double e = sqrt(ep(a) * ep(b));
            t[a * NTYPE + b] = make_double2(48.0 * e * s6, s6);
        }
    return t;
}

// the configuration preset's LJ pair table, Lorentz-Berthelot over its kinds
std::vector<double2> make_lj_table_cfg(const CfgField &F) {
    std::vector<double2> t(NTYPE * NTYPE, make_double2(0.0, 0.0));
    for (int a = 0; a < 2 + NCH; a++)
        for (int b = 0; b < 2 + NCH; b++) {
            if (a == 1 || b == 1) continue;
            const double s = (F.sg[a] + F.sg[b]) / 2.0, s2 = s * s, s6 = s2 * s2 * s2;
            t[a * NTYPE + b] = make_double2(48.0 * sqrt(F.ep[a] * F.ep[b]) * s6, s6);
        }
    return t;
}

// per-kind charge, mass and graphite (eps, sg^6) of either force field
void kind_tables(int preset, std::vector<double> &q, std::vector<double> &mass, std::vector<double2> &gr) {
    q.assign(NTYPE, 0.0); mass.assign(NTYPE, 1.0); gr.assign(NTYPE, make_double2(0.0, 0.0));
    if (preset == SESP_PRESET_CONFIG) {
        const CfgField F = make_cfg_field();
        for (int k = 0; k < 2 + NCH; k++) {
            q[k] = F.q[k];
            mass[k] = F.mass[k];
            if (k == 1) continue;
            const double s = (F.sg[k] + CFG_SG_C) / 2.0, s2 = s * s, s6 = s2 * s2 * s2;
            gr[k] = make_double2(sqrt(F.ep[k] * CFG_EP_C), s6);
        }
        return;
    }
    const Tables T = make_tables();
    for (int k = 0; k < NTYPE; k++) { q[k] = T.q[k]; mass[k] = T.mass[k]; }
    gr[0] = make_double2(T.epcw, T.sgcw6);
    for (int i = 0; i < NSURF; i++) gr[2 + i] = make_double2(T.epcs[i], T.sgcs6[i]);
}

// ------------------------------------------------------------------ translation operators (src/ifma.f90)

double legendre(int l, int m, double x) {
    if (l == -1 && m == 0) return 1.0;
    if (m > l || l < 0) return 0.0;
    double pmm = 1.0;
    if (m > 0) {
        double s = sqrt((1.0 - x) * (1.0 + x)), f = 1.0;
        for (int i = 1; i <= m; i++) { pmm = -pmm * f * s; f += 2.0; }
    }
    if (l == m) return pmm;
    double p1 = x * (2 * m + 1) * pmm;
    if (l == m + 1) return p1;
    double p0 = pmm, pl = 0.0;
    for (int ll = m + 2; ll <= l; ll++) { pl = (x * (2 * ll - 1) * p1 - (ll + m - 1) * p0) / (ll - m); p0 = p1; p1 = pl; }
    return pl;
}
std::complex<double> Ylm(int n, int m, double al, double be) {
    int am = abs(m);
    return sqrt(fact(n - am) / fact(n + am)) * legendre(n, am, cos(al)) * std::complex<double>(cos(m * be), sin(m * be));
}
double sgn(int n) { return (n % 2 == 0) ? 1.0 : -1.0; }
double rAnm(int n, int m) { return sgn(n) / sqrt(fact(n - m) * fact(n + m)); }
double iIkm1(int k, int m) { return sgn(abs((abs(k) - abs(m) - abs(k - m)) / 2)); }
double iIkm2(int k, int m) { return sgn(abs((abs(k - m) - abs(k) - abs(m)) / 2)); }
double iIkm3(int k, int m) { return sgn(abs((abs(m) - abs(m - k) - abs(k)) / 2)); }
int oidx(int j, int k) { return j * (j + 1) / 2 + k; }
int cidx(int n, int m) { return n * (n + 1) + m; }
void sph(double x, double y, double z, double &rho, double &al, double &be) {
    rho = sqrt(x * x + y * y + z * z);
    al = acos(z / rho);
    be = atan2(y, x);
}

// M2L factors (src/computeLjk4.f90:134-158): the operator entry for output
// (j,k) and input (n,m) at source - target vector d is
//   iIkm2(k,m) rAnm(j,k) rAnm(n,m) / (sgn(n) rAnm(j+n,m-k)) * Y(j+n,m-k) / rho^(j+n+1);
// the first factor is the same for every offset (m2l_coef), the second is
// H_{j+n}^{m-k} (harm_m2l stores l = 0..8, q = 0..l; H_l^{-q} = conj(H_l^q)).
void harm_m2l(double x, double y, double z, double2 *h) {
    double rho, al, be;
    sph(x, y, z, rho, al, be);
    for (int l = 0; l <= 2 * P; l++)
        for (int q = 0; q <= l; q++) {
            std::complex<double> c = Ylm(l, q, al, be) / pow(rho, l + 1);
            h[l * (l + 1) / 2 + q] = make_double2(c.real(), c.imag());
        }
}
void m2l_coef(double *cf) {
    for (int j = 0; j <= P; j++)
        for (int k = 0; k <= j; k++)
            for (int n = 0; n <= P; n++)
                for (int m = -n; m <= n; m++)
                    cf[oidx(j, k) * LP + cidx(n, m)] =
                        iIkm2(k, m) * rAnm(j, k) * rAnm(n, m) / (sgn(n) * rAnm(j + n, m - k));
}
// Real form of the M2L operator at one offset (h: its 45 H_l^q).  With
// O_n^-m = conj(O_n^m) the complex 15 x 25 operator T acts on the 25 real
// components of a multipole and gives the 25 real components of the local
// expansion (Im L_j^0 vanishes and is dropped): for m > 0, with
// T = T[(j,k),(n,m)] and T' = T[(j,k),(n,-m)],
//   Re L += (Re T + Re T') Re O + (Im T' - Im T) Im O,
//   Im L += (Im T + Im T') Re O + (Re T - Re T') Im O.
// rop is [input 25][output, padded to M2C_LD].
void m2l_real(const double *cf, const double2 *h, double *rop) {
    for (int i = 0; i < LP * M2C_LD; i++) rop[i] = 0.0;
    auto op = [&](int j, int k, int n, int m) {
        const int l = j + n, q = m - k;
        const double c = cf[oidx(j, k) * LP + cidx(n, m)];
        const double2 hv = h[l * (l + 1) / 2 + abs(q)];
        return make_double2(c * hv.x, (q < 0 ? -c : c) * hv.y);
    };
    for (int j = 0; j <= P; j++)
        for (int k = 0; k <= j; k++) {
            const int ore = oidx(j, k), oim = k > 0 ? LPH + ore - (j + 1) : -1;
            for (int n = 0; n <= P; n++)
                for (int m = 0; m <= n; m++) {
                    const int ire = oidx(n, m), iim = m > 0 ? LPH + ire - (n + 1) : -1;
                    const double2 t = op(j, k, n, m);
                    if (m == 0) {
                        rop[ire * M2C_LD + ore] += t.x;
                        if (oim >= 0) rop[ire * M2C_LD + oim] += t.y;
                        continue;
                    }
                    const double2 u = op(j, k, n, -m);
                    rop[ire * M2C_LD + ore] += t.x + u.x;
                    rop[iim * M2C_LD + ore] += u.y - t.y;
                    if (oim >= 0) {
                        rop[ire * M2C_LD + oim] += t.y + u.y;
                        rop[iim * M2C_LD + oim] += t.x - u.x;
                    }
                }
        }
}
// M2M operator at child - parent vector d, src/computeOnm3.f90:51-81
void op_m2m(double x, double y, double z, double2 *op) {
    double rho, al, be;
    sph(x, y, z, rho, al, be);
    for (int i = 0; i < LPH * LP; i++) op[i] = make_double2(0.0, 0.0);
    for (int j = 0; j <= P; j++)
        for (int k = 0; k <= j; k++)
            for (int n = 0; n <= j; n++)
                for (int m = -n; m <= n; m++) {
                    if (j - n - abs(k - m) < 0) continue;
                    double rt = iIkm1(k, m) * rAnm(n, m) * rAnm(j - n, k - m) * pow(rho, n) / rAnm(j, k);
                    std::complex<double> c = rt * Ylm(n, -m, al, be);
                    double2 &o = op[oidx(j, k) * LP + cidx(j - n, k - m)];
                    o.x += c.real(); o.y += c.imag();
                }
}
// L2L operator at parent - child vector d, src/shiftLjk3.f90:46-76
void op_l2l(double x, double y, double z, double2 *op) {
    double rho, al, be;
    sph(x, y, z, rho, al, be);
    for (int i = 0; i < LPH * LP; i++) op[i] = make_double2(0.0, 0.0);
    for (int j = 0; j <= P; j++)
        for (int k = 0; k <= j; k++)
            for (int n = 0; n <= P; n++)
                for (int m = -n; m <= n; m++) {
                    if (n - j - abs(m - k) < 0) continue;
                    double rt = iIkm3(k, m) * rAnm(n - j, m - k) * rAnm(j, k) * pow(rho, n - j) / (sgn(n + j) * rAnm(n, m));
                    std::complex<double> c = rt * Ylm(n - j, m - k, al, be);
                    double2 &o = op[oidx(j, k) * LP + cidx(n, m)];
                    o.x += c.real(); o.y += c.imag();
                }
}

}  // namespace

// ------------------------------------------------------------------ context

struct sesp_ctx {
    sesp_params p;
    cudaStream_t st = nullptr;
    bool uploaded = false, have_force = false;
    int nrep = 0, nsite = 0, nmol = 0, ncell = 0, n3 = 0, n2 = 0, nwm = 0, nsm = 0;
    int3 d2 = {1, 1, 1};   // largest L2 offset per axis of the far field's H table
    int chains = 0;        // configuration preset: surfactants are 12-bead flexible chains
    int ssite = NSURF;     // sites per surfactant
    std::vector<Rep> reps;
    Dev d;
    int *wmols = nullptr, *smols = nullptr;
    std::vector<void *> allocs;
    size_t bytes = 0;
    int64_t steps = 0;
    // graphs of one step with / without a rebuild
    cudaGraphExec_t g_step[2] = {nullptr, nullptr};
    // side stream of a step: the graphite and intramolecular terms run there,
    // beside the far-field build and the pair field (fork after the gather,
    // join before the site forces)
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_eta = nullptr;
    NearShape near = {64, 0};   // pair-field launch shape (autotuned or set; results do not depend on it)
    ConstraintShape cshape = {0, 4, 1};   // constraint halves of the mixed paths (likewise)
    int n_sm = 0;               // streaming multiprocessors of the device
    // SESP_SYNC_CHECK set in the environment: every kernel family is followed
    // by a stream synchronisation, and the first failing family is named
    bool sync_check = false;
    const char *fault = nullptr;
    // timing
    bool timing = false;
    cudaEvent_t ev[16];
    double t_acc[8] = {0};
    int64_t t_n[8] = {0};
    bool t_rec[8] = {false};
    // host copies for downloads
    std::vector<double> h3;
};

namespace {

template <typename T>
int dalloc(sesp_ctx *c, T **p, size_t n) {
    void *q = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess) return fail(SESP_ENOMEM, "cudaMalloc of %zu bytes: %s", n * sizeof(T), cudaGetErrorString(e));
    cudaMemsetAsync(q, 0, n * sizeof(T), c->st);
    c->allocs.push_back(q);
    c->bytes += n * sizeof(T);
    *p = (T *)q;
    return 0;
}

// work items of the pair field: at most 9 rows x ceil(sites / 32) chunks per cell
size_t near_items_max(int nsite, int ncell) { return 9 * ((size_t)nsite / 32 + ncell) + 16; }

void free_state(sesp_ctx *c) {
    for (auto &g : c->g_step)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (void *q : c->allocs) cudaFree(q);
    c->allocs.clear();
    c->bytes = 0;
    c->uploaded = false;
    c->have_force = false;
}

// cell centres along one axis of a replica: rcen4 of the owning rank,
// src/init_box_dimensions.f90:40-42 and :79-94
void axis_centres(const Rep &r, int a, std::vector<double> &out) {
    double b = (double)r.nr[a];
    for (int k = 0; k < r.nc[a]; k++) {
        int rk = k / 4, i = k % 4 + 1;
        double c2 = r.rsd[a] * (rk + 1) / b - r.rhs[a] - r.rsd[a] / b / 2.0;
        out.push_back(4.0 * RS * i / 4.0 - 2.0 * RS - 4.0 * RS / 8.0 + c2);
    }
}

// pair-field arithmetic: 0 FP64, 1 FP32, 2 FP32 with compensated sums
int near_mode(const sesp_ctx *c) {
    return c->p.precision == SESP_PLAIN_FP64 ? 0 : (c->p.precision == SESP_MIXED_COMP ? 2 : 1);
}

int check_ctx(sesp_ctx *c, bool need_state) {
    if (!c) return fail(SESP_EINVAL, "null context");
    if (need_state && !c->uploaded) return fail(SESP_ESTATE, "no state uploaded");
    return 0;
}

int set_device(sesp_ctx *c) {
    CK(cudaSetDevice(c->p.device));
    return 0;
}

}  // namespace

// ------------------------------------------------------------------ sequences

namespace {

void tstart(sesp_ctx *c, int k) {
    if (!c->timing) return;
    cudaEventRecord(c->ev[2 * k], c->st);
    c->t_rec[k] = true;
}
void tstop(sesp_ctx *c, int k) { if (c->timing) cudaEventRecord(c->ev[2 * k + 1], c->st); }
// only families recorded since the last collection are read
void tcollect(sesp_ctx *c, int k) {
    if (!c->timing || !c->t_rec[k]) return;
    c->t_rec[k] = false;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[2 * k], c->ev[2 * k + 1]) == cudaSuccess) { c->t_acc[k] += ms; c->t_n[k]++; }
    else cudaGetLastError();
}

// with sync_check, wait for the family just launched and remember the first that failed
void family(sesp_ctx *c, const char *name) {
    if (!c->sync_check || c->fault) return;
    if (cudaStreamSynchronize(c->st) != cudaSuccess) c->fault = name;
}

void seq_force(sesp_ctx *c, int rebuild, int terms) {
    const Dev &d = c->d;
    const int mixed = c->p.precision != SESP_PLAIN_FP64;
    if (rebuild) {
        tstart(c, 5);
        cudaMemsetAsync(d.ccount, 0, sizeof(int) * c->ncell, c->st);
        launch_locate(d, c->nmol, c->smols, c->nsm * c->ssite, c->chains, c->nsite, c->st);
        family(c, "locate");
        launch_sort(d, c->nsite, c->ncell, c->st);
        family(c, "cell sort");
        launch_near_items(d, c->ncell, (int)near_items_max(c->nsite, c->ncell), c->near.tile, c->st);
        family(c, "near-field items");
        launch_isub(d, c->nsm * c->ssite, c->smols, c->chains, c->st);
        family(c, "isub");
        launch_graphite_list(d, c->nsite, c->st);
        family(c, "graphite list");
        if (mixed) launch_water_order(d, c->wmols, c->nwm, c->st);
        family(c, "water order");
        tstop(c, 5);
    }
    launch_gather(d, c->nsite, c->ncell, mixed, c->st);
    family(c, "gather");
    // graphite and intramolecular terms into the side forces (fside), on the
    // side stream beside the far-field build and the pair field on the mixed
    // paths; in order on the main stream on the plain path (its FP64 pair
    // field beside them ran a batched step at 581 ms against 259 ms in order)
    // and when kernels are timed or checked one by one
    const bool fork = mixed && !c->timing && !c->sync_check;
    if (fork) {
        cudaEventRecord(c->ev_fork, c->st);
        cudaStreamWaitEvent(c->st2, c->ev_fork, 0);
        launch_graphite(d, terms, mixed, c->st2);
        launch_intra(d, c->smols, c->nsm, terms, mixed, c->chains, c->st2);
        cudaEventRecord(c->ev_join, c->st2);
    }
    if (rebuild) {
        tstart(c, 6);
        launch_fma_build(d, c->ncell, c->n3, c->n2, mixed, c->d2, c->st);
        family(c, "far-field build");
        tstop(c, 6);
    }
    tstart(c, 0);
    launch_near(d, c->ncell, c->nsite, near_mode(c), terms, c->near, c->st, false, c->chains);
    family(c, "near field");
    tstop(c, 0);
    tstart(c, 4);
    if (fork) {
        cudaStreamWaitEvent(c->st, c->ev_join, 0);
    } else {
        launch_graphite(d, terms, mixed, c->st);
        family(c, "graphite");
        launch_intra(d, c->smols, c->nsm, terms, mixed, c->chains, c->st);
        family(c, "intramolecular");
    }
    launch_site_forces(d, c->nsite, terms, mixed, c->st);
    family(c, "site forces");
    tstop(c, 4);
}

// fork_eta: the eta update goes to the side stream, beside the next force
// call, which joins it before the site forces (a step's sequence on the
// mixed paths); otherwise it follows the SHAKE half on the main stream
void seq_move_a(sesp_ctx *c, bool fork_eta = false) {
    tstart(c, 2);
    launch_move_a(c->d, c->wmols, c->nwm, c->smols, c->nsm, c->nrep, c->nmol, c->nsite, c->p.shake_tol, c->p.shake_maxit,
                  c->p.precision, c->cshape, c->chains, c->st);
    if (fork_eta) {
        cudaEventRecord(c->ev_eta, c->st);
        cudaStreamWaitEvent(c->st2, c->ev_eta, 0);
        launch_eta(c->d, c->nrep, c->st2);
    } else {
        launch_eta(c->d, c->nrep, c->st);
    }
    family(c, "move_a");
    tstop(c, 2);
}
void seq_move_b(sesp_ctx *c) {
    tstart(c, 3);
    launch_move_b(c->d, c->wmols, c->nwm, c->smols, c->nsm, c->nmol, c->nsite, c->p.shake_tol, c->p.shake_maxit,
                  c->p.precision, c->cshape, c->chains, c->st);
    family(c, "move_b");
    tstop(c, 3);
}

void collect_all(sesp_ctx *c) {
    if (!c->timing) return;
    cudaStreamSynchronize(c->st);
    for (int k = 0; k < 7; k++) tcollect(c, k);
}

}  // namespace

// ------------------------------------------------------------------ ABI

extern "C" {

int sesp_abi_version(void) { return SESP_ABI_VERSION; }

int sesp_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return SESP_EINVAL;
    snprintf(buf, len, "%s", g_err.c_str());
    return 0;
}

int sesp_default_params(sesp_params *p) {
    if (!p) return fail(SESP_EINVAL, "null params");
    memset(p, 0, sizeof *p);
    p->n_cells[0] = p->n_cells[1] = p->n_cells[2] = 12;
    p->precision = SESP_PLAIN_FP64;
    p->rebuild_interval = 10;
    p->graphite_on = 1;
    p->tr = 3.81087;
    p->tau_steps = 7.5;
    p->shake_tol = 0.0001;
    p->shake_maxit = 100;
    p->device = 0;
    p->max_cell_sites = 0;
    p->preset = SESP_PRESET_REFERENCE;
    return 0;
}

int sesp_default_config_params(sesp_params *p) {
    if (int e = sesp_default_params(p)) return e;
    p->n_cells[0] = p->n_cells[1] = p->n_cells[2] = 8;
    p->preset = SESP_PRESET_CONFIG;
    p->tr = 8.314462618 * 300.0 / EPSILON;   // 300 K
    p->tau_steps = 0.1e-12 / 2.0e-15;         // 0.1 ps of 2 fs steps
    p->shake_tol = 1e-8;
    p->shake_maxit = 100;
    return 0;
}

int sesp_create(const sesp_params *p, sesp_ctx **out) {
    if (!p || !out) return fail(SESP_EINVAL, "null argument");
    for (int a = 0; a < 3; a++)
        if (p->n_cells[a] <= 0 || p->n_cells[a] % 4) return fail(SESP_EINVAL, "n_cells must be positive multiples of 4");
    if (p->precision != SESP_PLAIN_FP64 && p->precision != SESP_MIXED && p->precision != SESP_MIXED_FP32C &&
        p->precision != SESP_MIXED_COMP)
        return fail(SESP_EINVAL, "unknown precision");
    if (p->rebuild_interval <= 0) return fail(SESP_EINVAL, "rebuild_interval must be positive");
    if (p->preset != SESP_PRESET_REFERENCE && p->preset != SESP_PRESET_CONFIG) return fail(SESP_EINVAL, "unknown preset %d", p->preset);
    if (p->preset == SESP_PRESET_CONFIG && (p->n_cells[0] < 8 || p->n_cells[1] < 8))
        return fail(SESP_EINVAL, "the periodic preset needs at least 8 cells in x and y");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(SESP_ECUDA, "no CUDA device");
    if (p->device < 0 || p->device >= ndev) return fail(SESP_EINVAL, "device %d out of range", p->device);
    sesp_ctx *c = new sesp_ctx();
    c->p = *p;
    c->chains = p->preset == SESP_PRESET_CONFIG;
    c->ssite = c->chains ? NCH : NSURF;
    if (set_device(c)) { delete c; return SESP_ECUDA; }
    if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_eta, cudaEventDisableTiming) != cudaSuccess) {
        delete c;
        return fail(SESP_ECUDA, "stream");
    }
    for (int k = 0; k < 16; k++) cudaEventCreate(&c->ev[k]);
    init_force_kernels();
    init_constraint_kernels();
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, dev);
        const int mixed = c->p.precision != SESP_PLAIN_FP64;
        c->near.tile = 64;   // 128 (mixed paths) only where the autotuner measures it faster
        c->near.grid = c->n_sm * near_max_ctas_per_sm(near_mode(c), c->near.tile, c->chains);
        c->cshape.grid = c->n_sm;
    }
    c->sync_check = getenv("SESP_SYNC_CHECK") != nullptr;
    Tables T = make_tables();
    {
        std::vector<unsigned char> map = make_intra_map(T);
        upload_intra_map(map.data(), c->st);
    }
    upload_tables_exact(T, c->st);
    upload_tables_force(T, c->st);
    upload_chain_tables(make_cfg_field().ch, c->st);
    if (!upload_tables_fast(T, c->st)) { delete c; return fail(SESP_ECUDA, "constraint table upload"); }
    if (cudaStreamSynchronize(c->st) != cudaSuccess) { delete c; return fail(SESP_ECUDA, "table upload"); }
    *out = c;
    return 0;
}

int sesp_destroy(sesp_ctx *c) {
    if (!c) return 0;
    cudaSetDevice(c->p.device);
    cudaStreamSynchronize(c->st);
    free_state(c);
    for (int k = 0; k < 16; k++) cudaEventDestroy(c->ev[k]);
    cudaEventDestroy(c->ev_fork);
    cudaEventDestroy(c->ev_join);
    cudaEventDestroy(c->ev_eta);
    cudaStreamDestroy(c->st2);
    cudaStreamDestroy(c->st);
    delete c;
    return 0;
}

}  // extern "C"

namespace {

struct RepIn {
    int nw, ns, nc[3], ncarb;
    const double *pos, *vel, *carb;
};

// Lay out one or more replica systems back to back and upload them.
int upload_impl(sesp_ctx *c, const std::vector<RepIn> &in) {
    // SESP_TRACE_UPLOAD set: host time of each phase to stderr
    const bool trace = getenv("SESP_TRACE_UPLOAD") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) {
        if (!trace) return;
        cudaStreamSynchronize(c->st);
        const auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "sesp upload: %-22s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(now - t_last).count());
        t_last = now;
    };
    if (set_device(c)) return SESP_ECUDA;
    cudaStreamSynchronize(c->st);
    free_state(c);
    const int R = (int)in.size();
    c->reps.assign(R, Rep());
    int nsite = 0, nmol = 0, ncell = 0, n3 = 0, n2 = 0, naxis = 0, ncol = 0, nwm = 0, nsm = 0;
    int3 d2 = {1, 1, 1};
    const int per = c->chains;   // the configuration preset: periodic in x and y
    size_t npk4 = 0, npk3 = 0;
    for (int q = 0; q < R; q++) {
        const RepIn &ri = in[q];
        Rep &r = c->reps[q];
        memset(&r, 0, sizeof r);
        for (int a = 0; a < 3; a++) {
            if (ri.nc[a] <= 0 || ri.nc[a] % 4) return fail(SESP_EINVAL, "replica %d: cells must be positive multiples of 4", q);
            if (per && a < 2 && ri.nc[a] < 8) return fail(SESP_EINVAL, "replica %d: the periodic preset needs at least 8 cells in x and y", q);
            r.nc[a] = ri.nc[a];
            r.nr[a] = r.nc[a] / 4;
            r.rsd[a] = r.nc[a] * RS;
            r.rhs[a] = r.rsd[a] / 2.0;
            r.irsd[a] = 1.0 / r.rsd[a];
            // offsets of the shared L2 table (closed boxes; the periodic
            // preset has per-replica image-summed tables instead)
            int &dd = a == 0 ? d2.x : (a == 1 ? d2.y : d2.z);
            dd = std::max(dd, r.nr[a] - 1);
        }
        r.per = per;
        r.ssite = c->ssite;
        r.igz = -1;
        r.gymax = GYMAX;
        if (ri.nw < 0 || ri.ns < 0 || ri.nw + ri.ns == 0) return fail(SESP_EINVAL, "replica %d: empty system", q);
        if (!ri.pos) return fail(SESP_EINVAL, "replica %d: null positions", q);
        if (ri.ncarb < 0 || (ri.ncarb > 0 && !ri.carb)) return fail(SESP_EINVAL, "replica %d: bad carbons", q);
        r.nw = ri.nw; r.ns = ri.ns;
        r.nsite = 3 * ri.nw + c->ssite * ri.ns;
        r.nmol = ri.nw + ri.ns;
        r.graphite_on = c->p.graphite_on;
        int np = r.nsite, ncon = 3 * ri.nw + (c->chains ? 0 : NBOND) * ri.ns, df = 3 * np - ncon;
        r.ncon = ncon;
        double rlx = c->p.tau_steps * DT;
        r.pnh1 = DT / df / c->p.tr / (rlx * rlx);
        r.pnh2 = -2.0 * df * c->p.tr;
        r.site0 = nsite; r.mol0 = nmol; r.cell0 = ncell; r.l3_0 = n3; r.l2_0 = n2; r.axis0 = naxis; r.gcol0 = ncol;
        r.pk4 = (int)npk4; r.pk3 = (int)npk3;
        npk4 += (size_t)8 * LP * (r.nc[0] / 2 + 4) * (r.nc[1] / 2 + 4) * (r.nc[2] / 2 + 4);
        npk3 += (size_t)8 * LP * (r.nc[0] / 4 + 4) * (r.nc[1] / 4 + 4) * (r.nc[2] / 4 + 4);
        if (npk4 >= (1u << 31)) return fail(SESP_EINVAL, "too many cells");
        int cc = r.nc[0] * r.nc[1] * r.nc[2];
        nsite += r.nsite; nmol += r.nmol; ncell += cc; n3 += cc / 8; n2 += cc / 64;
        naxis += r.nc[0] + r.nc[1] + r.nc[2]; ncol += r.nc[0] * r.nc[1];
        nwm += ri.nw; nsm += ri.ns;
        for (int g = 0; g < r.nsite; g++)
            for (int a = 0; a < 3; a++) {
                double v = ri.pos[3 * g + a];
                if (per && a < 2) {   // periodic axes: any position a rebuild can wrap
                    if (!(fabs(v) < 1e8)) return fail(SESP_EINVAL, "replica %d: site %d position %g (axis %d)", q, g, v, a);
                } else if (!(v > -r.rhs[a] && v < r.rhs[a])) {
                    return fail(SESP_EINVAL, "replica %d: site %d outside the box (axis %d: %g)", q, g, a, v);
                }
            }
    }
    c->nrep = R; c->nsite = nsite; c->nmol = nmol; c->ncell = ncell; c->n3 = n3; c->n2 = n2;
    c->nwm = nwm; c->nsm = nsm; c->d2 = d2;
    Dev &d = c->d;
    memset(&d, 0, sizeof d);
    int N = nsite, M = nmol, C = ncell;
    d.nsite = N;
    int e = 0;
    double **a12[12] = {&d.x, &d.y, &d.z, &d.vx, &d.vy, &d.vz, &d.ax, &d.ay, &d.az, &d.fx, &d.fy, &d.fz};
    for (auto q : a12) if ((e = dalloc(c, q, N))) return e;
    lap("replica checks");
    if ((e = dalloc(c, &d.ptype, N)) || (e = dalloc(c, &d.smol, N)) || (e = dalloc(c, &d.mrep, M)) ||
        (e = dalloc(c, &d.mfirst, M)) || (e = dalloc(c, &d.mkind, M)) || (e = dalloc(c, &d.mkey, M)) ||
        (e = dalloc(c, &d.mw1, M)) || (e = dalloc(c, &d.ke, 2 * M)) || (e = dalloc(c, &d.mfail, M)) ||
        (e = dalloc(c, &d.rep, R)) || (e = dalloc(c, &d.eta, R)) || (e = dalloc(c, &d.crep, C)) ||
        (e = dalloc(c, &d.b3rep, n3)) || (e = dalloc(c, &d.b2rep, n2)) || (e = dalloc(c, &d.cstart, C + 1)) ||
        (e = dalloc(c, &d.ccount, C)) || (e = dalloc(c, &d.cfill, C)) || (e = dalloc(c, &d.sloc, N)) ||
        (e = dalloc(c, &d.sslot, N)) || (e = dalloc(c, &d.srt_site, N)) || (e = dalloc(c, &d.srt_pos, N)) ||
        (e = dalloc(c, &d.srt_pos32, N)) || (e = dalloc(c, &d.srt_meta, N)) || (e = dalloc(c, &d.srt_key, N)) ||
        (e = dalloc(c, &d.srt_xmask, N)) || (e = dalloc(c, &d.nf, 3 * (size_t)N)) ||
        (e = dalloc(c, &d.near_part, 27 * (size_t)N)) || (e = dalloc(c, &d.near_items, near_items_max(N, C))) ||
        (e = dalloc(c, &d.near_items_tmp, near_items_max(N, C))) || (e = dalloc(c, &d.near_cls, near_items_max(N, C))) ||
        (e = dalloc(c, &d.near_icount, C + 1)) || (e = dalloc(c, &d.near_ctl, 66)) ||
        (e = dalloc(c, &d.isub, (size_t)c->ssite * nsm)) || (e = dalloc(c, &d.O4, (size_t)LP * C)) ||
        (e = dalloc(c, &d.L4, (size_t)LP * C)) || (e = dalloc(c, &d.L4f, (size_t)LP * C)) ||
        (e = dalloc(c, &d.fside, 3 * (size_t)N)) || (e = dalloc(c, &d.stage, 12 * (size_t)N)) ||
        (e = dalloc(c, &d.O3, (size_t)LP * n3)) ||
        (e = dalloc(c, &d.L3, (size_t)LP * n3)) || (e = dalloc(c, &d.O2, (size_t)LP * n2)) ||
        (e = dalloc(c, &d.L2, (size_t)LP * n2)) || (e = dalloc(c, &d.counters, 8)) ||
        (e = dalloc(c, &d.ljt, NTYPE * NTYPE)) || (e = dalloc(c, &d.ljt32, NTYPE * NTYPE)) || (e = dalloc(c, &c->wmols, nwm)) || (e = dalloc(c, &c->smols, nsm)) ||
        (e = dalloc(c, &d.wlist_a, nwm)) || (e = dalloc(c, &d.wlist_b, nwm)) || (e = dalloc(c, &d.wsw_a, M)) ||
        (e = dalloc(c, &d.wsw_b, M)) || (e = dalloc(c, &d.cctl, 8)) || (e = dalloc(c, &d.wsort_off, 256)) ||
        (e = dalloc(c, &d.eta_part, 64 * (size_t)R)) || (e = dalloc(c, &d.eta_ctl, R)) ||
        (e = dalloc(c, &d.cnh, C)) || (e = dalloc(c, &d.tq, NTYPE)) || (e = dalloc(c, &d.tmass, NTYPE)) ||
        (e = dalloc(c, &d.tgr, NTYPE)) || (e = dalloc(c, &d.simg, N)) || (e = dalloc(c, &d.tbuf, (size_t)R * (1 + TEMP_SLICES))))
        return e;
    const int w2x = 2 * d2.x + 1, w2y = 2 * d2.y + 1, w2z = 2 * d2.z + 1;
    const size_t nh2 = (size_t)w2x * w2y * w2z * NHARM;
    lap("allocation");
    // real-form M2L at L4 and L3: work items of M2C_TILE targets of one parity
    // class, each split into M2C_GROUPS offset groups (a constant, so a
    // replica's sums do not depend on what else is batched with it)
    const int mixed = c->p.precision != SESP_PLAIN_FP64;
    const size_t rsz = mixed ? sizeof(float) : sizeof(double);
    std::vector<int4> m2c_items;
    for (int lev = 4; lev >= 3; lev--)
        for (int q = 0; q < R; q++) {
            const Rep &r = c->reps[q];
            const int div = lev == 4 ? 2 : 4;
            const int ncls = (r.nc[0] / div) * (r.nc[1] / div) * (r.nc[2] / div);
            for (int cls = 0; cls < 8; cls++)
                for (int t0 = 0; t0 < ncls; t0 += M2C_TILE)
                    m2c_items.push_back(make_int4(lev << 28 | q, cls, t0, std::min(M2C_TILE, ncls - t0)));
        }
    d.m2c_nitems = (int)m2c_items.size();
    d.m2c_groups = M2C_GROUPS;
    {
        char *p4 = nullptr, *p3 = nullptr, *q4 = nullptr, *q3 = nullptr, *o4 = nullptr, *o3 = nullptr;
        if ((e = dalloc(c, &o4, (size_t)343 * LP * M2C_LD * rsz)) || (e = dalloc(c, &o3, (size_t)343 * LP * M2C_LD * rsz)) ||
            (e = dalloc(c, &p4, npk4 * rsz)) || (e = dalloc(c, &p3, npk3 * rsz)) ||
            (e = dalloc(c, &q4, (size_t)d.m2c_groups * LP * C * rsz)) ||
            (e = dalloc(c, &q3, (size_t)d.m2c_groups * LP * n3 * rsz)) ||
            (e = dalloc(c, &d.m2c_items, m2c_items.size())) || (e = dalloc(c, &d.m2c_off, (size_t)8 * M2C_NOFF)))
            return e;
        d.rop4 = o4; d.rop3 = o3; d.pk4 = p4; d.pk3 = p3; d.part4 = q4; d.part3 = q3;
    }
    CK(cudaMemcpyAsync(d.m2c_items, m2c_items.data(), m2c_items.size() * sizeof(int4), cudaMemcpyHostToDevice, c->st));
    {
        // per parity class (bit a: odd cell index on axis a) the offsets of
        // the children of the parent's neighbours that are not adjacent
        std::vector<int> off;
        for (int cls = 0; cls < 8; cls++)
            for (int dz = -3; dz <= 3; dz++)
                for (int dy = -3; dy <= 3; dy++)
                    for (int dx = -3; dx <= 3; dx++) {
                        const int dd[3] = {dx, dy, dz};
                        bool ok = !(abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1);
                        for (int a = 0; a < 3; a++) {
                            const int par = (cls >> a) & 1;
                            ok = ok && dd[a] >= -2 - par && dd[a] <= 3 - par;
                        }
                        if (ok) off.push_back((dx + 3) + 7 * (dy + 3) + 49 * (dz + 3));
                    }
        if (off.size() != (size_t)8 * M2C_NOFF) return fail(SESP_EINVAL, "M2L offset lists");
        CK(cudaMemcpyAsync(d.m2c_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
    }
    if ((e = dalloc(c, &d.h_m2l2, nh2)) || (e = dalloc(c, &d.h32_m2l2, nh2)) ||
        (e = dalloc(c, &d.m2l_cf, (size_t)LPH * LP)) || (e = dalloc(c, &d.m2l_cf32, (size_t)LPH * LP)) ||
        (e = dalloc(c, &d.op_m2m43, (size_t)8 * LPH * LP)) || (e = dalloc(c, &d.op_m2m32, (size_t)8 * LPH * LP)) ||
        (e = dalloc(c, &d.op_l2l23, (size_t)8 * LPH * LP)) || (e = dalloc(c, &d.op_l2l34, (size_t)8 * LPH * LP)) ||
        (e = dalloc(c, &d.op32_m2m43, (size_t)8 * LPH * LP)) || (e = dalloc(c, &d.op32_m2m32, (size_t)8 * LPH * LP)) ||
        (e = dalloc(c, &d.op32_l2l23, (size_t)8 * LPH * LP)) || (e = dalloc(c, &d.op32_l2l34, (size_t)8 * LPH * LP)))
        return e;
    lap("M2L work items");
    // static per-site / per-molecule / per-box data
    std::vector<uint8_t> ptype(N);
    std::vector<int> smol(N), mrep(M), mfirst(M), mkind(M), wm, sm, crep(C), b3(n3), b2(n2);
    std::vector<double> axis, rcen2, sx(N), sy(N), sz(N), vxa(N, 0.0), vya(N, 0.0), vza(N, 0.0), eta0(R, 0.0);
    std::vector<int> gstart(1, 0);
    std::vector<double4> gpos;
    std::vector<float4> gpos32;   // relative to the column's (x, y) centre and the bottom cell layer's z centre
    std::vector<int> gbin;        // per column and group: GBIN + 1 bin starts (the last is the group's end)
    std::vector<float2> ggrp_z;   // per column and group: z range in the gpos32 frame
    double rcut = RC + sqrt(2.0) * RS / 2.0;
    rcut *= rcut;
    for (int q = 0; q < R; q++) {
        Rep &r = c->reps[q];
        const RepIn &ri = in[q];
        for (int m = 0; m < ri.nw; m++) {
            int gm = r.mol0 + m, g0 = r.site0 + 3 * m;
            mfirst[gm] = g0; mkind[gm] = 0; mrep[gm] = q; wm.push_back(gm);
            for (int t = 0; t < 3; t++) { ptype[g0 + t] = t == 0 ? 0 : 1; smol[g0 + t] = gm; }
        }
        for (int k = 0; k < ri.ns; k++) {
            int gm = r.mol0 + ri.nw + k, g0 = r.site0 + 3 * ri.nw + c->ssite * k;
            mfirst[gm] = g0; mkind[gm] = 1; mrep[gm] = q; sm.push_back(gm);
            for (int t = 0; t < c->ssite; t++) { ptype[g0 + t] = (uint8_t)(2 + t); smol[g0 + t] = gm; }
        }
        for (int g = 0; g < r.nsite; g++) {
            sx[r.site0 + g] = ri.pos[3 * g]; sy[r.site0 + g] = ri.pos[3 * g + 1]; sz[r.site0 + g] = ri.pos[3 * g + 2];
            if (ri.vel) { vxa[r.site0 + g] = ri.vel[3 * g]; vya[r.site0 + g] = ri.vel[3 * g + 1]; vza[r.site0 + g] = ri.vel[3 * g + 2]; }
        }
        int cc = r.nc[0] * r.nc[1] * r.nc[2];
        for (int k = 0; k < cc; k++) crep[r.cell0 + k] = q;
        for (int k = 0; k < cc / 8; k++) b3[r.l3_0 + k] = q;
        for (int k = 0; k < cc / 64; k++) b2[r.l2_0 + k] = q;
        size_t a0 = axis.size();
        for (int a = 0; a < 3; a++) {
            if (per)   // uniform cells from the lower face
                for (int k = 0; k < r.nc[a]; k++) axis.push_back(-r.rhs[a] + (k + 0.5) * RS);
            else
                axis_centres(r, a, axis);
        }
        for (int a = 0; a < 3; a++) {   // the reference's operation order (rcen2xtmp)
            const double b = (double)r.nr[a];
            for (int rk = 0; rk < r.nr[a]; rk++) rcen2.push_back(r.rsd[a] * (rk + 1) / b - r.rhs[a] - r.rsd[a] / b / 2.0);
        }
        // periodic preset: carbons binned by column; a column's list takes
        // its neighbours' carbons (and their images across the periodic
        // faces) within rc + half a cell diagonal + the 2 A list skin
        std::vector<int> cbin_start, cbin;
        double rcut_per = RC + sqrt(2.0) * RS / 2.0 + (RS - RC);
        if (per) {
            r.gymax = (float)rcut_per + 1e-3f;
            const int ncc = r.nc[0] * r.nc[1];
            cbin_start.assign(ncc + 1, 0);
            std::vector<int> bof(ri.ncarb);
            double ztop = -1e300;
            for (int k = 0; k < ri.ncarb; k++) {
                int bx = (int)floor((ri.carb[3 * k] + r.rhs[0]) / RS), by = (int)floor((ri.carb[3 * k + 1] + r.rhs[1]) / RS);
                bx = ((bx % r.nc[0]) + r.nc[0]) % r.nc[0];
                by = ((by % r.nc[1]) + r.nc[1]) % r.nc[1];
                bof[k] = bx + r.nc[0] * by;
                cbin_start[bof[k] + 1]++;
                ztop = std::max(ztop, ri.carb[3 * k + 2]);
            }
            for (int b = 0; b < ncc; b++) cbin_start[b + 1] += cbin_start[b];
            cbin.resize(ri.ncarb);
            std::vector<int> fill(ncc, 0);
            for (int k = 0; k < ri.ncarb; k++) cbin[cbin_start[bof[k]] + fill[bof[k]]++] = k;
            // the layers of cells the graphite acts on: up to the one holding
            // the top carbon plane + rs (rc plus the list skin)
            if (ri.ncarb && c->p.graphite_on) {
                const int iz = (int)floor((ztop + RS + r.rhs[2]) * (1.0 / RS));
                r.igz = iz < 0 ? 0 : (iz >= r.nc[2] ? r.nc[2] - 1 : iz);
            }
        }
        // carbons per bottom-layer column, pre-filtered as src/read_graphite.f90:9-35
        // (lp: the listed carbons' coordinates as the column sees them).
        // Columns are independent: built on host threads, then appended in
        // column order (the same arrays as a serial loop).
        struct ColOut {
            std::vector<double4> gpos;
            std::vector<float4> gpos32;
            std::vector<int> gbin;        // relative to the column's first carbon
            std::vector<float2> ggrp_z;
        };
        const int ncol_r = r.nc[0] * r.nc[1];
        std::vector<ColOut> cols(ncol_r);
        auto build_col = [&](int col) {
            const int ix = col % r.nc[0], iy = col / r.nc[0];
            ColOut &co = cols[col];
            std::vector<double> lp;
            double cx = axis[a0 + ix], cy = axis[a0 + r.nc[0] + iy], cz = axis[a0 + r.nc[0] + r.nc[1]];
            if (per) {
                const double rc2 = rcut_per * rcut_per;
                for (int by = iy - 2; by <= iy + 2; by++)      // 5 x 5 columns cover rcut_per (< 2.5 cells);
                    for (int bx = ix - 2; bx <= ix + 2; bx++) { // at least 8 per axis: no column twice
                        const int wx = ((bx % r.nc[0]) + r.nc[0]) % r.nc[0], wy = ((by % r.nc[1]) + r.nc[1]) % r.nc[1];
                        const int b = wx + r.nc[0] * wy;
                        for (int t = cbin_start[b]; t < cbin_start[b + 1]; t++) {
                            const int k = cbin[t];
                            // the image of the carbon nearest the column centre
                            double gx = ri.carb[3 * k], gy = ri.carb[3 * k + 1];
                            gx -= r.rsd[0] * floor((gx - cx) / r.rsd[0] + 0.5);
                            gy -= r.rsd[1] * floor((gy - cy) / r.rsd[1] + 0.5);
                            const double dx = gx - cx, dy = gy - cy;
                            if (dx * dx + dy * dy <= rc2) { lp.push_back(gx); lp.push_back(gy); lp.push_back(ri.carb[3 * k + 2]); }
                        }
                    }
            } else {
                for (int k = 0; k < ri.ncarb; k++) {
                    double dx = ri.carb[3 * k] - cx, dy = ri.carb[3 * k + 1] - cy;
                    if (dx * dx + dy * dy <= rcut)
                        for (int a = 0; a < 3; a++) lp.push_back(ri.carb[3 * k + a]);
                }
            }
            std::vector<int> ks(lp.size() / 3);
            for (size_t i = 0; i < ks.size(); i++) ks[i] = (int)i;
            // groups: the column's carbons by z (a graphite layer each, at
            // most GGRP groups of neighbouring z), each group in order of
            // its FP32 y with GBIN uniform y bins over [-ymax, ymax], so a
            // site visits only the groups and the y window within rc
            std::sort(ks.begin(), ks.end(), [&](int a, int b) {
                return lp[3 * a + 2] != lp[3 * b + 2] ? lp[3 * a + 2] < lp[3 * b + 2] : a < b;
            });
            std::vector<int> bounds(1, 0);
            for (size_t t = 1; t < ks.size(); t++)
                if (lp[3 * ks[t] + 2] != lp[3 * ks[t - 1] + 2]) bounds.push_back((int)t);
            bounds.push_back((int)ks.size());
            const int nz = (int)bounds.size() - 1;
            std::vector<int> gb(1, 0);   // group bounds: every z level, or GGRP equal runs of them
            for (int l = 1; l <= GGRP; l++)
                gb.push_back(bounds[nz <= GGRP ? (l <= nz ? l : nz) : (int)((long long)nz * l / GGRP)]);
            auto y32 = [&](int k) { return (float)(lp[3 * k + 1] - cy); };
            for (int l = 0; l < GGRP; l++) {
                const int b0 = gb[l], b1 = gb[l + 1];
                std::sort(ks.begin() + b0, ks.begin() + b1,
                          [&](int a, int b) { return y32(a) != y32(b) ? y32(a) < y32(b) : a < b; });
                float zlo = 0.f, zhi = -1.f;   // empty group
                for (int t = b0; t < b1; t++) {
                    const float z = (float)(lp[3 * ks[t] + 2] - cz);
                    zlo = t == b0 ? z : std::min(zlo, z);
                    zhi = t == b0 ? z : std::max(zhi, z);
                }
                co.ggrp_z.push_back(make_float2(zlo, zhi));
                // bin edge j at -ymax + j * bw: the first carbon at or above it
                int t = b0;
                for (int j = 0; j < GBIN; j++) {
                    const double edge = -(double)r.gymax + j * ((double)r.gymax * 2.0 / GBIN);
                    while (t < b1 && (double)y32(ks[t]) < edge) t++;
                    co.gbin.push_back(j ? t : b0);
                }
                co.gbin.push_back(b1);
            }
            for (int k : ks) {
                double dx = lp[3 * k] - cx, dy = lp[3 * k + 1] - cy;
                co.gpos.push_back(make_double4(lp[3 * k], lp[3 * k + 1], lp[3 * k + 2], 0.0));
                co.gpos32.push_back(make_float4((float)dx, (float)dy, (float)(lp[3 * k + 2] - cz), 0.f));
            }
        };
        {
            const int nth = std::max(1, std::min({(int)std::thread::hardware_concurrency(), 32, ncol_r / 16}));
            std::atomic<int> next{0};
            auto worker = [&]() {
                for (int col; (col = next.fetch_add(1)) < ncol_r;) build_col(col);
            };
            std::vector<std::thread> pool;
            for (int t = 1; t < nth; t++) pool.emplace_back(worker);
            worker();
            for (auto &th : pool) th.join();
        }
        for (int col = 0; col < ncol_r; col++) {
            const ColOut &co = cols[col];
            const int base = (int)gpos.size();
            for (int v : co.gbin) gbin.push_back(base + v);
            ggrp_z.insert(ggrp_z.end(), co.ggrp_z.begin(), co.ggrp_z.end());
            gpos.insert(gpos.end(), co.gpos.begin(), co.gpos.end());
            gpos32.insert(gpos32.end(), co.gpos32.begin(), co.gpos32.end());
            gstart.push_back((int)gpos.size());
        }
    }
    if ((e = dalloc(c, &d.axis, axis.size())) || (e = dalloc(c, &d.rcen2, rcen2.size())) ||
        (e = dalloc(c, &d.gcol_start, gstart.size())) ||
        (e = dalloc(c, &d.gpos, gpos.size())) || (e = dalloc(c, &d.gpos32, gpos32.size())) ||
        (e = dalloc(c, &d.gbin, gbin.size())) || (e = dalloc(c, &d.ggrp_z, ggrp_z.size())) ||
        (e = dalloc(c, &d.gsite, N)) || (e = dalloc(c, &d.gcount, 1)))
        return e;
    lap("per-site data, carbons");
    // translation operators
    // M2L factors: H per offset at L4 (cell edge rs), L3 (2 rs) and L2 (4 rs), and the coefficients
    auto put = [&](const std::vector<double2> &h, double2 *dst, float2 *dst32) -> int {
        std::vector<float2> h32(h.size());
        for (size_t i = 0; i < h.size(); i++) h32[i] = make_float2((float)h[i].x, (float)h[i].y);
        CK(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(dst32, h32.data(), h32.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
        return 0;
    };
    std::vector<double> cf(LPH * LP);
    m2l_coef(cf.data());
    // real-form operators of the 7^3 offsets at L4 (cell edge rs) and L3 (2 rs)
    auto fill_win = [&](double scale, void *dst) -> int {
        std::vector<double> rop((size_t)343 * LP * M2C_LD, 0.0);
        double2 h[NHARM];
        for (int dz = -3; dz <= 3; dz++)
            for (int dy = -3; dy <= 3; dy++)
                for (int dx = -3; dx <= 3; dx++) {
                    if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) continue;
                    const int oi = (dx + 3) + 7 * (dy + 3) + 49 * (dz + 3);
                    harm_m2l(dx * scale, dy * scale, dz * scale, h);
                    m2l_real(cf.data(), h, &rop[(size_t)oi * LP * M2C_LD]);
                }
        if (mixed) {
            std::vector<float> r32(rop.begin(), rop.end());
            CK(cudaMemcpyAsync(dst, r32.data(), r32.size() * sizeof(float), cudaMemcpyHostToDevice, c->st));
            CK(cudaStreamSynchronize(c->st));
        } else {
            CK(cudaMemcpyAsync(dst, rop.data(), rop.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
            CK(cudaStreamSynchronize(c->st));
        }
        return 0;
    };
    lap("operators, M2L factors");
    if ((e = fill_win(RS, d.rop4)) || (e = fill_win(2 * RS, d.rop3))) return e;
    {
        std::vector<double2> h(nh2, make_double2(0.0, 0.0));
        for (int dz = -d2.z; dz <= d2.z; dz++)
            for (int dy = -d2.y; dy <= d2.y; dy++)
                for (int dx = -d2.x; dx <= d2.x; dx++) {
                    if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) continue;
                    const int oi = (dx + d2.x) + w2x * ((dy + d2.y) + w2y * (dz + d2.z));
                    harm_m2l(dx * 4 * RS, dy * 4 * RS, dz * 4 * RS, &h[(size_t)oi * NHARM]);
                }
        if ((e = put(h, d.h_m2l2, d.h32_m2l2))) return e;
        // periodic preset: per replica, for each offset within the box, the
        // H of its images not adjacent to the target summed (M2L is linear
        // in H, so one pass over the box's sources takes every image)
        std::vector<double2> hp(NHARM, make_double2(0.0, 0.0));
        if (per) {
            // H of an L2 offset depends only on its integers: kept for the
            // life of the process (contexts formed again and again, as the
            // request server does, compute each offset once)
            static std::map<std::tuple<int, int, int>, std::vector<double2>> cache;
            static std::mutex cache_mu;
            std::lock_guard<std::mutex> cache_lock(cache_mu);
            hp.clear();
            for (int q = 0; q < R; q++) {
                Rep &r = c->reps[q];
                r.h2off = (int)(hp.size() / NHARM);
                const int n0 = r.nr[0], n1 = r.nr[1], n2z = r.nr[2];
                for (int dz = -(n2z - 1); dz <= n2z - 1; dz++)
                    for (int dy = -(n1 - 1); dy <= n1 - 1; dy++)
                        for (int dx = -(n0 - 1); dx <= n0 - 1; dx++) {
                            double2 acc[NHARM];
                            for (int k = 0; k < NHARM; k++) acc[k] = make_double2(0.0, 0.0);
                            for (int iy = -1; iy <= 1; iy++)
                                for (int ix = -1; ix <= 1; ix++) {
                                    const int ux = dx + ix * n0, uy = dy + iy * n1;
                                    if (abs(ux) <= 1 && abs(uy) <= 1 && abs(dz) <= 1) continue;
                                    auto key = std::make_tuple(ux, uy, dz);
                                    auto it = cache.find(key);
                                    if (it == cache.end()) {
                                        std::vector<double2> hv(NHARM);
                                        harm_m2l(ux * 4 * RS, uy * 4 * RS, dz * 4 * RS, hv.data());
                                        it = cache.emplace(key, std::move(hv)).first;
                                    }
                                    for (int k = 0; k < NHARM; k++) { acc[k].x += it->second[k].x; acc[k].y += it->second[k].y; }
                                }
                            hp.insert(hp.end(), acc, acc + NHARM);
                        }
            }
        }
        if ((e = dalloc(c, &d.h_per, hp.size())) || (e = dalloc(c, &d.h32_per, hp.size()))) return e;
        if ((e = put(hp, d.h_per, d.h32_per))) return e;
        std::vector<float> cf32(LPH * LP);
        for (int i = 0; i < LPH * LP; i++) cf32[i] = (float)cf[i];
        CK(cudaMemcpyAsync(d.m2l_cf, cf.data(), cf.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(d.m2l_cf32, cf32.data(), cf32.size() * sizeof(float), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
        std::vector<double2> o8((size_t)8 * LPH * LP);
        struct { double2 *dst; float2 *dst32; double s; int kind; } sets[4] = {
            {d.op_m2m43, d.op32_m2m43, RS, 0}, {d.op_m2m32, d.op32_m2m32, 2 * RS, 0},
            {d.op_l2l23, d.op32_l2l23, 2 * RS, 1}, {d.op_l2l34, d.op32_l2l34, RS, 1}};
        for (auto &st : sets) {
            for (int ch = 0; ch < 8; ch++) {
                double v[3] = {(ch & 1) - 0.5, ((ch >> 1) & 1) - 0.5, ((ch >> 2) & 1) - 0.5};
                if (st.kind == 0) op_m2m(v[0] * st.s, v[1] * st.s, v[2] * st.s, &o8[(size_t)ch * LPH * LP]);
                else op_l2l(-v[0] * st.s, -v[1] * st.s, -v[2] * st.s, &o8[(size_t)ch * LPH * LP]);
            }
            std::vector<float2> o8f(o8.size());
            for (size_t i = 0; i < o8.size(); i++) o8f[i] = make_float2((float)o8[i].x, (float)o8[i].y);
            CK(cudaMemcpyAsync(st.dst, o8.data(), o8.size() * sizeof(double2), cudaMemcpyHostToDevice, c->st));
            CK(cudaMemcpyAsync(st.dst32, o8f.data(), o8f.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
            CK(cudaStreamSynchronize(c->st));
        }
    }
    std::vector<double2> ljt = c->chains ? make_lj_table_cfg(make_cfg_field()) : make_lj_table();
    {
        std::vector<double> kq, km;
        std::vector<double2> kg;
        kind_tables(c->p.preset, kq, km, kg);
        CK(cudaMemcpyAsync(d.tq, kq.data(), NTYPE * sizeof(double), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(d.tmass, km.data(), NTYPE * sizeof(double), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(d.tgr, kg.data(), NTYPE * sizeof(double2), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
    }
    std::vector<float2> ljt32(ljt.size());
    for (size_t k = 0; k < ljt.size(); k++) ljt32[k] = make_float2((float)ljt[k].x, (float)ljt[k].y);
    CK(cudaMemcpyAsync(d.ljt32, ljt32.data(), ljt32.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.x, sx.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.y, sy.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.z, sz.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.vx, vxa.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.vy, vya.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.vz, vza.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.ptype, ptype.data(), N, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.smol, smol.data(), N * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.mrep, mrep.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.mfirst, mfirst.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.mkind, mkind.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->st));
    lap("window operators, H tables");
    if (nwm) {
        CK(cudaMemcpyAsync(c->wmols, wm.data(), nwm * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(d.wlist_a, wm.data(), nwm * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(d.wlist_b, wm.data(), nwm * sizeof(int), cudaMemcpyHostToDevice, c->st));
    }
    if (nsm) CK(cudaMemcpyAsync(c->smols, sm.data(), nsm * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.rep, c->reps.data(), R * sizeof(Rep), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.eta, eta0.data(), R * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.axis, axis.data(), axis.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.rcen2, rcen2.data(), rcen2.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.crep, crep.data(), C * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.b3rep, b3.data(), n3 * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.b2rep, b2.data(), n2 * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.gcol_start, gstart.data(), gstart.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
    if (!gpos.empty()) CK(cudaMemcpyAsync(d.gpos, gpos.data(), gpos.size() * sizeof(double4), cudaMemcpyHostToDevice, c->st));
    if (!gpos32.empty())
        CK(cudaMemcpyAsync(d.gpos32, gpos32.data(), gpos32.size() * sizeof(float4), cudaMemcpyHostToDevice, c->st));
    if (!gbin.empty()) {
        CK(cudaMemcpyAsync(d.gbin, gbin.data(), gbin.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(d.ggrp_z, ggrp_z.data(), ggrp_z.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    }
    CK(cudaMemcpyAsync(d.ljt, ljt.data(), ljt.size() * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemsetAsync(d.near_ctl, 0, 66 * sizeof(int), c->st));   // no near-field items before the first rebuild
    CK(cudaStreamSynchronize(c->st));
    c->uploaded = true;
    c->have_force = false;
    c->steps = 0;
    lap("water lists, graphite");
    return 0;
}

}  // namespace

extern "C" {

int sesp_upload_state(sesp_ctx *c, int n_water, int n_surf, const double *pos, const double *vel, int n_carbon,
                      const double *carbons) {
    if (int e = check_ctx(c, false)) return e;
    RepIn r;
    r.nw = n_water; r.ns = n_surf; r.ncarb = n_carbon;
    for (int a = 0; a < 3; a++) r.nc[a] = c->p.n_cells[a];
    r.pos = pos; r.vel = vel; r.carb = carbons;
    return upload_impl(c, std::vector<RepIn>(1, r));
}

int sesp_upload_batch(sesp_ctx *c, int n_rep, const int *n_water, const int *n_surf, const int *n_cells,
                      const double *pos, const double *vel, const int *n_carbon, const double *carbons) {
    if (int e = check_ctx(c, false)) return e;
    if (n_rep <= 0 || !n_water || !n_surf || !n_cells || !pos || !n_carbon) return fail(SESP_EINVAL, "bad batch arguments");
    std::vector<RepIn> in(n_rep);
    size_t so = 0, co = 0;
    for (int q = 0; q < n_rep; q++) {
        RepIn &r = in[q];
        r.nw = n_water[q]; r.ns = n_surf[q]; r.ncarb = n_carbon[q];
        for (int a = 0; a < 3; a++) r.nc[a] = n_cells[3 * q + a];
        r.pos = pos + 3 * so;
        r.vel = vel ? vel + 3 * so : nullptr;
        r.carb = carbons ? carbons + 3 * co : nullptr;
        so += (size_t)3 * r.nw + (size_t)c->ssite * r.ns;
        co += r.ncarb;
    }
    return upload_impl(c, in);
}

int sesp_replica_count(sesp_ctx *c) {
    if (!c) return -fail(SESP_EINVAL, "null context");
    return c->nrep;
}

int sesp_get_eta_batch(sesp_ctx *c, double *eta) {
    if (int e = check_ctx(c, true)) return e;
    if (!eta) return fail(SESP_EINVAL, "null output");
    CK(cudaMemcpyAsync(eta, c->d.eta, c->nrep * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_set_eta_batch(sesp_ctx *c, const double *eta) {
    if (int e = check_ctx(c, true)) return e;
    if (!eta) return fail(SESP_EINVAL, "null input");
    for (int q = 0; q < c->nrep; q++)
        if (!std::isfinite(eta[q])) return fail(SESP_EINVAL, "eta of a replica is not finite");
    CK(cudaMemcpyAsync(c->d.eta, eta, c->nrep * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

// (3, n) site-major host arrays <-> the device's x / y / z arrays: one
// contiguous copy per array through a device staging buffer, transposed by
// a kernel (array k of the staging buffer at k * 3n: positions, velocities,
// accelerations, forces)
__global__ void k_state_io(Dev d, double *stage, int n, int mask, int unpack) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    double *soa[4][3] = {{d.x, d.y, d.z}, {d.vx, d.vy, d.vz}, {d.ax, d.ay, d.az}, {d.fx, d.fy, d.fz}};
    for (int k = 0; k < 4; k++) {
        if (!(mask >> k & 1)) continue;
        double *aos = stage + (size_t)k * 3 * n + 3 * (size_t)g;
        for (int a = 0; a < 3; a++) {
            if (unpack) soa[k][a][g] = aos[a];
            else aos[a] = soa[k][a][g];
        }
    }
}

int sesp_download_state(sesp_ctx *c, double *pos, double *vel, double *acc) {
    if (int e = check_ctx(c, true)) return e;
    if (set_device(c)) return SESP_ECUDA;
    const int N = c->nsite;
    double *outs[3] = {pos, vel, acc};
    const int mask = (pos ? 1 : 0) | (vel ? 2 : 0) | (acc ? 4 : 0);
    if (!mask) return 0;
    k_state_io<<<(N + 255) / 256, 256, 0, c->st>>>(c->d, c->d.stage, N, mask, 0);
    CK(cudaGetLastError());
    for (int k = 0; k < 3; k++)
        if (outs[k])
            CK(cudaMemcpyAsync(outs[k], c->d.stage + (size_t)k * 3 * N, 3 * (size_t)N * sizeof(double),
                               cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_set_state(sesp_ctx *c, const double *pos, const double *vel, const double *acc, double eta) {
    if (int e = check_ctx(c, true)) return e;
    if (set_device(c)) return SESP_ECUDA;
    const int N = c->nsite;
    const double *ins[3] = {pos, vel, acc};
    const int mask = (pos ? 1 : 0) | (vel ? 2 : 0) | (acc ? 4 : 0);
    for (int k = 0; k < 3; k++)
        if (ins[k])
            CK(cudaMemcpyAsync(c->d.stage + (size_t)k * 3 * N, ins[k], 3 * (size_t)N * sizeof(double),
                               cudaMemcpyHostToDevice, c->st));
    if (mask) {
        k_state_io<<<(N + 255) / 256, 256, 0, c->st>>>(c->d, c->d.stage, N, mask, 1);
        CK(cudaGetLastError());
    }
    const std::vector<double> etas(c->nrep, eta);   // every replica
    CK(cudaMemcpyAsync(c->d.eta, etas.data(), c->nrep * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_force_terms(sesp_ctx *c, int rebuild, int terms) {
    if (int e = check_ctx(c, true)) return e;
    if (!rebuild && !c->have_force) return fail(SESP_ESTATE, "the first force call must rebuild the lists");
    if (set_device(c)) return SESP_ECUDA;
    seq_force(c, rebuild, terms);
    if (c->fault) return fail(SESP_ECUDA, "kernel family '%s' failed: %s", c->fault, cudaGetErrorString(cudaGetLastError()));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    collect_all(c);
    c->have_force = true;
    return 0;
}

int sesp_force(sesp_ctx *c, int rebuild) { return sesp_force_terms(c, rebuild, SESP_T_ALL); }

int sesp_download_forces(sesp_ctx *c, double *f) {
    if (int e = check_ctx(c, true)) return e;
    if (!f) return fail(SESP_EINVAL, "null output");
    if (set_device(c)) return SESP_ECUDA;
    const int N = c->nsite;
    k_state_io<<<(N + 255) / 256, 256, 0, c->st>>>(c->d, c->d.stage, N, 8, 0);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(f, c->d.stage + (size_t)9 * N, 3 * (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_init_accel(sesp_ctx *c) {
    if (int e = check_ctx(c, true)) return e;
    if (set_device(c)) return SESP_ECUDA;
    launch_init_accel(c->d, c->nsite, c->st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_move_a(sesp_ctx *c) {
    if (int e = check_ctx(c, true)) return e;
    if (set_device(c)) return SESP_ECUDA;
    seq_move_a(c);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    collect_all(c);
    return 0;
}

int sesp_move_b(sesp_ctx *c) {
    if (int e = check_ctx(c, true)) return e;
    if (set_device(c)) return SESP_ECUDA;
    seq_move_b(c);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    collect_all(c);
    return 0;
}

static int launch_steps(sesp_ctx *c, int kb0, int nsteps) {
    if (int e = check_ctx(c, true)) return e;
    if (nsteps < 0) return fail(SESP_EINVAL, "negative step count");
    if (set_device(c)) return SESP_ECUDA;
    for (int k = 0; k < nsteps; k++) {
        int kb = kb0 + k;
        int rb = (kb % c->p.rebuild_interval == 0) || !c->have_force;
        if (c->timing || c->sync_check) {
            seq_move_a(c);
            seq_force(c, rb, SESP_T_ALL);
            seq_move_b(c);
            collect_all(c);
            if (c->fault) return fail(SESP_ECUDA, "step %d: kernel family '%s' failed: %s", kb, c->fault,
                                      cudaGetErrorString(cudaGetLastError()));
        } else {
            cudaGraphExec_t &ge = c->g_step[rb];
            if (!ge) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
                // on the mixed paths the force call forks its side stream and
                // joins it before the site forces, which also joins the eta update
                seq_move_a(c, c->p.precision != SESP_PLAIN_FP64);
                seq_force(c, rb, SESP_T_ALL);
                seq_move_b(c);
                CK(cudaStreamEndCapture(c->st, &g));
                CK(cudaGraphInstantiate(&ge, g, 0));
                cudaGraphDestroy(g);
            }
            CK(cudaGraphLaunch(ge, c->st));
        }
        c->have_force = true;
        c->steps++;
    }
    CK(cudaGetLastError());
    return 0;
}

int sesp_run_timed(sesp_ctx *c, int kb0, int nsteps, int flush_l2, double *step_ms) {
    if (int e = check_ctx(c, true)) return e;
    if (!step_ms || nsteps < 0) return fail(SESP_EINVAL, "bad arguments");
    if (c->timing) return fail(SESP_ESTATE, "disable per-kernel timing first");
    if (set_device(c)) return SESP_ECUDA;
    const size_t fbytes = (size_t)256 << 20;
    void *fbuf = nullptr;
    if (flush_l2) CK(cudaMalloc(&fbuf, fbytes));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = 0;
    for (int k = 0; k < nsteps && !rc; k++) {
        if (flush_l2) launch_flush(fbuf, fbytes, c->st);
        cudaEventRecord(e0, c->st);
        rc = launch_steps(c, kb0 + k, 1);
        cudaEventRecord(e1, c->st);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(SESP_ECUDA, "timed step failed");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        step_ms[k] = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (fbuf) cudaFree(fbuf);
    return rc;
}

// ------------------------------------------------------------------ autotuning of the pair-field launch

namespace {
void drop_graphs(sesp_ctx *c) {
    for (auto &g : c->g_step)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}
}  // namespace

int sesp_set_tuning(sesp_ctx *c, int tile, int ctas_per_sm) {
    if (int e = check_ctx(c, true)) return e;
    const int mixed = c->p.precision != SESP_PLAIN_FP64;
    if (tile != 32 && tile != 64 && !(mixed && tile == 128))
        return fail(SESP_EINVAL, "tile must be 32 or 64 (or 128 on the mixed paths)");
    if (ctas_per_sm < 1 || ctas_per_sm > near_max_ctas_per_sm(near_mode(c), tile, c->chains))
        return fail(SESP_EINVAL, "ctas_per_sm must be 1..%d", near_max_ctas_per_sm(near_mode(c), tile, c->chains));
    if (set_device(c)) return SESP_ECUDA;
    const bool retile = tile != c->near.tile;
    c->near = {tile, c->n_sm * ctas_per_sm};
    if (retile && c->have_force) launch_near_items(c->d, c->ncell, (int)near_items_max(c->nsite, c->ncell), tile, c->st);   // items of the current lists
    drop_graphs(c);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_tuning(sesp_ctx *c, int out[3]) {
    if (int e = check_ctx(c, false)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    out[0] = c->near.tile;
    out[1] = c->n_sm ? c->near.grid / c->n_sm : 0;
    out[2] = near_max_ctas_per_sm(near_mode(c), c->near.tile, c->chains);
    return 0;
}

int sesp_set_constraint_tuning(sesp_ctx *c, int surf_warps, int mols_per_warp) {
    if (int e = check_ctx(c, false)) return e;
    if (surf_warps < 1 || surf_warps > constraint_max_surf_warps())
        return fail(SESP_EINVAL, "surf_warps must be 1..%d", constraint_max_surf_warps());
    if (mols_per_warp < 1 || mols_per_warp > constraint_max_mols_per_warp(c->p.precision == SESP_MIXED_FP32C))
        return fail(SESP_EINVAL, "mols_per_warp must be 1..%d", constraint_max_mols_per_warp(c->p.precision == SESP_MIXED_FP32C));
    c->cshape.s_warps = surf_warps;
    c->cshape.mpw = mols_per_warp;
    drop_graphs(c);
    return 0;
}

int sesp_constraint_tuning(sesp_ctx *c, int out[4]) {
    if (int e = check_ctx(c, false)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    out[0] = c->cshape.s_warps;
    out[1] = c->cshape.mpw;
    out[2] = constraint_max_surf_warps();
    out[3] = constraint_max_mols_per_warp(c->p.precision == SESP_MIXED_FP32C);
    return 0;
}

namespace {
// Times both constraint halves of the mixed paths for every surfactant-warp
// count and surfactants per warp (1, 2, 4, 8), median of 3, restoring the
// state the halves change before every trial and at the end, and keeps the
// fastest.
int tune_constraints(sesp_ctx *c) {
    const Dev &d = c->d;
    const size_t N = c->nsite, M = c->nmol, R = c->nrep;
    struct Arr { void *p; size_t bytes; };
    const Arr arrs[] = {{d.x, 8 * N}, {d.y, 8 * N}, {d.z, 8 * N}, {d.vx, 8 * N}, {d.vy, 8 * N}, {d.vz, 8 * N},
                        {d.ax, 8 * N}, {d.ay, 8 * N}, {d.az, 8 * N}, {d.ke, 16 * M}, {d.mfail, 4 * M},
                        {d.eta, 8 * R}, {d.counters, 64}, {d.wsw_a, M}, {d.wsw_b, M}};
    size_t total = 0;
    for (const Arr &a : arrs) total += (a.bytes + 255) & ~(size_t)255;
    unsigned char *save = nullptr;
    CK(cudaMalloc(&save, total));
    auto copy = [&](bool out) {
        size_t off = 0;
        for (const Arr &a : arrs) {
            if (out) cudaMemcpyAsync(save + off, a.p, a.bytes, cudaMemcpyDeviceToDevice, c->st);
            else cudaMemcpyAsync(a.p, save + off, a.bytes, cudaMemcpyDeviceToDevice, c->st);
            off += (a.bytes + 255) & ~(size_t)255;
        }
    };
    copy(true);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    ConstraintShape pick = c->cshape;
    for (int sw = 1; sw <= constraint_max_surf_warps(); sw++)
    for (int mpw = 1; mpw <= constraint_max_mols_per_warp(c->p.precision == SESP_MIXED_FP32C); mpw *= 2) {
        const ConstraintShape sh = {c->cshape.grid, sw, mpw};
        float t[3];
        for (int r = 0; r < 3; r++) {
            copy(false);
            cudaEventRecord(e0, c->st);
            launch_move_a(d, c->wmols, c->nwm, c->smols, c->nsm, c->nrep, c->nmol, c->nsite, c->p.shake_tol, c->p.shake_maxit,
                          c->p.precision, sh, c->chains, c->st);
            launch_move_b(d, c->wmols, c->nwm, c->smols, c->nsm, c->nmol, c->nsite, c->p.shake_tol, c->p.shake_maxit, c->p.precision, sh,
                          c->chains, c->st);
            cudaEventRecord(e1, c->st);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&t[r], e0, e1);
        }
        std::sort(t, t + 3);
        if (t[1] < best) { best = t[1]; pick = sh; }
    }
    copy(false);
    cudaError_t err = cudaStreamSynchronize(c->st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(save);
    if (err != cudaSuccess) return fail(SESP_ECUDA, "constraint autotuning: %s", cudaGetErrorString(err));
    c->cshape = pick;
    return 0;
}
}  // namespace

// Times the pair field on the current state for every candidate shape (tile
// 128 (mixed paths), 64 or 32 sites per work item; 1/4, 1/2, 3/4 or all of
// the CTAs per SM the kernel can hold), median of 5 launches each, and keeps
// the fastest; on the
// mixed paths with surfactants, then the constraint halves' surfactant warps
// per CTA (the state is restored afterwards).
int sesp_autotune(sesp_ctx *c, int out[3]) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    if (!c->have_force) return fail(SESP_ESTATE, "autotuning needs a force call first (cell lists)");
    if (set_device(c)) return SESP_ECUDA;
    const int mixed = c->p.precision != SESP_PLAIN_FP64;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    NearShape pick = c->near;
    for (int tile : {128, 64, 32}) {
        if (tile == 128 && !mixed) continue;
        const int mx = near_max_ctas_per_sm(near_mode(c), tile, c->chains);
        const int cands[4] = {mx, (3 * mx) / 4, mx / 2, mx / 4};
        launch_near_items(c->d, c->ncell, (int)near_items_max(c->nsite, c->ncell), tile, c->st);
        for (int k = 0; k < 4; k++) {
            const int cps = cands[k];
            if (cps < 1 || (k > 0 && cps == cands[k - 1])) continue;
            const NearShape sh = {tile, c->n_sm * cps};
            launch_near(c->d, c->ncell, c->nsite, near_mode(c), SESP_T_NEAR, sh, c->st, true, c->chains);   // warm
            float t[5];
            for (int r = 0; r < 5; r++) {
                cudaEventRecord(e0, c->st);
                launch_near(c->d, c->ncell, c->nsite, near_mode(c), SESP_T_NEAR, sh, c->st, true, c->chains);
                cudaEventRecord(e1, c->st);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&t[r], e0, e1);
            }
            std::sort(t, t + 5);
            if (t[2] < best) { best = t[2]; pick = sh; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->near = pick;
    launch_near_items(c->d, c->ncell, (int)near_items_max(c->nsite, c->ncell), pick.tile, c->st);
    if (mixed && c->nsm > 0 && !c->chains)   // flexible chains have no constraint sweeps to shape
        if (int e = tune_constraints(c)) return e;
    drop_graphs(c);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    out[0] = pick.tile;
    out[1] = pick.grid / c->n_sm;
    out[2] = near_max_ctas_per_sm(near_mode(c), pick.tile, c->chains);
    return 0;
}

int sesp_pair_counts(sesp_ctx *c, int64_t out[2]) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    if (!c->have_force) return fail(SESP_ESTATE, "pair counts need a force call first");
    if (set_device(c)) return SESP_ECUDA;
    unsigned long long *dc = nullptr, h[2] = {0, 0};
    CK(cudaMalloc(&dc, sizeof h));
    cudaMemsetAsync(dc, 0, sizeof h, c->st);
    launch_gather(c->d, c->nsite, c->ncell, 0, c->st);
    launch_count_pairs(c->d, c->ncell, dc, c->st);
    cudaMemcpyAsync(h, dc, sizeof h, cudaMemcpyDeviceToHost, c->st);
    cudaError_t err = cudaStreamSynchronize(c->st);
    cudaFree(dc);
    if (err != cudaSuccess) return fail(SESP_ECUDA, "pair counts: %s", cudaGetErrorString(err));
    out[0] = (int64_t)h[0];
    out[1] = (int64_t)h[1];
    return 0;
}

int sesp_step(sesp_ctx *c, int kb) {
    int e = launch_steps(c, kb, 1);
    if (e) return e;
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_run(sesp_ctx *c, int kb0, int nsteps) {
    int e = launch_steps(c, kb0, nsteps);
    if (e) return e;
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_run_async(sesp_ctx *c, int kb0, int nsteps) { return launch_steps(c, kb0, nsteps); }

int sesp_query(sesp_ctx *c) {
    if (!c) return -fail(SESP_EINVAL, "null context");
    if (set_device(c)) return -SESP_ECUDA;
    cudaError_t e = cudaStreamQuery(c->st);
    if (e == cudaSuccess) return 0;
    if (e == cudaErrorNotReady) return 1;
    return -fail(SESP_ECUDA, "stream query: %s", cudaGetErrorString(e));
}

int sesp_device_bytes(sesp_ctx *c, int64_t *bytes) {
    if (int e = check_ctx(c, false)) return e;
    if (!bytes) return fail(SESP_EINVAL, "null output");
    *bytes = (int64_t)c->bytes;
    return 0;
}

int sesp_sync(sesp_ctx *c) {
    if (int e = check_ctx(c, false)) return e;
    if (set_device(c)) return SESP_ECUDA;
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_temperature(sesp_ctx *c, double *t) {
    if (int e = check_ctx(c, true)) return e;
    if (!t) return fail(SESP_EINVAL, "null output");
    if (set_device(c)) return SESP_ECUDA;
    launch_temperature(c->d, c->nrep, c->st);
    CK(cudaGetLastError());
    std::vector<double> sums(c->nrep);
    CK(cudaMemcpyAsync(sums.data(), c->d.tbuf, c->nrep * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    double s = 0.0;
    long dof = 0;
    for (int q = 0; q < c->nrep; q++) {
        s += sums[q];
        dof += 3L * c->reps[q].nsite - c->reps[q].ncon;
    }
    *t = s / (DT * DT) / (double)dof;   // src/compute_temperature.f90:240-242
    return 0;
}

int sesp_get_eta(sesp_ctx *c, double *eta) {
    if (int e = check_ctx(c, true)) return e;
    if (!eta) return fail(SESP_EINVAL, "null output");
    CK(cudaMemcpyAsync(eta, c->d.eta, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_set_eta(sesp_ctx *c, double eta) {
    if (int e = check_ctx(c, true)) return e;
    std::vector<double> v(c->nrep, eta);
    CK(cudaMemcpyAsync(c->d.eta, v.data(), c->nrep * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return 0;
}

int sesp_energies(sesp_ctx *c, double out[8]) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    if (!c->have_force) return fail(SESP_ESTATE, "energies need a force call first (lists and expansions)");
    if (set_device(c)) return SESP_ECUDA;
    int N = c->nsite;
    double *es = nullptr, *ei = nullptr, *em = nullptr;
    // the scratch is freed on every path (a failed allocation frees the earlier ones)
    struct Scratch {
        double **p[3];
        ~Scratch() { for (double **q : p) if (*q) cudaFree(*q); }
    } guard = {{&es, &ei, &em}};
    cudaError_t err = cudaMalloc(&es, 3 * sizeof(double) * N);
    if (err == cudaSuccess) err = cudaMalloc(&ei, 3 * sizeof(double) * N);
    if (err == cudaSuccess) err = cudaMalloc(&em, 3 * sizeof(double) * (c->nsm + 1));
    if (err != cudaSuccess) return fail(SESP_ENOMEM, "energies: scratch allocation: %s", cudaGetErrorString(err));
    std::vector<double> hs(3 * (size_t)N), hi(3 * (size_t)N), hm(3 * (size_t)(c->nsm + 1));
    err = cudaMemsetAsync(es, 0, 3 * sizeof(double) * N, c->st);
    if (err == cudaSuccess) {
        launch_gather(c->d, c->nsite, c->ncell, 0, c->st);
        launch_energies(c->d, c->ncell, N, c->smols, c->nsm, c->chains, es, ei, em, c->st);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(hs.data(), es, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(hi.data(), ei, hi.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(hm.data(), em, 3 * sizeof(double) * c->nsm, cudaMemcpyDeviceToHost, c->st);
    // wait for the queued work before the guard frees the scratch it uses
    const cudaError_t e2 = cudaStreamSynchronize(c->st);
    if (err == cudaSuccess) err = e2;
    if (err != cudaSuccess) return fail(SESP_ECUDA, "energies: %s", cudaGetErrorString(err));
    for (int k = 0; k < 8; k++) out[k] = 0.0;
    for (int s = 0; s < N; s++) { out[0] += hs[3 * s]; out[1] += hs[3 * s + 1]; out[2] += hs[3 * s + 2]; }
    for (int q = 0; q < c->nsm; q++) { out[4] += hm[3 * q]; out[3] += hm[3 * q + 1]; out[2] += hm[3 * q + 2]; }
    for (int g = 0; g < N; g++) { out[5] += hi[3 * g]; out[6] += hi[3 * g + 1]; out[7] += hi[3 * g + 2]; }
    return 0;
}

// ------------------------------------------------------------------ energies without allocation
//
// sesp_energies takes its per-site scratch from cudaMalloc and gives it back
// with cudaFree on every call.  Callers that share the GPU with runs they must
// not disturb cannot afford that: cudaFree waits for all work on the device,
// so a monitoring call from a loop that keeps several contexts busy at once
// (the request loop of the serving layer, where every admitted run has its own
// stream) would stall every run, and once an HBM budget has been handed out in
// full a cudaMalloc can fail.  sesp_energies_static computes the same eight
// energies with its scratch in one fixed array compiled into this library.
//
// The array holds SESP_NOALLOC_MAX_SITES x 6 + (SESP_NOALLOC_MAX_SURF + 1) x 3
// + 8 doubles (6.1 MiB); every GPU that loads the library keeps it until the
// process exits.  In host code its name is only a stand-in: its device
// address is looked up with cudaGetSymbolAddress, once per device, by the
// first call on that device, with that device current.  That first call
// should therefore come before any stream capture, and the address is kept
// for the life of the process: the function must not be used after
// something in the process resets the device's primary context
// (cudaDeviceReset), whose new context has the array elsewhere.  All calls on one device
// share the array and it keeps the last call's contents: each call clears the
// per-slot part (slots that no site occupies are summed as zeros), and calls
// hold a per-device lock until their result has reached the host, because two
// calls whose work overlapped on the GPU would race on the array.
static __device__ __align__(256) double sesp_energy_scratch[6 * (size_t)SESP_NOALLOC_MAX_SITES +
                                                             3 * ((size_t)SESP_NOALLOC_MAX_SURF + 1) + 8];

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_lock[NOALLOC_MAX_DEVICES];
double *g_noalloc_scratch[NOALLOC_MAX_DEVICES];   // device address per device, null until looked up

// The eight totals, each summed by one thread in the order sesp_energies sums
// them on the host (sites in order, then surfactants), so both entry points
// give the same bits.
__global__ void k_energy_totals(const double *e_slot, const double *e_site, const double *e_mol, int nsite, int ns,
                                double *out) {
    const int k = threadIdx.x;
    if (k >= 8) return;
    double s = 0.0;
    if (k <= 2) {
        for (int i = 0; i < nsite; i++) s += e_slot[3 * (size_t)i + k];
        if (k == 2)
            for (int q = 0; q < ns; q++) s += e_mol[3 * q + 2];
    } else if (k == 3) {
        for (int q = 0; q < ns; q++) s += e_mol[3 * q + 1];
    } else if (k == 4) {
        for (int q = 0; q < ns; q++) s += e_mol[3 * q];
    } else {
        for (int g = 0; g < nsite; g++) s += e_site[3 * (size_t)g + (k - 5)];
    }
    out[k] = s;
}

}  // namespace

int sesp_energies_static(sesp_ctx *c, double out[8]) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    if (c->nsite > SESP_NOALLOC_MAX_SITES || c->nsm > SESP_NOALLOC_MAX_SURF)
        return fail(SESP_EINVAL,
                    "sesp_energies_static: %d sites and %d surfactants exceed its fixed scratch (at most %d sites "
                    "and %d surfactants); call sesp_energies instead",
                    c->nsite, c->nsm, SESP_NOALLOC_MAX_SITES, SESP_NOALLOC_MAX_SURF);
    if (!c->have_force) return fail(SESP_ESTATE, "energies need a force call first (lists and expansions)");
    const int dev = c->p.device;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return fail(SESP_EINVAL, "sesp_energies_static: device %d is beyond the %d it serves", dev, NOALLOC_MAX_DEVICES);
    if (set_device(c)) return SESP_ECUDA;
    // the context's earlier work first, outside the lock: the lock then
    // covers only this call's kernels and copy, not other runs' queues
    CK(cudaStreamSynchronize(c->st));
    std::lock_guard<std::mutex> hold(g_noalloc_lock[dev]);
    if (!g_noalloc_scratch[dev]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, sesp_energy_scratch);
        if (e != cudaSuccess || !p)
            return fail(SESP_ECUDA, "sesp_energies_static: device address of the scratch: %s", cudaGetErrorString(e));
        g_noalloc_scratch[dev] = p;
    }
    const int N = c->nsite;
    double *es = g_noalloc_scratch[dev];
    double *ei = es + 3 * (size_t)SESP_NOALLOC_MAX_SITES;
    double *em = ei + 3 * (size_t)SESP_NOALLOC_MAX_SITES;
    double *tot = em + 3 * ((size_t)SESP_NOALLOC_MAX_SURF + 1);
    cudaError_t err = cudaMemsetAsync(es, 0, 3 * sizeof(double) * N, c->st);
    if (err == cudaSuccess) {
        launch_gather(c->d, c->nsite, c->ncell, 0, c->st);
        launch_energies(c->d, c->ncell, N, c->smols, c->nsm, c->chains, es, ei, em, c->st);
        k_energy_totals<<<1, 32, 0, c->st>>>(es, ei, em, N, c->nsm, tot);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(out, tot, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    // whatever failed, the lock is released only once the GPU is done with the array
    const cudaError_t e2 = cudaStreamSynchronize(c->st);
    if (err == cudaSuccess) err = e2;
    if (err != cudaSuccess) return fail(SESP_ECUDA, "sesp_energies_static: %s", cudaGetErrorString(err));
    return 0;
}

int sesp_failures_batch(sesp_ctx *c, int64_t *out) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    const int M = c->reps.empty() ? 0 : c->reps.back().mol0 + c->reps.back().nmol;
    std::vector<int> h(M > 0 ? M : 1);
    if (M > 0) CK(cudaMemcpyAsync(h.data(), c->d.mfail, M * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int q = 0; q < c->nrep; q++) {
        const Rep &r = c->reps[q];
        int64_t n = 0;
        for (int m = r.mol0; m < r.mol0 + r.nmol; m++) n += h[m];
        out[q] = n;
    }
    return 0;
}

int sesp_counters(sesp_ctx *c, int64_t out[8]) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    unsigned long long h[8];
    CK(cudaMemcpyAsync(h, c->d.counters, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int k = 0; k < 8; k++) out[k] = (int64_t)h[k];
    out[3] = c->steps;
    out[4] = (int64_t)h[3];
    return 0;
}

}  // extern "C"

namespace {

constexpr int CHECK_THREADS = 256;

// The counts of sesp_checks for one replica per block: molecules located
// whole, charge of the slots (srt_pos.w = q of the site), water O / H and
// unlocated sites.  Each thread strides over its share, then one fixed tree
// sums the block, so the charge total does not depend on timing.
__global__ void k_checks(Dev d, double *out) {
    __shared__ double s_q[CHECK_THREADS];
    __shared__ long long s_n[4][CHECK_THREADS];
    const Rep r = d.rep[blockIdx.x];
    const int t = threadIdx.x;
    long long mol_ok = 0, n_o = 0, n_h = 0, n_out = 0;
    double q = 0.0;
    for (int m = t; m < r.nmol; m += CHECK_THREADS) {
        const int g0 = d.mfirst[r.mol0 + m];
        const int ns = d.mkind[r.mol0 + m] == 0 ? 3 : r.ssite;
        int ok = 1;
        for (int k = 0; k < ns; k++) ok &= d.sloc[g0 + k] >= 0;
        mol_ok += ok;
    }
    for (int g = r.site0 + t; g < r.site0 + r.nsite; g += CHECK_THREADS) {
        if (d.sloc[g] < 0) { n_out++; continue; }
        const int pt = d.ptype[g];
        n_o += pt == 0;
        n_h += pt == 1;
    }
    const int s0 = d.cstart[r.cell0], s1 = d.cstart[r.cell0 + r.nc[0] * r.nc[1] * r.nc[2]];
    for (int s = s0 + t; s < s1; s += CHECK_THREADS) q += d.srt_pos[s].w;
    s_q[t] = q;
    s_n[0][t] = mol_ok; s_n[1][t] = n_o; s_n[2][t] = n_h; s_n[3][t] = n_out;
    __syncthreads();
    for (int w = CHECK_THREADS / 2; w > 0; w >>= 1) {
        if (t < w) {
            s_q[t] += s_q[t + w];
            for (int k = 0; k < 4; k++) s_n[k][t] += s_n[k][t + w];
        }
        __syncthreads();
    }
    if (t == 0) {
        double *o = out + 8 * (size_t)blockIdx.x;
        o[0] = (double)s_n[0][0]; o[1] = (double)r.nmol; o[2] = s_q[0];
        o[3] = (double)s_n[1][0]; o[4] = (double)s_n[2][0]; o[5] = (double)r.nw;
        o[6] = (double)s_n[3][0]; o[7] = 0.0;
    }
}

__global__ void k_scale_velocities(Dev d, int nsite, double f) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nsite) return;
    d.vx[g] = f * d.vx[g]; d.vy[g] = f * d.vy[g]; d.vz[g] = f * d.vz[g];
}

}  // namespace

extern "C" {

int sesp_check_flags(const double c[7]) {
    if (!c) return 0;
    int f = 0;
    if (c[0] != c[1]) f |= SESP_CHECK_MOLECULES_LOST;
    if (c[2] * c[2] > 0.001) f |= SESP_CHECK_CHARGE;
    const long long n_o = (long long)c[3], n_h = (long long)c[4];
    // the reference divides H by O as integers; with no O it would divide by
    // zero, here H without O is flagged and an empty system is not
    if (n_o > 0 ? n_h / n_o != 2 : n_h != 0) f |= SESP_CHECK_OH_RATIO;
    if (c[3] != c[5]) f |= SESP_CHECK_MISSING_OXYGEN;
    return f;
}

int sesp_checks(sesp_ctx *c, double *out) {
    if (int e = check_ctx(c, true)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    if (!c->have_force) return fail(SESP_ESTATE, "checks need a force call first (cell lists)");
    if (set_device(c)) return SESP_ECUDA;
    double *dout = nullptr;
    CK(cudaMallocAsync((void **)&dout, 8 * sizeof(double) * c->nrep, c->st));
    k_checks<<<c->nrep, CHECK_THREADS, 0, c->st>>>(c->d, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, 8 * sizeof(double) * c->nrep, cudaMemcpyDeviceToHost, c->st);
    cudaFreeAsync(dout, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) return fail(SESP_ECUDA, "sesp_checks: %s", cudaGetErrorString(e));
    for (int q = 0; q < c->nrep; q++) out[8 * q + 7] = (double)sesp_check_flags(out + 8 * q);
    return 0;
}

int sesp_rescale_temperature(sesp_ctx *c, double target, double *t_before) {
    if (int e = check_ctx(c, true)) return e;
    if (!(target > 0.0)) return fail(SESP_EINVAL, "target temperature %g is not positive", target);
    double t = 0.0;
    if (int e = sesp_temperature(c, &t)) return e;
    if (!(t > 0.0)) return fail(SESP_EINVAL, "temperature %g cannot be rescaled", t);
    if (set_device(c)) return SESP_ECUDA;
    const double f = sqrt(target / t);   // tscale, src/compute_temperature_rescale.f90:243
    k_scale_velocities<<<(c->nsite + 255) / 256, 256, 0, c->st>>>(c->d, c->nsite, f);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    if (t_before) *t_before = t;
    return 0;
}

int sesp_fp32_peak(int device, double *tflops) {
    if (!tflops) return fail(SESP_EINVAL, "null output");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return fail(SESP_EINVAL, "device %d not available", device);
    CK(cudaSetDevice(device));
    int n_sm = 0;
    CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const double v = measure_fp32_peak(n_sm, st);
    cudaStreamDestroy(st);
    CK(cudaGetLastError());
    if (!(v > 0.0)) return fail(SESP_ECUDA, "FP32 peak measurement failed");
    *tflops = v;
    return 0;
}

int sesp_kernel_times(sesp_ctx *c, double out[8], int reset) {
    if (int e = check_ctx(c, false)) return e;
    if (!out) return fail(SESP_EINVAL, "null output");
    for (int k = 0; k < 8; k++) out[k] = c->t_n[k] ? c->t_acc[k] / c->t_n[k] : 0.0;
    if (reset) for (int k = 0; k < 8; k++) { c->t_acc[k] = 0.0; c->t_n[k] = 0; }
    return 0;
}

int sesp_enable_timing(sesp_ctx *c, int on) {
    if (int e = check_ctx(c, false)) return e;
    c->timing = on != 0;
    return 0;
}

}  // extern "C"
