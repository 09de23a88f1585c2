// Constraint halves of the mixed paths: SHAKE (move_*_a) and RATTLE
// (move_*_b) for waters and surfactants in one persistent launch per half
// (src/move_w1_a.f90:36-134, src/move_surfactant_a.f90:36-134,
// src/move_w1_b.f90:30-119, src/move_surfactant_b.f90:30-118).
//
// The FP64 state is split once per call into
//   * the FP64 predictor (positions for SHAKE, velocities for RATTLE), which
//     is written to the state arrays at the start, and
//   * corrections per site (type C: FP64 for SESP_MIXED, FP32 for
//     SESP_MIXED_FP32C), which the Gauss-Seidel sweeps update.
// Each bond's constants are formed once in FP64 and rounded to C: for SHAKE
// from the predictor bond vector P, the old bond vector R, D0 = d^2 - |P|^2
// and R.P; for RATTLE from R and R.V (V the predictor velocity difference).
// A sweep then evaluates, with c the difference of the two sites'
// corrections,
//     d^2 - |P + c|^2 = D0 - c.(c + 2P),     R.(P + c) = R.P + R.c,
//     R.(V + c) = R.V + R.c,
// so nothing cancels.  With FP32 corrections a residual within 2 % of its
// threshold is recomputed in FP64 from the predictor plus the corrections, so
// the sweeps take the decisions an FP64 evaluation of the same state takes.
// At the end the corrections are added to the FP64 state.  Same bond order,
// tolerance tests, iteration limit and failure counting as the FP64 kernels
// of the plain path; only the rounding differs.
//
// Scheduling.  GB300 issues FP64 at one warp instruction per ~19 cycles per
// SM whatever the active lanes, with ~64 cycles of dependent latency.  A water
// (one thread, 3 bonds) is FP64-throughput work; a surfactant (4 lanes, 28
// bonds swept as a wavefront, 8 molecules per warp) is one long FP64
// dependency chain, latency work.  One launch of gridDim = SM count CTAs of
// 8 warps runs both: the first n_scta CTAs start s_warps warps each on the
// surfactant queue (groups of 8 molecules; few chains per SM, so they do not
// wait behind water instructions), every other warp takes items of 32 waters
// from the water queue, and surfactant warps join the water queue when no
// surfactant is left.  The water list is ordered
// by each molecule's sweep count in the previous call (most first, reordered
// at every list rebuild), so the 32 lanes of an item iterate alike and the
// longest items start first.  Which warp takes which molecule changes no
// result: every molecule is computed alone and its kinetic sums are stored
// per molecule.  The queues are atomic counters; the last CTA to finish
// resets them for the next launch.  Nothing waits on another CTA.
#include <type_traits>

#include "k_launch.cuh"

namespace sesp {

namespace {

struct Fast32 {
    double dsq64_w[3], dsq64_s[NBOND];
    double fb64_w[3], fb64_s[NBOND];
    double hfa64_w[3], hfa64_s[NBOND];     // 1 / (2 (1/m_i + 1/m_j))
    double mass64[NTYPE], rm64[NTYPE], rmdt64[NTYPE];
    double dt2m64[NTYPE];                  // dt^2 / (2 m)
    // the FP32 steering terms of the water matrix kernels, rounded once
    // here instead of in every water (GB300 converts at its FP64 rate)
    float rm32_w[2];                       // (float) rm64 of O and H
    float wk32[3][3];                      // (float) K_bc of the water triangle
};
__constant__ Fast32 cF;

// surfactant bond graph of src/init_arrays.f90:229-264: bond b joins site
// b + 1 to the earlier site sbi32(b) (checked against the uploaded
// tables on the host)
// {0, 1, ..., 17, 17, 19, 20, 20, 20, 17, 24, 25, 25, 25}
__host__ __device__ constexpr int sbi32(int b) {
    return b < 18 ? b : b == 18 ? 17 : b == 19 ? 19 : b <= 22 ? 20 : b == 23 ? 17 : b == 24 ? 24 : 25;
}

// 1 / b: the FP32 estimate and one Newton step in FP64, relative error
// ~2^-46 (for step lengths and scale factors, whose last bits matter to
// nothing; GB300's FP64 division costs ~15 FP64 instructions)
__device__ __forceinline__ double recip64(double b) {
    const double y = (double)__frcp_rn((float)b);
    return fma(y, fma(-b, y, 1.0), y);
}

// the FP64 predictors of the FP64 kernels, rounded the same way
__device__ inline double pred_a(double x, double v, double a, double escale) {
    return __dadd_rn(__dadd_rn(x, __dmul_rn(v, escale)), a);
}
__device__ inline double vel_a(double v, double a, double escale) { return __dadd_rn(__dmul_rn(v, escale), a); }


// SHAKE decision in FP64 for a residual near its threshold: predictor
// difference (state arrays hold the predictor) plus the FP32 corrections
__device__ __noinline__ bool shake_active64(const Dev &d, int gi, int gj, float dxi, float dyi, float dzi, float dxj,
                                            float dyj, float dzj, double dsq, double tol2) {
    double px = __dadd_rn(__dsub_rn(d.x[gi], d.x[gj]), __dsub_rn((double)dxi, (double)dxj));
    double py = __dadd_rn(__dsub_rn(d.y[gi], d.y[gj]), __dsub_rn((double)dyi, (double)dyj));
    double pz = __dadd_rn(__dsub_rn(d.z[gi], d.z[gj]), __dsub_rn((double)dzi, (double)dzj));
    double pabsq = __dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz));
    double diffsq = __dsub_rn(dsq, pabsq);
    return fabs(diffsq) > __dmul_rn(dsq, tol2);
}

// RATTLE decision in FP64 (state arrays hold positions and the velocity
// predictor), the FP64 kernels' formula -(r.v / DT) / ((1/mi + 1/mj) d^2)
__device__ __noinline__ bool rattle_active64(const Dev &d, int gi, int gj, int ki, int kj, float dvxi, float dvyi,
                                             float dvzi, float dvxj, float dvyj, float dvzj, double dsq, double tol) {
    double vx = __dadd_rn(__dsub_rn(d.vx[gi], d.vx[gj]), __dsub_rn((double)dvxi, (double)dvxj));
    double vy = __dadd_rn(__dsub_rn(d.vy[gi], d.vy[gj]), __dsub_rn((double)dvyi, (double)dvyj));
    double vz = __dadd_rn(__dsub_rn(d.vz[gi], d.vz[gj]), __dsub_rn((double)dvzi, (double)dvzj));
    double rx = __dsub_rn(d.x[gi], d.x[gj]), ry = __dsub_rn(d.y[gi], d.y[gj]), rz = __dsub_rn(d.z[gi], d.z[gj]);
    double rv = __dadd_rn(__dadd_rn(__dmul_rn(rx, vx), __dmul_rn(ry, vy)), __dmul_rn(rz, vz));
    double g = -__ddiv_rn(__ddiv_rn(rv, DT), __dmul_rn(__dadd_rn(cF.rm64[ki], cF.rm64[kj]), dsq));
    return fabs(g) > tol;
}

constexpr float BAND = 0.02f;   // relative half-width of the FP64 decision band of the FP32 sweeps
constexpr unsigned FULL = 0xffffffffu;

// |x| > t for t > 0: on the IEEE bit patterns for FP64, so the test runs on
// the integer pipe (GB300's FP64 pipe takes ~19 cycles per warp instruction
// whatever the active lanes, and 64 cycles of latency)
__device__ __forceinline__ bool gt_abs(double x, double t) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > __double_as_longlong(t);
}
__device__ __forceinline__ bool gt_abs(float x, float t) { return fabsf(x) > t; }

// Per-bond constants, formed once per call in FP64 and rounded to C.
// SHAKE, with P and R the predictor and old bond vectors, rp = R.P and
// y0 = 1 / (2 (1/m_i + 1/m_j) rp): 2P, R / rp, the correction directions
// R / m_i and R / m_j, D0 = d^2 - |P|^2, y0 and the threshold 2 tol d^2 (and
// one unused slot, so a record is 16 values).
template <typename C>
struct ShakeK {
    C p2[3], rr[3], a[3], b[3], d0, y0, thr, pad;
};
// RATTLE, with fb = (1/dt) / ((1/m_i + 1/m_j) d^2): -fb R, the correction
// directions R dt / m_i and R dt / m_j, -fb R.V of the velocity predictor
// (and one unused slot: 11 values).
template <typename C>
struct RattleK {
    C rs[3], a[3], b[3], rvs, pad;
};

template <typename C>
__device__ inline void shake_make(double rx, double ry, double rz, double px, double py, double pz, double dsq,
                                  double rmi, double rmj, double hfa, double tol2, ShakeK<C> &k) {
    const double rp = rx * px + ry * py + rz * pz;
    const double irp = recip64(rp);
    const double y0 = hfa * irp;
    k.p2[0] = (C)(2.0 * px); k.p2[1] = (C)(2.0 * py); k.p2[2] = (C)(2.0 * pz);
    k.rr[0] = (C)(rx * irp); k.rr[1] = (C)(ry * irp); k.rr[2] = (C)(rz * irp);
    k.a[0] = (C)(rmi * rx); k.a[1] = (C)(rmi * ry); k.a[2] = (C)(rmi * rz);
    k.b[0] = (C)(rmj * rx); k.b[1] = (C)(rmj * ry); k.b[2] = (C)(rmj * rz);
    k.d0 = (C)(dsq - (px * px + py * py + pz * pz));
    k.y0 = (C)y0;
    k.thr = (C)(dsq * tol2);
    k.pad = C(0);
}
template <typename C>
__device__ inline void rattle_make(double rx, double ry, double rz, double wx, double wy, double wz, double dti,
                                   double dtj, double fb, RattleK<C> &k) {
    k.rs[0] = (C)(-fb * rx); k.rs[1] = (C)(-fb * ry); k.rs[2] = (C)(-fb * rz);
    k.a[0] = (C)(dti * rx); k.a[1] = (C)(dti * ry); k.a[2] = (C)(dti * rz);
    k.b[0] = (C)(dtj * rx); k.b[1] = (C)(dtj * ry); k.b[2] = (C)(dtj * rz);
    k.rvs = (C)(-fb * (rx * wx + ry * wy + rz * wz));
    k.pad = C(0);
}

// One SHAKE bond update on the corrections of its two sites; true if the
// bond was corrected.  With c the difference of the sites' corrections the
// residual is d^2 - |P + c|^2 = D0 - c.(c + 2P), formed as one chain of
// FMAs from D0, so nothing cancels.  The step divides it by
// 2 (1/m_i + 1/m_j) R.(P + c) = (1 + t) / y0 with t = R.c / R.P, a few
// per cent at most; 1 / (1 + t) is taken as (1 - t)(1 + t^2)(1 + t^4),
// relative error t^8, which leaves the converged state within rounding of
// the exact quotient's (the tolerance test is on the residual itself;
// stopping at t^4 already moved ~1 % of the sites by more than 1e-8).
// FP64 operations per bond: 9 for the test, 16 more for a correction (with
// a full quotient 13 more, on a longer dependent chain).
template <typename C>
__device__ __forceinline__ bool shake_bond(const Dev &d, int gi, int gj, double dsq64, double tol2d, const ShakeK<C> &k,
                                           C &xi, C &yi, C &zi, C &xj, C &yj, C &zj) {
    const C dx = xi - xj, dy = yi - yj, dz = zi - zj;
    const C wx = dx + k.p2[0], wy = dy + k.p2[1], wz = dz + k.p2[2];
    C diffsq = fma(-dx, wx, k.d0);
    diffsq = fma(-dy, wy, diffsq);
    diffsq = fma(-dz, wz, diffsq);
    bool act = gt_abs(diffsq, k.thr);
    if constexpr (sizeof(C) == 4) {
        if (fabsf(fabsf(diffsq) - k.thr) < BAND * k.thr)
            act = shake_active64(d, gi, gj, xi, yi, zi, xj, yj, zj, dsq64, tol2d);
    }
    if (act) {   // the step only for a corrected bond: a bond within tolerance costs 9 operations
        C t = k.rr[2] * dz;
        t = fma(k.rr[1], dy, t);
        t = fma(k.rr[0], dx, t);
        const C t2 = t * t;
        const C ya = fma(-k.y0, t, k.y0), yb = fma(t, t, C(1)), yc = fma(t2, t2, C(1));
        const C gab = (diffsq * ya) * (yb * yc);
        xi += k.a[0] * gab; yi += k.a[1] * gab; zi += k.a[2] * gab;
        xj -= k.b[0] * gab; yj -= k.b[1] * gab; zj -= k.b[2] * gab;
    }
    return act;
}

// One RATTLE bond update: g = -fb R.(V + c) = -fb R.V + (-fb R).c, one FMA
// chain (the factor fb folded into the constants).
template <typename C>
__device__ __forceinline__ bool rattle_bond(const Dev &d, int gi, int gj, int ki, int kj, double dsq64, double told,
                                            C tolc, const RattleK<C> &k, C &xi, C &yi, C &zi, C &xj, C &yj, C &zj) {
    const C dx = xi - xj, dy = yi - yj, dz = zi - zj;
    C gab = fma(k.rs[0], dx, k.rvs);
    gab = fma(k.rs[1], dy, gab);
    gab = fma(k.rs[2], dz, gab);
    bool act = gt_abs(gab, tolc);
    if constexpr (sizeof(C) == 4) {
        if (fabsf(fabsf(gab) - tolc) < BAND * tolc)
            act = rattle_active64(d, gi, gj, ki, kj, xi, yi, zi, xj, yj, zj, dsq64, told);
    }
    if (act) {
        xi += k.a[0] * gab; yi += k.a[1] * gab; zi += k.a[2] * gab;
        xj -= k.b[0] * gab; yj -= k.b[1] * gab; zj -= k.b[2] * gab;
    }
    return act;
}

// ---------------------------------------------------------------- waters

// bonds (0,1), (1,2), (2,0); kinds 0 (O), 1 (H)
__host__ __device__ constexpr int wbi(int b) { return b; }
__host__ __device__ constexpr int wbj(int b) { return b == 2 ? 0 : b + 1; }
__host__ __device__ constexpr int wkind(int i) { return i == 0 ? 0 : 1; }

// SHAKE half of one water (one thread); returns the sweeps it ran
template <typename C>
__device__ __forceinline__ int water_a(const Dev &d, int m, double tol, int maxit) {
    const int g0 = d.mfirst[m];
    const double escale = __dsub_rn(1.0, __dmul_rn(d.eta[d.mrep[m]], DT) * 0.5);
    double rx[3], ry[3], rz[3], px[3], py[3], pz[3];
    double ke0 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        double vx = d.vx[g], vy = d.vy[g], vz = d.vz[g], ax = d.ax[g], ay = d.ay[g], az = d.az[g];
        rx[i] = d.x[g]; ry[i] = d.y[g]; rz[i] = d.z[g];
        ke0 = __dadd_rn(ke0, __dmul_rn(cF.mass64[wkind(i)],
                                       __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
        px[i] = pred_a(rx[i], vx, ax, escale);
        py[i] = pred_a(ry[i], vy, ay, escale);
        pz[i] = pred_a(rz[i], vz, az, escale);
        d.x[g] = px[i]; d.y[g] = py[i]; d.z[g] = pz[i];
        d.vx[g] = vel_a(vx, ax, escale);
        d.vy[g] = vel_a(vy, ay, escale);
        d.vz[g] = vel_a(vz, az, escale);
    }
    const double tol2d = 2.0 * tol;
    ShakeK<C> k[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int i = wbi(b), j = wbj(b);
        shake_make<C>(rx[i] - rx[j], ry[i] - ry[j], rz[i] - rz[j], px[i] - px[j], py[i] - py[j], pz[i] - pz[j],
                      cF.dsq64_w[b], cF.rm64[wkind(i)], cF.rm64[wkind(j)], cF.hfa64_w[b], tol2d, k[b]);
    }
    C cx[3] = {0, 0, 0}, cy[3] = {0, 0, 0}, cz[3] = {0, 0, 0};
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int i = wbi(b), j = wbj(b);
            if (shake_bond<C>(d, g0 + i, g0 + j, cF.dsq64_w[b], tol2d, k[b], cx[i], cy[i], cz[i], cx[j], cy[j],
                                     cz[j]))
                ldone = false;
        }
        it++;
    }
    double ke1 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        d.x[g] = __dadd_rn(px[i], (double)cx[i]);
        d.y[g] = __dadd_rn(py[i], (double)cy[i]);
        d.z[g] = __dadd_rn(pz[i], (double)cz[i]);
        double vx = __dadd_rn(d.vx[g], (double)cx[i]), vy = __dadd_rn(d.vy[g], (double)cy[i]),
               vz = __dadd_rn(d.vz[g], (double)cz[i]);
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        ke1 = __dadd_rn(ke1, __dmul_rn(cF.mass64[wkind(i)],
                                       __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
    }
    d.ke[2 * m] = ke0;
    d.ke[2 * m + 1] = ke1;
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
    return it;
}

// RATTLE half of one water (one thread); returns the sweeps it ran
template <typename C>
__device__ __forceinline__ int water_b(const Dev &d, int m, double tol, int maxit) {
    const int g0 = d.mfirst[m];
    const double escale = 2.0 * recip64(__dadd_rn(2.0, __dmul_rn(d.eta[d.mrep[m]], DT)));
    double rx[3], ry[3], rz[3], vx[3], vy[3], vz[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        const double h = cF.dt2m64[wkind(i)];
        const double ax = d.fx[g] * h, ay = d.fy[g] * h, az = d.fz[g] * h;
        d.ax[g] = ax; d.ay[g] = ay; d.az[g] = az;
        vx[i] = __dmul_rn(escale, __dadd_rn(d.vx[g], ax));
        vy[i] = __dmul_rn(escale, __dadd_rn(d.vy[g], ay));
        vz[i] = __dmul_rn(escale, __dadd_rn(d.vz[g], az));
        d.vx[g] = vx[i]; d.vy[g] = vy[i]; d.vz[g] = vz[i];
        rx[i] = d.x[g]; ry[i] = d.y[g]; rz[i] = d.z[g];
    }
    RattleK<C> k[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int i = wbi(b), j = wbj(b);
        rattle_make<C>(rx[i] - rx[j], ry[i] - ry[j], rz[i] - rz[j], vx[i] - vx[j], vy[i] - vy[j], vz[i] - vz[j],
                       cF.rmdt64[wkind(i)], cF.rmdt64[wkind(j)], cF.fb64_w[b], k[b]);
    }
    C cx[3] = {0, 0, 0}, cy[3] = {0, 0, 0}, cz[3] = {0, 0, 0};
    const C tolc = (C)tol;
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int i = wbi(b), j = wbj(b);
            if (rattle_bond<C>(d, g0 + i, g0 + j, wkind(i), wkind(j), cF.dsq64_w[b], tol, tolc, k[b], cx[i], cy[i],
                               cz[i], cx[j], cy[j], cz[j]))
                ldone = false;
        }
        it++;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        d.vx[g] = __dadd_rn(vx[i], (double)cx[i]);
        d.vy[g] = __dadd_rn(vy[i], (double)cy[i]);
        d.vz[g] = __dadd_rn(vz[i], (double)cz[i]);
    }
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
    return it;
}

// ---------------------------------------------------------------- waters in matrix form

// Configuration preset, mixed path: the SHAKE / RATTLE of a water as the 3 x 3
// system of its three constraints (matrix SHAKE: Kraeutler, van Gunsteren and
// Huenenberger, J. Comput. Chem. 22, 501 (2001)).  The corrections keep
// SHAKE's form - bond b moves its sites along its old bond vector R_b,
// site k by g_b s_kb R_b / m_k (s = +1 for the bond's first site, -1 for its
// second) - and the same stopping test, |d^2 - |P_b|^2| <= 2 tol d^2 for
// every bond; only the update differs: instead of Gauss-Seidel sweeps over
// the bonds (about 31 of them at this preset's tolerance 1e-8, where the
// water triangle's coupling slows them), Newton steps with the Jacobian of
// the predictor, J_bc = -2 P_b . K_bc R_c (K_bc = dP_b / d(g_c R_c)), about 4
// at 1e-8.  RATTLE's constraints R_b . V_b = 0 are linear in the corrections:
// one solve of A h = -R.V (A_bc = R_b . K_bc R_c) meets them, checked with
// RATTLE's own test.  Both converge to the constrained state the sweeps
// approach, so the result differs from the sweeps' by less than the
// tolerance.  The 3 x 3 matrices, their inverses and the steps are FP32
// (GB300 issues FP32 at 64 times its FP64 rate): they only steer.  The
// residuals, the tolerance tests, the state and the sums of the corrections
// stay FP64.  A FP32 residual resolves only about the tolerance band, so the
// last step or two start from the FP64 residual.

// K_bc of the water triangle (bond b joins sites b and b + 1 mod 3): the
// sum of the inverse masses on the diagonal, minus the inverse mass of the
// shared site off it (FP64; rounded to FP32 once, into cF.wk32)
inline double wk_host(const double *rm, int b, int c) {
    if (b == c) return rm[wkind(wbi(b))] + rm[wkind(wbj(b))];
    const int shared = (wbi(b) == wbi(c) || wbi(b) == wbj(c)) ? wbi(b) : wbj(b);
    return -rm[wkind(shared)];
}
// s_kb: +1 if site k is bond b's first site, -1 if its second, else 0
__device__ __forceinline__ double wsgn(int k, int b) { return k == wbi(b) ? 1.0 : (k == wbj(b) ? -1.0 : 0.0); }

__device__ __forceinline__ void inv3f(const float (&A)[3][3], float (&B)[3][3]) {
    B[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    B[0][1] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
    B[0][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
    B[1][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    B[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
    B[1][2] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
    B[2][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    B[2][1] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
    B[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    const float id = 1.f / (A[0][0] * B[0][0] + A[0][1] * B[1][0] + A[0][2] * B[2][0]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) B[i][j] *= id;
}

// site corrections of bond multipliers h: site k moves by s_kb h_b R_b / m_k
__device__ __forceinline__ void water_move32(const float (&R)[3][3], const float (&h)[3], float (&c)[3][3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float rm = cF.rm32_w[wkind(k)];
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const float w = (float)wsgn(k, b) * rm * h[b];
            if (w != 0.f) { c[k][0] += w * R[b][0]; c[k][1] += w * R[b][1]; c[k][2] += w * R[b][2]; }
        }
    }
}

// one Newton step on the corrections from residuals f: g = -J^-1 f
__device__ __forceinline__ void water_step32(const float (&Ji)[3][3], const float (&R)[3][3], const float (&f)[3],
                                             float (&c)[3][3]) {
    float g[3];
#pragma unroll
    for (int b = 0; b < 3; b++) g[b] = -(Ji[b][0] * f[0] + Ji[b][1] * f[1] + Ji[b][2] * f[2]);
    water_move32(R, g, c);
}

// FP32 Newton steps of a water's SHAKE before its FP64 tests (about 4 meet
// the FP32 residual's resolution)
constexpr int WMAT_FP32_STEPS = 8;

// SHAKE half of one water in matrix form; returns the Newton steps it ran
__device__ __forceinline__ int water_a_mat(const Dev &d, int m, double tol, int maxit) {
    const int g0 = d.mfirst[m];
    const double escale = __dsub_rn(1.0, __dmul_rn(d.eta[d.mrep[m]], DT) * 0.5);
    // (the velocity predictor is formed again at the end from the state, so
    // it holds no registers through the iterations)
    double r[3][3], p[3][3];
    double ke0 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        const double vx = d.vx[g], vy = d.vy[g], vz = d.vz[g], ax = d.ax[g], ay = d.ay[g], az = d.az[g];
        r[i][0] = d.x[g]; r[i][1] = d.y[g]; r[i][2] = d.z[g];
        ke0 = __dadd_rn(ke0, __dmul_rn(cF.mass64[wkind(i)],
                                       __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
        p[i][0] = pred_a(r[i][0], vx, ax, escale);
        p[i][1] = pred_a(r[i][1], vy, ay, escale);
        p[i][2] = pred_a(r[i][2], vz, az, escale);
    }
    double R[3][3], P[3][3], D0[3], thr[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int i = wbi(b), j = wbj(b);
#pragma unroll
        for (int a = 0; a < 3; a++) { R[b][a] = r[i][a] - r[j][a]; P[b][a] = p[i][a] - p[j][a]; }
        D0[b] = cF.dsq64_w[b] - (P[b][0] * P[b][0] + P[b][1] * P[b][1] + P[b][2] * P[b][2]);
        thr[b] = cF.dsq64_w[b] * (2.0 * tol);
    }
    // the Jacobian and its inverse in FP32: they only steer the steps
    float R32[3][3], P32[3][3], J[3][3], Ji[3][3];
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int a = 0; a < 3; a++) { R32[b][a] = (float)R[b][a]; P32[b][a] = (float)P[b][a]; }
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            J[b][c] = -2.f * cF.wk32[b][c] * (P32[b][0] * R32[c][0] + P32[b][1] * R32[c][1] + P32[b][2] * R32[c][2]);
    inv3f(J, Ji);
    // FP32 steps on the corrections until the FP32 residual is inside the
    // tolerance (its rounding, ~1e-9 of d^2 ~ 0.1, is about the tolerance
    // band itself, so these only bring the corrections near the answer)
    float c32[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    const float D0f[3] = {(float)D0[0], (float)D0[1], (float)D0[2]};
    const float thrf[3] = {(float)thr[0], (float)thr[1], (float)thr[2]};
    int it = 0;
    for (int k32 = 0; k32 < WMAT_FP32_STEPS && it <= maxit; k32++) {
        float f[3];
        bool in = true;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int i = wbi(b), j = wbj(b);
            float q = 0.f;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float cd = c32[i][a] - c32[j][a];
                q += cd * (cd + 2.f * P32[b][a]);
            }
            f[b] = D0f[b] - q;
            in = in && !(fabsf(f[b]) > thrf[b]);
        }
        if (in) break;
        water_step32(Ji, R32, f, c32);
        it++;
    }
    double cc[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int a = 0; a < 3; a++) cc[k][a] = (double)c32[k][a];
    // the tolerance test in FP64, as the reference's; a failed test takes
    // one more step from the FP64 residual (solved in FP32: it is small)
    bool done = false;
    while (it <= maxit) {
        double f[3];
        done = true;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int i = wbi(b), j = wbj(b);
            double q = 0.0;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const double cd = cc[i][a] - cc[j][a];
                q += cd * (cd + 2.0 * P[b][a]);
            }
            f[b] = D0[b] - q;   // d^2 - |P_b + c_i - c_j|^2
            done = done && !(fabs(f[b]) > thr[b]);
        }
        if (done) break;
        float f32[3] = {(float)f[0], (float)f[1], (float)f[2]}, d32[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        water_step32(Ji, R32, f32, d32);
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int a = 0; a < 3; a++) cc[k][a] += (double)d32[k][a];
        it++;
    }
    double ke1 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        const double v0 = vel_a(d.vx[g], d.ax[g], escale), v1 = vel_a(d.vy[g], d.ay[g], escale),
                     v2 = vel_a(d.vz[g], d.az[g], escale);
        d.x[g] = p[i][0] + cc[i][0]; d.y[g] = p[i][1] + cc[i][1]; d.z[g] = p[i][2] + cc[i][2];
        const double vx = v0 + cc[i][0], vy = v1 + cc[i][1], vz = v2 + cc[i][2];
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        ke1 = __dadd_rn(ke1, __dmul_rn(cF.mass64[wkind(i)],
                                       __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
    }
    d.ke[2 * m] = ke0;
    d.ke[2 * m + 1] = ke1;
    if (!done) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
    return it + 1;
}

// RATTLE half of one water in matrix form; returns the solves it ran
__device__ __forceinline__ int water_b_mat(const Dev &d, int m, double tol, int maxit) {
    const int g0 = d.mfirst[m];
    const double escale = 2.0 * recip64(__dadd_rn(2.0, __dmul_rn(d.eta[d.mrep[m]], DT)));
    double r[3][3], v[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        const double h = cF.dt2m64[wkind(i)];
        const double ax = d.fx[g] * h, ay = d.fy[g] * h, az = d.fz[g] * h;
        d.ax[g] = ax; d.ay[g] = ay; d.az[g] = az;
        v[i][0] = __dmul_rn(escale, __dadd_rn(d.vx[g], ax));
        v[i][1] = __dmul_rn(escale, __dadd_rn(d.vy[g], ay));
        v[i][2] = __dmul_rn(escale, __dadd_rn(d.vz[g], az));
        r[i][0] = d.x[g]; r[i][1] = d.y[g]; r[i][2] = d.z[g];
    }
    double R[3][3];
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int a = 0; a < 3; a++) R[b][a] = r[wbi(b)][a] - r[wbj(b)][a];
    // the matrix and its inverse in FP32 (they steer the solve; the test is FP64)
    float R32[3][3], A[3][3], Ai[3][3];
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++) R32[b][c] = (float)R[b][c];
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            A[b][c] = cF.wk32[b][c] * (R32[b][0] * R32[c][0] + R32[b][1] * R32[c][1] + R32[b][2] * R32[c][2]);
    inv3f(A, Ai);
    int it = 0;
    bool done = false;
    while (it <= maxit) {
        double rv[3];
        done = true;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int i = wbi(b), j = wbj(b);
            rv[b] = R[b][0] * (v[i][0] - v[j][0]) + R[b][1] * (v[i][1] - v[j][1]) + R[b][2] * (v[i][2] - v[j][2]);
            // RATTLE's test: -(R.V / dt) / ((1/m_i + 1/m_j) d^2)
            done = done && !(fabs(cF.fb64_w[b] * rv[b]) > tol);
        }
        if (done) break;
        // A h = -R.V in FP32 (R.V is small: the rounding of h is far below the tolerance)
        float rv32[3] = {(float)rv[0], (float)rv[1], (float)rv[2]}, d32[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        float h[3];
#pragma unroll
        for (int b = 0; b < 3; b++) h[b] = -(Ai[b][0] * rv32[0] + Ai[b][1] * rv32[1] + Ai[b][2] * rv32[2]);
        water_move32(R32, h, d32);
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int a = 0; a < 3; a++) v[k][a] += (double)d32[k][a];
        it++;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        d.vx[g] = v[i][0]; d.vy[g] = v[i][1]; d.vz[g] = v[i][2];
    }
    if (!done) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
    return it + 1;
}

// ---------------------------------------------------------------- surfactants

// Gauss-Seidel sweeps as a wavefront: sweep k starts WF_LAG bonds after
// sweep k - 1 and runs on wavefront lane k mod WF_LANES, one bond per lane
// and step.  Two bonds that share a site are never more than 7 apart in the
// bond order (site 17: bonds 16 and 23), so with a lag of 8 every site sees
// the updates of the sequential order, in that order, and no two lanes touch
// the same site in one step: the result is that of the sequential sweeps.
// Sweeps started after the first sweep without a correction make no
// correction either (they see the same, converged state), so the state at
// that point is final.  No more than maxit + 1 sweeps run, as in the
// sequential loop.
//
// A warp carries up to MPW = 8 molecules, one per group of 4 lanes (the
// launch picks how many: mpw).  An FP64 warp instruction costs a scheduler
// partition ~64 cycles whatever its active lanes, so a wavefront step costs
// the same for 1 molecule as for 8: more molecules per warp is more
// throughput for many surfactants, while with one molecule per warp a step
// whose 4 bonds all lie within tolerance more often skips the correction
// arithmetic.  Each group stops when its molecule has converged or failed;
// the warp stops when all have.
constexpr int WF_LAG = 8;
constexpr int WF_LANES = 4;   // ceil(NBOND / WF_LAG) sweeps in flight
constexpr int MPW = 32 / WF_LANES;   // molecules per warp

// Shared memory of one molecule: bond records and site corrections
// field-major with the index skewed by one slot every 8 (i -> i + i / 8), so
// the four lanes of a wavefront step (bonds b, b-8, b-16, b-24 and their
// sites) fall on different banks; the FP64 site vectors of the setup; and a
// stagger of 4 slots, so that the 8 molecules of a warp, whose lanes access
// the same offsets in the same step, fall on different banks as well.
__device__ __forceinline__ int skew8(int i) { return i + (i >> 3); }
constexpr int SK = 32;   // padded length (largest skewed index 28 + 3)
template <typename C, int NF>
struct MolSmem {
    C rec[NF][SK];
    C sc[3][SK];
    double sv[6][SK];   // per site: old position, then predictor position (SHAKE) or velocity (RATTLE)
    double kes[SK];     // per site m v^2 (SHAKE)
    C stagger[4];
    template <typename K>
    __device__ void put(int b, const K &k) {
        const C *f = reinterpret_cast<const C *>(&k);
#pragma unroll
        for (int q = 0; q < NF; q++) rec[q][skew8(b)] = f[q];
    }
    template <typename K>
    __device__ void get(int b, K &k) const {
        C *f = reinterpret_cast<C *>(&k);
#pragma unroll
        for (int q = 0; q < NF; q++) f[q] = rec[q][skew8(b)];
    }
};

// sum over the 4 lanes of a group (fixed order), result in every lane of it
__device__ __forceinline__ double group_sum(double v) {
    v += __shfl_xor_sync(FULL, v, 1);
    v += __shfl_xor_sync(FULL, v, 2);
    return v;
}

// The wavefront of SHAKE (SHAKE = true) or RATTLE over the 8 molecules of a
// warp.  Lane (g, w): molecule g, wavefront lane w.  Returns through fail
// whether its molecule ran out of sweeps.
// The wavefront with one bond per lane (FP32 corrections): lane (g, w),
// molecule g of the warp, wavefront lane w.  Returns a ballot whose bit 4g
// is set if molecule g ran out of sweeps.
template <typename C, bool SHAKE>
__device__ __forceinline__ unsigned surf_wavefront(const Dev &d, MolSmem<C, SHAKE ? 16 : 11> *sms, int g0, int n,
                                                   double tol, int maxit) {
    const int lane = threadIdx.x & 31, w = lane & (WF_LANES - 1), grp = lane >> 2;
    const unsigned gmask = 0xFu << (4 * grp);
    MolSmem<C, SHAKE ? 16 : 11> &sm = sms[grp < n ? grp : 0];
    const double tol2d = 2.0 * tol;
    const C tolc = (C)tol;
    int kmine = w;
    bool changed = false, done = grp >= n, fail = false;
    for (int t = 0;; t++) {
        bool clean = false, last = false;
        const int b = t - WF_LAG * kmine;
        if (!done && kmine <= maxit && b >= 0 && b < NBOND) {
            const int i = sbi32(b), j = b + 1, si = skew8(i), sj = skew8(j);
            C xi = sm.sc[0][si], yi = sm.sc[1][si], zi = sm.sc[2][si];
            C xj = sm.sc[0][sj], yj = sm.sc[1][sj], zj = sm.sc[2][sj];
            bool act;
            if constexpr (SHAKE) {
                ShakeK<C> k;
                sm.get(b, k);
                act = shake_bond<C>(d, g0 + i, g0 + j, cF.dsq64_s[b], tol2d, k, xi, yi, zi, xj, yj, zj);
            } else {
                RattleK<C> k;
                sm.get(b, k);
                act = rattle_bond<C>(d, g0 + i, g0 + j, 2 + i, 2 + j, cF.dsq64_s[b], tol, tolc, k, xi, yi, zi, xj, yj,
                                     zj);
            }
            if (act) {
                sm.sc[0][si] = xi; sm.sc[1][si] = yi; sm.sc[2][si] = zi;
                sm.sc[0][sj] = xj; sm.sc[1][sj] = yj; sm.sc[2][sj] = zj;
                changed = true;
            }
            if (b == NBOND - 1) {
                clean = !changed;
                last = changed && kmine == maxit;
                changed = false;
                kmine += WF_LANES;
            }
        }
        __syncwarp();
        const unsigned bc = __ballot_sync(FULL, clean), bl = __ballot_sync(FULL, last);
        if (!done) {
            if (bc & gmask) done = true;
            else if (bl & gmask) { done = true; fail = true; }
        }
        if (__all_sync(FULL, done)) break;
    }
    return __ballot_sync(FULL, fail && w == 0);
}

// sum of v over lanes base, base + 1, base + 2 (the same bits in all three)
__device__ __forceinline__ double tri_sum(double v, int base) {
    const double v0 = __shfl_sync(FULL, v, base), v1 = __shfl_sync(FULL, v, base + 1),
                 v2 = __shfl_sync(FULL, v, base + 2);
    return (v0 + v1) + v2;
}

// The wavefront for FP64 corrections with each bond split over 3 lanes, one
// per Cartesian component: lane 12 q + 3 w + k works on component k of
// wavefront lane w of molecule q (q < 2; lanes 24..31 idle).  Every FP64
// warp instruction costs the same whatever its active lanes, so splitting
// the components takes a SHAKE bond from 25 to 18 FP64 warp instructions
// (9 to 6 for a bond within tolerance) and a RATTLE bond from 12 to 7; the
// two dot products go over shuffles.  Returns a ballot whose bit 12 q is set
// if molecule q ran out of sweeps.
template <bool SHAKE>
__device__ __forceinline__ unsigned surf_wavefront3(const Dev &d, MolSmem<double, SHAKE ? 16 : 11> *sms, int n,
                                                    double tol, int maxit) {
    const int lane = threadIdx.x & 31;
    const int q = lane < 24 ? lane / 12 : 0, r = lane - 12 * q, w = lane < 24 ? r / 3 : 0, k = lane < 24 ? r % 3 : 0;
    const int base = lane - k;
    const unsigned gmask = 0xFFFu << (12 * q);
    MolSmem<double, SHAKE ? 16 : 11> &sm = sms[q < n ? q : 0];
    double *rec = &sm.rec[0][0];
    int kmine = w;
    bool changed = false, done = lane >= 24 || q >= n, fail = false;
    for (int t = 0;; t++) {
        bool clean = false, last = false;
        const int b = t - WF_LAG * kmine;
        const bool valid = !done && kmine <= maxit && b >= 0 && b < NBOND;
        const int sb = skew8(valid ? b : 0), i = valid ? sbi32(b) : 0, si = skew8(i), sj = skew8(valid ? b + 1 : 0);
        double ci = 0.0, cj = 0.0, dx = 0.0, pr = 0.0;
        if (valid) {
            ci = sm.sc[k][si];
            cj = sm.sc[k][sj];
            dx = ci - cj;
            pr = SHAKE ? dx * (dx + rec[k * SK + sb]) : rec[k * SK + sb] * dx;   // c_k (c_k + 2P_k)  /  -fb R_k c_k
        }
        const double sum = tri_sum(pr, base);
        double gab = 0.0;
        bool act = false;
        if constexpr (SHAKE) {
            const double diffsq = valid ? rec[12 * SK + sb] - sum : 0.0;   // D0 - c.(c + 2P)
            act = valid && gt_abs(diffsq, rec[14 * SK + sb]);
            if (__any_sync(FULL, act)) {   // the step only when some bond of the warp is corrected
                const double tk = valid ? rec[(3 + k) * SK + sb] * dx : 0.0;
                const double tt = tri_sum(tk, base);
                const double y0 = valid ? rec[13 * SK + sb] : 0.0;
                const double t2 = tt * tt;
                const double ya = fma(-y0, tt, y0), yb = fma(tt, tt, 1.0), yc = fma(t2, t2, 1.0);
                gab = (diffsq * ya) * (yb * yc);
            }
        } else {
            gab = valid ? rec[9 * SK + sb] + sum : 0.0;   // -fb R.(V + c)
            act = valid && gt_abs(gab, tol);
        }
        if (act) {
            const int fa = SHAKE ? 6 : 3, fb = SHAKE ? 9 : 6;
            sm.sc[k][si] = fma(rec[(fa + k) * SK + sb], gab, ci);
            sm.sc[k][sj] = fma(-rec[(fb + k) * SK + sb], gab, cj);
            changed = true;
        }
        if (valid && b == NBOND - 1) {
            clean = !changed;
            last = changed && kmine == maxit;
            changed = false;
            kmine += WF_LANES;
        }
        __syncwarp();
        const unsigned bc = __ballot_sync(FULL, clean), bl = __ballot_sync(FULL, last);
        if (!done) {
            if (bc & gmask) done = true;
            else if (bl & gmask) { done = true; fail = true; }
        }
        if (__all_sync(FULL, done)) break;
    }
    return __ballot_sync(FULL, fail && r == 0 && lane < 24);
}

// whether molecule g of the warp ran out of sweeps, from the wavefront's ballot
template <typename C>
__device__ __forceinline__ bool surf_failed(unsigned ballot, int g) {
    return (ballot >> (sizeof(C) == 8 ? 12 * g : 4 * g)) & 1u;
}

// molecules per warp the wavefront of corrections of type C takes
template <typename C>
__host__ __device__ constexpr int wavefront_mols() { return sizeof(C) == 8 ? 2 : MPW; }

// Per-molecule values of the warp's molecules, held by the lanes of each
// molecule's group and fetched by any lane with a shuffle.
struct SurfMol {
    int m, g0;
    double escale;
};
__device__ __forceinline__ SurfMol surf_mol(const SurfMol &mine, int q) {
    SurfMol o;
    o.m = __shfl_sync(FULL, mine.m, 4 * q);
    o.g0 = __shfl_sync(FULL, mine.g0, 4 * q);
    o.escale = __shfl_sync(FULL, mine.escale, 4 * q);
    return o;
}

// SHAKE half of up to 8 surfactants (the whole warp): molecules mols[0..n).
// The per-site and per-bond work of the n molecules is spread over all 32
// lanes (an FP64 warp instruction costs the same for 4 lanes as for 32), the
// sweeps run in the molecules' groups of 4 lanes.
template <typename C>
__device__ __forceinline__ void surf_a(const Dev &d, const int *mols, int n, double tol, int maxit,
                                       MolSmem<C, 16> *sms) {
    static_assert(sizeof(ShakeK<C>) == 16 * sizeof(C), "ShakeK is 16 values");
    const int lane = threadIdx.x & 31, w = lane & (WF_LANES - 1), grp = lane >> 2;
    const bool live = grp < n;
    SurfMol mine = {0, 0, 0.0};
    if (live) {
        mine.m = mols[grp];
        mine.g0 = d.mfirst[mine.m];
        mine.escale = __dsub_rn(1.0, __dmul_rn(d.eta[d.mrep[mine.m]], DT) * 0.5);
    }
    // sites: predictor, m v^2 before, FP64 site vectors
    for (int base = 0; base < n * NSURF; base += 32) {
        const int it = base + lane, q = it < n * NSURF ? it / NSURF : 0, s = it - q * NSURF;
        const SurfMol mq = surf_mol(mine, q);
        if (it < n * NSURF) {
            MolSmem<C, 16> &sm = sms[q];
            const int g = mq.g0 + s;
            const double vx = d.vx[g], vy = d.vy[g], vz = d.vz[g], ax = d.ax[g], ay = d.ay[g], az = d.az[g];
            const double rx = d.x[g], ry = d.y[g], rz = d.z[g];
            sm.kes[s] = __dmul_rn(cF.mass64[2 + s],
                                  __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz)));
            const double px = pred_a(rx, vx, ax, mq.escale), py = pred_a(ry, vy, ay, mq.escale),
                         pz = pred_a(rz, vz, az, mq.escale);
            d.x[g] = px; d.y[g] = py; d.z[g] = pz;
            d.vx[g] = vel_a(vx, ax, mq.escale);
            d.vy[g] = vel_a(vy, ay, mq.escale);
            d.vz[g] = vel_a(vz, az, mq.escale);
            sm.sv[0][s] = rx; sm.sv[1][s] = ry; sm.sv[2][s] = rz;
            sm.sv[3][s] = px; sm.sv[4][s] = py; sm.sv[5][s] = pz;
            sm.sc[0][skew8(s)] = sm.sc[1][skew8(s)] = sm.sc[2][skew8(s)] = C(0);
        }
    }
    __syncwarp();
    // bonds: constants
    const double tol2d = 2.0 * tol;
    for (int it = lane; it < n * NBOND; it += 32) {
        const int q = it / NBOND, b = it - q * NBOND, i = sbi32(b), j = b + 1;
        MolSmem<C, 16> &sm = sms[q];
        ShakeK<C> k;
        shake_make<C>(sm.sv[0][i] - sm.sv[0][j], sm.sv[1][i] - sm.sv[1][j], sm.sv[2][i] - sm.sv[2][j],
                      sm.sv[3][i] - sm.sv[3][j], sm.sv[4][i] - sm.sv[4][j], sm.sv[5][i] - sm.sv[5][j],
                      cF.dsq64_s[b], cF.rm64[2 + i], cF.rm64[2 + j], cF.hfa64_s[b], tol2d, k);
        sm.put(b, k);
    }
    __syncwarp();
    // kinetic sum before: lane w of a group adds sites w, w + 4, ..., then the group
    double ke0 = 0.0;
    if (live)
        for (int s = w; s < NSURF; s += WF_LANES) ke0 = __dadd_rn(ke0, sms[grp].kes[s]);
    ke0 = group_sum(ke0);
    unsigned failed;
    if constexpr (sizeof(C) == 8) failed = surf_wavefront3<true>(d, sms, n, tol, maxit);
    else failed = surf_wavefront<C, true>(d, sms, mine.g0, n, tol, maxit);
    // sites: positions, velocities, m v^2 after
    for (int it = lane; it < n * NSURF; it += 32) {
        const int q = it / NSURF, s = it - q * NSURF;
        MolSmem<C, 16> &sm = sms[q];
        const int g = d.mfirst[mols[q]] + s;
        const double cxi = sm.sc[0][skew8(s)], cyi = sm.sc[1][skew8(s)], czi = sm.sc[2][skew8(s)];
        d.x[g] = __dadd_rn(sm.sv[3][s], cxi);
        d.y[g] = __dadd_rn(sm.sv[4][s], cyi);
        d.z[g] = __dadd_rn(sm.sv[5][s], czi);
        const double vx = __dadd_rn(d.vx[g], cxi), vy = __dadd_rn(d.vy[g], cyi), vz = __dadd_rn(d.vz[g], czi);
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        sm.kes[s] = __dmul_rn(cF.mass64[2 + s],
                              __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz)));
    }
    __syncwarp();
    double ke1 = 0.0;
    if (live)
        for (int s = w; s < NSURF; s += WF_LANES) ke1 = __dadd_rn(ke1, sms[grp].kes[s]);
    ke1 = group_sum(ke1);
    if (live && w == 0) {
        d.ke[2 * mine.m] = ke0;
        d.ke[2 * mine.m + 1] = ke1;
        if (surf_failed<C>(failed, grp)) { d.mfail[mine.m] += 1; atomicAdd(&d.counters[0], 1ull); }
    }
    __syncwarp();   // the shared records are reused by the warp's next molecules
}

// RATTLE half of up to 8 surfactants (the whole warp), laid out as surf_a
template <typename C>
__device__ __forceinline__ void surf_b(const Dev &d, const int *mols, int n, double tol, int maxit,
                                       MolSmem<C, 11> *sms) {
    static_assert(sizeof(RattleK<C>) == 11 * sizeof(C), "RattleK is 11 values");
    const int lane = threadIdx.x & 31, grp = lane >> 2;
    const bool live = grp < n;
    SurfMol mine = {0, 0, 0.0};
    if (live) {
        mine.m = mols[grp];
        mine.g0 = d.mfirst[mine.m];
        mine.escale = 2.0 * recip64(__dadd_rn(2.0, __dmul_rn(d.eta[d.mrep[mine.m]], DT)));
    }
    for (int base = 0; base < n * NSURF; base += 32) {
        const int it = base + lane, q = it < n * NSURF ? it / NSURF : 0, s = it - q * NSURF;
        const SurfMol mq = surf_mol(mine, q);
        if (it < n * NSURF) {
            MolSmem<C, 11> &sm = sms[q];
            const int g = mq.g0 + s;
            const double h = cF.dt2m64[2 + s];
            const double ax = d.fx[g] * h, ay = d.fy[g] * h, az = d.fz[g] * h;
            d.ax[g] = ax; d.ay[g] = ay; d.az[g] = az;
            const double vx = __dmul_rn(mq.escale, __dadd_rn(d.vx[g], ax));
            const double vy = __dmul_rn(mq.escale, __dadd_rn(d.vy[g], ay));
            const double vz = __dmul_rn(mq.escale, __dadd_rn(d.vz[g], az));
            d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
            sm.sv[0][s] = d.x[g]; sm.sv[1][s] = d.y[g]; sm.sv[2][s] = d.z[g];
            sm.sv[3][s] = vx; sm.sv[4][s] = vy; sm.sv[5][s] = vz;
            sm.sc[0][skew8(s)] = sm.sc[1][skew8(s)] = sm.sc[2][skew8(s)] = C(0);
        }
    }
    __syncwarp();
    for (int it = lane; it < n * NBOND; it += 32) {
        const int q = it / NBOND, b = it - q * NBOND, i = sbi32(b), j = b + 1;
        MolSmem<C, 11> &sm = sms[q];
        RattleK<C> k;
        rattle_make<C>(sm.sv[0][i] - sm.sv[0][j], sm.sv[1][i] - sm.sv[1][j], sm.sv[2][i] - sm.sv[2][j],
                       sm.sv[3][i] - sm.sv[3][j], sm.sv[4][i] - sm.sv[4][j], sm.sv[5][i] - sm.sv[5][j],
                       cF.rmdt64[2 + i], cF.rmdt64[2 + j], cF.fb64_s[b], k);
        sm.put(b, k);
    }
    __syncwarp();
    unsigned failed;
    if constexpr (sizeof(C) == 8) failed = surf_wavefront3<false>(d, sms, n, tol, maxit);
    else failed = surf_wavefront<C, false>(d, sms, mine.g0, n, tol, maxit);
    for (int it = lane; it < n * NSURF; it += 32) {
        const int q = it / NSURF, s = it - q * NSURF;
        MolSmem<C, 11> &sm = sms[q];
        const int g = d.mfirst[mols[q]] + s;
        d.vx[g] = __dadd_rn(sm.sv[3][s], (double)sm.sc[0][skew8(s)]);
        d.vy[g] = __dadd_rn(sm.sv[4][s], (double)sm.sc[1][skew8(s)]);
        d.vz[g] = __dadd_rn(sm.sv[5][s], (double)sm.sc[2][skew8(s)]);
    }
    if (live && (lane & 3) == 0 && surf_failed<C>(failed, grp)) { d.mfail[mine.m] += 1; atomicAdd(&d.counters[0], 1ull); }
    __syncwarp();   // the shared records are reused by the warp's next molecules
}

// ---------------------------------------------------------------- the persistent launch

constexpr int CW = 8;                 // warps per CTA
constexpr int CW_THREADS = 32 * CW;
constexpr int MAX_SURF_WARPS = 4;     // surfactant warps per CTA (shared memory: 8 molecules each)

struct CPlan {
    const int *smols;   // surfactant molecules
    const int *wlist;   // water molecules in work order
    uint8_t *wsw;       // per molecule: sweeps of this half's last call (waters)
    unsigned *ctl;      // [0] next surfactant group, [1] next water item, [2] CTAs finished
    int ns, nw;
    int n_scta;         // CTAs that start on the surfactant queue
    int s_warps;        // surfactant warps in each of them
    int mpw;            // surfactants per warp (groups of 4 lanes), 1..MPW
    int nmol, nsite;    // bounds every listed molecule is checked against
    int mat;            // waters in matrix form (configuration preset, FP64 corrections)
};

// a listed molecule with its nsites sites inside the state arrays; a list
// entry that is not is counted in counters[7] and skipped, never followed
__device__ __forceinline__ bool mol_ok(const Dev &d, const CPlan &p, int m, int nsites) {
    if (m < 0 || m >= p.nmol) return false;
    const int g0 = d.mfirst[m];
    return g0 >= 0 && g0 + nsites <= p.nsite;
}

template <typename C, bool SHAKE>
__global__ void __launch_bounds__(CW_THREADS) k_constrain(Dev d, CPlan p, double tol, int maxit) {
    griddep_wait();
    constexpr int NF = SHAKE ? 16 : 11;
    extern __shared__ __align__(16) unsigned char cs_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool surf_cta = (int)blockIdx.x < p.n_scta;
    if (surf_cta && warp < p.s_warps) {
        MolSmem<C, NF> *sms = reinterpret_cast<MolSmem<C, NF> *>(cs_smem) + p.mpw * warp;
        for (;;) {
            unsigned s = 0;
            if (lane == 0) s = atomicAdd(&p.ctl[0], 1u);
            s = __shfl_sync(FULL, s, 0);
            const long long s0 = (long long)p.mpw * s;
            if (s0 >= p.ns) break;
            const int n = p.ns - (int)s0 < p.mpw ? p.ns - (int)s0 : p.mpw;
            const bool bad = lane < n && !mol_ok(d, p, p.smols[s0 + lane], NSURF);
            if (__any_sync(FULL, bad)) {
                if (lane == 0) atomicAdd(&d.counters[7], 1ull);
                continue;
            }
            if constexpr (SHAKE) surf_a<C>(d, p.smols + s0, n, tol, maxit, sms);
            else surf_b<C>(d, p.smols + s0, n, tol, maxit, sms);
        }
    }
    // the other warps of a surfactant CTA stay idle, so its chains keep the SM's FP64 pipe
    if (!surf_cta || warp < p.s_warps) {
        for (;;) {
            unsigned item = 0;
            if (lane == 0) item = atomicAdd(&p.ctl[1], 1u);
            item = __shfl_sync(FULL, item, 0);
            const long long t0 = 32LL * item;
            if (t0 >= p.nw) break;
            const int t = (int)t0 + lane;
            if (t < p.nw) {
                const int m = p.wlist[t];
                if (!mol_ok(d, p, m, 3)) {
                    atomicAdd(&d.counters[7], 1ull);
                    continue;
                }
                int sweeps;
                if (std::is_same<C, double>::value && p.mat)
                    sweeps = SHAKE ? water_a_mat(d, m, tol, maxit) : water_b_mat(d, m, tol, maxit);
                else
                    sweeps = SHAKE ? water_a<C>(d, m, tol, maxit) : water_b<C>(d, m, tol, maxit);
                p.wsw[m] = (uint8_t)(sweeps < 255 ? sweeps : 255);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // every CTA counts itself once it has left both queues; the last one
        // (all others have stopped taking work) resets them for the next launch
        __threadfence();
        if (atomicAdd(&p.ctl[2], 1u) == gridDim.x - 1) { p.ctl[0] = 0u; p.ctl[1] = 0u; p.ctl[2] = 0u; }
    }
}

// Configuration preset, mixed path: its chains carry no constraints, so the
// half is the water queue of k_constrain alone (matrix form), in a kernel
// without the surfactant wavefront's registers and shared memory: several
// CTAs per SM instead of one, to hide the FP64 latency of the per-water
// chains.  Same queue, same per-water arithmetic, same counter reset.
template <bool SHAKE>
__global__ void __launch_bounds__(CW_THREADS) k_water_mat(Dev d, CPlan p, double tol, int maxit) {
    griddep_wait();
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned item = 0;
        if (lane == 0) item = atomicAdd(&p.ctl[1], 1u);
        item = __shfl_sync(FULL, item, 0);
        const long long t0 = 32LL * item;
        if (t0 >= p.nw) break;
        const int t = (int)t0 + lane;
        if (t < p.nw) {
            const int m = p.wlist[t];
            if (!mol_ok(d, p, m, 3)) {
                atomicAdd(&d.counters[7], 1ull);
                continue;
            }
            const int sweeps = SHAKE ? water_a_mat(d, m, tol, maxit) : water_b_mat(d, m, tol, maxit);
            p.wsw[m] = (uint8_t)(sweeps < 255 ? sweeps : 255);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&p.ctl[2], 1u) == gridDim.x - 1) { p.ctl[0] = 0u; p.ctl[1] = 0u; p.ctl[2] = 0u; }
    }
}

// ---------------------------------------------------------------- water order

// Counting sort of the water list by the sweeps of the last call, most
// first, for each half (bins 0..127; placement within a bin is free)
constexpr int WS_BINS = 128;
__device__ __forceinline__ int wbin(uint8_t s) { return WS_BINS - 1 - (s < WS_BINS - 1 ? (int)s : WS_BINS - 1); }

__global__ void k_worder_count(const int *wmols, int nw, const uint8_t *swa, const uint8_t *swb, int *off) {
    __shared__ int h[2 * WS_BINS];
    for (int k = threadIdx.x; k < 2 * WS_BINS; k += blockDim.x) h[k] = 0;
    __syncthreads();
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nw; t += gridDim.x * blockDim.x) {
        const int m = wmols[t];
        atomicAdd(&h[wbin(swa[m])], 1);
        atomicAdd(&h[WS_BINS + wbin(swb[m])], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * WS_BINS; k += blockDim.x)
        if (h[k]) atomicAdd(&off[k], h[k]);
}

__global__ void k_worder_scan(int *off) {   // one thread per half: exclusive scan of its bins
    int *o = off + threadIdx.x * WS_BINS;
    int acc = 0;
    for (int k = 0; k < WS_BINS; k++) { const int v = o[k]; o[k] = acc; acc += v; }
}

__global__ void k_worder_place(const int *wmols, int nw, const uint8_t *swa, const uint8_t *swb, int *off, int *la,
                               int *lb, unsigned long long *bad) {
    __shared__ int cnt[2 * WS_BINS], base[2 * WS_BINS];
    for (int k = threadIdx.x; k < 2 * WS_BINS; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int m = -1, ba = 0, bb = 0, ra = 0, rb = 0;
    if (t < nw) {
        m = wmols[t];
        ba = wbin(swa[m]);
        bb = WS_BINS + wbin(swb[m]);
        ra = atomicAdd(&cnt[ba], 1);
        rb = atomicAdd(&cnt[bb], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * WS_BINS; k += blockDim.x)
        if (cnt[k]) base[k] = atomicAdd(&off[k], cnt[k]);
    __syncthreads();
    if (m >= 0) {
        const int pa = base[ba] + ra, pb = base[bb] + rb;
        if (pa < nw && pb < nw) {
            la[pa] = m;
            lb[pb] = m;
        } else {
            atomicAdd(bad, 1ull);
        }
    }
}

}  // namespace

bool upload_tables_fast(const Tables &t, cudaStream_t st) {
    for (int b = 0; b < NBOND; b++)
        if (t.bi[b] != sbi32(b) || t.bj[b] != b + 1) return false;
    Fast32 f;
    for (int k = 0; k < NTYPE; k++) {
        f.mass64[k] = t.mass[k];
        f.rm64[k] = 1.0 / t.mass[k];
        f.rmdt64[k] = DT / t.mass[k];
        f.dt2m64[k] = DTSQ2 / t.mass[k];
    }
    for (int k = 0; k < 2; k++) f.rm32_w[k] = (float)f.rm64[k];
    for (int b = 0; b < 3; b++)
        for (int c = 0; c < 3; c++) f.wk32[b][c] = (float)wk_host(f.rm64, b, c);
    for (int b = 0; b < 3; b++) {
        const int ki = b == 0 ? 0 : 1, kj = b == 2 ? 0 : 1;
        const double rs = 1.0 / t.mass[ki] + 1.0 / t.mass[kj];
        f.dsq64_w[b] = t.dsqw[b];
        f.fb64_w[b] = (1.0 / DT) / (rs * t.dsqw[b]);
        f.hfa64_w[b] = 1.0 / (2.0 * rs);
    }
    for (int b = 0; b < NBOND; b++) {
        const double rs = 1.0 / t.mass[2 + t.bi[b]] + 1.0 / t.mass[2 + t.bj[b]];
        f.dsq64_s[b] = t.dsqs[b];
        f.fb64_s[b] = (1.0 / DT) / (rs * t.dsqs[b]);
        f.hfa64_s[b] = 1.0 / (2.0 * rs);
    }
    return cudaMemcpyToSymbolAsync(cF, &f, sizeof f, 0, cudaMemcpyHostToDevice, st) == cudaSuccess;
}

int constraint_max_surf_warps() { return MAX_SURF_WARPS; }
int constraint_max_mols_per_warp(int fp32) { return fp32 ? wavefront_mols<float>() : wavefront_mols<double>(); }

namespace {
int g_water_mat_ctas[2] = {0, 0};   // CTAs per SM of k_water_mat<RATTLE / SHAKE> (set once)

template <typename C, bool SHAKE>
constexpr size_t surf_smem(int s_warps, int mpw) {
    return (size_t)s_warps * mpw * sizeof(MolSmem<C, SHAKE ? 16 : 11>);
}

template <typename C, bool SHAKE>
void launch_constrain_t(const Dev &d, const int *smols, int ns, int nw, int nmol, int nsite, const ConstraintShape &sh,
                        double tol, int maxit, cudaStream_t st, int mat) {
    CPlan p;
    p.mat = mat;
    p.smols = smols;
    p.wlist = SHAKE ? d.wlist_a : d.wlist_b;
    p.wsw = SHAKE ? d.wsw_a : d.wsw_b;
    p.ctl = d.cctl + (SHAKE ? 0 : 4);
    p.ns = ns;
    p.nw = nw;
    p.nmol = nmol;
    p.nsite = nsite;
    p.s_warps = sh.s_warps < 1 ? 1 : (sh.s_warps > MAX_SURF_WARPS ? MAX_SURF_WARPS : sh.s_warps);
    p.mpw = sh.mpw < 1 ? 1 : (sh.mpw > wavefront_mols<C>() ? wavefront_mols<C>() : sh.mpw);
    const int groups = (ns + p.mpw - 1) / p.mpw;
    const int need = (groups + p.s_warps - 1) / p.s_warps;
    p.n_scta = ns ? (need < sh.grid ? need : sh.grid) : 0;
    if (std::is_same<C, double>::value && mat && ns == 0) {
        // waters only, in matrix form: as many CTAs per SM as fit
        const int occ = g_water_mat_ctas[SHAKE ? 1 : 0] > 0 ? g_water_mat_ctas[SHAKE ? 1 : 0] : 1;
        launch_pdl(k_water_mat<SHAKE>, dim3(sh.grid * occ), dim3(CW_THREADS), 0, st, d, p, tol, maxit);
        return;
    }
    const size_t smem = p.n_scta ? surf_smem<C, SHAKE>(p.s_warps, p.mpw) : 0;
    launch_pdl(k_constrain<C, SHAKE>, dim3(sh.grid), dim3(CW_THREADS), smem, st, d, p, tol, maxit);
}
}  // namespace

void init_constraint_kernels() {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_water_mat_ctas[0], k_water_mat<false>, CW_THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_water_mat_ctas[1], k_water_mat<true>, CW_THREADS, 0);
    cudaFuncSetAttribute(k_constrain<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)surf_smem<double, true>(MAX_SURF_WARPS, MPW));
    cudaFuncSetAttribute(k_constrain<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)surf_smem<double, false>(MAX_SURF_WARPS, MPW));
    cudaFuncSetAttribute(k_constrain<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)surf_smem<float, true>(MAX_SURF_WARPS, MPW));
    cudaFuncSetAttribute(k_constrain<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)surf_smem<float, false>(MAX_SURF_WARPS, MPW));
}

// fp32: 1 for FP32 sweeps, 0 for FP64 sweeps
void launch_move_a32(const Dev &d, int nw, const int *smols, int ns, int nmol, int nsite, const ConstraintShape &sh,
                     cudaStream_t st, double tol, int maxit, int fp32, int mat) {
    if (!nw && !ns) return;
    if (fp32) launch_constrain_t<float, true>(d, smols, ns, nw, nmol, nsite, sh, tol, maxit, st, 0);
    else launch_constrain_t<double, true>(d, smols, ns, nw, nmol, nsite, sh, tol, maxit, st, mat);
}

void launch_move_b32(const Dev &d, int nw, const int *smols, int ns, int nmol, int nsite, const ConstraintShape &sh,
                     cudaStream_t st, double tol, int maxit, int fp32, int mat) {
    if (!nw && !ns) return;
    if (fp32) launch_constrain_t<float, false>(d, smols, ns, nw, nmol, nsite, sh, tol, maxit, st, 0);
    else launch_constrain_t<double, false>(d, smols, ns, nw, nmol, nsite, sh, tol, maxit, st, mat);
}

void launch_water_order(const Dev &d, const int *wmols, int nw, cudaStream_t st) {
    if (!nw) return;
    cudaMemsetAsync(d.wsort_off, 0, 2 * WS_BINS * sizeof(int), st);
    const int nb = (nw + 255) / 256;
    k_worder_count<<<nb < 256 ? nb : 256, 256, 0, st>>>(wmols, nw, d.wsw_a, d.wsw_b, d.wsort_off);
    k_worder_scan<<<1, 2, 0, st>>>(d.wsort_off);
    k_worder_place<<<nb, 256, 0, st>>>(wmols, nw, d.wsw_a, d.wsw_b, d.wsort_off, d.wlist_a, d.wlist_b, d.counters + 7);
}

}  // namespace sesp
