// Constraint halves of the mixed path: SHAKE (move_*_a) and RATTLE
// (move_*_b) iterated in FP32 (src/move_w1_a.f90:36-134,
// src/move_surfactant_a.f90:36-134, src/move_w1_b.f90:30-119,
// src/move_surfactant_b.f90:30-118).
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and a Gauss-Seidel
// sweep is one long dependent chain per molecule, so the FP64 sweeps of the
// plain path cost ~1000 cycles per bond.  Here the FP64 state is split once
// per call into
//   * the FP64 predictor (positions for SHAKE, velocities for RATTLE), which
//     is written to the state arrays at the start, and
//   * FP32 corrections per site, which the sweeps update.
// Each bond's constants are formed once in FP64 and rounded to FP32: for
// SHAKE the predictor bond vector P, the old bond vector R, D0 = d^2 - |P|^2
// and R.P; for RATTLE R and R.V (V the predictor velocity difference).  A
// sweep then evaluates, with c the difference of the two sites' corrections,
//     d^2 - |P + c|^2 = D0 - (2 P.c + c.c),     R.(P + c) = R.P + R.c,
//     R.(V + c) = R.V + R.c,
// so nothing cancels in FP32: the residual carries ~1e-10 absolute error
// against a threshold of 2e-4 d^2 (SHAKE) or an equivalent 1e-4 (RATTLE).  A
// residual within 2 % of its threshold is recomputed in FP64 from the
// predictor plus the corrections, so the sweeps take the decisions an FP64
// evaluation of the same state takes.  At the end the corrections are added
// to the FP64 state.  Same bond order, tolerance tests, iteration limit and
// failure counting as the FP64 kernels; only the rounding differs.
//
// Waters: one thread per molecule.  Surfactants: one warp per molecule, its
// 29 lanes doing the per-site FP64 work and the bond constants in parallel,
// lane 0 the serial sweeps (the bond constants stream from shared memory one
// bond ahead of use).
#include <type_traits>

#include "k_launch.cuh"

namespace sesp {

namespace {

struct Fast32 {
    float rm[NTYPE];            // 1 / mass by site kind
    float rmdt[NTYPE];          // DT / mass
    float dsq_w[3], fa_w[3], fb_w[3];
    float dsq_s[NBOND], fa_s[NBOND], fb_s[NBOND];
    double dsq64_w[3], dsq64_s[NBOND];
    double mass64[NTYPE], rm64[NTYPE];
};
__constant__ Fast32 cF;

// surfactant bond graph of src/init_arrays.f90:229-264: bond b joins site
// b + 1 to the earlier site sbi32(b) (checked against the uploaded
// tables on the host)
// {0, 1, ..., 17, 17, 19, 20, 20, 20, 17, 24, 25, 25, 25}
__host__ __device__ constexpr int sbi32(int b) {
    return b < 18 ? b : b == 18 ? 17 : b == 19 ? 19 : b <= 22 ? 20 : b == 23 ? 17 : b == 24 ? 24 : 25;
}

template <int NS>
struct G32;
template <>
struct G32<3> {
    static constexpr int NB = 3, BLOCK = 128;
    __device__ static constexpr int bi(int b) { return b; }
    __device__ static constexpr int bj(int b) { return b == 2 ? 0 : b + 1; }
    __device__ static constexpr int kind(int i) { return i == 0 ? 0 : 1; }
    __device__ static float dsq(int b) { return cF.dsq_w[b]; }
    __device__ static float fa(int b) { return cF.fa_w[b]; }
    __device__ static float fb(int b) { return cF.fb_w[b]; }
    __device__ static double dsq64(int b) { return cF.dsq64_w[b]; }
};
template <>
struct G32<NSURF> {
    static constexpr int NB = NBOND, BLOCK = 32;
    __device__ static constexpr int bi(int b) { return sbi32(b); }
    __device__ static constexpr int bj(int b) { return b + 1; }
    __device__ static constexpr int kind(int i) { return 2 + i; }
    __device__ static float dsq(int b) { return cF.dsq_s[b]; }
    __device__ static float fa(int b) { return cF.fa_s[b]; }
    __device__ static float fb(int b) { return cF.fb_s[b]; }
    __device__ static double dsq64(int b) { return cF.dsq64_s[b]; }
};

// the FP64 predictors of the FP64 kernels, rounded the same way
__device__ inline double pred_a(double x, double v, double a, double escale) {
    return __dadd_rn(__dadd_rn(x, __dmul_rn(v, escale)), a);
}
__device__ inline double vel_a(double v, double a, double escale) { return __dadd_rn(__dmul_rn(v, escale), a); }

// v as hi + lo, both FP32 (hi the rounded value, lo the rounded remainder)
template <typename F>
__device__ inline void split(double v, F &hi, F &lo) {
    const float h = (float)v;
    hi = h;
    lo = (float)__dsub_rn(v, (double)h);
}

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

constexpr float BAND = 0.02f;   // relative half-width of the FP64 decision band
constexpr unsigned FULL = 0xffffffffu;

// One SHAKE bond update.  k = {P.x, P.y, P.z, R.x, R.y, R.z, D0, R.P}.
template <int NS, int B>
__device__ __forceinline__ bool shake_step(const Dev &d, int g0, const float (&k)[8], float (&cx)[NS],
                                           float (&cy)[NS], float (&cz)[NS], float tol2, double tol2d) {
    using Gr = G32<NS>;
    constexpr int i = Gr::bi(B), j = Gr::bj(B);
    const float dx = cx[i] - cx[j], dy = cy[i] - cy[j], dz = cz[i] - cz[j];
    const float pc = k[0] * dx + k[1] * dy + k[2] * dz;
    const float cc = dx * dx + dy * dy + dz * dz;
    const float diffsq = k[6] - (2.f * pc + cc);
    const float thr = Gr::dsq(B) * tol2;
    bool act = fabsf(diffsq) > thr;
    if (fabsf(fabsf(diffsq) - thr) < BAND * thr)
        act = shake_active64(d, g0 + i, g0 + j, cx[i], cy[i], cz[i], cx[j], cy[j], cz[j], Gr::dsq64(B), tol2d);
    if (act) {
        const float rpab = k[7] + (k[3] * dx + k[4] * dy + k[5] * dz);
        const float gab = __fdividef(diffsq, Gr::fa(B) * rpab);
        const float ga = cF.rm[Gr::kind(i)] * gab, gb = cF.rm[Gr::kind(j)] * gab;
        cx[i] += k[3] * ga; cy[i] += k[4] * ga; cz[i] += k[5] * ga;
        cx[j] -= k[3] * gb; cy[j] -= k[4] * gb; cz[j] -= k[5] * gb;
    }
    return act;
}

// One RATTLE bond update.  k = {R.x, R.y, R.z, R.V}.
template <int NS, int B>
__device__ __forceinline__ bool rattle_step(const Dev &d, int g0, const float (&k)[4], float (&cx)[NS],
                                            float (&cy)[NS], float (&cz)[NS], float tol, double told) {
    using Gr = G32<NS>;
    constexpr int i = Gr::bi(B), j = Gr::bj(B);
    const float dx = cx[i] - cx[j], dy = cy[i] - cy[j], dz = cz[i] - cz[j];
    const float gab = -(k[3] + (k[0] * dx + k[1] * dy + k[2] * dz)) * Gr::fb(B);
    bool act = fabsf(gab) > tol;
    if (fabsf(fabsf(gab) - tol) < BAND * tol)
        act = rattle_active64(d, g0 + i, g0 + j, Gr::kind(i), Gr::kind(j), cx[i], cy[i], cz[i], cx[j], cy[j], cz[j],
                              Gr::dsq64(B), told);
    if (act) {
        const float ga = cF.rmdt[Gr::kind(i)] * gab, gb = cF.rmdt[Gr::kind(j)] * gab;
        cx[i] += k[0] * ga; cy[i] += k[1] * ga; cz[i] += k[2] * ga;
        cx[j] -= k[0] * gb; cy[j] -= k[1] * gb; cz[j] -= k[2] * gb;
    }
    return act;
}

// SHAKE constants of one bond from FP64 old positions r and predictors p
__device__ inline void shake_consts(double rxi, double ryi, double rzi, double rxj, double ryj, double rzj, double pxi,
                                    double pyi, double pzi, double pxj, double pyj, double pzj, double dsq,
                                    float (&k)[8]) {
    const double rx = rxi - rxj, ry = ryi - ryj, rz = rzi - rzj;
    const double px = pxi - pxj, py = pyi - pyj, pz = pzi - pzj;
    k[0] = (float)px; k[1] = (float)py; k[2] = (float)pz;
    k[3] = (float)rx; k[4] = (float)ry; k[5] = (float)rz;
    k[6] = (float)(dsq - (px * px + py * py + pz * pz));
    k[7] = (float)(rx * px + ry * py + rz * pz);
}

// static-index unrolling helper: f(integral_constant<B>) for B = 0..N-1
template <int B, int N, typename F>
__device__ __forceinline__ void unroll(F &&f) {
    if constexpr (B < N) {
        f(std::integral_constant<int, B>{});
        unroll<B + 1, N>(f);
    }
}

// ---------------------------------------------------------------- waters

__global__ void __launch_bounds__(128) k_move_a32w(Dev d, const int *mols, int nm, double tol, int maxit) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    const int m = mols[t];
    const int g0 = d.mfirst[m];
    const double escale = __dsub_rn(1.0, __dmul_rn(d.eta[d.mrep[m]], DT) * 0.5);
    double rx[3], ry[3], rz[3], px[3], py[3], pz[3];
    double ke0 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        double vx = d.vx[g], vy = d.vy[g], vz = d.vz[g], ax = d.ax[g], ay = d.ay[g], az = d.az[g];
        rx[i] = d.x[g]; ry[i] = d.y[g]; rz[i] = d.z[g];
        ke0 = __dadd_rn(ke0, __dmul_rn(cF.mass64[G32<3>::kind(i)],
                                       __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
        px[i] = pred_a(rx[i], vx, ax, escale);
        py[i] = pred_a(ry[i], vy, ay, escale);
        pz[i] = pred_a(rz[i], vz, az, escale);
        d.x[g] = px[i]; d.y[g] = py[i]; d.z[g] = pz[i];
        d.vx[g] = vel_a(vx, ax, escale);
        d.vy[g] = vel_a(vy, ay, escale);
        d.vz[g] = vel_a(vz, az, escale);
    }
    float k[3][8];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int i = G32<3>::bi(b), j = G32<3>::bj(b);
        shake_consts(rx[i], ry[i], rz[i], rx[j], ry[j], rz[j], px[i], py[i], pz[i], px[j], py[j], pz[j],
                     G32<3>::dsq64(b), k[b]);
    }
    float cx[3] = {0.f, 0.f, 0.f}, cy[3] = {0.f, 0.f, 0.f}, cz[3] = {0.f, 0.f, 0.f};
    const float tol2 = (float)(2.0 * tol);
    const double tol2d = 2.0 * tol;
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
        unroll<0, 3>([&](auto B) {
            if (shake_step<3, decltype(B)::value>(d, g0, k[B], cx, cy, cz, tol2, tol2d)) ldone = false;
        });
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
        ke1 = __dadd_rn(ke1, __dmul_rn(cF.mass64[G32<3>::kind(i)],
                                       __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
    }
    d.ke[2 * m] = ke0;
    d.ke[2 * m + 1] = ke1;
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
}

__global__ void __launch_bounds__(128) k_move_b32w(Dev d, const int *mols, int nm, double tol, int maxit) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    const int m = mols[t];
    const int g0 = d.mfirst[m];
    const double escale = __ddiv_rn(2.0, __dadd_rn(2.0, __dmul_rn(d.eta[d.mrep[m]], DT)));
    double rx[3], ry[3], rz[3], vx[3], vy[3], vz[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int g = g0 + i;
        const double mi = cF.mass64[G32<3>::kind(i)];
        double ax = __ddiv_rn(__dmul_rn(d.fx[g], DTSQ2), mi), ay = __ddiv_rn(__dmul_rn(d.fy[g], DTSQ2), mi),
               az = __ddiv_rn(__dmul_rn(d.fz[g], DTSQ2), mi);
        d.ax[g] = ax; d.ay[g] = ay; d.az[g] = az;
        vx[i] = __dmul_rn(escale, __dadd_rn(d.vx[g], ax));
        vy[i] = __dmul_rn(escale, __dadd_rn(d.vy[g], ay));
        vz[i] = __dmul_rn(escale, __dadd_rn(d.vz[g], az));
        d.vx[g] = vx[i]; d.vy[g] = vy[i]; d.vz[g] = vz[i];
        rx[i] = d.x[g]; ry[i] = d.y[g]; rz[i] = d.z[g];
    }
    float k[3][4];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int i = G32<3>::bi(b), j = G32<3>::bj(b);
        const double ex = rx[i] - rx[j], ey = ry[i] - ry[j], ez = rz[i] - rz[j];
        k[b][0] = (float)ex; k[b][1] = (float)ey; k[b][2] = (float)ez;
        k[b][3] = (float)(ex * (vx[i] - vx[j]) + ey * (vy[i] - vy[j]) + ez * (vz[i] - vz[j]));
    }
    float cx[3] = {0.f, 0.f, 0.f}, cy[3] = {0.f, 0.f, 0.f}, cz[3] = {0.f, 0.f, 0.f};
    const float tolf = (float)tol;
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
        unroll<0, 3>([&](auto B) {
            if (rattle_step<3, decltype(B)::value>(d, g0, k[B], cx, cy, cz, tolf, tol)) ldone = false;
        });
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
}

// ---------------------------------------------------------------- surfactants

__device__ inline double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    return v;   // lane 0
}

__global__ void __launch_bounds__(32) k_move_a32s(Dev d, const int *mols, int nm, double tol, int maxit) {
    __shared__ float sk[NBOND][8];
    __shared__ float sc[3][NSURF];
    __shared__ int sfail;
    if (blockIdx.x >= nm) return;
    const int lane = threadIdx.x;
    const int m = mols[blockIdx.x];
    const int g0 = d.mfirst[m];
    const double escale = __dsub_rn(1.0, __dmul_rn(d.eta[d.mrep[m]], DT) * 0.5);
    const bool site = lane < NSURF;
    const int g = g0 + (site ? lane : 0);
    double rx = 0.0, ry = 0.0, rz = 0.0, px = 0.0, py = 0.0, pz = 0.0, ke = 0.0;
    if (site) {
        double vx = d.vx[g], vy = d.vy[g], vz = d.vz[g], ax = d.ax[g], ay = d.ay[g], az = d.az[g];
        rx = d.x[g]; ry = d.y[g]; rz = d.z[g];
        ke = __dmul_rn(cF.mass64[2 + lane], __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz)));
        px = pred_a(rx, vx, ax, escale);
        py = pred_a(ry, vy, ay, escale);
        pz = pred_a(rz, vz, az, escale);
        d.x[g] = px; d.y[g] = py; d.z[g] = pz;
        d.vx[g] = vel_a(vx, ax, escale);
        d.vy[g] = vel_a(vy, ay, escale);
        d.vz[g] = vel_a(vz, az, escale);
    }
    const double ke0 = warp_sum(ke);
    {   // bond lane: sites sbi32(lane) and lane + 1
        const int bi = lane < NBOND ? sbi32(lane) : 0, bj = lane < NBOND ? lane + 1 : 0;
        const double rxi = __shfl_sync(FULL, rx, bi), ryi = __shfl_sync(FULL, ry, bi), rzi = __shfl_sync(FULL, rz, bi);
        const double rxj = __shfl_sync(FULL, rx, bj), ryj = __shfl_sync(FULL, ry, bj), rzj = __shfl_sync(FULL, rz, bj);
        const double pxi = __shfl_sync(FULL, px, bi), pyi = __shfl_sync(FULL, py, bi), pzi = __shfl_sync(FULL, pz, bi);
        const double pxj = __shfl_sync(FULL, px, bj), pyj = __shfl_sync(FULL, py, bj), pzj = __shfl_sync(FULL, pz, bj);
        if (lane < NBOND) {
            float k[8];
            shake_consts(rxi, ryi, rzi, rxj, ryj, rzj, pxi, pyi, pzi, pxj, pyj, pzj, cF.dsq64_s[lane], k);
#pragma unroll
            for (int q = 0; q < 8; q++) sk[lane][q] = k[q];
        }
    }
    __syncwarp();   // bond constants and the predictor stores, for lane 0
    if (lane == 0) {
        float cx[NSURF], cy[NSURF], cz[NSURF];
#pragma unroll
        for (int i = 0; i < NSURF; i++) cx[i] = cy[i] = cz[i] = 0.f;
        volatile float(*vk)[8] = sk;
        float kc[8], kn[8];
#pragma unroll
        for (int q = 0; q < 8; q++) kc[q] = vk[0][q];
        const float tol2 = (float)(2.0 * tol);
        const double tol2d = 2.0 * tol;
        int it = 0;
        bool ldone = false;
        while (!ldone && it <= maxit) {
            ldone = true;
            unroll<0, NBOND>([&](auto B) {
                constexpr int b = decltype(B)::value;
                constexpr int bn = b + 1 < NBOND ? b + 1 : 0;
#pragma unroll
                for (int q = 0; q < 8; q++) kn[q] = vk[bn][q];   // next bond's constants, ahead of use
                if (shake_step<NSURF, b>(d, g0, kc, cx, cy, cz, tol2, tol2d)) ldone = false;
#pragma unroll
                for (int q = 0; q < 8; q++) kc[q] = kn[q];
            });
            it++;
        }
#pragma unroll
        for (int i = 0; i < NSURF; i++) { sc[0][i] = cx[i]; sc[1][i] = cy[i]; sc[2][i] = cz[i]; }
        sfail = !ldone;
    }
    __syncwarp();
    double ke1 = 0.0;
    if (site) {
        const double cxi = sc[0][lane], cyi = sc[1][lane], czi = sc[2][lane];
        d.x[g] = __dadd_rn(px, cxi);
        d.y[g] = __dadd_rn(py, cyi);
        d.z[g] = __dadd_rn(pz, czi);
        double vx = __dadd_rn(d.vx[g], cxi), vy = __dadd_rn(d.vy[g], cyi), vz = __dadd_rn(d.vz[g], czi);
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        ke1 = __dmul_rn(cF.mass64[2 + lane], __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz)));
    }
    ke1 = warp_sum(ke1);
    if (lane == 0) {
        d.ke[2 * m] = ke0;
        d.ke[2 * m + 1] = ke1;
        if (sfail) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
    }
}

__global__ void __launch_bounds__(32) k_move_b32s(Dev d, const int *mols, int nm, double tol, int maxit) {
    __shared__ float sk[NBOND][4];
    __shared__ float sc[3][NSURF];
    __shared__ int sfail;
    if (blockIdx.x >= nm) return;
    const int lane = threadIdx.x;
    const int m = mols[blockIdx.x];
    const int g0 = d.mfirst[m];
    const double escale = __ddiv_rn(2.0, __dadd_rn(2.0, __dmul_rn(d.eta[d.mrep[m]], DT)));
    const bool site = lane < NSURF;
    const int g = g0 + (site ? lane : 0);
    double rx = 0.0, ry = 0.0, rz = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
    if (site) {
        const double mi = cF.mass64[2 + lane];
        double ax = __ddiv_rn(__dmul_rn(d.fx[g], DTSQ2), mi), ay = __ddiv_rn(__dmul_rn(d.fy[g], DTSQ2), mi),
               az = __ddiv_rn(__dmul_rn(d.fz[g], DTSQ2), mi);
        d.ax[g] = ax; d.ay[g] = ay; d.az[g] = az;
        vx = __dmul_rn(escale, __dadd_rn(d.vx[g], ax));
        vy = __dmul_rn(escale, __dadd_rn(d.vy[g], ay));
        vz = __dmul_rn(escale, __dadd_rn(d.vz[g], az));
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        rx = d.x[g]; ry = d.y[g]; rz = d.z[g];
    }
    {
        const int bi = lane < NBOND ? sbi32(lane) : 0, bj = lane < NBOND ? lane + 1 : 0;
        const double ex = __shfl_sync(FULL, rx, bi) - __shfl_sync(FULL, rx, bj);
        const double ey = __shfl_sync(FULL, ry, bi) - __shfl_sync(FULL, ry, bj);
        const double ez = __shfl_sync(FULL, rz, bi) - __shfl_sync(FULL, rz, bj);
        const double wx = __shfl_sync(FULL, vx, bi) - __shfl_sync(FULL, vx, bj);
        const double wy = __shfl_sync(FULL, vy, bi) - __shfl_sync(FULL, vy, bj);
        const double wz = __shfl_sync(FULL, vz, bi) - __shfl_sync(FULL, vz, bj);
        if (lane < NBOND) {
            sk[lane][0] = (float)ex; sk[lane][1] = (float)ey; sk[lane][2] = (float)ez;
            sk[lane][3] = (float)(ex * wx + ey * wy + ez * wz);
        }
    }
    __syncwarp();
    if (lane == 0) {
        float cx[NSURF], cy[NSURF], cz[NSURF];
#pragma unroll
        for (int i = 0; i < NSURF; i++) cx[i] = cy[i] = cz[i] = 0.f;
        volatile float(*vk)[4] = sk;
        float kc[4], kn[4];
#pragma unroll
        for (int q = 0; q < 4; q++) kc[q] = vk[0][q];
        const float tolf = (float)tol;
        int it = 0;
        bool ldone = false;
        while (!ldone && it <= maxit) {
            ldone = true;
            unroll<0, NBOND>([&](auto B) {
                constexpr int b = decltype(B)::value;
                constexpr int bn = b + 1 < NBOND ? b + 1 : 0;
#pragma unroll
                for (int q = 0; q < 4; q++) kn[q] = vk[bn][q];
                if (rattle_step<NSURF, b>(d, g0, kc, cx, cy, cz, tolf, tol)) ldone = false;
#pragma unroll
                for (int q = 0; q < 4; q++) kc[q] = kn[q];
            });
            it++;
        }
#pragma unroll
        for (int i = 0; i < NSURF; i++) { sc[0][i] = cx[i]; sc[1][i] = cy[i]; sc[2][i] = cz[i]; }
        sfail = !ldone;
    }
    __syncwarp();
    if (site) {
        d.vx[g] = __dadd_rn(vx, (double)sc[0][lane]);
        d.vy[g] = __dadd_rn(vy, (double)sc[1][lane]);
        d.vz[g] = __dadd_rn(vz, (double)sc[2][lane]);
    }
    if (lane == 0 && sfail) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
}

}  // namespace

bool upload_tables_fast(const Tables &t, cudaStream_t st) {
    for (int b = 0; b < NBOND; b++)
        if (t.bi[b] != sbi32(b) || t.bj[b] != b + 1) return false;
    Fast32 f;
    for (int k = 0; k < NTYPE; k++) {
        f.mass64[k] = t.mass[k];
        f.rm64[k] = 1.0 / t.mass[k];
        f.rm[k] = (float)(1.0 / t.mass[k]);
        f.rmdt[k] = (float)(DT / t.mass[k]);
    }
    for (int b = 0; b < 3; b++) {
        const int ki = b == 0 ? 0 : 1, kj = b == 2 ? 0 : 1;
        const double rs = 1.0 / t.mass[ki] + 1.0 / t.mass[kj];
        f.dsq64_w[b] = t.dsqw[b];
        f.dsq_w[b] = (float)t.dsqw[b];
        f.fa_w[b] = (float)(2.0 * rs);
        f.fb_w[b] = (float)((1.0 / DT) / (rs * t.dsqw[b]));
    }
    for (int b = 0; b < NBOND; b++) {
        const double rs = 1.0 / t.mass[2 + t.bi[b]] + 1.0 / t.mass[2 + t.bj[b]];
        f.dsq64_s[b] = t.dsqs[b];
        f.dsq_s[b] = (float)t.dsqs[b];
        f.fa_s[b] = (float)(2.0 * rs);
        f.fb_s[b] = (float)((1.0 / DT) / (rs * t.dsqs[b]));
    }
    return cudaMemcpyToSymbolAsync(cF, &f, sizeof f, 0, cudaMemcpyHostToDevice, st) == cudaSuccess;
}

void launch_move_a32(const Dev &d, const int *wmols, int nw, const int *smols, int ns, cudaStream_t st, double tol,
                     int maxit) {
    if (ns) k_move_a32s<<<ns, 32, 0, st>>>(d, smols, ns, tol, maxit);
    if (nw) k_move_a32w<<<(nw + 127) / 128, 128, 0, st>>>(d, wmols, nw, tol, maxit);
}

void launch_move_b32(const Dev &d, const int *wmols, int nw, const int *smols, int ns, cudaStream_t st, double tol,
                     int maxit) {
    if (ns) k_move_b32s<<<ns, 32, 0, st>>>(d, smols, ns, tol, maxit);
    if (nw) k_move_b32w<<<(nw + 127) / 128, 128, 0, st>>>(d, wmols, nw, tol, maxit);
}

}  // namespace sesp
