// Kernels whose FP64 arithmetic must round exactly like the reference's:
// cell assignment (the discrete ibox2 / ibox64 / isCentral decisions), the
// intramolecular-correction lists, and the SHAKE / RATTLE velocity-Verlet
// halves with the Nose-Hoover friction.  This translation unit is compiled
// with -fmad=false so no multiply-add is contracted, as in the reference.
#include "k_launch.cuh"

namespace sesp {

static __constant__ Tables cT;

void upload_tables_exact(const Tables &t, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(cT, &t, sizeof(Tables), 0, cudaMemcpyHostToDevice, st);
}

constexpr double IRS = 1.0 / RS;

// (int)(q / s) rounded as the reference divides, from q * (1 / s): with
// |q / s| below 1e6 the product and the rounded quotient differ by less
// than 1e-9, so they truncate alike unless the product lies within 1e-9 of
// an integer, where the division itself decides
__device__ inline int trunc_div(double q, double s, double inv_s) {
    const double t = q * inv_s;
    if (fabs(t - rint(t)) > 1e-9) return (int)t;
    return (int)(q / s);
}
// ibox2 - 1 along one axis, src/ibox.f90:127-139
__device__ inline int rank_axis(const Rep &r, int a, double v) {
    int k = trunc_div((v + r.rhs[a]) * r.nr[a], r.rsd[a], r.irsd[a]);
    return k < 0 ? 0 : (k >= r.nr[a] ? r.nr[a] - 1 : k);
}
// rcen2xtmp, src/init_box_dimensions.f90:40-42, tabulated at upload per
// replica, axis and rank (rsd (rk + 1) / nr - rhs - rsd / nr / 2)
__device__ inline double rcen2_axis(const Dev &d, const Rep &r, int a, int rk) {
    const double *t = d.rcen2 + r.axis0 / 4;
    return t[(a > 0 ? r.nr[0] : 0) + (a > 1 ? r.nr[1] : 0) + rk];
}
// ibox64 along one axis relative to a rank centre, src/ibox.f90:172-186
__device__ inline int local_axis(double v, double c2) {
    int k = trunc_div(v - c2 + 2.0 * RS, RS, IRS);
    return k < 0 ? 0 : (k > 3 ? 3 : k);
}
// global key-cell coordinate along one axis (rank by ibox2, cell by ibox64)
__device__ inline int key_axis(const Dev &d, const Rep &r, int a, double v, int *rk) {
    *rk = rank_axis(r, a, v);
    return 4 * (*rk) + local_axis(v, rcen2_axis(d, r, a, *rk));
}
// isCentral along one axis (src/ibox.f90:101-124): the cell whose
// [centre - rs/2, centre + rs/2) holds v, -1 if none (the product only
// picks the three candidates; the comparisons decide)
__device__ inline int central_axis(const double *cen, int n, double v, double rhs) {
    int k0 = (int)floor((v + rhs) * IRS);
    const double rs2 = RS / 2.0;
    for (int k = k0 - 1; k <= k0 + 1; k++) {
        if (k < 0 || k >= n) continue;
        double c = cen[k];
        if (v < c + rs2 && v >= c - rs2) return k;
    }
    return -1;
}

// the cell a site is Central in, or -1
__device__ inline int central_cell(const Dev &d, const Rep &r, int g) {
    const double *cx = d.axis + r.axis0;
    const double *cy = cx + r.nc[0];
    const double *cz = cy + r.nc[1];
    int ix = central_axis(cx, r.nc[0], d.x[g], r.rhs[0]);
    int iy = central_axis(cy, r.nc[1], d.y[g], r.rhs[1]);
    int iz = central_axis(cz, r.nc[2], d.z[g], r.rhs[2]);
    return (ix < 0 || iy < 0 || iz < 0) ? -1 : cell_index(r, ix, iy, iz);
}

// Re-key molecules (src/read_config.f90:44-175 and the delete/add pairs
// src/delete_w1.f90:54-195, src/delete_s.f90:33-43; key site O for water,
// 14 for surfactants) and locate every site in the cell it is Central in.
// A w1 water (all three sites in one rank and one ibox64 cell) has its
// sites located in its key cell, as the reference stores it there.
// Threads [0, nmol) take one molecule each (a water with its sites);
// threads [nmol, nmol + nss) one surfactant site each.
__global__ void k_locate(Dev d, int nmol, const int *smols, int nss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmol) {
        if (t - nmol >= nss) return;
        const int m = smols[(t - nmol) / NSURF], g = d.mfirst[m] + (t - nmol) % NSURF;
        const int loc = central_cell(d, d.rep[d.mrep[m]], g);
        d.sloc[g] = loc;
        if (loc >= 0) atomicAdd(&d.ccount[loc], 1);
        else atomicAdd(&d.counters[2], 1ull);
        return;
    }
    const int m = t;
    const Rep r = d.rep[d.mrep[m]];
    int g0 = d.mfirst[m];
    int kind = d.mkind[m];
    int ks = kind == 0 ? g0 : g0 + 13;
    double p[3] = {d.x[ks], d.y[ks], d.z[ks]};
    int rk[3], kc[3];
    for (int a = 0; a < 3; a++) kc[a] = key_axis(d, r, a, p[a], &rk[a]);
    int key = cell_index(r, kc[0], kc[1], kc[2]);
    d.mkey[m] = key;
    if (kind != 0) {
        d.mw1[m] = 0;
        return;
    }
    int w1 = 1;
    for (int s = 1; s < 3; s++) {
        double q[3] = {d.x[g0 + s], d.y[g0 + s], d.z[g0 + s]};
        for (int a = 0; a < 3; a++) {
            if (rank_axis(r, a, q[a]) != rk[a]) w1 = 0;
            else if (4 * rk[a] + local_axis(q[a], rcen2_axis(d, r, a, rk[a])) != kc[a]) w1 = 0;
        }
    }
    d.mw1[m] = w1;
    for (int s = 0; s < 3; s++) {
        const int g = g0 + s;
        const int loc = w1 ? key : central_cell(d, r, g);
        d.sloc[g] = loc;
        if (loc >= 0) atomicAdd(&d.ccount[loc], 1);
        else atomicAdd(&d.counters[2], 1ull);
    }
}

// Sites of each surfactant that lie outside the 27-cell block of a site's
// own cell (src/buildinternal.f90:13-63); cells on the 10^3 grid of the
// key rank (ibox1000, rcen1000: src/ibox.f90:206-220,
// src/init_box_dimensions.f90:155-170).  One thread per surfactant site.
__global__ void k_isub(Dev d, int nsurf_sites, const int *surf_mol_of) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsurf_sites) return;
    int m = surf_mol_of[t / NSURF];
    int j = t % NSURF;
    const Rep r = d.rep[d.mrep[m]];
    int g0 = d.mfirst[m];
    int key = d.mkey[m] - r.cell0;
    int kc[3] = {key % r.nc[0], (key / r.nc[0]) % r.nc[1], key / (r.nc[0] * r.nc[1])};
    double pm[3] = {d.x[g0 + j], d.y[g0 + j], d.z[g0 + j]};
    double cen[3];
    for (int a = 0; a < 3; a++) {
        double c2 = rcen2_axis(d, r, a, kc[a] / 4);
        int li = trunc_div(pm[a] - c2 + 5.0 * RS, RS, IRS) + 1;
        cen[a] = 10.0 * RS * li / 10.0 - 10.0 * RS / 2.0 - 10.0 * RS / 20.0 + c2;
    }
    const double r15 = 1.5 * RS;
    uint32_t mask = 0;
    for (int k = 0; k < NSURF; k++) {
        if (k == j) continue;
        double pk[3] = {d.x[g0 + k], d.y[g0 + k], d.z[g0 + k]};
        bool near = true;
        for (int a = 0; a < 3; a++) near = near && (pk[a] < cen[a] + r15 && pk[a] >= cen[a] - r15);
        if (!near) mask |= (1u << k);
    }
    d.isub[t] = mask;
}

// ---------------------------------------------------------------- integrator

template <int NSITE>
struct MolTopo;

template <>
struct MolTopo<3> {
    static constexpr int NB = 3;
    __device__ static int bi(int b) { return b; }
    __device__ static int bj(int b) { return b == 2 ? 0 : b + 1; }
    __device__ static double dsq(int b) { return cT.dsqw[b]; }
    __device__ static double mass(int i) { return cT.mass[i == 0 ? 0 : 1]; }
};
template <>
struct MolTopo<NSURF> {
    static constexpr int NB = NBOND;
    __device__ static int bi(int b) { return cT.bi[b]; }
    __device__ static int bj(int b) { return cT.bj[b]; }
    __device__ static double dsq(int b) { return cT.dsqs[b]; }
    __device__ static double mass(int i) { return cT.mass[2 + i]; }
};

// move_*_a for one molecule: Nose-Hoover scaled predictor, SHAKE
// (src/move_w1_a.f90:36-134, src/move_surfactant_a.f90:36-134), and the
// kinetic sums before and after (src/nh_water1.f90, src/nh_surfactant.f90)
template <int NSITE>
__global__ void k_move_a(Dev d, const int *mols, int nm, double tol, int maxit) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    int m = mols[t];
    int rep = d.mrep[m];
    int g0 = d.mfirst[m];
    double escale = 1.0 - d.eta[rep] * DT / 2.0;
    double rx[NSITE], ry[NSITE], rz[NSITE], px[NSITE], py[NSITE], pz[NSITE], vx[NSITE], vy[NSITE], vz[NSITE];
    double ke0 = 0.0;
    for (int i = 0; i < NSITE; i++) {
        int g = g0 + i;
        double vxg = d.vx[g], vyg = d.vy[g], vzg = d.vz[g];
        ke0 += MolTopo<NSITE>::mass(i) * (vxg * vxg + vyg * vyg + vzg * vzg);
        rx[i] = d.x[g]; ry[i] = d.y[g]; rz[i] = d.z[g];
        px[i] = d.x[g] + vxg * escale + d.ax[g];
        py[i] = d.y[g] + vyg * escale + d.ay[g];
        pz[i] = d.z[g] + vzg * escale + d.az[g];
        vx[i] = vxg * escale + d.ax[g];
        vy[i] = vyg * escale + d.ay[g];
        vz[i] = vzg * escale + d.az[g];
    }
    const double tol2 = 2.0 * tol;
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
        for (int b = 0; b < MolTopo<NSITE>::NB; b++) {
            int i = MolTopo<NSITE>::bi(b), j = MolTopo<NSITE>::bj(b);
            double pxab = px[i] - px[j], pyab = py[i] - py[j], pzab = pz[i] - pz[j];
            double pabsq = pxab * pxab + pyab * pyab + pzab * pzab;
            double rabsq = MolTopo<NSITE>::dsq(b);
            double diffsq = rabsq - pabsq;
            if (fabs(diffsq) > rabsq * tol2) {
                double rxab = rx[i] - rx[j], ryab = ry[i] - ry[j], rzab = rz[i] - rz[j];
                double rpab = rxab * pxab + ryab * pyab + rzab * pzab;
                double rma = 1.0 / MolTopo<NSITE>::mass(i), rmb = 1.0 / MolTopo<NSITE>::mass(j);
                double gab = diffsq / (2.0 * (rma + rmb) * rpab);
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                px[i] = px[i] + rma * dx; py[i] = py[i] + rma * dy; pz[i] = pz[i] + rma * dz;
                px[j] = px[j] - rmb * dx; py[j] = py[j] - rmb * dy; pz[j] = pz[j] - rmb * dz;
                vx[i] = vx[i] + rma * dx; vy[i] = vy[i] + rma * dy; vz[i] = vz[i] + rma * dz;
                vx[j] = vx[j] - rmb * dx; vy[j] = vy[j] - rmb * dy; vz[j] = vz[j] - rmb * dz;
                ldone = false;
            }
        }
        it++;
    }
    double ke1 = 0.0;
    for (int i = 0; i < NSITE; i++) {
        int g = g0 + i;
        d.x[g] = px[i]; d.y[g] = py[i]; d.z[g] = pz[i];
        d.vx[g] = vx[i]; d.vy[g] = vy[i]; d.vz[g] = vz[i];
        ke1 += MolTopo<NSITE>::mass(i) * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
    }
    d.ke[2 * m] = ke0;
    d.ke[2 * m + 1] = ke1;
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
}

// The surfactant halves with the bond graph of src/init_arrays.f90:229-264
// unrolled at compile time, so the 29 iterated positions (SHAKE) or
// velocities (RATTLE) live in registers; the fixed positions and the velocity
// copies sit in shared memory.  Same Gauss-Seidel order and arithmetic as the
// generic kernel above (and as src/move_surfactant_a.f90 / _b.f90).
__device__ constexpr int SBI[NBOND] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17,
                                        17, 19, 20, 20, 20, 17, 24, 25, 25, 25};
__device__ constexpr int SBJ[NBOND] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18,
                                        19, 20, 21, 22, 23, 24, 25, 26, 27, 28};
constexpr int SURF_BLOCK = 32;

__global__ void __launch_bounds__(SURF_BLOCK) k_move_a_surf(Dev d, const int *mols, int nm, double tol, int maxit) {
    __shared__ double s_rm[NSURF], s_dsq[NBOND];
    if (threadIdx.x < NSURF) s_rm[threadIdx.x] = 1.0 / cT.mass[2 + threadIdx.x];
    if (threadIdx.x < NBOND) s_dsq[threadIdx.x] = cT.dsqs[threadIdx.x];
    __syncthreads();
    volatile double *vrm = s_rm, *vdsq = s_dsq;
    __shared__ double sr[3][NSURF][SURF_BLOCK];
    __shared__ double sv[3][NSURF][SURF_BLOCK];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    const int l = threadIdx.x;
    int m = mols[t];
    int g0 = d.mfirst[m];
    double escale = 1.0 - d.eta[d.mrep[m]] * DT / 2.0;
    double px[NSURF], py[NSURF], pz[NSURF];
    double ke0 = 0.0;
#pragma unroll
    for (int i = 0; i < NSURF; i++) {
        int g = g0 + i;
        double vxg = d.vx[g], vyg = d.vy[g], vzg = d.vz[g];
        ke0 += cT.mass[2 + i] * (vxg * vxg + vyg * vyg + vzg * vzg);
        sr[0][i][l] = d.x[g]; sr[1][i][l] = d.y[g]; sr[2][i][l] = d.z[g];
        px[i] = d.x[g] + vxg * escale + d.ax[g];
        py[i] = d.y[g] + vyg * escale + d.ay[g];
        pz[i] = d.z[g] + vzg * escale + d.az[g];
        sv[0][i][l] = vxg * escale + d.ax[g];
        sv[1][i][l] = vyg * escale + d.ay[g];
        sv[2][i][l] = vzg * escale + d.az[g];
    }
    const double tol2 = 2.0 * tol;
    volatile double(*vr)[NSURF][SURF_BLOCK] = sr;
    volatile double(*vv)[NSURF][SURF_BLOCK] = sv;
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
#pragma unroll
        for (int b = 0; b < NBOND; b++) {
            const int i = SBI[b], j = SBJ[b];
            double pxab = px[i] - px[j], pyab = py[i] - py[j], pzab = pz[i] - pz[j];
            double pabsq = pxab * pxab + pyab * pyab + pzab * pzab;
            double rabsq = vdsq[b];
            double diffsq = rabsq - pabsq;
            if (fabs(diffsq) > rabsq * tol2) {
                double rxab = vr[0][i][l] - vr[0][j][l], ryab = vr[1][i][l] - vr[1][j][l], rzab = vr[2][i][l] - vr[2][j][l];
                double rpab = rxab * pxab + ryab * pyab + rzab * pzab;
                double rma = vrm[i], rmb = vrm[j];
                double gab = diffsq / (2.0 * (rma + rmb) * rpab);
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                px[i] = px[i] + rma * dx; py[i] = py[i] + rma * dy; pz[i] = pz[i] + rma * dz;
                px[j] = px[j] - rmb * dx; py[j] = py[j] - rmb * dy; pz[j] = pz[j] - rmb * dz;
                vv[0][i][l] = vv[0][i][l] + rma * dx; vv[1][i][l] = vv[1][i][l] + rma * dy; vv[2][i][l] = vv[2][i][l] + rma * dz;
                vv[0][j][l] = vv[0][j][l] - rmb * dx; vv[1][j][l] = vv[1][j][l] - rmb * dy; vv[2][j][l] = vv[2][j][l] - rmb * dz;
                ldone = false;
            }
        }
        it++;
    }
    double ke1 = 0.0;
#pragma unroll
    for (int i = 0; i < NSURF; i++) {
        int g = g0 + i;
        double vx = sv[0][i][l], vy = sv[1][i][l], vz = sv[2][i][l];
        d.x[g] = px[i]; d.y[g] = py[i]; d.z[g] = pz[i];
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        ke1 += cT.mass[2 + i] * (vx * vx + vy * vy + vz * vz);
    }
    d.ke[2 * m] = ke0;
    d.ke[2 * m + 1] = ke1;
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
}

__global__ void __launch_bounds__(SURF_BLOCK) k_move_b_surf(Dev d, const int *mols, int nm, double tol, int maxit) {
    __shared__ double s_rm[NSURF], s_dsq[NBOND];
    if (threadIdx.x < NSURF) s_rm[threadIdx.x] = 1.0 / cT.mass[2 + threadIdx.x];
    if (threadIdx.x < NBOND) s_dsq[threadIdx.x] = cT.dsqs[threadIdx.x];
    __syncthreads();
    volatile double *vrm = s_rm, *vdsq = s_dsq;
    __shared__ double sr[3][NSURF][SURF_BLOCK];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    const int l = threadIdx.x;
    int m = mols[t];
    int g0 = d.mfirst[m];
    double escale = 2.0 / (2.0 + d.eta[d.mrep[m]] * DT);
    double vx[NSURF], vy[NSURF], vz[NSURF];
#pragma unroll
    for (int i = 0; i < NSURF; i++) {
        int g = g0 + i;
        double mi = cT.mass[2 + i];
        sr[0][i][l] = d.x[g]; sr[1][i][l] = d.y[g]; sr[2][i][l] = d.z[g];
        double axg = d.fx[g] * DTSQ2 / mi, ayg = d.fy[g] * DTSQ2 / mi, azg = d.fz[g] * DTSQ2 / mi;
        d.ax[g] = axg; d.ay[g] = ayg; d.az[g] = azg;
        vx[i] = escale * (d.vx[g] + axg);
        vy[i] = escale * (d.vy[g] + ayg);
        vz[i] = escale * (d.vz[g] + azg);
    }
    volatile double(*vr)[NSURF][SURF_BLOCK] = sr;
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
#pragma unroll
        for (int b = 0; b < NBOND; b++) {
            const int i = SBI[b], j = SBJ[b];
            double vxab = vx[i] - vx[j], vyab = vy[i] - vy[j], vzab = vz[i] - vz[j];
            double rxab = vr[0][i][l] - vr[0][j][l], ryab = vr[1][i][l] - vr[1][j][l], rzab = vr[2][i][l] - vr[2][j][l];
            double rvab = rxab * vxab + ryab * vyab + rzab * vzab;
            double rma = vrm[i], rmb = vrm[j];
            rvab = rvab / DT;
            double gab = -rvab / ((rma + rmb) * vdsq[b]);
            if (fabs(gab) > tol) {
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                vx[i] = vx[i] + rma * dx * DT; vy[i] = vy[i] + rma * dy * DT; vz[i] = vz[i] + rma * dz * DT;
                vx[j] = vx[j] - rmb * dx * DT; vy[j] = vy[j] - rmb * dy * DT; vz[j] = vz[j] - rmb * dz * DT;
                ldone = false;
            }
        }
        it++;
    }
#pragma unroll
    for (int i = 0; i < NSURF; i++) {
        int g = g0 + i;
        d.vx[g] = vx[i]; d.vy[g] = vy[i]; d.vz[g] = vz[i];
    }
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
}

// eta update of src/move_w2_a.f90:145-157.  ETA_BLOCKS blocks per replica
// each sum a fixed contiguous share of its molecules' kinetic sums
// (thread-strided, then a tree); the last of them to finish adds the shares
// in block order and updates eta.  The summation order is fixed, whichever
// block finishes last; nothing waits.
constexpr int ETA_BLOCKS = 32, ETA_THREADS = 256;
__global__ void __launch_bounds__(ETA_THREADS) k_eta(Dev d) {
    const int rep = blockIdx.x / ETA_BLOCKS, j = blockIdx.x % ETA_BLOCKS;
    const Rep r = d.rep[rep];
    __shared__ double s0[ETA_THREADS], s1[ETA_THREADS];
    __shared__ bool last;
    const int per = (r.nmol + ETA_BLOCKS - 1) / ETA_BLOCKS;
    const int m0 = r.mol0 + j * per, m1 = min(r.mol0 + r.nmol, m0 + per);
    double a = 0.0, b = 0.0;
    for (int m = m0 + threadIdx.x; m < m1; m += ETA_THREADS) { a += d.ke[2 * m]; b += d.ke[2 * m + 1]; }
    s0[threadIdx.x] = a; s1[threadIdx.x] = b;
    __syncthreads();
    for (int w = ETA_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { s0[threadIdx.x] += s0[threadIdx.x + w]; s1[threadIdx.x] += s1[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        d.eta_part[2 * blockIdx.x] = s0[0];
        d.eta_part[2 * blockIdx.x + 1] = s1[0];
        __threadfence();
        last = atomicAdd(&d.eta_ctl[rep], 1u) == ETA_BLOCKS - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const volatile double *p = d.eta_part + 2 * ETA_BLOCKS * rep;
        double sum1 = 0.0, sum2 = 0.0;
        for (int k = 0; k < ETA_BLOCKS; k++) { sum1 += p[2 * k]; sum2 += p[2 * k + 1]; }
        sum1 = sum1 / (DT * DT);
        sum2 = sum2 / (DT * DT);
        d.eta[rep] = d.eta[rep] + r.pnh1 * (sum1 + r.pnh2 + sum2);
        d.eta_ctl[rep] = 0u;
    }
}

// move_*_b for one molecule: acceleration from force, friction, RATTLE
// (src/move_w1_b.f90:30-119, src/move_surfactant_b.f90:30-118)
template <int NSITE>
__global__ void k_move_b(Dev d, const int *mols, int nm, double tol, int maxit) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    int m = mols[t];
    int rep = d.mrep[m];
    int g0 = d.mfirst[m];
    double escale = 2.0 / (2.0 + d.eta[rep] * DT);
    double rx[NSITE], ry[NSITE], rz[NSITE], vx[NSITE], vy[NSITE], vz[NSITE];
    for (int i = 0; i < NSITE; i++) {
        int g = g0 + i;
        double mi = MolTopo<NSITE>::mass(i);
        rx[i] = d.x[g]; ry[i] = d.y[g]; rz[i] = d.z[g];
        double axg = d.fx[g] * DTSQ2 / mi, ayg = d.fy[g] * DTSQ2 / mi, azg = d.fz[g] * DTSQ2 / mi;
        d.ax[g] = axg; d.ay[g] = ayg; d.az[g] = azg;
        vx[i] = escale * (d.vx[g] + axg);
        vy[i] = escale * (d.vy[g] + ayg);
        vz[i] = escale * (d.vz[g] + azg);
    }
    int it = 0;
    bool ldone = false;
    while (!ldone && it <= maxit) {
        ldone = true;
        for (int b = 0; b < MolTopo<NSITE>::NB; b++) {
            int i = MolTopo<NSITE>::bi(b), j = MolTopo<NSITE>::bj(b);
            double vxab = vx[i] - vx[j], vyab = vy[i] - vy[j], vzab = vz[i] - vz[j];
            double rxab = rx[i] - rx[j], ryab = ry[i] - ry[j], rzab = rz[i] - rz[j];
            double rvab = rxab * vxab + ryab * vyab + rzab * vzab;
            double rma = 1.0 / MolTopo<NSITE>::mass(i), rmb = 1.0 / MolTopo<NSITE>::mass(j);
            rvab = rvab / DT;
            double gab = -rvab / ((rma + rmb) * MolTopo<NSITE>::dsq(b));
            if (fabs(gab) > tol) {
                double dx = rxab * gab, dy = ryab * gab, dz = rzab * gab;
                vx[i] = vx[i] + rma * dx * DT; vy[i] = vy[i] + rma * dy * DT; vz[i] = vz[i] + rma * dz * DT;
                vx[j] = vx[j] - rmb * dx * DT; vy[j] = vy[j] - rmb * dy * DT; vz[j] = vz[j] - rmb * dz * DT;
                ldone = false;
            }
        }
        it++;
    }
    for (int i = 0; i < NSITE; i++) {
        int g = g0 + i;
        d.vx[g] = vx[i]; d.vy[g] = vy[i]; d.vz[g] = vz[i];
    }
    if (!ldone) { d.mfail[m] += 1; atomicAdd(&d.counters[0], 1ull); }
}

// src/init_accel.f90:10-46
__global__ void k_init_accel(Dev d, int nsite) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nsite) return;
    double m = d.tmass[d.ptype[g]];
    d.ax[g] = d.fx[g] * DTSQ2 / m;
    d.ay[g] = d.fy[g] * DTSQ2 / m;
    d.az[g] = d.fz[g] * DTSQ2 / m;
}

// ---------------------------------------------------------------- configuration preset

// floor division (b > 0)
__device__ inline int floor_div(int a, int b) { const int q = a / b; return (a % b != 0 && a < 0) ? q - 1 : q; }

// Periodic cell location (configuration preset), one thread per site: the
// cell index along each axis is floor((r + rhs) / rs); x and y are wrapped
// into the box and the integer image is kept (positions stay unwrapped, so
// molecules stay whole); a site outside the z range is in no cell.  The
// molecule's key is the cell of its first site.
__global__ void k_locate_cfg(Dev d, int nsite) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nsite) return;
    const int m = d.smol[g];
    const Rep r = d.rep[d.mrep[m]];
    const double x = d.x[g], y = d.y[g], z = d.z[g];
    int loc = -1, kx = 0, ky = 0;
    const double lim = 1e9;   // far outside any box: treated as lost (no cell)
    if (fabs(x) < lim && fabs(y) < lim && fabs(z) < lim) {
        const int ex = (int)floor((x + r.rhs[0]) * IRS), ey = (int)floor((y + r.rhs[1]) * IRS);
        const int ez = (int)floor((z + r.rhs[2]) * IRS);
        kx = floor_div(ex, r.nc[0]);
        ky = floor_div(ey, r.nc[1]);
        if (ez >= 0 && ez < r.nc[2] && abs(kx) < 30000 && abs(ky) < 30000)
            loc = cell_index(r, ex - kx * r.nc[0], ey - ky * r.nc[1], ez);
    }
    d.sloc[g] = loc;
    d.simg[g] = make_short2((short)(loc >= 0 ? kx : 0), (short)(loc >= 0 ? ky : 0));
    if (loc >= 0) atomicAdd(&d.ccount[loc], 1);
    else atomicAdd(&d.counters[2], 1ull);
    if (g == d.mfirst[m]) { d.mkey[m] = loc; d.mw1[m] = 0; }
}

// Same-molecule sites of each chain bead whose (unwrapped) cells are not
// adjacent to the bead's own: the pairs the far field counts and the
// correction removes.  One thread per bead.
__global__ void k_isub_cfg(Dev d, int nbeads, const int *chain_mols) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nbeads) return;
    const int m = chain_mols[t / NCH], j = t % NCH;
    const Rep r = d.rep[d.mrep[m]];
    const int g0 = d.mfirst[m];
    auto ext = [&](int g, int a) {
        const double v = a == 0 ? d.x[g] : (a == 1 ? d.y[g] : d.z[g]);
        const double c = fabs(v) < 1e9 ? floor((v + r.rhs[a]) * IRS) : 0.0;
        return (int)c;
    };
    const int ej[3] = {ext(g0 + j, 0), ext(g0 + j, 1), ext(g0 + j, 2)};
    uint32_t mask = 0;
    for (int k = 0; k < NCH; k++) {
        if (k == j) continue;
        const int g = g0 + k;
        if (abs(ext(g, 0) - ej[0]) > 1 || abs(ext(g, 1) - ej[1]) > 1 || abs(ext(g, 2) - ej[2]) > 1) mask |= 1u << k;
    }
    d.isub[t] = mask;
}

// move_a of flexible chains: the Nose-Hoover scaled predictor of
// src/move_surfactant_a.f90:36-60 with no constraint, and the kinetic sums
// before and after.  16 lanes per chain, one bead each; the sums are added
// by a fixed shuffle tree within the 16 lanes.
__global__ void k_move_free_a(Dev d, const int *mols, int nm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = t >> 4, i = t & 15;
    double ke0 = 0.0, ke1 = 0.0;
    if (q < nm && i < NCH) {
        const int m = mols[q], g = d.mfirst[m] + i;
        const double escale = 1.0 - d.eta[d.mrep[m]] * DT / 2.0;
        const double mi = d.tmass[d.ptype[g]];
        double vx = d.vx[g], vy = d.vy[g], vz = d.vz[g];
        ke0 = mi * (vx * vx + vy * vy + vz * vz);
        d.x[g] = d.x[g] + vx * escale + d.ax[g];
        d.y[g] = d.y[g] + vy * escale + d.ay[g];
        d.z[g] = d.z[g] + vz * escale + d.az[g];
        vx = vx * escale + d.ax[g]; vy = vy * escale + d.ay[g]; vz = vz * escale + d.az[g];
        d.vx[g] = vx; d.vy[g] = vy; d.vz[g] = vz;
        ke1 = mi * (vx * vx + vy * vy + vz * vz);
    }
    for (int o = 8; o > 0; o >>= 1) {
        ke0 += __shfl_xor_sync(0xffffffffu, ke0, o);
        ke1 += __shfl_xor_sync(0xffffffffu, ke1, o);
    }
    if (q < nm && i == 0) {
        const int m = mols[q];
        d.ke[2 * m] = ke0;
        d.ke[2 * m + 1] = ke1;
    }
}

// move_b of flexible chains: acceleration from force and friction
// (src/move_surfactant_b.f90:30-55) with no constraint
__global__ void k_move_free_b(Dev d, const int *mols, int nm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm * NCH) return;
    const int m = mols[t / NCH], g = d.mfirst[m] + t % NCH;
    const double escale = 2.0 / (2.0 + d.eta[d.mrep[m]] * DT);
    const double mi = d.tmass[d.ptype[g]];
    const double axg = d.fx[g] * DTSQ2 / mi, ayg = d.fy[g] * DTSQ2 / mi, azg = d.fz[g] * DTSQ2 / mi;
    d.ax[g] = axg; d.ay[g] = ayg; d.az[g] = azg;
    d.vx[g] = escale * (d.vx[g] + axg);
    d.vy[g] = escale * (d.vy[g] + ayg);
    d.vz[g] = escale * (d.vz[g] + azg);
}

// ---------------------------------------------------------------- launchers

void launch_locate(const Dev &d, int nmol, const int *smols, int nsurf_sites, int per, int nsite, cudaStream_t st) {
    if (per) k_locate_cfg<<<(nsite + 127) / 128, 128, 0, st>>>(d, nsite);
    else k_locate<<<(nmol + nsurf_sites + 127) / 128, 128, 0, st>>>(d, nmol, smols, nsurf_sites);
}
void launch_isub(const Dev &d, int nsurf_sites, const int *surf_mols, int per, cudaStream_t st) {
    if (!nsurf_sites) return;
    if (per) k_isub_cfg<<<(nsurf_sites + 127) / 128, 128, 0, st>>>(d, nsurf_sites, surf_mols);
    else k_isub<<<(nsurf_sites + 31) / 32, 32, 0, st>>>(d, nsurf_sites, surf_mols);
}
// fast = 0 (plain path): the FP64 sweeps above, dividing exactly as the
// reference does; fast = 1 / 2 (mixed paths): the FP64 / FP32 sweeps of
// k_constraint.cu.
void launch_move_a(const Dev &d, const int *wmols, int nw, const int *smols, int ns, int nrep, int nmol, int nsite,
                   double tol, int maxit, int fast, const ConstraintShape &sh, int chains, cudaStream_t st) {
    if (chains) {   // flexible chains: constraints on the waters only
        if (fast) launch_move_a32(d, nw, smols, 0, nmol, nsite, sh, st, tol, maxit, fast == 2, 1);
        else if (nw) k_move_a<3><<<(nw + 127) / 128, 128, 0, st>>>(d, wmols, nw, tol, maxit);
        if (ns) k_move_free_a<<<(ns * 16 + 127) / 128, 128, 0, st>>>(d, smols, ns);
        return;
    }
    if (fast) {
        launch_move_a32(d, nw, smols, ns, nmol, nsite, sh, st, tol, maxit, fast == 2, 0);
    } else {
        if (ns) k_move_a_surf<<<(ns + SURF_BLOCK - 1) / SURF_BLOCK, SURF_BLOCK, 0, st>>>(d, smols, ns, tol, maxit);
        if (nw) k_move_a<3><<<(nw + 127) / 128, 128, 0, st>>>(d, wmols, nw, tol, maxit);
    }
}
void launch_eta(const Dev &d, int nrep, cudaStream_t st) { k_eta<<<nrep * ETA_BLOCKS, ETA_THREADS, 0, st>>>(d); }
void launch_move_b(const Dev &d, const int *wmols, int nw, const int *smols, int ns, int nmol, int nsite, double tol,
                   int maxit, int fast, const ConstraintShape &sh, int chains, cudaStream_t st) {
    if (chains) {
        if (fast) launch_move_b32(d, nw, smols, 0, nmol, nsite, sh, st, tol, maxit, fast == 2, 1);
        else if (nw) k_move_b<3><<<(nw + 127) / 128, 128, 0, st>>>(d, wmols, nw, tol, maxit);
        if (ns) k_move_free_b<<<(ns * NCH + 255) / 256, 256, 0, st>>>(d, smols, ns);
        return;
    }
    if (fast) {
        launch_move_b32(d, nw, smols, ns, nmol, nsite, sh, st, tol, maxit, fast == 2, 0);
    } else {
        if (ns) k_move_b_surf<<<(ns + SURF_BLOCK - 1) / SURF_BLOCK, SURF_BLOCK, 0, st>>>(d, smols, ns, tol, maxit);
        if (nw) k_move_b<3><<<(nw + 127) / 128, 128, 0, st>>>(d, wmols, nw, tol, maxit);
    }
}
void launch_init_accel(const Dev &d, int nsite, cudaStream_t st) {
    k_init_accel<<<(nsite + 255) / 256, 256, 0, st>>>(d, nsite);
}

}  // namespace sesp
