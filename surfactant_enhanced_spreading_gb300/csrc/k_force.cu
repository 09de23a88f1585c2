// Force kernels of the GB300 engine: cell sort, the full-shell short-range
// pair kernel (FP64, or FP32 with compensated accumulation) with the local
// expansion force fused into its epilogue, the order-4 multipole passes,
// walls, graphite and the surfactant intramolecular terms.
//
// The reference splits its short-range work into 39 list kernels
// (src/eval[wS]*.f90) over "Central" and "26" lists built every 10 steps
// (src/build*.f90).  Together they give every site the Coulomb force of all
// sites of other molecules that sit in the 27 cells around its own cell, plus
// the LJ force within rc for the site kinds that carry LJ.  Here that rule is
// one kernel: one CTA per cell, the 27 neighbour cells staged through shared
// memory, each thread accumulating the full force on its own site (no
// third-law scatter, no atomics, so results are bit-reproducible).
#include "k_launch.cuh"

namespace sesp {

static __constant__ Tables cT;

void upload_tables_force(const Tables &t, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(cT, &t, sizeof(Tables), 0, cudaMemcpyHostToDevice, st);
}

constexpr int NEAR_THREADS = 128;
constexpr int SORT_CAP = 2048;

__device__ inline void cell_xyz(const Rep &r, int c, int &ix, int &iy, int &iz) {
    int l = c - r.cell0;
    ix = l % r.nc[0];
    iy = (l / r.nc[0]) % r.nc[1];
    iz = l / (r.nc[0] * r.nc[1]);
}

// ------------------------------------------------------------------ sort

// exclusive prefix sum over one block (blockDim.x a multiple of 32, at most
// 1024): warp shuffles, then the warps' totals; *total gets the block's sum
__device__ inline int block_exscan(int v, int *total) {
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < nw ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    const int res = (w ? ws[w - 1] : 0) + x - v;
    *total = ws[nw - 1];
    __syncthreads();
    return res;
}

__global__ void k_scan(Dev d, int ncell) {
    int per = (ncell + blockDim.x - 1) / blockDim.x;
    int b = threadIdx.x * per, e = min(ncell, b + per);
    int s = 0;
    for (int c = b; c < e; c++) s += d.ccount[c];
    int total;
    int acc = block_exscan(s, &total);
    if (threadIdx.x == 0) d.cstart[ncell] = total;
    for (int c = b; c < e; c++) { d.cstart[c] = acc; acc += d.ccount[c]; d.cfill[c] = 0; }
}

__global__ void k_scatter(Dev d, int nsite) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nsite) return;
    int c = d.sloc[g];
    d.sslot[g] = -1;
    if (c < 0) return;
    int slot = d.cstart[c] + atomicAdd(&d.cfill[c], 1);
    d.srt_site[slot] = g;
}

// The cells around c (offsets -1..1 per axis, wrapped in x and y on the
// periodic preset) that hold a site of site v's molecule, v itself included:
// bit (dx + 1) + 3 (dy + 1) + 9 (dz + 1).
__device__ int molecule_cells(const Dev &d, int c, int v) {
    const Rep r = d.rep[d.crep[c]];
    const int m = d.smol[v], g0 = d.mfirst[m], ns = d.mkind[m] == 0 ? 3 : r.ssite;
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    int mask = 0;
    for (int k = 0; k < ns; k++) {
        const int ck = d.sloc[g0 + k];
        if (ck < 0) continue;
        int jx, jy, jz;
        cell_xyz(r, ck, jx, jy, jz);
        int dx = jx - ix, dy = jy - iy;
        const int dz = jz - iz;
        if (r.per) {
            if (2 * dx > r.nc[0]) dx -= r.nc[0];
            else if (2 * dx < -r.nc[0]) dx += r.nc[0];
            if (2 * dy > r.nc[1]) dy -= r.nc[1];
            else if (2 * dy < -r.nc[1]) dy += r.nc[1];
        }
        if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) mask |= 1 << ((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1));
    }
    return mask;
}

// order the sites of each cell by site index, so the slot order (and with it
// every floating-point sum) is independent of the scatter's atomics
// (order within a cell: sites with LJ first - every kind but water H - then
// water H, each group by site index; cnh[c] counts the first group, so the
// FP32 pair loop runs its LJ test on a prefix of every partner cell only)
constexpr int SORT_HBIT = 1 << 30;   // site indices stay below 2^30
__global__ void k_sort_cells(Dev d) {
    __shared__ int buf[SORT_CAP];
    __shared__ int nonh;
    int c = blockIdx.x;
    int s0 = d.cstart[c], n = d.cstart[c + 1] - s0;
    if (threadIdx.x == 0) nonh = 0;
    if (threadIdx.x == 0 && n > 0) atomicMax(&d.counters[3], (unsigned long long)n);
    __syncthreads();
    if (n > SORT_CAP) {
        // counted as an overflow; the cell keeps the scatter's order (its sums
        // then depend on timing), with every per-slot field still written
        if (threadIdx.x == 0) atomicAdd(&d.counters[1], 1ull);
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int v = d.srt_site[s0 + t];
            d.sslot[v] = s0 + t;
            d.srt_meta[s0 + t] = make_int2(d.smol[v], (int)d.ptype[v]);
            d.srt_key[s0 + t] = d.smol[v] << 5 | (int)d.ptype[v];
            d.srt_xmask[s0 + t] = molecule_cells(d, c, v);
        }
        if (threadIdx.x == 0) d.cnh[c] = n;   // the pair loop then tests every slot for LJ
        return;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int v = d.srt_site[s0 + t];
        const bool h = d.ptype[v] == 1;
        buf[t] = v | (h ? SORT_HBIT : 0);
        if (!h) atomicAdd(&nonh, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) d.cnh[c] = nonh;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int k = buf[t], v = k & (SORT_HBIT - 1);
        int rank = 0;
        for (int u = 0; u < n; u++) rank += buf[u] < k;
        d.srt_site[s0 + rank] = v;
        d.sslot[v] = s0 + rank;
        d.srt_meta[s0 + rank] = make_int2(d.smol[v], (int)d.ptype[v]);
        d.srt_key[s0 + rank] = d.smol[v] << 5 | (int)d.ptype[v];
        d.srt_xmask[s0 + rank] = molecule_cells(d, c, v);
    }
}

void launch_sort(const Dev &d, int nsite, int ncell, cudaStream_t st) {
    k_scan<<<1, 1024, 0, st>>>(d, ncell);
    k_scatter<<<(nsite + 255) / 256, 256, 0, st>>>(d, nsite);
    k_sort_cells<<<ncell, 256, 0, st>>>(d);
}

// ------------------------------------------------------------------ gather

__device__ inline double cell_centre(const Dev &d, const Rep &r, int a, int i) {
    const double *t = d.axis + r.axis0 + (a > 0 ? r.nc[0] : 0) + (a > 1 ? r.nc[1] : 0);
    return t[i];
}

// Slot positions of the step: the site's position (on the periodic preset
// wrapped by the image it had at the last rebuild, so it stays beside its
// frozen cell) and charge, FP64; on the mixed path also FP32 relative to the
// cell centre.
__global__ void k_gather(Dev d, int nslot, int ncell, int mixed) {
    griddep_wait();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) d.near_ctl[0] = 0;   // the pair field's work counter
    if (s >= nslot || s >= d.cstart[ncell]) return;
    int g = d.srt_site[s];
    double x = d.x[g], y = d.y[g], z = d.z[g];
    double q = d.tq[d.ptype[g]];
    const int c = d.sloc[g];
    const Rep &rr = d.rep[d.crep[c]];
    if (rr.per) {
        const short2 im = d.simg[g];
        x -= (double)im.x * rr.rsd[0];
        y -= (double)im.y * rr.rsd[1];
    }
    d.srt_pos[s] = make_double4(x, y, z, q);
    if (mixed) {
        const Rep r = rr;
        int ix, iy, iz;
        cell_xyz(r, c, ix, iy, iz);
        d.srt_pos32[s] = make_float4((float)(x - cell_centre(d, r, 0, ix)), (float)(y - cell_centre(d, r, 1, iy)),
                                     (float)(z - cell_centre(d, r, 2, iz)), (float)q);
    }
}

void launch_gather(const Dev &d, int nslot, int ncell, int mixed, cudaStream_t st) {
    launch_pdl(k_gather, dim3((nslot + 255) / 256 > 0 ? (nslot + 255) / 256 : 1), dim3(256), 0, st, d, nslot, ncell,
               mixed);
}

// ------------------------------------------------------------------ solid harmonics

// T_n^m = r^n P_n^m(cos theta) e^{i m phi} (Condon-Shortley phase), m >= 0,
// built by the Cartesian recurrences
//   T_m^m = -(2m-1)(x+iy) T_{m-1}^{m-1},  T_{m+1}^m = (2m+1) z T_m^m,
//   T_n^m = ((2n-1) z T_{n-1}^m - (n+m-1) r^2 T_{n-2}^m) / (n-m),
// which avoid the angles and the 1/(x^2+y^2) of the reference's spherical
// form (src/evalLjk4.f90:42-66) and so stay accurate next to the z axis.
template <typename R>
struct Cx {
    R re, im;
};
template <typename R>
__device__ inline Cx<R> cmul(Cx<R> a, Cx<R> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <typename R>
__device__ inline Cx<R> cscale(Cx<R> a, R s) { return {a.re * s, a.im * s}; }
template <typename R>
__device__ inline Cx<R> cadd(Cx<R> a, Cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R>
__device__ inline Cx<R> csub(Cx<R> a, Cx<R> b) { return {a.re - b.re, a.im - b.im}; }

// rfctr(n, m) of coefficient ic in the arithmetic's type (the FP32 copy is
// rounded once on the host: GB300 converts at its FP64 rate)
template <typename R>
__device__ __forceinline__ R rfctr_r(int ic) {
    if constexpr (std::is_same<R, float>::value) return cT.rfctr32[ic];
    else return cT.rfctr[ic];
}

// gradient of Phi = sum_n sum_m w_m rfctr(n,m) Re(L_n^m T_n^m) (w_0 = 1, w_m = 2):
// the potential of the local expansion L (25 coefficients, m >= 0 used),
// read as L(ic, re, im).  Both loops unroll, so every coefficient index is a
// constant: the expansion is read straight from its row (no per-thread copy
// in local memory).
template <typename R, typename LF>
__device__ inline void local_grad(const LF &L, R x, R y, R z, R &gx, R &gy, R &gz, R *phi) {
    R r2 = x * x + y * y + z * z;
    Cx<R> Tmm = {R(1), R(0)};
    Cx<R> dmm[3] = {{R(0), R(0)}, {R(0), R(0)}, {R(0), R(0)}};
    R ax = 0, ay = 0, az = 0, pp = 0;
    Cx<R> xy = {x, y};
#pragma unroll
    for (int m = 0; m <= P; m++) {
        if (m > 0) {
            R f = -(R)(2 * m - 1);
            Cx<R> nT = cscale(cmul(xy, Tmm), f);
            Cx<R> nd0 = cscale(cadd(Tmm, cmul(xy, dmm[0])), f);
            Cx<R> nd1 = cscale(cadd(Cx<R>{-Tmm.im, Tmm.re}, cmul(xy, dmm[1])), f);
            Cx<R> nd2 = cscale(cmul(xy, dmm[2]), f);
            Tmm = nT; dmm[0] = nd0; dmm[1] = nd1; dmm[2] = nd2;
        }
        Cx<R> T2 = Tmm, T1 = {R(0), R(0)};
        Cx<R> d2[3] = {dmm[0], dmm[1], dmm[2]};
        Cx<R> d1[3] = {{R(0), R(0)}, {R(0), R(0)}, {R(0), R(0)}};
#pragma unroll
        for (int n = m; n <= P; n++) {
            Cx<R> Tn;
            Cx<R> dn[3];
            if (n == m) {
                Tn = Tmm; dn[0] = dmm[0]; dn[1] = dmm[1]; dn[2] = dmm[2];
            } else if (n == m + 1) {
                R f = (R)(2 * m + 1);
                Tn = cscale(Tmm, f * z);
                dn[0] = cscale(dmm[0], f * z);
                dn[1] = cscale(dmm[1], f * z);
                dn[2] = cscale(cadd(Tmm, cscale(dmm[2], z)), f);
            } else {
                R a = (R)(2 * n - 1), b = (R)(n + m - 1), inv = R(1) / (R)(n - m);
                Tn = cscale(csub(cscale(T1, a * z), cscale(T2, b * r2)), inv);
                dn[0] = cscale(csub(cscale(d1[0], a * z), cadd(cscale(T2, b * 2 * x), cscale(d2[0], b * r2))), inv);
                dn[1] = cscale(csub(cscale(d1[1], a * z), cadd(cscale(T2, b * 2 * y), cscale(d2[1], b * r2))), inv);
                dn[2] = cscale(csub(cadd(cscale(T1, a), cscale(d1[2], a * z)), cadd(cscale(T2, b * 2 * z), cscale(d2[2], b * r2))), inv);
            }
            int ic = n * (n + 1) + m;
            R w = (m == 0 ? R(1) : R(2)) * rfctr_r<R>(ic);
            R lr, li;
            L(ic, lr, li);
            ax += w * (lr * dn[0].re - li * dn[0].im);
            ay += w * (lr * dn[1].re - li * dn[1].im);
            az += w * (lr * dn[2].re - li * dn[2].im);
            pp += w * (lr * Tn.re - li * Tn.im);
            if (n > m) { T2 = T1; d2[0] = d1[0]; d2[1] = d1[1]; d2[2] = d1[2]; }
            T1 = Tn; d1[0] = dn[0]; d1[1] = dn[1]; d1[2] = dn[2];
            if (n == m) { T2 = Tn; d2[0] = dn[0]; d2[1] = dn[1]; d2[2] = dn[2]; }
        }
    }
    gx = ax; gy = ay; gz = az;
    if (phi) *phi = pp;
}

// ------------------------------------------------------------------ near field

// 1/sqrt(r2) in FP64 from the FP32 hardware estimate and two Newton steps
// (relative error of the seed ~2^-22, after two steps at the FP64 rounding level)
__device__ inline double rsqrt_fp64(double r2) {
    double y = (double)rsqrtf((float)r2);
    double h = 0.5 * r2;
    y = y * (1.5 - h * y * y);
    y = y * (1.5 - h * y * y);
    return y;
}

// Work items, rebuilt with the cell lists: one per (target cell, partner row,
// chunk of `tile` target sites).  A partner row is the (up to) 3 cells at
// (dy, dz) from the target cell along x, contiguous in slot order; the 9 rows
// (3 planes x 3 rows) of a cell cover its 27-cell shell.  tile is 64 (two
// target sites per lane of a warp) or 32 (one); the autotuner picks it.
// item.x = cell, item.y = (plane * 3 + row) << 8 | chunk.

// rows of the 27-cell shell inside the box (periodic preset: every row in y)
__device__ inline int near_row_mask(const Rep &r, int iy, int iz) {
    int mask = 0;
    for (int pl = 0; pl < 3; pl++) {
        const int jz = iz + pl - 1;
        if (jz < 0 || jz >= r.nc[2]) continue;
        for (int rw = 0; rw < 3; rw++) {
            const int jy = iy + rw - 1;
            if (!r.per && (jy < 0 || jy >= r.nc[1])) continue;
            mask |= 1 << (pl * 3 + rw);
        }
    }
    return mask;
}

// index along a periodic axis of n cells (j within one box of [0, n))
__device__ __forceinline__ int wrap1(int j, int n) { return j < 0 ? j + n : (j >= n ? j - n : j); }

// the cell (x, y wrapped on the periodic preset) of unwrapped coordinates
__device__ __forceinline__ int shell_cell(const Rep &r, int jx, int jy, int jz) {
    return r.per ? cell_index(r, wrap1(jx, r.nc[0]), wrap1(jy, r.nc[1]), jz) : cell_index(r, jx, jy, jz);
}

// first and last cell along x of a partner row (clipped to a closed box)
__device__ __forceinline__ void row_x(const Rep &r, int ix, int &jx0, int &jx1) {
    if (r.per) { jx0 = ix - 1; jx1 = ix + 1; }
    else { jx0 = ix > 0 ? ix - 1 : 0; jx1 = ix + 1 < r.nc[0] ? ix + 1 : r.nc[0] - 1; }
}

__global__ void k_near_items_count(Dev d, int ncell, int tile) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int ni = d.cstart[c + 1] - d.cstart[c];
    int n = 0;
    if (ni > 0) {
        const Rep r = d.rep[d.crep[c]];
        int ix, iy, iz;
        cell_xyz(r, c, ix, iy, iz);
        n = __popc(near_row_mask(r, iy, iz)) * ((ni + tile - 1) / tile);
    }
    d.near_icount[c] = n;
}

// exclusive scan of the item counts in place (one block), total to near_ctl[1]
__global__ void k_near_items_scan(Dev d, int ncell) {
    const int per = (ncell + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(ncell, b + per);
    int s = 0;
    for (int c = b; c < e; c++) s += d.near_icount[c];
    int total;
    int acc = block_exscan(s, &total);
    if (threadIdx.x == 0) d.near_ctl[1] = total;
    for (int c = b; c < e; c++) { int v = d.near_icount[c]; d.near_icount[c] = acc; acc += v; }
}

// the work items of one cell, counted per cost class in the block's histogram
__device__ inline void near_items_fill_cell(const Dev &d, int c, int ni, int tile, int *hist) {
    const Rep r = d.rep[d.crep[c]];
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    const int mask = near_row_mask(r, iy, iz);
    const int nch = (ni + tile - 1) / tile;
    int jx0, jx1;
    row_x(r, ix, jx0, jx1);
    int k = d.near_icount[c];
    for (int pr = 0; pr < 9; pr++) {
        if (!(mask >> pr & 1)) continue;
        int npart = 0;
        if (r.per) {
            for (int jx = jx0; jx <= jx1; jx++) {
                const int cn = shell_cell(r, jx, iy + pr % 3 - 1, iz + pr / 3 - 1);
                npart += d.cstart[cn + 1] - d.cstart[cn];
            }
        } else {
            const int c0 = cell_index(r, jx0, iy + pr % 3 - 1, iz + pr / 3 - 1);
            npart = d.cstart[c0 + (jx1 - jx0) + 1] - d.cstart[c0];
        }
        for (int ch = 0; ch < nch; ch++) {
            const int nt = min(tile, ni - ch * tile);
            const int cls = 31 - __clz(nt * npart + 1);
            d.near_items_tmp[k] = make_int2(c, pr << 24 | ch);
            d.near_cls[k] = cls;
            atomicAdd(&hist[cls], 1);
            k++;
        }
    }
}

// Items in cell order into near_items_tmp, each with a cost class:
// floor(log2(targets x partners in its row)).
__global__ void k_near_items_fill(Dev d, int ncell, int tile) {
    __shared__ int hist[32];   // the block's items per class, added to the global counts once
    if (threadIdx.x < 32) hist[threadIdx.x] = 0;
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int ni = c < ncell ? d.cstart[c + 1] - d.cstart[c] : 0;
    if (ni > 0) near_items_fill_cell(d, c, ni, tile, hist);
    __syncthreads();
    if (threadIdx.x < 32 && hist[threadIdx.x]) atomicAdd(&d.near_ctl[2 + threadIdx.x], hist[threadIdx.x]);
}

// start of each cost class in the final order, most expensive class first
__global__ void k_near_items_classes(Dev d) {
    if (threadIdx.x != 0) return;
    int *bcount = d.near_ctl + 2, *bnext = d.near_ctl + 34;
    int acc = 0;
    for (int b = 31; b >= 0; b--) { bnext[b] = acc; acc += bcount[b]; }
}

// Items into near_items by class.  Within a class the order depends on
// thread timing; it only decides which warp takes which item first, and every
// item's arithmetic is the same whatever its position.
__global__ void k_near_items_place(Dev d) {
    __shared__ int cnt[32], base[32];   // the block's items per class and their reserved range
    if (threadIdx.x < 32) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int cls = -1, rank = 0;
    if (k < d.near_ctl[1]) {
        cls = d.near_cls[k];
        rank = atomicAdd(&cnt[cls], 1);
    }
    __syncthreads();
    if (threadIdx.x < 32 && cnt[threadIdx.x]) base[threadIdx.x] = atomicAdd(&d.near_ctl[34 + threadIdx.x], cnt[threadIdx.x]);
    __syncthreads();
    if (cls >= 0) d.near_items[base[cls] + rank] = d.near_items_tmp[k];
}

void launch_near_items(const Dev &d, int ncell, int nitems_max, int tile, cudaStream_t st) {
    cudaMemsetAsync(d.near_ctl + 2, 0, 64 * sizeof(int), st);
    k_near_items_count<<<(ncell + 255) / 256, 256, 0, st>>>(d, ncell, tile);
    k_near_items_scan<<<1, 1024, 0, st>>>(d, ncell);
    k_near_items_fill<<<(ncell + 255) / 256, 256, 0, st>>>(d, ncell, tile);
    k_near_items_classes<<<1, 32, 0, st>>>(d);
    k_near_items_place<<<(nitems_max + 255) / 256, 256, 0, st>>>(d);
}

// One partner's force on the two target sites of a lane (src/evalw1w1n.f90:86-104
// form): qq / r^3 without cutoff plus 48 eps sg6 r^-6 (sg6 r^-6 - 1/2) / r^2
// within rc; zero for a partner of the same molecule (src/evalSS.f90:36).  The
// LJ part runs only when some lane of the warp has a target within rc of the
// partner (the partner is the same for the whole warp).
// The pair's (48 eps sg6, sg6) from the kind-pair table (the
// Lorentz-Berthelot rule of src/init_arrays.f90:476-502, formed in FP64;
// FP32 copy for the FP32 path).
struct Tgt32 {
    float x, y, z, q;   // position relative to the target cell's centre, shifted into the partner cell's frame; q * xpi
    int m;              // molecule
    int trow;           // kind * NTYPE: the target's row of the kind-pair table
};
struct Tgt64 {
    double x, y, z, q;
    int m, trow;        // molecule, type * NTYPE
};

// 1/sqrt(x) of the special-function unit (the approximation rsqrtf uses)
// without the handling of denormal inputs: pair distances are never
// denormal, so the result is rsqrtf's and the fix-up instructions go
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Per-target force sums of an FP32 work item.  COMP: compensated (Kahan)
// summation, each term's rounding error carried in a second register and
// folded back when the sum is read.
template <int K, bool COMP>
struct Acc32 {
    float f[K][3];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int j = 0; j < K; j++) f[j][0] = f[j][1] = f[j][2] = 0.f;
    }
    __device__ __forceinline__ void add(int j, float dx, float dy, float dz, float ft) {
        f[j][0] = __fmaf_rn(dx, ft, f[j][0]); f[j][1] = __fmaf_rn(dy, ft, f[j][1]); f[j][2] = __fmaf_rn(dz, ft, f[j][2]);
    }
    __device__ __forceinline__ float get(int j, int a) const { return f[j][a]; }
};
template <int K>
struct Acc32<K, true> {
    float f[K][3], e[K][3];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int j = 0; j < K; j++)
#pragma unroll
            for (int a = 0; a < 3; a++) f[j][a] = e[j][a] = 0.f;
    }
    __device__ __forceinline__ void add1(float &s, float &c, float v) {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ void add(int j, float dx, float dy, float dz, float ft) {
        add1(f[j][0], e[j][0], __fmul_rn(dx, ft));
        add1(f[j][1], e[j][1], __fmul_rn(dy, ft));
        add1(f[j][2], e[j][2], __fmul_rn(dz, ft));
    }
    __device__ __forceinline__ float get(int j, int a) const { return __fsub_rn(f[j][a], e[j][a]); }
};

// FP32 path, K target sites per lane: one partner against targets t[0..K),
// Coulomb plus, for a partner with LJ, the LJ term of each target within rc
// (run when some lane of the warp has one); pairk_coul32 for a water-H
// partner (no LJ).  A partner of the target's own molecule (and the target
// itself, at r = 0) is excluded by one select that zeroes the reciprocal
// distance: its Coulomb and LJ terms are then exactly zero (EXCL: only
// in partner cells that hold a site of some target's molecule).
template <int K, bool EXCL, bool COMP>
__device__ __forceinline__ void pairk_acc32(const Tgt32 (&t)[K], float4 pj, int key, const float2 *ljt, float rc2,
                                            Acc32<K, COMP> &f) {
    const int mj = key >> 5, tj = key & 31;
    float dx[K], dy[K], dz[K], r2[K], ir2[K], ft[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
        dx[j] = __fsub_rn(t[j].x, pj.x); dy[j] = __fsub_rn(t[j].y, pj.y); dz[j] = __fsub_rn(t[j].z, pj.z);
        r2[j] = __fmaf_rn(dz[j], dz[j], __fmaf_rn(dy[j], dy[j], __fmul_rn(dx[j], dx[j])));
        const float ira = EXCL && mj == t[j].m ? 0.f : rsqrt_ftz(r2[j]);
        ir2[j] = __fmul_rn(ira, ira);
        ft[j] = __fmul_rn(__fmul_rn(__fmul_rn(t[j].q, pj.w), ira), ir2[j]);
    }
    {   // (a water H in the prefix, only in an overflowing cell, has zero LJ table entries)
        bool n[K], any = false;
#pragma unroll
        for (int j = 0; j < K; j++) { n[j] = r2[j] <= rc2; any = any || n[j]; }
        if (__any_sync(0xffffffffu, any)) {
#pragma unroll
            for (int j = 0; j < K; j++) {
                const float2 v = ljt[t[j].trow + tj];
                const float r6 = __fmul_rn(__fmul_rn(ir2[j], ir2[j]), ir2[j]);   // zero for an excluded partner
                const float w = __fmaf_rn(v.y, r6, -0.5f);
                ft[j] = __fmaf_rn(__fmul_rn(__fmul_rn(n[j] ? v.x : 0.f, r6), w), ir2[j], ft[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < K; j++) f.add(j, dx[j], dy[j], dz[j], ft[j]);
}
// (t[j].q already holds q_target xpi q_H: every water H carries the same charge)
template <int K, bool EXCL, bool COMP>
__device__ __forceinline__ void pairk_coul32(const Tgt32 (&t)[K], float4 pj, int mj, Acc32<K, COMP> &f) {
#pragma unroll
    for (int j = 0; j < K; j++) {
        const float dx = __fsub_rn(t[j].x, pj.x), dy = __fsub_rn(t[j].y, pj.y), dz = __fsub_rn(t[j].z, pj.z);
        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
        const float ira = EXCL && mj == t[j].m ? 0.f : rsqrt_ftz(r2);
        const float ft = __fmul_rn(__fmul_rn(t[j].q, ira), __fmul_rn(ira, ira));
        f.add(j, dx, dy, dz, ft);
    }
}

// Two targets per lane in Blackwell's paired FP32 arithmetic (fma / add /
// mul .rn.f32x2: one instruction for both targets; the reciprocal square
// root stays one MUFU each).  The pair field is issue-bound, so half the
// FP32 instructions of the two-target items is most of its gain.  The
// scalar forms above spell out the same roundings in the same order
// (explicit __fmaf_rn / __fmul_rn / __fsub_rn, so the compiler contracts
// nothing of its own): a target's force does not depend on whether its item
// took one, two or four targets per lane, i.e. on the launch shape.
// Water-H partners, no exclusion test, plain sums:
__device__ __forceinline__ void coul_h_x2(const Tgt32 (&u)[2], const float4 *wpos, int n, float (&f)[2][3]) {
    const float2 tx = make_float2(u[0].x, u[1].x), ty = make_float2(u[0].y, u[1].y), tz = make_float2(u[0].z, u[1].z);
    const float2 tq = make_float2(u[0].q, u[1].q);
    float2 fx = make_float2(f[0][0], f[1][0]), fy = make_float2(f[0][1], f[1][1]), fz = make_float2(f[0][2], f[1][2]);
#pragma unroll 2
    for (int k = 0; k < n; k++) {
        const float4 p = wpos[k];
        const float2 dx = __fadd2_rn(tx, make_float2(-p.x, -p.x));
        const float2 dy = __fadd2_rn(ty, make_float2(-p.y, -p.y));
        const float2 dz = __fadd2_rn(tz, make_float2(-p.z, -p.z));
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        const float2 ira = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
        const float2 ft = __fmul2_rn(__fmul2_rn(tq, ira), __fmul2_rn(ira, ira));
        fx = __ffma2_rn(dx, ft, fx); fy = __ffma2_rn(dy, ft, fy); fz = __ffma2_rn(dz, ft, fz);
    }
    f[0][0] = fx.x; f[1][0] = fx.y; f[0][1] = fy.x; f[1][1] = fy.y; f[0][2] = fz.x; f[1][2] = fz.y;
}
// the LJ-carrying prefix with both targets of a lane in f32x2 arithmetic
// (same-molecule test per target; LJ only when some lane has a target within rc)
__device__ __forceinline__ void lj_x2(const Tgt32 (&u)[2], const float4 *wpos, const int *wkey, int n, const float2 *ljt,
                                      float rc2, float (&f)[2][3]) {
    const float2 tx = make_float2(u[0].x, u[1].x), ty = make_float2(u[0].y, u[1].y), tz = make_float2(u[0].z, u[1].z);
    const float2 tq = make_float2(u[0].q, u[1].q);
    float2 fx = make_float2(f[0][0], f[1][0]), fy = make_float2(f[0][1], f[1][1]), fz = make_float2(f[0][2], f[1][2]);
#pragma unroll 2
    for (int k = 0; k < n; k++) {
        const float4 p = wpos[k];
        const int key = wkey[k], mj = key >> 5, tj = key & 31;
        const float2 dx = __fadd2_rn(tx, make_float2(-p.x, -p.x));
        const float2 dy = __fadd2_rn(ty, make_float2(-p.y, -p.y));
        const float2 dz = __fadd2_rn(tz, make_float2(-p.z, -p.z));
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        const float2 ira = make_float2(mj == u[0].m ? 0.f : rsqrt_ftz(r2.x), mj == u[1].m ? 0.f : rsqrt_ftz(r2.y));
        const float2 ir2 = __fmul2_rn(ira, ira);
        float2 ft = __fmul2_rn(__fmul2_rn(__fmul2_rn(tq, make_float2(p.w, p.w)), ira), ir2);
        const bool n0 = r2.x <= rc2, n1 = r2.y <= rc2;
        if (__any_sync(0xffffffffu, n0 || n1)) {
            const float2 v0 = ljt[u[0].trow + tj], v1 = ljt[u[1].trow + tj];
            const float2 r6 = __fmul2_rn(__fmul2_rn(ir2, ir2), ir2);
            const float2 on = make_float2(n0 ? v0.x : 0.f, n1 ? v1.x : 0.f);
            const float2 w = __ffma2_rn(make_float2(v0.y, v1.y), r6, make_float2(-0.5f, -0.5f));
            ft = __ffma2_rn(__fmul2_rn(__fmul2_rn(on, r6), w), ir2, ft);
        }
        fx = __ffma2_rn(dx, ft, fx); fy = __ffma2_rn(dy, ft, fy); fz = __ffma2_rn(dz, ft, fz);
    }
    f[0][0] = fx.x; f[1][0] = fx.y; f[0][1] = fy.x; f[1][1] = fy.y; f[0][2] = fz.x; f[1][2] = fz.y;
}
// water-H partners with the same-molecule test, f32x2
__device__ __forceinline__ void coul_h_x2_excl(const Tgt32 (&u)[2], const float4 *wpos, const int *wkey, int n,
                                               float (&f)[2][3]) {
    const float2 tx = make_float2(u[0].x, u[1].x), ty = make_float2(u[0].y, u[1].y), tz = make_float2(u[0].z, u[1].z);
    const float2 tq = make_float2(u[0].q, u[1].q);
    float2 fx = make_float2(f[0][0], f[1][0]), fy = make_float2(f[0][1], f[1][1]), fz = make_float2(f[0][2], f[1][2]);
#pragma unroll 1
    for (int k = 0; k < n; k++) {
        const float4 p = wpos[k];
        const int mj = wkey[k] >> 5;
        const float2 dx = __fadd2_rn(tx, make_float2(-p.x, -p.x));
        const float2 dy = __fadd2_rn(ty, make_float2(-p.y, -p.y));
        const float2 dz = __fadd2_rn(tz, make_float2(-p.z, -p.z));
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        const float2 ira = make_float2(mj == u[0].m ? 0.f : rsqrt_ftz(r2.x), mj == u[1].m ? 0.f : rsqrt_ftz(r2.y));
        const float2 ft = __fmul2_rn(__fmul2_rn(tq, ira), __fmul2_rn(ira, ira));
        fx = __ffma2_rn(dx, ft, fx); fy = __ffma2_rn(dy, ft, fy); fz = __ffma2_rn(dz, ft, fz);
    }
    f[0][0] = fx.x; f[1][0] = fx.y; f[0][1] = fy.x; f[1][1] = fy.y; f[0][2] = fz.x; f[1][2] = fz.y;
}

// One partner cell's sites (slots t0..t1, LJ-carrying ones before th) on
// the targets u, in the partner cell's frame.  The LJ-carrying prefix always
// tests for partners of a target's own molecule; the water-H suffix (about
// two thirds of the pairs) does so only when EXCL says some target's molecule
// has a site in this cell.  Only that loop comes in two versions, and the
// testing one is not unrolled: a second LJ loop and more unrolling cost more
// in instruction-cache stalls than they saved in instructions.  The warp
// stages 32 partners at a time in its shared-memory slot (one coalesced
// load per lane) and reads them back as broadcasts: shorter load latency
// than a broadcast L1 load per partner.
// Two-target items of the plain mixed path take the paired forms above.
template <int K, bool EXCL, bool COMP>
__device__ __forceinline__ void near_cell32(const float4 *__restrict__ pos32, const int *__restrict__ keys,
                                            Tgt32 (&u)[K], int t0, int th, int t1, const float2 *ljt, float rc2,
                                            Acc32<K, COMP> &f, float4 *wpos, int *wkey, int lane) {
    for (int b0 = t0; b0 < th; b0 += 32) {
        const int n = min(32, th - b0);
        __syncwarp();
        if (lane < n) { wpos[lane] = pos32[b0 + lane]; wkey[lane] = keys[b0 + lane]; }
        __syncwarp();
        if constexpr (K == 2 && !COMP) {
            lj_x2(u, wpos, wkey, n, ljt, rc2, f.f);
        } else {
#pragma unroll 2
            for (int k = 0; k < n; k++) pairk_acc32<K, true, COMP>(u, wpos[k], wkey[k], ljt, rc2, f);
        }
    }
    if (th < t1) {
        const float qh = pos32[th].w;
#pragma unroll
        for (int j = 0; j < K; j++) u[j].q *= qh;
    }
    if constexpr (EXCL) {
        for (int b0 = th; b0 < t1; b0 += 32) {
            const int n = min(32, t1 - b0);
            __syncwarp();
            if (lane < n) { wpos[lane] = pos32[b0 + lane]; wkey[lane] = keys[b0 + lane]; }
            __syncwarp();
            if constexpr (K == 2 && !COMP) {
                coul_h_x2_excl(u, wpos, wkey, n, f.f);
            } else {
#pragma unroll 1
                for (int k = 0; k < n; k++) pairk_coul32<K, true, COMP>(u, wpos[k], wkey[k] >> 5, f);
            }
        }
    } else {
        for (int b0 = th; b0 < t1; b0 += 32) {
            const int n = min(32, t1 - b0);
            __syncwarp();
            if (lane < n) wpos[lane] = pos32[b0 + lane];
            __syncwarp();
            if constexpr (K == 2 && !COMP) {
                coul_h_x2(u, wpos, n, f.f);
            } else {
#pragma unroll 2
                for (int k = 0; k < n; k++) pairk_coul32<K, false, COMP>(u, wpos[k], 0, f);
            }
        }
    }
}

// One FP32 work item with K target sites per lane (lane + 32 j of the chunk):
// the force of partner row pr on them, written to that row's partial.
template <int K, bool PER, bool COMP>
__device__ __forceinline__ void near_item32(const Dev &d, const float2 *ljt, int nslot, int c, int pr, int first,
                                            int ni, int lane, float4 *wpos, int *wkey) {
    const float4 *__restrict__ pos32 = d.srt_pos32;
    const int *__restrict__ keys = d.srt_key;
    const int dzc = pr / 3 - 1, dyc = pr % 3 - 1;
    const int s0 = d.cstart[c];
    const Rep r = d.rep[d.crep[c]];
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    const int jy = iy + dyc, jz = iz + dzc;
    int jx0, jx1;
    if constexpr (PER) { jx0 = ix - 1; jx1 = ix + 1; }
    else row_x(r, ix, jx0, jx1);
    const int wy = PER ? wrap1(jy, r.nc[1]) : jy;
    Tgt32 t[K];
    bool act[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
        const int i = first + lane + 32 * j;
        act[j] = i < ni;
        t[j] = {0.f, 0.f, 0.f, 0.f, -1, 0};
        if (act[j]) {
            const float4 p = pos32[s0 + i];
            const int kk = keys[s0 + i];
            t[j] = {p.x, p.y, p.z, p.w * (float)XPI, kk >> 5, (kk & 31) * NTYPE};
        }
    }
    // the row's partner cells holding a site of some target's molecule:
    // bit jx - ix + 1 (from the targets' molecule-cell masks)
    unsigned xm = 0;
    const int rowsh = 3 * (dyc + 1) + 9 * (dzc + 1);
#pragma unroll
    for (int j = 0; j < K; j++)
        if (act[j]) xm |= ((unsigned)d.srt_xmask[s0 + first + lane + 32 * j] >> rowsh) & 7u;
    const unsigned excl = __reduce_or_sync(0xffffffffu, xm);
    const float rc2 = (float)(RC * RC);
    const float sy = (float)(-dyc * RS), sz = (float)(-dzc * RS);
    Acc32<K, COMP> f;
    f.zero();
    for (int jx = jx0; jx <= jx1; jx++) {
        // positions are cell-relative: the shift is the unwrapped offset
        const int cn = cell_index(r, PER ? wrap1(jx, r.nc[0]) : jx, wy, jz);
        const int t0 = d.cstart[cn], t1 = d.cstart[cn + 1];
        const float sx = (float)((ix - jx) * RS);
        Tgt32 u[K];   // targets in the partner cell's frame
#pragma unroll
        for (int j = 0; j < K; j++) { u[j] = t[j]; u[j].x += sx; u[j].y += sy; u[j].z += sz; }
        // partners with LJ first (the cell sort puts water H last)
        const int th = t0 + d.cnh[cn];
        // (items of one target per lane keep one loop body: less code)
        if (K == 1 || ((excl >> (jx - ix + 1)) & 1u)) near_cell32<K, true, COMP>(pos32, keys, u, t0, th, t1, ljt, rc2, f, wpos, wkey, lane);
        else near_cell32<K, false, COMP>(pos32, keys, u, t0, th, t1, ljt, rc2, f, wpos, wkey, lane);
    }
    float *part = (float *)d.near_part + (size_t)pr * 3 * nslot;   // FP32 row partials on the mixed path
#pragma unroll
    for (int j = 0; j < K; j++)
        if (act[j]) {
            const size_t o = 3 * (size_t)(s0 + first + lane + 32 * j);
            part[o] = f.get(j, 0); part[o + 1] = f.get(j, 1); part[o + 2] = f.get(j, 2);
        }
}

__device__ __forceinline__ void pair2_acc64(const Tgt64 &a, const Tgt64 &b, bool two, double4 pj, int key,
                                            const double2 *lj, double rc2, double (&fa)[3], double (&fb)[3]) {
    const int mj = key >> 5, tj = key & 31;
    const double dxa = a.x - pj.x, dya = a.y - pj.y, dza = a.z - pj.z;
    const bool samea = mj == a.m;
    const double r2a = samea ? 1.0 : dxa * dxa + dya * dya + dza * dza;
    const double ira = rsqrt_fp64(r2a), ir2a = ira * ira;
    double fta = (samea ? 0.0 : a.q * pj.w) * ira * ir2a;
    double dxb = 0.0, dyb = 0.0, dzb = 0.0, r2b = 1.0, ir2b = 0.0, ftb = 0.0;
    bool sameb = true;
    if (two) {
        dxb = b.x - pj.x; dyb = b.y - pj.y; dzb = b.z - pj.z;
        sameb = mj == b.m;
        r2b = sameb ? 1.0 : dxb * dxb + dyb * dyb + dzb * dzb;
        const double irb = rsqrt_fp64(r2b);
        ir2b = irb * irb;
        ftb = (sameb ? 0.0 : b.q * pj.w) * irb * ir2b;
    }
    if (tj != 1) {
        const bool na = r2a <= rc2 && !samea, nb = two && r2b <= rc2 && !sameb;
        if (__any_sync(0xffffffffu, na || nb)) {   // a zero LJ term leaves the sum unchanged, so skipping it is exact
            {
                const double2 v = lj[a.trow + tj];
                const double on = na ? v.x : 0.0;
                const double r6 = ir2a * ir2a * ir2a;
                fta += on * r6 * (v.y * r6 - 0.5) * ir2a;
            }
            if (two) {
                const double2 v = lj[b.trow + tj];
                const double on = nb ? v.x : 0.0;
                const double r6 = ir2b * ir2b * ir2b;
                ftb += on * r6 * (v.y * r6 - 0.5) * ir2b;
            }
        }
    }
    fa[0] += dxa * fta; fa[1] += dya * fta; fa[2] += dza * fta;
    if (two) { fb[0] += dxb * ftb; fb[1] += dyb * ftb; fb[2] += dzb * ftb; }
}

// Near field as a persistent kernel: each warp takes items from a global
// counter until none are left, and for its item sums the force of one
// partner row on 64 target sites (2 per lane), reading the partners as
// broadcasts (FP32: staged 32 at a time in the warp's shared-memory slot;
// FP64: one broadcast L1 load per partner).  Each item
// writes its own partial per slot (near_part[plane * 3 + row]); k_near_finish
// adds the 9 partials in a fixed order.  Which warp takes which item does not
// change any arithmetic, so results are bit-reproducible.
// MIXED: FP32 positions relative to the cell centres, FP32 pair terms summed
// in FP32 over one row (at most 3 cells).
// PER: the periodic preset's instantiation (rows wrap around x and y)
// COMP: compensated (Kahan) FP32 sums per target (SESP_MIXED_COMP)
// (the FP32 two-target instantiations are held to 8 CTAs per SM, 64
// registers: the paired loops want 67 and the compensated ones 80, and
// fewer CTAs per SM ran slower)
template <bool MIXED, int KMAX, bool PER, bool COMP = false>
__global__ void __launch_bounds__(NEAR_THREADS, (MIXED && KMAX == 2) ? 8 : 1) k_near(Dev d, int nslot, int tile) {
    griddep_wait();
    __shared__ float2 s_lj32[MIXED ? NTYPE * NTYPE : 1];
    __shared__ float4 s_stage[MIXED ? NEAR_THREADS / 32 : 1][32];
    __shared__ int s_key[MIXED ? NEAR_THREADS / 32 : 1][32];
    __shared__ double2 s_lj64[MIXED ? 1 : NTYPE * NTYPE];
    if constexpr (MIXED) {
        for (int t = threadIdx.x; t < NTYPE * NTYPE; t += blockDim.x) s_lj32[t] = d.ljt32[t];
    } else {
        for (int t = threadIdx.x; t < NTYPE * NTYPE; t += blockDim.x) s_lj64[t] = d.ljt[t];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int nitems = d.near_ctl[1];
    const float4 *__restrict__ pos32 = d.srt_pos32;
    const double4 *__restrict__ pos64 = d.srt_pos;
    const int *__restrict__ keys = d.srt_key;
    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&d.near_ctl[0], 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= nitems) break;
        const int2 item = d.near_items[k];
        const int c = item.x, pr = item.y >> 24, chunk = item.y & 0xFFFFFF;
        const int dzc = pr / 3 - 1, dyc = pr % 3 - 1;
        const int s0 = d.cstart[c], ni = d.cstart[c + 1] - s0;
        const int i0 = chunk * tile + lane, i1 = tile == 64 ? i0 + 32 : ni;
        const bool a0 = i0 < ni, a1 = i1 < ni;
        const bool two = __any_sync(0xffffffffu, a1);
        const Rep r = d.rep[d.crep[c]];
        int ix, iy, iz;
        cell_xyz(r, c, ix, iy, iz);
        const int jy = iy + dyc, jz = iz + dzc;
        int jx0, jx1;
        row_x(r, ix, jx0, jx1);
        double *part = d.near_part + (size_t)pr * 3 * nslot;
        if constexpr (MIXED) {
            // K = targets per lane: ceil(targets of the chunk / 32), at most KMAX
            const int nt = min(tile, ni - chunk * tile), kk = (nt + 31) >> 5;
            if (kk <= 1) near_item32<1, PER, COMP>(d, s_lj32, nslot, c, pr, chunk * tile, ni, lane, s_stage[threadIdx.x >> 5], s_key[threadIdx.x >> 5]);
            else if (kk == 2 || KMAX == 2) near_item32<2, PER, COMP>(d, s_lj32, nslot, c, pr, chunk * tile, ni, lane, s_stage[threadIdx.x >> 5], s_key[threadIdx.x >> 5]);
            else if (kk == 3) near_item32<(KMAX > 2 ? 3 : 2), PER, COMP>(d, s_lj32, nslot, c, pr, chunk * tile, ni, lane, s_stage[threadIdx.x >> 5], s_key[threadIdx.x >> 5]);
            else near_item32<KMAX, PER, COMP>(d, s_lj32, nslot, c, pr, chunk * tile, ni, lane, s_stage[threadIdx.x >> 5], s_key[threadIdx.x >> 5]);
        } else {
            Tgt64 ta = {0.0, 0.0, 0.0, 0.0, -1, 0}, tb = ta;
            if (a0) {
                const double4 p = pos64[s0 + i0];
                const int kk = keys[s0 + i0];
                ta = {p.x, p.y, p.z, p.w * XPI, kk >> 5, (kk & 31) * NTYPE};
            }
            if (a1) {
                const double4 p = pos64[s0 + i1];
                const int kk = keys[s0 + i1];
                tb = {p.x, p.y, p.z, p.w * XPI, kk >> 5, (kk & 31) * NTYPE};
            }
            const double rc2 = RC * RC;
            double fa[3] = {0.0, 0.0, 0.0}, fb[3] = {0.0, 0.0, 0.0};
            if constexpr (PER) {
                // one cell at a time: a partner cell across a periodic face
                // holds positions one box length away, so the targets move
                // by that length into its frame
                const int wy = wrap1(jy, r.nc[1]);
                const double sy = (double)(jy - wy) * RS;
                for (int jx = jx0; jx <= jx1; jx++) {
                    const int wx = wrap1(jx, r.nc[0]);
                    const double sx = (double)(jx - wx) * RS;
                    Tgt64 ua = ta, ub = tb;
                    ua.x -= sx; ua.y -= sy; ub.x -= sx; ub.y -= sy;
                    const int cn = cell_index(r, wx, wy, jz);
                    const int t0 = d.cstart[cn], t1 = d.cstart[cn + 1];
#pragma unroll 2
                    for (int sl = t0; sl < t1; sl++) pair2_acc64(ua, ub, two, pos64[sl], keys[sl], s_lj64, rc2, fa, fb);
                }
            } else {
                const int ca = cell_index(r, jx0, jy, jz);
                const int t0 = d.cstart[ca], t1 = d.cstart[ca + (jx1 - jx0) + 1];
#pragma unroll 2
                for (int sl = t0; sl < t1; sl++) pair2_acc64(ta, tb, two, pos64[sl], keys[sl], s_lj64, rc2, fa, fb);
            }
            if (a0) {
                const size_t o = 3 * (size_t)(s0 + i0);
                part[o] = fa[0]; part[o + 1] = fa[1]; part[o + 2] = fa[2];
            }
            if (a1) {
                const size_t o = 3 * (size_t)(s0 + i1);
                part[o] = fb[0]; part[o + 1] = fb[1]; part[o + 2] = fb[2];
            }
        }
    }
}

// Sum of the 9 row partials (fixed order) plus the local-expansion force of
// src/evalLjk4.f90:31-282 for every slot; writes nf.
template <bool MIXED, bool COMP = false>
__global__ void k_near_finish(Dev d, int nslot, int ncell, int terms) {
    griddep_wait();
    typedef typename std::conditional<MIXED, float, double>::type R;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslot || s >= d.cstart[ncell]) return;
    const int g = d.srt_site[s];
    const int c = d.sloc[g];
    const Rep r = d.rep[d.crep[c]];
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    // the 9 row partials in row order: FP32 rows summed in FP32 on the mixed
    // path (one conversion to FP64 per component), FP64 on the plain path
    // (COMP: compensated FP32 sums of the rows, as in the pair field)
    R fx = 0, fy = 0, fz = 0;
    if (terms & SESP_T_NEAR) {
        const int mask = near_row_mask(r, iy, iz);
        const R *part = (const R *)d.near_part;
        R ex = 0, ey = 0, ez = 0;
        for (int pr = 0; pr < 9; pr++) {
            if (!(mask >> pr & 1)) continue;
            const R *p = part + (size_t)pr * 3 * nslot + 3 * (size_t)s;
            if constexpr (COMP) {
                R v[3] = {p[0], p[1], p[2]}, *sm[3] = {&fx, &fy, &fz}, *em[3] = {&ex, &ey, &ez};
                for (int a = 0; a < 3; a++) {
                    const float y = __fsub_rn(v[a], *em[a]);
                    const float t = __fadd_rn(*sm[a], y);
                    *em[a] = __fsub_rn(__fsub_rn(t, *sm[a]), y);
                    *sm[a] = t;
                }
            } else {
                fx += p[0]; fy += p[1]; fz += p[2];
            }
        }
        if constexpr (COMP) { fx = __fsub_rn(fx, ex); fy = __fsub_rn(fy, ey); fz = __fsub_rn(fz, ez); }
    }
    if (terms & SESP_T_FAR) {
        R x, y, z, q;
        // the cell's local expansion: the FP32 copy of L4 on the mixed path
        typedef typename std::conditional<MIXED, float2, double2>::type R2;
        const R2 *Lc = (MIXED ? (const R2 *)d.L4f : (const R2 *)d.L4) + (size_t)c * LP;
        auto L = [&](int k, R &re, R &im) { const R2 v = Lc[k]; re = v.x; im = v.y; };
        if constexpr (MIXED) {   // the cell-relative FP32 position: no FP64 work
            const float4 p = d.srt_pos32[s];
            x = p.x; y = p.y; z = p.z; q = p.w * (float)XPI;
        } else {
            const double4 pd = d.srt_pos[s];
            x = pd.x - cell_centre(d, r, 0, ix); y = pd.y - cell_centre(d, r, 1, iy); z = pd.z - cell_centre(d, r, 2, iz);
            q = pd.w * XPI;
        }
        R gx, gy, gz;
        local_grad<R>(L, x, y, z, gx, gy, gz, nullptr);
        fx -= q * gx; fy -= q * gy; fz -= q * gz;
    }
    d.nf[3 * (size_t)s] = (double)fx; d.nf[3 * (size_t)s + 1] = (double)fy; d.nf[3 * (size_t)s + 2] = (double)fz;
}

// mixed: 0 plain FP64, 1 FP32, 2 FP32 with compensated sums
template <bool PER>
int near_max_ctas_t(int mixed, int tile) {
    int nb = 0;
    if (mixed == 2 && tile > 64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_near<true, 4, PER, true>, NEAR_THREADS, 0);
    else if (mixed == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_near<true, 2, PER, true>, NEAR_THREADS, 0);
    else if (mixed && tile > 64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_near<true, 4, PER>, NEAR_THREADS, 0);
    else if (mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_near<true, 2, PER>, NEAR_THREADS, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_near<false, 2, PER>, NEAR_THREADS, 0);
    return nb > 0 ? nb : 1;
}
int near_max_ctas_per_sm(int mixed, int tile, int per) {
    return per ? near_max_ctas_t<true>(mixed, tile) : near_max_ctas_t<false>(mixed, tile);
}

// reset_counter: the work counter is cleared here (otherwise the step's
// gather kernel has cleared it)
template <bool PER>
void launch_near_t(const Dev &d, int nslot, int mixed, const NearShape &shape, cudaStream_t st) {
    const dim3 g(shape.grid), b(NEAR_THREADS);
    if (mixed == 2 && shape.tile > 64) launch_pdl(k_near<true, 4, PER, true>, g, b, 0, st, d, nslot, shape.tile);
    else if (mixed == 2) launch_pdl(k_near<true, 2, PER, true>, g, b, 0, st, d, nslot, shape.tile);
    else if (mixed && shape.tile > 64) launch_pdl(k_near<true, 4, PER>, g, b, 0, st, d, nslot, shape.tile);
    else if (mixed) launch_pdl(k_near<true, 2, PER>, g, b, 0, st, d, nslot, shape.tile);
    else launch_pdl(k_near<false, 2, PER>, g, b, 0, st, d, nslot, shape.tile);
}

void launch_near(const Dev &d, int ncell, int nslot, int mixed, int terms, const NearShape &shape, cudaStream_t st,
                 bool reset_counter, int per) {
    if (terms & SESP_T_NEAR) {
        if (reset_counter) cudaMemsetAsync(d.near_ctl, 0, sizeof(int), st);
        if (per) launch_near_t<true>(d, nslot, mixed, shape, st);
        else launch_near_t<false>(d, nslot, mixed, shape, st);
    }
    const dim3 g((nslot + 127) / 128 > 0 ? (nslot + 127) / 128 : 1), b(128);
    if (mixed == 2) launch_pdl(k_near_finish<true, true>, g, b, 0, st, d, nslot, ncell, terms);
    else if (mixed) launch_pdl(k_near_finish<true>, g, b, 0, st, d, nslot, ncell, terms);
    else launch_pdl(k_near_finish<false>, g, b, 0, st, d, nslot, ncell, terms);
}

// ------------------------------------------------------------------ multipoles

// P2M, src/computeOnm4.f90:142-162: O_n^m = sum_sites q rho^n Y(n,-m)
//                                          = sum q rfctr(n,m) conj(T_n^m)
template <typename R>
__global__ void k_p2m(Dev d) {
    griddep_wait();
    const int c = blockIdx.x;
    const int s0 = d.cstart[c], n = d.cstart[c + 1] - s0;
    const Rep r = d.rep[d.crep[c]];
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    const double cx = cell_centre(d, r, 0, ix), cy = cell_centre(d, r, 1, iy), cz = cell_centre(d, r, 2, iz);
    R acc[2 * LPH];
    for (int k = 0; k < 2 * LPH; k++) acc[k] = R(0);
    for (int s = threadIdx.x; s < n; s += blockDim.x) {
        R x, y, z, q;
        if constexpr (sizeof(R) == 4) {   // cell-relative FP32 positions of the mixed path
            const float4 p = d.srt_pos32[s0 + s];
            x = p.x; y = p.y; z = p.z; q = p.w;
        } else {
            const double4 p = d.srt_pos[s0 + s];
            x = p.x - cx; y = p.y - cy; z = p.z - cz; q = p.w;
        }
        R r2 = x * x + y * y + z * z;
        Cx<R> Tmm = {R(1), R(0)};
        Cx<R> xy = {x, y};
        int o = 0;
        for (int m = 0; m <= P; m++) {
            if (m > 0) Tmm = cscale(cmul(xy, Tmm), -(R)(2 * m - 1));
            Cx<R> T2 = Tmm, T1 = Tmm;
            for (int nn = m; nn <= P; nn++) {
                Cx<R> Tn;
                if (nn == m) Tn = Tmm;
                else if (nn == m + 1) Tn = cscale(Tmm, (R)(2 * m + 1) * z);
                else Tn = cscale(csub(cscale(T1, (R)(2 * nn - 1) * z), cscale(T2, (R)(nn + m - 1) * r2)), R(1) / (R)(nn - m));
                if (nn > m) T2 = T1;
                T1 = Tn;
                int ic = nn * (nn + 1) + m;
                R w = q * rfctr_r<R>(ic);
                // ordering index among m >= 0 coefficients: o(n,m) = n(n+1)/2 + m
                int oi = nn * (nn + 1) / 2 + m;
                acc[2 * oi] += w * Tn.re;
                acc[2 * oi + 1] -= w * Tn.im;
                o++;
            }
        }
    }
    __shared__ R red[2 * LPH][64];
    for (int k = 0; k < 2 * LPH; k++) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    if (threadIdx.x < 2 * LPH) {
        R s = R(0);
        for (int t = 0; t < blockDim.x; t++) s += red[threadIdx.x][t];
        red[threadIdx.x][0] = s;
    }
    __syncthreads();
    if (threadIdx.x < LPH) {
        int oi = threadIdx.x;
        int nn = 0;
        while ((nn + 1) * (nn + 2) / 2 <= oi) nn++;
        int m = oi - nn * (nn + 1) / 2;
        double re = (double)red[2 * oi][0], im = (double)red[2 * oi + 1][0];
        double2 *O = d.O4 + (size_t)c * LP;
        O[nn * (nn + 1) + m] = make_double2(re, im);
        if (m > 0) O[nn * (nn + 1) - m] = make_double2(re, -im);
    }
}

// output coefficient (j, k >= 0) of thread o (0..14)
__device__ inline void out_jk(int o, int &j, int &k) {
    j = 0;
    while ((j + 1) * (j + 2) / 2 <= o) j++;
    k = o - j * (j + 1) / 2;
}

__device__ inline void store_jk(double2 *L, int o, double re, double im, bool add) {
    int j, k;
    out_jk(o, j, k);
    double2 v = add ? L[j * (j + 1) + k] : make_double2(0.0, 0.0);
    v.x += re; v.y += im;
    L[j * (j + 1) + k] = v;
    if (k > 0) L[j * (j + 1) - k] = make_double2(v.x, -v.y);
}

// M2M, src/computeOnm3.f90:27-98 and src/computeOnm2.f90:13-62: parent box
// from its 8 children (level 4 -> 3 or 3 -> 2)
template <typename R, typename OP>
__device__ inline void apply_op_r(const OP *op, const double2 *in, R &re, R &im) {
#pragma unroll 5
    for (int c = 0; c < LP; c++) {
        const OP a = op[c];
        const double2 b = in[c];
        const R ax = (R)a.x, ay = (R)a.y, bx = (R)b.x, by = (R)b.y;
        re += ax * bx - ay * by;
        im += ax * by + ay * bx;
    }
}

// one CTA per parent: thread (child, output) applies one child's operator,
// the 8 children are added in a fixed order
template <typename R, typename OP>
__global__ void __launch_bounds__(128) k_m2m(Dev d, const double2 *Oc, double2 *Op, const OP *ops, const int *brep,
                                             int level) {
    griddep_wait();
    __shared__ R sre[8][LPH], sim[8][LPH];
    const int b = blockIdx.x;
    const Rep r = d.rep[brep[b]];
    const int div = level == 3 ? 2 : 4;   // parent grid = nc / div
    const int base_p = level == 3 ? r.l3_0 : r.l2_0;
    const int base_c = level == 3 ? r.cell0 : r.l3_0;
    const int np[3] = {r.nc[0] / div, r.nc[1] / div, r.nc[2] / div};
    const int nc[3] = {np[0] * 2, np[1] * 2, np[2] * 2};
    const int l = b - base_p;
    const int px = l % np[0], py = (l / np[0]) % np[1], pz = l / (np[0] * np[1]);
    const int ch = threadIdx.x / LPH, o = threadIdx.x % LPH;
    if (ch < 8) {
        const int cx = 2 * px + (ch & 1), cy = 2 * py + ((ch >> 1) & 1), cz = 2 * pz + ((ch >> 2) & 1);
        const int ci = base_c + cx + nc[0] * (cy + nc[1] * cz);
        R re = 0, im = 0;
        apply_op_r<R>(ops + ((size_t)ch * LPH + o) * LP, Oc + (size_t)ci * LP, re, im);
        sre[ch][o] = re;
        sim[ch][o] = im;
    }
    __syncthreads();
    if (threadIdx.x < LPH) {
        R re = 0, im = 0;
        for (int k = 0; k < 8; k++) { re += sre[k][threadIdx.x]; im += sim[k][threadIdx.x]; }
        store_jk(Op + (size_t)b * LP, threadIdx.x, (double)re, (double)im, false);
    }
}

// L2L, src/shiftLjk2.f90:16-60 and src/shiftLjk3.f90:27-91: child box
// from its parent (level 2 -> 3 or 3 -> 4), plus the child's M2L partial
// sums of its G offset groups (real form, [box][group][25]), added in
// group order
template <typename R, typename OP>
__global__ void k_l2l(Dev d, const double2 *Lp, double2 *Lc, const OP *ops, const int *brep, int level,
                      const R *part, int G, float2 *Lf, int nbox) {
    griddep_wait();
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);   // one warp per child box
    if (b >= nbox) return;
    const Rep r = d.rep[brep[b]];
    const int div = level == 3 ? 2 : 1;  // child grid = nc / div
    const int base_c = level == 3 ? r.l3_0 : r.cell0;
    const int base_p = level == 3 ? r.l2_0 : r.l3_0;
    const int nc[3] = {r.nc[0] / div, r.nc[1] / div, r.nc[2] / div};
    const int np[3] = {nc[0] / 2, nc[1] / 2, nc[2] / 2};
    int l = b - base_c;
    int cx = l % nc[0], cy = (l / nc[0]) % nc[1], cz = l / (nc[0] * nc[1]);
    int ch = (cx & 1) + 2 * (cy & 1) + 4 * (cz & 1);
    int pi = base_p + cx / 2 + np[0] * (cy / 2 + np[1] * (cz / 2));
    int o = threadIdx.x & 31;
    if (o >= LPH) return;
    R re = 0, im = 0;
    apply_op_r<R>(ops + ((size_t)ch * LPH + o) * LP, Lp + (size_t)pi * LP, re, im);
    int j, k;
    out_jk(o, j, k);
    R pre = 0, pim = 0;
    const R *pb = part + (size_t)b * G * LP;
    for (int g = 0; g < G; g++) {
        pre += pb[g * LP + o];
        if (k > 0) pim += pb[g * LP + LPH + o - (j + 1)];
    }
    const double vre = (double)re + (double)pre, vim = (double)im + (double)pim;
    store_jk(Lc + (size_t)b * LP, o, vre, vim, false);
    if (Lf) {   // FP32 copy of the finished L4 for the mixed path's L2P
        Lf[(size_t)b * LP + j * (j + 1) + k] = make_float2((float)vre, (float)vim);
        if (k > 0) Lf[(size_t)b * LP + j * (j + 1) - k] = make_float2((float)vre, (float)-vim);
    }
}

// M2L with the operator of src/computeLjk4.f90:134-158 factored as
//   op[(j,k),(n,m)] = cf[(j,k),(n,m)] * H_{j+n}^{m-k}(d),  H_l^q = Y_l^q(d) / |d|^(l+1),
// d the source - target vector and H_l^{-q} = conj(H_l^q): per offset 45
// complex H instead of 375 operator entries, so the tables stay in L1/L2
// and the kernels need no operator staging.  cf holds the offset-independent
// iIkm2(k,m) rAnm(j,k) rAnm(n,m) / (sgn(n) rAnm(j+n,m-k)).
constexpr int NH = 45;   // (l, q), l = 0..8, q = 0..l

template <typename R>
struct C2 {
    R x, y;
};
// the 25 terms of output coefficient o: index of H, coefficient for the real
// and the imaginary part of H (the sign of the latter conjugates H for m < k)
template <typename R>
__device__ inline void m2l_terms(int o, const R *cf, int (&h)[LP], R (&cr)[LP], R (&ci)[LP]) {
    int j, k;
    out_jk(o, j, k);
#pragma unroll
    for (int nm = 0; nm < LP; nm++) {
        const int n = nm < 1 ? 0 : nm < 4 ? 1 : nm < 9 ? 2 : nm < 16 ? 3 : 4;
        const int m = nm - n * (n + 1);
        const int l = j + n, q = m - k;
        h[nm] = l * (l + 1) / 2 + (q < 0 ? -q : q);
        const R c = cf[o * LP + nm];
        cr[nm] = c;
        ci[nm] = q < 0 ? -c : c;
    }
}

// one term table entry of an L2 M2L output: H index and coefficient (the
// conjugate's sign folded into ci)
template <typename R>
struct M2LTerm { int h; R cr, ci; };
template <typename R, typename S>
__device__ __forceinline__ void m2l_acc_s(const C2<R> *__restrict__ H, const S *src, const M2LTerm<R> *tm, R &re, R &im) {
#pragma unroll 5
    for (int nm = 0; nm < LP; nm++) {
        const M2LTerm<R> t = tm[nm];
        const C2<R> hv = H[t.h];
        const S mv = src[nm];
        const R mx = (R)mv.x, my = (R)mv.y;
        const R t1 = t.cr * hv.x, t2 = t.ci * hv.y;
        re += t1 * mx - t2 * my;
        im += t1 * my + t2 * mx;
    }
}

// M2L at L4 and L3 (src/computeLjk4.f90, src/computeLjk3.f90) in real form.
// A cell's interaction list (children of its parent's neighbours, less its
// own neighbours) depends only on its parity class (bit a: odd index on axis
// a): 189 offsets with each component in [-2-p, 3-p].  So for one class and
// one offset, every target applies the same 25 x 25 real operator to its
// source's 25 real components: a lane takes two targets of a class, the CTA
// stages the operators of its offset group in shared memory (read as
// broadcasts), and the sources come from the class-packed copy of the
// multipoles, whose zero margin of 2 stands for the cells outside the box.
// Each offset group writes its partial sums; k_l2l adds the groups in a
// fixed order.

// multipoles of L4 and L3 to the class-packed real layout (margins stay zero)
template <typename R>
__global__ void k_m2l_pack(Dev d, int ncell, int n3) {
    griddep_wait();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (ncell + n3) * LP) return;
    const int i = idx % LP, c = idx / LP;
    const bool l4 = c < ncell;
    const int cc = l4 ? c : c - ncell;
    const Rep r = d.rep[l4 ? d.crep[cc] : d.b3rep[cc]];
    const int div = l4 ? 1 : 2;
    const int n0 = r.nc[0] / div, n1 = r.nc[1] / div, n2 = r.nc[2] / div;
    const int l = cc - (l4 ? r.cell0 : r.l3_0);
    const int x = l % n0, y = (l / n0) % n1, z = l / (n0 * n1);
    const int p0 = n0 / 2 + 4, p1 = n1 / 2 + 4, vol = p0 * p1 * (n2 / 2 + 4);
    const int q = (x & 1) + 2 * (y & 1) + 4 * (z & 1);
    int n, m;
    bool im = i >= LPH;
    if (!im) {
        out_jk(i, n, m);
    } else {   // Im X_n^m, m > 0: index 15 + n(n-1)/2 + m - 1
        const int s = i - LPH;
        n = 1;
        while ((n + 1) * n / 2 <= s) n++;
        m = s - n * (n - 1) / 2 + 1;
    }
    const double2 v = (l4 ? d.O4 : d.O3)[(size_t)cc * LP + n * (n + 1) + m];
    R *pk = (R *)(l4 ? d.pk4 : d.pk3) + (l4 ? r.pk4 : r.pk3);
    const R val = (R)(im ? v.y : v.x);
    const int xc = x / 2, yc = y / 2, zc = z / 2;
    R *base = pk + ((size_t)q * LP + i) * vol + (size_t)(zc + 2) * p1 * p0;
    if (!r.per) {
        base[(yc + 2) * p0 + xc + 2] = val;
        return;
    }
    // periodic in x and y: the margins hold the class cells of the opposite
    // side (one box length away; an even cell count keeps the parity class),
    // so the interaction lists wrap around the box
    const int hx = n0 / 2, hy = n1 / 2;
    int xs[3] = {xc, 0, 0}, ys[3] = {yc, 0, 0}, nx = 1, ny = 1;
    if (xc < 2) xs[nx++] = xc + hx;
    if (xc >= hx - 2) xs[nx++] = xc - hx;
    if (yc < 2) ys[ny++] = yc + hy;
    if (yc >= hy - 2) ys[ny++] = yc - hy;
    for (int a = 0; a < ny; a++)
        for (int b = 0; b < nx; b++) base[(ys[a] + 2) * p0 + xs[b] + 2] = val;
}

constexpr int M2C_CH = 4;   // operators staged per chunk

// one input row of a staged operator applied to two targets
__device__ __forceinline__ void m2c_row(const float *op, float va, float vb, float (&aa)[LP], float (&ab)[LP]) {
#pragma unroll
    for (int o4 = 0; o4 < M2C_LD / 4; o4++) {
        const float4 w = *(const float4 *)(op + 4 * o4);
        const float ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (4 * o4 + u < LP) {
                aa[4 * o4 + u] += ws[u] * va;
                ab[4 * o4 + u] += ws[u] * vb;
            }
    }
}
__device__ __forceinline__ void m2c_row(const double *op, double va, double vb, double (&aa)[LP], double (&ab)[LP]) {
#pragma unroll
    for (int o2 = 0; o2 < M2C_LD / 2; o2++) {
        const double2 w = *(const double2 *)(op + 2 * o2);
        if (2 * o2 < LP) { aa[2 * o2] += w.x * va; ab[2 * o2] += w.x * vb; }
        if (2 * o2 + 1 < LP) { aa[2 * o2 + 1] += w.y * va; ab[2 * o2 + 1] += w.y * vb; }
    }
}

// FP32 rows in Blackwell's paired arithmetic: the operator row's outputs
// (o, o + 1) against one target's input, one fma.rn.f32x2 for both outputs
// (each element rounds as a scalar FMA, so the sums are the scalar ones)
constexpr int M2C_P = (LP + 1) / 2;   // output pairs (the last one padded)
__device__ __forceinline__ void m2c_row2(const float *op, float va, float vb, float2 (&aa)[M2C_P], float2 (&ab)[M2C_P]) {
    const float2 a2 = make_float2(va, va), b2 = make_float2(vb, vb);
#pragma unroll
    for (int o4 = 0; o4 < (2 * M2C_P + 3) / 4; o4++) {
        const float4 w = *(const float4 *)(op + 4 * o4);
        const float2 w0 = make_float2(w.x, w.y), w1 = make_float2(w.z, w.w);
        aa[2 * o4] = __ffma2_rn(w0, a2, aa[2 * o4]);
        ab[2 * o4] = __ffma2_rn(w0, b2, ab[2 * o4]);
        if (2 * o4 + 1 < M2C_P) {
            aa[2 * o4 + 1] = __ffma2_rn(w1, a2, aa[2 * o4 + 1]);
            ab[2 * o4 + 1] = __ffma2_rn(w1, b2, ab[2 * o4 + 1]);
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(32 * M2C_W) k_m2l_cls(Dev d) {
    griddep_wait();
    extern __shared__ __align__(16) unsigned char smraw[];
    R *sop = (R *)smraw;   // [M2C_CH][LP][M2C_LD]
    const int4 it = d.m2c_items[blockIdx.x];
    const int level = it.x >> 28, cls = it.y, t0 = it.z, cnt = it.w;
    const Rep r = d.rep[it.x & 0x0FFFFFFF];
    const int G = d.m2c_groups, g = blockIdx.y;
    const int k0 = g * M2C_NOFF / G, k1 = (g + 1) * M2C_NOFF / G;
    const int div = level == 4 ? 2 : 4;   // class grid = nc / div
    const int h0 = r.nc[0] / div, h1 = r.nc[1] / div;
    const int p0 = h0 + 4, p1 = h1 + 4, vol = p0 * p1 * (r.nc[2] / div + 4);
    const int px = cls & 1, py = (cls >> 1) & 1, pz = cls >> 2;
    const R *rop = (const R *)(level == 4 ? d.rop4 : d.rop3);
    const R *pk = (const R *)(level == 4 ? d.pk4 : d.pk3) + (level == 4 ? r.pk4 : r.pk3);
    const int *offs = d.m2c_off + cls * M2C_NOFF;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ta = t0 + w * 64 + lane, tb = ta + 32, last = t0 + cnt - 1;
    // padded class-grid index of a target (loads of lanes past the tile use its last target)
    auto pidx = [&](int t) {
        t = min(t, last);
        const int x = t % h0, y = (t / h0) % h1, z = t / (h0 * h1);
        return ((z + 2) * p1 + (y + 2)) * p0 + x + 2;
    };
    const int ia = pidx(ta), ib = pidx(tb);
    // the class-packed sources of offset k (shifted so that a target's own padded index addresses them)
    auto src_of = [&](int k) {
        const int oi = offs[k];
        const int ex = px + oi % 7 - 3, ey = py + (oi / 7) % 7 - 3, ez = pz + oi / 49 - 3;
        const int q = (ex & 1) + 2 * (ey & 1) + 4 * (ez & 1);
        return pk + (size_t)q * LP * vol + ((ez >> 1) * p1 + (ey >> 1)) * p0 + (ex >> 1);
    };
    R aa[LP], ab[LP];
#pragma unroll
    for (int i = 0; i < LP; i++) aa[i] = ab[i] = R(0);
    float2 pa[M2C_P], pb[M2C_P];   // FP32: the sums in output pairs
#pragma unroll
    for (int i = 0; i < M2C_P; i++) pa[i] = pb[i] = make_float2(0.f, 0.f);
    for (int c0 = k0; c0 < k1; c0 += M2C_CH) {
        const int nch = min(M2C_CH, k1 - c0);
        __syncthreads();
        for (int idx = threadIdx.x; idx < nch * LP * M2C_LD; idx += blockDim.x) {
            const int kk = idx / (LP * M2C_LD);
            sop[idx] = rop[(size_t)offs[c0 + kk] * (LP * M2C_LD) + (idx - kk * (LP * M2C_LD))];
        }
        __syncthreads();
        for (int kk = 0; kk < nch; kk++) {
            const R *src = src_of(c0 + kk);
            const R *op = sop + kk * LP * M2C_LD;
            if constexpr (std::is_same<R, float>::value) {
#pragma unroll
                for (int i = 0; i < LP; i++)
                    m2c_row2(op + i * M2C_LD, src[(size_t)i * vol + ia], src[(size_t)i * vol + ib], pa, pb);
            } else {
#pragma unroll
                for (int i = 0; i < LP; i++) m2c_row(op + i * M2C_LD, src[(size_t)i * vol + ia], src[(size_t)i * vol + ib], aa, ab);
            }
        }
    }
    if constexpr (std::is_same<R, float>::value) {
#pragma unroll
        for (int i = 0; i < LP; i++) {
            aa[i] = (i & 1) ? pa[i >> 1].y : pa[i >> 1].x;
            ab[i] = (i & 1) ? pb[i >> 1].y : pb[i >> 1].x;
        }
    }
    R *part = (R *)(level == 4 ? d.part4 : d.part3);
    const int base = level == 4 ? r.cell0 : r.l3_0, n0 = 2 * h0, n1 = 2 * h1;
    auto cell = [&](int t) {
        const int x = t % h0, y = (t / h0) % h1, z = t / (h0 * h1);
        return base + (2 * x + px) + n0 * ((2 * y + py) + n1 * (2 * z + pz));
    };
    if (ta <= last) {
        const int cg = cell(ta);
#pragma unroll
        for (int i = 0; i < LP; i++) part[((size_t)cg * G + g) * LP + i] = aa[i];
    }
    if (tb <= last) {
        const int cg = cell(tb);
#pragma unroll
        for (int i = 0; i < LP; i++) part[((size_t)cg * G + g) * LP + i] = ab[i];
    }
}

// M2L at L2 over all non-adjacent L2 boxes of the replica (src/computeLjk2.f90:17-72):
// one CTA per target box; each half-warp takes every 16th of the replica's
// boxes as sources (one at a time, the same for its lanes), lane o < 15 the
// output o; the 16 half-warps' sums are added in a fixed order
// Periodic preset: every (source box, image) pair of the 3 x 3 supercell of
// images in x and y that is not adjacent to the target (the reach of the far
// field; nearer images come through the wrapped lists of L3, L4 and the
// near field).  d2: the largest offset per axis of the H table.
template <typename R>
__global__ void __launch_bounds__(256) k_m2l_all(Dev d, const C2<R> *Htab, const C2<R> *Hper, const R *cf, int3 d2) {
    griddep_wait();
    __shared__ R scf[LPH * LP];
    __shared__ R sre[16][LPH], sim[16][LPH];
    const int b = blockIdx.x;
    const Rep r = d.rep[d.b2rep[b]];
    const int *n = r.nr;
    const int l = b - r.l2_0;
    const int t[3] = {l % n[0], (l / n[0]) % n[1], l / (n[0] * n[1])};
    for (int idx = threadIdx.x; idx < LPH * LP; idx += blockDim.x) scf[idx] = cf[idx];
    __syncthreads();
    const int hw = threadIdx.x >> 4, o = threadIdx.x & 15;
    // the term tables of the 15 outputs in shared memory, not registers (128
    // -> 48 registers: more CTAs per SM to hide the H and O loads)
    __shared__ M2LTerm<R> sterm[LPH][LP];
    if (threadIdx.x < LPH) {
        int h[LP];
        R cr[LP], ci[LP];
        m2l_terms<R>(threadIdx.x, scf, h, cr, ci);
        for (int nm = 0; nm < LP; nm++) sterm[threadIdx.x][nm] = {h[nm], cr[nm], ci[nm]};
    }
    __syncthreads();
    const M2LTerm<R> *tm = sterm[o < LPH ? o : LPH - 1];
    const int nb = n[0] * n[1] * n[2];
    // a half-warp's current source, rounded to R once by its 16 lanes and
    // read back as broadcasts (the 15 outputs each converting all 25 FP64
    // components kept GB300's FP64 pipe, which converts, busy 97% of cycles)
    __shared__ C2<R> ssrc[16][LP];
    const unsigned hmask = 0xFFFFu << (16 * (hw & 1));   // the half-warp's lanes (its trip count is its own)
    auto source = [&](int s) -> const C2<R> * {
        const double2 *src = d.O2 + (size_t)(r.l2_0 + s) * LP;
        __syncwarp(hmask);   // the previous source's reads are done
        for (int q = o; q < LP; q += 16) ssrc[hw][q] = {(R)src[q].x, (R)src[q].y};
        __syncwarp(hmask);
        return ssrc[hw];
    };
    R re = 0, im = 0;
    if (r.per) {
        // the image-summed factors of the replica: one pass over the box's sources
        const int wx = 2 * n[0] - 1, wy = 2 * n[1] - 1;
        const C2<R> *Hr = Hper + (size_t)r.h2off * NH;
        for (int s = hw; s < nb; s += 16) {
            const int sx = s % n[0], sy = (s / n[0]) % n[1], sz = s / (n[0] * n[1]);
            const int oi = (sx - t[0] + n[0] - 1) + wx * ((sy - t[1] + n[1] - 1) + wy * (sz - t[2] + n[2] - 1));
            m2l_acc_s<R>(Hr + (size_t)oi * NH, source(s), tm, re, im);
        }
    } else {
        const int wx = 2 * d2.x + 1, wy = 2 * d2.y + 1;
        for (int s = hw; s < nb; s += 16) {
            const int sx = s % n[0], sy = (s / n[0]) % n[1], sz = s / (n[0] * n[1]);
            const int dx = sx - t[0], dy = sy - t[1], dz = sz - t[2];
            if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) continue;
            const int oi = (dx + d2.x) + wx * ((dy + d2.y) + wy * (dz + d2.z));
            m2l_acc_s<R>(Htab + (size_t)oi * NH, source(s), tm, re, im);
        }
    }
    if (o < LPH) { sre[hw][o] = re; sim[hw][o] = im; }
    __syncthreads();
    if (threadIdx.x < LPH) {
        R a = 0, c = 0;
        for (int q = 0; q < 16; q++) { a += sre[q][threadIdx.x]; c += sim[q][threadIdx.x]; }
        store_jk(d.L2 + (size_t)b * LP, threadIdx.x, (double)a, (double)c, false);
    }
}

// opt-in shared-memory sizes, called once per context creation; every
// force kernel now fits the default 48 KB
void init_force_kernels() {}

template <typename R>
size_t m2c_smem() { return sizeof(R) * M2C_CH * LP * M2C_LD; }

template <typename R, typename OP>
void fma_build(const Dev &d, int ncell, int n3, int n2, int3 d2, const OP *m43, const OP *m32, const OP *l23,
               const OP *l34, const C2<R> *h2, const C2<R> *hper, const R *cf, cudaStream_t st) {
    // one chain of dependent launches (programmatic: each waits for its predecessor first)
    launch_pdl(k_p2m<R>, dim3(ncell), dim3(64), 0, st, d);
    launch_pdl(k_m2m<R, OP>, dim3(n3), dim3(128), 0, st, d, d.O4, d.O3, m43, d.b3rep, 3);
    launch_pdl(k_m2m<R, OP>, dim3(n2), dim3(128), 0, st, d, d.O3, d.O2, m32, d.b2rep, 2);
    launch_pdl(k_m2l_pack<R>, dim3(((ncell + n3) * LP + 255) / 256), dim3(256), 0, st, d, ncell, n3);
    launch_pdl(k_m2l_cls<R>, dim3(d.m2c_nitems, d.m2c_groups), dim3(32 * M2C_W), m2c_smem<R>(), st, d);
    launch_pdl(k_m2l_all<R>, dim3(n2), dim3(256), 0, st, d, h2, hper, cf, d2);
    launch_pdl(k_l2l<R, OP>, dim3((n3 + 3) / 4), dim3(128), 0, st, d, (const double2 *)d.L2, d.L3, l23,
               (const int *)d.b3rep, 3, (const R *)d.part3, d.m2c_groups, (float2 *)nullptr, n3);
    launch_pdl(k_l2l<R, OP>, dim3((ncell + 3) / 4), dim3(128), 0, st, d, (const double2 *)d.L3, d.L4, l34,
               (const int *)d.crep, 4, (const R *)d.part4, d.m2c_groups, sizeof(R) == 4 ? d.L4f : (float2 *)nullptr,
               ncell);
}

void launch_fma_build(const Dev &d, int ncell, int n3, int n2, int mixed, int3 d2, cudaStream_t st) {
    if (mixed)
        fma_build<float>(d, ncell, n3, n2, d2, d.op32_m2m43, d.op32_m2m32, d.op32_l2l23, d.op32_l2l34,
                         (const C2<float> *)d.h32_m2l2, (const C2<float> *)d.h32_per, d.m2l_cf32, st);
    else
        fma_build<double>(d, ncell, n3, n2, d2, d.op_m2m43, d.op_m2m32, d.op_l2l23, d.op_l2l34,
                          (const C2<double> *)d.h_m2l2, (const C2<double> *)d.h_per, d.m2l_cf, st);
}

// ------------------------------------------------------------------ per-site terms

__device__ inline double pow13(double v) { double v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4 * v; }
__device__ inline double pow12(double v) { double v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4; }

// graphite LJ of one site over its column's carbons (src/eval_graphite.f90:104-126)
__device__ inline void graphite_site(const Dev &d, int col, double x, double y, double z, double eps, double sg6,
                                     double &fx, double &fy, double &fz, double *e) {
    const double rc2 = RC * RC;
    for (int k = d.gcol_start[col]; k < d.gcol_start[col + 1]; k++) {
        double4 c = d.gpos[k];
        double xij = x - c.x, yij = y - c.y, zij = z - c.z;
        double r2 = xij * xij + yij * yij + zij * zij;
        if (r2 <= rc2) {
            double rsi = 1.0 / r2, r6 = rsi * rsi * rsi;
            double flj = 48.0 * eps * sg6 * r6 * (sg6 * r6 - 0.5) * rsi;
            fx += xij * flj; fy += yij * flj; fz += zij * flj;
            if (e) *e += 4.0 * eps * (sg6 * sg6 * r6 * r6 - sg6 * r6);
        }
    }
}

// graphite acts on LJ sites that sit in their molecule's key cell in the
// bottom layer of cells: water O (w1 and split) and surfactant sites in
// SCentral (src/eval_graphite.f90:13-132)
// Configuration preset: every LJ site whose cell lies in the bottom cell
// layers up to r.igz (those within rc plus the 2 A list skin of the top
// carbon plane), in the column of its cell.
__device__ inline int graphite_column(const Dev &d, const Rep &r, int g, double &eps, double &sg6) {
    if (!r.graphite_on) return -1;
    int pt = d.ptype[g];
    int loc = d.sloc[g];
    const double2 lj = d.tgr[pt];   // (eps, sg^6) with carbon; zero for water H
    if (lj.x == 0.0 || loc < 0) return -1;
    if (!r.per && loc != d.mkey[d.smol[g]]) return -1;
    int ix, iy, iz;
    cell_xyz(r, loc, ix, iy, iz);
    if (iz > (r.per ? r.igz : 0)) return -1;
    eps = lj.x;
    sg6 = lj.y;
    return r.gcol0 + ix + r.nc[0] * iy;
}

// a site's position wrapped by the image of the last rebuild (periodic preset)
__device__ inline void site_pos(const Dev &d, const Rep &r, int g, double &x, double &y, double &z) {
    x = d.x[g]; y = d.y[g]; z = d.z[g];
    if (r.per) {
        const short2 im = d.simg[g];
        x -= (double)im.x * r.rsd[0];
        y -= (double)im.y * r.rsd[1];
    }
}

// walls, src/eval_wall.f90:17-23: 48 / (v - h)^13 + 48 / (h + v)^13 per
// axis.  The mixed path forms the distances in FP64 (they cancel near a
// wall) and the rest in FP32 (at most 91 sigma across: no overflow).
__device__ inline float pow13f(float v) { float v2 = v * v, v4 = v2 * v2, v8 = v4 * v4; return v8 * v4 * v; }

// what one site's force assembly reads
struct SiteIn {
    int per;
    double rhs0, rhs1, rhs2;
    double nx, ny, nz;   // the pair-field force of its slot (0 without one)
    double x, y, z;
    double sx, sy, sz;   // the side forces
};

__device__ __forceinline__ void site_load(const Dev &d, int g, int terms, SiteIn &in) {
    const Rep &r = d.rep[d.mrep[d.smol[g]]];
    in.per = r.per;
    in.rhs2 = r.rhs[2];
    in.nx = in.ny = in.nz = 0.0;
    const int slot = d.sslot[g];
    if ((terms & (SESP_T_NEAR | SESP_T_FAR)) && slot >= 0) {
        in.nx = d.nf[3 * (size_t)slot]; in.ny = d.nf[3 * (size_t)slot + 1]; in.nz = d.nf[3 * (size_t)slot + 2];
    }
    in.z = d.z[g];
    // x and y enter only the side walls of a closed box (fewer registers
    // held for the periodic preset)
    in.x = in.y = in.rhs0 = in.rhs1 = 0.0;
    if ((terms & SESP_T_WALL) && !in.per) { in.x = d.x[g]; in.y = d.y[g]; in.rhs0 = r.rhs[0]; in.rhs1 = r.rhs[1]; }
    const size_t n = d.nsite;
    in.sx = d.fside[g]; in.sy = d.fside[n + g]; in.sz = d.fside[2 * n + g];
}

template <bool MIXED>
__device__ __forceinline__ void site_store(const Dev &d, int g, int terms, const SiteIn &in) {
    double fx = in.nx, fy = in.ny, fz = in.nz;
    const double x = in.x, y = in.y, z = in.z;
    if (terms & SESP_T_WALL) {   // the periodic preset has walls at the z faces only
        if constexpr (MIXED) {
            if (!in.per) {
                fx += (double)(48.f / pow13f((float)(x - in.rhs0)) + 48.f / pow13f((float)(in.rhs0 + x)));
                fy += (double)(48.f / pow13f((float)(y - in.rhs1)) + 48.f / pow13f((float)(in.rhs1 + y)));
            }
            fz += (double)(48.f / pow13f((float)(z - in.rhs2)) + 48.f / pow13f((float)(in.rhs2 + z)));
        } else {
            if (!in.per) {
                fx += 48.0 / pow13(x - in.rhs0); fx += 48.0 / pow13(in.rhs0 + x);
                fy += 48.0 / pow13(y - in.rhs1); fy += 48.0 / pow13(in.rhs1 + y);
            }
            fz += 48.0 / pow13(z - in.rhs2); fz += 48.0 / pow13(in.rhs2 + z);
        }
    }
    // the step's graphite and intramolecular forces, cleared for the next step
    const size_t n = d.nsite;
    fx += in.sx; fy += in.sy; fz += in.sz;
    d.fside[g] = 0.0; d.fside[n + g] = 0.0; d.fside[2 * n + g] = 0.0;
    d.fx[g] = fx; d.fy[g] = fy; d.fz[g] = fz;
}

// Total site forces: the slot's pair-field force, walls, side forces.  A
// thread takes SITE_PER sites (blockDim.x apart) and issues every load of
// all of them before it sums and stores any.  The kernel is a chain of
// dependent loads (site -> molecule -> replica, site -> slot -> force).  With
// one site per thread, 312,000 sites took 1.34 waves of CTAs, and the second
// wave waited out the whole chain again.  Two sites per thread (64 registers)
// run the two chains side by side, in 1.003 waves.
constexpr int SITE_PER = 2;
template <bool MIXED>
__global__ void k_site_forces(Dev d, int nsite, int terms) {
    griddep_wait();
    const int g0 = blockIdx.x * SITE_PER * blockDim.x + threadIdx.x;
    SiteIn in[SITE_PER];
#pragma unroll
    for (int k = 0; k < SITE_PER; k++)
        if (g0 + k * (int)blockDim.x < nsite) site_load(d, g0 + k * blockDim.x, terms, in[k]);
#pragma unroll
    for (int k = 0; k < SITE_PER; k++)
        if (g0 + k * (int)blockDim.x < nsite) site_store<MIXED>(d, g0 + k * blockDim.x, terms, in[k]);
}

// sites the graphite acts on, listed at every rebuild (their cells are frozen
// until the next one); list order does not enter any sum
__global__ void k_graphite_list(Dev d, int nsite) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nsite) return;
    const Rep r = d.rep[d.mrep[d.smol[g]]];
    double eps, sg6;
    if (graphite_column(d, r, g, eps, sg6) >= 0) d.gsite[atomicAdd(d.gcount, 1)] = g;
}

// graphite LJ (src/eval_graphite.f90:104-126), one warp per listed site.
// Lanes 0..GGRP-1 each take one carbon group (a graphite layer) of the
// site's column: a group farther than rc in z is skipped, and of the others
// only the y bins within sqrt(rc^2 - dz^2) of the site are visited (bounds
// widened by 1e-3, far above the FP32 rounding of the window arithmetic; the
// exact r^2 <= rc^2 test still decides every pair).  The lanes then stride
// the visited carbons of all groups and a fixed shuffle tree sums them.
// FP32 (mixed path): site and carbons relative to the column centre, so each
// carbon costs FP32 arithmetic only.
// A warp takes a run of up to 32 consecutive listed sites (the list split
// evenly over the warps): lane j does the FP64 set-up of the run's site j
// (column, position, parameters) and, at the end, its FP64 force update, so
// those run once per run instead of once per site on every lane (GB300
// issues FP64 and its conversions at 1/64 of the FP32 rate, whatever the
// active lanes); in between the warp walks the run's sites with their set-up
// broadcast.
template <typename R>
__global__ void k_graphite(Dev d) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int n = *d.gcount;
    const R rc2 = (R)(RC * RC);
    const float reach = (float)RC + 1e-3f;
    const int run = min(32, (n + nwarp - 1) / nwarp);
    for (int k0 = warp * run; k0 < n; k0 += nwarp * run) {
        // lane set-up of site k0 + lane
        const bool mine = lane < run && k0 + lane < n;
        int my_g = 0, my_col = 0;
        float my_gymax = 1.f, my_xs = 0.f, my_ys = 0.f, my_zs = 0.f;
        R my_e48 = 0, my_s6 = 0;
        double my_xd = 0.0, my_yd = 0.0, my_zd = 0.0;
        if (mine) {
            my_g = d.gsite[k0 + lane];
            const Rep r = d.rep[d.mrep[d.smol[my_g]]];
            my_gymax = r.gymax;
            double eps, sg6;
            my_col = graphite_column(d, r, my_g, eps, sg6);
            site_pos(d, r, my_g, my_xd, my_yd, my_zd);
            const int lc = my_col - r.gcol0, ix = lc % r.nc[0], iy = lc / r.nc[0];
            my_xs = (float)(my_xd - cell_centre(d, r, 0, ix));
            my_ys = (float)(my_yd - cell_centre(d, r, 1, iy));
            my_zs = (float)(my_zd - cell_centre(d, r, 2, 0));
            my_e48 = (R)(48.0 * eps * sg6);
            my_s6 = (R)sg6;
        }
        const int cnt = min(run, n - k0);
        R my_fx = 0, my_fy = 0, my_fz = 0;
        for (int j = 0; j < cnt; j++) {
            const int col = __shfl_sync(0xffffffffu, my_col, j);
            const float gymax = __shfl_sync(0xffffffffu, my_gymax, j), bin_scale = GBIN / (2.f * gymax);
            const float xs = __shfl_sync(0xffffffffu, my_xs, j), ys = __shfl_sync(0xffffffffu, my_ys, j),
                        zs = __shfl_sync(0xffffffffu, my_zs, j);
            const R e48 = __shfl_sync(0xffffffffu, my_e48, j), s6 = __shfl_sync(0xffffffffu, my_s6, j);
            double xd = 0.0, yd = 0.0, zd = 0.0;
            if constexpr (!std::is_same<R, float>::value) {
                xd = __shfl_sync(0xffffffffu, my_xd, j);
                yd = __shfl_sync(0xffffffffu, my_yd, j);
                zd = __shfl_sync(0xffffffffu, my_zd, j);
            }
            int s0 = 0, len = 0;
            if (lane < GGRP) {
                const size_t gi = (size_t)col * GGRP + lane;
                const float2 zr = d.ggrp_z[gi];
                const float dz = fmaxf(fmaxf(zr.x - zs, zs - zr.y), 0.f);
                if (zr.x <= zr.y && dz < reach) {
                    const float w = sqrtf(fmaxf(reach * reach - dz * dz, 0.f)) + 1e-3f;
                    const int b0 = min(max((int)floorf((ys - w + gymax) * bin_scale), 0), GBIN);
                    const int b1 = min(max((int)floorf((ys + w + gymax) * bin_scale) + 1, 0), GBIN);
                    const int *bins = d.gbin + gi * (GBIN + 1);
                    s0 = bins[b0];
                    len = bins[b1] - s0;
                }
            }
            int incl = len;   // inclusive prefix over the group lanes
            for (int o = 1; o < GGRP; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            int st[GGRP], pe[GGRP];
#pragma unroll
            for (int q = 0; q < GGRP; q++) {
                st[q] = __shfl_sync(0xffffffffu, s0, q);
                pe[q] = __shfl_sync(0xffffffffu, incl, q);
            }
            const int total = pe[GGRP - 1];
            R fx = 0, fy = 0, fz = 0;
            for (int t = lane; t < total; t += 32) {
                int q = st[0] + t;
#pragma unroll
                for (int u = 1; u < GGRP; u++)
                    if (t >= pe[u - 1]) q = st[u] + t - pe[u - 1];
                if constexpr (std::is_same<R, float>::value) {
                    const float4 c = d.gpos32[q];
                    const float xij = xs - c.x, yij = ys - c.y, zij = zs - c.z;
                    const float r2 = xij * xij + yij * yij + zij * zij;
                    if (r2 <= rc2) {
                        const float rsi = __fdividef(1.f, r2), r6 = rsi * rsi * rsi;
                        const float flj = e48 * r6 * (s6 * r6 - 0.5f) * rsi;
                        fx += xij * flj; fy += yij * flj; fz += zij * flj;
                    }
                } else {
                    const double4 c = d.gpos[q];
                    R xij = (R)(xd - c.x), yij = (R)(yd - c.y), zij = (R)(zd - c.z);
                    R r2 = xij * xij + yij * yij + zij * zij;
                    if (r2 <= rc2) {
                        R rsi = R(1) / r2, r6 = rsi * rsi * rsi;
                        R flj = e48 * r6 * (s6 * r6 - R(0.5)) * rsi;
                        fx += xij * flj; fy += yij * flj; fz += zij * flj;
                    }
                }
            }
            for (int off = 16; off > 0; off >>= 1) {
                fx += __shfl_down_sync(0xffffffffu, fx, off);
                fy += __shfl_down_sync(0xffffffffu, fy, off);
                fz += __shfl_down_sync(0xffffffffu, fz, off);
            }
            // lane 0 holds the sums; lane j keeps them for its update
            fx = __shfl_sync(0xffffffffu, fx, 0);
            fy = __shfl_sync(0xffffffffu, fy, 0);
            fz = __shfl_sync(0xffffffffu, fz, 0);
            if (lane == j) { my_fx = fx; my_fy = fy; my_fz = fz; }
        }
        if (mine) {
            const size_t ns = d.nsite;
            d.fside[my_g] += (double)my_fx; d.fside[ns + my_g] += (double)my_fy; d.fside[2 * ns + my_g] += (double)my_fz;
        }
    }
}

void launch_graphite_list(const Dev &d, int nsite, cudaStream_t st) {
    cudaMemsetAsync(d.gcount, 0, sizeof(int), st);
    k_graphite_list<<<(nsite + 255) / 256, 256, 0, st>>>(d, nsite);
}

void launch_site_forces(const Dev &d, int nsite, int terms, int mixed, cudaStream_t st) {
    const dim3 g((nsite + SITE_PER * 256 - 1) / (SITE_PER * 256)), b(256);
    if (mixed) launch_pdl(k_site_forces<true>, g, b, 0, st, d, nsite, terms);
    else launch_pdl(k_site_forces<false>, g, b, 0, st, d, nsite, terms);
}

void launch_graphite(const Dev &d, int terms, int mixed, cudaStream_t st) {
    if (terms & SESP_T_GRAPHITE) {
        if (mixed) k_graphite<float><<<152 * 4, 256, 0, st>>>(d);
        else k_graphite<double><<<152 * 4, 256, 0, st>>>(d);
    }
}

// ------------------------------------------------------------------ surfactant intramolecular

// positions of one surfactant (shared memory in the force kernel); the FP32
// form holds them relative to the molecule's first site
template <typename R, int N>
struct PosN {
    R x[N], y[N], z[N];
};
template <typename R = double>
using Pos29 = PosN<R, NSURF>;

// one harmonic angle (src/eval_valence.f90:104-145) at vertex b with
// equilibrium th0 and constant kth: forces on a, b, c
template <typename R, int N>
__device__ R angle_core(const PosN<R, N> &m, int a, int b, int c, double th0, double kth, R f[3][3]) {
    R rxji = m.x[a] - m.x[b], ryji = m.y[a] - m.y[b], rzji = m.z[a] - m.z[b];
    R rxki = m.x[c] - m.x[b], ryki = m.y[c] - m.y[b], rzki = m.z[c] - m.z[b];
    R dp = rxji * rxki + ryji * ryki + rzji * rzki;
    R rjin = sqrt(rxji * rxji + ryji * ryji + rzji * rzji);
    R rkin = sqrt(rxki * rxki + ryki * ryki + rzki * rzki);
    R th = acos(dp / rjin / rkin);
    R costh = cos(th);
    R dth = th - (R)th0;
    R r1 = (R)kth * dth / sin(th);
    R fjx = rxki / rjin / rkin - costh * rxji / (rjin * rjin);
    R fjy = ryki / rjin / rkin - costh * ryji / (rjin * rjin);
    R fjz = rzki / rjin / rkin - costh * rzji / (rjin * rjin);
    R fkx = rxji / rjin / rkin - costh * rxki / (rkin * rkin);
    R fky = ryji / rjin / rkin - costh * ryki / (rkin * rkin);
    R fkz = rzji / rjin / rkin - costh * rzki / (rkin * rkin);
    f[0][0] = r1 * fjx; f[0][1] = r1 * fjy; f[0][2] = r1 * fjz;
    f[1][0] = -r1 * (fjx + fkx); f[1][1] = -r1 * (fjy + fky); f[1][2] = -r1 * (fjz + fkz);
    f[2][0] = r1 * fkx; f[2][1] = r1 * fky; f[2][2] = r1 * fkz;
    return R(0.5) * (R)kth * dth * dth;
}
template <typename R>
__device__ R angle_term(const Pos29<R> &m, int i, R f[3][3]) {
    return angle_core<R, NSURF>(m, cT.ai[i], cT.aj[i], cT.ak[i], cT.th[i], cT.rkth[i], f);
}

// one dihedral: r1 = -dU/dcos(phi) applied with the cross-product algebra of
// src/eval_dihedral.f90:116-271 (triple cosine, dihedrals 1-18) or
// src/eval_dihedral_berendsen.f90 (cos 3 phi, dihedrals 19-30)
// FP32: with c = cos(phi) the ratios are the exact identities
// sin(2 phi) / sin(phi) = 2c and sin(3 phi) / sin(phi) = 4c^2 - 1, which need
// neither acos nor a division by sin(phi) (the FP64 form follows the reference).
template <typename R, int N>
__device__ R dihedral_core(const PosN<R, N> &m, int iv, int jv, int kv, int lv, bool berendsen, R dva, R dvb, R dvc,
                          R f[4][3]) {
    R ax = m.x[jv] - m.x[iv], ay = m.y[jv] - m.y[iv], az = m.z[jv] - m.z[iv];   // r_ji
    R bx = m.x[kv] - m.x[jv], by = m.y[kv] - m.y[jv], bz = m.z[kv] - m.z[jv];   // r_kj
    R cx = m.x[lv] - m.x[kv], cy = m.y[lv] - m.y[kv], cz = m.z[lv] - m.z[kv];   // r_nk
    R u1 = ax * by - ay * bx, u2 = ax * bz - az * bx, u3 = ay * bz - az * by;
    R v1 = bx * cy - by * cx, v2 = bx * cz - bz * cx, v3 = by * cz - bz * cy;
    R nu = sqrt(u1 * u1 + u2 * u2 + u3 * u3), nv = sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    R arg = (u1 * v1 + u2 * v2 + u3 * v3) / nu / nv;
    R r1, e, costh;
    if constexpr (std::is_same<R, double>::value) {
        const double clampv = berendsen ? 0.999999 : 0.99999999999;
        if (arg <= -1.0) arg = -clampv;
        if (arg >= 1.0) arg = clampv;
        double th = acos(arg), sinth = sin(th);
        costh = cos(th);
        if (berendsen) {
            r1 = -3.0 * dva * sin(3.0 * th) / sinth;
            e = dva * (1.0 + cos(3.0 * th));
        } else {
            r1 = -dva + 2.0 * dvb * sin(2.0 * th) / sinth - 3.0 * dvc * sin(3.0 * th) / sinth;
            e = dva * (1.0 + cos(th)) + dvb * (1.0 - cos(2.0 * th)) + dvc * (1.0 + cos(3.0 * th));
        }
    } else {
        const R clampv = berendsen ? R(0.999999) : R(1);
        if (arg <= R(-1)) arg = -clampv;
        if (arg >= R(1)) arg = clampv;
        const R c = arg, c2 = c * c;
        costh = c;
        const R s3 = R(4) * c2 - R(1), c3 = (R(4) * c2 - R(3)) * c;
        if (berendsen) {
            r1 = R(-3) * dva * s3;
            e = dva * (R(1) + c3);
        } else {
            r1 = -dva + R(4) * dvb * c - R(3) * dvc * s3;
            e = dva * (R(1) + c) + dvb * (R(2) - R(2) * c2) + dvc * (R(1) + c3);
        }
    }
    R nuv = nu * nv, nu2 = nu * nu, nv2 = nv * nv;
    R fix = (bx * (-by * cy - bz * cz) + cx * (by * by + bz * bz)) / nuv;
    R fiy = (by * (-bx * cx - bz * cz) + cy * (bx * bx + bz * bz)) / nuv;
    R fiz = (bz * (-bx * cx - by * cy) + cz * (bx * bx + by * by)) / nuv;
    R gix = (R(2) * ax * (-by * by - bz * bz) + R(2) * bx * (ay * by + az * bz)) / nu2;
    R giy = (R(2) * ay * (-bx * bx - bz * bz) + R(2) * by * (ax * bx + az * bz)) / nu2;
    R giz = (R(2) * az * (-bx * bx - by * by) + R(2) * bz * (ax * bx + ay * by)) / nu2;
    R fjx = (ax * (-by * cy - bz * cz) + bx * (by * cy + bz * cz) + cx * (-ay * by - az * bz - by * by - bz * bz) +
                  R(2) * bx * (ay * cy + az * cz)) / nuv;
    R fjy = (ay * (-bx * cx - bz * cz) + by * (bx * cx + bz * cz) + cy * (-ax * bx - az * bz - bx * bx - bz * bz) +
                  R(2) * by * (ax * cx + az * cz)) / nuv;
    R fjz = (az * (-bx * cx - by * cy) + bz * (bx * cx + by * cy) + cz * (-ax * bx - ay * by - bx * bx - by * by) +
                  R(2) * bz * (ax * cx + ay * cy)) / nuv;
    R gjx = (R(2) * ax * (by * by + bz * bz + ay * by + az * bz) + R(2) * bx * (-ay * ay - az * az - ay * by - az * bz)) / nu2 +
                 (R(2) * cx * (by * cy + bz * cz) + R(2) * bx * (-cy * cy - cz * cz)) / nv2;
    R gjy = (R(2) * ay * (bx * bx + bz * bz + ax * bx + az * bz) + R(2) * by * (-ax * ax - az * az - ax * bx - az * bz)) / nu2 +
                 (R(2) * cy * (bx * cx + bz * cz) + R(2) * by * (-cx * cx - cz * cz)) / nv2;
    R gjz = (R(2) * az * (bx * bx + by * by + ax * bx + ay * by) + R(2) * bz * (-ax * ax - ay * ay - ax * bx - ay * by)) / nu2 +
                 (R(2) * cz * (bx * cx + by * cy) + R(2) * bz * (-cx * cx - cy * cy)) / nv2;
    R fkx = (ax * (by * by + bz * bz + by * cy + bz * cz) + bx * (-ay * by - az * bz) + cx * (ay * by + az * bz) +
                  R(2) * bx * (-ay * cy - az * cz)) / nuv;
    R fky = (ay * (bx * bx + bz * bz + bx * cx + bz * cz) + by * (-ax * bx - az * bz) + cy * (ax * bx + az * bz) +
                  R(2) * by * (-ax * cx - az * cz)) / nuv;
    R fkz = (az * (bx * bx + by * by + bx * cx + by * cy) + bz * (-ax * bx - ay * by) + cz * (ax * bx + ay * by) +
                  R(2) * bz * (-ax * cx - ay * cy)) / nuv;
    R gkx = (R(2) * ax * (-ay * by - az * bz) + R(2) * bx * (ay * ay + az * az)) / nu2 +
                 (R(2) * cx * (-by * by - bz * bz - by * cy - bz * cz) + R(2) * bx * (cy * cy + cz * cz + by * cy + bz * cz)) / nv2;
    R gky = (R(2) * ay * (-ax * bx - az * bz) + R(2) * by * (ax * ax + az * az)) / nu2 +
                 (R(2) * cy * (-bx * bx - bz * bz - bx * cx - bz * cz) + R(2) * by * (cx * cx + cz * cz + bx * cx + bz * cz)) / nv2;
    R gkz = (R(2) * az * (-ax * bx - ay * by) + R(2) * bz * (ax * ax + ay * ay)) / nu2 +
                 (R(2) * cz * (-bx * bx - by * by - bx * cx - by * cy) + R(2) * bz * (cx * cx + cy * cy + bx * cx + by * cy)) / nv2;
    R fnx = (ax * (-by * by - bz * bz) + bx * (ay * by + az * bz)) / nuv;
    R fny = (ay * (-bx * bx - bz * bz) + by * (ax * bx + az * bz)) / nuv;
    R fnz = (az * (-bx * bx - by * by) + bz * (ax * bx + ay * by)) / nuv;
    R gnx = (R(2) * cx * (by * by + bz * bz) + R(2) * bx * (-by * cy - bz * cz)) / nv2;
    R gny = (R(2) * cy * (bx * bx + bz * bz) + R(2) * by * (-bx * cx - bz * cz)) / nv2;
    R gnz = (R(2) * cz * (bx * bx + by * by) + R(2) * bz * (-bx * cx - by * cy)) / nv2;
    R h = R(0.5) * costh;
    f[0][0] = r1 * (fix - h * gix); f[0][1] = r1 * (fiy - h * giy); f[0][2] = r1 * (fiz - h * giz);
    f[1][0] = r1 * (fjx - h * gjx); f[1][1] = r1 * (fjy - h * gjy); f[1][2] = r1 * (fjz - h * gjz);
    f[2][0] = r1 * (fkx - h * gkx); f[2][1] = r1 * (fky - h * gky); f[2][2] = r1 * (fkz - h * gkz);
    f[3][0] = r1 * (fnx - h * gnx); f[3][1] = r1 * (fny - h * gny); f[3][2] = r1 * (fnz - h * gnz);
    return e;
}
template <typename R>
__device__ R dihedral_term(const Pos29<R> &m, int i, R f[4][3]) {
    return dihedral_core<R, NSURF>(m, cT.di[i], cT.dj[i], cT.dk[i], cT.dl[i], i >= 18, (R)cT.dva[i], (R)cT.dvb[i],
                                   (R)cT.dvc[i], f);
}

// one intramolecular nonbonded pair, Coulomb + LJ without cutoff
// (src/eval_surfactant_internal.f90:33-66, 70-108)
template <typename R>
__device__ inline R ipair_term(const Dev &d, const Pos29<R> &m, int a, int b, R f[2][3]) {
    R x = m.x[a] - m.x[b], y = m.y[a] - m.y[b], z = m.z[a] - m.z[b];
    R rsq = x * x + y * y + z * z;
    R rsi = R(1) / rsq, ir = sqrt(rsi), r6 = rsi * rsi * rsi;
    R qq = (R)(cT.q[2 + a] * cT.q[2 + b] * XPI);
    const double2 lj = d.ljt[(2 + a) * NTYPE + 2 + b];   // (48 eps sg6, sg6)
    const R e48 = (R)lj.x, s6 = (R)lj.y;
    R ft = qq * ir * rsi + e48 * r6 * (s6 * r6 - R(0.5)) * rsi;
    f[0][0] = x * ft; f[0][1] = y * ft; f[0][2] = z * ft;
    f[1][0] = -x * ft; f[1][1] = -y * ft; f[1][2] = -z * ft;
    return qq * ir + (e48 / R(12)) * (s6 * r6 * r6 - r6);
}

// the far-field correction of one site (src/eval_subtract_fma.f90:14-53):
// minus the Coulomb force of its own molecule's sites outside its 27-cell block
template <typename R>
__device__ inline R subtract_site(const Pos29<R> &m, int j, uint32_t bits, R f[3]) {
    R e = 0;
    f[0] = f[1] = f[2] = 0;
    while (bits) {
        int k = __ffs(bits) - 1;
        bits &= bits - 1;
        R x = m.x[j] - m.x[k], y = m.y[j] - m.y[k], z = m.z[j] - m.z[k];
        R rmn = sqrt(x * x + y * y + z * z);
        R qq = (R)(cT.q[2 + j] * cT.q[2 + k] * XPI);
        R fel = qq / (rmn * rmn * rmn);
        f[0] -= x * fel; f[1] -= y * fel; f[2] -= z * fel;
        e -= R(0.5) * qq / rmn;
    }
    return e;
}

// One block per surfactant: the 36 angles, 30 dihedrals and 312
// intramolecular pairs take one thread each (INTRA_THREADS >= their count,
// so a block is one term deep), each writing its site forces to its own
// slots in shared memory; then thread s sums the slots of site s in the
// fixed order of the contribution table (deterministic, no atomics) and adds
// its far-field correction.
constexpr int NIPAIR = 270 + NSELF;                 // k >= j+4 pairs of sites 1..15, then the 42 listed
constexpr int NSLOT = NANGLE * 3 + NDIH * 4 + NIPAIR * 2;
constexpr int NTERM = NANGLE + NDIH + NIPAIR;
constexpr int INTRA_THREADS = 384;
static_assert(INTRA_THREADS >= NTERM, "one term per thread");

struct IntraMap {
    short off[NSURF + 1];  // slots of site s: list[off[s] .. off[s+1])
    short list[NSLOT];
    unsigned char pa[NIPAIR], pb[NIPAIR];
};
static __constant__ IntraMap cMap;

void upload_intra_map(const void *host_map, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(cMap, host_map, sizeof(IntraMap), 0, cudaMemcpyHostToDevice, st);
}
size_t intra_map_size() { return sizeof(IntraMap); }

template <typename R>
__global__ void __launch_bounds__(INTRA_THREADS) k_intra_block(Dev d, const int *smols, int terms) {
    __shared__ Pos29<R> m;
    __shared__ R sf[NSLOT][3];
    const int t = blockIdx.x;
    const int g0 = d.mfirst[smols[t]];
    if (threadIdx.x < NSURF) {
        if constexpr (std::is_same<R, double>::value) {
            m.x[threadIdx.x] = d.x[g0 + threadIdx.x];
            m.y[threadIdx.x] = d.y[g0 + threadIdx.x];
            m.z[threadIdx.x] = d.z[g0 + threadIdx.x];
        } else {
            m.x[threadIdx.x] = (R)(d.x[g0 + threadIdx.x] - d.x[g0]);
            m.y[threadIdx.x] = (R)(d.y[g0 + threadIdx.x] - d.y[g0]);
            m.z[threadIdx.x] = (R)(d.z[g0 + threadIdx.x] - d.z[g0]);
        }
    }
    __syncthreads();
    for (int w = threadIdx.x; w < NTERM; w += blockDim.x) {
        if (w < NANGLE) {
            R f[3][3] = {{0}};
            if (terms & SESP_T_VALENCE) angle_term<R>(m, w, f);
            for (int k = 0; k < 3; k++) for (int c = 0; c < 3; c++) sf[w * 3 + k][c] = f[k][c];
        } else if (w < NANGLE + NDIH) {
            int i = w - NANGLE;
            R f[4][3] = {{0}};
            if ((i < 18 && (terms & SESP_T_DIHEDRAL)) || (i >= 18 && (terms & SESP_T_BERENDSEN))) dihedral_term<R>(m, i, f);
            for (int k = 0; k < 4; k++) for (int c = 0; c < 3; c++) sf[NANGLE * 3 + i * 4 + k][c] = f[k][c];
        } else {
            int q = w - NANGLE - NDIH;
            R f[2][3] = {{0}};
            if (terms & SESP_T_INTERNAL) ipair_term<R>(d, m, cMap.pa[q], cMap.pb[q], f);
            int s0 = NANGLE * 3 + NDIH * 4 + 2 * q;
            for (int k = 0; k < 2; k++) for (int c = 0; c < 3; c++) sf[s0 + k][c] = f[k][c];
        }
    }
    __syncthreads();
    if (threadIdx.x < NSURF) {
        int s = threadIdx.x;
        R fx = 0, fy = 0, fz = 0;
        for (int k = cMap.off[s]; k < cMap.off[s + 1]; k++) {
            int sl = cMap.list[k];
            fx += sf[sl][0]; fy += sf[sl][1]; fz += sf[sl][2];
        }
        if (terms & SESP_T_SUBTRACT) {
            R f[3];
            subtract_site<R>(m, s, d.isub[(size_t)t * NSURF + s], f);
            fx += f[0]; fy += f[1]; fz += f[2];
        }
        const size_t n = d.nsite;
        d.fside[g0 + s] += (double)fx; d.fside[n + g0 + s] += (double)fy; d.fside[2 * n + g0 + s] += (double)fz;
    }
}


// ------------------------------------------------------------------ chains (configuration preset)

static __constant__ ChainTables cCh;

void upload_chain_tables(const ChainTables &t, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(cCh, &t, sizeof(ChainTables), 0, cudaMemcpyHostToDevice, st);
}

// term slots of one chain: bond b -> 2b + {b, b+1}; angle a -> CH_A0 + 3a +
// {a, vertex a+1, a+2}; dihedral q -> CH_D0 + 4q + {q .. q+3}; pair p ->
// CH_P0 + 2p + {a, b} (pairs four or more bonds apart, a ascending, then b)
constexpr int CH_A0 = 2 * NCH_BOND, CH_D0 = CH_A0 + 3 * NCH_ANGLE, CH_P0 = CH_D0 + 4 * NCH_DIH;
constexpr int CH_SLOTS = CH_P0 + 2 * NCH_PAIR;
constexpr int CH_TERMS = NCH_BOND + NCH_ANGLE + NCH_DIH + NCH_PAIR;
constexpr int CH_THREADS = 96;
static_assert(CH_THREADS >= CH_TERMS, "one term per thread");

// the p-th pair four or more bonds apart
__device__ __forceinline__ void chain_pair(int p, int &a, int &b) {
    a = 0;
    while (p >= NCH - 4 - a) { p -= NCH - 4 - a; a++; }
    b = a + 4 + p;
}

template <typename R>
__device__ inline R chain_bond(const PosN<R, NCH> &m, int i, R f[2][3]) {
    const R x = m.x[i] - m.x[i + 1], y = m.y[i] - m.y[i + 1], z = m.z[i] - m.z[i + 1];
    const R r = sqrt(x * x + y * y + z * z), dr = r - (R)cCh.r0, fm = -(R)cCh.kb * dr / r;
    f[0][0] = fm * x; f[0][1] = fm * y; f[0][2] = fm * z;
    f[1][0] = -fm * x; f[1][1] = -fm * y; f[1][2] = -fm * z;
    return R(0.5) * (R)cCh.kb * dr * dr;
}

// LJ + Coulomb without cutoff between beads a and b of one chain
template <typename R>
__device__ inline R chain_ipair(const Dev &d, const PosN<R, NCH> &m, int a, int b, R f[2][3]) {
    const R x = m.x[a] - m.x[b], y = m.y[a] - m.y[b], z = m.z[a] - m.z[b];
    const R rsq = x * x + y * y + z * z;
    const R rsi = R(1) / rsq, ir = sqrt(rsi), r6 = rsi * rsi * rsi;
    const R qq = (R)(d.tq[2 + a] * d.tq[2 + b] * XPI);
    const double2 lj = d.ljt[(2 + a) * NTYPE + 2 + b];   // (48 eps sg6, sg6)
    const R e48 = (R)lj.x, s6 = (R)lj.y;
    const R ft = qq * ir * rsi + e48 * r6 * (s6 * r6 - R(0.5)) * rsi;
    f[0][0] = x * ft; f[0][1] = y * ft; f[0][2] = z * ft;
    f[1][0] = -x * ft; f[1][1] = -y * ft; f[1][2] = -z * ft;
    return qq * ir + (e48 / R(12)) * (s6 * r6 * r6 - r6);
}

// far-field correction of one bead: minus the Coulomb of its own chain's
// beads in cells not adjacent to its own
template <typename R>
__device__ inline R chain_subtract(const Dev &d, const PosN<R, NCH> &m, int j, uint32_t bits, R f[3]) {
    R e = 0;
    f[0] = f[1] = f[2] = 0;
    while (bits) {
        const int k = __ffs(bits) - 1;
        bits &= bits - 1;
        const R x = m.x[j] - m.x[k], y = m.y[j] - m.y[k], z = m.z[j] - m.z[k];
        const R rmn = sqrt(x * x + y * y + z * z);
        const R qq = (R)(d.tq[2 + j] * d.tq[2 + k] * XPI);
        const R fel = qq / (rmn * rmn * rmn);
        f[0] -= x * fel; f[1] -= y * fel; f[2] -= z * fel;
        e -= R(0.5) * qq / rmn;
    }
    return e;
}

// One block per chain: the 11 bonds, 10 angles, 9 dihedrals and 36 pairs
// take one thread each and write their site forces to their own slots in
// shared memory; thread s then sums site s's slots in slot order (no
// atomics: deterministic) and adds its far-field correction.  FP32: positions
// relative to the chain's first bead.
template <typename R>
__global__ void __launch_bounds__(CH_THREADS) k_chain_block(Dev d, const int *smols, int terms) {
    __shared__ PosN<R, NCH> m;
    __shared__ R sf[CH_SLOTS][3];
    const int t = blockIdx.x;
    const int g0 = d.mfirst[smols[t]];
    if (threadIdx.x < NCH) {
        if constexpr (std::is_same<R, double>::value) {
            m.x[threadIdx.x] = d.x[g0 + threadIdx.x];
            m.y[threadIdx.x] = d.y[g0 + threadIdx.x];
            m.z[threadIdx.x] = d.z[g0 + threadIdx.x];
        } else {
            m.x[threadIdx.x] = (R)(d.x[g0 + threadIdx.x] - d.x[g0]);
            m.y[threadIdx.x] = (R)(d.y[g0 + threadIdx.x] - d.y[g0]);
            m.z[threadIdx.x] = (R)(d.z[g0 + threadIdx.x] - d.z[g0]);
        }
    }
    __syncthreads();
    const int w = threadIdx.x;
    if (w < NCH_BOND) {
        R f[2][3] = {{0}};
        if (terms & SESP_T_BOND) chain_bond<R>(m, w, f);
        for (int k = 0; k < 2; k++) for (int c = 0; c < 3; c++) sf[2 * w + k][c] = f[k][c];
    } else if (w < NCH_BOND + NCH_ANGLE) {
        const int a = w - NCH_BOND;
        R f[3][3] = {{0}};
        if (terms & SESP_T_VALENCE) angle_core<R, NCH>(m, a, a + 1, a + 2, cCh.th0, cCh.kth, f);
        for (int k = 0; k < 3; k++) for (int c = 0; c < 3; c++) sf[CH_A0 + 3 * a + k][c] = f[k][c];
    } else if (w < NCH_BOND + NCH_ANGLE + NCH_DIH) {
        const int q = w - NCH_BOND - NCH_ANGLE;
        R f[4][3] = {{0}};
        if (terms & SESP_T_DIHEDRAL)
            dihedral_core<R, NCH>(m, q, q + 1, q + 2, q + 3, false, (R)cCh.dva, (R)cCh.dvb, (R)cCh.dvc, f);
        for (int k = 0; k < 4; k++) for (int c = 0; c < 3; c++) sf[CH_D0 + 4 * q + k][c] = f[k][c];
    } else if (w < CH_TERMS) {
        const int p = w - NCH_BOND - NCH_ANGLE - NCH_DIH;
        int a, b;
        chain_pair(p, a, b);
        R f[2][3] = {{0}};
        if (terms & SESP_T_INTERNAL) chain_ipair<R>(d, m, a, b, f);
        for (int k = 0; k < 2; k++) for (int c = 0; c < 3; c++) sf[CH_P0 + 2 * p + k][c] = f[k][c];
    }
    __syncthreads();
    if (threadIdx.x < NCH) {
        const int s = threadIdx.x;
        R fx = 0, fy = 0, fz = 0;
        auto add = [&](int sl) { fx += sf[sl][0]; fy += sf[sl][1]; fz += sf[sl][2]; };
        if (s >= 1) add(2 * (s - 1) + 1);
        if (s < NCH_BOND) add(2 * s);
        if (s < NCH_ANGLE) add(CH_A0 + 3 * s);
        if (s >= 1 && s - 1 < NCH_ANGLE) add(CH_A0 + 3 * (s - 1) + 1);
        if (s >= 2) add(CH_A0 + 3 * (s - 2) + 2);
        for (int k = 0; k < 4; k++)
            if (s - k >= 0 && s - k < NCH_DIH) add(CH_D0 + 4 * (s - k) + k);
        for (int p = 0; p < NCH_PAIR; p++) {
            int a, b;
            chain_pair(p, a, b);
            if (a == s) add(CH_P0 + 2 * p);
            else if (b == s) add(CH_P0 + 2 * p + 1);
        }
        if (terms & SESP_T_SUBTRACT) {
            R f[3];
            chain_subtract<R>(d, m, s, d.isub[(size_t)t * NCH + s], f);
            fx += f[0]; fy += f[1]; fz += f[2];
        }
        const size_t n = d.nsite;
        d.fside[g0 + s] += (double)fx; d.fside[n + g0 + s] += (double)fy; d.fside[2 * n + g0 + s] += (double)fz;
    }
}

// energies of one chain's terms (diagnostic path): bonded, pairs, far-field correction
__global__ void k_chain_energy(Dev d, const int *smols, int ns, double *e_mol) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    const int g0 = d.mfirst[smols[t]];
    PosN<double, NCH> m;
    for (int i = 0; i < NCH; i++) { m.x[i] = d.x[g0 + i]; m.y[i] = d.y[g0 + i]; m.z[i] = d.z[g0 + i]; }
    double eb = 0.0, ei = 0.0, es = 0.0, f2[2][3], f3[3][3], f4[4][3], f1[3];
    for (int b = 0; b < NCH_BOND; b++) eb += chain_bond<double>(m, b, f2);
    for (int a = 0; a < NCH_ANGLE; a++) eb += angle_core<double, NCH>(m, a, a + 1, a + 2, cCh.th0, cCh.kth, f3);
    for (int q = 0; q < NCH_DIH; q++) eb += dihedral_core<double, NCH>(m, q, q + 1, q + 2, q + 3, false, cCh.dva, cCh.dvb, cCh.dvc, f4);
    for (int p = 0; p < NCH_PAIR; p++) {
        int a, b;
        chain_pair(p, a, b);
        ei += chain_ipair<double>(d, m, a, b, f2);
    }
    for (int j = 0; j < NCH; j++) es += chain_subtract<double>(d, m, j, d.isub[(size_t)t * NCH + j], f1);
    e_mol[3 * t] = eb; e_mol[3 * t + 1] = ei; e_mol[3 * t + 2] = es;
}

void launch_intra(const Dev &d, const int *smols, int ns, int terms, int mixed, int chains, cudaStream_t st) {
    const int bits = SESP_T_VALENCE | SESP_T_DIHEDRAL | SESP_T_BERENDSEN | SESP_T_INTERNAL | SESP_T_SUBTRACT | SESP_T_BOND;
    if (ns && chains && (terms & bits)) {
        if (mixed) k_chain_block<float><<<ns, CH_THREADS, 0, st>>>(d, smols, terms);
        else k_chain_block<double><<<ns, CH_THREADS, 0, st>>>(d, smols, terms);
        return;
    }
    if (ns && (terms & bits)) {
        if (mixed) k_intra_block<float><<<ns, INTRA_THREADS, 0, st>>>(d, smols, terms);
        else k_intra_block<double><<<ns, INTRA_THREADS, 0, st>>>(d, smols, terms);
    }
}

// energies of one surfactant's intramolecular terms (diagnostic path)
__global__ void k_intra_energy(Dev d, const int *smols, int ns, double *e_mol) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    int g0 = d.mfirst[smols[t]];
    Pos29<double> m;
    for (int i = 0; i < NSURF; i++) { m.x[i] = d.x[g0 + i]; m.y[i] = d.y[g0 + i]; m.z[i] = d.z[g0 + i]; }
    double eb = 0.0, ei = 0.0, es = 0.0;
    double f4[4][3], f3[3][3], f2[2][3], f1[3];
    for (int i = 0; i < NANGLE; i++) eb += angle_term<double>(m, i, f3);
    for (int i = 0; i < NDIH; i++) eb += dihedral_term<double>(m, i, f4);
    for (int q = 0; q < NIPAIR; q++) ei += ipair_term<double>(d, m, cMap.pa[q], cMap.pb[q], f2);
    for (int j = 0; j < NSURF; j++) es += subtract_site<double>(m, j, d.isub[(size_t)t * NSURF + j], f1);
    e_mol[3 * t] = eb; e_mol[3 * t + 1] = ei; e_mol[3 * t + 2] = es;
}

// ------------------------------------------------------------------ energies (diagnostic path)

// near-field pair energy (1/2 per ordered pair) and far-field potential
// energy per slot, FP64
__global__ void k_energy_slot(Dev d, double *e_slot) {
    const int c = blockIdx.x;
    const int s0 = d.cstart[c], ni = d.cstart[c + 1] - s0;
    const Rep r = d.rep[d.crep[c]];
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    const double cx = cell_centre(d, r, 0, ix), cy = cell_centre(d, r, 1, iy), cz = cell_centre(d, r, 2, iz);
    __shared__ double Lre[LP], Lim[LP];
    if (threadIdx.x < LP) { double2 v = d.L4[(size_t)c * LP + threadIdx.x]; Lre[threadIdx.x] = v.x; Lim[threadIdx.x] = v.y; }
    __syncthreads();
    const double rc2 = RC * RC;
    for (int i = threadIdx.x; i < ni; i += blockDim.x) {
        double4 pi = d.srt_pos[s0 + i];
        int2 mi = d.srt_meta[s0 + i];
        double ec = 0.0, el = 0.0;
        for (int dzc = -1; dzc <= 1; dzc++)
            for (int dyc = -1; dyc <= 1; dyc++)
                for (int dxc = -1; dxc <= 1; dxc++) {
                    int jx = ix + dxc, jy = iy + dyc, jz = iz + dzc;
                    if (jz < 0 || jz >= r.nc[2]) continue;
                    if (!r.per && (jx < 0 || jy < 0 || jx >= r.nc[0] || jy >= r.nc[1])) continue;
                    const int cn = shell_cell(r, jx, jy, jz);
                    const double sx = r.per ? (double)(jx - wrap1(jx, r.nc[0])) * RS : 0.0;
                    const double sy = r.per ? (double)(jy - wrap1(jy, r.nc[1])) * RS : 0.0;
                    for (int s = d.cstart[cn]; s < d.cstart[cn + 1]; s++) {
                        int2 mj = d.srt_meta[s];
                        if (mj.x == mi.x) continue;
                        double4 pj = d.srt_pos[s];
                        double dx = pi.x - (pj.x + sx), dy = pi.y - (pj.y + sy), dz = pi.z - pj.z;
                        double r2 = dx * dx + dy * dy + dz * dz;
                        double ir = rsqrt(r2);
                        ec += 0.5 * pi.w * pj.w * XPI * ir;
                        double2 lj = d.ljt[mi.y * NTYPE + mj.y];
                        if (r2 <= rc2 && lj.x != 0.0) {
                            double r6 = ir * ir * ir * ir * ir * ir;
                            el += 0.5 * (lj.x / 12.0) * (lj.y * r6 * r6 - r6);
                        }
                    }
                }
        double gx, gy, gz, phi;
        auto L = [&](int k, double &re, double &im) { re = Lre[k]; im = Lim[k]; };
        local_grad<double>(L, pi.x - cx, pi.y - cy, pi.z - cz, gx, gy, gz, &phi);
        e_slot[3 * (size_t)(s0 + i)] = ec;
        e_slot[3 * (size_t)(s0 + i) + 1] = el;
        e_slot[3 * (size_t)(s0 + i) + 2] = 0.5 * pi.w * XPI * phi;
    }
}

// walls, graphite and kinetic energy per site
__global__ void k_energy_site(Dev d, int nsite, double *e_site) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nsite) return;
    const Rep r = d.rep[d.mrep[d.smol[g]]];
    double x = d.x[g], y = d.y[g], z = d.z[g];
    double ew = 4.0 / pow12(z - r.rhs[2]) + 4.0 / pow12(r.rhs[2] + z);
    if (!r.per)
        ew = 4.0 / pow12(x - r.rhs[0]) + 4.0 / pow12(r.rhs[0] + x) + 4.0 / pow12(y - r.rhs[1]) +
             4.0 / pow12(r.rhs[1] + y) + 4.0 / pow12(z - r.rhs[2]) + 4.0 / pow12(r.rhs[2] + z);
    double eg = 0.0, fx = 0, fy = 0, fz = 0, eps, sg6;
    int col = graphite_column(d, r, g, eps, sg6);
    if (col >= 0) {
        double xw, yw, zw;
        site_pos(d, r, g, xw, yw, zw);
        graphite_site(d, col, xw, yw, zw, eps, sg6, fx, fy, fz, &eg);
    }
    double m = d.tmass[d.ptype[g]];
    double ek = 0.5 * m * (d.vx[g] * d.vx[g] + d.vy[g] * d.vy[g] + d.vz[g] * d.vz[g]) / (DT * DT);
    e_site[3 * (size_t)g] = ew; e_site[3 * (size_t)g + 1] = eg; e_site[3 * (size_t)g + 2] = ek;
}

// ordered near-field pairs and LJ-active pairs within rc (for the
// algorithmic flop count of the pair kernel)
__global__ void k_count_pairs(Dev d, unsigned long long *out) {
    const int c = blockIdx.x;
    const int s0 = d.cstart[c], ni = d.cstart[c + 1] - s0;
    const Rep r = d.rep[d.crep[c]];
    int ix, iy, iz;
    cell_xyz(r, c, ix, iy, iz);
    const double rc2 = RC * RC;
    unsigned long long nc = 0, nl = 0;
    for (int i = threadIdx.x; i < ni; i += blockDim.x) {
        double4 pi = d.srt_pos[s0 + i];
        int2 mi = d.srt_meta[s0 + i];
        for (int dzc = -1; dzc <= 1; dzc++)
            for (int dyc = -1; dyc <= 1; dyc++)
                for (int dxc = -1; dxc <= 1; dxc++) {
                    int jx = ix + dxc, jy = iy + dyc, jz = iz + dzc;
                    if (jz < 0 || jz >= r.nc[2]) continue;
                    if (!r.per && (jx < 0 || jy < 0 || jx >= r.nc[0] || jy >= r.nc[1])) continue;
                    const int cn = shell_cell(r, jx, jy, jz);
                    const double sx = r.per ? (double)(jx - wrap1(jx, r.nc[0])) * RS : 0.0;
                    const double sy = r.per ? (double)(jy - wrap1(jy, r.nc[1])) * RS : 0.0;
                    for (int s = d.cstart[cn]; s < d.cstart[cn + 1]; s++) {
                        int2 mj = d.srt_meta[s];
                        if (mj.x == mi.x) continue;
                        nc++;
                        double4 pj = d.srt_pos[s];
                        double dx = pi.x - (pj.x + sx), dy = pi.y - (pj.y + sy), dz = pi.z - pj.z;
                        if (dx * dx + dy * dy + dz * dz <= rc2 && d.ljt[mi.y * NTYPE + mj.y].x != 0.0) nl++;
                    }
                }
    }
    atomicAdd(&out[0], nc);
    atomicAdd(&out[1], nl);
}

void launch_count_pairs(const Dev &d, int ncell, unsigned long long *out, cudaStream_t st) {
    k_count_pairs<<<ncell, 128, 0, st>>>(d, out);
}

// sum m v^2 of each replica (src/compute_temperature.f90:240-242): one block
// per replica, thread-strided partial sums and a fixed tree, so the result
// does not depend on timing
constexpr int TEMP_THREADS = 256;
// sum of m v^2 per replica in a fixed order: TEMP_SLICES blocks per replica
// each sum one fixed slice of its sites (a tree in shared memory), then one
// block per replica adds the slices as a tree; the slices depend only on the
// replica's site count
__global__ void __launch_bounds__(TEMP_THREADS) k_temperature(Dev d, int nrep) {
    __shared__ double sh[TEMP_THREADS];
    const int q = blockIdx.x / TEMP_SLICES, b = blockIdx.x % TEMP_SLICES;
    const Rep r = d.rep[q];
    const int per = (r.nsite + TEMP_SLICES - 1) / TEMP_SLICES;
    const int g0 = r.site0 + b * per, g1 = min(r.site0 + r.nsite, g0 + per);
    double a = 0.0;
    for (int g = g0 + threadIdx.x; g < g1; g += TEMP_THREADS)
        a += d.tmass[d.ptype[g]] * (d.vx[g] * d.vx[g] + d.vy[g] * d.vy[g] + d.vz[g] * d.vz[g]);
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int w = TEMP_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) d.tbuf[nrep + blockIdx.x] = sh[0];
}
__global__ void __launch_bounds__(TEMP_SLICES) k_temperature_sum(Dev d, int nrep) {
    __shared__ double sh[TEMP_SLICES];
    sh[threadIdx.x] = d.tbuf[nrep + blockIdx.x * TEMP_SLICES + threadIdx.x];
    __syncthreads();
    for (int w = TEMP_SLICES / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) d.tbuf[blockIdx.x] = sh[0];
}

void launch_temperature(const Dev &d, int nrep, cudaStream_t st) {
    k_temperature<<<nrep * TEMP_SLICES, TEMP_THREADS, 0, st>>>(d, nrep);
    k_temperature_sum<<<nrep, TEMP_SLICES, 0, st>>>(d, nrep);
}

// FP32 FMA throughput: every thread runs 8 independent chains of `iters`
// fused multiply-adds (enough to cover the pipe's latency), and writes one
// value so nothing is optimised away.  2 flops per FMA.
__global__ void __launch_bounds__(256) k_fma_peak(float *out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (float)(threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// best of 5 launches of k_fma_peak over (SMs x 8) CTAs of 256 threads, in TFLOP/s
double measure_fp32_peak(int n_sm, cudaStream_t st) {
    float *out = nullptr;
    if (cudaMalloc(&out, (size_t)n_sm * 8 * 256 * sizeof(float)) != cudaSuccess) return 0.0;
    const int iters = 8192;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r < 6; r++) {
        cudaEventRecord(e0, st);
        k_fma_peak<<<n_sm * 8, 256, 0, st>>>(out, iters, 0.999f, 0.001f);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;   // the first launch warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * iters * (double)n_sm * 8 * 256;
    return best < 1e29f ? flops / (best * 1e-3) / 1e12 : 0.0;
}

// writes a buffer larger than the L2 cache so the next launch starts cold
__global__ void k_flush(float4 *buf, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i < n; i += (size_t)gridDim.x * blockDim.x) buf[i] = make_float4(0.f, 0.f, 0.f, (float)i);
}

void launch_flush(void *buf, size_t bytes, cudaStream_t st) {
    k_flush<<<152 * 8, 256, 0, st>>>((float4 *)buf, bytes / sizeof(float4));
}

void launch_energies(const Dev &d, int ncell, int nsite, const int *smols, int ns, int chains, double *e_slot,
                     double *e_site, double *e_mol, cudaStream_t st) {
    k_energy_slot<<<ncell, 128, 0, st>>>(d, e_slot);
    k_energy_site<<<(nsite + 255) / 256, 256, 0, st>>>(d, nsite, e_site);
    if (ns && chains) k_chain_energy<<<(ns + 63) / 64, 64, 0, st>>>(d, smols, ns, e_mol);
    else if (ns) k_intra_energy<<<(ns + 63) / 64, 64, 0, st>>>(d, smols, ns, e_mol);
}

}  // namespace sesp
