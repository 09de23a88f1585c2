// Internal definitions of the GB300 engine (sm_103a).
//
// Device layout (one context may hold several replica systems back to back):
//  * sites in the reference's order per replica (waters O,H,H, then 29-site
//    surfactants); FP64 structure-of-arrays positions, velocities,
//    accelerations and forces;
//  * L4 cells of rs = 12 A, flat over replicas; every rebuild sorts the sites
//    by the cell they sit in (the reference's "Central" test) into contiguous
//    slots, which the pair kernel reads cell by cell;
//  * multipole and local expansions (25 complex coefficients, order 4) per
//    L4, L3 and L2 box.
// Two force fields share the layout (Rep::per tells them apart): the
// reference's (29-site surfactants, closed box) and the configuration
// preset (12-bead chains, periodic in x and y; every site keeps the integer
// image of its last rebuild, and the slot arrays hold positions wrapped by it).
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>
#include <cuda_runtime.h>

#include "../../include/sesp.h"

namespace sesp {

// Programmatic dependent launch: a kernel launched by launch_pdl may be
// scheduled while its stream predecessor finishes, and calls griddep_wait()
// first, which returns once that predecessor has completed and its writes
// are visible (and at once after an ordinary launch).
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
template <typename... K, typename... A>
inline cudaError_t launch_pdl(void (*k)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

constexpr int P = 4;
constexpr int LP = 25;        // (P+1)^2 coefficients
constexpr int LPH = 15;       // coefficients with m >= 0
constexpr int NTYPE = 31;     // 0 water O, 1 water H, 2..30 surfactant sites 1..29
constexpr int NSURF = 29;
constexpr int NBOND = 28;
constexpr int NANGLE = 36;
constexpr int NDIH = 30;
constexpr int NSELF = 42;
constexpr int NHARM = 45;    // M2L factors H_l^q, l = 0..2P, q = 0..l
constexpr int NM2L = 316;     // 7^3 - 3^3 source offsets at L4 and L3
// configuration preset: 12-bead chains (types 2..13), 11 bonds, 10 angles,
// 9 dihedrals, 36 pairs four or more bonds apart
constexpr int NCH = 12;
constexpr int NCH_BOND = NCH - 1, NCH_ANGLE = NCH - 2, NCH_DIH = NCH - 3;
constexpr int NCH_PAIR = (NCH - 4) * (NCH - 3) / 2;

// reduced-unit constants of src/mybox.cmns:36-44 (xpi is a single-precision
// literal in the reference, hence the float)
constexpr double SIGMA = 3.166;
constexpr double EPSILON = 650.2;
constexpr double RC = 10.0 / 3.166;
constexpr double RS = 10.0 / 3.166 + 2.0 / 3.166;
constexpr double XPI = (double)675.05f;
constexpr double DT = 0.00127362;
constexpr double DTSQ2 = 0.00127362 * 0.00127362 / 2.0;

constexpr int M2C_NOFF = 189; // M2L offsets of a cell (6^3 - 3^3 for its parity class)
constexpr int M2C_LD = 28;    // padded output stride of a real M2L operator row
constexpr int M2C_W = 2;      // warps of an M2L CTA, 64 targets each (2 per lane)
constexpr int M2C_TILE = 64 * M2C_W;
constexpr int M2C_GROUPS = 21; // offset groups of an M2L work item, 9 offsets each (partial sums added in group order)
constexpr int GGRP = 8;       // carbon groups per graphite column
constexpr int GBIN = 32;      // y bins per group
// y extent of a column's carbons about its centre: rc + half the L4 cell diagonal
constexpr float GYMAX = (float)(RC + 1.4142135623730951 * RS / 2.0) + 1e-3f;

struct Rep {
    int nc[3];        // L4 cells per axis
    int nr[3];        // L2 boxes (4^3 L4 cells each) per axis
    int cell0;        // first L4 cell
    int l3_0, l2_0;   // first L3 / L2 box
    int site0, nsite; // sites
    int mol0, nmol;   // molecules
    int nw, ns;       // waters, surfactants
    int axis0;        // offset of this replica's cell-centre tables (x, then y, then z)
    int gcol0;        // first bottom-layer column of the carbon lists
    int graphite_on;
    int pk4, pk3;     // first element of this replica's class-packed L4 / L3 multipoles
    double rhs[3], rsd[3];
    double pnh1, pnh2;
    double irsd[3];   // 1 / rsd
    int per;          // periodic in x and y (configuration preset)
    int ssite;        // sites per surfactant (29, or 12 for the chains)
    int igz;          // configuration preset: last cell layer the graphite acts on (-1: none)
    int ncon;         // constraints (degrees of freedom removed)
    float gymax;      // half-extent in y of a graphite column's carbons (bins)
    int h2off;        // periodic preset: first record of this replica's image-summed L2 M2L factors
};

// constant topology and force-field tables (reference values, src/init_arrays.f90)
struct Tables {
    double q[NTYPE];          // charges
    double mass[NTYPE];       // masses / m_O
    int bi[NBOND], bj[NBOND]; // surfactant constraints (0-based sites)
    double dsqs[NBOND];
    double dsqw[3];
    int ai[NANGLE], aj[NANGLE], ak[NANGLE];
    double th[NANGLE], rkth[NANGLE];
    int di[NDIH], dj[NDIH], dk[NDIH], dl[NDIH];
    double dva[NDIH], dvb[NDIH], dvc[NDIH];
    int si[NSELF], sj[NSELF];
    double sgcs6[NSURF], epcs[NSURF];   // carbon - surfactant site LJ
    double sgcw6, epcw;                 // carbon - water O LJ
    double rfctr[LP];                   // sqrt((n-|m|)!/(n+|m|)!) by coefficient
    float rfctr32[LP];                  // the same rounded to FP32 (the FP32 multipole kernels)
};

// bonded terms of the configuration preset's chains (one table for every
// chain; beads are types 2 + b)
struct ChainTables {
    double kb, r0;          // bonds: U = kb / 2 (r - r0)^2
    double kth, th0;        // angles: U = kth / 2 (th - th0)^2
    double dva, dvb, dvc;   // dihedrals: a (1 + cos) + b (1 - cos 2) + c (1 + cos 3)
};

struct Dev {
    // sites
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *fx, *fy, *fz;
    uint8_t *ptype;
    int *smol;
    // molecules
    int *mrep, *mfirst, *mkind, *mkey, *mw1;
    double *ke;          // [2 * nmol]: sum m v^2 before / after SHAKE
    int *mfail;
    // constraint halves of the mixed paths: water work order per half, sweeps
    // of each water's last call per half, queue counters ([0..2] SHAKE,
    // [4..6] RATTLE) and the bins of the reordering
    int *wlist_a, *wlist_b;
    uint8_t *wsw_a, *wsw_b;
    unsigned *cctl;
    int *wsort_off;
    // replicas
    Rep *rep;
    double *eta;         // [nrep]
    double *eta_part;    // [nrep][32][2] partial kinetic sums of the eta update
    unsigned *eta_ctl;   // [nrep] blocks of the eta update finished
    double *axis;        // cell centre tables
    double *rcen2;       // rank centres per replica (at axis0 / 4) and axis (src/init_box_dimensions.f90:40-42)
    // cells
    int *crep, *b3rep, *b2rep;
    int *cstart, *ccount, *cfill;
    int *sloc, *sslot;
    int *cnh;            // per cell: slots with LJ (every kind but water H), which the sort puts first
    int *srt_site;
    double4 *srt_pos;    // x, y, z, q in slot order (FP64)
    float4 *srt_pos32;   // x, y, z relative to the slot's own cell centre, q (mixed)
    int2 *srt_meta;      // molecule, type
    int *srt_key;        // molecule << 5 | type
    int *srt_xmask;      // per slot: bit dx + 3 dy + 9 dz (each offset + 1) set when the cell at that
                         // offset from the slot's own holds a site of the slot's molecule (itself
                         // included), so the pair loop tests same-molecule partners there only
    double *nf;          // near + far force by slot [3 * nslot]
    double *near_part;   // per partner row partial near force [9][3 * nslot] (float on the mixed path)
    int2 *near_items;    // near-field work items (cell, row << 24 | chunk), most expensive first
    int2 *near_items_tmp;   // the same in cell order
    int *near_cls;       // cost class of each item in cell order
    int *near_icount;    // per cell: item count, then first item
    int *near_ctl;       // [0] item counter of the running launch, [1] item count,
                         // [2..33] items per cost class, [34..65] next slot per class
    // graphite columns of the bottom layer
    int *gcol_start;
    double4 *gpos;
    float4 *gpos32;      // the same carbons relative to the column centre (x, y) and the bottom layer's centre (z)
    int *gbin;           // per column GGRP groups of its carbons (z levels, each in FP32 y order):
                         // GBIN + 1 starts of uniform y bins over [-GYMAX, GYMAX], the last one the group's end
    float2 *ggrp_z;      // z range of each group in the gpos32 frame (lo > hi: empty)
    int *gsite, *gcount;   // sites the graphite acts on (rebuilt with the lists)
    // intramolecular correction lists (bit k: site k+1 of the molecule)
    uint32_t *isub;
    // multipoles / local expansions (double2 = complex)
    double2 *O4, *L4, *O3, *L3, *O2, *L2;
    float2 *L4f;         // FP32 copy of L4 (mixed path)
    double *fside;       // graphite + intramolecular forces of the step, [3][nsite]; the site forces add and clear them
    double *stage;       // transfers: positions, velocities, accelerations, forces as (3, nsite) site-major arrays
    double2 *op_m2m43, *op_m2m32, *op_l2l23, *op_l2l34;
    float2 *op32_m2m43, *op32_m2m32, *op32_l2l23, *op32_l2l34;   // FP32 copies for the mixed path
    // L2 M2L factors: H_l^q of every offset (45 per offset, (2 d2 + 1)^3
    // offsets) and the offset-independent coefficients (15 x 25)
    double2 *h_m2l2;
    float2 *h32_m2l2;    // FP32 copy for the mixed path
    // periodic preset: per replica, for every L2 offset (dx, dy, dz) within
    // the box, the sum of H over the offset's non-adjacent periodic images
    // (image shifts -1, 0, 1 in x and y), 45 per offset
    double2 *h_per;
    float2 *h32_per;
    double *m2l_cf;
    float *m2l_cf32;
    // L4 and L3 M2L in real form.  A multipole or local expansion is carried
    // as 25 reals: Re X_n^m for m >= 0 (index n(n+1)/2 + m), then Im X_n^m for
    // m > 0 (index 15 + n(n-1)/2 + m - 1); X_n^-m = conj(X_n^m) supplies the
    // rest.  Per offset (dx + 3) + 7 (dy + 3) + 49 (dz + 3) a real operator
    // [input 25][output, padded to M2C_LD] (FP64 or FP32 by precision).
    void *rop4, *rop3;
    // multipoles of each replica repacked per parity class of its cells:
    // [class 8][component 25][class grid with a zero margin of 2 per side]
    void *pk4, *pk3;
    // partial sums per offset group: [cell of the level][group][component 25]
    void *part4, *part3;
    int4 *m2c_items;     // work items: (level << 28 | replica, class, first target, targets)
    int *m2c_off;        // per class its 189 offsets, (dx + 3) + 7 (dy + 3) + 49 (dz + 3)
    int m2c_nitems, m2c_groups;
    // LJ pair table (eps, sg6), NTYPE^2
    double2 *ljt;
    float2 *ljt32;       // FP32 copy of ljt
    // per site kind (NTYPE): charge, mass, graphite LJ (48 eps sg6, sg6; zero
    // without); the force field's values, so kernels shared by both presets
    // read them here
    double *tq, *tmass;
    double2 *tgr;
    short2 *simg;        // per site: x / y image of the last rebuild (periodic preset)
    double *tbuf;        // [nrep] temperature sums, then [nrep][TEMP_SLICES] slice sums
    // counters: [0] fails, [1] overflow, [2] unlocated, [3] max cell, [5] pairs, [6] LJ pairs
    unsigned long long *counters;
    int max_cell;
    int nsite;           // sites of all replicas (the stride of fside)
};


// ---------------------------------------------------------------- helpers
__host__ __device__ inline int cell_index(const Rep &r, int ix, int iy, int iz) {
    return r.cell0 + ix + r.nc[0] * (iy + r.nc[1] * iz);
}

}  // namespace sesp
