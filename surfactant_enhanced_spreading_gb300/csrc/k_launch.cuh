// Host-side launchers of the engine's kernels (one declaration per kernel
// family); the kernels live in k_exact.cu and k_force.cu.
#pragma once

#include "sesp_internal.cuh"

namespace sesp {

// k_exact.cu
void upload_tables_exact(const Tables &t, cudaStream_t st);
// per: the configuration preset's periodic cells (every site located on its own)
void launch_locate(const Dev &d, int nmol, const int *smols, int nsurf_sites, int per, int nsite, cudaStream_t st);
void launch_isub(const Dev &d, int nsurf_sites, const int *surf_mols, int per, cudaStream_t st);
// launch shape of the mixed paths' constraint halves (results do not depend on it)
struct ConstraintShape {
    int grid;      // CTAs of the persistent launch (one per SM)
    int s_warps;   // surfactant warps per CTA that starts on the surfactant queue
    int mpw;       // surfactants per such warp (1..8)
};
// nmol / nsite: the state's molecules and sites (bounds of the list checks);
// chains: the surfactants are the configuration preset's flexible chains
// (no constraints; the waters' halves as for the reference preset)
void launch_move_a(const Dev &d, const int *wmols, int nw, const int *smols, int ns, int nrep, int nmol, int nsite,
                   double tol, int maxit, int fast, const ConstraintShape &sh, int chains, cudaStream_t st);
void launch_move_b(const Dev &d, const int *wmols, int nw, const int *smols, int ns, int nmol, int nsite, double tol,
                   int maxit, int fast, const ConstraintShape &sh, int chains, cudaStream_t st);
void launch_init_accel(const Dev &d, int nsite, cudaStream_t st);
// the eta update after the SHAKE half (reads the halves' kinetic sums; the
// RATTLE half reads eta)
void launch_eta(const Dev &d, int nrep, cudaStream_t st);

// k_constraint.cu (mixed paths: FP64 or FP32 sweeps); false if the uploaded
// bond graph is not the one the kernels are specialised for
bool upload_tables_fast(const Tables &t, cudaStream_t st);
// mat: waters as the 3 x 3 system of their constraints (matrix SHAKE /
// RATTLE; the configuration preset's FP64 corrections)
void launch_move_a32(const Dev &d, int nw, const int *smols, int ns, int nmol, int nsite, const ConstraintShape &sh,
                     cudaStream_t st, double tol, int maxit, int fp32, int mat);
void launch_move_b32(const Dev &d, int nw, const int *smols, int ns, int nmol, int nsite, const ConstraintShape &sh,
                     cudaStream_t st, double tol, int maxit, int fp32, int mat);
// reorders the halves' water lists by the sweeps of their last call (at list rebuilds)
void launch_water_order(const Dev &d, const int *wmols, int nw, cudaStream_t st);
int constraint_max_surf_warps();
int constraint_max_mols_per_warp(int fp32);   // fp32: FP32 corrections (SESP_MIXED_FP32C)
void init_constraint_kernels();   // shared-memory limits of the constraint launches

// k_force.cu
void upload_tables_force(const Tables &t, cudaStream_t st);
void launch_sort(const Dev &d, int nsite, int ncell, cudaStream_t st);
void launch_gather(const Dev &d, int nslot, int ncell, int mixed, cudaStream_t st);
// launch shape of the pair field (results do not depend on it)
struct NearShape {
    int tile;   // target sites per work item: 32, 64 or (FP32 path) 128, up to 4 per lane
    int grid;   // CTAs of the persistent kernel
};
void launch_near_items(const Dev &d, int ncell, int nitems_max, int tile, cudaStream_t st);
// per: the periodic preset's kernels
int near_max_ctas_per_sm(int mixed, int tile, int per);
// reset_counter: clear the pair field's work counter first; without it the
// caller must have launched launch_gather (which clears it) on the same
// stream since the last pair-field launch, or the launch finds every work
// item taken and computes nothing
void launch_near(const Dev &d, int ncell, int nslot, int mixed, int terms, const NearShape &shape, cudaStream_t st,
                 bool reset_counter, int per);
// d2: the largest L2 offset per axis (the H table's half-widths)
void launch_fma_build(const Dev &d, int ncell, int n3, int n2, int mixed, int3 d2, cudaStream_t st);
void launch_site_forces(const Dev &d, int nsite, int terms, int mixed, cudaStream_t st);
void launch_graphite(const Dev &d, int terms, int mixed, cudaStream_t st);
void launch_graphite_list(const Dev &d, int nsite, cudaStream_t st);
void init_force_kernels();
void upload_intra_map(const void *host_map, cudaStream_t st);
size_t intra_map_size();
// chains: the surfactants are the configuration preset's 12-bead chains
void launch_intra(const Dev &d, const int *smols, int ns, int terms, int mixed, int chains, cudaStream_t st);
void upload_chain_tables(const ChainTables &t, cudaStream_t st);
void launch_count_pairs(const Dev &d, int ncell, unsigned long long *out, cudaStream_t st);
void launch_flush(void *buf, size_t bytes, cudaStream_t st);
// FP32 FMA throughput of the device in TFLOP/s (an FMA loop timed with CUDA events)
double measure_fp32_peak(int n_sm, cudaStream_t st);
void launch_energies(const Dev &d, int ncell, int nsite, const int *smols, int ns, int chains, double *e_slot,
                     double *e_site, double *e_mol, cudaStream_t st);
// per-replica sums of m v^2 in a fixed order (TEMP_SLICES slices per replica,
// then their tree sum) into d.tbuf[0..nrep); the slices go to d.tbuf[nrep..)
constexpr int TEMP_SLICES = 64;
void launch_temperature(const Dev &d, int nrep, cudaStream_t st);

}  // namespace sesp
