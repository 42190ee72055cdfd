// psim_kernels.cuh -- launch interfaces between the host layer (psim_api.cu)
// and the kernel translation units:
//   psim_exact.cu  FP64 kernels built without FMA contraction (the plain
//                  force form, the vGB update, the cell hash)
//   psim_mixed.cu  the FP32-pair / Kahan-sum force form, from the cell list or
//                  from a Verlet pair list
//   psim_cells.cu  counting sort, scan, reorder, layout conversions
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "psim_device.cuh"

namespace psim {

// A plugin's device functor set, built on the host from psim_force_params.
struct ForceSetup {
    int kind;          // psim_force_kind
    AOPair ao;
    LJPair lj;
    CalPair cal;
    double rc_max;     // largest cutoff: cell_size must be >= rc_max
    float pre_rc2f;    // conservative FP32 prefilter bound on r^2 (FP64 form)
    int tile;          // 0: a warp per 32 consecutive particles; 1: a block per home cell
    int walk;          // with tile 0, the mixed form's walk: 0 direct (default), 1 staged, 2 direct
    int lj_pure;       // LennardJones with yukawaStrength 0 in every replica
};

// Positions and cell ranges in sorted (cell) order, as the force kernels read them.
struct CellView {
    const double4_32a* posd;  // {x, y, z, R}  (FP64 form)
    const float4* posh;   // {x, y, z, R} rounded to FP32
    const float4* posl;   // {x - xh, y - yh, z - zh, slot bits} (mixed form)
    const int* cellid;    // cell hash of each sorted slot
    const int* cstart;    // first sorted slot of each cell
    const int* ccount;    // particles in each cell
};

struct ForceOut {
    double* fx;
    double* fy;
    double* fz;
    uint32_t* err;
    const int* gate;   // may be null; else the pass runs only when *gate != 0
    // updateInteractions fused into the pass (systemHandling.cpp:94-161): when
    // coor is set, the number of neighbours closer than `cont` is written per
    // particle in the pass's order (the FP64 form tests sqrt(r^2) < cont as the
    // reference does; the mixed form r^2 < cont2f).  The caller widens the
    // candidate bound to cover cont; the block-per-cell layout does not count.
    int* coor;
    double cont;
    float cont2f;
};

// Independent replicas in one launch: per warp a task (replica, first
// particle) inside the replica's particle range, and per replica its
// geometry, pair functor (the body's Pair type) and FP32 prefilter bound.
struct BatchView {
    const int2* tasks;   // null: one system
    int n_tasks;
    const DevGeom* geoms;
    const void* pairs;
    const float* pre;
};

cudaError_t launch_forces_fp64(const ForceSetup& fs, const DevGeom& g, const CellView& cv,
                               const ForceOut& out, cudaStream_t st,
                               const BatchView* bv = nullptr);
cudaError_t launch_forces_mixed(const ForceSetup& fs, const DevGeom& g, const CellView& cv,
                                const ForceOut& out, cudaStream_t st,
                                const BatchView* bv = nullptr);

// Verlet pair list of the mixed form (psim_force_list.cuh).  Entries are
// record slots: a particle's list slot (< n), the ghost n that pads lists, or
// n + 1 + h for halo record h -- a periodic image of a particle near a face,
// kept up to date beside it.  The list of slot s is list[k * stride + s].
constexpr int kListFold = 8;   // pair terms per Kahan fold
constexpr int kHaloBaseMax = (1 << 25) - 1;   // halo records per system
struct PairList {
    const int* lslot;      // list slot of each current storage slot (null: the same slot)
    // list order, unwrapped, one record per slot (+ the ghost slot n and the
    // halo records): full, pos[2 s] = {x, y, z, R} high parts and pos[2 s + 1]
    // the low parts; or compact (one float4, compact_record: fixed-point
    // coordinates in units of `unit`) when every particle has the radius `radius`
    const float4* pos;
    const int* count;      // entries of each list slot (a multiple of kListFold)
    const uint32_t* list;
    int stride;
    int compact;
    float radius;
    float unit;            // compact records: the fixed-point unit 2^-k (compact_record)
    // a batch of replicas (rep null: one system): each storage slot's replica
    // and the replicas' pair functors
    const int* rep;
    const void* pairs;
    // threads per particle of the force pass (0 or 1, 2, 4): each lane of a
    // particle takes its 8 / lanes entries of every group and the lanes' sums
    // are added in lane order (compact records; full records take one lane).
    // The ghost record is slot `stride` (n).
    int lanes;
};
cudaError_t launch_forces_list(const ForceSetup& fs, const DevGeom& g, const PairList& pl,
                               const ForceOut& out, cudaStream_t st);
// Builds the list from the cell list of cv (list order = cell order) when
// *gate != 0; pre_r2: FP32 bound on r^2 for (rc + skin) with the rounding margin.
struct ListBuild {
    uint32_t* list;
    int* count;
    int stride;
    int cap;
    float pre_r2;
    const int* gate;
    const int* lhalo;      // per list slot: first halo record << 6 | halo_flags
    int ghost;             // the ghost record (n); halo records follow it
    // a batch of replicas (rep null: one system): each slot's replica, the
    // replicas' geometries and list radii squared (pre_r2 per replica)
    const int* rep;
    const DevGeom* geoms;
    const float* pre;
    // 1: each cell's particles are sorted by x (CanonArgs::xorder), so a row
    // of cells is an x-sorted run that the build trims to the home's reach
    int xsorted;
};
cudaError_t launch_list_build(const DevGeom& g, const CellView& cv, const ListBuild& lb,
                              uint32_t* err, cudaStream_t st);

// vGB coefficients and per-step switches for the integrator kernels.
struct VgbParams {
    double dt, dt2, dt3, dt_inv, c0;
    double coeff0, coeff1, coeff2, coeff3;
    double sig1, sig2, corr, dev, goy2, goy3, hn;
    // the mixed form's normal step: dt^2 coeff1, dt^2 coeff2, and the noise
    // coefficients in FP32
    double dt2c1, dt2c2;
    float sig1f, sig2f, corrf, devf, coeff0f, dt2c1f, dt2c2f;
    int vel_freq;
    uint32_t seed;
};

// Device-side step state, advanced by the rebuild's last kernel so a captured
// CUDA graph replays without host-side argument changes.
struct StepState {
    long long step;       // steps taken since upload (0 -> firstStep)
    int vel_counter;      // brownianIntegrator::velCounter
    int list_builds;      // pair-list rebuilds while stepping
};

struct NoiseView {
    int mode;             // psim_noise_mode
    const double* buf;    // injected noise, [step - first][tag][6]
    long long first;
    long long n_steps;
};

// The system-order integrator: gathers the previous state through perm,
// writes the new state in the current cell order, hashes the new positions
// and counts them into the next grid.
struct VgbSystemArgs {
    int n;
    const int* perm;            // current slot -> previous-order slot (null: the same)
    const int* tag;             // original index of each current slot
    const double* inv_mass;     // 1/m, current order
    const double* x; const double* y; const double* z;       // previous order
    const double* x0; const double* y0; const double* z0;
    const double* mx; const double* my; const double* mz;    // memX/Y/Z
    const double* fx; const double* fy; const double* fz;    // F, current order
    const double* gx; const double* gy; const double* gz;    // F0, previous order
    double* vel;                // 3n, original order (tag-indexed)
    double* ox; double* oy; double* oz;                      // new pos, current order
    double* ox0; double* oy0; double* oz0;
    double* omx; double* omy; double* omz;
    int* key;                   // new cell hash, current order
    int* rank;                  // slot inside the new cell (atomic order)
    int* count;                 // per-cell counts of the next grid (zeroed; null: no hash)
    uint32_t* err;
    const StepState* state;
    // mixed form with a pair list (lbuild null: none).  The new position is
    // also written in list order as the image nearest the list-build position
    // (an exact float pair), and *lflag_set is raised when it lies more than
    // sqrt(ldisp2) from that position; *lflag_clear (the other step parity's
    // flag) is cleared.  lslot: the list slot of each storage slot (null: the
    // same slot, when the storage order is the list order).
    const int* lslot;
    const float4* lbuild;       // list order: positions at the build, .w radius
    float4* lpos;               // PairList::pos
    float linv_unit;            // 1 / PairList::unit (compact), or 0 (full records)
    int* lflag_set;
    int* lflag_clear;
    float ldisp2;
    const int* lhalo;           // per list slot: first halo record << 6 | halo_flags
    int* lhcount;               // halo records handed out (reset here for the next build)
    // a batch of replicas (rep null: one system): the replica of each storage
    // slot, their geometries and Philox seeds (a replica's noise is keyed by
    // its own seed and its particles' indices within it)
    const int* rep;
    const DevGeom* geoms;
    const uint32_t* seeds;
    // box images each particle has crossed (3n, original order; may be null):
    // the unwrapped position is x + img L
    int* img;
};
cudaError_t launch_vgb_system(const VgbSystemArgs& a, const VgbParams& p, const DevGeom& g,
                              const NoiseView& nz, cudaStream_t st);
// The same update with FMA contraction (psim_mixed.cu), for the mixed form.
cudaError_t launch_vgb_system_fast(const VgbSystemArgs& a, const VgbParams& p, const DevGeom& g,
                                   const NoiseView& nz, cudaStream_t st);

// Reference-layout integrator (brownianIntegrator::nextSystem on AoS arrays
// in original order).  mem/mem_corr: 3n device arrays owned by the integrator.
struct VgbAosArgs {
    int n;
    int offset;             // index of the first particle (arrays start there): its noise key
    int first;
    int vel_step;
    double* pos; double* pos0; double* vel;
    const double* frc; const double* frc0;
    const double* mass;
    double* mem; double* mem_corr;
    const double* noise;        // n*6 (injected) or null
    uint32_t seed;
    long long philox_step;
    uint32_t* err;
};
cudaError_t launch_vgb_aos(const VgbAosArgs& a, const VgbParams& p, double L, cudaStream_t st);

// nextSystem straight on the caller's host arrays (original order), which
// the GPU reads and writes in place over the coherent host link -- no copies.
// F/F0: this step's force and the previous one (host); with frc_out set the
// pushed forces are written back (frc0_out <- F0, frc_out <- F).
struct VgbHostArgs {
    int n;
    int first;
    int vel_step;
    double* pos; double* pos0; double* vel;   // host, read and written
    const double* F; const double* F0;        // host
    double* frc_out; double* frc0_out;        // host, or null: no push
    const double* mass;                       // host
    double* mem; double* mem_corr;            // device
    const double* noise;                      // host n*6 (injected) or null
    uint32_t seed;
    long long philox_step;
    uint32_t* err;
};
cudaError_t launch_vgb_host(const VgbHostArgs& a, const VgbParams& p, double L, cudaStream_t st);

// Cell hash + atomic count of positions given as three coordinate arrays.
// rep/geoms (may be null): a batch's replica of each particle and their grids.
cudaError_t launch_hash_count(int n, const double* x, const double* y, const double* z,
                              const DevGeom& g, int* key, int* rank, int* count,
                              uint32_t* err, cudaStream_t st, const int* rep = nullptr,
                              const DevGeom* geoms = nullptr);

// ---------------------------------------------------------- cells (psim_cells.cu)
// Exclusive scan of count[ncell] into start[ncell]; scratch needs
// scan_scratch_ints(ncell) ints.
size_t scan_scratch_ints(int ncell);
cudaError_t launch_scan(const int* count, int* start, int ncell, int* scratch, cudaStream_t st);

// tmp[start[key[f]] + rank[f]] = f
cudaError_t launch_scatter(int n, const int* key, const int* rank, const int* start, int* tmp,
                           const uint32_t* err, cudaStream_t st);

// Canonical order inside each cell (by original index), the permutation and
// the sorted-order arrays the force kernel reads.
struct CanonArgs {
    int n;
    const int* tmp;         // atomic-order slot -> previous-order index
    const int* key;         // cell of each previous-order index
    const int* start;
    const int* count;
    const int* tag_in;      // previous order
    const double* radius_in;
    const double* inv_mass_in;
    const double* x; const double* y; const double* z;   // positions, previous order
    int* perm;              // new slot -> previous index
    int* tag_out;
    double* radius_out;
    double* inv_mass_out;   // may be null
    int* cellid;
    double4_32a* posd;          // may be null
    float4* posh;
    float4* posl;           // may be null
    StepState* state;       // may be null: advanced once per rebuild
    int advance;            // 1: this rebuild ends a step (advance state)
    int vel_freq;           // brownianIntegrator::velFreq
    uint32_t* err;          // non-zero: a previous kernel failed, skip the work
    // pair-list bookkeeping (null: none).  lslot is carried with the particles;
    // when *rebuild != 0 the list is rebuilt on the new order, so lslot becomes
    // the identity and posh/posl/lbuild are written -- otherwise posh/posl
    // hold the list-order positions and are left alone.
    const int* rebuild;
    const int* lslot_in;
    int* lslot_out;
    float4* lbuild;
    float4* lpos;           // PairList::pos, written with posh/posl
    float linv_unit;        // 1 / PairList::unit (compact), or 0 (full records)
    // halo records of the particles within hr of a face (rebuild only):
    // lhalo per slot, records n + 1 + [0, hcap) handed out by *lhcount
    int* lhalo;
    int* lhcount;
    int hcap;
    float hr, Lf, Lhi, Llo;
    // a batch of replicas (rep null: one system): the halo radius and the box
    // of each slot's replica
    const int* rep;
    const DevGeom* geoms;
    const float* hr_rep;
    // order within a cell: 0 by tag (the reference layout), 1 by x then tag
    // (a pair-list order: each row of cells is sorted by x, which the list
    // build uses to trim its runs)
    int xorder;
};
cudaError_t launch_canonicalize(const CanonArgs& a, cudaStream_t st);

// Full 32-byte pair-list records of the sorted positions (posh, posl) and
// the halo images of the particles within hr of a face (lhalo per slot,
// records n + 1 + [0, hcap) handed out by *lhcount, zeroed by the caller).
// inv_unit != 0: compact 16-byte records of that low-part unit (every
// particle has one radius), else full records.
cudaError_t launch_list_records(int n, const float4* posh, const float4* posl, float4* lpos,
                                int* lhalo, int* lhcount, int hcap, float hr, const DevGeom& g,
                                uint32_t* err, cudaStream_t st, float inv_unit = 0.f);

// The force drop-in's kept pair list on a later call: the records at the
// build's slots (slot_of: original index -> slot) rewritten from this call's
// sorted positions (tag: slot -> original index), each as the image nearest
// its build position (lbuild), with its halo images (lhalo); *flag = 1 when
// a particle has moved more than sqrt(disp2) since the build, or (compact
// records, inv_unit != 0) when its radius is not the build's `radius`.
cudaError_t launch_list_refresh(int n, const double4_32a* posd, const int* tag,
                                const int* slot_of, const float4* lbuild, const int* lhalo,
                                float4* lpos, float disp2, const DevGeom& g, float inv_unit,
                                float radius, int* flag, cudaStream_t st);
// slot_of[tag[k]] = k (tag: every value in [0, n)).
cudaError_t launch_invert_tags(int n, const int* tag, int* slot_of, cudaStream_t st);

// End of a step whose cell list is rebuilt only with its pair list: advances
// the step state (canonicalize_kernel's bookkeeping) and decides the rebuild
// -- the flag the integrator raised, unless an error is latched.  In a graph
// (use_handle) the decision sets the conditional node that runs the rebuild.
cudaError_t launch_step_end(StepState* state, const int* lflag, const uint32_t* err,
                            int vel_freq, cudaGraphConditionalHandle handle, int use_handle,
                            cudaStream_t st);

// dst[k][g] = src[k][perm[g]] for the first narr arrays (the state carried
// into a new cell order).
struct PermuteArgs {
    int n;
    const int* perm;
    int narr;
    const double* src[16];
    double* dst[16];
};
cudaError_t launch_permute(const PermuteArgs& a, const uint32_t* err, cudaStream_t st);

// Reference layout exports (outputs may be host memory written in place).
cudaError_t launch_export_cells(int n, int ncell, const int* cellid, const int* tag,
                                const double4_32a* posd, const int* start, const int* count,
                                int32_t* hash_index, uint32_t* cse, double* sorted,
                                cudaStream_t st);
// Sorted-order SoA force -> original-order AoS (particle_force layout).
cudaError_t launch_unsort_force(int n, const int* tag, const double* fx, const double* fy,
                                const double* fz, double* out, cudaStream_t st);
// Reference layout imports for psim_force_evaluate.
// Also hashes each position into cellid (EBIT_CELL when outside the grid).
// sorted/hash_index may be host memory the device can read in place.
// *mixed_radii (if not null) = 1 when the radii are not all equal.
cudaError_t launch_import_sorted(int n, const double* sorted, const int32_t* hash_index,
                                 const DevGeom& g, double4_32a* posd, float4* posh, float4* posl,
                                 int* cellid, int* tag, uint32_t* err, cudaStream_t st,
                                 int* mixed_radii = nullptr);
// out[3 i + k] = f_k[inv[i]]: forces from the force pass's order to the
// original order (out may be host memory written in place).
cudaError_t launch_export_force(int n, const int* inv, const double* fx, const double* fy,
                                const double* fz, double* out, cudaStream_t st);
// Counts from (start, end) pairs, starts re-derived by a scan (so empty
// cells keep the back-to-back layout the row walk of the force pass needs);
// a range beyond n, or a start that disagrees with that layout, sets
// EBIT_INDEX.  scratch: scan_scratch_ints(ncell) ints.
cudaError_t launch_import_cse(int ncell, int n, const uint32_t* cse, int* start, int* count,
                              int* scratch, uint32_t* err, cudaStream_t st);
// Positions (3n AoS) and radii, possibly host memory read in place, into
// SoA x, y, z and a device copy of the radii.
cudaError_t launch_import_positions(int n, const double* aos, const double* radius, double* x,
                                    double* y, double* z, double* radius_out, cudaStream_t st);
// AoS xyz -> three arrays, optionally scattered by tag (gather == 0) or
// gathered (gather == 1: out[i] = in[tag[i]]).
cudaError_t launch_split_xyz(int n, const double* aos, const int* tag, int gather, double* x,
                             double* y, double* z, cudaStream_t st);
// three arrays in storage order -> AoS original order: out[tag[i]] = (x[i], y[i], z[i]);
// with perm != null the source index is perm[i].
cudaError_t launch_merge_xyz(int n, const double* x, const double* y, const double* z,
                             const int* tag, const int* perm, double* aos, cudaStream_t st);
cudaError_t launch_fill_int_iota(int n, int* v, cudaStream_t st);
// out[i] = (x[perm[i]], y[perm[i]], z[perm[i]], radius[i])
// Sorted-order float4 {x, y, z, R} from storage-order FP64 positions.
cudaError_t launch_gather_posh(int n, const int* perm, const double* x, const double* y,
                               const double* z, const double* radius, float4* out,
                               cudaStream_t st);
cudaError_t launch_gather_posd(int n, const int* perm, const double* x, const double* y,
                               const double* z, const double* radius, double4_32a* out,
                               cudaStream_t st);
cudaError_t launch_occupancy(int ncell, const int* count, int* max_out, cudaStream_t st);
// Ordered pairs closer than rc (FP32 test on posh) summed into *total.
cudaError_t launch_pair_count(const DevGeom& g, const CellView& cv, float rc2,
                              unsigned long long* total, cudaStream_t st);
// FMA-chain throughput probe: `iters` rounds of 8 independent FMA chains per thread.
cudaError_t launch_fma_probe(int blocks, int threads, int iters, float* sink, cudaStream_t st);
// Host-link probe: copies `bytes` (a multiple of 16) from src to dst with
// SM loads and stores; either may be host memory.
cudaError_t launch_link_copy(int blocks, const void* src, void* dst, size_t bytes,
                             cudaStream_t st);

// Observables of the device-resident state (psim_observe.cu).
enum ObserveWhat { OBS_MEAN_DISP = 0, OBS_TRACKED = 1, OBS_POTENTIAL = 2 };
struct ObserveArgs {
    int n;
    int what;                   // ObserveWhat
    const double* x; const double* y; const double* z;      // positions, storage order
    const double* x0; const double* y0; const double* z0;   // previous positions, same order
    const double* fx; const double* fy; const double* fz;   // force of the last step, same order
    const double* gx; const double* gy; const double* gz;   // the force before, previous order
    const int* perm_prev;       // storage slot -> slot of the previous order
    const int* tag;             // original index of each storage slot
    const int* img;             // box images crossed (3n, original order)
    const double* start;        // positions when tracking started (3n, original order)
    double L;
};
// sum of v[i]^2 (count values); scratch: observe_scratch_doubles() doubles
cudaError_t launch_sum_squares(long long count, const double* v, double* scratch, double* out,
                               cudaStream_t st);
cudaError_t launch_observe(const ObserveArgs& a, double* scratch, double* out, cudaStream_t st);
int observe_scratch_doubles();
// 27-cell walk over sorted FP64 positions: coordination numbers (r < r_contact,
// written at the original index) and a histogram of r in [r_min, r_max)
struct PairScanArgs {
    DevGeom g;
    const double4_32a* posd;
    const int* cellid;
    const int* cstart;
    const int* ccount;
    const int* tag;
    double r_contact;
    int* coor;                      // may be null
    unsigned long long* n_pairs;    // may be null: sum of the coordination numbers
    double r_min, r_max, inv_dr;
    int n_bins;                     // 0: no histogram
    unsigned long long* hist;
};
cudaError_t launch_pair_scan(const PairScanArgs& a, cudaStream_t st);
// FP64 potential energy and virial of the plugin's pair force over the 27-cell
// walk of a: out[0] = sum over pairs of u(r), out[1] = sum over pairs of
// r_ij . f_ij (f_ij the force on i from j).  scratch: 2 * ceil(n / 128) doubles.
// cudaErrorInvalidValue for a force kind without an energy.
cudaError_t launch_energy(const ForceSetup& fs, const PairScanArgs& a, double* scratch,
                          double* out, cudaStream_t st);
// Clusters of the contact graph (r < a.r_contact): root[original index] = the
// smallest original index of its cluster, size[root] = cluster size (zeroed
// by the caller); label: union-find scratch (n ints).
cudaError_t launch_clusters(const PairScanArgs& a, int* label, int* root, int* size,
                            uint32_t* err, cudaStream_t st);

}  // namespace psim
