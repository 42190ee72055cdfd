// psim_cells.cu -- the hashed cell list as a counting sort (integer work).
//
// The reference hashes, sorts (hash, index) pairs with an unstable parallel
// sort and then walks the sorted list to fill cellStartEnd and gather the
// packed positions (ClusteredCore/src/system/systemHandling.cpp:33-85).  Here:
//   1. hash + histogram: every particle's cell and an atomic slot in it
//      (fused into the integrator epilogue, psim_exact.cu)
//   2. exclusive scan of the per-cell counts -> cell start
//   3. scatter each particle to start + atomic slot
//   4. canonicalise: inside a cell, rank the members by original index, so
//      the order is deterministic (that of a stable sort on (hash, index));
//      fused with the gather of everything the force pass reads
// The cell hashes and memberships equal the reference's bit for bit.
#include "psim_kernels.cuh"

namespace psim {

namespace {
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;

__device__ __forceinline__ int block_scan_exclusive(int v, int* warp_tot, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    total = warp_tot[(blockDim.x >> 5) - 1];
    const int excl = x - v + (warp > 0 ? warp_tot[warp - 1] : 0);
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(kScanBlock) scan_tile_sums(const int* in, int n, int* sums) {
    __shared__ int wt[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) v += in[base + k];
    int total;
    block_scan_exclusive(v, wt, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) scan_sums_inplace(int* sums, int nb) {
    __shared__ int wt[32];
    const int base = threadIdx.x * kScanItems;
    int loc[kScanItems];
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        loc[k] = (base + k < nb) ? sums[base + k] : 0;
        v += loc[k];
    }
    int total;
    int run = block_scan_exclusive(v, wt, total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < nb) sums[base + k] = run;
        run += loc[k];
    }
}

__global__ void __launch_bounds__(kScanBlock)
scan_finalize(const int* in, int n, const int* sums, int* out) {
    __shared__ int wt[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int loc[kScanItems];
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        loc[k] = (base + k < n) ? in[base + k] : 0;
        v += loc[k];
    }
    int total;
    int run = block_scan_exclusive(v, wt, total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += loc[k];
    }
}
}  // namespace

size_t scan_scratch_ints(int ncell) { return (size_t)(ncell + kScanTile - 1) / kScanTile + 1; }

cudaError_t launch_scan(const int* count, int* start, int ncell, int* scratch, cudaStream_t st) {
    if (ncell <= 0) return cudaSuccess;
    const int nb = (ncell + kScanTile - 1) / kScanTile;
    if (nb > kScanTile) return cudaErrorInvalidValue;  // > 16.7M cells
    scan_tile_sums<<<nb, kScanBlock, 0, st>>>(count, ncell, scratch);
    scan_sums_inplace<<<1, kScanBlock, 0, st>>>(scratch, nb);
    scan_finalize<<<nb, kScanBlock, 0, st>>>(count, ncell, scratch, start);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
scatter_kernel(int n, const int* key, const int* rank, const int* start, int* tmp,
               const uint32_t* err) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n || (err && *err)) return;
    tmp[start[key[f]] + rank[f]] = f;
}

cudaError_t launch_scatter(int n, const int* key, const int* rank, const int* start, int* tmp,
                           const uint32_t* err, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    scatter_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, key, rank, start, tmp, err);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) canonicalize_kernel(CanonArgs a, int vel_freq) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (a.err && *a.err) return;
    if (p < a.n) {
        const int f = a.tmp[p];
        const int c = a.key[f];
        const int st = a.start[c];
        const int cnt = a.count[c];
        const int mine = a.tag_in[f];
        int r = 0;
        if (a.xorder) {
            // by x, then tag: the bit patterns of the (non-negative) positions
            // order like their values, and every pattern is comparable
            const long long mx = __double_as_longlong(a.x[f]);
            for (int q = st; q < st + cnt; ++q) {
                const int fq = a.tmp[q];
                const long long xq = __double_as_longlong(a.x[fq]);
                r += (xq < mx || (xq == mx && a.tag_in[fq] < mine)) ? 1 : 0;
            }
        } else {
            for (int q = st; q < st + cnt; ++q) r += (a.tag_in[a.tmp[q]] < mine) ? 1 : 0;
        }
        const int g = st + r;
        a.perm[g] = f;
        a.tag_out[g] = mine;
        a.cellid[g] = c;
        const double R = a.radius_in[f];
        a.radius_out[g] = R;
        if (a.inv_mass_out) a.inv_mass_out[g] = a.inv_mass_in[f];
        // with a pair list, the sorted positions are written only when the
        // list is rebuilt on this order (they are the list's positions)
        const bool pos_out = !a.rebuild || *a.rebuild != 0;
        if (a.lslot_out) a.lslot_out[g] = (pos_out || !a.lslot_in) ? g : a.lslot_in[f];
        if (pos_out) {
            const double x = a.x[f], y = a.y[f], z = a.z[f];
            if (a.posd) a.posd[g] = make_double4_32a(x, y, z, R);
            float4 h, l;
            split_f64(x, h.x, l.x);
            split_f64(y, h.y, l.y);
            split_f64(z, h.z, l.z);
            h.w = (float)R;
            l.w = __int_as_float(g);  // the slot, which the pair-list build reads
            a.posh[g] = h;
            if (a.posl) a.posl[g] = l;
            if (a.lbuild) a.lbuild[g] = h;
            if (a.lpos) {
                l.w = 0.f;
                store_record(a.lpos, a.linv_unit, (size_t)g, h, l);
                // images of a particle near a face, as halo records (in a
                // batch, of its replica's box)
                float hr = a.hr, Lf = a.Lf, Lhi = a.Lhi, Llo = a.Llo;
                if (a.rep) {
                    const int r = a.rep[g];
                    hr = a.hr_rep[r];
                    Lf = Lhi = a.geoms[r].Lhi;
                    Llo = a.geoms[r].Llo;
                }
                uint32_t fl = halo_flags(h, hr, Lf);
                const int m = halo_copies(fl);
                int base = 0;
                if (m > 0) {
                    base = atomicAdd(a.lhcount, m);
                    if (base + m > a.hcap) {
                        atomicOr(a.err, EBIT_LIST);
                        fl = 0;
                        base = 0;
                    } else {
                        halo_write(a.lpos + (a.linv_unit != 0.f ? 1 : 2) * ((size_t)a.n + 1),
                                   a.linv_unit, base, fl, h, l, Lhi, Llo);
                    }
                }
                a.lhalo[g] = (base << 6) | (int)fl;
            }
        }
    }
    if (a.state && a.advance && p == 0) {
        // end of a step: brownianIntegrator's velCounter bookkeeping
        // (brownianIntegrator.cpp:291-292) runs only after normal steps
        StepState s = *a.state;
        if (s.step > 0) s.vel_counter = (s.vel_counter == vel_freq) ? 0 : s.vel_counter + 1;
        s.step += 1;
        if (a.rebuild && *a.rebuild) s.list_builds += 1;
        *a.state = s;
    }
}

cudaError_t launch_canonicalize(const CanonArgs& a, cudaStream_t st) {
    const int blocks = a.n > 0 ? (a.n + 255) / 256 : 1;
    canonicalize_kernel<<<blocks, 256, 0, st>>>(a, a.vel_freq);
    return cudaGetLastError();
}

// The reference-layout outputs, which may be host memory written in place:
// each block stages its spans through shared memory and writes them as
// coalesced runs.
__global__ void __launch_bounds__(256)
export_particles_kernel(int n, const int* cellid, const int* tag, const double4_32a* posd,
                        int32_t* hash_index, double* sorted) {
    __shared__ double ss[4 * 256];
    __shared__ int32_t sh[2 * 256];
    const int b0 = blockIdx.x * blockDim.x;
    const int m = min((int)blockDim.x, n - b0);
    const int i = b0 + threadIdx.x, u = threadIdx.x;
    if (i < n) {
        if (hash_index) {
            sh[2 * u] = cellid[i];
            sh[2 * u + 1] = tag[i];
        }
        if (sorted) {
            const double4_32a p = posd[i];
            ss[4 * u] = p.x;
            ss[4 * u + 1] = p.y;
            ss[4 * u + 2] = p.z;
            ss[4 * u + 3] = p.w;
        }
    }
    __syncthreads();
    if (hash_index)
        for (int k = u; k < 2 * m; k += blockDim.x) hash_index[2 * (size_t)b0 + k] = sh[k];
    if (sorted)
        for (int k = u; k < 4 * m; k += blockDim.x) sorted[4 * (size_t)b0 + k] = ss[k];
}

__global__ void __launch_bounds__(256)
export_cells_kernel(int ncell, const int* start, const int* count, uint32_t* cse) {
    __shared__ uint32_t sc[2 * 256];
    const int b0 = blockIdx.x * blockDim.x;
    const int m = min((int)blockDim.x, ncell - b0);
    const int c = b0 + threadIdx.x;
    if (c < ncell) {
        const int k = count[c];
        // empty cells keep clearCells' sentinel (system.h:166)
        sc[2 * threadIdx.x] = k > 0 ? (uint32_t)start[c] : 0xffffffffu;
        sc[2 * threadIdx.x + 1] = k > 0 ? (uint32_t)(start[c] + k) : 0xffffffffu;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * m; k += blockDim.x) cse[2 * (size_t)b0 + k] = sc[k];
}

cudaError_t launch_export_cells(int n, int ncell, const int* cellid, const int* tag,
                                const double4_32a* posd, const int* start, const int* count,
                                int32_t* hash_index, uint32_t* cse, double* sorted,
                                cudaStream_t st) {
    if (n > 0 && (hash_index || sorted))
        export_particles_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, cellid, tag, posd,
                                                                 hash_index, sorted);
    if (ncell > 0 && cse)
        export_cells_kernel<<<(ncell + 255) / 256, 256, 0, st>>>(ncell, start, count, cse);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
unsort_force_kernel(int n, const int* tag, const double* fx, const double* fy, const double* fz,
                    double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t o = 3 * (size_t)tag[i];
    out[o] = fx[i];
    out[o + 1] = fy[i];
    out[o + 2] = fz[i];
}

cudaError_t launch_unsort_force(int n, const int* tag, const double* fx, const double* fy,
                                const double* fz, double* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    unsort_force_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, tag, fx, fy, fz, out);
    return cudaGetLastError();
}

// The caller's sorted particles and hash index, which may be host memory
// read in place: a block stages its spans through shared memory so that each
// access is a coalesced run.  *mixed_radii (if not null) is set when a radius
// differs from the first particle's.
__global__ void __launch_bounds__(256)
import_sorted_kernel(int n, const double* sorted, const int32_t* hi, DevGeom g, double4_32a* posd,
                     float4* posh, float4* posl, int* cellid, int* tag, uint32_t* err,
                     int* mixed_radii) {
    __shared__ double ss[4 * 256];
    __shared__ int32_t sh[2 * 256];
    __shared__ double r0;
    const int b0 = blockIdx.x * blockDim.x;
    const int m = min((int)blockDim.x, n - b0);
    if (threadIdx.x == 0 && mixed_radii) r0 = sorted[3];
    for (int k = threadIdx.x; k < 4 * m; k += blockDim.x) ss[k] = sorted[4 * (size_t)b0 + k];
    for (int k = threadIdx.x; k < 2 * m; k += blockDim.x) sh[k] = hi[2 * (size_t)b0 + k];
    __syncthreads();
    const int i = b0 + threadIdx.x;
    if (i >= n) return;
    const int u = threadIdx.x;
    const double x = ss[4 * u], y = ss[4 * u + 1], z = ss[4 * u + 2], R = ss[4 * u + 3];
    if (mixed_radii && R != r0) *mixed_radii = 1;
    posd[i] = make_double4_32a(x, y, z, R);
    float4 h, l;
    split_f64(x, h.x, l.x);
    split_f64(y, h.y, l.y);
    split_f64(z, h.z, l.z);
    h.w = (float)R;
    l.w = __int_as_float(i);
    posh[i] = h;
    if (posl) posl[i] = l;
    int t = sh[2 * u + 1];
    if (t < 0 || t >= n) {  // an original index outside [0, n): refuse, stay in bounds
        atomicOr(err, (uint32_t)EBIT_INDEX);
        t = 0;
    }
    tag[i] = t;
    // the home cell, as getAcceleration recomputes it from the position
    // (AOPotential.cpp:143-145)
    int c[3];
    const double p[3] = {x, y, z};
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int q = cell_coord(p[k], g);
        if (q < 0 || q >= g.s) { bad = true; q = q < 0 ? 0 : g.s - 1; }
        c[k] = q;
    }
    cellid[i] = c[0] + g.s * c[1] + g.s2 * c[2];
    if (bad) atomicOr(err, (uint32_t)EBIT_CELL);
}

cudaError_t launch_import_sorted(int n, const double* sorted, const int32_t* hash_index,
                                 const DevGeom& g, double4_32a* posd, float4* posh, float4* posl,
                                 int* cellid, int* tag, uint32_t* err, cudaStream_t st,
                                 int* mixed_radii) {
    if (n == 0) return cudaSuccess;
    import_sorted_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, sorted, hash_index, g, posd, posh,
                                                          posl, cellid, tag, err, mixed_radii);
    return cudaGetLastError();
}

// The force of each original index i, read at its slot inv[i] of the force
// pass's order, written to `out` (3n, original order; may be host memory
// written in place) through shared memory in coalesced runs.
__global__ void __launch_bounds__(256)
export_force_kernel(int n, const int* inv, const double* fx, const double* fy, const double* fz,
                    double* out) {
    __shared__ double so[3 * 256];
    const int b0 = blockIdx.x * blockDim.x;
    const int m = min((int)blockDim.x, n - b0);
    const int i = b0 + threadIdx.x;
    if (i < n) {
        const int s = inv[i];
        so[3 * threadIdx.x] = fx[s];
        so[3 * threadIdx.x + 1] = fy[s];
        so[3 * threadIdx.x + 2] = fz[s];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m; k += blockDim.x) out[3 * (size_t)b0 + k] = so[k];
}

cudaError_t launch_export_force(int n, const int* inv, const double* fx, const double* fy,
                                const double* fz, double* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    export_force_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, inv, fx, fy, fz, out);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
import_cse_kernel(int ncell, int n, const uint32_t* cse, int* count, uint32_t* err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const uint32_t s = cse[2 * (size_t)c], e = cse[2 * (size_t)c + 1];
    bool empty = (s == 0xffffffffu) || (e == 0xffffffffu);
    if (!empty && (e < s || e > (uint32_t)n)) {  // a range outside the particle list
        atomicOr(err, (uint32_t)EBIT_INDEX);
        empty = true;
    }
    count[c] = empty ? 0 : (int)(e - s);
}

// Every non-empty cell must start where the counting-sort layout puts it
// (the layout reorderParticles produces: cells in hash order, back to back).
__global__ void __launch_bounds__(256)
check_cse_kernel(int ncell, const uint32_t* cse, const int* start, const int* count,
                 uint32_t* err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    if (count[c] > 0 && cse[2 * (size_t)c] != (uint32_t)start[c])
        atomicOr(err, (uint32_t)EBIT_INDEX);
}

cudaError_t launch_import_cse(int ncell, int n, const uint32_t* cse, int* start, int* count,
                              int* scratch, uint32_t* err, cudaStream_t st) {
    if (ncell == 0) return cudaSuccess;
    const int blocks = (ncell + 255) / 256;
    import_cse_kernel<<<blocks, 256, 0, st>>>(ncell, n, cse, count, err);
    cudaError_t e = launch_scan(count, start, ncell, scratch, st);
    if (e != cudaSuccess) return e;
    check_cse_kernel<<<blocks, 256, 0, st>>>(ncell, cse, start, count, err);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
split_xyz_kernel(int n, const double* aos, const int* tag, int gather, double* x, double* y,
                 double* z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t s = 3 * (size_t)((tag && gather) ? tag[i] : i);
    x[i] = aos[s];
    y[i] = aos[s + 1];
    z[i] = aos[s + 2];
}

// Positions (3n AoS) and radii of the caller, which may be host memory read
// in place, into SoA coordinates and a device copy of the radii, each block
// reading its spans as coalesced runs through shared memory.
__global__ void __launch_bounds__(256)
import_positions_kernel(int n, const double* aos, const double* radius, double* x, double* y,
                        double* z, double* radius_out) {
    __shared__ double sp[3 * 256];
    const int b0 = blockIdx.x * blockDim.x;
    const int m = min((int)blockDim.x, n - b0);
    for (int k = threadIdx.x; k < 3 * m; k += blockDim.x) sp[k] = aos[3 * (size_t)b0 + k];
    __syncthreads();
    const int i = b0 + threadIdx.x;
    if (i >= n) return;
    x[i] = sp[3 * threadIdx.x];
    y[i] = sp[3 * threadIdx.x + 1];
    z[i] = sp[3 * threadIdx.x + 2];
    radius_out[i] = radius[i];
}

cudaError_t launch_import_positions(int n, const double* aos, const double* radius, double* x,
                                    double* y, double* z, double* radius_out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    import_positions_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, aos, radius, x, y, z, radius_out);
    return cudaGetLastError();
}

cudaError_t launch_split_xyz(int n, const double* aos, const int* tag, int gather, double* x,
                             double* y, double* z, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    split_xyz_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, aos, tag, gather, x, y, z);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
merge_xyz_kernel(int n, const double* x, const double* y, const double* z, const int* tag,
                 const int* perm, double* aos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = perm ? perm[i] : i;
    const size_t d = 3 * (size_t)(tag ? tag[i] : i);
    aos[d] = x[src];
    aos[d + 1] = y[src];
    aos[d + 2] = z[src];
}

cudaError_t launch_merge_xyz(int n, const double* x, const double* y, const double* z,
                             const int* tag, const int* perm, double* aos, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    merge_xyz_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, x, y, z, tag, perm, aos);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) iota_kernel(int n, int* v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

cudaError_t launch_fill_int_iota(int n, int* v, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    iota_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, v);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
gather_posh_kernel(int n, const int* perm, const double* x, const double* y, const double* z,
                   const double* radius, float4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm[i];
    out[i] = make_float4((float)x[o], (float)y[o], (float)z[o], (float)radius[i]);
}

cudaError_t launch_gather_posh(int n, const int* perm, const double* x, const double* y,
                               const double* z, const double* radius, float4* out,
                               cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    gather_posh_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, perm, x, y, z, radius, out);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
gather_posd_kernel(int n, const int* perm, const double* x, const double* y, const double* z,
                   const double* radius, double4_32a* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm[i];
    out[i] = make_double4_32a(x[o], y[o], z[o], radius[i]);
}

cudaError_t launch_gather_posd(int n, const int* perm, const double* x, const double* y,
                               const double* z, const double* radius, double4_32a* out,
                               cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    gather_posd_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, perm, x, y, z, radius, out);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) occupancy_kernel(int ncell, const int* count, int* mx) {
    int best = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x)
        best = max(best, count[c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, best);
}

cudaError_t launch_occupancy(int ncell, const int* count, int* max_out, cudaStream_t st) {
    if (ncell == 0) return cudaSuccess;
    int blocks = (ncell + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    occupancy_kernel<<<blocks, 256, 0, st>>>(ncell, count, max_out);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(128)
pair_count_kernel(DevGeom g, CellView cv, float rc2, unsigned long long* total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int cnt = 0;
    if (i < g.n) {
        const float4 hi = cv.posh[i];
        const int c = cv.cellid[i];
        const int cx = c % g.s, cy = (c / g.s) % g.s, cz = c / g.s2;
        for (int dx = -1; dx <= 1; ++dx) {
            int shx;
            const int x = wrap_cell(cx + dx, g.s, shx);
            for (int dy = -1; dy <= 1; ++dy) {
                int shy;
                const int y = wrap_cell(cy + dy, g.s, shy);
                for (int dz = -1; dz <= 1; ++dz) {
                    int shz;
                    const int z = wrap_cell(cz + dz, g.s, shz);
                    const int cell = x + g.s * y + g.s2 * z;
                    const int st = cv.cstart[cell], en = st + cv.ccount[cell];
                    for (int j = st; j < en; ++j) {
                        const float4 hj = cv.posh[j];
                        const float ex = (hj.x + shx * g.Lhi) - hi.x;
                        const float ey = (hj.y + shy * g.Lhi) - hi.y;
                        const float ez = (hj.z + shz * g.Lhi) - hi.z;
                        cnt += (j != i && ex * ex + ey * ey + ez * ez < rc2) ? 1u : 0u;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(total, (unsigned long long)cnt);
}

cudaError_t launch_pair_count(const DevGeom& g, const CellView& cv, float rc2,
                              unsigned long long* total, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    pair_count_kernel<<<(g.n + 127) / 128, 128, 0, st>>>(g, cv, rc2, total);
    return cudaGetLastError();
}

// The pair-list records of a sorted order, one 32-byte float-pair record per
// slot (radius in the high part), and the halo images of the particles within
// hr of a face (the list records the canonicalisation writes, for positions
// that are already sorted).
__global__ void __launch_bounds__(256)
list_records_kernel(int n, const float4* posh, const float4* posl, float4* lpos, int* lhalo,
                    int* lhcount, int hcap, float hr, float Lf, float Lhi, float Llo,
                    float inv_unit, uint32_t* err) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || *err) return;
    const float4 h = posh[g];
    float4 l = posl[g];
    l.w = 0.f;
    store_record(lpos, inv_unit, (size_t)g, h, l);
    uint32_t fl = halo_flags(h, hr, Lf);
    const int m = halo_copies(fl);
    int base = 0;
    if (m > 0) {
        base = atomicAdd(lhcount, m);
        if (base + m > hcap) {
            atomicOr(err, EBIT_LIST);
            fl = 0;
            base = 0;
        } else {
            halo_write(lpos + (inv_unit != 0.f ? 1 : 2) * ((size_t)n + 1), inv_unit, base, fl,
                       h, l, Lhi, Llo);
        }
    }
    lhalo[g] = (base << 6) | (int)fl;
}

cudaError_t launch_list_records(int n, const float4* posh, const float4* posl, float4* lpos,
                                int* lhalo, int* lhcount, int hcap, float hr, const DevGeom& g,
                                uint32_t* err, cudaStream_t st, float inv_unit) {
    if (n == 0) return cudaSuccess;
    list_records_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, posh, posl, lpos, lhalo, lhcount, hcap,
                                                         hr, (float)g.L, g.Lhi, g.Llo, inv_unit,
                                                         err);
    return cudaGetLastError();
}

// The drop-in force pass's kept pair list on a later call.  Each particle
// (sorted slot k of this call, original index tag[k]) has its record at its
// slot of the build rewritten from this call's position: the image nearest
// its position at the build, as an exact float pair, with its halo images --
// as the integrator of a system with a pair list writes them.  *flag is set
// when a particle has moved more than sqrt(disp2) since the build, or when
// its original index has no slot of the build.
__global__ void __launch_bounds__(256)
list_refresh_kernel(int n, const double4_32a* posd, const int* tag, const int* slot_of,
                    const float4* lbuild, const int* lhalo, float4* lpos, float disp2, float Lhi,
                    float Llo, double L, float inv_unit, float radius, int* flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int s = slot_of[tag[k]];
    if (s < 0 || s >= n) {
        *flag = 1;
        return;
    }
    const double4_32a p = posd[k];
    const float4 b = lbuild[s];
    const double x[3] = {p.x, p.y, p.z};
    const float bb[3] = {b.x, b.y, b.z};
    const float halff = 0.5f * Lhi;
    float h[3], l[3], d2 = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        split_f64(x[a], h[a], l[a]);
        const float da = h[a] - bb[a];
        if (da > halff || da < -halff)  // wrapped since the build: the other image
            split_f64(da > 0.f ? x[a] - L : x[a] + L, h[a], l[a]);
        const float e = h[a] - bb[a];
        d2 += e * e;
    }
    const float4 hv = make_float4(h[0], h[1], h[2], (float)p.w);
    const float4 lv = make_float4(l[0], l[1], l[2], 0.f);
    store_record(lpos, inv_unit, (size_t)s, hv, lv);
    const int hal = lhalo[s];
    if (hal & 63)
        halo_write(lpos + (inv_unit != 0.f ? 1 : 2) * ((size_t)n + 1), inv_unit, hal >> 6,
                   (uint32_t)(hal & 63), hv, lv, Lhi, Llo);
    // compact records hold no radius: every particle must keep the build's
    if (d2 > disp2 || (inv_unit != 0.f && (float)p.w != radius)) *flag = 1;
}

cudaError_t launch_list_refresh(int n, const double4_32a* posd, const int* tag,
                                const int* slot_of, const float4* lbuild, const int* lhalo,
                                float4* lpos, float disp2, const DevGeom& g, float inv_unit,
                                float radius, int* flag, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    list_refresh_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, posd, tag, slot_of, lbuild, lhalo,
                                                         lpos, disp2, g.Lhi, g.Llo, g.L, inv_unit,
                                                         radius, flag);
    return cudaGetLastError();
}

// slot_of[tag[k]] = k: the slot of each original index in a sorted order
__global__ void __launch_bounds__(256)
invert_tags_kernel(int n, const int* tag, int* slot_of) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) slot_of[tag[k]] = k;
}

cudaError_t launch_invert_tags(int n, const int* tag, int* slot_of, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    invert_tags_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, tag, slot_of);
    return cudaGetLastError();
}

__global__ void step_end_kernel(StepState* state, const int* lflag, const uint32_t* err,
                                int vel_freq, cudaGraphConditionalHandle handle, int use_handle) {
    const int rebuild = (*err == 0 && *lflag != 0) ? 1 : 0;
    StepState s = *state;
    if (*err == 0) {
        // brownianIntegrator's velCounter bookkeeping (brownianIntegrator.cpp:291-292)
        // runs only after normal steps
        if (s.step > 0) s.vel_counter = (s.vel_counter == vel_freq) ? 0 : s.vel_counter + 1;
        s.step += 1;
        s.list_builds += rebuild;
        *state = s;
    }
    if (use_handle) cudaGraphSetConditional(handle, (unsigned int)rebuild);
}

cudaError_t launch_step_end(StepState* state, const int* lflag, const uint32_t* err,
                            int vel_freq, cudaGraphConditionalHandle handle, int use_handle,
                            cudaStream_t st) {
    step_end_kernel<<<1, 1, 0, st>>>(state, lflag, err, vel_freq, handle, use_handle);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) permute_kernel(PermuteArgs a, const uint32_t* err) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n || *err) return;
    const int o = a.perm[g];
    for (int k = 0; k < a.narr; ++k) a.dst[k][g] = a.src[k][o];
}

cudaError_t launch_permute(const PermuteArgs& a, const uint32_t* err, cudaStream_t st) {
    if (a.n == 0 || a.narr == 0) return cudaSuccess;
    permute_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a, err);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, float* sink) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    const float b = 0.999999f, c = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678f) sink[0] = s;  // keeps the chains live
}

cudaError_t launch_fma_probe(int blocks, int threads, int iters, float* sink, cudaStream_t st) {
    fma_probe_kernel<<<blocks, threads, 0, st>>>(iters, sink);
    return cudaGetLastError();
}

// Host-link probe: dst[i] = src[i] over n 16-byte words, four in flight per
// thread; either side may be host memory the device reads or writes in place.
__global__ void __launch_bounds__(256) link_copy_kernel(const uint4* __restrict__ src,
                                                        uint4* __restrict__ dst, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride],
                    d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

cudaError_t launch_link_copy(int blocks, const void* src, void* dst, size_t bytes,
                             cudaStream_t st) {
    link_copy_kernel<<<blocks, 256, 0, st>>>(static_cast<const uint4*>(src),
                                             static_cast<uint4*>(dst), bytes / 16);
    return cudaGetLastError();
}

}  // namespace psim
