// psim_exact.cu -- FP64 kernels, compiled with --fmad=false so every a*b+c
// rounds twice as in the reference's x86-64 build (no FMA contraction).
//
//   F64Body             plain form of the plugin force pass (the pair body of
//                       force_pass_kernel, psim_force.cuh)
//   vgb_system_kernel   brownianIntegrator::nextSystem fused with the gather
//                       into the new cell order and the cell hash + count of
//                       the next rebuild (brownianIntegrator.cpp:181-356,
//                       systemHandling.cpp:33-48)
//   vgb_aos_kernel      nextSystem on the reference's own AoS arrays
//   hash_count_kernel   system::hashParticles + the counting-sort histogram
#include <cmath>

#include "psim_body.cuh"
#include "psim_force.cuh"
#include "psim_force_cell.cuh"
#include "psim_vgb.cuh"

namespace psim {

// ------------------------------------------------------------------ forces


template <class Pair>
static cudaError_t run_fp64(const Pair& p, const DevGeom& g, const CellView& cv,
                            const ForceOut& out, float pre, cudaStream_t st, int tile,
                            const BatchView* bv) {
    F64Body<Pair> body{p, g};
    body.cont = out.coor ? out.cont : 0.0;   // updateInteractions fused into the pass
    if (tile && !bv) return launch_force_cells(body, g, cv, out, pre, st);
    return launch_force_pass(body, g, cv, out, pre, st, bv);
}

template <int N>
static cudaError_t run_lj_fp64(const LJPair& lj, const DevGeom& g, const CellView& cv,
                               const ForceOut& out, float pre, cudaStream_t st, int tile,
                               const BatchView* bv) {
    LJFixed<N> p;
    static_cast<LJPair&>(p) = lj;
    return run_fp64(p, g, cv, out, pre, st, tile, bv);
}

cudaError_t launch_forces_fp64(const ForceSetup& fs, const DevGeom& g, const CellView& cv,
                               const ForceOut& out, cudaStream_t st, const BatchView* bv) {
    const int t = fs.tile;
    const float pre = fs.pre_rc2f;
    switch (fs.kind) {
    case 1: return run_fp64(fs.ao, g, cv, out, pre, st, t, bv);
    case 2:
        switch (fs.lj.n) {
        case 0: return run_lj_fp64<0>(fs.lj, g, cv, out, pre, st, t, bv);
        case 6: return run_lj_fp64<6>(fs.lj, g, cv, out, pre, st, t, bv);
        case 12: return run_lj_fp64<12>(fs.lj, g, cv, out, pre, st, t, bv);
        case 18: return run_lj_fp64<18>(fs.lj, g, cv, out, pre, st, t, bv);
        default: return run_fp64(fs.lj, g, cv, out, pre, st, t, bv);
        }
    case 3: return run_fp64(fs.cal, g, cv, out, pre, st, t, bv);
    case 4: {
        if (bv) return cudaErrorInvalidValue;  // batches hold single-plugin replicas
        ComboPair cp{fs.ao, fs.lj, fs.ao.rc2 > fs.lj.rc2 ? fs.ao.rc2 : fs.lj.rc2};
        return run_fp64(cp, g, cv, out, pre, st, t, bv);
    }
    }
    return cudaErrorInvalidValue;
}

// -------------------------------------------------------------- integrator
// The update is psim_vgb.cuh; this translation unit is built without FMA
// contraction, so these instances round every product and sum separately,
// in the reference's order.

cudaError_t launch_vgb_system(const VgbSystemArgs& a, const VgbParams& p, const DevGeom& g,
                              const NoiseView& nz, cudaStream_t st) {
    return launch_vgb_system_t<VgbExact>(a, p, g, nz, st);
}

cudaError_t launch_vgb_aos(const VgbAosArgs& a, const VgbParams& p, double L, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    vgb_aos_kernel<VgbExact><<<(a.n + 255) / 256, 256, 0, st>>>(a, p, L);
    return cudaGetLastError();
}

cudaError_t launch_vgb_host(const VgbHostArgs& a, const VgbParams& p, double L, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    vgb_host_kernel<VgbExact><<<(a.n + kHostBlock - 1) / kHostBlock, kHostBlock, 0, st>>>(a, p, L);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ hashing

__global__ void __launch_bounds__(256)
hash_count_kernel(int n, const double* x, const double* y, const double* z, DevGeom g0,
                  int* key, int* rank, int* count, uint32_t* err_out, const int* rep,
                  const DevGeom* geoms) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    const double p[3] = {x[i], y[i], z[i]};
    const int k = hash_pos(p, rep ? geoms[rep[i]] : g0, err);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
    if (err) atomicOr(err_out, err);
}

cudaError_t launch_hash_count(int n, const double* x, const double* y, const double* z,
                              const DevGeom& g, int* key, int* rank, int* count, uint32_t* err,
                              cudaStream_t st, const int* rep, const DevGeom* geoms) {
    if (n == 0) return cudaSuccess;
    hash_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, x, y, z, g, key, rank, count, err, rep,
                                                       geoms);
    return cudaGetLastError();
}

}  // namespace psim
