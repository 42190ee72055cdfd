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

#include "psim_force.cuh"
#include "psim_force_cell.cuh"
#include "psim_vgb.cuh"

namespace psim {

// ------------------------------------------------------------------ forces

struct ComboPair {  // AO + LJ(n) summed; each part inside its own cutoff
    AOPair ao;
    LJPair lj;
    double rc2;
    static constexpr bool kCheckNan = true;
    __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double size) const {
        double f = 0.0;
        if (r2 < ao.rc2) f += ao.fnet64(r2, r, rinv, size);
        if (r2 < lj.rc2) f += lj.fnet64(r2, r, rinv, size);
        return f;
    }
};

// Plain form of one pair (i <- j): the reference's own minimum-image rules,
// pbcDist's |dx| > L/2.0 for r^2 (utilities.cpp:79-104) and unitVectorAdv's
// |dx| > int(L)/2 for the unit vector (utilities.cpp:114-142), the overlap
// check (AOPotential.cpp:83-88) and, for AO, the NaN check (:105-109).
// Each row's partial sum is folded into the total, as the reference folds
// each cell's partial (AOPotential.cpp:165-167).
template <class Pair>
struct F64Body {
    Pair pf;
    using Aux = double4_32a;  // the FP64 neighbour positions {x, y, z, R}
    static constexpr bool kBatchable = !std::is_same<Pair, ComboPair>::value;
    struct Home {
        double4_32a p;
    };
    using Shifted = Home;     // the FP64 form takes raw differences
    struct Acc {
        double n0, n1, n2, c0, c1, c2;
    };
    __device__ __forceinline__ const Aux* aux(const CellView& cv) const { return cv.posd; }
    // the body of replica r of a batch: its own pair functor and box
    __device__ __forceinline__ F64Body for_replica(const void* pairs, int r,
                                                   const DevGeom& g) const {
        F64Body b = *this;
        b.pf = static_cast<const Pair*>(pairs)[r];
        b.geom = g;
        return b;
    }
    __device__ __forceinline__ void init(Acc& a) const {
        a.n0 = a.n1 = a.n2 = a.c0 = a.c1 = a.c2 = 0.0;
    }
    __device__ __forceinline__ void load_home(const CellView& cv, int i, Home& h) const {
        h.p = cv.posd[i];
    }
    __device__ __forceinline__ void shift(const Home& h, const float4&, int, int, int,
                                          const DevGeom&, Shifted& o) const {
        o = h;
    }
    __device__ __forceinline__ void eval(const float4&, const double4_32a& pj, const Home& h,
                                         Acc& a, uint32_t& err) const {
        const DevGeom& g = geom;
        double d0 = pj.x - h.p.x, d1 = pj.y - h.p.y, d2 = pj.z - h.p.z;
        double a0 = fabs(d0), a1 = fabs(d1), a2 = fabs(d2);
        if (a0 > g.half) a0 -= g.L;
        if (a1 > g.half) a1 -= g.L;
        if (a2 > g.half) a2 -= g.L;
        const double r2 = (a0 * a0) + (a1 * a1) + (a2 * a2);
        if (r2 < pf.rc2) {
            const double r = sqrt(r2);
            const double size = h.p.w + pj.w;
            if (r < 0.8 * size) err |= EBIT_OVERLAP;
            const double rinv = 1.0 / r;
            const double f = pf.fnet64(r2, r, rinv, size);
            if (Pair::kCheckNan && isnan(f)) err |= EBIT_NAN;
            if (fabs(d0) > g.half_uv) d0 = (d0 < 0) ? d0 + g.L : d0 - g.L;
            if (fabs(d1) > g.half_uv) d1 = (d1 < 0) ? d1 + g.L : d1 - g.L;
            if (fabs(d2) > g.half_uv) d2 = (d2 < 0) ? d2 + g.L : d2 - g.L;
            a.c0 += f * (d0 * rinv);
            a.c1 += f * (d1 * rinv);
            a.c2 += f * (d2 * rinv);
        }
    }
    __device__ __forceinline__ void fold(Acc& a) const {
        a.n0 += a.c0;
        a.n1 += a.c1;
        a.n2 += a.c2;
        a.c0 = a.c1 = a.c2 = 0.0;
    }
    // the FP64 form takes raw differences; only the FP32 test copy is imaged
    __device__ __forceinline__ void image(float4& h, double4_32a&, int sx, int sy, int sz,
                                          const DevGeom& g) const {
        h.x += (float)sx * g.Lhi;
        h.y += (float)sy * g.Lhi;
        h.z += (float)sz * g.Lhi;
    }
    __device__ __forceinline__ void partial(const Acc& a, double* red, int tid,
                                            int stride) const {
        red[0 * stride + tid] = a.n0;
        red[1 * stride + tid] = a.n1;
        red[2 * stride + tid] = a.n2;
    }
    __device__ __forceinline__ void reduce_store(const ForceOut& out, int i, const double* red,
                                                 int stride, int h, int nh, int k) const {
        double t0 = 0.0, t1 = 0.0, t2 = 0.0;
        for (int q = 0; q < k; ++q) {
            const int t = q * nh + h;
            t0 += red[0 * stride + t];
            t1 += red[1 * stride + t];
            t2 += red[2 * stride + t];
        }
        out.fx[i] = t0;
        out.fy[i] = t1;
        out.fz[i] = t2;
    }
    __device__ __forceinline__ void store(const ForceOut& out, int i, const Acc& a) const {
        out.fx[i] = a.n0;
        out.fy[i] = a.n1;
        out.fz[i] = a.n2;
    }
    DevGeom geom;
};

template <class Pair>
static cudaError_t run_fp64(const Pair& p, const DevGeom& g, const CellView& cv,
                            const ForceOut& out, float pre, cudaStream_t st, int tile,
                            const BatchView* bv) {
    if (tile && !bv) return launch_force_cells(F64Body<Pair>{p, g}, g, cv, out, pre, st);
    return launch_force_pass(F64Body<Pair>{p, g}, g, cv, out, pre, st, bv);
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
