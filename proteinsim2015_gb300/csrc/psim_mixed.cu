// psim_mixed.cu -- the mixed-precision form of the plugin force pass.
//
// Pair forces are computed in FP32 and summed in FP32 with Kahan-compensated
// per-particle totals; the update, wrap and coefficients stay FP64 (in
// psim_exact.cu).  Positions are carried as FP32 pairs (hi + lo == the FP64
// position to ~1e-14).  For a row of cells the home position minus the
// row's periodic image (0 or +-L, L itself a float pair) is formed exactly
// as a float pair (h, l) by TwoSum, and a pair separation is
//     d = (x_j,hi - h) + (x_j,lo - l)
// where the first difference is exact for nearby values (Sterbenz), so d
// carries one FP32 rounding of a number of size <= rc, not of the box.
// The pair loop itself is force_pass_kernel (psim_force.cuh).
#include <algorithm>
#include <cmath>

#include "psim_body.cuh"
#include "psim_force.cuh"
#include "psim_force_cell.cuh"
#include "psim_force_list.cuh"
#include "psim_vgb.cuh"

namespace psim {

// The plugin's pair functor handed to run(pair, rc2f): LennardJones without
// a Yukawa term gets its exponent fixed at compile time for the common ljNum
// values 6, 12 and 18, the pure Yukawa form (ljNum 0) likewise; other
// LennardJones settings run the general functor.
template <class Run>
static cudaError_t with_pair(const ForceSetup& fs, Run&& run) {
    switch (fs.kind) {
    case 1: return run(fs.ao, fs.ao.rc2f);
    case 2: {
        auto fixed = [&](auto p) {
            static_cast<LJPair&>(p) = fs.lj;
            return run(p, fs.lj.rc2f);
        };
        if (fs.lj_pure) {
            switch (fs.lj.n) {
            case 6: return fixed(LJPure<6>{});
            case 12: return fixed(LJPure<12>{});
            case 18: return fixed(LJPure<18>{});
            }
        }
        if (fs.lj.n == 0) return fixed(LJFixed<0>{});
        return run(fs.lj, fs.lj.rc2f);
    }
    case 3: return run(fs.cal, fs.cal.rc2f);
    case 4: {
        const float rc2f = fs.ao.rc2f > fs.lj.rc2f ? fs.ao.rc2f : fs.lj.rc2f;
        return run(ComboPairF{fs.ao, fs.lj}, rc2f);
    }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_forces_mixed(const ForceSetup& fs, const DevGeom& g, const CellView& cv,
                                const ForceOut& out, cudaStream_t st, const BatchView* bv) {
    if (bv && fs.kind == 4) return cudaErrorInvalidValue;  // batches hold single-plugin replicas
    return with_pair(fs, [&](auto p, float rc2f) {
        MixedBody<decltype(p)> body{p, rc2f};
        body.cont2f = out.coor ? out.cont2f : 0.f;   // updateInteractions fused into the pass
        if (fs.tile && !bv) return launch_force_cells(body, g, cv, out, fs.pre_rc2f, st);
        return launch_force_pass(body, g, cv, out, fs.pre_rc2f, st, bv, fs.walk);
    });
}

cudaError_t launch_forces_list(const ForceSetup& fs, const DevGeom& g, const PairList& pl,
                               const ForceOut& out, cudaStream_t st) {
    return with_pair(fs, [&](auto p, float rc2f) {
        MixedBody<decltype(p)> body{p, rc2f};
        body.cont2f = out.coor ? out.cont2f : 0.f;
        return launch_force_list(body, g, pl, out, st);
    });
}

cudaError_t launch_list_build(const DevGeom& g, const CellView& cv, const ListBuild& lb,
                              uint32_t* err, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    // 32 blocks per SM of the current device (looked up per call: the
    // attribute query is a cached read in the runtime)
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const int blocks = 32 * sms;
    list_build_kernel<<<std::min(blocks, (g.n + 127) / 128), 128, 0, st>>>(g, cv, lb, err);
    return cudaGetLastError();
}

// The update of the mixed form: the same FP64 arithmetic as psim_exact.cu's
// instance, with a*b+c contracted into FMA by this translation unit.
cudaError_t launch_vgb_system_fast(const VgbSystemArgs& a, const VgbParams& p, const DevGeom& g,
                                   const NoiseView& nz, cudaStream_t st) {
    return launch_vgb_system_t<VgbFast>(a, p, g, nz, st);
}

}  // namespace psim
