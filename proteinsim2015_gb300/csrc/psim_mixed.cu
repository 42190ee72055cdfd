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

#include "psim_force.cuh"
#include "psim_force_cell.cuh"
#include "psim_force_list.cuh"
#include "psim_vgb.cuh"

namespace psim {

struct ComboPairF {
    AOPair ao;
    LJPair lj;
    __device__ __forceinline__ float fnet32(float r2, float r, float rinv, float size) const {
        float f = 0.0f;
        if (r2 < ao.rc2f) f += ao.fnet32(r2, r, rinv, size);
        if (r2 < lj.rc2f) f += lj.fnet32(r2, r, rinv, size);
        return f;
    }
};

// The FP32 cutoff of a pair functor (the larger one for the composite).
template <class P>
__device__ __forceinline__ float pair_rc2f(const P& p) { return p.rc2f; }
__device__ __forceinline__ float pair_rc2f(const ComboPairF& p) {
    return p.ao.rc2f > p.lj.rc2f ? p.ao.rc2f : p.lj.rc2f;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// One pair (i <- j) in FP32; each row's plain FP32 partial is added to the
// particle's total with Kahan compensation.
template <class Pair>
struct MixedBody {
    Pair pf;
    float rc2f;
    using Aux = float4;  // the low parts of the neighbour positions
    static constexpr bool kBatchable = !std::is_same<Pair, ComboPairF>::value;
    struct Home {
        float4 lo;
    };
    struct Shifted {     // home position minus the row's image, as a float pair
        float4 h;        // xyz: high part, w: radius
        float lx, ly, lz;
    };
    struct Acc {
        float s0, s1, s2, k0, k1, k2, p0, p1, p2;
    };
    __device__ __forceinline__ const Aux* aux(const CellView& cv) const { return cv.posl; }
    // the body of replica r of a batch: its own pair functor and cutoff
    __device__ __forceinline__ MixedBody for_replica(const void* pairs, int r,
                                                     const DevGeom&) const {
        MixedBody b = *this;
        b.pf = static_cast<const Pair*>(pairs)[r];
        b.rc2f = pair_rc2f(b.pf);
        return b;
    }
    __device__ __forceinline__ void init(Acc& a) const {
        a.s0 = a.s1 = a.s2 = a.k0 = a.k1 = a.k2 = a.p0 = a.p1 = a.p2 = 0.f;
    }
    __device__ __forceinline__ void load_home(const CellView& cv, int i, Home& h) const {
        h.lo = cv.posl[i];
    }
    __device__ __forceinline__ void shift(const Home& h, const float4& hi, int sx, int sy, int sz,
                                          const DevGeom& g, Shifted& o) const {
        float ex, ey, ez;
        two_sum(hi.x, -(float)sx * g.Lhi, o.h.x, ex);
        two_sum(hi.y, -(float)sy * g.Lhi, o.h.y, ey);
        two_sum(hi.z, -(float)sz * g.Lhi, o.h.z, ez);
        o.h.w = hi.w;
        o.lx = (ex + h.lo.x) - (float)sx * g.Llo;
        o.ly = (ey + h.lo.y) - (float)sy * g.Llo;
        o.lz = (ez + h.lo.z) - (float)sz * g.Llo;
    }
    __device__ __forceinline__ void eval(const float4& hj, const float4& lj, const Shifted& hs,
                                         Acc& a, uint32_t& err) const {
        const float d0 = (hj.x - hs.h.x) + (lj.x - hs.lx);
        const float d1 = (hj.y - hs.h.y) + (lj.y - hs.ly);
        const float d2 = (hj.z - hs.h.z) + (lj.z - hs.lz);
        const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
        if (r2 < rc2f) {
            const float rinv = rsqrtf(r2);
            const float r = r2 * rinv;
            const float size = hs.h.w + hj.w;
            if (r < 0.8f * size) err |= EBIT_OVERLAP;
            const float f = pf.fnet32(r2, r, rinv, size) * rinv;
            a.p0 += f * d0;
            a.p1 += f * d1;
            a.p2 += f * d2;
        }
    }
    // the pair-list pass: one entry at separation d (the float-pair difference
    // already formed), masked by the cutoff.  kUniform: every pair has the
    // contact diameter `size` (s2 = size^2), and the overlap test runs once
    // per particle on the smallest r^2 (rmin); otherwise per pair.
    template <bool kUniform>
    __device__ __forceinline__ void eval_list(float d0, float d1, float d2, float size, float s2,
                                              Acc& a, float& rmin, uint32_t& err) const {
        const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
        const bool in = r2 < rc2f;
        const float fr = list_fr32(pf, r2, size, s2);
        if (kUniform)
            rmin = fminf(rmin, r2);
        else if (in && r2 < 0.64f * s2)
            err |= EBIT_OVERLAP;
        const float f = in ? fr : 0.0f;
        a.p0 += f * d0;
        a.p1 += f * d1;
        a.p2 += f * d2;
    }
    // the overlap test of eval_list<true>: r < 0.8 size for an in-range pair
    __device__ __forceinline__ void list_overlap(float rmin, float s2, uint32_t& err) const {
        if (rmin < fminf(0.64f * s2, rc2f)) err |= EBIT_OVERLAP;
    }
    __device__ __forceinline__ void fold(Acc& a) const {
        kahan_add(a.s0, a.k0, a.p0);
        kahan_add(a.s1, a.k1, a.p1);
        kahan_add(a.s2, a.k2, a.p2);
        a.p0 = a.p1 = a.p2 = 0.f;
    }
    // a staged neighbour with its periodic image s L applied, exactly as a
    // float pair: (h + l) + s (Lhi + Llo)
    __device__ __forceinline__ void image(float4& h, float4& l, int sx, int sy, int sz,
                                          const DevGeom& g) const {
        image_shift(h, l, sx, sy, sz, g.Lhi, g.Llo);
    }
    // per-lane partial sums for the cross-lane reduction: 6 floats per lane
    __device__ __forceinline__ void partial(const Acc& a, double* red, int tid,
                                            int stride) const {
        float* f = reinterpret_cast<float*>(red);
        f[0 * stride + tid] = a.s0;
        f[1 * stride + tid] = a.s1;
        f[2 * stride + tid] = a.s2;
        f[3 * stride + tid] = a.k0;
        f[4 * stride + tid] = a.k1;
        f[5 * stride + tid] = a.k2;
    }
    // the k lanes of home h (slots h, h + nh, ...), Kahan-summed in lane order
    __device__ __forceinline__ void reduce_store(const ForceOut& out, int i, const double* red,
                                                 int stride, int h, int nh, int k) const {
        const float* f = reinterpret_cast<const float*>(red);
        float S0 = 0.f, S1 = 0.f, S2 = 0.f, C0 = 0.f, C1 = 0.f, C2 = 0.f;
        for (int q = 0; q < k; ++q) {
            const int t = q * nh + h;
            kahan_add(S0, C0, f[0 * stride + t]);
            kahan_add(S1, C1, f[1 * stride + t]);
            kahan_add(S2, C2, f[2 * stride + t]);
            kahan_add(S0, C0, -f[3 * stride + t]);
            kahan_add(S1, C1, -f[4 * stride + t]);
            kahan_add(S2, C2, -f[5 * stride + t]);
        }
        out.fx[i] = (double)S0 - (double)C0;
        out.fy[i] = (double)S1 - (double)C1;
        out.fz[i] = (double)S2 - (double)C2;
    }
    __device__ __forceinline__ void store(const ForceOut& out, int i, const Acc& a) const {
        out.fx[i] = (double)a.s0 - (double)a.k0;
        out.fy[i] = (double)a.s1 - (double)a.k1;
        out.fz[i] = (double)a.s2 - (double)a.k2;
    }
};

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
        const MixedBody<decltype(p)> body{p, rc2f};
        if (fs.tile && !bv) return launch_force_cells(body, g, cv, out, fs.pre_rc2f, st);
        return launch_force_pass(body, g, cv, out, fs.pre_rc2f, st, bv);
    });
}

cudaError_t launch_forces_list(const ForceSetup& fs, const DevGeom& g, const PairList& pl,
                               const ForceOut& out, cudaStream_t st) {
    return with_pair(fs, [&](auto p, float rc2f) {
        return launch_force_list(MixedBody<decltype(p)>{p, rc2f}, g, pl, out, st);
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
