// psim_body.cuh -- the per-pair bodies the force-pass templates
// (psim_force.cuh, psim_force_cell.cuh, psim_force_list.cuh) are
// instantiated with, one per precision form, each over a plugin's pair
// functor:
//   F64Body<Pair>    the plain FP64 form in the reference's operation order
//                    (a translation unit built with --fmad=false)
//   MixedBody<Pair>  FP32 pair terms, Kahan-compensated FP32 sums over
//                    float-pair positions
// Header-only, so that a force plugin compiles the same passes with its own
// functor (psim_plugin.cuh).
#pragma once

#include <type_traits>

#include "psim_force.cuh"

namespace psim {

struct ComboPair {  // AO + LJ(n) summed; each part inside its own cutoff
    AOPair ao;
    LJPair lj;
    double rc2;
    static constexpr bool kCheckNan = true;
    __host__ __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double size) const {
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
    // the reference's summation order and image rules: always the staged walk
    static constexpr bool kDirectWalk = false;
    struct Home {
        double4_32a p;
    };
    using Shifted = Home;     // the FP64 form takes raw differences
    struct Acc {
        double n0, n1, n2, c0, c1, c2;
        int cnt;
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
        a.cnt = 0;
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
        // updateInteractions' test: r = sqrt(pbcDist) < 1.2 (systemHandling.cpp:112-115)
        if (cont > 0.0 && sqrt(r2) < cont) ++a.cnt;
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
        if (out.coor) out.coor[i] = a.cnt;
    }
    DevGeom geom;
    double cont = 0.0;   // > 0: count the neighbours closer than cont (ForceOut::coor)
};

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
    float cont2f = 0.f;  // > 0: count the neighbours with r^2 < cont2f (ForceOut::coor)
    using Aux = float4;  // the low parts of the neighbour positions
    static constexpr bool kBatchable = !std::is_same<Pair, ComboPairF>::value;
    // the 27-cell walk that keeps its queues across rows (force_direct_kernel)
    static constexpr bool kDirectWalk = true;
    struct Home {
        float4 lo;
    };
    struct Shifted {     // home position minus the row's image, as a float pair
        float4 h;        // xyz: high part, w: radius
        float lx, ly, lz;
    };
    struct Acc {
        float s0, s1, s2, k0, k1, k2, p0, p1, p2;
        int cnt;
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
        a.cnt = 0;
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
        if (cont2f > 0.f && r2 < cont2f) ++a.cnt;
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
    // per particle on the smallest r^2 (rmin); otherwise per pair.  bias is
    // added to r^2: 0, or the compact ghost record's kGhostBias.
    template <bool kUniform, bool kCount = false>
    __device__ __forceinline__ void eval_list(float d0, float d1, float d2, float size, float s2,
                                              Acc& a, float& rmin, uint32_t& err,
                                              float bias = 0.f) const {
        const float r2 = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, bias)));
        if (kCount) a.cnt += r2 < cont2f ? 1 : 0;
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
    // the sums `own` of another lane of the same particle (mask: that
    // particle's lanes, src: the lane within its width-lane segment), added
    // into a with compensation; every lane of the mask calls it with its own
    // unmerged sums, and lane 0 keeps the result
    __device__ __forceinline__ void merge_lane(Acc& a, const Acc& own, unsigned mask, int src,
                                               int width) const {
        const float t[6] = {__shfl_sync(mask, own.s0, src, width),
                            __shfl_sync(mask, own.s1, src, width),
                            __shfl_sync(mask, own.s2, src, width),
                            __shfl_sync(mask, own.k0, src, width),
                            __shfl_sync(mask, own.k1, src, width),
                            __shfl_sync(mask, own.k2, src, width)};
        const int c = __shfl_sync(mask, own.cnt, src, width);
        kahan_add(a.s0, a.k0, t[0]);
        kahan_add(a.s1, a.k1, t[1]);
        kahan_add(a.s2, a.k2, t[2]);
        kahan_add(a.s0, a.k0, -t[3]);
        kahan_add(a.s1, a.k1, -t[4]);
        kahan_add(a.s2, a.k2, -t[5]);
        a.cnt += c;
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
        out.fx[i] = widen_f32(S0) - widen_f32(C0);
        out.fy[i] = widen_f32(S1) - widen_f32(C1);
        out.fz[i] = widen_f32(S2) - widen_f32(C2);
    }
    // the compensated sum s - k formed in FP64 (exact: both parts fit 48
    // bits); the floats are widened with integer operations, as the FP64
    // unit that would convert them runs at 1/64 of the FP32 rate on GB300
    __device__ __forceinline__ void store(const ForceOut& out, int i, const Acc& a) const {
        out.fx[i] = widen_f32(a.s0) - widen_f32(a.k0);
        out.fy[i] = widen_f32(a.s1) - widen_f32(a.k1);
        out.fz[i] = widen_f32(a.s2) - widen_f32(a.k2);
        if (out.coor) out.coor[i] = a.cnt;
    }
};

}  // namespace psim
