// psim_vgb.cuh -- the van Gunsteren-Berendsen update (brownianIntegrator.cpp:
// 181-356) with the periodic wrap (particle.cpp:61-99, utilities.cpp:26-50)
// and the cell hash of the next rebuild (systemHandling.cpp:33-48).
//
// Included by two translation units: psim_exact.cu (built with --fmad=false:
// the plain form, every product and sum rounded separately in the reference's
// order) and psim_mixed.cu (FMA contraction allowed: the update of the mixed
// form, still FP64).  The Tag template argument keeps the two instances apart.
//
// GB300 issues FP64 arithmetic at 1/64 of the FP32 rate, so only the update's
// own arithmetic is FP64: sign and range tests of the wrap read the IEEE bit
// patterns as integers (same order as the floating-point comparison for the
// values involved), the wrap's additions sit behind warp-uniform branches
// (almost no particle crosses the box in one step), and the cell hash is
// computed in FP32 unless the position lies within a guard band of a cell
// face (a few times the FP32 error of the hash), where the FP64 division of
// the reference decides.
#pragma once

#include <type_traits>

#include "psim_kernels.cuh"

namespace psim {

struct VgbExact {};
struct VgbFast {};

// v < 0 for a non-NaN double: sign bit set and not -0.0
__device__ __forceinline__ bool neg_d(double v) {
    const long long b = __double_as_longlong(v);
    return b < 0 && b != (long long)0x8000000000000000ull;
}
// v >= base for v >= +0 and base > 0 (a positive NaN counts as >= base)
__device__ __forceinline__ bool ge_pos_d(double v, double base) {
    return __double_as_longlong(v) >= __double_as_longlong(base);
}
// |d| > h for h > 0
__device__ __forceinline__ bool abs_gt_d(double d, double h) {
    return (__double_as_longlong(d) & 0x7fffffffffffffffll) > __double_as_longlong(h);
}

// One particle of nextSystem (see the file comment).  x/x0: current position
// and previous position; mx: memX/Y/Z in, new memX/Y/Z out; F/F0: pushed
// forces; v: velocity in/out; xi: 6 Gaussians in draw order.  Writes the
// wrapped new position xn and the re-imaged previous position x0n.
__device__ __forceinline__ void vgb_particle(const VgbParams& p, double L, double half_L,
                                             bool first, bool vel_step, const double x[3],
                                             const double x0[3], double mx[3], double mc[3],
                                             const double F[3], const double F0[3], double v[3],
                                             const double xi[6], double m, double xn[3],
                                             double x0n[3], uint32_t& err) {
    double nw[3];
    if (first) {  // firstStep, brownianIntegrator.cpp:191-223 (G&B eq. 2.26)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mc[k] = 0.0;
            mx[k] = xi[k];
            nw[k] = x[k] + (v[k] * p.coeff1 * p.dt) + (F[k] * p.coeff3 * p.dt * p.dt * m)
                    + (p.sig1 * mx[k]);
        }
    } else {      // normalStep, brownianIntegrator.cpp:225-296
        const double c1 = m * p.dt2 * p.coeff1;
        const double c2 = m * p.dt2 * p.coeff2;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mc[k] = p.sig2 * ((p.corr * mx[k]) + (p.dev * xi[k]));
            mx[k] = xi[3 + k];
            double t = (p.c0 * x[k]);
            t -= (p.coeff0 * x0[k]);
            t += (c1 * F[k]);
            t += (c2 * (F[k] - F0[k]));
            t += (p.sig1 * mx[k]) + (p.coeff0 * mc[k]);
            nw[k] = t;
        }
    }
    // safeMod (one +-L), then safeMod0 re-images the old position next to the
    // new one (particle::setX/Y/Z, particle.cpp:61-92)
    bool lo[3], hi[3];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = neg_d(nw[k]);
        hi[k] = !lo[k] && ge_pos_d(nw[k], L);
        any |= lo[k] | hi[k];
        xn[k] = nw[k];
    }
    if (__any_sync(__activemask(), any)) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (lo[k]) xn[k] = nw[k] + L;
            else if (hi[k]) xn[k] = nw[k] - L;
        }
    }
    bool far[3];
    any = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        far[k] = abs_gt_d(xn[k] - x[k], half_L);
        any |= far[k];
        x0n[k] = x[k];
    }
    if (__any_sync(__activemask(), any)) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (far[k]) x0n[k] = (xn[k] - x[k] < 0) ? x[k] - L : x[k] + L;
    }
    if (vel_step) {  // velocityStep, brownianIntegrator.cpp:298-356
        const double g2 = m * p.dt2 * p.goy2;
        const double g3 = m * p.dt3 * p.goy3;
        const double g4 = p.hn * p.dt_inv;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double d0 = x[k] - x0[k];
            double vv = (xn[k] - x0n[k]) + d0;  // the new position's wrap and re-image
            vv += (g2 * F[k]);
            vv -= (g3 * (F[k] - F0[k]));
            vv += (mc[k] - p.sig1 * mx[k]);
            vv *= g4;
            v[k] = vv;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        // the reference exits with 7703 when the wrapped value is outside
        // [0, L) (particle.cpp:67-69); a NaN coordinate is flagged too
        const bool inside = !neg_d(xn[k]) && !ge_pos_d(xn[k], L) && (xn[k] == xn[k]);
        if (!inside) err |= EBIT_BOUNDS;
    }
}

// normalStep of the mixed form (brownianIntegrator.cpp:225-296), written as
//   x_new = x + [coEff0 (x - x0) + dt^2 coEff1 F/m + dt^2 coEff2 (F - F0)/m + noise]
// (c0 = 1 + coEff0): the bracket -- a displacement of ~v dt -- is summed in
// FP32 from FP32 cuts of its terms (the random numbers are drawn in FP32) and
// added to the FP64 position once, so each step carries ~1e-10 of rounding
// on top of the FP64 form's, four orders of magnitude below the step's own
// noise.  GB300 runs FP64 at 1/64 of the FP32 rate: this leaves two FP64
// additions per axis.  The wrap is normalStep's; the previous position's
// re-image test runs in FP32 with a wide margin and falls back to FP64 near
// L/2.  xf: the 6 Gaussians.  A NaN in any input reaches the position and
// the bounds test.
__device__ __forceinline__ void vgb_normal_fast(const VgbParams& p, double L, double half_L,
                                                const double x[3], const double x0[3],
                                                double mx[3], const double F[3],
                                                const double F0[3], const float xf[6], double m,
                                                double xn[3], double x0n[3], uint32_t& err) {
    // explicit roundings (no contraction left to the compiler), so every
    // instance of this update -- one system or a batch -- rounds alike
    const float mf = f32_cut(m);
    const float c1 = __fmul_rn(mf, p.dt2c1f);
    const float c2 = __fmul_rn(mf, p.dt2c2f);
    double nw[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float mcf =
            __fmul_rn(p.sig2f, __fmaf_rn(p.corrf, f32_trunc(mx[k]), __fmul_rn(p.devf, xf[k])));
        const float noise = __fmaf_rn(p.sig1f, xf[3 + k], __fmul_rn(p.coeff0f, mcf));
        const float d = f32_cut(x[k] - x0[k]);
        const float fk = f32_cut(F[k]), f0k = f32_cut(F0[k]);
        const float step =
            __fmaf_rn(p.coeff0f, d, __fmaf_rn(c1, fk, __fmaf_rn(c2, __fsub_rn(fk, f0k), noise)));
        nw[k] = x[k] + widen_f32(step);
        mx[k] = widen_f32(xf[3 + k]);
    }
    bool lo[3], hi[3];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = neg_d(nw[k]);
        hi[k] = !lo[k] && ge_pos_d(nw[k], L);
        any |= lo[k] | hi[k];
        xn[k] = nw[k];
    }
    if (__any_sync(__activemask(), any)) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (lo[k]) xn[k] = nw[k] + L;
            else if (hi[k]) xn[k] = nw[k] - L;
        }
    }
    const float Lf = (float)L;   // a uniform value: converted once per thread
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float df = fabsf(f32_trunc(xn[k]) - f32_trunc(x[k]));
        bool far = df > 0.6f * Lf;
        if (df >= 0.4f * Lf && df <= 0.6f * Lf) far = abs_gt_d(xn[k] - x[k], half_L);
        x0n[k] = far ? ((xn[k] - x[k] < 0) ? x[k] - L : x[k] + L) : x[k];
        // [0, L) as normalStep requires; a NaN (either sign) fails one of the two
        const bool inside = !neg_d(xn[k]) && !ge_pos_d(xn[k], L);
        if (!inside) err |= EBIT_BOUNDS;
    }
}

// floor(x / cs) as the reference computes it (systemHandling.cpp:39-41).
__device__ __forceinline__ int cell_coord_fast(double x, const DevGeom& g) {
    const float q = f32_trunc(x) * g.inv_csf;
    const float f = floorf(q);
    const float fr = q - f;
    if (fr > g.hash_guard && fr < 1.0f - g.hash_guard) return (int)f;
    return cell_coord(x, g);
}

__device__ __forceinline__ int hash_pos(const double xn[3], const DevGeom& g, uint32_t& err) {
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int q = cell_coord_fast(xn[k], g);
        if (q < 0 || q >= g.s) {
            err |= EBIT_CELL;
            q = q < 0 ? 0 : g.s - 1;
        }
        c[k] = q;
    }
    return g.c0 + c[0] + g.s * c[1] + g.s2 * c[2];  // systemHandling.cpp:43 (+ the batch offset)
}

// tag: the particle's index in the injected buffer; ptag: its Philox key
__device__ __forceinline__ void load_noise(const NoiseView& nz, uint32_t seed, int n, int tag,
                                           int ptag, long long step, double xi[6],
                                           uint32_t& err) {
    if (nz.mode == 1) {
        const long long idx = step - nz.first;
        if (idx < 0 || idx >= nz.n_steps) {
            err |= EBIT_NOISE;
#pragma unroll
            for (int k = 0; k < 6; ++k) xi[k] = 0.0;
            return;
        }
        const double* b = nz.buf + ((size_t)idx * (size_t)n + (size_t)tag) * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) xi[k] = b[k];
    } else {
        philox_gaussians6(seed, (uint32_t)ptag, (uint32_t)step, xi);
    }
}

// The same draws as FP32 values (injected noise is cut to FP32).
__device__ __forceinline__ void load_noise_f(const NoiseView& nz, uint32_t seed, int n, int tag,
                                             int ptag, long long step, float xf[6],
                                             uint32_t& err) {
    if (nz.mode == 1) {
        const long long idx = step - nz.first;
        if (idx < 0 || idx >= nz.n_steps) {
            err |= EBIT_NOISE;
#pragma unroll
            for (int k = 0; k < 6; ++k) xf[k] = 0.f;
            return;
        }
        const double* b = nz.buf + ((size_t)idx * (size_t)n + (size_t)tag) * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) xf[k] = f32_trunc(b[k]);
    } else {
        philox_gaussians6f(seed, (uint32_t)ptag, (uint32_t)step, xf);
    }
}

// The system-order update: gathers the previous state through perm, writes
// the new state in the current cell order, and hashes + counts the new
// positions into the next grid.
// The new position in pair-list order: the periodic image nearest the
// position at the list build (|x - build| < L/2 picks it), as an exact float
// pair; raises the rebuild flag when it has moved more than sqrt(ldisp2).
// s, b, hal: the particle's list slot, its position at the build and its halo
// word, loaded before the update so that their latency overlaps it.
__device__ __forceinline__ void list_position(const VgbSystemArgs& a, int s, const float4& b,
                                              int hal, const double xn[3], const DevGeom& g) {
    const float bb[3] = {b.x, b.y, b.z};
    const float halff = 0.5f * g.Lhi;
    float h[3], l[3], d2 = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        split_f64(xn[k], h[k], l[k]);
        const float dk = h[k] - bb[k];
        if (dk > halff || dk < -halff)  // wrapped since the build: the other image
            split_f64(dk > 0.f ? xn[k] - g.L : xn[k] + g.L, h[k], l[k]);
        const float e = h[k] - bb[k];
        d2 += e * e;
    }
    const float4 hv = make_float4(h[0], h[1], h[2], b.w), lv = make_float4(l[0], l[1], l[2], 0.f);
    store_record(a.lpos, a.linv_unit, (size_t)s, hv, lv);
    if (hal & 63)  // the particle's periodic images in the halo records
        halo_write(a.lpos + (a.linv_unit != 0.f ? 1 : 2) * ((size_t)a.n + 1), a.linv_unit,
                   hal >> 6, (uint32_t)(hal & 63), hv, lv, g.Lhi, g.Llo);
    if (d2 > a.ldisp2) *a.lflag_set = 1;
}

// One particle of the system-order update (slot f), with its system's
// geometry g and parameters p.
template <class Tag>
__device__ __forceinline__ void vgb_system_one(const VgbSystemArgs& a, const VgbParams& p,
                                               const DevGeom& g, const NoiseView& nz, int f) {
    const long long step = a.state->step;
    const int vc = a.state->vel_counter;
    const bool first = (step == 0);
    const bool vel_step = !first && (p.vel_freq == 0 || vc == p.vel_freq);
    // the previous order's slot (no permutation: the order has not changed)
    const int o = a.perm ? a.perm[f] : f;
    const int tag = a.tag[f];
    const int ntag = tag - g.p0;   // the index within the replica keys its Philox noise
    const double m = a.inv_mass[f];
    uint32_t err = 0;
    const double x[3] = {a.x[o], a.y[o], a.z[o]};
    const double x0[3] = {a.x0[o], a.y0[o], a.z0[o]};
    double mx[3] = {a.mx[o], a.my[o], a.mz[o]};
    const double F[3] = {a.fx[f], a.fy[f], a.fz[f]};
    const double F0[3] = {a.gx[o], a.gy[o], a.gz[o]};
    int ls = 0, lhal = 0;
    float4 lb = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.lbuild) {
        // list slot: carried with the particle, or its storage slot when the
        // storage order is the list order
        ls = a.lslot ? __ldg(a.lslot + f) : f;
        lb = __ldg(a.lbuild + ls);
        lhal = __ldg(a.lhalo + ls);
    }
    double v[3] = {0.0, 0.0, 0.0};
    if (first || vel_step) {
        v[0] = a.vel[3 * (size_t)tag];
        v[1] = a.vel[3 * (size_t)tag + 1];
        v[2] = a.vel[3 * (size_t)tag + 2];
    }
    double xn[3], x0n[3];
    if (std::is_same<Tag, VgbFast>::value && !first && !vel_step) {
        float xf[6];
        load_noise_f(nz, p.seed, a.n, tag, ntag, step, xf, err);
        vgb_normal_fast(p, g.L, g.half, x, x0, mx, F, F0, xf, m, xn, x0n, err);
    } else {
        double xi[6], mc[3];
        load_noise(nz, p.seed, a.n, tag, ntag, step, xi, err);
        vgb_particle(p, g.L, g.half, first, vel_step, x, x0, mx, mc, F, F0, v, xi, m, xn, x0n, err);
    }
    a.ox[f] = xn[0]; a.oy[f] = xn[1]; a.oz[f] = xn[2];
    a.ox0[f] = x0n[0]; a.oy0[f] = x0n[1]; a.oz0[f] = x0n[2];
    a.omx[f] = mx[0]; a.omy[f] = mx[1]; a.omz[f] = mx[2];
    if (a.img) {
        // a wrap re-imaged the previous position by one box: count it
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (__double_as_longlong(x0n[k]) != __double_as_longlong(x[k]))
                a.img[3 * (size_t)tag + k] += (x0n[k] < x[k]) ? 1 : -1;
    }
    if (vel_step) {
        a.vel[3 * (size_t)tag] = v[0];
        a.vel[3 * (size_t)tag + 1] = v[1];
        a.vel[3 * (size_t)tag + 2] = v[2];
    }
    if (a.lbuild) list_position(a, ls, lb, lhal, xn, g);
    if (f == 0 && a.lflag_clear) {
        *a.lflag_clear = 0;
        *a.lhcount = 0;   // halo records are handed out afresh at the next build
    }
    if (a.count) {   // the next cell list (not when it is rebuilt only with the pair list)
        const int key = hash_pos(xn, g, err);
        a.key[f] = key;
        a.rank[f] = atomicAdd(&a.count[key], 1);
    }
    if (err) atomicOr(a.err, err);
}

// One system (the geometry is a kernel parameter) or, with kBatch, each
// particle's replica of a batch (its geometry and Philox seed from tables).
template <class Tag, bool kBatch>
__global__ void __launch_bounds__(256, 4)
vgb_system_kernel(VgbSystemArgs a, VgbParams p, DevGeom g0, NoiseView nz) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n || *a.err) return;
    if constexpr (kBatch) {
        const int r = a.rep[f];
        VgbParams pr = p;
        pr.seed = a.seeds[r];
        vgb_system_one<Tag>(a, pr, a.geoms[r], nz, f);
    } else {
        vgb_system_one<Tag>(a, p, g0, nz, f);
    }
}

template <class Tag>
cudaError_t launch_vgb_system_t(const VgbSystemArgs& a, const VgbParams& p, const DevGeom& g,
                                const NoiseView& nz, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    const int blocks = (a.n + 255) / 256;
    if (a.rep)
        vgb_system_kernel<Tag, true><<<blocks, 256, 0, st>>>(a, p, g, nz);
    else
        vgb_system_kernel<Tag, false><<<blocks, 256, 0, st>>>(a, p, g, nz);
    return cudaGetLastError();
}

// nextSystem on the reference's own AoS arrays in original order.
template <class Tag>
__global__ void __launch_bounds__(256) vgb_aos_kernel(VgbAosArgs a, VgbParams p, double L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    uint32_t err = 0;
    double x[3], x0[3], mx[3], F[3], F0[3], v[3], xi[6], mc[3], xn[3], x0n[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k] = a.pos[3 * (size_t)i + k];
        x0[k] = a.pos0[3 * (size_t)i + k];
        mx[k] = a.mem[3 * (size_t)i + k];
        F[k] = a.frc[3 * (size_t)i + k];
        F0[k] = a.frc0[3 * (size_t)i + k];
        v[k] = a.vel[3 * (size_t)i + k];
    }
    if (a.noise) {
#pragma unroll
        for (int k = 0; k < 6; ++k) xi[k] = a.noise[6 * (size_t)i + k];
    } else {
        philox_gaussians6(a.seed, (uint32_t)(a.offset + i), (uint32_t)a.philox_step, xi);
    }
    const double m = 1.0 / a.mass[i];
    vgb_particle(p, L, L / 2, a.first != 0, a.vel_step != 0, x, x0, mx, mc, F, F0, v, xi, m, xn,
                 x0n, err);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a.pos[3 * (size_t)i + k] = xn[k];
        a.pos0[3 * (size_t)i + k] = x0n[k];
        a.mem[3 * (size_t)i + k] = mx[k];
        a.mem_corr[3 * (size_t)i + k] = mc[k];
        if (a.vel_step) a.vel[3 * (size_t)i + k] = v[k];
    }
    if (err) atomicOr(a.err, err);
}

// nextSystem on the caller's host arrays in place.  A block of kHostBlock
// particles stages the AoS spans it reads (positions, previous positions, the
// two forces, velocities when the step reads them, injected noise) through
// shared memory, so that every host access is one coalesced run of doubles,
// updates its particles, and writes its spans back the same way.  The state
// of a particle is read before anything of it is written, so the in/out
// arrays may be the same (pos, pos0, vel) or overlap the push (F0 = frc).
constexpr int kHostBlock = 128;
template <class Tag>
__global__ void __launch_bounds__(kHostBlock) vgb_host_kernel(VgbHostArgs a, VgbParams p,
                                                               double L) {
    __shared__ double sx[3 * kHostBlock], sx0[3 * kHostBlock], sf[3 * kHostBlock],
        sf0[3 * kHostBlock], sv[3 * kHostBlock], sxi[6 * kHostBlock];
    const int b0 = blockIdx.x * kHostBlock;
    const int m = min(kHostBlock, a.n - b0);
    const int t = threadIdx.x;
    const size_t o3 = 3 * (size_t)b0;
    const bool read_vel = a.first || a.vel_step;
    for (int k = t; k < 3 * m; k += kHostBlock) {
        sx[k] = a.pos[o3 + k];
        sx0[k] = a.pos0[o3 + k];
        sf[k] = a.F[o3 + k];
        sf0[k] = a.F0[o3 + k];
        sv[k] = read_vel ? a.vel[o3 + k] : 0.0;
    }
    if (a.noise)
        for (int k = t; k < 6 * m; k += kHostBlock) sxi[k] = a.noise[6 * (size_t)b0 + k];
    __syncthreads();
    if (t < m) {
        const int i = b0 + t;
        uint32_t err = 0;
        double x[3], x0[3], mx[3], F[3], F0[3], v[3], xi[6], mc[3], xn[3], x0n[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            x[k] = sx[3 * t + k];
            x0[k] = sx0[3 * t + k];
            F[k] = sf[3 * t + k];
            F0[k] = sf0[3 * t + k];
            v[k] = sv[3 * t + k];
            mx[k] = a.mem[3 * (size_t)i + k];
        }
        if (a.noise) {
#pragma unroll
            for (int k = 0; k < 6; ++k) xi[k] = sxi[6 * t + k];
        } else {
            philox_gaussians6(a.seed, (uint32_t)i, (uint32_t)a.philox_step, xi);
        }
        const double minv = 1.0 / a.mass[i];
        vgb_particle(p, L, L / 2, a.first != 0, a.vel_step != 0, x, x0, mx, mc, F, F0, v, xi,
                     minv, xn, x0n, err);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sx[3 * t + k] = xn[k];
            sx0[3 * t + k] = x0n[k];
            sv[3 * t + k] = v[k];
            a.mem[3 * (size_t)i + k] = mx[k];
            a.mem_corr[3 * (size_t)i + k] = mc[k];
        }
        if (err) atomicOr(a.err, err);
    }
    __syncthreads();
    for (int k = t; k < 3 * m; k += kHostBlock) {
        a.pos[o3 + k] = sx[k];
        a.pos0[o3 + k] = sx0[k];
        if (a.vel_step) a.vel[o3 + k] = sv[k];
        if (a.frc_out) {
            a.frc0_out[o3 + k] = sf0[k];
            a.frc_out[o3 + k] = sf[k];
        }
    }
}

}  // namespace psim
