// psim_mixed.cu -- the mixed-precision form of the plugin force pass.
//
// Pair forces are computed in FP32 and summed in FP32 with Kahan-compensated
// per-particle totals; the update, wrap and coefficients stay FP64 (in
// psim_exact.cu).  Positions are carried as FP32 pairs (hi + lo == the FP64
// position to ~1e-14), so a pair separation is
//     d = ((x_j,hi + s_hi) - x_i,hi) + ((x_j,lo + s_lo) - x_i,lo)
// with s = 0 or +-L (also a float pair) for a periodic image: the first
// bracket is exact when the image is applied (Sterbenz), and the rounding of
// d is then one FP32 rounding of a number of size <= rc, not of the box.
#include <cmath>

#include "psim_kernels.cuh"

namespace psim {

struct ComboPairF {
    AOPair ao;
    LJPair lj;
    float rc2f;
    __device__ __forceinline__ float fnet32(float r2, float r, float rinv, float size) const {
        float f = 0.0f;
        if (r2 < ao.rc2f) f += ao.fnet32(r2, r, rinv, size);
        if (r2 < lj.rc2f) f += lj.fnet32(r2, r, rinv, size);
        return f;
    }
};

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

template <class Pair>
__global__ void __launch_bounds__(128)
force_mixed_kernel(Pair pair, float rc2f, DevGeom g, CellView cv, ForceOut out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n || *out.err) return;
    const float4 hi = cv.posh[i];
    const float4 lo = cv.posl[i];
    const int c = cv.cellid[i];
    const int cx = c % g.s, cy = (c / g.s) % g.s, cz = c / g.s2;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, k0 = 0.f, k1 = 0.f, k2 = 0.f;
    uint32_t err = 0;
    for (int dx = -1; dx <= 1; ++dx) {
        int shx;
        const int x = wrap_cell(cx + dx, g.s, shx);
        const float sxh = (float)shx * g.Lhi, sxl = (float)shx * g.Llo;
        for (int dy = -1; dy <= 1; ++dy) {
            int shy;
            const int y = wrap_cell(cy + dy, g.s, shy);
            const float syh = (float)shy * g.Lhi, syl = (float)shy * g.Llo;
            for (int dz = -1; dz <= 1; ++dz) {
                int shz;
                const int z = wrap_cell(cz + dz, g.s, shz);
                const float szh = (float)shz * g.Lhi, szl = (float)shz * g.Llo;
                const int cell = x + g.s * y + g.s2 * z;
                const int start = cv.cstart[cell];
                const int end = start + cv.ccount[cell];
                float p0 = 0.f, p1 = 0.f, p2 = 0.f;
                for (int j = start; j < end; ++j) {
                    const float4 hj = __ldg(&cv.posh[j]);
                    const float4 lj = __ldg(&cv.posl[j]);
                    const float d0 = ((hj.x + sxh) - hi.x) + ((lj.x + sxl) - lo.x);
                    const float d1 = ((hj.y + syh) - hi.y) + ((lj.y + syl) - lo.y);
                    const float d2 = ((hj.z + szh) - hi.z) + ((lj.z + szl) - lo.z);
                    const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
                    if (r2 < rc2f && j != i) {
                        const float rinv = rsqrtf(r2);
                        const float r = r2 * rinv;
                        const float size = hi.w + hj.w;
                        if (r < 0.8f * size) err |= EBIT_OVERLAP;
                        const float f = pair.fnet32(r2, r, rinv, size) * rinv;
                        p0 += f * d0;
                        p1 += f * d1;
                        p2 += f * d2;
                    }
                }
                kahan_add(s0, k0, p0);
                kahan_add(s1, k1, p1);
                kahan_add(s2, k2, p2);
            }
        }
    }
    out.fx[i] = (double)s0 - (double)k0;
    out.fy[i] = (double)s1 - (double)k1;
    out.fz[i] = (double)s2 - (double)k2;
    if (err) atomicOr(out.err, err);
}

template <class Pair>
static cudaError_t run_mixed(const Pair& p, float rc2f, const DevGeom& g, const CellView& cv,
                             const ForceOut& out, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    const int bs = 128;
    force_mixed_kernel<Pair><<<(g.n + bs - 1) / bs, bs, 0, st>>>(p, rc2f, g, cv, out);
    return cudaGetLastError();
}

cudaError_t launch_forces_mixed(const ForceSetup& fs, const DevGeom& g, const CellView& cv,
                                const ForceOut& out, cudaStream_t st) {
    switch (fs.kind) {
    case 1: return run_mixed(fs.ao, fs.ao.rc2f, g, cv, out, st);
    case 2: return run_mixed(fs.lj, fs.lj.rc2f, g, cv, out, st);
    case 3: return run_mixed(fs.cal, fs.cal.rc2f, g, cv, out, st);
    case 4: {
        float rc2f = fs.ao.rc2f > fs.lj.rc2f ? fs.ao.rc2f : fs.lj.rc2f;
        ComboPairF cp{fs.ao, fs.lj, rc2f};
        return run_mixed(cp, rc2f, g, cv, out, st);
    }
    }
    return cudaErrorInvalidValue;
}

}  // namespace psim
