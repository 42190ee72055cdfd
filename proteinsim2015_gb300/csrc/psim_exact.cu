// psim_exact.cu -- FP64 kernels, compiled with --fmad=false so every a*b+c
// rounds twice as in the reference's x86-64 build (no FMA contraction).
//
//   force_fp64_kernel   plain form of the plugin force pass
//                       (defaultForceManager.cpp:55-65 + <plugin>::iterCells)
//   vgb_system_kernel   brownianIntegrator::nextSystem fused with the gather
//                       into the new cell order and the cell hash + count of
//                       the next rebuild (brownianIntegrator.cpp:181-356,
//                       systemHandling.cpp:33-48)
//   vgb_aos_kernel      nextSystem on the reference's own AoS arrays
//   hash_count_kernel   system::hashParticles + the counting-sort histogram
#include <cmath>

#include "psim_kernels.cuh"

namespace psim {

// ------------------------------------------------------------------ forces

struct ComboPair {  // AO + LJ(n) summed; each part inside its own cutoff
    AOPair ao;
    LJPair lj;
    double rc2;
    float rc2f;
    static constexpr bool kCheckNan = true;
    __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double size) const {
        double f = 0.0;
        if (r2 < ao.rc2) f += ao.fnet64(r2, r, rinv, size);
        if (r2 < lj.rc2) f += lj.fnet64(r2, r, rinv, size);
        return f;
    }
};

// One thread per sorted particle.  The 27 neighbour cells are visited in the
// reference's order (x outer, y, z inner; AOPotential.cpp:147-170) and each
// cell's partial sum is added to the total, as iterCells returns it.  An FP32
// test on the rounded positions (with a margin that covers their rounding)
// discards pairs that are certainly beyond the cutoff; every surviving pair
// is decided and evaluated in FP64 with the reference's own minimum-image
// rules: pbcDist's |dx| > L/2.0 for r^2 (utilities.cpp:79-104) and
// unitVectorAdv's |dx| > int(L)/2 for the unit vector (utilities.cpp:114-142).
template <class Pair>
__global__ void __launch_bounds__(128)
force_fp64_kernel(Pair pair, DevGeom g, CellView cv, ForceOut out, float pre_rc2f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n || *out.err) return;
    const double4_32a pi = cv.posd[i];
    const float4 hi = cv.posh[i];
    const int c = cv.cellid[i];
    const int cx = c % g.s, cy = (c / g.s) % g.s, cz = c / g.s2;
    double n0 = 0.0, n1 = 0.0, n2 = 0.0;
    uint32_t err = 0;
    for (int dx = -1; dx <= 1; ++dx) {
        int shx;
        const int x = wrap_cell(cx + dx, g.s, shx);
        const float sx = (float)shx * g.Lhi;
        for (int dy = -1; dy <= 1; ++dy) {
            int shy;
            const int y = wrap_cell(cy + dy, g.s, shy);
            const float sy = (float)shy * g.Lhi;
            for (int dz = -1; dz <= 1; ++dz) {
                int shz;
                const int z = wrap_cell(cz + dz, g.s, shz);
                const float sz = (float)shz * g.Lhi;
                const int cell = x + g.s * y + g.s2 * z;
                const int start = cv.cstart[cell];
                const int end = start + cv.ccount[cell];
                double c0 = 0.0, c1 = 0.0, c2 = 0.0;
                for (int j = start; j < end; ++j) {
                    if (j == i) continue;
                    const float4 hj = __ldg(&cv.posh[j]);
                    const float ex = (hj.x + sx) - hi.x;
                    const float ey = (hj.y + sy) - hi.y;
                    const float ez = (hj.z + sz) - hi.z;
                    const float r2f = ex * ex + ey * ey + ez * ez;
                    if (!(r2f < pre_rc2f)) continue;
                    const double4_32a pj = cv.posd[j];
                    double d0 = pj.x - pi.x, d1 = pj.y - pi.y, d2 = pj.z - pi.z;
                    double a0 = fabs(d0), a1 = fabs(d1), a2 = fabs(d2);
                    if (a0 > g.half) a0 -= g.L;
                    if (a1 > g.half) a1 -= g.L;
                    if (a2 > g.half) a2 -= g.L;
                    const double r2 = (a0 * a0) + (a1 * a1) + (a2 * a2);
                    if (r2 < pair.rc2) {
                        const double r = sqrt(r2);
                        const double size = pi.w + pj.w;
                        if (r < 0.8 * size) err |= EBIT_OVERLAP;
                        const double rinv = 1.0 / r;
                        const double f = pair.fnet64(r2, r, rinv, size);
                        if (Pair::kCheckNan && isnan(f)) err |= EBIT_NAN;
                        if (fabs(d0) > g.half_uv) d0 = (d0 < 0) ? d0 + g.L : d0 - g.L;
                        if (fabs(d1) > g.half_uv) d1 = (d1 < 0) ? d1 + g.L : d1 - g.L;
                        if (fabs(d2) > g.half_uv) d2 = (d2 < 0) ? d2 + g.L : d2 - g.L;
                        c0 += f * (d0 * rinv);
                        c1 += f * (d1 * rinv);
                        c2 += f * (d2 * rinv);
                    }
                }
                n0 += c0;
                n1 += c1;
                n2 += c2;
            }
        }
    }
    out.fx[i] = n0;
    out.fy[i] = n1;
    out.fz[i] = n2;
    if (err) atomicOr(out.err, err);
}

template <class Pair>
static cudaError_t run_fp64(const Pair& p, const DevGeom& g, const CellView& cv,
                            const ForceOut& out, float pre, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    const int bs = 128;
    force_fp64_kernel<Pair><<<(g.n + bs - 1) / bs, bs, 0, st>>>(p, g, cv, out, pre);
    return cudaGetLastError();
}

cudaError_t launch_forces_fp64(const ForceSetup& fs, const DevGeom& g, const CellView& cv,
                               const ForceOut& out, cudaStream_t st) {
    switch (fs.kind) {
    case 1: return run_fp64(fs.ao, g, cv, out, fs.pre_rc2f, st);
    case 2: return run_fp64(fs.lj, g, cv, out, fs.pre_rc2f, st);
    case 3: return run_fp64(fs.cal, g, cv, out, fs.pre_rc2f, st);
    case 4: {
        ComboPair cp{fs.ao, fs.lj, fs.ao.rc2 > fs.lj.rc2 ? fs.ao.rc2 : fs.lj.rc2, 0.f};
        return run_fp64(cp, g, cv, out, fs.pre_rc2f, st);
    }
    }
    return cudaErrorInvalidValue;
}

// -------------------------------------------------------------- integrator

__device__ __forceinline__ double safe_mod(double v, double base) {  // utilities.cpp:26-39
    if (v < 0) return v + base;
    if (v >= base) return v - base;
    return v;
}
__device__ __forceinline__ double safe_mod0(double v0, double v, double base) {  // :41-50
    double d = v - v0;
    return (fabs(d) > (base / 2)) ? ((d < 0) ? v0 - base : v0 + base) : v0;
}

// One particle of nextSystem.  x/x0: current position and previous position;
// mx: memX/Y/Z in, new memX/Y/Z out; F/F0: pushed forces; v: velocity in/out;
// xi: 6 Gaussians in draw order.  Writes the wrapped new position xn and the
// re-imaged previous position x0n (particle::setPos, particle.cpp:61-99).
__device__ __forceinline__ void vgb_particle(const VgbParams& p, double L, bool first,
                                             bool vel_step, const double x[3],
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
        if (vel_step) {  // velocityStep, brownianIntegrator.cpp:298-356
            const double g2 = m * p.dt2 * p.goy2;
            const double g3 = m * p.dt3 * p.goy3;
            const double g4 = p.hn * p.dt_inv;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double d0 = x[k] - x0[k];
                const double xw = safe_mod(nw[k], L);
                const double xo = safe_mod0(x[k], xw, L);
                double vv = (xw - xo) + d0;
                vv += (g2 * F[k]);
                vv -= (g3 * (F[k] - F0[k]));
                vv += (mc[k] - p.sig1 * mx[k]);
                vv *= g4;
                v[k] = vv;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // particle::setX/Y/Z
        xn[k] = safe_mod(nw[k], L);
        x0n[k] = safe_mod0(x[k], xn[k], L);
        // the reference exits with 7703 when the wrapped value is outside
        // [0, L); a NaN coordinate is flagged here too
        if (!(xn[k] >= 0.0 && xn[k] < L)) err |= EBIT_BOUNDS;
    }
}

__device__ __forceinline__ int hash_pos(const double xn[3], const DevGeom& g, uint32_t& err) {
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int q = cell_coord(xn[k], g);
        if (q < 0 || q >= g.s) {
            err |= EBIT_CELL;
            q = q < 0 ? 0 : g.s - 1;
        }
        c[k] = q;
    }
    return c[0] + g.s * c[1] + g.s2 * c[2];  // systemHandling.cpp:43
}

__device__ __forceinline__ void load_noise(const NoiseView& nz, uint32_t seed, int n, int tag,
                                           long long step, double xi[6], uint32_t& err) {
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
        philox_gaussians6(seed, (uint32_t)tag, (uint32_t)step, xi);
    }
}

__global__ void __launch_bounds__(256)
vgb_system_kernel(VgbSystemArgs a, VgbParams p, DevGeom g, NoiseView nz) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n || *a.err) return;
    const long long step = a.state->step;
    const int vc = a.state->vel_counter;
    const bool first = (step == 0);
    const bool vel_step = !first && (p.vel_freq == 0 || vc == p.vel_freq);
    const int o = a.perm[f];
    const int tag = a.tag[f];
    const double m = a.inv_mass[f];
    uint32_t err = 0;
    double x[3] = {a.x[o], a.y[o], a.z[o]};
    double x0[3] = {a.x0[o], a.y0[o], a.z0[o]};
    double mx[3] = {a.mx[o], a.my[o], a.mz[o]};
    const double F[3] = {a.fx[f], a.fy[f], a.fz[f]};
    const double F0[3] = {a.gx[o], a.gy[o], a.gz[o]};
    double v[3] = {0.0, 0.0, 0.0};
    if (first || vel_step) {
        v[0] = a.vel[3 * (size_t)tag];
        v[1] = a.vel[3 * (size_t)tag + 1];
        v[2] = a.vel[3 * (size_t)tag + 2];
    }
    double xi[6];
    load_noise(nz, p.seed, a.n, tag, step, xi, err);
    double mc[3], xn[3], x0n[3];
    vgb_particle(p, g.L, first, vel_step, x, x0, mx, mc, F, F0, v, xi, m, xn, x0n, err);
    a.ox[f] = xn[0]; a.oy[f] = xn[1]; a.oz[f] = xn[2];
    a.ox0[f] = x0n[0]; a.oy0[f] = x0n[1]; a.oz0[f] = x0n[2];
    a.omx[f] = mx[0]; a.omy[f] = mx[1]; a.omz[f] = mx[2];
    if (vel_step) {
        a.vel[3 * (size_t)tag] = v[0];
        a.vel[3 * (size_t)tag + 1] = v[1];
        a.vel[3 * (size_t)tag + 2] = v[2];
    }
    const int key = hash_pos(xn, g, err);
    a.key[f] = key;
    a.rank[f] = atomicAdd(&a.count[key], 1);
    if (err) atomicOr(a.err, err);
}

cudaError_t launch_vgb_system(const VgbSystemArgs& a, const VgbParams& p, const DevGeom& g,
                              const NoiseView& nz, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    vgb_system_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a, p, g, nz);
    return cudaGetLastError();
}

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
        philox_gaussians6(a.seed, (uint32_t)i, (uint32_t)a.philox_step, xi);
    }
    const double m = 1.0 / a.mass[i];
    vgb_particle(p, L, a.first != 0, a.vel_step != 0, x, x0, mx, mc, F, F0, v, xi, m, xn, x0n,
                 err);
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

cudaError_t launch_vgb_aos(const VgbAosArgs& a, const VgbParams& p, double L, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    vgb_aos_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a, p, L);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ hashing

__global__ void __launch_bounds__(256)
hash_count_kernel(int n, const double* x, const double* y, const double* z, DevGeom g,
                  int* key, int* rank, int* count, uint32_t* err_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    const double p[3] = {x[i], y[i], z[i]};
    const int k = hash_pos(p, g, err);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
    if (err) atomicOr(err_out, err);
}

cudaError_t launch_hash_count(int n, const double* x, const double* y, const double* z,
                              const DevGeom& g, int* key, int* rank, int* count, uint32_t* err,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    hash_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, x, y, z, g, key, rank, count, err);
    return cudaGetLastError();
}

}  // namespace psim
