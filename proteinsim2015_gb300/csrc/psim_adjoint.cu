// psim_adjoint.cu -- gradients of a trajectory loss through the vGB step.
//
// The loss of the differentiable-trajectory workload is the squared distance
// between the time-averaged, Gaussian-smoothed g(r) of a trajectory and a
// target; its gradient with respect to the plugin parameters (and the
// initial positions) is taken with the noise held fixed, by an adjoint
// (reverse-time) recursion through the positions-only form of the vGB
// normal step (brownianIntegrator.cpp:225-296):
//
//   x_1     = x_0 + c_v v_0 + c_f F(x_0) + N_0                    (firstStep)
//   x_{t+1} = c0 x_t - a0 x_{t-1} + b1 F(x_t) - b2 F(x_{t-1}) + N_t
//
// with c0 = 1 + coEff0, a0 = coEff0, b1 = dt^2 (coEff1 + coEff2) / m,
// b2 = dt^2 coEff2 / m, c_v = coEff1 dt, c_f = coEff3 dt^2 / m, and N_t the
// noise terms (Philox-keyed by particle and step, as the system's).  Writing
// u_t = b1 lam_{t+1} - b2 lam_{t+2} (u_0 = c_f lam_1 - b2 lam_2) and J the
// force Jacobian (symmetric: F is minus a potential gradient),
//
//   lam_t  = dL/dx_t + c0 lam_{t+1} - a0 lam_{t+2} + J(x_t) u_t   (lam_0: 1, -a0)
//   dL/dth = sum_t u_t . dF/dth (x_t)
//
// Each reverse step is one fused pair pass (J u, dF/dth . u and the loss's
// position gradient) over a cell list of x_t.  The forward pass keeps a
// checkpoint (x_t, x_{t-1}, F(x_{t-1})) every K steps; the reverse pass
// recomputes each K-step segment from its checkpoint, so memory is
// (T/K + K) positions and the cost two forward passes plus the reverse.
//
// All arithmetic is FP64 and the forward matches the system's plain form
// (same coefficients and Philox draws) up to rounding.  The pair force is the
// AO plugin (AOPotential.cpp:50-130), the Yukawa term of the LennardJones
// plugin with ljNum = 0 and the plugin's LJ(n) term (LJPotential.cpp:96-109),
// each inside its own cutoff; parameters th = (c1, c2, Y, lambda, eps,
// sigma): the AO coefficients, the Yukawa amplitude kT wellDepth
// yukawaStrength and its length, and the LJ energy kT wellDepth and contact
// diameter (the plugin's size, L = (sigma/r)^n).  The cutoffs are fixed: a
// pair crossing a cutoff changes the force by a step, which no derivative of
// the smooth part carries.
#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/psim_gb300.h"
#include "psim_kernels.cuh"

namespace psim {
namespace {

constexpr int kAdjTh = 6;    // parameters: c1, c2, Y, lambda, eps, sigma

struct AdjPair {
    double c1, c2, ao_rc2;   // ao_rc2 = 0: no AO term
    double Y, lam, y_rc2;    // y_rc2 = 0: no Yukawa term
    double inv_lam;          // 1 / lam
    double eps, sig, lj_rc2; // lj_rc2 = 0: no LJ(n) term
    int ljn;
};

// s(r) = F_pair / r (force on i along x_j - x_i), ds/dr and ds/dth
__device__ __forceinline__ void pair_terms(const AdjPair& q, double r2, double& s, double& ds,
                                           double dth[kAdjTh]) {
    const double ri = rsqrt(r2), r = r2 * ri;
    s = 0.0;
    ds = 0.0;
    for (int k = 0; k < kAdjTh; ++k) dth[k] = 0.0;
    const double ri2 = ri * ri, ri3 = ri2 * ri;
    if (r2 < q.ao_rc2) {
        const double ri4 = ri2 * ri2, ri8 = ri4 * ri4, ri16 = ri8 * ri8, ri32 = ri16 * ri16;
        const double ri39 = ri32 * ri4 * ri3;
        s += -(36.0 * ri39 + q.c1 * ri2 + q.c2);
        ds += 36.0 * 39.0 * ri39 * ri + 2.0 * q.c1 * ri3;
        dth[0] = -ri2;
        dth[1] = -1.0;
    }
    if (r2 < q.y_rc2) {
        const double e = exp(-r * q.inv_lam);
        const double lr = q.lam + r;
        s += -q.Y * e * lr * ri3;
        ds += q.Y * e * ri3 * (r * q.inv_lam + 3.0 * lr * ri);
        dth[2] = -e * lr * ri3;
        dth[3] = -q.Y * e * ri3 * (r * lr * q.inv_lam * q.inv_lam + 1.0);
    }
    if (r2 < q.lj_rc2) {
        // fNet = -eps (2L - 1) 4n L / r, L = (sigma / r)^n: s = -4n eps (2L - 1) L / r^2,
        // ds/dr = 4n eps L (n (4L - 1) + 2 (2L - 1)) / r^3,
        // ds/dsigma = -4n^2 eps (4L - 1) L / (sigma r^2)
        const double n = (double)q.ljn;
        const double L = powi_binary(q.sig * ri, q.ljn);
        const double base = -4.0 * n * (2.0 * L - 1.0) * L * ri2;
        s += q.eps * base;
        ds += 4.0 * n * q.eps * L * (n * (4.0 * L - 1.0) + 2.0 * (2.0 * L - 1.0)) * ri3;
        dth[4] = base;
        dth[5] = -4.0 * n * n * q.eps * (4.0 * L - 1.0) * L * ri2 / q.sig;
    }
}

struct AdjGrid {
    double L, inv_cs;
    int s, s2, ncell;
};

__device__ __forceinline__ double wrap_box(double x, double L) { return x - L * floor(x / L); }

__device__ __forceinline__ int cell_of(double xw, const AdjGrid& g) {
    int c = (int)(xw * g.inv_cs);
    return c < 0 ? 0 : (c >= g.s ? g.s - 1 : c);
}

__global__ void __launch_bounds__(256) adj_hash_kernel(int n, const double* x, AdjGrid g, int* key,
                                                       int* rank, int* count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = wrap_box(x[i], g.L), b = wrap_box(x[n + i], g.L), c = wrap_box(x[2 * n + i], g.L);
    const int k = cell_of(a, g) + g.s * cell_of(b, g) + g.s2 * cell_of(c, g);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

// sorted positions, wrapped into the box: FP64 and an FP32 copy for the
// candidate test
__global__ void __launch_bounds__(256) adj_place_kernel(int n, const double* x, const int* key,
                                                        const int* rank, const int* start,
                                                        int* order, double4_32a* sp, float4* spf,
                                                        double L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = start[key[i]] + rank[i];
    order[p] = i;
    const double a = wrap_box(x[i], L), b = wrap_box(x[n + i], L), c = wrap_box(x[2 * n + i], L);
    sp[p] = make_double4_32a(a, b, c, 0.0);
    spf[p] = make_float4((float)a, (float)b, (float)c, 0.f);
}

struct AdjWalk {
    AdjGrid g;
    AdjPair q;
    int n;
    const int* order;
    const double4_32a* sp;   // sorted positions, wrapped
    const float4* spf;       // the same in FP32
    const int* start;
    const int* count;
    const int* key;
};

// minimum image of a difference of two wrapped coordinates
template <class T>
__device__ __forceinline__ T min_image(T d, T L, T half) {
    return d > half ? d - L : (d < -half ? d + L : d);
}

// every neighbour j of sorted slot p within the largest cutoff: fn(j, d, r2).
// Candidates are tested in FP32 with a margin first; FP64 decides.
template <class Fn>
__device__ __forceinline__ void for_pairs(const AdjWalk& w, int p, const double4_32a& pi,
                                          double rc2, Fn&& fn) {
    const int c = w.key[w.order[p]];
    const int cx = c % w.g.s, cy = (c / w.g.s) % w.g.s, cz = c / w.g.s2;
    const double L = w.g.L, half = 0.5 * L;
    const float Lf = (float)L, hf = 0.5f * Lf;
    const float4 pf = w.spf[p];
    const float rcf = (float)sqrt(rc2) + 1e-3f + 4e-6f * Lf;
    const float pre = rcf * rcf;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                int sh;
                const int cell = wrap_cell(cx + dx, w.g.s, sh) + w.g.s * wrap_cell(cy + dy, w.g.s, sh) +
                                 w.g.s2 * wrap_cell(cz + dz, w.g.s, sh);
                const int st = w.start[cell], en = st + w.count[cell];
                for (int q = st; q < en; ++q) {
                    if (q == p) continue;
                    const float4 qf = w.spf[q];
                    const float ex = min_image(qf.x - pf.x, Lf, hf), ey = min_image(qf.y - pf.y, Lf, hf),
                                ez = min_image(qf.z - pf.z, Lf, hf);
                    if (ex * ex + ey * ey + ez * ez >= pre) continue;
                    const double4_32a pj = w.sp[q];
                    const double d[3] = {min_image(pj.x - pi.x, L, half), min_image(pj.y - pi.y, L, half),
                                         min_image(pj.z - pi.z, L, half)};
                    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    if (r2 < rc2) fn(q, d, r2);
                }
            }
}

__global__ void __launch_bounds__(128) adj_force_kernel(AdjWalk w, double rc2, double* F) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.n) return;
    const double4_32a pi = w.sp[p];
    double f[3] = {0.0, 0.0, 0.0};
    for_pairs(w, p, pi, rc2, [&](int, const double* d, double r2) {
        double s, ds, dth[kAdjTh];
        pair_terms(w.q, r2, s, ds, dth);
        for (int k = 0; k < 3; ++k) f[k] += s * d[k];
    });
    const int i = w.order[p];
    for (int k = 0; k < 3; ++k) F[(size_t)k * w.n + i] = f[k];
}

// smoothed g(r): Gaussian kernels at the bin centres, summed over ordered pairs
struct AdjHist {
    double r_min, dr, inv_sig, norm;   // norm: 1 / (sqrt(2 pi) sigma)
    int n_bins, reach;                 // bins within reach of a distance contribute
};

__device__ __forceinline__ double gauss(double z, double norm) { return norm * exp(-0.5 * z * z); }

// The kernel values G_b = norm exp(-z_b^2 / 2) of distance r at the bins
// b_lo..b_hi, z_b = (r - r_b) / sigma, by the recurrence of consecutive bins
// (z_{b+1} = z_b - dz): G_{b+1} = G_b q_b, q_{b+1} = q_b e^{-dz^2},
// q_b = e^{dz z_b - dz^2 / 2} -- two exponentials per distance.  fn(b, z, G).
template <class Fn>
__device__ __forceinline__ void gauss_bins(const AdjHist& h, double r, Fn&& fn) {
    const int b0 = (int)floor((r - h.r_min) / h.dr);
    const int lo = max(0, b0 - h.reach), hi = min(h.n_bins - 1, b0 + h.reach);
    if (lo > hi) return;
    const double dz = h.dr * h.inv_sig;
    double z = (r - (h.r_min + (lo + 0.5) * h.dr)) * h.inv_sig;
    double G = gauss(z, h.norm);
    double q = exp(dz * z - 0.5 * dz * dz);
    const double qq = exp(-dz * dz);
    for (int b = lo; b <= hi; ++b) {
        fn(b, z, G);
        G *= q;
        q *= qq;
        z -= dz;
    }
}

__global__ void __launch_bounds__(128) adj_hist_kernel(AdjWalk w, double rc2, AdjHist h,
                                                       double* hist) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.n) return;
    const double4_32a pi = w.sp[p];
    for_pairs(w, p, pi, rc2, [&](int, const double*, double r2) {
        gauss_bins(h, sqrt(r2), [&](int b, double, double G) { atomicAdd(&hist[b], h.dr * G); });
    });
}

struct AdjReverse {
    const double* u;      // u_t, 3n original order
    const double* lam1;   // lam_{t+1}
    const double* lam2;   // lam_{t+2}
    double* lam0;         // lam_t (out)
    double* u_prev;       // u_{t-1} (out)
    double c_self1, c_self2;   // lam_t = g + c_self1 lam1 + c_self2 lam2 + J u
    double cu0, cu1;           // u_{t-1} = cu0 lam_t + cu1 lam1
    const double* wgt;    // per bin: dL/d(smoothed count) of this step, or null
    AdjHist h;
    double* part;         // per block: kAdjTh parameter partials
};

__global__ void __launch_bounds__(128) adj_reverse_kernel(AdjWalk w, double rc2, AdjReverse a) {
    __shared__ double red[kAdjTh][128];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double th[kAdjTh] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (p < w.n) {
        const int i = w.order[p];
        const int n = w.n;
        const double4_32a pi = w.sp[p];
        const double ui[3] = {a.u[i], a.u[n + i], a.u[2 * (size_t)n + i]};
        double ju[3] = {0.0, 0.0, 0.0}, gl[3] = {0.0, 0.0, 0.0};
        for_pairs(w, p, pi, rc2, [&](int q, const double* d, double r2) {
            const int j = w.order[q];
            double s, ds, dth[kAdjTh];
            pair_terms(w.q, r2, s, ds, dth);
            const double r = sqrt(r2);
            const double du[3] = {a.u[j] - ui[0], a.u[n + j] - ui[1], a.u[2 * (size_t)n + j] - ui[2]};
            const double ddu = d[0] * du[0] + d[1] * du[1] + d[2] * du[2];
            const double c = ds / r;
            const double dui = d[0] * ui[0] + d[1] * ui[1] + d[2] * ui[2];
            for (int k = 0; k < 3; ++k) ju[k] += s * du[k] + c * d[k] * ddu;
            for (int k = 0; k < kAdjTh; ++k) th[k] += dth[k] * dui;
            if (a.wgt) {
                // d/dx_i of the smoothed counts of pairs (i, j) and (j, i)
                double wr = 0.0;
                gauss_bins(a.h, r, [&](int b, double z, double G) {
                    wr += a.wgt[b] * a.h.dr * G * (-z * a.h.inv_sig);
                });
                for (int k = 0; k < 3; ++k) gl[k] += 2.0 * wr * (-d[k] / r);
            }
        });
        for (int k = 0; k < 3; ++k) {
            const size_t o = (size_t)k * n + i;
            const double l0 = gl[k] + a.c_self1 * a.lam1[o] + a.c_self2 * a.lam2[o] + ju[k];
            a.lam0[o] = l0;
            a.u_prev[o] = a.cu0 * l0 + a.cu1 * a.lam1[o];
        }
    }
    for (int k = 0; k < kAdjTh; ++k) red[k][threadIdx.x] = th[k];
    __syncthreads();
    if (threadIdx.x < kAdjTh) {
        double t = 0.0;
        for (int m = 0; m < blockDim.x; ++m) t += red[threadIdx.x][m];
        a.part[kAdjTh * (size_t)blockIdx.x + threadIdx.x] = t;
    }
}

// adds the block partials into acc[kAdjTh] in block order (one thread block)
__global__ void adj_accumulate_kernel(const double* part, int blocks, double* acc) {
    if (threadIdx.x < kAdjTh) {
        double t = 0.0;
        for (int b = 0; b < blocks; ++b) t += part[kAdjTh * (size_t)b + threadIdx.x];
        acc[threadIdx.x] += t;
    }
}

struct AdjStep {
    int n;
    double c0, a0, b1, b2, cv, cf;
    double sig1, sig2, corr, dev, coeff0;
    uint32_t seed;
};

// x_new from x, x_prev, F, F_prev and the step's noise (mem: the previous
// draws of the noise memory, updated in place)
__global__ void __launch_bounds__(256) adj_step_kernel(AdjStep c, long long step, const double* x,
                                                       const double* xp, const double* F,
                                                       const double* Fp, const double* v0,
                                                       double* mem, double* xn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double xi[6];
    philox_gaussians6(c.seed, (uint32_t)i, (uint32_t)step, xi);
    for (int k = 0; k < 3; ++k) {
        const size_t o = (size_t)k * c.n + i;
        if (step == 0) {   // firstStep: memX = the first three draws
            mem[o] = xi[k];
            xn[o] = x[o] + c.cv * v0[o] + c.cf * F[o] + c.sig1 * xi[k];
        } else {
            const double mc = c.sig2 * (c.corr * mem[o] + c.dev * xi[k]);
            mem[o] = xi[3 + k];
            xn[o] = c.c0 * x[o] - c.a0 * xp[o] + c.b1 * F[o] - c.b2 * Fp[o] + c.sig1 * xi[3 + k] +
                    c.coeff0 * mc;
        }
    }
}

__global__ void __launch_bounds__(256) philox_noise_kernel(uint32_t seed, int n, long long first,
                                                           int n_steps, double* out) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)n * n_steps) return;
    const int t = (int)(idx / n), i = (int)(idx % n);
    double xi[6];
    philox_gaussians6(seed, (uint32_t)i, (uint32_t)(first + t), xi);
    for (int k = 0; k < 6; ++k) out[6 * idx + k] = xi[k];
}

}  // namespace
}  // namespace psim

using namespace psim;

extern "C" void psim_internal_set_error(const char* msg);

namespace {

int adj_fail(int code, const char* msg) {
    psim_internal_set_error(msg);
    return code;
}

#define ADJ_CUDA(call)                                                             \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return adj_fail(PSIM_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b ? b : 16);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
    ~Buf() { if (p) cudaFree(p); }
};

// AO coefficients c1, c2 (AOPotential.cpp:50-55) and their derivatives with
// respect to wellDepth and cutOff
void ao_coeffs_d(double kT, double wd, double rc, double c[2], double dwd[2], double drc[2]) {
    const double q = rc / (rc - 1.0);
    const double a1 = -kT * wd * q * q * q, a2 = -3.0 / (2.0 * rc), a3 = 1.0 / (2.0 * rc * rc * rc);
    c[0] = -a1 * a2;
    c[1] = -3.0 * a1 * a3;
    const double a1_wd = -kT * q * q * q;
    const double a1_rc = 3.0 * kT * wd * rc * rc / std::pow(rc - 1.0, 4);
    const double a2_rc = 3.0 / (2.0 * rc * rc), a3_rc = -3.0 / (2.0 * rc * rc * rc * rc);
    dwd[0] = -a1_wd * a2;
    dwd[1] = -3.0 * a1_wd * a3;
    drc[0] = -(a1_rc * a2 + a1 * a2_rc);
    drc[1] = -3.0 * (a1_rc * a3 + a1 * a3_rc);
}

}  // namespace

struct psim_adjoint {
    psim_adjoint_config cfg{};
    int device = 0, n = 0, T = 0, K = 0, S = 0;
    cudaStream_t st = nullptr;
    AdjGrid grid{};
    AdjStep step{};
    AdjHist hist{};
    double rc2 = 0.0, walk_rc2 = 0.0;
    int blocks128 = 0;
    Buf key, rank, count, start, scan, order, sp, spf, F[3], mem, v0, traj, ck, lam[3], u[2], part, acc,
        hsum, wgt, x0;
};

namespace {

// the cell list of positions x (3n SoA) into the walk
int build_walk(psim_adjoint* a, const double* x, AdjWalk& w) {
    const int n = a->n;
    ADJ_CUDA(cudaMemsetAsync(a->count.p, 0, 4 * (size_t)a->grid.ncell, a->st));
    adj_hash_kernel<<<(n + 255) / 256, 256, 0, a->st>>>(n, x, a->grid, a->key.as<int>(),
                                                        a->rank.as<int>(), a->count.as<int>());
    ADJ_CUDA(launch_scan(a->count.as<int>(), a->start.as<int>(), a->grid.ncell, a->scan.as<int>(),
                         a->st));
    adj_place_kernel<<<(n + 255) / 256, 256, 0, a->st>>>(n, x, a->key.as<int>(), a->rank.as<int>(),
                                                         a->start.as<int>(), a->order.as<int>(),
                                                         a->sp.as<double4_32a>(),
                                                         a->spf.as<float4>(), a->grid.L);
    w.g = a->grid;
    w.n = n;
    w.order = a->order.as<int>();
    w.sp = a->sp.as<double4_32a>();
    w.spf = a->spf.as<float4>();
    w.start = a->start.as<int>();
    w.count = a->count.as<int>();
    w.key = a->key.as<int>();
    ADJ_CUDA(cudaGetLastError());
    return PSIM_OK;
}

double* pos_at(psim_adjoint* a, Buf& b, int k) { return b.as<double>() + (size_t)k * 3 * a->n; }

// Forward from step t0 (x = x_t0, xp = x_{t0-1}, Fp = F(x_{t0-1}), mem before
// step t0) to t1, storing x_t0..x_t1 in out[0..] (out may hold just two
// slots when keep == false: then positions alternate) and, when hist is
// given, the smoothed counts of the sampled steps.  Checkpoints every K steps
// go to ck when save_ck.
int run_forward(psim_adjoint* a, const AdjPair& q, int t0, int t1, double* x_seg, bool save_ck,
                bool do_hist, bool hist_t1) {
    const int n = a->n;
    const size_t b3 = 3 * (size_t)n * sizeof(double);
    AdjWalk w{};
    w.q = q;
    for (int t = t0; t <= t1; ++t) {
        double* x = x_seg + (size_t)(t - t0) * 3 * n;
        int rc = build_walk(a, x, w);
        if (rc) return rc;
        if (do_hist && t > 0 && t % a->cfg.sample_every == 0 && (t < t1 || hist_t1))
            adj_hist_kernel<<<a->blocks128, 128, 0, a->st>>>(w, a->walk_rc2, a->hist,
                                                             a->hsum.as<double>());
        if (t == t1) break;
        // F(x_t) into the rotating buffer of step t; F(x_{t-1}) is the previous one
        double* Ft = a->F[t % 3].as<double>();
        double* Fp = a->F[(t + 2) % 3].as<double>();
        adj_force_kernel<<<a->blocks128, 128, 0, a->st>>>(w, a->rc2, Ft);
        if (save_ck && t % a->K == 0) {   // resume point: x_t, x_{t-1}, F(x_{t-1}), noise memory
            double* c = a->ck.as<double>() + (size_t)(t / a->K) * 9 * n;
            ADJ_CUDA(cudaMemcpyAsync(c, x, b3, cudaMemcpyDeviceToDevice, a->st));
            if (t > 0) {
                ADJ_CUDA(cudaMemcpyAsync(c + 3 * (size_t)n, x - 3 * (size_t)n, b3,
                                         cudaMemcpyDeviceToDevice, a->st));
                ADJ_CUDA(cudaMemcpyAsync(c + 6 * (size_t)n, Fp, b3, cudaMemcpyDeviceToDevice, a->st));
            }
            ADJ_CUDA(cudaMemcpyAsync(a->mem.as<double>() + 3 * (size_t)n * (t / a->K + 1), a->mem.p,
                                     b3, cudaMemcpyDeviceToDevice, a->st));
        }
        const double* xp = t > 0 ? x - 3 * (size_t)n : x;
        adj_step_kernel<<<(n + 255) / 256, 256, 0, a->st>>>(a->step, t, x, xp, Ft, Fp,
                                                            a->v0.as<double>(), a->mem.as<double>(),
                                                            x + 3 * (size_t)n);
        ADJ_CUDA(cudaGetLastError());
    }
    return PSIM_OK;
}

}  // namespace

namespace {

void set_pair(const psim_adjoint_params* p, AdjPair& q, double dwd[2], double drc[2]) {
    double c[2] = {0.0, 0.0};
    dwd[0] = dwd[1] = drc[0] = drc[1] = 0.0;
    q = AdjPair{};
    if (p->ao_cutoff > 0.0) {
        // the coefficients' range (1 + q) and the cutoff distance: the same
        // unless ao_range is given, which holds the cutoff while q moves
        const double range = p->ao_range > 0.0 ? p->ao_range : p->ao_cutoff;
        ao_coeffs_d(p->kT, p->ao_well_depth, range, c, dwd, drc);
        q.c1 = c[0];
        q.c2 = c[1];
        q.ao_rc2 = p->ao_cutoff * p->ao_cutoff;
    }
    if (p->yuk_cutoff > 0.0) {
        q.Y = p->yuk_amplitude;
        q.lam = p->yuk_length;
        q.inv_lam = 1.0 / p->yuk_length;
        q.y_rc2 = p->yuk_cutoff * p->yuk_cutoff;
    }
    if (p->lj_cutoff > 0.0) {
        q.eps = p->lj_epsilon;
        q.sig = p->lj_sigma;
        q.ljn = p->lj_n;
        q.lj_rc2 = p->lj_cutoff * p->lj_cutoff;
    }
}

// positions (3n AoS, original order) into a SoA device slot
int upload_soa(psim_adjoint* a, const double* host, double* dev) {
    const int n = a->n;
    ADJ_CUDA(a->x0.ensure(24 * (size_t)n));
    ADJ_CUDA(cudaMemcpyAsync(a->x0.p, host, 24 * (size_t)n, cudaMemcpyHostToDevice, a->st));
    ADJ_CUDA(launch_split_xyz(n, a->x0.as<double>(), nullptr, 0, dev, dev + n, dev + 2 * (size_t)n,
                              a->st));
    return PSIM_OK;
}

// The whole forward in K-step segments (traj holds x_{t0-1}, x_t0 .. x_t0+K),
// with checkpoints and the smoothed counts of the sampled steps.
int forward_all(psim_adjoint* a, const AdjPair& q, const double* pos0, const double* vel0) {
    const int n = a->n;
    const size_t b3 = 24 * (size_t)n;
    double* slot0 = pos_at(a, a->traj, 0);
    double* slot1 = pos_at(a, a->traj, 1);
    int rc = upload_soa(a, pos0, slot1);
    if (rc) return rc;
    if (vel0) {
        if ((rc = upload_soa(a, vel0, a->v0.as<double>()))) return rc;
    } else {
        ADJ_CUDA(cudaMemsetAsync(a->v0.p, 0, b3, a->st));
    }
    ADJ_CUDA(cudaMemcpyAsync(slot0, slot1, b3, cudaMemcpyDeviceToDevice, a->st));
    ADJ_CUDA(cudaMemsetAsync(a->hsum.p, 0, 8 * (size_t)a->cfg.n_bins, a->st));
    for (int t0 = 0; t0 < a->T; t0 += a->K) {
        const int t1 = std::min(t0 + a->K, a->T);
        // the counts of x_t1 belong to the next segment unless it is the last
        if ((rc = run_forward(a, q, t0, t1, slot1, true, true, t1 == a->T))) return rc;
        if (t1 < a->T)   // carry x_{t1-1}, x_t1 to the front
            ADJ_CUDA(cudaMemcpyAsync(slot0, pos_at(a, a->traj, t1 - t0), 2 * b3,
                                     cudaMemcpyDeviceToDevice, a->st));
    }
    return PSIM_OK;
}

int mean_g(psim_adjoint* a, std::vector<double>& g) {
    const int nb = a->cfg.n_bins;
    std::vector<double> h((size_t)nb);
    ADJ_CUDA(cudaMemcpyAsync(h.data(), a->hsum.p, 8 * (size_t)nb, cudaMemcpyDeviceToHost, a->st));
    ADJ_CUDA(cudaStreamSynchronize(a->st));
    const double L = a->cfg.geom.box_size;
    const double rho = a->n / (L * L * L);
    g.assign((size_t)nb, 0.0);
    for (int b = 0; b < nb; ++b) {
        const double rb = a->hist.r_min + (b + 0.5) * a->hist.dr;
        const double Cb = a->n * rho * 4.0 * M_PI * rb * rb * a->hist.dr;
        g[(size_t)b] = h[(size_t)b] / (a->S * Cb);
    }
    return PSIM_OK;
}

}  // namespace

extern "C" {

psim_adjoint* psim_adjoint_create(const psim_adjoint_config* cfg, int32_t device) {
    if (!cfg) { adj_fail(PSIM_ERR_INPUT, "NULL config"); return nullptr; }
    const psim_geometry& gm = cfg->geom;
    const int n = gm.n_particles;
    if (n <= 0 || gm.cell_scale < 3 || !(gm.box_size > 0.0) ||
        std::fabs(gm.cell_size * gm.cell_scale - gm.box_size) > 1e-9 * gm.box_size) {
        adj_fail(PSIM_ERR_INPUT, "adjoint: bad geometry (n > 0, cellScale >= 3, cellSize * cellScale == box)");
        return nullptr;
    }
    if (cfg->n_steps <= 0 || cfg->checkpoint_every <= 0 || cfg->sample_every <= 0 ||
        cfg->sample_every > cfg->n_steps || cfg->n_bins <= 0 || !(cfg->r_max > cfg->r_min) ||
        !(cfg->sigma > 0.0) || !(cfg->mass > 0.0)) {
        adj_fail(PSIM_ERR_INPUT, "adjoint: bad steps, checkpoint/sample interval, bins, sigma or mass");
        return nullptr;
    }
    const double reach = cfg->r_max + 4.0 * cfg->sigma;
    if (reach > gm.cell_size) {
        adj_fail(PSIM_ERR_INPUT, "adjoint: cellSize must cover r_max + 4 sigma");
        return nullptr;
    }
    psim_vgb_coeffs vc;
    if (psim_vgb_coefficients(cfg->integ.gamma, cfg->integ.dt, cfg->integ.kT, &vc)) return nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        adj_fail(PSIM_ERR_NO_DEVICE, "adjoint: no such CUDA device");
        return nullptr;
    }
    cudaSetDevice(device);
    psim_adjoint* a = new psim_adjoint();
    a->cfg = *cfg;
    a->device = device;
    a->n = n;
    a->T = cfg->n_steps;
    a->K = std::min(std::max(cfg->checkpoint_every, 2), cfg->n_steps);
    a->S = cfg->n_steps / cfg->sample_every;
    a->grid = AdjGrid{gm.box_size, 1.0 / gm.cell_size, gm.cell_scale, gm.cell_scale * gm.cell_scale,
                      gm.cell_scale * gm.cell_scale * gm.cell_scale};
    const double dt = cfg->integ.dt, dt2 = dt * dt, m = 1.0 / cfg->mass;
    a->step = AdjStep{n, 1.0 + vc.coeff0, vc.coeff0, m * dt2 * (vc.coeff1 + vc.coeff2),
                      m * dt2 * vc.coeff2, vc.coeff1 * dt, vc.coeff3 * dt2 * m, vc.sig1, vc.sig2,
                      vc.corr, vc.dev, vc.coeff0, (uint32_t)cfg->integ.seed};
    const double dr = (cfg->r_max - cfg->r_min) / cfg->n_bins;
    a->hist = AdjHist{cfg->r_min, dr, 1.0 / cfg->sigma, 1.0 / (std::sqrt(2.0 * M_PI) * cfg->sigma),
                      cfg->n_bins, (int)std::ceil(4.0 * cfg->sigma / dr) + 1};
    a->walk_rc2 = reach * reach;
    a->blocks128 = (n + 127) / 128;
    const size_t b3 = 24 * (size_t)n, nc = (size_t)a->grid.ncell;
    const int nck = (a->T + a->K - 1) / a->K + 1;
    bool ok = cudaStreamCreateWithFlags(&a->st, cudaStreamNonBlocking) == cudaSuccess &&
              !a->key.ensure(4 * (size_t)n) && !a->rank.ensure(4 * (size_t)n) &&
              !a->count.ensure(4 * nc) && !a->start.ensure(4 * nc) &&
              !a->scan.ensure(4 * (size_t)scan_scratch_ints((int)nc)) &&
              !a->order.ensure(4 * (size_t)n) && !a->sp.ensure(32 * (size_t)n) &&
              !a->spf.ensure(16 * (size_t)n) &&
              !a->F[0].ensure(b3) && !a->F[1].ensure(b3) && !a->F[2].ensure(b3) &&
              !a->mem.ensure(b3 * (size_t)(nck + 1)) && !a->v0.ensure(b3) &&
              !a->traj.ensure(b3 * (size_t)(a->K + 2)) && !a->ck.ensure(3 * b3 * (size_t)nck) &&
              !a->lam[0].ensure(b3) && !a->lam[1].ensure(b3) && !a->lam[2].ensure(b3) &&
              !a->u[0].ensure(b3) && !a->u[1].ensure(b3) &&
              !a->part.ensure(8 * kAdjTh * (size_t)a->blocks128) && !a->acc.ensure(8 * kAdjTh) &&
              !a->hsum.ensure(8 * (size_t)cfg->n_bins) && !a->wgt.ensure(8 * (size_t)cfg->n_bins);
    if (!ok) {
        adj_fail(PSIM_ERR_CUDA, "adjoint: device allocation failed");
        psim_adjoint_destroy(a);
        return nullptr;
    }
    return a;
}

int psim_philox_noise(uint32_t seed, int32_t n, int64_t first_step, int32_t n_steps,
                      double* out, int32_t device) {
    if (!out || n < 0 || n_steps < 0 || first_step < 0)
        return adj_fail(PSIM_ERR_INPUT, "philox noise: bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return adj_fail(PSIM_ERR_NO_DEVICE, "philox noise: no such CUDA device");
    const long long cnt = (long long)n * n_steps;
    if (cnt == 0) return PSIM_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaError_t e;
    {   // the buffer is freed with `device` current
        Buf b;
        e = b.ensure(48 * (size_t)cnt);
        if (e == cudaSuccess) {
            philox_noise_kernel<<<(unsigned)((cnt + 255) / 256), 256>>>(seed, n, first_step,
                                                                        n_steps, b.as<double>());
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpy(out, b.p, 48 * (size_t)cnt, cudaMemcpyDeviceToHost);
    }
    cudaSetDevice(prev);
    return e == cudaSuccess ? PSIM_OK : adj_fail(PSIM_ERR_CUDA, cudaGetErrorString(e));
}

void psim_adjoint_destroy(psim_adjoint* a) {
    if (!a) return;
    cudaSetDevice(a->device);
    if (a->st) {
        cudaStreamSynchronize(a->st);
        cudaStreamDestroy(a->st);
    }
    delete a;
}

int psim_adjoint_forward(psim_adjoint* a, const psim_adjoint_params* p, const double* pos0,
                         const double* vel0, double* g_mean, double* pos_final) {
    if (!a || !p || !pos0 || !g_mean) return adj_fail(PSIM_ERR_INPUT, "NULL argument");
    cudaSetDevice(a->device);
    AdjPair q;
    double dwd[2], drc[2];
    set_pair(p, q, dwd, drc);
    a->rc2 = std::max(std::max(q.ao_rc2, q.y_rc2), q.lj_rc2);
    if (a->rc2 > a->cfg.geom.cell_size * a->cfg.geom.cell_size)
        return adj_fail(PSIM_ERR_INPUT, "adjoint: a cutoff exceeds the cell size");
    int rc = forward_all(a, q, pos0, vel0);
    if (rc) return rc;
    std::vector<double> g;
    if ((rc = mean_g(a, g))) return rc;
    std::copy(g.begin(), g.end(), g_mean);
    if (pos_final) {
        const int last = a->T - ((a->T - 1) / a->K) * a->K;   // slot of x_T in the last segment
        const double* x = pos_at(a, a->traj, 1 + last);
        ADJ_CUDA(launch_merge_xyz(a->n, x, x + a->n, x + 2 * (size_t)a->n, nullptr, nullptr,
                                  a->x0.as<double>(), a->st));
        ADJ_CUDA(cudaMemcpyAsync(pos_final, a->x0.p, 24 * (size_t)a->n, cudaMemcpyDeviceToHost,
                                 a->st));
        ADJ_CUDA(cudaStreamSynchronize(a->st));
    }
    return PSIM_OK;
}

int psim_adjoint_gradient(psim_adjoint* a, const psim_adjoint_params* p, const double* pos0,
                          const double* vel0, const double* g_target, double* loss,
                          double* g_mean, double* grad, double* grad_pos0) {
    if (!a || !p || !pos0 || !g_target || !loss || !grad)
        return adj_fail(PSIM_ERR_INPUT, "NULL argument");
    cudaSetDevice(a->device);
    const int n = a->n, T = a->T, K = a->K, nb = a->cfg.n_bins;
    const size_t b3 = 24 * (size_t)n;
    AdjPair q;
    double dwd[2], drc[2];
    set_pair(p, q, dwd, drc);
    a->rc2 = std::max(std::max(q.ao_rc2, q.y_rc2), q.lj_rc2);
    if (a->rc2 > a->cfg.geom.cell_size * a->cfg.geom.cell_size)
        return adj_fail(PSIM_ERR_INPUT, "adjoint: a cutoff exceeds the cell size");
    if (q.lj_rc2 > 0.0 && (!(q.sig > 0.0) || q.ljn < 0 || q.ljn > 64))
        return adj_fail(PSIM_ERR_INPUT, "adjoint: LJ term needs sigma > 0 and 0 <= n <= 64");
    // forward: checkpoints and the loss
    int rc = forward_all(a, q, pos0, vel0);
    if (rc) return rc;
    std::vector<double> g;
    if ((rc = mean_g(a, g))) return rc;
    double L = 0.0;
    std::vector<double> wgt((size_t)nb);
    const double box = a->cfg.geom.box_size, rho = n / (box * box * box);
    for (int b = 0; b < nb; ++b) {
        const double diff = g[(size_t)b] - g_target[b];
        L += diff * diff;
        const double rb = a->hist.r_min + (b + 0.5) * a->hist.dr;
        const double Cb = n * rho * 4.0 * M_PI * rb * rb * a->hist.dr;
        wgt[(size_t)b] = 2.0 * diff / (a->S * Cb);   // dL / d(smoothed count of one sample)
    }
    *loss = L;
    if (g_mean) std::copy(g.begin(), g.end(), g_mean);
    ADJ_CUDA(cudaMemcpyAsync(a->wgt.p, wgt.data(), 8 * (size_t)nb, cudaMemcpyHostToDevice, a->st));
    // reverse: lam_{T+1} = lam_{T+2} = 0, u_T = 0
    for (int k = 0; k < 3; ++k) ADJ_CUDA(cudaMemsetAsync(a->lam[k].p, 0, b3, a->st));
    ADJ_CUDA(cudaMemsetAsync(a->u[0].p, 0, b3, a->st));
    ADJ_CUDA(cudaMemsetAsync(a->acc.p, 0, 8 * kAdjTh, a->st));
    int l0 = 0, l1 = 1, l2 = 2, uc = 0;   // lam_t, lam_{t+1}, lam_{t+2}; u_t
    double* slot0 = pos_at(a, a->traj, 0);
    double* slot1 = pos_at(a, a->traj, 1);
    const int nseg = (T + K - 1) / K;
    const double rwalk = std::max(a->rc2, a->walk_rc2);
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int t0 = seg * K, t1 = std::min(t0 + K, T);
        // recompute the segment from its checkpoint
        const double* c = a->ck.as<double>() + (size_t)seg * 9 * n;
        ADJ_CUDA(cudaMemcpyAsync(slot1, c, b3, cudaMemcpyDeviceToDevice, a->st));
        ADJ_CUDA(cudaMemcpyAsync(slot0, t0 > 0 ? c + 3 * (size_t)n : c, b3, cudaMemcpyDeviceToDevice,
                                 a->st));
        if (t0 > 0)
            ADJ_CUDA(cudaMemcpyAsync(a->F[(t0 + 2) % 3].p, c + 6 * (size_t)n, b3,
                                     cudaMemcpyDeviceToDevice, a->st));
        ADJ_CUDA(cudaMemcpyAsync(a->mem.p, a->mem.as<double>() + 3 * (size_t)n * (seg + 1), b3,
                                 cudaMemcpyDeviceToDevice, a->st));
        if ((rc = run_forward(a, q, t0, t1, slot1, false, false, false))) return rc;
        for (int t = (seg == nseg - 1 ? t1 : t1 - 1); t >= t0; --t) {
            AdjWalk w{};
            w.q = q;
            if ((rc = build_walk(a, pos_at(a, a->traj, 1 + t - t0), w))) return rc;
            AdjReverse r{};
            r.u = a->u[uc].as<double>();
            r.lam1 = a->lam[l1].as<double>();
            r.lam2 = a->lam[l2].as<double>();
            r.lam0 = a->lam[l0].as<double>();
            r.u_prev = a->u[1 - uc].as<double>();
            r.c_self1 = t > 0 ? a->step.c0 : 1.0;
            r.c_self2 = -a->step.a0;
            r.cu0 = t - 1 >= 1 ? a->step.b1 : a->step.cf;
            r.cu1 = -a->step.b2;
            r.wgt = (t > 0 && t % a->cfg.sample_every == 0) ? a->wgt.as<double>() : nullptr;
            r.h = a->hist;
            r.part = a->part.as<double>();
            adj_reverse_kernel<<<a->blocks128, 128, 0, a->st>>>(w, rwalk, r);
            adj_accumulate_kernel<<<1, 32, 0, a->st>>>(a->part.as<double>(), a->blocks128,
                                                       a->acc.as<double>());
            ADJ_CUDA(cudaGetLastError());
            // lam_t becomes lam_{t+1} of the next (earlier) step
            const int old2 = l2;
            l2 = l1;
            l1 = l0;
            l0 = old2;
            uc = 1 - uc;
        }
    }
    double th[kAdjTh];
    ADJ_CUDA(cudaMemcpyAsync(th, a->acc.p, 8 * kAdjTh, cudaMemcpyDeviceToHost, a->st));
    if (grad_pos0) {   // lam_0 (now lam[l1]) in original order
        const double* l = a->lam[l1].as<double>();
        ADJ_CUDA(launch_merge_xyz(n, l, l + n, l + 2 * (size_t)n, nullptr, nullptr,
                                  a->x0.as<double>(), a->st));
        ADJ_CUDA(cudaMemcpyAsync(grad_pos0, a->x0.p, b3, cudaMemcpyDeviceToHost, a->st));
    }
    ADJ_CUDA(cudaStreamSynchronize(a->st));
    // th = dL/d(c1, c2, Y, lambda, eps, sigma) -> dL/d(AO wellDepth, AO range,
    // Y, lambda, eps, sigma)
    grad[0] = th[0] * dwd[0] + th[1] * dwd[1];
    grad[1] = th[0] * drc[0] + th[1] * drc[1];
    grad[2] = th[2];
    grad[3] = th[3];
    grad[4] = th[4];
    grad[5] = th[5];
    return PSIM_OK;
}

}  // extern "C"
