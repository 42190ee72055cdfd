// psim_observe.cu -- observables of the device-resident state: the analysis
// the reference runs between steps, on the GPU so the state stays in HBM.
//
//   temperature          analysisManager::getTemperature  (analysisGeneral.cpp:26-43)
//   mean displacement    analysisManager::meanDisplacement (analysisGeneral.cpp:45-55)
//   tracked displacement trackedDisplacement (analysisTracker.cpp:26-85), every wrap counted
//   potential ("EAP")    particle::calculatePotential (particle.cpp:133-149), summed
//   coordination         system::updateInteractions (systemHandling.cpp:94-161)
//   g(r)                 a pair-distance histogram over the same 27-cell walk
//   energy and virial    FP64 sums over pairs of the plugin's u(r) and r.f
//
// Sums are deterministic: each block writes its partial, one block adds the
// partials in block order.
#include "psim_kernels.cuh"

namespace psim {

namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 512;

__device__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    __syncthreads();
    return t;  // valid in thread 0
}

__global__ void __launch_bounds__(kRedThreads) finish_kernel(const double* part, int n, double* out) {
    __shared__ double sh[kRedThreads / 32];
    // each thread adds a fixed stride of partials, then the block in lane order
    double v = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) v += part[k];
    const double t = block_sum(v, sh);
    if (threadIdx.x == 0) *out = t;
}

// sum of |v|^2 over count values
__global__ void __launch_bounds__(kRedThreads) sumsq_kernel(long long count, const double* v,
                                                            double* part) {
    __shared__ double sh[kRedThreads / 32];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        s += v[i] * v[i];
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(kRedThreads) observe_kernel(ObserveArgs a, double* part) {
    __shared__ double sh[kRedThreads / 32];
    double s = 0.0;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.n; f += gridDim.x * blockDim.x) {
        const double x[3] = {a.x[f], a.y[f], a.z[f]};
        if (a.what == OBS_MEAN_DISP) {
            const double d0 = x[0] - a.x0[f], d1 = x[1] - a.y0[f], d2 = x[2] - a.z0[f];
            s += d0 * d0 + d1 * d1 + d2 * d2;
        } else if (a.what == OBS_TRACKED) {
            const int t = a.tag[f];
            for (int k = 0; k < 3; ++k) {
                // the reference sums this in FP32 (analysisTracker.cpp:68-83)
                const double d = (x[k] + a.L * a.img[3 * (size_t)t + k]) - a.start[3 * (size_t)t + k];
                s += d * d;
            }
        } else {  // OBS_POTENTIAL: particle::calculatePotential in FP32
            const int o = a.perm_prev ? a.perm_prev[f] : f;
            const float dx = (float)(x[0] - a.x0[f]), dy = (float)(x[1] - a.y0[f]),
                        dz = (float)(x[2] - a.z0[f]);
            const double F[3] = {a.fx[f], a.fy[f], a.fz[f]};
            const double G[3] = {a.gx[o], a.gy[o], a.gz[o]};
            const float dfx = (float)(F[0] - G[0]), dfy = (float)(F[1] - G[1]),
                        dfz = (float)(F[2] - G[2]);
            const float dr = sqrtf(dx * dx + dy * dy + dz * dz);
            const float df = sqrtf(dfx * dfx + dfy * dfy + dfz * dfz);
            const float f0 = sqrtf((float)(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]));
            const float p = (f0 * dr) + (0.5f * df * dr);
            s += (double)(-p);
        }
    }
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// The 27-cell walk of updateInteractions (systemHandling.cpp:126-161) on
// the sorted FP64 positions: neighbours closer than r_contact are counted
// (pbcDist's minimum image, utilities.cpp:79-104), and distances in
// [r_min, r_max) are binned for g(r).
__global__ void __launch_bounds__(128) pairs_kernel(PairScanArgs a) {
    extern __shared__ unsigned int hist[];
    for (int b = threadIdx.x; b < a.n_bins; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.g.n) {
        const double4_32a pi = a.posd[i];
        const int c = a.cellid[i];
        const int cx = c % a.g.s, cy = (c / a.g.s) % a.g.s, cz = c / a.g.s2;
        int coor = 0;
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    int sh;
                    const int x = wrap_cell(cx + dx, a.g.s, sh);
                    const int y = wrap_cell(cy + dy, a.g.s, sh);
                    const int z = wrap_cell(cz + dz, a.g.s, sh);
                    const int cell = x + a.g.s * y + a.g.s2 * z;
                    const int st = a.cstart[cell], en = st + a.ccount[cell];
                    for (int j = st; j < en; ++j) {
                        if (j == i) continue;
                        const double4_32a pj = a.posd[j];
                        double d0 = fabs(pj.x - pi.x), d1 = fabs(pj.y - pi.y),
                               d2 = fabs(pj.z - pi.z);
                        if (d0 > a.g.half) d0 -= a.g.L;
                        if (d1 > a.g.half) d1 -= a.g.L;
                        if (d2 > a.g.half) d2 -= a.g.L;
                        const double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                        if (r < a.r_contact) ++coor;
                        if (a.n_bins > 0 && r >= a.r_min && r < a.r_max) {
                            int b = (int)((r - a.r_min) * a.inv_dr);
                            b = b < a.n_bins ? b : a.n_bins - 1;
                            atomicAdd(&hist[b], 1u);
                        }
                    }
                }
        if (a.coor) a.coor[a.tag[i]] = coor;
        if (a.n_pairs) atomicAdd(a.n_pairs, (unsigned long long)coor);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < a.n_bins; b += blockDim.x)
        if (hist[b]) atomicAdd(&a.hist[b], (unsigned long long)hist[b]);
}

// ---------------------------------------------------------------- clusters
// Connected components of the contact graph (r < r_contact), the clusters of
// analysisManager::findClusters (analysisCluster.cpp:26-62), by lock-free
// union-find over original indices: an edge hooks the larger of its two roots
// under the smaller with atomicCAS, so each component's root ends as its
// smallest original index -- the order findClusters visits clusters in.
// Parents always have smaller indices, so a chain is at most n long and a
// failed hook means the root was hooked by another thread (at most n times);
// both loops are capped at n + 1 anyway and report EBIT_INDEX past it.

__device__ int uf_find(const int* label, int x, int n, uint32_t& err) {
    int p = ((const volatile int*)label)[x];
    for (int k = 0; p != x; ++k) {
        if (k > n) {
            err |= EBIT_INDEX;
            return x;
        }
        x = p;
        p = ((const volatile int*)label)[x];
    }
    return x;
}

__device__ void uf_union(int* label, int a, int b, int n, uint32_t& err) {
    for (int it = 0; it <= n; ++it) {
        a = uf_find(label, a, n, err);
        b = uf_find(label, b, n, err);
        if (a == b || err) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(&label[b], b, a);
        if (old == b) return;   // hooked; else b gained a parent meanwhile: retry
    }
    err |= EBIT_INDEX;
}

__global__ void __launch_bounds__(256) uf_init_kernel(int n, int* label) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) label[i] = i;
}

__global__ void __launch_bounds__(128) uf_edges_kernel(PairScanArgs a, int* label,
                                                        uint32_t* err_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.g.n) return;
    uint32_t err = 0;
    const double4_32a pi = a.posd[i];
    const int ti = a.tag[i];
    const int c = a.cellid[i];
    const int cx = c % a.g.s, cy = (c / a.g.s) % a.g.s, cz = c / a.g.s2;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                int sh;
                const int x = wrap_cell(cx + dx, a.g.s, sh);
                const int y = wrap_cell(cy + dy, a.g.s, sh);
                const int z = wrap_cell(cz + dz, a.g.s, sh);
                const int cell = x + a.g.s * y + a.g.s2 * z;
                const int st = a.cstart[cell], en = st + a.ccount[cell];
                for (int j = st; j < en; ++j) {
                    const int tj = a.tag[j];
                    if (tj <= ti) continue;   // each undirected edge once
                    const double4_32a pj = a.posd[j];
                    double d0 = fabs(pj.x - pi.x), d1 = fabs(pj.y - pi.y), d2 = fabs(pj.z - pi.z);
                    if (d0 > a.g.half) d0 -= a.g.L;
                    if (d1 > a.g.half) d1 -= a.g.L;
                    if (d2 > a.g.half) d2 -= a.g.L;
                    if (sqrt(d0 * d0 + d1 * d1 + d2 * d2) < a.r_contact)
                        uf_union(label, ti, tj, a.g.n, err);
                }
            }
    if (err) atomicOr(err_out, err);
}

__global__ void __launch_bounds__(256) uf_final_kernel(int n, const int* label, int* root,
                                                        int* size, uint32_t* err_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t err = 0;
    const int r = uf_find(label, i, n, err);
    root[i] = r;
    atomicAdd(&size[r], 1);
    if (err) atomicOr(err_out, err);
}

// ------------------------------------------------------ energy and virial
// One pair term of the energy walk: u(r) and fNet(r) inside the cutoff.
template <class Pair>
struct OneTerm {
    Pair p;
    __device__ double rc2() const { return p.rc2; }
    __device__ void eval(double r2, double r, double rinv, double size, double& u,
                         double& f) const {
        if (r2 < p.rc2) {
            u += p.u64(r2, r, rinv, size);
            f += p.fnet64(r2, r, rinv, size);
        }
    }
};
struct ComboTerms {  // the AO + LJ(n) composite: each part inside its own cutoff
    AOPair ao;
    LJPair lj;
    __device__ double rc2() const { return ao.rc2 > lj.rc2 ? ao.rc2 : lj.rc2; }
    __device__ void eval(double r2, double r, double rinv, double size, double& u,
                         double& f) const {
        if (r2 < ao.rc2) {
            u += ao.u64(r2, r, rinv, size);
            f += ao.fnet64(r2, r, rinv, size);
        }
        if (r2 < lj.rc2) {
            u += lj.u64(r2, r, rinv, size);
            f += lj.fnet64(r2, r, rinv, size);
        }
    }
};

// Per particle i: half the sum over its neighbours j of u(r_ij) and of
// r_ij . f_ij = -fNet(r_ij) r_ij (pbcDist's minimum image), in FP64; block
// partials of both, added in block order by finish_kernel.
template <class Terms>
__global__ void __launch_bounds__(128) energy_kernel(PairScanArgs a, Terms t, double* part,
                                                     int stride) {
    __shared__ double sh[4];
    double eu = 0.0, ew = 0.0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.g.n) {
        const double4_32a pi = a.posd[i];
        const int c = a.cellid[i];
        const int cx = c % a.g.s, cy = (c / a.g.s) % a.g.s, cz = c / a.g.s2;
        const double rc2 = t.rc2();
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    int sh_;
                    const int x = wrap_cell(cx + dx, a.g.s, sh_);
                    const int y = wrap_cell(cy + dy, a.g.s, sh_);
                    const int z = wrap_cell(cz + dz, a.g.s, sh_);
                    const int cell = x + a.g.s * y + a.g.s2 * z;
                    const int st = a.cstart[cell], en = st + a.ccount[cell];
                    for (int j = st; j < en; ++j) {
                        if (j == i) continue;
                        const double4_32a pj = a.posd[j];
                        double d0 = fabs(pj.x - pi.x), d1 = fabs(pj.y - pi.y),
                               d2 = fabs(pj.z - pi.z);
                        if (d0 > a.g.half) d0 -= a.g.L;
                        if (d1 > a.g.half) d1 -= a.g.L;
                        if (d2 > a.g.half) d2 -= a.g.L;
                        const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
                        if (!(r2 < rc2)) continue;
                        const double r = sqrt(r2), rinv = 1.0 / r;
                        double u = 0.0, f = 0.0;
                        t.eval(r2, r, rinv, pi.w + pj.w, u, f);
                        eu += u;
                        ew -= f * r;
                    }
                }
    }
    const double su = block_sum(0.5 * eu, sh);
    const double sw = block_sum(0.5 * ew, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = su;
        part[stride + blockIdx.x] = sw;
    }
}

template <class Terms>
cudaError_t run_energy(const Terms& t, const PairScanArgs& a, double* scratch, double* out,
                       cudaStream_t st) {
    const int blocks = (a.g.n + 127) / 128;
    energy_kernel<Terms><<<blocks, 128, 0, st>>>(a, t, scratch, blocks);
    finish_kernel<<<1, kRedThreads, 0, st>>>(scratch, blocks, out);
    finish_kernel<<<1, kRedThreads, 0, st>>>(scratch + blocks, blocks, out + 1);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_energy(const ForceSetup& fs, const PairScanArgs& a, double* scratch,
                          double* out, cudaStream_t st) {
    if (a.g.n == 0) return cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
    switch (fs.kind) {
    case 1: return run_energy(OneTerm<AOPair>{fs.ao}, a, scratch, out, st);
    case 2: return run_energy(OneTerm<LJPair>{fs.lj}, a, scratch, out, st);
    case 3: return run_energy(OneTerm<CalPair>{fs.cal}, a, scratch, out, st);
    case 4: return run_energy(ComboTerms{fs.ao, fs.lj}, a, scratch, out, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_clusters(const PairScanArgs& a, int* label, int* root, int* size,
                            uint32_t* err, cudaStream_t st) {
    const int n = a.g.n;
    if (n == 0) return cudaSuccess;
    uf_init_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, label);
    uf_edges_kernel<<<(n + 127) / 128, 128, 0, st>>>(a, label, err);
    uf_final_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, label, root, size, err);
    return cudaGetLastError();
}

cudaError_t launch_sum_squares(long long count, const double* v, double* scratch, double* out,
                               cudaStream_t st) {
    sumsq_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(count, v, scratch);
    finish_kernel<<<1, kRedThreads, 0, st>>>(scratch, kRedBlocks, out);
    return cudaGetLastError();
}

cudaError_t launch_observe(const ObserveArgs& a, double* scratch, double* out, cudaStream_t st) {
    observe_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(a, scratch);
    finish_kernel<<<1, kRedThreads, 0, st>>>(scratch, kRedBlocks, out);
    return cudaGetLastError();
}

int observe_scratch_doubles() { return kRedBlocks; }

cudaError_t launch_pair_scan(const PairScanArgs& a, cudaStream_t st) {
    if (a.g.n == 0) return cudaSuccess;
    const size_t smem = sizeof(unsigned int) * (size_t)(a.n_bins > 0 ? a.n_bins : 1);
    pairs_kernel<<<(a.g.n + 127) / 128, 128, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace psim
