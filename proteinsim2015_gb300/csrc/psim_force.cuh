// psim_force.cuh -- the plugin force pass as a two-phase warp kernel.
//
// The reference evaluates, for every particle, all particles of the 27
// neighbour cells (defaultForceManager.cpp:55-65 -> <plugin>::getAcceleration
// -> iterCells, e.g. AOPotential.cpp:61-175).  With cellSize >= cutOff only
// ~15% of those candidates are inside the cutoff, so a thread-per-particle
// loop that evaluates the pair force under a branch runs the pair body in
// almost every iteration with a few lanes active.  Here each warp owns 32
// consecutive sorted particles and works in two phases:
//
//   A. candidate test: the 27 cells are walked as 9 rows of 3 x-adjacent
//      cells, each row a contiguous run of the sorted particle list (two runs
//      when the row wraps around the box).  Each lane tests its own row with
//      an FP32 distance on the rounded positions (a margin covers their
//      rounding) and appends in-range candidates (index + periodic image) to
//      its own queue in shared memory.  Loop bounds are warp-uniform (the
//      longest run of the warp), so there is no divergent control flow.
//   B. pair forces: when a queue fills (and at the end) every lane drains its
//      own queue with the plugin's pair body; lanes stay busy because each
//      holds ~a queue's worth of pairs, and each lane sums only its own
//      particle's force, so no atomics or reductions are needed.
//
// Body supplies the precision-specific parts (psim_exact.cu: FP64 plain form
// with the reference's image rules; psim_mixed.cu: FP32 pairs with Kahan
// sums).
#pragma once

#include "psim_kernels.cuh"

namespace psim {

constexpr int kForceWarps = 4;              // warps per block
constexpr int kQueue = 48;                  // drain when a lane holds this many
constexpr int kUnroll = 4;                  // candidates tested between drains
constexpr int kQueueCap = kQueue + kUnroll; // slots per lane
constexpr uint32_t kIndexMask = (1u << 27) - 1u;  // queue entry: j | image << 27
constexpr uint32_t kNoImage = 13u;                // (0, 0, 0)

// n < 2^27 particles so a queue entry packs the index with the image code
// ((sx+1) + 3(sy+1) + 9(sz+1), 0..26).
__device__ __forceinline__ void decode_image(uint32_t e, int& sx, int& sy, int& sz) {
    const int code = (int)(e >> 27);
    sx = code % 3 - 1;
    sy = (code / 3) % 3 - 1;
    sz = code / 9 - 1;
}

template <class Body>
__global__ void __launch_bounds__(kForceWarps * 32)
force_pass_kernel(Body body, DevGeom g, CellView cv, ForceOut out, float pre_rc2) {
    __shared__ uint32_t queue[kForceWarps][kQueueCap][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // an error latched by an earlier kernel stops the pass; read once and
    // broadcast so every lane of the warp takes the same path
    const bool failed = __shfl_sync(0xffffffffu, (lane == 0) ? (*out.err != 0) : false, 0);
    const bool active = (i < g.n) && !failed;
    uint32_t (*q)[32] = queue[w];

    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f);
    int cx = 0, cy = 0, cz = 0;
    typename Body::Home home;
    typename Body::Acc acc;
    body.init(acc);
    if (active) {
        hi = cv.posh[i];
        const int c = cv.cellid[i];
        cx = c % g.s;
        cy = (c / g.s) % g.s;
        cz = c / g.s2;
        body.load_home(cv, i, home);
    }
    uint32_t err = 0;
    int cnt = 0;

    auto drain = [&]() {
        const int kmax = __reduce_max_sync(0xffffffffu, cnt);
        for (int k = 0; k < kmax; ++k) {
            if (k < cnt) body.eval(g, cv, home, hi, q[k][lane], acc, err);
        }
        body.fold(acc);
        cnt = 0;
        __syncwarp();
    };

    for (int row = 0; row < 9; ++row) {
        const int dy = row / 3 - 1, dz = row % 3 - 1;
        int sy, sz;
        const int y = wrap_cell(cy + dy, g.s, sy);
        const int z = wrap_cell(cz + dz, g.s, sz);
        const int base = g.s * y + g.s2 * z;
#pragma unroll 1
        for (int part = 0; part < 2; ++part) {
            // part 0: the cells of [cx-1, cx+1] inside the grid, contiguous;
            // part 1: the one cell that wraps around in x (if any)
            int a = 0, len = 0, sx = 0;
            if (active) {
                if (part == 0) {
                    const int xa = cx > 0 ? cx - 1 : 0;
                    const int xb = cx < g.s - 1 ? cx + 1 : g.s - 1;
                    a = cv.cstart[base + xa];
                    len = cv.cstart[base + xb] + cv.ccount[base + xb] - a;
                } else if (cx == 0 || cx == g.s - 1) {
                    const int xw = cx == 0 ? g.s - 1 : 0;
                    sx = cx == 0 ? -1 : 1;
                    a = cv.cstart[base + xw];
                    len = cv.ccount[base + xw];
                }
            }
            const int lmax = __reduce_max_sync(0xffffffffu, len);
            if (lmax == 0) continue;
            // the image is applied to the home position: d = x_j - (x_i - s L)
            const float hx = hi.x - (float)sx * g.Lhi;
            const float hy = hi.y - (float)sy * g.Lhi;
            const float hz = hi.z - (float)sz * g.Lhi;
            const uint32_t img = (uint32_t)((sx + 1) + 3 * (sy + 1) + 9 * (sz + 1)) << 27;
            // Branch-free test: the load index is clamped into the list (the
            // tail of a shorter run reads a valid particle and is masked out),
            // every candidate is written to the next free slot and only an
            // in-range one advances the counter.
            const int jlast = g.n - 1;
            for (int t0 = 0; t0 < lmax; t0 += kUnroll) {
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) {
                    const int t = t0 + u;
                    const int j = a + t;
                    const float4 hj = __ldg(&cv.posh[min(j, jlast)]);
                    const float ex = hj.x - hx, ey = hj.y - hy, ez = hj.z - hz;
                    const float r2 = ex * ex + ey * ey + ez * ez;
                    const bool in = (t < len) & (r2 < pre_rc2) & (j != i);
                    q[cnt][lane] = (uint32_t)j | img;
                    cnt += in ? 1 : 0;
                }
                if (__any_sync(0xffffffffu, cnt >= kQueue)) drain();
            }
        }
    }
    drain();
    if (active) body.store(out, i, acc);
    if (err) atomicOr(out.err, err);
}

template <class Body>
cudaError_t launch_force_pass(const Body& body, const DevGeom& g, const CellView& cv,
                              const ForceOut& out, float pre_rc2, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    if (g.n >= (1 << 27)) return cudaErrorInvalidValue;
    const int threads = kForceWarps * 32;
    force_pass_kernel<Body><<<(g.n + threads - 1) / threads, threads, 0, st>>>(body, g, cv, out,
                                                                              pre_rc2);
    return cudaGetLastError();
}

// LennardJones with the exponent fixed at compile time (the common ljNum
// values 0, 6, 12, 18); LJPair's runtime loop covers the rest.
template <int N>
struct LJFixed : LJPair {
    __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double size) const {
        double lj = powi_fixed<N>(size * rinv);
        double attract = (2.0 * lj) - 1.0;
        attract *= (four_n * rinv * lj);
        double repel = 0.0;
        if (yuk != 0.0) {
            double e = exp(-1.0 * (r * inv_lambda));
            repel = e * (rinv * rinv * (lambda + r) * yuk);
        }
        return -kTwd * (attract + repel);
    }
    __device__ __forceinline__ float fnet32(float r2, float r, float rinv, float size) const {
        float attract = 0.0f;
        if (N > 0) {
            const float lj = powi_fixed<N>(size * rinv);
            attract = (2.0f * lj - 1.0f) * (four_nf * rinv * lj);
        }
        float repel = 0.0f;
        if (yukf != 0.0f) repel = __expf(-r * inv_lambdaf) * (rinv * rinv * (lambdaf + r) * yukf);
        return -kTwdf * (attract + repel);
    }
};

}  // namespace psim
