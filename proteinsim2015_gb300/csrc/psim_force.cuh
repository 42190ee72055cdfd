// psim_force.cuh -- the plugin force pass as a two-phase warp kernel.
//
// The reference evaluates, for every particle, all particles of the 27
// neighbour cells (defaultForceManager.cpp:55-65 -> <plugin>::getAcceleration
// -> iterCells, e.g. AOPotential.cpp:61-175).  With cellSize >= cutOff only
// ~15% of those candidates are inside the cutoff, so a thread-per-particle
// loop that evaluates the pair force under a branch runs the pair body in
// almost every iteration with a few lanes active.  Here each warp owns 32
// consecutive sorted particles and walks the 27 cells as 9 rows of 3
// x-adjacent cells: in the sorted list a row is one contiguous run (the x-wrap
// at the box edge adds a second, one-cell run).  For each row:
//
//   stage  the union of the 32 lanes' runs (~5 cells, ~70 particles) is
//          copied into shared memory with coalesced 16-byte loads;
//   A      each lane tests its own run from shared memory with an FP32
//          distance on the rounded positions (a margin covers their rounding)
//          and appends in-range candidates to its own queue -- branch-free:
//          every candidate is written to the next free slot and only an
//          in-range one advances the count; loop bounds are warp-uniform;
//   B      every lane drains its own queue with the plugin's pair body, so
//          each lane sums only its own particle's force (no atomics).
//
// The row's periodic image is folded into a per-lane shifted home position,
// so neither phase handles images per pair.  Runs that wrap around the box
// in x, and unions too long for the stage, are read from global memory.
//
// Body supplies the precision-specific parts (psim_exact.cu: FP64 plain form
// with the reference's image rules; psim_mixed.cu: FP32 pairs with Kahan
// sums).  The staged walk serves the FP64 form; the mixed form takes the
// direct walk (force_direct_kernel, below), which reads the rows through L1
// and keeps its queues across rows.
#pragma once

#include <climits>

#include "psim_kernels.cuh"

namespace psim {

constexpr int kForceWarps = 4;                // warps per block
constexpr int kStage = 96;                    // staged particles per warp and row
constexpr int kQueue = 20;                    // drain when a lane holds this many
constexpr int kUnroll = 4;                    // candidates tested between drain checks
constexpr int kQueueCap = kQueue + kUnroll;   // slots per lane
// A lane reads its run at stage[rel + t] for t < (longest run of the warp,
// rounded up to kUnroll); rel + len <= union length <= kStage, so reads stay
// below 2 kStage + kUnroll.  Slots past the union hold stale data that the
// t < len test masks.
constexpr int kStagePad = 2 * kStage + kUnroll;

// The warp's walk: particle i of the lane (inactive lanes i >= g.p1), with
// the warp's shared stage and queues.
template <class Body>
__device__ __forceinline__ void force_pass_warp(const Body& body, const DevGeom& g,
                                                const CellView& cv, const ForceOut& out,
                                                float pre_rc2, int i, int lane,
                                                float4* st_hi, typename Body::Aux* st_aux,
                                                uint32_t (*q)[32]) {
    using Aux = typename Body::Aux;
    const bool active = i < g.p1;
    const Aux* g_aux = body.aux(cv);

    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f);
    int cx = 0, cy = 0, cz = 0;
    typename Body::Home home;
    typename Body::Acc acc;
    body.init(acc);
    if (active) {
        hi = cv.posh[i];
        const int c = cv.cellid[i] - g.c0;
        cx = c % g.s;
        cy = (c / g.s) % g.s;
        cz = c / g.s2;
        body.load_home(cv, i, home);
    }
    uint32_t err = 0;
    int cnt = 0;
    const int jlast = g.p1 - 1;

    for (int row = 0; row < 9; ++row) {
        // z-major rows: runs come in increasing sorted-slot order
        const int dz = row / 3 - 1, dy = row % 3 - 1;
        int sy, sz;
        const int y = wrap_cell(cy + dy, g.s, sy);
        const int z = wrap_cell(cz + dz, g.s, sz);
        const int base = g.c0 + g.s * y + g.s2 * z;
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
            typename Body::Shifted hs;
            body.shift(home, hi, sx, sy, sz, g, hs);
            const float hx = hi.x - (float)sx * g.Lhi;
            const float hy = hi.y - (float)sy * g.Lhi;
            const float hz = hi.z - (float)sz * g.Lhi;
            const int u0 = __reduce_min_sync(0xffffffffu, len > 0 ? a : INT_MAX);
            const int u1 = __reduce_max_sync(0xffffffffu, len > 0 ? a + len : 0);
            const int ulen = u1 - u0;
            if (part == 0 && ulen <= kStage) {
                for (int k = lane; k < ulen; k += 32) {
                    st_hi[k] = cv.posh[u0 + k];
                    st_aux[k] = g_aux[u0 + k];
                }
                __syncwarp();
                const int rel = len > 0 ? a - u0 : 0;
                // candidate t of this lane is stage[rel + t]; it is the home
                // particle itself when rel + t == i - u0
                const int dself = (i >= u0 && i < u1) ? rel - (i - u0) : INT_MIN / 2;
                const float4* sp = st_hi + rel;
                uint32_t* qp = &q[0][lane];
                uint32_t* const qlim = &q[kQueue][lane];
                for (int t0 = 0; t0 < lmax; t0 += kUnroll, sp += kUnroll) {
                    const int rem = len - t0;      // candidate u is in the run iff u < rem
                    const int ds = dself + t0;     // candidate u is the home iff ds + u == 0
#pragma unroll
                    for (int u = 0; u < kUnroll; ++u) {
                        const float4 hj = sp[u];
                        const float ex = hj.x - hx, ey = hj.y - hy, ez = hj.z - hz;
                        const float r2 = ex * ex + ey * ey + ez * ez;
                        const bool in = (u < rem) & (r2 < pre_rc2) & (ds + u != 0);
                        *qp = (uint32_t)(rel + t0 + u);
                        qp += in ? 32 : 0;
                    }
                    if (__any_sync(0xffffffffu, qp >= qlim) || t0 + kUnroll >= lmax) {
                        const int n_in = (int)(qp - &q[0][lane]) >> 5;
                        const int kmax = __reduce_max_sync(0xffffffffu, n_in);
                        for (int k = 0; k < kmax; ++k) {
                            if (k < n_in) {
                                const uint32_t sidx = q[k][lane];
                                body.eval(st_hi[sidx], st_aux[sidx], hs, acc, err);
                            }
                        }
                        qp = &q[0][lane];
                    }
                }
                __syncwarp();  // the stage is rewritten by the next row
            } else {
                for (int t0 = 0; t0 < lmax; t0 += kUnroll) {
#pragma unroll
                    for (int u = 0; u < kUnroll; ++u) {
                        const int t = t0 + u;
                        const int j = min(a + t, jlast);
                        const float4 hj = __ldg(&cv.posh[j]);
                        const float ex = hj.x - hx, ey = hj.y - hy, ez = hj.z - hz;
                        const float r2 = ex * ex + ey * ey + ez * ez;
                        const bool in = (t < len) & (r2 < pre_rc2) & (j != i);
                        q[cnt][lane] = (uint32_t)j;
                        cnt += in ? 1 : 0;
                    }
                    if (__any_sync(0xffffffffu, cnt >= kQueue) || t0 + kUnroll >= lmax) {
                        const int kmax = __reduce_max_sync(0xffffffffu, cnt);
                        for (int k = 0; k < kmax; ++k) {
                            if (k < cnt) {
                                const uint32_t j2 = q[k][lane];
                                body.eval(__ldg(&cv.posh[j2]), g_aux[j2], hs, acc, err);
                            }
                        }
                        cnt = 0;
                    }
                }
            }
            body.fold(acc);
        }
    }
    if (active) body.store(out, i, acc);
    if (err) atomicOr(out.err, err);
}

// An error latched by an earlier kernel (or a closed gate) stops the pass;
// read once by lane 0 and broadcast so every lane takes the same path.
__device__ __forceinline__ bool pass_failed(const ForceOut& out, int lane) {
    return __shfl_sync(0xffffffffu,
                       (lane == 0) ? (*out.err != 0 || (out.gate && *out.gate == 0)) : false, 0);
}

// One system: the geometry and body are kernel parameters.
template <class Body>
__global__ void __launch_bounds__(kForceWarps * 32)
force_pass_kernel(Body body, DevGeom g, CellView cv, ForceOut out, float pre_rc2) {
    __shared__ float4 s_hi[kForceWarps][kStagePad];
    __shared__ typename Body::Aux s_aux[kForceWarps][kStage];
    __shared__ uint32_t s_q[kForceWarps][kQueueCap][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (pass_failed(out, lane)) return;  // warp-uniform; warps synchronise only themselves
    force_pass_warp(body, g, cv, out, pre_rc2, blockIdx.x * blockDim.x + threadIdx.x, lane,
                    s_hi[w], s_aux[w], s_q[w]);
}

// The mixed form's 27-cell walk (the direct walk): a thread per sorted
// particle walks its 9 rows of cells straight from global memory and keeps
// its in-range candidates in a queue across rows, each entry with its row's
// periodic image (5 bits above the 27-bit slot).  The warp drains the queues
// when one is nearly full and at the end, so a lane runs the pair body about
// as often as the warp's busiest lane has neighbours in all 27 cells, where
// the staged walk drains after every row.  The particles of a warp mostly
// share their rows' runs, so the candidate reads broadcast through L1 about
// as well as they would from a shared-memory stage.  Measured on GB300 the
// direct walk beat the staged walk at every occupancy tried (1 to 21
// particles per cell: force pass 3-37% shorter).  The image is applied to
// the neighbour (Body::image).  A single system and each replica of a batch
// follow the same rule, so that a replica steps alike in both.  The FP64
// form keeps the staged walk, whose sums follow the reference's cell order:
// a direct walk with a fold marker at each row's end gave the same bits but
// measured 6-18% slower (its 32-byte FP64 neighbour loads through L1).
constexpr int kDirectQueue = kQueue;          // the staged walk's queue rows, reused
constexpr int kDirectMaxN = 1 << 27;          // slots the queue entries can hold
constexpr int kDirectCentre = 13;             // image code of (0, 0, 0)

// walk: 0 the body's own choice, 1 the staged walk, 2 the direct walk (where
// the body allows it).  A queue entry holds a storage slot in 27 bits: the
// grid's particles (a replica's, in a batch: global slots up to p1) must end
// below 2^27.
template <class Body>
__host__ __device__ __forceinline__ bool direct_walk(const DevGeom& g, int walk = 0) {
    if constexpr (Body::kDirectWalk) return g.p1 <= kDirectMaxN && walk != 1;
    return false;
}

template <class Body>
__device__ __forceinline__ void force_direct_warp(const Body& body, const DevGeom& g,
                                                  const CellView& cv, const ForceOut& out,
                                                  float pre_rc2, int i, int lane,
                                                  uint32_t (*q)[32]) {
    using Aux = typename Body::Aux;
    const Aux* g_aux = body.aux(cv);
    const bool active = i < g.p1;
    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f);
    int cx = 0, cy = 0, cz = 0;
    typename Body::Home home;
    typename Body::Acc acc;
    body.init(acc);
    if (active) {
        hi = cv.posh[i];
        const int c = cv.cellid[i] - g.c0;
        cx = c % g.s;
        cy = (c / g.s) % g.s;
        cz = c / g.s2;
        body.load_home(cv, i, home);
    }
    typename Body::Shifted hs;
    body.shift(home, hi, 0, 0, 0, g, hs);
    uint32_t err = 0;
    int cnt = 0;
    const int jlast = g.p1 - 1;
    auto drain = [&]() {
        const int kmax = __reduce_max_sync(0xffffffffu, cnt);
        for (int k = 0; k < kmax; ++k) {
            if (k < cnt) {
                const uint32_t e = q[k][lane];
                const int j = (int)(e & (uint32_t)(kDirectMaxN - 1));
                const int img = (int)(e >> 27);
                float4 hj = __ldg(&cv.posh[j]);
                Aux aj = g_aux[j];
                if (img != kDirectCentre)
                    body.image(hj, aj, img % 3 - 1, (img / 3) % 3 - 1, img / 9 - 1, g);
                body.eval(hj, aj, hs, acc, err);
            }
        }
        body.fold(acc);
        cnt = 0;
    };
    for (int row = 0; row < 9; ++row) {
        const int dz = row / 3 - 1, dy = row % 3 - 1;
        int sy, sz;
        const int y = wrap_cell(cy + dy, g.s, sy);
        const int z = wrap_cell(cz + dz, g.s, sz);
        const int base = g.c0 + g.s * y + g.s2 * z;
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
            // the neighbour's image is +s L: x_j + s L - x_i
            const float hx = hi.x - (float)sx * g.Lhi;
            const float hy = hi.y - (float)sy * g.Lhi;
            const float hz = hi.z - (float)sz * g.Lhi;
            const uint32_t code = (uint32_t)((sx + 1) + 3 * (sy + 1) + 9 * (sz + 1)) << 27;
            for (int t0 = 0; t0 < lmax; t0 += kUnroll) {
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) {
                    const int t = t0 + u;
                    const int j = min(a + t, jlast);
                    const float4 hj = __ldg(&cv.posh[j]);
                    const float ex = hj.x - hx, ey = hj.y - hy, ez = hj.z - hz;
                    const float r2 = ex * ex + ey * ey + ez * ez;
                    const bool in = (t < len) & (r2 < pre_rc2) & (j != i);
                    q[cnt][lane] = (uint32_t)j | code;
                    cnt += in ? 1 : 0;
                }
                // at most kDirectQueue - kUnroll entries before a batch of
                // kUnroll: slots stay below kQueueCap
                if (__any_sync(0xffffffffu, cnt > kDirectQueue - kUnroll)) drain();
            }
        }
    }
    drain();
    if (active) body.store(out, i, acc);
    if (err) atomicOr(out.err, err);
}

template <class Body>
__global__ void __launch_bounds__(kForceWarps * 32)
force_direct_kernel(Body body, DevGeom g, CellView cv, ForceOut out, float pre_rc2) {
    __shared__ uint32_t s_q[kForceWarps][kQueueCap][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (pass_failed(out, lane)) return;  // warp-uniform
    force_direct_warp(body, g, cv, out, pre_rc2, blockIdx.x * blockDim.x + threadIdx.x, lane,
                      s_q[w]);
}

// A batch of replicas: each warp takes a task (replica, first particle) and
// that replica's geometry, pair functor and prefilter bound.
template <class Body>
__global__ void __launch_bounds__(kForceWarps * 32)
force_batch_kernel(Body body0, CellView cv, ForceOut out, BatchView bv, int walk) {
    __shared__ float4 s_hi[kForceWarps][kStagePad];
    __shared__ typename Body::Aux s_aux[kForceWarps][kStage];
    __shared__ uint32_t s_q[kForceWarps][kQueueCap][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (pass_failed(out, lane)) return;
    const int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (task >= bv.n_tasks) return;
    const int2 t = bv.tasks[task];
    const DevGeom g = bv.geoms[t.x];
    const Body body = body0.for_replica(bv.pairs, t.x, g);
    if (direct_walk<Body>(g, walk))   // the rule a single system of this replica follows
        force_direct_warp(body, g, cv, out, bv.pre[t.x], t.y + lane, lane, s_q[w]);
    else
        force_pass_warp(body, g, cv, out, bv.pre[t.x], t.y + lane, lane, s_hi[w], s_aux[w],
                        s_q[w]);
}

template <class Body>
cudaError_t launch_force_pass(const Body& body, const DevGeom& g, const CellView& cv,
                              const ForceOut& out, float pre_rc2, cudaStream_t st,
                              const BatchView* bv = nullptr, int walk = 0) {
    const int threads = kForceWarps * 32;
    if (bv && bv->tasks) {
        if constexpr (Body::kBatchable) {
            if (bv->n_tasks == 0) return cudaSuccess;
            const int blocks = (bv->n_tasks + kForceWarps - 1) / kForceWarps;
            force_batch_kernel<Body><<<blocks, threads, 0, st>>>(body, cv, out, *bv, walk);
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    if (g.n == 0) return cudaSuccess;
    if (direct_walk<Body>(g, walk)) {
        force_direct_kernel<Body><<<(g.n + threads - 1) / threads, threads, 0, st>>>(
            body, g, cv, out, pre_rc2);
        return cudaGetLastError();
    }
    force_pass_kernel<Body><<<(g.n + threads - 1) / threads, threads, 0, st>>>(body, g, cv, out,
                                                                              pre_rc2);
    return cudaGetLastError();
}

// LennardJones with the exponent fixed at compile time (the common ljNum
// values 0, 6, 12, 18); LJPair's runtime loop covers the rest.
template <int N>
struct LJFixed : LJPair {
    __host__ __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double size) const {
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

// LennardJones with an even exponent fixed at compile time and no Yukawa term
// (yukawaStrength 0, the plain 2n-n potential): fNet = -kT wd (2L-1) 4n L / r
// with L = (size^2 / r^2)^(n/2), a function of r^2 alone.
template <int N>
struct LJPure : LJPair {
    static_assert(N > 0 && N % 2 == 0, "an even, positive exponent");
    __device__ __forceinline__ float fnet32(float, float, float rinv, float size) const {
        const float lj = powi_fixed<N>(size * rinv);
        return -kTwdf * ((2.0f * lj - 1.0f) * (four_nf * rinv * lj));
    }
};

static_assert(sizeof(LJPure<6>) == sizeof(LJPair), "batches store LJPair parameters");

// FP32 reciprocal, approximate (rcp.approx: max error ~1 ulp)
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// F(r)/r of a pair at r^2 for the pair-list pass, the value the cell walk's
// body forms as fnet32(r2, r, 1/r, size) / r.  s2 = size^2.
template <class P>
__device__ __forceinline__ float list_fr32(const P& p, float r2, float size, float) {
    const float rinv = rsqrtf(r2);
    return p.fnet32(r2, r2 * rinv, rinv, size) * rinv;
}
// the plain LJ form needs only 1/r^2: C (2L - 1) L / r^2 with C = -kT wd 4n
// and L = (s2 / r^2)^(n/2), one reciprocal and no square root
template <int N>
__device__ __forceinline__ float list_fr32(const LJPure<N>& p, float r2, float, float s2) {
    const float rinv2 = rcp_approx(r2);
    const float lj = powi_fixed<N / 2>(s2 * rinv2);
    const float c = -p.kTwdf * p.four_nf;
    return fmaf(2.0f * c, lj, -c) * (lj * rinv2);
}

}  // namespace psim
