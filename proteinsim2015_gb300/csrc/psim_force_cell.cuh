// psim_force_cell.cuh -- the plugin force pass with one block per home cell.
//
// All particles of a home cell share one 27-cell neighbourhood
// (AOPotential.cpp:147-170), so a block of 128 threads takes one home cell:
//
//   stage  the 27 cells are 9 rows of 3 x-adjacent cells, each a contiguous
//          run of the sorted list (a wrap in x splits a row in two): up to 18
//          runs.  Threads 0..17 describe one run each, a warp prefix sum lays
//          them end to end, and the block copies the neighbourhood into
//          shared memory in one flat loop of coalesced 16-byte loads.  A run
//          across the box edge is stored with its periodic image applied, as
//          an exact float pair (TwoSum), so no per-pair image arithmetic is
//          needed.  The stage is padded with far-away dummies so the test loop
//          needs no bounds checks.  A neighbourhood larger than the stage is
//          processed in several chunks.
//   A      the home particles are spread over the block, k = 128 / n lanes
//          each; lane p of a home tests stage slots p, p+k, p+2k, ... (lanes
//          with the same p read the same slot: a broadcast) with an FP32
//          distance widened to cover the rounding of the positions, and
//          appends in-range ones to its own queue -- branch-free.
//   B      every lane drains its queue through the plugin's pair body.
//   reduce the k partial forces of each home are summed in lane order
//          through shared memory (deterministic) and stored.
#pragma once

#include "psim_kernels.cuh"

namespace psim {

constexpr int kCellThreads = 128;
constexpr int kCellStage = 384;                  // staged particles per chunk
constexpr int kCellQueue = 16;                   // drain when a lane holds this many
constexpr int kCellUnroll = 4;
constexpr int kCellQueueCap = kCellQueue + kCellUnroll;
// lane p of a home reads slots p + m k for m < ceil(chunk / k) rounded up to
// kCellUnroll: below chunk + kCellUnroll * kCellThreads
constexpr int kCellPad = kCellUnroll * kCellThreads;

// c + d for |d| <= 1 and c in [0, s): the wrapped cell and its image
__device__ __forceinline__ int wrap_near(int c, int s, int& shift) {
    shift = 0;
    if (c < 0) {
        c += s;
        shift = -1;
    } else if (c >= s) {
        c -= s;
        shift = 1;
    }
    return c;
}

template <class Body>
__global__ void __launch_bounds__(kCellThreads)
force_cell_kernel(Body body, DevGeom g, CellView cv, ForceOut out, float pre_rc2) {
    using Aux = typename Body::Aux;
    __shared__ float4 s_hi[kCellStage + kCellPad];
    __shared__ Aux s_aux[kCellStage];
    __shared__ uint16_t s_q[kCellQueueCap][kCellThreads];
    __shared__ double s_red[3 * kCellThreads];  // the body's partial sums, per lane
    __shared__ int s_run_a[18], s_run_off[19], s_run_img[18];
    __shared__ int s_failed;

    const int c = blockIdx.x;
    const int tid = threadIdx.x;
    const int n_c = cv.ccount[c];
    if (n_c == 0) return;  // block-uniform: no barrier has been reached
    const int start_c = cv.cstart[c];
    const int cx = c % g.s, cy = (c / g.s) % g.s, cz = c / g.s2;
    // run descriptors, one per thread of warp 0; an error latched by an
    // earlier kernel is read once for the whole block
    if (tid < 32) {
        int len = 0, a = 0, img = 13;
        if (tid < 18) {
            const int row = tid >> 1, part = tid & 1;
            int sy, sz;
            const int y = wrap_near(cy + row / 3 - 1, g.s, sy);
            const int z = wrap_near(cz + row % 3 - 1, g.s, sz);
            const int base = g.s * y + g.s2 * z;
            int sx = 0;
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
            img = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
        }
        int incl = len;  // inclusive prefix of the run lengths
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (tid >= o) incl += v;
        }
        if (tid < 18) {
            s_run_a[tid] = a;
            s_run_off[tid] = incl - len;
            s_run_img[tid] = img;
        }
        if (tid == 17) s_run_off[18] = incl;
        if (tid == 0) s_failed = (*out.err != 0) ? 1 : 0;
    }
    __syncthreads();
    if (s_failed) return;
    const int total = s_run_off[18];
    // the home cell is row (0, 0), part 0: run 8
    const int home_off = s_run_off[8] + (start_c - s_run_a[8]);
    const Aux* g_aux = body.aux(cv);

    for (int hb = 0; hb < n_c; hb += kCellThreads) {
        const int nh = min(n_c - hb, kCellThreads);
        const int k = kCellThreads / nh;         // lanes per home
        const int h = tid % nh, p = tid / nh;
        const bool active = p < k;
        const int gi = start_c + hb + h;         // this lane's home particle
        float4 hi = cv.posh[gi];
        typename Body::Home home;
        typename Body::Shifted hs;
        typename Body::Acc acc;
        body.init(acc);
        body.load_home(cv, gi, home);
        body.shift(home, hi, 0, 0, 0, g, hs);
        const float thr = active ? pre_rc2 : -1.0f;  // inactive lanes accept nothing
        uint32_t err = 0;

        for (int c0 = 0; c0 < total; c0 += kCellStage) {
            const int fill = min(total - c0, kCellStage);
            __syncthreads();  // the previous readers of the stage are done
            for (int m = tid; m < fill + kCellPad; m += kCellThreads) {
                if (m < fill) {
                    const int gm = c0 + m;
                    int r = 0;
#pragma unroll
                    for (int q = 1; q < 18; ++q) r += (gm >= s_run_off[q]) ? 1 : 0;
                    const int j = s_run_a[r] + (gm - s_run_off[r]);
                    float4 hj = cv.posh[j];
                    Aux aj = g_aux[j];
                    const int img = s_run_img[r];
                    if (img != 13)
                        body.image(hj, aj, img % 3 - 1, (img / 3) % 3 - 1, img / 9 - 1, g);
                    s_hi[m] = hj;
                    s_aux[m] = aj;
                } else {
                    s_hi[m] = make_float4(1e30f, 1e30f, 1e30f, 0.f);  // never in range
                }
            }
            __syncthreads();
            const int self_t = home_off + hb + h - c0;  // outside [0, fill) when not staged
            int cnt = 0;
            const int iters = (fill + k - 1) / k;
            for (int m0 = 0; m0 < iters; m0 += kCellUnroll) {
#pragma unroll
                for (int u = 0; u < kCellUnroll; ++u) {
                    const int t = (m0 + u) * k + p;
                    const float4 hj = s_hi[t];
                    const float ex = hj.x - hi.x, ey = hj.y - hi.y, ez = hj.z - hi.z;
                    const float r2 = ex * ex + ey * ey + ez * ez;
                    const bool in = (r2 < thr) & (t != self_t);
                    s_q[cnt][tid] = (uint16_t)t;
                    cnt += in ? 1 : 0;
                }
                if (__any_sync(0xffffffffu, cnt >= kCellQueue) || m0 + kCellUnroll >= iters) {
                    const int kmax = __reduce_max_sync(0xffffffffu, cnt);
                    for (int q = 0; q < kmax; ++q) {
                        if (q < cnt) {
                            const int s = s_q[q][tid];
                            body.eval(s_hi[s], s_aux[s], hs, acc, err);
                        }
                    }
                    body.fold(acc);
                    cnt = 0;
                }
            }
        }
        // the k partial forces of each home, summed in lane order
        __syncthreads();
        body.partial(acc, s_red, tid, kCellThreads);
        __syncthreads();
        if (p == 0) body.reduce_store(out, gi, s_red, kCellThreads, h, nh, k);
        if (err) atomicOr(out.err, err);
    }
}

template <class Body>
cudaError_t launch_force_cells(const Body& body, const DevGeom& g, const CellView& cv,
                               const ForceOut& out, float pre_rc2, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    force_cell_kernel<Body><<<g.ncell, kCellThreads, 0, st>>>(body, g, cv, out, pre_rc2);
    return cudaGetLastError();
}

}  // namespace psim
