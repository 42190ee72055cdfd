// psim_force_list.cuh -- the mixed form's force pass through a Verlet pair list.
//
// The plugin force on particle i is the sum over the particles j of its 27
// neighbour cells with |x_j - x_i| < rc (AOPotential.cpp:61-175,
// LJPotential.cpp:64-182).  Every such j lies within rc + skin of i's position
// at any earlier time at which neither particle had yet moved skin/2 -- so a
// list of the pairs within rc + skin, built from the cell list at one step,
// holds every pair the cell walk would find for as long as no particle has
// moved more than skin/2 since.  The list is rebuilt on the step after one
// has.  The force of each step is then the same set of pair terms, read from
// ~(rc+skin)^3/(27 cs^3) as many candidates as the cell walk tests.
//
//   build  the warp kernel of psim_force.cuh with a body that appends, rather
//          than evaluates, the candidates within rc + skin (plus the rounding
//          margin of its FP32 test).  It runs on the step's own cell list, so
//          list order is the cell order of the build step, and it needs
//          cellSize >= rc + skin.  A pair across the box edge refers to a
//          halo record: a copy of the neighbour shifted by the box, made for
//          every particle within rc + skin of a face and rewritten with it
//          each step, so the force pass does no periodic arithmetic.
//   force  a thread per particle walks its list in FP32 with the plugin's pair
//          body and Kahan-compensated sums (MixedBody, psim_mixed.cu).
//
// Positions in list order are kept as exact float pairs and *unwrapped*: the
// integrator writes each particle's new position as the image nearest its
// build position (and its halo images beside it), so a pair's periodic image
// found at the build stays right for the life of the list (the box is larger
// than 2 (rc + skin)).
#pragma once

#include "psim_force.cuh"

namespace psim {

// The pair-list build, a thread per particle i (sorted order of the build
// step, whose list slots are the sorted positions).  It walks the 27
// neighbour cells as 9 rows of x-adjacent cells -- one contiguous run of the
// sorted list per row, plus a one-cell run where the row wraps in x -- and
// appends every candidate within the list radius (rc + skin, widened by the
// FP32 test's rounding margin).  A neighbour cell beyond that radius from
// the particle (by its distance to the cell's faces) is not read: about a
// quarter of the 27 cells on average when cellSize ~ rc + skin.  A pair
// across the box edge refers to the neighbour's halo record for that image.
// When each cell's particles are sorted by x (ListBuild::xsorted), a row's
// run is sorted by x too, and two binary searches cut it to the particles
// within the row's x reach of the home: about 250 candidates per particle
// instead of about 410 at cellSize ~ rc + skin.
// Lists are padded to a multiple of kListFold with the ghost record, a dummy
// out of range of every particle, so the force pass reads whole batches.
// st.global of v at p when w holds; no branch around it
__device__ __forceinline__ void store_if(uint32_t* p, uint32_t v, bool w) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.u32 [%0], %1;\n\t}"
                 :: "l"(p), "r"(v), "r"((uint32_t)w) : "memory");
}

// A home's list is stored in groups of kListFold = 8 entries: group q of the
// home in slot i is 32 contiguous bytes at element (q stride + i) 8, so the
// force pass reads a group with one 32-byte load per thread.  The build
// appends entry n of home i at element o = ((n / 8) stride + i) 8 + n % 8,
// kept as a 32-bit offset (the host keeps (cap + 8) stride below 2^32);
// entries past the cap go to the scratch group cap / 8 and are counted, so
// that the overflow is reported.
__device__ __forceinline__ void list_append(const ListBuild& lb, uint32_t ocap, uint32_t v,
                                            bool in, int& n, uint32_t& o) {
    store_if(lb.list + min(o, ocap), v, in);
    n += in ? 1 : 0;
    // next element: the following word, or the next group's first
    const uint32_t step = (n & (kListFold - 1)) ? 1u : (uint32_t)lb.stride * kListFold - 7u;
    o += in ? step : 0u;
}

// Appends the candidates of one run [a, a + len) of the sorted list within
// the list radius of the home position (hx, hy, hz) (the home particle i
// minus the run's image s L) to i's list, n entries so far.  Candidates are
// read four at a time, up to three past the run (the sorted positions are
// padded by four), and masked.  Only the home row's run (kSelf) can hold i
// itself; a shifted run appends the neighbour's halo record for that image.
template <bool kShifted, bool kSelf>
__device__ __forceinline__ void list_run(const CellView& cv, const ListBuild& lb, float R2, int i,
                                         int a, int len, float hx, float hy, float hz, int sx,
                                         int sy, int sz, int& n, uint32_t& o, uint32_t& err) {
    const uint32_t ocap = ((uint32_t)(lb.cap / kListFold) * (uint32_t)lb.stride + (uint32_t)i) *
                          kListFold;
    const float4* pp = cv.posh + a;
    for (int t0 = 0; t0 < len; t0 += 4, pp += 4) {
        float4 hj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) hj[u] = __ldg(pp + u);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float ex = hj[u].x - hx, ey = hj[u].y - hy, ez = hj[u].z - hz;
            const float r2 = ex * ex + ey * ey + ez * ez;
            bool in = (t0 + u < len) & (r2 < R2);
            if (kSelf) in &= (a + t0 + u != i);
            if (!kShifted) {
                list_append(lb, ocap, (uint32_t)(a + t0 + u), in, n, o);
            } else if (in) {
                // image number: one bit per flagged axis, set where this run shifts
                const int j = a + t0 + u;
                const int hal = lb.lhalo[j];
                const uint32_t fl = (uint32_t)(hal & 63);
                const int sh[3] = {sx, sy, sz};
                int num = 0, bit = 0;
                bool ok = true;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int fk = halo_axis(fl, k);
                    if (sh[k] != 0) {
                        ok = ok && fk == sh[k];
                        num |= 1 << bit;
                    }
                    if (fk != 0) ++bit;
                }
                if (!ok)   // no record of that image: the margin failed
                    err |= EBIT_LIST;
                else
                    list_append(lb, ocap, (uint32_t)(lb.ghost + 1 + (hal >> 6) + num - 1),
                                true, n, o);
            }
        }
    }
}

__device__ __forceinline__ void list_build_one(const DevGeom& g, const CellView& cv,
                                               const ListBuild& lb, float R2, int i,
                                               uint32_t& err) {
    const float4 hi = cv.posh[i];
    const int c = cv.cellid[i] - g.c0;
    const int cx = c % g.s, cy = (c / g.s) % g.s, cz = c / g.s2;
    const int ghost = lb.ghost;
    // distances to the lower and upper faces of the home cell, less a margin
    // for the FP32 rounding of the position and of the cell bounds
    const float csf = (float)g.cs;
    const float m = 8.0f * ulp_of(g.Lhi);
    const float fx = hi.x - (float)cx * csf, fy = hi.y - (float)cy * csf,
                fz = hi.z - (float)cz * csf;
    const float lo[3] = {fmaxf(fx - m, 0.f), fmaxf(fy - m, 0.f), fmaxf(fz - m, 0.f)};
    const float up[3] = {fmaxf(csf - fx - m, 0.f), fmaxf(csf - fy - m, 0.f),
                         fmaxf(csf - fz - m, 0.f)};
    int n = 0;
    uint32_t o = (uint32_t)i * kListFold;
    for (int row = 0; row < 9; ++row) {
        const int dz = row / 3 - 1, dy = row % 3 - 1;
        const float ey = dy < 0 ? lo[1] : (dy > 0 ? up[1] : 0.f);
        const float ez = dz < 0 ? lo[2] : (dz > 0 ? up[2] : 0.f);
        const float e2 = ey * ey + ez * ez;
        if (e2 >= R2) continue;
        int sy, sz;
        const int y = wrap_cell(cy + dy, g.s, sy);
        const int z = wrap_cell(cz + dz, g.s, sz);
        const int base = g.c0 + g.s * y + g.s2 * z;
        const bool left = e2 + lo[0] * lo[0] < R2, right = e2 + up[0] * up[0] < R2;
#pragma unroll 1
        for (int part = 0; part < 2; ++part) {
            // part 0: the reachable cells of [cx-1, cx+1] inside the grid;
            // part 1: the one cell that wraps around in x (if reachable)
            int a = 0, len = 0, sx = 0;
            if (part == 0) {
                const int xa = (left && cx > 0) ? cx - 1 : cx;
                const int xb = (right && cx < g.s - 1) ? cx + 1 : cx;
                a = cv.cstart[base + xa];
                len = cv.cstart[base + xb] + cv.ccount[base + xb] - a;
            } else if ((cx == 0 && left) || (cx == g.s - 1 && right)) {
                const int xw = cx == 0 ? g.s - 1 : 0;
                sx = cx == 0 ? -1 : 1;
                a = cv.cstart[base + xw];
                len = cv.ccount[base + xw];
            }
            if (len <= 0) continue;
            // the row's image is applied to the home position
            const float hx = hi.x - (float)sx * g.Lhi;
            const float hy = hi.y - (float)sy * g.Lhi;
            const float hz = hi.z - (float)sz * g.Lhi;
            if (lb.xsorted) {
                // the run is sorted by x: keep the candidates within the
                // row's x reach sqrt(R^2 - e^2) of the home, found by two
                // binary searches.  e^2 is a lower bound of a candidate's
                // y-z distance^2 (the face distances carry the margin m); the
                // reach is widened by 1e-5 R^2 under the root, far above the
                // FP32 rounding of the r^2 test, and by m outside it.
                const float rx = sqrtf(fmaxf(R2 - e2, 0.f) + 1e-5f * R2) + m;
                const float xlo = hx - rx, xhi = hx + rx;
                // the two searches run interleaved (independent load chains)
                const float4* pp = cv.posh + a;
                int l0 = 0, h0 = len, l1 = 0, h1 = len;
                while (l0 < h0 || l1 < h1) {
                    const int m0 = (l0 + h0) >> 1, m1 = (l1 + h1) >> 1;
                    const float x0 = l0 < h0 ? __ldg(&pp[m0].x) : 0.f;
                    const float x1 = l1 < h1 ? __ldg(&pp[m1].x) : 0.f;
                    if (l0 < h0) {
                        if (x0 < xlo) l0 = m0 + 1;
                        else h0 = m0;
                    }
                    if (l1 < h1) {
                        if (x1 <= xhi) l1 = m1 + 1;
                        else h1 = m1;
                    }
                }
                a += l0;
                len = l1 - l0;
                if (len <= 0) continue;
            }
            if ((sx | sy | sz) != 0)
                list_run<true, false>(cv, lb, R2, i, a, len, hx, hy, hz, sx, sy, sz, n, o, err);
            else if (row == 4 && part == 0)
                list_run<false, true>(cv, lb, R2, i, a, len, hx, hy, hz, 0, 0, 0, n, o, err);
            else
                list_run<false, false>(cv, lb, R2, i, a, len, hx, hy, hz, 0, 0, 0, n, o, err);
        }
    }
    // the open group padded with the ghost record
    const uint32_t ocap = ((uint32_t)(lb.cap / kListFold) * (uint32_t)lb.stride + (uint32_t)i) *
                          kListFold;
    while (n & (kListFold - 1)) list_append(lb, ocap, (uint32_t)ghost, true, n, o);
    if (n > lb.cap) {
        err |= EBIT_LIST;
        n = lb.cap;
    }
    lb.count[i] = n;
}

// A grid of a few blocks per SM striding over the particles, so that a step
// whose rebuild gate is closed costs one short launch.
__global__ void __launch_bounds__(128)
list_build_kernel(DevGeom g, CellView cv, ListBuild lb, uint32_t* errp) {
    if (*errp != 0 || (lb.gate && *lb.gate == 0)) return;
    uint32_t err = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        if (lb.rep) {   // a batch: the particle's replica's grid and list radius
            const int r = lb.rep[i];
            list_build_one(lb.geoms[r], cv, lb, lb.pre[r], i, err);
        } else {
            list_build_one(g, cv, lb, lb.pre_r2, i, err);
        }
    }
    if (err) atomicOr(errp, err);
}

// One 32-byte record (high and low float4 halves) in a single 256-bit load
// through the read-only path; the records are 32-byte aligned.
__device__ __forceinline__ void load_record(const float4* pos, uint32_t j, float4& h, float4& l) {
    const float4* a = pos + 2 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(h.x), "=f"(h.y), "=f"(h.z), "=f"(h.w), "=f"(l.x), "=f"(l.y), "=f"(l.z), "=f"(l.w)
        : "l"(a));
}

// One group of kListFold = 8 list entries (32 bytes, 32-byte aligned) in a
// single 256-bit load through the read-only path: a warp's request covers
// its 1 KB once, where two 128-bit loads would each cover all of it.
__device__ __forceinline__ void load_group(const uint32_t* p, uint4& a, uint4& b) {
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
        : "l"(p));
}

// A neighbour record as the force pass holds it between its load and its
// pair term: one float4 (compact) or the high and low halves (full).
template <bool kCompact>
struct ListRec {
    float4 h;
};
template <>
struct ListRec<false> {
    float4 h, l;
};
__device__ __forceinline__ ListRec<true> load_rec(const float4* pos, uint32_t j,
                                                  ListRec<true>) {
    return ListRec<true>{__ldg(pos + j)};
}
__device__ __forceinline__ ListRec<false> load_rec(const float4* pos, uint32_t j,
                                                   ListRec<false>) {
    ListRec<false> r;
    load_record(pos, j, r.h, r.l);
    return r;
}

// A thread per particle (current storage order f) -- or kLanes threads, lane
// l taking entries [l E, (l + 1) E) of every group of 8 (E = 8 / kLanes) --
// its list slot, its list, its neighbours' records; the force is stored at f.
// With several lanes a warp covers 32 / kLanes particles, mostly of one cell,
// whose entries at the same place of their lists lie close together in the
// same rows of cells: fewer L1 wavefronts per record gather, and the lanes of
// a particle do equal work.  A lane walks its entries in views of 8 (kLanes
// groups' parts; a group past the list's end reads as the ghost record), in
// batches of 4 (lists are padded to multiples of 8, kListFold).  Each
// batch's records are loaded one batch ahead of its pair terms, and its list
// entries -- streamed from DRAM -- one batch ahead of the records, so the
// latency of both overlaps the terms of the batch before.  Every record holds
// the image the pair needs: no periodic arithmetic per pair.  A separation
// is, for compact records, the exact integer difference of the fixed-point
// coordinates, converted and scaled by a power of two (fixed_sep); for full
// records d = (x_j,hi - x_i,hi) + (x_j,lo - x_i,lo), the first difference
// exact for nearby values.  Either way d carries one FP32 rounding.  The
// lanes of a particle are adjacent in one warp; lane 0 adds the others' sums
// in lane order, so the result does not depend on scheduling.
template <class Body, bool kCompact, bool kReplicas, bool kCount = false, int kLanes = 1>
__global__ void __launch_bounds__(256)
force_list_kernel(Body body0, DevGeom g, PairList pl, ForceOut out) {
    constexpr int kBatch = 4;
    static_assert(kListFold == 2 * kBatch, "a fold is two batches");
    static_assert(kLanes == 1 || kLanes == 2 || kLanes == 4, "1, 2 or 4 lanes per particle");
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = t / kLanes;
    const int lane = t % kLanes;
    if (kLanes == 1) {
        if (f >= g.n || *out.err) return;
    } else {
        // every lane of a particle must take the same path: the error word
        // is read once per warp (all 32 threads are present here)
        const bool failed =
            __shfl_sync(0xffffffffu, (threadIdx.x & 31) == 0 ? (*out.err != 0) : false, 0);
        if (failed || f >= g.n) return;   // f is the same for all lanes of a particle
    }
    // a batch: the pair functor of the particle's replica (its neighbours are
    // all of the same replica)
    const Body body = kReplicas ? body0.for_replica(pl.pairs, pl.rep[f], g) : body0;
    const int s = pl.lslot ? pl.lslot[f] : f;   // no slot table: storage order is list order
    float4 hh, hl;
    // compact records: the home's fixed-point coordinates
    uint32_t ux = 0u, uy = 0u, uz = 0u;
    const float unit = pl.unit;
    if (kCompact) {
        const float4 c = pl.pos[s];
        ux = __float_as_uint(c.x);
        uy = __float_as_uint(c.y);
        uz = __float_as_uint(c.z);
        hh = make_float4(0.f, 0.f, 0.f, pl.radius);
        hl = hh;
    } else {
        hh = pl.pos[2 * (size_t)s];
        hl = pl.pos[2 * (size_t)s + 1];
    }
    const float usize = 2.0f * pl.radius, us2 = usize * usize;
    typename Body::Acc acc;
    body.init(acc);
    uint32_t err = 0;
    float rmin = 3.0e38f;
    // this lane's views of 8 entries: its parts of kLanes groups each
    const int groups = pl.count[s] / kListFold;
    const int views = (groups + kLanes - 1) / kLanes;
    using Rec = ListRec<kCompact>;
    const Rec none{};
    auto terms = [&](const Rec* r) {
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            if constexpr (kCompact) {
                const float d0 = fixed_sep(r[u].h.x, ux, unit);
                const float d1 = fixed_sep(r[u].h.y, uy, unit);
                const float d2 = fixed_sep(r[u].h.z, uz, unit);
                body.template eval_list<true, kCount>(d0, d1, d2, usize, us2, acc, rmin, err,
                                                      r[u].h.w);
            } else {
                const float d0 = (r[u].h.x - hh.x) + (r[u].l.x - hl.x);
                const float d1 = (r[u].h.y - hh.y) + (r[u].l.y - hl.y);
                const float d2 = (r[u].h.z - hh.z) + (r[u].l.z - hl.z);
                const float size = hh.w + r[u].h.w;
                body.template eval_list<false, kCount>(d0, d1, d2, size, size * size, acc, rmin,
                                                       err);
            }
        }
    };
    // groups of 8 entries (one 32-byte load) one group ahead; records one
    // batch of 4 ahead of their pair terms
    constexpr int kE = kListFold / kLanes;   // entries of each group this lane takes
    const uint32_t* gp = pl.list + (size_t)s * kListFold + lane * kE;
    const size_t gs = (size_t)pl.stride * kListFold;   // one group
    const uint32_t gh = (uint32_t)pl.stride;           // the ghost record (slot n)
    // view m of this lane: its parts of groups kLanes m ... kLanes m + kLanes - 1
    // (gp at the first; group kLanes m exists)
    auto load_view = [&](const uint32_t* p, int m, uint4& a, uint4& b) {
        if constexpr (kLanes == 1) {
            load_group(p, a, b);
        } else if constexpr (kLanes == 2) {
            a = __ldg(reinterpret_cast<const uint4*>(p));
            b = 2 * m + 1 < groups ? __ldg(reinterpret_cast<const uint4*>(p + gs))
                                   : make_uint4(gh, gh, gh, gh);
        } else {
            const uint2 gg = make_uint2(gh, gh);
            const uint2 q0 = __ldg(reinterpret_cast<const uint2*>(p));
            const uint2 q1 = 4 * m + 1 < groups ? __ldg(reinterpret_cast<const uint2*>(p + gs)) : gg;
            const uint2 q2 =
                4 * m + 2 < groups ? __ldg(reinterpret_cast<const uint2*>(p + 2 * gs)) : gg;
            const uint2 q3 =
                4 * m + 3 < groups ? __ldg(reinterpret_cast<const uint2*>(p + 3 * gs)) : gg;
            a = make_uint4(q0.x, q0.y, q1.x, q1.y);
            b = make_uint4(q2.x, q2.y, q3.x, q3.y);
        }
    };
    // past the list's end the entries read as slot 0, a valid record: the
    // record loads need no condition
    uint4 ea = make_uint4(0u, 0u, 0u, 0u), eb = ea;
    Rec r[kBatch], rn[kBatch];
    if (views > 0) load_view(gp, 0, ea, eb);
    r[0] = load_rec(pl.pos, ea.x, none);
    r[1] = load_rec(pl.pos, ea.y, none);
    r[2] = load_rec(pl.pos, ea.z, none);
    r[3] = load_rec(pl.pos, ea.w, none);
    for (int m = 0; m < views; ++m) {
        const bool more = m + 1 < views;
        gp += gs * kLanes;
        uint4 na = make_uint4(0u, 0u, 0u, 0u), nb = na;
        if (more) load_view(gp, m + 1, na, nb);
        rn[0] = load_rec(pl.pos, eb.x, none);
        rn[1] = load_rec(pl.pos, eb.y, none);
        rn[2] = load_rec(pl.pos, eb.z, none);
        rn[3] = load_rec(pl.pos, eb.w, none);
        terms(r);
        r[0] = load_rec(pl.pos, na.x, none);
        r[1] = load_rec(pl.pos, na.y, none);
        r[2] = load_rec(pl.pos, na.z, none);
        r[3] = load_rec(pl.pos, na.w, none);
        terms(rn);
        body.fold(acc);
        eb = nb;
    }
    if constexpr (kLanes > 1) {
        // lane 0 adds the other lanes' sums in lane order
        const unsigned seg = (threadIdx.x & 31) & ~(unsigned)(kLanes - 1);
        const unsigned mask = ((1u << kLanes) - 1u) << seg;
        const typename Body::Acc own = acc;
#pragma unroll
        for (int o = 1; o < kLanes; ++o) body.merge_lane(acc, own, mask, o, kLanes);
#pragma unroll
        for (int o = kLanes / 2; o > 0; o >>= 1) {
            rmin = fminf(rmin, __shfl_xor_sync(mask, rmin, o, kLanes));
            err |= __shfl_xor_sync(mask, err, o, kLanes);
        }
        if (lane != 0) return;
    }
    if (kCompact) body.list_overlap(rmin, us2, err);
    body.store(out, f, acc);
    if (err) atomicOr(out.err, err);
}

// The list pass with `lanes` threads per particle (kMulti: the 2- and 4-lane
// kernels are built for this variant; otherwise one lane).
template <class Body, bool kCompact, bool kReplicas, bool kCount, bool kMulti>
cudaError_t launch_list_lanes(const Body& body, const DevGeom& g, const PairList& pl,
                              const ForceOut& out, int lanes, cudaStream_t st) {
    if constexpr (kMulti) {
        if (lanes == 2 || lanes == 4) {
            const int blocks = (int)(((long long)g.n * lanes + 255) / 256);
            if (lanes == 4)
                force_list_kernel<Body, kCompact, kReplicas, kCount, 4>
                    <<<blocks, 256, 0, st>>>(body, g, pl, out);
            else
                force_list_kernel<Body, kCompact, kReplicas, kCount, 2>
                    <<<blocks, 256, 0, st>>>(body, g, pl, out);
            return cudaGetLastError();
        }
    }
    force_list_kernel<Body, kCompact, kReplicas, kCount, 1><<<(g.n + 255) / 256, 256, 0, st>>>(
        body, g, pl, out);
    return cudaGetLastError();
}

template <class Body>
cudaError_t launch_force_list(const Body& body, const DevGeom& g, const PairList& pl,
                              const ForceOut& out, cudaStream_t st) {
    if (g.n == 0) return cudaSuccess;
    // several lanes per particle for compact records without the count; one
    // lane otherwise
    const int lanes = (pl.compact && !out.coor && (pl.lanes == 2 || pl.lanes == 4)) ? pl.lanes : 1;
    if (pl.rep) {
        if constexpr (Body::kBatchable) {
            if (pl.compact)
                return launch_list_lanes<Body, true, true, false, true>(body, g, pl, out, lanes, st);
            return launch_list_lanes<Body, false, true, false, false>(body, g, pl, out, 1, st);
        }
        return cudaErrorInvalidValue;
    }
    if (out.coor) {   // the coordination numbers with the forces (one system)
        if (pl.compact)
            return launch_list_lanes<Body, true, false, true, false>(body, g, pl, out, 1, st);
        return launch_list_lanes<Body, false, false, true, false>(body, g, pl, out, 1, st);
    }
    if (pl.compact)
        return launch_list_lanes<Body, true, false, false, true>(body, g, pl, out, lanes, st);
    return launch_list_lanes<Body, false, false, false, false>(body, g, pl, out, 1, st);
}

}  // namespace psim
