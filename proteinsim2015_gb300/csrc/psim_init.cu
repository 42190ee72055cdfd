// psim_init.cu -- seeded initial states on the host (set-up, not the hot path).
//
// The reference places particles uniformly with mt19937 and then removes
// overlaps by an O(N^2) sweep (ClusteredCore/src/system/systemInit.cpp:31-160),
// which cannot build the dense or large systems the GPU runs.  This is random
// sequential addition instead: trial positions drawn uniformly in the periodic
// box are kept when no earlier particle lies closer than min_sep, found through
// a cell grid of side >= min_sep (27 cells per trial).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/psim_gb300.h"

extern "C" void psim_internal_set_error(const char* msg);

namespace {

// SplitMix64 (Steele, Lea, Flood, OOPSLA 2014): a 64-bit state stepped by a
// Weyl increment and mixed; the 53 high bits give a double in [0, 1).
struct SplitMix {
    uint64_t x;
    uint64_t next() {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

extern "C" int psim_init_rsa(int32_t n, double box, double min_sep, uint64_t seed,
                             int64_t max_trials, double* pos) {
    if (n < 0 || !(box > 0.0) || !(min_sep >= 0.0) || (n > 0 && !pos)) {
        psim_internal_set_error("psim_init_rsa: bad arguments");
        return PSIM_ERR_INPUT;
    }
    const int s = std::max(1, std::min(1024, (int)std::floor(box / std::max(min_sep, 1e-12))));
    const double cs = box / s;
    const double sep2 = min_sep * min_sep;
    // per cell: the particles placed in it (head/next lists)
    std::vector<int> head((size_t)s * s * s, -1), next((size_t)n, -1);
    SplitMix rng{seed};
    int64_t trials = 0;
    auto cell = [&](double x) {
        int c = (int)std::floor(x / cs);
        return c < 0 ? 0 : (c >= s ? s - 1 : c);
    };
    for (int i = 0; i < n; ++i) {
        for (;;) {
            if (max_trials > 0 && ++trials > max_trials) {
                psim_internal_set_error("psim_init_rsa: no room left (the volume fraction is "
                                        "too close to the RSA jamming limit)");
                return PSIM_ERR_INIT;
            }
            const double p[3] = {rng.uniform() * box, rng.uniform() * box, rng.uniform() * box};
            const int c[3] = {cell(p[0]), cell(p[1]), cell(p[2])};
            bool ok = true;
            for (int dx = -1; dx <= 1 && ok; ++dx)
                for (int dy = -1; dy <= 1 && ok; ++dy)
                    for (int dz = -1; dz <= 1 && ok; ++dz) {
                        const int x = (c[0] + dx + s) % s, y = (c[1] + dy + s) % s,
                                  z = (c[2] + dz + s) % s;
                        for (int j = head[(size_t)x + (size_t)s * (y + (size_t)s * z)]; j >= 0;
                             j = next[j]) {
                            double r2 = 0.0;
                            for (int k = 0; k < 3; ++k) {
                                double d = pos[3 * (size_t)j + k] - p[k];
                                d -= box * std::nearbyint(d / box);
                                r2 += d * d;
                            }
                            if (r2 < sep2) {
                                ok = false;
                                break;
                            }
                        }
                    }
            if (!ok) continue;
            for (int k = 0; k < 3; ++k) pos[3 * (size_t)i + k] = p[k];
            const size_t h = (size_t)c[0] + (size_t)s * (c[1] + (size_t)s * c[2]);
            next[i] = head[h];
            head[h] = i;
            break;
        }
    }
    return PSIM_OK;
}

// ------------------------------------------------------------- on the GPU
//
// The same random sequential addition on the GPU, trial for trial: trial t
// draws SplitMix64 outputs 3t .. 3t + 2 (the generator is a Weyl sequence, so
// draw k is the mix of seed + (k + 1) * gamma) and is kept when no earlier
// kept trial lies closer than min_sep.  Trials are evaluated in chunks:
//   test     each trial of the chunk against the particles already placed
//            (a cell table of at most kRsaCap particles per cell);
//   resolve  among the chunk's survivors, a trial is kept when every earlier
//            survivor closer than min_sep is rejected, and rejected when one
//            of them is kept -- repeated until every survivor is decided (the
//            first undecided survivor is decided in each round);
//   commit   the kept trials in trial order, up to n in all.
// The particles placed and their order are those of the host version run
// with the same arithmetic (FP64, no contraction): the decision of a trial
// depends only on earlier trials, not on the chunk size.
namespace {

constexpr int kRsaCap = 16;     // placed particles per cell (a cube of side
                                // < 1.34 min_sep holds at most ~10)
constexpr int kRsaChunkCap = 32;

__device__ __forceinline__ double rsa_draw(uint64_t seed, uint64_t k) {
    uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return __dmul_rn((double)(z >> 11), 1.0 / 9007199254740992.0);
}

struct RsaArgs {
    int s;
    double box, cs, sep2;
    uint64_t seed;
    long long t0;          // first trial of the chunk
    int T;                 // trials in the chunk
    const double* placed;  // 3 per placed particle
    const int* cell_n;     // placed particles per cell
    const int* cell_id;    // kRsaCap per cell
    double* tp;            // 3 per trial of the chunk
    int* tcell;            // cell of each trial
    int* state;            // 0 undecided, 1 kept, 2 rejected
    int* ccount;           // chunk survivors per cell
    int* cid;              // kRsaChunkCap per cell: survivor indices (any order)
    int* flag;             // [0] overflow, [1] undecided count
};

__device__ __forceinline__ int rsa_cell(double x, double cs, int s) {
    int c = (int)floor(__ddiv_rn(x, cs));
    return c < 0 ? 0 : (c >= s ? s - 1 : c);
}

__device__ __forceinline__ bool rsa_close(const double* a, const double* b, double box,
                                          double sep2) {
    double r2 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double d = __dsub_rn(a[k], b[k]);
        d = __dsub_rn(d, __dmul_rn(box, rint(__ddiv_rn(d, box))));
        r2 = __dadd_rn(r2, __dmul_rn(d, d));
    }
    return r2 < sep2;
}

__global__ void rsa_test_kernel(RsaArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.T) return;
    const uint64_t k = 3ull * (uint64_t)(a.t0 + t);
    double p[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) p[d] = __dmul_rn(rsa_draw(a.seed, k + d), a.box);
    const int c[3] = {rsa_cell(p[0], a.cs, a.s), rsa_cell(p[1], a.cs, a.s),
                      rsa_cell(p[2], a.cs, a.s)};
    bool ok = true;
    for (int dx = -1; dx <= 1 && ok; ++dx)
        for (int dy = -1; dy <= 1 && ok; ++dy)
            for (int dz = -1; dz <= 1 && ok; ++dz) {
                const int x = (c[0] + dx + a.s) % a.s, y = (c[1] + dy + a.s) % a.s,
                          z = (c[2] + dz + a.s) % a.s;
                const size_t h = (size_t)x + (size_t)a.s * (y + (size_t)a.s * z);
                const int m = min(a.cell_n[h], kRsaCap);
                for (int e = 0; e < m && ok; ++e)
                    ok = !rsa_close(a.placed + 3 * (size_t)a.cell_id[h * kRsaCap + e], p, a.box,
                                    a.sep2);
            }
    a.tp[3 * (size_t)t] = p[0];
    a.tp[3 * (size_t)t + 1] = p[1];
    a.tp[3 * (size_t)t + 2] = p[2];
    const int h = c[0] + a.s * (c[1] + a.s * c[2]);
    a.tcell[t] = h;
    a.state[t] = ok ? 0 : 2;
    if (ok) {
        const int slot = atomicAdd(a.ccount + h, 1);
        if (slot < kRsaChunkCap)
            a.cid[(size_t)h * kRsaChunkCap + slot] = t;
        else
            a.flag[0] = 1;   // too many survivors in one cell: a smaller chunk
    }
}

// One round of decisions: a survivor is kept when every earlier survivor
// within min_sep is rejected, rejected when one of them is kept.
__global__ void rsa_resolve_kernel(RsaArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.T || a.state[t] != 0) return;
    const double* p = a.tp + 3 * (size_t)t;
    const int h = a.tcell[t];
    const int cx = h % a.s, cy = (h / a.s) % a.s, cz = h / (a.s * a.s);
    bool pending = false, beaten = false;
    for (int dx = -1; dx <= 1 && !beaten; ++dx)
        for (int dy = -1; dy <= 1 && !beaten; ++dy)
            for (int dz = -1; dz <= 1 && !beaten; ++dz) {
                const int x = (cx + dx + a.s) % a.s, y = (cy + dy + a.s) % a.s,
                          z = (cz + dz + a.s) % a.s;
                const size_t q = (size_t)x + (size_t)a.s * (y + (size_t)a.s * z);
                const int m = min(a.ccount[q], kRsaChunkCap);
                for (int e = 0; e < m && !beaten; ++e) {
                    const int u = a.cid[q * kRsaChunkCap + e];
                    if (u >= t) continue;
                    const int su = a.state[u];
                    if (su == 2) continue;
                    if (!rsa_close(a.tp + 3 * (size_t)u, p, a.box, a.sep2)) continue;
                    if (su == 1) beaten = true;
                    else pending = true;
                }
            }
    if (beaten) {
        a.state[t] = 2;
    } else if (!pending) {
        a.state[t] = 1;
    } else {
        atomicAdd(a.flag + 1, 1);
    }
}

// The particles placed by a chunk (indices first .. first + m - 1) into the
// cell table.
__global__ void rsa_insert_kernel(RsaArgs a, int* cell_n, int* cell_id, int first, int m) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const int i = first + k;
    const double* p = a.placed + 3 * (size_t)i;
    const int h = rsa_cell(p[0], a.cs, a.s) + a.s * (rsa_cell(p[1], a.cs, a.s) +
                                                     a.s * rsa_cell(p[2], a.cs, a.s));
    const int slot = atomicAdd(cell_n + h, 1);
    if (slot < kRsaCap)
        cell_id[(size_t)h * kRsaCap + slot] = i;
    else
        a.flag[0] = 1;
}

}  // namespace

extern "C" int psim_init_rsa_device(int32_t n, double box, double min_sep, uint64_t seed,
                                    int64_t max_trials, double* pos, int32_t device) {
    if (n < 0 || !(box > 0.0) || !(min_sep > 0.0) || (n > 0 && !pos)) {
        psim_internal_set_error("psim_init_rsa_device: bad arguments");
        return PSIM_ERR_INPUT;
    }
    const int s = std::max(1, std::min(1024, (int)std::floor(box / min_sep)));
    if (s < 3 || n == 0)  // the 27-cell search needs 3 cells a side
        return psim_init_rsa(n, box, min_sep, seed, max_trials, pos);
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        psim_internal_set_error("psim_init_rsa_device: no such device");
        return PSIM_ERR_CUDA;
    }
    const size_t ncell = (size_t)s * s * s;
    int Tmax = (int)std::min<size_t>(1u << 18, std::max<size_t>(1024, ncell / 8));
    std::vector<void*> bufs;
    auto alloc = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return p;
    };
    auto done = [&](int rc) {
        for (void* p : bufs) cudaFree(p);
        cudaSetDevice(prev);
        return rc;
    };
    RsaArgs a{};
    a.s = s;
    a.box = box;
    a.cs = box / s;
    a.sep2 = min_sep * min_sep;
    a.seed = seed;
    double* placed = (double*)alloc(24 * (size_t)n);
    int* cell_n = (int*)alloc(4 * ncell);
    int* cell_id = (int*)alloc(4 * ncell * kRsaCap);
    a.tp = (double*)alloc(24 * (size_t)Tmax);
    a.tcell = (int*)alloc(4 * (size_t)Tmax);
    a.state = (int*)alloc(4 * (size_t)Tmax);
    a.ccount = (int*)alloc(4 * ncell);
    a.cid = (int*)alloc(4 * ncell * kRsaChunkCap);
    a.flag = (int*)alloc(8);
    for (void* p : bufs)
        if (!p) {
            psim_internal_set_error("psim_init_rsa_device: out of device memory");
            return done(PSIM_ERR_CUDA);
        }
    a.placed = placed;
    a.cell_n = cell_n;
    a.cell_id = cell_id;
    if (cudaMemset(cell_n, 0, 4 * ncell) != cudaSuccess ||
        cudaMemset(a.ccount, 0, 4 * ncell) != cudaSuccess) {
        psim_internal_set_error("psim_init_rsa_device: memset failed");
        return done(PSIM_ERR_CUDA);
    }
    std::vector<double> tp;
    std::vector<int> state;
    int placed_n = 0;
    long long t0 = 0;
    int T = Tmax;
    auto fail_cuda = [&](const char* what) {
        psim_internal_set_error(what);
        return done(PSIM_ERR_CUDA);
    };
    while (placed_n < n) {
        if (max_trials > 0 && t0 >= max_trials) {
            psim_internal_set_error("psim_init_rsa: no room left (the volume fraction is too close "
                                    "to the RSA jamming limit)");
            return done(PSIM_ERR_INIT);
        }
        a.t0 = t0;
        a.T = T;
        // the chunk's survivor table starts empty
        if (cudaMemset(a.ccount, 0, 4 * ncell) != cudaSuccess || cudaMemset(a.flag, 0, 8))
            return fail_cuda("psim_init_rsa_device: memset failed");
        rsa_test_kernel<<<(T + 255) / 256, 256>>>(a);
        int flag[2] = {0, 0};
        if (cudaMemcpy(flag, a.flag, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail_cuda("psim_init_rsa_device: kernel failed");
        if (flag[0]) {   // a crowded cell among this chunk's survivors: fewer trials
            if (T <= 64) return fail_cuda("psim_init_rsa_device: survivor table overflow");
            T /= 4;
            continue;
        }
        for (int round = 0;; ++round) {
            if (cudaMemset(a.flag + 1, 0, 4) != cudaSuccess)
                return fail_cuda("psim_init_rsa_device: memset failed");
            rsa_resolve_kernel<<<(T + 255) / 256, 256>>>(a);
            int undecided = 0;
            if (cudaMemcpy(&undecided, a.flag + 1, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
                return fail_cuda("psim_init_rsa_device: kernel failed");
            if (undecided == 0) break;
            // each round decides at least the first undecided survivor
            if (round > T) return fail_cuda("psim_init_rsa_device: no progress");
        }
        // commit in trial order on the host (a few percent of the trials are kept)
        state.resize((size_t)T);
        tp.resize(3 * (size_t)T);
        if (cudaMemcpy(state.data(), a.state, 4 * (size_t)T, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(tp.data(), a.tp, 24 * (size_t)T, cudaMemcpyDeviceToHost))
            return fail_cuda("psim_init_rsa_device: copy failed");
        const int first_new = placed_n;
        for (int t = 0; t < T && placed_n < n; ++t) {
            if (state[(size_t)t] != 1) continue;
            if (max_trials > 0 && t0 + t + 1 > max_trials) {
                psim_internal_set_error("psim_init_rsa: no room left (the volume fraction is "
                                        "too close to the RSA jamming limit)");
                return done(PSIM_ERR_INIT);
            }
            for (int d = 0; d < 3; ++d) pos[3 * (size_t)placed_n + d] = tp[3 * (size_t)t + d];
            ++placed_n;
        }
        // the new particles into the device table
        const int m = placed_n - first_new;
        if (m > 0) {
            if (cudaMemcpy(placed + 3 * (size_t)first_new, pos + 3 * (size_t)first_new,
                           24 * (size_t)m, cudaMemcpyHostToDevice) != cudaSuccess)
                return fail_cuda("psim_init_rsa_device: copy failed");
            rsa_insert_kernel<<<(m + 255) / 256, 256>>>(a, cell_n, cell_id, first_new, m);
            if (cudaMemcpy(flag, a.flag, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
                return fail_cuda("psim_init_rsa_device: kernel failed");
            if (flag[0]) return fail_cuda("psim_init_rsa_device: cell table overflow");
        }
        t0 += T;
        if (T < Tmax) T = std::min(Tmax, T * 2);
    }
    return done(PSIM_OK);
}
