// psim_noalloc.cu -- the cell-list build for callers that cannot allocate
// device memory.
//
// Some hosts of this library own every byte of device memory themselves: an
// embedding engine that hands out buffers from its own pool and forbids
// cudaMalloc/cudaFree inside its step loop (they synchronise the device and
// fragment the pool), or a real-time caller that cannot take an allocation's
// latency mid-run.  They can pass their own device buffers for inputs and
// outputs, but the build also needs scratch (keys, slots, permutation, tags,
// split coordinates, per-cell counts).  Here that scratch is a file-scope
// static device array of kNoAllocBytes (32 MiB), so this entry point
// allocates nothing.
//
// Costs and rules, stated for the caller:
//   * every GPU that loads this library holds the 32 MiB array until the
//     process exits;
//   * every call looks the array's device address up (cudaGetSymbolAddress)
//     with the caller's device current, so a device reset, after which the
//     library's module is loaded again and the array may sit elsewhere, needs
//     nothing from the caller;
//   * the call waits for its own work (it reads the error word back), so it
//     blocks until the build is done and cannot be called while a stream is
//     being captured;
//   * all calls share the one array and it keeps the last call's contents:
//     calls whose work overlaps on the GPU (other streams, other host
//     threads) race on it -- serialise them;
//   * a problem too large for the array is refused with PSIM_ERR_INPUT and a
//     message giving the bytes needed.
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cmath>

#include "../../include/psim_gb300.h"
#include "psim_kernels.cuh"

using namespace psim;

namespace {

constexpr size_t kNoAllocBytes = size_t(32) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// bump allocator over the static array (256-byte aligned pieces)
struct Carve {
    char* base;
    size_t used = 0;
    void* take(size_t bytes) {
        void* p = base + used;
        used += (bytes + 255) & ~size_t(255);
        return p;
    }
};

size_t scratch_bytes(size_t n, size_t ncell) {
    auto r = [](size_t b) { return (b + 255) & ~size_t(255); };
    return r(24 * n) + 7 * r(4 * n) + r(8 * n) + r(16 * n) + 2 * r(4 * ncell) +
           r(4 * scan_scratch_ints((int)ncell)) + r(4);
}

}  // namespace

extern "C" void psim_internal_set_error(const char* msg);

static int refuse(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    psim_internal_set_error(buf);
    return code;
}

extern "C" int psim_cells_build_noalloc(const psim_geometry* gm, const double* d_pos,
                                        const double* d_radius, int32_t* d_hash_index,
                                        uint32_t* d_cell_start_end, double* d_sorted,
                                        void* stream) {
    if (!gm) return refuse(PSIM_ERR_INPUT, "geometry is NULL");
    if (gm->n_particles < 0) return refuse(PSIM_ERR_INPUT, "negative particle count");
    if (gm->cell_scale < 3 || gm->cell_scale > 256)
        return refuse(PSIM_ERR_INPUT, "cellScale %d outside [3, 256]", gm->cell_scale);
    if (!(gm->box_size > 0.0) || !(gm->cell_size > 0.0))
        return refuse(PSIM_ERR_INPUT, "box and cell size must be positive");
    if (std::fabs(gm->cell_size * gm->cell_scale - gm->box_size) > 1e-9 * gm->box_size)
        return refuse(PSIM_ERR_INPUT, "cellSize * cellScale != boxSize");
    const size_t n = (size_t)gm->n_particles;
    const size_t ncell = (size_t)gm->cell_scale * gm->cell_scale * gm->cell_scale;
    const size_t need = scratch_bytes(n, ncell);
    if (need > kNoAllocBytes)
        return refuse(PSIM_ERR_INPUT,
                      "%zu particles and %zu cells need %zu bytes of scratch; the static "
                      "scratch of psim_cells_build_noalloc holds %zu",
                      n, ncell, need, kNoAllocBytes);
    if (n > 0 && (!d_pos || !d_radius || !d_hash_index || !d_sorted))
        return refuse(PSIM_ERR_INPUT, "NULL device buffer");
    if (!d_cell_start_end) return refuse(PSIM_ERR_INPUT, "NULL device buffer");
    if (reinterpret_cast<uintptr_t>(d_sorted) % 32 != 0)
        return refuse(PSIM_ERR_INPUT, "sorted_particles must be 32-byte aligned");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return refuse(PSIM_ERR_NO_DEVICE, "no usable CUDA device (%s)", cudaGetErrorString(e));
    // The host-side name g_noalloc_scratch is not a device address.  Look the
    // address up on every call, with the caller's device current: it is cheap
    // once the module is loaded, and it stays right after a device reset.
    void* base = nullptr;
    e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
    if (e != cudaSuccess || !base)
        return refuse(PSIM_ERR_CUDA, "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));

    DevGeom g{};
    g.n = (int)n;
    g.s = gm->cell_scale;
    g.s2 = g.s * g.s;
    g.ncell = (int)ncell;
    g.L = gm->box_size;
    g.half = g.L / 2.0;
    g.cs = gm->cell_size;
    g.inv_cs = 1.0 / gm->cell_size;
    g.inv_csf = (float)g.inv_cs;
    g.hash_guard = 0.5f;  // FP64 hash everywhere: this path is not performance critical
    g.c0 = 0;
    g.p0 = 0;
    g.p1 = g.n;

    Carve c{static_cast<char*>(base)};
    double* x = static_cast<double*>(c.take(24 * n));
    int* key = static_cast<int*>(c.take(4 * n));
    int* rank = static_cast<int*>(c.take(4 * n));
    int* tmp = static_cast<int*>(c.take(4 * n));
    int* perm = static_cast<int*>(c.take(4 * n));
    int* tag_in = static_cast<int*>(c.take(4 * n));
    int* tag_out = static_cast<int*>(c.take(4 * n));
    int* cellid = static_cast<int*>(c.take(4 * n));
    double* radius_out = static_cast<double*>(c.take(8 * n));
    float4* posh = static_cast<float4*>(c.take(16 * n));
    int* count = static_cast<int*>(c.take(4 * ncell));
    int* start = static_cast<int*>(c.take(4 * ncell));
    int* scan = static_cast<int*>(c.take(4 * scan_scratch_ints((int)ncell)));
    uint32_t* err = static_cast<uint32_t*>(c.take(4));

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the array keeps the previous call's contents: clear what must start at zero
#define NA_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return refuse(PSIM_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
    } while (0)
    NA_CUDA(cudaMemsetAsync(count, 0, 4 * ncell, st));
    NA_CUDA(cudaMemsetAsync(err, 0, 4, st));
    NA_CUDA(launch_split_xyz((int)n, d_pos, nullptr, 0, x, x + n, x + 2 * n, st));
    NA_CUDA(launch_hash_count((int)n, x, x + n, x + 2 * n, g, key, rank, count, err, st));
    NA_CUDA(launch_scan(count, start, (int)ncell, scan, st));
    NA_CUDA(launch_scatter((int)n, key, rank, start, tmp, nullptr, st));
    NA_CUDA(launch_fill_int_iota((int)n, tag_in, st));
    CanonArgs ca{};
    ca.n = (int)n;
    ca.tmp = tmp;
    ca.key = key;
    ca.start = start;
    ca.count = count;
    ca.tag_in = tag_in;
    ca.radius_in = d_radius;
    ca.x = x;
    ca.y = x + n;
    ca.z = x + 2 * n;
    ca.perm = perm;
    ca.tag_out = tag_out;
    ca.radius_out = radius_out;
    ca.cellid = cellid;
    ca.posd = reinterpret_cast<double4_32a*>(d_sorted);  // {x, y, z, R}: the sorted layout
    ca.posh = posh;
    NA_CUDA(launch_canonicalize(ca, st));
    NA_CUDA(launch_export_cells((int)n, (int)ncell, cellid, tag_out, nullptr, start, count,
                                d_hash_index, d_cell_start_end, nullptr, st));
    uint32_t bits = 0;
    NA_CUDA(cudaMemcpyAsync(&bits, err, 4, cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
#undef NA_CUDA
    if (bits & EBIT_CELL) return refuse(PSIM_ERR_CELL_BOUNDS, "particle hashed outside the cell grid");
    return PSIM_OK;
}
