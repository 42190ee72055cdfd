// psim_device.cuh -- device-side building blocks shared by the kernels.
//
//   DevGeom      the cell grid (systemState's boxSize/cellSize/cellScale)
//   error bits   latched by kernels, mapped to the reference's exit codes
//   pair functors, one per IForce plugin: the __device__ form of the
//                plugin's per-pair force (AOPotential.cpp:90-110,
//                LJPotential.cpp:96-109, Calibration.cpp:75-81)
//   Philox4x32-10 counter-based Gaussians (Salmon et al., SC'11)
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace psim {

// ----------------------------------------------------------------- errors
enum : uint32_t {
    EBIT_BOUNDS = 1u,     // 7703 particle outside [0, L) after the wrap
    EBIT_OVERLAP = 2u,    // 7704 r < 0.8 (Ri + Rj)
    EBIT_NAN = 4u,        // 7705 non-finite AO force
    EBIT_CELL = 8u,       // 7702 particle hashed outside the grid
    EBIT_NOISE = 16u,     // 7706 injected noise buffer does not cover the step
    EBIT_INDEX = 32u,     // 7706 a caller-supplied index or cell range is out of bounds
    EBIT_LIST = 64u,      // 7706 a pair list is full (more neighbours within rc + skin than it holds)
};

// ----------------------------------------------------------------- geometry
struct DevGeom {
    int n;          // particles
    int s;          // cellScale
    int s2;         // s*s
    int ncell;      // s^3
    double L;       // boxSize
    double half;    // L / 2.0          (pbcDist, utilities.cpp:85)
    double half_uv; // int(L) / 2       (unitVectorAdv with int L, utilities.cpp:124)
    double cs;      // cellSize
    double inv_cs;  // 1 / cellSize (fast path of the cell hash)
    float Lhi, Llo; // L as a float pair (Lhi + Llo == L to ~1e-14)
    float inv_csf;  // 1 / cellSize in FP32 (the FP32 cell hash)
    float hash_guard; // distance from a cell face (in cells) below which FP64 decides
    // a system's place in a batch of independent replicas (one system: 0, 0, n):
    // its first global cell and its particle range in every storage order
    int c0, p0, p1;
};

// The grid of n particles in a box of edge L cut into s cells of edge cs
// (checked by the caller: s >= 3, s * cs == L).  One system: its cells and
// particles start at 0.
inline void fill_geom(int n, int s, double L, double cs, DevGeom* g) {
    g->n = n;
    g->s = s;
    g->s2 = s * s;
    g->ncell = g->s2 * s;
    g->L = L;
    g->half = L / 2.0;
    const double fl = std::floor(L);
    g->half_uv = (fl == L && L < 2147483647.0) ? (double)(((int)L) / 2) : L / 2.0;
    g->cs = cs;
    g->inv_cs = 1.0 / cs;
    g->Lhi = (float)L;
    g->Llo = (float)(L - (double)g->Lhi);
    g->inv_csf = (float)g->inv_cs;
    // FP32 hash error: x cut or rounded to FP32 (< ulp(L)) scaled by 1/cs, plus
    // the roundings of 1/cs and of the product (each ~s 2^-24 cells); 4x that
    // is the guard
    const double ex = std::ldexp(1.0, std::ilogb(std::max(L, 1.0)) - 23) * g->inv_cs +
                      2.0 * s * std::ldexp(1.0, -24);
    const double guard = 4.0 * ex + 1e-6;
    g->hash_guard = guard < 0.25 ? (float)guard : 0.5f;  // 0.5: always the FP64 path
    g->c0 = 0;
    g->p0 = 0;
    g->p1 = n;
}

// floor(x / cs) exactly as the reference computes it (systemHandling.cpp:39-41):
// a multiply by 1/cs decides unless x/cs lies within 1e-9 of an integer, in
// which case the correctly rounded division decides.
__device__ __forceinline__ int cell_coord(double x, const DevGeom& g) {
    double q = x * g.inv_cs;
    double f = floor(q);
    double fr = q - f;
    if (fr > 1e-9 && fr < 1.0 - 1e-9) return (int)f;
    return (int)floor(x / g.cs);
}

// x = hi + lo: hi is x with its significand cut to FP32's 24 bits (toward
// zero), lo the remainder rounded to FP32 (|hi + lo - x| <= 2^-47 |x|).  Built
// from the bits of x with integer and FP32 operations only: on GB300 the FP64
// unit, which also performs double<->float conversions, runs at 1/64 of the
// FP32 rate.  Positions outside [2^-74, 2^127) in magnitude are not used
// here: below 2^-126 hi = 0, below 2^-74 lo = 0.
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t top = (uint32_t)(b >> 32);
    const uint32_t sign = top & 0x80000000u;
    const int e = (int)((top >> 20) & 0x7FFu);               // biased FP64 exponent
    const uint32_t m23 = (uint32_t)(b >> 29) & 0x7FFFFFu;    // the significand's top 23 bits
    const uint32_t rem = (uint32_t)b & 0x1FFFFFFFu;          // the 29 bits below them
    hi = (e > 896 && e < 1151) ? __uint_as_float(sign | ((uint32_t)(e - 896) << 23) | m23) : 0.f;
    // rem is an integer in units of 2^(e - 1075)
    const float unit = (e > 948) ? __uint_as_float((uint32_t)(e - 948) << 23) : 0.f;
    const float r = __uint2float_rn(rem) * unit;
    lo = sign ? -r : r;
}

// x cut to FP32 toward zero (the hi part of split_f64), by integer operations.
__device__ __forceinline__ float f32_trunc(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t top = (uint32_t)(b >> 32);
    const int e = (int)((top >> 20) & 0x7FFu);
    const uint32_t m23 = (uint32_t)(b >> 29) & 0x7FFFFFu;
    return (e > 896 && e < 1151)
               ? __uint_as_float((top & 0x80000000u) | ((uint32_t)(e - 896) << 23) | m23)
               : 0.f;
}

// x cut to FP32 toward zero like f32_trunc, except that a value beyond the
// FP32 range becomes an infinity and a NaN stays a NaN.
__device__ __forceinline__ float f32_cut(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t top = (uint32_t)(b >> 32);
    const uint32_t sign = top & 0x80000000u;
    const int e = (int)((top >> 20) & 0x7FFu);
    const uint32_t m23 = (uint32_t)(b >> 29) & 0x7FFFFFu;
    const bool nan = e == 2047 && (b << 12) != 0ull;
    const uint32_t big = sign | 0x7F800000u | (nan ? 0x400000u : 0u);
    return __uint_as_float(e >= 1151 ? big
                                     : (e > 896 ? sign | ((uint32_t)(e - 896) << 23) | m23 : sign));
}

// A float widened to double exactly, by integer operations (FP32 subnormals,
// which the noise never produces, become zero).
__device__ __forceinline__ double widen_f32(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xFFu;
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    const unsigned long long ed = e == 0u ? 0ull : (e == 255u ? 2047ull : (unsigned long long)(e + 896u));
    const unsigned long long m = e == 0u ? 0ull : (unsigned long long)(b & 0x7FFFFFu) << 29;
    return __longlong_as_double((long long)(sign | (ed << 52) | m));
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// A position held as a float pair (h + l) moved by (sx, sy, sz) boxes, with
// the box L = Lhi + Llo: the high parts exactly by TwoSum, the low parts
// absorbing the rounding.
__device__ __forceinline__ void image_shift(float4& h, float4& l, int sx, int sy, int sz,
                                            float Lhi, float Llo) {
    float ex, ey, ez;
    two_sum(h.x, (float)sx * Lhi, h.x, ex);
    two_sum(h.y, (float)sy * Lhi, h.y, ey);
    two_sum(h.z, (float)sz * Lhi, h.z, ez);
    l.x = (l.x + ex) + (float)sx * Llo;
    l.y = (l.y + ey) + (float)sy * Llo;
    l.z = (l.z + ez) + (float)sz * Llo;
}

// Periodic images a pair list needs of one particle: flag 2 bits per axis
// (0: none, 1: the +L image -- the particle is within r of the low face --,
// 3: the -L image, near the high face).  The images of a particle are its
// copies shifted along every non-empty subset of its flagged axes, numbered
// by the subset's bits in x, y, z order (1 .. 2^axes - 1).
__device__ __forceinline__ uint32_t halo_flags(const float4& h, float r, float L) {
    uint32_t f = 0;
    f |= h.x < r ? 1u : (h.x > L - r ? 3u : 0u);
    f |= (h.y < r ? 1u : (h.y > L - r ? 3u : 0u)) << 2;
    f |= (h.z < r ? 1u : (h.z > L - r ? 3u : 0u)) << 4;
    return f;
}
__device__ __forceinline__ int halo_axis(uint32_t flags, int axis) {
    return (int)(flags << (30 - 2 * axis)) >> 30;  // sign-extend the 2-bit field
}
// The number of images of a particle with these flags.
__device__ __forceinline__ int halo_copies(uint32_t flags) {
    const int axes = (flags & 3u ? 1 : 0) + (flags & 12u ? 1 : 0) + (flags & 48u ? 1 : 0);
    return (1 << axes) - 1;
}
// Image `num` (1 .. halo_copies) of a particle: its shift per axis.
__device__ __forceinline__ void halo_shift(uint32_t flags, int num, int sh[3]) {
    int bit = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int fk = halo_axis(flags, k);
        sh[k] = 0;
        if (fk != 0) {
            if (num & (1 << bit)) sh[k] = fk;
            ++bit;
        }
    }
}
// ------------------------------------------------- pair-list position records
// A full record is 32 bytes: {x, y, z, R} high parts and the low parts.  When
// every particle has the same radius a compact 16-byte record suffices: each
// coordinate as a 32-bit fixed-point number, the position in units of
// unit = 2^-k rounded to the nearest and taken modulo 2^32, and in .w an r^2
// bias (0; the ghost record's is kGhostBias, which puts it out of range of
// every particle).  k is chosen so that every separation a list can hold is
// below 2^31 units: the separation of two records is then the exact integer
// difference of their coordinates (wrapping modulo 2^32 cancels), and one
// conversion to FP32 and a power-of-two scale make it a float with a single
// rounding.  Each coordinate is within one unit of the position (unit
// 2^-27 ~ 7.5e-9 for LJ rc 2.5 with skin 0.4, fixed_unit).
constexpr float kGhostBias = 1e30f;
__device__ __forceinline__ uint32_t fixed_coord(float h, float l, float inv_unit) {
    // h 2^k is exact (a power-of-two scale) and an integer for |h| >= 2^(24-k);
    // the low part adds its rounded share
    const long long a = __float2ll_rn(h * inv_unit);
    const long long b = (long long)__float2int_rn(l * inv_unit);
    return (uint32_t)(unsigned long long)(a + b);
}
__device__ __forceinline__ float4 compact_record(const float4& h, const float4& l,
                                                 float inv_unit) {
    return make_float4(__uint_as_float(fixed_coord(h.x, l.x, inv_unit)),
                       __uint_as_float(fixed_coord(h.y, l.y, inv_unit)),
                       __uint_as_float(fixed_coord(h.z, l.z, inv_unit)), 0.f);
}
// The separation coordinate b - a of two compact-record coordinates (raw
// bits), in length units: the integer difference, converted and scaled.
__device__ __forceinline__ float fixed_sep(float b, uint32_t a, float unit) {
    return (float)(int)(__float_as_uint(b) - a) * unit;
}
// record `slot` of a full (inv_unit == 0) or compact record array
__device__ __forceinline__ void store_record(float4* pos, float inv_unit, size_t slot,
                                             const float4& h, const float4& l) {
    if (inv_unit != 0.f) {
        pos[slot] = compact_record(h, l, inv_unit);
    } else {
        pos[2 * slot] = h;
        pos[2 * slot + 1] = l;
    }
}

// Writes the images of a particle (positions h, l) into its halo records
// base + num - 1 of `pos` (the records after the ghost).
__device__ __forceinline__ void halo_write(float4* pos, float inv_unit, int base, uint32_t flags,
                                           const float4& h, const float4& l, float Lhi,
                                           float Llo) {
    const int m = halo_copies(flags);
    for (int num = 1; num <= m; ++num) {
        int sh[3];
        halo_shift(flags, num, sh);
        float4 hh = h, ll = l;
        image_shift(hh, ll, sh[0], sh[1], sh[2], Lhi, Llo);
        store_record(pos, inv_unit, (size_t)(base + num - 1), hh, ll);
    }
}

// Neighbour cell index wrapped into [0, s) as the reference does
// ((c % s) + s when negative, AOPotential.cpp:154-160), and the periodic
// image it implies (-1, 0 or +1 boxes).
// The spacing of floats at x (x > 0 and normal, 2^(e-23) for x in [2^e, 2^(e+1))),
// from the exponent bits; the smallest normal float when that is smaller.
__device__ __forceinline__ float ulp_of(float x) {
    const int eb = (int)((__float_as_uint(x) >> 23) & 0xffu) - 23;
    return __uint_as_float((uint32_t)(eb > 1 ? eb : 1) << 23);
}

__device__ __forceinline__ int wrap_cell(int c, int s, int& shift) {
    int w = c % s;
    if (w < 0) w += s;
    shift = (c - w) / s;
    return w;
}

// ------------------------------------------------------------ pair functors
// fnet64: the plugin's FP64 per-pair magnitude in the reference's operation
// order, except that integer powers use binary powering and divisions by r2
// or r multiply by 1/r (a few ulp, far inside the 1e-12 parity tolerance).
// It is host-callable too: a plugin's CPU getAcceleration (the reference's
// per-particle entry) evaluates the same functor.
// fnet32: the same formula in FP32 for the mixed form.

template <typename T>
__host__ __device__ __forceinline__ T powi_binary(T base, int e) {  // utilities.cpp:144-154
    T ans = T(1);
    while (e) {
        if (e & 1) ans *= base;
        e >>= 1;
        base *= base;
    }
    return ans;
}

// powi_binary with the exponent known at compile time: the same products in
// the same order (multiplying by the initial 1 is exact), fully unrolled.
template <int N, typename T>
__host__ __device__ __forceinline__ T powi_fixed(T base) {
    T ans = T(1);
#pragma unroll
    for (int e = N; e; e >>= 1) {
        if (e & 1) ans *= base;
        base *= base;
    }
    return ans;
}

template <typename T>
__host__ __device__ __forceinline__ T pow36(T rinv) {
    T r2 = rinv * rinv, r4 = r2 * r2, r8 = r4 * r4, r16 = r8 * r8, r32 = r16 * r16;
    return r32 * r4;
}

// AOPotential: fNet = -(36 r^-38 + coEff1/r + coEff2 r)   (AOPotential.cpp:90-99)
struct AOPair {
    double rc2, c1, c2;
    float rc2f, c1f, c2f;
    static constexpr bool kCheckNan = true;
    __host__ __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double) const {
        double r36 = pow36(rinv);
        double r38 = r36 * (rinv * rinv);
        double f = 36.0 * r38 + c1 * rinv + c2 * r;
        return -f;
    }
    __device__ __forceinline__ float fnet32(float r2, float r, float rinv, float) const {
        float r36 = pow36(rinv);
        float r38 = r36 * (rinv * rinv);
        return -(36.0f * r38 + c1f * rinv + c2f * r);
    }
    // the pair energy whose derivative is fnet64 (u' = fNet), zero at the
    // cutoff: 36/37 (r^-37 - rc^-37) + coEff1 ln(rc/r) + coEff2 (rc^2 - r^2)/2
    __host__ __device__ __forceinline__ double u64(double r2, double, double rinv, double) const {
        const double rc = sqrt(rc2), rcinv = 1.0 / rc;
        return (36.0 / 37.0) * (pow36(rinv) * rinv - pow36(rcinv) * rcinv) + c1 * log(rc * rinv) +
               0.5 * c2 * (rc2 - r2);
    }
};

// LennardJones: fNet = -kT wd [(2L-1) 4n L / r + yukStr e^{-r/lambda} (lambda + r)/r^2],
// L = (size/r)^n                                          (LJPotential.cpp:96-109)
struct LJPair {
    double rc2, kTwd, four_n, yuk, lambda, inv_lambda;
    float rc2f, kTwdf, four_nf, yukf, lambdaf, inv_lambdaf;
    int n;
    static constexpr bool kCheckNan = false;
    __host__ __device__ __forceinline__ double fnet64(double r2, double r, double rinv, double size) const {
        double lj = powi_binary(size * rinv, n);
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
        float lj = powi_binary(size * rinv, n);
        float attract = (2.0f * lj - 1.0f) * (four_nf * rinv * lj);
        float repel = 0.0f;
        if (yukf != 0.0f) repel = __expf(-r * inv_lambdaf) * (rinv * rinv * (lambdaf + r) * yukf);
        return -kTwdf * (attract + repel);
    }
    // the pair energy whose derivative is fnet64, zero at the cutoff:
    // kT wd [4 (L^2 - L) + yukStr lambda e^{-r/lambda} / r] - (the same at rc)
    __host__ __device__ __forceinline__ double u64(double, double r, double rinv, double size) const {
        const double rc = sqrt(rc2);
        const double L = powi_binary(size * rinv, n), Lc = powi_binary(size / rc, n);
        double u = 4.0 * ((L * L - L) - (Lc * Lc - Lc));
        if (yuk != 0.0)
            u += yuk * lambda * (exp(-r * inv_lambda) * rinv - exp(-rc * inv_lambda) / rc);
        return kTwd * u;
    }
};

// Calibration: fNet = -36 r^-37                           (Calibration.cpp:75-81)
struct CalPair {
    double rc2;
    float rc2f;
    static constexpr bool kCheckNan = false;
    __host__ __device__ __forceinline__ double fnet64(double, double, double rinv, double) const {
        return -(36.0 * (pow36(rinv) * rinv));
    }
    __device__ __forceinline__ float fnet32(float, float, float rinv, float) const {
        return -(36.0f * (pow36(rinv) * rinv));
    }
    // the pair energy whose derivative is fnet64, zero at the cutoff: r^-36 - rc^-36
    __host__ __device__ __forceinline__ double u64(double, double, double rinv, double) const {
        return pow36(rinv) - pow36(1.0 / sqrt(rc2));
    }
};

// The functors of the three reference plugins from their settings values,
// with the FP32 copies the mixed form reads.
inline void ao_coeffs(double kT, double wd, double rc, double* c1, double* c2) {  // AOPotential.cpp:50-55
    double q = rc / (rc - 1.0);
    double a1 = -kT * wd * q * q * q;
    double a2 = -3.0 / (2.0 * rc);
    double a3 = 1.0 / (2.0 * rc * rc * rc);
    *c1 = -a1 * a2;
    *c2 = -3.0 * a1 * a3;
}
inline AOPair make_ao_pair(double kT, double wd, double rc) {
    AOPair p{};
    ao_coeffs(kT, wd, rc, &p.c1, &p.c2);
    p.rc2 = rc * rc;
    p.rc2f = (float)p.rc2;
    p.c1f = (float)p.c1;
    p.c2f = (float)p.c2;
    return p;
}
inline LJPair make_lj_pair(double kT, double wd, int n, double yuk, double lambda, double rc) {
    LJPair p{};
    p.rc2 = rc * rc;
    p.kTwd = kT * wd;
    p.n = n;
    p.four_n = 4.0 * n;
    p.yuk = yuk;
    p.lambda = lambda;
    p.inv_lambda = 1.0 / lambda;
    p.rc2f = (float)p.rc2;
    p.kTwdf = (float)p.kTwd;
    p.four_nf = (float)p.four_n;
    p.yukf = (float)p.yuk;
    p.lambdaf = (float)p.lambda;
    p.inv_lambdaf = (float)p.inv_lambda;
    return p;
}
inline CalPair make_cal_pair(double rc) {
    CalPair p{};
    p.rc2 = rc * rc;
    p.rc2f = (float)p.rc2;
    return p;
}

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): counter (step, draw-group, particle, 0), key
// (seed, stream tag).
struct Philox4 {
    uint32_t v[4];
};

__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                 uint32_t c3, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
        uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += W0; k1 += W1;
    }
    return Philox4{{c0, c1, c2, c3}};
}

// Two Gaussians from two 32-bit words by the Box-Muller transform in FP32
// (the reference itself stores every other deviate as a float,
// fastRandom.h:16).
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
    float u1 = ((float)(a >> 8) + 1.0f) * (1.0f / 16777216.0f);  // (0, 1]
    float u2 = (float)(b >> 8) * (1.0f / 16777216.0f);            // [0, 1)
    float rad = sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    z0 = rad * cs;
    z1 = rad * sn;
}

// Six Gaussians for (particle tag, step): the normal step's xi_x..z, mem_x..z.
__device__ __forceinline__ void philox_gaussians6f(uint32_t seed, uint32_t tag, uint32_t step,
                                                   float g[6]) {
    Philox4 a = philox4x32_10(step, 0u, tag, 0u, seed, 0x5053494Du);
    Philox4 b = philox4x32_10(step, 1u, tag, 0u, seed, 0x5053494Du);
    box_muller(a.v[0], a.v[1], g[0], g[1]);
    box_muller(a.v[2], a.v[3], g[2], g[3]);
    box_muller(b.v[0], b.v[1], g[4], g[5]);
}
__device__ __forceinline__ void philox_gaussians6(uint32_t seed, uint32_t tag, uint32_t step,
                                                  double g[6]) {
    float f[6];
    philox_gaussians6f(seed, tag, step, f);
#pragma unroll
    for (int k = 0; k < 6; ++k) g[k] = widen_f32(f[k]);
}

}  // namespace psim
