// psim_api.cu -- host implementation of the C ABI (include/psim_gb300.h).
//
// Validation, settings.cfg parsing for the plugin parameters, the reference-
// layout drop-ins, and the device-resident system whose step is
//   force -> memset(next counts) -> vGB (+hash, count) -> scan -> scatter ->
//   canonicalise (+gather, step counter)
// captured once per buffer phase into CUDA graphs.
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/psim_gb300.h"
#include "psim_kernels.cuh"

using namespace psim;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define PSIM_CUDA(call)                                                                     \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(PSIM_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                \
    } while (0)

int code_from_bits(uint32_t bits) {
    // the reference's exit order inside a step: force pass (overlap, NaN),
    // then the integrator (bounds), then the hash
    if (bits & EBIT_OVERLAP) return PSIM_ERR_OVERLAP;
    if (bits & EBIT_NAN) return PSIM_ERR_NAN_FORCE;
    if (bits & EBIT_BOUNDS) return PSIM_ERR_PARTICLE_BOUNDS;
    if (bits & EBIT_CELL) return PSIM_ERR_CELL_BOUNDS;
    if (bits & (EBIT_NOISE | EBIT_INDEX | EBIT_LIST)) return PSIM_ERR_INPUT;
    return PSIM_OK;
}

const char* bits_text(uint32_t bits) {
    if (bits & EBIT_OVERLAP) return "significant particle overlap (r < 0.8 (Ri + Rj))";
    if (bits & EBIT_NAN) return "non-finite force";
    if (bits & EBIT_BOUNDS) return "particle out of bounds after the periodic wrap";
    if (bits & EBIT_CELL) return "particle hashed outside the cell grid";
    if (bits & EBIT_NOISE) return "injected noise does not cover the step";
    if (bits & EBIT_INDEX) return "an index or cell range in the input is out of bounds";
    if (bits & EBIT_LIST)
        return "pair list full: a particle has more neighbours within cutOff + skin than the "
               "list holds (lower the skin)";
    return "";
}

// ------------------------------------------------------------- settings.cfg

// config.cpp:27-56: "key = value" lines, '#' in column 0 starts a comment,
// whitespace around key and value is trimmed.  Values parse like std::stod /
// std::stoi: the leading number counts ("10;" is 10).
struct Settings {
    std::vector<std::pair<std::string, std::string>> kv;
    explicit Settings(const char* text) {
        if (!text) return;
        const char* p = text;
        while (*p) {
            const char* e = p;
            while (*e && *e != '\n') ++e;
            std::string line(p, e);
            if (!line.empty() && line.back() == '\r') line.pop_back();
            if (!line.empty() && line[0] != '#') {
                size_t eq = line.find('=');
                std::string key = line.substr(0, eq), val = eq == std::string::npos ? "" : line.substr(eq + 1);
                auto trim = [](std::string& s) {
                    size_t a = s.find_first_not_of(" \t\r\n\v\f");
                    size_t b = s.find_last_not_of(" \t\r\n\v\f");
                    s = (a == std::string::npos) ? std::string() : s.substr(a, b - a + 1);
                };
                trim(key);
                trim(val);
                bool found = false;
                for (auto& q : kv)
                    if (q.first == key) { q.second = val; found = true; }
                if (!found) kv.emplace_back(key, val);
            }
            p = *e ? e + 1 : e;
        }
    }
    const std::string* find(const std::string& k) const {
        for (auto& q : kv)
            if (q.first == k) return &q.second;
        return nullptr;
    }
    bool get_double(const std::string& k, double def, double* out) const {
        const std::string* v = find(k);
        if (!v) { *out = def; return true; }
        char* end = nullptr;
        double d = strtod(v->c_str(), &end);
        if (end == v->c_str()) return false;
        *out = d;
        return true;
    }
    bool get_int(const std::string& k, int def, int* out) const {
        const std::string* v = find(k);
        if (!v) { *out = def; return true; }
        char* end = nullptr;
        long d = strtol(v->c_str(), &end, 10);
        if (end == v->c_str()) return false;
        *out = (int)d;
        return true;
    }
};

// ------------------------------------------------------------- validation

// plugin: the force runs through a plugin's device entry, which owns the
// meaning of every parameter but the cutoff.
int check_params(const psim_force_params* p, bool plugin = false) {
    if (!p) return fail(PSIM_ERR_INPUT, "force params are NULL");
    if (plugin) {
        if (!(p->cutoff > 0.0) || !std::isfinite(p->cutoff))
            return fail(PSIM_ERR_INPUT, "cutOff must be positive and finite");
        if (p->kind == 4 && !(p->cutoff2 > 0.0))
            return fail(PSIM_ERR_INPUT, "the composite needs the LJ part's cutOff");
        return PSIM_OK;
    }
    if (p->kind == PSIM_FORCE_PLUGIN)
        return fail(PSIM_ERR_INPUT, "force kind PSIM_FORCE_PLUGIN needs the plugin's psim_force_launch");
    if (p->kind < 1 || p->kind > 4) return fail(PSIM_ERR_INPUT, "unknown force kind %d", p->kind);
    if (!(p->cutoff > 0.0) || !std::isfinite(p->cutoff))
        return fail(PSIM_ERR_INPUT, "cutOff must be positive and finite");
    if ((p->kind == 1 || p->kind == 4) && !(p->cutoff > 1.0))
        return fail(PSIM_ERR_INPUT, "AO cutOff must exceed 1 (coefficients divide by cutOff - 1)");
    if (p->kind == 2 || p->kind == 4) {
        if (p->lj_num < 0 || p->lj_num > 64) return fail(PSIM_ERR_INPUT, "ljNum out of range");
        if (!(p->debye_length > 0.0)) return fail(PSIM_ERR_INPUT, "debyeLength must be positive");
    }
    if (p->kind == 4 && !(p->cutoff2 > 0.0))
        return fail(PSIM_ERR_INPUT, "the composite needs the LJ part's cutOff");
    return PSIM_OK;
}

double max_cutoff(const psim_force_params* p) {
    return p->kind == 4 ? std::max(p->cutoff, p->cutoff2) : p->cutoff;
}

// The unit 2^-k of compact list records (compact_record).  A listed pair is
// within rc + skin at the build and each particle moves less than skin / 2
// before the next one, so separations stay below B = rc + 2 skin + 1; k is
// the largest with 2 B 2^k <= 2^31, so that the integer difference of two
// coordinates never wraps (B < 2^(ilogb(B) + 1)).
float fixed_unit(double rc, double skin) {
    const double B = rc + 2.0 * skin + 1.0;
    return (float)std::ldexp(1.0, std::ilogb(B) + 2 - 31);
}

int make_geom(const psim_geometry* gm, double rc_max, DevGeom* g) {
    if (!gm) return fail(PSIM_ERR_INPUT, "geometry is NULL");
    if (gm->n_particles < 0) return fail(PSIM_ERR_INPUT, "negative particle count");
    if (gm->cell_scale < 3)
        return fail(PSIM_ERR_INPUT, "cellScale %d < 3: the 27-cell stencil would visit a cell twice",
                    gm->cell_scale);
    if (gm->cell_scale > 256) return fail(PSIM_ERR_INPUT, "cellScale %d > 256", gm->cell_scale);
    if (!(gm->box_size > 0.0) || !(gm->cell_size > 0.0))
        return fail(PSIM_ERR_INPUT, "box and cell size must be positive");
    double span = gm->cell_size * gm->cell_scale;
    if (std::fabs(span - gm->box_size) > 1e-9 * gm->box_size)
        return fail(PSIM_ERR_INPUT, "cellSize * cellScale (%.17g) != boxSize (%.17g)", span,
                    gm->box_size);
    if (rc_max > 0.0 && gm->cell_size < rc_max)
        return fail(PSIM_ERR_INPUT, "cellSize %.9g is below the cutoff %.9g", gm->cell_size, rc_max);
    fill_geom(gm->n_particles, gm->cell_scale, gm->box_size, gm->cell_size, g);
    return PSIM_OK;
}


// The FP32 candidate test sees positions rounded to FP32 (ulp(L)/2 each),
// L rounded (ulp(L)/2), the imaged home position rounded (ulp(L)) and the
// difference rounded: a separation is off by at most ~4.3 ulp(L), so the
// test's radius is widened by 8 ulp(L).
float prefilter_r2(double r, double L) {
    double ulpL = std::ldexp(1.0, std::ilogb(std::max(L, 1.0)) - 23);
    double rpre = r * (1.0 + 1e-6) + 8.0 * ulpL + 1e-6;
    return (float)(rpre * rpre * (1.0 + 1e-6));
}

// The pair list's sizes for cutoff rc, skin and grid g: the entries per
// particle (room for 1.5x the mean number of neighbours within rc + skin,
// + 32), the list radius squared (the FP32 test's widened bound), the
// rebuild test's displacement squared (half the skin, less the FP32 rounding
// of the positions, each off by ulp(L)/2), the halo radius (beyond the list
// test's radius, so every pair the build finds across an edge has an image)
// and the halo records to hold.
struct ListSizes {
    int cap;
    float pre, disp2, hr;
    int hcap;
};
ListSizes list_sizes(double rc, double skin, const DevGeom& g) {
    ListSizes z{};
    const double rl = rc + skin;
    const double mean = 4.0 / 3.0 * M_PI * rl * rl * rl * g.n / (g.L * g.L * g.L);
    z.cap = ((int)(1.5 * mean) + 32 + 31) / 32 * 32;
    z.pre = prefilter_r2(rl, g.L);
    const double ulpL = std::ldexp(1.0, std::ilogb(std::max(g.L, 1.0)) - 23);
    const double dmax = 0.5 * skin * (1.0 - 1e-3) - 4.0 * ulpL;
    z.disp2 = dmax > 0.0 ? (float)(dmax * dmax) : 0.f;
    z.hr = (float)(std::sqrt((double)z.pre) + 1e-3 * rl + 16.0 * ulpL);
    const double p = 2.0 * z.hr / g.L;   // a particle's chance of an image per axis
    const double expect = g.n * ((1.0 + p) * (1.0 + p) * (1.0 + p) - 1.0);
    z.hcap = (int)std::min(std::min(7.0 * g.n, 1.3 * expect + 1024.0), (double)kHaloBaseMax);
    return z;
}

// The skin of the force drop-in's pair list on grid g: `want` (clamped to
// the room the cell size leaves over cutOff), or with want < 0 the smaller of
// 0.4 and that room, if at least 0.1; 0: no skin.
double dropin_skin(double want, const DevGeom& g, double rc) {
    const double room = (g.cs - rc) * (1.0 - 1e-9);
    if (room <= 0.0 || want == 0.0) return 0.0;
    if (want > 0.0) return std::min(want, room);
    const double s = std::min(0.4, room);
    return s >= 0.1 ? s : 0.0;
}

ForceSetup make_setup(const psim_force_params* p, double L) {
    ForceSetup fs{};
    fs.kind = p->kind;
    const double rc_lj = p->kind == 4 ? p->cutoff2 : p->cutoff;
    const double wd_lj = p->kind == 4 ? p->well_depth2 : p->well_depth;
    fs.ao = make_ao_pair(p->kT, p->well_depth, p->cutoff);
    fs.lj = make_lj_pair(p->kT, wd_lj, p->lj_num, p->yukawa_strength, p->debye_length, rc_lj);
    fs.cal = make_cal_pair(p->cutoff);
    fs.rc_max = max_cutoff(p);
    fs.pre_rc2f = prefilter_r2(fs.rc_max, L);
    fs.lj_pure = p->kind == PSIM_FORCE_LJ && p->yukawa_strength == 0.0;
    return fs;
}

// Force-pass layout: a warp per 32 consecutive sorted particles (rows), or a
// block per home cell whose homes share one staged 27-cell neighbourhood
// (cells).  Rows is the default: on the rho = 0.8 LJ liquid at 2^20
// particles (13 per cell) it measured 0.67 ms against 0.71 ms for cells.
// PSIM_FORCE_PASS=cells|rows picks one (both give the same forces up to
// summation order); it is read when a system or a drop-in force evaluation is
// set up.
int choose_tile(const DevGeom&) {
    if (const char* v = std::getenv("PSIM_FORCE_PASS")) {
        if (!std::strcmp(v, "cells")) return 1;
    }
    return 0;
}

// The mixed form's 27-cell walk: the direct walk (0), or as PSIM_FORCE_WALK
// names it ("staged": 1, "direct": 2), for measurement.
int choose_walk() {
    if (const char* v = std::getenv("PSIM_FORCE_WALK")) {
        if (!std::strcmp(v, "staged")) return 1;
        if (!std::strcmp(v, "direct")) return 2;
    }
    return 0;
}

// One force pass: the library's own functor for the parameters' kind, or a
// plugin's device entry (psim_force_launch) with the same arrays.  pass:
// psim_force_pass; cv for the cell walks, pl for the pair list.
struct ForceRunner {
    const ForceSetup* fs;
    psim_force_launch_fn plugin;
    const psim_force_params* params;
    cudaError_t run(int pass, const DevGeom& g, const CellView* cv, const PairList* pl,
                    const ForceOut& out, cudaStream_t st) const {
        if (!plugin) {
            if (pass == PSIM_PASS_LIST) return launch_forces_list(*fs, g, *pl, out, st);
            if (pass == PSIM_PASS_FP64) return launch_forces_fp64(*fs, g, *cv, out, st);
            return launch_forces_mixed(*fs, g, *cv, out, st);
        }
        psim_force_args a{};
        a.abi = PSIM_FORCE_ABI;
        a.pass = pass;
        a.params = params;
        a.n_particles = g.n;
        a.cell_scale = g.s;
        a.box_size = g.L;
        a.cell_size = g.cs;
        if (cv) {
            a.pos_fp64 = cv->posd;
            a.pos_hi = cv->posh;
            a.pos_lo = cv->posl;
            a.cell_id = cv->cellid;
            a.cell_start = cv->cstart;
            a.cell_count = cv->ccount;
        }
        a.prefilter_r2 = fs->pre_rc2f;
        a.tile = fs->tile;
        if (pl) {
            a.list_pos = pl->pos;
            a.list_count = pl->count;
            a.list = pl->list;
            a.list_stride = pl->stride;
            a.list_compact = pl->compact;
            a.list_radius = pl->radius;
            a.list_unit = pl->unit;
        }
        a.fx = out.fx;
        a.fy = out.fy;
        a.fz = out.fz;
        a.err = out.err;
        a.gate = out.gate;
        // the plugin's own CUDA runtime reports its launch errors as a status
        return plugin(&a, st) == PSIM_OK ? cudaSuccess : cudaErrorLaunchFailure;
    }
};

// brownianIntegrator.cpp:27-99 with setupHigh/setupLow/setupZero (:111-175)
void vgb_coeffs(double gamma, double dt, double kT, psim_vgb_coeffs* c) {
    double y = gamma * dt;
    c->y = y;
    {
        double ty = 2.0 * y;
        c->coeff0 = exp(-y);
        double aa1 = 1.0 - c->coeff0;
        double aa2 = 0.5 * y * (1.0 + c->coeff0) - aa1;
        double aa3 = y - aa1;
        c->coeff1 = aa1 / y;
        c->coeff2 = aa2 / (y * y);
        c->coeff3 = aa3 / (y * y);
        c->sig1 = 2.0 * y - 3.0 + 4.0 * exp(-y) - exp(-ty);
        c->sig2 = -2.0 * y - 3.0 + 4.0 * exp(y) - exp(ty);
        c->gn = exp(y) - ty - exp(-y);
        c->goy2 = c->gn / (y * y);
        c->goy3 = c->gn / (y * y * y);
        c->hn = y / (exp(y) - exp(-y));
    }
    if (gamma < 0.05) {  // series expansion (setupLow); coEff0 keeps setupHigh's value
        double y1 = y, y2 = y1 * y1, y3 = y2 * y1, y4 = y3 * y1, y5 = y4 * y1;
        double y6 = y5 * y1, y7 = y6 * y1, y8 = y7 * y1, y9 = y8 * y1;
        c->coeff1 = 1.0 - 0.5 * y1 + (1.0 / 6.0) * y2 - (1.0 / 24.0) * y3 + (1.0 / 120.0) * y4;
        c->coeff2 = (1.0 / 12.0) * y1 - (1.0 / 24.0) * y2 + (1.0 / 80.0) * y3 - (1.0 / 360.0) * y4;
        c->coeff3 = 0.5 - (1.0 / 6.0) * y1 + (1.0 / 24.0) * y2 - (1.0 / 120.0) * y3;
        c->sig1 = +(2.0 / 3.0) * y3 - 0.5 * y4 + (7.0 / 30.0) * y5 - (1.0 / 12.0) * y6
                  + (31.0 / 1260.0) * y7 - (1.0 / 160.0) * y8 + (127.0 / 90720.0) * y9;
        c->sig2 = -(2.0 / 3.0) * y3 - 0.5 * y4 - (7.0 / 30.) * y5 - (1.0 / 12.0) * y6
                  - (31.0 / 1260.0) * y7 - (1.0 / 160.0) * y8 - (127.0 / 90720.0) * y9;
        c->goy2 = (1.0 / 3.0) * y1 + (1.0 / 60.0) * y3;
        c->goy3 = 1.0 / 3.0 + (1.0 / 60.0) * y2;
        c->hn = 0.5 - (1.00 / 12.0) * y2 + (7.0 / 720.0) * y4;
        c->gn = (1.0 / 3.0) * y3 + (1.0 / 60.0) * y5;
    }
    if (gamma == 0) {
        c->coeff0 = 1.0;
        c->coeff1 = 1.0;
        c->coeff2 = 0.0;
        c->coeff3 = 0.5;
    }
    double gamma2 = gamma * gamma;
    c->sig1 = sqrt(+kT * c->sig1 / gamma2);
    c->sig2 = sqrt(-kT * c->sig2 / gamma2);
    c->corr = (kT / (gamma2)) * (c->gn / (c->sig1 * c->sig2));
    c->dev = sqrt(1.0 - (c->corr * c->corr));
}

int make_vgb_params(const psim_integrator_config* ic, VgbParams* p) {
    if (!ic) return fail(PSIM_ERR_INPUT, "integrator config is NULL");
    if (!(ic->dt > 0.0)) return fail(PSIM_ERR_INPUT, "timeStep must be positive");
    if (ic->vel_freq < 0) return fail(PSIM_ERR_INPUT, "velFreq must be >= 0");
    psim_vgb_coeffs c;
    vgb_coeffs(ic->gamma, ic->dt, ic->kT, &c);
    const double v[] = {c.coeff0, c.coeff1, c.coeff2, c.coeff3, c.sig1,
                        c.sig2,   c.corr,   c.dev,    c.goy2,   c.goy3, c.hn};
    for (double x : v)
        if (!std::isfinite(x))
            return fail(PSIM_ERR_INPUT,
                        "vGB coefficients are not finite for gamma=%g dt=%g kT=%g (the "
                        "reference's gamma == 0 set-up divides by gamma^2)",
                        ic->gamma, ic->dt, ic->kT);
    p->dt = ic->dt;
    p->dt2 = ic->dt * ic->dt;
    p->dt3 = ic->dt * p->dt2;
    p->dt_inv = 1.0 / ic->dt;
    p->c0 = 1.0 + c.coeff0;
    p->coeff0 = c.coeff0;
    p->coeff1 = c.coeff1;
    p->coeff2 = c.coeff2;
    p->coeff3 = c.coeff3;
    p->sig1 = c.sig1;
    p->sig2 = c.sig2;
    p->corr = c.corr;
    p->dev = c.dev;
    p->goy2 = c.goy2;
    p->goy3 = c.goy3;
    p->hn = c.hn;
    p->dt2c1 = p->dt2 * c.coeff1;
    p->dt2c2 = p->dt2 * c.coeff2;
    p->sig1f = (float)c.sig1;
    p->sig2f = (float)c.sig2;
    p->corrf = (float)c.corr;
    p->devf = (float)c.dev;
    p->coeff0f = (float)c.coeff0;
    p->dt2c1f = (float)p->dt2c1;
    p->dt2c2f = (float)p->dt2c2;
    p->vel_freq = ic->vel_freq;
    p->seed = (uint32_t)ic->seed;
    return PSIM_OK;
}

int ensure_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(PSIM_ERR_NO_DEVICE, "no CUDA device available (%s)",
                    e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
    }
    return PSIM_OK;
}

// ------------------------------------------------------------- buffers

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b ? b : 16);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// A temporary device buffer freed when it leaves scope.
struct ScopedBuf : DevBuf {
    ~ScopedBuf() { release(); }
};

// Scratch for the reference-layout drop-ins, grown on demand, one set per
// process (calls are serialised by a mutex).
struct Workspace {
    std::mutex mu;
    int device = -1;
    cudaStream_t st = nullptr;
    DevBuf pos, radius, radius_in, xyz, key, rank, tmp, perm, tag_in, tag_out, radius_out,
        cellid, count, start, scratch, posd, posh, posl, hash_index, cse, sorted, force, fxyz, err;
    // the mixed form's pair list (records, halo words and count, entries),
    // kept across calls while no particle has moved skin/2 since its build:
    // the build's slot of each original index and original index of each
    // slot, the build positions (high parts), the displacement flag
    DevBuf lpos, lhalo, lhcount, list, lcount, lslot_of, lbuild, lflag, inv;
    // the kept list's records: compact (one radius lradius, low-part unit
    // lunit) or full
    bool lcompact = false;
    float lradius = 0.f, lunit = 0.f;
    // the device reads and writes the callers' host arrays in place (a device
    // with access to pageable host memory); PSIM_DROPIN_COPIES=1 copies them
    bool direct = false;
    int pageable = 0;
    struct ListKey {
        bool valid = false;
        int n = 0, s = 0, cap = 0, hcap = 0;
        double L = 0.0, cs = 0.0, rc = 0.0, skin = 0.0;
        bool operator==(const ListKey& o) const {
            return valid && o.valid && n == o.n && s == o.s && cap == o.cap && hcap == o.hcap &&
                   L == o.L && cs == o.cs && rc == o.rc && skin == o.skin;
        }
    } lkey;
    // the list's skin: 0 (default) none -- each call stands alone, as the
    // reference's call does; < 0 automatic; > 0 that skin
    double lskin = 0.0;
    long long lbuilds = 0, lcalls = 0;
};
Workspace g_ws;

int ws_begin(Workspace& w) {
    int dev = 0;
    PSIM_CUDA(cudaGetDevice(&dev));
    if (w.st && w.device != dev) {
        // the caller switched devices: free the old device's buffers and
        // stream on that device, then make the caller's device current again
        DevBuf* all[] = {&w.pos, &w.radius, &w.radius_in, &w.xyz, &w.key, &w.rank, &w.tmp, &w.perm, &w.tag_in,
                         &w.tag_out, &w.radius_out, &w.cellid, &w.count, &w.start, &w.scratch,
                         &w.posd, &w.posh, &w.posl, &w.hash_index, &w.cse, &w.sorted, &w.force,
                         &w.fxyz, &w.err, &w.lpos, &w.lhalo, &w.lhcount, &w.list, &w.lcount,
                         &w.lslot_of, &w.lbuild, &w.lflag, &w.inv};
        if (cudaSetDevice(w.device) == cudaSuccess) {
            cudaStreamSynchronize(w.st);
            for (DevBuf* b : all) b->release();
            cudaStreamDestroy(w.st);
        } else {
            // the old device is gone (reset or lost): its memory went with it
            cudaGetLastError();
            for (DevBuf* b : all) { b->p = nullptr; b->bytes = 0; }
        }
        PSIM_CUDA(cudaSetDevice(dev));
        w.lkey.valid = false;
        w.st = nullptr;
    }
    if (!w.st) {
        PSIM_CUDA(cudaStreamCreateWithFlags(&w.st, cudaStreamNonBlocking));
        w.device = dev;
        if (cudaDeviceGetAttribute(&w.pageable, cudaDevAttrPageableMemoryAccess, dev) !=
            cudaSuccess)
            w.pageable = 0;
    }
    const char* copies = std::getenv("PSIM_DROPIN_COPIES");
    w.direct = w.pageable == 1 && !(copies && copies[0] == '1');
    return PSIM_OK;
}

}  // namespace

// ===================================================================== C ABI

extern "C" {

int psim_abi_version(void) { return 4; }

// Lets other translation units of this library report through
// psim_last_error_string (not part of the public header).
void psim_internal_set_error(const char* msg) { g_last_error = msg ? msg : ""; }

const char* psim_last_error_string(void) { return g_last_error.c_str(); }

int psim_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int psim_ao_coefficients(double kT, double well_depth, double cutoff, double* coeff1,
                         double* coeff2) {
    if (!coeff1 || !coeff2) return fail(PSIM_ERR_INPUT, "NULL output");
    ao_coeffs(kT, well_depth, cutoff, coeff1, coeff2);
    return PSIM_OK;
}

int psim_force_params_from_settings(const char* plugin, const char* text, psim_force_params* out) {
    if (!plugin || !out) return fail(PSIM_ERR_INPUT, "NULL argument");
    Settings s(text);
    std::string name(plugin);
    psim_force_params p{};
    bool ok = true;
    double kT = 1.0;
    ok &= s.get_double("kT", 1.0, &kT);
    p.kT = kT;
    if (name == "AOPotential" || name == "AO") {            // AOPotential.cpp:40-47
        p.kind = PSIM_FORCE_AO;
        ok &= s.get_double("wellDepth", 0.261, &p.well_depth);
        ok &= s.get_double("cutOff", 1.1, &p.cutoff);
        p.lj_num = 18;
        p.debye_length = 0.5;
    } else if (name == "LennardJones" || name == "LJ") {    // LJPotential.cpp:31-55
        p.kind = PSIM_FORCE_LJ;
        ok &= s.get_double("wellDepth", 10.0, &p.well_depth);
        ok &= s.get_double("yukawaStrength", 8.0, &p.yukawa_strength);
        ok &= s.get_int("ljNum", 18, &p.lj_num);
        ok &= s.get_double("cutOff", 2.5, &p.cutoff);
        ok &= s.get_double("debyeLength", 0.5, &p.debye_length);
    } else if (name == "Calibration" || name == "Cal") {    // Calibration.cpp:33-36
        p.kind = PSIM_FORCE_CALIBRATION;
        ok &= s.get_double("cutOff", 1.1, &p.cutoff);
        p.lj_num = 18;
        p.debye_length = 0.5;
    } else if (name == "AOYukawa") {
        p.kind = PSIM_FORCE_AO_YUKAWA;
        ok &= s.get_double("wellDepth", 0.261, &p.well_depth);
        ok &= s.get_double("cutOff", 1.1, &p.cutoff);
        ok &= s.get_double("yukawa.wellDepth", 10.0, &p.well_depth2);
        ok &= s.get_double("yukawa.yukawaStrength", 8.0, &p.yukawa_strength);
        ok &= s.get_int("yukawa.ljNum", 0, &p.lj_num);
        ok &= s.get_double("yukawa.cutOff", 2.5, &p.cutoff2);
        ok &= s.get_double("yukawa.debyeLength", 0.5, &p.debye_length);
    } else {
        return fail(PSIM_ERR_LOAD, "unknown force plugin '%s'", plugin);
    }
    if (!ok) return fail(PSIM_ERR_INPUT, "a settings value for plugin '%s' is not a number", plugin);
    *out = p;
    return PSIM_OK;
}

int psim_vgb_coefficients(double gamma, double dt, double kT, psim_vgb_coeffs* out) {
    if (!out) return fail(PSIM_ERR_INPUT, "NULL output");
    vgb_coeffs(gamma, dt, kT, out);
    return PSIM_OK;
}

// ----------------------------------------------------------- cells drop-in

int psim_cells_build(const psim_geometry* gm, const double* pos, const double* radius,
                     int32_t* hash_index, uint32_t* cse, double* sorted) {
    DevGeom g;
    int rc = make_geom(gm, 0.0, &g);
    if (rc) return rc;
    if (g.n > 0 && (!pos || !radius)) return fail(PSIM_ERR_INPUT, "NULL positions or radii");
    if ((rc = ensure_device())) return rc;
    Workspace& w = g_ws;
    std::lock_guard<std::mutex> lk(w.mu);
    if ((rc = ws_begin(w))) return rc;
    const size_t n = (size_t)g.n, nc = (size_t)g.ncell;
    PSIM_CUDA(w.radius.ensure(8 * n));
    PSIM_CUDA(w.xyz.ensure(24 * n));
    PSIM_CUDA(w.key.ensure(4 * n));
    PSIM_CUDA(w.rank.ensure(4 * n));
    PSIM_CUDA(w.tmp.ensure(4 * n));
    PSIM_CUDA(w.perm.ensure(4 * n));
    PSIM_CUDA(w.tag_in.ensure(4 * n));
    PSIM_CUDA(w.tag_out.ensure(4 * n));
    PSIM_CUDA(w.radius_out.ensure(8 * n));
    PSIM_CUDA(w.cellid.ensure(4 * n));
    PSIM_CUDA(w.count.ensure(4 * nc));
    PSIM_CUDA(w.start.ensure(4 * nc));
    PSIM_CUDA(w.scratch.ensure(4 * scan_scratch_ints(g.ncell)));
    PSIM_CUDA(w.posd.ensure(32 * n));
    PSIM_CUDA(w.posh.ensure(16 * n));
    PSIM_CUDA(w.err.ensure(4));
    cudaStream_t st = w.st;
    double* x = w.xyz.as<double>();
    // the caller's arrays: read and written in place by the device, or copied
    const double* d_pos = pos;
    const double* d_radius = radius;
    if (!w.direct) {
        PSIM_CUDA(w.pos.ensure(24 * n));
        PSIM_CUDA(w.radius_in.ensure(8 * n));
        PSIM_CUDA(w.hash_index.ensure(8 * n));
        PSIM_CUDA(w.cse.ensure(8 * nc));
        PSIM_CUDA(w.sorted.ensure(32 * n));
        PSIM_CUDA(cudaMemcpyAsync(w.pos.p, pos, 24 * n, cudaMemcpyHostToDevice, st));
        PSIM_CUDA(cudaMemcpyAsync(w.radius_in.p, radius, 8 * n, cudaMemcpyHostToDevice, st));
        d_pos = w.pos.as<double>();
        d_radius = w.radius_in.as<double>();
    }
    PSIM_CUDA(cudaMemsetAsync(w.count.p, 0, 4 * nc, st));
    PSIM_CUDA(cudaMemsetAsync(w.err.p, 0, 4, st));
    PSIM_CUDA(launch_import_positions(g.n, d_pos, d_radius, x, x + n, x + 2 * n,
                                      w.radius.as<double>(), st));
    PSIM_CUDA(launch_hash_count(g.n, x, x + n, x + 2 * n, g, w.key.as<int>(), w.rank.as<int>(),
                                w.count.as<int>(), w.err.as<uint32_t>(), st));
    PSIM_CUDA(launch_scan(w.count.as<int>(), w.start.as<int>(), g.ncell, w.scratch.as<int>(), st));
    PSIM_CUDA(launch_scatter(g.n, w.key.as<int>(), w.rank.as<int>(), w.start.as<int>(),
                             w.tmp.as<int>(), nullptr, st));
    PSIM_CUDA(launch_fill_int_iota(g.n, w.tag_in.as<int>(), st));
    CanonArgs ca{};
    ca.n = g.n;
    ca.tmp = w.tmp.as<int>();
    ca.key = w.key.as<int>();
    ca.start = w.start.as<int>();
    ca.count = w.count.as<int>();
    ca.tag_in = w.tag_in.as<int>();
    ca.radius_in = w.radius.as<double>();
    ca.x = x;
    ca.y = x + n;
    ca.z = x + 2 * n;
    ca.perm = w.perm.as<int>();
    ca.tag_out = w.tag_out.as<int>();
    ca.radius_out = w.radius_out.as<double>();
    ca.cellid = w.cellid.as<int>();
    ca.posd = w.posd.as<double4_32a>();
    ca.posh = w.posh.as<float4>();
    PSIM_CUDA(launch_canonicalize(ca, st));
    if (w.direct) {
        PSIM_CUDA(launch_export_cells(g.n, g.ncell, w.cellid.as<int>(), w.tag_out.as<int>(),
                                      w.posd.as<double4_32a>(), w.start.as<int>(),
                                      w.count.as<int>(), hash_index, cse, sorted, st));
    } else {
        PSIM_CUDA(launch_export_cells(g.n, g.ncell, w.cellid.as<int>(), w.tag_out.as<int>(),
                                      w.posd.as<double4_32a>(), w.start.as<int>(),
                                      w.count.as<int>(), w.hash_index.as<int32_t>(),
                                      w.cse.as<uint32_t>(), w.sorted.as<double>(), st));
        if (hash_index)
            PSIM_CUDA(cudaMemcpyAsync(hash_index, w.hash_index.p, 8 * n, cudaMemcpyDeviceToHost,
                                      st));
        if (cse) PSIM_CUDA(cudaMemcpyAsync(cse, w.cse.p, 8 * nc, cudaMemcpyDeviceToHost, st));
        if (sorted)
            PSIM_CUDA(cudaMemcpyAsync(sorted, w.sorted.p, 32 * n, cudaMemcpyDeviceToHost, st));
    }
    uint32_t bits = 0;
    PSIM_CUDA(cudaMemcpyAsync(&bits, w.err.p, 4, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaStreamSynchronize(st));
    if (bits) return fail(code_from_bits(bits), "%s", bits_text(bits));
    return PSIM_OK;
}

// ----------------------------------------------------------- force drop-in

namespace {
int force_evaluate(psim_force_launch_fn plugin, const psim_force_params* params,
                   const psim_geometry* gm, int32_t precision, const double* sorted,
                   const int32_t* hash_index, const uint32_t* cse, double* force) {
    int rc = check_params(params, plugin != nullptr);
    if (rc) return rc;
    DevGeom g;
    if ((rc = make_geom(gm, max_cutoff(params), &g))) return rc;
    if (precision != PSIM_PRECISION_FP64 && precision != PSIM_PRECISION_MIXED)
        return fail(PSIM_ERR_INPUT, "unknown precision %d", precision);
    if (g.n > 0 && (!sorted || !hash_index || !cse || !force))
        return fail(PSIM_ERR_INPUT, "NULL array");
    if ((rc = ensure_device())) return rc;
    ForceSetup fs = make_setup(params, g.L);
    fs.tile = choose_tile(g);
    fs.walk = choose_walk();
    const ForceRunner fr{&fs, plugin, params};
    Workspace& w = g_ws;
    std::lock_guard<std::mutex> lk(w.mu);
    if ((rc = ws_begin(w))) return rc;
    const size_t n = (size_t)g.n, nc = (size_t)g.ncell;
    PSIM_CUDA(w.posd.ensure(32 * n));
    PSIM_CUDA(w.posh.ensure(16 * n));
    PSIM_CUDA(w.posl.ensure(16 * n));
    PSIM_CUDA(w.cellid.ensure(4 * n));
    PSIM_CUDA(w.tag_out.ensure(4 * n));
    PSIM_CUDA(w.start.ensure(4 * nc));
    PSIM_CUDA(w.count.ensure(4 * nc));
    PSIM_CUDA(w.scratch.ensure(4 * scan_scratch_ints(g.ncell)));
    PSIM_CUDA(w.fxyz.ensure(24 * n));
    PSIM_CUDA(w.inv.ensure(4 * n));
    PSIM_CUDA(w.err.ensure(4));
    PSIM_CUDA(w.lflag.ensure(8));
    cudaStream_t st = w.st;
    // the caller's arrays: read in place by the device, or copied in
    const double* d_sorted = sorted;
    const int32_t* d_hi = hash_index;
    const uint32_t* d_cse = cse;
    if (!w.direct) {
        PSIM_CUDA(w.sorted.ensure(32 * n));
        PSIM_CUDA(w.hash_index.ensure(8 * n));
        PSIM_CUDA(w.cse.ensure(8 * nc));
        PSIM_CUDA(w.force.ensure(24 * n));
        PSIM_CUDA(cudaMemcpyAsync(w.sorted.p, sorted, 32 * n, cudaMemcpyHostToDevice, st));
        PSIM_CUDA(cudaMemcpyAsync(w.hash_index.p, hash_index, 8 * n, cudaMemcpyHostToDevice, st));
        PSIM_CUDA(cudaMemcpyAsync(w.cse.p, cse, 8 * nc, cudaMemcpyHostToDevice, st));
        d_sorted = w.sorted.as<double>();
        d_hi = w.hash_index.as<int32_t>();
        d_cse = w.cse.as<uint32_t>();
    }
    PSIM_CUDA(cudaMemsetAsync(w.err.p, 0, 4, st));
    // flags: [0] a particle moved too far for the kept list, [1] mixed radii
    int* flags = w.lflag.as<int>();
    PSIM_CUDA(cudaMemsetAsync(flags, 0, 8, st));
    PSIM_CUDA(launch_import_sorted(g.n, d_sorted, d_hi, g, w.posd.as<double4_32a>(),
                                   w.posh.as<float4>(), w.posl.as<float4>(), w.cellid.as<int>(),
                                   w.tag_out.as<int>(), w.err.as<uint32_t>(), st, flags + 1));
    PSIM_CUDA(launch_import_cse(g.ncell, g.n, d_cse, w.start.as<int>(), w.count.as<int>(),
                                w.scratch.as<int>(), w.err.as<uint32_t>(), st));
    // The mixed form walks a pair list: the pairs within cutOff + skin of a
    // build, kept across calls while no particle has moved skin/2 since (every
    // pair within cutOff is then in it), or, with no skin, a list of this
    // call's pairs only.  Building a list and walking it costs about half the
    // 27-cell walk; walking a kept one, about a fifth.  Records are compact
    // (16 bytes) when every particle has the same radius.
    const double rcm = max_cutoff(params);
    const double skin = precision == PSIM_PRECISION_MIXED ? dropin_skin(w.lskin, g, rcm) : 0.0;
    const ListSizes z = list_sizes(rcm, skin, g);
    const bool one_list = precision == PSIM_PRECISION_MIXED && g.n > 0 &&
                          (double)(z.cap + kListFold) * (double)g.n < 4294967296.0;
    Workspace::ListKey key;
    key.valid = skin > 0.0;
    key.n = g.n;
    key.s = g.s;
    key.cap = z.cap;
    key.hcap = z.hcap;
    key.L = g.L;
    key.cs = g.cs;
    key.rc = rcm;
    key.skin = skin;
    const bool kept = one_list && w.lkey == key;
    double* f = w.fxyz.as<double>();
    CellView cv{w.posd.as<double4_32a>(), w.posh.as<float4>(), w.posl.as<float4>(),
                w.cellid.as<int>(), w.start.as<int>(), w.count.as<int>()};
    ForceOut out{f, f + n, f + 2 * n, w.err.as<uint32_t>()};
    if (kept) {
        // this call's positions into the kept records with the displacement
        // test, and the force pass over the kept list in the same stream: the
        // usual call ends at the one synchronisation below; a call that finds
        // a particle moved too far discards this force and builds a new list
        PSIM_CUDA(launch_list_refresh(g.n, w.posd.as<double4_32a>(), w.tag_out.as<int>(),
                                      w.lslot_of.as<int>(), w.lbuild.as<float4>(),
                                      w.lhalo.as<int>(), w.lpos.as<float4>(), z.disp2, g,
                                      w.lcompact ? 1.0f / w.lunit : 0.f, w.lradius, flags, st));
        const PairList pl{nullptr, w.lpos.as<float4>(), w.lcount.as<int>(),
                          w.list.as<uint32_t>(), g.n, w.lcompact, w.lradius, w.lunit};
        PSIM_CUDA(fr.run(PSIM_PASS_LIST, g, nullptr, &pl, out, st));
        PSIM_CUDA(launch_export_force(g.n, w.lslot_of.as<int>(), f, f + n, f + 2 * n,
                                      w.direct ? force : w.force.as<double>(), st));
        if (!w.direct)
            PSIM_CUDA(cudaMemcpyAsync(force, w.force.p, 24 * n, cudaMemcpyDeviceToHost, st));
    }
    w.lcalls += precision == PSIM_PRECISION_MIXED ? 1 : 0;
    // a position outside the grid has no home cell: stop before the force pass
    uint32_t bits = 0;
    int hflags[2] = {0, 0};
    PSIM_CUDA(cudaMemcpyAsync(&bits, w.err.p, 4, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaMemcpyAsync(hflags, flags, 8, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaStreamSynchronize(st));
    if (bits) {
        w.lkey.valid = false;
        return fail(code_from_bits(bits), "%s", bits_text(bits));
    }
    if (kept && hflags[0] == 0) return PSIM_OK;
    // the forces come out in the list's order (the sorted order of its
    // build) or this call's sorted order; inv maps original index -> slot
    const int* inv = nullptr;
    if (precision == PSIM_PRECISION_MIXED && one_list) {
        bool listed = false;   // a kept list that is still good has returned above
        w.lkey.valid = false;
        const bool compact = hflags[1] == 0;
        const float R = compact ? (float)sorted[3] : 0.f;
        const float unit = fixed_unit(rcm, skin);
        const size_t rec = compact ? 16 : 32;
        PSIM_CUDA(w.lpos.ensure(rec * (n + 1 + (size_t)z.hcap)));
        PSIM_CUDA(w.lhalo.ensure(4 * n));
        PSIM_CUDA(w.lhcount.ensure(4));
        PSIM_CUDA(w.list.ensure(4 * n * (size_t)(z.cap + kListFold)));
        PSIM_CUDA(w.lcount.ensure(4 * n));
        PSIM_CUDA(w.lslot_of.ensure(4 * n));
        PSIM_CUDA(cudaMemsetAsync(w.lhcount.p, 0, 4, st));
        // the ghost record that pads the lists, out of range of every particle
        static const float4 ghost_full[2] = {make_float4(1e18f, 1e18f, 1e18f, 0.f),
                                             make_float4(0.f, 0.f, 0.f, 0.f)};
        static const float4 ghost_compact = make_float4(0.f, 0.f, 0.f, kGhostBias);
        PSIM_CUDA(cudaMemcpyAsync(w.lpos.as<char>() + rec * n,
                                  compact ? &ghost_compact : ghost_full, rec,
                                  cudaMemcpyHostToDevice, st));
        PSIM_CUDA(launch_list_records(g.n, w.posh.as<float4>(), w.posl.as<float4>(),
                                      w.lpos.as<float4>(), w.lhalo.as<int>(),
                                      w.lhcount.as<int>(), z.hcap, z.hr, g,
                                      w.err.as<uint32_t>(), st, compact ? 1.0f / unit : 0.f));
        ListBuild lb{w.list.as<uint32_t>(), w.lcount.as<int>(), g.n, z.cap, z.pre, nullptr,
                     w.lhalo.as<int>(), g.n};
        PSIM_CUDA(launch_list_build(g, cv, lb, w.err.as<uint32_t>(), st));
        PSIM_CUDA(cudaMemcpyAsync(&bits, w.err.p, 4, cudaMemcpyDeviceToHost, st));
        PSIM_CUDA(cudaStreamSynchronize(st));
        w.lbuilds++;
        if (bits == EBIT_LIST) {
            // a denser neighbourhood than the list has room for: the cell walk
            bits = 0;
            PSIM_CUDA(cudaMemsetAsync(w.err.p, 0, 4, st));
            PSIM_CUDA(fr.run(PSIM_PASS_MIXED, g, &cv, nullptr, out, st));
        } else if (bits == 0) {
            listed = true;
            w.lcompact = compact;
            w.lradius = R;
            w.lunit = unit;
            PSIM_CUDA(cudaMemsetAsync(w.lslot_of.p, 0xff, 4 * n, st));
            PSIM_CUDA(launch_invert_tags(g.n, w.tag_out.as<int>(), w.lslot_of.as<int>(), st));
            if (key.valid) {   // kept: the build positions
                PSIM_CUDA(w.lbuild.ensure(16 * n));
                PSIM_CUDA(cudaMemcpyAsync(w.lbuild.p, w.posh.p, 16 * n,
                                          cudaMemcpyDeviceToDevice, st));
                w.lkey = key;
            }
        }
        if (listed) {
            const PairList pl{nullptr, w.lpos.as<float4>(), w.lcount.as<int>(),
                              w.list.as<uint32_t>(), g.n, w.lcompact, w.lradius, w.lunit};
            PSIM_CUDA(fr.run(PSIM_PASS_LIST, g, nullptr, &pl, out, st));
            inv = w.lslot_of.as<int>();
        }
    } else if (precision == PSIM_PRECISION_FP64) {
        PSIM_CUDA(fr.run(PSIM_PASS_FP64, g, &cv, nullptr, out, st));
    } else {
        PSIM_CUDA(fr.run(PSIM_PASS_MIXED, g, &cv, nullptr, out, st));
    }
    if (!inv) {   // this call's sorted order
        PSIM_CUDA(launch_invert_tags(g.n, w.tag_out.as<int>(), w.inv.as<int>(), st));
        inv = w.inv.as<int>();
    }
    PSIM_CUDA(launch_export_force(g.n, inv, f, f + n, f + 2 * n,
                                  w.direct ? force : w.force.as<double>(), st));
    PSIM_CUDA(cudaMemcpyAsync(&bits, w.err.p, 4, cudaMemcpyDeviceToHost, st));
    if (!w.direct)
        PSIM_CUDA(cudaMemcpyAsync(force, w.force.p, 24 * n, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaStreamSynchronize(st));
    if (bits) {
        w.lkey.valid = false;
        return fail(code_from_bits(bits), "%s", bits_text(bits));
    }
    return PSIM_OK;
}
}  // namespace

int psim_force_evaluate(const psim_force_params* params, const psim_geometry* gm,
                        int32_t precision, const double* sorted, const int32_t* hash_index,
                        const uint32_t* cse, double* force) {
    return force_evaluate(nullptr, params, gm, precision, sorted, hash_index, cse, force);
}

int psim_force_evaluate_plugin(psim_force_launch_fn launch, const psim_force_params* params,
                               const psim_geometry* gm, int32_t precision,
                               const double* sorted, const int32_t* hash_index,
                               const uint32_t* cse, double* force) {
    if (!launch) return fail(PSIM_ERR_INPUT, "the plugin's psim_force_launch is NULL");
    return force_evaluate(launch, params, gm, precision, sorted, hash_index, cse, force);
}

int psim_force_set_list_skin(double skin) {
    if (!(skin == skin)) return fail(PSIM_ERR_INPUT, "skin is NaN");
    Workspace& w = g_ws;
    std::lock_guard<std::mutex> lk(w.mu);
    w.lskin = skin;
    w.lkey.valid = false;
    return PSIM_OK;
}

int psim_force_list_stats(int64_t* calls, int64_t* builds) {
    Workspace& w = g_ws;
    std::lock_guard<std::mutex> lk(w.mu);
    if (calls) *calls = w.lcalls;
    if (builds) *builds = w.lbuilds;
    return PSIM_OK;
}

}  // extern "C"

// ------------------------------------------------------------ integrator

constexpr int kAosChunks = 8;   // chunks of the drop-in integrator's copies

struct psim_integrator {
    int device = 0;
    int n = 0;
    cudaStream_t st = nullptr;
    // the copies in and out run on their own streams, chunk by chunk, so that
    // they overlap each other and the update of the chunks before
    cudaStream_t st_in = nullptr, st_out = nullptr;
    cudaEvent_t ev_in[kAosChunks] = {}, ev_run[kAosChunks] = {};
    // the GPU reads and writes the caller's arrays in place (a device with
    // access to pageable host memory: Grace's coherent link) instead of
    // copying them; PSIM_DROPIN_COPIES=1 keeps the copies
    bool direct = false;
    VgbParams vp{};
    int vel_counter = 0;
    long long steps = 0;
    DevBuf mem, mem_corr, pos, pos0, vel, frc, frc0, mass, noise, err;
};

extern "C" {

psim_integrator* psim_integrator_create(const psim_integrator_config* cfg, int32_t n) {
    if (n < 0) { fail(PSIM_ERR_INPUT, "negative particle count"); return nullptr; }
    VgbParams vp;
    if (make_vgb_params(cfg, &vp)) return nullptr;
    if (ensure_device()) return nullptr;
    psim_integrator* it = new psim_integrator();
    it->n = n;
    it->vp = vp;
    cudaGetDevice(&it->device);
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, it->device) !=
        cudaSuccess)
        pageable = 0;
    const char* copies = std::getenv("PSIM_DROPIN_COPIES");
    it->direct = pageable == 1 && !(copies && copies[0] == '1');
    const size_t b = 24 * (size_t)n;
    bool ev_ok = cudaStreamCreateWithFlags(&it->st_in, cudaStreamNonBlocking) == cudaSuccess &&
                 cudaStreamCreateWithFlags(&it->st_out, cudaStreamNonBlocking) == cudaSuccess;
    for (int k = 0; k < kAosChunks && ev_ok; ++k)
        ev_ok = cudaEventCreateWithFlags(&it->ev_in[k], cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&it->ev_run[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ev_ok || cudaStreamCreateWithFlags(&it->st, cudaStreamNonBlocking) != cudaSuccess ||
        it->mem.ensure(b) || it->mem_corr.ensure(b) || it->pos.ensure(b) || it->pos0.ensure(b) ||
        it->vel.ensure(b) || it->frc.ensure(b) || it->frc0.ensure(b) ||
        it->mass.ensure(8 * (size_t)n) || it->err.ensure(4) ||
        cudaMemset(it->mem.p, 0, b) || cudaMemset(it->mem_corr.p, 0, b)) {
        fail(PSIM_ERR_CUDA, "integrator allocation failed: %s", cudaGetErrorString(cudaGetLastError()));
        psim_integrator_destroy(it);
        return nullptr;
    }
    return it;
}

void psim_integrator_destroy(psim_integrator* it) {
    if (!it) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(it->device);
    DevBuf* all[] = {&it->mem, &it->mem_corr, &it->pos, &it->pos0, &it->vel, &it->frc,
                     &it->frc0, &it->mass, &it->noise, &it->err};
    for (DevBuf* b : all) b->release();
    for (int k = 0; k < kAosChunks; ++k) {
        if (it->ev_in[k]) cudaEventDestroy(it->ev_in[k]);
        if (it->ev_run[k]) cudaEventDestroy(it->ev_run[k]);
    }
    if (it->st_in) cudaStreamDestroy(it->st_in);
    if (it->st_out) cudaStreamDestroy(it->st_out);
    if (it->st) cudaStreamDestroy(it->st);
    cudaSetDevice(prev);
    delete it;
}

int psim_integrator_next_system(psim_integrator* it, double current_time, double box,
                                int32_t noise_mode, const double* noise,
                                const double* particle_force, double* pos, double* pos0,
                                double* vel, double* frc, double* frc0, const double* mass) {
    if (!it) return fail(PSIM_ERR_INPUT, "NULL integrator");
    if (!(box > 0.0)) return fail(PSIM_ERR_INPUT, "box size must be positive");
    if (noise_mode == PSIM_NOISE_INJECTED && !noise && it->n > 0)
        return fail(PSIM_ERR_INPUT, "injected noise mode needs a noise array");
    if (it->n > 0 && (!pos || !pos0 || !vel || !frc || !frc0 || !mass))
        return fail(PSIM_ERR_INPUT, "NULL particle array");
    int prev = 0;
    PSIM_CUDA(cudaGetDevice(&prev));
    PSIM_CUDA(cudaSetDevice(it->device));
    const size_t n = (size_t)it->n;
    cudaStream_t st = it->st;
    const bool first = (current_time == 0);  // nextSystem, brownianIntegrator.cpp:183
    const bool vel_step = !first && (it->vp.vel_freq == 0 || it->vel_counter == it->vp.vel_freq);
    // the previous force and this one on the device (pushParticleForce:
    // frc0 <- frc, frc <- particleForce)
    const double* F0 = particle_force ? frc : frc0;
    const double* F = particle_force ? particle_force : frc;
    if (it->direct) {
        // one pass over the caller's arrays in place
        PSIM_CUDA(cudaMemsetAsync(it->err.p, 0, 4, st));
        VgbHostArgs a{};
        a.n = (int)n;
        a.first = first ? 1 : 0;
        a.vel_step = vel_step ? 1 : 0;
        a.pos = pos;
        a.pos0 = pos0;
        a.vel = vel;
        a.F = F;
        a.F0 = F0;
        a.frc_out = particle_force ? frc : nullptr;
        a.frc0_out = particle_force ? frc0 : nullptr;
        a.mass = mass;
        a.mem = it->mem.as<double>();
        a.mem_corr = it->mem_corr.as<double>();
        a.noise = noise_mode == PSIM_NOISE_INJECTED ? noise : nullptr;
        a.seed = it->vp.seed;
        a.philox_step = it->steps;
        a.err = it->err.as<uint32_t>();
        PSIM_CUDA(launch_vgb_host(a, it->vp, box, st));
        uint32_t bits = 0;
        PSIM_CUDA(cudaMemcpyAsync(&bits, it->err.p, 4, cudaMemcpyDeviceToHost, st));
        PSIM_CUDA(cudaStreamSynchronize(st));
        if (!first)  // brownianIntegrator.cpp:291-292
            it->vel_counter = (it->vel_counter == it->vp.vel_freq) ? 0 : it->vel_counter + 1;
        it->steps++;
        cudaSetDevice(prev);
        if (bits) return fail(code_from_bits(bits), "%s", bits_text(bits));
        return PSIM_OK;
    }
    if (noise_mode == PSIM_NOISE_INJECTED) PSIM_CUDA(it->noise.ensure(48 * n));
    PSIM_CUDA(cudaMemsetAsync(it->err.p, 0, 4, st));
    cudaEvent_t ev0 = it->ev_run[0];
    PSIM_CUDA(cudaEventRecord(ev0, st));   // the error word is cleared before any chunk runs
    PSIM_CUDA(cudaStreamWaitEvent(it->st_in, ev0, 0));
    // chunks of whole particles: copies in (st_in), the update (st), copies out
    // (st_out); velocities move only when the step reads (firstStep) or writes
    // (velocityStep) them
    const size_t chunk = (n + kAosChunks - 1) / kAosChunks;
    for (int k = 0; k < kAosChunks; ++k) {
        const size_t a0 = std::min(n, (size_t)k * chunk), a1 = std::min(n, a0 + chunk);
        const size_t m = a1 - a0;
        if (m == 0) continue;
        const size_t o3 = 3 * a0, b3 = 24 * m;
        auto in = [&](DevBuf& d, const double* h, size_t off, size_t bytes) {
            return cudaMemcpyAsync(d.as<double>() + off, h + off, bytes, cudaMemcpyHostToDevice,
                                   it->st_in);
        };
        PSIM_CUDA(in(it->pos, pos, o3, b3));
        PSIM_CUDA(in(it->pos0, pos0, o3, b3));
        PSIM_CUDA(in(it->frc0, F0, o3, b3));
        PSIM_CUDA(in(it->frc, F, o3, b3));
        PSIM_CUDA(in(it->mass, mass, a0, 8 * m));
        if (first || vel_step) PSIM_CUDA(in(it->vel, vel, o3, b3));
        if (noise_mode == PSIM_NOISE_INJECTED) PSIM_CUDA(in(it->noise, noise, 6 * a0, 48 * m));
        PSIM_CUDA(cudaEventRecord(it->ev_in[k], it->st_in));
        PSIM_CUDA(cudaStreamWaitEvent(st, it->ev_in[k], 0));
        VgbAosArgs a{};
        a.n = (int)m;
        a.offset = (int)a0;
        a.first = first ? 1 : 0;
        a.vel_step = vel_step ? 1 : 0;
        a.pos = it->pos.as<double>() + o3;
        a.pos0 = it->pos0.as<double>() + o3;
        a.vel = it->vel.as<double>() + o3;
        a.frc = it->frc.as<double>() + o3;
        a.frc0 = it->frc0.as<double>() + o3;
        a.mass = it->mass.as<double>() + a0;
        a.mem = it->mem.as<double>() + o3;
        a.mem_corr = it->mem_corr.as<double>() + o3;
        a.noise = noise_mode == PSIM_NOISE_INJECTED ? it->noise.as<double>() + 6 * a0 : nullptr;
        a.seed = it->vp.seed;
        a.philox_step = it->steps;
        a.err = it->err.as<uint32_t>();
        PSIM_CUDA(launch_vgb_aos(a, it->vp, box, st));
        PSIM_CUDA(cudaEventRecord(it->ev_run[k], st));
        // the pushed forces back to the host arrays as soon as they are in
        if (particle_force) {
            PSIM_CUDA(cudaStreamWaitEvent(it->st_out, it->ev_in[k], 0));
            PSIM_CUDA(cudaMemcpyAsync(frc0 + o3, it->frc0.as<double>() + o3, b3,
                                      cudaMemcpyDeviceToHost, it->st_out));
            PSIM_CUDA(cudaMemcpyAsync(frc + o3, it->frc.as<double>() + o3, b3,
                                      cudaMemcpyDeviceToHost, it->st_out));
        }
        PSIM_CUDA(cudaStreamWaitEvent(it->st_out, it->ev_run[k], 0));
        PSIM_CUDA(cudaMemcpyAsync(pos + o3, it->pos.as<double>() + o3, b3,
                                  cudaMemcpyDeviceToHost, it->st_out));
        PSIM_CUDA(cudaMemcpyAsync(pos0 + o3, it->pos0.as<double>() + o3, b3,
                                  cudaMemcpyDeviceToHost, it->st_out));
        if (vel_step)
            PSIM_CUDA(cudaMemcpyAsync(vel + o3, it->vel.as<double>() + o3, b3,
                                      cudaMemcpyDeviceToHost, it->st_out));
    }
    uint32_t bits = 0;
    PSIM_CUDA(cudaMemcpyAsync(&bits, it->err.p, 4, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaStreamSynchronize(it->st_in));
    PSIM_CUDA(cudaStreamSynchronize(it->st_out));
    PSIM_CUDA(cudaStreamSynchronize(st));
    if (!first)  // brownianIntegrator.cpp:291-292
        it->vel_counter = (it->vel_counter == it->vp.vel_freq) ? 0 : it->vel_counter + 1;
    it->steps++;
    cudaSetDevice(prev);
    if (bits) return fail(code_from_bits(bits), "%s", bits_text(bits));
    return PSIM_OK;
}

}  // extern "C"

// ================================================================ system

struct psim_system {
    psim_system_config cfg{};
    int device = 0;
    cudaStream_t st = nullptr, side = nullptr;
    cudaEvent_t ev_snap_ready = nullptr, ev_snap_done = nullptr;
    cudaEvent_t ev[5] = {};
    DevGeom g{};
    ForceSetup fs{};
    VgbParams vp{};
    int n = 0, ncell = 0;
    // storage-order state (ping-pong) and order-dependent arrays
    DevBuf pos[2], pos0[2], mem[2], frc[3], tag[2], radius[2], inv_mass[2], perm[2], count[2];
    DevBuf cellid, key, rank, tmp, start, scratch, posd, posh, posl, vel, err, state, occ, noise,
        snap;
    long long noise_first = 0, noise_steps = 0;
    long long total = 0;      // steps since upload, as the host has enqueued them
    bool uploaded = false;
    bool snap_pending = false;
    // one graph per buffer phase (one step), and one of kGraphSteps steps
    // starting at phase 0 (fewer graph launches for small systems)
    cudaGraphExec_t graph[6] = {};
    cudaGraphExec_t graph_multi = nullptr;
    uint32_t latched = 0;
    // Verlet pair list of the mixed form (list_on): list slot of each storage
    // slot (ping-pong with the order), positions at the build, entries,
    // counts, and the two step-parity rebuild flags
    bool list_on = false;
    int list_lanes = 1;   // threads per particle of the list force pass (1, 2 or 4)
    double skin = 0.0;
    int lcap = 0, hcap = 0;
    float lpre = 0.f, ldisp2 = 0.f, hr = 0.f;
    DevBuf lslot[2], lbuild, lpos, list, lcount, lflag, lhalo, lhcount;
    // With a pair list the cell list is rebuilt only with the list (the
    // storage order then stays the list order between builds): the state is
    // carried into the new order through pscratch (15 n doubles), and the
    // per-slot arrays live in buffer 0 (buffer 1 receives a new order or the
    // cell view of the current positions that refresh_cells computes).
    DevBuf pscratch;
    cudaGraphConditionalHandle cond = 0;   // the rebuild's conditional node (graph capture)
    // compact 16-byte records when every particle has one radius (set by the upload)
    int lcompact = 0;
    float lradius = 0.f, lunit = 0.f;
    // a batch of independent replicas (psim_batch_create): per-warp tasks,
    // per-replica grids, pair functors, prefilter bounds and seeds, and the
    // replica of each storage slot (fixed: the cells of a replica are
    // contiguous, so its particles keep their slot range in every cell order)
    int n_reps = 0, n_tasks = 0;
    DevBuf b_tasks, b_geoms, b_pairs, b_pre, b_rep, b_seeds;
    // a batch with a pair list: per replica the list radius squared and the
    // halo radius; the largest cutoff (the compact records' unit)
    DevBuf b_lpre, b_hr;
    double lmaxrc = 0.0;
    // displacement tracker: box images crossed per particle and the start
    // positions (original order), counted by the integrator once started
    DevBuf img, track_start;
};

namespace {

struct Phase {
    int sb, ob, cb, pb, fprev, fcur;
};

// steps in one multi-step graph: a whole number of buffer periods (6)
constexpr int kGraphSteps = 12;

// Buffer roles after `t` steps (t = 0: just uploaded).  Period 6: the
// ping-pong pairs flip every step, the three force buffers rotate.
Phase phase_of(long long t) {
    Phase p;
    const int par = (int)(t & 1);
    p.sb = par;
    p.ob = par;
    p.cb = par;
    p.pb = par;
    p.fprev = (int)(t % 3);
    p.fcur = (p.fprev + 1) % 3;
    return p;
}

double* d3(DevBuf& b, int n, int k) { return b.as<double>() + (size_t)k * n; }

// The list-order records the canonicalisation writes when the list is
// rebuilt: positions, build positions and halo images.
void set_halo_args(psim_system* s, CanonArgs& ca) {
    ca.xorder = 1;   // each row of cells sorted by x: the list build trims its runs
    ca.lbuild = s->lbuild.as<float4>();
    ca.lpos = s->lpos.as<float4>();
    ca.linv_unit = s->lcompact ? 1.0f / s->lunit : 0.f;
    ca.lhalo = s->lhalo.as<int>();
    ca.lhcount = s->lhcount.as<int>();
    ca.hcap = s->hcap;
    ca.hr = s->hr;
    ca.Lf = (float)s->g.L;
    ca.Lhi = s->g.Lhi;
    ca.Llo = s->g.Llo;
    if (s->n_reps) {   // each replica's own box and halo radius
        ca.rep = s->b_rep.as<int>();
        ca.geoms = s->b_geoms.as<DevGeom>();
        ca.hr_rep = s->b_hr.as<float>();
    }
}

// The pair-list build on the cell order just made (count buffer cb), run
// only when *gate != 0.
cudaError_t enqueue_list_build(psim_system* s, int cb, const int* gate) {
    CellView cv{nullptr, s->posh.as<float4>(), s->posl.as<float4>(), s->cellid.as<int>(),
                s->start.as<int>(), s->count[cb].as<int>()};
    ListBuild lb{s->list.as<uint32_t>(), s->lcount.as<int>(), s->n, s->lcap, s->lpre, gate,
                 s->lhalo.as<int>(), s->n};
    lb.xsorted = 1;   // the order set_halo_args asks the canonicalisation for
    if (s->n_reps) {   // each replica's own grid and list radius
        lb.rep = s->b_rep.as<int>();
        lb.geoms = s->b_geoms.as<DevGeom>();
        lb.pre = s->b_lpre.as<float>();
    }
    return launch_list_build(s->g, cv, lb, s->err.as<uint32_t>(), s->st);
}

// The force pass on the state after `total` steps (phase ph): the cell walk,
// or the pair list in the mixed form with a skin; forces in storage order.
cudaError_t enqueue_force(psim_system* s, const Phase& ph, const ForceOut& fo) {
    CellView cv{s->posd.as<double4_32a>(), s->posh.as<float4>(), s->posl.as<float4>(),
                s->cellid.as<int>(), s->start.as<int>(), s->count[ph.cb].as<int>()};
    if (s->cfg.force_launch) {   // a plugin's device entry (single systems only)
        const ForceRunner fr{&s->fs, s->cfg.force_launch, &s->cfg.force};
        if (s->cfg.precision == PSIM_PRECISION_FP64)
            return fr.run(PSIM_PASS_FP64, s->g, &cv, nullptr, fo, s->st);
        if (s->list_on) {
            PairList pl{nullptr, s->lpos.as<float4>(), s->lcount.as<int>(),
                        s->list.as<uint32_t>(), s->n, s->lcompact, s->lradius, s->lunit};
            return fr.run(PSIM_PASS_LIST, s->g, nullptr, &pl, fo, s->st);
        }
        return fr.run(PSIM_PASS_MIXED, s->g, &cv, nullptr, fo, s->st);
    }
    if (s->n_reps && s->list_on) {   // each particle with its replica's pair functor
        PairList pl{nullptr, s->lpos.as<float4>(), s->lcount.as<int>(), s->list.as<uint32_t>(),
                    s->n, s->lcompact, s->lradius, s->lunit, s->b_rep.as<int>(), s->b_pairs.p};
        pl.lanes = s->list_lanes;
        return launch_forces_list(s->fs, s->g, pl, fo, s->st);
    }
    if (s->n_reps) {
        BatchView bv{s->b_tasks.as<int2>(), s->n_tasks, s->b_geoms.as<DevGeom>(),
                     s->b_pairs.p, s->b_pre.as<float>()};
        if (s->cfg.precision == PSIM_PRECISION_FP64)
            return launch_forces_fp64(s->fs, s->g, cv, fo, s->st, &bv);
        return launch_forces_mixed(s->fs, s->g, cv, fo, s->st, &bv);
    }
    if (s->cfg.precision == PSIM_PRECISION_FP64) return launch_forces_fp64(s->fs, s->g, cv, fo, s->st);
    if (s->list_on) {
        // the storage order is the list order: no slot table
        PairList pl{nullptr, s->lpos.as<float4>(), s->lcount.as<int>(),
                    s->list.as<uint32_t>(), s->n, s->lcompact, s->lradius, s->lunit};
        pl.lanes = s->list_lanes;
        return launch_forces_list(s->fs, s->g, pl, fo, s->st);
    }
    return launch_forces_mixed(s->fs, s->g, cv, fo, s->st);
}

// ---- the step with a pair list: the cell list is rebuilt with the list only
//
// force (list) -> vGB (no permutation, no hash) -> step end, then, on the
// steps whose integrator raised the rebuild flag, the rebuild: hash + count,
// scan, scatter, canonicalisation into the new cell order (list records and
// halo images included), the state carried into that order, the list build.
// In a graph the rebuild is the body of a conditional node that the step end
// sets; so a step without a rebuild launches three kernels.  The forces and
// the trajectory are those of the cell list rebuilt every step: the same
// pair terms in the same list order, the same per-particle arithmetic.

// The rebuild after step t (phase of t): the state the integrator wrote (in
// the storage order) sorted into the new cell order.
int enqueue_rebuild_lazy(psim_system* s, long long t) {
    const Phase ph = phase_of(t);
    const int n = s->n, nsb = 1 - ph.sb;
    cudaStream_t st = s->st;
    uint32_t* err = s->err.as<uint32_t>();
    PSIM_CUDA(cudaMemsetAsync(s->count[0].p, 0, 4 * (size_t)s->ncell, st));
    PSIM_CUDA(launch_hash_count(n, d3(s->pos[nsb], n, 0), d3(s->pos[nsb], n, 1),
                                d3(s->pos[nsb], n, 2), s->g, s->key.as<int>(), s->rank.as<int>(),
                                s->count[0].as<int>(), err, st,
                                s->n_reps ? s->b_rep.as<int>() : nullptr,
                                s->n_reps ? s->b_geoms.as<DevGeom>() : nullptr));
    PSIM_CUDA(launch_scan(s->count[0].as<int>(), s->start.as<int>(), s->ncell,
                          s->scratch.as<int>(), st));
    PSIM_CUDA(launch_scatter(n, s->key.as<int>(), s->rank.as<int>(), s->start.as<int>(),
                             s->tmp.as<int>(), err, st));
    CanonArgs ca{};
    ca.n = n;
    ca.tmp = s->tmp.as<int>();
    ca.key = s->key.as<int>();
    ca.start = s->start.as<int>();
    ca.count = s->count[0].as<int>();
    ca.tag_in = s->tag[0].as<int>();
    ca.radius_in = s->radius[0].as<double>();
    ca.inv_mass_in = s->inv_mass[0].as<double>();
    ca.x = d3(s->pos[nsb], n, 0); ca.y = d3(s->pos[nsb], n, 1); ca.z = d3(s->pos[nsb], n, 2);
    ca.perm = s->perm[0].as<int>();
    ca.tag_out = s->tag[1].as<int>();
    ca.radius_out = s->radius[1].as<double>();
    ca.inv_mass_out = s->inv_mass[1].as<double>();
    ca.cellid = s->cellid.as<int>();
    ca.posh = s->posh.as<float4>();
    ca.vel_freq = s->vp.vel_freq;
    ca.err = err;
    set_halo_args(s, ca);   // list records, build positions and halo images on the new order
    PSIM_CUDA(launch_canonicalize(ca, st));
    // the state into the new order: positions, previous positions, noise
    // memory, and the forces of this step and the one before
    DevBuf* arrs[5] = {&s->pos[nsb], &s->pos0[nsb], &s->mem[nsb], &s->frc[ph.fcur],
                       &s->frc[ph.fprev]};
    PermuteArgs pa{};
    pa.n = n;
    pa.perm = s->perm[0].as<int>();
    pa.narr = 15;
    double* scr = s->pscratch.as<double>();
    for (int a = 0; a < 5; ++a)
        for (int k = 0; k < 3; ++k) {
            pa.src[3 * a + k] = d3(*arrs[a], n, k);
            pa.dst[3 * a + k] = scr + (size_t)(3 * a + k) * n;
        }
    PSIM_CUDA(launch_permute(pa, err, st));
    for (int a = 0; a < 5; ++a)
        PSIM_CUDA(cudaMemcpyAsync(arrs[a]->p, scr + (size_t)3 * a * n, 24 * (size_t)n,
                                  cudaMemcpyDeviceToDevice, st));
    PSIM_CUDA(cudaMemcpyAsync(s->tag[0].p, s->tag[1].p, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    PSIM_CUDA(cudaMemcpyAsync(s->radius[0].p, s->radius[1].p, 8 * (size_t)n,
                              cudaMemcpyDeviceToDevice, st));
    PSIM_CUDA(cudaMemcpyAsync(s->inv_mass[0].p, s->inv_mass[1].p, 8 * (size_t)n,
                              cudaMemcpyDeviceToDevice, st));
    PSIM_CUDA(enqueue_list_build(s, 0, nullptr));
    return PSIM_OK;
}

// Step t with a pair list.  In a graph (evs null) this enqueues the force
// pass, the integrator and the step end; the caller adds the conditional
// rebuild.  Timed directly (evs: 4 events), the rebuild decision is read back.
int enqueue_step_lazy(psim_system* s, long long t, cudaEvent_t* evs) {
    const Phase ph = phase_of(t);
    const int n = s->n, sb = ph.sb, nsb = 1 - ph.sb;
    cudaStream_t st = s->st;
    int* lflag = s->lflag.as<int>() + (t & 1);
    if (evs) PSIM_CUDA(cudaEventRecord(evs[0], st));
    ForceOut fo{d3(s->frc[ph.fcur], n, 0), d3(s->frc[ph.fcur], n, 1), d3(s->frc[ph.fcur], n, 2),
                s->err.as<uint32_t>(), nullptr};
    PSIM_CUDA(enqueue_force(s, ph, fo));
    if (evs) PSIM_CUDA(cudaEventRecord(evs[1], st));
    VgbSystemArgs a{};
    a.n = n;
    a.perm = nullptr;   // the storage order has not changed since the last rebuild
    a.tag = s->tag[0].as<int>();
    a.inv_mass = s->inv_mass[0].as<double>();
    a.x = d3(s->pos[sb], n, 0); a.y = d3(s->pos[sb], n, 1); a.z = d3(s->pos[sb], n, 2);
    a.x0 = d3(s->pos0[sb], n, 0); a.y0 = d3(s->pos0[sb], n, 1); a.z0 = d3(s->pos0[sb], n, 2);
    a.mx = d3(s->mem[sb], n, 0); a.my = d3(s->mem[sb], n, 1); a.mz = d3(s->mem[sb], n, 2);
    a.fx = fo.fx; a.fy = fo.fy; a.fz = fo.fz;
    a.gx = d3(s->frc[ph.fprev], n, 0); a.gy = d3(s->frc[ph.fprev], n, 1);
    a.gz = d3(s->frc[ph.fprev], n, 2);
    a.vel = s->vel.as<double>();
    a.ox = d3(s->pos[nsb], n, 0); a.oy = d3(s->pos[nsb], n, 1); a.oz = d3(s->pos[nsb], n, 2);
    a.ox0 = d3(s->pos0[nsb], n, 0); a.oy0 = d3(s->pos0[nsb], n, 1); a.oz0 = d3(s->pos0[nsb], n, 2);
    a.omx = d3(s->mem[nsb], n, 0); a.omy = d3(s->mem[nsb], n, 1); a.omz = d3(s->mem[nsb], n, 2);
    a.count = nullptr;  // no hash: the cell list is rebuilt with the list
    a.err = s->err.as<uint32_t>();
    a.state = s->state.as<StepState>();
    a.lslot = nullptr;  // list slot = storage slot
    a.lbuild = s->lbuild.as<float4>();
    a.lpos = s->lpos.as<float4>();
    a.linv_unit = s->lcompact ? 1.0f / s->lunit : 0.f;
    a.lflag_set = lflag;
    a.lflag_clear = s->lflag.as<int>() + (1 - (t & 1));
    a.ldisp2 = s->ldisp2;
    a.lhalo = s->lhalo.as<int>();
    a.lhcount = s->lhcount.as<int>();
    a.img = s->img.as<int>();
    if (s->n_reps) {
        a.rep = s->b_rep.as<int>();
        a.geoms = s->b_geoms.as<DevGeom>();
        a.seeds = s->b_seeds.as<uint32_t>();
    }
    NoiseView nz{s->cfg.noise_mode, s->noise.as<double>(), s->noise_first, s->noise_steps};
    PSIM_CUDA(launch_vgb_system_fast(a, s->vp, s->g, nz, st));
    if (evs) PSIM_CUDA(cudaEventRecord(evs[2], st));
    PSIM_CUDA(launch_step_end(s->state.as<StepState>(), lflag, s->err.as<uint32_t>(),
                              s->vp.vel_freq, s->cond, evs ? 0 : 1, st));
    if (evs) {
        int flag = 0;
        uint32_t bits = 0;
        PSIM_CUDA(cudaMemcpyAsync(&flag, lflag, 4, cudaMemcpyDeviceToHost, st));
        PSIM_CUDA(cudaMemcpyAsync(&bits, s->err.p, 4, cudaMemcpyDeviceToHost, st));
        PSIM_CUDA(cudaStreamSynchronize(st));
        if (flag && !bits) {
            const int rc = enqueue_rebuild_lazy(s, t);
            if (rc) return rc;
        }
        PSIM_CUDA(cudaEventRecord(evs[3], st));
    }
    return PSIM_OK;
}

int enqueue_step(psim_system* s, long long t, cudaEvent_t* evs) {
    if (s->list_on) return enqueue_step_lazy(s, t, evs);
    const Phase ph = phase_of(t);
    const int n = s->n;
    cudaStream_t st = s->st;
    const int sb = ph.sb, nsb = 1 - ph.sb, ob = ph.ob, nob = 1 - ph.ob, cb = ph.cb, ncb = 1 - ph.cb;
    const int pb = ph.pb, npb = 1 - ph.pb;
    // the rebuild flag of this step's parity (pair list only)
    int* lflag = s->list_on ? s->lflag.as<int>() + (t & 1) : nullptr;
    if (evs) PSIM_CUDA(cudaEventRecord(evs[0], st));
    ForceOut fo{d3(s->frc[ph.fcur], n, 0), d3(s->frc[ph.fcur], n, 1), d3(s->frc[ph.fcur], n, 2),
                s->err.as<uint32_t>(), nullptr};
    PSIM_CUDA(enqueue_force(s, ph, fo));
    if (evs) PSIM_CUDA(cudaEventRecord(evs[1], st));
    // integrator: pushParticleForce + nextSystem, hash + count into the next grid
    PSIM_CUDA(cudaMemsetAsync(s->count[ncb].p, 0, 4 * (size_t)s->ncell, st));
    VgbSystemArgs a{};
    a.n = n;
    a.perm = s->perm[pb].as<int>();
    a.tag = s->tag[ob].as<int>();
    a.inv_mass = s->inv_mass[ob].as<double>();
    a.x = d3(s->pos[sb], n, 0); a.y = d3(s->pos[sb], n, 1); a.z = d3(s->pos[sb], n, 2);
    a.x0 = d3(s->pos0[sb], n, 0); a.y0 = d3(s->pos0[sb], n, 1); a.z0 = d3(s->pos0[sb], n, 2);
    a.mx = d3(s->mem[sb], n, 0); a.my = d3(s->mem[sb], n, 1); a.mz = d3(s->mem[sb], n, 2);
    a.fx = fo.fx; a.fy = fo.fy; a.fz = fo.fz;
    a.gx = d3(s->frc[ph.fprev], n, 0); a.gy = d3(s->frc[ph.fprev], n, 1);
    a.gz = d3(s->frc[ph.fprev], n, 2);
    a.vel = s->vel.as<double>();
    a.ox = d3(s->pos[nsb], n, 0); a.oy = d3(s->pos[nsb], n, 1); a.oz = d3(s->pos[nsb], n, 2);
    a.ox0 = d3(s->pos0[nsb], n, 0); a.oy0 = d3(s->pos0[nsb], n, 1); a.oz0 = d3(s->pos0[nsb], n, 2);
    a.omx = d3(s->mem[nsb], n, 0); a.omy = d3(s->mem[nsb], n, 1); a.omz = d3(s->mem[nsb], n, 2);
    a.key = s->key.as<int>();
    a.rank = s->rank.as<int>();
    a.count = s->count[ncb].as<int>();
    a.err = s->err.as<uint32_t>();
    a.state = s->state.as<StepState>();
    if (s->list_on) {
        a.lslot = s->lslot[ob].as<int>();
        a.lbuild = s->lbuild.as<float4>();
        a.lpos = s->lpos.as<float4>();
        a.linv_unit = s->lcompact ? 1.0f / s->lunit : 0.f;
        a.lflag_set = lflag;
        a.lflag_clear = s->lflag.as<int>() + (1 - (t & 1));
        a.ldisp2 = s->ldisp2;
        a.lhalo = s->lhalo.as<int>();
        a.lhcount = s->lhcount.as<int>();
    }
    if (s->n_reps) {
        a.rep = s->b_rep.as<int>();
        a.geoms = s->b_geoms.as<DevGeom>();
        a.seeds = s->b_seeds.as<uint32_t>();
    }
    a.img = s->img.as<int>();   // null until the displacement tracker starts
    NoiseView nz{s->cfg.noise_mode, s->noise.as<double>(), s->noise_first, s->noise_steps};
    if (s->cfg.precision == PSIM_PRECISION_FP64)
        PSIM_CUDA(launch_vgb_system(a, s->vp, s->g, nz, st));
    else
        PSIM_CUDA(launch_vgb_system_fast(a, s->vp, s->g, nz, st));
    if (evs) PSIM_CUDA(cudaEventRecord(evs[2], st));
    // rebuild: scan, scatter, canonicalise into the next order
    PSIM_CUDA(launch_scan(s->count[ncb].as<int>(), s->start.as<int>(), s->ncell,
                          s->scratch.as<int>(), st));
    PSIM_CUDA(launch_scatter(n, s->key.as<int>(), s->rank.as<int>(), s->start.as<int>(),
                             s->tmp.as<int>(), s->err.as<uint32_t>(), st));
    CanonArgs ca{};
    ca.n = n;
    ca.tmp = s->tmp.as<int>();
    ca.key = s->key.as<int>();
    ca.start = s->start.as<int>();
    ca.count = s->count[ncb].as<int>();
    ca.tag_in = s->tag[ob].as<int>();
    ca.radius_in = s->radius[ob].as<double>();
    ca.inv_mass_in = s->inv_mass[ob].as<double>();
    ca.x = a.ox; ca.y = a.oy; ca.z = a.oz;
    ca.perm = s->perm[npb].as<int>();
    ca.tag_out = s->tag[nob].as<int>();
    ca.radius_out = s->radius[nob].as<double>();
    ca.inv_mass_out = s->inv_mass[nob].as<double>();
    ca.cellid = s->cellid.as<int>();
    ca.posd = s->cfg.precision == PSIM_PRECISION_FP64 ? s->posd.as<double4_32a>() : nullptr;
    ca.posh = s->posh.as<float4>();
    ca.posl = s->cfg.precision == PSIM_PRECISION_MIXED ? s->posl.as<float4>() : nullptr;
    ca.state = s->state.as<StepState>();
    ca.advance = 1;
    ca.vel_freq = s->vp.vel_freq;
    ca.err = s->err.as<uint32_t>();
    if (s->list_on) {
        ca.rebuild = lflag;
        ca.lslot_in = s->lslot[ob].as<int>();
        ca.lslot_out = s->lslot[nob].as<int>();
        set_halo_args(s, ca);
    }
    PSIM_CUDA(launch_canonicalize(ca, st));
    if (s->list_on) PSIM_CUDA(enqueue_list_build(s, ncb, lflag));
    if (evs) PSIM_CUDA(cudaEventRecord(evs[3], st));
    return PSIM_OK;
}

// The step graph with a pair list: the step, then a conditional node (set by
// the step end) whose body is the rebuild.
// Steps phase .. phase + steps - 1 with a pair list, captured into one graph:
// each step's kernels followed by a conditional node whose body is that
// step's rebuild (the step end sets the node's condition).
int graph_lazy_steps(psim_system* s, int phase, int steps, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    PSIM_CUDA(cudaGraphCreate(&g, 0));
    auto done = [&](int rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    };
    // a condition handle per conditional node: the step end that sets it is
    // captured with s->cond holding that step's handle
    std::vector<cudaGraphConditionalHandle> conds(steps);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < steps && e == cudaSuccess; ++k)
        e = cudaGraphConditionalHandleCreate(&conds[k], g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess)
        return done(fail(PSIM_ERR_CUDA, "conditional handle: %s", cudaGetErrorString(e)));
    std::vector<cudaGraph_t> bodies;
    e = cudaStreamBeginCaptureToGraph(s->st, g, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return done(fail(PSIM_ERR_CUDA, "capture: %s", cudaGetErrorString(e)));
    int rc = PSIM_OK;
    for (int k = 0; k < steps && !rc; ++k) {
        s->cond = conds[k];
        rc = enqueue_step_lazy(s, phase + k, nullptr);
        if (rc) break;
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaGraph_t cg = nullptr;
        e = cudaStreamGetCaptureInfo(s->st, &cs, nullptr, &cg, &deps, nullptr, &nd);
        cudaGraphNode_t cn = nullptr;
        cudaGraphNodeParams cp{};
        if (e == cudaSuccess) {
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = s->cond;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            std::vector<cudaGraphNode_t> dv(deps, deps + nd);
            e = cudaGraphAddNode(&cn, cg, dv.data(), nullptr, dv.size(), &cp);
        }
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(s->st, &cn, nullptr, 1,
                                                    cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess)
            rc = fail(PSIM_ERR_CUDA, "conditional node: %s", cudaGetErrorString(e));
        else
            bodies.push_back(cp.conditional.phGraph_out[0]);
    }
    cudaGraph_t captured = g;
    e = cudaStreamEndCapture(s->st, &captured);
    if (rc) return done(rc);
    if (e != cudaSuccess) return done(fail(PSIM_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e)));
    // the bodies: each step's rebuild, captured into its node's own graph
    for (int k = 0; k < steps; ++k) {
        cudaGraph_t body = bodies[k];
        e = cudaStreamBeginCaptureToGraph(s->st, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return done(fail(PSIM_ERR_CUDA, "capture: %s", cudaGetErrorString(e)));
        rc = enqueue_rebuild_lazy(s, phase + k);
        cudaGraph_t bcap = body;
        e = cudaStreamEndCapture(s->st, &bcap);
        if (rc) return done(rc);
        if (e != cudaSuccess)
            return done(fail(PSIM_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e)));
    }
    e = cudaGraphInstantiate(out, g, 0);
    if (e != cudaSuccess)
        return done(fail(PSIM_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e)));
    return done(PSIM_OK);
}

// Steps phase .. phase + steps - 1, captured into one graph.
int graph_steps(psim_system* s, int phase, int steps, cudaGraphExec_t* out) {
    if (s->list_on) return graph_lazy_steps(s, phase, steps, out);
    cudaGraph_t g = nullptr;
    PSIM_CUDA(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    int rc = PSIM_OK;
    for (int k = 0; k < steps && !rc; ++k) rc = enqueue_step(s, phase + k, nullptr);
    cudaError_t e = cudaStreamEndCapture(s->st, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return fail(PSIM_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(PSIM_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    return PSIM_OK;
}

int graph_for(psim_system* s, int phase, cudaGraphExec_t* out) {
    if (!s->graph[phase]) {
        int rc = graph_steps(s, phase, 1, &s->graph[phase]);
        if (rc) return rc;
    }
    *out = s->graph[phase];
    return PSIM_OK;
}

void drop_graphs(psim_system* s) {
    for (auto& g : s->graph)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    if (s->graph_multi) { cudaGraphExecDestroy(s->graph_multi); s->graph_multi = nullptr; }
}

struct DeviceGuard {
    int prev = 0;
    explicit DeviceGuard(int d) { cudaGetDevice(&prev); cudaSetDevice(d); }
    ~DeviceGuard() { cudaSetDevice(prev); }
};

// Waits for the stream, reads the error word and the device step counter,
// and re-aligns the host's step count with the steps the device completed.
int settle(psim_system* s) {
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    uint32_t bits = 0;
    StepState ss{};
    PSIM_CUDA(cudaMemcpy(&bits, s->err.p, 4, cudaMemcpyDeviceToHost));
    PSIM_CUDA(cudaMemcpy(&ss, s->state.p, sizeof ss, cudaMemcpyDeviceToHost));
    s->total = ss.step;
    if (bits) {
        s->latched = bits;
        return fail(code_from_bits(bits), "step %lld: %s", ss.step, bits_text(bits));
    }
    return PSIM_OK;
}

// The tags of the storage order (the order of the state arrays) after the
// steps taken: the previous cell order, or with a pair list the order of the
// last rebuild.
const int* store_tags(psim_system* s) {
    if (s->list_on) return s->tag[0].as<int>();
    return s->tag[1 - phase_of(s->total).ob].as<int>();
}
// The permutation from the storage order to the order of the force two steps
// back (null: the same order).
const int* prev_perm(psim_system* s) {
    return s->list_on ? nullptr : s->perm[1 - phase_of(s->total).pb].as<int>();
}

// A cell list of the current positions: per cell-order slot its storage slot,
// tag and radius, and the counts per cell (with start and cellid in the
// system's buffers).
struct CellRefs {
    const int* perm;
    const int* tag;
    const double* radius;
    const int* count;
};
// Without a pair list: the one the last step built.  With one, the stored cell
// list is that of the last rebuild, so it is computed afresh into buffer 1
// from the current positions; the system's order, list and state are left
// alone (the float positions posh it rewrites are read only by a rebuild,
// after rewriting them).
int cell_refs(psim_system* s, CellRefs& c) {
    const Phase ph = phase_of(s->total);
    if (!s->list_on) {
        c = CellRefs{s->perm[ph.pb].as<int>(), s->tag[ph.ob].as<int>(),
                     s->radius[ph.ob].as<double>(), s->count[ph.cb].as<int>()};
        return PSIM_OK;
    }
    const int n = s->n;
    cudaStream_t st = s->st;
    uint32_t* err = s->err.as<uint32_t>();
    PSIM_CUDA(cudaMemsetAsync(s->count[0].p, 0, 4 * (size_t)s->ncell, st));
    PSIM_CUDA(launch_hash_count(n, d3(s->pos[ph.sb], n, 0), d3(s->pos[ph.sb], n, 1),
                                d3(s->pos[ph.sb], n, 2), s->g, s->key.as<int>(), s->rank.as<int>(),
                                s->count[0].as<int>(), err, st,
                                s->n_reps ? s->b_rep.as<int>() : nullptr,
                                s->n_reps ? s->b_geoms.as<DevGeom>() : nullptr));
    PSIM_CUDA(launch_scan(s->count[0].as<int>(), s->start.as<int>(), s->ncell,
                          s->scratch.as<int>(), st));
    PSIM_CUDA(launch_scatter(n, s->key.as<int>(), s->rank.as<int>(), s->start.as<int>(),
                             s->tmp.as<int>(), err, st));
    CanonArgs ca{};
    ca.n = n;
    ca.tmp = s->tmp.as<int>();
    ca.key = s->key.as<int>();
    ca.start = s->start.as<int>();
    ca.count = s->count[0].as<int>();
    ca.tag_in = s->tag[0].as<int>();
    ca.radius_in = s->radius[0].as<double>();
    ca.x = d3(s->pos[ph.sb], n, 0); ca.y = d3(s->pos[ph.sb], n, 1); ca.z = d3(s->pos[ph.sb], n, 2);
    ca.perm = s->perm[1].as<int>();
    ca.tag_out = s->tag[1].as<int>();
    ca.radius_out = s->radius[1].as<double>();
    ca.cellid = s->cellid.as<int>();
    ca.posh = s->posh.as<float4>();
    ca.err = err;
    PSIM_CUDA(launch_canonicalize(ca, st));
    c = CellRefs{s->perm[1].as<int>(), s->tag[1].as<int>(), s->radius[1].as<double>(),
                 s->count[0].as<int>()};
    return PSIM_OK;
}

}  // namespace

namespace {
psim_system* system_new(const psim_system_config* cfg, const DevGeom& g, bool batch = false);

}

extern "C" {

psim_system* psim_system_create(const psim_system_config* cfg) {
    if (!cfg) { fail(PSIM_ERR_INPUT, "NULL config"); return nullptr; }
    if (check_params(&cfg->force, cfg->force_launch != nullptr)) return nullptr;
    if (cfg->precision != PSIM_PRECISION_FP64 && cfg->precision != PSIM_PRECISION_MIXED) {
        fail(PSIM_ERR_INPUT, "unknown precision %d", cfg->precision);
        return nullptr;
    }
    if (cfg->noise_mode != PSIM_NOISE_PHILOX && cfg->noise_mode != PSIM_NOISE_INJECTED) {
        fail(PSIM_ERR_INPUT, "unknown noise mode %d", cfg->noise_mode);
        return nullptr;
    }
    DevGeom g;
    if (make_geom(&cfg->geom, max_cutoff(&cfg->force), &g)) return nullptr;
    return system_new(cfg, g);
}

psim_system* psim_batch_create(const psim_replica* reps, int32_t n_reps,
                               const psim_integrator_config* integ, int32_t precision,
                               int32_t noise_mode, int32_t device) {
    return psim_batch_create_list(reps, n_reps, integ, precision, noise_mode, device, 0.0);
}

psim_system* psim_batch_create_list(const psim_replica* reps, int32_t n_reps,
                                    const psim_integrator_config* integ, int32_t precision,
                                    int32_t noise_mode, int32_t device, double skin) {
    if (!reps || n_reps <= 0 || !integ) {
        fail(PSIM_ERR_INPUT, "a batch needs at least one replica and an integrator config");
        return nullptr;
    }
    if (!(skin >= 0.0) || (skin > 0.0 && precision != PSIM_PRECISION_MIXED)) {
        fail(PSIM_ERR_INPUT, "a pair-list skin needs the mixed precision form (skin %g)", skin);
        return nullptr;
    }
    for (int r = 0; r < n_reps && skin > 0.0; ++r) {
        const double need = max_cutoff(&reps[r].force) + skin;
        if (reps[r].geom.cell_size < need) {
            fail(PSIM_ERR_INPUT, "replica %d: pair-list skin %g needs cellSize >= cutOff + skin "
                 "(%g < %g)", r, skin, reps[r].geom.cell_size, need);
            return nullptr;
        }
    }
    const int kind = reps[0].force.kind;
    if (kind == PSIM_FORCE_AO_YUKAWA) {
        fail(PSIM_ERR_INPUT, "a batch holds single-plugin replicas (not the AO + Yukawa composite)");
        return nullptr;
    }
    std::vector<DevGeom> geoms((size_t)n_reps);
    long long P = 0, C = 0;
    for (int r = 0; r < n_reps; ++r) {
        const psim_force_params* f = &reps[r].force;
        if (check_params(f)) return nullptr;
        if (f->kind != kind || (kind == PSIM_FORCE_LJ && f->lj_num != reps[0].force.lj_num)) {
            fail(PSIM_ERR_INPUT, "replica %d: every replica of a batch uses the same plugin "
                 "(and ljNum)", r);
            return nullptr;
        }
        DevGeom& g = geoms[r];
        if (make_geom(&reps[r].geom, max_cutoff(f), &g)) return nullptr;
        g.c0 = (int)C;
        g.p0 = (int)P;
        g.p1 = (int)(P + g.n);
        P += g.n;
        C += g.ncell;
        if (P > INT32_MAX / 2 || C > INT32_MAX / 2) {
            fail(PSIM_ERR_INPUT, "the batch holds too many particles or cells");
            return nullptr;
        }
    }
    // the whole batch as one grid for the kernels that need no geometry
    DevGeom gt = geoms[0];
    gt.n = (int)P;
    gt.ncell = (int)C;
    gt.c0 = 0;
    gt.p0 = 0;
    gt.p1 = (int)P;
    psim_system_config cfg{};
    cfg.geom = reps[0].geom;
    cfg.geom.n_particles = (int)P;
    cfg.integ = *integ;
    cfg.force = reps[0].force;
    cfg.precision = precision;
    cfg.noise_mode = noise_mode;
    cfg.device = device;
    cfg.skin = skin;
    if (precision != PSIM_PRECISION_FP64 && precision != PSIM_PRECISION_MIXED) {
        fail(PSIM_ERR_INPUT, "unknown precision %d", precision);
        return nullptr;
    }
    if (noise_mode != PSIM_NOISE_PHILOX && noise_mode != PSIM_NOISE_INJECTED) {
        fail(PSIM_ERR_INPUT, "unknown noise mode %d", noise_mode);
        return nullptr;
    }
    psim_system* s = system_new(&cfg, gt, true);
    if (!s) return nullptr;
    DeviceGuard dg(s->device);
    s->fs.tile = 0;
    s->fs.walk = choose_walk();
    // warp tasks aligned to the replicas' particle ranges
    std::vector<int2> tasks;
    std::vector<int> rep((size_t)P);
    std::vector<float> pre((size_t)n_reps);
    std::vector<uint32_t> seeds((size_t)n_reps);
    std::vector<unsigned char> pairs;
    for (int r = 0; r < n_reps; ++r) {
        const DevGeom& g = geoms[r];
        for (int i0 = g.p0; i0 < g.p1; i0 += 32) tasks.push_back(make_int2(r, i0));
        for (int i = g.p0; i < g.p1; ++i) rep[(size_t)i] = r;
        const ForceSetup fr = make_setup(&reps[r].force, g.L);
        s->fs.lj_pure = s->fs.lj_pure && fr.lj_pure;
        pre[(size_t)r] = fr.pre_rc2f;
        seeds[(size_t)r] = (uint32_t)reps[r].seed;
        const void* src = kind == PSIM_FORCE_AO ? (const void*)&fr.ao
                          : kind == PSIM_FORCE_LJ ? (const void*)&fr.lj : (const void*)&fr.cal;
        const size_t sz = kind == PSIM_FORCE_AO ? sizeof(AOPair)
                          : kind == PSIM_FORCE_LJ ? sizeof(LJPair) : sizeof(CalPair);
        const unsigned char* b = static_cast<const unsigned char*>(src);
        pairs.insert(pairs.end(), b, b + sz);
    }
    s->n_reps = n_reps;
    s->n_tasks = (int)tasks.size();
    auto put = [&](DevBuf& d, const void* h, size_t bytes) {
        return !d.ensure(bytes ? bytes : 16) &&
               (bytes == 0 || cudaMemcpy(d.p, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess);
    };
    const bool ok = put(s->b_tasks, tasks.data(), tasks.size() * sizeof(int2)) &&
                    put(s->b_geoms, geoms.data(), geoms.size() * sizeof(DevGeom)) &&
                    put(s->b_pairs, pairs.data(), pairs.size()) &&
                    put(s->b_pre, pre.data(), pre.size() * sizeof(float)) &&
                    put(s->b_rep, rep.data(), rep.size() * sizeof(int)) &&
                    put(s->b_seeds, seeds.data(), seeds.size() * sizeof(uint32_t));
    if (!ok) {
        fail(PSIM_ERR_CUDA, "batch tables: %s", cudaGetErrorString(cudaGetLastError()));
        psim_system_destroy(s);
        return nullptr;
    }
    if (s->list_on) {
        // the list's sizes per replica: entries and halo records for the
        // densest, the rebuild test of the strictest, each radius its own
        std::vector<float> lpre((size_t)n_reps), hr((size_t)n_reps);
        int cap = 0;
        long long hcap = 0;
        float disp2 = 3.0e38f, pre_max = 0.f;
        for (int r = 0; r < n_reps; ++r) {
            const ListSizes z = list_sizes(max_cutoff(&reps[r].force), skin, geoms[r]);
            cap = std::max(cap, z.cap);
            hcap += z.hcap;
            disp2 = std::min(disp2, z.disp2);
            pre_max = std::max(pre_max, z.pre);
            lpre[(size_t)r] = z.pre;
            hr[(size_t)r] = z.hr;
            s->lmaxrc = std::max(s->lmaxrc, max_cutoff(&reps[r].force));
        }
        s->lcap = cap;
        s->hcap = (int)std::min(hcap, (long long)kHaloBaseMax);
        s->ldisp2 = disp2;
        s->lpre = pre_max;
        const size_t n = (size_t)P;
        const bool ok2 = (double)(cap + kListFold) * (double)P < 4294967296.0 &&
                         put(s->b_lpre, lpre.data(), lpre.size() * sizeof(float)) &&
                         put(s->b_hr, hr.data(), hr.size() * sizeof(float)) &&
                         !s->list.ensure(4 * n * (size_t)(cap + kListFold)) &&
                         !s->lpos.ensure(32 * (n + 1 + (size_t)s->hcap));
        if (!ok2) {
            fail(PSIM_ERR_INPUT, "the batch's pair list does not fit (%lld particles, %d entries "
                 "each)", (long long)P, cap);
            psim_system_destroy(s);
            return nullptr;
        }
    }
    return s;
}

}  // extern "C"

namespace {

// The system's streams, events and buffers for grid g (the whole batch's
// particles and cells for a batch); validates the rest of cfg.
psim_system* system_new(const psim_system_config* cfg, const DevGeom& g, bool batch) {
    VgbParams vp;
    if (make_vgb_params(&cfg->integ, &vp)) return nullptr;
    const double rc = max_cutoff(&cfg->force);
    const double skin = cfg->skin;
    const bool list_on = skin > 0.0 && cfg->precision == PSIM_PRECISION_MIXED;
    if (!(skin >= 0.0) || (skin > 0.0 && cfg->precision != PSIM_PRECISION_MIXED)) {
        fail(PSIM_ERR_INPUT, "a pair-list skin needs the mixed precision form (skin %g)", skin);
        return nullptr;
    }
    if (list_on && g.cs < rc + skin) {
        // the list is built from the 27-cell walk, which sees every pair
        // within cellSize only
        fail(PSIM_ERR_INPUT, "pair-list skin %g needs cellSize >= cutOff + skin (%g < %g)", skin,
             g.cs, rc + skin);
        return nullptr;
    }
    if (list_on && g.n > (1 << 28)) {
        fail(PSIM_ERR_INPUT, "the pair list indexes at most 2^28 particles");
        return nullptr;
    }
    if (ensure_device()) return nullptr;
    int ndev = 0;
    cudaGetDeviceCount(&ndev);
    if (cfg->device < 0 || cfg->device >= ndev) {
        fail(PSIM_ERR_INPUT, "device %d out of range", cfg->device);
        return nullptr;
    }
    DeviceGuard dg(cfg->device);
    psim_system* s = new psim_system();
    s->cfg = *cfg;
    s->device = cfg->device;
    s->g = g;
    s->vp = vp;
    s->fs = make_setup(&cfg->force, g.L);
    s->fs.tile = choose_tile(g);
    s->fs.walk = choose_walk();
    s->n = g.n;
    s->ncell = g.ncell;
    if (list_on) {
        // (a batch sizes its list per replica once its tables are made)
        const ListSizes z = batch ? ListSizes{0, 0.f, 0.f, 0.f, 0} : list_sizes(rc, skin, g);
        s->list_on = true;
        s->skin = skin;
        s->lcap = z.cap;
        if ((double)(s->lcap + kListFold) * (double)g.n >= 4294967296.0) {
            // the list build addresses entries with 32-bit offsets
            const int cap = s->lcap;
            delete s;
            fail(PSIM_ERR_INPUT, "the pair list of %d particles (%d entries each) is too large; "
                 "use a smaller skin", g.n, cap);
            return nullptr;
        }
        s->lpre = z.pre;
        s->ldisp2 = z.disp2;
        s->hr = z.hr;
        s->hcap = z.hcap;
    }
    const size_t n = (size_t)g.n, nc = (size_t)g.ncell;
    bool ok = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->ev_snap_ready, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->ev_snap_done, cudaEventDisableTiming) == cudaSuccess;
    for (auto& e : s->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    for (int k = 0; k < 2 && ok; ++k) {
        ok = !s->pos[k].ensure(24 * n) && !s->pos0[k].ensure(24 * n) && !s->mem[k].ensure(24 * n) &&
             !s->tag[k].ensure(4 * n) && !s->radius[k].ensure(8 * n) &&
             !s->inv_mass[k].ensure(8 * n) && !s->perm[k].ensure(4 * n) &&
             !s->count[k].ensure(4 * nc);
    }
    for (int k = 0; k < 3 && ok; ++k) ok = !s->frc[k].ensure(24 * n);
    ok = ok && !s->cellid.ensure(4 * n) && !s->key.ensure(4 * n) && !s->rank.ensure(4 * n) &&
         !s->tmp.ensure(4 * n) && !s->start.ensure(4 * nc) &&
         !s->scratch.ensure(4 * scan_scratch_ints(g.ncell)) &&
         !s->posh.ensure(16 * (n + 4)) &&   // + 4: the list build reads up to 3 past a run
         !s->vel.ensure(24 * n) && !s->err.ensure(4) && !s->state.ensure(sizeof(StepState)) &&
         !s->occ.ensure(4);
    if (ok && cfg->precision == PSIM_PRECISION_FP64) ok = !s->posd.ensure(32 * n);
    if (ok && cfg->precision == PSIM_PRECISION_MIXED)
        ok = !s->posl.ensure(16 * n);
    if (ok && list_on) {
        ok = !s->lslot[0].ensure(4 * n) && !s->lslot[1].ensure(4 * n) && !s->lbuild.ensure(16 * n) &&
             !s->lpos.ensure(32 * (n + 1 + (size_t)s->hcap)) &&
             !s->list.ensure(4 * n * (size_t)(s->lcap + kListFold)) && !s->lcount.ensure(4 * n) &&
             !s->lflag.ensure(8) && !s->lhalo.ensure(4 * n) && !s->lhcount.ensure(4) &&
             !s->pscratch.ensure(15 * 8 * (size_t)n) &&
             cudaMemset(s->lflag.p, 0, 8) == cudaSuccess &&
             cudaMemset(s->lhcount.p, 0, 4) == cudaSuccess;
    }
    if (ok) ok = cudaMemset(s->err.p, 0, 4) == cudaSuccess &&
                 cudaMemset(s->state.p, 0, sizeof(StepState)) == cudaSuccess;
    if (!ok) {
        fail(PSIM_ERR_CUDA, "system allocation failed: %s", cudaGetErrorString(cudaGetLastError()));
        psim_system_destroy(s);
        return nullptr;
    }
    if (cfg->force_launch) {
        // One call of the plugin's pass with its error word already set (and
        // every cell empty): each kernel of the pass launches and returns at
        // once.  It brings the plugin's own CUDA runtime up and loads its
        // kernels here, outside the stream capture of the step graphs.
        DevBuf word;
        double* f = s->frc[0].as<double>();
        ForceOut fo{f, f + n, f + 2 * n, nullptr, nullptr};
        ok = !word.ensure(4) && cudaMemset(word.p, 0xff, 4) == cudaSuccess &&
             cudaMemset(s->count[0].p, 0, 4 * nc) == cudaSuccess &&
             cudaMemset(s->start.p, 0, 4 * nc) == cudaSuccess;
        if (ok) {
            fo.err = word.as<uint32_t>();
            const ForceRunner fr{&s->fs, cfg->force_launch, &s->cfg.force};
            CellView cv{s->posd.as<double4_32a>(), s->posh.as<float4>(), s->posl.as<float4>(),
                        s->cellid.as<int>(), s->start.as<int>(), s->count[0].as<int>()};
            PairList pl{nullptr, s->lpos.as<float4>(), s->lcount.as<int>(),
                        s->list.as<uint32_t>(), s->n, 0, 0.f, 0.f};
            const int pass = cfg->precision == PSIM_PRECISION_FP64
                                 ? PSIM_PASS_FP64
                                 : (list_on ? PSIM_PASS_LIST : PSIM_PASS_MIXED);
            ok = fr.run(pass, g, &cv, &pl, fo, s->st) == cudaSuccess &&
                 cudaStreamSynchronize(s->st) == cudaSuccess;
        }
        word.release();
        if (!ok) {
            fail(PSIM_ERR_CUDA, "the plugin's psim_force_launch failed on a first, empty pass");
            psim_system_destroy(s);
            return nullptr;
        }
    }
    return s;
}

}  // namespace

extern "C" {

void psim_system_destroy(psim_system* s) {
    if (!s) return;
    DeviceGuard dg(s->device);
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->side) cudaStreamSynchronize(s->side);
    drop_graphs(s);
    DevBuf* arrs[] = {&s->cellid, &s->key, &s->rank, &s->tmp, &s->start, &s->scratch, &s->posd,
                      &s->posh, &s->posl, &s->vel, &s->err, &s->state, &s->occ, &s->noise,
                      &s->snap, &s->lslot[0], &s->lslot[1], &s->lbuild, &s->lpos, &s->list,
                      &s->lcount, &s->lflag, &s->lhalo, &s->lhcount, &s->pscratch, &s->b_tasks,
                      &s->b_geoms, &s->b_pairs, &s->b_pre, &s->b_rep, &s->b_seeds,
                      &s->img, &s->track_start, &s->b_lpre, &s->b_hr};
    for (DevBuf* b : arrs) b->release();
    for (int k = 0; k < 2; ++k) {
        s->pos[k].release(); s->pos0[k].release(); s->mem[k].release(); s->tag[k].release();
        s->radius[k].release(); s->inv_mass[k].release(); s->perm[k].release();
        s->count[k].release();
    }
    for (int k = 0; k < 3; ++k) s->frc[k].release();
    for (auto& e : s->ev) if (e) cudaEventDestroy(e);
    if (s->ev_snap_ready) cudaEventDestroy(s->ev_snap_ready);
    if (s->ev_snap_done) cudaEventDestroy(s->ev_snap_done);
    if (s->st) cudaStreamDestroy(s->st);
    if (s->side) cudaStreamDestroy(s->side);
    delete s;
}

int psim_system_upload(psim_system* s, const double* pos, const double* pos0, const double* vel,
                       const double* frc, const double* frc0, const double* radius,
                       const double* mass) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (s->n > 0 && (!pos || !radius)) return fail(PSIM_ERR_INPUT, "positions and radii are required");
    DeviceGuard dg(s->device);
    const int n = s->n;
    const size_t b = 24 * (size_t)n;
    cudaStream_t st = s->st;
    PSIM_CUDA(cudaStreamSynchronize(st));
    // the upload is "after step -1": storage order = original order
    const Phase ph = phase_of(0);
    const int sb = ph.sb, ob = ph.ob, pb = ph.pb;
    ScopedBuf stage;
    PSIM_CUDA(stage.ensure(b));
    auto load3 = [&](const double* src, DevBuf& dst) -> int {
        if (src) {
            PSIM_CUDA(cudaMemcpyAsync(stage.p, src, b, cudaMemcpyHostToDevice, st));
            PSIM_CUDA(launch_split_xyz(n, stage.as<double>(), nullptr, 0, d3(dst, n, 0),
                                       d3(dst, n, 1), d3(dst, n, 2), st));
        } else {
            PSIM_CUDA(cudaMemsetAsync(dst.p, 0, b, st));
        }
        return PSIM_OK;
    };
    int rc;
    if ((rc = load3(pos, s->pos[sb]))) return rc;
    if ((rc = load3(pos0 ? pos0 : pos, s->pos0[sb]))) return rc;
    PSIM_CUDA(cudaMemsetAsync(s->mem[sb].p, 0, b, st));
    if ((rc = load3(frc, s->frc[ph.fprev]))) return rc;
    if ((rc = load3(frc0, s->frc[(ph.fprev + 2) % 3]))) return rc;
    if (vel) PSIM_CUDA(cudaMemcpyAsync(s->vel.p, vel, b, cudaMemcpyHostToDevice, st));
    else PSIM_CUDA(cudaMemsetAsync(s->vel.p, 0, b, st));
    // original-order tags, radii and 1/m of "order -1"
    std::vector<double> inv((size_t)n, 1.0);
    if (mass)
        for (int i = 0; i < n; ++i) inv[i] = 1.0 / mass[i];
    PSIM_CUDA(cudaMemcpyAsync(s->radius[1 - ob].p, radius, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    PSIM_CUDA(cudaMemcpyAsync(s->inv_mass[1 - ob].p, inv.data(), 8 * (size_t)n,
                              cudaMemcpyHostToDevice, st));
    PSIM_CUDA(launch_fill_int_iota(n, s->tag[1 - ob].as<int>(), st));
    PSIM_CUDA(launch_fill_int_iota(n, s->perm[1 - pb].as<int>(), st));
    PSIM_CUDA(cudaMemsetAsync(s->err.p, 0, 4, st));
    PSIM_CUDA(cudaMemsetAsync(s->state.p, 0, sizeof(StepState), st));
    // first cell list (system.cpp:101-103)
    PSIM_CUDA(cudaMemsetAsync(s->count[ph.cb].p, 0, 4 * (size_t)s->ncell, st));
    PSIM_CUDA(launch_hash_count(n, d3(s->pos[sb], n, 0), d3(s->pos[sb], n, 1),
                                d3(s->pos[sb], n, 2), s->g, s->key.as<int>(), s->rank.as<int>(),
                                s->count[ph.cb].as<int>(), s->err.as<uint32_t>(), st,
                                s->n_reps ? s->b_rep.as<int>() : nullptr,
                                s->n_reps ? s->b_geoms.as<DevGeom>() : nullptr));
    PSIM_CUDA(launch_scan(s->count[ph.cb].as<int>(), s->start.as<int>(), s->ncell,
                          s->scratch.as<int>(), st));
    PSIM_CUDA(launch_scatter(n, s->key.as<int>(), s->rank.as<int>(), s->start.as<int>(),
                             s->tmp.as<int>(), nullptr, st));
    CanonArgs ca{};
    ca.n = n;
    ca.tmp = s->tmp.as<int>();
    ca.key = s->key.as<int>();
    ca.start = s->start.as<int>();
    ca.count = s->count[ph.cb].as<int>();
    ca.tag_in = s->tag[1 - ob].as<int>();
    ca.radius_in = s->radius[1 - ob].as<double>();
    ca.inv_mass_in = s->inv_mass[1 - ob].as<double>();
    ca.x = d3(s->pos[sb], n, 0); ca.y = d3(s->pos[sb], n, 1); ca.z = d3(s->pos[sb], n, 2);
    ca.perm = s->perm[pb].as<int>();
    ca.tag_out = s->tag[ob].as<int>();
    ca.radius_out = s->radius[ob].as<double>();
    ca.inv_mass_out = s->inv_mass[ob].as<double>();
    ca.cellid = s->cellid.as<int>();
    ca.posd = s->cfg.precision == PSIM_PRECISION_FP64 ? s->posd.as<double4_32a>() : nullptr;
    ca.posh = s->posh.as<float4>();
    ca.posl = s->cfg.precision == PSIM_PRECISION_MIXED ? s->posl.as<float4>() : nullptr;
    if (s->list_on) {
        // compact records when all radii are equal; the ghost record n that
        // pads the lists is out of range of every particle (far away for
        // full records, an r^2 bias for compact ones)
        int compact = n > 0 ? 1 : 0;
        for (int i = 1; i < n && compact; ++i) compact = radius[i] == radius[0];
        const float R = n > 0 ? (float)radius[0] : 0.f;
        if (compact != s->lcompact || R != s->lradius) drop_graphs(s);
        s->lcompact = compact;
        s->lradius = R;
        s->lunit = fixed_unit(s->n_reps ? s->lmaxrc : max_cutoff(&s->cfg.force), s->skin);
        const float4 ghost[2] = {compact ? make_float4(0.f, 0.f, 0.f, kGhostBias)
                                         : make_float4(1e18f, 1e18f, 1e18f, R),
                                 make_float4(0.f, 0.f, 0.f, 0.f)};
        float4* grec = s->lpos.as<float4>() + (compact ? 1 : 2) * (size_t)n;
        PSIM_CUDA(cudaMemcpyAsync(grec, ghost, compact ? 16 : 32, cudaMemcpyHostToDevice, st));
    }
    if (s->list_on) {
        // the first list, on the first cell order (the list slots are the
        // storage slots: the state is carried into that order below)
        PSIM_CUDA(cudaMemsetAsync(s->lflag.p, 0, 8, st));
        set_halo_args(s, ca);
        PSIM_CUDA(cudaMemsetAsync(s->lhcount.p, 0, 4, st));
    }
    PSIM_CUDA(launch_canonicalize(ca, st));
    if (s->list_on) {
        // the uploaded state (original order) into the first cell order
        DevBuf* arrs[5] = {&s->pos[sb], &s->pos0[sb], &s->mem[sb], &s->frc[ph.fprev],
                           &s->frc[(ph.fprev + 2) % 3]};
        PermuteArgs pa{};
        pa.n = n;
        pa.perm = s->perm[pb].as<int>();
        pa.narr = 15;
        double* scr = s->pscratch.as<double>();
        for (int a = 0; a < 5; ++a)
            for (int k = 0; k < 3; ++k) {
                pa.src[3 * a + k] = d3(*arrs[a], n, k);
                pa.dst[3 * a + k] = scr + (size_t)(3 * a + k) * n;
            }
        PSIM_CUDA(launch_permute(pa, s->err.as<uint32_t>(), st));
        for (int a = 0; a < 5; ++a)
            PSIM_CUDA(cudaMemcpyAsync(arrs[a]->p, scr + (size_t)3 * a * n, 24 * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
        PSIM_CUDA(enqueue_list_build(s, ph.cb, nullptr));
    }
    uint32_t bits = 0;
    PSIM_CUDA(cudaMemcpyAsync(&bits, s->err.p, 4, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaStreamSynchronize(st));
    stage.release();
    s->total = 0;
    s->latched = 0;
    s->uploaded = true;
    if (bits) {
        s->latched = bits;
        return fail(code_from_bits(bits), "upload: %s", bits_text(bits));
    }
    return PSIM_OK;
}

int psim_system_set_noise(psim_system* s, const double* noise, int32_t n_steps, int32_t first) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (n_steps < 0 || first < 0) return fail(PSIM_ERR_INPUT, "negative noise range");
    if (n_steps > 0 && !noise) return fail(PSIM_ERR_INPUT, "NULL noise");
    DeviceGuard dg(s->device);
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    const size_t b = (size_t)n_steps * (size_t)s->n * 6 * sizeof(double);
    void* old = s->noise.p;
    PSIM_CUDA(s->noise.ensure(b));
    if (s->noise.p != old) drop_graphs(s);  // graphs hold the buffer address
    if (b) PSIM_CUDA(cudaMemcpy(s->noise.p, noise, b, cudaMemcpyHostToDevice));
    if (s->noise_first != first || s->noise_steps != n_steps) drop_graphs(s);
    s->noise_first = first;
    s->noise_steps = n_steps;
    return PSIM_OK;
}

int psim_system_step_async(psim_system* s, int32_t n_steps) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    if (s->latched) return fail(code_from_bits(s->latched), "%s", bits_text(s->latched));
    if (n_steps < 0) return fail(PSIM_ERR_INPUT, "negative step count");
    DeviceGuard dg(s->device);
    for (int ph = 0; ph < 6 && n_steps > 0; ++ph) {  // capture before anything is in flight
        cudaGraphExec_t ge;
        if (!s->graph[ph]) {
            PSIM_CUDA(cudaStreamSynchronize(s->st));
            int rc = graph_for(s, ph, &ge);
            if (rc) return rc;
        }
    }
    if (n_steps >= kGraphSteps + 5 && !s->graph_multi) {
        PSIM_CUDA(cudaStreamSynchronize(s->st));
        int rc = graph_steps(s, 0, kGraphSteps, &s->graph_multi);
        if (rc) return rc;
    }
    // single steps up to a multiple of 6, then kGraphSteps steps per launch
    while (n_steps > 0) {
        if (s->graph_multi && s->total % 6 == 0 && n_steps >= kGraphSteps) {
            PSIM_CUDA(cudaGraphLaunch(s->graph_multi, s->st));
            s->total += kGraphSteps;
            n_steps -= kGraphSteps;
            continue;
        }
        cudaGraphExec_t ge;
        int rc = graph_for(s, (int)(s->total % 6), &ge);
        if (rc) return rc;
        PSIM_CUDA(cudaGraphLaunch(ge, s->st));
        s->total++;
        --n_steps;
    }
    return PSIM_OK;
}

int psim_system_sync(psim_system* s) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    DeviceGuard dg(s->device);
    return settle(s);
}

int psim_system_step(psim_system* s, int32_t n_steps) {
    int rc = psim_system_step_async(s, n_steps);
    if (rc) return rc;
    return psim_system_sync(s);
}

int psim_system_download(psim_system* s, double* pos, double* pos0, double* vel, double* frc,
                         double* frc0) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc && rc != code_from_bits(s->latched)) return rc;
    const Phase ph = phase_of(s->total);
    const int n = s->n;
    const size_t b = 24 * (size_t)n;
    cudaStream_t st = s->st;
    // storage order is the previous cell order: its tags are tag[1 - ob]
    const int* tg = store_tags(s);
    ScopedBuf stage;
    PSIM_CUDA(stage.ensure(b));
    auto get3 = [&](DevBuf& src, const int* perm, double* dst) -> int {
        if (!dst) return PSIM_OK;
        PSIM_CUDA(launch_merge_xyz(n, d3(src, n, 0), d3(src, n, 1), d3(src, n, 2), tg, perm,
                                   stage.as<double>(), st));
        PSIM_CUDA(cudaMemcpyAsync(dst, stage.p, b, cudaMemcpyDeviceToHost, st));
        PSIM_CUDA(cudaStreamSynchronize(st));
        return PSIM_OK;
    };
    if ((rc = get3(s->pos[ph.sb], nullptr, pos))) return rc;
    if ((rc = get3(s->pos0[ph.sb], nullptr, pos0))) return rc;
    if ((rc = get3(s->frc[ph.fprev], nullptr, frc))) return rc;
    // frc0 is the force of two orders back, reached through the previous permutation
    if ((rc = get3(s->frc[(ph.fprev + 2) % 3], prev_perm(s), frc0))) return rc;
    if (vel) {
        PSIM_CUDA(cudaMemcpyAsync(vel, s->vel.p, b, cudaMemcpyDeviceToHost, st));
        PSIM_CUDA(cudaStreamSynchronize(st));
    }
    stage.release();
    return s->latched ? code_from_bits(s->latched) : PSIM_OK;
}

int psim_system_download_cells(psim_system* s, int32_t* hash_index, uint32_t* cse,
                               double* sorted) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc && rc != code_from_bits(s->latched)) return rc;
    const Phase ph = phase_of(s->total);
    const int n = s->n;
    cudaStream_t st = s->st;
    ScopedBuf hb, cb, sb, pd;
    PSIM_CUDA(hb.ensure(8 * (size_t)n));
    PSIM_CUDA(cb.ensure(8 * (size_t)s->ncell));
    PSIM_CUDA(sb.ensure(32 * (size_t)n));
    CellRefs c;
    if ((rc = cell_refs(s, c))) return rc;
    const double4_32a* posd = s->posd.as<double4_32a>();
    if (s->cfg.precision != PSIM_PRECISION_FP64) {
        // the mixed form keeps no FP64 sorted copy: gather one from the storage order
        PSIM_CUDA(pd.ensure(32 * (size_t)n));
        PSIM_CUDA(launch_gather_posd(n, c.perm, d3(s->pos[ph.sb], n, 0), d3(s->pos[ph.sb], n, 1),
                                     d3(s->pos[ph.sb], n, 2), c.radius, pd.as<double4_32a>(), st));
        posd = pd.as<double4_32a>();
    }
    PSIM_CUDA(launch_export_cells(n, s->ncell, s->cellid.as<int>(), c.tag, posd,
                                  s->start.as<int>(), c.count,
                                  hb.as<int32_t>(), cb.as<uint32_t>(), sb.as<double>(), st));
    if (hash_index)
        PSIM_CUDA(cudaMemcpyAsync(hash_index, hb.p, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (cse) PSIM_CUDA(cudaMemcpyAsync(cse, cb.p, 8 * (size_t)s->ncell, cudaMemcpyDeviceToHost, st));
    if (sorted) PSIM_CUDA(cudaMemcpyAsync(sorted, sb.p, 32 * (size_t)n, cudaMemcpyDeviceToHost, st));
    PSIM_CUDA(cudaStreamSynchronize(st));
    return PSIM_OK;
}

int psim_system_snapshot_async(psim_system* s, double* host_pos) {
    if (!s || !host_pos) return fail(PSIM_ERR_INPUT, "NULL argument");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    DeviceGuard dg(s->device);
    const int n = s->n;
    const size_t b = 24 * (size_t)n;
    PSIM_CUDA(s->snap.ensure(b));
    const Phase ph = phase_of(s->total);
    // the previous snapshot's copy must have left the staging buffer
    if (s->snap_pending) PSIM_CUDA(cudaStreamWaitEvent(s->st, s->ev_snap_done, 0));
    PSIM_CUDA(launch_merge_xyz(n, d3(s->pos[ph.sb], n, 0), d3(s->pos[ph.sb], n, 1),
                               d3(s->pos[ph.sb], n, 2), store_tags(s), nullptr,
                               s->snap.as<double>(), s->st));
    PSIM_CUDA(cudaEventRecord(s->ev_snap_ready, s->st));
    PSIM_CUDA(cudaStreamWaitEvent(s->side, s->ev_snap_ready, 0));
    PSIM_CUDA(cudaMemcpyAsync(host_pos, s->snap.p, b, cudaMemcpyDeviceToHost, s->side));
    PSIM_CUDA(cudaEventRecord(s->ev_snap_done, s->side));
    s->snap_pending = true;
    return PSIM_OK;
}

int psim_system_snapshot_wait(psim_system* s) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    DeviceGuard dg(s->device);
    if (s->snap_pending) PSIM_CUDA(cudaEventSynchronize(s->ev_snap_done));
    s->snap_pending = false;
    return PSIM_OK;
}

int psim_system_get_step(psim_system* s, int64_t* step, int32_t* vel_counter) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    DeviceGuard dg(s->device);
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    StepState ss{};
    PSIM_CUDA(cudaMemcpy(&ss, s->state.p, sizeof ss, cudaMemcpyDeviceToHost));
    if (step) *step = ss.step;
    if (vel_counter) *vel_counter = ss.vel_counter;
    return PSIM_OK;
}

int psim_system_forces(psim_system* s, double* force) {
    if (!s || !force) return fail(PSIM_ERR_INPUT, "NULL argument");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    const Phase ph = phase_of(s->total);
    const int n = s->n;
    ScopedBuf f3, out;
    PSIM_CUDA(f3.ensure(24 * (size_t)n));
    PSIM_CUDA(out.ensure(24 * (size_t)n));
    ForceOut fo{f3.as<double>(), f3.as<double>() + n, f3.as<double>() + 2 * (size_t)n,
                s->err.as<uint32_t>(), nullptr};
    PSIM_CUDA(enqueue_force(s, ph, fo));
    // the pass writes in its order: the next cell order, or with a pair list
    // the storage order
    PSIM_CUDA(launch_unsort_force(n, s->list_on ? store_tags(s) : s->tag[ph.ob].as<int>(),
                                  fo.fx, fo.fy, fo.fz,
                                  out.as<double>(), s->st));
    PSIM_CUDA(cudaMemcpyAsync(force, out.p, 24 * (size_t)n, cudaMemcpyDeviceToHost, s->st));
    return settle(s);
}

// ------------------------------------------------------------ observables

namespace {

int ready(psim_system* s, const void* out) {
    if (!s || !out) return fail(PSIM_ERR_INPUT, "NULL argument");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    return PSIM_OK;
}

// One reduction of the state after `total` steps, copied to the host.
int reduce(psim_system* s, ObserveArgs& a, double* out) {
    const Phase ph = phase_of(s->total);
    const int n = s->n;
    a.n = n;
    a.x = d3(s->pos[ph.sb], n, 0); a.y = d3(s->pos[ph.sb], n, 1); a.z = d3(s->pos[ph.sb], n, 2);
    a.x0 = d3(s->pos0[ph.sb], n, 0); a.y0 = d3(s->pos0[ph.sb], n, 1);
    a.z0 = d3(s->pos0[ph.sb], n, 2);
    a.fx = d3(s->frc[ph.fprev], n, 0); a.fy = d3(s->frc[ph.fprev], n, 1);
    a.fz = d3(s->frc[ph.fprev], n, 2);
    const int fb = (ph.fprev + 2) % 3;
    a.gx = d3(s->frc[fb], n, 0); a.gy = d3(s->frc[fb], n, 1); a.gz = d3(s->frc[fb], n, 2);
    a.perm_prev = prev_perm(s);
    a.tag = store_tags(s);   // the storage order's tags (as download)
    a.L = s->g.L;
    ScopedBuf scratch, res;
    PSIM_CUDA(scratch.ensure(8 * (size_t)observe_scratch_doubles()));
    PSIM_CUDA(res.ensure(8));
    PSIM_CUDA(launch_observe(a, scratch.as<double>(), res.as<double>(), s->st));
    PSIM_CUDA(cudaMemcpyAsync(out, res.p, 8, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    return PSIM_OK;
}

// The sorted FP64 positions of the current cell list (into pd) and the cell
// ranges, for a 27-cell walk.
int sorted_view(psim_system* s, ScopedBuf& pd, PairScanArgs& a) {
    if (s->n_reps) return fail(PSIM_ERR_INPUT, "pair observables are per system, not per batch");
    const Phase ph = phase_of(s->total);
    PSIM_CUDA(pd.ensure(32 * (size_t)s->n));
    CellRefs c;
    if (int rc = cell_refs(s, c)) return rc;
    PSIM_CUDA(launch_gather_posd(s->n, c.perm, d3(s->pos[ph.sb], s->n, 0),
                                 d3(s->pos[ph.sb], s->n, 1), d3(s->pos[ph.sb], s->n, 2),
                                 c.radius, pd.as<double4_32a>(), s->st));
    a.g = s->g;
    a.posd = pd.as<double4_32a>();
    a.cellid = s->cellid.as<int>();
    a.cstart = s->start.as<int>();
    a.ccount = c.count;
    a.tag = c.tag;
    return PSIM_OK;
}

int pair_scan(psim_system* s, PairScanArgs& a) {
    ScopedBuf pd;
    int rc = sorted_view(s, pd, a);
    if (rc) return rc;
    PSIM_CUDA(launch_pair_scan(a, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    return PSIM_OK;
}

}  // namespace

int psim_system_temperature(psim_system* s, double* kT) {
    int rc = ready(s, kT);
    if (rc) return rc;
    DeviceGuard dg(s->device);
    if ((rc = settle(s))) return rc;
    ScopedBuf scratch, res;
    PSIM_CUDA(scratch.ensure(8 * (size_t)observe_scratch_doubles()));
    PSIM_CUDA(res.ensure(8));
    PSIM_CUDA(launch_sum_squares(3LL * s->n, s->vel.as<double>(), scratch.as<double>(),
                                 res.as<double>(), s->st));
    double v2 = 0.0;
    PSIM_CUDA(cudaMemcpyAsync(&v2, res.p, 8, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    *kT = s->n ? v2 / 3.0 / s->n : 0.0;
    return PSIM_OK;
}

int psim_system_mean_displacement(psim_system* s, double* msd) {
    int rc = ready(s, msd);
    if (rc) return rc;
    DeviceGuard dg(s->device);
    if ((rc = settle(s))) return rc;
    ObserveArgs a{};
    a.what = OBS_MEAN_DISP;
    double sum = 0.0;
    if ((rc = reduce(s, a, &sum))) return rc;
    *msd = s->n ? sum / s->n : 0.0;
    return PSIM_OK;
}

int psim_system_potential(psim_system* s, double* eap) {
    int rc = ready(s, eap);
    if (rc) return rc;
    DeviceGuard dg(s->device);
    if ((rc = settle(s))) return rc;
    ObserveArgs a{};
    a.what = OBS_POTENTIAL;
    double sum = 0.0;
    if ((rc = reduce(s, a, &sum))) return rc;
    *eap = s->n ? sum / s->n : 0.0;
    return PSIM_OK;
}

int psim_system_track_start(psim_system* s) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    if (s->n_reps) return fail(PSIM_ERR_INPUT, "the tracker is per system, not per batch");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    const size_t b = 24 * (size_t)s->n;
    const bool fresh = s->img.p == nullptr;
    PSIM_CUDA(s->img.ensure(12 * (size_t)s->n));
    PSIM_CUDA(s->track_start.ensure(b));
    if (fresh) drop_graphs(s);   // the captured steps start counting images
    const Phase ph = phase_of(s->total);
    PSIM_CUDA(cudaMemsetAsync(s->img.p, 0, 12 * (size_t)s->n, s->st));
    PSIM_CUDA(launch_merge_xyz(s->n, d3(s->pos[ph.sb], s->n, 0), d3(s->pos[ph.sb], s->n, 1),
                               d3(s->pos[ph.sb], s->n, 2), store_tags(s), nullptr,
                               s->track_start.as<double>(), s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    return PSIM_OK;
}

int psim_system_tracked_displacement(psim_system* s, double* msd) {
    int rc = ready(s, msd);
    if (rc) return rc;
    if (!s->img.p) return fail(PSIM_ERR_INPUT, "the displacement tracker was not started");
    DeviceGuard dg(s->device);
    if ((rc = settle(s))) return rc;
    ObserveArgs a{};
    a.what = OBS_TRACKED;
    a.img = s->img.as<int>();
    a.start = s->track_start.as<double>();
    double sum = 0.0;
    if ((rc = reduce(s, a, &sum))) return rc;
    *msd = s->n ? sum / s->n : 0.0;
    return PSIM_OK;
}

int psim_system_interactions(psim_system* s, double r_contact, int32_t* coor, int64_t* total) {
    if (!s || !s->uploaded) return fail(PSIM_ERR_INPUT, "NULL system or no state uploaded");
    if (!(r_contact > 0.0) || r_contact > s->g.cs)
        return fail(PSIM_ERR_INPUT, "contact distance %g outside (0, cellSize]", r_contact);
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    ScopedBuf cb, tot;
    PSIM_CUDA(cb.ensure(4 * (size_t)s->n));
    // updateInteractions fused into one force pass on the current state: the
    // FP64 walk (the reference's own test, sqrt(r^2) < r_contact), the mixed
    // walk, or the mixed pair list when every pair closer than r_contact is
    // guaranteed to be in it (r_contact <= cutOff).  A plugin's pass, a batch,
    // the block-per-cell layout or a list of a shorter cutoff take a separate
    // walk instead.
    if (!s->n_reps && !s->cfg.force_launch && s->fs.tile == 0 &&
        (!s->list_on || r_contact <= max_cutoff(&s->cfg.force))) {
        const Phase ph = phase_of(s->total);
        const int n = s->n;
        ScopedBuf f3;
        PSIM_CUDA(f3.ensure(24 * (size_t)n));
        ForceOut fo{f3.as<double>(), f3.as<double>() + n, f3.as<double>() + 2 * (size_t)n,
                    s->err.as<uint32_t>(), nullptr};
        fo.coor = cb.as<int>();
        fo.cont = r_contact;
        fo.cont2f = (float)(r_contact * r_contact);
        const float keep = s->fs.pre_rc2f;   // the candidate bound must cover r_contact
        s->fs.pre_rc2f = std::max(keep, prefilter_r2(r_contact, s->g.L));
        const cudaError_t e = enqueue_force(s, ph, fo);
        s->fs.pre_rc2f = keep;
        PSIM_CUDA(e);
        if ((rc = settle(s))) return rc;
        std::vector<int> c((size_t)n), tg((size_t)n);
        PSIM_CUDA(cudaMemcpy(c.data(), cb.p, 4 * (size_t)n, cudaMemcpyDeviceToHost));
        PSIM_CUDA(cudaMemcpy(tg.data(), s->list_on ? store_tags(s) : s->tag[ph.ob].as<int>(),
                             4 * (size_t)n, cudaMemcpyDeviceToHost));
        int64_t t = 0;
        for (int i = 0; i < n; ++i) {
            t += c[(size_t)i];
            if (coor) coor[tg[(size_t)i]] = c[(size_t)i];
        }
        if (total) *total = t;
        return PSIM_OK;
    }
    PSIM_CUDA(tot.ensure(8));
    PSIM_CUDA(cudaMemsetAsync(tot.p, 0, 8, s->st));
    PairScanArgs a{};
    a.r_contact = r_contact;
    a.coor = cb.as<int>();
    a.n_pairs = tot.as<unsigned long long>();
    if ((rc = pair_scan(s, a))) return rc;
    if (coor) PSIM_CUDA(cudaMemcpy(coor, cb.p, 4 * (size_t)s->n, cudaMemcpyDeviceToHost));
    unsigned long long t = 0;
    PSIM_CUDA(cudaMemcpy(&t, tot.p, 8, cudaMemcpyDeviceToHost));
    if (total) *total = (int64_t)t;
    return PSIM_OK;
}

int psim_system_clusters(psim_system* s, double r_contact, int32_t min_size, int32_t* root,
                         int32_t* n_clusters, int32_t* avg_size) {
    if (!s || !s->uploaded) return fail(PSIM_ERR_INPUT, "NULL system or no state uploaded");
    if (!(r_contact > 0.0) || r_contact > s->g.cs)
        return fail(PSIM_ERR_INPUT, "contact distance %g outside (0, cellSize]", r_contact);
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    const size_t n = (size_t)s->n;
    ScopedBuf pd, lab, rt, sz, eb;
    PSIM_CUDA(lab.ensure(4 * n));
    PSIM_CUDA(rt.ensure(4 * n));
    PSIM_CUDA(sz.ensure(4 * n));
    PSIM_CUDA(eb.ensure(4));
    PSIM_CUDA(cudaMemsetAsync(sz.p, 0, 4 * n, s->st));
    PSIM_CUDA(cudaMemsetAsync(eb.p, 0, 4, s->st));
    PairScanArgs a{};
    a.r_contact = r_contact;
    if ((rc = sorted_view(s, pd, a))) return rc;
    PSIM_CUDA(launch_clusters(a, lab.as<int>(), rt.as<int>(), sz.as<int>(), eb.as<uint32_t>(),
                              s->st));
    std::vector<int> hroot(n), hsize(n);
    uint32_t bits = 0;
    PSIM_CUDA(cudaMemcpyAsync(hroot.data(), rt.p, 4 * n, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaMemcpyAsync(hsize.data(), sz.p, 4 * n, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaMemcpyAsync(&bits, eb.p, 4, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    if (bits) return fail(PSIM_ERR_INPUT, "cluster search did not converge");
    if (root) std::copy(hroot.begin(), hroot.end(), root);
    // analysisManager::writeClusters (analysisCluster.cpp:64-78): clusters of
    // more than min_size particles, and their integer mean size
    long long members = 0, count = 0;
    for (size_t i = 0; i < n; ++i)
        if (hroot[i] == (int)i && hsize[i] > min_size) {
            ++count;
            members += hsize[i];
        }
    if (n_clusters) *n_clusters = (int32_t)count;
    if (avg_size) *avg_size = count ? (int32_t)(members / count) : 0;
    return PSIM_OK;
}

int psim_system_rdf(psim_system* s, double r_min, double r_max, int32_t n_bins, double* g_r) {
    if (!s || !g_r || !s->uploaded) return fail(PSIM_ERR_INPUT, "NULL argument or no state");
    if (!(r_min >= 0.0) || !(r_max > r_min) || r_max > s->g.cs || n_bins <= 0 || n_bins > 8192)
        return fail(PSIM_ERR_INPUT, "g(r) range [%g, %g) with %d bins: need 0 <= r_min < r_max "
                    "<= cellSize and 1..8192 bins", r_min, r_max, n_bins);
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    ScopedBuf hb;
    PSIM_CUDA(hb.ensure(8 * (size_t)n_bins));
    PSIM_CUDA(cudaMemsetAsync(hb.p, 0, 8 * (size_t)n_bins, s->st));
    PairScanArgs a{};
    a.r_contact = 0.0;
    a.r_min = r_min;
    a.r_max = r_max;
    a.inv_dr = n_bins / (r_max - r_min);
    a.n_bins = n_bins;
    a.hist = hb.as<unsigned long long>();
    if ((rc = pair_scan(s, a))) return rc;
    std::vector<unsigned long long> h((size_t)n_bins);
    PSIM_CUDA(cudaMemcpy(h.data(), hb.p, 8 * (size_t)n_bins, cudaMemcpyDeviceToHost));
    // ordered pairs per particle in each shell over the ideal-gas count
    const double rho = s->n / (s->g.L * s->g.L * s->g.L);
    const double dr = (r_max - r_min) / n_bins;
    for (int k = 0; k < n_bins; ++k) {
        const double r0 = r_min + k * dr, r1 = r0 + dr;
        const double shell = 4.0 / 3.0 * M_PI * (r1 * r1 * r1 - r0 * r0 * r0);
        g_r[k] = s->n ? (double)h[(size_t)k] / (s->n * rho * shell) : 0.0;
    }
    return PSIM_OK;
}

int psim_system_set_list_lanes(psim_system* s, int32_t lanes) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    if (lanes != 1 && lanes != 2 && lanes != 4)
        return fail(PSIM_ERR_INPUT, "lanes per particle must be 1, 2 or 4 (got %d)", lanes);
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    if (lanes != s->list_lanes) {
        drop_graphs(s);   // the captured steps hold the kernel of the old setting
        s->list_lanes = lanes;
    }
    return PSIM_OK;
}

int psim_system_energy(psim_system* s, double* potential, double* virial) {
    if (!s || !s->uploaded) return fail(PSIM_ERR_INPUT, "NULL system or no state");
    if (s->n_reps) return fail(PSIM_ERR_INPUT, "energy: single systems only");
    if (s->cfg.force_launch || s->cfg.force.kind == PSIM_FORCE_PLUGIN)
        return fail(PSIM_ERR_INPUT, "energy: the plugin's pair energy is not known to the library");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    PairScanArgs a{};
    ScopedBuf pd, scratch, res;
    if ((rc = sorted_view(s, pd, a))) return rc;
    PSIM_CUDA(scratch.ensure(16 * (size_t)((s->n + 127) / 128 + 1)));
    PSIM_CUDA(res.ensure(16));
    PSIM_CUDA(launch_energy(s->fs, a, scratch.as<double>(), res.as<double>(), s->st));
    double out[2] = {0.0, 0.0};
    PSIM_CUDA(cudaMemcpyAsync(out, res.p, 16, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    if (potential) *potential = s->n ? out[0] / s->n : 0.0;
    if (virial) *virial = s->n ? out[1] / s->n : 0.0;
    return PSIM_OK;
}

int psim_system_list_builds(psim_system* s, int32_t* builds) {
    if (!s || !builds) return fail(PSIM_ERR_INPUT, "NULL argument");
    DeviceGuard dg(s->device);
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    StepState ss{};
    PSIM_CUDA(cudaMemcpy(&ss, s->state.p, sizeof ss, cudaMemcpyDeviceToHost));
    *builds = ss.list_builds;
    return PSIM_OK;
}

void* psim_system_stream(psim_system* s) { return s ? (void*)s->st : nullptr; }

int psim_system_profile(psim_system* s, int32_t n_steps, double* out_ms) {
    if (!s || !out_ms) return fail(PSIM_ERR_INPUT, "NULL argument");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    DeviceGuard dg(s->device);
    double acc[4] = {0, 0, 0, 0};
    for (int k = 0; k < n_steps; ++k) {
        int rc = enqueue_step(s, s->total, s->ev);
        if (rc) return rc;
        s->total++;
        PSIM_CUDA(cudaEventSynchronize(s->ev[3]));
        float a = 0, b = 0, c = 0;
        PSIM_CUDA(cudaEventElapsedTime(&a, s->ev[0], s->ev[1]));
        PSIM_CUDA(cudaEventElapsedTime(&b, s->ev[1], s->ev[2]));
        PSIM_CUDA(cudaEventElapsedTime(&c, s->ev[2], s->ev[3]));
        acc[0] += a; acc[1] += b; acc[2] += c; acc[3] += a + b + c;
    }
    for (int k = 0; k < 4; ++k) out_ms[k] = n_steps > 0 ? acc[k] / n_steps : 0.0;
    return settle(s);
}

int psim_system_launches_per_step(psim_system* s) {
    // force, vGB, scan x3, scatter, canonicalise (+1 memset node); with a
    // pair list: force, vGB, step end (the rebuild's kernels run on the
    // steps that rebuild: psim_system_launches_per_rebuild)
    return (s && s->list_on) ? 3 : 7;
}

int psim_system_launches_per_rebuild(psim_system* s) {
    // hash + count, scan x3, scatter, canonicalise, state permutation, list
    // build (+ memset and copy nodes)
    return (s && s->list_on) ? 8 : 0;
}

int psim_system_cell_occupancy(psim_system* s, int32_t* max_occ, double* mean_occ) {
    if (!s) return fail(PSIM_ERR_INPUT, "NULL system");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc && rc != code_from_bits(s->latched)) return rc;
    const Phase ph = phase_of(s->total);
    PSIM_CUDA(cudaMemsetAsync(s->occ.p, 0, 4, s->st));
    CellRefs c;
    if ((rc = cell_refs(s, c))) return rc;
    PSIM_CUDA(launch_occupancy(s->ncell, c.count, s->occ.as<int>(), s->st));
    int mx = 0;
    PSIM_CUDA(cudaMemcpyAsync(&mx, s->occ.p, 4, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    if (max_occ) *max_occ = mx;
    if (mean_occ) *mean_occ = s->ncell ? (double)s->n / s->ncell : 0.0;
    return PSIM_OK;
}

int psim_system_time_steps(psim_system* s, int32_t n_steps, double* ms) {
    if (!s || !ms) return fail(PSIM_ERR_INPUT, "NULL argument");
    DeviceGuard dg(s->device);
    // capture the graphs first so the timed region holds only launches
    int rc = psim_system_step_async(s, 0);
    if (rc) return rc;
    for (int ph = 0; ph < 6; ++ph) {
        cudaGraphExec_t ge;
        if (!s->graph[ph]) {
            PSIM_CUDA(cudaStreamSynchronize(s->st));
            if ((rc = graph_for(s, ph, &ge))) return rc;
        }
    }
    if (n_steps >= kGraphSteps + 5 && !s->graph_multi) {
        PSIM_CUDA(cudaStreamSynchronize(s->st));
        if ((rc = graph_steps(s, 0, kGraphSteps, &s->graph_multi))) return rc;
    }
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    PSIM_CUDA(cudaEventRecord(s->ev[0], s->st));
    if ((rc = psim_system_step_async(s, n_steps))) return rc;
    PSIM_CUDA(cudaEventRecord(s->ev[1], s->st));
    PSIM_CUDA(cudaEventSynchronize(s->ev[1]));
    float t = 0.f;
    PSIM_CUDA(cudaEventElapsedTime(&t, s->ev[0], s->ev[1]));
    *ms = t;
    return settle(s);
}

int psim_system_pair_count(psim_system* s, double cutoff, double* mean_pairs) {
    if (!s || !mean_pairs) return fail(PSIM_ERR_INPUT, "NULL argument");
    if (!s->uploaded) return fail(PSIM_ERR_INPUT, "no state uploaded");
    if (cutoff > s->g.cs) return fail(PSIM_ERR_INPUT, "cutoff beyond the cell size");
    DeviceGuard dg(s->device);
    int rc = settle(s);
    if (rc) return rc;
    const Phase ph = phase_of(s->total);
    ScopedBuf tot, ph4;
    PSIM_CUDA(tot.ensure(8));
    PSIM_CUDA(ph4.ensure(16 * (size_t)s->n));
    PSIM_CUDA(cudaMemsetAsync(tot.p, 0, 8, s->st));
    // sorted positions gathered from the FP64 state (with a pair list the
    // float copies are in list order)
    CellRefs c;
    if ((rc = cell_refs(s, c))) return rc;
    PSIM_CUDA(launch_gather_posh(s->n, c.perm, d3(s->pos[ph.sb], s->n, 0),
                                 d3(s->pos[ph.sb], s->n, 1), d3(s->pos[ph.sb], s->n, 2),
                                 c.radius, ph4.as<float4>(), s->st));
    CellView cv{nullptr, ph4.as<float4>(), nullptr, s->cellid.as<int>(), s->start.as<int>(),
                c.count};
    PSIM_CUDA(launch_pair_count(s->g, cv, (float)(cutoff * cutoff), tot.as<unsigned long long>(),
                                s->st));
    unsigned long long h = 0;
    PSIM_CUDA(cudaMemcpyAsync(&h, tot.p, 8, cudaMemcpyDeviceToHost, s->st));
    PSIM_CUDA(cudaStreamSynchronize(s->st));
    *mean_pairs = s->n ? (double)h / s->n : 0.0;
    return PSIM_OK;
}

int psim_measure_fp32_peak(int32_t device, double* tflops) {
    if (!tflops) return fail(PSIM_ERR_INPUT, "NULL argument");
    int rc = ensure_device();
    if (rc) return rc;
    DeviceGuard dg(device);
    int sms = 0;
    PSIM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int threads = 256, blocks = sms * 8, iters = 4096;
    ScopedBuf sink;
    PSIM_CUDA(sink.ensure(4));
    cudaEvent_t a, b;
    PSIM_CUDA(cudaEventCreate(&a));
    PSIM_CUDA(cudaEventCreate(&b));
    PSIM_CUDA(launch_fma_probe(blocks, threads, 64, sink.as<float>(), 0));  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        PSIM_CUDA(cudaEventRecord(a, 0));
        PSIM_CUDA(launch_fma_probe(blocks, threads, iters, sink.as<float>(), 0));
        PSIM_CUDA(cudaEventRecord(b, 0));
        PSIM_CUDA(cudaEventSynchronize(b));
        float t = 0.f;
        PSIM_CUDA(cudaEventElapsedTime(&t, a, b));
        if (t < best) best = t;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * (double)blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return PSIM_OK;
}

int psim_measure_host_link(int32_t device, double* read_gbs, double* write_gbs,
                           double* both_gbs) {
    if (!read_gbs || !write_gbs || !both_gbs) return fail(PSIM_ERR_INPUT, "NULL argument");
    int rc = ensure_device();
    if (rc) return rc;
    DeviceGuard dg(device);
    int sms = 0;
    PSIM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const size_t bytes = 128ull << 20;
    ScopedBuf d;
    PSIM_CUDA(d.ensure(bytes));
    PSIM_CUDA(cudaMemset(d.p, 0, bytes));
    void* h[2] = {nullptr, nullptr};
    for (void*& p : h) {
        if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            for (void* q : h)
                if (q) cudaFreeHost(q);
            return fail(PSIM_ERR_CUDA, "pinned host allocation failed");
        }
        std::memset(p, 1, bytes);
    }
    void* hd[2] = {nullptr, nullptr};   // the device's addresses of the host buffers
    rc = PSIM_OK;
    for (int k = 0; k < 2 && rc == PSIM_OK; ++k)
        if (cudaHostGetDevicePointer(&hd[k], h[k], 0) != cudaSuccess)
            rc = fail(PSIM_ERR_CUDA, "host buffer not mapped");
    cudaEvent_t a = nullptr, b = nullptr;
    if (rc == PSIM_OK && (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess))
        rc = fail(PSIM_ERR_CUDA, "event creation failed");
    // read: host -> device; write: device -> host; both: host -> host through
    // the SMs (each byte crosses the link twice, as in the in-place drop-ins)
    const void* src[3] = {hd[0], d.p, hd[0]};
    void* dst[3] = {d.p, hd[1], hd[1]};
    double* out[3] = {read_gbs, write_gbs, both_gbs};
    for (int k = 0; k < 3 && rc == PSIM_OK; ++k) {
        float best = 1e30f;
        for (int r = 0; r < 4 && rc == PSIM_OK; ++r) {
            if (cudaEventRecord(a, 0) != cudaSuccess ||
                launch_link_copy(sms * 4, src[k], dst[k], bytes, 0) != cudaSuccess ||
                cudaEventRecord(b, 0) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
                rc = fail(PSIM_ERR_CUDA, "link probe failed: %s",
                          cudaGetErrorString(cudaGetLastError()));
                break;
            }
            float t = 0.f;
            cudaEventElapsedTime(&t, a, b);
            if (r > 0 && t < best) best = t;   // the first run warms the mappings
        }
        *out[k] = (k == 2 ? 2.0 : 1.0) * (double)bytes / (best * 1e-3) / 1e9;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    for (void* q : h) cudaFreeHost(q);
    return rc;
}

}  // extern "C"
