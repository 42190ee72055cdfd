// psim_plugin.cuh -- what a force plugin compiles against.
//
// A force plugin is one shared object that keeps the reference's plugin
// contract -- the factory extern "C" getForce(config*) returning an IForce
// whose getAcceleration(index, ...) is called per particle
// (ClusteredCore/include/interfaces/IForce.h:35-65, AOPotential.h:77-80) --
// and adds a device entry, psim_force_launch (psim_gb300.h), that runs the
// library's force passes instantiated with the plugin's own __device__ pair
// functor.  A new potential therefore needs no rebuild of the library.
//
// A plugin source (one .cu file) defines
//   * its pair functor Pair with
//       double rc2; float rc2f;                     the cutoff squared
//       static constexpr bool kCheckNan;            7705 on a NaN force (AO)
//       __host__ __device__ double fnet64(r2, r, 1/r, size)   F(r) in FP64
//       __device__ float fnet32(r2, r, 1/r, size)              F(r) in FP32
//     where F(r) is the reference's fNet: positive attracts, and the pair
//     term on i is F(r) times the unit vector from i to j;
//   * its force class, deriving from psim::PluginForce<Class, Pair>: a
//     constructor from PSim::config* that fills params_ (kind
//     PSIM_FORCE_PLUGIN, the cutoff, any values in params_.user) and sets
//     `name`, and a static Pair pair(const psim_force_params&).  A plugin
//     with several functor types (one per parameter regime) instead
//     defines static dispatch(params, f), calling f with the functor it
//     picks;
//   * PSIM_FORCE_PLUGIN(Class) once, at file scope.
// The build (proteinsim2015_gb300.build.build_force_plugin) compiles the file
// twice: with PSIM_PLUGIN_PART=1 and --fmad=false for the plain FP64 pass
// (two roundings per a*b+c, as the reference's x86-64 build), and with
// PSIM_PLUGIN_PART=2 for the mixed passes and the host entries, and links
// both into <name>.so.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "../../include/psim_gb300.hpp"
#include "psim_body.cuh"
#include "psim_force_cell.cuh"
#if !defined(PSIM_PLUGIN_PART) || PSIM_PLUGIN_PART != 1
#include "psim_force_list.cuh"
#endif

namespace psim {

// ------------------------------------------------------ the device entry

inline DevGeom plugin_geom(const psim_force_args* a) {
    DevGeom g{};
    fill_geom(a->n_particles, a->cell_scale, a->box_size, a->cell_size, &g);
    return g;
}

inline CellView plugin_cells(const psim_force_args* a) {
    return CellView{static_cast<const double4_32a*>(a->pos_fp64),
                    static_cast<const float4*>(a->pos_hi), static_cast<const float4*>(a->pos_lo),
                    a->cell_id, a->cell_start, a->cell_count};
}

inline ForceOut plugin_out(const psim_force_args* a) {
    return ForceOut{a->fx, a->fy, a->fz, a->err, a->gate};
}

inline int plugin_status(cudaError_t e) { return e == cudaSuccess ? PSIM_OK : PSIM_ERR_CUDA; }

// The plain FP64 pass with functor p (a translation unit built with --fmad=false).
template <class Pair>
int plugin_launch_fp64(const Pair& p, const psim_force_args* a, cudaStream_t st) {
    const DevGeom g = plugin_geom(a);
    const F64Body<Pair> body{p, g};
    const CellView cv = plugin_cells(a);
    const ForceOut out = plugin_out(a);
    if (a->tile) return plugin_status(launch_force_cells(body, g, cv, out, a->prefilter_r2, st));
    return plugin_status(launch_force_pass(body, g, cv, out, a->prefilter_r2, st));
}

#if !defined(PSIM_PLUGIN_PART) || PSIM_PLUGIN_PART != 1
// The mixed passes with functor p: the 27-cell walk or the pair list.
template <class Pair>
int plugin_launch_mixed(const Pair& p, const psim_force_args* a, cudaStream_t st) {
    const DevGeom g = plugin_geom(a);
    const MixedBody<Pair> body{p, p.rc2f};
    const ForceOut out = plugin_out(a);
    if (a->pass == PSIM_PASS_LIST) {
        PairList pl{};
        pl.pos = static_cast<const float4*>(a->list_pos);
        pl.count = a->list_count;
        pl.list = a->list;
        pl.stride = a->list_stride;
        pl.compact = a->list_compact;
        pl.radius = a->list_radius;
        pl.unit = a->list_unit;
        return plugin_status(launch_force_list(body, g, pl, out, st));
    }
    const CellView cv = plugin_cells(a);
    if (a->tile) return plugin_status(launch_force_cells(body, g, cv, out, a->prefilter_r2, st));
    return plugin_status(launch_force_pass(body, g, cv, out, a->prefilter_r2, st));
}
#endif

// ------------------------------------------- the reference's CPU entry

// The force on the particle at sorted index `index` with pair functor pf,
// as the reference plugins compute it (AOPotential.cpp:132-175 with
// iterCells :61-130; the same walk in LJPotential.cpp:64-182 and
// Calibration.cpp:41-147): its home cell from its position, the 27 cells
// around it (wrapped), every other particle of each within the cutoff, the
// minimum image of pbcDist (|d| > L/2.0, utilities.cpp:79-104) for r^2 and
// of unitVectorAdv (|d| > int(L)/2, utilities.cpp:114-142) for the
// direction, each cell's partial added to the total.  Errors end the
// process with the reference's exit codes: 7704 for an overlap
// (r < 0.8 (Ri + Rj)), 7705 for a NaN force when Pair::kCheckNan.
template <class Pair>
void cpu_get_acceleration(const Pair& pf, int index, const double* sorted, double* force,
                          const std::vector<std::tuple<int, int>>* hash_index,
                          const std::vector<std::tuple<int, int>>* cell_start_end,
                          const PSim::systemState* st) {
    const double L = st->boxSize;
    const double half = L / 2.0;
    const double half_uv = (double)(st->boxSize / 2);
    const int s = st->cellScale;
    const double* pi = sorted + 4 * (size_t)index;
    int home[3];
    for (int k = 0; k < 3; ++k) home[k] = (int)std::floor(pi[k] / st->cellSize);
    double net[3] = {0.0, 0.0, 0.0};
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                int c[3] = {home[0] + dx, home[1] + dy, home[2] + dz};
                for (int k = 0; k < 3; ++k) {
                    c[k] %= s;
                    if (c[k] < 0) c[k] += s;
                }
                const auto& range = (*cell_start_end)[c[0] + s * c[1] + s * s * c[2]];
                const uint32_t first = (uint32_t)std::get<0>(range);
                if (first == 0xffffffffu) continue;
                const int last = std::get<1>(range);
                double part[3] = {0.0, 0.0, 0.0};
                for (int j = (int)first; j < last; ++j) {
                    if (j == index) continue;
                    const double* pj = sorted + 4 * (size_t)j;
                    double a[3], d[3];
                    for (int k = 0; k < 3; ++k) {
                        d[k] = pj[k] - pi[k];
                        a[k] = std::fabs(d[k]);
                        if (a[k] > half) a[k] -= L;
                    }
                    const double r2 = (a[0] * a[0]) + (a[1] * a[1]) + (a[2] * a[2]);
                    if (!(r2 < pf.rc2)) continue;
                    const double r = std::sqrt(r2);
                    const double size = pi[3] + pj[3];
                    if (r < 0.8 * size) {
                        std::fprintf(stderr, "Particle overlap: %d and %d at r = %g\n", index, j, r);
                        std::exit(PSIM_ERR_OVERLAP);
                    }
                    const double rinv = 1.0 / r;
                    const double f = pf.fnet64(r2, r, rinv, size);
                    if (Pair::kCheckNan && std::isnan(f)) {
                        std::fprintf(stderr, "Non-finite force on particle %d\n", index);
                        std::exit(PSIM_ERR_NAN_FORCE);
                    }
                    for (int k = 0; k < 3; ++k) {
                        if (std::fabs(d[k]) > half_uv) d[k] = (d[k] < 0) ? d[k] + L : d[k] - L;
                        part[k] += f * (d[k] * rinv);
                    }
                }
                for (int k = 0; k < 3; ++k) net[k] += part[k];
            }
    const int o = 3 * std::get<1>((*hash_index)[index]);
    force[o] = net[0];
    force[o + 1] = net[1];
    force[o + 2] = net[2];
}

// The base of a GB300 force plugin: the reference's IForce with its
// per-particle CPU entry, and the parameters the device entry receives.
// Derived supplies a constructor from PSim::config* (filling params_ and
// name) and static Pair pair(const psim_force_params&).
template <class Derived, class Pair>
class PluginForce : public PSim::IForce {
protected:
    psim_force_params params_{};

public:
    const psim_force_params& deviceParams() const { return params_; }
    // f(functor) with the functor of parameters p (one type by default)
    template <class F>
    static int dispatch(const psim_force_params& p, F&& f) {
        return f(Derived::pair(p));
    }
    void getAcceleration(int index, double* sortedParticles, double* particleForce,
                         std::vector<std::tuple<int, int>>* particleHashIndex,
                         std::vector<std::tuple<int, int>>* cellStartEnd,
                         PSim::systemState* state) override {
        Derived::dispatch(params_, [&](const auto& pf) {
            cpu_get_acceleration(pf, index, sortedParticles, particleForce, particleHashIndex,
                                 cellStartEnd, state);
            return 0;
        });
    }
    bool isTimeDependent() override { return false; }
};

}  // namespace psim

// The plugin's exported entries.  Part 1 holds the FP64 pass; part 2 the
// mixed passes, the device entry that dispatches on the pass, the reference
// factory getForce and the entries the GB300 host looks up beside it.
#if defined(PSIM_PLUGIN_PART) && PSIM_PLUGIN_PART == 1
#define PSIM_FORCE_PLUGIN(Class)                                                               \
    extern "C" __attribute__((visibility("default"))) int psim_plugin_launch_fp64(            \
        const psim_force_args* a, void* st) {                                                  \
        return Class::dispatch(*a->params, [&](const auto& pf) {                               \
            return psim::plugin_launch_fp64(pf, a, static_cast<cudaStream_t>(st));             \
        });                                                                                    \
    }
#else
#define PSIM_FORCE_PLUGIN(Class)                                                               \
    extern "C" int psim_plugin_launch_fp64(const psim_force_args* a, void* st);                \
    extern "C" __attribute__((visibility("default"))) int psim_force_launch(                   \
        const psim_force_args* a, void* st) {                                                  \
        if (!a || a->abi != PSIM_FORCE_ABI || !a->params) return PSIM_ERR_INPUT;               \
        if (a->pass == PSIM_PASS_FP64) return psim_plugin_launch_fp64(a, st);                  \
        if (a->pass != PSIM_PASS_MIXED && a->pass != PSIM_PASS_LIST) return PSIM_ERR_INPUT;    \
        return Class::dispatch(*a->params, [&](const auto& pf) {                               \
            return psim::plugin_launch_mixed(pf, a, static_cast<cudaStream_t>(st));            \
        });                                                                                    \
    }                                                                                          \
    extern "C" __attribute__((visibility("default"))) PSim::IForce* getForce(                  \
        PSim::config* cfg) {                                                                   \
        return new Class(cfg);                                                                 \
    }                                                                                          \
    extern "C" __attribute__((visibility("default"))) int psim_plugin_abi(void) {              \
        return PSIM_FORCE_ABI;                                                                 \
    }                                                                                          \
    extern "C" __attribute__((visibility("default"))) int psim_plugin_device_params(           \
        PSim::IForce* f, psim_force_params* out) {                                             \
        if (!f || !out) return PSIM_ERR_INPUT;                                                 \
        *out = static_cast<Class*>(f)->deviceParams();                                         \
        return PSIM_OK;                                                                        \
    }                                                                                          \
    extern "C" __attribute__((visibility("default"))) int psim_plugin_params(                  \
        const char* settings_text, psim_force_params* out) {                                   \
        if (!out) return PSIM_ERR_INPUT;                                                       \
        PSim::config cfg = PSim::config::fromText(settings_text ? settings_text : "");         \
        Class f(&cfg);                                                                         \
        *out = f.deviceParams();                                                               \
        return PSIM_OK;                                                                        \
    }
#endif
