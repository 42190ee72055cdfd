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
