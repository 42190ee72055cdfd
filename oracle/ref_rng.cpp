// ref_rng.cpp -- TEST INFRASTRUCTURE ONLY.
// Exposes the reference's own per-particle generator (fastRandom, compiled
// from ClusteredCore/src/utilities/fastRandom.cpp) to pin the oracle's
// restatement of psdrand/g250.
#include "fastRandom.h"

extern "C" void psimref_rng_draw(int seed, int count, double* out) {
    PSim::fastRandom r;
    for (int k = 0; k < count; k++) out[k] = r.g250(seed);
}
