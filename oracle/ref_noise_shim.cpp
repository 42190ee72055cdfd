// ref_noise_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Link-time stand-in for the reference's per-particle generator
// (ClusteredCore/src/utilities/fastRandom.cpp) that serves pre-drawn
// Gaussians instead of computing them.  It implements the class declared in
// the reference's own header ClusteredCore/include/fastRandom.h:6-41, so the
// reference integrator (brownianIntegrator.cpp) runs unmodified on injected
// noise.  Generators are numbered in construction order, which is particle
// order (brownianIntegrator.cpp:48-50); `jrand` holds that number and
// istack[0] counts the draws made in the current step.
#include "fastRandom.h"

#include <cstddef>

namespace psimref {
const double* g_noise = nullptr;  // n x 6 Gaussians for the current step
int g_next_id = 0;
}  // namespace psimref

namespace PSim {

fastRandom::fastRandom() {
    deviateAvailable = false;
    storedDeviate = 0;
    jrand = psimref::g_next_id++;
    istack = new int[58]();
    init = false;
}

fastRandom::~fastRandom() {}

double fastRandom::psdrand(int) { return 0.0; }

double fastRandom::g250(int, double mu, double sigma) {
    int k = istack[0]++;
    return psimref::g_noise[(std::size_t)jrand * 6 + (std::size_t)k] * sigma + mu;
}

}  // namespace PSim
