// yukawa_plugin.cu -- a force plugin written outside the library, to show the
// plugin contract: a pure screened-Coulomb repulsion
//     U(r) = A exp(-kappa (r - sigma)) / r,
//     F(r) = -dU/dr = A e^{kappa sigma} e^{-kappa r} (1 + kappa r) / r^2,
// with settings keys yukawaAmplitude (A, in kT), kappa, sigma and cutOff.
// In the reference's sign convention (fNet < 0 repels) this is the
// LennardJones plugin's Yukawa term with ljNum 0 (LJPotential.cpp:96-109)
// at kT wellDepth yukawaStrength = A kappa e^{kappa sigma} and debyeLength
// = 1/kappa, which is how the tests check it against the oracle.
//
// Built by proteinsim2015_gb300.build.build_force_plugin(this file); it
// includes the library's plugin header and nothing else of it.
#include "psim_plugin.cuh"

namespace {

struct YukawaPair {
    double rc2, amp, kappa;   // amp = A e^{kappa sigma}
    float rc2f, ampf, kappaf;
    static constexpr bool kCheckNan = false;
    __host__ __device__ double fnet64(double, double r, double rinv, double) const {
        return -(amp * exp(-kappa * r) * (1.0 + kappa * r) * (rinv * rinv));
    }
    __device__ float fnet32(float, float r, float rinv, float) const {
        return -(ampf * __expf(-kappaf * r) * (1.0f + kappaf * r) * (rinv * rinv));
    }
};

class Yukawa : public psim::PluginForce<Yukawa, YukawaPair> {
public:
    explicit Yukawa(PSim::config* cfg) {
        name = "Yukawa";
        const double A = cfg->getParam<double>("yukawaAmplitude", 10.0);
        const double kappa = cfg->getParam<double>("kappa", 4.0);
        const double sigma = cfg->getParam<double>("sigma", 1.0);
        params_.kind = PSIM_FORCE_PLUGIN;
        params_.kT = cfg->getParam<double>("kT", 1.0);
        params_.cutoff = cfg->getParam<double>("cutOff", 3.0);
        params_.user[0] = A * std::exp(kappa * sigma);
        params_.user[1] = kappa;
    }
    static YukawaPair pair(const psim_force_params& p) {
        YukawaPair y{};
        y.rc2 = p.cutoff * p.cutoff;
        y.amp = p.user[0];
        y.kappa = p.user[1];
        y.rc2f = (float)y.rc2;
        y.ampf = (float)y.amp;
        y.kappaf = (float)y.kappa;
        return y;
    }
};

}  // namespace

PSIM_FORCE_PLUGIN(Yukawa)
