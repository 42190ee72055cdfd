// AOPotential.so -- the reference's AOPotential plugin (AOPotential/src/
// AOPotential.cpp, factory AOPotential/include/AOPotential.h:77-80) as a
// GB300 force plugin: the same settings keys and defaults (:33-59), the
// soft-core + Asakura-Oosawa pair force as the __device__ functor AOPair,
// its device entry psim_force_launch and the per-particle CPU
// getAcceleration of the reference contract.
#include "../psim_plugin.cuh"

namespace {

class AOPotential : public psim::PluginForce<AOPotential, psim::AOPair> {
public:
    explicit AOPotential(PSim::config* cfg) {
        name = "AOPotential";
        params_.kind = PSIM_FORCE_AO;
        params_.kT = cfg->getParam<double>("kT", 1.0);
        params_.well_depth = cfg->getParam<double>("wellDepth", 0.261);
        params_.cutoff = cfg->getParam<double>("cutOff", 1.1);
        params_.lj_num = 18;
        params_.debye_length = 0.5;
    }
    static psim::AOPair pair(const psim_force_params& p) {
        return psim::make_ao_pair(p.kT, p.well_depth, p.cutoff);
    }
};

}  // namespace

PSIM_FORCE_PLUGIN(AOPotential)
