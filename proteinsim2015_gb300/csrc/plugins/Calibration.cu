// Calibration.so -- the reference's Calibration plugin (Calibration/src/
// Calibration.cpp, factory Calibration/include/Calibration.h:65-68) as a
// GB300 force plugin: the same settings key and default (:30-39), the
// r^-36 repulsion as the __device__ functor CalPair, its device entry
// psim_force_launch and the per-particle CPU getAcceleration of the
// reference contract.
#include "../psim_plugin.cuh"

namespace {

class Calibration : public psim::PluginForce<Calibration, psim::CalPair> {
public:
    explicit Calibration(PSim::config* cfg) {
        name = "Calibration";
        params_.kind = PSIM_FORCE_CALIBRATION;
        params_.kT = cfg->getParam<double>("kT", 1.0);
        params_.cutoff = cfg->getParam<double>("cutOff", 1.1);
        params_.lj_num = 18;
        params_.debye_length = 0.5;
    }
    static psim::CalPair pair(const psim_force_params& p) { return psim::make_cal_pair(p.cutoff); }
};

}  // namespace

PSIM_FORCE_PLUGIN(Calibration)
