// psim_plugin.cpp -- the force plugins as drop-in shared objects.
//
// Built three times (PSIM_PLUGIN_NAME = AOPotential, LennardJones,
// Calibration) into <name>.so, each exporting the reference's factory
//     extern "C" PSim::IForce* getForce(PSim::config* cfg)
// (AOPotential/include/AOPotential.h:77-80, LennardJones/include/LJPotential.h:74-77,
//  Calibration/include/Calibration.h:65-68).  The object reads the same
// settings.cfg keys with the same defaults as the reference constructors and
// hands the values to the device pair functor through deviceParams().
#include "psim_gb300.hpp"

#ifndef PSIM_PLUGIN_NAME
#error "PSIM_PLUGIN_NAME must name the plugin"
#endif

namespace {

class GB300Force : public PSim::IForce {
    psim_force_params p_{};

public:
    explicit GB300Force(PSim::config* cfg) {
        const std::string plugin = PSIM_PLUGIN_NAME;
        name = plugin;
        p_.kT = cfg->getParam<double>("kT", 1.0);
        p_.debye_length = 0.5;
        p_.lj_num = 18;
        if (plugin == "AOPotential") {            // AOPotential.cpp:40-47
            p_.kind = PSIM_FORCE_AO;
            p_.well_depth = cfg->getParam<double>("wellDepth", 0.261);
            p_.cutoff = cfg->getParam<double>("cutOff", 1.1);
        } else if (plugin == "LennardJones") {    // LJPotential.cpp:31-55
            p_.kind = PSIM_FORCE_LJ;
            p_.well_depth = cfg->getParam<double>("wellDepth", 10.0);
            p_.yukawa_strength = cfg->getParam<double>("yukawaStrength", 8.0);
            p_.lj_num = cfg->getParam<int>("ljNum", 18);
            p_.cutoff = cfg->getParam<double>("cutOff", 2.5);
            p_.debye_length = cfg->getParam<double>("debyeLength", 0.5);
        } else {                                  // Calibration.cpp:33-36
            p_.kind = PSIM_FORCE_CALIBRATION;
            p_.cutoff = cfg->getParam<double>("cutOff", 1.1);
        }
    }
    psim_force_params deviceParams() const override { return p_; }
    bool isTimeDependent() override { return false; }
};

}  // namespace

extern "C" PSim::IForce* getForce(PSim::config* cfg) { return new GB300Force(cfg); }

// C entry for callers without the C++ ABI (ctypes): the parameters the
// factory would produce from settings.cfg text.
extern "C" int psim_plugin_params(const char* settings_text, psim_force_params* out) {
    PSim::config cfg = PSim::config::fromText(settings_text ? settings_text : "");
    GB300Force f(&cfg);
    *out = f.deviceParams();
    return 0;
}
