// LennardJones.so -- the reference's LennardJones plugin (LennardJones/src/
// LJPotential.cpp, factory LennardJones/include/LJPotential.h:74-77) as a
// GB300 force plugin: the same settings keys and defaults (:29-62), the
// LJ(n) + Yukawa pair force as __device__ functors, its device entry
// psim_force_launch and the per-particle CPU getAcceleration of the
// reference contract.  The functor is picked per parameter regime: the
// exponent fixed at compile time for the plain 12-6 form without a Yukawa
// term, and for the pure Yukawa form (ljNum 0); the general functor for the
// rest.
#include "../psim_plugin.cuh"

namespace {

class LennardJones : public psim::PluginForce<LennardJones, psim::LJPair> {
public:
    explicit LennardJones(PSim::config* cfg) {
        name = "LennardJones";
        params_.kind = PSIM_FORCE_LJ;
        params_.kT = cfg->getParam<double>("kT", 1.0);
        params_.well_depth = cfg->getParam<double>("wellDepth", 10.0);
        params_.yukawa_strength = cfg->getParam<double>("yukawaStrength", 8.0);
        params_.lj_num = cfg->getParam<int>("ljNum", 18);
        params_.cutoff = cfg->getParam<double>("cutOff", 2.5);
        params_.debye_length = cfg->getParam<double>("debyeLength", 0.5);
    }
    static psim::LJPair pair(const psim_force_params& p) {
        return psim::make_lj_pair(p.kT, p.well_depth, p.lj_num, p.yukawa_strength,
                                  p.debye_length, p.cutoff);
    }
    template <class F>
    static int dispatch(const psim_force_params& p, F&& f) {
        const psim::LJPair lj = pair(p);
        if (p.yukawa_strength == 0.0 && p.lj_num == 6) {
            psim::LJPure<6> q;
            static_cast<psim::LJPair&>(q) = lj;
            return f(q);
        }
        if (p.lj_num == 0) {
            psim::LJFixed<0> q;
            static_cast<psim::LJPair&>(q) = lj;
            return f(q);
        }
        return f(lj);
    }
};

}  // namespace

PSIM_FORCE_PLUGIN(LennardJones)
