// psim_gb300.hpp -- C++ host interface mirroring the reference's classes, on
// top of the C ABI in psim_gb300.h.  Link with -lpsim_gb300 -ldl.
//
//   PSim::config               settings.cfg reader   (ClusteredCore/include/config.h:15-63)
//   PSim::IForce               plugin contract       (ClusteredCore/include/interfaces/IForce.h:13-65)
//   PSim::create_Force         getForce factory type (IForce.h:65)
//   PSim::loadForces           dlopen("./<force>.so") + getForce (ClusteredUI/src/runSim.cpp:29-79)
//   PSim::defaultForceManager  whole-system force call (forceManager.h:20-121)
//   PSim::brownianIntegrator   nextSystem            (integrator.h:20-158)
//   PSim::system               device-resident step loop (system.h:17-301, run at system.cpp:170-212)
//
// The GB300 IForce keeps the factory, the settings keys and isTimeDependent/
// quench/getName; the per-particle virtual getAcceleration(index, ...) of the
// reference is replaced by deviceParams(): the parameters of the plugin's
// __device__ pair functor, which the GPU force pass evaluates for every
// particle at once (a virtual call per particle cannot run on the device).
#ifndef PSIM_GB300_HPP
#define PSIM_GB300_HPP

#include <dlfcn.h>

#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "psim_gb300.h"

namespace PSim {

// settings.cfg: "key = value" lines, '#' at column 0 for comments
// (config.cpp:27-56); values parse like std::stod/std::stoi.
class config {
public:
    static const int version = 1;
    config() {}
    explicit config(const std::string& fileName) {
        std::ifstream in(fileName);
        std::stringstream ss;
        ss << in.rdbuf();
        text_ = ss.str();
        parse(text_);
    }
    static config fromText(const std::string& text) {
        config c;
        c.text_ = text;
        c.parse(text);
        return c;
    }
    template <typename T> T getParam(const std::string& key, T def) const;
    bool containsKey(const std::string& key) const { return options_.count(key) != 0; }
    void set(const std::string& key, const std::string& val) {
        options_[key] = val;
        text_ += "\n" + key + " = " + val;
    }
    const std::string& text() const { return text_; }

private:
    void parse(const std::string& text) {
        std::istringstream is(text);
        for (std::string line; std::getline(is, line);) {
            if (line.empty() || line[0] == '#') continue;
            size_t eq = line.find('=');
            std::string key = trim(line.substr(0, eq));
            std::string val = eq == std::string::npos ? std::string() : trim(line.substr(eq + 1));
            options_[key] = val;
        }
    }
    static std::string trim(const std::string& s) {
        size_t a = s.find_first_not_of(" \t\r\n\v\f"), b = s.find_last_not_of(" \t\r\n\v\f");
        return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    }
    std::map<std::string, std::string> options_;
    std::string text_;
};

template <> inline double config::getParam<double>(const std::string& k, double def) const {
    auto it = options_.find(k);
    return it == options_.end() ? def : std::stod(it->second);
}
template <> inline int config::getParam<int>(const std::string& k, int def) const {
    auto it = options_.find(k);
    return it == options_.end() ? def : std::stoi(it->second);
}
template <> inline std::string config::getParam<std::string>(const std::string& k,
                                                             std::string def) const {
    auto it = options_.find(k);
    return it == options_.end() ? def : it->second;
}

// systemState (structs/systemState.h:7-19) with the box and cell edge as double.
struct systemState {
    int nParticles = 0;
    double concentration = 0;
    double boxSize = 0;
    double cellSize = 0;
    int cellScale = 0;
    double temp = 1;
    double currentTime = 0;
    double dTime = 0.001;
    int seed = 90210;
    int outputFreq = 1000;
    double endTime = 0;
};

class IForce {
protected:
    std::string name;

public:
    static const int version = 1;
    virtual ~IForce() {}
    // Parameters of the plugin's __device__ pair functor.
    virtual psim_force_params deviceParams() const = 0;
    virtual bool isTimeDependent() = 0;
    // Called after integration (IForce.h:48); no caller exists in the reference either.
    virtual void quench(systemState*) {}
    std::string getName() { return name; }
};

typedef IForce* create_Force(config*);

inline void check(int rc) {
    if (rc != PSIM_OK)
        throw std::runtime_error("psim error " + std::to_string(rc) + ": " +
                                 psim_last_error_string());
}

// runSim.cpp:29-79: open "./<force>.so" (or a path), resolve getForce, call it.
// Exit code 100 of the reference becomes an exception carrying PSIM_ERR_LOAD.
inline IForce* loadForces(config* cfg, const std::string& dir = ".") {
    std::string forceName = cfg->getParam<std::string>("force", "");
    std::string fileName = dir + "/" + forceName + ".so";
    void* lib = dlopen(fileName.c_str(), RTLD_LAZY);
    if (!lib) throw std::runtime_error("psim error 100: cannot load " + fileName);
    dlerror();
    create_Force* factory = (create_Force*)dlsym(lib, "getForce");
    if (dlerror()) throw std::runtime_error("psim error 100: no getForce in " + fileName);
    return factory(cfg);
}

inline psim_geometry geometryOf(const systemState& s) {
    psim_geometry g;
    g.n_particles = s.nParticles;
    g.cell_scale = s.cellScale;
    g.box_size = s.boxSize;
    g.cell_size = s.cellSize;
    return g;
}

// defaultForceManager (forceManager.h:20-121): holds the forces; only the
// first is evaluated, as the reference does (defaultForceManager.cpp:56).
class defaultForceManager {
    std::vector<IForce*> flist;
    bool timeDependent = false;
    int precision = PSIM_PRECISION_FP64;

public:
    void addForce(IForce* f) {
        flist.push_back(f);
        if (f->isTimeDependent()) timeDependent = true;
    }
    bool isTimeDependent() { return timeDependent; }
    void setPrecision(int p) { precision = p; }
    IForce* first() const { return flist.empty() ? nullptr : flist[0]; }
    // defaultForceManager::getAcceleration on the reference's own arrays
    // (defaultForceManager.cpp:55-65).
    void getAcceleration(const double* sortedParticles, double* particleForce,
                         const int32_t* particleHashIndex, const uint32_t* cellStartEnd,
                         const systemState* state) {
        if (flist.empty()) throw std::runtime_error("no force loaded");
        psim_force_params p = flist[0]->deviceParams();
        psim_geometry g = geometryOf(*state);
        check(psim_force_evaluate(&p, &g, precision, sortedParticles, particleHashIndex,
                                  cellStartEnd, particleForce));
    }
};

// brownianIntegrator (integrator.h:20-158) over host arrays in original order.
class brownianIntegrator {
    psim_integrator* it_ = nullptr;

public:
    brownianIntegrator(config* cfg) {
        psim_integrator_config c;
        c.gamma = cfg->getParam<double>("gamma", 0.5);
        c.dt = cfg->getParam<double>("timeStep", 0.001);
        c.kT = cfg->getParam<double>("kT", 1.0);
        c.vel_freq = cfg->getParam<int>("velFreq", 1000);
        c.seed = cfg->getParam<int>("seed", 90210);
        it_ = psim_integrator_create(&c, cfg->getParam<int>("nParticles", 1000));
        if (!it_) check(PSIM_ERR_INPUT);
    }
    ~brownianIntegrator() { psim_integrator_destroy(it_); }
    brownianIntegrator(const brownianIntegrator&) = delete;
    brownianIntegrator& operator=(const brownianIntegrator&) = delete;
    int nextSystem(double* pos, double* pos0, double* vel, double* frc, double* frc0,
                   const double* mass, systemState* state, const double* particleForce = nullptr,
                   const double* injectedNoise = nullptr) {
        return psim_integrator_next_system(
            it_, state->currentTime, state->boxSize,
            injectedNoise ? PSIM_NOISE_INJECTED : PSIM_NOISE_PHILOX, injectedNoise,
            particleForce, pos, pos0, vel, frc, frc0, mass);
    }
};

// system (system.h:17-301): the state lives on the GPU; run() is the hot
// loop of system::run (system.cpp:187-206) without the analysis output.
class system {
    psim_system* sys_ = nullptr;
    systemState state_;

public:
    system(config* cfg, IForce* force, int precision = PSIM_PRECISION_MIXED, int device = 0) {
        state_.nParticles = cfg->getParam<int>("nParticles", 1000);
        state_.dTime = cfg->getParam<double>("timeStep", 0.001);
        state_.temp = cfg->getParam<double>("kT", 1.0);
        state_.seed = cfg->getParam<int>("seed", 90210);
        state_.cellScale = cfg->getParam<int>("scale", 4);
        state_.boxSize = cfg->getParam<double>("boxSize", 0.0);
        state_.cellSize = state_.boxSize / state_.cellScale;
        psim_system_config c{};
        c.geom = geometryOf(state_);
        c.integ.gamma = cfg->getParam<double>("gamma", 0.5);
        c.integ.dt = state_.dTime;
        c.integ.kT = state_.temp;
        c.integ.vel_freq = cfg->getParam<int>("velFreq", 1000);
        c.integ.seed = state_.seed;
        c.force = force->deviceParams();
        c.precision = precision;
        c.noise_mode = PSIM_NOISE_PHILOX;
        c.device = device;
        // settings key "skin": the mixed form's Verlet pair-list skin (0: none)
        c.skin = precision == PSIM_PRECISION_MIXED ? cfg->getParam<double>("skin", 0.0) : 0.0;
        sys_ = psim_system_create(&c);
        if (!sys_) check(PSIM_ERR_INPUT);
    }
    ~system() { psim_system_destroy(sys_); }
    system(const system&) = delete;
    system& operator=(const system&) = delete;
    void upload(const double* pos, const double* vel, const double* radius,
                const double* mass = nullptr) {
        check(psim_system_upload(sys_, pos, nullptr, vel, nullptr, nullptr, radius, mass));
        state_.currentTime = 0;
    }
    void run(double endTime) {
        state_.endTime = endTime;
        int64_t steps = 0;
        double t = state_.currentTime;
        while (t < endTime) {  // the reference's loop test and time accumulation
            t += state_.dTime;
            ++steps;
        }
        check(psim_system_step(sys_, (int32_t)steps));
        state_.currentTime = t;
    }
    void download(double* pos, double* pos0, double* vel, double* frc, double* frc0) {
        check(psim_system_download(sys_, pos, pos0, vel, frc, frc0));
    }
    const systemState& state() const { return state_; }
    psim_system* handle() { return sys_; }
};

}  // namespace PSim

#endif  // PSIM_GB300_HPP
