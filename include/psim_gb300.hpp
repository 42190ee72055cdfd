// psim_gb300.hpp -- C++ host interface mirroring the reference's classes, on
// top of the C ABI in psim_gb300.h.  Link with -lpsim_gb300 -ldl.
//
//   PSim::config               settings.cfg reader   (ClusteredCore/include/config.h:15-63)
//   PSim::systemState          run constants         (ClusteredCore/include/structs/systemState.h:7-19)
//   PSim::IForce               plugin contract       (ClusteredCore/include/interfaces/IForce.h:13-65)
//   PSim::create_Force         getForce factory type (IForce.h:65)
//   PSim::loadForces           dlopen("./<force>.so") + getForce (ClusteredUI/src/runSim.cpp:29-79)
//   PSim::systemConstants      the box from settings.cfg (ClusteredCore/src/system/system.cpp:28-65)
//   PSim::defaultForceManager  whole-system force call (forceManager.h:20-121)
//   PSim::brownianIntegrator   nextSystem            (integrator.h:20-158)
//   PSim::system               device-resident step loop (system.h:17-301, run at system.cpp:170-212)
//
// config, systemState and IForce have the reference's memory layout and
// virtual-function order, so a plugin built against this header loads into a
// host built from the reference's sources and the reverse: the reference
// calls getAcceleration(index, ...) per particle through the vtable.  A
// GB300 plugin also exports C entries beside getForce (psim_plugin_abi,
// psim_plugin_device_params, psim_force_launch): loadForces looks them up
// and records them, and the GPU paths run the plugin's device pair functor
// through psim_force_launch.  A reference plugin, which has none, still
// loads; the GPU paths refuse it (it can only run on the CPU).
#ifndef PSIM_GB300_HPP
#define PSIM_GB300_HPP

#include <dlfcn.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "psim_gb300.h"

namespace PSim {

// settings.cfg: "key = value" lines, '#' at column 0 for comments
// (config.cpp:27-56); values parse like std::stod/std::stoi.  The first two
// members are the reference's (options, suppressOutput), in its order.
class config {
    std::map<std::string, std::string> options_;
    bool suppressOutput_ = true;
    std::string text_;

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
    void showOutput() { suppressOutput_ = false; }
    void hideOutput() { suppressOutput_ = true; }

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

// systemState (structs/systemState.h:7-19), the reference's layout: an
// integer box and cell edge.  A real-valued box (a GB300 extension) travels
// as psim_geometry beside it.
struct systemState {
    int nParticles = 0;
    double concentration = 0;
    int boxSize = 0;
    int cellSize = 0;
    int cellScale = 0;
    double temp = 1;
    double currentTime = 0;
    double dTime = 0.001;
    int seed = 90210;
    int outputFreq = 1000;
    double endTime = 0;
};

// IForce.h:13-65, in its virtual-function order.
class IForce {
protected:
    std::string name;

public:
    static const int version = 1;
    virtual ~IForce() {}
    // IForce.h:35: the force on the particle at sorted index `index`, written
    // to particleForce[3 * original index ...] (called concurrently for
    // distinct indices).  GB300 plugins implement it on the CPU with their
    // pair functor, for hosts built from the reference; the GPU paths of
    // this library never call it.
    virtual void getAcceleration(int index, double* sortedParticles, double* particleForce,
                                 std::vector<std::tuple<int, int>>* particleHashIndex,
                                 std::vector<std::tuple<int, int>>* cellStartEnd,
                                 systemState* state) = 0;
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

// The C entries a GB300 plugin exports beside getForce.
typedef int psim_plugin_abi_fn(void);
typedef int psim_plugin_device_params_fn(IForce*, psim_force_params*);

// The device side of a loaded force: its parameters and launch entry.
struct DeviceForce {
    psim_force_params params;
    psim_force_launch_fn launch;
};

inline std::map<const IForce*, DeviceForce>& deviceForceTable() {
    static std::map<const IForce*, DeviceForce> table;
    return table;
}
inline std::mutex& deviceForceMutex() {
    static std::mutex mu;
    return mu;
}

// The device side of a force that loadForces loaded from a GB300 plugin, or
// nullptr (a reference plugin, or a force not loaded through loadForces).
inline const DeviceForce* deviceForce(const IForce* f) {
    std::lock_guard<std::mutex> lk(deviceForceMutex());
    auto it = deviceForceTable().find(f);
    return it == deviceForceTable().end() ? nullptr : &it->second;
}

// runSim.cpp:29-79: open "./<force>.so" (or a path), resolve getForce, call
// it; for a GB300 plugin also resolve its device entry.  Exit code 100 of
// the reference becomes an exception carrying PSIM_ERR_LOAD.
inline IForce* loadForces(config* cfg, const std::string& dir = ".") {
    std::string forceName = cfg->getParam<std::string>("force", "");
    std::string fileName = dir + "/" + forceName + ".so";
    void* lib = dlopen(fileName.c_str(), RTLD_LAZY);
    if (!lib) throw std::runtime_error("psim error 100: cannot load " + fileName);
    dlerror();
    create_Force* factory = (create_Force*)dlsym(lib, "getForce");
    if (dlerror()) throw std::runtime_error("psim error 100: no getForce in " + fileName);
    IForce* f = factory(cfg);
    auto abi = (psim_plugin_abi_fn*)dlsym(lib, "psim_plugin_abi");
    auto params = (psim_plugin_device_params_fn*)dlsym(lib, "psim_plugin_device_params");
    auto launch = (psim_force_launch_fn)dlsym(lib, "psim_force_launch");
    if (abi && params && launch) {
        if (abi() != PSIM_FORCE_ABI)
            throw std::runtime_error("psim error 100: " + fileName +
                                     " was built for another device-entry ABI");
        DeviceForce d{};
        d.launch = launch;
        if (params(f, &d.params) != 0)
            throw std::runtime_error("psim error 100: " + fileName + " refused its parameters");
        std::lock_guard<std::mutex> lk(deviceForceMutex());
        deviceForceTable()[f] = d;
    }
    return f;
}

// The device side of f, or an exception naming why a GPU path cannot run it.
inline const DeviceForce& requireDevice(const IForce* f) {
    const DeviceForce* d = f ? deviceForce(f) : nullptr;
    if (!d)
        throw std::runtime_error("psim error 100: the force has no device entry "
                                 "(psim_force_launch); it can only run on the CPU");
    return *d;
}

// system::setSystemConstants (system.cpp:28-65): the run constants from
// settings.cfg.  The box holds nParticles spheres of `radius` at volume
// fraction `conc`, cut to a whole number of integer cells: L = int(cbrt(vP /
// conc)), cellSize = L / scale (integer division), L = cellSize * scale, and
// the concentration reported is that of the quantised box.  A `boxSize` key
// (which the reference never reads) gives a real-valued box instead, cut into
// `scale` cells; geom receives the grid either way (may be NULL).
inline systemState systemConstants(const config* cfg, psim_geometry* geom = nullptr) {
    systemState st;
    st.currentTime = 0;
    st.dTime = cfg->getParam<double>("timeStep", 0.001);
    st.seed = cfg->getParam<int>("seed", 90210);
    st.temp = cfg->getParam<double>("kT", 1.0);
    st.nParticles = cfg->getParam<int>("nParticles", 1000);
    st.outputFreq = cfg->getParam<int>("outputFreq", int(1.0 / st.dTime));
    const double conc = cfg->getParam<double>("conc", 0.01);
    const int scale = cfg->getParam<int>("scale", 4);
    const double r = cfg->getParam<double>("radius", 0.5);
    const double vP = st.nParticles * (4.0 / 3.0) * std::atan(1.0) * 4.0 * r * r * r;
    psim_geometry g{};
    g.n_particles = st.nParticles;
    g.cell_scale = scale;
    st.cellScale = scale;
    if (cfg->containsKey("boxSize")) {
        const double L = cfg->getParam<double>("boxSize", 0.0);
        g.box_size = L;
        g.cell_size = L / scale;
        st.boxSize = (int)L;
        st.cellSize = (int)g.cell_size;
        st.concentration = vP / (L * L * L);
    } else {
        st.boxSize = (int)(std::cbrt(vP / conc));
        st.cellSize = scale != 0 ? st.boxSize / scale : 0;
        st.boxSize = st.cellSize * scale;
        st.concentration = vP / std::pow((double)st.boxSize, 3.0);
        g.box_size = st.boxSize;
        g.cell_size = st.cellSize;
    }
    if (geom) *geom = g;
    return st;
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
// first is evaluated, as the reference does (defaultForceManager.cpp:56), on
// the GPU through its device entry.
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
    // defaultForceManager::getAcceleration (defaultForceManager.cpp:55-65) on
    // the reference's arrays as flat pairs: particleHashIndex (hash, index)
    // and cellStartEnd (start, end) int32 pairs.
    void getAcceleration(const double* sortedParticles, double* particleForce,
                         const int32_t* particleHashIndex, const uint32_t* cellStartEnd,
                         const psim_geometry& g) {
        if (flist.empty()) throw std::runtime_error("no force loaded");
        const DeviceForce& d = requireDevice(flist[0]);
        check(psim_force_evaluate_plugin(d.launch, &d.params, &g, precision, sortedParticles,
                                         particleHashIndex, cellStartEnd, particleForce));
    }
    void getAcceleration(const double* sortedParticles, double* particleForce,
                         const int32_t* particleHashIndex, const uint32_t* cellStartEnd,
                         const systemState* state) {
        getAcceleration(sortedParticles, particleForce, particleHashIndex, cellStartEnd,
                        geometryOf(*state));
    }
    // The reference's own signature, on its vectors of (hash, index) and
    // (start, end) tuples.
    void getAcceleration(double* sortedParticles, double* particleForce,
                         std::vector<std::tuple<int, int>>* particleHashIndex,
                         std::vector<std::tuple<int, int>>* cellStartEnd, systemState* state) {
        std::vector<int32_t> phi(2 * particleHashIndex->size());
        std::vector<uint32_t> cse(2 * cellStartEnd->size());
        for (size_t i = 0; i < particleHashIndex->size(); ++i) {
            phi[2 * i] = std::get<0>((*particleHashIndex)[i]);
            phi[2 * i + 1] = std::get<1>((*particleHashIndex)[i]);
        }
        for (size_t c = 0; c < cellStartEnd->size(); ++c) {
            cse[2 * c] = (uint32_t)std::get<0>((*cellStartEnd)[c]);
            cse[2 * c + 1] = (uint32_t)std::get<1>((*cellStartEnd)[c]);
        }
        getAcceleration(sortedParticles, particleForce, phi.data(), cse.data(), state);
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
                   const double* mass, double currentTime, double boxSize,
                   const double* particleForce = nullptr, const double* injectedNoise = nullptr) {
        return psim_integrator_next_system(
            it_, currentTime, boxSize, injectedNoise ? PSIM_NOISE_INJECTED : PSIM_NOISE_PHILOX,
            injectedNoise, particleForce, pos, pos0, vel, frc, frc0, mass);
    }
    int nextSystem(double* pos, double* pos0, double* vel, double* frc, double* frc0,
                   const double* mass, systemState* state, const double* particleForce = nullptr,
                   const double* injectedNoise = nullptr) {
        return nextSystem(pos, pos0, vel, frc, frc0, mass, state->currentTime,
                          (double)state->boxSize, particleForce, injectedNoise);
    }
};

// system (system.h:17-301): the state lives on the GPU; run() is the hot
// loop of system::run (system.cpp:187-206) without the analysis output.  The
// box comes from settings.cfg as the reference derives it (systemConstants);
// the force runs through the plugin's device entry.
class system {
    psim_system* sys_ = nullptr;
    systemState state_;
    psim_geometry geom_{};
    double radius_ = 0.5, mass_ = 1.0;

public:
    system(config* cfg, IForce* force, int precision = PSIM_PRECISION_MIXED, int device = 0) {
        const DeviceForce& d = requireDevice(force);
        state_ = systemConstants(cfg, &geom_);
        radius_ = cfg->getParam<double>("radius", 0.5);
        mass_ = cfg->getParam<double>("mass", 1.0);
        psim_system_config c{};
        c.geom = geom_;
        c.integ.gamma = cfg->getParam<double>("gamma", 0.5);
        c.integ.dt = state_.dTime;
        c.integ.kT = state_.temp;
        c.integ.vel_freq = cfg->getParam<int>("velFreq", 1000);
        c.integ.seed = state_.seed;
        c.force = d.params;
        c.force_launch = d.launch;
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
    // radius / mass NULL: every particle has the settings' radius / mass
    // (initParticles, system.cpp:88-95)
    void upload(const double* pos, const double* vel, const double* radius = nullptr,
                const double* mass = nullptr) {
        std::vector<double> r, m;
        if (!radius) {
            r.assign(state_.nParticles, radius_);
            radius = r.data();
        }
        if (!mass) {
            m.assign(state_.nParticles, mass_);
            mass = m.data();
        }
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
    const psim_geometry& geometry() const { return geom_; }
    psim_system* handle() { return sys_; }
};

}  // namespace PSim

#endif  // PSIM_GB300_HPP
