// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own hot-path code, compiled from its sources by
// oracle/build_ref.sh, on states injected from the caller:
//   system::hashParticles / sortParticles / clearCells / reorderParticles
//       (ClusteredCore/src/system/systemHandling.cpp:33-85, system.h:166)
//   defaultForceManager::getAcceleration + plugin getForce factories
//       (defaultForceManager.cpp:55-65; AOPotential.h:77-80, LJPotential.h:74-77,
//        Calibration.h:65-68)
//   brownianIntegrator(cfg) + nextSystem (brownianIntegrator.cpp:27-356)
//   the loop body of system::run (system.cpp:187-211)
// Private members are reached by compiling this file with `private` defined
// as `public` after every standard header is in; the reference's own
// translation units are compiled unchanged.  The system object is laid out
// in raw storage and only the members its hot-path methods touch are
// constructed, which skips the reference's O(N^2) random initialisation.
#include <bits/stdc++.h>
#include <dlfcn.h>
#include <parallel/algorithm>
#include <omp.h>
#include <sys/sendfile.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#define private public
#define protected public
#include "system.h"
#undef private
#undef protected

using PSim::particle;
using PSim::type3;

extern "C" PSim::IForce* psimref_getForce_AO(PSim::config*);
extern "C" PSim::IForce* psimref_getForce_LJ(PSim::config*);
extern "C" PSim::IForce* psimref_getForce_Cal(PSim::config*);

namespace psimref {
extern const double* g_noise;
extern int g_next_id;
}

namespace {

class NullAnalysis : public PSim::IAnalysisManager {
public:
    void postAnalysis(std::queue<std::string>*, particle**, PSim::systemState*) override {}
    void writeInitialState(particle**, PSim::systemState*) override {}
    void writeFinalState(particle**, PSim::systemState*) override {}
    void writeRunTimeState(particle**, PSim::systemState*) override {}
};

struct Geometry {
    int n, box, cell_size, scale;
};

PSim::system* make_system(const Geometry& g, const double* pos, const double* pos0,
                          const double* vel, const double* frc, const double* frc0,
                          const double* radius, const double* mass) {
    void* mem = ::operator new(sizeof(PSim::system));
    std::memset(mem, 0, sizeof(PSim::system));
    PSim::system* s = static_cast<PSim::system*>(mem);
    const int ncell = g.scale * g.scale * g.scale;
    new (&s->particleHashIndex) std::vector<std::tuple<int, int>>(g.n, std::tuple<int, int>());
    new (&s->cellStartEnd) std::vector<std::tuple<int, int>>(
        ncell, std::tuple<int, int>(0xffffffff, 0xffffffff));
    new (&s->trialName) std::string("/tmp/psimref_trial");
    s->state = PSim::systemState();
    s->state.nParticles = g.n;
    s->state.boxSize = g.box;
    s->state.cellSize = g.cell_size;
    s->state.cellScale = g.scale;
    s->state.currentTime = 0;
    s->state.outputFreq = 1 << 30;
    s->particles = new particle*[g.n];
    for (int i = 0; i < g.n; i++) {
        particle* p = new particle(i);
        p->pos = type3<double>(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        if (pos0) p->pos0 = type3<double>(pos0[3 * i], pos0[3 * i + 1], pos0[3 * i + 2]);
        if (vel) p->vel = type3<double>(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        if (frc) p->frc = type3<double>(frc[3 * i], frc[3 * i + 1], frc[3 * i + 2]);
        if (frc0) p->frc0 = type3<double>(frc0[3 * i], frc0[3 * i + 1], frc0[3 * i + 2]);
        p->r = radius[i];
        p->m = mass ? mass[i] : 1.0;
        s->particles[i] = p;
    }
    s->sortedParticles = new double[4 * (size_t)g.n];
    s->particleForce = new double[3 * (size_t)g.n]();
    s->analysis = new NullAnalysis();
    return s;
}

void export_cells(PSim::system* s, int* hash_index, uint32_t* cse, double* sorted) {
    const int n = s->state.nParticles;
    if (hash_index)
        for (int i = 0; i < n; i++) {
            hash_index[2 * i] = std::get<0>(s->particleHashIndex[i]);
            hash_index[2 * i + 1] = std::get<1>(s->particleHashIndex[i]);
        }
    if (cse)
        for (size_t c = 0; c < s->cellStartEnd.size(); c++) {
            cse[2 * c] = (uint32_t)std::get<0>(s->cellStartEnd[c]);
            cse[2 * c + 1] = (uint32_t)std::get<1>(s->cellStartEnd[c]);
        }
    if (sorted) std::memcpy(sorted, s->sortedParticles, sizeof(double) * 4 * (size_t)n);
}

void export_particles(PSim::system* s, double* pos, double* pos0, double* vel, double* frc,
                      double* frc0) {
    for (int i = 0; i < s->state.nParticles; i++) {
        particle* p = s->particles[i];
        if (pos) { pos[3 * i] = p->pos.x; pos[3 * i + 1] = p->pos.y; pos[3 * i + 2] = p->pos.z; }
        if (pos0) { pos0[3 * i] = p->pos0.x; pos0[3 * i + 1] = p->pos0.y; pos0[3 * i + 2] = p->pos0.z; }
        if (vel) { vel[3 * i] = p->vel.x; vel[3 * i + 1] = p->vel.y; vel[3 * i + 2] = p->vel.z; }
        if (frc) { frc[3 * i] = p->frc.x; frc[3 * i + 1] = p->frc.y; frc[3 * i + 2] = p->frc.z; }
        if (frc0) { frc0[3 * i] = p->frc0.x; frc0[3 * i + 1] = p->frc0.y; frc0[3 * i + 2] = p->frc0.z; }
    }
}

PSim::IForce* make_force(const char* plugin, PSim::config* cfg) {
    std::string p(plugin);
    if (p == "AO") return psimref_getForce_AO(cfg);
    if (p == "LJ") return psimref_getForce_LJ(cfg);
    if (p == "Cal") return psimref_getForce_Cal(cfg);
    return nullptr;
}

void set_threads(int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
}

}  // namespace

extern "C" {

// system::setSystemConstants (system.cpp:28-65) on a settings.cfg file: the
// integer box and cell edge the reference derives from nParticles, conc,
// radius and scale, and the concentration it reports.
int psimref_system_constants(const char* settings_path, int* n, int* box, int* cell_size,
                             int* scale, double* concentration) {
    PSim::config cfg{std::string(settings_path)};
    void* mem = ::operator new(sizeof(PSim::system));
    std::memset(mem, 0, sizeof(PSim::system));
    PSim::system* s = static_cast<PSim::system*>(mem);
    new (&s->trialName) std::string("/tmp/psimref_trial");
    s->setSystemConstants(&cfg, nullptr, nullptr);
    *n = s->state.nParticles;
    *box = s->state.boxSize;
    *cell_size = s->state.cellSize;
    *scale = s->state.cellScale;
    *concentration = s->state.concentration;
    return 0;
}

// Reference cell-list build on the given positions (original order).
int psimref_build_cells(int n, int box, int cell_size, int scale, const double* pos,
                        const double* radius, int* hash_index, uint32_t* cse, double* sorted,
                        int nthreads) {
    set_threads(nthreads);
    Geometry g{n, box, cell_size, scale};
    PSim::system* s = make_system(g, pos, nullptr, nullptr, nullptr, nullptr, radius, nullptr);
    s->hashParticles();
    s->sortParticles();
    s->clearCells();
    s->reorderParticles();
    export_cells(s, hash_index, cse, sorted);
    return 0;
}

// Reference force evaluation on a cell list given in the reference's layout.
int psimref_forces(const char* plugin, const char* settings_path, int n, int box,
                   int cell_size, int scale, const double* sorted, const int* hash_index,
                   const uint32_t* cse, double* force, int nthreads) {
    PSim::config cfg{std::string(settings_path)};
    PSim::IForce* f = make_force(plugin, &cfg);
    if (!f) return 100;
    PSim::defaultForceManager* mgr = new PSim::defaultForceManager();
    mgr->addForce(f);
    set_threads(nthreads);
    PSim::systemState st = PSim::systemState();
    st.nParticles = n;
    st.boxSize = box;
    st.cellSize = cell_size;
    st.cellScale = scale;
    std::vector<std::tuple<int, int>> phi(n), cells((size_t)scale * scale * scale);
    for (int i = 0; i < n; i++) phi[i] = std::make_tuple(hash_index[2 * i], hash_index[2 * i + 1]);
    for (size_t c = 0; c < cells.size(); c++)
        cells[c] = std::make_tuple((int)cse[2 * c], (int)cse[2 * c + 1]);
    std::vector<double> sp(sorted, sorted + 4 * (size_t)n);
    mgr->getAcceleration(sp.data(), force, &phi, &cells, &st);
    return 0;
}

// The reference's own force call on a plugin it loads the way runSim.cpp:
// 35-61 does (dlopen + dlsym "getForce"), given by path: a plugin built
// outside the reference (a GB300 plugin) driven through the reference's
// config, IForce vtable and defaultForceManager::getAcceleration.  Returns
// 100 when the plugin does not load.
int psimref_foreign_forces(const char* plugin_path, const char* settings_path, int n, int box,
                           int cell_size, int scale, const double* sorted,
                           const int* hash_index, const uint32_t* cse, double* force,
                           int nthreads) {
    void* lib = dlopen(plugin_path, RTLD_NOW | RTLD_LOCAL);
    if (!lib) return 100;
    typedef PSim::IForce* factory_t(PSim::config*);
    factory_t* factory = (factory_t*)dlsym(lib, "getForce");
    if (!factory) return 100;
    PSim::config cfg{std::string(settings_path)};
    PSim::IForce* f = factory(&cfg);
    PSim::defaultForceManager* mgr = new PSim::defaultForceManager();
    mgr->addForce(f);
    set_threads(nthreads);
    PSim::systemState st = PSim::systemState();
    st.nParticles = n;
    st.boxSize = box;
    st.cellSize = cell_size;
    st.cellScale = scale;
    std::vector<std::tuple<int, int>> phi(n), cells((size_t)scale * scale * scale);
    for (int i = 0; i < n; i++) phi[i] = std::make_tuple(hash_index[2 * i], hash_index[2 * i + 1]);
    for (size_t c = 0; c < cells.size(); c++)
        cells[c] = std::make_tuple((int)cse[2 * c], (int)cse[2 * c + 1]);
    std::vector<double> sp(sorted, sorted + 4 * (size_t)n);
    mgr->getAcceleration(sp.data(), force, &phi, &cells, &st);
    return 0;
}

// The reference's analysis of an injected state: the cell list and
// system::updateInteractions (systemHandling.cpp:94-161) -> every particle's
// coordination number (coor, original order); analysisManager::findClusters
// (analysisCluster.cpp:26-83) -> the cluster of every particle in the order
// findClusters returns them (-1: in no cluster of more than 4); getTemperature,
// meanDisplacement (analysisGeneral.cpp:26-55) and the FP32 sum of
// particle::calculatePotential (analysisOutput.cpp:117-123) -> stats[0..2];
// writeSystem and writeSystemXYZ (analysisOutput.cpp:31-74) -> the files
// out_prefix.txt and out_prefix.xyz.
int psimref_analysis(int n, int box, int cell_size, int scale, const double* pos,
                     const double* pos0, const double* vel, const double* frc,
                     const double* frc0, const double* radius, const double* mass,
                     double current_time, int* coor, int* cluster_of, int* n_clusters,
                     double* stats, const char* out_prefix) {
    Geometry g{n, box, cell_size, scale};
    PSim::system* s = make_system(g, pos, pos0, vel, frc, frc0, radius, mass);
    s->hashParticles();
    s->sortParticles();
    s->clearCells();
    s->reorderParticles();
    s->updateInteractions();
    for (int i = 0; i < n; i++) coor[i] = s->particles[i]->getCoorNumber();
    PSim::analysisManager am(std::string("/tmp/psimref_trial"), &s->state);
    std::vector<std::vector<particle*>> clusters = am.findClusters(s->particles, n);
    for (int i = 0; i < n; i++) cluster_of[i] = -1;
    for (size_t c = 0; c < clusters.size(); c++)
        for (particle* p : clusters[c]) cluster_of[(int)p->getName()] = (int)c;
    *n_clusters = (int)clusters.size();
    float pot = 0;
    for (int i = 0; i < n; i++) pot += s->particles[i]->calculatePotential();
    stats[0] = am.getTemperature(s->particles, n);
    stats[1] = am.meanDisplacement(s->particles, n);
    stats[2] = pot / double(n);
    am.writeSystem(s->particles, n, std::string(out_prefix));
    am.writeSystemXYZ(s->particles, n, 1, current_time, std::string(out_prefix));
    return 0;
}

// vGB coefficients as the reference integrator's constructor computes them.
void psimref_vgb_coeffs(const char* settings_path, double* out) {
    PSim::config cfg{std::string(settings_path)};
    psimref::g_next_id = 0;
    PSim::brownianIntegrator integ(&cfg);
    double v[13] = {integ.y,    integ.coEff0, integ.coEff1, integ.coEff2, integ.coEff3,
                    integ.sig1, integ.sig2,   integ.corr,   integ.dev,    integ.goy2,
                    integ.goy3, integ.hn,     integ.gn};
    std::memcpy(out, v, sizeof v);
}

// The reference hot loop, system::run, for n_steps steps with injected noise
// noise[(step * n + i) * 6 + k].  Inputs are the particle state in original
// order; outputs overwrite it, plus the final cell list and the last force.
int psimref_run(const char* plugin, const char* settings_path, int n, int box, int cell_size,
                int scale, int n_steps, const double* noise, double* pos, double* pos0,
                double* vel, double* frc, double* frc0, const double* radius,
                const double* mass, int* hash_index, uint32_t* cse, double* sorted,
                double* last_force, int nthreads) {
    PSim::config cfg{std::string(settings_path)};
    PSim::IForce* f = make_force(plugin, &cfg);
    if (!f) return 100;
    PSim::defaultForceManager* mgr = new PSim::defaultForceManager();
    mgr->addForce(f);
    psimref::g_next_id = 0;
    PSim::brownianIntegrator* integ = new PSim::brownianIntegrator(&cfg);
    set_threads(nthreads);
    Geometry g{n, box, cell_size, scale};
    PSim::system* s = make_system(g, pos, pos0, vel, frc, frc0, radius, mass);
    s->integrator = integ;
    s->sysForces = mgr;
    s->state.dTime = cfg.getParam<double>("timeStep", 0.001);
    s->state.temp = cfg.getParam<double>("kT", 1.0);
    // the constructor's first cell list (system.cpp:101-103)
    s->hashParticles();
    s->sortParticles();
    s->reorderParticles();
    for (int t = 0; t < n_steps; t++) {
        psimref::g_noise = noise + (size_t)t * (size_t)n * 6;
        for (int i = 0; i < n; i++) integ->rndGens[i]->istack[0] = 0;
        // The body of system::run's loop (system.cpp:187-211) minus the
        // analysis-only updateInteractions sweep and the output calls.
        // system::run itself is not called: for an endTime below 1 its
        // progress bar (utilities.cpp:52-77) divides 0 by 0 and then prints
        // about 2^31 characters.
        s->sysForces->getAcceleration(s->sortedParticles, s->particleForce,
                                      &s->particleHashIndex, &s->cellStartEnd, &s->state);
        s->pushParticleForce();
        s->integrator->nextSystem(s->particles, &s->state);
        s->hashParticles();
        s->sortParticles();
        s->clearCells();
        s->reorderParticles();
        s->state.currentTime += s->state.dTime;
    }
    export_particles(s, pos, pos0, vel, frc, frc0);
    export_cells(s, hash_index, cse, sorted);
    if (last_force) std::memcpy(last_force, s->particleForce, sizeof(double) * 3 * (size_t)n);
    return 0;
}

}  // extern "C"
