// plugin_host.cpp -- a C++ host of the reference's shape (runSim.cpp:29-79,
// system.cpp:28-65) on include/psim_gb300.hpp, for the tests.  Modes:
//   constants SETTINGS
//       prints nParticles boxSize cellSize cellScale concentration, as
//       PSim::systemConstants derives them from the settings file
//   cpu_forces SETTINGS PLUGIN_DIR N BOX CELL SCALE SORTED HASH CSE OUT
//       loads the plugin the settings name, checks it has a device entry,
//       and writes the force of every particle from the plugin's CPU
//       getAcceleration (the reference's per-particle entry) to OUT
//   system SETTINGS PLUGIN_DIR PRECISION POS OUT_FORCE OUT_POS END_TIME
//       builds PSim::system from the settings (box, grid, radius, mass, the
//       plugin's device entry), uploads POS, writes the force of that state
//       (psim_system_forces) and, after run(END_TIME), the positions
// Binary files hold raw doubles / int32 / uint32 in the reference layouts.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "psim_gb300.hpp"

template <class T>
static std::vector<T> read_file(const char* path) {
    std::ifstream in(path, std::ios::binary);
    std::vector<char> raw((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    std::vector<T> v(raw.size() / sizeof(T));
    std::memcpy(v.data(), raw.data(), v.size() * sizeof(T));
    return v;
}

template <class T>
static void write_file(const char* path, const std::vector<T>& v) {
    std::ofstream out(path, std::ios::binary);
    out.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::string mode = argv[1];
    PSim::config cfg(argv[2]);
    if (mode == "constants") {
        PSim::systemState st = PSim::systemConstants(&cfg);
        std::printf("%d %d %d %d %.17g\n", st.nParticles, st.boxSize, st.cellSize, st.cellScale,
                    st.concentration);
        return 0;
    }
    try {
        if (mode == "cpu_forces" && argc == 12) {
            PSim::IForce* f = PSim::loadForces(&cfg, argv[3]);
            if (!PSim::deviceForce(f)) return 3;
            PSim::systemState st;
            st.nParticles = std::atoi(argv[4]);
            st.boxSize = std::atoi(argv[5]);
            st.cellSize = std::atoi(argv[6]);
            st.cellScale = std::atoi(argv[7]);
            std::vector<double> sorted = read_file<double>(argv[8]);
            std::vector<int32_t> hi = read_file<int32_t>(argv[9]);
            std::vector<uint32_t> cse = read_file<uint32_t>(argv[10]);
            std::vector<std::tuple<int, int>> phi(st.nParticles), cells(cse.size() / 2);
            for (int i = 0; i < st.nParticles; ++i) phi[i] = std::make_tuple(hi[2 * i], hi[2 * i + 1]);
            for (size_t c = 0; c < cells.size(); ++c)
                cells[c] = std::make_tuple((int)cse[2 * c], (int)cse[2 * c + 1]);
            std::vector<double> force(3 * (size_t)st.nParticles, 0.0);
            for (int i = 0; i < st.nParticles; ++i)
                f->getAcceleration(i, sorted.data(), force.data(), &phi, &cells, &st);
            write_file(argv[11], force);
            std::printf("%s\n", f->getName().c_str());
            return 0;
        }
        if (mode == "system" && argc == 9) {
            PSim::IForce* f = PSim::loadForces(&cfg, argv[3]);
            PSim::system sys(&cfg, f, std::atoi(argv[4]));
            const int n = sys.state().nParticles;
            std::vector<double> pos = read_file<double>(argv[5]);
            if ((int)pos.size() != 3 * n) return 4;
            std::vector<double> vel(3 * (size_t)n, 0.0), force(3 * (size_t)n);
            sys.upload(pos.data(), vel.data());
            PSim::check(psim_system_forces(sys.handle(), force.data()));
            write_file(argv[6], force);
            sys.run(std::atof(argv[8]));
            sys.download(pos.data(), nullptr, nullptr, nullptr, nullptr);
            write_file(argv[7], pos);
            std::printf("%d %d %d %d\n", sys.state().boxSize, sys.state().cellSize,
                        sys.state().cellScale, n);
            return 0;
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 5;
    }
    return 2;
}
