// qtlsim_gb300.cpp -- QTLSim-style driver (examples/QTLSim/qtlsim_main.cpp:89-192)
// over the C++ policy adapters: G generations of a population on the GPU,
// per-generation status on stdout, the reference's performance JSON at the end.
//
//   qtlsim_gb300 [N] [generations] [mu] [rho] [traits] [staged(0|1)] [seed]
#include <cstdio>
#include <cstdlib>
#include <random>

#include "clotho_gb300.hpp"

int main(int argc, char** argv) {
    clotho::gb300::Parameters p;
    p.max_individuals = argc > 1 ? (uint32_t)std::atoi(argv[1]) : 10000u;
    const unsigned G = argc > 2 ? (unsigned)std::atoi(argv[2]) : 100u;
    p.mu = argc > 3 ? std::atof(argv[3]) : 0.01;
    p.rho = argc > 4 ? std::atof(argv[4]) : 0.01;
    p.traits = argc > 5 ? (uint32_t)std::atoi(argv[5]) : 1u;
    const bool staged = argc > 6 && std::atoi(argv[6]) != 0;
    p.seed = argc > 7 ? (uint64_t)std::atoll(argv[7]) : 1u;
    p.max_alleles = 1u << 16;
    p.fitness = CLOTHO_FIT_GAUSSIAN;
    std::mt19937_64 rng(p.seed);
    try {
        clotho::gb300::EngineGB300<std::mt19937_64> engine(&rng, p);
        for (unsigned g = 0; g < G; ++g) {
            engine.simulate(staged);
            if ((g + 1) % 10 == 0 || g + 1 == G) {
                clotho_info i = engine.population().info();
                std::printf("{\"generation\":%u,\"N\":%u,\"alleles\":%u,\"free\":%u,\"fixed_total\":%u,"
                            "\"mean_fitness\":%.6g,\"device_error\":%u}\n",
                            i.generation - 1, i.N, i.A, i.free_count, i.fixed_total, i.mean_fitness,
                            i.device_error);
                if (i.device_error) return 2;
            }
        }
        std::printf("%s\n", engine.performance_json().c_str());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "qtlsim_gb300: %s\n", e.what());
        return 1;
    }
    return 0;
}
