// qtlsim_gb300.cpp -- QTLSim-style driver (examples/QTLSim/qtlsim_main.cpp:89-192)
// over the C++ policy adapters: G generations of a population on the GPU,
// per-generation status on stdout, the reference's performance JSON at the end.
//
//   qtlsim_gb300 [N] [generations] [mu] [rho] [traits] [staged(0|1)] [seed] [growth]
//
// growth: "linear:A:B" or "predefined:n0,n1,..." (the population_growth
// toolkit's models); N is then the capacity and the sizes follow the model.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <sstream>
#include <string>

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
        std::shared_ptr<clotho::gb300::PopulationGrowth> growth;
        if (argc > 8) {  // "name:v0:v1" or "name:v0,v1,..."
            std::string spec(argv[8]);
            const size_t c = spec.find(':');
            const std::string name = spec.substr(0, c);
            std::vector<double> vals;
            std::string rest = c == std::string::npos ? "" : spec.substr(c + 1);
            for (char& ch : rest)
                if (ch == ':' ) ch = ',';
            std::stringstream ss(rest);
            for (std::string tok; std::getline(ss, tok, ',');)
                if (!tok.empty()) vals.push_back(std::atof(tok.c_str()));
            clotho::gb300::GrowthToolkit::Params prm;
            if (name == "linear") {
                if (vals.size() > 0) prm["A"] = {vals[0]};
                if (vals.size() > 1) prm["B"] = {vals[1]};
            } else {
                prm["sizes"] = vals;
            }
            growth = clotho::gb300::GrowthToolkit::instance().get_tool(name, prm);
        }
        clotho::gb300::EngineGB300<std::mt19937_64> engine(&rng, p, growth);
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
