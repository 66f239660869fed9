// The reference engine's shape over the GPU adapters.
//
// Engine<RNG, Real, Block, Size, batched_task> selects its stage policies through member typedefs
// (examples/QTLSim/engine_batched_task.hpp:84-103) and runs them in simulate() (:163-223) with the
// policies' own member signatures.  StageEngine below is written the same way: a template over a policy
// set, calling
//   FreeSpace::operator()(space*, Pool&), fixed_begin/fixed_end, free_size      (updateFixedAlleles, :303-345)
//   space::grow(N, A, T)                                                         (:192)
//   Selection::update(const Fitness&, unsigned)                                  (:195)
//   Crossover::operator()(const Selection&, space*, space*, AlleleSpace*, Pool&) (:198)
//   Mutation::generateNewMutation(unsigned), operator()(space*, AlleleSpace*, TraitSpace*, FreeSpace*,
//                                             unsigned, unsigned, Pool&, unsigned)  (:175, :202)
//   TraitSpace::isAllNeutral, Phenotype::operator()(space*, space*, TraitSpace*, Pool&),
//   Phenotype::constant_phenotype(space*, TraitSpace*)                           (:205-211)
//   Fitness::operator()(const Phenotype&)                                        (:213)
// It is instantiated with the GPU policy set (clotho_gb300/cpp/clotho_gb300.hpp) and a stand-in for the
// reference's thread_pool (include/clotho/data_spaces/task/thread_pool.hpp:31-139, which needs Boost).
//
// Run: G generations of StageEngine and of the fused engine (EngineGB300, one tape call a generation)
// from the same seed give bit-identical genomes, allele tables and free lists; phenotypes agree within
// the FP32 bound of a full re-sum against carried sums.  A second StageEngine draws its parents on the
// device (clotho_select) and must report pairs that index the parent population.  Prints "ok".
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "clotho_gb300/cpp/clotho_gb300.hpp"

using namespace clotho::gb300;

// thread_pool<RNG> with no workers: the master thread runs every task (T = 0, thread_count_parameter.hpp:22)
struct PoolStandIn {
    unsigned pool_size() const { return 0u; }
};

template <class RNG>
struct GpuPolicies {
    typedef RNG random_engine_type;
    typedef PopulationSpaceGPU sequence_space_type;
    typedef AlleleSpaceGPU allele_type;
    typedef TraitSpaceGPU trait_space_type;
    typedef FreeSpaceGPU free_space_type;
    typedef MutationGPU<RNG> mutation_type;
    typedef FitnessGPU fitness_type;
    typedef SelectionGPU<RNG> selection_type;
    typedef CrossoverGPU<RNG> crossover_type;
    typedef PhenotypeGPU phenotype_eval_type;
    typedef PoolStandIn thread_pool_type;
};

template <class P>
class StageEngine {
public:
    typedef typename P::random_engine_type random_engine_type;
    typedef typename P::sequence_space_type sequence_space_type;
    typedef typename P::allele_type allele_type;
    typedef typename P::trait_space_type trait_space_type;
    typedef typename P::free_space_type free_space_type;
    typedef typename P::mutation_type mutation_type;
    typedef typename P::fitness_type fitness_type;
    typedef typename P::selection_type selection_type;
    typedef typename P::crossover_type crossover_type;
    typedef typename P::phenotype_eval_type phenotype_eval_type;
    typedef typename P::thread_pool_type thread_pool_type;

    StageEngine(random_engine_type* rng, Context* pop, unsigned N, bool device_selection)
        : m_pop0(pop), m_pop1(pop), m_parent(&m_pop0), m_child(&m_pop1), m_allele_space(pop), m_trait_space(pop),
          select_gen(rng, device_selection), cross_gen(rng, pop->params().rho, pop->params().bias),
          mutate_gen(rng, pop->params(), pop), m_fit(pop), m_N(N), m_generation(1) {
        check(clotho_init(pop->get(), N), pop->get(), "clotho_init");
        m_fit.resize(N);
    }

    void simulate() {
        std::swap(m_child, m_parent);
        const unsigned pN = m_N;
        const unsigned pM = mutate_gen.generateNewMutation(2 * pN);
        const unsigned free_count = updateFixedAlleles(m_parent);
        const size_t all_size = child_max_alleles(m_allele_space.size(), free_count, pM);
        m_child->grow(pN, (unsigned)all_size, m_trait_space.trait_count());
        select_gen.update(m_fit, pN);
        cross_gen(select_gen, m_parent, m_child, &m_allele_space, m_thread_pool);
        mutate_gen(m_child, &m_allele_space, &m_trait_space, &m_free_space, pM, m_generation, m_thread_pool, 1);
        if (!m_trait_space.isAllNeutral()) {
            m_pheno(m_parent, m_child, &m_trait_space, m_thread_pool);
        } else {
            m_pheno.constant_phenotype(m_child, &m_trait_space);
        }
        m_fit(m_pheno);
        ++m_generation;
    }

    const selection_type& selection() const { return select_gen; }

private:
    unsigned updateFixedAlleles(sequence_space_type* ss) {
        m_free_space(ss, m_thread_pool);
        for (auto it = m_free_space.fixed_begin(); it != m_free_space.fixed_end(); ++it) ss->remove_fixed_allele(*it);
        return m_free_space.free_size();
    }
    static size_t child_max_alleles(size_t N_parent, size_t F_parent, size_t M_child) {
        return F_parent >= M_child ? N_parent : N_parent + (M_child - F_parent);
    }

    sequence_space_type m_pop0, m_pop1;
    sequence_space_type *m_parent, *m_child;
    allele_type m_allele_space;
    trait_space_type m_trait_space;
    free_space_type m_free_space;
    selection_type select_gen;
    crossover_type cross_gen;
    mutation_type mutate_gen;
    phenotype_eval_type m_pheno;
    fitness_type m_fit;
    thread_pool_type m_thread_pool;
    unsigned m_N, m_generation;
};

#define REQUIRE(c)                                                        \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::printf("failed: %s (line %d)\n", #c, __LINE__);          \
            return 1;                                                     \
        }                                                                 \
    } while (0)

template <class T>
static std::vector<T> read(clotho_ctx* c, int (*fn)(clotho_ctx*, T*), size_t n) {
    std::vector<T> v(n);
    if (n) check(fn(c, v.data()), c, "read-back");
    return v;
}

int main() {
    Parameters p;
    p.max_individuals = 400;
    p.max_alleles = 8192;
    p.traits = 2;
    p.mu = 0.2;
    p.rho = 1.5;
    p.p_neutral = 0.3;
    p.fitness = CLOTHO_FIT_GAUSSIAN_VS;
    p.fit_param = 4.0;
    p.seed = 11;
    const unsigned N = 400, G = 15;
    try {
        std::mt19937_64 rng_a(2024), rng_b(2024);
        Context staged_pop(p);
        StageEngine<GpuPolicies<std::mt19937_64>> staged(&rng_a, &staged_pop, N, false);
        EngineGB300<std::mt19937_64> fused(&rng_b, p);
        for (unsigned g = 0; g < G; ++g) {
            staged.simulate();
            fused.simulate(false);
        }
        clotho_info a = staged_pop.info(), b = fused.population().info();
        REQUIRE(a.device_error == 0 && b.device_error == 0);
        REQUIRE(a.generation == b.generation && a.N == b.N && a.A == b.A && a.W == b.W);
        REQUIRE(a.A > 100 && a.free_count == b.free_count && a.fixed_total == b.fixed_total);
        std::vector<uint64_t> ra((size_t)2 * a.N * a.W), rb(ra.size());
        check(clotho_get_rows(staged_pop.get(), ra.data(), ra.size()), staged_pop.get(), "rows");
        check(clotho_get_rows(fused.population().get(), rb.data(), rb.size()), fused.population().get(), "rows");
        REQUIRE(ra == rb);
        REQUIRE(read(staged_pop.get(), clotho_get_free, a.free_count) ==
                read(fused.population().get(), clotho_get_free, b.free_count));
        std::vector<double> pa(a.A), pb(b.A);
        std::vector<uint32_t> ga(a.A), gb(b.A);
        std::vector<float> ea((size_t)a.A * p.traits), eb(ea.size());
        check(clotho_get_alleles(staged_pop.get(), pa.data(), ga.data(), ea.data()), staged_pop.get(), "alleles");
        check(clotho_get_alleles(fused.population().get(), pb.data(), gb.data(), eb.data()),
              fused.population().get(), "alleles");
        REQUIRE(pa == pb && ga == gb && ea == eb);
        // staged: full re-sum of every genome; fused: carried sums -- both FP32 sums of the same effects
        std::vector<double> za = read(staged_pop.get(), clotho_get_phenotypes, (size_t)a.N * p.traits);
        std::vector<double> zb = read(fused.population().get(), clotho_get_phenotypes, (size_t)b.N * p.traits);
        double sumabs = 0.0;
        for (float e : ea) sumabs += std::fabs((double)e);
        for (size_t i = 0; i < za.size(); ++i) REQUIRE(std::fabs(za[i] - zb[i]) <= 1e-5 * (1.0 + sumabs));

        // device-drawn parents through the same stage sequence
        std::mt19937_64 rng_c(7);
        Context dev_pop(p);
        StageEngine<GpuPolicies<std::mt19937_64>> dev(&rng_c, &dev_pop, N, true);
        for (unsigned g = 0; g < 5; ++g) {
            dev.simulate();
            REQUIRE(dev.selection().individual_count() == N);
            for (const auto& pr : dev.selection().getMatePairs()) REQUIRE(pr.first < N && pr.second < N);
        }
        std::vector<uint32_t> pairs = read(dev_pop.get(), clotho_get_pairs, (size_t)2 * N);
        size_t k = 0;
        for (const auto& pr : dev.selection().getMatePairs()) REQUIRE(pairs[k++] == pr.first && pairs[k++] == pr.second);
        REQUIRE(dev_pop.info().device_error == 0 && dev_pop.info().generation == 6);
    } catch (const std::exception& e) {
        std::printf("failed: %s\n", e.what());
        return 1;
    }
    std::printf("ok\n");
    return 0;
}
