// clotho_gb300.hpp -- C++ policy adapters over the C-ABI (include/clotho_gpu.h).
//
// Header-only mirror of the stage policies that
// Engine<RNG,Real,Block,Size,batched_task> selects through its member
// typedefs (examples/QTLSim/engine_batched_task.hpp:84-103).  Each adapter keeps
// the reference member names and argument meaning; the work runs in
// libclotho_gpu.so.  EngineGB300 restates Engine::simulate()
// (engine_batched_task.hpp:163-223): the host draws the generation's random
// numbers in the reference's order into an event tape and the device does the
// rest.  Errors throw clotho::gb300::Error (the reference asserts).
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/clotho_gpu.h"

namespace clotho {
namespace gb300 {

struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void check(int rc, clotho_ctx* ctx, const char* what) {
    if (rc != CLOTHO_OK)
        throw Error(std::string(what) + " failed (" + std::to_string(rc) + "): " + clotho_last_error(ctx));
}

// Simulation parameters with the reference's configuration keys.
struct Parameters {
    uint32_t max_individuals = 10000;  // population_growth predefined default (predefined_population_growth_generator.cpp:21)
    uint32_t max_alleles = 1u << 16;
    uint32_t traits = 1;               // traits.N (trait_count_parameter.hpp:23)
    double mu = 1e-4;                  // mutation.mu (mutation_rate_parameter.hpp:24)
    double rho = 1e-4;                 // recombination.rho (recombination_rate_parameter.hpp:24)
    double bias = 0.5;                 // recombination.sequence_bias.p (sequence_bias_parameter.hpp:23)
    double p_neutral = 0.5;            // neutral.p (neutral_parameter.hpp:35)
    double eff_mean = 0.0, eff_sigma = 1.0;  // traits.mean / traits.sigma
    int fitness = CLOTHO_FIT_GAUSSIAN;       // fitness.name
    double fit_param = 1.0;                  // fitness.params.scale (quadratic) or Vs
    bool q1 = true;                    // second gamete never recombines (reference behaviour)
    uint64_t seed = 1;
};

// The generation the engine is about to run.  Mutation::generateNewMutation(2N) is the first stage of the
// reference's sequence that knows the generation's size and new-mutation count
// (engine_batched_task.hpp:166-175): it records them here; the first stage that needs the device (the
// free-space analysis of the parent) begins the generation on the device with them, and the last stage
// (fitness, :213) ends it.  The reference swaps its parent and child spaces by pointer (:164); the device
// swaps its buffers when the generation begins.
struct StepState {
    bool pending = false, begun = false;
    uint32_t N = 0, M = 0;
};

// Owns one resident population (clotho_ctx).
class Context {
public:
    explicit Context(const Parameters& p) : p_(p) {
        clotho_desc d{};
        d.max_individuals = p.max_individuals;
        d.max_alleles = p.max_alleles;
        d.traits = p.traits;
        const double S = 2.0 * p.max_individuals;
        d.max_events = (uint32_t)(S * p.rho + 10.0 * std::sqrt(S * p.rho + 1.0) + 64);
        d.max_mutations = (uint32_t)(S * p.mu + 10.0 * std::sqrt(S * p.mu + 1.0) + 64);
        d.max_fixed = std::max<uint32_t>(1024, p.max_alleles);
        d.fitness = p.fitness;
        d.flags = p.q1 ? CLOTHO_FLAG_Q1 : 0u;
        d.fit_param = p.fit_param;
        d.mu = p.mu;
        d.rho = p.rho;
        d.bias = p.bias;
        d.p_neutral = p.p_neutral;
        d.eff_mean = p.eff_mean;
        d.eff_sigma = p.eff_sigma;
        d.seed = p.seed;
        if (clotho_create(&d, &ctx_) != CLOTHO_OK) throw Error("clotho_create failed");
    }
    ~Context() {
        if (ctx_) clotho_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    clotho_ctx* get() const { return ctx_; }
    const Parameters& params() const { return p_; }
    clotho_info info() const {
        clotho_info i{};
        check(clotho_get_info(ctx_, &i), ctx_, "clotho_get_info");
        return i;
    }
    StepState& step() { return step_; }

private:
    Parameters p_;
    clotho_ctx* ctx_ = nullptr;
    StepState step_;
};

// ---- The spaces.  The reference passes its population, allele and trait spaces to every policy by raw
// pointer (population_space_row, AlleleSpace, trait_space_vector: engine_batched_task.hpp:84-95).  Here
// they live on the device, inside one Context; these types are the host-side views the policies take, with
// the reference's member names.  Host copies are read back on demand and dropped when the device state
// changes.

inline void begin_pending(Context* c) {
    StepState& st = c->step();
    if (st.begun) return;
    if (!st.pending) throw Error("no generation pending: Mutation::generateNewMutation comes first");
    check(clotho_begin_generation(c->get(), st.N, st.M), c->get(), "clotho_begin_generation");
    st.begun = true;
    st.pending = false;
}
inline void end_begun(Context* c) {
    StepState& st = c->step();
    if (!st.begun) return;
    check(clotho_end_generation(c->get()), c->get(), "clotho_end_generation");
    st.begun = false;
}

// population_space_row<uint64_t, double> (population_space_row_block.hpp:25-260): row i is haploid genome
// i, individual j owns rows 2j and 2j+1.  Two views (the parent and child roles the engine swaps by
// pointer) share one Context; between generations both read the rows of the last generation.
class PopulationSpaceGPU {
public:
    typedef uint64_t block_type;
    typedef double weight_type;
    typedef const block_type* genome_iterator;

    explicit PopulationSpaceGPU(Context* ctx) : ctx_(ctx) {}

    Context* context() const { return ctx_; }

    // grow(I, A, T) (:64-72): the device sizes the child itself (the same child_max_alleles rule,
    // :287-301, is applied on the device); this checks that the sizes fit the context's capacities.
    void grow(unsigned I, unsigned A, unsigned T) {
        const Parameters& p = ctx_->params();
        if (I > p.max_individuals || A > p.max_alleles || T != p.traits)
            throw Error("grow: the population exceeds the context's capacities");
    }
    // remove_fixed_allele (:127-147): the free-space analysis clears fixed columns on the device (the
    // generation kernel masks them out of every parent word), so nothing is left to do here.
    void remove_fixed_allele(unsigned /*index*/) {}

    unsigned getMaxBlocks() const { return ctx_->info().W; }                       // :94-101
    unsigned getMaxAlleles() const { return ctx_->info().A; }
    unsigned haploid_genome_count() const { return 2 * ctx_->info().N; }
    unsigned getIndividualCount() const { return ctx_->info().N; }
    unsigned getTraitCount() const { return ctx_->params().traits; }

    // begin_genome / end_genome (:176-188): the words of row i, from a host copy of the current rows
    genome_iterator begin_genome(unsigned i) { return rows().data() + (size_t)i * width_; }
    genome_iterator end_genome(unsigned i) { return begin_genome(i) + width_; }
    void invalidate() { rows_.clear(); }

private:
    const std::vector<block_type>& rows() {
        if (rows_.empty()) {
            const clotho_info i = ctx_->info();
            width_ = i.W;
            rows_.assign((size_t)2 * i.N * i.W, 0);
            if (!rows_.empty())
                check(clotho_get_rows(ctx_->get(), rows_.data(), rows_.size()), ctx_->get(), "clotho_get_rows");
        }
        return rows_;
    }
    Context* ctx_;
    std::vector<block_type> rows_;
    unsigned width_ = 0;
};

// AlleleSpace<double, unsigned> (allele_space_vector.hpp:31-227): positions and ages by slot.
class AlleleSpaceGPU {
public:
    typedef double position_type;
    explicit AlleleSpaceGPU(Context* ctx) : ctx_(ctx) {}
    size_t size() const { return ctx_->info().A; }
    // grow (:115-137): slots appended by a mutation are added by the device
    void grow() {}
    position_type getPositionAt(size_t i) {
        load();
        return pos_.at(i);
    }
    unsigned getAgeAt(size_t i) {
        load();
        return age_.at(i);
    }
    void invalidate() { pos_.clear(); }

private:
    void load() {
        if (!pos_.empty()) return;
        const unsigned A = ctx_->info().A, T = ctx_->params().traits;
        pos_.assign(A, 0.0);
        age_.assign(A, 0);
        std::vector<float> eff((size_t)A * T);
        if (A) check(clotho_get_alleles(ctx_->get(), pos_.data(), age_.data(), eff.data()), ctx_->get(),
                     "clotho_get_alleles");
    }
    Context* ctx_;
    std::vector<double> pos_;
    std::vector<uint32_t> age_;
};

// trait_space_vector<double> (trait_space_vector.hpp:26-198): T effects per slot.
class TraitSpaceGPU {
public:
    typedef float weight_type;
    typedef std::vector<float>::const_iterator iterator;
    explicit TraitSpaceGPU(Context* ctx) : ctx_(ctx) {}
    unsigned trait_count() const { return ctx_->params().traits; }
    size_t size() const { return ctx_->info().A; }
    void grow() {}  // the device writes the effects of appended slots
    // isAllNeutral: every effect zero (the engine then takes the constant phenotype, :205-211)
    bool isAllNeutral() {
        load();
        return std::all_of(w_.begin(), w_.end(), [](float x) { return x == 0.0f; });
    }
    iterator begin(size_t slot) {
        load();
        return w_.begin() + slot * trait_count();
    }
    iterator end(size_t slot) { return begin(slot) + trait_count(); }
    void invalidate() { loaded_ = false; }

private:
    void load() {
        if (loaded_) return;
        const unsigned A = ctx_->info().A, T = trait_count();
        std::vector<double> pos(A);
        std::vector<uint32_t> age(A);
        w_.assign((size_t)A * T, 0.0f);
        if (A) check(clotho_get_alleles(ctx_->get(), pos.data(), age.data(), w_.data()), ctx_->get(),
                     "clotho_get_alleles");
        loaded_ = true;
    }
    Context* ctx_;
    std::vector<float> w_;
    bool loaded_ = false;
};

// ---- FreeSpaceAnalyzerMT<population_space_row> (free_space_mt_population_space_row_interlaced.hpp:41-89)
// with the free_space_details accessors (free_space_details.hpp:193-277).  The analysis of the parent,
// the removal of its fixed alleles and the fixed-allele table (Engine::updateFixedAlleles,
// engine_batched_task.hpp:303-345) run on the device in one call.
class FreeSpaceGPU {
public:
    typedef uint32_t size_type;
    typedef std::vector<size_type>::const_iterator iterator;

    template <class PoolType>
    void operator()(PopulationSpaceGPU* ss, PoolType&) {
        begin_pending(ss->context());
        uint32_t c[3];
        check(clotho_free_space(ss->context()->get(), c), ss->context()->get(), "clotho_free_space");
        fixed_ = c[0];
        lost_ = c[1];
        idx_.assign(c[2], 0);
        if (c[2]) check(clotho_get_free(ss->context()->get(), idx_.data()), ss->context()->get(), "clotho_get_free");
        width_ = ss->context()->info().A;
    }
    // the same analysis through a bare Context (the fused engine's bookkeeping)
    template <class PoolType>
    void operator()(Context* ss, PoolType&) {
        uint32_t c[3];
        check(clotho_free_space(ss->get(), c), ss->get(), "clotho_free_space");
        fixed_ = c[0];
        lost_ = c[1];
        idx_.assign(c[2], 0);
        if (c[2]) check(clotho_get_free(ss->get(), idx_.data()), ss->get(), "clotho_get_free");
        width_ = ss->info().A;
    }
    size_type fixed_size() const { return fixed_; }
    size_type lost_size() const { return lost_; }
    size_type free_size() const { return fixed_ + lost_; }
    size_type variable_count() const { return width_ - free_size(); }
    iterator free_begin() const { return idx_.begin(); }
    iterator free_end() const { return idx_.end(); }
    iterator fixed_begin() const { return idx_.begin(); }
    iterator fixed_end() const { return idx_.begin() + fixed_; }
    iterator lost_begin() const { return idx_.begin() + fixed_; }
    iterator lost_end() const { return idx_.end(); }

private:
    std::vector<size_type> idx_;
    size_type fixed_ = 0, lost_ = 0, width_ = 0;
};

class PhenotypeGPU;

// ---- GeneralFitness (general_fitness.hpp:101-276): one fitness value per individual, the toolkit metric
// applied on the device; begin()/end() iterate a host copy.
class FitnessGPU {
public:
    typedef double fitness_type;
    typedef std::vector<double>::const_iterator const_iterator;

    FitnessGPU() = default;
    explicit FitnessGPU(Context* ctx) : ctx_(ctx) {}
    void bind(Context* ctx) { ctx_ = ctx; }
    Context* context() const { return ctx_; }

    // GeneralFitness::operator()(phenos) (:101-119)
    inline void operator()(const PhenotypeGPU& phenos);
    void operator()(Context* pop) {
        check(clotho_fitness(pop->get()), pop->get(), "clotho_fitness");
        load(pop);
    }
    // resize(N) (:238-243): new entries are 1.0
    void resize(unsigned N) {
        while (f_.size() < N) f_.push_back(1.0);
    }
    unsigned individual_count() const { return (unsigned)f_.size(); }
    unsigned size() const { return (unsigned)f_.size(); }
    const_iterator begin() const { return f_.begin(); }
    const_iterator end() const { return f_.end(); }
    const std::vector<double>& values() const { return f_; }
    std::vector<double> values(Context* pop) const {  // the current population's fitness, read back
        clotho_info i = pop->info();
        std::vector<double> f(i.N);
        if (i.N) check(clotho_get_fitness(pop->get(), f.data()), pop->get(), "clotho_get_fitness");
        return f;
    }
    void load(Context* pop) { f_ = values(pop); }

private:
    Context* ctx_ = nullptr;
    std::vector<double> f_;
};

// ---- SelectionGenerator<RNG, fitness_selection<GeneralFitness>>
// (general_fitness_selection_generator.hpp:45-113): N (id0,id1) pairs, uniform when every fitness is equal,
// else fitness-proportional.  Host draws (the default) follow the reference with the caller's RNG; with
// device draws the pairs come from the device's FP64 prefix sum of fitness and Philox uniforms
// (clotho_select), which needs the generation begun on the device.
template <class RNG>
class SelectionGPU {
public:
    typedef std::vector<std::pair<uint32_t, uint32_t>> mate_pair_vector;

    explicit SelectionGPU(RNG* rng, bool device_draws = false) : rng_(rng), device_(device_draws) {}

    void update(const FitnessGPU& fit, unsigned N) {
        if (device_ && fit.context()) {
            std::vector<uint32_t> ids(2 * (size_t)N);
            check(clotho_select(fit.context()->get(), ids.data()), fit.context()->get(), "clotho_select");
            pairs_.clear();
            for (unsigned k = 0; k < N; ++k) pairs_.emplace_back(ids[2 * k], ids[2 * k + 1]);
            return;
        }
        update(fit.values(), N);
    }
    void update(const std::vector<double>& fit, unsigned N) {
        pairs_.clear();
        const size_t M = fit.size();
        bool constant = true;
        for (size_t i = 1; i < M && constant; ++i) constant = fit[i] == fit[0];
        if (constant) {
            std::uniform_int_distribution<uint32_t> uni(0, M ? (uint32_t)(M - 1) : 0u);
            while (pairs_.size() < N) {
                uint32_t a = uni(*rng_), b = uni(*rng_);
                pairs_.emplace_back(a, b);
            }
        } else {
            std::discrete_distribution<uint32_t> disc(fit.begin(), fit.end());
            while (pairs_.size() < N) {
                uint32_t a = disc(*rng_), b = disc(*rng_);
                pairs_.emplace_back(a, b);
            }
        }
    }
    bool device_draws() const { return device_; }
    const mate_pair_vector& getMatePairs() const { return pairs_; }
    unsigned individual_count() const { return (unsigned)pairs_.size(); }

private:
    RNG* rng_;
    bool device_;
    mate_pair_vector pairs_;
};

// ---- BatchCrossoverMTWE (batch_crossover_mtwe.hpp:51-145): the event pool, lookup and bias pool are drawn
// on the host in the reference's order; the splice runs on the device.
template <class RNG>
class CrossoverGPU {
public:
    CrossoverGPU(RNG* rng, double rho, double bias) : rng_(rng), rho_(rho), bias_(bias) {}

    // operator()(parents, parental, offspring, alleles, pool) (:51-55)
    template <class Selection, class PoolType>
    void operator()(const Selection& parents, PopulationSpaceGPU* /*parental*/, PopulationSpaceGPU* offspring,
                    AlleleSpaceGPU* /*alleles*/, PoolType& pool) {
        (*this)(parents, (Context*)nullptr, offspring->context(), pool);
        offspring->invalidate();
    }
    template <class Selection, class PoolType>
    void operator()(const Selection& parents, Context* /*parental*/, Context* offspring, PoolType&) {
        const size_t S = 2 * parents.individual_count();
        draw(S);
        std::vector<uint32_t> pairs;
        pairs.reserve(S);
        for (const auto& pr : parents.getMatePairs()) {
            pairs.push_back(pr.first);
            pairs.push_back(pr.second);
        }
        check(clotho_set_pairs(offspring->get(), pairs.data()), offspring->get(), "clotho_set_pairs");
        check(clotho_crossover(offspring->get(), swap_.data(), lookup_.data(), events_.data()), offspring->get(),
              "clotho_crossover");
    }
    // fill_event_pool / fill_bias_pool (:117-145)
    void draw(size_t gametes) {
        std::poisson_distribution<uint32_t> n_events(rho_);
        std::uniform_real_distribution<double> pos(0.0, 1.0);
        std::bernoulli_distribution b(bias_);
        lookup_.clear();
        events_.clear();
        for (size_t g = 0; g < gametes; ++g) {
            lookup_.push_back((uint32_t)events_.size());
            uint32_t n = rho_ > 0 ? n_events(*rng_) : 0u;
            while (n--) events_.push_back(pos(*rng_));
        }
        lookup_.push_back((uint32_t)events_.size());
        swap_.resize(gametes);
        for (size_t g = 0; g < gametes; ++g) swap_[g] = b(*rng_) ? 1 : 0;
    }
    const std::vector<uint32_t>& lookup() const { return lookup_; }
    const std::vector<double>& events() const { return events_; }
    const std::vector<uint8_t>& bias() const { return swap_; }

private:
    RNG* rng_;
    double rho_, bias_;
    std::vector<uint32_t> lookup_;
    std::vector<double> events_;
    std::vector<uint8_t> swap_;
};

// ---- BatchMutationMT (batch_mutation_mt.hpp:57-81) with the allele and trait generators: per mutation the
// target row, the position, then per trait the neutral draw and the Normal effect.  The free list, slot reuse
// and appended slots (:69-80) are applied on the device from its own analysis.
template <class RNG>
class MutationGPU {
public:
    // pop: the population whose coming generation generateNewMutation announces (may be null)
    MutationGPU(RNG* rng, const Parameters& p, Context* pop = nullptr) : rng_(rng), p_(p), pop_(pop) {}

    // generateNewMutation (:57-59, mutation_allocator.hpp:41-47); also records the coming generation
    uint32_t generateNewMutation(unsigned N_hap) {
        std::poisson_distribution<uint32_t> d(p_.mu * N_hap);
        const uint32_t M = p_.mu > 0 ? d(*rng_) : 0u;
        if (pop_) {
            StepState& st = pop_->step();
            if (st.begun) throw Error("a generation is still open on the device");
            st.pending = true;
            st.N = N_hap / 2;
            st.M = M;
        }
        return M;
    }

    // operator()(pop, alleles, traits, free_space, N, age, pool[, TC]) (:61-81)
    template <class PoolType>
    void operator()(PopulationSpaceGPU* pop, AlleleSpaceGPU* alleles, TraitSpaceGPU* traits, FreeSpaceGPU* free_space,
                    unsigned M, unsigned age, PoolType& pool, unsigned TC = 1) {
        (void)free_space;
        (void)TC;  // the reference forces one mutation task (engine_batched_task.hpp:202)
        const clotho_info i = pop->context()->info();
        if (age != i.generation) throw Error("mutation age differs from the device's generation");
        (*this)(pop->context(), M, 2 * i.N, pool);
        pop->invalidate();
        alleles->invalidate();
        traits->invalidate();
    }
    template <class PoolType>
    void operator()(Context* pop, unsigned M, unsigned S, PoolType&) {
        std::uniform_int_distribution<uint32_t> seq(0, S ? S - 1 : 0);
        std::uniform_real_distribution<double> pos(0.0, 1.0);
        std::bernoulli_distribution neutral(p_.p_neutral);
        std::normal_distribution<double> w(p_.eff_mean, p_.eff_sigma);
        seq_.resize(M);
        pos_.resize(M);
        eff_.assign((size_t)M * p_.traits, 0.0f);
        for (unsigned i = 0; i < M; ++i) {
            seq_[i] = seq(*rng_);
            pos_[i] = pos(*rng_);
            for (unsigned t = 0; t < p_.traits; ++t)
                if (!neutral(*rng_)) eff_[(size_t)i * p_.traits + t] = (float)w(*rng_);
        }
        check(clotho_mutate(pop->get(), seq_.data(), pos_.data(), eff_.data()), pop->get(), "clotho_mutate");
    }

private:
    RNG* rng_;
    Parameters p_;
    Context* pop_;
    std::vector<uint32_t> seq_;
    std::vector<double> pos_;
    std::vector<float> eff_;
};

// ---- BatchPhenotypeMT<population_space_row> (batch_phenotype_mt_population_space_row.hpp:48-104).  The
// per-individual phenotype is a T-vector (individual_count() is N; the reference's returns T*N, which makes
// its multi-trait fitness abort: a quirk not followed).
class PhenotypeGPU {
public:
    typedef std::vector<double>::const_iterator phenotype_iterator;

    // operator()(parent, child, traits, pool) (:62-72)
    template <class PoolType>
    void operator()(PopulationSpaceGPU* /*parent*/, PopulationSpaceGPU* pop, TraitSpaceGPU* traits, PoolType&) {
        ctx_ = pop->context();
        trait_count_ = traits->trait_count();
        check(clotho_phenotype(ctx_->get()), ctx_->get(), "clotho_phenotype");
        z_.clear();
    }
    template <class PoolType>
    void operator()(Context* /*parent*/, Context* pop, PoolType&) {
        ctx_ = pop;
        trait_count_ = pop->params().traits;
        check(clotho_phenotype(pop->get()), pop->get(), "clotho_phenotype");
        z_.clear();
    }
    // constant_phenotype(pop, traits) (:48-59): every effect is zero, so the device's fitness stage sees
    // the constant phenotype 1.0 (engine_batched_task.hpp:207-211)
    void constant_phenotype(PopulationSpaceGPU* pop, TraitSpaceGPU* traits) {
        ctx_ = pop->context();
        trait_count_ = traits->trait_count();
        check(clotho_phenotype(ctx_->get()), ctx_->get(), "clotho_phenotype");
        z_.clear();
    }
    Context* context() const { return ctx_; }
    unsigned individual_count() const { return ctx_ ? ctx_->info().N : 0u; }
    unsigned trait_count() const { return trait_count_; }
    // begin/end_individual_phenotype(i) (:86-92): individual i's T values, from a host copy read after the
    // fitness stage (the device fills the per-individual values there)
    phenotype_iterator begin_individual_phenotype(unsigned i) { return values().begin() + (size_t)i * trait_count_; }
    phenotype_iterator end_individual_phenotype(unsigned i) { return begin_individual_phenotype(i) + trait_count_; }
    const std::vector<double>& values() {
        if (z_.empty() && ctx_) z_ = phenotypes(ctx_);
        return z_;
    }
    std::vector<double> phenotypes(Context* pop) const {
        clotho_info i = pop->info();
        std::vector<double> z((size_t)i.N * pop->params().traits);
        if (!z.empty()) check(clotho_get_phenotypes(pop->get(), z.data()), pop->get(), "clotho_get_phenotypes");
        return z;
    }
    void invalidate() { z_.clear(); }

private:
    Context* ctx_ = nullptr;
    unsigned trait_count_ = 0;
    std::vector<double> z_;
};

// the last stage of the reference's sequence (:213): also ends a generation begun on the device
inline void FitnessGPU::operator()(const PhenotypeGPU& phenos) {
    Context* c = phenos.context() ? phenos.context() : ctx_;
    if (!c) throw Error("fitness: no population");
    ctx_ = c;
    check(clotho_fitness(c->get()), c->get(), "clotho_fitness");
    end_begun(c);
    load(c);
}

// ---- population growth: the reference's runtime plugins and their registry
// (population_growth_toolkit.hpp:27-53).  A model maps (current N, generation)
// to the next N; the engine asks once at set-up with (0, 0) and before every
// generation with (previous N, generation) (engine_batched_task.hpp:143-170).
struct PopulationGrowth {
    virtual ~PopulationGrowth() = default;
    virtual unsigned operator()(unsigned N, unsigned generation) const = 0;
    virtual std::string name() const = 0;
};

// N' = (unsigned)(A N + B) (linear_population_growth.cpp:23-25); A = 1, B = 0 by default
struct LinearGrowth : PopulationGrowth {
    double A = 1.0, B = 0.0;
    LinearGrowth(double a = 1.0, double b = 0.0) : A(a), B(b) {}
    unsigned operator()(unsigned N, unsigned) const override {
        const double v = A * N + B;
        return v > 0.0 ? (unsigned)v : 0u;
    }
    std::string name() const override { return "linear"; }
};

// N' = sizes[g % size] (predefined_population_growth.cpp:26-28); default {10000}
struct PredefinedGrowth : PopulationGrowth {
    std::vector<unsigned> sizes;
    explicit PredefinedGrowth(std::vector<unsigned> s = {10000u}) : sizes(s.empty() ? std::vector<unsigned>{10000u} : s) {}
    unsigned operator()(unsigned, unsigned generation) const override { return sizes[generation % sizes.size()]; }
    std::string name() const override { return "predefined"; }
};

// String-keyed registry: name -> factory taking numeric parameters
// ("A", "B" for linear; "sizes" for predefined).
class GrowthToolkit {
public:
    using Params = std::map<std::string, std::vector<double>>;
    using Factory = std::function<std::shared_ptr<PopulationGrowth>(const Params&)>;

    static GrowthToolkit& instance() {
        static GrowthToolkit tk;
        return tk;
    }
    void register_tool(const std::string& name, Factory f) { tools_[name] = std::move(f); }
    std::shared_ptr<PopulationGrowth> get_tool(const std::string& name, const Params& p = {}) const {
        auto it = tools_.find(name);
        if (it == tools_.end()) throw Error("unknown population growth model: " + name);
        return it->second(p);
    }

private:
    GrowthToolkit() {
        auto first = [](const Params& p, const char* k, double d) {
            auto it = p.find(k);
            return (it == p.end() || it->second.empty()) ? d : it->second[0];
        };
        register_tool("linear", [first](const Params& p) {
            return std::make_shared<LinearGrowth>(first(p, "A", 1.0), first(p, "B", 0.0));
        });
        register_tool("predefined", [](const Params& p) {
            std::vector<unsigned> s;
            auto it = p.find("sizes");
            if (it != p.end())
                for (double v : it->second) s.push_back((unsigned)v);
            return std::make_shared<PredefinedGrowth>(s);
        });
    }
    std::map<std::string, Factory> tools_;
};

// ---- QTLSim configuration trees (boost::property_tree::ptree, or any tree with get<T>(path, default),
// get_child_optional(path), get_child(path), iteration over (key, child) pairs and data()): the keys
// QTLSim reads, from its "configuration" block or the root (qtlsim_main.cpp:111-113), with the
// defaults of the reference's parameter objects.  The allele and individual capacities have no key.
template <class Tree>
const Tree& configuration_block(const Tree& config) {
    auto b = config.get_child_optional("configuration");
    return b ? config.get_child("configuration") : config;
}

template <class Tree>
Parameters params_from(const Tree& config, uint32_t max_individuals, uint32_t max_alleles) {
    const Tree& c = configuration_block(config);
    Parameters p;
    p.max_individuals = max_individuals;
    p.max_alleles = max_alleles;
    p.mu = c.template get<double>("mutation.mu", 1e-4);                       // mutation_rate_parameter.hpp:24-39
    p.rho = c.template get<double>("recombination.rho", 1e-4);                // recombination_rate_parameter.hpp:24-39
    p.bias = c.template get<double>("recombination.sequence_bias.p", 0.5);    // sequence_bias_parameter.hpp:23-42
    p.traits = c.template get<uint32_t>("traits.N", 1u);                      // trait_count_parameter.hpp:23-38
    p.eff_mean = c.template get<double>("traits.mean", 0.0);                  // normal_distribution_parameter.hpp:23-41
    p.eff_sigma = c.template get<double>("traits.sigma", 1.0);
    p.p_neutral = c.template get<double>("neutral.p", 0.5);                   // neutral_parameter.hpp:35-50
    const std::string f = c.template get<std::string>("fitness.name", "");    // fitness_toolkit.cpp:50-69
    if (f.empty() || f == "constant") p.fitness = CLOTHO_FIT_CONSTANT;
    else if (f == "gaussian") p.fitness = CLOTHO_FIT_GAUSSIAN;
    else if (f == "quadratic") p.fitness = CLOTHO_FIT_QUADRATIC;
    else throw Error("unknown fitness metric: " + f);
    p.fit_param = p.fitness == CLOTHO_FIT_QUADRATIC ? c.template get<double>("fitness.params.scale", 1.0) : 1.0;
    p.seed = c.template get<uint64_t>("random_number.seed", 0u);              // seed_parameter.hpp:25-46
    if (p.traits < 1 || p.traits > 4) throw Error("traits.N must be 1..4");
    return p;
}

// population_growth.{name, params} (population_growth_toolkit.cpp:36-58): null without a model.
template <class Tree>
std::shared_ptr<PopulationGrowth> growth_from(const Tree& config) {
    const Tree& c = configuration_block(config);
    const std::string name = c.template get<std::string>("population_growth.name", "");
    if (name.empty()) return nullptr;
    GrowthToolkit::Params prm;
    if (c.get_child_optional("population_growth.params")) {
        for (const auto& kv : c.get_child("population_growth.params")) {
            std::vector<double>& v = prm[kv.first];
            if (!kv.second.data().empty()) v.push_back(std::stod(kv.second.data()));
            for (const auto& item : kv.second) v.push_back(std::stod(item.second.data()));  // lists ("sizes")
        }
    }
    return GrowthToolkit::instance().get_tool(name, prm);
}

// generations.size (examples/generation_parameter.cpp:17-33)
template <class Tree>
unsigned generations_from(const Tree& config) {
    return configuration_block(config).template get<unsigned>("generations.size", 10000u);
}

// ---- Engine<...> restated on the device (engine_batched_task.hpp:110-223).
// staged = true drives the policies one by one with the reference's member signatures; false uses the
// fused call with the same host draws (same RNG, same order), so both give the same genomes.
template <class RNG = std::mt19937_64>
class EngineGB300 {
public:
    typedef PopulationSpaceGPU sequence_space_type;
    typedef AlleleSpaceGPU allele_type;
    typedef TraitSpaceGPU trait_space_type;
    typedef FreeSpaceGPU free_space_type;
    typedef SelectionGPU<RNG> selection_type;
    typedef CrossoverGPU<RNG> crossover_type;
    typedef MutationGPU<RNG> mutation_type;
    typedef PhenotypeGPU phenotype_eval_type;
    typedef FitnessGPU fitness_type;

    EngineGB300(RNG* rng, const Parameters& p, std::shared_ptr<PopulationGrowth> growth = nullptr,
                bool device_selection = false)
        : rng_(rng), pop_(p), pop0_(&pop_), pop1_(&pop_), parent_(&pop0_), child_(&pop1_), alleles_(&pop_),
          traits_(&pop_), sel_(rng, device_selection), xover_(rng, p.rho, p.bias), mut_(rng, p, &pop_),
          N_(p.max_individuals), growth_(std::move(growth)) {
        // Engine::init (:143-161): the initial size is growth(0, 0) with a growth model
        if (growth_) N_ = (*growth_)(0u, 0u);
        if (N_ > p.max_individuals) throw Error("growth: initial size exceeds max_individuals");
        fit_.bind(&pop_);
        fit_.resize(N_);  // GeneralFitness::resize fills 1.0 (general_fitness.hpp:238-243)
        check(clotho_init(pop_.get(), N_), pop_.get(), "clotho_init");
    }

    void simulate(bool staged = false) {
        const auto t0 = std::chrono::steady_clock::now();
        if (staged) {
            simulate_staged();
        } else {
            simulate_fused();
        }
        const auto t1 = std::chrono::steady_clock::now();
        sim_times_.push_back(std::chrono::duration<double>(t1 - t0).count());
        clotho_info i = pop_.info();
        free_sizes_.push_back(i.free_count);
        var_sizes_.push_back(i.variable_count);
        fixed_sizes_.push_back(i.fixed_count);
    }

    Context& population() { return pop_; }
    sequence_space_type* getChildPopulation() const { return child_; }
    sequence_space_type* getParentPopulation() const { return parent_; }
    const fitness_type& fitness() const { return fit_; }

    // getPerformanceResults (engine_batched_task.hpp:233-242) as JSON
    std::string performance_json() const {
        auto arr = [](const auto& v) {
            std::string s = "[";
            for (size_t k = 0; k < v.size(); ++k) s += (k ? "," : "") + std::to_string(v[k]);
            return s + "]";
        };
        return std::string("{\"performance\":{\"simulate\":") + arr(sim_times_) + "},\"memory\":{\"free_count\":" +
               arr(free_sizes_) + ",\"variable_count\":" + arr(var_sizes_) + ",\"fixed_count\":" +
               arr(fixed_sizes_) + "}}";
    }

private:
    struct Pool {
        unsigned pool_size() const { return 0u; }  // the master thread alone (thread_count_parameter.hpp:22)
    };

    // the size of the coming generation (engine_batched_task.hpp:167-170)
    unsigned next_size() {
        unsigned pN = N_;
        if (growth_) {
            pN = (*growth_)(N_, pop_.info().generation);
            if (pN > pop_.params().max_individuals) throw Error("growth: size exceeds max_individuals");
        }
        return pN;
    }

    // Engine::simulate (engine_batched_task.hpp:163-223), stage by stage
    void simulate_staged() {
        std::swap(child_, parent_);                                   // :164
        const unsigned pN = next_size();                              // :166-170
        const uint32_t pM = mut_.generateNewMutation(2 * pN);         // :175
        const uint32_t free_count = updateFixedAlleles(parent_);      // :178
        const size_t all_size = child_max_alleles(alleles_.size(), free_count, pM);  // :182
        child_->grow(pN, (unsigned)all_size, traits_.trait_count());  // :192
        sel_.update(fit_, pN);                                        // :195
        xover_(sel_, parent_, child_, &alleles_, pool_);              // :198
        mut_(child_, &alleles_, &traits_, &free_, pM, pop_.info().generation, pool_, 1);  // :202
        if (!traits_.isAllNeutral()) {                                // :205-211
            pheno_(parent_, child_, &traits_, pool_);
        } else {
            pheno_.constant_phenotype(child_, &traits_);
        }
        fit_(pheno_);                                                 // :213 (ends the device generation)
        parent_->invalidate();
        child_->invalidate();
        N_ = pN;
    }

    // Engine::updateFixedAlleles (:303-345): the analysis removes the fixed alleles and records them on the
    // device; the loop over fixed indices is kept for the reference's call shape
    uint32_t updateFixedAlleles(sequence_space_type* ss) {
        free_(ss, pool_);
        for (auto it = free_.fixed_begin(); it != free_.fixed_end(); ++it) ss->remove_fixed_allele(*it);
        return free_.free_size();
    }
    // child_max_alleles (:287-301)
    static size_t child_max_alleles(size_t N_parent, size_t F_parent, size_t M_child) {
        return F_parent >= M_child ? N_parent : N_parent + (M_child - F_parent);
    }

    // the fused call: the same host draws in the same order, one tape call
    void simulate_fused() {
        const unsigned N = next_size();
        const uint32_t M = mut_.generateNewMutation(2 * N);
        pop_.step().pending = false;  // the tape call below runs the whole generation
        sel_.update(fit_.values(), N);
        xover_.draw(2 * (size_t)N);
        std::vector<uint32_t> pairs;
        pairs.reserve(2 * (size_t)N);
        for (const auto& pr : sel_.getMatePairs()) {
            pairs.push_back(pr.first);
            pairs.push_back(pr.second);
        }
        std::uniform_int_distribution<uint32_t> seq(0, 2 * N - 1);
        std::uniform_real_distribution<double> pos(0.0, 1.0);
        std::bernoulli_distribution neutral(pop_.params().p_neutral);
        std::normal_distribution<double> w(pop_.params().eff_mean, pop_.params().eff_sigma);
        const unsigned T = pop_.params().traits;
        std::vector<uint32_t> ms(M);
        std::vector<double> mp(M);
        std::vector<float> me((size_t)M * T, 0.0f);
        for (uint32_t i = 0; i < M; ++i) {
            ms[i] = seq(*rng_);
            mp[i] = pos(*rng_);
            for (unsigned t = 0; t < T; ++t)
                if (!neutral(*rng_)) me[(size_t)i * T + t] = (float)w(*rng_);
        }
        clotho_gen_tape tape{N, M, pairs.data(), xover_.bias().data(), xover_.lookup().data(),
                             xover_.events().data(), ms.data(), mp.data(), me.data()};
        check(clotho_generation_tape(pop_.get(), &tape), pop_.get(), "clotho_generation_tape");
        fit_.load(&pop_);
        std::swap(child_, parent_);
        child_->invalidate();
        parent_->invalidate();
        N_ = N;
    }

    RNG* rng_;
    Context pop_;
    PopulationSpaceGPU pop0_, pop1_;
    PopulationSpaceGPU *parent_, *child_;
    AlleleSpaceGPU alleles_;
    TraitSpaceGPU traits_;
    FreeSpaceGPU free_;
    SelectionGPU<RNG> sel_;
    CrossoverGPU<RNG> xover_;
    MutationGPU<RNG> mut_;
    PhenotypeGPU pheno_;
    FitnessGPU fit_;
    Pool pool_;
    unsigned N_;
    std::shared_ptr<PopulationGrowth> growth_;
    std::vector<double> sim_times_;
    std::vector<uint32_t> free_sizes_, var_sizes_, fixed_sizes_;
};

}  // namespace gb300
}  // namespace clotho
