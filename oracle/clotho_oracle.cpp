// clotho_oracle.cpp -- CPU restatement of the QTLSimMT per-generation step.
//
// TEST INFRASTRUCTURE ONLY (the checker and the CPU baseline; never shipped,
// never called by the product library).  Every function cites the reference
// file:line whose behaviour it restates.  Paths are relative to the
// putnampp/clotho source tree.
//
// Parity status: pinned against the known-answer tests of the reference's
// unit tests (see tests/test_oracle_kat.py).  The reference cannot be built
// here (Boost is absent), so the Boost.Random draw stream is not reproduced:
// parity is "same tape in, same genomes out".

#include "clotho_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

constexpr unsigned kBitsPerBlock = 64;        // bit_helper<8>
constexpr unsigned kBitsPerCacheLine = 512;   // utility/bit_helper.hpp:68
constexpr unsigned kBlocksPerCacheLine = 8;   // utility/bit_helper.hpp:69
constexpr uint64_t kAllSet = ~0ull;
constexpr uint64_t kAllUnset = 0ull;

// population_space_row::setMaxAlleles
// (data_spaces/population_space/population_space_row_block.hpp:94-101):
// the row width is the allele count rounded up to whole 512-bit cache lines.
inline unsigned ref_block_columns(unsigned A) {
    unsigned lines = A / kBitsPerCacheLine + ((A % kBitsPerCacheLine) ? 1u : 0u);
    return lines * kBlocksPerCacheLine;
}

// debruijn_bit_walker<uint64>::next_and_shift
// (utility/debruijn_bit_walker.hpp:111-127) visits set bits in ascending order;
// the walk below yields the same index sequence.
template <class F>
inline void walk_bits(uint64_t b, F&& f) {
    while (b) {
        unsigned j = (unsigned)__builtin_ctzll(b);
        f(j);
        b &= b - 1;
    }
}

// ---------------------------------------------------------------------------
// Executor: restates thread_pool<RNG> (data_spaces/task/thread_pool.hpp:37-139):
// TC-1 workers plus the master thread, which runs the last batch, then sync.
class Pool {
public:
    explicit Pool(unsigned tc) : tc_(tc < 1 ? 1 : tc) {
        for (unsigned i = 0; i + 1 < tc_; ++i) workers_.emplace_back([this, i] { loop(i); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    unsigned size() const { return tc_; }

    // Runs fn(part) for part in [0, nparts).  Parts 0..nparts-2 are posted to
    // the workers, the last part runs on the calling (master) thread.
    void run(unsigned nparts, const std::function<void(unsigned)>& fn) {
        if (nparts == 0) return;
        if (workers_.empty() || nparts == 1) {
            for (unsigned p = 0; p < nparts; ++p) fn(p);
            return;
        }
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &fn;
            nposted_ = nparts - 1;
            next_ = 0;
            pending_ = nparts - 1;
        }
        cv_.notify_all();
        fn(nparts - 1);
        std::unique_lock<std::mutex> lk(m_);
        done_cv_.wait(lk, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    // A part is claimed under the lock, so a worker can never pick up a part
    // of a job whose run() has already returned.
    void loop(unsigned) {
        std::unique_lock<std::mutex> lk(m_);
        for (;;) {
            cv_.wait(lk, [this] { return stop_ || (job_ != nullptr && next_ < nposted_); });
            if (stop_) return;
            unsigned p = next_++;
            const std::function<void(unsigned)>* job = job_;
            lk.unlock();
            (*job)(p);
            lk.lock();
            if (--pending_ == 0) done_cv_.notify_all();
        }
    }

    unsigned tc_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(unsigned)>* job_ = nullptr;
    unsigned nposted_ = 0, pending_ = 0, next_ = 0;
    bool stop_ = false;
};

// Batch size rule used by every MT stage of the reference, e.g.
// free_space_mt_population_space_row_interlaced.hpp:101.
inline unsigned batch_size(unsigned n, unsigned tc) { return n / tc + ((n % tc) ? 1u : 0u); }

// Partitions [0,n) into contiguous ranges of the reference batch size and
// runs them on the pool.
void partitioned(Pool& pool, unsigned n, const std::function<void(unsigned, unsigned)>& body) {
    if (n == 0) return;
    unsigned bs = batch_size(n, pool.size());
    unsigned parts = (n + bs - 1) / bs;
    pool.run(parts, [&](unsigned p) {
        unsigned lo = p * bs, hi = std::min(n, lo + bs);
        body(lo, hi);
    });
}

// ---------------------------------------------------------------------------
// Tape-recorder RNG: xoshiro256** (Blackman & Vigna) seeded by splitmix64.
// It stands in for boost::random::mt19937; only the tape it writes matters.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            v = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform_01 (generators/position_distribution_helper.hpp:27-41): [0,1).
    double u01() { return (double)(next() >> 11) * 0x1.0p-53; }
    // uniform_int_distribution(0, n-1) (general_fitness_selection_generator.hpp:63,
    // batch_mutation_task_population_space_row.hpp:77).
    uint32_t uint_below(uint32_t n) {
        if (n <= 1) return 0;
        uint64_t v = (uint64_t)(u01() * (double)n);
        return (uint32_t)(v >= n ? n - 1 : v);
    }
    // bernoulli_distribution(p) (batch_crossover_mtwe.hpp:139, neutral_parameter.hpp:30).
    bool bernoulli(double p) { return u01() < p; }
    // normal_distribution(mean, sigma) (weight_distribution_helper.hpp:28-48):
    // Marsaglia's polar method.
    double normal(double mean, double sigma) {
        if (have_spare) { have_spare = false; return mean + sigma * spare; }
        double u, v, q;
        do {
            u = 2.0 * u01() - 1.0;
            v = 2.0 * u01() - 1.0;
            q = u * u + v * v;
        } while (q >= 1.0 || q == 0.0);
        double f = std::sqrt(-2.0 * std::log(q) / q);
        spare = v * f;
        have_spare = true;
        return mean + sigma * u * f;
    }
    // poisson_distribution(lambda) (mutation_allocator.hpp:41-47,
    // crossover_event_distribution_helper.hpp:25-36): inversion for small
    // means, Hoermann's PTRS transformed rejection (1993) for large ones.
    uint32_t poisson(double lam) {
        if (!(lam > 0.0)) return 0;
        if (lam < 12.0) {
            double u = u01(), p = std::exp(-lam), F = p;
            uint32_t k = 0;
            while (u > F && k < 1000) { ++k; p *= lam / k; F += p; }
            return k;
        }
        double slam = std::sqrt(lam), loglam = std::log(lam);
        double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
        double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
        for (;;) {
            double U = u01() - 0.5, V = u01(), us = 0.5 - std::fabs(U);
            double k = std::floor((2.0 * a / us + b) * U + lam + 0.43);
            if (us >= 0.07 && V <= vr) return (uint32_t)k;
            if (k < 0.0 || (us < 0.013 && V > us)) continue;
            if (std::log(V) + std::log(invalpha) - std::log(a / (us * us) + b) <=
                -lam + k * loglam - std::lgamma(k + 1.0))
                return (uint32_t)k;
        }
    }
    bool have_spare = false;
    double spare = 0.0;
};

// ---------------------------------------------------------------------------
// population_space_row<uint64_t,double>
// (data_spaces/population_space/population_space_row_block.hpp:25-260).
struct PopSpace {
    std::vector<uint64_t> g;
    unsigned rows = 0, B = 0, A = 0, T = 0;
    std::vector<double> genome_traits;

    // grow(I, A, T) :64-72 with resize() :231-251 (content is not kept when
    // the buffer grows; every child word is rewritten by crossover).
    void grow(unsigned I, unsigned A_, unsigned T_) {
        rows = 2 * I;
        A = A_;
        B = ref_block_columns(A_);
        T = T_;
        size_t tot = (size_t)rows * B;
        if (tot > g.size()) g.assign(tot, 0);
        size_t nt = (size_t)T * rows;
        if (genome_traits.size() < nt) genome_traits.resize(nt, 0.0);
    }
    void clear() { std::fill(g.begin(), g.end(), 0); }  // :219-221
    uint64_t* row(unsigned i) { return g.data() + (size_t)i * B; }
    const uint64_t* row(unsigned i) const { return g.data() + (size_t)i * B; }
    // mutate :111-125 (XOR of one bit)
    void mutate(unsigned seq, unsigned slot) {
        row(seq)[slot / kBitsPerBlock] ^= (1ull << (slot % kBitsPerBlock));
    }
    // remove_fixed_allele :127-147 (clear one column in every row)
    void remove_fixed_allele(unsigned slot) {
        uint64_t mask = ~(1ull << (slot % kBitsPerBlock));
        for (unsigned i = 0; i < rows; ++i) row(i)[slot / kBitsPerBlock] &= mask;
    }
};

// AlleleSpace<double,uint> (data_spaces/allele_space/allele_space_vector.hpp:31-227);
// the std::map position multiset is bookkeeping only and is not restated.
struct AlleleTable {
    std::vector<double> pos;
    std::vector<uint32_t> age;
    size_t size() const { return pos.size(); }
    void grow() { pos.push_back(0.0); age.push_back(0); }                      // :185-192
    void setAllele(unsigned i, double p, uint32_t a) { pos[i] = p; age[i] = a; } // :115-137
    void append(const AlleleTable& o, unsigned i) {                            // :159-183
        pos.push_back(o.pos[i]);
        age.push_back(o.age[i]);
    }
};

// trait_space_vector<double> (data_spaces/phenotype_evaluator/trait_space_vector.hpp:26-198).
struct TraitTable {
    unsigned T = 1;
    std::vector<double> w;
    void grow() { for (unsigned i = 0; i < T; ++i) w.push_back(0.0); }
    void set(double v, unsigned row, unsigned col) { w[(size_t)row * T + col] = v; }
    // isAllNeutral :73-78 (every stored weight, stale ones included)
    bool all_neutral() const {
        for (double v : w) if (v != 0.0) return false;
        return true;
    }
};

// free_space_details (data_spaces/free_space/free_space_details.hpp:176-357).
struct FreeSpace {
    std::vector<uint32_t> idx;
    unsigned fixed = 0, lost = 0, size = 0;
    unsigned free_size() const { return fixed + lost; }
    unsigned variable_count() const { return size - (fixed + lost); }
};

// FreeSpaceAnalyzerMT<population_space_row>::operator()
// (free_space/free_space_mt_population_space_row_interlaced.hpp:41-89, tasks
// free_space_task_population_space_row_interlaced.hpp:51-72) followed by
// analyze_free_indices (free_space_details.hpp:299-357).
void analyze_free_space(const uint64_t* rows, unsigned S, unsigned B, unsigned A, Pool& pool,
                        FreeSpace& fs) {
    if (A == 0) return;  // :46, previous state is kept
    fs.size = A;
    std::vector<uint64_t> d(2 * (size_t)B);
    if (S == 0) {
        std::fill(d.begin(), d.end(), 0);
    } else {
        for (unsigned w = 0; w < B; ++w) d[2 * w] = d[2 * w + 1] = rows[w];  // :58-66
        if (A / kBitsPerBlock != B) {                                         // :68-81
            size_t s = 2 * (size_t)(A / kBitsPerBlock);
            uint64_t pad = kAllSet << (A % kBitsPerBlock);
            d[s] &= ~pad;
            d[s + 1] |= pad;
            for (size_t e = s + 2; e < d.size(); e += 2) { d[e] = kAllUnset; d[e + 1] = kAllSet; }
        }
        // process_space :96-121: columns split into batches across threads.
        partitioned(pool, B, [&](unsigned lo, unsigned hi) {
            for (unsigned i = 1; i < S; ++i) {
                const uint64_t* r = rows + (size_t)i * B;
                for (unsigned w = lo; w < hi; ++w) { d[2 * w] &= r[w]; d[2 * w + 1] |= r[w]; }
            }
        });
    }
    fs.idx.assign(std::max<size_t>(A, (size_t)B * kBitsPerBlock), 0);
    unsigned off = 0;
    for (unsigned w = 0; w < B; ++w)  // fixed indices, ascending (:305-326)
        walk_bits(d[2 * w], [&](unsigned j) { fs.idx[off++] = w * kBitsPerBlock + j; });
    fs.fixed = off;
    for (unsigned w = 0; w < B; ++w)  // lost indices, ascending (:328-350)
        walk_bits(~d[2 * w + 1], [&](unsigned j) { fs.idx[off++] = w * kBitsPerBlock + j; });
    fs.lost = off - fs.fixed;
}

// region_classifier + binary_classifier<is_odd_tag> through PositionClassifier
// (crossover/position_classifier.hpp:59-93, classifiers/region_classifier.hpp:62-77,
// classifiers/binary_classifier.hpp:35-38, classifiers/tags/is_odd_tag.hpp:23-25):
// odd number of (sorted) events <= position  ->  take the bottom strand.
struct Classifier {
    std::vector<double> ev;  // sorted in the region_classifier constructor :62-64
    const std::vector<double>* pos;
    bool operator()(unsigned slot) const {
        if (ev.empty()) return false;
        size_t c = std::upper_bound(ev.begin(), ev.end(), pos->at(slot)) - ev.begin();
        return (c & 1) != 0;
    }
};

// block_crossover::crossover (crossover/block_crossover.hpp:46-63).
inline uint64_t block_crossover(const Classifier& cls, uint64_t top, uint64_t bottom, unsigned offset) {
    uint64_t hets = top ^ bottom, mask = 0;
    walk_bits(hets, [&](unsigned j) {
        if (cls(offset + j)) mask |= (1ull << j);
    });
    return (top & ~mask) | (bottom & mask);
}

// batch_crossover_taskwe<...population_space_row>::run_crossover_task /
// crossover_task (crossover/batch_crossover_taskwe_population_space_row.hpp:157-217).
void crossover_gamete(const Classifier& cls, const uint64_t* p0, unsigned n0, const uint64_t* p1,
                      unsigned n1, uint64_t* off, unsigned noff, bool swap) {
    if (cls.ev.empty()) {
        const uint64_t* src = swap ? p1 : p0;
        unsigned n = swap ? n1 : n0, i = 0;
        for (; i < n; ++i) off[i] = src[i];
        for (; i < noff; ++i) off[i] = kAllUnset;
        return;
    }
    if (swap) { std::swap(p0, p1); std::swap(n0, n1); }
    unsigned i = 0, k = 0;
    for (;; ++k) {
        if (k >= n0) {
            for (; k < n1; ++k) off[i++] = block_crossover(cls, kAllUnset, p1[k], k * kBitsPerBlock);
            break;
        } else if (k >= n1) {
            for (; k < n0; ++k) off[i++] = block_crossover(cls, p0[k], kAllUnset, k * kBitsPerBlock);
            break;
        }
        off[i++] = block_crossover(cls, p0[k], p1[k], k * kBitsPerBlock);
    }
    for (; i < noff; ++i) off[i] = kAllUnset;
}

// batch_phenotype_task<...row>::accumulate_allele_weights_alt2
// (phenotype_evaluator/batch_phenotype_task_population_space_row.hpp:127-153):
// words ascending, set bits of a word accumulated in descending order.
void genome_weights(const uint64_t* row, unsigned B, const double* w, unsigned T, double* out) {
    for (unsigned t = 0; t < T; ++t) out[t] = 0.0;
    unsigned idx[64];
    for (unsigned k = 0; k < B; ++k) {
        unsigned n = 0;
        walk_bits(row[k], [&](unsigned j) { idx[n++] = k * kBitsPerBlock + j; });
        while (n--) {
            const double* e = w + (size_t)idx[n] * T;
            for (unsigned t = 0; t < T; ++t) out[t] += e[t];
        }
    }
}

uint32_t seed_hash(uint64_t seed, uint32_t row, uint32_t slot) {
    uint64_t x = seed + 0x9E3779B97F4A7C15ull * ((((uint64_t)row) << 32) + (uint64_t)slot + 1ull);
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (uint32_t)(x >> 32);
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// Engine<RNG,double,uint64_t,uint,batched_task> (examples/QTLSim/engine_batched_task.hpp:70-373).
struct Engine {
    orc_params prm;
    Pool pool;
    Rng rng;
    PopSpace pop0, pop1;
    PopSpace *parent = &pop0, *child = &pop1;
    AlleleTable alleles, fixed;
    TraitTable traits, fixed_traits;
    FreeSpace fs;
    std::vector<double> phenos;   // N*T individual phenotypes
    std::vector<double> fitness;  // N
    uint32_t generation = 0;
    uint32_t last_M = 0;
    bool all_neutral = true;
    double times[6] = {0, 0, 0, 0, 0, 0};

    // recorded tape (orc_step_record)
    std::vector<uint32_t> t_pairs, t_evoff, t_mseq;
    std::vector<uint8_t> t_swap;
    std::vector<double> t_evpos, t_mpos;
    std::vector<float> t_meff;
    orc_tape rec{};

    explicit Engine(const orc_params& p) : prm(p), pool(p.threads ? p.threads : 1), rng(p.seed) {
        traits.T = fixed_traits.T = p.T;
    }

    // init(0) :143-161
    void init(uint32_t N0) {
        pop0.grow(N0, 0, prm.T);
        pop1.grow(N0, 0, prm.T);
        pop1.clear();
        pop0.clear();
        parent = &pop0;
        child = &pop1;
        fitness.assign(N0, 1.0);  // GeneralFitness::resize (general_fitness.hpp:230-235)
        phenos.clear();
        generation = 1;
    }

    void seed(uint32_t N, uint32_t A, const double* pos, const float* eff, const uint32_t* thr,
              uint64_t s) {
        init(N);
        child->grow(N, A, prm.T);
        std::fill(child->g.begin(), child->g.end(), 0);
        partitioned(pool, child->rows, [&](unsigned lo, unsigned hi) {
            for (uint32_t r = lo; r < hi; ++r) {
                uint64_t* row = child->row(r);
                for (uint32_t a = 0; a < A; ++a)
                    if (seed_hash(s, r, a) < thr[a]) row[a / 64] |= 1ull << (a % 64);
            }
        });
        alleles.pos.assign(pos, pos + A);
        alleles.age.assign(A, 0);
        traits.w.assign(A * (size_t)prm.T, 0.0);
        for (size_t i = 0; i < (size_t)A * prm.T; ++i) traits.w[i] = (double)eff[i];
        evaluate_child();
    }

    void load(uint32_t N, uint32_t A, const uint64_t* rows, const double* pos, const float* eff) {
        init(N);
        child->grow(N, A, prm.T);
        std::copy(rows, rows + (size_t)child->rows * child->B, child->g.begin());
        alleles.pos.assign(pos, pos + A);
        alleles.age.assign(A, 0);
        traits.w.assign(A * (size_t)prm.T, 0.0);
        for (size_t i = 0; i < (size_t)A * prm.T; ++i) traits.w[i] = (double)eff[i];
        evaluate_child();
    }

    // child_max_alleles :287-301
    static size_t child_max_alleles(size_t Np, size_t Fp, size_t Mc) {
        return (Fp >= Mc) ? Np : Np + (Mc - Fp);
    }

    // updateFixedAlleles :303-345
    uint32_t update_fixed(PopSpace* ss) {
        analyze_free_space(ss->g.data(), ss->rows, ss->B, ss->A, pool, fs);
        for (unsigned i = 0; i < fs.fixed; ++i) {
            unsigned f = fs.idx[i];
            ss->remove_fixed_allele(f);
            fixed.append(alleles, f);
            for (unsigned t = 0; t < prm.T; ++t) fixed_traits.w.push_back(traits.w[(size_t)f * prm.T + t]);
        }
        return fs.free_size();
    }

    // BatchCrossoverMTWE::batch_generate (crossover/batch_crossover_mtwe.hpp:62-113)
    void crossover(const orc_tape& t) {
        const bool q1 = (prm.flags & ORC_FLAG_Q1) != 0;
        partitioned(pool, t.N, [&](unsigned lo, unsigned hi) {
            for (unsigned k = lo; k < hi; ++k) {
                for (unsigned h = 0; h < 2; ++h) {
                    unsigned g = 2 * k + h;
                    unsigned pid = 2 * t.pairs[g];
                    Classifier cls;
                    cls.pos = &alleles.pos;
                    if (!(q1 && h == 1))
                        cls.ev.assign(t.ev_pos + t.ev_off[g], t.ev_pos + t.ev_off[g + 1]);
                    std::sort(cls.ev.begin(), cls.ev.end());
                    crossover_gamete(cls, parent->row(pid), parent->B, parent->row(pid + 1), parent->B,
                                     child->row(g), child->B, t.swap[g] != 0);
                }
            }
        });
    }

    // BatchMutationMT::operator() (mutation/batch_mutation_mt.hpp:67-81) with
    // BatchMutationTask<...row> (batch_mutation_task_population_space_row.hpp:76-88);
    // the task count is forced to 1 (engine_batched_task.hpp:202).
    void mutate(const orc_tape& t) {
        std::vector<uint32_t> free_indices(fs.idx.begin(), fs.idx.begin() + fs.free_size());
        if (t.M > fs.free_size()) {
            unsigned add = t.M - fs.free_size();
            for (unsigned b = 0; b < add; ++b) {
                free_indices.push_back((uint32_t)alleles.size());
                alleles.grow();
                traits.grow();
            }
        }
        for (unsigned i = 0; i < t.M; ++i) {
            unsigned slot = free_indices[i];
            child->mutate(t.mut_seq[i], slot);
            alleles.setAllele(slot, t.mut_pos[i], generation);
            for (unsigned tt = 0; tt < prm.T; ++tt) traits.set((double)t.mut_eff[(size_t)i * prm.T + tt], slot, tt);
        }
    }

    // BatchPhenotypeMT<...row>::operator() / constant_phenotype
    // (phenotype_evaluator/batch_phenotype_mt_population_space_row.hpp:48-72,111-156),
    // individual_reducer_task (individual_reducer_task_population_space_row.hpp:51-79).
    void phenotype() {
        const unsigned T = prm.T, S = child->rows, N = S / 2;
        phenos.assign((size_t)N * T, 0.0);
        all_neutral = traits.all_neutral();
        if (all_neutral) {  // engine_batched_task.hpp:207-211
            std::fill(phenos.begin(), phenos.end(), 1.0);
            return;
        }
        partitioned(pool, S, [&](unsigned lo, unsigned hi) {
            for (unsigned i = lo; i < hi; ++i)
                genome_weights(child->row(i), child->B, traits.w.data(), T, &child->genome_traits[(size_t)i * T]);
        });
        partitioned(pool, N, [&](unsigned lo, unsigned hi) {
            for (unsigned i = lo; i < hi; ++i)
                for (unsigned t = 0; t < T; ++t)
                    phenos[(size_t)i * T + t] =
                        child->genome_traits[(size_t)(2 * i) * T + t] + child->genome_traits[(size_t)(2 * i + 1) * T + t];
        });
    }

    // GeneralFitness::operator()(BatchPhenotypeMT<row>&) (fitness/general_fitness.hpp:101-119)
    // with the toolkit metrics: normal_fitness_metric.cpp:25-31 (+generator
    // normal_fitness_generator.cpp:36-52), quadratic_fitness_metric.cpp:23-28
    // (+quadratic_fitness_generator.cpp:42-54), constant; gaussian_vs is the
    // exp(-|z|^2/2Vs) metric the multi-trait configurations need.
    void compute_fitness() {
        const unsigned T = prm.T, N = child->rows / 2;
        fitness.assign(N, 1.0);
        const double n4 = std::sqrt(4.0 * (double)N * prm.mu);
        for (unsigned i = 0; i < N; ++i) {
            const double* z = &phenos[(size_t)i * T];
            double f = 1.0;
            switch (prm.fitness) {
                case ORC_FIT_GAUSSIAN: {
                    double sigma = n4;
                    double coeff = (1.0 / sigma) * 0.398942280401432677939946059934;  // 1/sqrt(2 pi)
                    double ex = z[0] * z[0] / (2.0 * sigma * sigma);
                    f = coeff * std::exp(-ex);
                } break;
                case ORC_FIT_QUADRATIC: {
                    double s = prm.fit_param * n4;
                    double r = z[0] / s;
                    r *= r;
                    f = (r >= 1.0) ? 0.0 : 1.0 - r;
                } break;
                case ORC_FIT_GAUSSIAN_VS: {
                    double ss = 0.0;
                    for (unsigned t = 0; t < T; ++t) ss += z[t] * z[t];
                    f = std::exp(-ss / (2.0 * prm.fit_param));
                } break;
                default: f = 1.0;
            }
            fitness[i] = f;
        }
    }

    void evaluate_child() {
        phenotype();
        compute_fitness();
    }

    // Engine::simulate (engine_batched_task.hpp:163-223) on a tape.
    int step(const orc_tape& t) {
        double t0 = now_s();
        std::swap(child, parent);
        double tf0 = now_s();
        uint32_t free_count = update_fixed(parent);
        double tf1 = now_s();
        size_t all_size = child_max_alleles(alleles.size(), free_count, t.M);
        child->grow(t.N, (unsigned)all_size, prm.T);
        double tx0 = now_s();
        crossover(t);
        double tx1 = now_s();
        mutate(t);
        double tm1 = now_s();
        phenotype();
        double tp1 = now_s();
        compute_fitness();
        double tfit = now_s();
        last_M = t.M;
        ++generation;
        times[0] = tf1 - tf0; times[1] = tx1 - tx0; times[2] = tm1 - tx1;
        times[3] = tp1 - tm1; times[4] = tfit - tp1; times[5] = tfit - t0;
        return 0;
    }

    // Draws one generation in the reference's draw order
    // (engine_batched_task.hpp:175-202):
    // M (mutation_allocator.hpp:41-47); selection pairs
    // (general_fitness_selection_generator.hpp:45-69,104-113); per gamete E then
    // E positions (batch_crossover_mtwe.hpp:117-133); all bias bits (:135-145);
    // per mutation: sequence, position, then per trait [neutral, normal]
    // (batch_mutation_task_population_space_row.hpp:76-88,
    // trait_space_generator.hpp:118-129).  The free-space analysis is done
    // first because the tape's M must be known to the analysis consumer only;
    // it draws nothing.
    int step_record(uint32_t N) {
        const unsigned T = prm.T;
        uint32_t M = rng.poisson(prm.mu * 2.0 * (double)N);
        // selection over the current (soon parent) fitness
        t_pairs.resize(2 * (size_t)N);
        const size_t P = fitness.size();
        bool constant = true;
        for (size_t i = 1; i < P && constant; ++i) constant = (fitness[i] == fitness[0]);
        if (constant) {
            for (size_t i = 0; i < 2 * (size_t)N; ++i) t_pairs[i] = rng.uint_below((uint32_t)(P == 0 ? 1 : P));
        } else {
            std::vector<double> cdf(P);
            double acc = 0.0;
            for (size_t i = 0; i < P; ++i) { acc += fitness[i]; cdf[i] = acc; }
            for (size_t i = 0; i < 2 * (size_t)N; ++i) {
                double x = rng.u01() * acc;
                size_t k = std::upper_bound(cdf.begin(), cdf.end(), x) - cdf.begin();
                t_pairs[i] = (uint32_t)(k >= P ? P - 1 : k);
            }
        }
        t_evoff.assign(2 * (size_t)N + 1, 0);
        t_evpos.clear();
        for (size_t g = 0; g < 2 * (size_t)N; ++g) {
            t_evoff[g] = (uint32_t)t_evpos.size();
            uint32_t E = rng.poisson(prm.rho);
            while (E--) t_evpos.push_back(rng.u01());
        }
        t_evoff[2 * (size_t)N] = (uint32_t)t_evpos.size();
        t_swap.resize(2 * (size_t)N);
        for (size_t g = 0; g < 2 * (size_t)N; ++g) t_swap[g] = rng.bernoulli(prm.bias) ? 1 : 0;
        t_mseq.resize(M);
        t_mpos.resize(M);
        t_meff.resize((size_t)M * T);
        for (uint32_t i = 0; i < M; ++i) {
            t_mseq[i] = rng.uint_below(2 * N);
            t_mpos[i] = rng.u01();
            for (unsigned tt = 0; tt < T; ++tt) {
                double w = 0.0;
                if (!rng.bernoulli(prm.p_neutral)) w = rng.normal(prm.eff_mean, prm.eff_sigma);
                t_meff[(size_t)i * T + tt] = (float)w;
            }
        }
        rec.N = N; rec.M = M;
        rec.pairs = t_pairs.data(); rec.swap = t_swap.data();
        rec.ev_off = t_evoff.data(); rec.ev_pos = t_evpos.data();
        rec.mut_seq = t_mseq.data(); rec.mut_pos = t_mpos.data(); rec.mut_eff = t_meff.data();
        return step(rec);
    }
};

}  // namespace

extern "C" {

void* orc_create(const orc_params* p) { return new Engine(*p); }
void orc_destroy(void* h) { delete static_cast<Engine*>(h); }
void orc_init(void* h, uint32_t N0) { static_cast<Engine*>(h)->init(N0); }
void orc_seed_population(void* h, uint32_t N, uint32_t A, const double* pos, const float* eff,
                         const uint32_t* thr, uint64_t seed) {
    static_cast<Engine*>(h)->seed(N, A, pos, eff, thr, seed);
}
void orc_load_population(void* h, uint32_t N, uint32_t A, const uint64_t* rows, const double* pos,
                         const float* eff) {
    static_cast<Engine*>(h)->load(N, A, rows, pos, eff);
}
int orc_step_tape(void* h, const orc_tape* t) { return static_cast<Engine*>(h)->step(*t); }
int orc_step_record(void* h, uint32_t N) { return static_cast<Engine*>(h)->step_record(N); }
void orc_last_tape(void* h, orc_tape* out, uint32_t* ev_total) {
    Engine* e = static_cast<Engine*>(h);
    *out = e->rec;
    *ev_total = e->t_evoff.empty() ? 0 : e->t_evoff.back();
}

void orc_get_info(void* h, orc_info* o) {
    Engine* e = static_cast<Engine*>(h);
    o->generation = e->generation;
    o->S = e->child->rows;
    o->N = e->child->rows / 2;
    o->A = e->child->A;
    o->B = e->child->B;
    o->fixed_count = e->fs.fixed;
    o->lost_count = e->fs.lost;
    o->free_count = e->fs.free_size();
    o->variable_count = e->fs.variable_count();
    o->fixed_total = (uint32_t)e->fixed.size();
    o->all_neutral = e->all_neutral ? 1u : 0u;
    o->last_M = e->last_M;
}
void orc_get_rows(void* h, uint64_t* dst) {
    Engine* e = static_cast<Engine*>(h);
    std::memcpy(dst, e->child->g.data(), sizeof(uint64_t) * (size_t)e->child->rows * e->child->B);
}
void orc_get_alleles(void* h, double* pos, uint32_t* age, double* eff) {
    Engine* e = static_cast<Engine*>(h);
    std::copy(e->alleles.pos.begin(), e->alleles.pos.end(), pos);
    std::copy(e->alleles.age.begin(), e->alleles.age.end(), age);
    std::copy(e->traits.w.begin(), e->traits.w.end(), eff);
}
void orc_get_fixed(void* h, double* pos, uint32_t* age, double* eff) {
    Engine* e = static_cast<Engine*>(h);
    std::copy(e->fixed.pos.begin(), e->fixed.pos.end(), pos);
    std::copy(e->fixed.age.begin(), e->fixed.age.end(), age);
    std::copy(e->fixed_traits.w.begin(), e->fixed_traits.w.end(), eff);
}
void orc_get_free(void* h, uint32_t* dst) {
    Engine* e = static_cast<Engine*>(h);
    std::copy(e->fs.idx.begin(), e->fs.idx.begin() + e->fs.free_size(), dst);
}
void orc_get_genome_traits(void* h, double* dst) {
    Engine* e = static_cast<Engine*>(h);
    std::copy(e->child->genome_traits.begin(), e->child->genome_traits.begin() + (size_t)e->child->rows * e->prm.T, dst);
}
void orc_get_phenotypes(void* h, double* dst) {
    Engine* e = static_cast<Engine*>(h);
    std::copy(e->phenos.begin(), e->phenos.end(), dst);
}
void orc_get_fitness(void* h, double* dst) {
    Engine* e = static_cast<Engine*>(h);
    std::copy(e->fitness.begin(), e->fitness.end(), dst);
}
void orc_get_times(void* h, double* dst6) {
    Engine* e = static_cast<Engine*>(h);
    for (int i = 0; i < 6; ++i) dst6[i] = e->times[i];
}

uint32_t orc_bit_walk(uint64_t w, uint32_t* idx) {
    uint32_t n = 0;
    walk_bits(w, [&](unsigned j) { idx[n++] = j; });
    return n;
}
void orc_free_space(const uint64_t* rows, uint32_t S, uint32_t B, uint32_t A, uint32_t threads,
                    uint32_t* out, uint32_t* counts) {
    Pool pool(threads ? threads : 1);
    FreeSpace fs;
    analyze_free_space(rows, S, B, A, pool, fs);
    for (unsigned i = 0; i < fs.free_size(); ++i) out[i] = fs.idx[i];
    counts[0] = fs.fixed;
    counts[1] = fs.lost;
    counts[2] = fs.free_size();
}
uint64_t orc_block_crossover(uint64_t top, uint64_t bottom, uint32_t offset, const double* positions,
                             uint32_t npos, const double* events, uint32_t nev) {
    std::vector<double> pos(positions, positions + npos);
    Classifier c;
    c.pos = &pos;
    c.ev.assign(events, events + nev);
    std::sort(c.ev.begin(), c.ev.end());
    return block_crossover(c, top, bottom, offset);
}
void orc_genome_weights(const uint64_t* row, uint32_t B, const double* w, uint32_t T, double* out) {
    genome_weights(row, B, w, T, out);
}
uint32_t orc_seed_hash(uint64_t seed, uint32_t row, uint32_t slot) { return seed_hash(seed, row, slot); }

}  // extern "C"
