/*
 * clotho_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the
 * per-generation hot path of putnampp/clotho's QTLSimMT engine
 * (examples/QTLSim/engine_batched_task.hpp:163-345).  It is the checker that
 * GPU results are compared against, and the CPU baseline that bench.py times.
 * Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
 * --impl reference arm) may load it.  The product library never links it.
 *
 * Parity status: the reference itself cannot be compiled here (every
 * hot-path header includes Boost, which is absent), so the restatement is
 * pinned against the known-answer tests of the reference's own unit tests
 * (unittest/data_spaces/{free_space,crossover,linear_phenotype,mutation}_test.cpp,
 * unittest/utility/{debruijn_bit_walker,popcount}_test.cpp), restated as
 * tests/test_oracle_kat.py.  The random stream of Boost.Random is not pinned:
 * parity is defined as identical genomes given the same event tape.
 */
#ifndef CLOTHO_ORACLE_H_
#define CLOTHO_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One generation of the event tape, in the reference's draw order
 * (engine_batched_task.hpp:175-202).  Identical layout to clotho_gen_tape in
 * include/clotho_gpu.h so one buffer set feeds both engines. */
typedef struct orc_tape {
    uint32_t N;              /* offspring individuals (pairs)                */
    uint32_t M;              /* new mutations                                */
    const uint32_t *pairs;   /* [2N] (id0,id1) parent individuals            */
    const uint8_t  *swap;    /* [2N] strand-swap (bias) bit per gamete       */
    const uint32_t *ev_off;  /* [2N+1] event lookup offsets                  */
    const double   *ev_pos;  /* [ev_off[2N]] crossover positions, draw order */
    const uint32_t *mut_seq; /* [M] target offspring sequence                */
    const double   *mut_pos; /* [M] allele position                          */
    const float    *mut_eff; /* [M*T] allele effects (FP32 on the tape)      */
} orc_tape;

enum {
    ORC_FIT_CONSTANT = 0,
    ORC_FIT_GAUSSIAN = 1,    /* normal_fitness_metric, sigma = sqrt(4 N mu)   */
    ORC_FIT_QUADRATIC = 2,   /* quadratic_fitness_metric, s = scale*sqrt(4Nmu)*/
    ORC_FIT_GAUSSIAN_VS = 3  /* exp(-|z|^2 / (2 Vs)), Vs = fit_param          */
};

enum {
    ORC_FLAG_Q1 = 1u        /* reference behaviour: second gamete of each pair
                               never recombines (batch_crossover_taskwe_
                               population_space_row.hpp:133-138)            */
};

typedef struct orc_params {
    uint32_t T;            /* traits                                        */
    int32_t  fitness;      /* ORC_FIT_*                                     */
    double   fit_param;    /* quadratic scale, or Vs                        */
    double   mu;           /* mutation.mu (per sequence)                    */
    double   rho;          /* recombination.rho (per gamete)                */
    double   bias;         /* recombination.sequence_bias.p                 */
    double   p_neutral;    /* neutral.p                                     */
    double   eff_mean;     /* traits.mean                                   */
    double   eff_sigma;    /* traits.sigma                                  */
    uint32_t flags;        /* ORC_FLAG_*                                    */
    uint32_t threads;      /* worker threads + master (>=1)                 */
    uint64_t seed;         /* tape-recorder RNG seed                        */
} orc_params;

typedef struct orc_info {
    uint32_t generation;   /* next generation number (== ages of new alleles) */
    uint32_t N;            /* individuals of the current child population   */
    uint32_t S;            /* haploid genomes (rows) = 2N                   */
    uint32_t A;            /* allele slots of the child (getMaxAlleles)     */
    uint32_t B;            /* block columns of the child (row width)        */
    uint32_t fixed_count;  /* from the last free-space analysis             */
    uint32_t lost_count;
    uint32_t free_count;
    uint32_t variable_count;
    uint32_t fixed_total;  /* alleles recorded in the fixed table           */
    uint32_t all_neutral;  /* trait space all zero -> constant phenotype    */
    uint32_t last_M;
} orc_info;

void *orc_create(const orc_params *p);
void  orc_destroy(void *h);
/* Engine::init(0): both populations grown to (N0, 0, T) and cleared. */
void  orc_init(void *h, uint32_t N0);
/* Pre-seeded start (measurement setup): A slots with given positions and
 * effects; bit (row, slot) set iff clotho_seed_hash(seed,row,slot) < thr[slot].
 * The same rule is implemented by the device (clotho_seed_population). */
void  orc_seed_population(void *h, uint32_t N, uint32_t A, const double *pos,
                          const float *eff, const uint32_t *thr, uint64_t seed);
/* Explicit start: 2N rows of ceil(A/512)*8 words, positions pos[A], effects
 * eff[A*T]; ages 0.  Phenotypes and fitness are evaluated. */
void  orc_load_population(void *h, uint32_t N, uint32_t A, const uint64_t *rows,
                          const double *pos, const float *eff);
/* One generation consuming a tape.  Returns 0 or a negative error. */
int   orc_step_tape(void *h, const orc_tape *t);
/* One generation drawing from the oracle's own RNG in the reference's draw
 * order, recording the tape.  N = offspring individuals. */
int   orc_step_record(void *h, uint32_t N);
/* Access to the last recorded tape (valid until the next step). */
void  orc_last_tape(void *h, orc_tape *out, uint32_t *ev_total);

void  orc_get_info(void *h, orc_info *out);
/* Child rows, S x B words (row-major, reference width). */
void  orc_get_rows(void *h, uint64_t *dst);
/* Allele table of length A: positions, ages, effects (A*T, FP64). */
void  orc_get_alleles(void *h, double *pos, uint32_t *age, double *eff);
void  orc_get_fixed(void *h, double *pos, uint32_t *age, double *eff);
/* Free list of the last analysis: fixed (ascending) then lost (ascending). */
void  orc_get_free(void *h, uint32_t *dst);
/* Per-genome trait sums (S*T), individual phenotypes (N*T), fitness (N). */
void  orc_get_genome_traits(void *h, double *dst);
void  orc_get_phenotypes(void *h, double *dst);
void  orc_get_fitness(void *h, double *dst);
/* Per-stage wall times of the last step in seconds:
 * [fixed, crossover, mutate, phenotypes, fitness, total]. */
void  orc_get_times(void *h, double *dst6);

/* ---- stage-level entry points used by the known-answer tests ---- */
/* debruijn_bit_walker order: set-bit indices, ascending. Returns count. */
uint32_t orc_bit_walk(uint64_t w, uint32_t *idx);
/* FreeSpaceAnalyzerMT over S rows of B words, A alleles. Writes the free
 * list to out (capacity >= B*64) and counts[3] = {fixed, lost, free}. */
void orc_free_space(const uint64_t *rows, uint32_t S, uint32_t B, uint32_t A,
                    uint32_t threads, uint32_t *out, uint32_t *counts);
/* block_crossover::crossover for one word, with the PositionClassifier over
 * positions[] and the (unsorted) events[]. */
uint64_t orc_block_crossover(uint64_t top, uint64_t bottom, uint32_t offset,
                             const double *positions, uint32_t npos,
                             const double *events, uint32_t nev);
/* accumulate_allele_weights_alt2 over one genome of B words, T traits. */
void orc_genome_weights(const uint64_t *row, uint32_t B, const double *w,
                        uint32_t T, double *out);
/* Bit rule shared with the device seeding kernel. */
uint32_t orc_seed_hash(uint64_t seed, uint32_t row, uint32_t slot);

#ifdef __cplusplus
}
#endif
#endif /* CLOTHO_ORACLE_H_ */
