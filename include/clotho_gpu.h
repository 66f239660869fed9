/*
 * clotho_gpu.h -- C-ABI of the GB300 (sm_103a) engine for the per-generation
 * hot path of a putnampp/clotho forward-time simulation.
 *
 * The reference plugs its stages into Engine<RNG,Real,Block,Size,batched_task>
 * through member typedefs (examples/QTLSim/engine_batched_task.hpp:84-103);
 * each entry point below names the reference member it replaces.  Paths are
 * relative to the putnampp/clotho source tree.
 *
 * Conventions
 *  - Every call returns an int status: 0 on success, a negative CLOTHO_E_*
 *    code on failure; clotho_last_error() gives the message.  No exception
 *    crosses the ABI.
 *  - A context owns one population (parent + child bitset spaces, allele and
 *    trait tables, free-space lists) in device memory, and one CUDA stream.
 *    Buffers are sized once at creation from clotho_desc capacities.
 *  - Host pointers passed in are read before the call returns (host->device
 *    copies complete before return); device work may still be in flight until
 *    clotho_sync() or a call that returns host data.
 *  - Bitset layout is the reference's population_space_row: row i is haploid
 *    genome i, individual j owns rows 2j and 2j+1; allele slot a is bit a%64 of
 *    word a/64; a row of A alleles has ceil(A/512)*8 words
 *    (population_space_row_block.hpp:94-101).
 *  - One context per host thread at a time.
 */
#ifndef CLOTHO_GPU_H_
#define CLOTHO_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLOTHO_ABI_VERSION 1

typedef struct clotho_ctx clotho_ctx;

/* status codes */
#define CLOTHO_OK              0
#define CLOTHO_E_ARG          -1   /* bad argument                            */
#define CLOTHO_E_CUDA         -2   /* CUDA runtime error                      */
#define CLOTHO_E_CAPACITY     -3   /* a size exceeds the context capacity     */
#define CLOTHO_E_STATE        -4   /* call out of order                        */
#define CLOTHO_E_DEVICE       -5   /* device-side check failed (see message)  */
#define CLOTHO_E_NOMEM        -6   /* device allocation refused               */

/* fitness metrics (fitness_toolkit registry, src/clotho/fitness/fitness_toolkit.cpp:50-78) */
#define CLOTHO_FIT_CONSTANT    0   /* 1.0                                      */
#define CLOTHO_FIT_GAUSSIAN    1   /* normal_fitness_metric.cpp:25-31, sigma = sqrt(4 N mu)
                                      (normal_fitness_generator.cpp:36-52), trait 0 */
#define CLOTHO_FIT_QUADRATIC   2   /* quadratic_fitness_metric.cpp:23-28,
                                      s = scale*sqrt(4 N mu), trait 0        */
#define CLOTHO_FIT_GAUSSIAN_VS 3   /* exp(-|z|^2 / (2 Vs)) over all traits     */

/* flags */
#define CLOTHO_FLAG_Q1         1u  /* reference behaviour: the second gamete of a
                                      mate pair never recombines
                                      (batch_crossover_taskwe_population_space_row.hpp:133-138) */

typedef struct clotho_desc {
    uint32_t max_individuals; /* N capacity; rows = 2N                        */
    uint32_t max_alleles;     /* allele slot capacity (A)                      */
    uint32_t traits;          /* T, 1..4 (traits.N)                            */
    uint32_t max_events;      /* crossover events per generation (tape mode)  */
    uint32_t max_mutations;   /* new mutations per generation                  */
    uint32_t max_fixed;       /* fixed-allele table capacity                   */
    int32_t  fitness;         /* CLOTHO_FIT_*                                  */
    uint32_t flags;           /* CLOTHO_FLAG_*                                 */
    double   fit_param;       /* quadratic: fitness.params.scale; gaussian_vs: Vs */
    double   mu;              /* mutation.mu per sequence                       */
    double   rho;             /* recombination.rho per gamete                   */
    double   bias;            /* recombination.sequence_bias.p                  */
    double   p_neutral;       /* neutral.p                                      */
    double   eff_mean;        /* traits.mean                                    */
    double   eff_sigma;       /* traits.sigma                                   */
    uint64_t seed;            /* Philox-4x32-10 key for device-drawn generations */
} clotho_desc;

/* One generation of the event tape, in the reference's draw order
 * (engine_batched_task.hpp:175-202).  These are the draws the reference's
 * policies make with Boost.Random; given the same tape the engine produces
 * the reference's genomes bit for bit. */
typedef struct clotho_gen_tape {
    uint32_t N;               /* offspring individuals                          */
    uint32_t M;               /* new mutations (mutation_allocator.hpp:41-47)   */
    const uint32_t *pairs;    /* [2N] (id0,id1) parent individuals per offspring
                                 (general_fitness_selection_generator.hpp:104-113) */
    const uint8_t  *swap;     /* [2N] strand-swap bit per gamete (batch_crossover_mtwe.hpp:135-145) */
    const uint32_t *ev_off;   /* [2N+1] event lookup (batch_crossover_mtwe.hpp:117-133) */
    const double   *ev_pos;   /* [ev_off[2N]] breakpoint positions, any order   */
    const uint32_t *mut_seq;  /* [M] target offspring row (batch_mutation_task_population_space_row.hpp:77-81) */
    const double   *mut_pos;  /* [M] allele position in [0,1) (allele_generator_vector.hpp:76-83) */
    const float    *mut_eff;  /* [M*T] allele effects (trait_space_generator.hpp:118-129) */
} clotho_gen_tape;

typedef struct clotho_info {
    uint32_t generation;      /* number of the next generation (age of its mutations) */
    uint32_t N;               /* individuals of the current (child) population  */
    uint32_t A;               /* allele slots (getMaxAlleles)                   */
    uint32_t W;               /* row width in 64-bit words (getMaxBlocks)       */
    uint32_t fixed_count;     /* last free-space analysis (free_space_details.hpp:193-277) */
    uint32_t lost_count;
    uint32_t free_count;
    uint32_t variable_count;
    uint32_t fixed_total;     /* alleles in the fixed table                     */
    uint32_t last_M;          /* mutations of the last generation               */
    uint32_t all_neutral;     /* phenotype was the constant 1.0 path            */
    uint32_t device_error;    /* sticky CLOTHO_DEVERR_* bits                    */
    double   mean_fitness;    /* of the current population                     */
} clotho_info;

/* device error bits reported in clotho_info.device_error */
#define CLOTHO_DEVERR_ALLELES  1u   /* allele capacity exceeded               */
#define CLOTHO_DEVERR_FIXED    2u   /* fixed table capacity exceeded          */
#define CLOTHO_DEVERR_EVENTS   4u   /* more than 128 device-drawn events per gamete */
#define CLOTHO_DEVERR_PARENT   8u   /* tape parent index out of range         */
#define CLOTHO_DEVERR_SEQ     16u   /* tape mutation row out of range         */
#define CLOTHO_DEVERR_MUT     32u   /* mutation capacity exceeded             */
#define CLOTHO_DEVERR_FITNESS 64u   /* all fitness zero: uniform selection used */
#define CLOTHO_DEVERR_STALL  128u   /* a parent strand's asynchronous copy outlived the wait limit
                                       (clotho_set_copy_wait_limit); the warp kept waiting for it, so
                                       the row is complete unless CLOTHO_DEVERR_ABANDONED is also set */
#define CLOTHO_DEVERR_ABANDONED 256u /* such a copy had still not landed after 2^22 more rounds: its
                                       row was written without the parent strand and that warp did no
                                       further rows (the generation is invalid) */

/* ---- lifetime ---------------------------------------------------------- */
int  clotho_create(const clotho_desc *desc, clotho_ctx **out);
int  clotho_destroy(clotho_ctx *ctx);
const char *clotho_last_error(const clotho_ctx *ctx);
/* Device bytes held by the context. */
size_t clotho_footprint(const clotho_ctx *ctx);
/* Bytes a context with this descriptor would allocate (admission control). */
size_t clotho_footprint_for(const clotho_desc *desc);
int  clotho_sync(clotho_ctx *ctx);
/* The stream the context's kernels run on: the caller's cudaStream_t (cast
 * to void *), or NULL for the context's own stream.  Work already queued on
 * the previous stream is finished first.  The caller keeps ownership of its
 * stream and must not destroy it while the context uses it.  The graph calls
 * (clotho_run_philox*) capture on this stream, so it must not be the legacy
 * default stream for them. */
int  clotho_set_stream(clotho_ctx *ctx, void *stream);

/* ---- population set-up ------------------------------------------------- */
/* Engine::init(0) (engine_batched_task.hpp:143-161): N0 individuals, no alleles. */
int  clotho_init(clotho_ctx *ctx, uint32_t N0);
/* Pre-seeded start: A slots with positions pos[A] and effects eff[A*T]; bit
 * (row, slot) is set iff the seed hash of (seed,row,slot) < thr[slot]
 * (splitmix64 finaliser of seed + 0x9E3779B97F4A7C15*((row<<32)+slot+1),
 * upper 32 bits).  Ages are 0.  Phenotypes and fitness are evaluated. */
int  clotho_seed_population(clotho_ctx *ctx, uint32_t N, uint32_t A, const double *pos,
                            const float *eff, const uint32_t *thr, uint64_t seed);

/* Explicit start: rows [2N * ceil(A/512)*8] words in the reference layout
 * (bits at slots >= A are ignored), positions pos[A], effects eff[A*T];
 * ages 0.  Phenotypes and fitness are evaluated. */
int  clotho_load_population(clotho_ctx *ctx, uint32_t N, uint32_t A, const uint64_t *rows,
                            const double *pos, const float *eff);

/* ---- checkpoint / resume --------------------------------------------------
 * The reference keeps its state in host objects and writes logs only
 * (engine_batched_task.hpp:233-242); these calls save and restore one
 * population between generations so that a run can be resumed.  A snapshot
 * holds the description, the status word (generation, sizes, counts), the
 * current rows, the allele and fixed-allele tables, the last free list,
 * per-genome trait sums,
 * phenotypes, fitness and its prefix sum.  Device-drawn generations are keyed
 * by (seed, generation), so a restored population continues bit for bit as
 * the uninterrupted one.  Restore needs a single-population context whose
 * parameters (traits, fitness, flags, fit_param, mu, rho, bias, p_neutral,
 * eff_mean, eff_sigma, seed) equal the snapshot's and whose capacities hold
 * it; clotho_snapshot_size returns 0 when no snapshot can be taken. */
size_t clotho_snapshot_size(clotho_ctx *ctx);
int  clotho_snapshot(clotho_ctx *ctx, void *dst, size_t len);
int  clotho_restore(clotho_ctx *ctx, const void *src, size_t len);

/* ---- fused generation (the hot path) ------------------------------------ */
/* Engine::simulate() (engine_batched_task.hpp:163-223) with the tape standing
 * in for the RNG draws: free space + fixed removal (FreeSpaceAnalyzerMT,
 * updateFixedAlleles :303-345), crossover (BatchCrossoverMTWE), mutation
 * (BatchMutationMT), phenotype (BatchPhenotypeMT) and fitness (GeneralFitness),
 * with no host synchronisation. */
int  clotho_generation_tape(clotho_ctx *ctx, const clotho_gen_tape *tape);
/* The same step with every draw made on the device (Philox-4x32-10 keyed by
 * (seed, generation, stream, index)); parents are sampled by an FP64 inclusive
 * prefix sum of fitness.  N = offspring individuals. */
int  clotho_generation_philox(clotho_ctx *ctx, uint32_t N);
/* G device-drawn generations replayed from one captured CUDA graph. */
int  clotho_run_philox(clotho_ctx *ctx, uint32_t N, uint32_t G);

/* ---- staged entry points (one per reference policy) --------------------- */
/* Start a generation: swap parent/child (engine_batched_task.hpp:164). */
int  clotho_begin_generation(clotho_ctx *ctx, uint32_t N, uint32_t M);
/* FreeSpaceAnalyzerMT::operator() (free_space_mt_population_space_row_interlaced.hpp:41-89)
 * + analyze_free_indices (free_space_details.hpp:299-357) + fixed removal
 * (engine_batched_task.hpp:303-345) + child_max_alleles (:287-301).
 * counts[3] = {fixed, lost, free} (may be NULL). */
int  clotho_free_space(clotho_ctx *ctx, uint32_t *counts);
/* SelectionGenerator::update from tape pairs (general_fitness_selection_generator.hpp:45-69). */
int  clotho_set_pairs(clotho_ctx *ctx, const uint32_t *pairs);
/* SelectionGenerator::update on the device: FP64 prefix sum of the parent
 * fitness and one uniform per draw (2N draws); pairs_out may be NULL. */
int  clotho_select(clotho_ctx *ctx, uint32_t *pairs_out);
/* BatchCrossoverMTWE::operator() (batch_crossover_mtwe.hpp:51-113). */
int  clotho_crossover(clotho_ctx *ctx, const uint8_t *swap, const uint32_t *ev_off,
                      const double *ev_pos);
/* BatchMutationMT::operator() (batch_mutation_mt.hpp:67-81). */
int  clotho_mutate(clotho_ctx *ctx, const uint32_t *mut_seq, const double *mut_pos,
                   const float *mut_eff);
/* BatchPhenotypeMT::operator() (batch_phenotype_mt_population_space_row.hpp:62-72). */
int  clotho_phenotype(clotho_ctx *ctx);
/* GeneralFitness::operator() (general_fitness.hpp:101-119). */
int  clotho_fitness(clotho_ctx *ctx);
/* Finish the generation (++m_generation, engine_batched_task.hpp:222). */
int  clotho_end_generation(clotho_ctx *ctx);

/* ---- read-back (synchronising) ------------------------------------------ */
int  clotho_get_info(clotho_ctx *ctx, clotho_info *out);
/* Asynchronous read-back of the same fields: the request copies the status
 * behind the work issued so far and returns at once with a ticket, so the
 * caller can issue the next generation (and its tape upload) before
 * clotho_info_wait blocks for the copy.  Tickets count up from 0 per context;
 * at most 8 are outstanding (a ninth request waits for the oldest copy).  No
 * reference counterpart: the reference engine returns to its caller only
 * after a generation (engine_batched_task.hpp:163-223). */
int  clotho_info_request(clotho_ctx *ctx, uint32_t *ticket);
int  clotho_info_wait(clotho_ctx *ctx, uint32_t ticket, clotho_info *out);
/* Current child rows, 2N x W words (reference width). */
int  clotho_get_rows(clotho_ctx *ctx, uint64_t *dst, size_t dst_words);
/* Allele table [A]: positions, ages, effects [A*T] (FP32). */
int  clotho_get_alleles(clotho_ctx *ctx, double *pos, uint32_t *age, float *eff);
/* Fixed-allele table [fixed_total]. */
int  clotho_get_fixed(clotho_ctx *ctx, double *pos, uint32_t *age, float *eff);
/* Free list of the last analysis [free_count]: fixed ascending, then lost ascending. */
int  clotho_get_free(clotho_ctx *ctx, uint32_t *dst);
/* Per-genome trait sums [2N*T] and individual phenotypes [N*T]: FP32 partial
 * sums of FP32 effects, accumulated per genome in FP64. */
int  clotho_get_genome_traits(clotho_ctx *ctx, double *dst);
int  clotho_get_phenotypes(clotho_ctx *ctx, double *dst);
int  clotho_get_fitness(clotho_ctx *ctx, double *dst);        /* [N]    */
int  clotho_get_pairs(clotho_ctx *ctx, uint32_t *dst);        /* [2N] of the last generation */

/* ---- statistics (allele_frequency, population_space_row_frequency_evaluator.hpp:37-62) */
typedef struct clotho_stats {
    uint32_t segregating;     /* slots with 0 < count < 2N                      */
    uint32_t fixed_now;       /* slots with count == 2N                         */
    double   mean_fitness;
    double   mean_phenotype[4];
    double   heterozygosity;  /* mean over slots of 2p(1-p) (sum over slots)    */
} clotho_stats;
/* sfs may be NULL; else sfs[k] for k in [0, sfs_len) counts slots carried by
 * exactly k rows (k = 2N folded into the last bin when sfs_len <= 2N). */
int  clotho_stats_compute(clotho_ctx *ctx, clotho_stats *out, uint32_t *sfs, uint32_t sfs_len);
/* Margins of the current rows (population_space_row_frequency_evaluator.hpp:37-62,
 * margin_details.hpp:50-98): col_counts[A] = sequences carrying each allele
 * slot, row_counts[2N] = alleles carried by each sequence.  Either may be NULL. */
int  clotho_margins(clotho_ctx *ctx, uint32_t *col_counts, uint32_t *row_counts);

/* Pairwise differences (association_matrix_pairwise_difference.hpp:75-120,
 * cuda/analysis/pairwise_difference_kernel.hpp:56-339): for every pair i < j
 * of the n sampled rows, the number of allele slots where they differ.
 * sample[n] are row indices (< 2N; NULL = rows 0..n-1), n <= 65,536.  dist,
 * if not NULL, receives the n(n-1)/2 distances in row-major upper-triangle
 * order (pair (i,j) at i*n - i(i+1)/2 + j-i-1); it needs n <= 16,384. */
typedef struct clotho_pairwise {
    uint64_t count;           /* pairs                                          */
    uint64_t total;           /* sum of the distances                           */
    uint32_t min, max;
    double   mean, variance;  /* variance divided by the count (Boost.Accumulators) */
} clotho_pairwise;
int  clotho_pairwise_difference(clotho_ctx *ctx, const uint32_t *sample, uint32_t n, uint32_t *dist,
                                clotho_pairwise *out);

/* ---- timing ------------------------------------------------------------- */
/* CUDA events on the context stream around the fused generation kernel.
 * After enabling, clotho_kernel_time returns total ms and launch count of the
 * dominant kernel since the last reset.  enable = 2 also switches the kernel
 * to its build with phase clocks (clotho_phase_clocks), which runs slower. */
int  clotho_profile(clotho_ctx *ctx, int enable);
int  clotho_kernel_time(clotho_ctx *ctx, double *total_ms, uint32_t *launches,
                        uint64_t *rows_processed, uint64_t *words_processed);
/* Phase cycles of the fused generation kernel while profiling is enabled
 * with enable = 2 (that build clocks every suffix-table row): SM cycles
 * summed over warps, reset by clotho_profile.  out[0..n) receives, in order:
 *   0 copy rows, 1 copy set-up, 2 copy body, 3 copy phenotype,
 *   4 crossover rows, 5 crossover set-up, 6 switch-mask build,
 *   7 crossover body (streaming + gather), 8 effect gather (within 7),
 *   9 crossover phenotype, 10 long-event rows, 11 their cycles,
 *   12 warp residency cycles, 13 warps.
 * No reference counterpart: the reference times whole stages
 * (engine_batched_task.hpp:233-242); here the stages are fused in one kernel.
 * n <= CLOTHO_PHASE_COUNT. */
#define CLOTHO_PHASE_COUNT 14u
int  clotho_phase_clocks(clotho_ctx *ctx, uint64_t *out, uint32_t n);
int  clotho_timer_begin(clotho_ctx *ctx);
int  clotho_timer_end(clotho_ctx *ctx, double *ms);
/* Count of kernels this context launched since creation. */
uint64_t clotho_launch_count(const clotho_ctx *ctx);

/* ---- pinned host memory for tape staging (page-locked, so host->device
 * copies run at link speed).  No reference counterpart: the reference keeps
 * its event pool in ordinary host memory (batch_crossover_mtwe.hpp:80-84). */
int  clotho_host_alloc(size_t bytes, void **out);
int  clotho_host_free(void *p);

/* ---- batched and served populations ------------------------------------
 * One context can hold up to 256 resident populations of uneven N, allele
 * width and trait count.  Every step runs one launch per stage over all of
 * them (the kernels walk a descriptor table), and clotho_batch_run_philox
 * replays the step from one CUDA graph.  Populations join and leave between
 * steps, which is what a continuous-batching serving loop needs.  No reference
 * counterpart: the reference runs one population per process
 * (examples/QTLSim/qtlsim_main.cpp:117-179). */
int  clotho_batch_create(const clotho_desc *descs, uint32_t n, clotho_ctx **out);
uint32_t clotho_pop_count(const clotho_ctx *ctx);
/* Allocate and append a population (its index goes to *index). */
int  clotho_pop_add(clotho_ctx *ctx, const clotho_desc *desc, uint32_t *index);
/* Free a population; later indices shift down by one. */
int  clotho_pop_remove(clotho_ctx *ctx, uint32_t index);
int  clotho_pop_init(clotho_ctx *ctx, uint32_t index, uint32_t N0);
int  clotho_pop_info(clotho_ctx *ctx, uint32_t index, clotho_info *out);
int  clotho_pop_info_request(clotho_ctx *ctx, uint32_t index, uint32_t *ticket);  /* clotho_info_wait */
int  clotho_pop_rows(clotho_ctx *ctx, uint32_t index, uint64_t *dst, size_t dst_words);
int  clotho_pop_stats(clotho_ctx *ctx, uint32_t index, clotho_stats *out, uint32_t *sfs, uint32_t sfs_len);
int  clotho_pop_margins(clotho_ctx *ctx, uint32_t index, uint32_t *col_counts, uint32_t *row_counts);
int  clotho_pop_pairwise_difference(clotho_ctx *ctx, uint32_t index, const uint32_t *sample, uint32_t n,
                                    uint32_t *dist, clotho_pairwise *out);
/* Column counts fused into the generation step.  With enable = 1 every later
 * fused step of population `index` also counts, for each allele slot, the
 * child rows that carry it (bit-sliced counters in the generation kernel's
 * shared memory, added as each child word is finished), so that
 * clotho_pop_stats / clotho_stats_compute read the counts instead of making a
 * pass over the rows (the allele_frequency analysis,
 * population_space_row_frequency_evaluator.hpp:37-62).  The counting build
 * runs while a population asks for it and its rows are at most 712 words;
 * otherwise the statistics count on demand as before.  enable = 0 stops it.
 * Works on single-population contexts with index 0. */
int  clotho_pop_count_columns(clotho_ctx *ctx, uint32_t index, int enable);
/* One device-drawn generation of every population (N[i] offspring). */
int  clotho_batch_generation_philox(clotho_ctx *ctx, const uint32_t *N);
/* G such generations, replayed from one captured CUDA graph. */
int  clotho_batch_run_philox(clotho_ctx *ctx, const uint32_t *N, uint32_t G);
/* G device-drawn generations with a size schedule: N[g * npops + i] offspring
 * individuals of population i in generation g (population growth,
 * predefined_population_growth.cpp:26-28, linear_population_growth.cpp:23-25).
 * One captured CUDA graph serves every generation; the sizes are copied to
 * the device once and each replay reads its own.  Works on single-population
 * and batched contexts. */
int  clotho_run_philox_schedule(clotho_ctx *ctx, const uint32_t *N, uint32_t G);
/* Rounds of mbarrier try_wait a copy row's bulk copy of its parent strand may
 * take before CLOTHO_DEVERR_STALL is raised (0 = the default, 2^22; at most
 * 2^30).  The warp keeps waiting for the copy after that, 2^22 rounds more at
 * most, before it touches the copy's buffer.  A diagnostic knob: a limit of 1
 * makes the flag fire on ordinary copies without changing any result.  No
 * reference counterpart (the reference has no asynchronous copies). */
int  clotho_set_copy_wait_limit(clotho_ctx *ctx, uint32_t rounds);
/* Rows per scheduling item of the generation kernel (autotuner knob of
 * batched contexts; a single-population context has its warps claim one row
 * at a time and ignores it). */
int  clotho_set_rows_per_item(clotho_ctx *ctx, uint32_t rows);
/* Launch shapes chosen by an autotuner (clotho_gb300/autotune.py).  None
 * changes a result: the kernels are deterministic in every shape.
 *   rows_per_item      rows per scheduling item of the generation kernel in
 *                      batched contexts (0 = keep the current value)
 *   narrow_build       1 = run the generation kernel's narrow build when every
 *                      row is at most 128 words (the default), 0 = always the
 *                      wide build
 *   row_blocks_per_sm  blocks per SM of the per-individual kernels of a step
 *                      (parent sampling; phenotype and fitness); 0 = the
 *                      default, 16
 * No reference counterpart: the reference's work partition is its thread
 * pool's fixed batches (thread_pool.hpp:31-139). */
typedef struct clotho_tuning {
    uint32_t rows_per_item;
    uint32_t narrow_build;
    uint32_t row_blocks_per_sm;
} clotho_tuning;
int  clotho_set_tuning(clotho_ctx *ctx, const clotho_tuning *t);
int  clotho_get_tuning(clotho_ctx *ctx, clotho_tuning *t);
/* Free and total device memory (admission control). */
int  clotho_mem_info(size_t *free_bytes, size_t *total_bytes);

/* ---- free-space analysis that allocates nothing --------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (their device memory is owned by another allocator, or allocation is
 * forbidden after start-up): the analysis of clotho_free_space on rows the
 * caller owns, with its working state in a fixed array inside the library.
 *   rows       device pointer, S rows of row_stride_words words (reference
 *              layout; row_stride_words >= ceil(A/512)*8)
 *   free_list  device pointer, room for ceil(A/512)*512 entries: fixed slots
 *              ascending, then lost slots ascending
 *   counts     device pointer to {fixed, lost, free}
 *   stream     cudaStream_t to run on (NULL: the default stream)
 * At most 16,384 words per row (A <= 1,048,576); larger A returns
 * CLOTHO_E_CAPACITY.  The fixed array (256 KB) stays on every device that
 * loaded the library until the process exits.  The first call on a device
 * looks up the array's address; make it before any stream capture (inside a
 * capture it returns CLOTHO_E_STATE).  Calls on a stream that is not
 * capturing look the address up again, so a context made after
 * cudaDeviceReset is followed.  S = 0 reads every slot of every word as
 * lost, as the reference's analysis of an empty population does.  All calls
 * share the array: calls that overlap on the GPU race, so order them on one
 * stream.  Work is enqueued on `stream`; results are ready when it completes. */
int  clotho_free_space_noalloc(const uint64_t *rows, uint32_t S, uint32_t row_stride_words, uint32_t A,
                               uint32_t *free_list, uint32_t *counts, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CLOTHO_GPU_H_ */
