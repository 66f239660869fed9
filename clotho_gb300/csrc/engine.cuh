// engine.cuh -- device data layout and shared device helpers of the GB300
// engine for Clotho's per-generation hot path.
//
// One PopDev describes one resident population.  Every kernel takes an array
// of PopDev and walks all of them, so the plain engine is a batch of one and
// the batched/served forms reuse the same launches.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace clotho {

constexpr uint32_t kMaxTraits = 4;
#ifndef CLOTHO_GEN_THREADS
#define CLOTHO_GEN_THREADS 512
#endif
constexpr uint32_t kGenThreads = CLOTHO_GEN_THREADS;  // one CTA per SM in the generation kernel
constexpr uint32_t kRowsPerItem = 512;     // default child rows per scheduling item (tunable)
constexpr uint32_t kMaxEvReg = 16;         // events held in registers
constexpr uint32_t kMaxEvDevice = 128;     // device-drawn events per gamete
constexpr uint32_t kMaxMutReg = 32;        // mutations per row held in registers
constexpr uint32_t kWordAlign = 64;        // row stride granularity (words)
constexpr uint32_t kSufMaxSlots = 65536;   // allele capacity up to which suffix-table masks are built in per-warp bitmaps
#ifndef CLOTHO_TABLE_MAX_SLOTS
#define CLOTHO_TABLE_MAX_SLOTS (1u << 19)
#endif
// allele capacity up to which a population has a suffix table (above kSufMaxSlots its masks are XORed chunk
// by chunk); at least kSufMaxSlots
constexpr uint32_t kTableMaxSlots = CLOTHO_TABLE_MAX_SLOTS;

// sticky device error bits (CLOTHO_DEVERR_* in clotho_gpu.h)
constexpr uint32_t kErrAlleles = 1u, kErrFixed = 2u, kErrEvents = 4u, kErrParent = 8u,
                   kErrSeq = 16u, kErrMut = 32u, kErrFitness = 64u, kErrStall = 128u, kErrAbandon = 256u;

enum Mode : uint32_t { kModeTape = 0, kModePhilox = 1 };

// Philox counter streams
enum Stream : uint32_t {
    kStreamGamete = 1, kStreamSelect = 2, kStreamMutCount = 3, kStreamMutAllele = 4
};

struct DevStatus {
    uint32_t gen;          // generation number of the step in progress / next step
    uint32_t cur;          // rows buffer holding the current child
    uint32_t N, A, W;      // current child: individuals, alleles, reference width
    uint32_t pN, pA, pW;   // parent of the step in progress
    uint32_t M;            // mutations of the step in progress
    uint32_t fixed_cnt, lost_cnt, free_cnt;
    uint32_t fixed_total;
    int32_t  nz_eff;       // nonzero effect entries in eff[0, A*T)
    uint32_t fs_valid;     // accF/accV hold AND/OR over the current child rows
    uint32_t err;
    uint32_t fit_const;    // every fitness value equal (selection is uniform)
    uint32_t all_neutral;  // phenotype took the constant path
    uint32_t last_M;
    uint32_t ev_used;      // crossover-plan event entries allocated in the step in progress
    uint32_t count_cols;   // the host asked for per-column counts of every fused step's child rows
    uint32_t cols_valid;   // colcnt holds the column counts of the current child rows
    double   fit_total;    // sum of fitness of the current population
    double   fixsum[4];    // effect sums of the alleles fixed in this step's parent
};

struct PopDev {
    uint64_t* rows[2];     // [Scap * Wcap] each
    uint64_t* fixmask;     // [Wcap] fixed columns of the parent
    uint64_t* accF;        // [Wcap] AND over current child rows
    uint64_t* accV;        // [Wcap] OR over current child rows
    uint32_t* free_list;   // [Acap]
    double*   pos;         // [Acap] allele positions (non-negative: ordered as u64)
    uint32_t* age;         // [Acap]
    float*    eff;         // [Acap * 4] effects, traits padded to 4 (unused traits 0)
    double*   fx_pos;      // [FXcap]
    uint32_t* fx_age;      // [FXcap]
    float*    fx_eff;      // [FXcap * T]
    double*   zg[2];       // [Scap * 4] per-genome trait sums, one array per rows buffer
    double*   zi;          // [Ncap * 4] per-individual phenotypes
    double*   fit;         // [Ncap]
    double*   cdf;         // [Ncap]
    double*   scan_part;   // [Ncap / 1024 + 2]
    uint32_t* scan_upart;  // [Scap / 1024 + 2]
    uint32_t* scan_opart;  // [Scap / 1024 + 2] the row-ordering scan's own partials (it runs beside the others)
    uint32_t* pairs;       // [2 * Ncap]
    uint8_t*  swap;        // [Scap]
    uint32_t* ev_off;      // [Scap + 1]
    double*   ev_pos;      // [EVcap]
    uint32_t* mut_seq;     // [Mcap]
    double*   mut_pos;     // [Mcap]
    float*    mut_eff;     // [Mcap * T]
    uint32_t* mut_slot;    // [Mcap]
    uint32_t* row_cnt;     // [Scap + 1] per-row mutation counts (zero between steps)
    uint32_t* row_off;     // [Scap + 1] exclusive prefix of row_cnt
    uint32_t* row_cur;     // [Scap] scatter cursors (zero between steps)
    uint32_t* row_mut;     // [Mcap] mutation indices grouped by row
    uint32_t* bcnt;        // [NB + 1] positions per bucket (zero between steps)
    uint32_t* boff;        // [NB + 1] exclusive prefix of bcnt
    uint32_t* bcur;        // [NB] bucket scatter cursors (zero between steps)
    double*   bpos;        // [Acap] positions grouped by bucket
    uint32_t* bslot;       // [Acap] slot of each bpos entry
    uint32_t* rank;        // [Acap] rank of each slot (position, then slot index) among the A slots
    uint32_t* inv;         // [Acap] slot of each rank (Acap <= kTableMaxSlots, else null)
    uint64_t* suf;         // [(Acap/64 + 1) * Wcap] suffix table of the crossover classifier (Acap <= kTableMaxSlots, else null)
    uint4*    plan_row;    // [Scap] crossover plans in processing order: row, top strand, event base, events | flags << 30
    uint32_t* ord_cnt;     // [Scap + 1] rows per ordering key (zero between steps)
    uint32_t* ord_off;     // [Scap + 1] exclusive prefix of ord_cnt
    uint32_t* ord_cur;     // [Scap] scatter cursors (zero between steps)
    uint32_t* ord_pos;     // [Scap] processing position of each row
    uint32_t* plan_go;     // [EVcap] table row offset per planned event (with suf)
    uint32_t* plan_cr;     // [EVcap] correction ranks per planned event: first | count << 20 (with suf)
    uint2*    plan_mut;    // [Scap] new alleles of the planned row (processing order): CSR offset, count
    double*   plan_z;      // [Scap * 4] phenotype base of the planned row: z(base strand) - sum(fixed)
    uint32_t* colcnt;      // [Acap] per-column counts of the child rows (counting steps)
    DevStatus* st;
    uint32_t Scap, Ncap, Wcap, Acap, Mcap, EVcap, FXcap, T;
    uint32_t NB, pad2;     // position buckets (power of two)
    double mu, rho, bias, p_neutral, eff_mean, eff_sigma, fit_param;
    double exp_neg_rho, exp_neg_mu;   // Poisson inversion seeds, computed on the host
    uint64_t seed;
    int32_t fitness;
    uint32_t flags;
    uint32_t mode;
    uint32_t pad1;
};

// Work control shared by the persistent kernels of one step.
struct WorkCtl {
    uint32_t gen_counter;           // dynamic item counter of k_generation
    uint32_t gen_items;             // total items
    uint32_t rows_per_item;         // scheduling granularity (set by the host)
    uint32_t wait_limit;            // try_wait rounds before a bulk copy is flagged late (0: default)
    uint32_t item_base[257];        // item prefix per population (<= 256 pops)
    uint32_t gen_counter_iv;        // item counter of the interval-classifier pass of a mixed batch
    uint32_t gen_counter_cm;        // item counter of the chunk-mask pass of a mixed batch
    uint64_t rows_done;             // profiling: rows processed
    uint64_t words_done;            // profiling: words written
    uint64_t phase[16];             // profiling: k_generation phase cycles (kPh*)
};

// Phase counters of the profiling build of k_generation (suffix-table rows):
// SM cycles summed over warps, per kind of row, and the rows of each kind.
enum : uint32_t {
    kPhCopyRows = 0, kPhCopySetup, kPhCopyBody, kPhCopyPheno,
    kPhXoRows, kPhXoSetup, kPhXoMask, kPhXoBody, kPhXoGather, kPhXoPheno,
    kPhLongRows, kPhLongCyc, kPhWarpCyc, kPhWarps, kPhCount
};

constexpr uint32_t kMaxPops = 256;

// ---------------------------------------------------------------------------
// small helpers

__host__ __device__ inline uint32_t ref_width(uint32_t A) {
    // population_space_row::setMaxAlleles (population_space_row_block.hpp:94-101)
    return ((A + 511u) / 512u) * 8u;
}

__device__ inline uint64_t dkey(double d) { return (uint64_t)__double_as_longlong(d); }

// seed rule shared with the oracle (orc_seed_hash)
__host__ __device__ inline uint32_t seed_hash(uint64_t seed, uint32_t row, uint32_t slot) {
    uint64_t x = seed + 0x9E3779B97F4A7C15ull * ((((uint64_t)row) << 32) + (uint64_t)slot + 1ull);
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (uint32_t)(x >> 32);
}

// Philox-4x32-10 counter-based generator, written from the published
// description (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): multipliers 0xD2511F53/0xCD9E8D57, Weyl key increments
// 0x9E3779B9/0xBB67AE85, ten rounds.
struct U4 { uint32_t x, y, z, w; };

__device__ inline U4 philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t key) {
    uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

// [0,1) double from 53 random bits: v * 2^-53, assembled as IEEE-754 bits with
// integer operations (exactly the value of the FP64 conversion and scaling, which
// would occupy GB300's narrow FP64 pipe).
__device__ inline double u01(uint32_t hi, uint32_t lo) {
    const uint64_t v = ((((uint64_t)hi) << 32) | lo) >> 11;
    const int msb = 63 - __clzll((long long)(v | 1ull));          // highest set bit, 0..52
    const uint64_t frac = (v << (52 - msb)) & 0x000FFFFFFFFFFFFFull;
    const uint64_t bits = ((uint64_t)(1023 - 53 + msb) << 52) | frac;
    return __longlong_as_double((long long)(v ? bits : 0ull));
}

// x < y for non-negative, non-NaN doubles, as an integer compare of their bit
// patterns (IEEE-754 order); exact, and off the FP64 pipe.
__device__ inline bool lt_nonneg(double x, double y) {
    return (unsigned long long)__double_as_longlong(x) < (unsigned long long)__double_as_longlong(y);
}

// 1/k for the Poisson inversion (k = 1..kRecip-1); multiplying by it avoids
// FP64 divisions, which are slow on this part.  Every translation unit that
// draws Poisson numbers has its own copy (no relocatable device code), filled
// on the current device by that unit's init_recip_* function.
constexpr uint32_t kRecip = 256;
static __constant__ double c_recip[kRecip];
static inline int fill_recip_table() {
    double h[kRecip];
    h[0] = 0.0;
    for (uint32_t k = 1; k < kRecip; ++k) h[k] = 1.0 / (double)k;
    return cudaMemcpyToSymbol(c_recip, h, sizeof(h)) == cudaSuccess ? 0 : -1;
}

// Poisson draw by sequential inversion of the CDF; e = exp(-lambda) from the
// host.  Used only for small means (per-gamete events, per-row mutations).
// One step of the Poisson CDF recurrence p_k = p_{k-1} lambda / k, F_k = F_{k-1} + p_k, with
// explicitly rounded operations (never contracted into FMAs), so every copy of it -- the inversion
// loop and the plan kernel's table -- gives the same bits.
__device__ inline void poisson_step(double& p, double& F, double lambda, uint32_t k) {
    p = __dmul_rn(p, __dmul_rn(lambda, k < kRecip ? c_recip[k] : 1.0 / (double)k));
    F = __dadd_rn(F, p);
}

__device__ inline uint32_t poisson_inv(double u, double lambda, double e) {
    double p = e, F = e;
    uint32_t k = 0;
    while (u > F && k < 4096u) {
        ++k;
        poisson_step(p, F, lambda, k);
    }
    return k;
}

__device__ inline uint32_t lane_id() { return threadIdx.x & 31u; }

// Monotone bucket of a position in [0,1) (values outside are clamped).
// floor(x * NB) for x in (0, 1), from the bits with integer operations: 0 for
// x <= 0 (and subnormals), NB - 1 for x >= 1.  Monotone, which is all the
// bucket index needs (the rank kernels and the threshold search use this one
// function; ranks are exact within a bucket), and off the FP64 pipe.
__device__ inline uint32_t pos_bucket(double x, uint32_t NB) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    if ((b >> 63) || b == 0ull) return 0u;
    const int ex = (int)((b >> 52) & 0x7FFu) - 1023;                     // x = 1.f * 2^ex
    if (ex >= 0) return NB - 1u;
    const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);      // 53-bit significand
    const int sh = -ex - 1;                                              // x * 2^53 = m >> sh
    const uint64_t v = sh >= 64 ? 0ull : (m >> sh);
    const uint32_t k = (uint32_t)__umul64hi(v << 11, (uint64_t)NB);     // floor(v * NB / 2^53)
    return k < NB - 1u ? k : NB - 1u;
}

// x < y for positions (doubles >= 0, -0.0 included) as an integer compare of
// the bit patterns with the sign cleared.
__device__ inline bool pos_lt(double x, double y) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull) <
           ((unsigned long long)__double_as_longlong(y) & 0x7FFFFFFFFFFFFFFFull);
}

}  // namespace clotho

// ---------------------------------------------------------------------------
// Host-side launch wrappers (defined in the kernel translation units).
namespace clotho {
struct LaunchCfg {
    cudaStream_t stream;
    int num_sms;
    uint32_t ind_per_sm = 16;     // blocks per SM of the per-individual kernels (selection, fitness)
    bool narrow_ok = true;        // the narrow build of k_generation may run when every row fits it
};

// Population-parallel launches: blockIdx.z walks the populations, so small
// populations of a batch run side by side; blockIdx.x (and .y) stride inside
// one population.  per_pop bounds the useful blocks of one population.
inline dim3 pop_grid(uint32_t npops, uint32_t per_pop, int num_sms, uint32_t per_sm = 4) {
    const uint32_t gz = npops < 1u ? 1u : (npops > 65535u ? 65535u : npops);
    uint32_t gx = (uint32_t)num_sms * per_sm / gz;
    if (gx > per_pop) gx = per_pop;
    if (gx < 1u) gx = 1u;
    return dim3(gx, 1u, gz);
}
inline uint32_t blocks_for(uint64_t n, uint32_t per_block) {
    const uint64_t b = (n + per_block - 1) / per_block;
    return b < 1 ? 1u : (b > 0x7fffffffull ? 0x7fffffffu : (uint32_t)b);
}
// which: 0 = current child rows, 1 = parent rows of the step in progress
void launch_fs_reduce(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxW, uint32_t which);
// count_on: the step's generation kernel counts columns for the populations that asked (see
// generation_counts_fit); their counts are zeroed here and marked valid
void launch_fs_finalize(const LaunchCfg&, const PopDev* pops, uint32_t npops, bool count_on = false);
void launch_begin(const LaunchCfg&, const PopDev* pops, uint32_t npops, const uint32_t* hdr,
                  WorkCtl* ctl);
void launch_mut_csr_tape(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxS);
void launch_mut_counts_philox(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxS);
void launch_mut_resolve(const LaunchCfg&, const PopDev* pops, uint32_t npops);
void launch_select_philox(const LaunchCfg&, const PopDev* pops, uint32_t npops);
// Generation-kernel builds: suffix-table masks in per-warp bitmaps (capacity <= kSufMaxSlots), chunk by
// chunk from the table (populations with a table above that), interval classifier (populations without a
// table).  mixed: the batch holds populations of more than one kind; this launch runs only the populations
// of its own kind (build; maxW, maxA are theirs) and skips the others' items, so each population keeps the
// build it runs alone whatever it is batched with
enum GenBuild : int { kBuildInterval = 0, kBuildBitmap = 1, kBuildChunk = 2 };
cudaError_t launch_generation(const LaunchCfg&, const PopDev* pops, uint32_t npops, WorkCtl* ctl,
                              uint32_t maxW, uint32_t maxA, uint32_t fuse, int profile, GenBuild build,
                              bool count_on = false, bool mixed = false);
// whether the generation kernel's counting build fits this launch (suffix-table rows, counters in shared memory)
bool generation_counts_fit(uint32_t maxW, uint32_t maxA);
void launch_mut_scatter(const LaunchCfg&, const PopDev* pops, uint32_t npops);
void launch_phenotype(const LaunchCfg&, const PopDev* pops, uint32_t npops);
void launch_individuals(const LaunchCfg&, const PopDev* pops, uint32_t npops);
void launch_cdf(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxN);
void launch_end(const LaunchCfg&, const PopDev* pops, uint32_t npops);
void launch_seed_rows(const LaunchCfg&, const PopDev* pops, uint32_t npops, const uint32_t* thr,
                      uint64_t seed, uint32_t A);
void launch_stats(const LaunchCfg&, const PopDev* pops, uint32_t p, uint32_t* counts, uint32_t A);
void launch_row_counts(const LaunchCfg&, const PopDev* pops, uint32_t p, uint32_t* counts, uint32_t S);
// device accumulators of the pairwise-difference kernel
struct PairwiseOut {
    unsigned long long count, total, sumsq;
    unsigned int min, max;
};
void launch_pairwise(const LaunchCfg&, const PopDev* pops, uint32_t p, const uint32_t* sample, uint32_t n,
                     uint32_t* dist, PairwiseOut* out);
void launch_ranks(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxNB, uint32_t maxW, bool suf);
void launch_uscan_buckets(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxNB);
void launch_uscan_order(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxS);

void launch_plan(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxS);
// the two halves of launch_plan: the rows' processing order (by parent; needs only the pairs and the step
// header) and the per-row plans (needs the ranks, the suffix tables and the new alleles as well)
void launch_order(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxS);
void launch_row_plan(const LaunchCfg&, const PopDev* pops, uint32_t npops, uint32_t maxS);
int init_recip_step();  // k_step.cu's copy of the reciprocal table
int init_recip_gen();   // k_generation.cu's copy

// crossover-plan row flags
constexpr uint32_t kPlanInv = 1u, kPlanLong = 2u, kPlanFlagShift = 30u;
constexpr uint32_t kPlanMaxEvents = (1u << kPlanFlagShift) - 1u;

// fuse flags of k_generation
constexpr uint32_t kFuseMut = 1u, kFusePheno = 2u, kFuseFs = 4u;
}  // namespace clotho
