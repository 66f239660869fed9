// k_generation.cu -- the fused generation pass: one warp builds one offspring
// row in a single sweep over its parent's two rows.
//
// Per row (gamete g of mate pair g/2, parent individual pairs[g]):
//   crossover  batch_crossover_taskwe<...population_space_row>::run_crossover_task
//              (crossover/batch_crossover_taskwe_population_space_row.hpp:157-217)
//              and block_crossover::crossover (crossover/block_crossover.hpp:46-63):
//              a heterozygous bit takes the bottom strand iff an odd number of
//              breakpoints is <= its position (upper_bound in region_classifier,
//              classifiers/region_classifier.hpp:62-77).  Positions are replaced by
//              integer ranks: rank(s) = #{slots t with pos(t) < pos(s), or equal
//              position and t < s} (a bijection onto [0, A)); breakpoint e becomes
//              r(e) = #{slots with pos < e}, and e <= pos(s)  <=>  r(e) <= rank(s)
//              for every slot, ties included.  Fixed columns are masked on load:
//              the in-register form of remove_fixed_allele
//              (population_space_row_block.hpp:127-147).
//   mutation   XOR of the row's new alleles (population_space_row_block.hpp:111-125)
//              in registers before the store.
//   phenotype  z(child) = z(top strand) - sum(fixed) + sum(switched bits: bottom-top)
//              + sum(new alleles): the per-genome sum of
//              batch_phenotype_task_population_space_row.hpp:127-153, carried
//              from the parent row instead of re-walking every set bit.
//              Per-lane FP32 partial sums reduced across the warp in FP32,
//              FP64 per-genome values.
//   free space AND/OR of the finished words, the next generation's
//              FreeSpaceAnalyzerMT input (free_space_task_population_space_row_interlaced.hpp:51-72).
//
// Two crossover classifiers:
//   suffix table (A <= 524,288 slots): the switch mask of a gamete with rank
//              thresholds r_1..r_E is XOR_k G(r_k), G(r) = {slots with rank >= r}.
//              G at every multiple of 64 is a per-generation table in L2
//              (suf[g * Wcap + w], built by k_suf_build); G(r) differs from the
//              nearest table row by at most 32 slots, which the warp toggles in
//              its own correction bitmap in shared memory.  Per word: E table
//              loads and XORs, no per-bit work.  Rows too wide for a bitmap per
//              warp (A > 65,536) take each chunk's mask words straight from the
//              table and toggle the correction slots that fall in the chunk
//              (chunk-mask build); their copy rows stream through registers.
//   intervals  (wider allele spaces): sorted thresholds pair into half-open rank
//              intervals; every heterozygous bit is classified by its rank.
//
// Rows are 64-word chunks, two words (one 128-bit load) per lane; a crossover
// row's parent words are loaded one chunk ahead of use and the whole parent row
// is prefetched into L2 at row start.  Effects of switched alleles are gathered
// from a per-warp queue, kRoundLane entries per lane a round, so lanes stay
// balanced.  The kernel is persistent, one CTA per SM: with one population each
// warp claims rows one at a time from a device counter; a batch hands each CTA
// items of rows, which its warps claim one at a time.
#include "engine.cuh"

#include <algorithm>
#include <mutex>

namespace clotho {

namespace {

constexpr int kMaxGenDevices = 64;

// Rare paths: inlined (measured faster than out-of-line calls for this kernel).
#define CLOTHO_COLD __forceinline__

constexpr uint32_t kWarps = kGenThreads / 32;
constexpr uint32_t kMaxIvSmem = 64;     // rank intervals in shared memory (E <= 128)
constexpr uint32_t kMaxIv = 8;          // rank intervals held in registers (E <= 16)
constexpr uint32_t kQueueCap = 512;     // entries of the per-warp queue (power of two)

// ---------------------------------------------------------------------------
// shared pieces

// L2 prefetch of [p, p + bytes) in 2 KB pieces, one piece per lane.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t off = lane * 2048u;
    if (off < bytes) {
        const uint32_t n = min(2048u, bytes - off);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<const char*>(p) + off),
                     "r"(n)
                     : "memory");
    }
}

// d += (+1 if the bottom strand brings the allele, -1 if it drops it) * eff
// over the switched bits of the lane's two words; two chains, two loads in flight.
__device__ __forceinline__ void switched_effects(uint64_t x0, uint64_t x1, uint64_t b0, uint64_t b1, uint32_t s0,
                                                 const float4* __restrict__ eff4, float (&d)[kMaxTraits]) {
    while (x0 | x1) {
        const bool n0 = x0 != 0ull, n1 = x1 != 0ull;
        const uint32_t j0 = n0 ? (uint32_t)(__ffsll((long long)x0) - 1) : 0u;
        const uint32_t j1 = n1 ? (uint32_t)(__ffsll((long long)x1) - 1) : 0u;
        x0 &= x0 - 1ull;
        x1 &= x1 - 1ull;
        const float4 e0 = __ldg(eff4 + s0 + j0);
        const float4 e1 = __ldg(eff4 + s0 + 64u + j1);
        const float g0 = n0 ? (((b0 >> j0) & 1ull) ? 1.0f : -1.0f) : 0.0f;
        const float g1 = n1 ? (((b1 >> j1) & 1ull) ? 1.0f : -1.0f) : 0.0f;
        d[0] = fmaf(g0, e0.x, fmaf(g1, e1.x, d[0]));
        d[1] = fmaf(g0, e0.y, fmaf(g1, e1.y, d[1]));
        d[2] = fmaf(g0, e0.z, fmaf(g1, e1.z, d[2]));
        d[3] = fmaf(g0, e0.w, fmaf(g1, e1.w, d[3]));
    }
}

// Bits of h whose slot position is >= an odd number of the events (direct
// double compares against the event list; used only for very long lists).
__device__ __forceinline__ uint64_t sw_mask_events(uint64_t h, uint32_t base, const double* __restrict__ pos,
                                                   const double* __restrict__ ev, uint32_t E) {
    uint64_t m = 0;
    while (h) {
        const uint32_t j = (uint32_t)(__ffsll((long long)h) - 1);
        h &= h - 1ull;
        const double p = __ldg(pos + base + j);
        uint32_t c = 0;
        for (uint32_t k = 0; k < E; ++k) c += (__ldg(ev + k) <= p) ? 1u : 0u;
        m |= (uint64_t)(c & 1u) << j;
    }
    return m;
}

// r(e) = #{slots with position < e} through the position buckets.
__device__ __forceinline__ uint32_t threshold_rank(const PopDev& P, double e) {
    const uint32_t b = pos_bucket(e, P.NB);
    const uint32_t k0 = __ldg(P.boff + b), k1 = __ldg(P.boff + b + 1u);
    uint32_t r = k0;
    for (uint32_t k = k0; k < k1; ++k) r += pos_lt(__ldg(P.bpos + k), e) ? 1u : 0u;
    return r;
}

struct RowArgs {
    const uint64_t* top;
    const uint64_t* bot;
    uint64_t* out;
    uint32_t Wc, Wp;
    uint32_t mc, mo, my_slot;
    uint32_t E;
    uint32_t topr;
    double zbase;         // lanes 0..3: z(top strand) - sum(fixed effects), trait = lane
    const double* evg;
    bool philox;
};

__device__ __forceinline__ void load_pair(ulonglong2& t, ulonglong2& b, const RowArgs& R, uint32_t w, bool xo) {
    if (w < R.Wp) {
        t = __ldg(reinterpret_cast<const ulonglong2*>(R.top + w));
        b = xo ? __ldg(reinterpret_cast<const ulonglong2*>(R.bot + w)) : make_ulonglong2(0, 0);
    } else {
        t = make_ulonglong2(0, 0);
        b = make_ulonglong2(0, 0);
    }
}

// AND/OR into the CTA accumulators; the atomic is issued only when it would
// change the word (both operations are monotone, so skipping is exact).
__device__ __forceinline__ void fold_fs(uint64_t* sF, uint64_t* sV, uint32_t w, uint64_t x0, uint64_t x1) {
    const ulonglong2 f = *reinterpret_cast<const ulonglong2*>(sF + w);
    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(sV + w);
    if (f.x & ~x0) atomicAnd((unsigned long long*)&sF[w], (unsigned long long)x0);
    if (f.y & ~x1) atomicAnd((unsigned long long*)&sF[w + 1u], (unsigned long long)x1);
    if (x0 & ~v.x) atomicOr((unsigned long long*)&sV[w], (unsigned long long)x0);
    if (x1 & ~v.y) atomicOr((unsigned long long*)&sV[w + 1u], (unsigned long long)x1);
}

// Per-column counts of the finished child words, bit-sliced: plane b (cnt + b * stride) holds bit b of every
// column's count in the CTA since its last flush.  Adding a word is a ripple-carry increment of every column
// whose bit is set; each step is an atomic XOR whose old value gives the carry, so adds from other warps
// interleave exactly.  Up to 2^kCountPlanes - 1 rows between flushes.
constexpr uint32_t kCountPlanes = 16;

__device__ __forceinline__ void count_add(uint64_t* cnt, uint32_t stride, uint32_t w, uint64_t x0, uint64_t x1) {
    unsigned long long c0 = x0, c1 = x1;
    for (uint32_t b = 0; b < kCountPlanes && (c0 | c1); ++b) {
        unsigned long long* pl = reinterpret_cast<unsigned long long*>(cnt + (size_t)b * stride + w);
        if (c0) c0 &= atomicXor(pl, c0);
        if (c1) c1 &= atomicXor(pl + 1, c1);
    }
}

// What the free-space epilogue folds a finished word pair into: the AND/OR accumulators and, in the
// counting build, the column-count planes (cnt null otherwise, and the branch folds away).
struct Fold {
    uint64_t* F;
    uint64_t* V;
    uint64_t* cnt;
    uint32_t stride;
};
__device__ __forceinline__ void fold(const Fold& fo, uint32_t w, uint64_t x0, uint64_t x1) {
    fold_fs(fo.F, fo.V, w, x0, x1);
    if (fo.cnt) count_add(fo.cnt, fo.stride, w, x0, x1);
}
constexpr uint32_t kCountMax = (1u << kCountPlanes) - 1u;   // rows a CTA may add between flushes

// Adds the CTA's counters of words [0, W) to the population's column counts colcnt[0, A) and clears them.
// The whole block calls it, after a barrier (every add is done) and before one (the planes are reused).
__device__ __noinline__ void count_flush(uint64_t* planes, uint32_t stride, uint32_t W, uint32_t A,
                                         uint32_t* __restrict__ colcnt) {
    for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) {
        uint64_t pl[kCountPlanes];
        uint64_t any = 0;
#pragma unroll
        for (uint32_t b = 0; b < kCountPlanes; ++b) {
            pl[b] = planes[(size_t)b * stride + w];
            planes[(size_t)b * stride + w] = 0ull;
            any |= pl[b];
        }
        for (uint64_t m = any; m; m &= m - 1ull) {
            const uint32_t j = (uint32_t)(__ffsll((long long)m) - 1);
            uint32_t c = 0;
#pragma unroll
            for (uint32_t b = 0; b < kCountPlanes; ++b) c |= (uint32_t)((pl[b] >> j) & 1ull) << b;
            const uint32_t slot = w * 64u + j;
            if (slot < A) atomicAdd(colcnt + slot, c);
        }
    }
}

// XOR masks of the lane's two words (w, w+1) from the row's new alleles.
// Called by the whole warp (the shuffles need every lane).
__device__ __forceinline__ void mutation_masks(const PopDev& P, const DevStatus& st, const RowArgs& R, uint32_t w,
                                               uint64_t& mx0, uint64_t& mx1) {
    mx0 = 0;
    mx1 = 0;
    const uint32_t lim = R.mc < 32u ? R.mc : 32u;
    for (uint32_t j = 0; j < lim; ++j) {
        const uint32_t s = __shfl_sync(0xffffffffu, R.my_slot, j);
        if (s == 0xffffffffu) continue;
        const uint32_t sw = s >> 6;
        if (sw == w) mx0 ^= 1ull << (s & 63u);
        else if (sw == w + 1u) mx1 ^= 1ull << (s & 63u);
    }
    for (uint32_t j = 32; j < R.mc; ++j) {  // rows with more than 32 new alleles
        const uint32_t mi = R.philox ? R.mo + j : P.row_mut[R.mo + j];
        if (mi >= st.M) continue;
        const uint32_t s = P.mut_slot[mi];
        if (s == 0xffffffffu) continue;
        const uint32_t sw = s >> 6;
        if (sw == w) mx0 ^= 1ull << (s & 63u);
        else if (sw == w + 1u) mx1 ^= 1ull << (s & 63u);
    }
}

__device__ __forceinline__ void row_mutation_setup(const PopDev& P, const DevStatus& st, uint32_t g, bool do_mut,
                                                   bool gather, RowArgs& R, float (&d)[kMaxTraits]);

// Parents, strand swap and breakpoint count of gamete g (interval classifier);
// the new alleles of the row (lanes hold up to 32 slot indices) and their effects.
__device__ __forceinline__ void row_setup(const PopDev& P, const DevStatus& st, uint32_t g, bool do_mut,
                                          bool do_ph, bool gather, RowArgs& R, float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t* prow = P.rows[st.cur ^ 1u];
    const bool q1 = (P.flags & 1u) != 0;
    const bool philox = P.mode == kModePhilox;
    uint32_t pind = P.pairs[g];
    if (pind >= st.pN) {
        if (lane == 0) atomicOr(&P.st->err, kErrParent);
        pind = 0;
    }
    const uint32_t h = g & 1u;
    bool swap;
    uint32_t E;
    const double* evg = nullptr;
    if (philox) {
        const U4 x = philox4x32(g, 0u, st.gen, kStreamGamete, P.seed);
        E = poisson_inv(u01(x.x, x.y), P.rho, P.exp_neg_rho);
        swap = u01(x.z, x.w) < P.bias;
        if (q1 && h) E = 0;
        if (E > kMaxEvDevice) {
            if (lane == 0) atomicOr(&P.st->err, kErrEvents);
            E = kMaxEvDevice;
        }
    } else {
        swap = P.swap[g] != 0;
        const uint32_t e0 = P.ev_off[g], e1 = P.ev_off[g + 1u];
        E = (q1 && h) ? 0u : e1 - e0;
        evg = P.ev_pos + e0;
    }
    const uint32_t topr = 2u * pind + (swap ? 1u : 0u);
    R.topr = topr;
    R.top = prow + (size_t)topr * P.Wcap;
    R.bot = prow + (size_t)(topr ^ 1u) * P.Wcap;
    R.out = P.rows[st.cur] + (size_t)g * P.Wcap;
    R.Wc = st.W;
    R.Wp = st.pW;
    R.E = E;
    R.evg = evg;
    R.philox = philox;
    R.zbase = 0.0;
    if (do_ph && lane < kMaxTraits)
        R.zbase = P.zg[st.cur ^ 1u][(size_t)topr * 4u + lane] - P.st->fixsum[lane];
    row_mutation_setup(P, st, g, do_mut, gather, R, d);
}

// The new alleles of row g (lanes hold up to 32 slot indices) and their effects.
// The new alleles of the row: CSR range [mo, mo + mc) of the mutation list.
__device__ __forceinline__ void row_mutation_setup(const PopDev& P, const DevStatus& st, uint32_t mo, uint32_t mc,
                                                   bool do_mut, bool gather, RowArgs& R, float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool philox = R.philox;
    R.mo = 0;
    R.mc = 0;
    R.my_slot = 0xffffffffu;
    const float4* eff4 = reinterpret_cast<const float4*>(P.eff);
    if (do_mut) {
        R.mo = mo;
        R.mc = mc;
        if (lane < R.mc) {
            const uint32_t i = R.mo + lane;
            const uint32_t mi = philox ? i : P.row_mut[i];
            R.my_slot = (mi < st.M) ? P.mut_slot[mi] : 0xffffffffu;
            if (gather && R.my_slot != 0xffffffffu) {
                const float4 e = __ldg(eff4 + R.my_slot);
                d[0] += e.x; d[1] += e.y; d[2] += e.z; d[3] += e.w;
            }
        }
        if (gather && R.mc > 32u && lane == 0) {
            for (uint32_t j = 32; j < R.mc; ++j) {
                const uint32_t mi = philox ? R.mo + j : P.row_mut[R.mo + j];
                if (mi >= st.M) continue;
                const uint32_t s = P.mut_slot[mi];
                if (s == 0xffffffffu) continue;
                const float4 e = __ldg(eff4 + s);
                d[0] += e.x; d[1] += e.y; d[2] += e.z; d[3] += e.w;
            }
        }
    }
}

__device__ __forceinline__ void row_mutation_setup(const PopDev& P, const DevStatus& st, uint32_t g, bool do_mut,
                                                   bool gather, RowArgs& R, float (&d)[kMaxTraits]) {
    const uint32_t mo = do_mut ? P.row_off[g] : 0u;
    row_mutation_setup(P, st, mo, do_mut ? P.row_off[g + 1u] - mo : 0u, do_mut, gather, R, d);
}

// Breakpoint k of the row as a double.
__device__ __forceinline__ double row_event(const PopDev& P, const DevStatus& st, const RowArgs& R, uint32_t g,
                                            uint32_t k) {
    if (R.philox) {
        const U4 a = philox4x32(g, 1u + (k >> 1), st.gen, kStreamGamete, P.seed);
        return (k & 1u) ? u01(a.z, a.w) : u01(a.x, a.y);
    }
    return __ldg(R.evg + k);
}

// z(child genome g) = z(top strand) - sum(fixed effects) + the row's delta (FP64 warp sum).
#ifndef CLOTHO_PHENO_F32
#define CLOTHO_PHENO_F32 1
#endif
__device__ __forceinline__ void row_phenotype(const PopDev& P, const DevStatus& st, uint32_t g, const RowArgs& R,
                                              const float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    double z[kMaxTraits] = {0.0, 0.0, 0.0, 0.0};
    // a copy row without new alleles has nothing to add: one vote instead of the reduction
    const bool any = __any_sync(0xffffffffu, (d[0] != 0.f) | (d[1] != 0.f) | (d[2] != 0.f) | (d[3] != 0.f));
    if (any) {
#if CLOTHO_PHENO_F32
        // the lanes' FP32 sums are reduced in FP32 (GB300's FP64 pipe is narrow); the row's phenotype stays FP64
#pragma unroll
        for (uint32_t t = 0; t < kMaxTraits; ++t) {
            float v = d[t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            z[t] = (double)v;
        }
#else
#pragma unroll
        for (uint32_t t = 0; t < kMaxTraits; ++t) {
            double v = (double)d[t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            z[t] = v;
        }
#endif
    }
    if (lane < kMaxTraits) {
        const double zz = lane == 0 ? z[0] : lane == 1 ? z[1] : lane == 2 ? z[2] : z[3];
        P.zg[st.cur][(size_t)g * 4u + lane] = R.zbase + zz;
    }
}

// ---------------------------------------------------------------------------
// Suffix-table rows.
//
// Setup builds the row's whole switch mask in the warp's mask bitmap (shared
// memory, one bit per slot): the correction slots of every breakpoint are
// toggled first, then XOR_k suf[g_k] is folded in, many table loads in flight
// at a time.  The streaming loop reads (and clears) two mask words per lane
// per chunk, so it waits on nothing but the parent words, which are loaded
// one chunk ahead.
//
// Effects of switched alleles go through the per-warp queue (slot | sign << 31)
// and are gathered kRoundLane per lane a round (loads folded in one round later).  A row gathers the smaller of two sets: the
// switched heterozygous bits (z = z(top) + sum (bottom - top) w), or, when the
// breakpoints switch more than half of the rank space, the unswitched ones
// (z = z(bottom) + sum (top - bottom) w); both give the same phenotype up to
// FP32 rounding.

struct WarpSmem {
    uint32_t q[kQueueCap];            // effect queue: slot | sign << 31
    unsigned long long mbar;          // completion barrier of the warp's bulk copies
    uint32_t dead;                    // a bulk copy of this warp never landed: it does no further row
    uint32_t pad;
};

// Copy rows of the bitmap builds: 1 = one bulk copy of the parent strand into the warp's bitmap,
// 0 = register streaming six chunks deep (what the chunk-mask build, which has no bitmaps, always does)
#ifndef CLOTHO_COPY_BULK
#define CLOTHO_COPY_BULK 1
#endif

// ---- bulk copies (cp.async.bulk) into the warp's bitmap, completed on an mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
constexpr uint32_t kWaitLimit = 1u << 22;   // default try_wait rounds before a copy is flagged late

__device__ __forceinline__ bool mbar_test_wait(unsigned long long* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Waits for the phase of the warp's barrier.  Round 1 is a probe that does not wait (test_wait),
// later rounds are try_waits.  A copy still in flight after `limit` unsuccessful rounds sets
// kErrStall and is waited for kWaitLimit rounds more, so its buffer is never touched while the copy
// can still land; if it has not landed by then, kErrAbandon is set and the result is false (the
// whole warp agrees).  No wait is unbounded.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t& phase, uint32_t* err,
                                          const uint32_t* wait_limit) {
    bool ok = true;
    if (!mbar_test_wait(bar, phase)) {
        // the limit is read only here, off the path of copies that have landed by the first probe
        const uint32_t lim = *wait_limit, limit = lim ? lim : kWaitLimit;
        for (uint32_t it = 1;; ++it) {
            if (it == limit) atomicOr(err, kErrStall);
            if (it >= limit + kWaitLimit) {
                atomicOr(err, kErrAbandon);
                ok = false;
                break;
            }
            if (mbar_try_wait(bar, phase)) break;
        }
    }
    ok = __all_sync(0xffffffffu, ok);
    if (ok) phase ^= 1u;
    return ok;
}

__device__ __forceinline__ void add4(float (&d)[kMaxTraits], const float4& e) {
    d[0] += e.x;
    d[1] += e.y;
    d[2] += e.z;
    d[3] += e.w;
}

__device__ CLOTHO_COLD float4 effects_direct(uint64_t m0, uint64_t m1, uint64_t b0, uint64_t b1, uint32_t s0,
                                              const float4* __restrict__ eff4) {
    float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
    switched_effects(m0, m1, b0, b1, s0, eff4, d);
    return make_float4(d[0], d[1], d[2], d[3]);
}

#ifndef CLOTHO_ROUND_LANE
#define CLOTHO_ROUND_LANE 3
#endif
#ifndef CLOTHO_TABLE_INFLIGHT
#define CLOTHO_TABLE_INFLIGHT 16
#endif
constexpr uint32_t kRoundLane = CLOTHO_ROUND_LANE;   // queue entries gathered per lane per round
constexpr uint32_t kRound = 32u * kRoundLane;
constexpr uint32_t kTableInflight = CLOTHO_TABLE_INFLIGHT;
constexpr uint32_t kFlatLoads = 4;   // table loads per lane when a narrow row's whole mask is built at once
constexpr uint32_t kDirectCopyChunks = 2;   // copy rows up to 128 words load their strand directly
constexpr uint32_t kCmMaxEv = 16;           // chunk-mask build: breakpoints a row takes through the table
constexpr uint32_t kCmCorr = 32u * kCmMaxEv;   // chunk-mask build: correction slots a warp holds
constexpr uint32_t kCmAccWords = 3072;      // chunk-mask build: widest rows folded in shared memory
#ifndef CLOTHO_WARP_CHUNK
#define CLOTHO_WARP_CHUNK 1
#endif
constexpr uint32_t kWarpChunk = CLOTHO_WARP_CHUNK;   // rows a warp claims at a time (one population)

// A gather round in flight: its effects are loaded when the round is issued
// and folded into the sums one round later, so the loads have a chunk of work
// to land behind.
struct EffRound {
    float4 ef[kRoundLane];
    uint32_t sg;  // bit k: entry k is added (else subtracted); an empty entry loads zeros
};

__device__ __forceinline__ void effq_issue(const uint32_t* Q, uint32_t head, uint32_t n,
                                           const float4* __restrict__ eff4, EffRound& r) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (uint32_t k = 0; k < kRoundLane; ++k) {
        const uint32_t i = lane + 32u * k;
        const bool ok = i < n;
        const uint32_t e = ok ? Q[(head + i) & (kQueueCap - 1u)] : 0u;
        if (k == 0) r.sg = 0u;
        r.sg |= (e >> 31) << k;
        r.ef[k] = ok ? __ldg(eff4 + (e & 0x7fffffffu)) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__device__ __forceinline__ void effq_complete(const EffRound& r, float (&d)[kMaxTraits]) {
#pragma unroll
    for (uint32_t k = 0; k < kRoundLane; ++k) {
        const float sg = ((r.sg >> k) & 1u) ? 1.0f : -1.0f;
        d[0] = fmaf(sg, r.ef[k].x, d[0]);
        d[1] = fmaf(sg, r.ef[k].y, d[1]);
        d[2] = fmaf(sg, r.ef[k].z, d[2]);
        d[3] = fmaf(sg, r.ef[k].w, d[3]);
    }
}

__device__ __forceinline__ void effq_clear(EffRound& r) {
    r.sg = 0u;
#pragma unroll
    for (uint32_t k = 0; k < kRoundLane; ++k) r.ef[k] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Queue the gathered bits (g0, g1) of the lane's words w, w+1 (sign +1 where
// s0/s1 has the bit); every complete round is issued, the previous one folded in.
__device__ __forceinline__ void effq_push(uint64_t g0, uint64_t g1, uint64_t s0, uint64_t s1, uint32_t w,
                                          uint32_t* Q, uint32_t& head, uint32_t& tail, EffRound& pend,
                                          const float4* __restrict__ eff4, float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t c = (uint32_t)(__popcll(g0) + __popcll(g1));
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t H = __shfl_sync(0xffffffffu, incl, 31);
    if (H == 0u) return;
    if (H > kQueueCap - kRound) {  // denser than the queue takes: per-lane chains
        add4(d, effects_direct(g0, g1, s0, s1, w * 64u, eff4));
        return;
    }
    uint32_t i = tail + incl - c;
    // the lane's four 32-bit mask words one after another: 32-bit bit scans
    const uint32_t gg[4] = {(uint32_t)g0, (uint32_t)(g0 >> 32), (uint32_t)g1, (uint32_t)(g1 >> 32)};
    const uint32_t ss[4] = {(uint32_t)s0, (uint32_t)(s0 >> 32), (uint32_t)s1, (uint32_t)(s1 >> 32)};
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
        const uint32_t base = w * 64u + 32u * k;
        // highest bit first: one leading-zero count per bit, the sign bit shifted into place by it
        for (uint32_t x = gg[k]; x;) {
            const uint32_t c = (uint32_t)__clz(x);
            Q[i & (kQueueCap - 1u)] = (base + 31u - c) | ((ss[k] << c) & 0x80000000u);
            x ^= 0x80000000u >> c;
            ++i;
        }
    }
    tail += H;
    __syncwarp();
    while (tail - head >= kRound) {
        effq_complete(pend, d);
        effq_issue(Q, head, kRound, eff4, pend);
        head += kRound;
    }
    __syncwarp();
}

__device__ CLOTHO_COLD ulonglong2 mutation_masks_tail(const PopDev& P, uint32_t M, uint32_t mo, uint32_t mc,
                                                       bool philox, uint32_t w) {
    ulonglong2 x = make_ulonglong2(0, 0);
    for (uint32_t j = 32; j < mc; ++j) {  // rows with more than 32 new alleles
        const uint32_t mi = philox ? mo + j : P.row_mut[mo + j];
        if (mi >= M) continue;
        const uint32_t s = P.mut_slot[mi];
        if (s == 0xffffffffu) continue;
        const uint32_t sw = s >> 6;
        if (sw == w) x.x ^= 1ull << (s & 63u);
        else if (sw == w + 1u) x.y ^= 1ull << (s & 63u);
    }
    return x;
}

// XOR masks of the lane's words w, w+1 from the row's new alleles (whole warp).
__device__ __forceinline__ void row_mutations(const PopDev& P, uint32_t M, const RowArgs& R, uint32_t w,
                                              uint64_t& mx0, uint64_t& mx1) {
    mx0 = 0;
    mx1 = 0;
    const uint32_t lim = R.mc < 32u ? R.mc : 32u;
    for (uint32_t j = 0; j < lim; ++j) {
        const uint32_t s = __shfl_sync(0xffffffffu, R.my_slot, j);
        if (s == 0xffffffffu) continue;
        const uint32_t sw = s >> 6;
        if (sw == w) mx0 ^= 1ull << (s & 63u);
        else if (sw == w + 1u) mx1 ^= 1ull << (s & 63u);
    }
    if (R.mc > 32u) {
        const ulonglong2 x = mutation_masks_tail(P, M, R.mo, R.mc, R.philox, w);
        mx0 ^= x.x;
        mx1 ^= x.y;
    }
}

// Copy rows (no breakpoint): the top strand with the fixed columns cleared and
// the new alleles added, streamed through registers six chunks ahead (the
// chunk-mask build, whose warps have no bitmap for a bulk copy to land in).
__device__ __forceinline__ void row_body_copy(const PopDev& P, uint32_t M, const RowArgs& R, const uint64_t* sfix,
                                              bool do_mut, bool do_fs, const Fold& fo) {
    const uint32_t lane = threadIdx.x & 31u;
    constexpr uint32_t D = 6;
    ulonglong2 t[D];
#pragma unroll
    for (uint32_t j = 0; j < D; ++j) {
        const uint32_t w = 2u * lane + 64u * j;
        t[j] = (w < R.Wp) ? __ldg(reinterpret_cast<const ulonglong2*>(R.top + w)) : make_ulonglong2(0, 0);
    }
    for (uint32_t w0 = 0; w0 < R.Wc; w0 += 64u) {
        const uint32_t w = w0 + 2u * lane;
        const ulonglong2 cur = t[0];
#pragma unroll
        for (uint32_t j = 0; j + 1 < D; ++j) t[j] = t[j + 1];
        const uint32_t wn = w + 64u * D;
        t[D - 1] = (wn < R.Wp) ? __ldg(reinterpret_cast<const ulonglong2*>(R.top + wn)) : make_ulonglong2(0, 0);
        uint64_t mx0 = 0, mx1 = 0;
        if (do_mut && R.mc) row_mutations(P, M, R, w, mx0, mx1);
        if (w < R.Wc) {
            ulonglong2 fm = make_ulonglong2(0, 0);
            if (w < R.Wp) fm = *reinterpret_cast<const ulonglong2*>(sfix + w);
            const uint64_t x0 = (cur.x & ~fm.x) ^ mx0, x1 = (cur.y & ~fm.y) ^ mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) fold(fo, w, x0, x1);
        }
    }
}

// Narrow copy rows (the narrow build of the kernel, every row <= 128 words):
// one 16-byte load a lane per chunk, all issued at once, cost less than arming
// a barrier and waiting for a bulk copy.  A separate build keeps the wide rows'
// code as it is (even an untaken branch to this path slowed them 2%).
__device__ __forceinline__ void row_body_copy_direct(const PopDev& P, uint32_t M, const RowArgs& R,
                                                  const uint64_t* sfix, bool do_mut, bool do_fs, const Fold& fo) {
    const uint32_t lane = threadIdx.x & 31u;
    ulonglong2 t[kDirectCopyChunks];
#pragma unroll
    for (uint32_t j = 0; j < kDirectCopyChunks; ++j) {
        const uint32_t w = 64u * j + 2u * lane;
        t[j] = w < R.Wp ? __ldg(reinterpret_cast<const ulonglong2*>(R.top + w)) : make_ulonglong2(0, 0);
    }
#pragma unroll
    for (uint32_t j = 0; j < kDirectCopyChunks; ++j) {
        const uint32_t w = 64u * j + 2u * lane;
        if (64u * j >= R.Wc) break;
        uint64_t mx0 = 0, mx1 = 0;
        if (do_mut && R.mc) row_mutations(P, M, R, w, mx0, mx1);
        if (w < R.Wc) {
            const ulonglong2 fm =
                w < R.Wp ? *reinterpret_cast<const ulonglong2*>(sfix + w) : make_ulonglong2(0, 0);
            const uint64_t x0 = (t[j].x & ~fm.x) ^ mx0, x1 = (t[j].y & ~fm.y) ^ mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) fold(fo, w, x0, x1);
        }
    }
    if (R.Wc > 64u * kDirectCopyChunks) {  // a child wider than its parent: the rest is new alleles only
        for (uint32_t w0 = 64u * kDirectCopyChunks; w0 < R.Wc; w0 += 64u) {
            const uint32_t w = w0 + 2u * lane;
            uint64_t mx0 = 0, mx1 = 0;
            if (do_mut && R.mc) row_mutations(P, M, R, w, mx0, mx1);
            if (w < R.Wc) {
                *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(mx0, mx1);
                if (do_fs) fold(fo, w, mx0, mx1);
            }
        }
    }
}

// Copy rows through a bulk copy: the whole parent strand (<= 8 KB) lands in
// the warp's (otherwise idle) bitmap in one asynchronous transfer, then the
// lanes mask, mutate, store and fold it, and clear the bitmap behind them.
// false: the strand's copy never landed (kErrAbandon); the row is written without it and the warp
// must not use its bitmap again, since the copy may still land there.
__device__ __forceinline__ bool row_body_copy_bulk(const PopDev& P, uint32_t M, const RowArgs& R,
                                                   const uint64_t* sfix, uint64_t* buf, unsigned long long* bar,
                                                   uint32_t& phase, const uint32_t* wait_limit, bool do_mut,
                                                   bool do_fs, const Fold& fo) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t bytes = R.Wp * 8u;
    bool ok = true;
    if (bytes) {
        // earlier generic-proxy reads and writes of buf come before the asynchronous write
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive_expect(bar, bytes);
        __syncwarp();
        const uint32_t off = lane * 2048u;
        if (off < bytes)
            bulk_load(reinterpret_cast<char*>(buf) + off, reinterpret_cast<const char*>(R.top) + off,
                      min(2048u, bytes - off), bar);
        ok = mbar_wait(bar, phase, &P.st->err, wait_limit);
    }
    for (uint32_t w0 = 0; w0 < R.Wc; w0 += 64u) {
        const uint32_t w = w0 + 2u * lane;
        uint64_t mx0 = 0, mx1 = 0;
        if (do_mut && R.mc) row_mutations(P, M, R, w, mx0, mx1);
        if (w < R.Wc) {
            ulonglong2 t = make_ulonglong2(0, 0), fm = make_ulonglong2(0, 0);
            if (w < R.Wp) {
                ulonglong2* bw = reinterpret_cast<ulonglong2*>(buf + w);
                if (ok) t = *bw;
                *bw = make_ulonglong2(0, 0);  // crossover rows expect the bitmap at zero
                fm = *reinterpret_cast<const ulonglong2*>(sfix + w);
            }
            const uint64_t x0 = (t.x & ~fm.x) ^ mx0, x1 = (t.y & ~fm.y) ^ mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) fold(fo, w, x0, x1);
        }
    }
    __syncwarp();
    return ok;
}

// Crossover rows.  MODE 0: switch mask from the warp's mask bitmap; MODE 1:
// direct event compares (tape rows with more than kMaxEvDevice events);
// MODE 2 (chunk-mask build): each chunk's mask words XORed from the table rows
// of the breakpoints (lane k < E holds row k's offset in my_go) and toggled at
// the row's correction slots (cs[32 k + lane], 0xffffffff for none).
// PROF: clock the effect gather into *gcyc (profiling build).
template <int MODE, bool PROF = false>
__device__ __forceinline__ void row_body_suf(const PopDev& P, uint32_t M, const RowArgs& R, const uint64_t* sfix,
                                             uint64_t* mask, uint32_t* Q, bool inv, bool do_mut, bool gather,
                                             bool do_fs, const Fold& fo, float (&d)[kMaxTraits],
                                             unsigned long long* gcyc = nullptr, const uint32_t* cs = nullptr,
                                             uint32_t my_go = 0u) {
    const uint32_t lane = threadIdx.x & 31u;
    constexpr bool xo = true;
    const float4* eff4 = reinterpret_cast<const float4*>(P.eff);
    uint32_t qh = 0, qt = 0;
    EffRound pend;
    effq_clear(pend);
    // parent words one chunk ahead (the strands are prefetched into L2 at row start;
    // a second chunk in registers measured slower: it takes the registers of the gather rounds)
    ulonglong2 t_a, b_a;
    load_pair(t_a, b_a, R, 2u * lane, xo);
    for (uint32_t w0 = 0; w0 < R.Wc; w0 += 64u) {
        const uint32_t w = w0 + 2u * lane;
        ulonglong2 t_b, b_b;
        load_pair(t_b, b_b, R, w + 64u, xo);
        uint64_t mx0 = 0, mx1 = 0;
        if (do_mut && R.mc) row_mutations(P, M, R, w, mx0, mx1);
        const bool live = w < R.Wc;
        ulonglong2 fm = make_ulonglong2(0, 0);
        if (live && w < R.Wp) fm = *reinterpret_cast<const ulonglong2*>(sfix + w);
        const uint64_t t0 = t_a.x & ~fm.x, t1 = t_a.y & ~fm.y;
        uint64_t x0, x1;
        {
            const uint64_t b0 = b_a.x & ~fm.x, b1 = b_a.y & ~fm.y;
            const uint64_t h0 = live ? (t0 ^ b0) : 0ull, h1 = live ? (t1 ^ b1) : 0ull;
            uint64_t m0 = 0, m1 = 0;
            if (MODE == 0) {
                if (live) {
                    ulonglong2* mw = reinterpret_cast<ulonglong2*>(mask + w);
                    const ulonglong2 m = *mw;
                    *mw = make_ulonglong2(0, 0);  // the bitmap starts every row at zero
                    m0 = m.x;
                    m1 = m.y;
                }
            } else if (MODE == 2) {
                // table rows (L2-resident) of the row's breakpoints, four loads in flight; words past the
                // parent's width take no switch.  The next chunk's words are prefetched into L1 behind this
                // chunk's work.
                for (uint32_t k0 = 0; k0 < R.E; k0 += 4u) {
                    ulonglong2 v[4];
#pragma unroll
                    for (uint32_t j = 0; j < 4u; ++j) {
                        const uint32_t k = k0 + j;
                        const uint64_t* tk = P.suf + __shfl_sync(0xffffffffu, my_go, k & 31u);
                        const bool on = k < R.E;
                        if (on && w + 64u < R.Wp) asm volatile("prefetch.global.L1 [%0];" ::"l"(tk + w + 64u));
                        v[j] = (on && live && w < R.Wp) ? __ldg(reinterpret_cast<const ulonglong2*>(tk + w))
                                                        : make_ulonglong2(0, 0);
                    }
#pragma unroll
                    for (uint32_t j = 0; j < 4u; ++j) {
                        m0 ^= v[j].x;
                        m1 ^= v[j].y;
                    }
                }
                // correction slots that fall in this chunk: each is toggled by the lane that owns its word
                for (uint32_t k = 0; k < R.E; ++k) {
                    const uint32_t rel = cs[32u * k + lane] - w0 * 64u;
                    uint32_t hits = __ballot_sync(0xffffffffu, rel < 4096u);
                    while (hits) {
                        const uint32_t l = (uint32_t)(__ffs(hits) - 1);
                        hits &= hits - 1u;
                        const uint32_t r = __shfl_sync(0xffffffffu, rel, l);
                        if ((r >> 7) == lane) {
                            const uint32_t bit = r & 127u;
                            if (bit < 64u) m0 ^= 1ull << bit;
                            else m1 ^= 1ull << (bit - 64u);
                        }
                    }
                }
            } else {
                m0 = sw_mask_events(h0, w * 64u, P.pos, R.evg, R.E);
                m1 = sw_mask_events(h1, w * 64u + 64u, P.pos, R.evg, R.E);
            }
            const uint64_t sw0 = m0 & h0, sw1 = m1 & h1;
            x0 = t0 ^ sw0;
            x1 = t1 ^ sw1;
            if (gather) {
                const long long c0 = PROF ? clock64() : 0;
                effq_push(inv ? (h0 ^ sw0) : sw0, inv ? (h1 ^ sw1) : sw1, inv ? t0 : b0, inv ? t1 : b1, w, Q, qh, qt,
                          pend, eff4, d);
                if (PROF) *gcyc += (unsigned long long)(clock64() - c0);
            }
        }
        if (live) {
            x0 ^= mx0;
            x1 ^= mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) fold(fo, w, x0, x1);
        }
        t_a = t_b; b_a = b_b;
    }
    if (gather) {
        const long long c0 = PROF ? clock64() : 0;
        effq_complete(pend, d);
        if (qt != qh) {
            effq_issue(Q, qh, qt - qh, eff4, pend);
            effq_complete(pend, d);
            __syncwarp();
        }
        if (PROF) *gcyc += (unsigned long long)(clock64() - c0);
    }
}

// inv: gather the unswitched heterozygous set (the plan chose the bottom strand's carried value as the base).
__device__ CLOTHO_COLD float4 row_body_events(const PopDev& P, uint32_t M, const RowArgs R, const uint64_t* sfix,
                                               uint32_t* Q, bool do_mut, bool gather, bool do_fs, const Fold& fo,
                                               bool inv = false) {
    float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
    row_body_suf<1>(P, M, R, sfix, nullptr, Q, inv, do_mut, gather, do_fs, fo, d);
    return make_float4(d[0], d[1], d[2], d[3]);
}

// Nearest suffix-table row b (a multiple of 64) of rank threshold r and the
// ranks between them: [c0, c0 + n), n <= 32.
__device__ __forceinline__ uint32_t table_row(uint32_t r, uint32_t A, uint32_t& c0, uint32_t& n) {
    const uint32_t lo = r & ~63u;
    const uint32_t b = (r - lo <= 32u) ? lo : lo + 64u;
    c0 = min(r, b);
    n = min(max(r, b), A) - c0;
    return b;
}

// Phase cycles of the profiling build, kept by every lane, flushed by lane 0.
struct PhaseClk {
    unsigned long long c[kPhCount];
};

// One offspring row, the whole warp (suffix-table classifier), from the plan
// at processing position v (k_row_plan): row, top strand, breakpoints, table
// rows and correction ranks.  PROF: clock the row's phases into pc.
// Returns false when the row's bulk copy was abandoned (the warp then stops working on rows).
template <bool PROF, bool NARROW, bool CM = false>
__device__ __forceinline__ bool gen_row_suf(const PopDev& P, const DevStatus& st, uint32_t v, const uint64_t* sfix,
                                            uint64_t* mask, WarpSmem& ws, uint32_t& phase,
                                            const uint32_t* wait_limit, bool do_mut, bool do_ph, bool gather, bool do_fs,
                                            const Fold& fo, PhaseClk& pc, uint32_t* cs = nullptr) {
    const uint32_t lane = threadIdx.x & 31u;
    const long long c0 = PROF ? clock64() : 0;
    long long c1 = 0, c2 = 0, c3 = 0;
    const uint4 pr = __ldg(P.plan_row + v);
    const uint2 pm = __ldg(P.plan_mut + v);
    const double pz = (do_ph && lane < kMaxTraits) ? __ldg(P.plan_z + (size_t)v * 4u + lane) : 0.0;
    const uint32_t g = pr.x, topr = pr.y, base = pr.z;
    const uint32_t E = pr.w & kPlanMaxEvents, flags = pr.w >> kPlanFlagShift;
    const bool inv = gather && (flags & kPlanInv) != 0;
    const uint64_t* prow = P.rows[st.cur ^ 1u];
    RowArgs R;
    R.topr = topr;
    R.top = prow + (size_t)topr * P.Wcap;
    R.bot = prow + (size_t)(topr ^ 1u) * P.Wcap;
    R.out = P.rows[st.cur] + (size_t)g * P.Wcap;
    R.Wc = st.W;
    R.Wp = st.pW;
    R.E = E;
    R.philox = P.mode == kModePhilox;
    R.evg = P.ev_pos + base;
    if (E > 0 || CM || !CLOTHO_COPY_BULK) prefetch_l2(R.top, R.Wp * 8u);
    if (E > 0) prefetch_l2(R.bot, R.Wp * 8u);
    R.zbase = pz;  // z(inv ? bottom : top) - sum(fixed), from the plan
    float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
    row_mutation_setup(P, st, pm.x, pm.y, do_mut, gather, R, d);
    bool landed = true;
    if (PROF) c1 = clock64();
    if ((flags & kPlanLong) || (CM && E > kCmMaxEv)) {
        add4(d, row_body_events(P, st.M, R, sfix, ws.q, do_mut, gather, do_fs, fo, inv));
    } else if (CM && E == 0) {
        row_body_copy(P, st.M, R, sfix, do_mut, do_fs, fo);
    } else if (CM) {
        // chunk masks: the breakpoints' table-row offsets in lanes 0..E-1, their correction slots in cs
        const uint32_t my_go = lane < E ? __ldg(P.plan_go + base + lane) : 0u;
        const uint32_t my_cr = lane < E ? __ldg(P.plan_cr + base + lane) : 0u;
        for (uint32_t k = 0; k < E; ++k) {  // the first chunk's table words, behind the corrections' set-up
            const uint64_t* tk = P.suf + __shfl_sync(0xffffffffu, my_go, k);  // every lane takes part
            if (2u * lane < R.Wp) asm volatile("prefetch.global.L1 [%0];" ::"l"(tk + 2u * lane));
        }
        __syncwarp();  // the previous row's reads of cs are done
        for (uint32_t k = 0; k < E; ++k) {
            const uint32_t pcr = __shfl_sync(0xffffffffu, my_cr, k);
            cs[32u * k + lane] = lane < (pcr >> 20) ? __ldg(P.inv + (pcr & 0xfffffu) + lane) : 0xffffffffu;
        }
        __syncwarp();
        row_body_suf<2>(P, st.M, R, sfix, nullptr, ws.q, inv, do_mut, gather, do_fs, fo, d, nullptr, cs, my_go);
    } else if (E == 0) {
#if CLOTHO_COPY_BULK
        if (NARROW)
            row_body_copy_direct(P, st.M, R, sfix, do_mut, do_fs, fo);
        else
            landed = row_body_copy_bulk(P, st.M, R, sfix, mask, &ws.mbar, phase, wait_limit, do_mut, do_fs, fo);
#else
        row_body_copy(P, st.M, R, sfix, do_mut, do_fs, fo);
#endif
    } else {
        uint32_t* m32 = reinterpret_cast<uint32_t*>(mask);
        const uint64_t* __restrict__ suf = P.suf;
        const uint32_t np = R.Wp >> 1;  // word pairs of a table row
        if (np != 0u && E <= 32u && E * np <= 32u * kFlatLoads) {
            // narrow rows (batches of small populations): the table rows' words of every breakpoint are
            // spread over the lanes and loaded at once, then XORed in with shared atomics, so the mask
            // costs one table round trip instead of one per breakpoint
            const uint32_t my_cr = lane < E ? __ldg(P.plan_cr + base + lane) : 0u;
            const uint32_t my_go = lane < E ? __ldg(P.plan_go + base + lane) : 0u;
            ulonglong2 v[kFlatLoads];
            uint32_t at[kFlatLoads];
#pragma unroll
            for (uint32_t j = 0; j < kFlatLoads; ++j) {
                const uint32_t i = lane + 32u * j;
                const uint32_t k = i / np;  // breakpoint of this word pair (np >= 4)
                const uint32_t go = __shfl_sync(0xffffffffu, my_go, k & 31u);
                at[j] = i < E * np ? i - k * np : 0xffffffffu;
                v[j] = i < E * np ? __ldg(reinterpret_cast<const ulonglong2*>(suf + go) + (i - k * np))
                                  : make_ulonglong2(0, 0);
            }
            // corrections: toggle the slots whose rank lies between threshold and table row
#pragma unroll 4
            for (uint32_t k = 0; k < E; ++k) {
                const uint32_t pc = __shfl_sync(0xffffffffu, my_cr, k);
                if (lane < (pc >> 20)) {
                    const uint32_t sl = __ldg(P.inv + (pc & 0xfffffu) + lane);
                    atomicXor(m32 + (sl >> 5), 1u << (sl & 31u));
                }
            }
#pragma unroll
            for (uint32_t j = 0; j < kFlatLoads; ++j) {
                if (at[j] != 0xffffffffu) {
                    uint32_t* mw = m32 + 4u * at[j];
                    if ((uint32_t)v[j].x) atomicXor(mw, (uint32_t)v[j].x);
                    if ((uint32_t)(v[j].x >> 32)) atomicXor(mw + 1, (uint32_t)(v[j].x >> 32));
                    if ((uint32_t)v[j].y) atomicXor(mw + 2, (uint32_t)v[j].y);
                    if ((uint32_t)(v[j].y >> 32)) atomicXor(mw + 3, (uint32_t)(v[j].y >> 32));
                }
            }
        } else {
            // corrections: toggle the slots whose rank lies between threshold and table row (the table-row
            // offsets of the first 32 breakpoints are fetched with their correction ranks)
            const uint32_t go0 = lane < E ? __ldg(P.plan_go + base + lane) : 0u;
            for (uint32_t k0 = 0; k0 < E; k0 += 32u) {
                const uint32_t my_cr = (k0 + lane < E) ? __ldg(P.plan_cr + base + k0 + lane) : 0u;
                const uint32_t ke = min(32u, E - k0);
    #pragma unroll 4
                for (uint32_t k = 0; k < ke; ++k) {
                    const uint32_t pc = __shfl_sync(0xffffffffu, my_cr, k);
                    if (lane < (pc >> 20)) {
                        const uint32_t s = __ldg(P.inv + (pc & 0xfffffu) + lane);
                        atomicXor(m32 + (s >> 5), 1u << (s & 31u));
                    }
                }
            }
            __syncwarp();
            // XOR of the events' table rows, kTableInflight 16-byte loads per lane in flight
            ulonglong2* m2 = reinterpret_cast<ulonglong2*>(mask);
            for (uint32_t k0 = 0; k0 < E; k0 += 32u) {
                const uint32_t my_go = k0 == 0 ? go0 : (k0 + lane < E) ? __ldg(P.plan_go + base + k0 + lane) : 0u;
                const uint32_t ke = min(32u, E - k0);
                for (uint32_t k = 0; k < ke; ++k) {
                    const uint64_t* tk = suf + __shfl_sync(0xffffffffu, my_go, k);
                    for (uint32_t wb = 0; wb < R.Wp; wb += 64u * kTableInflight) {
                        ulonglong2 v[kTableInflight];
    #pragma unroll
                        for (uint32_t j = 0; j < kTableInflight; ++j) {
                            const uint32_t w = wb + 64u * j + 2u * lane;
                            v[j] = (w < R.Wp) ? __ldg(reinterpret_cast<const ulonglong2*>(tk + w))
                                              : make_ulonglong2(0, 0);
                        }
    #pragma unroll
                        for (uint32_t j = 0; j < kTableInflight; ++j) {
                            const uint32_t w = wb + 64u * j + 2u * lane;
                            if (w < R.Wp) {
                                ulonglong2 x = m2[w >> 1];
                                x.x ^= v[j].x;
                                x.y ^= v[j].y;
                                m2[w >> 1] = x;
                            }
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (PROF) c2 = clock64();
        row_body_suf<0, PROF>(P, st.M, R, sfix, mask, ws.q, inv, do_mut, gather, do_fs, fo, d,
                              &pc.c[kPhXoGather]);
    }
    if (PROF) c3 = clock64();
    if (do_ph) row_phenotype(P, st, g, R, d);
    if (PROF) {
        const unsigned long long c4 = (unsigned long long)clock64();
        if (flags & kPlanLong) {
            pc.c[kPhLongRows] += 1;
            pc.c[kPhLongCyc] += c4 - c0;
        } else if (E == 0) {
            pc.c[kPhCopyRows] += 1;
            pc.c[kPhCopySetup] += c1 - c0;
            pc.c[kPhCopyBody] += c3 - c1;
            pc.c[kPhCopyPheno] += c4 - c3;
        } else {
            pc.c[kPhXoRows] += 1;
            pc.c[kPhXoSetup] += c1 - c0;
            pc.c[kPhXoMask] += c2 - c1;
            pc.c[kPhXoBody] += c3 - c2;
            pc.c[kPhXoPheno] += c4 - c3;
        }
    }
    return landed;
}

// ---------------------------------------------------------------------------
// Interval classifier (allele spaces beyond the suffix table).

// Sorted breakpoint thresholds of one gamete as half-open rank intervals:
// a het bit switches strand iff its slot rank lies in one of them.
struct RowXo {
    uint32_t a[kMaxIv];   // interval start (rank)
    uint32_t l[kMaxIv];   // length; 0 = empty
    const uint2* iv;      // the same intervals in shared memory (any count)
    uint32_t niv;
};

template <int NI>
__device__ __forceinline__ bool in_iv(uint32_t r, const RowXo& X) {
    bool s = false;
    if (NI > 0) {
#pragma unroll
        for (int k = 0; k < NI; ++k) s |= (r - X.a[k]) < X.l[k];
    } else {
        for (uint32_t k = 0; k < X.niv; ++k) s |= (r - X.iv[k].x) < X.iv[k].y;
    }
    return s;
}

// One branch-free step of a het-bit chain: classify the lowest bit of h.
template <int NI>
__device__ __forceinline__ void xo_step(uint32_t& h, uint32_t& m, uint32_t base, const uint32_t* __restrict__ grank,
                                        const RowXo& X) {
    const bool nz = h != 0u;
    const uint32_t j = nz ? (uint32_t)(__ffs(h) - 1) : 0u;
    h &= h - 1u;
    const uint32_t r = __ldg(grank + base + j);
    const bool s = nz && in_iv<NI>(r, X);
    m |= (uint32_t)s << j;
}

// Switched-strand masks of the lane's two words: four interleaved 32-bit chains.
template <int NI>
__device__ __forceinline__ void classify(uint64_t h0, uint64_t h1, uint32_t s0, const uint32_t* __restrict__ grank,
                                         const RowXo& X, uint64_t& m0, uint64_t& m1) {
    uint32_t a = (uint32_t)h0, b = (uint32_t)(h0 >> 32), c = (uint32_t)h1, d = (uint32_t)(h1 >> 32);
    uint32_t ma = 0, mb = 0, mc = 0, md = 0;
    while (a | b | c | d) {
        xo_step<NI>(a, ma, s0, grank, X);
        xo_step<NI>(b, mb, s0 + 32u, grank, X);
        xo_step<NI>(c, mc, s0 + 64u, grank, X);
        xo_step<NI>(d, md, s0 + 96u, grank, X);
    }
    m0 = (uint64_t)ma | ((uint64_t)mb << 32);
    m1 = (uint64_t)mc | ((uint64_t)md << 32);
}

// Warp-balanced classification of one 64-word chunk: the het bits of the
// warp go through the queue, four per lane; switched bits are ORed into the
// warp's chunk mask SM and their effects gathered.  H = total het bits (<= kQueueCap).
template <int NI>
__device__ __forceinline__ void classify_balanced(uint64_t h0, uint64_t h1, uint64_t b0, uint64_t b1, uint32_t w,
                                                  uint32_t w0, uint32_t off, uint32_t H, uint32_t* Q,
                                                  uint32_t* SM, const uint32_t* __restrict__ grank, const RowXo& X,
                                                  const float4* __restrict__ eff4, bool gather,
                                                  float (&d)[kMaxTraits], uint64_t& m0, uint64_t& m1) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) SM[4u * lane + k] = 0u;
    uint32_t q = off;
    const uint32_t hh[4] = {(uint32_t)h0, (uint32_t)(h0 >> 32), (uint32_t)h1, (uint32_t)(h1 >> 32)};
    const uint32_t bb[4] = {(uint32_t)b0, (uint32_t)(b0 >> 32), (uint32_t)b1, (uint32_t)(b1 >> 32)};
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
        const uint32_t base = w * 64u + 32u * k;
        for (uint32_t x = hh[k]; x; x &= x - 1u) {
            const uint32_t j = (uint32_t)(__ffs(x) - 1);
            Q[q++] = (base + j) | (((bb[k] >> j) & 1u) << 31);
        }
    }
    __syncwarp();
    const uint32_t sbase = w0 * 64u;
    for (uint32_t ib = 0; ib < H; ib += 128u) {
        uint32_t e[4];
        bool sw[4];
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
            const uint32_t i = ib + lane + 32u * k;
            e[k] = (i < H) ? Q[i] : 0u;
            const uint32_t r = __ldg(grank + (e[k] & 0x7fffffffu));
            sw[k] = (i < H) && in_iv<NI>(r, X);
        }
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
            if (sw[k]) {
                const uint32_t loc = (e[k] & 0x7fffffffu) - sbase;
                atomicOr(&SM[loc >> 5], 1u << (loc & 31u));
            }
        }
        if (gather) {
            float4 ef[4];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)
                ef[k] = sw[k] ? __ldg(eff4 + (e[k] & 0x7fffffffu)) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                const float g = sw[k] ? ((e[k] >> 31) ? 1.0f : -1.0f) : 0.0f;
                d[0] = fmaf(g, ef[k].x, d[0]);
                d[1] = fmaf(g, ef[k].y, d[1]);
                d[2] = fmaf(g, ef[k].z, d[2]);
                d[3] = fmaf(g, ef[k].w, d[3]);
            }
        }
    }
    __syncwarp();
    m0 = (uint64_t)SM[4u * lane] | ((uint64_t)SM[4u * lane + 1u] << 32);
    m1 = (uint64_t)SM[4u * lane + 2u] | ((uint64_t)SM[4u * lane + 3u] << 32);
    __syncwarp();
}

// Per-row crossover mode of the interval classifier
enum XoKind : int { kXoCopy = 0, kXoIv4 = 4, kXoIv8 = 8, kXoFar = -1, kXoEvents = -2 };

template <int KIND>
__device__ __forceinline__ void row_body_iv(const PopDev& P, const DevStatus& st, const RowArgs& R,
                                            const uint64_t* sfix, const RowXo& X, uint32_t* Q, uint32_t* SM,
                                            bool do_mut, bool gather, bool do_fs, const Fold& fo,
                                            float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    constexpr bool xo = (KIND != kXoCopy);
    const float4* eff4 = reinterpret_cast<const float4*>(P.eff);
    ulonglong2 t_a, b_a, t_b, b_b;
    load_pair(t_a, b_a, R, 2u * lane, xo);
    load_pair(t_b, b_b, R, 2u * lane + 64u, xo);
    for (uint32_t w0 = 0; w0 < R.Wc; w0 += 64u) {
        const uint32_t w = w0 + 2u * lane;
        ulonglong2 t_c, b_c;
        load_pair(t_c, b_c, R, w + 128u, xo);
        uint64_t mx0 = 0, mx1 = 0;
        if (do_mut && R.mc) mutation_masks(P, st, R, w, mx0, mx1);
        const bool live = w < R.Wc;
        ulonglong2 fm = make_ulonglong2(0, 0);
        if (live && w < R.Wp) fm = *reinterpret_cast<const ulonglong2*>(sfix + w);
        const uint64_t t0 = t_a.x & ~fm.x, t1 = t_a.y & ~fm.y;
        uint64_t x0 = t0, x1 = t1;
        if (xo) {
            const uint64_t b0 = b_a.x & ~fm.x, b1 = b_a.y & ~fm.y;
            const uint64_t h0 = live ? (t0 ^ b0) : 0ull, h1 = live ? (t1 ^ b1) : 0ull;
            uint64_t m0, m1;
            if (KIND != kXoEvents) {
                // warp prefix of het counts decides between the balanced queue and per-lane chains
                const uint32_t c = (uint32_t)(__popcll(h0) + __popcll(h1));
                uint32_t incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= (uint32_t)o) incl += y;
                }
                const uint32_t H = __shfl_sync(0xffffffffu, incl, 31);
                if (H <= kQueueCap) {
                    classify_balanced<(KIND > 0 ? KIND : 0)>(h0, h1, b0, b1, w, w0, incl - c, H, Q, SM, P.rank, X,
                                                             eff4, gather, d, m0, m1);
                } else {
                    classify<(KIND > 0 ? KIND : 0)>(h0, h1, w * 64u, P.rank, X, m0, m1);
                    if (gather) switched_effects(m0, m1, b0, b1, w * 64u, eff4, d);
                }
            } else {
                m0 = sw_mask_events(h0, w * 64u, P.pos, R.evg, R.E);
                m1 = sw_mask_events(h1, w * 64u + 64u, P.pos, R.evg, R.E);
                if (gather) switched_effects(m0, m1, b0, b1, w * 64u, eff4, d);
            }
            x0 = (t0 & ~m0) | (b0 & m0);
            x1 = (t1 & ~m1) | (b1 & m1);
        }
        if (live) {
            x0 ^= mx0;
            x1 ^= mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) fold(fo, w, x0, x1);
        }
        t_a = t_b; b_a = b_b;
        t_b = t_c; b_b = b_c;
    }
}

// One offspring row, the whole warp (interval classifier).
__device__ __forceinline__ void gen_row_iv(const PopDev& P, const DevStatus& st, uint32_t g, const uint64_t* sfix,
                                           uint2* s_iv, uint32_t* s_thr, uint32_t* Q, uint32_t* SM, bool do_mut,
                                           bool do_ph, bool gather, bool do_fs, const Fold& fo) {
    const uint32_t lane = threadIdx.x & 31u;
    RowArgs R;
    float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
    row_setup(P, st, g, do_mut, do_ph, gather, R, d);
    const uint32_t E = R.E;
    // ---- breakpoints -> sorted rank thresholds -> intervals
    RowXo X;
#pragma unroll
    for (uint32_t k = 0; k < kMaxIv; ++k) { X.a[k] = 0; X.l[k] = 0; }
    X.iv = s_iv;
    X.niv = 0;
    int kind = kXoCopy;
    if (E > 0 && E <= kMaxEvDevice) {
        for (uint32_t k = lane; k < E; k += 32u) s_thr[k] = threshold_rank(P, row_event(P, st, R, g, k));
        __syncwarp();
        // stable rank sort of the thresholds
        uint32_t mine[4], posn[4];
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            const uint32_t k = lane + 32u * q;
            mine[q] = (k < E) ? s_thr[k] : 0u;
            posn[q] = 0;
        }
        for (uint32_t j = 0; j < E; ++j) {
            const uint32_t tj = s_thr[j];
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                const uint32_t k = lane + 32u * q;
                posn[q] += (tj < mine[q] || (tj == mine[q] && j < k)) ? 1u : 0u;
            }
        }
        __syncwarp();
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            const uint32_t k = lane + 32u * q;
            if (k < E) s_thr[posn[q]] = mine[q];
        }
        __syncwarp();
        const uint32_t NI = (E + 1u) >> 1;
        for (uint32_t i = lane; i < NI; i += 32u) {
            const uint32_t a = s_thr[2u * i];
            uint32_t l;
            if (2u * i + 1u < E) l = s_thr[2u * i + 1u] - a;
            else l = a ? (uint32_t)(0x100000000ull - a) : 0xffffffffu;
            s_iv[i] = make_uint2(a, l);
        }
        __syncwarp();
        X.niv = NI;
        if (NI <= kMaxIv) {
#pragma unroll
            for (uint32_t k = 0; k < kMaxIv; ++k) {
                if (k < NI) { X.a[k] = s_iv[k].x; X.l[k] = s_iv[k].y; }
            }
            kind = NI <= 4 ? kXoIv4 : kXoIv8;
        } else {
            kind = kXoFar;
        }
    } else if (E > kMaxEvDevice) {
        kind = kXoEvents;  // tape rows with very long event lists
    }
    switch (kind) {
        case kXoCopy: row_body_iv<kXoCopy>(P, st, R, sfix, X, Q, SM, do_mut, gather, do_fs, fo, d); break;
        case kXoIv4: row_body_iv<kXoIv4>(P, st, R, sfix, X, Q, SM, do_mut, gather, do_fs, fo, d); break;
        case kXoIv8: row_body_iv<kXoIv8>(P, st, R, sfix, X, Q, SM, do_mut, gather, do_fs, fo, d); break;
        case kXoFar: row_body_iv<kXoFar>(P, st, R, sfix, X, Q, SM, do_mut, gather, do_fs, fo, d); break;
        default: row_body_iv<kXoEvents>(P, st, R, sfix, X, Q, SM, do_mut, gather, do_fs, fo, d); break;
    }
    if (do_ph) row_phenotype(P, st, g, R, d);
}

}  // namespace

// Dynamic shared memory: [AND acc: aw][OR acc: aw][fixed mask: aw] u64 (aw = maxW in the bitmap
// builds, acc_words in the chunk-mask and interval-classifier builds), then, in the bitmap builds,
// the warps' mask bitmaps and one WarpSmem per warp, in the chunk-mask build one WarpSmem and
// kCmCorr correction slots per warp.  A population whose current rows are wider than acc_words
// (chunk-mask and interval builds) folds into its global AND/OR accumulators and reads its fixed
// mask from global memory; the choice is made per population from its widths on the device, so a
// graph captured for a large capacity keeps the shared accumulators while the rows are narrow.
// PROF (suffix-table build only): per-phase cycle counters into ctl->phase.
// NARROW (suffix-table build only): every row is at most 128 words.
// CNT (suffix-table builds, shared accumulators): per-column counts of the child rows of the populations
// that asked (DevStatus::count_cols), in kCountPlanes bit-sliced planes after the WarpSmem array, flushed to
// PopDev::colcnt when the block moves to another population and at the kernel's end.
template <bool SUF, bool PROF, bool NARROW, bool CNT = false, bool CM = false>
__global__ void __launch_bounds__(kGenThreads, 1)
k_generation(const PopDev* __restrict__ pops, uint32_t npops, WorkCtl* __restrict__ ctl, uint32_t fuse,
             int profile, uint32_t maxW, uint32_t acc_words, uint32_t mixed) {
    const long long c_start = PROF ? clock64() : 0;
    PhaseClk pc;
    if (PROF)
        for (uint32_t i = 0; i < kPhCount; ++i) pc.c[i] = 0;
    extern __shared__ __align__(16) uint64_t s_dyn[];
    constexpr uint32_t kIvWarps = SUF ? 1 : kWarps;  // interval-classifier state, unused by the suffix table
    __shared__ uint2 s_iv[kIvWarps][kMaxIvSmem];
    __shared__ uint32_t s_thr[kIvWarps][kMaxEvDevice];
    __shared__ uint32_t s_q[kIvWarps][kQueueCap];
    __shared__ uint32_t s_sm[kIvWarps][128];
    __shared__ uint32_t s_item, s_next;
    __shared__ uint32_t s_crows;   // CNT, one population: rows the block has counted
    // the suffix-table builds keep their accumulators maxW words wide; the chunk-mask and interval builds
    // hold rows of up to acc_words words in shared memory
    const uint32_t aw = (SUF && !CM) ? maxW : acc_words;
    uint64_t* const sF0 = s_dyn;
    uint64_t* const sV0 = s_dyn + aw;
    uint64_t* const sfix0 = s_dyn + 2u * aw;
    uint64_t* sF = sF0;
    uint64_t* sV = sV0;
    uint64_t* sfix = sfix0;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // SUF: per-warp mask bitmaps [kWarps][maxW] u64, then one WarpSmem per warp; CM: no bitmaps, one WarpSmem
    // per warp, then kCmCorr correction slots per warp
    uint64_t* mask = s_dyn + (3u + ((SUF && !CM) ? warp : 0u)) * maxW;
    WarpSmem* const wsa = reinterpret_cast<WarpSmem*>(s_dyn + (CM ? 3u * aw : (3u + kWarps) * maxW));
    WarpSmem& ws = wsa[SUF ? warp : 0u];
    uint32_t* const cs = CM ? reinterpret_cast<uint32_t*>(wsa + kWarps) + warp * kCmCorr : nullptr;
    uint32_t bphase = 0;  // parity of the warp's bulk-copy barrier
    const uint32_t* wait_limit = &ctl->wait_limit;  // read only when a copy is late
    if (SUF) {
        if (!CM)
            for (uint32_t w = lane; w < maxW; w += 32u) mask[w] = 0ull;
        if (lane == 0) {
            mbar_init(&ws.mbar);
            ws.dead = 0u;
        }
        __syncwarp();
    }
    const bool do_mut = (fuse & kFuseMut) != 0, do_ph = (fuse & kFusePheno) != 0, do_fs = (fuse & kFuseFs) != 0;
    uint64_t* const cplanes =
        CNT ? reinterpret_cast<uint64_t*>(reinterpret_cast<WarpSmem*>(s_dyn + (3u + kWarps) * maxW) + kWarps) : nullptr;
    if (CNT) {
        for (uint32_t i = threadIdx.x; i < kCountPlanes * maxW; i += blockDim.x) cplanes[i] = 0ull;
        if (threadIdx.x == 0) s_crows = 0u;
    }
    int cur_pop = -1;
    uint32_t cur_W = 0, cur_A = 0;
    bool cur_cnt = false;      // CNT: the block's current population counts columns
    bool cur_g = false;        // the block's current population folds into its global accumulators
    uint32_t crows = 0;        // CNT, batches: rows the block has counted since its last flush (block-uniform)
    uint64_t rows_done = 0, words_done = 0;

    if (npops == 1) {
        // One population: each warp takes kWarpChunk rows at a time from the
        // step's counter, with no block barrier between them, so no warp waits
        // for the slowest warp of its block until the kernel's end.
        const PopDev& P = pops[0];
        const DevStatus st = *P.st;
        cur_pop = 0;
        cur_W = st.W;
        cur_g = (!SUF || CM) && max(st.W, st.pW) > acc_words;
        if (cur_g) {
            sF = P.accF;
            sV = P.accV;
            sfix = P.fixmask;
        } else {
            if (do_fs)
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) { sF[w] = ~0ull; sV[w] = 0ull; }
            for (uint32_t w = threadIdx.x; w < st.pW; w += blockDim.x) sfix[w] = P.fixmask[w];
        }
        __syncthreads();
        const bool gather = do_ph && st.nz_eff != 0;
        const uint32_t S = 2u * st.N;
        const uint32_t Se = (S + 1u) >> 1;
        cur_A = st.A;
        cur_cnt = CNT && do_fs && !cur_g && st.count_cols != 0u;
        Fold fo{sF, sV, cur_cnt ? cplanes : nullptr, maxW};
        // the next claim is taken before the current rows run, so its
        // round trip to the counter is hidden behind them
        uint32_t claim = 0;
        if (lane == 0) claim = atomicAdd(&ctl->gen_counter, kWarpChunk);
        for (;;) {
            const uint32_t k = __shfl_sync(0xffffffffu, claim, 0);
            if (k >= S) break;
            if (lane == 0) claim = atomicAdd(&ctl->gen_counter, kWarpChunk);
            const uint32_t k1 = min(S, k + kWarpChunk);
            for (uint32_t v = k; v < k1; ++v) {
                const uint32_t g = v < Se ? 2u * v : 2u * (v - Se) + 1u;
                if (CNT && fo.cnt) {  // a block counts at most kCountMax rows (one flush, at the end)
                    uint32_t n = 0;
                    if (lane == 0) n = atomicAdd(&s_crows, 1u);
                    n = __shfl_sync(0xffffffffu, n, 0);
                    if (n >= kCountMax) {
                        if (lane == 0 && n == kCountMax) atomicAnd(&P.st->cols_valid, 0u);
                        fo.cnt = nullptr;
                    }
                }
                if (SUF) {
                    if (!gen_row_suf<PROF, NARROW, CM>(P, st, v, sfix, mask, ws, bphase, wait_limit, do_mut, do_ph,
                                                       gather, do_fs, fo, pc, cs)) {
                        ws.dead = 1u;
                        break;
                    }
                } else
                    gen_row_iv(P, st, g, sfix, s_iv[warp], s_thr[warp], s_q[warp], s_sm[warp], do_mut, do_ph,
                               gather, do_fs, fo);
                if (profile && lane == 0) { rows_done += 1; words_done += st.W; }
            }
            if (SUF && ws.dead) break;  // no further row: the warp leaves the loop
        }
    }
    for (; npops > 1;) {
        if (threadIdx.x == 0) {
            // a mixed batch runs one pass per classifier, each on its own counter over the same items
            s_item = atomicAdd(!mixed || (SUF && !CM) ? &ctl->gen_counter
                               : CM                   ? &ctl->gen_counter_cm
                                                      : &ctl->gen_counter_iv,
                               1u);
            s_next = 0;
        }
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= ctl->gen_items) break;
        uint32_t p;
        {
            uint32_t lo = 0, hi = npops;  // last p with item_base[p] <= item
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (ctl->item_base[mid] <= item) lo = mid; else hi = mid;
            }
            p = lo;
        }
        const PopDev& P = pops[p];
        // the build of this population (by its capacity) against this launch's build
        const uint32_t kind = P.suf == nullptr ? 0u : P.Acap > kSufMaxSlots ? 2u : 1u;
        if (mixed && kind != (SUF ? (CM ? 2u : 1u) : 0u)) {  // another pass takes this item
            __syncthreads();
            continue;
        }
        const DevStatus st = *P.st;
        if ((int)p != cur_pop) {
            if (cur_pop >= 0 && do_fs && !cur_g) {
                const PopDev& Q = pops[cur_pop];
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) {
                    atomicAnd((unsigned long long*)&Q.accF[w], (unsigned long long)sF[w]);
                    atomicOr((unsigned long long*)&Q.accV[w], (unsigned long long)sV[w]);
                }
                if (CNT && cur_cnt) count_flush(cplanes, maxW, cur_W, cur_A, Q.colcnt);
            }
            __syncthreads();
            cur_pop = (int)p;
            cur_W = st.W;
            cur_A = st.A;
            cur_g = (!SUF || CM) && max(st.W, st.pW) > acc_words;
            cur_cnt = CNT && do_fs && !cur_g && st.count_cols != 0u;
            crows = 0;
            if (cur_g) {
                sF = P.accF;
                sV = P.accV;
                sfix = P.fixmask;
            } else {
                sF = sF0;
                sV = sV0;
                sfix = sfix0;
                if (do_fs)
                    for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) { sF[w] = ~0ull; sV[w] = 0ull; }
                for (uint32_t w = threadIdx.x; w < st.pW; w += blockDim.x) sfix[w] = P.fixmask[w];
            }
            __syncthreads();
        }
        // all effects zero: the gathered sums are exactly zero, skip them
        const bool gather = do_ph && st.nz_eff != 0;
        const uint32_t S = 2u * st.N;
        const uint32_t rpi = ctl->rows_per_item ? ctl->rows_per_item : kRowsPerItem;
        const uint32_t r0 = (item - ctl->item_base[p]) * rpi;
        const uint32_t r1 = min(S, r0 + rpi);
        const uint32_t Se = (S + 1u) >> 1;
        if (CNT && cur_cnt) {  // block-uniform: flush before the counters could overflow
            if (crows + (r1 - r0) > kCountMax) {
                count_flush(cplanes, maxW, cur_W, cur_A, P.colcnt);
                __syncthreads();
                crows = 0;
            }
            crows += r1 - r0;
        }
        const Fold fo{sF, sV, (CNT && cur_cnt) ? cplanes : nullptr, maxW};
        // narrow build: each warp claims its next row one ahead and fetches that row's plan entries into L1
        // behind the current row (narrow rows are bound by their chains of dependent loads)
        uint32_t kc = 0;
        if (NARROW && lane == 0) kc = atomicAdd(&s_next, 1u);
        for (;;) {
            uint32_t k = 0;
            if (NARROW) {
                k = kc;
                if (lane == 0) kc = atomicAdd(&s_next, 1u);
            } else if (lane == 0) {
                k = atomicAdd(&s_next, 1u);
            }
            const uint32_t v = r0 + __shfl_sync(0xffffffffu, k, 0);
            if (v >= r1) break;
            if (NARROW && SUF) {
                const uint32_t vn = r0 + __shfl_sync(0xffffffffu, kc, 0);
                if (vn < r1) {
                    const void* a = lane == 0   ? (const void*)(P.plan_row + vn)
                                    : lane == 1 ? (const void*)(P.plan_mut + vn)
                                                : (const void*)(P.plan_z + (size_t)vn * 4u);
                    if (lane < 3) asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
                }
            }
            // interval classifier: even gametes first, then odd ones (the second
            // gamete of a mate pair is a copy row under the reference's crossover
            // rule), so a CTA runs one kind of row at a time; the suffix-table
            // path takes its rows in plan order
            const uint32_t g = v < Se ? 2u * v : 2u * (v - Se) + 1u;
            if (SUF) {
                // a warp whose copy never landed keeps taking its rows (leaving them undone) and the
                // block's barriers
                if (ws.dead) continue;
                if (!gen_row_suf<PROF, NARROW, CM>(P, st, v, sfix, mask, ws, bphase, wait_limit, do_mut, do_ph, gather,
                                                   do_fs, fo, pc, cs))
                    ws.dead = 1u;
            } else
                gen_row_iv(P, st, g, sfix, s_iv[warp], s_thr[warp], s_q[warp], s_sm[warp], do_mut, do_ph, gather,
                           do_fs, fo);
            if (profile && lane == 0) { rows_done += 1; words_done += st.W; }
        }
        __syncthreads();
    }
    __syncthreads();
    if (cur_pop >= 0 && do_fs && !cur_g) {
        const PopDev& Q = pops[cur_pop];
        for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) {
            atomicAnd((unsigned long long*)&Q.accF[w], (unsigned long long)sF[w]);
            atomicOr((unsigned long long*)&Q.accV[w], (unsigned long long)sV[w]);
        }
        if (CNT && cur_cnt) count_flush(cplanes, maxW, cur_W, cur_A, Q.colcnt);
    }
    if (PROF && lane == 0) {
        pc.c[kPhWarpCyc] = (unsigned long long)(clock64() - c_start);
        pc.c[kPhWarps] = 1;
        for (uint32_t i = 0; i < kPhCount; ++i)
            if (pc.c[i]) atomicAdd((unsigned long long*)&ctl->phase[i], pc.c[i]);
    }
    if (profile && lane == 0 && rows_done) {
        atomicAdd((unsigned long long*)&ctl->rows_done, (unsigned long long)rows_done);
        atomicAdd((unsigned long long*)&ctl->words_done, (unsigned long long)words_done);
    }
}

// One launch of the generation kernel in the given build over the populations of that build (every
// population in a launch of one kind; in a mixed batch the others' items are skipped): per-warp bitmap
// masks (capacities <= kSufMaxSlots, maxW <= 1,024 words), chunk masks (other populations with a
// suffix table) or the interval classifier.  Returns the error of
// the shared-memory opt-in (the kernel is not launched then), else cudaSuccess.
namespace {
constexpr size_t kSmemLimit = 227u * 1024u;   // dynamic shared memory a block may opt into
size_t suf_smem(uint32_t maxW, bool count) {
    return (3ull + kWarps + (count ? kCountPlanes : 0u)) * maxW * sizeof(uint64_t) + kWarps * sizeof(WarpSmem);
}
}  // namespace

bool generation_counts_fit(uint32_t maxW, uint32_t maxA) {
    return maxA <= kSufMaxSlots && suf_smem(maxW, true) <= kSmemLimit;
}

cudaError_t launch_generation(const LaunchCfg& L, const PopDev* pops, uint32_t npops, WorkCtl* ctl, uint32_t maxW,
                              uint32_t maxA, uint32_t fuse, int profile, GenBuild build, bool count_on, bool mixed) {
    const uint32_t mx = mixed ? 1u : 0u;
    // suffix-table populations up to kSufMaxSlots slots build their masks in per-warp bitmaps; wider ones
    // (rows too wide for a bitmap per warp) chunk by chunk from the table
    const bool suf = build != kBuildInterval;
    const bool cm = build == kBuildChunk;
    // the counting build: column counters in shared memory (the phase-clock builds do not count)
    const bool cnt = count_on && profile != 2 && build == kBuildBitmap && generation_counts_fit(maxW, maxA);
    // the interval classifier keeps 3.5 KB of static shared memory per warp, the chunk-mask build a
    // WarpSmem and kCmCorr correction slots per warp in dynamic shared memory; their AND/OR accumulators and
    // fixed mask take what is left of 220 KB, rows of up to acc_words words (wider rows fold into the
    // global accumulators).  acc_words is a multiple of kWordAlign, so every region starts on a 16-byte
    // boundary: the lanes access them as 16-byte word pairs.
    const size_t per_warp = cm ? sizeof(WarpSmem) + kCmCorr * sizeof(uint32_t) : 3584u;
    const size_t acc_fit =
        (220u * 1024u - 4096u - kWarps * per_warp) / (3u * sizeof(uint64_t)) / kWordAlign * kWordAlign;
    // (the chunk-mask build keeps its accumulators to kCmAccWords words, so that L1 keeps room for the
    // table words it prefetches a chunk ahead)
    const uint32_t acc_words = (suf && !cm) ? maxW
                               : cm         ? (uint32_t)std::min<size_t>(maxW, std::min<size_t>(acc_fit, kCmAccWords))
                                            : (uint32_t)std::min<size_t>(maxW, acc_fit);
    const size_t smem = cm    ? 3ull * acc_words * sizeof(uint64_t) + kWarps * per_warp
                        : suf ? suf_smem(maxW, cnt)
                              : 3ull * acc_words * sizeof(uint64_t);
    // profile 2: the suffix-table kernel's build with phase clocks; rows of at most
    // 128 words: its narrow build (copy rows by direct loads)
    const bool narrow = L.narrow_ok && maxW <= 64u * kDirectCopyChunks;
    const int si = cm ? 7 : suf ? (profile == 2 ? (narrow ? 4 : 2) : cnt ? (narrow ? 6 : 5) : narrow ? 3 : 1) : 0;
    const void* fns[8] = {(const void*)k_generation<false, false, false>, (const void*)k_generation<true, false, false>,
                          (const void*)k_generation<true, true, false>, (const void*)k_generation<true, false, true>,
                          (const void*)k_generation<true, true, true>,
                          (const void*)k_generation<true, false, false, true>,
                          (const void*)k_generation<true, false, true, true>,
                          (const void*)k_generation<true, false, false, false, true>};
    // static shared memory is above 48 KB on its own, so the opt-in attribute is always needed; it is a
    // property of the function on each device, so it is kept per device (host threads share the table)
    {
        static std::mutex mu;
        static size_t configured[kMaxGenDevices][8] = {};
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kMaxGenDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(mu);
        size_t& c = configured[dev][si];
        if (smem > c || c == 0) {
            e = cudaFuncSetAttribute(fns[si], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            c = smem > 0 ? smem : 1;
        }
    }
    switch (si) {
        case 7:
            k_generation<true, false, false, false, true><<<L.num_sms, kGenThreads, smem, L.stream>>>(
                pops, npops, ctl, fuse, profile, maxW, acc_words, mx);
            break;
        case 6:
            k_generation<true, false, true, true><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                              profile, maxW, 0u, mx);
            break;
        case 5:
            k_generation<true, false, false, true><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                               profile, maxW, 0u, mx);
            break;
        case 4:
            k_generation<true, true, true><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                       profile, maxW, 0u, mx);
            break;
        case 3:
            k_generation<true, false, true><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                        profile, maxW, 0u, mx);
            break;
        case 2:
            k_generation<true, true, false><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                        profile, maxW, 0u, mx);
            break;
        case 1:
            k_generation<true, false, false><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                        profile, maxW, 0u, mx);
            break;
        default:
            k_generation<false, false, false><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse,
                                                                                         profile, maxW, acc_words, mx);
    }
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
constexpr uint32_t kPlanSmemEv = 16;  // breakpoints of a row the plan kernel ranks in shared memory
constexpr uint32_t kPoisTab = 64;     // entries of the plan kernel's Poisson CDF table

// poisson_inv(u, rho, exp(-rho)) from the table cdf[k] = F_k of the same recurrence: the first k with
// u <= F_k (u and F_k are non-negative, so their bit patterns compare as integers); past the table the
// recurrence goes on from (p, F) at k = kPoisTab - 1, as poisson_inv would.
__device__ __forceinline__ uint32_t poisson_tab(double u, const double* cdf, double plast, double lambda) {
    uint32_t k = 0;
    while (k < kPoisTab && lt_nonneg(cdf[k], u)) ++k;
    if (k < kPoisTab) return k;
    k = kPoisTab - 1u;
    double pk = plast, F = cdf[k];
    while (u > F && k < 4096u) {
        ++k;
        poisson_step(pk, F, lambda, k);
    }
    return k;
}

// Processing order of the offspring rows (parent-major): rows are sorted by
// parent individual, so rows reading the same parent strands run side by side
// and the second read of a strand is an L2 hit.  Counting sort by key; the
// order inside one key does not matter (rows are independent).  Keys 0 and 2
// (by gamete parity first) are kept for measurement.
#ifndef CLOTHO_ORDER_KEY
#define CLOTHO_ORDER_KEY 1
#endif
__device__ __forceinline__ uint32_t order_key(const PopDev& P, uint32_t g, uint32_t N, uint32_t pN) {
    uint32_t pind = P.pairs[g];
    if (pind >= pN) pind = 0;
#if CLOTHO_ORDER_KEY == 1
    return pind;                                  // parent only
#elif CLOTHO_ORDER_KEY == 2
    return (g & 1u) * N + (g >> 1);               // even rows, then odd rows
#else
    return (g & 1u) * N + pind;                   // parity, then parent
#endif
}

__global__ void k_ord_count(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        if (!P.plan_row) continue;
        const uint32_t N = P.st->N, pN = P.st->pN, S = 2u * N;
        for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < S; g += gridDim.x * blockDim.x)
            atomicAdd(&P.ord_cnt[order_key(P, g, N, pN)], 1u);
    }
}

__global__ void k_ord_scatter(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        if (!P.plan_row) continue;
        const uint32_t N = P.st->N, pN = P.st->pN, S = 2u * N;
        for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < S; g += gridDim.x * blockDim.x) {
            const uint32_t key = order_key(P, g, N, pN);
            P.ord_pos[g] = P.ord_off[key] + atomicAdd(&P.ord_cur[key], 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// Per-row crossover plans for the suffix-table classifier, one thread per row:
// the top strand (parent individual and strand swap), the breakpoint count,
// and for every breakpoint its nearest table row and correction ranks; plus
// the direction of the phenotype gather.  Device-drawn breakpoints get their
// plan entries from a block-aggregated counter; tape rows use the tape's own
// event offsets.
__global__ void __launch_bounds__(256) k_row_plan(const PopDev* __restrict__ pops, uint32_t npops) {
    const uint32_t lane = threadIdx.x & 31u;
    // a thread's thresholds (up to kPlanSmemEv) stay in shared memory while they are ranked
    // against each other; longer lists use their global slots
    __shared__ uint32_t s_cr[256][kPlanSmemEv + 1];
    // the population's Poisson(rho) CDF, built by the same FP64 recurrence as poisson_inv and
    // searched with integer compares, so a breakpoint count costs no FP64 work
    __shared__ double s_cdf[kPoisTab];
    __shared__ double s_plast;
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        if (!P.plan_row) continue;
        __syncthreads();  // the previous population's table is no longer read
        if (threadIdx.x == 0) {
            double pk = P.exp_neg_rho, F = pk;
            s_cdf[0] = F;
            for (uint32_t k = 1; k < kPoisTab; ++k) {
                poisson_step(pk, F, P.rho, k);
                s_cdf[k] = F;
            }
            s_plast = pk;
        }
        __syncthreads();
        const DevStatus st = *P.st;
        const uint32_t S = 2u * st.N, A = st.A, Se = (S + 1u) >> 1;
        const bool philox = P.mode == kModePhilox;
        const bool q1 = (P.flags & 1u) != 0;
        for (uint32_t v0 = blockIdx.x * blockDim.x; v0 < S; v0 += gridDim.x * blockDim.x) {
            const uint32_t v = v0 + threadIdx.x;
            const bool live = v < S;
            // even gametes on the first half of the threads, odd ones on the second:
            // under the reference's crossover rule odd gametes are copy rows, so a
            // warp holds one kind of row
            const uint32_t g = v < Se ? 2u * v : 2u * (v - Se) + 1u;
            uint32_t pind = 0, E = 0, base = 0, flags = 0;
            bool swap = false;
            if (live) {
                pind = P.pairs[g];
                if (pind >= st.pN) {
                    atomicOr(&P.st->err, kErrParent);
                    pind = 0;
                }
                if (philox) {
                    const U4 x = philox4x32(g, 0u, st.gen, kStreamGamete, P.seed);
                    E = (q1 && (g & 1u)) ? 0u : poisson_tab(u01(x.x, x.y), s_cdf, s_plast, P.rho);
                    swap = lt_nonneg(u01(x.z, x.w), P.bias);
                    if (E > kMaxEvDevice) {
                        atomicOr(&P.st->err, kErrEvents);
                        E = kMaxEvDevice;
                    }
                } else {
                    swap = P.swap[g] != 0;
                    base = P.ev_off[g];
                    E = (q1 && (g & 1u)) ? 0u : P.ev_off[g + 1u] - base;
                }
            }
            if (philox) {  // warp-aggregated allocation of the plan entries
                uint32_t incl = E;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= (uint32_t)o) incl += y;
                }
                const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
                uint32_t b0 = 0;
                if (lane == 0 && tot) b0 = atomicAdd(&P.st->ev_used, tot);
                base = __shfl_sync(0xffffffffu, b0, 0) + incl - E;
                if (E && base + E > P.EVcap) {
                    atomicOr(&P.st->err, kErrEvents);
                    E = 0;
                }
            }
            if (!live) continue;
            // what the plan entry needs besides the breakpoints, fetched before the breakpoint work so that
            // their round trips overlap it: the processing position, the new alleles' CSR range, and the
            // carried phenotypes of both parent strands (one 64-byte line; the gather direction picks one)
            const uint32_t at = P.ord_pos[g];
            const uint32_t mo = P.row_off[g], mend = P.row_off[g + 1u];
            const uint32_t topr = 2u * pind + (swap ? 1u : 0u);
            asm volatile("prefetch.global.L1 [%0];" ::"l"(P.zg[st.cur ^ 1u] + (size_t)(topr & ~1u) * 4u));
            if (E > kMaxEvDevice) {
                flags = kPlanLong;  // tape rows with very long event lists: direct compares
            } else if (E > 0) {
                uint32_t* cr = E <= kPlanSmemEv ? s_cr[threadIdx.x] : P.plan_cr + base;
                // the chunk-mask build classifies rows of more than kCmMaxEv breakpoints by direct compares
                // against their positions, which device-drawn rows keep in the event list for it (every
                // population's, to keep the plan kernel uniform; rare: E > 16)
                const bool keep_pos = philox && E > kCmMaxEv;
                for (uint32_t k = 0; k < E; k += 2u) {
                    double e0, e1 = 0.0;
                    if (philox) {
                        const U4 a = philox4x32(g, 1u + (k >> 1), st.gen, kStreamGamete, P.seed);
                        e0 = u01(a.x, a.y);
                        e1 = u01(a.z, a.w);
                        if (keep_pos) {
                            P.ev_pos[base + k] = e0;
                            if (k + 1u < E) P.ev_pos[base + k + 1u] = e1;
                        }
                    } else {
                        e0 = __ldg(P.ev_pos + base + k);
                        if (k + 1u < E) e1 = __ldg(P.ev_pos + base + k + 1u);
                    }
                    cr[k] = threshold_rank(P, e0);
                    if (k + 1u < E) cr[k + 1u] = threshold_rank(P, e1);
                }
                // share of the rank space the breakpoints switch: sorted thresholds pair into intervals
                int64_t len = (E & 1u) ? (int64_t)A : 0;
                for (uint32_t k = 0; k < E; ++k) {
                    const uint32_t rk = cr[k];
                    uint32_t posn = 0;
                    for (uint32_t j = 0; j < E; ++j) {
                        const uint32_t rj = cr[j];
                        posn += (rj < rk || (rj == rk && j < k)) ? 1u : 0u;
                    }
                    len += (posn & 1u) ? (int64_t)rk : -(int64_t)rk;
                }
                if (2 * len > (int64_t)A) flags |= kPlanInv;
                for (uint32_t k = 0; k < E; ++k) {
                    uint32_t c0, n;
                    const uint32_t b = table_row(cr[k], A, c0, n);
                    P.plan_go[base + k] = (b >> 6) * P.Wcap;
                    P.plan_cr[base + k] = c0 | (n << 20);
                }
            }
            if (E > kPlanMaxEvents) {
                atomicOr(&P.st->err, kErrEvents);
                E = 0;
                flags = 0;
            }
            P.plan_row[at] = make_uint4(g, topr, base, E | (flags << kPlanFlagShift));
            // what the row's set-up would otherwise fetch after its plan: the new alleles' CSR
            // range and the carried phenotype's base strand value less the fixed effects
            P.plan_mut[at] = make_uint2(mo, mend - mo);
            const uint32_t zs = ((flags & kPlanInv) && st.nz_eff != 0) ? topr ^ 1u : topr;
            const double* zp = P.zg[st.cur ^ 1u] + (size_t)zs * 4u;
#pragma unroll
            for (uint32_t t = 0; t < kMaxTraits; ++t) P.plan_z[(size_t)at * 4u + t] = zp[t] - P.st->fixsum[t];
        }
    }
}

int init_recip_gen() { return fill_recip_table(); }

void launch_order(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxS) {
    const dim3 g = pop_grid(npops, blocks_for(maxS, 256), L.num_sms, 8);
    k_ord_count<<<g, 256, 0, L.stream>>>(pops, npops);
    launch_uscan_order(L, pops, npops, maxS);
    k_ord_scatter<<<g, 256, 0, L.stream>>>(pops, npops);
}

void launch_row_plan(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxS) {
    k_row_plan<<<pop_grid(npops, blocks_for(maxS, 256), L.num_sms, 8), 256, 0, L.stream>>>(pops, npops);
}

void launch_plan(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxS) {
    launch_order(L, pops, npops, maxS);
    launch_row_plan(L, pops, npops, maxS);
}

// ---------------------------------------------------------------------------
// Position ranks for the crossover classifiers, rebuilt every generation over
// the slots [0, A): counting sort of positions into NB buckets, then each
// slot's rank = slots in lower buckets + slots of its own bucket with a
// smaller position (or the same position and a lower slot index).  inv is the
// inverse map (rank -> slot); suf is the suffix table of the classifier.
__global__ void k_rank_count(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const uint32_t A = P.st->A;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < A; s += gridDim.x * blockDim.x)
            atomicAdd(&P.bcnt[pos_bucket(P.pos[s], P.NB)], 1u);
    }
}
__global__ void k_rank_scatter(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const uint32_t A = P.st->A;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < A; s += gridDim.x * blockDim.x) {
            const double x = P.pos[s];
            const uint32_t b = pos_bucket(x, P.NB);
            const uint32_t k = P.boff[b] + atomicAdd(&P.bcur[b], 1u);
            P.bpos[k] = x;
            P.bslot[k] = s;
        }
    }
}
__global__ void k_rank_final(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const uint32_t A = P.st->A;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < A; s += gridDim.x * blockDim.x) {
            const double x = P.pos[s];
            const uint32_t b = pos_bucket(x, P.NB);
            const uint32_t k0 = P.boff[b], k1 = P.boff[b + 1u];
            uint32_t r = k0;
            for (uint32_t k = k0; k < k1; ++k) {
                const double y = P.bpos[k];
                r += (y < x || (y == x && P.bslot[k] < s)) ? 1u : 0u;
            }
            P.rank[s] = r;
            if (P.inv) P.inv[r] = s;
        }
    }
}

// suf[g * Wcap + w] = bits of word w whose slot has rank >= 64 g, for
// g = 0 .. ceil(A/64) (the last row is empty).  A unit of work is 32 words and
// every kSufSlices-th table row; the units are spread over the whole grid from
// the current width, so the blocks are busy however wide the capacity is.
constexpr uint32_t kSufSlices = 16;
__global__ void __launch_bounds__(256) k_suf_build(const PopDev* __restrict__ pops, uint32_t npops) {
    __shared__ uint32_t s_grp[32][65];  // (rank >> 6) + 1 per slot, 0 beyond A
    const uint32_t tx = threadIdx.x & 31u, ty = threadIdx.x >> 5;
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        if (!P.suf) continue;
        const uint32_t A = P.st->A, W = P.st->W;
        const uint32_t Gt = (A + 63u) >> 6;
        const uint32_t wblocks = (W + 31u) / 32u;
        for (uint32_t u = blockIdx.x; u < wblocks * kSufSlices; u += gridDim.x) {
            const uint32_t wb = (u % wblocks) * 32u, slice = u / wblocks;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < 2048u; i += blockDim.x) {
                const uint32_t s = wb * 64u + i;
                s_grp[i >> 6][i & 63u] = (s < A) ? (P.rank[s] >> 6) + 1u : 0u;
            }
            __syncthreads();
            const uint32_t w = wb + tx;
            if (w >= W) continue;
            for (uint32_t g = slice * 8u + ty; g <= Gt; g += kSufSlices * 8u) {
                uint64_t m = 0;
#pragma unroll 16
                for (uint32_t b = 0; b < 64u; ++b) m |= (uint64_t)(s_grp[tx][b] > g) << b;
                P.suf[(size_t)g * P.Wcap + w] = m;
            }
        }
    }
}

void launch_ranks(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxNB, uint32_t maxW,
                  bool suf) {
    const dim3 g = pop_grid(npops, L.num_sms * 2u, L.num_sms, 2);
    k_rank_count<<<g, 256, 0, L.stream>>>(pops, npops);
    launch_uscan_buckets(L, pops, npops, maxNB);
    k_rank_scatter<<<g, 256, 0, L.stream>>>(pops, npops);
    k_rank_final<<<g, 256, 0, L.stream>>>(pops, npops);
    if (suf) {
        const uint32_t units = (maxW + 31u) / 32u * kSufSlices;
        k_suf_build<<<pop_grid(npops, units, L.num_sms, 4), 256, 0, L.stream>>>(pops, npops);
    }
}

// ---------------------------------------------------------------------------
// Full per-genome phenotype (staged API and population set-up):
// BatchPhenotypeMT<...row>::updateHaploidGenomeWeights
// (batch_phenotype_mt_population_space_row.hpp:111-132), one warp per genome,
// FP32 lane sums combined in FP64.
__global__ void __launch_bounds__(256) k_phenotype(const PopDev* __restrict__ pops, uint32_t npops) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const DevStatus st = *P.st;
        const uint32_t S = 2u * st.N, W = st.W;
        const uint64_t* rows = P.rows[st.cur];
        double* zcur = P.zg[st.cur];
        for (uint32_t g = gw; g < S; g += nw) {
            float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
            const uint64_t* r = rows + (size_t)g * P.Wcap;
            for (uint32_t w = 2u * lane; w < W; w += 64u) {
                const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(r + w);
                // all set bits, sign +1 (b = x, so every bit counts as brought in)
                switched_effects(x.x, x.y, x.x, x.y, w * 64u, reinterpret_cast<const float4*>(P.eff), d);
            }
#pragma unroll
            for (uint32_t t = 0; t < kMaxTraits; ++t) {
                double v = (double)d[t];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == t) zcur[(size_t)g * 4u + t] = v;
            }
        }
    }
}
void launch_phenotype(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_phenotype<<<pop_grid(npops, L.num_sms * 8u, L.num_sms, 8), 256, 0, L.stream>>>(pops, npops);
}

}  // namespace clotho
