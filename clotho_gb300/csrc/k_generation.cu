// k_generation.cu -- the fused generation pass: one warp builds one offspring
// row in a single sweep over its parent's two rows.
//
// Per row (gamete g of mate pair g/2, parent individual pairs[g]):
//   crossover  batch_crossover_taskwe<...population_space_row>::run_crossover_task
//              (crossover/batch_crossover_taskwe_population_space_row.hpp:157-217)
//              and block_crossover::crossover (crossover/block_crossover.hpp:46-63):
//              only heterozygous bits are classified; a bit takes the bottom
//              strand iff an odd number of breakpoints is <= its position
//              (upper_bound in region_classifier, classifiers/region_classifier.hpp:62-77).
//              Positions are replaced by integer ranks (rank(s) = #{slots with a
//              smaller position}); breakpoint e becomes r(e) = #{slots with
//              position < e}, and e <= pos(s)  <=>  r(e) <= rank(s) for every slot,
//              ties included.  Sorted thresholds pair into half-open rank
//              intervals; a het bit switches strand iff its rank lies in one.
//              Fixed columns are masked on load: the in-register form of
//              remove_fixed_allele (population_space_row_block.hpp:127-147).
//   mutation   XOR of the row's new alleles (population_space_row_block.hpp:111-125)
//              in registers before the store.
//   phenotype  z(child) = z(top strand) - sum(fixed) + sum(switched bits: bottom-top)
//              + sum(new alleles): the per-genome sum of
//              batch_phenotype_task_population_space_row.hpp:127-153, carried
//              from the parent row instead of re-walking every set bit.
//              Per-lane FP32 partial sums, FP64 per-genome values.
//   free space AND/OR of the finished words, the next generation's
//              FreeSpaceAnalyzerMT input (free_space_task_population_space_row_interlaced.hpp:51-72).
//
// Rows are 64-word chunks, two words (one 128-bit load) per lane; parent words
// are loaded two chunks ahead of use.  The het-bit walk runs the lane's four
// 32-bit halves as independent chains (branch-free steps) so shared-memory
// and ALU latencies overlap.  The kernel is persistent: one CTA per SM takes
// 512-row items from a device counter and its warps claim rows one at a time,
// so warps never wait on each other inside an item.
#include "engine.cuh"

namespace clotho {

namespace {

constexpr uint32_t kWarps = kGenThreads / 32;
constexpr uint32_t kMaxIvSmem = 64;     // rank intervals in shared memory (E <= 128)

constexpr uint32_t kMaxIv = 8;          // rank intervals held in registers (E <= 16)

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

template <bool SR>
__device__ __forceinline__ uint32_t slot_rank(uint32_t s, const uint16_t* srank, const uint32_t* __restrict__ grank) {
    return SR ? (uint32_t)srank[s] : __ldg(grank + s);
}

// One branch-free step of a het-bit chain: classify the lowest bit of h.
template <int NI, bool SR>
__device__ __forceinline__ void xo_step(uint32_t& h, uint32_t& m, uint32_t base, const uint16_t* srank,
                                        const uint32_t* __restrict__ grank, const RowXo& X) {
    const bool nz = h != 0u;
    const uint32_t j = nz ? (uint32_t)(__ffs(h) - 1) : 0u;
    h &= h - 1u;
    const uint32_t r = slot_rank<SR>(base + j, srank, grank);
    const bool s = nz && in_iv<NI>(r, X);
    m |= (uint32_t)s << j;
}

// Switched-strand masks of the lane's two words: four interleaved 32-bit chains.
template <int NI, bool SR>
__device__ __forceinline__ void classify(uint64_t h0, uint64_t h1, uint32_t s0, const uint16_t* srank,
                                         const uint32_t* __restrict__ grank, const RowXo& X, uint64_t& m0,
                                         uint64_t& m1) {
    uint32_t a = (uint32_t)h0, b = (uint32_t)(h0 >> 32), c = (uint32_t)h1, d = (uint32_t)(h1 >> 32);
    uint32_t ma = 0, mb = 0, mc = 0, md = 0;
    while (a | b | c | d) {
        xo_step<NI, SR>(a, ma, s0, srank, grank, X);
        xo_step<NI, SR>(b, mb, s0 + 32u, srank, grank, X);
        xo_step<NI, SR>(c, mc, s0 + 64u, srank, grank, X);
        xo_step<NI, SR>(d, md, s0 + 96u, srank, grank, X);
    }
    m0 = (uint64_t)ma | ((uint64_t)mb << 32);
    m1 = (uint64_t)mc | ((uint64_t)md << 32);
}

constexpr uint32_t kQueueCap = 512;    // het bits per warp-chunk handled by the balanced path

// Warp-balanced classification of one 64-word chunk.  Each lane pushes the
// het bits of its two words into the warp's queue (slot, plus bit 31 when the
// bottom strand carries the allele); the whole warp then classifies the queue
// four entries per lane at a time, ORs switched bits into the warp's chunk
// mask and adds +-effect for each switched allele.  H = total het bits.
template <int NI, bool SR>
__device__ __forceinline__ void classify_balanced(uint64_t h0, uint64_t h1, uint64_t b0, uint64_t b1, uint32_t w,
                                                  uint32_t w0, uint32_t off, uint32_t H, uint32_t* Q,
                                                  uint32_t* SM, const uint16_t* srank,
                                                  const uint32_t* __restrict__ grank, const RowXo& X,
                                                  const float4* __restrict__ eff4, bool do_ph,
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
            const uint32_t slot = e[k] & 0x7fffffffu;
            const uint32_t r = slot_rank<SR>(slot, srank, grank);
            sw[k] = (i < H) && in_iv<NI>(r, X);
        }
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
            if (sw[k]) {
                const uint32_t loc = (e[k] & 0x7fffffffu) - sbase;
                atomicOr(&SM[loc >> 5], 1u << (loc & 31u));
            }
        }
        if (do_ph) {
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

// r(e) = #{slots with position < e} through the position buckets.
__device__ __forceinline__ uint32_t threshold_rank(const PopDev& P, double e) {
    const uint32_t b = pos_bucket(e, P.NB);
    const uint32_t k0 = __ldg(P.boff + b), k1 = __ldg(P.boff + b + 1u);
    uint32_t r = k0;
    for (uint32_t k = k0; k < k1; ++k) r += (__ldg(P.bpos + k) < e) ? 1u : 0u;
    return r;
}

// Per-row crossover mode
enum XoKind : int { kXoCopy = 0, kXoIv4 = 4, kXoIv8 = 8, kXoFar = -1, kXoEvents = -2 };

struct RowArgs {
    const uint64_t* top;
    const uint64_t* bot;
    uint64_t* out;
    uint32_t Wc, Wp;
    uint32_t mc, mo, my_slot;
    uint32_t E;
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

template <int KIND, bool SR>
__device__ __forceinline__ void row_body(const PopDev& P, const DevStatus& st, const RowArgs& R,
                                         const uint16_t* srank, const uint64_t* sfix, const RowXo& X, uint32_t* Q,
                                         uint32_t* SM, bool do_mut, bool do_ph, bool do_fs, uint64_t* sF,
                                         uint64_t* sV, float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    constexpr bool xo = (KIND != kXoCopy);
    const float4* eff4 = reinterpret_cast<const float4*>(P.eff);
    // two chunks of parent words in flight ahead of the one being processed
    ulonglong2 t_a, b_a, t_b, b_b;
    load_pair(t_a, b_a, R, 2u * lane, xo);
    load_pair(t_b, b_b, R, 2u * lane + 64u, xo);
    for (uint32_t w0 = 0; w0 < R.Wc; w0 += 64u) {
        const uint32_t w = w0 + 2u * lane;
        ulonglong2 t_c, b_c;
        load_pair(t_c, b_c, R, w + 128u, xo);
        // XOR masks of this lane's two words from the row's new alleles
        uint64_t mx0 = 0, mx1 = 0;
        if (do_mut && R.mc) {
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
                    classify_balanced<(KIND > 0 ? KIND : 0), SR>(h0, h1, b0, b1, w, w0, incl - c, H, Q, SM, srank,
                                                                  P.rank, X, eff4, do_ph, d, m0, m1);
                } else {
                    classify<(KIND > 0 ? KIND : 0), SR>(h0, h1, w * 64u, srank, P.rank, X, m0, m1);
                    if (do_ph) switched_effects(m0, m1, b0, b1, w * 64u, eff4, d);
                }
            } else {
                m0 = sw_mask_events(h0, w * 64u, P.pos, R.evg, R.E);
                m1 = sw_mask_events(h1, w * 64u + 64u, P.pos, R.evg, R.E);
                if (do_ph) switched_effects(m0, m1, b0, b1, w * 64u, eff4, d);
            }
            x0 = (t0 & ~m0) | (b0 & m0);
            x1 = (t1 & ~m1) | (b1 & m1);
        }
        if (live) {
            x0 ^= mx0;
            x1 ^= mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) fold_fs(sF, sV, w, x0, x1);
        }
        t_a = t_b; b_a = b_b;
        t_b = t_c; b_b = b_c;
    }
}

// One offspring row, the whole warp.
template <bool SR>
__device__ __forceinline__ void gen_row(const PopDev& P, const DevStatus& st, uint32_t g, const uint16_t* srank,
                                        const uint64_t* sfix, uint2* s_iv, uint32_t* s_thr, uint32_t* Q,
                                        uint32_t* SM, bool do_mut, bool do_ph, bool do_fs, uint64_t* sF,
                                        uint64_t* sV) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t* prow = P.rows[st.cur ^ 1u];
    uint64_t* crow = P.rows[st.cur];
    const bool q1 = (P.flags & 1u) != 0;
    const bool philox = P.mode == kModePhilox;
    // ---- parent strands and the strand-swap bit of gamete g
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
    RowArgs R;
    R.top = prow + (size_t)topr * P.Wcap;
    R.bot = prow + (size_t)(topr ^ 1u) * P.Wcap;
    R.out = crow + (size_t)g * P.Wcap;
    R.Wc = st.W;
    R.Wp = st.pW;
    R.E = E;
    R.evg = evg;
    R.philox = philox;

    // ---- breakpoints -> sorted rank thresholds -> intervals
    RowXo X;
#pragma unroll
    for (uint32_t k = 0; k < kMaxIv; ++k) { X.a[k] = 0; X.l[k] = 0; }
    X.iv = s_iv;
    X.niv = 0;
    int kind = kXoCopy;
    if (E > 0 && E <= kMaxEvDevice) {
        for (uint32_t k = lane; k < E; k += 32u) {
            double e;
            if (philox) {
                const U4 a = philox4x32(g, 1u + (k >> 1), st.gen, kStreamGamete, P.seed);
                e = (k & 1u) ? u01(a.z, a.w) : u01(a.x, a.y);
            } else {
                e = __ldg(evg + k);
            }
            s_thr[k] = threshold_rank(P, e);
        }
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

    // ---- new alleles of this row (slot indices), lanes hold up to 32
    R.mo = 0;
    R.mc = 0;
    R.my_slot = 0xffffffffu;
    float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
    const float4* eff4 = reinterpret_cast<const float4*>(P.eff);
    if (do_mut) {
        R.mo = P.row_off[g];
        R.mc = P.row_off[g + 1u] - R.mo;
        if (lane < R.mc) {
            const uint32_t i = R.mo + lane;
            const uint32_t mi = philox ? i : P.row_mut[i];
            R.my_slot = (mi < st.M) ? P.mut_slot[mi] : 0xffffffffu;
            if (do_ph && R.my_slot != 0xffffffffu) {
                const float4 e = __ldg(eff4 + R.my_slot);
                d[0] += e.x; d[1] += e.y; d[2] += e.z; d[3] += e.w;
            }
        }
        if (do_ph && R.mc > 32u && lane == 0) {
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

    switch (kind) {
        case kXoCopy: row_body<kXoCopy, SR>(P, st, R, srank, sfix, X, Q, SM, do_mut, do_ph, do_fs, sF, sV, d); break;
        case kXoIv4: row_body<kXoIv4, SR>(P, st, R, srank, sfix, X, Q, SM, do_mut, do_ph, do_fs, sF, sV, d); break;
        case kXoIv8: row_body<kXoIv8, SR>(P, st, R, srank, sfix, X, Q, SM, do_mut, do_ph, do_fs, sF, sV, d); break;
        case kXoFar: row_body<kXoFar, SR>(P, st, R, srank, sfix, X, Q, SM, do_mut, do_ph, do_fs, sF, sV, d); break;
        default: row_body<kXoEvents, SR>(P, st, R, srank, sfix, X, Q, SM, do_mut, do_ph, do_fs, sF, sV, d); break;
    }
    if (do_ph) {
        double z[kMaxTraits];
#pragma unroll
        for (uint32_t t = 0; t < kMaxTraits; ++t) {
            double v = (double)d[t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            z[t] = v;
        }
        if (lane < kMaxTraits) {
            const double zt = P.zg[st.cur ^ 1u][(size_t)topr * 4u + lane];
            const double zz = lane == 0 ? z[0] : lane == 1 ? z[1] : lane == 2 ? z[2] : z[3];
            P.zg[st.cur][(size_t)g * 4u + lane] = (zt - P.st->fixsum[lane]) + zz;
        }
    }
}

}  // namespace

// Dynamic shared memory: [AND acc: maxW][OR acc: maxW][fixed mask: maxW] u64,
// then (SR) the slot ranks as u16 [maxR].
template <bool SR>
__global__ void __launch_bounds__(kGenThreads, 1)
k_generation(const PopDev* __restrict__ pops, uint32_t npops, WorkCtl* __restrict__ ctl, uint32_t fuse,
             int profile, uint32_t maxW, uint32_t maxR) {
    extern __shared__ __align__(16) uint64_t s_dyn[];
    __shared__ uint2 s_iv[kWarps][kMaxIvSmem];
    __shared__ uint32_t s_thr[kWarps][kMaxEvDevice];
    __shared__ uint32_t s_q[kWarps][kQueueCap];
    __shared__ uint32_t s_sm[kWarps][128];
    __shared__ uint32_t s_item, s_next;
    uint64_t* sF = s_dyn;
    uint64_t* sV = s_dyn + maxW;
    uint64_t* sfix = s_dyn + 2u * maxW;
    uint16_t* srank = reinterpret_cast<uint16_t*>(s_dyn + 3u * maxW);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const bool do_mut = (fuse & kFuseMut) != 0, do_ph = (fuse & kFusePheno) != 0, do_fs = (fuse & kFuseFs) != 0;
    int cur_pop = -1;
    uint32_t cur_W = 0;
    uint64_t rows_done = 0, words_done = 0;

    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(&ctl->gen_counter, 1u);
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
        const DevStatus st = *P.st;
        if ((int)p != cur_pop) {
            if (cur_pop >= 0 && do_fs) {
                const PopDev& Q = pops[cur_pop];
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) {
                    atomicAnd((unsigned long long*)&Q.accF[w], (unsigned long long)sF[w]);
                    atomicOr((unsigned long long*)&Q.accV[w], (unsigned long long)sV[w]);
                }
            }
            __syncthreads();
            cur_pop = (int)p;
            cur_W = st.W;
            if (do_fs)
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) { sF[w] = ~0ull; sV[w] = 0ull; }
            for (uint32_t w = threadIdx.x; w < st.pW; w += blockDim.x) sfix[w] = P.fixmask[w];
            if (SR)
                for (uint32_t s = threadIdx.x; s < st.A && s < maxR; s += blockDim.x) srank[s] = (uint16_t)P.rank[s];
            __syncthreads();
        }
        const uint32_t S = 2u * st.N;
        const uint32_t rpi = ctl->rows_per_item ? ctl->rows_per_item : kRowsPerItem;
        const uint32_t r0 = (item - ctl->item_base[p]) * rpi;
        const uint32_t r1 = min(S, r0 + rpi);
        for (;;) {
            uint32_t k = 0;
            if (lane == 0) k = atomicAdd(&s_next, 1u);
            const uint32_t g = r0 + __shfl_sync(0xffffffffu, k, 0);
            if (g >= r1) break;
            gen_row<SR>(P, st, g, srank, sfix, s_iv[warp], s_thr[warp], s_q[warp], s_sm[warp], do_mut, do_ph, do_fs,
                        sF, sV);
            if (profile && lane == 0) { rows_done += 1; words_done += st.W; }
        }
        __syncthreads();
    }
    __syncthreads();
    if (cur_pop >= 0 && do_fs) {
        const PopDev& Q = pops[cur_pop];
        for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) {
            atomicAnd((unsigned long long*)&Q.accF[w], (unsigned long long)sF[w]);
            atomicOr((unsigned long long*)&Q.accV[w], (unsigned long long)sV[w]);
        }
    }
    if (profile && lane == 0 && rows_done) {
        atomicAdd((unsigned long long*)&ctl->rows_done, (unsigned long long)rows_done);
        atomicAdd((unsigned long long*)&ctl->words_done, (unsigned long long)words_done);
    }
}

// Shared-memory rank table: u16 ranks are used when every population has
// A <= 65,536 and the layout fits the opt-in shared-memory limit.
void launch_generation(const LaunchCfg& L, const PopDev* pops, uint32_t npops, WorkCtl* ctl, uint32_t maxW,
                       uint32_t maxA, uint32_t fuse, int profile) {
    const size_t static_smem = sizeof(uint2) * kWarps * kMaxIvSmem + sizeof(uint32_t) * kWarps * kMaxEvDevice +
                               sizeof(uint32_t) * kWarps * (kQueueCap + 128) + 64;
    const size_t base = 3ull * maxW * sizeof(uint64_t);
    uint32_t maxR = (maxA <= 65536u) ? ((maxA + 7u) & ~7u) : 0u;
    if (base + 2ull * maxR + static_smem > 227u * 1024u) maxR = 0;
    const size_t smem = base + 2ull * maxR;
    static size_t configured[2] = {0, 0};
    const int sr = maxR > 0 ? 1 : 0;
    if (smem + static_smem > 48u * 1024u && smem > configured[sr]) {
        if (sr) cudaFuncSetAttribute(k_generation<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        else cudaFuncSetAttribute(k_generation<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured[sr] = smem;
    }
    if (sr) k_generation<true><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse, profile, maxW, maxR);
    else k_generation<false><<<L.num_sms, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse, profile, maxW, 0u);
}

// ---------------------------------------------------------------------------
// Position ranks for the crossover classifier, rebuilt every generation over
// the slots [0, A): counting sort of positions into NB buckets, then each
// slot's rank = slots in lower buckets + smaller positions in its own bucket.
__global__ void k_rank_count(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = 0; p < npops; ++p) {
        const PopDev& P = pops[p];
        const uint32_t A = P.st->A;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < A; s += gridDim.x * blockDim.x)
            atomicAdd(&P.bcnt[pos_bucket(P.pos[s], P.NB)], 1u);
    }
}
__global__ void k_rank_scatter(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = 0; p < npops; ++p) {
        const PopDev& P = pops[p];
        const uint32_t A = P.st->A;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < A; s += gridDim.x * blockDim.x) {
            const double x = P.pos[s];
            const uint32_t b = pos_bucket(x, P.NB);
            const uint32_t k = atomicAdd(&P.bcur[b], 1u);
            P.bpos[P.boff[b] + k] = x;
        }
    }
}
__global__ void k_rank_final(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = 0; p < npops; ++p) {
        const PopDev& P = pops[p];
        const uint32_t A = P.st->A;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < A; s += gridDim.x * blockDim.x) {
            const double x = P.pos[s];
            const uint32_t b = pos_bucket(x, P.NB);
            const uint32_t k0 = P.boff[b], k1 = P.boff[b + 1u];
            uint32_t r = k0;
            for (uint32_t k = k0; k < k1; ++k) r += (P.bpos[k] < x) ? 1u : 0u;
            P.rank[s] = r;
        }
    }
}
void launch_ranks(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxNB) {
    const int g = L.num_sms * 2;
    k_rank_count<<<g, 256, 0, L.stream>>>(pops, npops);
    launch_uscan_buckets(L, pops, npops, maxNB);
    k_rank_scatter<<<g, 256, 0, L.stream>>>(pops, npops);
    k_rank_final<<<g, 256, 0, L.stream>>>(pops, npops);
}

// ---------------------------------------------------------------------------
// Full per-genome phenotype (staged API and population set-up):
// BatchPhenotypeMT<...row>::updateHaploidGenomeWeights
// (batch_phenotype_mt_population_space_row.hpp:111-132), one warp per genome,
// FP32 lane sums combined in FP64.
__global__ void __launch_bounds__(256) k_phenotype(const PopDev* __restrict__ pops, uint32_t npops) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = 0; p < npops; ++p) {
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
    k_phenotype<<<L.num_sms * 8, 256, 0, L.stream>>>(pops, npops);
}

}  // namespace clotho
