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
// Rows are 64-word chunks, two words (one 128-bit load) per lane; the next
// chunk's parent words are loaded while the current one is processed.  The
// kernel is persistent: CTAs take 64-row items from a device counter.
#include "engine.cuh"

namespace clotho {

namespace {

constexpr uint32_t kWarps = kGenThreads / 32;
constexpr uint32_t kMaxIv = 8;          // rank intervals held in registers (E <= 16)
constexpr uint32_t kMaxIvSmem = 64;     // rank intervals in shared memory (E <= 128)

struct Intervals {
    uint32_t a[kMaxIv];   // interval start (rank)
    uint32_t l[kMaxIv];   // length; 0 = empty
};

template <int NI>
__device__ __forceinline__ bool in_iv(uint32_t r, const Intervals& iv) {
    bool s = false;
#pragma unroll
    for (int k = 0; k < NI; ++k) s |= (r - iv.a[k]) < iv.l[k];
    return s;
}

__device__ __forceinline__ bool in_iv_far(uint32_t r, const uint2* iv, uint32_t n) {
    bool s = false;
    for (uint32_t k = 0; k < n; ++k) s |= (r - iv[k].x) < iv[k].y;
    return s;
}

// Parity mask of one 32-bit half: bits of h whose slot rank is inside an interval.
template <int NI>
__device__ __forceinline__ uint32_t sw_mask32(uint32_t h, uint32_t base, const uint32_t* __restrict__ rank,
                                              const Intervals& iv, const uint2* far, uint32_t nfar) {
    uint32_t m = 0;
    while (h) {
        const uint32_t j = __ffs(h) - 1u;
        h &= h - 1u;
        const uint32_t r = __ldg(rank + base + j);
        bool s;
        if (NI > 0) s = in_iv<NI>(r, iv);
        else s = in_iv_far(r, far, nfar);
        m |= (uint32_t)s << j;
    }
    return m;
}

// Bits of h whose slot position is >= an odd number of the events (direct
// double compares against the event list; used only for very long lists).
__device__ __forceinline__ uint32_t sw_mask32_events(uint32_t h, uint32_t base, const double* __restrict__ pos,
                                                     const double* __restrict__ ev, uint32_t E) {
    uint32_t m = 0;
    while (h) {
        const uint32_t j = __ffs(h) - 1u;
        h &= h - 1u;
        const double p = __ldg(pos + base + j);
        uint32_t c = 0;
        for (uint32_t k = 0; k < E; ++k) c += (__ldg(ev + k) <= p) ? 1u : 0u;
        m |= (c & 1u) << j;
    }
    return m;
}

__device__ __forceinline__ void acc_effects(uint64_t x, uint32_t base, const float* __restrict__ eff, uint32_t T,
                                            float sign, float (&d)[kMaxTraits]) {
    if (T == 4) {
        while (x) {
            const uint32_t j = (uint32_t)(__ffsll((long long)x) - 1);
            x &= x - 1ull;
            const float4 e = __ldg(reinterpret_cast<const float4*>(eff) + base + j);
            d[0] = fmaf(sign, e.x, d[0]); d[1] = fmaf(sign, e.y, d[1]);
            d[2] = fmaf(sign, e.z, d[2]); d[3] = fmaf(sign, e.w, d[3]);
        }
    } else {
        while (x) {
            const uint32_t j = (uint32_t)(__ffsll((long long)x) - 1);
            x &= x - 1ull;
            const float* e = eff + (size_t)(base + j) * T;
#pragma unroll
            for (uint32_t t = 0; t < kMaxTraits; ++t)
                if (t < T) d[t] = fmaf(sign, __ldg(e + t), d[t]);
        }
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
enum XoKind : int { kXoCopy = 0, kXoReg2 = 2, kXoReg4 = 4, kXoReg8 = 8, kXoSmem = -1, kXoEvents = -2 };

template <int NI>
__device__ __forceinline__ void chunk_xover(uint64_t& x0, uint64_t& x1, uint64_t t0, uint64_t t1, uint64_t b0,
                                            uint64_t b1, uint32_t w, const PopDev& P, const Intervals& iv,
                                            const uint2* far, uint32_t nfar, const double* evg, uint32_t E,
                                            uint64_t& m0, uint64_t& m1) {
    const uint64_t h0 = t0 ^ b0, h1 = t1 ^ b1;
    const uint32_t s0 = w * 64u, s1 = s0 + 64u;
    if (NI >= -1) {
        m0 = (uint64_t)sw_mask32<NI>((uint32_t)h0, s0, P.rank, iv, far, nfar) |
             ((uint64_t)sw_mask32<NI>((uint32_t)(h0 >> 32), s0 + 32u, P.rank, iv, far, nfar) << 32);
        m1 = (uint64_t)sw_mask32<NI>((uint32_t)h1, s1, P.rank, iv, far, nfar) |
             ((uint64_t)sw_mask32<NI>((uint32_t)(h1 >> 32), s1 + 32u, P.rank, iv, far, nfar) << 32);
    } else {
        m0 = (uint64_t)sw_mask32_events((uint32_t)h0, s0, P.pos, evg, E) |
             ((uint64_t)sw_mask32_events((uint32_t)(h0 >> 32), s0 + 32u, P.pos, evg, E) << 32);
        m1 = (uint64_t)sw_mask32_events((uint32_t)h1, s1, P.pos, evg, E) |
             ((uint64_t)sw_mask32_events((uint32_t)(h1 >> 32), s1 + 32u, P.pos, evg, E) << 32);
    }
    x0 = (t0 & ~m0) | (b0 & m0);
    x1 = (t1 & ~m1) | (b1 & m1);
}

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

template <int NI>
__device__ __forceinline__ void row_body(const PopDev& P, const DevStatus& st, const RowArgs& R, const Intervals& iv,
                                         const uint2* far, uint32_t nfar, bool do_mut, bool do_ph, bool do_fs,
                                         uint64_t* sF, uint64_t* sV, float (&d)[kMaxTraits]) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool xo = (NI != 0);
    uint32_t w = 2u * lane;
    // prefetch of chunk 0
    ulonglong2 tt = make_ulonglong2(0, 0), bb = make_ulonglong2(0, 0), fm = make_ulonglong2(0, 0);
    if (w < R.Wp) {
        tt = __ldg(reinterpret_cast<const ulonglong2*>(R.top + w));
        if (xo) bb = __ldg(reinterpret_cast<const ulonglong2*>(R.bot + w));
        fm = *reinterpret_cast<const ulonglong2*>(P.fixmask + w);
    }
    for (uint32_t w0 = 0; w0 < R.Wc; w0 += 64u) {
        w = w0 + 2u * lane;
        const uint32_t wn = w + 64u;
        ulonglong2 tn = make_ulonglong2(0, 0), bn = make_ulonglong2(0, 0), fn = make_ulonglong2(0, 0);
        if (wn < R.Wp) {
            tn = __ldg(reinterpret_cast<const ulonglong2*>(R.top + wn));
            if (xo) bn = __ldg(reinterpret_cast<const ulonglong2*>(R.bot + wn));
            fn = *reinterpret_cast<const ulonglong2*>(P.fixmask + wn);
        }
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
        if (w < R.Wc) {
            const uint64_t t0 = tt.x & ~fm.x, t1 = tt.y & ~fm.y;
            uint64_t x0 = t0, x1 = t1;
            if (xo) {
                const uint64_t b0 = bb.x & ~fm.x, b1 = bb.y & ~fm.y;
                uint64_t m0, m1;
                chunk_xover<NI>(x0, x1, t0, t1, b0, b1, w, P, iv, far, nfar, R.evg, R.E, m0, m1);
                if (do_ph) {
                    // switched bits: +w where the bottom strand brings the allele, -w where it drops it
                    acc_effects(m0 & b0, w * 64u, P.eff, P.T, 1.0f, d);
                    acc_effects(m0 & t0, w * 64u, P.eff, P.T, -1.0f, d);
                    acc_effects(m1 & b1, (w + 1u) * 64u, P.eff, P.T, 1.0f, d);
                    acc_effects(m1 & t1, (w + 1u) * 64u, P.eff, P.T, -1.0f, d);
                }
            }
            x0 ^= mx0;
            x1 ^= mx1;
            *reinterpret_cast<ulonglong2*>(R.out + w) = make_ulonglong2(x0, x1);
            if (do_fs) {
                atomicAnd((unsigned long long*)&sF[w], (unsigned long long)x0);
                atomicAnd((unsigned long long*)&sF[w + 1u], (unsigned long long)x1);
                atomicOr((unsigned long long*)&sV[w], (unsigned long long)x0);
                atomicOr((unsigned long long*)&sV[w + 1u], (unsigned long long)x1);
            }
        }
        tt = tn;
        bb = bn;
        fm = fn;
    }
}

}  // namespace

__global__ void __launch_bounds__(kGenThreads, 3)
k_generation(const PopDev* __restrict__ pops, uint32_t npops, WorkCtl* __restrict__ ctl, uint32_t fuse,
             int profile) {
    extern __shared__ uint64_t s_acc[];  // [2 * maxW]: AND then OR accumulators
    __shared__ uint2 s_iv[kWarps][kMaxIvSmem];
    __shared__ uint32_t s_thr[kWarps][kMaxEvDevice];
    __shared__ uint32_t s_item;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const bool do_mut = (fuse & kFuseMut) != 0, do_ph = (fuse & kFusePheno) != 0, do_fs = (fuse & kFuseFs) != 0;
    int cur_pop = -1;
    uint32_t cur_W = 0;
    uint64_t* sF = s_acc;
    uint64_t* sV = s_acc;
    uint64_t rows_done = 0, words_done = 0;

    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&ctl->gen_counter, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        __syncthreads();
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
                __syncthreads();
            }
            cur_pop = (int)p;
            cur_W = st.W;
            sV = s_acc + cur_W;
            if (do_fs)
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) { sF[w] = ~0ull; sV[w] = 0ull; }
            __syncthreads();
        }

        const uint32_t S = 2u * st.N;
        const uint64_t* prow = P.rows[st.cur ^ 1u];
        uint64_t* crow = P.rows[st.cur];
        const double* zpar = P.zg[st.cur ^ 1u];
        double* zcur = P.zg[st.cur];
        const bool q1 = (P.flags & 1u) != 0;
        const bool philox = P.mode == kModePhilox;
        const uint32_t row0 = (item - ctl->item_base[p]) * kRowsPerItem + warp * (kRowsPerItem / kWarps);

        for (uint32_t rr = 0; rr < kRowsPerItem / kWarps; ++rr) {
            const uint32_t g = row0 + rr;
            if (g >= S) break;
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
            Intervals iv;
#pragma unroll
            for (uint32_t k = 0; k < kMaxIv; ++k) { iv.a[k] = 0; iv.l[k] = 0; }
            uint32_t nfar = 0;
            int kind = kXoCopy;
            if (E > 0 && E <= kMaxEvDevice) {
                // thresholds, lane-strided, into the warp's shared buffer
                for (uint32_t k = lane; k < E; k += 32u) {
                    double e;
                    if (philox) {
                        const U4 a = philox4x32(g, 1u + (k >> 1), st.gen, kStreamGamete, P.seed);
                        e = (k & 1u) ? u01(a.z, a.w) : u01(a.x, a.y);
                    } else {
                        e = __ldg(evg + k);
                    }
                    s_thr[warp][k] = threshold_rank(P, e);
                }
                __syncwarp();
                // stable rank sort of the thresholds
                uint32_t mine[4], posn[4];
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) {
                    const uint32_t k = lane + 32u * q;
                    mine[q] = (k < E) ? s_thr[warp][k] : 0u;
                    posn[q] = 0;
                }
                for (uint32_t j = 0; j < E; ++j) {
                    const uint32_t tj = s_thr[warp][j];
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
                    if (k < E) s_thr[warp][posn[q]] = mine[q];
                }
                __syncwarp();
                const uint32_t NI = (E + 1u) >> 1;
                for (uint32_t i = lane; i < NI; i += 32u) {
                    const uint32_t a = s_thr[warp][2u * i];
                    uint32_t l;
                    if (2u * i + 1u < E) l = s_thr[warp][2u * i + 1u] - a;
                    else l = a ? (uint32_t)(0x100000000ull - a) : 0xffffffffu;
                    s_iv[warp][i] = make_uint2(a, l);
                }
                __syncwarp();
                if (NI <= kMaxIv) {
#pragma unroll
                    for (uint32_t k = 0; k < kMaxIv; ++k) {
                        if (k < NI) { iv.a[k] = s_iv[warp][k].x; iv.l[k] = s_iv[warp][k].y; }
                    }
                    kind = NI <= 2 ? kXoReg2 : (NI <= 4 ? kXoReg4 : kXoReg8);
                } else {
                    nfar = NI;
                    kind = kXoSmem;
                }
            } else if (E > kMaxEvDevice) {
                kind = kXoEvents;  // tape rows with very long event lists
            }

            // ---- new alleles of this row (slot indices), lanes hold up to 32
            R.mo = 0;
            R.mc = 0;
            R.my_slot = 0xffffffffu;
            float d[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
            if (do_mut) {
                R.mo = P.row_off[g];
                R.mc = P.row_off[g + 1u] - R.mo;
                if (lane < R.mc) {
                    const uint32_t i = R.mo + lane;
                    const uint32_t mi = philox ? i : P.row_mut[i];
                    R.my_slot = (mi < st.M) ? P.mut_slot[mi] : 0xffffffffu;
                    if (do_ph && R.my_slot != 0xffffffffu) {
#pragma unroll
                        for (uint32_t t = 0; t < kMaxTraits; ++t)
                            if (t < P.T) d[t] += __ldg(P.eff + (size_t)R.my_slot * P.T + t);
                    }
                }
                if (do_ph && R.mc > 32u && lane == 0) {
                    for (uint32_t j = 32; j < R.mc; ++j) {
                        const uint32_t mi = philox ? R.mo + j : P.row_mut[R.mo + j];
                        if (mi >= st.M) continue;
                        const uint32_t s = P.mut_slot[mi];
                        if (s == 0xffffffffu) continue;
#pragma unroll
                        for (uint32_t t = 0; t < kMaxTraits; ++t)
                            if (t < P.T) d[t] += __ldg(P.eff + (size_t)s * P.T + t);
                    }
                }
            }

            const uint2* far = s_iv[warp];
            switch (kind) {
                case kXoCopy: row_body<0>(P, st, R, iv, far, 0, do_mut, do_ph, do_fs, sF, sV, d); break;
                case kXoReg2: row_body<2>(P, st, R, iv, far, 0, do_mut, do_ph, do_fs, sF, sV, d); break;
                case kXoReg4: row_body<4>(P, st, R, iv, far, 0, do_mut, do_ph, do_fs, sF, sV, d); break;
                case kXoReg8: row_body<8>(P, st, R, iv, far, 0, do_mut, do_ph, do_fs, sF, sV, d); break;
                case kXoSmem: row_body<-1>(P, st, R, iv, far, nfar, do_mut, do_ph, do_fs, sF, sV, d); break;
                default: row_body<-2>(P, st, R, iv, far, 0, do_mut, do_ph, do_fs, sF, sV, d); break;
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
                    const double zt = zpar[(size_t)topr * 4u + lane];
                    const double zz = lane == 0 ? z[0] : lane == 1 ? z[1] : lane == 2 ? z[2] : z[3];
                    zcur[(size_t)g * 4u + lane] = (zt - P.st->fixsum[lane]) + zz;
                }
            }
            if (profile && lane == 0) { rows_done += 1; words_done += st.W; }
        }
    }
    if (cur_pop >= 0 && do_fs) {
        __syncthreads();
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

void launch_generation(const LaunchCfg& L, const PopDev* pops, uint32_t npops, WorkCtl* ctl, uint32_t maxW,
                       uint32_t fuse, int profile) {
    const size_t smem = 2ull * maxW * sizeof(uint64_t);
    static size_t configured = 0;
    static size_t occ_smem = ~(size_t)0;
    static int occ = 1;
    if (smem > 48u * 1024u && smem > configured) {
        cudaFuncSetAttribute(k_generation, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    if (occ_smem != smem) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_generation, kGenThreads, smem);
        occ = per_sm < 1 ? 1 : per_sm;
        occ_smem = smem;
    }
    k_generation<<<L.num_sms * occ, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse, profile);
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
                acc_effects(x.x, w * 64u, P.eff, P.T, 1.0f, d);
                acc_effects(x.y, (w + 1u) * 64u, P.eff, P.T, 1.0f, d);
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
