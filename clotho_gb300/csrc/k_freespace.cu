// k_freespace.cu -- free-space analysis of a population_space_row.
//
// Restates FreeSpaceAnalyzerMT<population_space_row>
// (data_spaces/free_space/free_space_mt_population_space_row_interlaced.hpp:41-121)
// and free_space_details::analyze_free_indices (free_space_details.hpp:299-357)
// for the GPU:
//  * k_fs_reduce  -- AND (fixed) / OR (variable) of every column over all rows,
//                    coalesced 128-bit row loads, folded into per-population
//                    accF/accV with global atomics.  In the fused path this
//                    reduction is done in the epilogue of the generation kernel
//                    and this kernel is only used for a freshly loaded population.
//  * k_fs_finalize -- tail padding, ordered compaction (fixed indices ascending,
//                    then lost indices ascending), fixed-table append
//                    (engine_batched_task.hpp:303-345) and the child allele
//                    count (child_max_alleles, :287-301).
#include "engine.cuh"

namespace clotho {

// which == 0: the current child rows; which == 1: the parent of the step in progress.
__global__ void __launch_bounds__(256) k_fs_reduce(const PopDev* __restrict__ pops, uint32_t npops,
                                                   uint32_t which) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const DevStatus st = *P.st;
        const uint32_t S = 2u * (which ? st.pN : st.N);
        const uint32_t W = which ? st.pW : st.W;
        const uint64_t* rows = P.rows[which ? (st.cur ^ 1u) : st.cur];
        const uint32_t nchunks = (W + 511u) / 512u;  // 256 threads x 2 words
        if (S == 0 || W == 0) continue;
        const uint32_t groups = gridDim.y;
        const uint32_t rows_per = (S + groups - 1) / groups;
        const uint32_t r0 = blockIdx.y * rows_per, r1 = min(S, r0 + rows_per);
        if (r0 >= r1) continue;
        for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
            const uint32_t w = c * 512u + 2u * threadIdx.x;
            if (w >= W) continue;
            uint64_t f0 = ~0ull, f1 = ~0ull, v0 = 0, v1 = 0;
            for (uint32_t r = r0; r < r1; ++r) {
                const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(rows + (size_t)r * P.Wcap + w);
                f0 &= x.x; f1 &= x.y; v0 |= x.x; v1 |= x.y;
            }
            atomicAnd((unsigned long long*)&P.accF[w], (unsigned long long)f0);
            atomicAnd((unsigned long long*)&P.accF[w + 1], (unsigned long long)f1);
            atomicOr((unsigned long long*)&P.accV[w], (unsigned long long)v0);
            atomicOr((unsigned long long*)&P.accV[w + 1], (unsigned long long)v1);
        }
    }
}

void launch_fs_reduce(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxW, uint32_t which) {
    const dim3 pg = pop_grid(npops, 0x7fffffffu, L.num_sms, 4);  // blocks per population in pg.x
    const uint32_t gx = max(1u, min(16u, (maxW + 511u) / 512u));
    const dim3 grid(gx, max(1u, pg.x / gx), pg.z);
    k_fs_reduce<<<grid, 256, 0, L.stream>>>(pops, npops, which);
}

// Block-wide exclusive scan of one value per thread (1024 threads).
__device__ inline uint32_t block_excl_scan_1024(uint32_t v, uint32_t* s_warp, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        s_warp[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    total = s_warp[31];
    uint32_t excl = x - v + (warp ? s_warp[warp - 1] : 0u);
    __syncthreads();
    return excl;
}

// Column state of word w of the parent after the reference's tail padding
// (free_space_mt_population_space_row_interlaced.hpp:52-81): F = fixed bits,
// L = lost bits; padding bits are neither.
__device__ inline void padded_word(const PopDev& P, uint32_t w, uint32_t W, uint32_t A, uint32_t S,
                                   uint64_t& F, uint64_t& L) {
    if (w >= W) { F = 0; L = 0; return; }
    if (S == 0) {  // no genomes: every bit of every word reads as lost (:52-56)
        F = 0;
        L = ~0ull;
        return;
    }
    uint64_t valid;
    const uint32_t b = w * 64u;
    if (b + 64u <= A) valid = ~0ull;
    else if (b >= A) valid = 0ull;
    else valid = (1ull << (A - b)) - 1ull;
    F = P.accF[w] & valid;
    L = ~(P.accV[w] | ~valid);
}

__global__ void __launch_bounds__(1024) k_fs_finalize(const PopDev* __restrict__ pops, uint32_t count_on) {
    const PopDev& P = pops[blockIdx.x];
    DevStatus* st = P.st;
    // column counts of this step's child rows, for the populations that asked: zeroed here, added by the
    // generation kernel's counting build
    // the bitmap builds of the suffix-table classifier count (capacity <= kSufMaxSlots)
    const bool counting = count_on && st->count_cols != 0u && P.suf != nullptr && P.Acap <= kSufMaxSlots;
    if (counting)
        for (uint32_t a = threadIdx.x; a < P.Acap; a += 1024u) P.colcnt[a] = 0u;
    __shared__ uint32_t s_warp[32];
    const uint32_t pA = st->pA, pW = st->pW, pS = 2u * st->pN, M = st->M;
    const uint32_t fx_base = st->fixed_total;
    uint32_t totF = 0, totL = 0;
    __shared__ double s_fx[32][kMaxTraits];
    double fsum[kMaxTraits] = {0.0, 0.0, 0.0, 0.0};
    if (pA > 0) {
        // pass 1: totals
        uint32_t cf = 0, cl = 0;
        for (uint32_t w = threadIdx.x; w < pW; w += 1024u) {
            uint64_t F, L;
            padded_word(P, w, pW, pA, pS, F, L);
            cf += __popcll(F);
            cl += __popcll(L);
        }
        uint32_t t0, t1;
        block_excl_scan_1024(cf, s_warp, t0);
        block_excl_scan_1024(cl, s_warp, t1);
        totF = t0;
        totL = t1;
        // pass 2: ordered writes, 1024 words per round
        uint32_t base_f = 0, base_l = totF;
        for (uint32_t c = 0; c < pW; c += 1024u) {
            const uint32_t w = c + threadIdx.x;
            uint64_t F, L;
            padded_word(P, w, pW, pA, pS, F, L);
            uint32_t tf, tl;
            uint32_t of = block_excl_scan_1024(__popcll(F), s_warp, tf);
            uint32_t ol = block_excl_scan_1024(__popcll(L), s_warp, tl);
            if (w < pW) {
                uint32_t i = base_f + of;
                for (uint64_t b = F; b; b &= b - 1ull) {
                    const uint32_t slot = w * 64u + (uint32_t)(__ffsll((long long)b) - 1);
                    P.free_list[i] = slot;
                    const uint32_t k = fx_base + i;
                    for (uint32_t t = 0; t < P.T; ++t) fsum[t] += (double)P.eff[(size_t)slot * 4u + t];
                    if (k < P.FXcap) {  // m_fixed.append / m_fixed_traits.append (:315-324)
                        P.fx_pos[k] = P.pos[slot];
                        P.fx_age[k] = P.age[slot];
                        for (uint32_t t = 0; t < P.T; ++t) P.fx_eff[(size_t)k * P.T + t] = P.eff[(size_t)slot * 4u + t];
                    }
                    ++i;
                }
                i = base_l + ol;
                for (uint64_t b = L; b; b &= b - 1ull) P.free_list[i++] = w * 64u + (uint32_t)(__ffsll((long long)b) - 1);
                P.fixmask[w] = F;
            }
            base_f += tf;
            base_l += tl;
        }
    }
    // effect sum of the fixed alleles (every parent row carries them): the
    // generation pass subtracts it from the carried per-genome sums
#pragma unroll
    for (uint32_t t = 0; t < kMaxTraits; ++t) {
        double v = fsum[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31u) == 0) s_fx[threadIdx.x >> 5][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < kMaxTraits) {
        double v = 0.0;
        for (int i = 0; i < 32; ++i) v += s_fx[i][threadIdx.x];
        st->fixsum[threadIdx.x] = v;
    }
    // reset the accumulators for the child of this step
    for (uint32_t w = threadIdx.x; w < P.Wcap; w += 1024u) {
        P.accF[w] = ~0ull;
        P.accV[w] = 0ull;
    }
    if (threadIdx.x == 0) {
        if (pA > 0) {
            st->fixed_cnt = totF;
            st->lost_cnt = totL;
            st->free_cnt = totF + totL;
            if (fx_base + totF > P.FXcap) st->err |= kErrFixed;
            st->fixed_total = min(P.FXcap, fx_base + totF);
        }
        const uint32_t fr = st->free_cnt;
        const uint32_t Ac = st->pA + (M > fr ? M - fr : 0u);
        if (Ac > P.Acap) {
            st->err |= kErrAlleles;
            st->A = P.Acap;
        } else {
            st->A = Ac;
        }
        st->W = ref_width(st->A);
        st->cols_valid = counting ? 1u : 0u;
    }
}

void launch_fs_finalize(const LaunchCfg& L, const PopDev* pops, uint32_t npops, bool count_on) {
    k_fs_finalize<<<npops, 1024, 0, L.stream>>>(pops, count_on ? 1u : 0u);
}

}  // namespace clotho
